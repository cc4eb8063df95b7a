// ppf_step.cu -- sm_103a kernels of the explicit Moelans/KKS step.
//
// One kernel per time step replaces the reference's four passes
// (BC fill phasefield.c:1112-1189, pass A :325-335, pass B :347-391,
// pass C :393-401) -- the step is forward Euler, so reading the old state
// and writing the new one into a second buffer is exactly equivalent.
//
// Shape of the fused step: a CTA owns a TX x TY tile of one x-y plane and
// marches ZC planes up z.  For every plane it loads etaS/etaL/c of the tile
// plus a one-cell ring, evaluates the pointwise pass-A quantities (hS, mu,
// M) once per loaded cell, and keeps them in one of three shared-memory
// plane buffers; the z-neighbours of a thread's own cells stay in
// registers.  The 7-point stencils of pass B then read x/y neighbours from
// shared memory.  Loads of plane z+1 are issued before plane z is
// computed.  Boundary conditions are applied on the write side: a cell on
// a domain face also writes its value into the ghost it feeds (periodic
// wrap or no-flux copy), so the next step reads a ready ghost layer.
#include <cuda_runtime.h>

#include <cstdint>

#include "ppf_internal.h"

namespace ppf {

template <typename T>
__device__ __forceinline__ T rcp(T x);
template <>
__device__ __forceinline__ double rcp<double>(double x) { return __drcp_rn(x); }
template <>
__device__ __forceinline__ float rcp<float>(float x) { return __frcp_rn(x); }

// pass A of sweep_fields (phasefield.c:328-332) for one cell; also returns
// 1/(etaS^2+etaL^2) and 1/(AS+(AL-AS)hS), reused by pass B at the centre.
template <typename T>
__device__ __forceinline__ void point(const Coef<T> &k, T eS, T eL, T c, T &mu, T &M, T &h, T &rs,
                                      T &rA) {
    T s2 = eS * eS + eL * eL;
    rs = rcp(s2);
    h = eS * eS * rs;
    rA = rcp(k.AS + k.dA * h);
    mu = k.AsAl * rA * (c - k.cL0 + k.dc0 * h);
    M = k.ML + k.dM * h;
}

// Face-ghost targets of an interior index i in [0, n): the ghost that the
// BC fill would copy this cell into (-2 = none).
__device__ __forceinline__ void ghost_targets(int i, int n, int bc, int &g0, int &g1) {
    g0 = -2;
    g1 = -2;
    if (i == 0) g0 = (bc == 0) ? n : -1;          // periodic: ghost n = cell 0; no-flux: ghost -1
    if (i == n - 1) g1 = (bc == 0) ? -1 : n;      // periodic: ghost -1 = cell n-1
}

template <typename T>
__device__ __forceinline__ void store3(const Geom &g, Fields<T> out, int x, int y, int z, T s, T l, T c,
                                       bool c_only) {
    int64_t i = g.at(x, y, z);
    if (!c_only) {
        out.eS[i] = s;
        out.eL[i] = l;
    }
    out.c[i] = c;
}

template <typename T>
__device__ __forceinline__ void store_with_ghosts(const Geom &g, Fields<T> out, int x, int y, int z, T s,
                                                  T l, T c, bool c_only) {
    store3(g, out, x, y, z, s, l, c, c_only);
    int a, b;
    ghost_targets(x, g.nx, g.bc, a, b);
    if (a != -2) store3(g, out, a, y, z, s, l, c, c_only);
    if (b != -2) store3(g, out, b, y, z, s, l, c, c_only);
    ghost_targets(y, g.ny, g.bc, a, b);
    if (a != -2) store3(g, out, x, a, z, s, l, c, c_only);
    if (b != -2) store3(g, out, x, b, z, s, l, c, c_only);
    ghost_targets(z, g.nz, g.bc, a, b);
    if (a != -2) store3(g, out, x, y, a, s, l, c, c_only);
    if (b != -2) store3(g, out, x, y, b, s, l, c, c_only);
}

template <int TX, int TY>
__device__ __forceinline__ void ring_pos(int r, int &hx, int &hy) {
    if (r < TX) { hx = r; hy = -1; }
    else if (r < 2 * TX) { hx = r - TX; hy = TY; }
    else if (r < 2 * TX + TY) { hx = -1; hy = r - 2 * TX; }
    else { hx = TX; hy = r - 2 * TX - TY; }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NV doubles per thread; thread 0 writes partials[NV*b+i].
template <int NT, int NV>
__device__ __forceinline__ void block_sum_store(double (&v)[NV], double *partials, int b) {
    __shared__ double red[NT / 32][NV];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = warp_sum(v[i]);
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) red[w][i] = v[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = 0;
            for (int q = 0; q < NT / 32; ++q) s += red[q][i];
            partials[(int64_t)NV * b + i] = s;
        }
    }
}

template <typename T, int TX, int TY, int NT, bool STATS, bool C_ONLY>
__global__ void __launch_bounds__(NT, 2)
    step_kernel(Geom g, Coef<T> k, Fields<const T> in, Fields<T> out, int zc, double *__restrict__ partials) {
    constexpr int SX = TX + 2, SP = SX * (TY + 2);
    constexpr int CPT = TX * TY / NT;
    constexpr int ROWS = NT / TX;
    constexpr int RING = 2 * TX + 2 * TY;
    constexpr int RPT = (RING + NT - 1) / NT;
    constexpr int NF = C_ONLY ? 2 : 4;   // smem fields: [etaS, etaL,] mu, M
    constexpr int FMU = C_ONLY ? 0 : 2, FM = FMU + 1;
    static_assert((TX * TY) % NT == 0 && NT % TX == 0, "tile/threads mismatch");
    __shared__ T sm[3][NF][SP];

    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, g.nz);
    const int cx = tid % TX, cy0 = tid / TX;
    const int X = x0 + cx;

    // loaded (not yet computed) values of one plane
    T lS[CPT], lL[CPT], lc[CPT], rS[RPT], rL[RPT], rc[RPT];
    auto load_plane = [&](int pz) {
#pragma unroll
        for (int q = 0; q < CPT; ++q) {
            const int Y = y0 + cy0 + q * ROWS;
            lS[q] = T(1); lL[q] = T(0); lc[q] = T(0);
            if (X <= g.nx && Y <= g.ny) {
                const int64_t i = g.at(X, Y, pz);
                lS[q] = __ldg(in.eS + i);
                lL[q] = __ldg(in.eL + i);
                lc[q] = __ldg(in.c + i);
            }
        }
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            const int r = tid + q * NT;
            rS[q] = T(1); rL[q] = T(0); rc[q] = T(0);
            if (r < RING) {
                int hx, hy;
                ring_pos<TX, TY>(r, hx, hy);
                const int XX = x0 + hx, YY = y0 + hy;
                if (XX >= -1 && XX <= g.nx && YY >= -1 && YY <= g.ny) {
                    const int64_t i = g.at(XX, YY, pz);
                    rS[q] = __ldg(in.eS + i);
                    rL[q] = __ldg(in.eL + i);
                    rc[q] = __ldg(in.c + i);
                }
            }
        }
    };

    // plane q-1 (prev), plane q (cur) of the thread's own cells
    T pS[CPT], pL[CPT], pmu[CPT], pM[CPT];
    T qS[CPT], qL[CPT], qmu[CPT], qM[CPT], qc[CPT], qh[CPT], qrs[CPT], qrA[CPT];
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
        pS[q] = pL[q] = pmu[q] = pM[q] = T(0);
        qS[q] = qL[q] = qmu[q] = qM[q] = qc[q] = qh[q] = qrs[q] = qrA[q] = T(0);
    }
    double acc[3] = {0.0, 0.0, 0.0};

    load_plane(z0 - 1);
    for (int pz = z0 - 1; pz <= z1; ++pz) {
        const int bw = (pz - z0 + 1) % 3;   // buffer of plane pz
        const int br = (pz - z0 + 3) % 3;   // buffer of plane pz-1
        T cS_[CPT], cL_[CPT], cc_[CPT], crS[RPT], crL[RPT], crc[RPT];
#pragma unroll
        for (int q = 0; q < CPT; ++q) { cS_[q] = lS[q]; cL_[q] = lL[q]; cc_[q] = lc[q]; }
#pragma unroll
        for (int q = 0; q < RPT; ++q) { crS[q] = rS[q]; crL[q] = rL[q]; crc[q] = rc[q]; }
        if (pz + 1 <= z1) load_plane(pz + 1);

        // pass A for the plane: own cells into registers + smem, ring into smem
        T xS[CPT], xL[CPT], xmu[CPT], xM[CPT], xc[CPT], xh[CPT], xrs[CPT], xrA[CPT];
#pragma unroll
        for (int q = 0; q < CPT; ++q) {
            point(k, cS_[q], cL_[q], cc_[q], xmu[q], xM[q], xh[q], xrs[q], xrA[q]);
            xS[q] = cS_[q]; xL[q] = cL_[q]; xc[q] = cc_[q];
            const int s = (cy0 + q * ROWS + 1) * SX + cx + 1;
            if (!C_ONLY) { sm[bw][0][s] = xS[q]; sm[bw][1][s] = xL[q]; }
            sm[bw][FMU][s] = xmu[q];
            sm[bw][FM][s] = xM[q];
        }
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            const int r = tid + q * NT;
            if (r < RING) {
                int hx, hy;
                ring_pos<TX, TY>(r, hx, hy);
                T mu, M, h, rs, rA;
                point(k, crS[q], crL[q], crc[q], mu, M, h, rs, rA);
                const int s = (hy + 1) * SX + hx + 1;
                if (!C_ONLY) { sm[bw][0][s] = crS[q]; sm[bw][1][s] = crL[q]; }
                sm[bw][FMU][s] = mu;
                sm[bw][FM][s] = M;
            }
        }
        __syncthreads();

        // pass B + C for plane pz-1
        const int zq = pz - 1;
        if (zq >= z0) {
#pragma unroll
            for (int q = 0; q < CPT; ++q) {
                const int Y = y0 + cy0 + q * ROWS;
                if (X < g.nx && Y < g.ny) {
                    const int s = (cy0 + q * ROWS + 1) * SX + cx + 1;
                    const T *smu = sm[br][FMU], *sM = sm[br][FM];
                    const T mu = qmu[q], M = qM[q];
                    // solute: sum over faces of (M_nb + M_0)(mu_nb - mu_0), the
                    // flux form of phasefield.c:374-384
                    const T fl = (xM[q] + M) * (xmu[q] - mu) + (pM[q] + M) * (pmu[q] - mu) +
                                 (sM[s + SX] + M) * (smu[s + SX] - mu) + (sM[s - SX] + M) * (smu[s - SX] - mu) +
                                 (sM[s + 1] + M) * (smu[s + 1] - mu) + (sM[s - 1] + M) * (smu[s - 1] - mu);
                    const T dc = k.tmp3 * fl;
                    const T c = qc[q];
                    if (C_ONLY) {
                        store_with_ghosts(g, out, X, Y, zq, T(0), T(0), c + dc, true);
                        if (STATS) acc[0] += (double)dc * (double)dc;
                    } else {
                        const T eS = qS[q], eL = qL[q], h = qh[q], rA = qrA[q], rs = qrs[q];
                        const T *sS = sm[br][0], *sL = sm[br][1];
                        // KKS phase compositions and parabolas, :351-355
                        const T cSp = rA * (k.AL * c + (T(1) - h) * k.tmp2);
                        const T cLp = rA * (k.AS * c - h * k.tmp2);
                        const T fS = k.halfAS * (cSp - k.cS0) * (cSp - k.cS0) + k.CS;
                        const T fL = k.halfAL * (cLp - k.cL0) * (cLp - k.cL0) + k.CL;
                        const T dmu = T(2) * (eS * eL) * (rs * rs) * (fS - fL - mu * (cSp - cLp));   // :356-359
                        const T lapS = xS[q] + pS[q] + sS[s + SX] + sS[s - SX] + sS[s + 1] + sS[s - 1] - T(6) * eS;
                        const T lapL = xL[q] + pL[q] + sL[s + SX] + sL[s - SX] + sL[s + 1] + sL[s - 1] - T(6) * eL;
                        const T dS = k.tmp1 * (k.m * eS * (eS * eS - T(1) + k.twogam * eL * eL) - k.kh2 * lapS + eL * dmu);
                        const T dL = k.tmp1 * (k.m * eL * (eL * eL - T(1) + k.twogam * eS * eS) - k.kh2 * lapL - eS * dmu);
                        store_with_ghosts(g, out, X, Y, zq, eS + dS, eL + dL, c + dc, false);
                        if (STATS) {
                            acc[0] += (double)dc * (double)dc;
                            acc[1] += (double)dS * (double)dS;
                            acc[2] += (double)dL * (double)dL;
                        }
                    }
                }
            }
        }
        // rotate: q -> prev, x -> cur
#pragma unroll
        for (int q = 0; q < CPT; ++q) {
            pS[q] = qS[q]; pL[q] = qL[q]; pmu[q] = qmu[q]; pM[q] = qM[q];
            qS[q] = xS[q]; qL[q] = xL[q]; qmu[q] = xmu[q]; qM[q] = xM[q];
            qc[q] = xc[q]; qh[q] = xh[q]; qrs[q] = xrs[q]; qrA[q] = xrA[q];
        }
    }
    if (STATS) {
        const int b = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        block_sum_store<NT, 3>(acc, partials, b);
    }
}

template <typename T>
struct StepCfg;
template <>
struct StepCfg<float> {
    static constexpr int TX = 64, TY = 8, NT = 256;
};
template <>
struct StepCfg<double> {
    static constexpr int TX = 32, TY = 8, NT = 256;
};

template <typename T>
int step_blocks(const Geom &g, int zc) {
    using C = StepCfg<T>;
    return ((g.nx + C::TX - 1) / C::TX) * ((g.ny + C::TY - 1) / C::TY) * ((g.nz + zc - 1) / zc);
}

template <typename T>
cudaError_t launch_step(const Geom &g, const Coef<T> &k, Fields<const T> in, Fields<T> out, bool c_only,
                        double *partials, int zc, cudaStream_t s, int *nblocks) {
    using C = StepCfg<T>;
    if (zc < 1) zc = 1;
    dim3 grid((g.nx + C::TX - 1) / C::TX, (g.ny + C::TY - 1) / C::TY, (g.nz + zc - 1) / zc);
    if (nblocks) *nblocks = (int)(grid.x * grid.y * grid.z);
    const bool st = partials != nullptr;
    if (!c_only) {
        if (st) step_kernel<T, C::TX, C::TY, C::NT, true, false><<<grid, C::NT, 0, s>>>(g, k, in, out, zc, partials);
        else step_kernel<T, C::TX, C::TY, C::NT, false, false><<<grid, C::NT, 0, s>>>(g, k, in, out, zc, partials);
    } else {
        if (st) step_kernel<T, C::TX, C::TY, C::NT, true, true><<<grid, C::NT, 0, s>>>(g, k, in, out, zc, partials);
        else step_kernel<T, C::TX, C::TY, C::NT, false, true><<<grid, C::NT, 0, s>>>(g, k, in, out, zc, partials);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------- pack ----

template <typename T>
__global__ void pack_kernel(Geom g, const double *__restrict__ src, Fields<T> dst) {
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx);
        const int y = (int)((i / g.nx) % g.ny);
        const int z = (int)(i / ((int64_t)g.nx * g.ny));
        store_with_ghosts(g, dst, x, y, z, (T)src[i], (T)src[n + i], (T)src[2 * n + i], false);
    }
}

template <typename T>
__global__ void unpack_kernel(Geom g, Fields<const T> src, double *__restrict__ dst) {
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx);
        const int y = (int)((i / g.nx) % g.ny);
        const int z = (int)(i / ((int64_t)g.nx * g.ny));
        const int64_t j = g.at(x, y, z);
        dst[i] = (double)src.eS[j];
        dst[n + i] = (double)src.eL[j];
        dst[2 * n + i] = (double)src.c[j];
    }
}

static int grid_for(int64_t n, int nt) {
    int64_t b = (n + nt - 1) / nt;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

template <typename T>
cudaError_t launch_pack(const Geom &g, const double *src3, Fields<T> dst, cudaStream_t s) {
    pack_kernel<T><<<grid_for((int64_t)g.nx * g.ny * g.nz, 256), 256, 0, s>>>(g, src3, dst);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_unpack(const Geom &g, Fields<const T> src, double *dst3, cudaStream_t s) {
    unpack_kernel<T><<<grid_for((int64_t)g.nx * g.ny * g.nz, 256), 256, 0, s>>>(g, src, dst3);
    return cudaGetLastError();
}

// ----------------------------------------------------------- observables --
// Energy density in the step's precision, accumulated in double.  Free
// energy density (no counterpart in the reference; its variational
// derivative is the bracket of phasefield.c:360-373):
//   m f0(etaS, etaL) + kappa/2 |grad eta|^2 (forward differences) + hS fS + (1-hS) fL

template <typename T>
__global__ void __launch_bounds__(256) observe_kernel(Geom g, CoefD kd, Fields<const T> f, double *partials) {
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const T AS = (T)kd.AS, AL = (T)kd.AL, dA = (T)kd.dA, cS0 = (T)kd.cS0, cL0 = (T)kd.cL0;
    const T CS = (T)kd.CS, CL = (T)kd.CL, tmp2 = (T)kd.tmp2, m = (T)kd.m, gam = (T)kd.gamma;
    const T kg = (T)kd.kappa_h2_half;
    double acc[5] = {0, 0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx);
        const int y = (int)((i / g.nx) % g.ny);
        const int z = (int)(i / ((int64_t)g.nx * g.ny));
        const int64_t j = g.at(x, y, z);
        const T eS = f.eS[j], eL = f.eL[j], c = f.c[j];
        if (!isfinite((double)eS) || !isfinite((double)eL) || !isfinite((double)c)) {
            acc[4] += 1.0;
            continue;
        }
        // +x/+y/+z neighbours read through the ghost layer (periodic wrap or no-flux copy)
        const T sx = f.eS[j + 1], sy = f.eS[j + g.P], sz = f.eS[j + g.PS];
        const T lx = f.eL[j + 1], ly = f.eL[j + g.P], lz = f.eL[j + g.PS];
        const T s2 = eS * eS + eL * eL;
        const T h = eS * eS / s2;
        const T f0 = eS * eS * eS * eS / T(4) - eS * eS / T(2) + eL * eL * eL * eL / T(4) - eL * eL / T(2) +
                     gam * eS * eS * eL * eL + T(0.25);
        const T gr = (sx - eS) * (sx - eS) + (lx - eL) * (lx - eL) + (sy - eS) * (sy - eS) + (ly - eL) * (ly - eL) +
                     (sz - eS) * (sz - eS) + (lz - eL) * (lz - eL);
        const T rA = T(1) / (AS + dA * h);
        const T cSp = rA * (AL * c + (T(1) - h) * tmp2);
        const T cLp = rA * (AS * c - h * tmp2);
        const T fS = T(0.5) * AS * (cSp - cS0) * (cSp - cS0) + CS;
        const T fL = T(0.5) * AL * (cLp - cL0) * (cLp - cL0) + CL;
        acc[0] += (double)c;
        acc[1] += (double)h;
        acc[2] += eS > T(0.5) ? 1.0 : 0.0;
        acc[3] += kd.vol * ((double)(m * f0) + (double)(kg * gr) + (double)(h * fS) + (double)((T(1) - h) * fL));
    }
    block_sum_store<256, 5>(acc, partials, blockIdx.x);
}

template <typename T>
cudaError_t launch_observe(const Geom &g, const CoefD &k, Fields<const T> f, double *partials, int nblocks,
                           cudaStream_t s) {
    observe_kernel<T><<<nblocks, 256, 0, s>>>(g, k, f, partials);
    return cudaGetLastError();
}

__global__ void final_sum_kernel(const double *__restrict__ partials, int nblocks, int stride, int nvals,
                                 double *out) {
    __shared__ double red[256];
    for (int v = 0; v < nvals; ++v) {
        double s = 0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[(int64_t)stride * b + v];
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = 128; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[v] = red[0];
        __syncthreads();
    }
}

cudaError_t launch_final_sum(const double *partials, int nblocks, int stride, int nvals, double *out,
                             cudaStream_t s) {
    final_sum_kernel<<<1, 256, 0, s>>>(partials, nblocks, stride, nvals, out);
    return cudaGetLastError();
}

// explicit instantiations
template int step_blocks<float>(const Geom &, int);
template int step_blocks<double>(const Geom &, int);
template cudaError_t launch_step<float>(const Geom &, const Coef<float> &, Fields<const float>, Fields<float>,
                                        bool, double *, int, cudaStream_t, int *);
template cudaError_t launch_step<double>(const Geom &, const Coef<double> &, Fields<const double>,
                                         Fields<double>, bool, double *, int, cudaStream_t, int *);
template cudaError_t launch_pack<float>(const Geom &, const double *, Fields<float>, cudaStream_t);
template cudaError_t launch_pack<double>(const Geom &, const double *, Fields<double>, cudaStream_t);
template cudaError_t launch_unpack<float>(const Geom &, Fields<const float>, double *, cudaStream_t);
template cudaError_t launch_unpack<double>(const Geom &, Fields<const double>, double *, cudaStream_t);
template cudaError_t launch_observe<float>(const Geom &, const CoefD &, Fields<const float>, double *, int,
                                           cudaStream_t);
template cudaError_t launch_observe<double>(const Geom &, const CoefD &, Fields<const double>, double *, int,
                                            cudaStream_t);

}  // namespace ppf
