// ppf_state.cu -- state movement and reductions around the fused step:
// pack/unpack between the caller's compact [z][y][x] double arrays and the
// padded ghosted device layout (the BC fill of phasefield.c:207-211 is done
// on pack), the observables reduction (FP64 accumulation) and the
// deterministic final sum of per-CTA partials.
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "ppf_internal.h"

namespace ppf {

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
__global__ void pack_multi_kernel(const IoDesc *__restrict__ table) {
    const IoDesc &d = table[blockIdx.y];
    const Geom g = d.g;
    const Fields<T> dst = {(T *)d.fld[0][0], (T *)d.fld[0][1], (T *)d.fld[0][2]};
    const double *src = d.staging;
    if (blockIdx.x == 0 && threadIdx.x < 3) d.dres[threadIdx.x] = 0.0;
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx);
        const int y = (int)((i / g.nx) % g.ny);
        const int z = (int)(i / ((int64_t)g.nx * g.ny));
        store_with_ghosts(g, dst, x, y, z, (T)src[i], (T)src[n + i], (T)src[2 * n + i], false);
    }
}

template <typename T>
__global__ void unpack_multi_kernel(const IoDesc *__restrict__ table, int buf) {
    const IoDesc &d = table[blockIdx.y];
    const Geom g = d.g;
    const T *sS = (const T *)d.fld[buf][0], *sL = (const T *)d.fld[buf][1], *sC = (const T *)d.fld[buf][2];
    double *dst = d.staging;
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx);
        const int y = (int)((i / g.nx) % g.ny);
        const int z = (int)(i / ((int64_t)g.nx * g.ny));
        const int64_t j = g.at(x, y, z);
        dst[i] = (double)sS[j];
        dst[n + i] = (double)sL[j];
        dst[2 * n + i] = (double)sC[j];
    }
}

template <typename T>
cudaError_t launch_pack_multi(const IoDesc *table, int n, int64_t max_cells, cudaStream_t s) {
    pack_multi_kernel<T><<<dim3((unsigned)grid_for(max_cells, 256), (unsigned)n), 256, 0, s>>>(table);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_unpack_multi(const IoDesc *table, int n, int64_t max_cells, int buf, cudaStream_t s) {
    unpack_multi_kernel<T><<<dim3((unsigned)grid_for(max_cells, 256), (unsigned)n), 256, 0, s>>>(table, buf);
    return cudaGetLastError();
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

// A float sum carried with its rounding error (Knuth's TwoSum): about 48
// bits, enough for per-thread partial sums of FP32 cell terms; FP32 adds are
// far cheaper than FP64 ones on this GPU.
struct FSum {
    float hi, lo;
};
__device__ __forceinline__ void fsum_add(FSum &a, float x) {
    const float s = a.hi + x;
    const float bp = s - a.hi;
    const float err = (a.hi - (s - bp)) + (x - bp);
    a.hi = s;
    a.lo += err;
}

template <typename T>
__global__ void __launch_bounds__(256) observe_kernel(Geom g, CoefD kd, Fields<const T> f, double *partials) {
    const T AS = (T)kd.AS, AL = (T)kd.AL, dA = (T)kd.dA, cS0 = (T)kd.cS0, cL0 = (T)kd.cL0;
    const T CS = (T)kd.CS, CL = (T)kd.CL, tmp2 = (T)kd.tmp2, m = (T)kd.m, gam = (T)kd.gamma;
    const T kg = (T)kd.kappa_h2_half;
    constexpr bool F32 = std::is_same<T, float>::value;
    double acc[5] = {0, 0, 0, 0, 0};
    // FP32 state: the solid fraction and the free energy are summed per
    // thread as compensated float sums (the solute mass stays an FP64 sum of
    // the stored values, exact to rounding); FP64 state: FP64 throughout
    FSum hsum = {0.f, 0.f}, fsum = {0.f, 0.f};
    int nsolid = 0, nbad = 0;
    // one block per x row (grid-stride over rows): no per-cell index division
    const int nrows = g.ny * g.nz;
    for (int rr = blockIdx.x; rr < nrows; rr += gridDim.x) {
        const int64_t j0 = g.at(0, rr % g.ny, rr / g.ny);
        for (int x = threadIdx.x; x < g.nx; x += blockDim.x) {
            const int64_t j = j0 + x;
            const T eS = f.eS[j], eL = f.eL[j], c = f.c[j];
            if (!isfinite(eS) || !isfinite(eL) || !isfinite(c)) {
                ++nbad;
                continue;
            }
            // +x/+y/+z neighbours read through the ghost layer (periodic wrap or no-flux copy)
            const T sx = f.eS[j + 1], sy = f.eS[j + g.P], sz = f.eS[j + g.PS];
            const T lx = f.eL[j + 1], ly = f.eL[j + g.P], lz = f.eL[j + g.PS];
            const T s2 = eS * eS + eL * eL;
            const T h = eS * eS / s2;
            const T f0 = eS * eS * eS * eS / T(4) - eS * eS / T(2) + eL * eL * eL * eL / T(4) - eL * eL / T(2) +
                         gam * eS * eS * eL * eL + T(0.25);
            const T gr = (sx - eS) * (sx - eS) + (lx - eL) * (lx - eL) + (sy - eS) * (sy - eS) +
                         (ly - eL) * (ly - eL) + (sz - eS) * (sz - eS) + (lz - eL) * (lz - eL);
            const T rA = T(1) / (AS + dA * h);
            const T cSp = rA * (AL * c + (T(1) - h) * tmp2);
            const T cLp = rA * (AS * c - h * tmp2);
            const T fS = T(0.5) * AS * (cSp - cS0) * (cSp - cS0) + CS;
            const T fL = T(0.5) * AL * (cLp - cL0) * (cLp - cL0) + CL;
            acc[0] += (double)c;
            nsolid += eS > T(0.5) ? 1 : 0;
            if constexpr (F32) {
                fsum_add(hsum, h);
                // the terms differ by orders of magnitude (the parabola offsets
                // CS, CL against gradient and well terms): each added on its own
                fsum_add(fsum, m * f0);
                fsum_add(fsum, kg * gr);
                fsum_add(fsum, h * fS);
                fsum_add(fsum, (T(1) - h) * fL);
            } else {
                acc[1] += (double)h;
                acc[3] += ((double)(m * f0) + (double)(kg * gr)) + ((double)(h * fS) + (double)((T(1) - h) * fL));
            }
        }
    }
    if constexpr (F32) {
        acc[1] = (double)hsum.hi + (double)hsum.lo;
        acc[3] = (double)fsum.hi + (double)fsum.lo;
    }
    acc[2] = (double)nsolid;
    acc[4] = (double)nbad;
    acc[3] *= kd.vol;
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
template cudaError_t launch_pack<float>(const Geom &, const double *, Fields<float>, cudaStream_t);
template cudaError_t launch_pack<double>(const Geom &, const double *, Fields<double>, cudaStream_t);
template cudaError_t launch_unpack<float>(const Geom &, Fields<const float>, double *, cudaStream_t);
template cudaError_t launch_unpack<double>(const Geom &, Fields<const double>, double *, cudaStream_t);
template cudaError_t launch_pack_multi<float>(const IoDesc *, int, int64_t, cudaStream_t);
template cudaError_t launch_pack_multi<double>(const IoDesc *, int, int64_t, cudaStream_t);
template cudaError_t launch_unpack_multi<float>(const IoDesc *, int, int64_t, int, cudaStream_t);
template cudaError_t launch_unpack_multi<double>(const IoDesc *, int, int64_t, int, cudaStream_t);
template cudaError_t launch_observe<float>(const Geom &, const CoefD &, Fields<const float>, double *, int,
                                           cudaStream_t);
template cudaError_t launch_observe<double>(const Geom &, const CoefD &, Fields<const double>, double *, int,
                                            cudaStream_t);

}  // namespace ppf
