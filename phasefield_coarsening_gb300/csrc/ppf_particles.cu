// ppf_particles.cu -- particle analysis of a state on the GPU: connected
// components of the solid (etaS > threshold, 6-connected, wrapping across
// periodic faces), their volumes, equivalent-sphere radii, the mean radius
// R-bar, and the solid/liquid interface area.  The reference does this
// analysis outside the program (README.md:26: MATLAB post-processing); here
// it runs on the device state between steps.
//
// Labelling is a lock-free union-find over a label per cell: a solid cell
// starts as its own root; for every solid forward neighbour the two roots
// are joined by hooking the larger root onto the smaller with a
// compare-and-swap.  Parent labels therefore strictly decrease along every
// path, so each find terminates; retry loops are additionally capped and
// report PPF_ETIMEOUT if the cap is ever reached.
#include <cuda_runtime.h>

#include <cstdint>

#include "ppf_internal.h"
#include "ppf_particles.h"

namespace ppf {

namespace {

constexpr int kNT = 256;
constexpr int kMaxRetry = 1 << 20;

// Label reads and the halving writes bypass L1 (other SMs change labels
// through L2 while the merge runs).
__device__ __forceinline__ int find_root(int *lab, int i) {
    // path halving: each visited cell points two levels up (still an ancestor)
    for (int it = 0; it < kMaxRetry; ++it) {
        const int p = __ldcg(lab + i);
        if (p == i) return i;
        const int gp = __ldcg(lab + p);
        if (gp != p) __stcg(lab + i, gp);
        i = gp;
    }
    return -1;
}

__device__ __forceinline__ bool unite(int *lab, int a, int b) {
    for (int it = 0; it < kMaxRetry; ++it) {
        a = find_root(lab, a);
        b = find_root(lab, b);
        if (a < 0 || b < 0) return false;
        if (a == b) return true;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicCAS(lab + a, a, b);   // hook root a under b < a
        if (old == a) return true;
        a = old;                                     // a was hooked meanwhile: retry from there
    }
    return false;
}

template <typename T>
__device__ __forceinline__ bool solid_at(const Geom &g, const T *eS, int x, int y, int z, T thr) {
    return eS[g.at(x, y, z)] > thr;
}

template <typename T>
__global__ void __launch_bounds__(kNT) init_labels(Geom g, const T *__restrict__ eS, T thr, int *__restrict__ lab,
                                                   int *__restrict__ vol) {
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx), y = (int)((i / g.nx) % g.ny), z = (int)(i / ((int64_t)g.nx * g.ny));
        lab[i] = solid_at(g, eS, x, y, z, thr) ? (int)i : -1;
        vol[i] = 0;
    }
}

// joins every solid cell with its solid +x, +y, +z neighbours (wrapping for
// periodic boundaries); also counts solid/liquid faces (interface area)
template <typename T>
__global__ void __launch_bounds__(kNT) merge_labels(Geom g, const T *__restrict__ eS, T thr, int *lab,
                                                    double *__restrict__ partials, int *__restrict__ err) {
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    double faces = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx), y = (int)((i / g.nx) % g.ny), z = (int)(i / ((int64_t)g.nx * g.ny));
        const bool s = solid_at(g, eS, x, y, z, thr);
        const int nb[3][3] = {{x + 1, y, z}, {x, y + 1, z}, {x, y, z + 1}};
        const int lim[3] = {g.nx, g.ny, g.nz};
        for (int d = 0; d < 3; ++d) {
            int c[3] = {nb[d][0], nb[d][1], nb[d][2]};
            if (c[d] == lim[d]) {
                if (g.bc != 0) continue;              // no-flux: no neighbour across the face
                c[d] = 0;
            }
            const bool t = solid_at(g, eS, c[0], c[1], c[2], thr);
            if (s != t) faces += 1.0;
            if (s && t) {
                const int j = (c[2] * g.ny + c[1]) * g.nx + c[0];
                if (!unite(lab, (int)i, j)) atomicOr(err, 2);
            }
        }
    }
    // block sum of the face count
    __shared__ double red[kNT / 32];
    for (int o = 16; o > 0; o >>= 1) faces += __shfl_xor_sync(0xffffffffu, faces, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = faces;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < kNT / 32; ++w) s += red[w];
        partials[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kNT) count_volumes(int64_t n, int *lab, int *__restrict__ vol,
                                                     int *__restrict__ err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (lab[i] < 0) continue;
        const int r = find_root(lab, (int)i);
        if (r < 0) {
            atomicOr(err, 2);
            continue;
        }
        lab[i] = r;
        atomicAdd(vol + r, 1);
    }
}

// per root: count, sum of equivalent radii, sum of volumes, largest volume;
// optionally the list of volumes
__global__ void __launch_bounds__(kNT) root_stats(int64_t n, const int *__restrict__ lab, const int *__restrict__ vol,
                                                  double dx3, double *__restrict__ partials,
                                                  int64_t *__restrict__ list, int64_t cap,
                                                  unsigned long long *__restrict__ nlist) {
    double cnt = 0, rsum = 0, vsum = 0, vmax = 0;
    const double k = 3.0 / (4.0 * 3.14159265358979323846);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (lab[i] != (int)i) continue;
        const double v = (double)vol[i];
        cnt += 1.0;
        rsum += cbrt(k * v * dx3);
        vsum += v;
        vmax = v > vmax ? v : vmax;
        if (list) {
            const unsigned long long slot = atomicAdd(nlist, 1ull);
            if ((int64_t)slot < cap) list[slot] = (int64_t)v;
        }
    }
    __shared__ double red[kNT / 32][4];
    double v4[4] = {cnt, rsum, vsum, vmax};
    for (int q = 0; q < 4; ++q) {
        double a = v4[q];
        for (int o = 16; o > 0; o >>= 1) {
            const double b = __shfl_xor_sync(0xffffffffu, a, o);
            a = q == 3 ? (b > a ? b : a) : a + b;
        }
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][q] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[4] = {0, 0, 0, 0};
        for (int w = 0; w < kNT / 32; ++w) {
            s[0] += red[w][0];
            s[1] += red[w][1];
            s[2] += red[w][2];
            s[3] = red[w][3] > s[3] ? red[w][3] : s[3];
        }
        for (int q = 0; q < 4; ++q) partials[(int64_t)blockIdx.x * 4 + q] = s[q];
    }
}

__global__ void __launch_bounds__(kNT) finish_stats(const double *__restrict__ faces, const double *__restrict__ rs,
                                                    int nb, double *__restrict__ out) {
    __shared__ double red[kNT];
    // out: count, rsum, vsum, vmax, faces
    for (int q = 0; q < 5; ++q) {
        double a = q == 3 ? 0.0 : 0.0;
        for (int b = threadIdx.x; b < nb; b += kNT) {
            const double v = q < 4 ? rs[(int64_t)b * 4 + q] : faces[b];
            a = q == 3 ? (v > a ? v : a) : a + v;
        }
        red[threadIdx.x] = a;
        __syncthreads();
        for (int h = kNT / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) {
                const double o = red[threadIdx.x + h];
                red[threadIdx.x] = q == 3 ? (o > red[threadIdx.x] ? o : red[threadIdx.x]) : red[threadIdx.x] + o;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) out[q] = red[0];
        __syncthreads();
    }
}

}  // namespace

template <typename T>
cudaError_t launch_particles(const Geom &g, const T *etaS, double threshold, int *lab, int *vol, double *partials,
                             int nblocks, double dx, double *out, int64_t *list, int64_t cap,
                             unsigned long long *nlist, int *err, cudaStream_t s) {
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const T thr = (T)threshold;
    init_labels<T><<<nblocks, kNT, 0, s>>>(g, etaS, thr, lab, vol);
    merge_labels<T><<<nblocks, kNT, 0, s>>>(g, etaS, thr, lab, partials, err);
    count_volumes<<<nblocks, kNT, 0, s>>>(n, lab, vol, err);
    if (list) cudaMemsetAsync(nlist, 0, sizeof(unsigned long long), s);
    root_stats<<<nblocks, kNT, 0, s>>>(n, lab, vol, dx * dx * dx, partials + nblocks, list, cap, nlist);
    finish_stats<<<1, kNT, 0, s>>>(partials, partials + nblocks, nblocks, out);
    return cudaGetLastError();
}

template cudaError_t launch_particles<float>(const Geom &, const float *, double, int *, int *, double *, int, double,
                                             double *, int64_t *, int64_t, unsigned long long *, int *, cudaStream_t);
template cudaError_t launch_particles<double>(const Geom &, const double *, double, int *, int *, double *, int,
                                              double, double *, int64_t *, int64_t, unsigned long long *, int *,
                                              cudaStream_t);

}  // namespace ppf
