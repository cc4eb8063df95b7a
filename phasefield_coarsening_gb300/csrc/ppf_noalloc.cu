// ppf_noalloc.cu -- ppf_observe_noalloc: the observables reduction of
// ppf_reduce for callers that must not allocate device memory.
//
// Who needs it: code that runs inside someone else's memory discipline --
// an analysis hook called by a host application between its own time
// steps, whose device memory is owned by the application's pool or arena
// (a caching allocator, a preallocated MPI/NCCL buffer set), where a
// cudaMalloc the owner did not plan for can fail on a full device, fragment
// the application's memory pool, or stall the application's streams while the CUDA driver maps new
// memory.  Such a caller holds the fields in its own device buffers and only
// wants five numbers back.
//
// How: the per-CTA partial sums live in the file-scope array below instead
// of a context's allocation.  Host code cannot use the array's name as a
// device address (it names a host-side stand-in); its device address is
// looked up with cudaGetSymbolAddress once per device, the first time the
// entry point runs with that device current.  That first call therefore
// does set-up work and should come before any stream capture.  The address
// is kept together with the identity of the CUDA context it belongs to: if
// the caller resets the device (cudaDeviceReset), the next call finds a new
// context and looks the address up again instead of using a stale one.
//
// The array is shared by every call in the process and keeps the last
// call's contents.  Each call writes every partial slot it later reads, so
// nothing in it has to start at zero.  Calls whose work overlaps on the GPU
// (different streams, or different host threads) race on the array:
// serialize them, e.g. by issuing them on one stream.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "ppf.h"
#include "ppf_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 32;
constexpr int kCellsPerBlock = kThreads * kCellsPerThread;       // 8192
constexpr int kMaxBlocks = PPF_NOALLOC_MAX_CELLS / kCellsPerBlock; // 16384
constexpr int kVals = 5;
static_assert(PPF_NOALLOC_MAX_CELLS % kCellsPerBlock == 0, "scratch sizing");

// 16384 blocks x 5 doubles = 640 KiB, held by every GPU that loads the library
static __device__ __align__(256) double g_partials[kMaxBlocks * kVals];

// errors are reported through ppf_last_error(), like every other entry point
int fail(int code, const char *fmt, ...) {
    char msg[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    return ppf::set_last_error(code, msg);
}

struct Consts {
    double AS, dA, AL, cS0, cL0, CS, CL, tmp2, m, gamma, kg, vol;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Same observables and arithmetic as ppf_reduce: mass, solid fraction,
// solid cells, free energy (the functional whose variational derivative is
// the bracket of phasefield.c:360-373), non-finite cells.  Fields are
// compact [z][y][x]; the +x/+y/+z neighbour of a last cell wraps
// (periodic) or is the cell itself (no-flux), as the ghost layer would give.
__global__ void __launch_bounds__(kThreads) observe_compact(const double *__restrict__ eSf,
                                                             const double *__restrict__ eLf,
                                                             const double *__restrict__ cf, int nz, int ny, int nx,
                                                             int bc, Consts k, double *__restrict__ partials) {
    const long long n = (long long)nz * ny * nx;
    double acc[kVals] = {0, 0, 0, 0, 0};
    const long long base = (long long)blockIdx.x * kCellsPerBlock;
    for (int r = 0; r < kCellsPerThread; ++r) {
        const long long i = base + (long long)r * kThreads + threadIdx.x;
        if (i >= n) break;
        const int x = (int)(i % nx);
        const int y = (int)((i / nx) % ny);
        const int z = (int)(i / ((long long)nx * ny));
        const double eS = eSf[i], eL = eLf[i], c = cf[i];
        if (!isfinite(eS) || !isfinite(eL) || !isfinite(c)) {
            acc[4] += 1.0;
            continue;
        }
        const int xp = x + 1 < nx ? x + 1 : (bc == PPF_BC_PERIODIC ? 0 : x);
        const int yp = y + 1 < ny ? y + 1 : (bc == PPF_BC_PERIODIC ? 0 : y);
        const int zp = z + 1 < nz ? z + 1 : (bc == PPF_BC_PERIODIC ? 0 : z);
        const long long jx = ((long long)z * ny + y) * nx + xp;
        const long long jy = ((long long)z * ny + yp) * nx + x;
        const long long jz = ((long long)zp * ny + y) * nx + x;
        const double sx = eSf[jx], sy = eSf[jy], sz = eSf[jz];
        const double lx = eLf[jx], ly = eLf[jy], lz = eLf[jz];
        const double s2 = eS * eS + eL * eL;
        const double h = eS * eS / s2;
        const double f0 = eS * eS * eS * eS / 4.0 - eS * eS / 2.0 + eL * eL * eL * eL / 4.0 - eL * eL / 2.0 +
                          k.gamma * eS * eS * eL * eL + 0.25;
        const double gr = (sx - eS) * (sx - eS) + (lx - eL) * (lx - eL) + (sy - eS) * (sy - eS) +
                          (ly - eL) * (ly - eL) + (sz - eS) * (sz - eS) + (lz - eL) * (lz - eL);
        const double rA = 1.0 / (k.AS + k.dA * h);
        const double cSp = rA * (k.AL * c + (1.0 - h) * k.tmp2);
        const double cLp = rA * (k.AS * c - h * k.tmp2);
        const double fS = 0.5 * k.AS * (cSp - k.cS0) * (cSp - k.cS0) + k.CS;
        const double fL = 0.5 * k.AL * (cLp - k.cL0) * (cLp - k.cL0) + k.CL;
        acc[0] += c;
        acc[1] += h;
        acc[2] += eS > 0.5 ? 1.0 : 0.0;
        acc[3] += k.vol * ((k.m * f0) + (k.kg * gr) + (h * fS) + ((1.0 - h) * fL));
    }
    __shared__ double red[kThreads / 32][kVals];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v < kVals; ++v) {
        const double s = warp_sum(acc[v]);
        if (lane == 0) red[w][v] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int v = 0; v < kVals; ++v) {
            double s = 0;
            for (int q = 0; q < kThreads / 32; ++q) s += red[q][v];
            partials[(long long)blockIdx.x * kVals + v] = s;
        }
    }
}

// Fixed-order sum of the first `nblocks` partial slots into out[0..4].
__global__ void __launch_bounds__(kThreads) sum_partials(const double *__restrict__ partials, int nblocks,
                                                          double *__restrict__ out) {
    __shared__ double red[kThreads];
    for (int v = 0; v < kVals; ++v) {
        double s = 0;
        for (int b = threadIdx.x; b < nblocks; b += kThreads) s += partials[(long long)b * kVals + v];
        red[threadIdx.x] = s;
        __syncthreads();
        for (int h = kThreads / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[v] = red[0];
        __syncthreads();
    }
}

// device address of g_partials, looked up once per device and context
constexpr int kMaxDevices = 64;
struct ScratchAddr {
    double *addr;
    unsigned long long ctx_id;   // the CUDA context the address belongs to (unique per process)
};
ScratchAddr g_addr[kMaxDevices];
std::mutex g_lock;

// the unique id of the calling thread's current CUDA context (0: none yet)
unsigned long long current_context_id() {
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (PFN_cuCtxGetCurrent_v4000)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (PFN_cuCtxGetId_v12000)p;
        looked_up = true;
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

int scratch_for_current_device(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(PPF_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(PPF_ECUDA, "device %d out of range", dev);
    std::lock_guard<std::mutex> hold(g_lock);
    ScratchAddr &a = g_addr[dev];
    const unsigned long long id = current_context_id();
    if (!a.addr || id == 0 || id != a.ctx_id) {
        // first use on this device, or its context was recreated (cudaDeviceReset):
        // the symbol's address belongs to the context's copy of this module
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_partials);
        if (e != cudaSuccess || !p)
            return fail(PPF_ECUDA, "cudaGetSymbolAddress of the reduction scratch: %s", cudaGetErrorString(e));
        a.addr = static_cast<double *>(p);
        a.ctx_id = current_context_id();    // the lookup made the primary context current
    }
    *out = a.addr;
    return PPF_OK;
}

}  // namespace

extern "C" int ppf_observe_noalloc(int nz, int ny, int nx, const ppf_params *p, int bc, const double *etaS,
                                   const double *etaL, const double *c, double *out, void *stream) {
    if (!p || !etaS || !etaL || !c || !out) return fail(PPF_EINVAL, "ppf_observe_noalloc: null argument");
    if (nz < 1 || ny < 1 || nx < 1) return fail(PPF_EINVAL, "ppf_observe_noalloc: grid %dx%dx%d", nz, ny, nx);
    if (bc != PPF_BC_PERIODIC && bc != PPF_BC_NOFLUX) return fail(PPF_EINVAL, "ppf_observe_noalloc: bad bc %d", bc);
    const long long cells = (long long)nz * ny * nx;
    if (cells > (long long)PPF_NOALLOC_MAX_CELLS)
        return fail(PPF_EINVAL,
                    "ppf_observe_noalloc: %lld cells exceed the allocation-free limit of %d cells "
                    "(its fixed scratch holds %d partial sums); use ppf_reduce on a context instead",
                    cells, PPF_NOALLOC_MAX_CELLS, kMaxBlocks);
    ppf_derived d;
    if (ppf_params_derive(p, &d) != PPF_OK) return fail(PPF_EINVAL, "ppf_observe_noalloc: invalid parameters");
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    Consts k;
    k.AS = p->AS;
    k.AL = p->AL;
    k.dA = p->AL - p->AS;
    k.cS0 = p->cS0;
    k.cL0 = p->cL0;
    k.CS = p->CS;
    k.CL = p->CL;
    k.tmp2 = p->AS * p->cS0 - p->AL * p->cL0;
    k.m = d.m;
    k.gamma = p->gamma;
    k.kg = 0.5 * d.kappa * d.h2;
    k.vol = p->dx * p->dx * p->dx;
    const int nblocks = (int)((cells + kCellsPerBlock - 1) / kCellsPerBlock);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    observe_compact<<<nblocks, kThreads, 0, s>>>(etaS, etaL, c, nz, ny, nx, bc, k, scratch);
    sum_partials<<<1, kThreads, 0, s>>>(scratch, nblocks, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(PPF_ECUDA, "ppf_observe_noalloc launch: %s", cudaGetErrorString(e));
    return PPF_OK;
}
