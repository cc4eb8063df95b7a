// ppf_nn_conv.cu -- 3x3x3 convolutions of the surrogate network as
// implicit GEMMs on the fifth-generation tensor cores (tcgen05, BF16 in,
// FP32 accumulation in TMEM).
//
// conv_kernel<CI, CO, EPI>: out[v] = sum over the 27 taps of W_tap * in[v + tap].
//   One tile = 128 consecutive voxels of one x row (M = 128), N = CO,
//   K = 27 taps x CI.  A work item is a column of tiles marching in y
//   (rows y0..y1-1 of one z plane and x segment).  Each row of the march
//   needs the three input rows (y-1, y, y+1) at z-1, z, z+1; an input
//   "segment" is 130 voxels (the tile plus one each side) of one input row,
//   moved into shared memory by 1-D bulk copies, one per 8-channel plane.
//   A ring of RING row slots (3 segments each) holds rows y-1..y+1 while
//   the next rows load, so every input row is fetched once per work item.
//   The A operand of tap (dz, dy, dx) is its segment started dx+1 voxels
//   (16 bytes each) in; the B operand is that tap's CI x CO block of the
//   weight image, loaded once per CTA.
//   Warp roles (352 threads): warp 0 lane 0 issues the bulk copies, lane 0
//   of warps 1 and 10 issue the MMAs of alternate rows (warp 1 owns the
//   TMEM allocation), warps
//   2-9 run the epilogue on a double-buffered TMEM accumulator (warp w
//   reads TMEM lanes 32 (w % 4).., warps 2-5 the first half of the output
//   channels, warps 6-9 the second), so the epilogue of one tile overlaps
//   the MMAs of the next.  Operand descriptors are built once and advanced
//   by constant offsets.
//
// wgrad_kernel<CX, CZ>: dW[tap][co][ci] = sum over voxels v of
//   dZ[v][co] * X[v + tap][ci].  The reduction runs over voxels (K), both
//   operands are channel-contiguous (MN-major).  Per tile the nine (dz, dy)
//   segments sit in fixed slots laid out back to back, so one M = 128 block
//   covers 128/CX slots x CX channels at a uniform group stride; the three
//   dx shifts are three start offsets.  Per CTA the partial dW stays in
//   TMEM over all its tiles and is written once at the end.
//
// Every mbarrier wait is bounded by a time limit; on expiry the CTA sets
// the error word, stops issuing work, drains its own copies and MMAs
// (bounded) and exits.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "ppf_nn.h"
#include "ppf_ptx.h"

namespace ppf {
namespace nn {

using namespace ppf::ptx;

namespace {

// bounded wait that also gives up when another role flagged an abort
__device__ __forceinline__ bool wait_or_abort(uint32_t bar, uint32_t parity, unsigned long long limit_ns,
                                              volatile int *abort_flag) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    for (uint32_t it = 0;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 31u) == 31u) {
            if (*abort_flag) return false;
            if (globaltimer() - t0 > limit_ns) return false;
        }
    }
}

// the same with a short sleep between polls: for the many epilogue warps,
// whose spinning would otherwise take issue slots from the MMA thread
__device__ __forceinline__ bool wait_backoff(uint32_t bar, uint32_t parity, unsigned long long limit_ns,
                                             volatile int *abort_flag) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    for (uint32_t it = 0;; ++it) {
        __nanosleep(64);
        if (mbar_try(bar, parity)) return true;
        if ((it & 7u) == 7u) {
            if (*abort_flag) return false;
            if (globaltimer() - t0 > limit_ns) return false;
        }
    }
}

__device__ __forceinline__ void fail(volatile int *abort_flag, int *err, int code) {
    *abort_flag = 1;
    atomicOr(err, code);
}

// the halo image of interior coordinate x, or kNone (periodic: x=0 -> n,
// x=n-1 -> -1; no-flux: x=0 -> -1, x=n-1 -> n); needs n >= 2
constexpr int kNone = -0x40000000;
__device__ __forceinline__ int image_of(int x, int n, int bc) {
    return x == 0 ? (bc == 0 ? n : -1) : x == n - 1 ? (bc == 0 ? -1 : n) : kNone;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ uint4 pack8(const float *f) {
    return make_uint4(pack_bf16x2(f[0], f[1]), pack_bf16x2(f[2], f[3]), pack_bf16x2(f[4], f[5]),
                      pack_bf16x2(f[6], f[7]));
}

__device__ __forceinline__ void unpack8(uint4 q, float *f) {
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        f[2 * i] = __uint_as_float(w[i] << 16);
        f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
    }
}

// logistic function: sigma(z) = (1 + tanh(z/2)) / 2 with the hardware
// tanh (tanh.approx.f32, relative error about 2^-11, well below the BF16
// rounding of every value it feeds)
__device__ __forceinline__ float sigmoidf(float z) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
    return fmaf(0.5f, t, 0.5f);
}

template <int NP>
__device__ __forceinline__ void store_planes(uint16_t *base, int64_t Pst, int64_t p, const uint4 (&v)[NP]) {
#pragma unroll
    for (int j = 0; j < NP; ++j)
        *reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(base) + ((int64_t)j * Pst + p) * 16) = v[j];
}

// store at (x, y, z) and at every halo image of it
template <int NP>
__device__ __forceinline__ void store_with_images(const NNGeom &g, uint16_t *base, int x, int y, int z,
                                                  const uint4 (&v)[NP]) {
    store_planes<NP>(base, g.Pst, g.p(x, y, z), v);
    const int ax = image_of(x, g.nx, g.bc), ay = image_of(y, g.ny, g.bc), az = image_of(z, g.nz, g.bc);
    if (ax == kNone && ay == kNone && az == kNone) return;
    for (int k = 1; k < 8; ++k) {
        const int xx = (k & 1) ? ax : x, yy = (k & 2) ? ay : y, zz = (k & 4) ? az : z;
        if (xx == kNone || yy == kNone || zz == kNone) continue;
        store_planes<NP>(base, g.Pst, g.p(xx, yy, zz), v);
    }
}

constexpr int kConvThreads = 352;   // producer warp, MMA warp, 8 epilogue warps, second MMA warp
constexpr int kMmaWarp2 = 10;
constexpr int kEpiThreads = 256;

template <int CI, int CO>
struct ConvCfg {
    static constexpr int RING = CI == 32 ? 6 : 5;        // input-row slots in shared memory
    static constexpr int ND = 5;                         // TMEM tiles (one per input row)
    static constexpr int NCOL = 3 * CO;                  // one tile: contributions to rows y+1, y, y-1
    static constexpr int SEGB = (CI / 8) * kSegPlane;    // one segment, all channel planes
    static constexpr int ROWB = 3 * SEGB;                // one slot: segments at z-1, z, z+1
    static constexpr int WB = 27 * CI * CO * 2;          // weight image
    static constexpr int HALF = CO / 2;                  // output channels per epilogue warp
    static constexpr int OFF_W = RING * ROWB;
    static constexpr int OFF_BAR = OFF_W + WB;
    static constexpr int NBAR = 2 * RING + 2 * ND + 3;   // full, empty, dfull, dempty, wbar, drain x2
    static constexpr int OFF_SLOT = OFF_BAR + NBAR * 8;  // TMEM base, abort flag
    static constexpr int OFF_RED = OFF_SLOT + 16;        // [8][HALF + 1] floats
    static constexpr int OFF_BIAS = OFF_RED + 8 * (HALF + 1) * 4;   // CO floats
    static constexpr int OFF_REDD = (OFF_BIAS + CO * 4 + 7) / 8 * 8;  // [4] doubles
    static constexpr int SMEM = OFF_REDD + 4 * 8;
    static constexpr int TMEM_COLS = ND * NCOL <= 256 ? 256 : 512;
    static_assert(CI % 16 == 0 && CO % 16 == 0 && CO <= 32, "channel counts");
    static_assert(ND * NCOL <= 512 && NCOL <= 256, "TMEM / MMA N");
    static_assert(OFF_W % 16 == 0 && OFF_BAR % 8 == 0, "alignment");
};

struct Item {
    int z, x0, y0, y1;
};

__device__ __forceinline__ Item item_of(const NNGeom &g, int yc, int it) {
    const int nxt = g.nx / kTileX;
    const int nyc = (g.ny + yc - 1) / yc;
    Item r;
    const int xt = it % nxt;
    const int rest = it / nxt;
    const int yi = rest % nyc;
    r.z = rest / nyc;
    r.x0 = xt * kTileX;
    r.y0 = yi * yc;
    r.y1 = min(g.ny, r.y0 + yc);
    return r;
}

// Work order inside a CTA: items in turn, and in an item the input rows
// y0-1 .. y1 in order; input row number q (counted over the CTA's items)
// owns shared-memory slot q % RING and TMEM tile q % ND.  The MMAs of row q
// compute, for the 128 voxels of the tile and all three dy at once
// (N = 3 CO), D_q[v][(dy, co)] = sum over (dz, dx, ci) of
// W[dz][dy][dx][co][ci] in[z+dz][row q][x+dx][ci]; output row y is
// D_{y-1}[dy=-1] + D_y[dy=0] + D_{y+1}[dy=+1], summed by the epilogue.
template <int CI, int CO, int EPI>
__global__ void __launch_bounds__(kConvThreads, 1) conv_kernel(const ConvArgs a) {
    using C = ConvCfg<CI, CO>;
    constexpr int HALF = C::HALF;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sb = smem_u32(smem);
    const uint32_t ring = sb, wsm = sb + C::OFF_W, bars = sb + C::OFF_BAR;
    const uint32_t wbar = bars + 8 * (2 * C::RING + 2 * C::ND), dbar = wbar + 8;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + C::OFF_SLOT);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + C::OFF_SLOT + 4);
    float *red = reinterpret_cast<float *>(smem + C::OFF_RED);
    float *sbias = reinterpret_cast<float *>(smem + C::OFF_BIAS);
    auto full = [&](uint32_t s) { return bars + 8 * s; };
    auto empty = [&](uint32_t s) { return bars + 8 * (C::RING + s); };
    auto dfull = [&](uint32_t s) { return bars + 8 * (2 * C::RING + s); };
    auto dempty = [&](uint32_t s) { return bars + 8 * (2 * C::RING + C::ND + s); };
    const NNGeom &g = a.g;

    if (tid < CO) sbias[tid] = a.bias[tid];
    if (tid == 0) {
        for (int s = 0; s < C::RING; ++s) {
            mbar_init(full(s), 1);
            mbar_init(empty(s), 1);
        }
        for (int s = 0; s < C::ND; ++s) {
            mbar_init(dfull(s), 1);
            mbar_init(dempty(s), kEpiThreads);
        }
        mbar_init(wbar, 1);
        mbar_init(dbar, 1);
        mbar_init(dbar + 8, 1);
        *abort_flag = 0;
        mbar_init_fence();
    }
    if (warp == 1) tmem_alloc(smem_u32(tslot), C::TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *reinterpret_cast<volatile uint32_t *>(tslot);

    if (warp == 0) {
        // ---------------- producer: bulk copies of input rows ----------------
        if (lane == 0) {
            uint32_t issued_q[C::RING];
#pragma unroll
            for (int s = 0; s < C::RING; ++s) issued_q[s] = 0xFFFFFFFFu;
            mbar_expect_tx(wbar, C::WB);
            bulk_load(wsm, a.wimg, C::WB, wbar);
            uint32_t q = 0;
            bool ok = true;
            for (int it = blockIdx.x; ok && it < a.items; it += gridDim.x) {
                const Item w = item_of(g, a.yc, it);
                for (int r = w.y0 - 1; r <= w.y1; ++r, ++q) {
                    const uint32_t s = q % C::RING;
                    // the producer runs ahead of the MMAs: its waits for a free slot
                    // sleep between polls instead of taking issue slots
                    if (q >= (uint32_t)C::RING &&
                        !wait_backoff(empty(s), ((q / C::RING) + 1) & 1, a.limit_ns, abort_flag)) {
                        fail(abort_flag, a.err, 1);
                        ok = false;
                        break;
                    }
                    // test hook: the second row's barrier expects 16 bytes that never come
                    mbar_expect_tx(full(s), C::ROWB + ((a.inject_stall && q == 1) ? 16u : 0u));
#pragma unroll
                    for (int k = 0; k < C::RING; ++k)
                        if (k == (int)s) issued_q[k] = q;
#pragma unroll
                    for (int dz = 0; dz < 3; ++dz) {
                        const int64_t pv = g.p(w.x0 - 1, r, w.z + dz - 1);
#pragma unroll
                        for (int j = 0; j < CI / 8; ++j) {
                            const unsigned char *src =
                                reinterpret_cast<const unsigned char *>(a.x) + ((int64_t)j * g.Pst + pv) * 16;
                            bulk_load(ring + s * C::ROWB + dz * C::SEGB + j * kSegPlane, src, kSegPlane, full(s));
                        }
                    }
                }
            }
            // drain: every issued copy has landed before the CTA may exit
#pragma unroll
            for (int s = 0; s < C::RING; ++s)
                if (issued_q[s] != 0xFFFFFFFFu && !mbar_wait(full(s), (issued_q[s] / C::RING) & 1, a.limit_ns))
                    atomicOr(a.err, 4);
            if (!mbar_wait(wbar, 0, a.limit_ns)) atomicOr(a.err, 4);
        }
    } else if (warp == 1 || warp == kMmaWarp2) {
        // ---------------- MMA issuers: one D tile per input row; warp 1
        // takes the even rows, warp 10 the odd ones, so that one thread's
        // waits and bookkeeping overlap the other's MMAs ----------------
        if (lane == 0) {
            const uint32_t mine = warp == 1 ? 0u : 1u;
            const uint32_t mydbar = warp == 1 ? dbar : dbar + 8;
            const uint32_t idesc = idesc_bf16(128, C::NCOL, false, false);
            // descriptors of slot 0 and of the weight image; every operand
            // below is one of these plus a byte offset / 16 (no carry: all
            // shared addresses stay below 2^18).  Weight image rows for
            // (dz, dx, 8-channel group j) are (dy, co): N = 3 CO rows.
            const uint64_t a0 = smem_desc(ring, kSegPlane, 128);
            const uint64_t b0 = smem_desc(wsm, C::NCOL * 16, 128);
            bool ok = wait_or_abort(wbar, 0, a.limit_ns, abort_flag);
            if (!ok) fail(abort_flag, a.err, 1);
            uint32_t q = 0;
            for (int it = blockIdx.x; ok && it < a.items; it += gridDim.x) {
                const Item w = item_of(g, a.yc, it);
                for (int r = w.y0 - 1; r <= w.y1; ++r, ++q) {
                    if ((q & 1u) != mine) continue;
                    const uint32_t s = q % C::RING, ds = q % C::ND;
                    if (!wait_or_abort(full(s), (q / C::RING) & 1, a.limit_ns, abort_flag) ||
                        (q >= (uint32_t)C::ND &&
                         !wait_or_abort(dempty(ds), ((q / C::ND) + 1) & 1, a.limit_ns, abort_flag))) {
                        fail(abort_flag, a.err, 1);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = tbase + ds * C::NCOL;
                    const uint64_t ab = a0 + ((s * C::ROWB) >> 4);
#pragma unroll
                    for (int dz = 0; dz < 3; ++dz)
#pragma unroll
                        for (int dx = 0; dx < 3; ++dx)
#pragma unroll
                            for (int kk = 0; kk < CI / 16; ++kk) {
                                const uint64_t ad = ab + ((dz * C::SEGB + dx * 16 + kk * 2 * kSegPlane) >> 4);
                                const uint64_t bd = b0 + ((((dz * 3 + dx) * (CI / 8) + 2 * kk) * C::NCOL * 16) >> 4);
                                mma_bf16(d, ad, bd, idesc, (dz | dx | kk) ? 1u : 0u);
                            }
                    mma_commit(empty(s));
                    mma_commit(dfull(ds));
                }
            }
            // drain: all issued MMAs complete before TMEM is released
            mma_commit(mydbar);
            if (!mbar_wait(mydbar, 0, a.limit_ns)) atomicOr(a.err, 4);
        }
    } else {
        // ---------------- epilogue: warps 2-9; TMEM lane quarter = warp % 4,
        // output channels [c0, c0 + HALF) by warp group ----------------
        const int ew = warp - 2;
        const int quarter = warp & 3;
        const int c0 = (ew >> 2) * HALF;
        const int row = quarter * 32 + lane;
        const uint32_t tl = tbase + ((uint32_t)(quarter * 32) << 16) + c0;
        constexpr bool STATE_OUT = EPI == EPI_STATE || EPI == EPI_LOSS;
        const bool active = !STATE_OUT || c0 == 0;
        float sums[HALF + 1];
#pragma unroll
        for (int c = 0; c <= HALF; ++c) sums[c] = 0.f;
        double mass = 0.0;
        uint32_t q = 0;
        bool ok = true;
        for (int it = blockIdx.x; ok && it < a.items; it += gridDim.x) {
            const Item w = item_of(g, a.yc, it);
            const uint32_t qb = q;                 // input row y0 - 1
            q += (uint32_t)(w.y1 - w.y0) + 2;
            for (int y = w.y0; y < w.y1; ++y) {
                const uint32_t qy = qb + (uint32_t)(y - w.y0) + 1;   // input row y
                const int x = w.x0 + row, z = w.z;
                const int64_t p = g.p(x, y, z);
                // loads that do not depend on the accumulators go first
                float zl[HALF];
                float s0v[3] = {0.f, 0.f, 0.f}, s1v[3] = {0.f, 0.f, 0.f};
                int64_t sa = 0;
                if (EPI == EPI_DGRAD) {
#pragma unroll
                    for (int j = 0; j < HALF / 8; ++j)
                        unpack8(*reinterpret_cast<const uint4 *>(reinterpret_cast<const unsigned char *>(a.zlow) +
                                                                  ((int64_t)(c0 / 8 + j) * g.Pst + p) * 16),
                                zl + 8 * j);
                }
                if (STATE_OUT && active) {
                    sa = a.sg.at(x, y, z);
                    s0v[0] = a.s0.eS[sa];
                    s0v[1] = a.s0.eL[sa];
                    s0v[2] = a.s0.c[sa];
                    if (EPI == EPI_LOSS) {
                        s1v[0] = a.s1.eS[sa];
                        s1v[1] = a.s1.eL[sa];
                        s1v[2] = a.s1.c[sa];
                    }
                }
                if (!wait_backoff(dfull((qy - 1) % C::ND), ((qy - 1) / C::ND) & 1, a.limit_ns, abort_flag) ||
                    !wait_backoff(dfull(qy % C::ND), (qy / C::ND) & 1, a.limit_ns, abort_flag) ||
                    !wait_backoff(dfull((qy + 1) % C::ND), ((qy + 1) / C::ND) & 1, a.limit_ns, abort_flag)) {
                    fail(abort_flag, a.err, 1);
                    ok = false;
                    break;
                }
                tc_fence_after();
                float v[HALF];
                {
                    // out[y] = sum_dy W_dy in[y + dy]: the dy = -1 block of
                    // D_{y-1}, the dy = 0 block of D_y, the dy = +1 block of D_{y+1}
                    const uint32_t t0 = tl + ((qy - 1) % C::ND) * C::NCOL;
                    const uint32_t t1 = tl + (qy % C::ND) * C::NCOL + CO;
                    const uint32_t t2 = tl + ((qy + 1) % C::ND) * C::NCOL + 2 * CO;
                    if constexpr (HALF == 16) {
                        float u0[16], u1[16], u2[16];
                        tmem_ld16(t0, u0);
                        tmem_ld16(t1, u1);
                        tmem_ld16(t2, u2);
#pragma unroll
                        for (int i = 0; i < 16; ++i) v[i] = (u0[i] + u1[i]) + u2[i];
                    } else {
                        float u0[8], u1[8], u2[8];
                        tmem_ld8(t0, u0);
                        tmem_ld8(t1, u1);
                        tmem_ld8(t2, u2);
#pragma unroll
                        for (int i = 0; i < 8; ++i) v[i] = (u0[i] + u1[i]) + u2[i];
                    }
                }
                tc_fence_before();
                mbar_arrive(dempty((qy - 1) % C::ND));
                if (y == w.y1 - 1) {
                    mbar_arrive(dempty(qy % C::ND));
                    mbar_arrive(dempty((qy + 1) % C::ND));
                }

                if (EPI == EPI_ACT || EPI == EPI_ACT_TRAIN) {
                    uint4 o[HALF / 8], zz[HALF / 8];
#pragma unroll
                    for (int j = 0; j < HALF / 8; ++j) {
                        float h[8], sv[8];
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            h[i] = v[8 * j + i] + sbias[c0 + 8 * j + i];
                            sv[i] = h[i] * sigmoidf(h[i]);
                        }
                        o[j] = pack8(sv);
                        zz[j] = pack8(h);
                    }
                    uint16_t *ob = reinterpret_cast<uint16_t *>(reinterpret_cast<unsigned char *>(a.out) +
                                                                (int64_t)(c0 / 8) * g.Pst * 16);
                    store_with_images<HALF / 8>(g, ob, x, y, z, o);
                    if (EPI == EPI_ACT_TRAIN) {
                        uint16_t *zb = reinterpret_cast<uint16_t *>(reinterpret_cast<unsigned char *>(a.zout) +
                                                                    (int64_t)(c0 / 8) * g.Pst * 16);
                        store_planes<HALF / 8>(zb, g.Pst, p, zz);
                    }
                } else if (EPI == EPI_DGRAD) {
                    uint4 o[HALF / 8];
#pragma unroll
                    for (int j = 0; j < HALF / 8; ++j) {
                        float dd[8];
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const float zi = zl[8 * j + i];
                            const float sg = sigmoidf(zi);
                            dd[i] = v[8 * j + i] * sg * (1.0f + zi * (1.0f - sg));
                            sums[8 * j + i] += dd[i];
                        }
                        o[j] = pack8(dd);
                    }
                    uint16_t *ob = reinterpret_cast<uint16_t *>(reinterpret_cast<unsigned char *>(a.out) +
                                                                (int64_t)(c0 / 8) * g.Pst * 16);
                    store_with_images<HALF / 8>(g, ob, x, y, z, o);
                } else if (EPI == EPI_STATE) {
                    if (active) {
                        const Geom &sg = a.sg;
                        float nv[3];
#pragma unroll
                        for (int k = 0; k < 3; ++k) nv[k] = s0v[k] + a.oscale[k] * (v[k] + sbias[k]);
                        // the stencil's face ghosts: written by the cell they mirror
                        const int ax = image_of(x, sg.nx, sg.bc), ay = image_of(y, sg.ny, sg.bc),
                                  az = image_of(z, sg.nz, sg.bc);
                        a.s1.eS[sa] = nv[0];
                        a.s1.eL[sa] = nv[1];
                        a.s1.c[sa] = nv[2];
                        mass += (double)nv[2];
                        if (ax != kNone) {
                            const int64_t b = sg.at(ax, y, z);
                            a.s1.eS[b] = nv[0]; a.s1.eL[b] = nv[1]; a.s1.c[b] = nv[2];
                        }
                        if (ay != kNone) {
                            const int64_t b = sg.at(x, ay, z);
                            a.s1.eS[b] = nv[0]; a.s1.eL[b] = nv[1]; a.s1.c[b] = nv[2];
                        }
                        if (az != kNone) {
                            const int64_t b = sg.at(x, y, az);
                            a.s1.eS[b] = nv[0]; a.s1.eL[b] = nv[1]; a.s1.c[b] = nv[2];
                        }
                    }
                } else if (EPI == EPI_LOSS) {
                    if (active) {
                        float gr[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            const float tg = (s1v[c] - s0v[c]) / a.oscale[c];
                            const float diff = v[c] + sbias[c] - tg;
                            sums[HALF] += a.lw[c] * diff * diff;
                            gr[c] = 2.0f * a.lw[c] * diff;
                            sums[c] += gr[c];
                        }
                        const uint4 o[1] = {pack8(gr)};
                        store_with_images<1>(g, a.out, x, y, z, o);
                    }
                }
            }
        }
        if (EPI == EPI_STATE) {
            // deterministic per-CTA FP64 sum of the new c (warps 2-5 hold it)
            double* redd = reinterpret_cast<double *>(smem + C::OFF_REDD);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mass += __shfl_xor_sync(0xffffffffu, mass, o);
            if (lane == 0 && ew < 4) redd[ew] = mass;
            asm volatile("bar.sync 1, %0;" ::"r"(kEpiThreads) : "memory");
            if (ew == 0 && lane == 0 && a.mass_part)
                a.mass_part[blockIdx.x] = ((redd[0] + redd[1]) + redd[2]) + redd[3];
        }
        if (EPI == EPI_DGRAD || EPI == EPI_LOSS) {
            // deterministic per-CTA sums: warp shuffle, then the four warps
            // of each column group in a fixed order
#pragma unroll
            for (int c = 0; c <= HALF; ++c) {
                float sv = sums[c];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, o);
                if (lane == 0) red[ew * (HALF + 1) + c] = sv;
            }
            asm volatile("bar.sync 1, %0;" ::"r"(kEpiThreads) : "memory");
            if (ew == 0) {
                float *dst = a.partials + (int64_t)blockIdx.x * (CO + 1);
                for (int c = lane; c < CO; c += 32) {
                    const int grp = c / HALF, cc = c % HALF;
                    const float *r = red + grp * 4 * (HALF + 1) + cc;
                    dst[c] = ((r[0] + r[HALF + 1]) + r[2 * (HALF + 1)]) + r[3 * (HALF + 1)];
                }
                if (lane == 0)
                    dst[CO] = ((red[HALF] + red[(HALF + 1) + HALF]) + red[2 * (HALF + 1) + HALF]) +
                              red[3 * (HALF + 1) + HALF];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tbase, C::TMEM_COLS);
    }
}

// ---------------------------------------------------------------------------

template <int CX, int CZ>
struct WgCfg {
    static constexpr int SPB = 128 / CX;                  // slots per M block
    static constexpr int NMB = (9 + SPB - 1) / SPB;       // M blocks
    static constexpr int NSLOT = NMB * SPB;
    static constexpr int SEGB = (CX / 8) * kSegPlane;
    static constexpr int XB = NSLOT * SEGB;
    static constexpr int ZB = (CZ / 8) * kTileX * 16;
    static constexpr int STB = XB + ZB;
    static constexpr int NST = 2;
    static constexpr int OFF_BAR = NST * STB;
    static constexpr int NBAR = 2 * NST + 1;
    static constexpr int OFF_SLOT = OFF_BAR + NBAR * 8;
    static constexpr int SMEM = OFF_SLOT + 16;
    static constexpr int NACC = NMB * 3;
    static constexpr int COLS = NACC * CZ;
    static constexpr int TMEM_COLS = COLS <= 32 ? 32 : COLS <= 64 ? 64 : COLS <= 128 ? 128 : COLS <= 256 ? 256 : 512;
    static_assert(COLS <= 512, "TMEM columns");
    static_assert(STB % 16 == 0, "alignment");
};

template <int CX, int CZ>
__global__ void __launch_bounds__(192, 1) wgrad_kernel(const WgradArgs a) {
    using C = WgCfg<CX, CZ>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sb = smem_u32(smem), bars = sb + C::OFF_BAR;
    auto full = [&](uint32_t s) { return bars + 8 * s; };
    auto empty = [&](uint32_t s) { return bars + 8 * (C::NST + s); };
    const uint32_t dbar = bars + 8 * (2 * C::NST);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + C::OFF_SLOT);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + C::OFF_SLOT + 4);
    const NNGeom &g = a.g;
    const int nxt = g.nx / kTileX;
    const int t0 = (int)((int64_t)a.ntiles * blockIdx.x / gridDim.x);
    const int t1 = (int)((int64_t)a.ntiles * (blockIdx.x + 1) / gridDim.x);

    // unused slots (past the nine taps) read as zeros
    for (int st = 0; st < C::NST; ++st)
        for (int i = tid; i < (C::NSLOT - 9) * C::SEGB / 16; i += blockDim.x)
            reinterpret_cast<uint4 *>(smem + st * C::STB + 9 * C::SEGB)[i] = make_uint4(0, 0, 0, 0);
    fence_proxy_async_smem();
    if (tid == 0) {
        for (int s = 0; s < C::NST; ++s) {
            mbar_init(full(s), 1);
            mbar_init(empty(s), 1);
        }
        mbar_init(dbar, 1);
        *abort_flag = 0;
        mbar_init_fence();
    }
    if (warp == 1) tmem_alloc(smem_u32(tslot), C::TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *reinterpret_cast<volatile uint32_t *>(tslot);

    if (warp == 0) {
        if (lane == 0) {
            uint32_t n = 0;
            for (int tt = t0; tt < t1; ++tt, ++n) {
                const uint32_t st = n % C::NST;
                if (n >= (uint32_t)C::NST &&
                    !wait_backoff(empty(st), ((n / C::NST) + 1) & 1, a.limit_ns, abort_flag)) {
                    fail(abort_flag, a.err, 1);
                    break;
                }
                const int xt = tt % nxt, y = (tt / nxt) % g.ny, z = tt / (nxt * g.ny);
                const int x0 = xt * kTileX;
                const uint32_t stage = sb + st * C::STB;
                mbar_expect_tx(full(st), 9 * C::SEGB + C::ZB);
                for (int dz = 0; dz < 3; ++dz)
                    for (int dy = 0; dy < 3; ++dy) {
                        const int64_t pv = g.p(x0 - 1, y + dy - 1, z + dz - 1);
                        for (int j = 0; j < CX / 8; ++j)
                            bulk_load(stage + (dz * 3 + dy) * C::SEGB + j * kSegPlane,
                                      reinterpret_cast<const unsigned char *>(a.x) + ((int64_t)j * g.Pst + pv) * 16,
                                      kSegPlane, full(st));
                    }
                const int64_t pz = g.p(x0, y, z);
                for (int j = 0; j < CZ / 8; ++j)
                    bulk_load(stage + C::XB + j * kTileX * 16,
                              reinterpret_cast<const unsigned char *>(a.dz) + ((int64_t)j * g.Pst + pz) * 16,
                              kTileX * 16, full(st));
            }
            // drain the copies of the last stages
            const uint32_t issued = n;
            for (uint32_t k = issued > (uint32_t)C::NST ? issued - C::NST : 0; k < issued; ++k)
                if (!mbar_wait(full(k % C::NST), (k / C::NST) & 1, a.limit_ns)) atomicOr(a.err, 4);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(128, CZ, true, true);
            // MN-major operands: LBO = stride of 8-voxel K groups (128 B),
            // SBO = stride of 8-channel groups (a segment plane / a dZ plane)
            const uint64_t a0 = smem_desc(sb, 128, kSegPlane);
            const uint64_t b0 = smem_desc(sb + C::XB, 128, kTileX * 16);
            uint32_t n = 0;
            for (int tt = t0; tt < t1; ++tt, ++n) {
                const uint32_t st = n % C::NST;
                if (!wait_or_abort(full(st), (n / C::NST) & 1, a.limit_ns, abort_flag)) {
                    fail(abort_flag, a.err, 1);
                    break;
                }
                tc_fence_after();
                const uint32_t so = (st * C::STB) >> 4;
#pragma unroll
                for (int kb = 0; kb < kTileX / 16; ++kb) {
                    const uint64_t bd = b0 + so + ((kb * 16 * 16) >> 4);
#pragma unroll
                    for (int mb = 0; mb < C::NMB; ++mb)
#pragma unroll
                        for (int dx = 0; dx < 3; ++dx) {
                            const uint64_t ad = a0 + so + ((mb * C::SPB * C::SEGB + (kb * 16 + dx) * 16) >> 4);
                            mma_bf16(tbase + (mb * 3 + dx) * CZ, ad, bd, idesc, (n > 0 || kb > 0) ? 1u : 0u);
                        }
                }
                mma_commit(empty(st));
            }
            mma_commit(dbar);
        }
    }
    // epilogue: all four lane quarters; wait for the last MMA
    if (warp >= 2) {
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;
        const bool have = t1 > t0;
        bool ok = true;
        if (!wait_or_abort(dbar, 0, a.limit_ns, abort_flag)) {
            fail(abort_flag, a.err, 1);
            ok = false;
        }
        tc_fence_after();
        float *out = a.partials + (int64_t)blockIdx.x * 27 * CZ * CX;
        for (int mb = 0; mb < C::NMB; ++mb) {
            const int slot = mb * C::SPB + row / CX, ci = row % CX;
            for (int dx = 0; dx < 3; ++dx) {
#pragma unroll
                for (int c16 = 0; c16 < CZ / 16; ++c16) {
                    float v[16];
                    tmem_ld16(tbase + ((uint32_t)(quarter * 32) << 16) + (mb * 3 + dx) * CZ + 16 * c16, v);
                    if (slot < 9) {
                        const int tap = (slot / 3) * 9 + (slot % 3) * 3 + dx;
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            out[((int64_t)tap * CZ + 16 * c16 + i) * CX + ci] = (ok && have) ? v[i] : 0.f;
                    }
                }
            }
        }
    } else if (warp == 1) {
        // the MMA warp's other lanes wait here too, so every role ends below
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        // make sure no MMA is still running on an aborted CTA
        if (lane == 0 && !mbar_wait(dbar, 0, a.limit_ns)) atomicOr(a.err, 4);
        __syncwarp();
        tmem_dealloc(tbase, C::TMEM_COLS);
    }
}

template <int CI, int CO, int EPI>
cudaError_t conv_launch(const ConvArgs &a, int grid, cudaStream_t s) {
    conv_kernel<CI, CO, EPI><<<grid, kConvThreads, ConvCfg<CI, CO>::SMEM, s>>>(a);
    return cudaGetLastError();
}

template <int CI, int CO>
cudaError_t conv_launch_epi(int epi, const ConvArgs &a, int grid, cudaStream_t s) {
    switch (epi) {
        case EPI_ACT: return conv_launch<CI, CO, EPI_ACT>(a, grid, s);
        case EPI_ACT_TRAIN: return conv_launch<CI, CO, EPI_ACT_TRAIN>(a, grid, s);
        case EPI_DGRAD: return conv_launch<CI, CO, EPI_DGRAD>(a, grid, s);
        case EPI_STATE: return CO == 16 ? conv_launch<CI, 16, EPI_STATE>(a, grid, s) : cudaErrorInvalidValue;
        case EPI_LOSS: return CO == 16 ? conv_launch<CI, 16, EPI_LOSS>(a, grid, s) : cudaErrorInvalidValue;
        default: return cudaErrorInvalidValue;
    }
}

template <int CI, int CO, int EPI>
cudaError_t conv_attr() {
    return cudaFuncSetAttribute(conv_kernel<CI, CO, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                ConvCfg<CI, CO>::SMEM);
}

template <int CI, int CO>
cudaError_t conv_attr_all() {
    cudaError_t e;
    if ((e = conv_attr<CI, CO, EPI_ACT>()) != cudaSuccess) return e;
    if ((e = conv_attr<CI, CO, EPI_ACT_TRAIN>()) != cudaSuccess) return e;
    if ((e = conv_attr<CI, CO, EPI_DGRAD>()) != cudaSuccess) return e;
    if (CO == 16) {
        if ((e = conv_attr<CI, 16, EPI_STATE>()) != cudaSuccess) return e;
        if ((e = conv_attr<CI, 16, EPI_LOSS>()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <int CX, int CZ>
cudaError_t wgrad_attr() {
    return cudaFuncSetAttribute(wgrad_kernel<CX, CZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                WgCfg<CX, CZ>::SMEM);
}

}  // namespace

template <int CI, int CO>
int conv_per_sm() {
    // shared memory (228 KB per SM, 1 KB reserved per CTA) and TMEM (512 columns per SM)
    const int by_smem = 233472 / (ConvCfg<CI, CO>::SMEM + 1024);
    const int by_tmem = 512 / ConvCfg<CI, CO>::TMEM_COLS;
    const int n = by_smem < by_tmem ? by_smem : by_tmem;
    return n < 1 ? 1 : n;
}

int conv_ctas_per_sm(int ci, int co) {
    if (ci == 16 && co == 16) return conv_per_sm<16, 16>();
    if (ci == 16 && co == 32) return conv_per_sm<16, 32>();
    if (ci == 32 && co == 16) return conv_per_sm<32, 16>();
    if (ci == 32 && co == 32) return conv_per_sm<32, 32>();
    return 1;
}

int conv_smem_bytes(int ci, int co) {
    if (ci == 16 && co == 16) return ConvCfg<16, 16>::SMEM;
    if (ci == 16 && co == 32) return ConvCfg<16, 32>::SMEM;
    if (ci == 32 && co == 16) return ConvCfg<32, 16>::SMEM;
    if (ci == 32 && co == 32) return ConvCfg<32, 32>::SMEM;
    return -1;
}

int wgrad_smem_bytes(int cx, int cz) {
    if (cx == 16 && cz == 16) return WgCfg<16, 16>::SMEM;
    if (cx == 16 && cz == 32) return WgCfg<16, 32>::SMEM;
    if (cx == 32 && cz == 16) return WgCfg<32, 16>::SMEM;
    if (cx == 32 && cz == 32) return WgCfg<32, 32>::SMEM;
    return -1;
}

cudaError_t conv_setup(int max_smem_optin) {
    if (WgCfg<32, 32>::SMEM > max_smem_optin || ConvCfg<32, 32>::SMEM > max_smem_optin) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = conv_attr_all<16, 16>()) != cudaSuccess) return e;
    if ((e = conv_attr_all<16, 32>()) != cudaSuccess) return e;
    if ((e = conv_attr_all<32, 16>()) != cudaSuccess) return e;
    if ((e = conv_attr_all<32, 32>()) != cudaSuccess) return e;
    if ((e = wgrad_attr<16, 16>()) != cudaSuccess) return e;
    if ((e = wgrad_attr<16, 32>()) != cudaSuccess) return e;
    if ((e = wgrad_attr<32, 16>()) != cudaSuccess) return e;
    return wgrad_attr<32, 32>();
}

cudaError_t launch_conv(int ci, int co, int epi, const ConvArgs &a, int grid, cudaStream_t s) {
    if (ci == 16 && co == 16) return conv_launch_epi<16, 16>(epi, a, grid, s);
    if (ci == 16 && co == 32) return conv_launch_epi<16, 32>(epi, a, grid, s);
    if (ci == 32 && co == 16) return conv_launch_epi<32, 16>(epi, a, grid, s);
    if (ci == 32 && co == 32) return conv_launch_epi<32, 32>(epi, a, grid, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_wgrad(int cx, int cz, const WgradArgs &a, int grid, cudaStream_t s) {
    if (cx == 16 && cz == 16) wgrad_kernel<16, 16><<<grid, 192, WgCfg<16, 16>::SMEM, s>>>(a);
    else if (cx == 16 && cz == 32) wgrad_kernel<16, 32><<<grid, 192, WgCfg<16, 32>::SMEM, s>>>(a);
    else if (cx == 32 && cz == 16) wgrad_kernel<32, 16><<<grid, 192, WgCfg<32, 16>::SMEM, s>>>(a);
    else if (cx == 32 && cz == 32) wgrad_kernel<32, 32><<<grid, 192, WgCfg<32, 32>::SMEM, s>>>(a);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

}  // namespace nn
}  // namespace ppf
