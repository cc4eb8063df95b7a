// ppf_step_tma.cuh -- the fused explicit step as a TMA-fed, z-marching,
// persistent sm_103a kernel (instantiated per precision by ppf_step_f32.cu
// and ppf_step_f64.cu for single domains and by ppf_step_f32_ens.cu and
// ppf_step_f64_ens.cu for ensembles, which compile in parallel).
//
// Replaces, per time step, the reference's BC fill (phasefield.c:1112-1189)
// and the three passes of sweep_fields (:325-335 pass A, :347-391 pass B,
// :393-401 pass C) -- or of sweep_fields_c (:406-476) in c-only mode.
//
// Data flow of one CTA:
//   * (z chunk, x-y tile) work items in chunk-major order, taken by the CTAs
//     of a persistent grid from a global counter (or dealt round-robin);
//     each item is a tile column segment marched up z;
//   * thread 0 streams every plane's etaS/etaL/c tile plus a one-cell ring
//     (a TX+2*XH by TY+2 box per field) from HBM into a S-stage shared ring
//     with cp.async.bulk.tensor.3d, completion signalled on an mbarrier per
//     stage; S-2 planes are in flight while one is computed;
//   * pass A (hS, mu, M) is evaluated once per loaded cell into a 3-plane
//     shared ring of mu/M; each thread owns CY cells stacked in y so that
//     its y and z neighbours stay in registers;
//   * pass B + C for plane z-1 then read x/y neighbours from shared memory,
//     and write the new state straight to HBM, including the face ghosts
//     the boundary condition defines (so the next step reads ready ghosts).
// Every mbarrier wait is bounded by a time limit: on expiry the waiting
// thread sets the error word, the plane barrier (__syncthreads_or) tells the
// whole CTA, which drains its own outstanding copies (again bounded) and
// exits uniformly; the host reports PPF_ETIMEOUT.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <type_traits>

#include "ppf_internal.h"
#include "ppf_step_tma.h"

namespace ppf {

// Tile shapes.  TILE 0: FP32 64 x 16 (S = 5: three planes in flight; two
// CTAs of 256 threads fit an SM), FP64 32 x 16.  TILE 1 (FP32 only): 32 x 32,
// which fills domains whose x edge is a multiple of 32 but not of 64; four
// stages (two planes in flight), so that two CTAs still fit an SM.
template <typename T, int TILE = 0>
struct TmaCfg;
template <>
struct TmaCfg<float, 0> {
    static constexpr int TX = 64, TY = 16, NT = 256, S = 5, XH = 4;
};
template <>
struct TmaCfg<float, 1> {
    static constexpr int TX = 32, TY = 32, NT = 256, S = 4, XH = 4;
};
template <>
struct TmaCfg<double, 0> {
    static constexpr int TX = 32, TY = 16, NT = 256, S = 4, XH = 2;
};
template <>
struct TmaCfg<double, 1> : TmaCfg<double, 0> {};   // (not instantiated: FP64 has one tile)

// tile shapes per precision
template <typename T>
constexpr int kTileShapes = std::is_same<T, float>::value ? 2 : 1;

template <typename T, int TILE = 0>
struct TmaGeo {
    using C = TmaCfg<T, TILE>;
    static constexpr int TX = C::TX, TY = C::TY, NT = C::NT, S = C::S, XH = C::XH;
    static constexpr int BX = TX + 2 * XH, BY = TY + 2;
    static constexpr int BOX = BX * BY;                                   // elements per field box
    static constexpr int BOX_BYTES = BOX * (int)sizeof(T);
    static constexpr int BOX_PAD = (BOX_BYTES + 127) / 128 * 128 / (int)sizeof(T);  // 128 B aligned slots
    static constexpr int WX = TX / 32, WY = (NT / 32) / WX, CY = TY / WY;
    static constexpr int RING = 2 * TX + 2 * TY;
    static_assert(TX % 32 == 0 && (NT / 32) % WX == 0 && TY % WY == 0, "tile/warp mismatch");
    static_assert(RING / 2 <= NT, "one ring pair per thread");
    static_assert(BX * sizeof(T) % 16 == 0 && (XH * sizeof(T)) % 16 == 0, "TMA box alignment");
};

template <typename T, int TILE = 0>
struct alignas(128) TmaSmem {
    using G = TmaGeo<T, TILE>;
    T raw[G::S][3][G::BOX_PAD];   // etaS, etaL, c boxes per stage
    T mm[3][2][G::BOX];           // mu, M of three consecutive planes (MmLay)
    unsigned long long bar[G::S];
};

template <typename T, int TILE = 0>
size_t tma_smem_bytes() { return sizeof(TmaSmem<T, TILE>) + 128; }

// ------------------------------------------------------------ PTX glue ----

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait on an mbarrier phase; false when the time limit ran out
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    for (uint32_t it = 0;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 31u) == 31u && globaltimer() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

template <typename T>
__device__ __forceinline__ T fast_rcp(T x);
template <>
__device__ __forceinline__ float fast_rcp<float>(float x) {
    // the hardware reciprocal (rcp.approx.ftz.f32, ~1 ulp): the operands are
    // sums of squares and interpolation weights, never denormal or huge
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
template <>
__device__ __forceinline__ double fast_rcp<double>(double x) { return __drcp_rn(x); }

// Two cells of one thread evaluated together.  For float this is the
// packed f32x2 arithmetic of sm_100+ (one instruction per pair); for double
// it is plain scalar code.  Each lane is rounded exactly as the scalar
// operation would be.
template <typename T>
struct V2;

template <>
struct V2<float> {
    float2 v;
    __device__ __forceinline__ V2() {}
    __device__ __forceinline__ V2(float a, float b) : v(make_float2(a, b)) {}
    __device__ __forceinline__ explicit V2(float2 w) : v(w) {}
    __device__ __forceinline__ float x() const { return v.x; }
    __device__ __forceinline__ float y() const { return v.y; }
};
__device__ __forceinline__ V2<float> operator+(V2<float> a, V2<float> b) { return V2<float>(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ V2<float> operator*(V2<float> a, V2<float> b) { return V2<float>(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ V2<float> operator-(V2<float> a, V2<float> b) {
    unsigned long long ra, xa, ya;
    memcpy(&xa, &a.v, 8);
    memcpy(&ya, &b.v, 8);
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(ra) : "l"(xa), "l"(ya));
    float2 r;
    memcpy(&r, &ra, 8);
    return V2<float>(r);
}
__device__ __forceinline__ V2<float> fma2(V2<float> a, V2<float> b, V2<float> c) {
    return V2<float>(__ffma2_rn(a.v, b.v, c.v));
}

template <>
struct V2<double> {
    double a, b;
    __device__ __forceinline__ V2() {}
    __device__ __forceinline__ V2(double p, double q) : a(p), b(q) {}
    __device__ __forceinline__ explicit V2(double2 w) : a(w.x), b(w.y) {}
    __device__ __forceinline__ double x() const { return a; }
    __device__ __forceinline__ double y() const { return b; }
};
__device__ __forceinline__ V2<double> operator+(V2<double> p, V2<double> q) { return V2<double>(p.a + q.a, p.b + q.b); }
__device__ __forceinline__ V2<double> operator*(V2<double> p, V2<double> q) { return V2<double>(p.a * q.a, p.b * q.b); }
__device__ __forceinline__ V2<double> operator-(V2<double> p, V2<double> q) { return V2<double>(p.a - q.a, p.b - q.b); }
__device__ __forceinline__ V2<double> fma2(V2<double> p, V2<double> q, V2<double> r) {
    return V2<double>(fma(p.a, q.a, r.a), fma(p.b, q.b, r.b));
}

template <typename T>
__device__ __forceinline__ V2<T> splat(T a) { return V2<T>(a, a); }

// a pair stored as two adjacent elements (one 2-element shared access)
__device__ __forceinline__ V2<float> ld2(const float *p) { return V2<float>(*reinterpret_cast<const float2 *>(p)); }
__device__ __forceinline__ V2<double> ld2(const double *p) { return V2<double>(*reinterpret_cast<const double2 *>(p)); }
__device__ __forceinline__ void st2(float *p, V2<float> v) { *reinterpret_cast<float2 *>(p) = v.v; }
__device__ __forceinline__ void st2(double *p, V2<double> v) { *reinterpret_cast<double2 *>(p) = make_double2(v.a, v.b); }

// Layout of one mu or M plane in shared memory (BOX elements): the TY rows
// of the tile as TY/2 pair rows -- pair row wy*H + i interleaves, element by
// element, the rows ty0 + i and ty0 + i + H of warp row wy, so that a
// thread's pair of cells and the pairs beside it in x are one 2-element
// access each -- then the ring rows -1 and TY as plain rows.  Column c of
// every row holds x = c - XH.
template <typename T, int TILE = 0>
struct MmLay {
    using G = TmaGeo<T, TILE>;
    static constexpr int H = G::CY / 2;
    static constexpr int TOP = G::TY * G::BX, BOT = TOP + G::BX;
    static_assert(BOT + G::BX == G::BOX, "mu/M plane size");
    __device__ static int pair(int pr, int col) { return (pr * G::BX + col) * 2; }
    __device__ static int row(int r, int col) {   // element of tile row r in [-1, TY]
        if (r < 0) return TOP + col;
        if (r >= G::TY) return BOT + col;
        const int w = r % G::CY;
        return pair((r / G::CY) * H + w % H, col) + w / H;
    }
};

// The constants of the packed arithmetic as (x, x) pairs, passed in
// parameter space: an f32x2 instruction then takes the pair as one operand
// instead of a register pair rebuilt from the scalar for every use.
template <typename T>
struct PairOf;
template <>
struct PairOf<float> { using type = float2; };
template <>
struct PairOf<double> { using type = double2; };

template <typename T>
struct CoefV {
    using P = typename PairOf<T>::type;
    P AS, dA, AsAl, A, cL0, dc0, Mt0, Mt1, dC, nq1, q1, q2, dm2, mt, tg, nkt, m6, one, zero;
};

template <typename T>
CoefV<T> make_coefv(const Coef<T> &k) {
    auto p = [](T x) {
        typename PairOf<T>::type r;
        r.x = x;
        r.y = x;
        return r;
    };
    CoefV<T> v;
    v.AS = p(k.AS); v.dA = p(k.dA); v.AsAl = p(k.AsAl); v.A = p(k.A);
    v.cL0 = p(k.cL0); v.dc0 = p(k.dc0); v.Mt0 = p(k.Mt0); v.Mt1 = p(k.Mt1);
    v.dC = p(k.dC); v.nq1 = p(-k.q1); v.q1 = p(k.q1); v.q2 = p(k.q2); v.dm2 = p(k.dm2);
    v.mt = p(k.mt); v.tg = p(k.tg); v.nkt = p(-k.kt);
    v.m6 = p(T(-6)); v.one = p(T(1)); v.zero = p(T(0));
    return v;
}

// pass A (phasefield.c:328-332) for a pair of cells: mu and M' = tmp3 M,
// with EQ (AS == AL) the denominator AS+(AL-AS)hS is the constant AS and
// mu = AS (c - cL0 + (cL0-cS0) hS); plus the centre-only part of pass B,
// tmp1 dmu of :351-359, through the identity
//   fS - fL - mu (cS - cL) = (CS-CL) - mu ((cS0-cL0) + (1/AS-1/AL)/2 mu).
template <typename T, bool EQ>
__device__ __forceinline__ void pass_a_own2(const CoefV<T> &kv, V2<T> eS, V2<T> eL, V2<T> c, V2<T> &mu, V2<T> &Mt,
                                            V2<T> &dmu) {
    const V2<T> S2 = eS * eS;
    const V2<T> s2 = fma2(eL, eL, S2);
    const V2<T> rs(fast_rcp(s2.x()), fast_rcp(s2.y()));
    const V2<T> h = S2 * rs;
    const V2<T> w = fma2(h, V2<T>(kv.dc0), c - V2<T>(kv.cL0));
    if (EQ) {
        mu = V2<T>(kv.A) * w;
    } else {
        const V2<T> den = fma2(h, V2<T>(kv.dA), V2<T>(kv.AS));
        mu = V2<T>(kv.AsAl) * V2<T>(fast_rcp(den.x()), fast_rcp(den.y())) * w;
    }
    Mt = fma2(h, V2<T>(kv.Mt1), V2<T>(kv.Mt0));
    const V2<T> D = EQ ? fma2(mu, V2<T>(kv.nq1), V2<T>(kv.dC))
                       : V2<T>(kv.dC) - mu * fma2(mu, V2<T>(kv.q2), V2<T>(kv.q1));
    dmu = V2<T>(kv.dm2) * (eS * eL) * (rs * rs) * D;
}

// pass A alone for a pair (c-only steps)
template <typename T, bool EQ>
__device__ __forceinline__ void pass_a2(const CoefV<T> &kv, V2<T> eS, V2<T> eL, V2<T> c, V2<T> &mu, V2<T> &Mt) {
    const V2<T> S2 = eS * eS;
    const V2<T> s2 = fma2(eL, eL, S2);
    const V2<T> rs(fast_rcp(s2.x()), fast_rcp(s2.y()));
    const V2<T> h = S2 * rs;
    const V2<T> w = fma2(h, V2<T>(kv.dc0), c - V2<T>(kv.cL0));
    if (EQ) {
        mu = V2<T>(kv.A) * w;
    } else {
        const V2<T> den = fma2(h, V2<T>(kv.dA), V2<T>(kv.AS));
        mu = V2<T>(kv.AsAl) * V2<T>(fast_rcp(den.x()), fast_rcp(den.y())) * w;
    }
    Mt = fma2(h, V2<T>(kv.Mt1), V2<T>(kv.Mt0));
}

// One face ghost cell at storage index `a` (the BC fill of
// phasefield.c:1112-1189 applied to the new state; the caller picks the
// ghost that each boundary cell feeds).
template <typename T, bool C_ONLY, typename I = int64_t>
__device__ __forceinline__ void put_ghost(const Fields<T> &o, I a, T s, T l, T c) {
    if (!C_ONLY) {
        o.eS[a] = s;
        o.eL[a] = l;
    }
    o.c[a] = c;
}

// Work items are (z chunk, x-y tile) pairs in chunk-major order, taken in
// that order by the persistent CTAs: CTAs resident at the same time march
// the same z window of neighbouring tiles, so the halo rows one tile reads
// from its neighbours' data are mostly still in L2.

// Registers of the own cells of one plane, as pairs (cell i, cell i+H) of
// the thread's column of CY = 2H cells: with that pairing the y neighbours
// of pair i are mostly the pairs i-1 and i+1 themselves.
template <typename T, int H>
struct PlaneRegs {
    V2<T> S[H], L[H], mu[H], M[H], c[H], d[H];
};

// A work item: one tile column segment of one domain (tile bx, by; interior
// planes z0 .. z1-1).
struct Item {
    int dom, bx, by, z0, z1;
};

// The tiles of one launch.  A step is one launch over every tile (SET_ALL;
// SET_WIDE with 64-bit offsets, for a domain whose fields exceed 2^32
// elements), or, when every tile lies inside the domain, over the whole
// tiles (SET_WHOLE: the nfx x nfy rectangle of tiles inside the domain,
// whose plane body needs no per-cell "inside" test), or two launches: the
// whole tiles and the edge tiles (SET_EDGE: the column of partial tiles at
// high x when nx is not a multiple of the tile width, then the row of
// partial tiles at high y).
enum { SET_WIDE = 0, SET_EDGE = 1, SET_WHOLE = 2, SET_ALL = 3 };

struct Tiles {
    int ntx, nty;   // tiles in x and y
    int nfx, nfy;   // whole tiles in x and y
};

__host__ __device__ inline int tiles_in_set(const Tiles &t, int set) {
    return set == SET_WHOLE ? t.nfx * t.nfy : set == SET_EDGE ? t.ntx * t.nty - t.nfx * t.nfy : t.ntx * t.nty;
}

// tile k of the set
template <int SET>
__device__ __forceinline__ void tile_of(int k, const Tiles &t, int &bx, int &by) {
    if (SET == SET_ALL || SET == SET_WIDE) {
        by = k / t.ntx;
        bx = k - by * t.ntx;
    } else if (SET == SET_WHOLE) {
        by = k / t.nfx;
        bx = k - by * t.nfx;
    } else {
        if (t.nfx < t.ntx) {           // the high-x column of partial tiles
            if (k < t.nty) {
                bx = t.nfx;
                by = k;
                return;
            }
            k -= t.nty;
        }
        bx = k;                        // the high-y row of partial tiles
        by = t.nfy;
    }
}

// How a single domain's z range is cut into work-item chunks: n1 chunks of
// zc planes, then chunks of zc2 planes up to nz (the last one may be
// shorter).  Shorter chunks at the top of z make the last items of a step
// short, so that the CTAs end closer together.
struct ZSplit {
    int zc, zc2, n1;
};

// Work item `item` of the launch.  Single domain: (z chunk, tile of the
// set) in chunk-major order.  Ensemble (MULTI): the items of each domain are
// contiguous, chunk-major within the domain (the set's item range of each
// domain in the table; a domain may have none).
template <bool MULTI, int SET>
__device__ __forceinline__ Item item_at(int item, const Tiles &t1, const ZSplit &zs, int nz, const DomainDesc *table,
                                        int ndom) {
    Item it;
    if (!MULTI) {
        const int nt = tiles_in_set(t1, SET);
        const int c = item / nt;
        it.dom = 0;
        tile_of<SET>(item - c * nt, t1, it.bx, it.by);
        it.z0 = c < zs.n1 ? c * zs.zc : zs.n1 * zs.zc + (c - zs.n1) * zs.zc2;
        it.z1 = min(nz, it.z0 + (c < zs.n1 ? zs.zc : zs.zc2));
        return it;
    }
    const int s = SET == SET_WHOLE ? 1 : SET == SET_EDGE ? 0 : 2;
    int lo = 0, hi = ndom - 1;                 // last domain with item0 <= item
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (table[mid].item0[s] <= item) lo = mid;
        else hi = mid - 1;
    }
    const DomainDesc &d = table[lo];
    const Tiles td = {d.ntx, d.nty, d.nfx, d.nfy};
    const int nt = tiles_in_set(td, SET);
    const int li = item - d.item0[s];
    const int c = li / nt;
    it.dom = lo;
    tile_of<SET>(li - c * nt, td, it.bx, it.by);
    it.z0 = c * d.zc;
    it.z1 = min(d.g.nz, it.z0 + d.zc);
    return it;
}

// SET: the launch's tiles (SET_WHOLE: no per-cell "inside the domain" test;
// SET_EDGE, SET_ALL: with it; SET_WIDE: with it and 64-bit element offsets,
// for fields of more than 2^32 elements; the other sets use 32-bit offsets).
template <typename T, bool STATS, bool C_ONLY, bool EQ, int ROLL, bool MULTI, int SET, int TILE>
__global__ void __launch_bounds__(TmaGeo<T, TILE>::NT, 2)
    step_tma_kernel(const __grid_constant__ CUtensorMap mapS, const __grid_constant__ CUtensorMap mapL,
                    const __grid_constant__ CUtensorMap mapC, Geom g1, Coef<T> k, CoefV<T> kv, Fields<T> out1,
                    Tiles t1, ZSplit zs1, double *__restrict__ partials, int *__restrict__ err, unsigned long long limit_ns,
                    int inject_stall, const DomainDesc *__restrict__ table, int ndom, int mitems, int parity,
                    int *__restrict__ sched, int second) {
    using G = TmaGeo<T, TILE>;
    constexpr int TX = G::TX, TY = G::TY, S = G::S, XH = G::XH, BX = G::BX, CY = G::CY;
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    // 128-byte alignment by an offset from the shared array itself, so that
    // every derived pointer stays a shared-window pointer (LDS/STS, 32-bit
    // addressing) rather than a generic one
    const uint32_t pad = (128u - (smem_u32(smem_dyn) & 127u)) & 127u;
    TmaSmem<T, TILE> &sm = *reinterpret_cast<TmaSmem<T, TILE> *>(smem_dyn + pad);

    // Programmatic dependent launch (no-ops when the launch does not allow
    // the overlap).  A step is one launch, or two over disjoint tile sets
    // that read the same input and write disjoint cells.  The first launch
    // of a step waits for the previous grid -- the previous step, which wrote
    // what it reads -- to complete, and then lets the next grid be scheduled
    // (its CTAs take SM slots as this grid's CTAs leave).  The second launch
    // of a step (`second`) depends on nothing of the first: its CTAs start
    // in the first launch's tail, since that launch let it be scheduled only
    // after the previous step had completed, and they wait for the first
    // launch to complete only before they exit, so that this grid's end
    // also ends the step.
    if (!second) asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tx = (warp % G::WX) * 32 + lane;        // own column in the tile
    const int ty0 = (warp / G::WX) * CY;              // first own row in the tile
    const int nitems = mitems;
    const int ob = (ty0 + 1) * BX + tx + XH;          // shared offset of the first own cell
    static_assert(!(MULTI && SET == SET_WIDE), "ensemble domains hold fewer than 2^32 elements per field");
    constexpr bool FULL = SET == SET_WHOLE;
    // the pair of cells of the one-cell ring around the tile that this thread
    // evaluates: the last RING/2 threads (warp 0 also feeds the TMA ring), each
    // a cell of the top row with the one below it in the bottom row, or a cell
    // of the left column with the one beside it in the right column
    constexpr int RP = G::RING / 2;
    const bool ring = tid >= G::NT - RP;
    int ring_o0 = 0, ring_o1 = 0, ring_m0 = 0, ring_m1 = 0;   // in the TMA box / the mu-M plane
    if (ring) {
        const int r = tid - (G::NT - RP);
        if (r < TX) {
            ring_o0 = XH + r;                               // (r, -1)
            ring_o1 = (TY + 1) * BX + XH + r;               // (r, TY)
            ring_m0 = MmLay<T, TILE>::row(-1, XH + r);
            ring_m1 = MmLay<T, TILE>::row(TY, XH + r);
        } else {
            ring_o0 = (r - TX + 1) * BX + XH - 1;           // (-1, r - TX)
            ring_o1 = (r - TX + 1) * BX + XH + TX;          // (TX, r - TX)
            ring_m0 = MmLay<T, TILE>::row(r - TX, XH - 1);
            ring_m1 = MmLay<T, TILE>::row(r - TX, XH + TX);
        }
    }
    // the thread's first pair in a mu/M plane, and its rows above and below
    const int pofs = MmLay<T, TILE>::pair((warp / G::WX) * (CY / 2), tx + XH);
    const int m_above = MmLay<T, TILE>::row(ty0 - 1, tx + XH), m_below = MmLay<T, TILE>::row(ty0 + CY, tx + XH);

    // increment sums of the statistics step: per thread and work item in the
    // state's precision (packed, one FMA per pair; FP32: at most 2 zc squares
    // per lane), then in FP64 across lanes, warps and items
    V2<T> acc[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) acc[i] = splat(T(0));
    __shared__ int s_next[2];
    // (with the scheduler every CTA takes part, so that the count of CTAs
    // that stopped taking items reaches the grid size)
    if (sched || (int)blockIdx.x < nitems) {
        if (tid == 0) {
            for (int s = 0; s < S; ++s) mbar_init(smem_u32(&sm.bar[s]), 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }

        // producer (thread 0): takes the CTA's items and walks their planes,
        // S-2 loads ahead of the consumers.  Items come round-robin
        // (blockIdx.x, + gridDim.x, ...) or, with a scheduler word pair,
        // blockIdx.x first and then gridDim.x + a global counter, in the same
        // chunk-major order, so that a CTA that runs faster takes more items
        // (the grid never exceeds the item count).  Each item id is published in s_next
        // (two slots: an item spans at least three planes, so the producer is
        // never more than one item ahead), written at least two plane
        // barriers before the consumers read it.
        int p_item = 0, p_pz = 0, p_xs = 0, p_ys = 0, p_seq = 0;
        bool p_done = sched == nullptr;           // stopped taking items (dynamic mode)
        auto take = [&]() {
            int v;
            if (sched) {
                // a CTA's first item is its own index (no counter round trip before
                // the first load); later ones come from the counter
                v = p_seq == 0 ? (int)blockIdx.x : (int)gridDim.x + atomicAdd(&sched[0], 1);
                if (v >= nitems) {
                    v = nitems;
                    // the last CTA to stop taking items resets the pair for the next launch
                    if (atomicAdd(&sched[1], 1) == (int)gridDim.x - 1) {
                        atomicExch(&sched[0], 0);
                        atomicExch(&sched[1], 0);
                    }
                    p_done = true;
                }
            } else {
                v = p_seq == 0 ? (int)blockIdx.x : min(nitems, p_item + (int)gridDim.x);
            }
            s_next[p_seq & 1] = v;
            ++p_seq;
            p_item = v;
        };
        const CUtensorMap *p_mS = &mapS, *p_mL = &mapL, *p_mC = &mapC;
        Item p_it;
        auto p_set = [&]() {
            if (p_item < nitems) {
                p_it = item_at<MULTI, SET>(p_item, t1, zs1, g1.nz, table, ndom);
                p_pz = p_it.z0 - 1;
                // the item's box corner: storage x of the box start (16-byte
                // aligned) and storage y of interior row y0-1
                const int xoff = MULTI ? table[p_it.dom].g.xoff : g1.xoff;
                p_xs = p_it.bx * TX + xoff - XH;
                p_ys = p_it.by * TY;
                if (MULTI) {
                    p_mS = &table[p_it.dom].maps[parity][0];
                    p_mL = &table[p_it.dom].maps[parity][1];
                    p_mC = &table[p_it.dom].maps[parity][2];
                }
            }
        };
        int ist = 0, issued = 0;
        auto issue = [&]() {
            const uint32_t bar = smem_u32(&sm.bar[ist]);
            const int zs = p_pz + 1;                   // storage z of the plane
            uint32_t bytes = 3u * (uint32_t)G::BOX_BYTES;
            if (inject_stall && issued == 1) bytes += 16u;   // test hook: this phase can never complete
            mbar_expect_tx(bar, bytes);
            tma_load_3d(smem_u32(sm.raw[ist][0]), p_mS, p_xs, p_ys, zs, bar);
            tma_load_3d(smem_u32(sm.raw[ist][1]), p_mL, p_xs, p_ys, zs, bar);
            tma_load_3d(smem_u32(sm.raw[ist][2]), p_mC, p_xs, p_ys, zs, bar);
            if (++p_pz > p_it.z1) {
                take();
                p_set();
            }
            ist = ist + 1 == S ? 0 : ist + 1;
            ++issued;
        };
        if (tid == 0) {
            take();
            p_set();
            for (int l = 0; l < S - 2 && p_item < nitems; ++l) issue();
        }
        __syncthreads();                              // barriers initialised, first item published

        // three register planes whose roles rotate: q-1, q, q+1
        constexpr int H = CY / 2;
        static_assert(CY % 2 == 0, "cells are processed in pairs");
        PlaneRegs<T, H> RA, RB, RC;
#pragma unroll
        for (int i = 0; i < H; ++i) {
            RA.S[i] = RA.L[i] = RA.mu[i] = RA.M[i] = RA.c[i] = RA.d[i] = splat(T(0));
            RB.S[i] = RB.L[i] = RB.mu[i] = RB.M[i] = RB.c[i] = RB.d[i] = splat(T(0));
        }

        int st = 0, mb = 0, consumed = 0;            // stage / mu-M buffer / count of the current load
        uint32_t par = 0;
        int st_prev = 0, mb_prev = 0;
        bool dead = false;
        for (int seq = 0; !dead; ++seq) {
            const int item = s_next[seq & 1];
            if (item >= nitems) break;
            const Item it = item_at<MULTI, SET>(item, t1, zs1, g1.nz, table, ndom);
            const Geom g = MULTI ? table[it.dom].g : g1;
            Fields<T> out = out1;
            if (MULTI) {
                out.eS = (T *)table[it.dom].fld[1 - parity][0];
                out.eL = (T *)table[it.dom].fld[1 - parity][1];
                out.c = (T *)table[it.dom].fld[1 - parity][2];
            }
            const int x0 = it.bx * TX, y0 = it.by * TY, z0 = it.z0, z1 = it.z1;
            const int X = x0 + tx;
            // per own row j: inside the domain (bit j of vmask)
            unsigned vmask = 0;
#pragma unroll
            for (int j = 0; j < CY; ++j) {
                const int Y = y0 + ty0 + j;
                if (X < g.nx && Y < g.ny) vmask |= 1u << j;
            }
            const int64_t col = (int64_t)(y0 + ty0 + 1) * g.P + X + g.xoff;   // storage of own cell j=0, z=-1

            // one plane: load/pass A of plane pz into Xr, pass B + C of plane pz-1
            // from (Pr = pz-2, Qr = pz-1, Xr = pz); false once the item is done
            auto plane = [&](int pz, PlaneRegs<T, H> &Pr, PlaneRegs<T, H> &Qr, PlaneRegs<T, H> &Xr) -> bool {
                if (pz > z1) return false;
                const bool late = !mbar_wait(smem_u32(&sm.bar[st]), par, limit_ns);
                if (late) atomicOr(err, 1);
                const T *rS = sm.raw[st][0], *rL = sm.raw[st][1], *rC = sm.raw[st][2];
                T *wmu = sm.mm[mb][0], *wM = sm.mm[mb][1];
#pragma unroll
                for (int i = 0; i < H; ++i) {
                    const int o0 = ob + i * BX, o1 = o0 + H * BX;     // cells i and i+H
                    Xr.S[i] = V2<T>(rS[o0], rS[o1]);
                    Xr.L[i] = V2<T>(rL[o0], rL[o1]);
                    Xr.c[i] = V2<T>(rC[o0], rC[o1]);
                    if (C_ONLY) {
                        pass_a2<T, EQ>(kv, Xr.S[i], Xr.L[i], Xr.c[i], Xr.mu[i], Xr.M[i]);
                    } else {
                        pass_a_own2<T, EQ>(kv, Xr.S[i], Xr.L[i], Xr.c[i], Xr.mu[i], Xr.M[i], Xr.d[i]);
                    }
                    st2(wmu + pofs + 2 * BX * i, Xr.mu[i]);
                    st2(wM + pofs + 2 * BX * i, Xr.M[i]);
                }
                if (ring) {                            // the one-cell ring around the tile
                    V2<T> mu, M;
                    pass_a2<T, EQ>(kv, V2<T>(rS[ring_o0], rS[ring_o1]), V2<T>(rL[ring_o0], rL[ring_o1]),
                                   V2<T>(rC[ring_o0], rC[ring_o1]), mu, M);
                    wmu[ring_m0] = mu.x();
                    wmu[ring_m1] = mu.y();
                    wM[ring_m0] = M.x();
                    wM[ring_m1] = M.y();
                }
                // the plane barrier also tells every thread whether any wait ran out
                if (__syncthreads_or(late)) { dead = true; return false; }
                if (tid == 0 && p_item < nitems) issue();   // refill the stage freed two planes ago

                const int q = pz - 1;
                if (q >= z0) {
                    const T *nS = sm.raw[st_prev][0], *nL = sm.raw[st_prev][1];
                    const T *nmu = sm.mm[mb_prev][0], *nM = sm.mm[mb_prev][1];
                    // 32-bit element offsets unless the fields exceed 2^32 elements
                    using Off = typename std::conditional<SET == SET_WIDE, int64_t, uint32_t>::type;
                    const Off base = (Off)col + (Off)(q + 1) * (Off)g.PS;
                    // the new values of the plane's own cells, kept for the face ghosts below
                    V2<T> gS[H], gL[H], gC[H];
#pragma unroll
                    for (int i = 0; i < H; ++i) {
                        const int j0 = i, j1 = i + H;                       // the pair's cells
                        const bool v0 = FULL || (vmask & (1u << j0)), v1 = FULL || (vmask & (1u << j1));
                        // (a pair outside the domain is computed from whatever the
                        // box holds there; nothing of it is stored or summed)
                        const int o0 = ob + j0 * BX, o1 = ob + j1 * BX;
                        const V2<T> mu = Qr.mu[i], M = Qr.M[i], c = Qr.c[i];
                        // y neighbours: pair i-1 / i+1, or a shared row at the column ends
                        const V2<T> muym = i > 0 ? Qr.mu[i - 1] : V2<T>(nmu[m_above], Qr.mu[H - 1].x());
                        const V2<T> Mym = i > 0 ? Qr.M[i - 1] : V2<T>(nM[m_above], Qr.M[H - 1].x());
                        const V2<T> muyp = i < H - 1 ? Qr.mu[i + 1] : V2<T>(Qr.mu[0].y(), nmu[m_below]);
                        const V2<T> Myp = i < H - 1 ? Qr.M[i + 1] : V2<T>(Qr.M[0].y(), nM[m_below]);
                        const int po = pofs + 2 * BX * i;              // the pair in the mu/M plane
                        const V2<T> muxp = ld2(nmu + po + 2), muxm = ld2(nmu + po - 2);
                        const V2<T> Mxp = ld2(nM + po + 2), Mxm = ld2(nM + po - 2);
                        // dc: the flux form of phasefield.c:374-384, tmp3 inside M'.
                        // The six face fluxes are summed first and added to c once,
                        // so c is rounded once per step.
                        V2<T> fl = (Xr.M[i] + M) * (Xr.mu[i] - mu);
                        fl = fma2(Pr.M[i] + M, Pr.mu[i] - mu, fl);
                        fl = fma2(Myp + M, muyp - mu, fl);
                        fl = fma2(Mym + M, muym - mu, fl);
                        fl = fma2(Mxp + M, muxp - mu, fl);
                        fl = fma2(Mxm + M, muxm - mu, fl);
                        const V2<T> cn = c + fl;
                        // a cell outside the domain stores to the first element of its
                        // plane (column 0 of ghost row -1: padding that nothing reads),
                        // so that the stores need no predicate
                        const Off sink = base - (Off)col;
                        const Off a0 = v0 ? base + (Off)j0 * (Off)g.P : sink;
                        const Off a1 = v1 ? base + (Off)j1 * (Off)g.P : sink;
                        if (C_ONLY) {
                            out.c[a0] = cn.x();
                            out.c[a1] = cn.y();
                            gS[i] = gL[i] = splat(T(0));
                            gC[i] = cn;
                            if (STATS) {
                                const V2<T> f = FULL ? fl : V2<T>(v0 ? fl.x() : T(0), v1 ? fl.y() : T(0));
                                acc[0] = fma2(f, f, acc[0]);
                            }
                        } else {
                            const V2<T> eS = Qr.S[i], eL = Qr.L[i], dmu = Qr.d[i];
                            const V2<T> Sym = i > 0 ? Qr.S[i - 1] : V2<T>(nS[o0 - BX], Qr.S[H - 1].x());
                            const V2<T> Lym = i > 0 ? Qr.L[i - 1] : V2<T>(nL[o0 - BX], Qr.L[H - 1].x());
                            const V2<T> Syp = i < H - 1 ? Qr.S[i + 1] : V2<T>(Qr.S[0].y(), nS[o1 + BX]);
                            const V2<T> Lyp = i < H - 1 ? Qr.L[i + 1] : V2<T>(Qr.L[0].y(), nL[o1 + BX]);
                            // detaS, detaL of phasefield.c:360-373 with tmp1 absorbed, in
                            // the reference's grouping  mt eta (eta^2 - 1 + 2 gamma other^2)
                            //   - kt (sum6 - 6 eta) -/+ other tmp1 dmu,  which is exactly
                            // zero for a pure phase (eta = 1, other = 0, flat neighbours)
                            const V2<T> S6 = Xr.S[i] + Pr.S[i] + Syp + Sym + V2<T>(nS[o0 + 1], nS[o1 + 1]) +
                                             V2<T>(nS[o0 - 1], nS[o1 - 1]);
                            const V2<T> L6 = Xr.L[i] + Pr.L[i] + Lyp + Lym + V2<T>(nL[o0 + 1], nL[o1 + 1]) +
                                             V2<T>(nL[o0 - 1], nL[o1 - 1]);
                            const V2<T> one(kv.one), tg(kv.tg), nkt(kv.nkt), m6(kv.m6), mt(kv.mt);
                            const V2<T> S2 = eS * eS, L2 = eL * eL;
                            const V2<T> lapS = fma2(m6, eS, S6), lapL = fma2(m6, eL, L6);
                            const V2<T> dS = fma2(mt * eS, fma2(tg, L2, S2 - one), fma2(nkt, lapS, eL * dmu));
                            const V2<T> dL = fma2(mt * eL, fma2(tg, S2, L2 - one), fma2(nkt, lapL, V2<T>(kv.zero) - eS * dmu));
                            const V2<T> Sn = eS + dS, Ln = eL + dL;
                            out.eS[a0] = Sn.x();
                            out.eL[a0] = Ln.x();
                            out.c[a0] = cn.x();
                            out.eS[a1] = Sn.y();
                            out.eL[a1] = Ln.y();
                            out.c[a1] = cn.y();
                            gS[i] = Sn;
                            gL[i] = Ln;
                            gC[i] = cn;
                            if (STATS) {
                                const V2<T> f = FULL ? fl : V2<T>(v0 ? fl.x() : T(0), v1 ? fl.y() : T(0));
                                const V2<T> ds = FULL ? dS : V2<T>(v0 ? dS.x() : T(0), v1 ? dS.y() : T(0));
                                const V2<T> dl = FULL ? dL : V2<T>(v0 ? dL.x() : T(0), v1 ? dL.y() : T(0));
                                acc[0] = fma2(f, f, acc[0]);
                                acc[1] = fma2(ds, ds, acc[1]);
                                acc[2] = fma2(dl, dl, acc[2]);
                            }
                        }
                    }
                    {
                        // face ghosts straight from the kept values.  An x face is a
                        // whole thread column, a y face one own row of a thread, a z face
                        // a plane; cells outside the domain (partial tiles) feed none.
                        // Periodic: cell 0 feeds ghost n, cell n-1 ghost -1; no-flux:
                        // cell 0 feeds ghost -1, cell n-1 ghost n.
                        const bool per = g.bc == 0;
                        const int Yf = y0 + ty0;
                        auto put_row = [&](int j, Off d) {    // own row j (a constant once unrolled)
                            if (!FULL && !(vmask & (1u << j))) return;
                            const Off a = base + (Off)j * (Off)g.P + d;
                            if (j < H) put_ghost<T, C_ONLY, Off>(out, a, gS[j].x(), gL[j].x(), gC[j].x());
                            else put_ghost<T, C_ONLY, Off>(out, a, gS[j - H].y(), gL[j - H].y(), gC[j - H].y());
                        };
                        // (a one-cell-wide domain feeds both x ghosts from the same cell)
                        if (X == 0) {
                            const Off d = per ? (Off)g.nx : (Off)-1;
#pragma unroll
                            for (int j = 0; j < CY; ++j) put_row(j, d);
                        }
                        if (X == g.nx - 1) {
                            const Off d = per ? (Off)-g.nx : (Off)1;
#pragma unroll
                            for (int j = 0; j < CY; ++j) put_row(j, d);
                        }
#pragma unroll
                        for (int j = 0; j < CY; ++j) {
                            // with whole tiles a y face row is a thread's first or last
                            if (FULL ? (j == 0 && Yf == 0) : (Yf + j == 0))
                                put_row(j, per ? (Off)g.ny * (Off)g.P : (Off)-g.P);
                            if (FULL ? (j == CY - 1 && Yf + CY == g.ny) : (Yf + j == g.ny - 1))
                                put_row(j, per ? (Off)(-g.ny) * (Off)g.P : (Off)g.P);
                        }
                        if (q == 0) {
                            const Off d = per ? (Off)g.nz * (Off)g.PS : (Off)-g.PS;
#pragma unroll
                            for (int j = 0; j < CY; ++j) put_row(j, d);
                        }
                        if (q == g.nz - 1) {
                            const Off d = per ? (Off)(-g.nz) * (Off)g.PS : (Off)g.PS;
#pragma unroll
                            for (int j = 0; j < CY; ++j) put_row(j, d);
                        }
                    }
                }
                st_prev = st;
                mb_prev = mb;
                if (++st == S) { st = 0; par ^= 1u; }
                mb = mb + 1 == 3 ? 0 : mb + 1;
                ++consumed;
                return true;
            };
            if (ROLL == 3) {
                // three copies of the plane body, the register planes renamed
                // instead of copied
                for (int pz = z0 - 1;; pz += 3) {
                    if (!plane(pz, RA, RB, RC)) break;
                    if (!plane(pz + 1, RB, RC, RA)) break;
                    if (!plane(pz + 2, RC, RA, RB)) break;
                }
            } else {
                // one copy of the plane body (a third of the code), the
                // register planes moved down after each plane
                for (int pz = z0 - 1;; ++pz) {
                    if (!plane(pz, RA, RB, RC)) break;
                    RA = RB;
                    RB = RC;
                }
            }
            if (STATS && !dead) {
                // the increment sums of each work item, summed later in item order
                // (the same bits whichever CTA took the item)
                __shared__ double ired[G::NT / 32][3];
                __syncthreads();
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    double v = (double)acc[i].x() + (double)acc[i].y();
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0) ired[warp][i] = v;
                    acc[i] = splat(T(0));
                }
                __syncthreads();
                if (tid == 0)
                    for (int i = 0; i < 3; ++i) {
                        double sv = 0;
                        for (int w = 0; w < G::NT / 32; ++w) sv += ired[w][i];
                        partials[(int64_t)item * 3 + i] = sv;
                    }
            }
        }
        if (dead) {
            // drain this CTA's own copies still in flight (bounded), stop taking
            // items (the remaining CTAs then reset the scheduler pair), leave
            if (tid == 0) {
                for (int d = 0; d < issued - consumed; ++d)
                    (void)mbar_wait(smem_u32(&sm.bar[(st + d) % S]), par ^ (uint32_t)(((st + d) / S) & 1), limit_ns);
                if (!p_done && atomicAdd(&sched[1], 1) == (int)gridDim.x - 1) {
                    atomicExch(&sched[0], 0);
                    atomicExch(&sched[1], 0);
                }
            }
        }
    }
    if (second) asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ------------------------------------------------------------------ host --

static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

template <typename T, int TILE>
static int make_field_map_t(const Geom &g, const T *base, CUtensorMap *map) {
    using G = TmaGeo<T, TILE>;
    auto enc = get_encode();
    if (!enc) return -1;
    if ((reinterpret_cast<uintptr_t>(base) & 15) || ((g.P * sizeof(T)) & 15)) return -2;
    const cuuint64_t dims[3] = {(cuuint64_t)g.P, (cuuint64_t)(g.ny + 2), (cuuint64_t)(g.nz + 2)};
    const cuuint64_t strides[2] = {(cuuint64_t)(g.P * sizeof(T)), (cuuint64_t)(g.PS * sizeof(T))};
    const cuuint32_t box[3] = {(cuuint32_t)G::BX, (cuuint32_t)G::BY, 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    CUresult r = enc(map, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
                     (void *)base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? 0 : -3;
}

template <typename T>
int make_field_map(const Geom &g, const T *base, CUtensorMap *map, int tile) {
    if (kTileShapes<T> > 1 && tile == 1) return make_field_map_t<T, 1>(g, base, map);
    return make_field_map_t<T, 0>(g, base, map);
}

template <typename T, bool ST, bool CO, bool EQ, int R, bool M, int TILE>
static cudaError_t set_attr1() {
    // (single-domain and ensemble variants are set up, and compiled, in
    // separate translation units)
    const int sh = (int)tma_smem_bytes<T, TILE>();
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e;
    // (the plane body is unrolled three times only for whole tiles)
    if ((e = cudaFuncSetAttribute(step_tma_kernel<T, ST, CO, EQ, R, M, SET_WHOLE, TILE>, a, sh))) return e;
    if constexpr (R == 1) {
        if ((e = cudaFuncSetAttribute(step_tma_kernel<T, ST, CO, EQ, 1, M, SET_EDGE, TILE>, a, sh)) ||
            (e = cudaFuncSetAttribute(step_tma_kernel<T, ST, CO, EQ, 1, M, SET_ALL, TILE>, a, sh)))
            return e;
        if constexpr (!M) return cudaFuncSetAttribute(step_tma_kernel<T, ST, CO, EQ, 1, false, SET_WIDE, TILE>, a, sh);
    }
    return cudaSuccess;
}

template <typename T, int R, bool M, int TILE>
static cudaError_t set_attrs_r() {
    cudaError_t e;
    if ((e = set_attr1<T, false, false, false, R, M, TILE>()) || (e = set_attr1<T, true, false, false, R, M, TILE>()) ||
        (e = set_attr1<T, false, true, false, R, M, TILE>()) || (e = set_attr1<T, true, true, false, R, M, TILE>()) ||
        (e = set_attr1<T, false, false, true, R, M, TILE>()) || (e = set_attr1<T, true, false, true, R, M, TILE>()) ||
        (e = set_attr1<T, false, true, true, R, M, TILE>()) || (e = set_attr1<T, true, true, true, R, M, TILE>()))
        return e;
    return cudaSuccess;
}

// CTAs per SM of the step kernels of one tile shape (M: the ensemble
// variants, else the single-domain ones), with their attributes set first;
// per device, once.  0 on failure.
template <typename T, bool M, int TILE>
static int step_occupancy() {
    static int occ_of[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    int &occ = occ_of[dev];
    if (!occ) {
        if (set_attrs_r<T, 1, M, TILE>() != cudaSuccess || set_attrs_r<T, 3, M, TILE>() != cudaSuccess) return 0;
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, step_tma_kernel<T, false, false, true, 1, M, SET_WHOLE, TILE>,
                                                          TmaGeo<T, TILE>::NT, tma_smem_bytes<T, TILE>()) != cudaSuccess ||
            o < 1)
            o = 1;
        occ = o;
    }
    return occ;
}

template <typename T, bool M>
static int step_occupancy(int tile) {
    if constexpr (kTileShapes<T> > 1)
        if (tile == 1) return step_occupancy<T, M, 1>();
    return step_occupancy<T, M, 0>();
}

template <typename T>
void step_tile(int *tx, int *ty, int tile) {
    if (kTileShapes<T> > 1 && tile == 1) {
        *tx = TmaGeo<T, 1>::TX;
        *ty = TmaGeo<T, 1>::TY;
    } else {
        *tx = TmaGeo<T, 0>::TX;
        *ty = TmaGeo<T, 0>::TY;
    }
}

template <typename T>
int step_tile_shapes() { return kTileShapes<T>; }

// Launch shape (the model behind the default z chunk).  Work items are
// (z chunk, tile) pairs dealt round-robin to a persistent grid of `slots`
// CTAs (occupancy x SMs).  The chunk length
// zc is chosen to minimise the busiest CTA's load count -- its planes plus
// two halo planes per item -- so that the resident CTAs end together;
// *zc_out receives it (for the first tile shape).
template <typename T>
int tma_grid(const Geom &g, int num_sms, int *zc_out) {
    using G = TmaGeo<T, 0>;
    const int occ = step_occupancy<T, false>(0);
    if (occ < 1) return -1;
    const int64_t ntiles = (int64_t)((g.nx + G::TX - 1) / G::TX) * ((g.ny + G::TY - 1) / G::TY);
    const int64_t slots = (int64_t)occ * num_sms;
    double best_cost = -1;
    int64_t best_zc = g.nz, best_grid = 1;
    for (int zc = 1; zc <= g.nz; ++zc) {
        const int64_t nc = (g.nz + zc - 1) / zc;
        if (nc > 1 && (nc - 1) * zc >= g.nz) continue;
        const int64_t items = ntiles * nc;
        if (items > ((int64_t)1 << 29)) continue;
        const int64_t grid = items < slots ? items : slots;
        // items of CTA b: b, b+grid, ...; chunk-major, the last chunk is short
        const int64_t last = g.nz - (nc - 1) * zc;
        int64_t worst = 0;
        for (int64_t b = 0; b < grid; b += (grid > 64 ? grid / 64 : 1)) {
            int64_t cost = 0;
            for (int64_t it = b; it < items; it += grid) cost += ((it / ntiles) == nc - 1 ? last : zc) + 2;
            if (cost > worst) worst = cost;
        }
        {   // the final CTA always holds a short item when items % grid != 0
            int64_t cost = 0;
            for (int64_t it = grid - 1; it < items; it += grid) cost += ((it / ntiles) == nc - 1 ? last : zc) + 2;
            if (cost > worst) worst = cost;
        }
        // the resident CTAs share the SMs: a wave with fewer CTAs than slots
        // runs each faster, roughly as slots/grid while memory is the limit
        const double cost = (double)worst * (grid < slots ? (double)slots / (double)grid : 1.0);
        if (best_cost < 0 || cost < best_cost) { best_cost = cost; best_zc = zc; best_grid = grid; }
    }
    *zc_out = (int)best_zc;
    return (int)best_grid;
}

// The z split of a launch choice: chunks of zc, the top `tail` planes
// (rounded so that the chunks below are whole) in chunks of zc2; zc2 = 0 or
// tail = 0 cuts uniformly.
static ZSplit zsplit(const Geom &g, const StepTune &t) {
    ZSplit s;
    s.zc = t.zc < 1 ? 1 : (t.zc > g.nz ? g.nz : t.zc);
    const bool two = t.zc2 > 0 && t.tail > 0 && t.zc2 < s.zc;
    s.zc2 = two ? t.zc2 : s.zc;
    const int below = two ? (t.tail < g.nz ? g.nz - t.tail : 0) : g.nz;
    s.n1 = below / s.zc;
    return s;
}

template <typename T>
Tiles tiles_of(const Geom &g, int tile) {
    int tx = 0, ty = 0;
    step_tile<T>(&tx, &ty, tile);
    Tiles t;
    t.ntx = (g.nx + tx - 1) / tx;
    t.nty = (g.ny + ty - 1) / ty;
    t.nfx = g.nx / tx;
    t.nfy = g.ny / ty;
    return t;
}

template <typename T>
int64_t tma_items(const Geom &g, const StepTune &t) {
    const ZSplit s = zsplit(g, t);
    const int64_t chunks = s.n1 + (g.nz - s.n1 * s.zc + s.zc2 - 1) / s.zc2;
    const Tiles tl = tiles_of<T>(g, t.tile);
    return (int64_t)tl.ntx * tl.nty * chunks;
}

template <typename T>
int tma_grid_for(const Geom &g, int num_sms, const StepTune &t) {
    const int occ = step_occupancy<T, false>(t.tile);
    if (occ < 1) return -1;
    const int64_t items = tma_items<T>(g, t);
    const int64_t slots = (int64_t)occ * num_sms;
    if (items > ((int64_t)1 << 29)) return -1;
    return (int)(items < slots ? items : slots);
}

// A launch of the step; with `pdl` the launch allows programmatic dependent
// launch (see the kernel's griddepcontrol use).
template <typename... KArgs, typename... Args>
static void launch_step_ex(bool pdl, void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t s,
                           Args... args) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    (void)cudaLaunchKernelEx(&cfg, kern, args...);
}

// One launch of the single-domain step over the items of one tile set.
template <typename T, int R, int SET, int TILE>
static void launch_r(const Geom &g, const Coef<T> &k, const CUtensorMap *maps, Fields<T> out, bool c_only, bool eqA,
                     double *partials, const StepTune &tune, int items, int *err, unsigned long long limit_ns,
                     int inject_stall, int *sched, int second, cudaStream_t s) {
    using G = TmaGeo<T, TILE>;
    const size_t sh = tma_smem_bytes<T, TILE>();
    const bool st = partials != nullptr;
    const CoefV<T> kv = make_coefv(k);
    const DomainDesc *no_table = nullptr;
    const ZSplit zs = zsplit(g, tune);
    const Tiles t = tiles_of<T>(g, TILE);
    const int grid = items < tune.grid ? items : tune.grid;
#define PPF_LAUNCH(ST, CO, EQ)                                                                                        \
    launch_step_ex(tune.pdl != 0, step_tma_kernel<T, ST, CO, EQ, R, false, SET, TILE>, grid, G::NT, sh, s, maps[0],   \
                   maps[1], maps[2], g, k, kv, out, t, zs, partials, err, limit_ns, inject_stall, no_table, 0, items,   \
                   0, tune.sched ? sched : nullptr, second)
    if (eqA) {
        if (!c_only) { if (st) PPF_LAUNCH(true, false, true); else PPF_LAUNCH(false, false, true); }
        else { if (st) PPF_LAUNCH(true, true, true); else PPF_LAUNCH(false, true, true); }
    } else {
        if (!c_only) { if (st) PPF_LAUNCH(true, false, false); else PPF_LAUNCH(false, false, false); }
        else { if (st) PPF_LAUNCH(true, true, false); else PPF_LAUNCH(false, true, false); }
    }
#undef PPF_LAUNCH
}

template <typename T, int R, int TILE>
static void launch_sets(const Geom &g, const Coef<T> &k, const CUtensorMap *maps, Fields<T> out, bool c_only,
                        bool eqA, double *partials, const StepTune &tune, int *err, unsigned long long limit_ns,
                        int inject_stall, int *sched, cudaStream_t s) {
    const Tiles t = tiles_of<T>(g, TILE);
    const int64_t chunks = tma_items<T>(g, tune) / ((int64_t)t.ntx * t.nty);
    const int na = (int)(chunks * t.ntx * t.nty);
    if (g.total > ((int64_t)1 << 32)) {        // 64-bit offsets: one launch over every tile
        launch_r<T, 1, SET_WIDE, TILE>(g, k, maps, out, c_only, eqA, partials, tune, na, err, limit_ns, inject_stall,
                                       sched, 0, s);
        return;
    }
    const int nw = (int)(chunks * tiles_in_set(t, SET_WHOLE)), ne = (int)(chunks * tiles_in_set(t, SET_EDGE));
    if (ne == 0) {                             // every tile inside the domain
        launch_r<T, R, SET_WHOLE, TILE>(g, k, maps, out, c_only, eqA, partials, tune, nw, err, limit_ns, inject_stall,
                                        sched, 0, s);
        return;
    }
    if (!tune.split || nw == 0) {              // one launch over every tile
        launch_r<T, 1, SET_ALL, TILE>(g, k, maps, out, c_only, eqA, partials, tune, na, err, limit_ns, inject_stall,
                                      sched, 0, s);
        return;
    }
    // the whole tiles, then the edge tiles (their increment sums follow the
    // whole tiles' in `partials`; their own scheduler pair, since the two
    // launches overlap)
    launch_r<T, R, SET_WHOLE, TILE>(g, k, maps, out, c_only, eqA, partials, tune, nw, err, limit_ns, inject_stall,
                                    sched, 0, s);
    launch_r<T, 1, SET_EDGE, TILE>(g, k, maps, out, c_only, eqA, partials ? partials + 3 * (int64_t)nw : nullptr, tune,
                                   ne, err, limit_ns, 0, sched ? sched + 2 : nullptr, 1, s);
}

template <typename T, int TILE>
static void launch_tile(const Geom &g, const Coef<T> &k, const CUtensorMap *maps, Fields<T> out, bool c_only,
                        bool eqA, double *partials, const StepTune &tune, int *err, unsigned long long limit_ns,
                        int inject_stall, int *sched, cudaStream_t s) {
    if (tune.roll == 1)
        launch_sets<T, 1, TILE>(g, k, maps, out, c_only, eqA, partials, tune, err, limit_ns, inject_stall, sched, s);
    else
        launch_sets<T, 3, TILE>(g, k, maps, out, c_only, eqA, partials, tune, err, limit_ns, inject_stall, sched, s);
}

template <typename T>
cudaError_t launch_step_tma(const Geom &g, const Coef<T> &k, const CUtensorMap *maps, Fields<T> out, bool c_only,
                            bool eqA, double *partials, const StepTune &tune, int *err, unsigned long long limit_ns,
                            int inject_stall, int *sched, cudaStream_t s) {
    if constexpr (kTileShapes<T> > 1)
        if (tune.tile == 1) {
            launch_tile<T, 1>(g, k, maps, out, c_only, eqA, partials, tune, err, limit_ns, inject_stall, sched, s);
            return cudaGetLastError();
        }
    launch_tile<T, 0>(g, k, maps, out, c_only, eqA, partials, tune, err, limit_ns, inject_stall, sched, s);
    return cudaGetLastError();
}

template <typename T, int R, int SET, int TILE>
static void launch_multi_r(const DomainDesc *table, int ndom, int items, const Coef<T> &k, bool c_only, bool eqA,
                           int parity, double *partials, int grid, int *err, unsigned long long limit_ns,
                           int *sched, bool pdl, int second, cudaStream_t s) {
    using G = TmaGeo<T, TILE>;
    const size_t sh = tma_smem_bytes<T, TILE>();
    const bool st = partials != nullptr;
    CUtensorMap none;
    memset(&none, 0, sizeof none);
    Geom g0;
    memset(&g0, 0, sizeof g0);
    const Fields<T> o0 = {nullptr, nullptr, nullptr};
    const CoefV<T> kv = make_coefv(k);
    const ZSplit z1 = {1, 1, 1};
    const Tiles t0 = {1, 1, 1, 1};
    if (items < grid) grid = items;
#define PPF_LAUNCH(ST, CO, EQ)                                                                                       \
    launch_step_ex(pdl, step_tma_kernel<T, ST, CO, EQ, R, true, SET, TILE>, grid, G::NT, sh, s, none, none, none, g0, \
                   k, kv, o0, t0, z1, partials, err, limit_ns, 0, table, ndom, items, parity, sched, second)
    if (eqA) {
        if (!c_only) { if (st) PPF_LAUNCH(true, false, true); else PPF_LAUNCH(false, false, true); }
        else { if (st) PPF_LAUNCH(true, true, true); else PPF_LAUNCH(false, true, true); }
    } else {
        if (!c_only) { if (st) PPF_LAUNCH(true, false, false); else PPF_LAUNCH(false, false, false); }
        else { if (st) PPF_LAUNCH(true, true, false); else PPF_LAUNCH(false, true, false); }
    }
#undef PPF_LAUNCH
}

template <typename T, int TILE>
static void launch_multi_tile(const DomainDesc *table, int ndom, const int *items, const Coef<T> &k, bool c_only,
                              bool eqA, int parity, double *partials, int grid, int roll, bool pdl, bool split,
                              int *err, unsigned long long limit_ns, int *sched, cudaStream_t s) {
    const int nw = items[1], ne = items[0], na = items[2];
    if (ne == 0) {                             // every tile of every domain inside its domain
        if (roll == 1)
            launch_multi_r<T, 1, SET_WHOLE, TILE>(table, ndom, nw, k, c_only, eqA, parity, partials, grid, err, limit_ns,
                                                  sched, pdl, 0, s);
        else
            launch_multi_r<T, 3, SET_WHOLE, TILE>(table, ndom, nw, k, c_only, eqA, parity, partials, grid, err, limit_ns,
                                                  sched, pdl, 0, s);
        return;
    }
    if (!split || nw == 0) {                   // one launch over every tile
        launch_multi_r<T, 1, SET_ALL, TILE>(table, ndom, na, k, c_only, eqA, parity, partials, grid, err, limit_ns, sched,
                                            pdl, 0, s);
        return;
    }
    // the whole tiles of every domain, then the edge tiles (their increment
    // sums follow the whole tiles' in `partials`; their own scheduler pair,
    // since the two launches overlap)
    if (roll == 1)
        launch_multi_r<T, 1, SET_WHOLE, TILE>(table, ndom, nw, k, c_only, eqA, parity, partials, grid, err, limit_ns,
                                              sched, pdl, 0, s);
    else
        launch_multi_r<T, 3, SET_WHOLE, TILE>(table, ndom, nw, k, c_only, eqA, parity, partials, grid, err, limit_ns,
                                              sched, pdl, 0, s);
    launch_multi_r<T, 1, SET_EDGE, TILE>(table, ndom, ne, k, c_only, eqA, parity,
                                         partials ? partials + 3 * (int64_t)nw : nullptr, grid, err, limit_ns,
                                         sched ? sched + 2 : nullptr, pdl, 1, s);
}

template <typename T>
cudaError_t launch_step_multi(const DomainDesc *table, int ndom, const int *items, const Coef<T> &k, bool c_only,
                              bool eqA, int parity, double *partials, int grid, int roll, bool pdl, bool split,
                              int tile, int *err, unsigned long long limit_ns, int *sched, cudaStream_t s) {
    if constexpr (kTileShapes<T> > 1)
        if (tile == 1) {
            launch_multi_tile<T, 1>(table, ndom, items, k, c_only, eqA, parity, partials, grid, roll, pdl, split, err,
                                    limit_ns, sched, s);
            return cudaGetLastError();
        }
    launch_multi_tile<T, 0>(table, ndom, items, k, c_only, eqA, parity, partials, grid, roll, pdl, split, err, limit_ns,
                            sched, s);
    return cudaGetLastError();
}

template <typename T>
int tma_grid_items(int64_t items, int num_sms, int tile) {
    const int occ = step_occupancy<T, true>(tile);
    if (occ < 1) return -1;
    const int64_t slots = (int64_t)occ * num_sms;
    return (int)(items < slots ? items : slots);
}

}  // namespace ppf
