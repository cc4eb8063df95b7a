// ppf_surrogate.cu -- the learned time-stepping surrogate (a 3-D
// convolutional network that advances an FP32 state by k explicit steps in
// one call), its training on the device, and the FP64 solute-mass
// projection.  No counterpart in the reference: the reference only has
// the explicit step (phasefield.c:301-476) that this network stands in for
// and that trains it, corrects it and measures its error.
//
// Network: six 3x3x3 convolutions, 16 -> W -> W -> W -> W -> W -> 16
// channels (W = 16 or 32), SiLU after the first five, residual output:
//   state(t + k dt) = state(t) + out_scale * net(features(state(t)))
// for the three fields (etaS, etaL, c); output channels 3..15 and input
// channels 5..15 are zero padding that keeps every GEMM K and N a multiple
// of 16.  Input features: etaS, etaL, (c - c_eq(h)) * in_scale_c with
// h = etaS^2 / (etaS^2 + etaL^2) (the reference's interpolation,
// phasefield.c:331) and c_eq(h) = h c_solid + (1-h) c_liquid, so the
// composition enters as its (small) departure from local equilibrium,
// which BF16 represents to 2^-8 relative; then 256 (etaS - bf16(etaS)) and
// 256 (etaL - bf16(etaL)), the part of each phase field BF16 drops.
//
// After every call the solute mass sum(c) is projected back, in FP64, to
// its value before the call: the deficit is spread over the cells as whole
// units of 2^-24 (one FP32 ulp on [0.5, 1)) by a Bresenham rule, so the
// FP32 sum lands on the target to within about one ulp; a second pass
// removes what rounding at other binades left.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ppf.h"
#include "ppf_ctx.h"
#include "ppf_internal.h"
#include "ppf_nn.h"

using namespace ppf;
using namespace ppf::nn;

namespace {

constexpr int kLayers = 6;
constexpr int kNT = 256;

int serr(int code, const char *fmt, ...) {
    char buf[400];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return set_last_error(code, buf);
}

#define SCU(x)                                                                                   \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) return serr(PPF_ECUDA, "%s: %s", #x, cudaGetErrorString(e_));     \
    } while (0)

__device__ __forceinline__ int face_images(int x, int n, int bc, int (&o)[3]) {
    int k = 0;
    o[k++] = x;
    if (x == 0) o[k++] = bc == 0 ? n : -1;
    if (x == n - 1) o[k++] = bc == 0 ? -1 : n;
    return k;
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// the halo image of interior coordinate x, or kNone (periodic: x=0 -> n,
// x=n-1 -> -1; no-flux: x=0 -> -1, x=n-1 -> n)
constexpr int kNone = -0x40000000;
__device__ __forceinline__ int image_of(int x, int n, int bc) {
    return x == 0 ? (bc == 0 ? n : -1) : x == n - 1 ? (bc == 0 ? -1 : n) : kNone;
}

__device__ __forceinline__ void block_sum_to(double s, double *out) {
    __shared__ double red[kNT / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < kNT / 32; ++w) t += red[w];
        *out = t;
    }
}

// state (FP32, stencil layout) -> first channel plane of the 16-channel
// BF16 features (etaS, etaL, composition feature; channels 8..15 live in
// the second plane, zero from allocation and never written), with every
// halo image; also the per-CTA FP64 sum of c (the mass before the call).
// One block per x row (grid-stride over rows).
__global__ void __launch_bounds__(kNT) features_kernel(Geom sg, Fields<const float> s, NNGeom g, uint16_t *act,
                                                       float cS, float cL, float kc, double *mass_part) {
    double m = 0;
    const int nrows = g.ny * g.nz;
    for (int rr = blockIdx.x; rr < nrows; rr += gridDim.x) {
        const int y = rr % g.ny, z = rr / g.ny;
        const int ay = image_of(y, g.ny, g.bc), az = image_of(z, g.nz, g.bc);
        const int64_t a0 = sg.at(0, y, z);
        for (int x = threadIdx.x; x < g.nx; x += kNT) {
            const float eS = s.eS[a0 + x], eL = s.eL[a0 + x], c = s.c[a0 + x];
            m += (double)c;
            const float s2 = eS * eS, l2 = eL * eL;
            const float h = s2 / fmaxf(s2 + l2, 1e-30f);
            const float f2 = (c - (cL + (cS - cL) * h)) * kc;
            // what BF16 drops of etaS and etaL, scaled into range: with
            // channels 0-1 the network sees both fields to ~16 bits
            const uint32_t hi = pack2(eS, eL);
            const float rS = (eS - __uint_as_float(hi << 16)) * 256.0f;
            const float rL = (eL - __uint_as_float(hi & 0xFFFF0000u)) * 256.0f;
            const uint4 v = make_uint4(hi, pack2(f2, rS), pack2(rL, 0.f), 0u);
            const int ax = image_of(x, g.nx, g.bc);
            for (int k = 0; k < 8; ++k) {
                const int xx = (k & 1) ? ax : x, yy = (k & 2) ? ay : y, zz = (k & 4) ? az : z;
                if (xx == kNone || yy == kNone || zz == kNone) continue;
                *reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(act) + g.p(xx, yy, zz) * 16) = v;
            }
        }
    }
    block_sum_to(m, mass_part + blockIdx.x);
}

// FP64 per-CTA sums of c over the interior, one block per x row
__global__ void __launch_bounds__(kNT) csum_kernel(Geom sg, const float *c, double *partials) {
    double m = 0;
    const int nrows = sg.ny * sg.nz;
    for (int rr = blockIdx.x; rr < nrows; rr += gridDim.x) {
        const float *row = c + sg.at(0, rr % sg.ny, rr / sg.ny);
        for (int x = threadIdx.x; x < sg.nx; x += kNT) m += (double)row[x];
    }
    block_sum_to(m, partials + blockIdx.x);
}

// The projection moves sum(c) by R = round((target - sum) / 2^-24) units of
// 2^-24: every cell by `base` units and `rem` cells by one more, where
// base = floor(R / n), rem = R - base n in [0, n); the cells taking the
// extra unit are i_k = ceil((k+1) n / rem) - 1, k < rem (evenly spread: the
// cells where floor((i+1) rem / n) steps up).
struct MassPlan {
    double target, sum;
    long long base, rem;
};

__global__ void plan_kernel(MassPlan *mp, long long n) {
    const double d = (mp->target - mp->sum) * 16777216.0;   // in units of 2^-24
    long long R = 0;
    if (fabs(d) < 4.0e18) R = llrint(d);                     // non-finite or absurd: leave c alone
    long long base = R / n, rem = R % n;
    if (rem < 0) {
        rem += n;
        base -= 1;
    }
    mp->base = base;
    mp->rem = rem;
}

__device__ __forceinline__ void put_c(const Geom &sg, float *c, int x, int y, int z, double add) {
    const int64_t a = sg.at(x, y, z);
    const float v = (float)((double)c[a] + add);
    c[a] = v;
    const int ax = image_of(x, sg.nx, sg.bc), ay = image_of(y, sg.ny, sg.bc), az = image_of(z, sg.nz, sg.bc);
    if (ax != kNone) c[sg.at(ax, y, z)] = v;
    if (ay != kNone) c[sg.at(x, ay, z)] = v;
    if (az != kNone) c[sg.at(x, y, az)] = v;
}

__global__ void __launch_bounds__(kNT) dense_kernel(Geom sg, float *c, const MassPlan *mp) {
    const long long base = mp->base;
    if (base == 0) return;
    const double add = (double)base * 5.9604644775390625e-08;
    const int nrows = sg.ny * sg.nz;
    for (int rr = blockIdx.x; rr < nrows; rr += gridDim.x) {
        const int y = rr % sg.ny, z = rr / sg.ny;
        for (int x = threadIdx.x; x < sg.nx; x += kNT) put_c(sg, c, x, y, z, add);
    }
}

__global__ void __launch_bounds__(kNT) sparse_kernel(Geom sg, float *c, const MassPlan *mp, long long n) {
    const long long rem = mp->rem;
    for (long long k = blockIdx.x * (long long)kNT + threadIdx.x; k < rem; k += (long long)gridDim.x * kNT) {
        const long long i = ((k + 1) * n + rem - 1) / rem - 1;
        const int x = (int)(i % sg.nx), y = (int)((i / sg.nx) % sg.ny), z = (int)(i / ((long long)sg.nx * sg.ny));
        put_c(sg, c, x, y, z, 5.9604644775390625e-08);
    }
}

// out[i] = sum_b part[b * stride + i] (fixed order, FP64 accumulation)
__global__ void __launch_bounds__(kNT) reduce_kernel(const float *part, int nb, int stride, int n, float *out) {
    for (int i = blockIdx.x * kNT + threadIdx.x; i < n; i += gridDim.x * kNT) {
        double s = 0;
        for (int b = 0; b < nb; ++b) s += (double)part[(int64_t)b * stride + i];
        out[i] = (float)s;
    }
}

__global__ void loss_kernel(const float *part, int nb, int stride, int idx, double *out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0;
        for (int b = 0; b < nb; ++b) s += (double)part[(int64_t)b * stride + idx];
        *out = s;
    }
}

__global__ void __launch_bounds__(kNT) adam_kernel(int64_t n, float *p, const float *g, float *m, float *v, float lr,
                                                   float b1, float b2, float eps, float c1, float c2) {
    for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNT) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// W[27][co][ci] (FP32, tap = 9 dz + 3 dy + dx over 0..2) -> the BF16
// B-operand images of the convolution kernel, [dz][dx][ci/8][dy][co][8]
// (one MMA's N = 3 co rows are the three dy taps), forward and for the
// input-gradient convolution (taps reversed, ci and co swapped).
__global__ void __launch_bounds__(kNT) pack_kernel(const float *W, int ci, int co, uint16_t *wf, uint16_t *wb) {
    const int n = 27 * ci * co;
    for (int i = blockIdx.x * kNT + threadIdx.x; i < n; i += gridDim.x * kNT) {
        const int c_in = i % ci, c_out = (i / ci) % co, tap = i / (ci * co);
        const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
        const __nv_bfloat16 h = __float2bfloat16_rn(W[i]);
        const uint16_t u = *reinterpret_cast<const uint16_t *>(&h);
        wf[((((int64_t)(dz * 3 + dx) * (ci / 8) + c_in / 8) * 3 + dy) * co + c_out) * 8 + (c_in & 7)] = u;
        const int rz = 2 - dz, ry = 2 - dy, rx = 2 - dx;
        wb[((((int64_t)(rz * 3 + rx) * (co / 8) + c_out / 8) * 3 + ry) * ci + c_in) * 8 + (c_out & 7)] = u;
    }
}

}  // namespace

struct ppf_surrogate {
    ppf_surrogate_config cfg;
    int W = 0;
    int dev = 0, num_sms = 0;
    int ci[kLayers], co[kLayers];
    int64_t woff[kLayers], boff[kLayers], nparams = 0;
    float *params = nullptr, *grads = nullptr, *mom1 = nullptr, *mom2 = nullptr;
    uint16_t *wf[kLayers] = {}, *wb[kLayers] = {};
    int64_t adam_t = 0;
    // workspace for one domain shape
    int wz = 0, wy = 0, wx = 0, wbc = -1;
    NNGeom g{};
    uint16_t *feat = nullptr, *act[5] = {}, *zp[5] = {}, *g16 = nullptr, *gw[2] = {};
    bool train_ready = false;    // g16, gw, zp allocated for the current shape
    float *wpart = nullptr, *bpart = nullptr;
    double *mpart = nullptr;     // per-CTA sums of c after a call (output layer)
    double *dscal = nullptr;     // [0] loss
    float *scratch = nullptr;    // predictions: zero state + output state
    double *stage = nullptr;
    size_t scratch_elems = 0;
    int conv_grid[2][2] = {}, wgrad_grid = 0;
    int inject = 0;              // test hook: the next convolution's wait runs out
};

namespace {

void free_train(ppf_surrogate *s) {
    for (auto &p : s->zp) cudaFree(p), p = nullptr;
    for (auto &p : s->gw) cudaFree(p), p = nullptr;
    cudaFree(s->g16);
    s->g16 = nullptr;
    s->train_ready = false;
}

// buffers may still be in use by work queued on any context's stream: the
// whole device is synchronised before anything is freed
void free_ws(ppf_surrogate *s) {
    cudaDeviceSynchronize();
    free_train(s);
    cudaFree(s->feat);
    for (auto &p : s->act) cudaFree(p), p = nullptr;
    cudaFree(s->scratch);
    cudaFree(s->stage);
    s->feat = nullptr;
    s->scratch = nullptr;
    s->stage = nullptr;
    s->scratch_elems = 0;
    s->wz = s->wy = s->wx = 0;
    s->wbc = -1;
}

int alloc_zero(void **p, size_t bytes, cudaStream_t st) {
    SCU(cudaMalloc(p, bytes));
    SCU(cudaMemsetAsync(*p, 0, bytes, st));
    return PPF_OK;
}

int check_ctx(ppf_ctx *c) {
    if (!c) return serr(PPF_EINVAL, "null context");
    if (c->prec != PPF_F32) return serr(PPF_EINVAL, "the surrogate runs on FP32 contexts");
    if (c->nx % kTileX != 0) return serr(PPF_EINVAL, "the surrogate needs an x edge that is a multiple of %d", kTileX);
    if (c->ny < 2 || c->nz < 2) return serr(PPF_EINVAL, "the surrogate needs y and z edges of at least 2");
    if (!c->uploaded) return serr(PPF_ESTATE, "no state uploaded");
    return PPF_OK;
}

int ensure_ws(ppf_surrogate *s, ppf_ctx *c, bool train) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->dev != s->dev) return serr(PPF_EINVAL, "context and surrogate on different devices");
    if (s->wz != c->nz || s->wy != c->ny || s->wx != c->nx || s->wbc != c->bc) {
        free_ws(s);
        s->g = make_nngeom(c->nz, c->ny, c->nx, c->bc);
        if ((rc = alloc_zero((void **)&s->feat, act_bytes(s->g, 16), c->stream))) return rc;
        for (auto &p : s->act)
            if ((rc = alloc_zero((void **)&p, act_bytes(s->g, s->W), c->stream))) return rc;
        s->wz = c->nz;
        s->wy = c->ny;
        s->wx = c->nx;
        s->wbc = c->bc;
    }
    if (train && !s->train_ready) {
        // all or nothing: a failure leaves no half-allocated training set
        rc = alloc_zero((void **)&s->g16, act_bytes(s->g, 16), c->stream);
        for (auto &p : s->gw)
            if (!rc) rc = alloc_zero((void **)&p, act_bytes(s->g, s->W), c->stream);
        for (auto &p : s->zp)
            if (!rc) rc = alloc_zero((void **)&p, act_bytes(s->g, s->W), c->stream);
        if (rc) {
            cudaDeviceSynchronize();
            free_train(s);
            return rc;
        }
        s->train_ready = true;
    }
    return PPF_OK;
}

int pick_yc(const NNGeom &g, int grid) {
    const int64_t nxt = g.nx / kTileX;
    int yc = 32;
    while (yc > 4 && (int64_t)g.nz * ((g.ny + yc - 1) / yc) * nxt < 8LL * grid) yc /= 2;
    return yc;
}

Fields<const float> cur_fields(ppf_ctx *c) {
    return {(const float *)c->fld[c->cur_eta][0], (const float *)c->fld[c->cur_eta][1],
            (const float *)c->fld[c->cur_c][2]};
}

ConvArgs conv_args(ppf_surrogate *s, ppf_ctx *c, int layer, const uint16_t *x, const uint16_t *wimg) {
    ConvArgs a{};
    a.g = s->g;
    a.x = x;
    a.wimg = wimg;
    a.bias = s->params + s->boff[layer];
    a.sg = c->g;
    const int grid = s->conv_grid[s->ci[layer] == 32][s->co[layer] == 32];
    a.yc = pick_yc(s->g, grid);
    a.items = s->g.nz * ((s->g.ny + a.yc - 1) / a.yc) * (s->g.nx / kTileX);
    a.err = c->derr;
    a.limit_ns = c->wait_limit_ns;
    for (int k = 0; k < 3; ++k) {
        a.oscale[k] = (float)s->cfg.out_scale[k];
        a.lw[k] = (float)(s->cfg.loss_weight[k] / (3.0 * (double)c->nz * c->ny * c->nx));
    }
    return a;
}

int run_conv(ppf_surrogate *s, ppf_ctx *c, int ci, int co, int epi, const ConvArgs &a) {
    const int grid = s->conv_grid[ci == 32][co == 32];
    ConvArgs b = a;
    b.inject_stall = s->inject;
    s->inject = 0;
    SCU(launch_conv(ci, co, epi, b, grid, c->stream));
    return PPF_OK;
}

MassPlan *plan_of(ppf_ctx *c) { return reinterpret_cast<MassPlan *>(c->dres + 16); }

int row_blocks(const ppf_ctx *c) { return (int)std::min<int64_t>((int64_t)c->ny * c->nz, 8LL * c->num_sms); }

// features of the current state; the mass before the call goes to the plan's target
int features(ppf_surrogate *s, ppf_ctx *c) {
    const int nb = row_blocks(c);
    int rc = ensure_partials(c, nb);
    if (rc) return rc;
    features_kernel<<<nb, kNT, 0, c->stream>>>(c->g, cur_fields(c), s->g, s->feat, (float)s->cfg.c_solid,
                                               (float)s->cfg.c_liquid, (float)s->cfg.in_scale_c, c->partials);
    SCU(cudaGetLastError());
    SCU(launch_final_sum(c->partials, nb, 1, 1, &plan_of(c)->target, c->stream));
    return PPF_OK;
}

// features + hidden layers 0..4 (train: keep pre-activations)
int forward_hidden(ppf_surrogate *s, ppf_ctx *c, bool train) {
    int rc = features(s, c);
    if (rc) return rc;
    for (int l = 0; l < 5; ++l) {
        ConvArgs a = conv_args(s, c, l, l == 0 ? s->feat : s->act[l - 1], s->wf[l]);
        a.out = s->act[l];
        a.zout = train ? s->zp[l] : nullptr;
        if ((rc = run_conv(s, c, s->ci[l], s->co[l], train ? EPI_ACT_TRAIN : EPI_ACT, a))) return rc;
    }
    return PPF_OK;
}

int reduce_into(ppf_surrogate *s, ppf_ctx *c, const float *part, int nb, int stride, int n, float *out) {
    const int blocks = std::max(1, std::min((n + kNT - 1) / kNT, 4 * s->num_sms));
    reduce_kernel<<<blocks, kNT, 0, c->stream>>>(part, nb, stride, n, out);
    SCU(cudaGetLastError());
    return PPF_OK;
}

int wgrad(ppf_surrogate *s, ppf_ctx *c, int layer, const uint16_t *x, const uint16_t *dz) {
    WgradArgs w{};
    w.g = s->g;
    w.x = x;
    w.dz = dz;
    w.partials = s->wpart;
    w.ntiles = s->g.nz * s->g.ny * (s->g.nx / kTileX);
    w.err = c->derr;
    w.limit_ns = c->wait_limit_ns;
    SCU(launch_wgrad(s->ci[layer], s->co[layer], w, s->wgrad_grid, c->stream));
    const int n = 27 * s->ci[layer] * s->co[layer];
    return reduce_into(s, c, s->wpart, s->wgrad_grid, n, n, s->grads + s->woff[layer]);
}

// loss and gradients of all parameters for one (input, target) pair
int loss_grad(ppf_surrogate *s, ppf_ctx *in, ppf_ctx *tg) {
    int rc = ensure_ws(s, in, true);
    if (rc) return rc;
    if ((rc = check_ctx(tg))) return rc;
    if (tg->nz != in->nz || tg->ny != in->ny || tg->nx != in->nx)
        return serr(PPF_EINVAL, "input and target shapes differ");
    if (in->bc != PPF_BC_PERIODIC) return serr(PPF_EINVAL, "training runs on periodic domains");
    if (tg->stream != in->stream) SCU(cudaStreamSynchronize(tg->stream));
    if ((rc = forward_hidden(s, in, true))) return rc;
    // output layer + loss: dZ5 -> g16
    {
        ConvArgs a = conv_args(s, in, 5, s->act[4], s->wf[5]);
        a.out = s->g16;
        a.partials = s->bpart;
        a.s0 = cur_fields(in);
        Fields<const float> t = cur_fields(tg);
        a.s1 = {const_cast<float *>(t.eS), const_cast<float *>(t.eL), const_cast<float *>(t.c)};
        if ((rc = run_conv(s, in, s->ci[5], 16, EPI_LOSS, a))) return rc;
        const int grid = s->conv_grid[s->ci[5] == 32][0];
        if ((rc = reduce_into(s, in, s->bpart, grid, 17, 16, s->grads + s->boff[5]))) return rc;
        loss_kernel<<<1, 32, 0, in->stream>>>(s->bpart, grid, 17, 16, s->dscal);
        SCU(cudaGetLastError());
    }
    if ((rc = wgrad(s, in, 5, s->act[4], s->g16))) return rc;
    const uint16_t *cur = s->g16;
    for (int l = 5; l >= 1; --l) {
        // dZ_{l-1} = conv^T(dZ_l, W_l) * silu'(z_{l-1}); bias gradient of layer l-1
        uint16_t *out = s->gw[(5 - l) % 2];
        ConvArgs a = conv_args(s, in, l, cur, s->wb[l]);
        a.out = out;
        a.zlow = s->zp[l - 1];
        a.partials = s->bpart;
        const int ci = s->co[l], co = s->ci[l];
        if ((rc = run_conv(s, in, ci, co, EPI_DGRAD, a))) return rc;
        if ((rc = reduce_into(s, in, s->bpart, s->conv_grid[ci == 32][co == 32], co + 1, co,
                              s->grads + s->boff[l - 1])))
            return rc;
        if ((rc = wgrad(s, in, l - 1, l - 1 == 0 ? s->feat : s->act[l - 2], out))) return rc;
        cur = out;
    }
    return PPF_OK;
}

int pack_all(ppf_surrogate *s, cudaStream_t st) {
    for (int l = 0; l < kLayers; ++l) {
        const int n = 27 * s->ci[l] * s->co[l];
        pack_kernel<<<(n + kNT - 1) / kNT, kNT, 0, st>>>(s->params + s->woff[l], s->ci[l], s->co[l], s->wf[l],
                                                        s->wb[l]);
        SCU(cudaGetLastError());
    }
    return PPF_OK;
}

int mass_sum(ppf_ctx *c, double *out) {
    const int nb = row_blocks(c);
    int rc = ensure_partials(c, nb);
    if (rc) return rc;
    csum_kernel<<<nb, kNT, 0, c->stream>>>(c->g, (const float *)c->fld[c->cur_c][2], c->partials);
    SCU(cudaGetLastError());
    SCU(launch_final_sum(c->partials, nb, 1, 1, out, c->stream));
    return PPF_OK;
}

// move sum(c) onto the plan's target; `have_sum`: the plan's sum is already
// that of the current state
int project(ppf_ctx *c, bool have_sum) {
    MassPlan *mp = plan_of(c);
    const long long n = (long long)c->nz * c->ny * c->nx;
    float *cc = (float *)c->fld[c->cur_c][2];
    for (int pass = 0; pass < 2; ++pass) {
        if (pass > 0 || !have_sum) {
            int rc = mass_sum(c, &mp->sum);
            if (rc) return rc;
        }
        plan_kernel<<<1, 1, 0, c->stream>>>(mp, n);
        dense_kernel<<<row_blocks(c), kNT, 0, c->stream>>>(c->g, cc, mp);
        sparse_kernel<<<4 * c->num_sms, kNT, 0, c->stream>>>(c->g, cc, mp, n);
        SCU(cudaGetLastError());
    }
    return PPF_OK;
}

}  // namespace

// ---------------------------------------------------------------- C-ABI --

extern "C" void ppf_surrogate_config_default(ppf_surrogate_config *cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof *cfg);
    cfg->width = 32;
    cfg->k_steps = 50;
    cfg->c_solid = 0.47603;
    cfg->c_liquid = 0.99903;
    cfg->in_scale_c = 1000.0;
    cfg->out_scale[0] = cfg->out_scale[1] = 1e-2;
    cfg->out_scale[2] = 1e-3;
    cfg->loss_weight[0] = cfg->loss_weight[1] = cfg->loss_weight[2] = 1.0;
}

extern "C" int ppf_surrogate_create(const ppf_surrogate_config *cfg, ppf_surrogate **out) {
    if (!cfg || !out) return serr(PPF_EINVAL, "null argument");
    *out = nullptr;
    if (cfg->width != 16 && cfg->width != 32) return serr(PPF_EINVAL, "width must be 16 or 32");
    if (cfg->k_steps < 1) return serr(PPF_EINVAL, "k_steps must be positive");
    for (int k = 0; k < 3; ++k)
        if (!(cfg->out_scale[k] > 0)) return serr(PPF_EINVAL, "out_scale must be positive");
    ppf_surrogate *s = new ppf_surrogate();
    s->cfg = *cfg;
    s->W = cfg->width;
    if (cudaGetDevice(&s->dev) != cudaSuccess) {
        delete s;
        return serr(PPF_ECUDA, "no CUDA device");
    }
    int optin = 0, major = 0;
    cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, s->dev);
    if (major < 10) {
        delete s;
        return serr(PPF_ECUDA, "the surrogate's kernels need a Blackwell (sm_10x) GPU");
    }
    cudaError_t e = conv_setup(optin);
    if (e != cudaSuccess) {
        delete s;
        return serr(PPF_ECUDA, "convolution set-up failed: %s", cudaGetErrorString(e));
    }
    const int chans[kLayers + 1] = {16, s->W, s->W, s->W, s->W, s->W, 16};
    int64_t off = 0;
    for (int l = 0; l < kLayers; ++l) {
        s->ci[l] = chans[l];
        s->co[l] = chans[l + 1];
        s->woff[l] = off;
        off += 27LL * s->ci[l] * s->co[l];
        s->boff[l] = off;
        off += s->co[l];
    }
    s->nparams = off;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) s->conv_grid[a][b] = conv_ctas_per_sm(a ? 32 : 16, b ? 32 : 16) * s->num_sms;
    s->wgrad_grid = s->num_sms;
    const size_t pb = (size_t)s->nparams * sizeof(float);
    bool ok = cudaMalloc(&s->params, pb) == cudaSuccess && cudaMalloc(&s->grads, pb) == cudaSuccess &&
              cudaMalloc(&s->mom1, pb) == cudaSuccess && cudaMalloc(&s->mom2, pb) == cudaSuccess &&
              cudaMalloc(&s->wpart, (size_t)s->wgrad_grid * 27 * 32 * 32 * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&s->bpart, (size_t)2 * s->num_sms * 33 * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&s->mpart, (size_t)2 * s->num_sms * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&s->dscal, 8 * sizeof(double)) == cudaSuccess;
    for (int l = 0; ok && l < kLayers; ++l)
        ok = cudaMalloc(&s->wf[l], 27 * s->ci[l] * s->co[l] * 2) == cudaSuccess &&
             cudaMalloc(&s->wb[l], 27 * s->ci[l] * s->co[l] * 2) == cudaSuccess;
    if (ok)
        ok = cudaMemset(s->params, 0, pb) == cudaSuccess && cudaMemset(s->grads, 0, pb) == cudaSuccess &&
             cudaMemset(s->mom1, 0, pb) == cudaSuccess && cudaMemset(s->mom2, 0, pb) == cudaSuccess &&
             cudaMemset(s->dscal, 0, 8 * sizeof(double)) == cudaSuccess;
    if (ok) ok = pack_all(s, 0) == PPF_OK && cudaDeviceSynchronize() == cudaSuccess;
    if (!ok) {
        ppf_surrogate_destroy(s);
        return serr(PPF_ENOMEM, "surrogate allocation failed");
    }
    *out = s;
    return PPF_OK;
}

extern "C" int ppf_surrogate_destroy(ppf_surrogate *s) {
    if (!s) return PPF_OK;
    cudaDeviceSynchronize();
    free_ws(s);
    for (int l = 0; l < kLayers; ++l) {
        cudaFree(s->wf[l]);
        cudaFree(s->wb[l]);
    }
    cudaFree(s->params);
    cudaFree(s->grads);
    cudaFree(s->mom1);
    cudaFree(s->mom2);
    cudaFree(s->wpart);
    cudaFree(s->bpart);
    cudaFree(s->mpart);
    cudaFree(s->dscal);
    delete s;
    return PPF_OK;
}

extern "C" int64_t ppf_surrogate_num_params(const ppf_surrogate *s) { return s ? s->nparams : -1; }

extern "C" int ppf_surrogate_get_config(const ppf_surrogate *s, ppf_surrogate_config *cfg) {
    if (!s || !cfg) return serr(PPF_EINVAL, "null argument");
    *cfg = s->cfg;
    return PPF_OK;
}

extern "C" int ppf_surrogate_set_params(ppf_surrogate *s, const float *host, int64_t n) {
    if (!s || !host) return serr(PPF_EINVAL, "null argument");
    if (n != s->nparams) return serr(PPF_EINVAL, "expected %lld parameters", (long long)s->nparams);
    SCU(cudaMemcpy(s->params, host, n * sizeof(float), cudaMemcpyHostToDevice));
    SCU(cudaMemset(s->mom1, 0, n * sizeof(float)));
    SCU(cudaMemset(s->mom2, 0, n * sizeof(float)));
    s->adam_t = 0;
    int rc = pack_all(s, 0);
    if (rc) return rc;
    SCU(cudaDeviceSynchronize());
    return PPF_OK;
}

extern "C" int ppf_surrogate_get_params(ppf_surrogate *s, float *host, int64_t n) {
    if (!s || !host) return serr(PPF_EINVAL, "null argument");
    if (n != s->nparams) return serr(PPF_EINVAL, "expected %lld parameters", (long long)s->nparams);
    SCU(cudaDeviceSynchronize());
    SCU(cudaMemcpy(host, s->params, n * sizeof(float), cudaMemcpyDeviceToHost));
    return PPF_OK;
}

extern "C" int ppf_surrogate_loss_grad(ppf_surrogate *s, ppf_ctx *input, ppf_ctx *target, double *loss,
                                       float *grad, int64_t n) {
    if (!s) return serr(PPF_EINVAL, "null surrogate");
    if (grad && n != s->nparams) return serr(PPF_EINVAL, "expected %lld gradient entries", (long long)s->nparams);
    int rc = loss_grad(s, input, target);
    if (rc) return rc;
    double l = 0;
    SCU(cudaMemcpyAsync(&l, s->dscal, sizeof(double), cudaMemcpyDeviceToHost, input->stream));
    if (grad)
        SCU(cudaMemcpyAsync(grad, s->grads, s->nparams * sizeof(float), cudaMemcpyDeviceToHost, input->stream));
    SCU(cudaStreamSynchronize(input->stream));
    if ((rc = check_device_error(input))) return rc;
    if (loss) *loss = l;
    return PPF_OK;
}

extern "C" int ppf_surrogate_train_step(ppf_surrogate *s, ppf_ctx *input, ppf_ctx *target, double lr,
                                        double *loss) {
    if (!s) return serr(PPF_EINVAL, "null surrogate");
    if (!(lr >= 0)) return serr(PPF_EINVAL, "learning rate must be non-negative");
    int rc = loss_grad(s, input, target);
    if (rc) return rc;
    s->adam_t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)s->adam_t), c2 = 1.f - powf(b2, (float)s->adam_t);
    const int nb = (int)std::min<int64_t>((s->nparams + kNT - 1) / kNT, 4LL * s->num_sms);
    adam_kernel<<<nb, kNT, 0, input->stream>>>(s->nparams, s->params, s->grads, s->mom1, s->mom2, (float)lr, b1, b2,
                                               1e-8f, c1, c2);
    SCU(cudaGetLastError());
    if ((rc = pack_all(s, input->stream))) return rc;
    if (loss) {
        SCU(cudaMemcpyAsync(loss, s->dscal, sizeof(double), cudaMemcpyDeviceToHost, input->stream));
        SCU(cudaStreamSynchronize(input->stream));
        return check_device_error(input);
    }
    return PPF_OK;
}

extern "C" int ppf_surrogate_predict(ppf_surrogate *s, ppf_ctx *c, double *out3) {
    if (!s || !out3) return serr(PPF_EINVAL, "null argument");
    int rc = ensure_ws(s, c, false);
    if (rc) return rc;
    const size_t elems = (size_t)c->g.total * 3;
    if (s->scratch_elems != elems) {
        cudaDeviceSynchronize();
        cudaFree(s->scratch);
        cudaFree(s->stage);
        s->scratch = nullptr;
        s->stage = nullptr;
        s->scratch_elems = 0;
        if ((rc = alloc_zero((void **)&s->scratch, 2 * elems * sizeof(float), c->stream))) return rc;
        SCU(cudaMalloc(&s->stage, (size_t)3 * c->nz * c->ny * c->nx * sizeof(double)));
        s->scratch_elems = elems;
    }
    if ((rc = forward_hidden(s, c, false))) return rc;
    const int64_t T = c->g.total;
    float *z0 = s->scratch, *o = s->scratch + elems;
    ConvArgs a = conv_args(s, c, 5, s->act[4], s->wf[5]);
    a.s0 = {z0, z0 + T, z0 + 2 * T};
    a.s1 = {o, o + T, o + 2 * T};
    a.mass_part = s->mpart;
    if ((rc = run_conv(s, c, s->ci[5], 16, EPI_STATE, a))) return rc;
    SCU(launch_unpack<float>(c->g, Fields<const float>{o, o + T, o + 2 * T}, s->stage, c->stream));
    SCU(cudaMemcpyAsync(out3, s->stage, (size_t)3 * c->nz * c->ny * c->nx * sizeof(double), cudaMemcpyDeviceToHost,
                        c->stream));
    SCU(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

extern "C" int ppf_surrogate_advance(ppf_surrogate *s, ppf_ctx *c, int ncalls) {
    if (!s) return serr(PPF_EINVAL, "null surrogate");
    if (ncalls < 0) return serr(PPF_EINVAL, "negative call count");
    int rc = ensure_ws(s, c, false);
    if (rc) return rc;
    for (int k = 0; k < ncalls; ++k) {
        if ((rc = forward_hidden(s, c, false))) return rc;     // features: mass before the call
        const int ie = c->cur_eta, ic = c->cur_c;
        ConvArgs a = conv_args(s, c, 5, s->act[4], s->wf[5]);
        a.s0 = cur_fields(c);
        a.s1 = {(float *)c->fld[1 - ie][0], (float *)c->fld[1 - ie][1], (float *)c->fld[1 - ic][2]};
        a.mass_part = s->mpart;
        if ((rc = run_conv(s, c, s->ci[5], 16, EPI_STATE, a))) return rc;
        SCU(launch_final_sum(s->mpart, s->conv_grid[s->ci[5] == 32][0], 1, 1, &plan_of(c)->sum, c->stream));
        c->cur_eta = 1 - ie;
        c->cur_c = 1 - ic;
        c->steps += s->cfg.k_steps;
        if ((rc = project(c, true))) return rc;
    }
    return PPF_OK;
}

extern "C" int ppf_surrogate_debug_inject(ppf_surrogate *s, int fault) {
    if (!s) return serr(PPF_EINVAL, "null surrogate");
    if (fault != PPF_INJECT_NONE && fault != PPF_INJECT_STALL_WAIT) return serr(PPF_EINVAL, "unknown fault");
    s->inject = fault == PPF_INJECT_STALL_WAIT;
    return PPF_OK;
}

extern "C" int ppf_mass_project(ppf_ctx *c, double target_mass) {
    if (!c) return serr(PPF_EINVAL, "null context");
    if (c->prec != PPF_F32) return serr(PPF_EINVAL, "mass projection applies to FP32 contexts");
    if (!c->uploaded) return serr(PPF_ESTATE, "no state uploaded");
    if (!std::isfinite(target_mass)) return serr(PPF_EINVAL, "target mass must be finite");
    SCU(cudaMemcpyAsync(&plan_of(c)->target, &target_mass, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int rc = project(c, false);
    if (rc) return rc;
    SCU(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

extern "C" int ppf_copy_state(ppf_ctx *dst, ppf_ctx *src) {
    if (!dst || !src) return serr(PPF_EINVAL, "null context");
    if (dst->nz != src->nz || dst->ny != src->ny || dst->nx != src->nx || dst->prec != src->prec ||
        dst->bc != src->bc)
        return serr(PPF_EINVAL, "contexts differ in shape, precision or boundary condition");
    if (!src->uploaded) return serr(PPF_ESTATE, "no state uploaded");
    if (dst == src) return PPF_OK;
    const size_t bytes = (size_t)src->g.total * (src->prec == PPF_F32 ? 4 : 8);
    SCU(cudaStreamSynchronize(src->stream));
    for (int k = 0; k < 3; ++k)
        SCU(cudaMemcpyAsync(dst->fld[0][k], src->fld[k < 2 ? src->cur_eta : src->cur_c][k], bytes,
                            cudaMemcpyDeviceToDevice, dst->stream));
    dst->cur_eta = dst->cur_c = 0;
    dst->uploaded = 1;
    dst->steps = src->steps;
    SCU(cudaStreamSynchronize(dst->stream));
    return PPF_OK;
}
