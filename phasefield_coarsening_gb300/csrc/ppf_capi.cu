// ppf_capi.cu -- the extern "C" boundary declared in include/ppf.h.
//
// A context replaces the reference's global state (phasefield.c:67-70,
// ten ghosted double arrays) with two ping-pong copies of the three
// evolving fields in device memory; hS, mu and M are never stored (the
// fused step recomputes them per plane in shared memory) and the
// increments detaS/detaL/dc are never stored either (only their squared
// sums, phasefield.c:228-238, are kept for the convergence test).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "ppf.h"
#include "ppf_internal.h"
#include "ppf_particles.h"
#include "ppf_step_tma.h"

using namespace ppf;

static thread_local char g_err[512];

// Consecutive steps overlap by programmatic dependent launch unless the
// autotuner finds the plain launch faster: the next step's CTAs are placed
// while this one's last CTAs drain (worth ~12 % per step at 128^3, nothing
// at 256^3, where the step is long against the launch gap).
static constexpr int kStepPdl = 1;

// CTAs take the step's work items from a global counter (in the same
// chunk-major order as the round-robin deal), so that CTAs that run faster
// take more items and the launch's CTAs end closer together.
static constexpr int kStepSched = 1;

// A domain whose x or y edge is not a multiple of the tile runs its whole
// tiles and its edge tiles as two launches, the second in the first one's
// tail, unless the autotuner finds one launch over every tile faster.
static constexpr int kStepSplit = 1;

static int seterr(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

int ppf::set_last_error(int code, const char *msg) { return seterr(code, "%s", msg); }

#define CU(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return seterr(PPF_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

#include "ppf_ctx.h"


extern "C" void ppf_params_default(ppf_params *p) {
    if (!p) return;
    // phasefield.c:76-97
    p->AS = 1e+09;
    p->AL = 1e+09;
    p->CS = -1e+06;
    p->CL = 1.e+07;
    p->cS0 = 0.455;
    p->cL0 = 0.978;
    p->cSeq = 0.999;
    p->cLeq = 0.476;
    p->DL = 1.0e-14;
    p->DS = 0.0;
    p->sigma = 2.0;
    p->gamma = 1.5;
    p->dx = 1;
    p->dt = 0;   // 0.125*dx*dx/DL
    p->l = 0;    // 7*dx
}

extern "C" int ppf_params_derive(const ppf_params *p, ppf_derived *d) {
    if (!p || !d) return seterr(PPF_EINVAL, "null argument");
    if (!(p->dx > 0) || !(p->AS > 0) || !(p->AL > 0) || !(p->DL > 0) || p->DS < 0 || !(p->sigma > 0) ||
        p->cSeq == p->cLeq)
        return seterr(PPF_EINVAL, "invalid parameters (need dx, AS, AL, DL, sigma > 0, DS >= 0, cSeq != cLeq)");
    d->ML = p->DL / p->AL;                              // :85
    d->MS = p->DS / p->AS;
    d->h2 = 1.0 / (p->dx * p->dx);                      // :91
    d->dt = p->dt > 0 ? p->dt : 0.125 * p->dx * p->dx / p->DL;   // :92
    d->l = p->l > 0 ? p->l : 7.0 * p->dx;              // :94
    d->m = 6.0 * p->sigma / d->l;                       // :95
    d->kappa = 3 * 0.25 * p->sigma * d->l;              // :96
    d->L = 4.0 / 3.0 * d->m / d->kappa *
           (0.5 * (d->MS + d->ML) / ((p->cSeq - p->cLeq) * (p->cSeq - p->cLeq)));   // :97
    const double D = p->DL > p->DS ? p->DL : p->DS;
    d->dt_limit = p->dx * p->dx / (6.0 * D);
    return PPF_OK;
}

template <typename T>
static Coef<T> make_coef(const ppf_params &p, const ppf_derived &d) {
    const double tmp1 = -1.0 * d.L * d.dt;         // :337
    const double tmp3 = d.dt * 0.5 * d.h2;          // :339
    const double kh2 = d.kappa * d.h2;
    Coef<T> k;
    k.AS = (T)p.AS;
    k.dA = (T)(p.AL - p.AS);
    k.AsAl = (T)(p.AS * p.AL);
    k.A = (T)p.AS;
    k.cL0 = (T)p.cL0;
    k.dc0 = (T)(p.cL0 - p.cS0);
    k.Mt0 = (T)(tmp3 * d.ML);
    k.Mt1 = (T)(tmp3 * (d.MS - d.ML));
    k.dC = (T)(p.CS - p.CL);
    k.q1 = (T)(p.cS0 - p.cL0);
    k.q2 = (T)(0.5 * (1.0 / p.AS - 1.0 / p.AL));
    k.dm2 = (T)(2.0 * tmp1);
    k.mt = (T)(tmp1 * d.m);
    k.tg = (T)(2.0 * p.gamma);
    k.kt = (T)(tmp1 * kh2);
    return k;
}

int check_device_error(ppf_ctx *c);

static Fields<float> ff(ppf_ctx *c, int be, int bc_) {
    return {(float *)c->fld[be][0], (float *)c->fld[be][1], (float *)c->fld[bc_][2]};
}
static Fields<double> fd(ppf_ctx *c, int be, int bc_) {
    return {(double *)c->fld[be][0], (double *)c->fld[be][1], (double *)c->fld[bc_][2]};
}
template <typename T>
static Fields<const T> cst(Fields<T> f) {
    return {f.eS, f.eL, f.c};
}

int ensure_partials(ppf_ctx *c, int ndoubles) {
    if (ndoubles <= c->partials_cap) return PPF_OK;
    if (c->partials) cudaFree(c->partials);
    c->partials = nullptr;
    c->partials_cap = 0;
    CU(cudaMalloc(&c->partials, (size_t)ndoubles * sizeof(double)));
    c->partials_cap = ndoubles;
    return PPF_OK;
}

extern "C" int ppf_create(int nz, int ny, int nx, const ppf_params *p, int bc, int precision, ppf_ctx **out) {
    if (!out) return seterr(PPF_EINVAL, "out is NULL");
    *out = nullptr;
    if (nz < 1 || ny < 1 || nx < 1 || nz > 8192 || ny > 8192 || nx > 8192)
        return seterr(PPF_EINVAL, "grid %dx%dx%d out of range [1, 8192]", nz, ny, nx);
    if (bc != PPF_BC_PERIODIC && bc != PPF_BC_NOFLUX) return seterr(PPF_EINVAL, "bad bc %d", bc);
    if (precision != PPF_F64 && precision != PPF_F32) return seterr(PPF_EINVAL, "bad precision %d", precision);
    ppf_params prm;
    if (p) prm = *p;
    else ppf_params_default(&prm);
    ppf_derived der;
    int rc = ppf_params_derive(&prm, &der);
    if (rc) return rc;
    int dev = 0, ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1)
        return seterr(PPF_ECUDA, "no CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
    CU(cudaGetDevice(&dev));
    ppf_ctx *c = new (std::nothrow) ppf_ctx();
    if (!c) return seterr(PPF_ENOMEM, "host allocation failed");
    c->nz = nz; c->ny = ny; c->nx = nx; c->bc = bc; c->prec = precision;
    c->p = prm;
    c->d = der;
    c->dev = dev;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
    c->g = precision == PPF_F32 ? make_geom<float>(nz, ny, nx, bc) : make_geom<double>(nz, ny, nx, bc);
    c->kf = make_coef<float>(prm, der);
    c->kd = make_coef<double>(prm, der);
    c->eqA = prm.AS == prm.AL;
    c->cd.AS = prm.AS; c->cd.AL = prm.AL; c->cd.dA = prm.AL - prm.AS;
    c->cd.cS0 = prm.cS0; c->cd.cL0 = prm.cL0; c->cd.CS = prm.CS; c->cd.CL = prm.CL;
    c->cd.tmp2 = prm.AS * prm.cS0 - prm.AL * prm.cL0;
    c->cd.m = der.m; c->cd.gamma = prm.gamma; c->cd.kappa_h2_half = 0.5 * der.kappa * der.h2;
    c->cd.vol = prm.dx * prm.dx * prm.dx;
    const size_t es = precision == PPF_F32 ? 4 : 8;
    const size_t fbytes = (size_t)c->g.total * es;
    const int64_t cells = (int64_t)nz * ny * nx;
    cudaError_t e1 = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
    cudaError_t e2 = e1 == cudaSuccess ? cudaMalloc(&c->state, 6 * fbytes) : e1;
    cudaError_t e3 = e2 == cudaSuccess ? cudaMalloc(&c->staging, 3 * (size_t)cells * sizeof(double)) : e2;
    cudaError_t e4 = e3 == cudaSuccess ? cudaMalloc(&c->dres, 32 * sizeof(double) + 64) : e3;
    if (e4 != cudaSuccess) {
        ppf_destroy(c);
        return seterr(e4 == cudaErrorMemoryAllocation ? PPF_ENOMEM : PPF_ECUDA, "device setup failed: %s",
                      cudaGetErrorString(e4));
    }
    c->stream = c->own;
    c->derr = (int *)(c->dres + 32);
    c->dsched = c->derr + 4;
    c->wait_limit_ns = 1000000000ULL;
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 3; ++f) c->fld[b][f] = (char *)c->state + (size_t)(3 * b + f) * fbytes;
    for (int tl = 0; tl < 2 && rc == PPF_OK; ++tl)
        for (int b = 0; b < 2; ++b)
            for (int f = 0; f < 3; ++f) {
                // (FP64 has one tile shape: its second set repeats the first)
                CUtensorMap *m = &c->maps[tl][b][f];
                int mr = precision == PPF_F32 ? make_field_map<float>(c->g, (const float *)c->fld[b][f], m, tl)
                                              : make_field_map<double>(c->g, (const double *)c->fld[b][f], m, 0);
                if (mr != 0) {
                    ppf_destroy(c);
                    return seterr(PPF_ECUDA, "TMA descriptor setup failed (%d)", mr);
                }
            }
    c->tune.roll = 1;
    c->tune.pdl = kStepPdl;
    c->tune.sched = kStepSched;
    c->tune.split = kStepSplit;
    c->tune.grid = precision == PPF_F32 ? tma_grid<float>(c->g, c->num_sms, &c->tune.zc)
                                        : tma_grid<double>(c->g, c->num_sms, &c->tune.zc);
    if (c->tune.grid < 1) {
        ppf_destroy(c);
        return seterr(PPF_ECUDA, "kernel attribute setup failed");
    }
    // zero the padding once so that unused ghost edges hold finite values
    e = cudaMemsetAsync(c->state, 0, 6 * fbytes, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dres, 0, 32 * sizeof(double) + 64, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        ppf_destroy(c);
        return seterr(PPF_ECUDA, "device init failed: %s", cudaGetErrorString(e));
    }
    *out = c;
    return PPF_OK;
}

extern "C" int ppf_destroy(ppf_ctx *c) {
    if (!c) return PPF_OK;
    if (c->own) cudaStreamSynchronize(c->own);
    if (c->stream && c->stream != c->own) cudaStreamSynchronize(c->stream);
    if (c->state) cudaFree(c->state);
    if (c->staging) cudaFree(c->staging);
    if (c->partials) cudaFree(c->partials);
    if (c->dres) cudaFree(c->dres);
    if (c->plab) cudaFree(c->plab);
    if (c->pvol) cudaFree(c->pvol);
    if (c->plist) cudaFree(c->plist);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
    return PPF_OK;
}

extern "C" int ppf_get_dims(const ppf_ctx *c, int *nz, int *ny, int *nx) {
    if (!c) return seterr(PPF_EINVAL, "null context");
    if (nz) *nz = c->nz;
    if (ny) *ny = c->ny;
    if (nx) *nx = c->nx;
    return PPF_OK;
}

extern "C" int ppf_set_stream(ppf_ctx *c, void *stream) {
    if (!c) return seterr(PPF_EINVAL, "null context");
    CU(cudaStreamSynchronize(c->stream));
    c->stream = stream ? (cudaStream_t)stream : c->own;
    return PPF_OK;
}

int do_pack(ppf_ctx *c) {
    c->cur_eta = 0;
    c->cur_c = 0;
    if (c->prec == PPF_F32) CU(launch_pack<float>(c->g, c->staging, ff(c, 0, 0), c->stream));
    else CU(launch_pack<double>(c->g, c->staging, fd(c, 0, 0), c->stream));
    CU(cudaMemsetAsync(c->dres, 0, 3 * sizeof(double), c->stream));
    c->uploaded = 1;
    c->steps = 0;
    return PPF_OK;
}

extern "C" int ppf_upload(ppf_ctx *c, const double *etaS, const double *etaL, const double *cc) {
    if (!c || !etaS || !etaL || !cc) return seterr(PPF_EINVAL, "null argument");
    const size_t n = (size_t)c->nz * c->ny * c->nx;
    CU(cudaMemcpyAsync(c->staging, etaS, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(c->staging + n, etaL, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(c->staging + 2 * n, cc, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int rc = do_pack(c);
    if (rc) return rc;
    CU(cudaStreamSynchronize(c->stream));
    return PPF_OK;
}

extern "C" int ppf_upload_device(ppf_ctx *c, const double *etaS, const double *etaL, const double *cc) {
    if (!c || !etaS || !etaL || !cc) return seterr(PPF_EINVAL, "null argument");
    const size_t n = (size_t)c->nz * c->ny * c->nx;
    CU(cudaMemcpyAsync(c->staging, etaS, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(c->staging + n, etaL, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(c->staging + 2 * n, cc, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    int rc = do_pack(c);
    if (rc) return rc;
    CU(cudaStreamSynchronize(c->stream));
    return PPF_OK;
}

int do_unpack(ppf_ctx *c) {
    if (!c->uploaded) return seterr(PPF_ESTATE, "no state uploaded");
    if (c->prec == PPF_F32)
        CU(launch_unpack<float>(c->g, cst(ff(c, c->cur_eta, c->cur_c)), c->staging, c->stream));
    else
        CU(launch_unpack<double>(c->g, cst(fd(c, c->cur_eta, c->cur_c)), c->staging, c->stream));
    return PPF_OK;
}

extern "C" int ppf_download(ppf_ctx *c, double *etaS, double *etaL, double *cc) {
    if (!c || !etaS || !etaL || !cc) return seterr(PPF_EINVAL, "null argument");
    int rc = do_unpack(c);
    if (rc) return rc;
    const size_t n = (size_t)c->nz * c->ny * c->nx;
    CU(cudaMemcpyAsync(etaS, c->staging, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(etaL, c->staging + n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(cc, c->staging + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

extern "C" int ppf_download_device(ppf_ctx *c, double *etaS, double *etaL, double *cc) {
    if (!c || !etaS || !etaL || !cc) return seterr(PPF_EINVAL, "null argument");
    int rc = do_unpack(c);
    if (rc) return rc;
    const size_t n = (size_t)c->nz * c->ny * c->nx;
    CU(cudaMemcpyAsync(etaS, c->staging, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(etaL, c->staging + n, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(cc, c->staging + 2 * n, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return PPF_OK;
}

// Reads and clears the device error word; PPF_ETIMEOUT when a kernel's
// bounded wait ran out since the last check.
int check_device_error(ppf_ctx *c) {
    int h = 0;
    CU(cudaMemcpyAsync(&h, c->derr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    if (h) {
        // the error word, and the scheduler pairs that an abandoned step may leave set
        CU(cudaMemsetAsync(c->derr, 0, 8 * sizeof(int), c->stream));
        CU(cudaStreamSynchronize(c->stream));
        return seterr(PPF_ETIMEOUT, "a device wait exceeded its limit; the state of that step is invalid");
    }
    return PPF_OK;
}

static int run_steps(ppf_ctx *c, int64_t nsteps, bool c_only) {
    if (!c) return seterr(PPF_EINVAL, "null context");
    if (nsteps < 0) return seterr(PPF_EINVAL, "negative step count");
    if (!c->uploaded) return seterr(PPF_ESTATE, "no state uploaded");
    if (nsteps == 0) return PPF_OK;
    const int64_t items = c->prec == PPF_F32 ? tma_items<float>(c->g, c->tune) : tma_items<double>(c->g, c->tune);
    if (items > ((int64_t)1 << 29)) return seterr(PPF_EINVAL, "too many work items");
    int rc = ensure_partials(c, 3 * (int)items);
    if (rc) return rc;
    for (int64_t s = 0; s < nsteps; ++s) {
        const bool last = s == nsteps - 1;
        const int ie = c->cur_eta, ic = c->cur_c;
        const int oe = c_only ? ie : 1 - ie, oc = 1 - ic;
        double *part = last ? c->partials : nullptr;
        const int inject = c->inject;
        c->inject = PPF_INJECT_NONE;
        cudaError_t e;
        if (c->prec == PPF_F32) {
            const int tl = c->tune.tile;
            const CUtensorMap m[3] = {c->maps[tl][ie][0], c->maps[tl][ie][1], c->maps[tl][ic][2]};
            e = launch_step_tma<float>(c->g, c->kf, m, ff(c, oe, oc), c_only, c->eqA, part, c->tune,
                                       c->derr, c->wait_limit_ns, inject, c->dsched, c->stream);
        } else {
            const CUtensorMap m[3] = {c->maps[0][ie][0], c->maps[0][ie][1], c->maps[0][ic][2]};
            e = launch_step_tma<double>(c->g, c->kd, m, fd(c, oe, oc), c_only, c->eqA, part, c->tune,
                                        c->derr, c->wait_limit_ns, inject, c->dsched, c->stream);
        }
        if (e != cudaSuccess) return seterr(PPF_ECUDA, "step launch failed: %s", cudaGetErrorString(e));
        c->cur_eta = oe;
        c->cur_c = oc;
        c->steps++;
        if (last) CU(launch_final_sum(c->partials, (int)items, 3, c_only ? 1 : 3, c->dres, c->stream));
    }
    return PPF_OK;
}

extern "C" int ppf_step(ppf_ctx *c, int64_t nsteps) { return run_steps(c, nsteps, false); }

extern "C" int ppf_step_c_only(ppf_ctx *c, int64_t nsteps) { return run_steps(c, nsteps, true); }

extern "C" int ppf_reduce(ppf_ctx *c, ppf_stats *out) {
    if (!c || !out) return seterr(PPF_EINVAL, "null argument");
    if (!c->uploaded) return seterr(PPF_ESTATE, "no state uploaded");
    const int64_t cells = (int64_t)c->nz * c->ny * c->nx;
    int nb = c->ny * c->nz;                     // one block per x row at most
    if (nb > 8 * c->num_sms) nb = 8 * c->num_sms;
    int rc = ensure_partials(c, 5 * nb);
    if (rc) return rc;
    if (c->prec == PPF_F32)
        CU(launch_observe<float>(c->g, c->cd, cst(ff(c, c->cur_eta, c->cur_c)), c->partials, nb, c->stream));
    else
        CU(launch_observe<double>(c->g, c->cd, cst(fd(c, c->cur_eta, c->cur_c)), c->partials, nb, c->stream));
    CU(launch_final_sum(c->partials, nb, 5, 5, c->dres + 3, c->stream));
    double h[8];
    CU(cudaMemcpyAsync(h, c->dres, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    rc = check_device_error(c);
    if (rc) return rc;
    out->sum_dc2 = h[0];
    out->sum_detaS2 = h[1];
    out->sum_detaL2 = h[2];
    out->mass = h[3];
    out->solid = h[4];
    out->solid_cells = h[5];
    out->free_energy = h[6];
    out->nonfinite = (int64_t)h[7];
    out->cells = cells;
    out->steps = c->steps;
    return PPF_OK;
}

extern "C" int ppf_sync(ppf_ctx *c) {
    if (!c) return seterr(PPF_EINVAL, "null context");
    CU(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

extern "C" int ppf_set_wait_limit(ppf_ctx *c, double seconds) {
    if (!c) return seterr(PPF_EINVAL, "null context");
    if (!(seconds > 0) || seconds > 60) return seterr(PPF_EINVAL, "wait limit must be in (0, 60] s");
    c->wait_limit_ns = (unsigned long long)(seconds * 1e9);
    return PPF_OK;
}

extern "C" int ppf_debug_inject(ppf_ctx *c, int fault) {
    if (!c) return seterr(PPF_EINVAL, "null context");
    if (fault != PPF_INJECT_NONE && fault != PPF_INJECT_STALL_WAIT) return seterr(PPF_EINVAL, "unknown fault %d", fault);
    c->inject = fault;
    return PPF_OK;
}

static int grid_for(ppf_ctx *c, const StepTune &t) {
    return c->prec == PPF_F32 ? tma_grid_for<float>(c->g, c->num_sms, t) : tma_grid_for<double>(c->g, c->num_sms, t);
}

static int grid_for(ppf_ctx *c, int zc) {
    StepTune t = c->tune;
    t.zc = zc;
    t.zc2 = t.tail = 0;
    return grid_for(c, t);
}

extern "C" int ppf_get_tune(const ppf_ctx *c, ppf_tune *t) {
    if (!c || !t) return seterr(PPF_EINVAL, "null argument");
    t->zc = c->tune.zc;
    t->roll = c->tune.roll;
    t->grid = c->tune.grid;
    t->pdl = c->tune.pdl;
    t->sched = c->tune.sched;
    t->zc2 = c->tune.zc2;
    t->tail = c->tune.tail;
    t->split = c->tune.split;
    t->tile = c->tune.tile;
    t->us_per_step = 0.0;
    return PPF_OK;
}

extern "C" int ppf_set_tune(ppf_ctx *c, const ppf_tune *t) {
    if (!c || !t) return seterr(PPF_EINVAL, "null argument");
    if (t->roll != 1 && t->roll != 3) return seterr(PPF_EINVAL, "roll must be 1 or 3");
    if (t->zc < 1 || t->zc > c->nz) return seterr(PPF_EINVAL, "zc must be in [1, nz]");
    if (t->pdl != 0 && t->pdl != 1) return seterr(PPF_EINVAL, "pdl must be 0 or 1");
    if (t->sched != 0 && t->sched != 1) return seterr(PPF_EINVAL, "sched must be 0 or 1");
    if (t->zc2 < 0 || t->tail < 0 || t->tail > c->nz) return seterr(PPF_EINVAL, "need zc2 >= 0 and 0 <= tail <= nz");
    if (t->split != 0 && t->split != 1) return seterr(PPF_EINVAL, "split must be 0 or 1");
    const int shapes = c->prec == PPF_F32 ? step_tile_shapes<float>() : step_tile_shapes<double>();
    if (t->tile < 0 || t->tile >= shapes) return seterr(PPF_EINVAL, "tile must be in [0, %d)", shapes);
    CU(cudaStreamSynchronize(c->stream));
    StepTune n = c->tune;
    n.zc = t->zc;
    n.roll = t->roll;
    n.pdl = t->pdl;
    n.sched = t->sched;
    n.split = t->split;
    n.tile = t->tile;
    n.zc2 = t->zc2 < t->zc ? t->zc2 : 0;
    n.tail = n.zc2 > 0 ? t->tail : 0;
    n.grid = grid_for(c, n);
    if (n.grid < 1) return seterr(PPF_ECUDA, "no launch shape for zc=%d", t->zc);
    c->tune = n;
    return PPF_OK;
}

extern "C" int ppf_autotune(ppf_ctx *c, int trial_steps, ppf_tune *best) {
    if (!c) return seterr(PPF_EINVAL, "null context");
    if (!c->uploaded) return seterr(PPF_ESTATE, "autotuning needs an uploaded state");
    if (trial_steps < 1) trial_steps = 1;
    // candidates: the model's chunk, powers of two and a few short chunks
    // (fine items for the counter's deal), a single chunk, and the chunks
    // that deal k = 3..7 items to nearly every CTA (so that the resident
    // CTAs end together); both unrolls; with and without programmatic
    // dependent launch; counter or round-robin deal
    int zcs[16], nzc = 0;
    auto add = [&](int z) {
        if (z < 1 || z > c->nz) return;
        for (int i = 0; i < nzc; ++i)
            if (zcs[i] == z) return;
        if (nzc < 16) zcs[nzc++] = z;
    };
    add(c->tune.zc);
    add(c->nz);
    for (int z = 8; z <= 128; z *= 2) add(z);
    add(4);
    add(12);
    add((c->tune.zc + 1) / 2);
    add(c->tune.zc * 2);
    {
        int tx = 0, ty = 0;
        if (c->prec == PPF_F32) step_tile<float>(&tx, &ty, 0);
        else step_tile<double>(&tx, &ty, 0);
        const int64_t ntiles = (int64_t)((c->nx + tx - 1) / tx) * ((c->ny + ty - 1) / ty);
        const int64_t slots = grid_for(c, 1);          // a grid that every CTA slot holds
        for (int k = 3; k <= 7 && ntiles > 0 && slots > 0; ++k) {
            const int64_t nc = k * slots / ntiles;     // chunks per tile column
            if (nc >= 1) add((int)((c->nz + nc - 1) / nc));
        }
    }
    // keep the state: the trials advance it, so save it and restore it after
    const int64_t steps0 = c->steps;
    int rc = do_unpack(c);
    if (rc) return rc;
    const StepTune keep = c->tune;
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    float best_ms = -1.0f;
    StepTune win = keep;
    auto trial = [&](StepTune t) {
        t.grid = grid_for(c, t);
        if (t.grid < 1) return;
        c->tune = t;
        if ((rc = run_steps(c, 2, false)) != PPF_OK) return;      // warm-up
        if (cudaEventRecord(e0, c->stream) != cudaSuccess) { rc = seterr(PPF_ECUDA, "event record"); return; }
        if ((rc = run_steps(c, trial_steps, false)) != PPF_OK) return;
        if (cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
            rc = seterr(PPF_ECUDA, "event timing failed");
            return;
        }
        if ((rc = check_device_error(c)) != PPF_OK) return;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (best_ms < 0 || ms < best_ms) { best_ms = ms; win = t; }
    };
    // uniform chunks; with edge tiles, as one launch or two; the first tile
    // shape with every deal and overlap, the others with the counter's deal
    // and programmatic dependent launch
    const int shapes = c->prec == PPF_F32 ? step_tile_shapes<float>() : step_tile_shapes<double>();
    for (int tl = 0; tl < shapes && rc == PPF_OK; ++tl) {
        int tx = 0, ty = 0;
        if (c->prec == PPF_F32) step_tile<float>(&tx, &ty, tl);
        else step_tile<double>(&tx, &ty, tl);
        const bool edges = c->nx % tx != 0 || c->ny % ty != 0, wholes = c->nx >= tx && c->ny >= ty;
        const int nsplit = edges && wholes ? 2 : 1;
        for (int sp = 0; sp < nsplit && rc == PPF_OK; ++sp)
        for (int sd = 1; sd >= (tl == 0 ? 0 : 1) && rc == PPF_OK; --sd)
        for (int pdl = 1; pdl >= (tl == 0 ? 0 : 1) && rc == PPF_OK; --pdl)
        for (int r = 0; r < 2 && rc == PPF_OK; ++r)
            for (int i = 0; i < nzc && rc == PPF_OK; ++i) {
                StepTune t = keep;
                t.tile = tl;
                t.split = nsplit == 2 ? sp : keep.split;
                t.sched = sd;
                t.pdl = pdl;
                t.roll = r == 0 ? 3 : 1;
                t.zc = zcs[i];
                t.zc2 = t.tail = 0;
                trial(t);
            }
    }
    // with the counter's deal: longer main chunks (the winner's and longer
    // ones, which pay fewer halo planes) with chunks of a half to a quarter
    // of their length at the top of z, covering about one or two waves of
    // the persistent grid's items
    if (rc == PPF_OK && win.sched == 1) {
        const StepTune base = win;
        int tx = 0, ty = 0;
        if (c->prec == PPF_F32) step_tile<float>(&tx, &ty, base.tile);
        else step_tile<double>(&tx, &ty, base.tile);
        const int64_t ntiles = (int64_t)((c->nx + tx - 1) / tx) * ((c->ny + ty - 1) / ty);
        const int64_t slots = grid_for(c, 1);
        int mains[5], nm = 0;
        for (int z : {base.zc, 2 * base.zc, 16, 24, 32}) {
            if (z < 4 || z > c->nz) continue;
            bool dup = false;
            for (int i = 0; i < nm; ++i) dup = dup || mains[i] == z;
            if (!dup) mains[nm++] = z;
        }
        for (int m = 0; m < nm && rc == PPF_OK; ++m)
            for (int q = 2; q <= 4 && rc == PPF_OK; ++q)
                for (int waves = 1; waves <= 2 && rc == PPF_OK; ++waves) {
                    StepTune t = base;
                    t.zc = mains[m];
                    t.zc2 = t.zc / q > 1 ? t.zc / q : 2;
                    const int64_t chunks = (waves * slots + ntiles - 1) / ntiles;
                    t.tail = (int)(chunks * t.zc2 < c->nz ? chunks * t.zc2 : c->nz / 2);
                    if (t.zc2 >= t.zc || t.tail < 1) continue;
                    trial(t);
                }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->tune = rc == PPF_OK ? win : keep;
    int rc2 = do_pack(c);           // restore the state saved above
    c->steps = steps0;
    if (rc2 == PPF_OK) {
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) rc2 = seterr(PPF_ECUDA, "restore failed: %s", cudaGetErrorString(e));
    }
    if (rc) return rc;
    if (rc2) return rc2;
    if (best) {
        best->zc = win.zc;
        best->roll = win.roll;
        best->grid = win.grid;
        best->pdl = win.pdl;
        best->sched = win.sched;
        best->zc2 = win.zc2;
        best->tail = win.tail;
        best->split = win.split;
        best->tile = win.tile;
        best->us_per_step = best_ms * 1000.0 / trial_steps;
    }
    return PPF_OK;
}

extern "C" int ppf_particles(ppf_ctx *c, double threshold, ppf_particle_stats *out, int64_t *volumes,
                             int64_t capacity, int64_t *nvolumes) {
    if (!c || !out) return seterr(PPF_EINVAL, "null argument");
    if (!c->uploaded) return seterr(PPF_ESTATE, "no state uploaded");
    if (volumes && capacity < 0) return seterr(PPF_EINVAL, "negative capacity");
    const int64_t cells = (int64_t)c->nz * c->ny * c->nx;
    if (cells >= ((int64_t)1 << 31)) return seterr(PPF_EINVAL, "particle labels hold at most 2^31-1 cells");
    if (!c->plab) CU(cudaMalloc(&c->plab, (size_t)cells * sizeof(int)));
    if (!c->pvol) CU(cudaMalloc(&c->pvol, (size_t)cells * sizeof(int)));
    int64_t cap = volumes ? capacity : 0;
    if (cap > 0 && cap > c->plist_cap) {
        if (c->plist) cudaFree(c->plist);
        c->plist = nullptr;
        c->plist_cap = 0;
        CU(cudaMalloc(&c->plist, (size_t)cap * sizeof(int64_t) + 64));
        c->plist_cap = cap;
    }
    int nb = (int)((cells + 255) / 256);
    if (nb > 8 * c->num_sms) nb = 8 * c->num_sms;
    int rc = ensure_partials(c, 5 * nb + 8);
    if (rc) return rc;
    unsigned long long *nlist = c->plist ? (unsigned long long *)(c->plist + c->plist_cap) : nullptr;
    double *dout = c->dres + 8;
    if (c->prec == PPF_F32)
        CU(launch_particles<float>(c->g, (const float *)c->fld[c->cur_eta][0], threshold, c->plab, c->pvol,
                                   c->partials, nb, c->p.dx, dout, cap > 0 ? c->plist : nullptr, cap, nlist, c->derr,
                                   c->stream));
    else
        CU(launch_particles<double>(c->g, (const double *)c->fld[c->cur_eta][0], threshold, c->plab, c->pvol,
                                    c->partials, nb, c->p.dx, dout, cap > 0 ? c->plist : nullptr, cap, nlist,
                                    c->derr, c->stream));
    double h[5];
    unsigned long long hn = 0;
    CU(cudaMemcpyAsync(h, dout, 5 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (cap > 0) CU(cudaMemcpyAsync(&hn, nlist, sizeof hn, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    rc = check_device_error(c);
    if (rc) return rc;
    const double dx = c->p.dx;
    out->count = (int64_t)h[0];
    out->mean_radius = h[0] > 0 ? h[1] / h[0] / dx : 0.0;
    out->solid_volume = h[2] * dx * dx * dx;
    out->largest_volume = h[3] * dx * dx * dx;
    out->interface_area = h[4] * dx * dx;
    if (nvolumes) *nvolumes = (int64_t)h[0];
    if (cap > 0) {
        const int64_t m = (int64_t)hn < cap ? (int64_t)hn : cap;
        CU(cudaMemcpy(volumes, c->plist, (size_t)m * sizeof(int64_t), cudaMemcpyDeviceToHost));
    }
    return PPF_OK;
}

extern "C" const char *ppf_last_error(void) { return g_err; }

extern "C" const char *ppf_version(void) { return "ppf-gb300 0.1 (sm_103a)"; }
