// ppf_ensemble.cu -- many independent domains of different sizes advanced
// together: one persistent launch of the fused step per time step covers
// the work items of every domain (the MULTI variant of step_tma_kernel,
// reading each item's geometry and TMA descriptors from a device table),
// and runs of steps are replayed from a captured CUDA graph.
//
// No counterpart in the reference, which runs one domain per program.
// Each domain is an ordinary ppf_ctx (its own buffers, descriptors,
// uploads, downloads and reductions); the ensemble only owns the table, the
// per-item partial sums, the graph and the launch choices.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "ppf_ctx.h"

using namespace ppf;

namespace {

int err_(int code, const char *fmt, ...) {
    char msg[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    return set_last_error(code, msg);
}

#define ECU(call)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return err_(PPF_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));   \
    } while (0)

// per-domain sums of the per-item increment partials (deterministic order).
// nwhole < 0: the step was one launch over every tile (the domain's range
// of it); else the domain's whole-tile items, then its edge-tile items,
// which follow all `nwhole` whole-tile items in `partials`
__global__ void domain_sums(const DomainDesc *__restrict__ table, const double *__restrict__ partials, int nwhole,
                            double *const *__restrict__ dres) {
    const DomainDesc &d = table[blockIdx.x];
    __shared__ double red[3][128];
    double a[3] = {0, 0, 0};
    const int n = nwhole < 0 ? d.nitems[2] : d.nitems[1] + d.nitems[0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int64_t r = nwhole < 0 ? (int64_t)d.item0[2] + i
                          : i < d.nitems[1] ? d.item0[1] + i : (int64_t)nwhole + d.item0[0] + (i - d.nitems[1]);
        for (int v = 0; v < 3; ++v) a[v] += partials[r * 3 + v];
    }
    for (int v = 0; v < 3; ++v) red[v][threadIdx.x] = a[v];
    __syncthreads();
    for (int h = 64; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int v = 0; v < 3; ++v) red[v][threadIdx.x] += red[v][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int v = 0; v < 3; ++v) dres[blockIdx.x][v] = red[v][0];
}

}  // namespace

struct ppf_ensemble {
    int n, prec, bc, eqA;
    std::vector<ppf_ctx *> dom;
    std::vector<int> order;      // table entry k describes domain order[k]: largest domains first
    DomainDesc *dtable;          // device
    double **ddres;              // device: each domain's dres pointer
    IoDesc *dio;                 // device: each domain's batched-I/O descriptor (domain order)
    int64_t max_cells;           // cells of the largest domain
    double *partials;            // 3 doubles per work item
    int partials_cap;
    int items[3];                // work items of the edge-tile [0], whole-tile [1] and every-tile [2] launches
    int split;                   // 1: whole and edge tiles as two overlapping launches; 0: one launch
    int tile;                    // tile shape
    int grid, zc, roll;
    int pdl;                     // 1: launches overlap by programmatic dependent launch
    int sched;                   // 1: work items from a counter (domain 0's scheduler pair; the
                                 // ensemble's stream orders every domain's launches)
    int parity;                  // buffer holding the current state of every domain
    int64_t steps;
    cudaStream_t stream;
    cudaGraphExec_t graph;       // kGraphSteps plain steps, starting and ending at parity 0
    int graph_ok;
    int num_sms;
};

static constexpr int kGraphSteps = 16;

static int build_table(ppf_ensemble *e) {
    int tx = 0, ty = 0;
    if (e->prec == PPF_F32) step_tile<float>(&tx, &ty, e->tile);
    else step_tile<double>(&tx, &ty, e->tile);
    std::vector<DomainDesc> h((size_t)e->n);
    int64_t item0s[3] = {0, 0, 0};
    for (int k = 0; k < e->n; ++k) {
        ppf_ctx *c = e->dom[(size_t)e->order[(size_t)k]];
        DomainDesc &t = h[(size_t)k];
        memset(&t, 0, sizeof t);
        for (int b = 0; b < 2; ++b)
            for (int f = 0; f < 3; ++f) {
                t.maps[b][f] = c->maps[e->prec == PPF_F32 ? e->tile : 0][b][f];
                t.fld[b][f] = c->fld[b][f];
            }
        t.g = c->g;
        t.ntx = (c->nx + tx - 1) / tx;
        t.nty = (c->ny + ty - 1) / ty;
        t.nfx = c->nx / tx;
        t.nfy = c->ny / ty;
        t.zc = e->zc < c->nz ? e->zc : c->nz;
        t.nc = (c->nz + t.zc - 1) / t.zc;
        t.nitems[1] = t.nfx * t.nfy * t.nc;
        t.nitems[0] = (t.ntx * t.nty - t.nfx * t.nfy) * t.nc;
        t.nitems[2] = t.ntx * t.nty * t.nc;
        for (int q = 0; q < 3; ++q) {
            t.item0[q] = (int)item0s[q];
            item0s[q] += t.nitems[q];
        }
    }
    if (item0s[0] + item0s[1] > ((int64_t)1 << 29)) return err_(PPF_EINVAL, "ensemble has too many work items");
    e->items[0] = (int)item0s[0];
    e->items[1] = (int)item0s[1];
    e->items[2] = (int)item0s[2];
    const int64_t item0 = item0s[2];
    e->grid = e->prec == PPF_F32 ? tma_grid_items<float>(item0, e->num_sms, e->tile)
                                 : tma_grid_items<double>(item0, e->num_sms, 0);
    if (e->grid < 1) return err_(PPF_ECUDA, "no launch shape for the ensemble");
    ECU(cudaMemcpyAsync(e->dtable, h.data(), h.size() * sizeof(DomainDesc), cudaMemcpyHostToDevice, e->stream));
    if (3 * item0 > e->partials_cap) {
        if (e->partials) cudaFree(e->partials);
        e->partials = nullptr;
        ECU(cudaMalloc(&e->partials, (size_t)3 * item0 * sizeof(double)));
        e->partials_cap = (int)(3 * item0);
    }
    ECU(cudaStreamSynchronize(e->stream));
    if (e->graph_ok) cudaGraphExecDestroy(e->graph);
    e->graph_ok = 0;
    return PPF_OK;
}

static int launch_one(ppf_ensemble *e, bool stats) {
    const int inj = 0;
    (void)inj;
    ppf_ctx *c0 = e->dom[0];
    cudaError_t r;
    if (e->prec == PPF_F32)
        r = launch_step_multi<float>(e->dtable, e->n, e->items, c0->kf, false, e->eqA, e->parity,
                                     stats ? e->partials : nullptr, e->grid, e->roll, e->pdl != 0, e->split != 0,
                                     e->tile, c0->derr, c0->wait_limit_ns, e->sched ? c0->dsched : nullptr, e->stream);
    else
        r = launch_step_multi<double>(e->dtable, e->n, e->items, c0->kd, false, e->eqA, e->parity,
                                      stats ? e->partials : nullptr, e->grid, e->roll, e->pdl != 0, e->split != 0,
                                      0, c0->derr, c0->wait_limit_ns, e->sched ? c0->dsched : nullptr, e->stream);
    if (r != cudaSuccess) return err_(PPF_ECUDA, "ensemble step launch: %s", cudaGetErrorString(r));
    e->parity ^= 1;
    return PPF_OK;
}

static int ensure_graph(ppf_ensemble *e) {
    if (e->graph_ok) return PPF_OK;
    cudaGraph_t g;
    const int p0 = e->parity;
    e->parity = 0;
    ECU(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = PPF_OK;
    for (int s = 0; s < kGraphSteps && rc == PPF_OK; ++s) rc = launch_one(e, false);
    cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    e->parity = p0;
    if (rc) return rc;
    if (ce != cudaSuccess) return err_(PPF_ECUDA, "graph capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&e->graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return err_(PPF_ECUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    e->graph_ok = 1;
    return PPF_OK;
}

extern "C" int ppf_ensemble_destroy(ppf_ensemble *e) {
    if (!e) return PPF_OK;
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->graph_ok) cudaGraphExecDestroy(e->graph);
    for (ppf_ctx *c : e->dom) ppf_destroy(c);
    if (e->dtable) cudaFree(e->dtable);
    if (e->ddres) cudaFree(e->ddres);
    if (e->dio) cudaFree(e->dio);
    if (e->partials) cudaFree(e->partials);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return PPF_OK;
}

extern "C" int ppf_ensemble_create(int n, const int *dims, const ppf_params *p, int bc, int precision,
                                   ppf_ensemble **out) {
    if (!out || !dims || n < 1 || n > 4096) return err_(PPF_EINVAL, "ensemble: bad arguments");
    for (int d = 0; d < n; ++d) {
        // the ensemble step addresses each domain with 32-bit element offsets
        const int64_t nz = dims[3 * d], ny = dims[3 * d + 1], nx = dims[3 * d + 2];
        if (nz > 0 && ny > 0 && nx > 0 && (nz + 2) * (ny + 2) * (nx + 16) > ((int64_t)1 << 32))
            return err_(PPF_EINVAL, "ensemble: domain %d holds 2^32 elements or more per field", d);
    }
    *out = nullptr;
    ppf_ensemble *e = new (std::nothrow) ppf_ensemble();
    if (!e) return err_(PPF_ENOMEM, "host allocation failed");
    e->n = n;
    e->prec = precision;
    e->bc = bc;
    e->zc = 32;
    e->roll = 1;
    e->sched = 1;
    e->pdl = 1;
    e->split = 0;
    e->tile = 0;
    int rc = PPF_OK;
    for (int d = 0; d < n && rc == PPF_OK; ++d) {
        ppf_ctx *c = nullptr;
        rc = ppf_create(dims[3 * d], dims[3 * d + 1], dims[3 * d + 2], p, bc, precision, &c);
        if (rc == PPF_OK) e->dom.push_back(c);
    }
    if (rc) {
        ppf_ensemble_destroy(e);
        return rc;
    }
    ppf_ctx *c0 = e->dom[0];
    e->num_sms = c0->num_sms;
    e->eqA = c0->eqA;
    cudaError_t ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaMalloc(&e->dtable, (size_t)n * sizeof(DomainDesc));
    if (ce == cudaSuccess) ce = cudaMalloc(&e->ddres, (size_t)n * sizeof(double *));
    if (ce == cudaSuccess) ce = cudaMalloc(&e->dio, (size_t)n * sizeof(IoDesc));
    if (ce != cudaSuccess) {
        ppf_ensemble_destroy(e);
        return err_(PPF_ECUDA, "ensemble setup: %s", cudaGetErrorString(ce));
    }
    // work items of the largest domains first: the persistent grid ends a
    // step on the small domains' items, which shortens its tail
    e->order.resize((size_t)n);
    for (int d = 0; d < n; ++d) e->order[(size_t)d] = d;
    std::stable_sort(e->order.begin(), e->order.end(), [&](int a, int b) {
        const ppf_ctx *x = e->dom[(size_t)a], *y = e->dom[(size_t)b];
        return (int64_t)x->nz * x->ny * x->nx > (int64_t)y->nz * y->ny * y->nx;
    });
    std::vector<double *> h((size_t)n);
    for (int k = 0; k < n; ++k) h[(size_t)k] = e->dom[(size_t)e->order[(size_t)k]]->dres;
    for (int d = 0; d < n; ++d) e->dom[(size_t)d]->stream = e->stream;   // one stream orders every domain's work
    ce = cudaMemcpy(e->ddres, h.data(), (size_t)n * sizeof(double *), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) {
        std::vector<IoDesc> io((size_t)n);
        for (int d = 0; d < n; ++d) {
            const ppf_ctx *x = e->dom[(size_t)d];
            IoDesc &t = io[(size_t)d];
            memset(&t, 0, sizeof t);
            t.g = x->g;
            t.staging = x->staging;
            for (int b = 0; b < 2; ++b)
                for (int f = 0; f < 3; ++f) t.fld[b][f] = x->fld[b][f];
            t.dres = x->dres;
            const int64_t cells = (int64_t)x->nz * x->ny * x->nx;
            if (cells > e->max_cells) e->max_cells = cells;
        }
        ce = cudaMemcpy(e->dio, io.data(), io.size() * sizeof(IoDesc), cudaMemcpyHostToDevice);
    }
    if (ce != cudaSuccess) {
        ppf_ensemble_destroy(e);
        return err_(PPF_ECUDA, "ensemble setup: %s", cudaGetErrorString(ce));
    }
    rc = build_table(e);
    if (rc) {
        ppf_ensemble_destroy(e);
        return rc;
    }
    *out = e;
    return PPF_OK;
}

static int check_domain(ppf_ensemble *e, int d) {
    if (!e) return err_(PPF_EINVAL, "null ensemble");
    if (d < 0 || d >= e->n) return err_(PPF_EINVAL, "domain %d out of range [0, %d)", d, e->n);
    return PPF_OK;
}

extern "C" int ppf_ensemble_domain(ppf_ensemble *e, int d, ppf_ctx **ctx) {
    int rc = check_domain(e, d);
    if (rc) return rc;
    if (!ctx) return err_(PPF_EINVAL, "null argument");
    *ctx = e->dom[(size_t)d];
    return PPF_OK;
}

extern "C" int ppf_ensemble_upload(ppf_ensemble *e, int d, const double *etaS, const double *etaL, const double *c) {
    int rc = check_domain(e, d);
    if (rc) return rc;
    if (e->parity != 0) {
        // the domains are stepped together; a fresh upload lands in buffer 0,
        // so bring every other domain to buffer 0 first
        for (ppf_ctx *x : e->dom)
            if (x->uploaded && (rc = do_unpack(x)) == PPF_OK) rc = do_pack(x);
        if (rc) return rc;
        e->parity = 0;
    }
    return ppf_upload(e->dom[(size_t)d], etaS, etaL, c);
}

extern "C" int ppf_ensemble_download(ppf_ensemble *e, int d, double *etaS, double *etaL, double *c) {
    int rc = check_domain(e, d);
    if (rc) return rc;
    return ppf_download(e->dom[(size_t)d], etaS, etaL, c);
}

extern "C" int ppf_ensemble_upload_all(ppf_ensemble *e, const double *const *etaS, const double *const *etaL,
                                       const double *const *c) {
    if (!e || !etaS || !etaL || !c) return err_(PPF_EINVAL, "null argument");
    for (int d = 0; d < e->n; ++d)
        if (!etaS[d] || !etaL[d] || !c[d]) return err_(PPF_EINVAL, "null array of domain %d", d);
    // every domain's copies, then one conversion launch for all domains
    // (which also clears their increment sums), then one synchronisation
    for (int d = 0; d < e->n; ++d) {
        ppf_ctx *x = e->dom[(size_t)d];
        const size_t n = (size_t)x->nz * x->ny * x->nx;
        ECU(cudaMemcpyAsync(x->staging, etaS[d], n * sizeof(double), cudaMemcpyHostToDevice, e->stream));
        ECU(cudaMemcpyAsync(x->staging + n, etaL[d], n * sizeof(double), cudaMemcpyHostToDevice, e->stream));
        ECU(cudaMemcpyAsync(x->staging + 2 * n, c[d], n * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    }
    if (e->prec == PPF_F32) ECU(launch_pack_multi<float>(e->dio, e->n, e->max_cells, e->stream));
    else ECU(launch_pack_multi<double>(e->dio, e->n, e->max_cells, e->stream));
    for (ppf_ctx *x : e->dom) {
        x->cur_eta = x->cur_c = 0;
        x->uploaded = 1;
        x->steps = 0;
    }
    e->parity = 0;
    ECU(cudaStreamSynchronize(e->stream));
    return PPF_OK;
}

extern "C" int ppf_ensemble_download_all(ppf_ensemble *e, double *const *etaS, double *const *etaL,
                                         double *const *c) {
    if (!e || !etaS || !etaL || !c) return err_(PPF_EINVAL, "null argument");
    bool together = true;                      // every domain's state in buffer `parity`
    for (int d = 0; d < e->n; ++d) {
        const ppf_ctx *x = e->dom[(size_t)d];
        if (!etaS[d] || !etaL[d] || !c[d]) return err_(PPF_EINVAL, "null array of domain %d", d);
        if (!x->uploaded) return err_(PPF_ESTATE, "domain %d has no uploaded state", d);
        together = together && x->cur_eta == e->parity && x->cur_c == e->parity;
    }
    if (!together) {                           // a domain was stepped on its own
        for (int d = 0; d < e->n; ++d) {
            const int rc = ppf_download(e->dom[(size_t)d], etaS[d], etaL[d], c[d]);
            if (rc) return rc;
        }
        return PPF_OK;
    }
    // one conversion launch for all domains, then every domain's copies, then
    // one synchronisation
    if (e->prec == PPF_F32) ECU(launch_unpack_multi<float>(e->dio, e->n, e->max_cells, e->parity, e->stream));
    else ECU(launch_unpack_multi<double>(e->dio, e->n, e->max_cells, e->parity, e->stream));
    for (int d = 0; d < e->n; ++d) {
        ppf_ctx *x = e->dom[(size_t)d];
        const size_t n = (size_t)x->nz * x->ny * x->nx;
        ECU(cudaMemcpyAsync(etaS[d], x->staging, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
        ECU(cudaMemcpyAsync(etaL[d], x->staging + n, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
        ECU(cudaMemcpyAsync(c[d], x->staging + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    }
    ECU(cudaStreamSynchronize(e->stream));
    return check_device_error(e->dom[0]);
}

extern "C" int ppf_ensemble_reduce(ppf_ensemble *e, int d, ppf_stats *out) {
    int rc = check_domain(e, d);
    if (rc) return rc;
    return ppf_reduce(e->dom[(size_t)d], out);
}

static int run(ppf_ensemble *e, int64_t nsteps) {
    for (ppf_ctx *x : e->dom)
        if (!x->uploaded) return err_(PPF_ESTATE, "every domain needs an uploaded state");
    int rc = PPF_OK;
    int64_t left = nsteps;
    // whole graphs of plain steps (they start at buffer 0) while at least one
    // step remains for the statistics step
    if (left - 1 > kGraphSteps && e->parity == 1) {
        if ((rc = launch_one(e, false)) != PPF_OK) return rc;
        --left;
    }
    if (left - 1 >= kGraphSteps && e->parity == 0) {
        if ((rc = ensure_graph(e)) != PPF_OK) return rc;
        while (left - 1 >= kGraphSteps) {
            ECU(cudaGraphLaunch(e->graph, e->stream));
            left -= kGraphSteps;
        }
    }
    for (; left > 0 && rc == PPF_OK; --left) rc = launch_one(e, left == 1);
    if (rc) return rc;
    // the layout of the statistics step's partials (launch_step_multi)
    const int nwhole = e->items[0] == 0 || (e->split && e->items[1] > 0) ? e->items[1] : -1;
    domain_sums<<<e->n, 128, 0, e->stream>>>(e->dtable, e->partials, nwhole, e->ddres);
    ECU(cudaGetLastError());
    for (ppf_ctx *x : e->dom) {
        x->cur_eta = x->cur_c = e->parity;
        x->steps += nsteps;
    }
    e->steps += nsteps;
    return PPF_OK;
}

extern "C" int ppf_ensemble_step(ppf_ensemble *e, int64_t nsteps) {
    if (!e) return err_(PPF_EINVAL, "null ensemble");
    if (nsteps < 0) return err_(PPF_EINVAL, "negative step count");
    if (nsteps == 0) return PPF_OK;
    return run(e, nsteps);
}

extern "C" int ppf_ensemble_sync(ppf_ensemble *e) {
    if (!e) return err_(PPF_EINVAL, "null ensemble");
    ECU(cudaStreamSynchronize(e->stream));
    return check_device_error(e->dom[0]);
}

extern "C" int ppf_ensemble_get_tune(const ppf_ensemble *e, ppf_tune *t) {
    if (!e || !t) return err_(PPF_EINVAL, "null argument");
    t->zc = e->zc;
    t->roll = e->roll;
    t->grid = e->grid;
    t->pdl = e->pdl;
    t->sched = e->sched;
    t->split = e->split;
    t->tile = e->tile;
    t->zc2 = t->tail = 0;
    t->us_per_step = 0;
    return PPF_OK;
}

extern "C" int ppf_ensemble_set_tune(ppf_ensemble *e, const ppf_tune *t) {
    if (!e || !t) return err_(PPF_EINVAL, "null argument");
    if (t->roll != 1 && t->roll != 3) return err_(PPF_EINVAL, "roll must be 1 or 3");
    if (t->zc < 1) return err_(PPF_EINVAL, "zc must be >= 1");
    if (t->sched != 0 && t->sched != 1) return err_(PPF_EINVAL, "sched must be 0 or 1");
    if (t->pdl != 0 && t->pdl != 1) return err_(PPF_EINVAL, "pdl must be 0 or 1");
    if (t->split != 0 && t->split != 1) return err_(PPF_EINVAL, "split must be 0 or 1");
    const int shapes = e->prec == PPF_F32 ? step_tile_shapes<float>() : step_tile_shapes<double>();
    if (t->tile < 0 || t->tile >= shapes) return err_(PPF_EINVAL, "tile must be in [0, %d)", shapes);
    e->tile = t->tile;
    ECU(cudaStreamSynchronize(e->stream));
    e->split = t->split;
    e->zc = t->zc;
    e->roll = t->roll;
    e->sched = t->sched;
    e->pdl = t->pdl;
    return build_table(e);
}

extern "C" int ppf_ensemble_autotune(ppf_ensemble *e, int trial_steps, ppf_tune *best) {
    if (!e) return err_(PPF_EINVAL, "null ensemble");
    if (trial_steps < 1) trial_steps = 1;
    for (ppf_ctx *x : e->dom)
        if (!x->uploaded) return err_(PPF_ESTATE, "autotuning needs every domain's state");
    int rc = PPF_OK;
    // keep every domain's state: save it, try the choices, restore it
    for (ppf_ctx *x : e->dom)
        if ((rc = do_unpack(x)) != PPF_OK) return rc;
    const int zcs[] = {4, 8, 12, 16, 24, 32, 48, 64, 128};
    const int keep_zc = e->zc, keep_roll = e->roll, keep_sched = e->sched, keep_pdl = e->pdl, keep_split = e->split;
    const int keep_tile = e->tile;
    const int64_t keep_steps = e->steps;
    int best_zc = keep_zc, best_roll = keep_roll, best_sched = keep_sched, best_pdl = keep_pdl, best_split = keep_split;
    int best_tile = keep_tile;
    const int shapes = e->prec == PPF_F32 ? step_tile_shapes<float>() : step_tile_shapes<double>();
    float best_ms = -1.0f;
    cudaEvent_t t0, t1;
    ECU(cudaEventCreate(&t0));
    ECU(cudaEventCreate(&t1));
    // every tile shape; both kinds of tile: one launch or two; the first
    // shape with every deal and overlap, the others with the counter's deal
    // and programmatic dependent launch
    for (int tl = 0; tl < shapes && rc == PPF_OK; ++tl) {
    e->tile = tl;
    e->zc = zcs[0];
    if ((rc = build_table(e)) != PPF_OK) break;
    const int nsplit = e->items[0] > 0 && e->items[1] > 0 ? 2 : 1;
    for (int sp = 0; sp < nsplit && rc == PPF_OK; ++sp)
    for (int pdl = 1; pdl >= (tl == 0 ? 0 : 1) && rc == PPF_OK; --pdl)
    for (int sd = 1; sd >= (tl == 0 ? 0 : 1) && rc == PPF_OK; --sd)
    for (int r = 0; r < 2 && rc == PPF_OK; ++r)
        for (int zc : zcs) {
            e->zc = zc;
            e->roll = r == 0 ? 1 : 3;
            e->sched = sd;
            e->pdl = pdl;
            e->split = sp;
            e->tile = tl;
            if ((rc = build_table(e)) != PPF_OK) break;
            for (int s = 0; s < 2 && rc == PPF_OK; ++s) rc = launch_one(e, false);     // warm-up
            if (rc) break;
            cudaEventRecord(t0, e->stream);
            for (int s = 0; s < trial_steps && rc == PPF_OK; ++s) rc = launch_one(e, false);
            cudaEventRecord(t1, e->stream);
            if (cudaEventSynchronize(t1) != cudaSuccess) { rc = err_(PPF_ECUDA, "event timing failed"); break; }
            if ((rc = check_device_error(e->dom[0])) != PPF_OK) break;
            float ms = 0;
            cudaEventElapsedTime(&ms, t0, t1);
            if (best_ms < 0 || ms < best_ms) {
                best_ms = ms;
                best_zc = e->zc;
                best_roll = e->roll;
                best_sched = e->sched;
                best_pdl = e->pdl;
                best_split = e->split;
                best_tile = e->tile;
            }
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    e->zc = rc == PPF_OK ? best_zc : keep_zc;
    e->roll = rc == PPF_OK ? best_roll : keep_roll;
    e->sched = rc == PPF_OK ? best_sched : keep_sched;
    e->pdl = rc == PPF_OK ? best_pdl : keep_pdl;
    e->split = rc == PPF_OK ? best_split : keep_split;
    e->tile = rc == PPF_OK ? best_tile : keep_tile;
    int rc2 = build_table(e);
    for (ppf_ctx *x : e->dom)
        if (rc2 == PPF_OK) {
            const int64_t s0 = x->steps;
            rc2 = do_pack(x);
            x->steps = s0;
        }
    e->parity = 0;
    e->steps = keep_steps;
    if (rc2 == PPF_OK && cudaStreamSynchronize(e->stream) != cudaSuccess) rc2 = err_(PPF_ECUDA, "restore failed");
    if (rc) return rc;
    if (rc2) return rc2;
    if (best) {
        best->zc = e->zc;
        best->roll = e->roll;
        best->grid = e->grid;
        best->pdl = e->pdl;
        best->sched = e->sched;
        best->split = e->split;
        best->tile = e->tile;
        best->zc2 = best->tail = 0;
        best->us_per_step = best_ms * 1000.0 / trial_steps;
    }
    return PPF_OK;
}
