// ppf_slabs.cu -- one domain split into z slabs, one context per slab, with
// one ghost-plane exchange per step: the decomposition of the reference's
// MPI build (init_mpi, phasefield.c:627-679, and exchange_ghost_layer,
// :683-708) reduced to its one-dimensional form.
//
// Each slab is an ordinary ppf_ctx of nz_s x ny x nx cells with the
// domain's BC in x and y.  After every step the fused kernel has written
// the slab's face ghosts as if the slab were the whole domain; the
// exchange then overwrites its two z ghost planes with the neighbours'
// boundary planes, in the receiving context's own storage (periodic: the
// first slab's lower neighbour is the last slab; no-flux: the end slabs keep
// their own mirror planes).  A plane of the padded layout is contiguous, so
// one copy per field and side moves it, x/y ghost rows included.  Every
// cell then sees exactly the neighbours it has in the undivided domain, so
// the result is bit-identical to stepping the whole domain.
//
// The slabs live on the current device and share one stream; the copies
// are cudaMemcpyAsync device to device.  Placing slabs on several GPUs
// would make the same copies peer copies; that path is not built here.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
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

#define SCU(call)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return err_(PPF_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));   \
    } while (0)

}  // namespace

extern "C" int ppf_slabs_plan(int nz, int nslabs, int bc, int *z0, int *nzs, int *lower, int *upper) {
    if (nz < 1 || nslabs < 1 || nslabs > nz || (bc != PPF_BC_PERIODIC && bc != PPF_BC_NOFLUX) || !z0 || !nzs ||
        !lower || !upper)
        return err_(PPF_EINVAL, "ppf_slabs_plan: need 1 <= nslabs <= nz, a valid bc and output arrays");
    // as even as possible: the first nz % nslabs slabs get one plane more
    const int base = nz / nslabs, extra = nz % nslabs;
    int z = 0;
    for (int s = 0; s < nslabs; ++s) {
        z0[s] = z;
        nzs[s] = base + (s < extra ? 1 : 0);
        z += nzs[s];
        const bool per = bc == PPF_BC_PERIODIC;
        lower[s] = s > 0 ? s - 1 : (per && nslabs > 1 ? nslabs - 1 : -1);
        upper[s] = s < nslabs - 1 ? s + 1 : (per && nslabs > 1 ? 0 : -1);
    }
    return PPF_OK;
}

struct ppf_slabs {
    int n, nz, ny, nx, bc, prec;
    std::vector<ppf_ctx *> ctx;
    std::vector<int> z0, nzs, lower, upper;
    cudaStream_t stream;
};

extern "C" int ppf_slabs_destroy(ppf_slabs *s) {
    if (!s) return PPF_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (ppf_ctx *c : s->ctx) ppf_destroy(c);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return PPF_OK;
}

extern "C" int ppf_slabs_create(int nz, int ny, int nx, int nslabs, const ppf_params *p, int bc, int precision,
                                ppf_slabs **out) {
    if (!out) return err_(PPF_EINVAL, "out is NULL");
    *out = nullptr;
    if (nslabs < 1 || nslabs > nz) return err_(PPF_EINVAL, "nslabs must be in [1, nz]");
    ppf_slabs *s = new (std::nothrow) ppf_slabs();
    if (!s) return err_(PPF_ENOMEM, "host allocation failed");
    s->n = nslabs;
    s->nz = nz;
    s->ny = ny;
    s->nx = nx;
    s->bc = bc;
    s->prec = precision;
    s->z0.resize((size_t)nslabs);
    s->nzs.resize((size_t)nslabs);
    s->lower.resize((size_t)nslabs);
    s->upper.resize((size_t)nslabs);
    int rc = ppf_slabs_plan(nz, nslabs, bc, s->z0.data(), s->nzs.data(), s->lower.data(), s->upper.data());
    if (rc) {
        delete s;
        return rc;
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return err_(PPF_ECUDA, "stream creation failed");
    }
    for (int k = 0; k < nslabs && rc == PPF_OK; ++k) {
        ppf_ctx *c = nullptr;
        rc = ppf_create(s->nzs[(size_t)k], ny, nx, p, bc, precision, &c);
        if (rc == PPF_OK) {
            s->ctx.push_back(c);
            rc = ppf_set_stream(c, s->stream);
        }
    }
    if (rc) {
        ppf_slabs_destroy(s);
        return rc;
    }
    *out = s;
    return PPF_OK;
}

// the z ghost planes of every slab := its neighbours' boundary planes
static int exchange(ppf_slabs *s) {
    for (int k = 0; k < s->n; ++k) {
        ppf_ctx *c = s->ctx[(size_t)k];
        const size_t es = c->prec == PPF_F32 ? 4 : 8;
        const size_t plane = (size_t)c->g.PS * es;
        for (int side = 0; side < 2; ++side) {
            const int nb = side == 0 ? s->lower[(size_t)k] : s->upper[(size_t)k];
            if (nb < 0) continue;                          // a no-flux end keeps its own mirror plane
            ppf_ctx *d = s->ctx[(size_t)nb];
            // storage plane 0 is z = -1, plane nz + 1 is z = nz
            const size_t dst_plane = side == 0 ? 0 : (size_t)c->nz + 1;
            const size_t src_plane = side == 0 ? (size_t)d->nz : 1;   // the neighbour's top / bottom row of cells
            for (int f = 0; f < 3; ++f) {
                const int bd = f < 2 ? c->cur_eta : c->cur_c, bs = f < 2 ? d->cur_eta : d->cur_c;
                char *dst = (char *)c->fld[bd][f] + dst_plane * plane;
                const char *src = (const char *)d->fld[bs][f] + src_plane * plane;
                SCU(cudaMemcpyAsync(dst, src, plane, cudaMemcpyDeviceToDevice, s->stream));
            }
        }
    }
    return PPF_OK;
}

extern "C" int ppf_slabs_upload(ppf_slabs *s, const double *etaS, const double *etaL, const double *c) {
    if (!s || !etaS || !etaL || !c) return err_(PPF_EINVAL, "null argument");
    const size_t pl = (size_t)s->ny * s->nx;
    for (int k = 0; k < s->n; ++k) {
        const size_t o = (size_t)s->z0[(size_t)k] * pl;
        int rc = ppf_upload(s->ctx[(size_t)k], etaS + o, etaL + o, c + o);
        if (rc) return rc;
    }
    int rc = exchange(s);
    if (rc) return rc;
    SCU(cudaStreamSynchronize(s->stream));
    return PPF_OK;
}

extern "C" int ppf_slabs_download(ppf_slabs *s, double *etaS, double *etaL, double *c) {
    if (!s || !etaS || !etaL || !c) return err_(PPF_EINVAL, "null argument");
    const size_t pl = (size_t)s->ny * s->nx;
    for (int k = 0; k < s->n; ++k) {
        const size_t o = (size_t)s->z0[(size_t)k] * pl;
        int rc = ppf_download(s->ctx[(size_t)k], etaS + o, etaL + o, c + o);
        if (rc) return rc;
    }
    return PPF_OK;
}

extern "C" int ppf_slabs_step(ppf_slabs *s, int64_t nsteps) {
    if (!s) return err_(PPF_EINVAL, "null slabs");
    if (nsteps < 0) return err_(PPF_EINVAL, "negative step count");
    for (int64_t t = 0; t < nsteps; ++t) {
        for (ppf_ctx *c : s->ctx) {
            int rc = ppf_step(c, 1);
            if (rc) return rc;
        }
        int rc = exchange(s);
        if (rc) return rc;
    }
    return PPF_OK;
}

extern "C" int ppf_slabs_reduce(ppf_slabs *s, ppf_stats *out) {
    if (!s || !out) return err_(PPF_EINVAL, "null argument");
    ppf_stats t;
    memset(out, 0, sizeof *out);
    for (int k = 0; k < s->n; ++k) {
        int rc = ppf_reduce(s->ctx[(size_t)k], &t);
        if (rc) return rc;
        out->sum_dc2 += t.sum_dc2;
        out->sum_detaS2 += t.sum_detaS2;
        out->sum_detaL2 += t.sum_detaL2;
        out->mass += t.mass;
        out->solid += t.solid;
        out->solid_cells += t.solid_cells;
        out->free_energy += t.free_energy;
        out->cells += t.cells;
        out->nonfinite += t.nonfinite;
        out->steps = t.steps;
    }
    return PPF_OK;
}

extern "C" int ppf_slabs_sync(ppf_slabs *s) {
    if (!s) return err_(PPF_EINVAL, "null slabs");
    for (ppf_ctx *c : s->ctx) {
        int rc = ppf_sync(c);
        if (rc) return rc;
    }
    return PPF_OK;
}
