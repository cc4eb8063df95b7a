// ppf_ctx.h -- the context behind the opaque ppf_ctx of include/ppf.h,
// shared by the C-ABI translation units (ppf_capi.cu, ppf_ensemble.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "ppf.h"
#include "ppf_internal.h"
#include "ppf_step_tma.h"

// A context replaces the reference's global state (phasefield.c:67-70).
struct ppf_ctx {
    int nz, ny, nx, bc, prec;
    ppf_params p;
    ppf_derived d;
    ppf::Geom g;
    int dev, num_sms;
    cudaStream_t own, stream;
    void *state;          // one allocation: 2 buffers x 3 fields x g.total elements
    void *fld[2][3];      // [buffer][etaS, etaL, c]
    int cur_eta, cur_c;   // buffer holding the current eta / c
    double *staging;      // 3 * cells doubles, compact [z][y][x]
    double *partials;     // partial sums (per work item of the step, per block of other kernels)
    int partials_cap;     // in doubles
    double *dres;         // device results: [0..2] increments, [3..7] observables, [8..12] particles,
                          // [16..19] mass-projection plan; the error word follows at dres + 32
    int *derr;            // device error word set by a kernel whose bounded wait ran out
    int *dsched;          // the step's two scheduler word pairs (dres + 32, after the error word)
    CUtensorMap maps[2][2][3];   // TMA maps of the fields of both buffers, per tile shape [tile][buffer][field]
    ppf::StepTune tune;        // launch choices of the fused step (grid, z chunk, unroll)
    unsigned long long wait_limit_ns;
    int inject;           // test hook: PPF_INJECT_*
    int *plab, *pvol;     // particle labels / volumes (allocated on first use)
    int64_t *plist;       // particle volume list (device), plist_cap entries
    int64_t plist_cap;
    int64_t steps;
    int uploaded;
    ppf::Coef<float> kf;
    ppf::Coef<double> kd;
    int eqA;              // AS == AL: the mu reciprocal is a constant
    ppf::CoefD cd;
};

// helpers of ppf_capi.cu (return PPF_* codes, set ppf_last_error)
int ensure_partials(ppf_ctx *c, int ndoubles);
int do_pack(ppf_ctx *c);        // staging -> state buffer 0 (+ ghosts)
int do_unpack(ppf_ctx *c);      // current state -> staging
int check_device_error(ppf_ctx *c);
