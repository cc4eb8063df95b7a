// ppf_step_tma.h -- launcher of the TMA-fed fused step (ppf_step_tma.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "ppf_internal.h"

namespace ppf {

// Launch choices of the fused step that the autotuner may change.
struct StepTune {
    int grid;   // persistent CTAs
    int zc;     // z planes per work item
    int roll;   // 3: plane body unrolled three times; 1: one copy
};

// Tensor map of one padded field (3-D: x pitch, ny+2 rows, nz+2 planes)
// with the kernel's box; 0 on success.
template <typename T>
int make_field_map(const Geom &g, const T *base, CUtensorMap *map);

// Persistent grid size (occupancy x SMs, capped by the work) and the z
// chunk length of a work item; < 0 on error.
template <typename T>
int tma_grid(const Geom &g, int num_sms, int *zc);

// Grid for a given z chunk length.
template <typename T>
int tma_grid_for_zc(const Geom &g, int num_sms, int zc);

// One fused step.  maps = {etaS, etaL, c} of the input state; eqA selects
// the specialisation for AS == AL (mu needs no reciprocal); `partials`
// (nullable) receives 3 doubles per CTA; `err` is a device word that a
// CTA sets when an mbarrier wait exceeds limit_ns.  inject_stall != 0 is a
// test hook that makes one wait per CTA run out.
template <typename T>
cudaError_t launch_step_tma(const Geom &g, const Coef<T> &k, const CUtensorMap *maps, Fields<T> out, bool c_only,
                            bool eqA, double *partials, const StepTune &tune, int *err, unsigned long long limit_ns,
                            int inject_stall, cudaStream_t s);

}  // namespace ppf
