// ppf_particles.h -- launcher of the particle analysis (ppf_particles.cu).
#pragma once

#include <cuda_runtime.h>

#include "ppf_internal.h"

namespace ppf {

// Labels the solid (etaS > threshold) of the state whose etaS is `etaS`
// (padded layout), then writes out[0..4] = {particles, sum of equivalent
// radii, solid cells, largest particle (cells), solid/liquid faces}.
// lab, vol: nx*ny*nz ints of scratch; partials: 5*nblocks doubles; list
// (nullable): up to `cap` particle volumes, *nlist = number of particles;
// err: a device word, bit 1 set if a retry cap was reached.
template <typename T>
cudaError_t launch_particles(const Geom &g, const T *etaS, double threshold, int *lab, int *vol, double *partials,
                             int nblocks, double dx, double *out, int64_t *list, int64_t cap,
                             unsigned long long *nlist, int *err, cudaStream_t s);

}  // namespace ppf
