// ppf_step_f32.cu -- the FP32 single-domain instantiations of the fused step
// (ppf_step_tma.cuh); the ensemble ones are in ppf_step_f32_ens.cu, so that
// the two sets of kernels compile in parallel.
#include "ppf_step_tma.cuh"

namespace ppf {

template void step_tile<float>(int *, int *, int);
template int step_tile_shapes<float>();
template int make_field_map<float>(const Geom &, const float *, CUtensorMap *, int);
template int tma_grid<float>(const Geom &, int, int *);
template int tma_grid_for<float>(const Geom &, int, const StepTune &);
template int64_t tma_items<float>(const Geom &, const StepTune &);
template cudaError_t launch_step_tma<float>(const Geom &, const Coef<float> &, const CUtensorMap *, Fields<float>, bool,
                                          bool, double *, const StepTune &, int *, unsigned long long, int, int *,
                                          cudaStream_t);

}  // namespace ppf
