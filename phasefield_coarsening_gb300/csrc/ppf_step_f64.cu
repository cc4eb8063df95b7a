// ppf_step_f64.cu -- the FP64 single-domain instantiations of the fused step
// (ppf_step_tma.cuh); the ensemble ones are in ppf_step_f64_ens.cu, so that
// the two sets of kernels compile in parallel.
#include "ppf_step_tma.cuh"

namespace ppf {

template void step_tile<double>(int *, int *, int);
template int step_tile_shapes<double>();
template int make_field_map<double>(const Geom &, const double *, CUtensorMap *, int);
template int tma_grid<double>(const Geom &, int, int *);
template int tma_grid_for<double>(const Geom &, int, const StepTune &);
template int64_t tma_items<double>(const Geom &, const StepTune &);
template cudaError_t launch_step_tma<double>(const Geom &, const Coef<double> &, const CUtensorMap *, Fields<double>, bool,
                                          bool, double *, const StepTune &, int *, unsigned long long, int, int *,
                                          cudaStream_t);

}  // namespace ppf
