// ppf_step_f32.cu -- the FP32 instantiations of the fused step (ppf_step_tma.cuh).
#include "ppf_step_tma.cuh"

namespace ppf {

template void step_tile<float>(int *, int *);
template int tma_grid_items<float>(int64_t, int);
template cudaError_t launch_step_multi<float>(const DomainDesc *, int, int, const Coef<float> &, bool, bool, int,
                                            double *, int, int, int *, unsigned long long, int *,
                                            cudaStream_t);
template int make_field_map<float>(const Geom &, const float *, CUtensorMap *);
template int tma_grid<float>(const Geom &, int, int *);
template int tma_grid_for<float>(const Geom &, int, const StepTune &);
template int64_t tma_items<float>(const Geom &, const StepTune &);
template cudaError_t launch_step_tma<float>(const Geom &, const Coef<float> &, const CUtensorMap *, Fields<float>, bool,
                                          bool, double *, const StepTune &, int *, unsigned long long, int, int *,
                                          cudaStream_t);

}  // namespace ppf
