// ppf_step_f32_ens.cu -- the FP32 ensemble instantiations of the fused step
// (ppf_step_tma.cuh).
#include "ppf_step_tma.cuh"

namespace ppf {

template int tma_grid_items<float>(int64_t, int, int);
template cudaError_t launch_step_multi<float>(const DomainDesc *, int, const int *, const Coef<float> &, bool, bool, int,
                                            double *, int, int, bool, bool, int, int *, unsigned long long,
                                            int *,
                                            cudaStream_t);

}  // namespace ppf
