// ppf_step_f64_ens.cu -- the FP64 ensemble instantiations of the fused step
// (ppf_step_tma.cuh).
#include "ppf_step_tma.cuh"

namespace ppf {

template int tma_grid_items<double>(int64_t, int, int);
template cudaError_t launch_step_multi<double>(const DomainDesc *, int, const int *, const Coef<double> &, bool, bool, int,
                                            double *, int, int, bool, bool, int, int *, unsigned long long,
                                            int *,
                                            cudaStream_t);

}  // namespace ppf
