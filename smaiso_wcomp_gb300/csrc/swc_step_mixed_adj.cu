// swc_step_mixed_adj.cu -- the mixed engine's FP32 discrete adjoint (the FP64 engine's
// adjoint kernels instantiated for float), in its own translation unit.
#include "swc_step_impl.cuh"
#include "swc_adjoint_impl.cuh"

namespace swc {
template int StepEngine<float>::backward_impl(const double* dpsi, const double* drho, double energy_lambda,
                                              double* dpsi0, double* drho0, swc_grad* out);
}  // namespace swc
