// swc_step_mixed_c.cu -- part C of the mixed engine's step, in its own
// translation unit (the enqueue functions of one step are split three ways so their
// pass instantiations compile in parallel).
#include "swc_step_part_c.cuh"

namespace swc {
template int StepEngine<float>::enqueue_part_c(bool relax, bool first, bool diag);
template int StepEngine<float>::inverse_velocity(int ax, float* in, float* out);
template int StepEngine<float>::transform_vsol();
}  // namespace swc
