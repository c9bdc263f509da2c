// swc_step_fp64_c.cu -- part C of the fp64 engine's step, in its own
// translation unit (the enqueue functions of one step are split three ways so their
// pass instantiations compile in parallel).
#include "swc_step_part_c.cuh"

namespace swc {
template int StepEngine<double>::enqueue_part_c(bool relax, bool first, bool diag);
template int StepEngine<double>::inverse_velocity(int ax, double* in, double* out);
template int StepEngine<double>::transform_vsol();
}  // namespace swc
