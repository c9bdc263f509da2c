// swc_step_fp64.cu -- the FP64 step engine (every transform and pointwise term in FP64).
#include "swc_step_impl.cuh"
#include "swc_adjoint_impl.cuh"

namespace swc {
int make_engine_fp64(const swc_params& p, EngineBase** out) {
  auto* e = new (std::nothrow) StepEngine<double>(p);
  if (!e) return SWC_ERR_OOM;
  int rc = e->init();
  if (rc) { delete e; return rc; }
  *out = e;
  return SWC_OK;
}
}  // namespace swc
