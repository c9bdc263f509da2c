// swc_step_mixed.cu -- the mixed engine: FP32 transforms and pointwise terms, FP64
// psiq/psiq_old/rho/f_rho state, FP64 CN/AB2 update, FP64 reductions.
#include "swc_step_impl.cuh"

namespace swc {
int make_engine_mixed(const swc_params& p, EngineBase** out) {
  auto* e = new (std::nothrow) StepEngine<float>(p);
  if (!e) return SWC_ERR_OOM;
  int rc = e->init();
  if (rc) { delete e; return rc; }
  *out = e;
  return SWC_OK;
}
}  // namespace swc
