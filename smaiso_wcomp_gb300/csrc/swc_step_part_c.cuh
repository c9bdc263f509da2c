// swc_step_part_c.cuh -- part C of the step: S11 velocities to real space, S12-S14
// density update, Nl transform, psiq update, psi back to real space and the diagnostic
// reductions (compiled by the engine's *_c.cu translation unit only).
#pragma once

#include "swc_step_impl.cuh"

namespace swc {

// The staggered inverse transform of one velocity component (REF:2093-2117): DST-III
// along its own axis, DCT-III along the other two.
template <typename T> int StepEngine<T>::inverse_velocity(int ax, T* in, T* out) {
  using LP = LdPlain<T, T>;
  using SP = StPlain<T, T>;
  if (ax == 2) SWC_TRY((pass<K_S3, 2>(LP{in}, SP{out})));
  else SWC_TRY((pass<K_C3, 2>(LP{in}, SP{out})));
  if (ax == 1) SWC_TRY((pass<K_S3, 1>(LP{out}, SP{out})));
  else SWC_TRY((pass<K_C3, 1>(LP{out}, SP{out})));
  if (ax == 0) SWC_TRY((pass<K_S3, 0>(LP{out}, SP{out})));
  else SWC_TRY((pass<K_C3, 0>(LP{out}, SP{out})));
  return SWC_OK;
}

// v_sol of the last step to real space, when a v_sol field is read (REF:2099-2117):
// the Stokes kernel keeps spectral v_sol on the last step of each swc_step call.
template <typename T> int StepEngine<T>::transform_vsol() {
  const int64_t keep = launches_;
  for (int ax = 0; ax < 3; ++ax) SWC_TRY(inverse_velocity(ax, vsol_[ax], vsolr_[ax]));
  launches_ = keep;
  return SWC_OK;
}

template <typename T> int StepEngine<T>::enqueue_part_c(bool relax, bool first, bool diag) {
  using LP = LdPlain<T, T>;
  using SP = StPlain<T, T>;
  // S11 (REF:2093-2117): v = vsol + virr (summed by the Stokes kernel into v_) to real
  // space in place; v_sol alone is transformed on demand (transform_vsol)
  for (int ax = 0; ax < 3; ++ax) SWC_TRY(inverse_velocity(ax, v_[ax], v_[ax]));
  // S12 + S13 + S14 (REF:2121-2197): rho update, Nl, its DCT, the psiq update, psi = iDCT(psiq_new)
  T* pout = (diag || cap_tape_) ? psi_new_ : psi_;  // the tape variant keeps the input psi
  if constexpr (std::is_same<T, double>::value) {
    // FP64 engine: the reference's expressions; the CN update in the Nl transform's last pass
    LdNl<T> ld{v_[0], v_[1], v_[2], gr_[0], gr_[1], gr_[2], divv_, mu_, amp_f_, psi_, gp_[0], gp_[1], gp_[2],
               rho_, frho_, p_.dt, kp_, p_.zeta, p_.rho_0};
    SWC_TRY((pass<K_C2, 2>(ld, SP{nlw_})));
    SWC_TRY((pass<K_C2, 1>(LP{nlw_}, SP{nlw_})));
    StNlUpdate<T> st{dq_, psiq_, psiq_old_, nlq_, vqd_[0], vqd_[1], vqd_[2], p_.ep, p_.alpha,
                     p_.q0 * p_.q0, p_.dt, rho_m_, p_.dt / 2, scale_, first ? 1 : 0};
    SWC_TRY((pass<K_C2, 0>(LP{nlw_}, st)));
    SWC_TRY((pass<K_C3, 2>(LdPlain<T, double>{psiq_}, SP{pout})));
  } else {
    // mixed engine: FP64-lean density update fused into the Nl transform, then the CN update
    LdNlMixed ld{v_[0], v_[1], v_[2], gr_[0], gr_[1], gr_[2], divv_, mu_, amp_f_, psi_, gp_[0], gp_[1], gp_[2],
                 rho_, frhot_, rhof_, rho_off_, (float)p_.dt, (float)kp_, (float)p_.zeta, (float)p_.rho_0,
                 (float)rho_off_, f_[0], f_[1], f_[2]};
    SWC_TRY((pass<K_C2, 2>(ld, SP{nlw_})));
    SWC_TRY((pass<K_C2, 1>(LP{nlw_}, SP{nlw_})));
    SWC_TRY((pass<K_C2, 0>(LP{nlw_}, SP{nlw_})));
    // the CN update as a full-occupancy pointwise kernel (it writes the FP32 copy psiqf of
    // the new psiq), then a plain TMA-fed pass from that copy
    LdNlUpdate lu{nlw_, nullptr, nlq_, psiq_, psiq_old_, vq_[0], vq_[1], vq_[2], (float)(p_.q0 * p_.q0), (float)p_.ep,
                  (float)p_.alpha, (float)(p_.dt * rho_m_), psiqf_, (float)(p_.dt / 2 * scale_), first ? 1 : 0,
                  g_, vqd_[0], vqd_[1], vqd_[2], p_.ep, p_.alpha, p_.q0 * p_.q0, p_.dt * rho_m_,
                  p_.dt / 2 * scale_};
    nl_update_kernel<<<(unsigned)((g_.ng / 4 + 255) / 256), 256, 0, stream_>>>(g_.ng, lu);
    SWC_CK(cudaGetLastError());
    ++launches_;
    SWC_TRY((pass<K_C3, 2>(LP{psiqf_}, SP{pout})));
  }
  SWC_TRY((pass<K_C3, 1>(LP{pout}, SP{pout})));
  SWC_TRY((pass<K_C3, 0>(LP{pout}, SP{pout})));
  if (diag) {
    DiagArgs<T> a{psi_new_, lpsi_, amp_f_, psi_, psi_old_, energy_, rho_, partial_,
                  p_.ep, p_.beta, p_.gamma, p_.zeta, p_.rho_0, kp_, rhof_,
                  (T)(-0.5 * p_.ep), (T)(0.25 * p_.beta), (T)(p_.gamma / 6), (T)(0.5 * p_.zeta),
                  (T)p_.rho_0, (T)kp_, (T)rho_off_};
    diag_kernel<T><<<diag_blocks_, kDiagThreads, 0, stream_>>>(g_, a);
    SWC_CK(cudaGetLastError());
    diag_final_kernel<<<1, kDiagFinalThreads, 0, stream_>>>(partial_, diag_blocks_, dsum_);
    SWC_CK(cudaGetLastError());
    launches_ += 2;
  }
  return SWC_OK;
}

}  // namespace swc
