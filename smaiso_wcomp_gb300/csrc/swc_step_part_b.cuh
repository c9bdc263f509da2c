// swc_step_part_b.cuh -- part B of the step: S5 relax tail + S6 pointwise terms, the
// S7 forward transforms, S8-S10 Stokes solve and divergence (compiled by the engine's
// *_b.cu translation unit only).
#pragma once

#include "swc_step_impl.cuh"

namespace swc {

template <typename T> int StepEngine<T>::enqueue_part_b(bool relax, bool first, bool diag) {
  using LP = LdPlain<T, T>;
  using SP = StPlain<T, T>;
  const unsigned pw_blocks = (unsigned)((g_.ng + 255) / 256);
  // S5 relax tail + S6 (REF:1363-1425)
  {
    S6Args<T> a{lapR_, lpsi_, psi_, amp_f_, gp_[0], gp_[1], gp_[2], gr_[0], gr_[1], gr_[2], rho_,
                fgrad_, ener_, S_[0], S_[1], S_[2], f_[0], f_[1], f_[2], mu_,
                p_.ep, p_.beta, p_.gamma, p_.zeta, kp_, p_.rho_0, amp_, relax ? 1 : 0, rhof_, rho_off_,
                (T)p_.rho_0, (T)kp_, (T)p_.zeta, (T)p_.ep, (T)p_.beta, (T)p_.gamma, (T)rho_off_};
    s6_kernel<T><<<(unsigned)((g_.ng / 4 + 255) / 256), 256, 0, stream_>>>(g_, a);
    SWC_CK(cudaGetLastError());
    ++launches_;
  }
  // S7 (REF:1427-1457): forward transforms
  T* cts[2] = {fgrad_, ener_};
  for (T* b : cts) {
    SWC_TRY((pass<K_C2, 2>(LP{b}, SP{b})));
    SWC_TRY((pass<K_C2, 1>(LP{b}, SP{b})));
    SWC_TRY((pass<K_C2, 0>(LP{b}, SP{b})));
  }
  // The mixed engine transforms S only: grad.f, which enters Nl alone, is taken in real
  // space below (the FP64 engine keeps the reference's spectral form, REF:2078-2090).
  constexpr bool mixed = !std::is_same<T, double>::value;
  for (int ax = 0; ax < 3; ++ax) {
    T* bs[2] = {S_[ax], f_[ax]};
    for (int q = 0; q < (mixed ? 1 : 2); ++q) {
      T* b = bs[q];
      if (ax == 2) SWC_TRY((pass<K_S2, 2>(LP{b}, SP{b})));
      else SWC_TRY((pass<K_C2, 2>(LP{b}, SP{b})));
      if (ax == 1) SWC_TRY((pass<K_S2, 1>(LP{b}, SP{b})));
      else SWC_TRY((pass<K_C2, 1>(LP{b}, SP{b})));
      if (ax == 0) SWC_TRY((pass<K_S2, 0>(LP{b}, SP{b})));
      else SWC_TRY((pass<K_C2, 0>(LP{b}, SP{b})));
    }
  }
  if constexpr (mixed) {
    // grad.f of REF:2078-2090 = DCT-III^3 (scale sum_a q_a f-hat_a(mode - e_a)), f-hat_a the
    // mixed forward transform of f_a (DST-II along a). Along the two other axes
    // DCT-III DCT-II = 2n: component a is (1/2n_a) DCT-III_a(q_a(m) z_(m-1)), z = DST-II_a f_a,
    // and q_a(m) = Vs_a(m-1) -- minus the transposed-derivative pass DCT-III_a M^T DST-II_a
    // with M the derivative's multiplier -Vs/(2n). One pass per component, in place;
    // the first pass of the Nl transform reads the three and adds them.
    const T cx = (T)(1.0 / (2.0 * g_.nx)), cy = (T)(1.0 / (2.0 * g_.ny)), cz = (T)(1.0 / (2.0 * g_.nz));
    SWC_TRY((pass<K_DERIVT, 2>(LP{f_[2]}, SP{f_[2]}, MulDeriv<T>{vs_[2], cz, 2})));
    SWC_TRY((pass<K_DERIVT, 1>(LP{f_[1]}, SP{f_[1]}, MulDeriv<T>{vs_[1], cy, 1})));
    SWC_TRY((pass<K_DERIVT, 0>(LP{f_[0]}, SP{f_[0]}, MulDeriv<T>{vs_[0], cx, 0})));
  }
  // S8 + S9 (REF:1468-1974); the mixed engine's Stokes kernel also writes div v-hat (S10)
  // and writes v_irr itself only for the adjoint's tape (the steps that keep v_sol)
  {
    StokesArgs<T> a{S_[0], S_[1], S_[2], fgrad_, ener_, vsol_[0], vsol_[1], vsol_[2], virr_[0], virr_[1],
                    virr_[2], vq_[0], vq_[1], vq_[2], vs_[0], vs_[1], vs_[2], gq_[0], gq_[1], gq_[2], gs_[0],
                    gs_[1], gs_[2], (T)scale_, (T)(1.0 / p_.nu), (T)(1.0 / (p_.lambda + 2 * p_.nu)),
                    p_.nx / p_.ref_ranks, v_[0], v_[1], v_[2], cap_vsol_ ? 1 : 0,
                    (mixed && !cap_vsol_) ? 0 : 1, divv_};
    stokes_kernel<T, mixed><<<(unsigned)((g_.ng / 4 + 255) / 256), 256, 0, stream_>>>(g_, a);
    SWC_CK(cudaGetLastError());
    ++launches_;
  }
  // S10 (REF:1977-2091): the FP64 engine's div v-hat and q.f
  if constexpr (!mixed) {
    DivArgs<T> a{virr_[0], virr_[1], virr_[2], f_[0], f_[1], f_[2], divv_, dq_, vq_[0], vq_[1], vq_[2]};
    div_kernel<T><<<pw_blocks, 256, 0, stream_>>>(g_, a);
    SWC_CK(cudaGetLastError());
    ++launches_;
  }
  SWC_TRY((pass<K_C3, 2>(LP{divv_}, SP{divv_})));
  SWC_TRY((pass<K_C3, 1>(LP{divv_}, SP{divv_})));
  SWC_TRY((pass<K_C3, 0>(LP{divv_}, SP{divv_})));
  return SWC_OK;
}

}  // namespace swc
