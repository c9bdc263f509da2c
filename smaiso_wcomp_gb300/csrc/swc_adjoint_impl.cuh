// swc_adjoint_impl.cuh -- the discrete adjoint of the time step and the recompute
// behind swc_backward (instantiated for the FP64 engine, T = double, and for the FP32
// adjoint of the mixed engine, T = float).
//
// Trajectory, two schedules. K = adjoint_ckpt > 0: swc_step kept the state every K
// steps (swc_set_state kept step 0); swc_backward walks the segments from the last,
// restores the segment's first state, reruns its steps keeping a tape of the
// intermediates each adjoint step reads, then applies the adjoint steps in reverse.
// Device memory: (T/K + 2) checkpoints + K tape slots of kTape N^3 values + the adjoint
// work arrays (kAdj N^3 values). adjoint_ckpt = -1: binomial checkpointing (Griewank's
// optimal schedule, reverse_binomial): only the initial state is kept by the forward;
// s snapshot slots (the largest count that fits under adjoint_cap_gb) and a one-step
// tape whose fields are mostly read in place; with S = s + 1 and t the least integer
// with C(S + t, t) >= T, the reversal advances t T - C(S + t, t - 1) steps plus one
// taped rerun per step.
#pragma once

#include "swc_adjoint_kernels.cuh"

namespace swc {

// tape slot layout (N^3 doubles each)
enum {
  TP_PSI = 0, TP_QOLD, TP_QNEW, TP_GPX, TP_GPY, TP_GPZ, TP_GRX, TP_GRY, TP_GRZ, TP_A, TP_L, TP_LAPR,
  TP_RHOIN, TP_RHONEW, TP_VX, TP_VY, TP_VZ, TP_DIVV, TP_VSX, TP_VSY, TP_VSZ, TP_VIX, TP_VIY, TP_VIZ, kTape
};
static_assert(PG_COUNT == 8, "pgrad_doubles() assumes 8 parameter slots");
static_assert(kTape <= 32, "tape_alias_ holds one pointer per tape field");

// adjoint work arrays
enum {
  AJ_Q = 0, AJ_QO, AJ_NLO, AJ_R, AJ_F, AJ_NL, AJ_FX, AJ_FY, AJ_FZ, AJ_MU, AJ_A, AJ_PSI, AJ_VX, AJ_VY, AJ_VZ,
  AJ_GPX, AJ_GPY, AJ_GPZ, AJ_GRX, AJ_GRY, AJ_GRZ, AJ_DIVV, AJ_DOTX, AJ_DOTY, AJ_DOTZ, AJ_SDX, AJ_SDY, AJ_SDZ,
  AJ_FGPX, AJ_FGPY, AJ_FGPZ, AJ_SX, AJ_SY, AJ_SZ, AJ_FG, AJ_E, AJ_LAPR, AJ_L,
  AJ_KEEPL, AJ_KEEPA,  // the final step's L and A, put back when swc_backward returns
  kAdj
};

// Fields the one-step tape of the binomial schedule copies (the others are read in
// place): the incoming density, and in the mixed engine the FP64 state narrowed to FP32.
constexpr int kTapeCopied(bool mixed) { return mixed ? 4 : 1; }

template <typename T> int StepEngine<T>::adjoint_alloc(size_t tape_fields) {
  const size_t ng = (size_t)g_.ng;
  if (!adj_) {
    if (cudaMalloc(&adj_, (size_t)kAdj * ng * sizeof(T)) != cudaSuccess ||
        cudaMalloc(&pgrad_, pgrad_doubles() * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc of the adjoint work arrays failed (%zu MB)", (kAdj * ng * sizeof(T)) >> 20);
      return SWC_ERR_OOM;
    }
  }
  if (tape_fields_ < tape_fields) {
    if (tape_) cudaFree(tape_);
    tape_ = nullptr;
    if (cudaMalloc(&tape_, tape_fields * ng * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      tape_fields_ = 0;
      set_error("cudaMalloc of the adjoint tape failed (%zu MB)", (tape_fields * ng * sizeof(T)) >> 20);
      return SWC_ERR_OOM;
    }
    tape_fields_ = tape_fields;
  }
  return SWC_OK;
}

template <typename T>
int StepEngine<T>::adjoint_step(size_t slot, bool relax, bool first, bool last) {
  const size_t ng = (size_t)g_.ng;
  const T* tp = tape_ + slot * (size_t)kTape * ng;
  auto TP = [&](int q) { return (tape_alias_on_ && tape_alias_[q]) ? tape_alias_[q] : tp + (size_t)q * ng; };
  auto AJ = [&](int q) { return adj_ + (size_t)q * ng; };
  const unsigned blocks = pt4_blocks(g_);
  const AdjScalars<T> sc{(T)p_.ep, (T)p_.alpha, (T)p_.beta, (T)p_.gamma, (T)p_.zeta, (T)kp_, (T)p_.rho_0,
                         (T)(p_.q0 * p_.q0), (T)p_.dt, (T)(p_.dt / 2), (T)rho_m_, (T)scale_, (T)p_.nu,
                         (T)(p_.lambda + 2 * p_.nu)};
  using LP = LdPlain<T, T>;
  using SP = StPlain<T, T>;
  const AxisWeights<T> w2{{0, 0, 0}, (T)2.0}, wh{{0, 0, 0}, (T)0.5};
  auto sine_w = [](int ax, double w) { AxisWeights<T> a{{ax == 0, ax == 1, ax == 2}, (T)w}; return a; };

  // (1) CN/AB2 update (REF:2177-2190)
  adj_cn_kernel<T><<<blocks, 256, 0, stream_>>>(g_, vq_[0], vq_[1], vq_[2], sc, first ? 1 : 0, TP(TP_QOLD),
                                             TP(TP_QNEW), AJ(AJ_Q), AJ(AJ_QO), AJ(AJ_NLO), AJ(AJ_NL), pgrad_);
  SWC_CK(cudaGetLastError());
  // (2) grad.f subtracted in spectral space, then Nl-hat = DCT-II^3 Nl -> Nl_bar = DCT-III^3 D0 Nlq_bar
  adj_dq_kernel<T><<<blocks, 256, 0, stream_>>>(g_, vq_[0], vq_[1], vq_[2], AJ(AJ_NL), AJ(AJ_FX), AJ(AJ_FY),
                                             AJ(AJ_FZ), sine_w(0, 2.0), sine_w(1, 2.0), sine_w(2, 2.0));
  SWC_CK(cudaGetLastError());
  SWC_TRY((pass<K_C3, 2>(LdW<T>{g_, AJ(AJ_NL), w2}, SP{AJ(AJ_NL)})));
  SWC_TRY((pass<K_C3, 1>(LP{AJ(AJ_NL)}, SP{AJ(AJ_NL)})));
  SWC_TRY((pass<K_C3, 0>(LP{AJ(AJ_NL)}, SP{AJ(AJ_NL)})));
  // (3) density update + Nl in real space (REF:2121-2160)
  {
    AdjNlArgs<T> a{AJ(AJ_NL), TP(TP_PSI), TP(TP_A), TP(TP_RHOIN), TP(TP_RHONEW), TP(TP_VX), TP(TP_VY), TP(TP_VZ),
                TP(TP_GPX), TP(TP_GPY), TP(TP_GPZ), TP(TP_GRX), TP(TP_GRY), TP(TP_GRZ), TP(TP_DIVV),
                adj_ + AJ_R * ng, adj_ + AJ_F * ng, adj_ + AJ_MU * ng, adj_ + AJ_A * ng, adj_ + AJ_PSI * ng,
                adj_ + AJ_VX * ng, adj_ + AJ_VY * ng, adj_ + AJ_VZ * ng, adj_ + AJ_GPX * ng, adj_ + AJ_GPY * ng,
                adj_ + AJ_GPZ * ng, adj_ + AJ_GRX * ng, adj_ + AJ_GRY * ng, adj_ + AJ_GRZ * ng,
                adj_ + AJ_DIVV * ng, pgrad_, sc, relax ? 1 : 0};
    adj_nl_kernel<T><<<blocks, 256, 0, stream_>>>(g_, a);
    SWC_CK(cudaGetLastError());
  }
  // (4) divv = DCT-III^3 divv-hat -> divv-hat_bar = D0^-1 DCT-II^3 divv_bar;
  //     v_a = inverse mixed of v-hat_a -> v-hat_bar = W^-1 forward-mixed(v_bar)
  //     (the output weights D0^-1, W^-1 are applied where adj_stokes1_kernel reads them)
  SWC_TRY((pass<K_C2, 2>(LP{AJ(AJ_DIVV)}, SP{AJ(AJ_DIVV)})));
  SWC_TRY((pass<K_C2, 1>(LP{AJ(AJ_DIVV)}, SP{AJ(AJ_DIVV)})));
  SWC_TRY((pass<K_C2, 0>(LP{AJ(AJ_DIVV)}, SP{AJ(AJ_DIVV)})));
  {
    T* bv[3] = {adj_ + AJ_VX * ng, adj_ + AJ_VY * ng, adj_ + AJ_VZ * ng};
    SWC_TRY((pass<K_C2, 2>(LP{bv[0]}, SP{bv[0]})));
    SWC_TRY((pass<K_C2, 1>(LP{bv[0]}, SP{bv[0]})));
    SWC_TRY((pass<K_S2, 0>(LP{bv[0]}, SP{bv[0]})));
    SWC_TRY((pass<K_C2, 2>(LP{bv[1]}, SP{bv[1]})));
    SWC_TRY((pass<K_S2, 1>(LP{bv[1]}, SP{bv[1]})));
    SWC_TRY((pass<K_C2, 0>(LP{bv[1]}, SP{bv[1]})));
    SWC_TRY((pass<K_S2, 2>(LP{bv[2]}, SP{bv[2]})));
    SWC_TRY((pass<K_C2, 1>(LP{bv[2]}, SP{bv[2]})));
    SWC_TRY((pass<K_C2, 0>(LP{bv[2]}, SP{bv[2]})));
  }
  // (5) Stokes solve + divergence (REF:1468-2078)
  {
    AdjStokesArgs<T> a{AJ(AJ_VX), AJ(AJ_VY), AJ(AJ_VZ), AJ(AJ_DIVV), TP(TP_VSX), TP(TP_VSY), TP(TP_VSZ), TP(TP_VIX),
                    TP(TP_VIY), TP(TP_VIZ), adj_ + AJ_DOTX * ng, adj_ + AJ_DOTY * ng, adj_ + AJ_DOTZ * ng,
                    adj_ + AJ_SDX * ng, adj_ + AJ_SDY * ng, adj_ + AJ_SDZ * ng, adj_ + AJ_FGPX * ng,
                    adj_ + AJ_FGPY * ng, adj_ + AJ_FGPZ * ng, vq_[0], vq_[1], vq_[2], vs_[0], vs_[1], vs_[2],
                    gq_[0], gq_[1], gq_[2], gs_[0], gs_[1], gs_[2], (T)scale_, (T)(1.0 / p_.nu),
                    (T)(1.0 / (p_.lambda + 2 * p_.nu)), (T)p_.nu, (T)(p_.lambda + 2 * p_.nu), p_.nx / p_.ref_ranks,
                    sine_w(0, 0.5), sine_w(1, 0.5), sine_w(2, 0.5), wh, pgrad_};
    adj_stokes1_kernel<T><<<blocks, 256, 0, stream_>>>(g_, a);
    SWC_CK(cudaGetLastError());
    AdjStokes2Args<T> b{AJ(AJ_DOTX), AJ(AJ_DOTY), AJ(AJ_DOTZ), AJ(AJ_SDX), AJ(AJ_SDY), AJ(AJ_SDZ), AJ(AJ_FGPX),
                     AJ(AJ_FGPY), AJ(AJ_FGPZ), adj_ + AJ_SX * ng, adj_ + AJ_SY * ng, adj_ + AJ_SZ * ng,
                     adj_ + AJ_FG * ng, adj_ + AJ_E * ng, vq_[0], vq_[1], vq_[2], vs_[0], vs_[1], vs_[2],
                     gq_[0], gq_[1], gq_[2], sine_w(0, 2.0), sine_w(1, 2.0), sine_w(2, 2.0), w2};
    adj_stokes2_kernel<T><<<blocks, 256, 0, stream_>>>(g_, b);
    SWC_CK(cudaGetLastError());
  }
  // (6) forward transforms of S7 (REF:1427-1457) transposed: DCT-II^T = DCT-III D0,
  //     DST-II^T = DST-III DL, applied in place to the spectral cotangents (their
  //     producers, adj_stokes2_kernel and adj_dq_kernel, stored them times D0 / DL)
  auto cos_t = [&](T* b) -> int {
    SWC_TRY((pass<K_C3, 2>(LP{b}, SP{b})));
    SWC_TRY((pass<K_C3, 1>(LP{b}, SP{b})));
    SWC_TRY((pass<K_C3, 0>(LP{b}, SP{b})));
    return SWC_OK;
  };
  SWC_TRY(cos_t(adj_ + AJ_FG * ng));
  SWC_TRY(cos_t(adj_ + AJ_E * ng));
  for (int c = 0; c < 2; ++c) {
    T* bx = adj_ + (c == 0 ? AJ_SX : AJ_FX) * ng;
    T* by = adj_ + (c == 0 ? AJ_SY : AJ_FY) * ng;
    T* bz = adj_ + (c == 0 ? AJ_SZ : AJ_FZ) * ng;
    SWC_TRY((pass<K_C3, 2>(LP{bx}, SP{bx})));
    SWC_TRY((pass<K_C3, 1>(LP{bx}, SP{bx})));
    SWC_TRY((pass<K_S3, 0>(LP{bx}, SP{bx})));
    SWC_TRY((pass<K_C3, 2>(LP{by}, SP{by})));
    SWC_TRY((pass<K_S3, 1>(LP{by}, SP{by})));
    SWC_TRY((pass<K_C3, 0>(LP{by}, SP{by})));
    SWC_TRY((pass<K_S3, 2>(LP{bz}, SP{bz})));
    SWC_TRY((pass<K_C3, 1>(LP{bz}, SP{bz})));
    SWC_TRY((pass<K_C3, 0>(LP{bz}, SP{bz})));
  }
  // (7) S6 and the relax reset (REF:1363-1425)
  {
    AdjS6Args<T> a{AJ(AJ_FG), AJ(AJ_E), AJ(AJ_SX), AJ(AJ_SY), AJ(AJ_SZ), AJ(AJ_FX), AJ(AJ_FY), AJ(AJ_FZ), AJ(AJ_MU),
                TP(TP_LAPR), TP(TP_RHOIN), TP(TP_L), TP(TP_PSI), TP(TP_A), TP(TP_GPX), TP(TP_GPY), TP(TP_GPZ),
                TP(TP_GRX), TP(TP_GRY), TP(TP_GRZ), adj_ + AJ_GPX * ng, adj_ + AJ_GPY * ng, adj_ + AJ_GPZ * ng,
                adj_ + AJ_GRX * ng, adj_ + AJ_GRY * ng, adj_ + AJ_GRZ * ng, adj_ + AJ_A * ng, adj_ + AJ_PSI * ng,
                adj_ + AJ_R * ng, adj_ + AJ_LAPR * ng, adj_ + AJ_L * ng, pgrad_, sc, relax ? 1 : 0,
                TP(TP_RHONEW), last ? (T)energy_w_ : (T)0.0};
    adj_s6_kernel<T><<<blocks, 256, 0, stream_>>>(g_, a);
    SWC_CK(cudaGetLastError());
  }
  // (8) S5 (REF:1312-1380)
  T* blap = adj_ + AJ_LAPR * ng;
  if (!relax) {
    // lapR = Delta_s(rho L), Delta_s = DCT-III^3 (-scale q^2) DCT-II^3 is symmetric
    SWC_TRY((pass<K_C2, 2>(LP{blap}, SP{blap})));
    SWC_TRY((pass<K_C2, 1>(LP{blap}, SP{blap})));
    SWC_TRY((pass<K_FILT, 0>(LP{blap}, SP{blap}, MulLap<T>{vq_[0], vq_[1], vq_[2], (T)scale_})));
    SWC_TRY((pass<K_C3, 1>(LP{blap}, SP{blap})));
    SWC_TRY((pass<K_C3, 2>(LP{blap}, StAdjLap<T>{TP(TP_L), TP(TP_RHOIN), adj_ + AJ_R * ng, adj_ + AJ_L * ng})));
  } else {
    // lapR_raw = DCT-III^3 (-q^2 alpha (q0^2 - q^2) psiq)
    SWC_TRY((pass<K_C2, 2>(LP{blap}, SP{blap})));
    SWC_TRY((pass<K_C2, 1>(LP{blap}, SP{blap})));
    SWC_TRY((pass<K_C2, 0>(LP{blap}, SP{blap})));
    adj_acc_spec_kernel<T><<<blocks, 256, 0, stream_>>>(g_, vq_[0], vq_[1], vq_[2], 1, (T)p_.alpha,
                                                     (T)(p_.q0 * p_.q0), wh, blap, TP(TP_QOLD), AJ(AJ_Q),
                                                     pgrad_);
    SWC_CK(cudaGetLastError());
  }
  // (9) dfDlapPsi = DCT-III^3 (alpha (q0^2 - q^2) psiq)  (REF:1293-1308)
  {
    T* bl = adj_ + AJ_L * ng;
    SWC_TRY((pass<K_C2, 2>(LP{bl}, SP{bl})));
    SWC_TRY((pass<K_C2, 1>(LP{bl}, SP{bl})));
    SWC_TRY((pass<K_C2, 0>(LP{bl}, SP{bl})));
    adj_acc_spec_kernel<T><<<blocks, 256, 0, stream_>>>(g_, vq_[0], vq_[1], vq_[2], 0, (T)p_.alpha,
                                                     (T)(p_.q0 * p_.q0), wh, bl, TP(TP_QOLD), AJ(AJ_Q), pgrad_);
    SWC_CK(cudaGetLastError());
  }
  // (10) amplitude filter A = F(A_raw) (symmetric) and A_raw = |psi, grad psi| (REF:1254-1289)
  {
    T* bA = adj_ + AJ_A * ng;
    SWC_TRY((pass<K_C2, 2>(LP{bA}, SP{bA})));
    SWC_TRY((pass<K_C2, 1>(LP{bA}, SP{bA})));
    SWC_TRY((pass<K_FILT, 0>(LP{bA}, SP{bA}, MulGauss<T>{gq_[0], gq_[1], gq_[2], (T)scale_})));
    SWC_TRY((pass<K_C3, 1>(LP{bA}, SP{bA})));
    SWC_TRY((pass<K_C3, 2>(LP{bA}, SP{bA})));
    adj_amp_kernel<T><<<blocks, 256, 0, stream_>>>(g_, bA, TP(TP_PSI), TP(TP_GPX), TP(TP_GPY), TP(TP_GPZ),
                                                (T)(p_.q0 * p_.q0), AJ(AJ_PSI), AJ(AJ_GPX), AJ(AJ_GPY),
                                                AJ(AJ_GPZ));
    SWC_CK(cudaGetLastError());
  }
  // (11) gradients (REF:1166-1250): the forward takes grad_a psi and grad_a rho with one
  //      derivative pass along axis a each (DCT-II, shifted multiply, DST-III); their
  //      transposes are one pass each of the transposed kind (DST-II, transposed shift,
  //      DCT-III), summed into psi_bar and rho_bar by adj_gsum_kernel
  {
    const T cx = (T)(1.0 / (2.0 * g_.nx)), cy = (T)(1.0 / (2.0 * g_.ny)), cz = (T)(1.0 / (2.0 * g_.nz));
    T* bgp[3] = {AJ(AJ_GPX), AJ(AJ_GPY), AJ(AJ_GPZ)};
    T* bgr[3] = {AJ(AJ_GRX), AJ(AJ_GRY), AJ(AJ_GRZ)};
    for (T* const* b : {bgp, bgr}) {
      SWC_TRY((pass<K_DERIVT, 2>(LP{b[2]}, SP{b[2]}, MulDeriv<T>{vs_[2], cz, 2})));
      SWC_TRY((pass<K_DERIVT, 1>(LP{b[1]}, SP{b[1]}, MulDeriv<T>{vs_[1], cy, 1})));
      SWC_TRY((pass<K_DERIVT, 0>(LP{b[0]}, SP{b[0]}, MulDeriv<T>{vs_[0], cx, 0})));
    }
    adj_gsum_kernel<T><<<blocks, 256, 0, stream_>>>(g_, bgp[0], bgp[1], bgp[2], bgr[0], bgr[1], bgr[2], AJ(AJ_PSI),
                                                 AJ(AJ_R));
    SWC_CK(cudaGetLastError());
  }
  // (13) the step's psi = DCT-III^3 psiq: psiq_bar += D0^-1 DCT-II^3 psi_bar
  T* bp = adj_ + AJ_PSI * ng;
  SWC_TRY((pass<K_C2, 2>(LP{bp}, SP{bp})));
  SWC_TRY((pass<K_C2, 1>(LP{bp}, SP{bp})));
  SWC_TRY((pass<K_C2, 0>(LP{bp}, SP{bp})));
  adj_fold_kernel<T><<<blocks, 256, 0, stream_>>>(g_, bp, wh, AJ(AJ_Q));
  SWC_CK(cudaGetLastError());
  return SWC_OK;
}

// Host FP64 field <-> device field of the engine's precision (the mixed engine goes
// through the FP64 staging buffer and narrows / widens on the device).
template <typename T> int StepEngine<T>::host_to_field(const double* src, T* dst) {
  const size_t ng = (size_t)g_.ng;
  if constexpr (std::is_same<T, double>::value) {
    SWC_CK(cudaMemcpyAsync(dst, src, ng * 8, cudaMemcpyHostToDevice, stream_));
  } else {
    SWC_TRY(stage_alloc());
    SWC_CK(cudaMemcpyAsync(stage_, src, ng * 8, cudaMemcpyHostToDevice, stream_));
    narrow_kernel<<<(unsigned)((ng / 4 + 255) / 256), 256, 0, stream_>>>(stage_, dst, (long long)ng);
    SWC_CK(cudaGetLastError());
  }
  return SWC_OK;
}
template <typename T> int StepEngine<T>::field_to_host(const T* src, double* dst) {
  const size_t ng = (size_t)g_.ng;
  if constexpr (std::is_same<T, double>::value) {
    SWC_CK(cudaMemcpyAsync(dst, src, ng * 8, cudaMemcpyDeviceToHost, stream_));
  } else {
    SWC_TRY(stage_alloc());
    widen_kernel<<<(unsigned)((ng / 4 + 255) / 256), 256, 0, stream_>>>(src, stage_, (long long)ng);
    SWC_CK(cudaGetLastError());
    SWC_CK(cudaMemcpyAsync(dst, stage_, ng * 8, cudaMemcpyDeviceToHost, stream_));
  }
  return SWC_OK;
}

// Step n (1-based) from the loaded state n-1 with its tape (slot 0), then its adjoint.
template <typename T> int StepEngine<T>::tape_and_adjoint(int64_t n) {
  SWC_TRY(record_tape(tape_, n, true));
  const bool relax = !(n > p_.divv_switch || p_.load == 1);
  tape_alias_on_ = true;
  const int rc = adjoint_step(0, relax, n == 1, n == nloop_);
  tape_alias_on_ = false;
  return rc;
}

// Run step n (1-based) from the loaded state n-1 and copy the fields its adjoint reads
// into the tape slot tp; the mixed engine's FP64 state fields are narrowed to FP32.
// alias: the adjoint of step n runs next, so the fields that hold their taped values
// until then (every one but the incoming density, and the narrowed FP64 state) are
// left where the step wrote them and read in place (tape_alias_).
template <typename T> int StepEngine<T>::record_tape(T* tp, int64_t n, bool alias) {
  const size_t ng = (size_t)g_.ng;
  constexpr bool mixed = !std::is_same<T, double>::value;
  int packed = 0;  // alias mode: the copied fields sit one after another in tp
  auto put = [&](int q, const void* src, bool is_double) -> int {
    T* dst = tp + (size_t)(alias ? packed++ : q) * ng;
    if (alias) tape_alias_[q] = dst;
    if (mixed && is_double) {
      narrow_kernel<<<(unsigned)((ng / 4 + 255) / 256), 256, 0, stream_>>>((const double*)src, (float*)dst,
                                                                           (long long)ng);
      SWC_CK(cudaGetLastError());
    } else {
      SWC_CK(cudaMemcpyAsync(dst, src, ng * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
    }
    return SWC_OK;
  };
  for (int q = 0; q < kTape; ++q) tape_alias_[q] = nullptr;
  SWC_TRY(put(TP_RHOIN, rho_, true));
  const bool relax = !(n > p_.divv_switch || p_.load == 1);
  // the diagnostic variant keeps the input psi in psi_old and writes v_sol; the tape
  // variant (alias mode: nothing runs between this step and its adjoint) writes v_sol and
  // leaves the input psi in psi_, without the diagnostic reductions
  if (alias) SWC_TRY(run_graph(relax, n == 1, false, true, true));
  else SWC_TRY(run_graph(relax, n == 1, true, true));
  const void* src[kTape] = {alias ? psi_ : psi_old_, psiq_old_, psiq_, gp_[0], gp_[1], gp_[2], gr_[0], gr_[1], gr_[2],
                            amp_f_, lpsi_, lapR_, nullptr, rho_, v_[0], v_[1], v_[2], divv_, vsol_[0],
                            vsol_[1], vsol_[2], virr_[0], virr_[1], virr_[2]};
  for (int q = 0; q < kTape; ++q) {
    if (!src[q]) continue;
    const bool is_double = q == TP_QOLD || q == TP_QNEW || q == TP_RHONEW;
    if (alias && !(mixed && is_double)) tape_alias_[q] = static_cast<const T*>(src[q]);
    else SWC_TRY(put(q, src[q], is_double));
  }
  ++fwd_steps_;
  return SWC_OK;
}

// k plain forward steps from the loaded state `from` (steps from+1 .. from+k).
template <typename T> int StepEngine<T>::advance(int64_t from, int64_t k) {
  for (int64_t n = from + 1; n <= from + k; ++n) {
    const bool relax = !(n > p_.divv_switch || p_.load == 1);
    SWC_TRY(run_graph(relax, n == 1, false, false));
  }
  fwd_steps_ += k;
  return SWC_OK;
}

// C(s + t, t), saturating: the most steps s held states reverse with each step
// advanced at most t times.
static inline int64_t binomial_reach(int64_t s, int64_t t) {
  double c = 1.0;
  for (int64_t i = 1; i <= t; ++i) {
    c = c * (double)(s + i) / (double)i;
    if (c > 9.0e18) return INT64_MAX;
  }
  return (int64_t)(c + 0.5);
}

// Reverse steps l+1 .. l+n given state l in checkpoint slot sl, with nfree snapshot slots
// ff, ff+1, ... free: place one snapshot where the binomial split puts it, reverse the
// right part with one slot less, then the left part with the slot back.
template <typename T>
int StepEngine<T>::reverse_binomial(int64_t l, int64_t n, size_t sl, size_t ff, int64_t nfree) {
  if (n <= 0) return SWC_OK;
  if (n == 1) {
    SWC_TRY(restore_ckpt(sl));
    return tape_and_adjoint(l + 1);
  }
  if (nfree == 0) {
    for (int64_t k = n; k >= 1; --k) {
      SWC_TRY(restore_ckpt(sl));
      SWC_TRY(advance(l, k - 1));
      SWC_TRY(tape_and_adjoint(l + k));
    }
    return SWC_OK;
  }
  // optimal first split (Griewank): with S = nfree + 1 states held (the loaded one
  // counts) and t the least integer with C(S + t, t) >= n, advance
  // m = max(n - C(S - 1 + t, t), C(S + t - 2, t - 2)) steps (within [1, n - 1]) before
  // the next snapshot; the reversal then costs t n - C(S + t, t - 1) advances in all
  int64_t t = 0;
  while (binomial_reach(nfree + 1, t) < n) ++t;
  int64_t m = n - std::min<int64_t>(n, binomial_reach(nfree, t));
  if (t >= 2) m = std::max<int64_t>(m, binomial_reach(nfree + 1, t - 2));
  m = std::min<int64_t>(std::max<int64_t>(m, 1), n - 1);
  const int64_t right = n - m;
  SWC_TRY(restore_ckpt(sl));
  SWC_TRY(advance(l, m));
  SWC_TRY(save_ckpt(ff, false));
  SWC_TRY(reverse_binomial(l + m, right, ff, ff + 1, nfree - 1));
  return reverse_binomial(l, m, sl, ff, nfree);
}

template <typename T>
int StepEngine<T>::backward_impl(const double* dpsi, const double* drho, double energy_lambda, double* dpsi0,
                                 double* drho0, swc_grad* out) {
  const int K = p_.adjoint_ckpt;
  if (K == 0) {
    set_error("swc_backward needs params.adjoint_ckpt > 0 or -1 at swc_create");
    return SWC_ERR_BAD_PARAM;
  }
  const bool binomial = K < 0;
  if (!have_state_ || !adj_valid_) {
    set_error("swc_backward: no trajectory from swc_set_state to differentiate");
    return SWC_ERR_STATE;
  }
  SWC_CK(cudaSetDevice(p_.device));
  SWC_TRY(finish_steps());  // steps enqueued by swc_step_async: their status first
  if (vsol_pending_) {  // the recompute below reuses the spectral v_sol buffers
    SWC_TRY(transform_vsol());
    vsol_pending_ = false;
  }
  SWC_CK(cudaStreamSynchronize(stream_));
  const size_t ng = (size_t)g_.ng;
  const int64_t Tn = nloop_;
  constexpr bool mixed = !std::is_same<T, double>::value;
  const size_t tape_fields = binomial ? (size_t)kTapeCopied(mixed)
                                      : (size_t)(Tn < K ? (Tn > 0 ? Tn : 1) : K) * kTape;
  SWC_TRY(adjoint_alloc(tape_fields));
  // the final state, restored when the call returns (slot past the trajectory's)
  const size_t last_slot = binomial ? 1 : (size_t)(Tn / K) + 1;
  SWC_TRY(save_ckpt(last_slot));
  int64_t nsnap = 0;
  if (binomial) {
    // snapshot slots under the cap: engine arrays + adjoint work + tape + slots 0, 1
    // (allocated) + s snapshots without psi
    const size_t slot_bytes = ckpt_slot_bytes(false);
    size_t held = 0;
    for (size_t b : ckpt_bytes_) held += b;
    const size_t used = engine_bytes_ + (size_t)kAdj * ng * sizeof(T) + pgrad_doubles() * 8 +
                        tape_fields_ * ng * sizeof(T) + held + (stage_ ? ng * 8 : 0);
    double cap = p_.adjoint_cap_gb * 1e9;
    if (cap <= 0) {
      size_t fr = 0, tot = 0;
      SWC_CK(cudaMemGetInfo(&fr, &tot));
      cap = (double)used + (double)fr - 1e9;
    }
    if (cap < (double)used) {
      set_error("adjoint_cap_gb %.3f is below the %.3f GB the reversal needs before any snapshot",
                p_.adjoint_cap_gb, (double)used / 1e9);
      return SWC_ERR_OOM;
    }
    nsnap = (int64_t)((cap - (double)used) / (double)slot_bytes);
    nsnap = std::min<int64_t>(nsnap, std::max<int64_t>(Tn - 1, 0));  // one per step is the most useful
    if (p_.adjoint_snapshots > 0) nsnap = std::min<int64_t>(nsnap, p_.adjoint_snapshots);
  }
  fwd_steps_ = 0;
  auto AJ = [&](int q) { return adj_ + (size_t)q * ng; };
  SWC_CK(cudaMemsetAsync(adj_, 0, (size_t)kAdj * ng * sizeof(T), stream_));
  SWC_CK(cudaMemsetAsync(pgrad_, 0, pgrad_doubles() * sizeof(double), stream_));
  // the final step's L and A (read by the energy term; the recompute overwrites them)
  SWC_CK(cudaMemcpyAsync(AJ(AJ_KEEPL), lpsi_, ng * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
  SWC_CK(cudaMemcpyAsync(AJ(AJ_KEEPA), amp_f_, ng * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
  // cotangent of the final state: psi(T) = DCT-III^3 psiq(T), rho(T), plus lambda times
  // that of the free-energy diagnostic of step T (REF:2214-2258)
  if (dpsi) SWC_TRY(host_to_field(dpsi, AJ(AJ_PSI)));
  if (drho) SWC_TRY(host_to_field(drho, AJ(AJ_R)));
  energy_w_ = energy_lambda * dx_ * dx_ * dx_;  // the diagnostic's dx^3 (REF:2258)
  if (energy_lambda != 0.0) {
    const AdjScalars<T> sc{(T)p_.ep, (T)p_.alpha, (T)p_.beta, (T)p_.gamma, (T)p_.zeta, (T)kp_, (T)p_.rho_0,
                           (T)(p_.q0 * p_.q0), (T)p_.dt, (T)(p_.dt / 2), (T)rho_m_, (T)scale_, (T)p_.nu,
                           (T)(p_.lambda + 2 * p_.nu)};
    adj_energy_final_kernel<T><<<pt4_blocks(g_), 256, 0, stream_>>>(
        g_, psi_, rho_, AJ(AJ_KEEPL), AJ(AJ_KEEPA), (T)energy_w_, sc, AJ(AJ_PSI), AJ(AJ_R), pgrad_);
    SWC_CK(cudaGetLastError());
  }
  if (dpsi || energy_lambda != 0.0) {
    using LP = LdPlain<T, T>;
    using SP = StPlain<T, T>;
    const AxisWeights<T> wh{{0, 0, 0}, (T)0.5};
    SWC_TRY((pass<K_C2, 2>(LP{AJ(AJ_PSI)}, SP{AJ(AJ_PSI)})));
    SWC_TRY((pass<K_C2, 1>(LP{AJ(AJ_PSI)}, SP{AJ(AJ_PSI)})));
    SWC_TRY((pass<K_C2, 0>(LP{AJ(AJ_PSI)}, StW<T>{g_, AJ(AJ_Q), wh, 0})));
  }
  if (binomial) {
    SWC_TRY(reverse_binomial(0, Tn, 0, 2, nsnap));
  } else {
    // segments [s0, s1), last first
    const int64_t nseg = (Tn + K - 1) / K;
    for (int64_t sg = nseg - 1; sg >= 0; --sg) {
      const int64_t s0 = sg * K, s1 = std::min<int64_t>(s0 + K, Tn);
      SWC_TRY(restore_ckpt((size_t)sg));
      for (int64_t n = s0 + 1; n <= s1; ++n) SWC_TRY(record_tape(tape_ + (size_t)(n - s0 - 1) * kTape * ng, n));
      for (int64_t n = s1; n > s0; --n) {
        const bool relax = !(n > p_.divv_switch || p_.load == 1);
        SWC_TRY(adjoint_step((size_t)(n - s0 - 1), relax, n == 1, n == Tn));
      }
    }
  }
  // swc_set_state: psiq0 = scale DCT-II^3 psi0 = psiq_old0  =>  psi0_bar = scale DCT-III^3 D0 (Q_bar + Qo_bar)
  const unsigned blocks = (unsigned)((g_.ng + 255) / 256);
  if (dpsi0) {
    axpby_kernel<T><<<blocks, 256, 0, stream_>>>(g_.ng, (T)1.0, AJ(AJ_Q), (T)1.0, AJ(AJ_QO), AJ(AJ_PSI));
    SWC_CK(cudaGetLastError());
    using LP = LdPlain<T, T>;
    using SP = StPlain<T, T>;
    const AxisWeights<T> w2{{0, 0, 0}, (T)2.0};
    SWC_TRY((pass<K_C3, 2>(LdW<T>{g_, AJ(AJ_PSI), w2}, SP{AJ(AJ_PSI)})));
    SWC_TRY((pass<K_C3, 1>(LP{AJ(AJ_PSI)}, SP{AJ(AJ_PSI)})));
    SWC_TRY((pass<K_C3, 0>(LP{AJ(AJ_PSI)}, SP{AJ(AJ_PSI)})));
    axpby_kernel<T><<<blocks, 256, 0, stream_>>>(g_.ng, (T)scale_, AJ(AJ_PSI), (T)0.0, nullptr, AJ(AJ_PSI));
    SWC_CK(cudaGetLastError());
    SWC_TRY(field_to_host(AJ(AJ_PSI), dpsi0));
  }
  if (drho0) SWC_TRY(field_to_host(AJ(AJ_R), drho0));
  pg_reduce_kernel<<<PG_COUNT, 256, 0, stream_>>>(pgrad_, blocks);
  SWC_CK(cudaGetLastError());
  double pg[PG_COUNT];
  SWC_CK(cudaMemcpyAsync(pg, pgrad_, sizeof(pg), cudaMemcpyDeviceToHost, stream_));
  SWC_TRY(restore_ckpt(last_slot));
  SWC_CK(cudaMemcpyAsync(lpsi_, AJ(AJ_KEEPL), ng * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
  SWC_CK(cudaMemcpyAsync(amp_f_, AJ(AJ_KEEPA), ng * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
  diag_step_ = -1;  // the recompute overwrote the energy density and the sums
  pending_diag_ = -1;
  SWC_CK(cudaStreamSynchronize(stream_));
  // chain rule through Amp(beta, gamma) and kp = (1 - rho_0)/Amp (REF:250-253); rho_s = 1, rho_m = 1/2
  const double disc = std::sqrt(9 * p_.beta * p_.beta + 40 * p_.ep * p_.gamma);
  const double dAmp_dX = 1.0 / (10.0 * amp_);
  const double dAmp_dbeta = dAmp_dX * (3.0 + 9.0 * p_.beta / disc);
  const double dAmp_dgamma = dAmp_dX * (20.0 * p_.ep / disc);
  const double dkp_dAmp = -kp_ / amp_, dkp_drho0 = -1.0 / amp_;
  out->alpha = pg[PG_ALPHA];
  out->beta = pg[PG_BETA] + pg[PG_KP] * dkp_dAmp * dAmp_dbeta;
  out->gamma = pg[PG_GAMMA] + pg[PG_KP] * dkp_dAmp * dAmp_dgamma;
  out->nu = pg[PG_NU];
  out->rho_0 = pg[PG_RHO0] + pg[PG_KP] * dkp_drho0;
  out->steps = Tn;
  out->forward_steps = fwd_steps_;
  out->snapshots = nsnap;
  return SWC_OK;
}

}  // namespace swc
