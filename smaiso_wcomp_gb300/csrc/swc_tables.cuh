// swc_tables.cuh -- per-length twiddle tables and pass shapes of the r2r kernels.
#pragma once

#include <cmath>
#include <vector>

#include "swc_r2r.cuh"
#include "swc_r2r_tma.cuh"

namespace swc {

inline bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
inline int ilog2(long long n) {
  int l = 0;
  while ((1LL << l) < n) ++l;
  return l;
}

// Stockham radix schedule of an M-point FFT (largest radix first).
inline void radix_plan(int M, int* radix, int& nst) {
  nst = 0;
  switch (M) {
    case 2: radix[nst++] = 2; break;
    case 4: radix[nst++] = 4; break;
    case 8: radix[nst++] = 8; break;
    case 16: radix[nst++] = 16; break;
    case 32: radix[nst++] = 8; radix[nst++] = 4; break;
    case 64: radix[nst++] = 8; radix[nst++] = 8; break;
    case 128: radix[nst++] = 16; radix[nst++] = 8; break;
    case 256: radix[nst++] = 16; radix[nst++] = 16; break;
    case 512: radix[nst++] = 16; radix[nst++] = 8; radix[nst++] = 4; break;
    default: nst = 0; break;
  }
}

// Shape of a pass over an array whose `axis` has length n, for element size `elem`.
inline PassShape make_shape(const Grid& g, int axis, size_t elem) {
  PassShape ps{};
  const int dims[3] = {g.nx, g.ny, g.nz};
  ps.n = dims[axis];
  ps.log2n = ilog2(ps.n);
  ps.axis = axis;
  const int M = ps.n / 2;
  radix_plan(M, ps.radix, ps.nst);
  int rmax = 1;
  for (int s = 0; s < ps.nst; ++s) rmax = ps.radix[s] > rmax ? ps.radix[s] : rmax;
  ps.tpl = M / rmax;
  ps.nlines = g.ng / ps.n;
  int L = 64;
  while (L > 1 && (L * ps.tpl > 256 || (L > 16 && L * ps.tpl > 128) ||
                   (2 * (size_t)M * (L + 1) + 5 * (size_t)M + 2) * 2 * elem > 80 * 1024 || L > ps.nlines))
    L >>= 1;
  ps.L = L;
  ps.log2L = ilog2(L);
  ps.P = L + 1;
  return ps;
}

// Host computation of the tables of one length n in double, converted to T.
//   fft[t]  = exp(-2 pi i t/M)
//   post[2k] = c_k = t_k (1 - i W_k),  post[2k+1] = d_k = t_k (1 + i W_k),
//              t_k = exp(-i pi k/2n), W_k = exp(-2 pi i k/n)   (k = 0..M; factor 2 folded)
//   pre[2k]  = a_k = (1 + i W'_k) exp(i pi k/2n), pre[2k+1] = b_k = (1 - i W'_k) exp(-i pi (M-k)/2n),
//              W'_k = exp(2 pi i k/n)                            (k < M)
template <typename T> struct HostTables {
  std::vector<T> fft, post, pre;  // interleaved (re, im)
  explicit HostTables(int n) {
    const int M = n / 2;
    const double pi = 3.14159265358979323846;
    fft.resize(2 * M);
    for (int t = 0; t < M; ++t) {
      fft[2 * t] = (T)std::cos(-2.0 * pi * t / M);
      fft[2 * t + 1] = (T)std::sin(-2.0 * pi * t / M);
    }
    post.resize(4 * (M + 1));
    for (int k = 0; k <= M; ++k) {
      const double tr = std::cos(-pi * k / (2.0 * n)), ti = std::sin(-pi * k / (2.0 * n));
      const double wr = std::cos(-2.0 * pi * k / n), wi = std::sin(-2.0 * pi * k / n);
      // i W = (-wi, wr);  1 - iW = (1 + wi, -wr);  1 + iW = (1 - wi, wr)
      const double cr = tr * (1 + wi) - ti * (-wr), ci = tr * (-wr) + ti * (1 + wi);
      const double dr = tr * (1 - wi) - ti * wr, di = tr * wr + ti * (1 - wi);
      post[4 * k] = (T)cr; post[4 * k + 1] = (T)ci;
      post[4 * k + 2] = (T)dr; post[4 * k + 3] = (T)di;
    }
    pre.resize(4 * M);
    for (int k = 0; k < M; ++k) {
      const double wr = std::cos(2.0 * pi * k / n), wi = std::sin(2.0 * pi * k / n);
      const double er = std::cos(pi * k / (2.0 * n)), ei = std::sin(pi * k / (2.0 * n));
      const double fr = std::cos(-pi * (M - k) / (2.0 * n)), fi = std::sin(-pi * (M - k) / (2.0 * n));
      // 1 + iW' = (1 - wi, wr); 1 - iW' = (1 + wi, -wr)
      const double ar = (1 - wi) * er - wr * ei, ai = (1 - wi) * ei + wr * er;
      const double br = (1 + wi) * fr - (-wr) * fi, bi = (1 + wi) * fi + (-wr) * fr;
      pre[4 * k] = (T)ar; pre[4 * k + 1] = (T)ai;
      pre[4 * k + 2] = (T)br; pre[4 * k + 3] = (T)bi;
    }
  }
};

template <typename U, int N, int KIND, int AX, class LD, class ST, class MUL>
cudaError_t launch_fast(const Grid& g, const R2RTables<U>& tb, cudaStream_t stream, LD ld, ST st, MUL mul) {
  using Cf = FastCfg<U, N>;
  const size_t smem = Cf::smem_bytes();
  auto kern = r2r_fast_kernel<U, N, KIND, AX, LD, ST, MUL>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const unsigned blocks = (unsigned)((g.ng / N) / Cf::L);
  kern<<<blocks, Cf::NT, smem, stream>>>(g, tb, ld, st, mul);
  return cudaGetLastError();
}

template <int N, int KIND, int AX, class LD, class ST, class MUL>
cudaError_t launch_pair(const Grid& g, const R2RTables<float>& tb, cudaStream_t stream, LD ld, ST st, MUL mul) {
  using Cf = PairCfg<N>;
  const size_t smem = Cf::smem_bytes();
  auto kern = r2r_pair_kernel<N, KIND, AX, LD, ST, MUL>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const unsigned blocks = (unsigned)((g.ng / N) / (2 * Cf::LP));
  kern<<<blocks, Cf::NT, smem, stream>>>(g, tb, ld, st, mul);
  return cudaGetLastError();
}

template <class F> struct IsLdMul : std::false_type {};
template <class M> struct IsLdMul<LdMul<M>> : std::true_type {};

// Whether launch_pass runs a pass in the TMA-fed form (on the shapes that form supports):
// the one form that honours R2RTables::rev.
template <typename U, int KIND, int AX, class LD> constexpr bool tma_fed_form() {
  return std::is_same<U, float>::value &&
         (std::is_same<LD, LdPlain<float, float>>::value || (IsLdMul<LD>::value && AX == 2 && KIND == K_C3));
}

// Launch one axis pass on `stream` (in place or out of place per the functors): for
// line lengths 64..512 the compile-time kernels (FP32: two lines per thread with packed
// arithmetic; FP64: one line per thread group), the runtime one otherwise.
template <typename U, int KIND, int AX, class LD, class ST, class MUL>
cudaError_t launch_pass(const Grid& g, const R2RTables<U>& tb, cudaStream_t stream, LD ld, ST st, MUL mul) {
  constexpr int axis = AX;
  const int dims[3] = {g.nx, g.ny, g.nz};
  const int n = dims[axis];
  if constexpr (std::is_same<U, float>::value && std::is_same<LD, LdPlain<float, float>>::value) {
    // plain FP32 input: TMA-fed persistent pass
    if (n == 256 && tma_pass_supported<256>(g, axis))
      return launch_tma<256, KIND, AX, ST, MUL>(g, tb, stream, ld.p, st, mul);
    if (n == 128 && tma_pass_supported<128>(g, axis))
      return launch_tma<128, KIND, AX, ST, MUL>(g, tb, stream, ld.p, st, mul);
    if (n == 512 && tma_pass_supported<512>(g, axis))
      return launch_tma<512, KIND, AX, ST, MUL>(g, tb, stream, ld.p, st, mul);
    if (n == 64 && tma_pass_supported<64>(g, axis))
      return launch_tma<64, KIND, AX, ST, MUL>(g, tb, stream, ld.p, st, mul);
  } else if constexpr (std::is_same<U, float>::value && IsLdMul<LD>::value && AX == 2 && KIND == K_C3) {
    // plain FP32 input times a pointwise multiplier: TMA-fed, applied to the staged tile
    if (n == 256 && tma_pass_supported<256>(g, axis))
      return launch_tma<256, KIND, AX, ST, MUL>(g, tb, stream, ld.p, st, mul, ld.m);
    if (n == 128 && tma_pass_supported<128>(g, axis))
      return launch_tma<128, KIND, AX, ST, MUL>(g, tb, stream, ld.p, st, mul, ld.m);
    if (n == 512 && tma_pass_supported<512>(g, axis))
      return launch_tma<512, KIND, AX, ST, MUL>(g, tb, stream, ld.p, st, mul, ld.m);
    if (n == 64 && tma_pass_supported<64>(g, axis))
      return launch_tma<64, KIND, AX, ST, MUL>(g, tb, stream, ld.p, st, mul, ld.m);
    if (n == 256 && pair_pass_supported<256>(g, axis))
      return launch_pair<256, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
    if (n == 128 && pair_pass_supported<128>(g, axis))
      return launch_pair<128, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
    if (n == 512 && pair_pass_supported<512>(g, axis))
      return launch_pair<512, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
    if (n == 64 && pair_pass_supported<64>(g, axis))
      return launch_pair<64, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
  } else if constexpr (std::is_same<U, float>::value) {
    // fused FP32 loaders: two lines per thread, direct loads
    if (n == 256 && pair_pass_supported<256>(g, axis))
      return launch_pair<256, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
    if (n == 128 && pair_pass_supported<128>(g, axis))
      return launch_pair<128, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
    if (n == 512 && pair_pass_supported<512>(g, axis))
      return launch_pair<512, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
    if (n == 64 && pair_pass_supported<64>(g, axis))
      return launch_pair<64, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
  } else {
    if (n == 256 && fast_pass_supported<U, 256>(g, axis))
      return launch_fast<U, 256, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
    if (n == 128 && fast_pass_supported<U, 128>(g, axis))
      return launch_fast<U, 128, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
    if (n == 512 && fast_pass_supported<U, 512>(g, axis))
      return launch_fast<U, 512, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
    if (n == 64 && fast_pass_supported<U, 64>(g, axis))
      return launch_fast<U, 64, KIND, AX, LD, ST, MUL>(g, tb, stream, ld, st, mul);
  }
  {
    const PassShape ps = make_shape(g, axis, sizeof(U));
    const size_t smem = pass_smem_bytes(ps, sizeof(U));
    auto kern = r2r_pass_kernel<U, KIND, 0, LD, ST, MUL>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    const unsigned blocks = (unsigned)(ps.nlines / ps.L);
    kern<<<blocks, ps.L * ps.tpl, smem, stream>>>(g, ps, tb, ld, st, mul);
    return cudaGetLastError();
  }
}

}  // namespace swc
