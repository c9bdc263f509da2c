// swc_r2r_pair.cuh -- the FP32 r2r axis pass with two lines per thread.
//
// Same transform, kinds, Makhoul mapping and Stockham plan as r2r_fast_kernel
// (swc_r2r_fast.cuh), but every thread carries the same butterfly of two adjacent
// lines A and B in "planar pair" registers: PC = {re = (re_A, re_B), im = (im_A, im_B)}.
// All arithmetic is then sm_100+ packed FP32 (FADD2 / FMUL2 / FFMA2 through
// __fadd2_rn / __fmul2_rn / __ffma2_rn), one instruction for both lines, with the
// twiddles broadcast to both halves from float4 tables {c, c, s, s} in shared memory.
// Global traffic is vectorised too: x/y passes load and store (A, B) as one float2
// (adjacent lines are adjacent addresses), z passes move four consecutive elements of
// a line as one float4 and scatter them into Makhoul order in registers.
#pragma once

#include <type_traits>
#include <utility>

#include "swc_r2r_fast.cuh"

// Radix plan of the 256-point lines: 1 = 16 x 8 (8 threads per line pair, 128-thread
// CTAs), 2 = 8 x 4 x 4 (16 threads per line pair, 256-thread CTAs: twice the warps for
// the same tile, one more shared-memory exchange). Measured on GB300 at 256^3: plan 1
// 0.0289 ms per pass, plan 2 0.0314 ms.
#ifndef SWC_PAIR_PLAN256
#define SWC_PAIR_PLAN256 1
#endif

namespace swc {

// ---- packed FP32 helpers -------------------------------------------------------------

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as a + (-1) b: exact product, one rounding, same as a subtraction
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

struct PC {
  float2 re, im;
};
__device__ __forceinline__ PC pmake(float2 re, float2 im) { PC r; r.re = re; r.im = im; return r; }
__device__ __forceinline__ PC padd(PC a, PC b) { return pmake(add2(a.re, b.re), add2(a.im, b.im)); }
__device__ __forceinline__ PC psub(PC a, PC b) { return pmake(sub2(a.re, b.re), sub2(a.im, b.im)); }
__device__ __forceinline__ PC pswap(PC a) { return pmake(a.im, a.re); }
// v * w for a twiddle w = (x, y) held as {x, x, y, y}
__device__ __forceinline__ PC pmul(PC v, float4 w) {
  const float2 wx = make_float2(w.x, w.y), wy = make_float2(w.z, w.w);
  return pmake(fma2(v.re, wx, mul2(v.im, neg2(wy))), fma2(v.re, wy, mul2(v.im, wx)));
}
// w * conj(v)
__device__ __forceinline__ PC pmulc(float4 w, PC v) {
  const float2 wx = make_float2(w.x, w.y), wy = make_float2(w.z, w.w);
  return pmake(fma2(v.re, wx, mul2(v.im, wy)), fma2(v.re, wy, mul2(v.im, neg2(wx))));
}
// a * x + b * conj(y)   (the Makhoul pre/post combination)
__device__ __forceinline__ PC pcomb(float4 a, PC x, float4 b, PC y) {
  const float2 ax = make_float2(a.x, a.y), ay = make_float2(a.z, a.w);
  const float2 bx = make_float2(b.x, b.y), by = make_float2(b.z, b.w);
  const float2 re = fma2(x.re, ax, fma2(x.im, neg2(ay), fma2(y.re, bx, mul2(y.im, by))));
  const float2 im = fma2(x.im, ax, fma2(x.re, ay, fma2(y.re, by, mul2(y.im, neg2(bx)))));
  return pmake(re, im);
}
// the same with the table entries a = (x, y), b = (x, y) broadcast to both lines
__device__ __forceinline__ PC pcomb(float2 a, PC x, float2 b, PC y) {
  return pcomb(make_float4(a.x, a.x, a.y, a.y), x, make_float4(b.x, b.x, b.y, b.y), y);
}

// ---- register DFT on planar pairs (forward, exp(-2 pi i/R)) ---------------------------

template <int R> struct PDft {
  // butterfly K of the radix-2 combine: v[K] = e + W^K o, v[K + R/2] = e - W^K o
  template <int K> __device__ __forceinline__ static void combine(PC* v, const PC* e, const PC* o) {
    if constexpr (K < R / 2) {
      constexpr int k16 = K * (16 / R);
      const PC a = e[K], b = o[K];
      if constexpr (k16 == 0) {
        v[K] = padd(a, b);
        v[K + R / 2] = psub(a, b);
      } else if constexpr (k16 == 4) {  // W = -i: t = (b.im, -b.re)
        v[K] = pmake(add2(a.re, b.im), sub2(a.im, b.re));
        v[K + R / 2] = pmake(sub2(a.re, b.im), add2(a.im, b.re));
      } else if constexpr (k16 == 2) {  // W = (1 - i)/sqrt2: t = r (b.re + b.im, b.im - b.re)
        const float2 s1 = add2(b.re, b.im), s2 = sub2(b.im, b.re);
        const float2 r = f2((float)SWC_R2H), nr = f2(-(float)SWC_R2H);
        v[K] = pmake(fma2(s1, r, a.re), fma2(s2, r, a.im));
        v[K + R / 2] = pmake(fma2(s1, nr, a.re), fma2(s2, nr, a.im));
      } else if constexpr (k16 == 6) {  // W = (-1 - i)/sqrt2: t = r (b.im - b.re, -(b.re + b.im))
        const float2 s1 = add2(b.re, b.im), s2 = sub2(b.im, b.re);
        const float2 r = f2((float)SWC_R2H), nr = f2(-(float)SWC_R2H);
        v[K] = pmake(fma2(s2, r, a.re), fma2(s1, nr, a.im));
        v[K + R / 2] = pmake(fma2(s2, nr, a.re), fma2(s1, r, a.im));
      } else {  // W = c - i s: t = (b.re c + b.im s, b.im c - b.re s)
        constexpr double cs[8] = {1.0, SWC_C16_1, SWC_R2H, SWC_S16_1, 0.0, -SWC_S16_1, -SWC_R2H, -SWC_C16_1};
        constexpr double sn[8] = {0.0, SWC_S16_1, SWC_R2H, SWC_C16_1, 1.0, SWC_C16_1, SWC_R2H, SWC_S16_1};
        const float2 c = f2((float)cs[k16]), s = f2((float)sn[k16]), ns = f2(-(float)sn[k16]);
        const float2 tr = fma2(b.re, c, mul2(b.im, s));
        const float2 ti = fma2(b.im, c, mul2(b.re, ns));
        v[K] = pmake(add2(a.re, tr), add2(a.im, ti));
        v[K + R / 2] = pmake(sub2(a.re, tr), sub2(a.im, ti));
      }
      combine<K + 1>(v, e, o);
    }
  }
  __device__ __forceinline__ static void run(PC* v) {
    PC e[R / 2], o[R / 2];
#pragma unroll
    for (int i = 0; i < R / 2; ++i) { e[i] = v[2 * i]; o[i] = v[2 * i + 1]; }
    PDft<R / 2>::run(e);
    PDft<R / 2>::run(o);
    combine<0>(v, e, o);
  }
};
template <> struct PDft<1> {
  __device__ __forceinline__ static void run(PC*) {}
};

// ---- configuration ---------------------------------------------------------------------

template <int N> struct PairCfg {
  using F = FastCfg<float, N>;
  static constexpr int M = N / 2;
  static constexpr bool P3 = (N == 256 && SWC_PAIR_PLAN256 == 2);
  // Stockham radices (R3 = 1: two stages)
  static constexpr int R1 = P3 ? 8 : F::R1, R2 = P3 ? 4 : F::R2, R3 = P3 ? 4 : 1;
  static_assert(R1 * R2 * R3 == M, "radix plan");
  static constexpr int RL = (R3 > 1) ? R3 : R2;            // last stage's radix
  static constexpr int NSL = (R3 > 1) ? R1 * R2 : R1;      // and its Stockham span
  static constexpr int TPL = M / R1;          // threads per line pair
  static constexpr int NT = P3 ? 256 : 128;   // threads per CTA
  static constexpr int LP = NT / TPL;         // line pairs per CTA
  static constexpr int PP = LP + 1;           // PC row pitch (staggers banks for the z phases)
  static constexpr int NQ = N / 4;            // float4 per line
  static constexpr int LOG2LP = (LP == 4) ? 2 : (LP == 8) ? 3 : (LP == 16) ? 4 : (LP == 32) ? 5 : 6;
  static constexpr int LOG2NQ = (NQ == 16) ? 4 : (NQ == 32) ? 5 : (NQ == 64) ? 6 : 7;
  static_assert((1 << LOG2LP) == LP && (1 << LOG2NQ) == NQ, "powers of two");
  static_assert(NT % TPL == 0 && LP >= 4, "line pairs per CTA");
  // PC buffer + stage twiddles (M, float4 {c, c, s, s}) + post (2(M+1)) and pre (2M)
  // Makhoul twiddles (float2, broadcast on use)
  static constexpr size_t table_bytes() { return (size_t)M * 16 + (size_t)(2 * (M + 1) + 2 * M) * 8; }
  static constexpr size_t smem_bytes() { return (size_t)M * PP * 16 + table_bytes(); }
};

// Line B of a pair is line A + 1: coordinate k + 1 for x/y passes (needs nz >= 2),
// j + 1 for z passes (needs ny >= 2). Indices are 32-bit.
template <int N> inline bool pair_pass_supported(const Grid& g, int axis) {
  const long long nlines = g.ng / N;
  if (nlines < 2 * PairCfg<N>::LP || g.ng >= (1LL << 31)) return false;
  return axis == 2 ? g.ny >= 2 : g.nz >= 2;
}

// ---- functor adapters: both lines of a pair, or four consecutive z elements --------------
// A functor may provide pair(i, j, k, idx[, v]) (x/y passes: elements idx, idx + 1 at
// k, k + 1) and quad(i, j, k, idx[, v]) (z passes: idx .. idx + 3 at k .. k + 3) to move
// them as vectors; otherwise the scalar operator() is called per element.

template <class F, class = void> struct HasLdPair : std::false_type {};
template <class F>
struct HasLdPair<F, std::void_t<decltype(std::declval<const F&>().pair(0, 0, 0, 0LL))>> : std::true_type {};
template <class F, class = void> struct HasLdQuad : std::false_type {};
template <class F>
struct HasLdQuad<F, std::void_t<decltype(std::declval<const F&>().quad(0, 0, 0, 0LL))>> : std::true_type {};
template <class F, class = void> struct HasStPair : std::false_type {};
template <class F>
struct HasStPair<F, std::void_t<decltype(std::declval<const F&>().pair(0, 0, 0, 0LL, float2()))>> : std::true_type {};
template <class F, class = void> struct HasStQuad : std::false_type {};
template <class F>
struct HasStQuad<F, std::void_t<decltype(std::declval<const F&>().quad(0, 0, 0, 0LL, float4()))>> : std::true_type {};

// element (i, j, k, idx) of line A and its partner on line B
template <int AX, class LD>
__device__ __forceinline__ float2 ld_ab(const Grid& g, const LD& ld, int i, int j, int k, long long idx) {
  if constexpr (AX != 2) {
    if constexpr (HasLdPair<LD>::value) return ld.pair(i, j, k, idx);
    else return make_float2(ld(i, j, k, idx), ld(i, j, k + 1, idx + 1));
  } else {
    return make_float2(ld(i, j, k, idx), ld(i, j + 1, k, idx + g.nz));
  }
}
template <int AX, class ST>
__device__ __forceinline__ void st_ab(const Grid& g, const ST& st, int i, int j, int k, long long idx, float2 v) {
  if constexpr (AX != 2) {
    if constexpr (HasStPair<ST>::value) {
      st.pair(i, j, k, idx, v);
    } else {
      st(i, j, k, idx, v.x);
      st(i, j, k + 1, idx + 1, v.y);
    }
  } else {
    st(i, j, k, idx, v.x);
    st(i, j + 1, k, idx + g.nz, v.y);
  }
}
template <int AX, class MUL> __device__ __forceinline__ float2 mul_ab(const MUL& mul, int i, int j, int k) {
  if constexpr (AX != 2) return make_float2(mul(i, j, k), mul(i, j, k + 1));
  else return make_float2(mul(i, j, k), mul(i, j + 1, k));
}
// elements k, k+1 of one z line (the pair form stores idx, idx + 1)
template <class ST>
__device__ __forceinline__ void st_z2(const ST& st, int i, int j, int k, long long idx, float2 v) {
  if constexpr (HasStPair<ST>::value) {
    st.pair(i, j, k, idx, v);
  } else {
    st(i, j, k, idx, v.x);
    st(i, j, k + 1, idx + 1, v.y);
  }
}
// elements k .. k+3 of one z line
template <class LD> __device__ __forceinline__ float4 ld_q(const LD& ld, int i, int j, int k, long long idx) {
  if constexpr (HasLdQuad<LD>::value) return ld.quad(i, j, k, idx);
  else return make_float4(ld(i, j, k, idx), ld(i, j, k + 1, idx + 1), ld(i, j, k + 2, idx + 2), ld(i, j, k + 3, idx + 3));
}
template <class ST>
__device__ __forceinline__ void st_q(const ST& st, int i, int j, int k, long long idx, float4 v) {
  if constexpr (HasStQuad<ST>::value) {
    st.quad(i, j, k, idx, v);
  } else {
    st(i, j, k, idx, v.x);
    st(i, j, k + 1, idx + 1, v.y);
    st(i, j, k + 2, idx + 2, v.z);
    st(i, j, k + 3, idx + 3, v.w);
  }
}

// real element r of line pair lp in the PC buffer viewed as float2 (A, B) pairs
template <int PP> __device__ __forceinline__ int rpi(int r, int lp) { return (((r >> 1) * PP + lp) << 1) + (r & 1); }

// ---- stages ------------------------------------------------------------------------------

// Radix-R Stockham stage from and to the PC buffer (read -> barrier -> write -> barrier).
template <int M, int R, int NS, int TPL, int PP>
__device__ __forceinline__ void pair_stage(PC* buf, const float4* tw, int lp, int tj) {
  constexpr int NB = M / R, PER = NB / TPL, STRIDE = M / R;
  PC v[PER][R];
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int jb = tj + b * TPL;
#pragma unroll
    for (int r = 0; r < R; ++r) v[b][r] = buf[(jb + r * STRIDE) * PP + lp];
    if constexpr (NS > 1) {
      const int jj = jb & (NS - 1);
      constexpr int TSTEP = M / (NS * R);
#pragma unroll
      for (int r = 1; r < R; ++r) v[b][r] = pmul(v[b][r], tw[r * jj * TSTEP]);
    }
    PDft<R>::run(v[b]);
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int jb = tj + b * TPL;
    const int jj = jb & (NS - 1);
    const int base = (jb - jj) * R + jj;
#pragma unroll
    for (int r = 0; r < R; ++r) buf[(base + r * NS) * PP + lp] = v[b][r];
  }
  __syncthreads();
}

// DCT-II post-processing on (k, M-k) pairs into the real layout, natural order
// (reversed for DST-II), times the filter multiplier for K_FILT. ROWS: one row of
// LP + 1 float2 per position instead (the z store's layout: conflict-free writes here
// and reads there).
template <int N, int KIND, int AX, class MUL, bool ROWS = false>
__device__ __forceinline__ void pair_post(const Grid& g, int lineA, PC* buf, const float2* post, int lp, int tj,
                                          const MUL& mul) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, PP = Cf::PP, TPL = Cf::TPL, NP = (M / 2) / TPL;
  float2 y[NP][4];
  float2 ymid[2] = {f2(0.f), f2(0.f)};
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    const PC zk = buf[k * PP + lp];
    const PC zm = buf[((M - k) & (M - 1)) * PP + lp];
    const PC u0 = pcomb(post[2 * k], zk, post[2 * k + 1], zm);
    const int km = M - k;
    const PC u1 = pcomb(post[2 * km], zm, post[2 * km + 1], zk);
    y[b][0] = u0.re;        // Y_k
    y[b][1] = neg2(u0.im);  // Y_{N-k}
    y[b][2] = u1.re;        // Y_{M-k}
    y[b][3] = neg2(u1.im);  // Y_{M+k}
  }
  if (tj == 0) {
    const PC z = buf[(M / 2) * PP + lp];
    const PC u = pcomb(post[M], z, post[M + 1], z);
    ymid[0] = u.re;
    ymid[1] = neg2(u.im);
  }
  __syncthreads();
  float2* rb2 = reinterpret_cast<float2*>(buf);
  auto put = [&](int pos, float2 v) {
    if constexpr (KIND == K_FILT) {
      int i, j, kk;
      long long idx;
      line_coords(g, AX, lineA, pos, i, j, kk, idx);
      v = mul2(v, mul_ab<AX>(mul, i, j, kk));
    }
    const int o = (KIND == K_S2) ? (N - 1 - pos) : pos;
    if constexpr (ROWS) rb2[o * PP + lp] = v;
    else rb2[rpi<PP>(o, lp)] = v;
  };
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    put(k, y[b][0]);
    put(M - k, y[b][2]);
    if (k > 0) {
      put(N - k, y[b][1]);
      put(M + k, y[b][3]);
    }
  }
  if (tj == 0) {
    put(M / 2, ymid[0]);
    put(M + M / 2, ymid[1]);
  }
  __syncthreads();
}

// DCT-III pre-processing of one (k, M-k) pair: reals X_k, X_{N-k}, X_{M-k}, X_{M+k}
// -> Z_k, Z_{M-k} (U_k = X_k - i X_{N-k}, Z_k = a_k U_k + b_k conj(U_{M-k})).
__device__ __forceinline__ void pair_pre_one(const float2* pre, int M, int k, float2 xk, float2 xnk, float2 xmk,
                                             float2 xmpk, PC& z0, PC& z1) {
  const PC U = pmake(xk, neg2(xnk)), Um = pmake(xmk, neg2(xmpk));
  z0 = pcomb(pre[2 * k], U, pre[2 * k + 1], Um);
  const int km = (M - k) & (M - 1);
  z1 = pcomb(pre[2 * km], Um, pre[2 * km + 1], U);
}

// DCT-III pre-processing from the real layout (natural order) to (im, re)-swapped Z.
template <int N> __device__ __forceinline__ void pair_pre(PC* buf, const float2* pre, int lp, int tj) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, PP = Cf::PP, TPL = Cf::TPL, NP = (M / 2) / TPL;
  const float2* rb2 = reinterpret_cast<const float2*>(buf);
  PC z[NP][2];
  PC zmid = pmake(f2(0.f), f2(0.f));
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    const float2 xnk = (k == 0) ? f2(0.f) : rb2[rpi<PP>(N - k, lp)];
    pair_pre_one(pre, M, k, rb2[rpi<PP>(k, lp)], xnk, rb2[rpi<PP>(M - k, lp)], rb2[rpi<PP>(M + k, lp)], z[b][0],
                 z[b][1]);
  }
  if (tj == 0) {
    const int k = M / 2;
    const PC U = pmake(rb2[rpi<PP>(k, lp)], neg2(rb2[rpi<PP>(N - k, lp)]));
    zmid = pcomb(pre[2 * k], U, pre[2 * k + 1], U);
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    buf[k * PP + lp] = pswap(z[b][0]);
    if (k > 0) buf[(M - k) * PP + lp] = pswap(z[b][1]);
  }
  if (tj == 0) buf[(M / 2) * PP + lp] = pswap(zmid);
  __syncthreads();
}

// K_DERIV between the two FFTs, in registers: the DCT-II post-processing of the slot
// pair (k, M-k) yields Y_k, Y_{N-k}, Y_{M-k}, Y_{M+k}; the DST-III input is the shifted,
// reversed X_r = w_{N-1-r} = mul(N-1-r) Y_{N-r} (X_0 = w_{N-1} = 0), and its
// pre-processing of the same slot pair reads X_k, X_{N-k}, X_{M-k}, X_{M+k} -- exactly
// those four Y times their multipliers. Each slot is read and written by one thread
// only, so no barrier separates the two steps (one after, before the inverse FFT).
template <int N, int AX, class MUL>
__device__ __forceinline__ void pair_deriv(const Grid& g, int lineA, PC* buf, const float2* post,
                                           const float2* pre, int lp, int tj, const MUL& mul) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, PP = Cf::PP, TPL = Cf::TPL, NP = (M / 2) / TPL;
  auto m = [&](int pos) -> float2 {  // the multiplier at position pos of both lines
    int i, j, k;
    long long idx;
    line_coords(g, AX, lineA, pos, i, j, k, idx);
    return mul_ab<AX>(mul, i, j, k);
  };
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    const PC zk = buf[k * PP + lp];
    const PC zm = buf[((M - k) & (M - 1)) * PP + lp];
    const PC u0 = pcomb(post[2 * k], zk, post[2 * k + 1], zm);
    const int km = M - k;
    const PC u1 = pcomb(post[2 * km], zm, post[2 * km + 1], zk);
    // Y_k = u0.re, Y_{N-k} = -u0.im, Y_{M-k} = u1.re, Y_{M+k} = -u1.im (k = 0: Y_M = u1.re)
    const float2 xk = (k > 0) ? mul2(m(N - 1 - k), neg2(u0.im)) : f2(0.f);
    const float2 xnk = (k > 0) ? mul2(m(k - 1), u0.re) : f2(0.f);
    const float2 xmk = (k > 0) ? mul2(m(M - 1 + k), neg2(u1.im)) : mul2(m(M - 1), u1.re);
    const float2 xmpk = mul2(m(M - 1 - k), u1.re);
    PC z0, z1;
    pair_pre_one(pre, M, k, xk, xnk, xmk, xmpk, z0, z1);
    buf[k * PP + lp] = pswap(z0);
    if (k > 0) buf[(M - k) * PP + lp] = pswap(z1);
  }
  if (tj == 0) {
    const int k = M / 2;
    const PC z = buf[k * PP + lp];
    const PC u = pcomb(post[M], z, post[M + 1], z);
    // Y_{M/2} = u.re, Y_{N-M/2} = -u.im: X_{M/2} = mul(N-1-M/2) Y_{N-M/2}, X_{N-M/2} = mul(M/2-1) Y_{M/2}
    const float2 xk = mul2(m(N - 1 - k), neg2(u.im)), xnk = mul2(m(k - 1), u.re);
    const PC U = pmake(xk, neg2(xnk));
    buf[k * PP + lp] = pswap(pcomb(pre[2 * k], U, pre[2 * k + 1], U));
  }
  __syncthreads();
}

// K_FILT between the two FFTs, in registers: X_p = Y_p mul(p) at the four positions
// k, N-k, M-k, M+k that the DCT-II post-processing of the slot pair (k, M-k) yields and
// the DCT-III pre-processing of the same pair reads (one barrier, as pair_deriv).
template <int N, int AX, class MUL>
__device__ __forceinline__ void pair_filt(const Grid& g, int lineA, PC* buf, const float2* post,
                                          const float2* pre, int lp, int tj, const MUL& mul) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, PP = Cf::PP, TPL = Cf::TPL, NP = (M / 2) / TPL;
  auto m = [&](int pos) -> float2 {
    int i, j, k;
    long long idx;
    line_coords(g, AX, lineA, pos, i, j, k, idx);
    return mul_ab<AX>(mul, i, j, k);
  };
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    const PC zk = buf[k * PP + lp];
    const PC zm = buf[((M - k) & (M - 1)) * PP + lp];
    const PC u0 = pcomb(post[2 * k], zk, post[2 * k + 1], zm);
    const int km = M - k;
    const PC u1 = pcomb(post[2 * km], zm, post[2 * km + 1], zk);
    const float2 xk = mul2(u0.re, m(k));
    const float2 xnk = (k > 0) ? mul2(neg2(u0.im), m(N - k)) : f2(0.f);
    const float2 xmk = mul2(u1.re, m(M - k));
    const float2 xmpk = (k > 0) ? mul2(neg2(u1.im), m(M + k)) : xmk;
    PC z0, z1;
    pair_pre_one(pre, M, k, xk, xnk, xmk, xmpk, z0, z1);
    buf[k * PP + lp] = pswap(z0);
    if (k > 0) buf[(M - k) * PP + lp] = pswap(z1);
  }
  if (tj == 0) {
    const int k = M / 2;
    const PC z = buf[k * PP + lp];
    const PC u = pcomb(post[M], z, post[M + 1], z);
    const float2 xk = mul2(u.re, m(k)), xnk = mul2(neg2(u.im), m(N - k));
    const PC U = pmake(xk, neg2(xnk));
    buf[k * PP + lp] = pswap(pcomb(pre[2 * k], U, pre[2 * k + 1], U));
  }
  __syncthreads();
}

// K_DERIVT between the two FFTs, in registers (as pair_deriv): the DST-II output is
// z_q = Y_{N-1-q} of the DCT-II post-processing, the DCT-III input u_j = mul(j-1) z_{j-1}
// = mul(j-1) Y_{N-j} (u_0 = 0), and the pre-processing of slot pair (k, M-k) reads
// u_k, u_{N-k}, u_{M-k}, u_{M+k}: the Y at N-k, k, M+k, M-k that its post-processing yields.
template <int N, int AX, class MUL>
__device__ __forceinline__ void pair_derivt(const Grid& g, int lineA, PC* buf, const float2* post,
                                            const float2* pre, int lp, int tj, const MUL& mul) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, PP = Cf::PP, TPL = Cf::TPL, NP = (M / 2) / TPL;
  auto m = [&](int pos) -> float2 {
    int i, j, k;
    long long idx;
    line_coords(g, AX, lineA, pos, i, j, k, idx);
    return mul_ab<AX>(mul, i, j, k);
  };
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    const PC zk = buf[k * PP + lp];
    const PC zm = buf[((M - k) & (M - 1)) * PP + lp];
    const PC u0 = pcomb(post[2 * k], zk, post[2 * k + 1], zm);
    const int km = M - k;
    const PC u1 = pcomb(post[2 * km], zm, post[2 * km + 1], zk);
    // Y_k = u0.re, Y_{N-k} = -u0.im, Y_{M-k} = u1.re, Y_{M+k} = -u1.im (k = 0: Y_M = u1.re)
    const float2 xk = (k > 0) ? mul2(m(k - 1), neg2(u0.im)) : f2(0.f);
    const float2 xnk = (k > 0) ? mul2(m(N - k - 1), u0.re) : f2(0.f);
    const float2 xmk = (k > 0) ? mul2(m(M - k - 1), neg2(u1.im)) : mul2(m(M - 1), u1.re);
    const float2 xmpk = mul2(m(M + k - 1), u1.re);
    PC z0, z1;
    pair_pre_one(pre, M, k, xk, xnk, xmk, xmpk, z0, z1);
    buf[k * PP + lp] = pswap(z0);
    if (k > 0) buf[(M - k) * PP + lp] = pswap(z1);
  }
  if (tj == 0) {
    const int k = M / 2;
    const PC z = buf[k * PP + lp];
    const PC u = pcomb(post[M], z, post[M + 1], z);
    // u_{M/2} = mul(M/2-1) Y_{N-M/2} = mul(M/2-1) (-u.im), u_{N-M/2} = mul(N-M/2-1) Y_{M/2}
    const float2 xk = mul2(m(k - 1), neg2(u.im)), xnk = mul2(m(N - k - 1), u.re);
    const PC U = pmake(xk, neg2(xnk));
    buf[k * PP + lp] = pswap(pcomb(pre[2 * k], U, pre[2 * k + 1], U));
  }
  __syncthreads();
}

// x/y forward kinds: post-processing with the outputs of both lines stored straight
// to global memory.
template <int N, int KIND, int AX, class ST>
__device__ __forceinline__ void pair_post_store(const Grid& g, int lineA, const PC* buf, const float2* post, int lp,
                                                int tj, const ST& st) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, PP = Cf::PP, TPL = Cf::TPL, NP = (M / 2) / TPL;
  auto put = [&](int pos, float2 v) {
    const int o = (KIND == K_S2) ? (N - 1 - pos) : pos;
    int i, j, k;
    long long idx;
    xy_coords<AX>(g, lineA, o, i, j, k, idx);
    st_ab<AX>(g, st, i, j, k, idx, v);
  };
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    const PC zk = buf[k * PP + lp];
    const PC zm = buf[((M - k) & (M - 1)) * PP + lp];
    const PC u0 = pcomb(post[2 * k], zk, post[2 * k + 1], zm);
    const int km = M - k;
    const PC u1 = pcomb(post[2 * km], zm, post[2 * km + 1], zk);
    put(k, u0.re);
    put(M - k, u1.re);
    if (k > 0) {
      put(N - k, neg2(u0.im));
      put(M + k, neg2(u1.im));
    }
  }
  if (tj == 0) {
    const PC z = buf[(M / 2) * PP + lp];
    const PC u = pcomb(post[M], z, post[M + 1], z);
    put(M / 2, u.re);
    put(M + M / 2, neg2(u.im));
  }
}

// x/y inverse kinds: the last Stockham stage with both lines' outputs stored straight
// to global memory (slot m holds the swapped z_m: v_2m = .im, v_2m+1 = .re, v_q at
// position mk_pos(q), negated at odd positions for DST-III).
template <int N, int KIND, int AX, class ST, int R = PairCfg<N>::RL, int NS = PairCfg<N>::NSL>
__device__ __forceinline__ void pair_last_store(const Grid& g, int lineA, const PC* buf, const float4* tw, int lp,
                                                int tj, const ST& st) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, PP = Cf::PP, TPL = Cf::TPL;
  constexpr int NB = M / R, PER = NB / TPL, STRIDE = M / R, TSTEP = M / (NS * R);
  PC v[PER][R];
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int jb = tj + b * TPL;
#pragma unroll
    for (int r = 0; r < R; ++r) v[b][r] = buf[(jb + r * STRIDE) * PP + lp];
    const int jj = jb & (NS - 1);
#pragma unroll
    for (int r = 1; r < R; ++r) v[b][r] = pmul(v[b][r], tw[r * jj * TSTEP]);
    PDft<R>::run(v[b]);
  }
  auto put = [&](int q, float2 val) {
    const int pos = mk_pos<N>(q);
    if ((KIND == K_S3 || KIND == K_DERIV) && (pos & 1)) val = neg2(val);
    int i, j, k;
    long long idx;
    xy_coords<AX>(g, lineA, pos, i, j, k, idx);
    st_ab<AX>(g, st, i, j, k, idx, val);
  };
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int jb = tj + b * TPL;
    const int jj = jb & (NS - 1);
    const int base = (jb - jj) * R + jj;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int m = base + r * NS;
      put(2 * m, v[b][r].im);
      put(2 * m + 1, v[b][r].re);
    }
  }
}


// ---- paired radix-8 stages next to the Makhoul steps (x/y passes, N = 256) ---------------
// In the 16 x 8 plan the stage adjacent to the post-processing (the last forward stage)
// and, in the 8 x 16 plan, the stage adjacent to the pre-processing (the first inverse
// stage) have 16 radix-8 butterflies per line pair, two per thread. Thread tj takes
// b0 = tj and b1 = 16 - tj (tj = 0: 0 and 8). Butterfly b covers the modes b + 16 r, and
// the Makhoul pair (k, M-k) of k = b0 + 16 r (r < 4) is element r of b0 with element
// 7 - r of b1, that of k = b1 + 16 r element r of b1 with element 7 - r of b0; for
// tj = 0, b0 = 0 pairs its own elements r and 8 - r (element 0 alone, element 4 the
// middle mode M/2) and b1 = 8 its elements r and 7 - r. So the DCT-II post-processing
// after the last forward stage, and the DCT-III pre-processing before the first inverse
// stage, run in the registers of one thread.
template <int N> struct PairR8 {
  using Cf = PairCfg<N>;
  static constexpr bool ok = N == 256 && Cf::R3 == 1 && Cf::R2 == 8 && Cf::M == 16 * Cf::TPL && Cf::R1 == 16;
};
__device__ __forceinline__ int pr_b1(int tj, int tpl) { return tj == 0 ? tpl : 2 * tpl - tj; }
__device__ __forceinline__ PC psel(bool c, const PC& a, const PC& b) {
  return pmake(make_float2(c ? a.re.x : b.re.x, c ? a.re.y : b.re.y),
               make_float2(c ? a.im.x : b.im.x, c ? a.im.y : b.im.y));
}

// Last forward stage (radix 8, span M/8) of butterfly b from the buffer: its outputs at
// modes b + 16 r in o[r].
template <int M, int PP>
__device__ __forceinline__ void pr_last_fwd(const PC* buf, const float4* tw, int lp, int b, PC (&o)[8]) {
  constexpr int R = 8, STRIDE = M / R;  // span M/8 = 16 > b, twiddle step 1
#pragma unroll
  for (int r = 0; r < R; ++r) o[r] = buf[(b + r * STRIDE) * PP + lp];
#pragma unroll
  for (int r = 1; r < R; ++r) o[r] = pmul(o[r], tw[r * b]);
  PDft<R>::run(o);
}

// The FFT outputs z_k and z_(M-k) of the pair k = b + 16 r from the outputs of b0 (o0)
// and b1 (o1): second == false for k in b0, true for k in b1.
template <bool second>
__device__ __forceinline__ void pr_pair_in(bool t0, int r, const PC (&o0)[8], const PC (&o1)[8], PC& zk, PC& zm) {
  if constexpr (!second) {
    zk = o0[r];
    zm = psel(t0, o0[(8 - r) & 7], o1[7 - r]);
  } else {
    zk = o1[r];
    zm = psel(t0, o1[7 - r], o0[7 - r]);
  }
}

// The first inverse stage (radix 8) of b0 and b1 from the pre-processed (im, re)-swapped
// Z of the pairs: Zk0[r], Zm0[r] of k = b0 + 16 r, Zk1[r], Zm1[r] of k = b1 + 16 r, and
// (tj = 0) the middle mode; written to the buffer as rows b 8 + r after a barrier (the
// caller's reads of the buffer end there) and a second one after.
template <int M, int PP>
__device__ __forceinline__ void pr_first_inv(PC* buf, bool t0, int lp, int b0, int b1, const PC (&Zk0)[4],
                                             const PC (&Zm0)[4], const PC (&Zk1)[4], const PC (&Zm1)[4],
                                             const PC& mid) {
  PC v0[8], v1[8];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    v0[r] = Zk0[r];
    v1[r] = Zk1[r];
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    v0[7 - r] = psel(t0, (r == 3) ? mid : Zm0[(r + 1) & 3], Zm1[r]);
    v1[7 - r] = psel(t0, Zm1[r], Zm0[r]);
  }
  PDft<8>::run(v0);
  PDft<8>::run(v1);
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    buf[(b0 * 8 + r) * PP + lp] = v0[r];
    buf[(b1 * 8 + r) * PP + lp] = v1[r];
  }
  __syncthreads();
}

// x/y forward kinds: the last forward stage in registers, the post-processing, and both
// lines' outputs stored straight to global memory.
template <int N, int KIND, int AX, class ST>
__device__ __forceinline__ void pr_post_store(const Grid& g, int lineA, const PC* buf, const float4* tw,
                                              const float2* post, int lp, int tj, const ST& st) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, PP = Cf::PP, TPL = Cf::TPL;
  const bool t0 = tj == 0;
  const int b0 = tj, b1 = pr_b1(tj, TPL);
  PC o0[8], o1[8];
  pr_last_fwd<M, PP>(buf, tw, lp, b0, o0);
  pr_last_fwd<M, PP>(buf, tw, lp, b1, o1);
  auto put = [&](int pos, float2 v) {
    const int o = (KIND == K_S2) ? (N - 1 - pos) : pos;
    int i, j, k;
    long long idx;
    xy_coords<AX>(g, lineA, o, i, j, k, idx);
    st_ab<AX>(g, st, i, j, k, idx, v);
  };
  auto one = [&](int k, const PC& zk, const PC& zm) {
    const PC u0 = pcomb(post[2 * k], zk, post[2 * k + 1], zm);
    const int km = M - k;
    const PC u1 = pcomb(post[2 * km], zm, post[2 * km + 1], zk);
    put(k, u0.re);
    put(M - k, u1.re);
    if (k > 0) {
      put(N - k, neg2(u0.im));
      put(M + k, neg2(u1.im));
    }
  };
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    PC zk, zm;
    pr_pair_in<false>(t0, r, o0, o1, zk, zm);
    one(b0 + 16 * r, zk, zm);
    pr_pair_in<true>(t0, r, o0, o1, zk, zm);
    one(b1 + 16 * r, zk, zm);
  }
  if (t0) {
    const PC z = o0[4];
    const PC u = pcomb(post[M], z, post[M + 1], z);
    put(M / 2, u.re);
    put(M + M / 2, neg2(u.im));
  }
}

// Shared-memory twiddle tables: stage twiddles as {c, c, s, s}, Makhoul tables as is.
template <int N, bool FWD, bool INV>
__device__ __forceinline__ void pair_tables(const R2RTables<float>& tb, float4* sfft, float2* spost, float2* spre,
                                            int tid) {
  constexpr int M = N / 2, NT = PairCfg<N>::NT;
  for (int t = tid; t < M; t += NT) {
    const float2 w = __ldg(&tb.fft[t]);
    sfft[t] = make_float4(w.x, w.x, w.y, w.y);
  }
  if constexpr (FWD)
    for (int t = tid; t < 2 * (M + 1); t += NT) spost[t] = __ldg(&tb.post[t]);
  if constexpr (INV)
    for (int t = tid; t < 2 * M; t += NT) spre[t] = __ldg(&tb.pre[t]);
}

// Everything after the load phase, shared by the direct and the TMA-fed kernels. On
// entry the PC buffer holds, per kind and axis: x/y forward -> stage-1 output; z forward
// -> the Makhoul-ordered z; x/y inverse -> the pre-processed, swapped Z; z inverse ->
// the natural-order reals. Outputs go to global memory through `st`.
// ZT (row-staged z passes): the loader has already run the first stage, of radix R1/2,
// of the FFT that follows the load -- the forward FFT of the forward kinds, or the
// inverse FFT (after the DCT-III pre-processing) of the inverse kinds -- so that FFT
// ends with one stage of radix 2 R2.
// PR (x/y passes of the plain kinds, PairR8<N>::ok): the stages next to the Makhoul
// steps are paired radix-8 ones -- the forward kinds' last stage and post-processing
// run in registers (pr_post_store); for the inverse kinds the loader has run the
// pre-processing and the first inverse stage (pr_first_inv), and the last inverse stage
// is radix 16.
template <int N, int KIND, int AX, class StoreOp, class MulOp, bool ZT = false, bool PR = false>
__device__ __forceinline__ void pair_tail(const Grid& g, int pair0, int lp, int tj, int tid, PC* buf,
                                          const float4* sfft, const float2* spost, const float2* spre,
                                          const StoreOp& st, const MulOp& mul) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, LP = Cf::LP, PP = Cf::PP, NT = Cf::NT, TPL = Cf::TPL, NQ = Cf::NQ;
  constexpr int R1 = Cf::R1;
  constexpr bool fwd_in = (KIND == K_C2 || KIND == K_S2 || KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);
  constexpr bool inv_out = (KIND == K_C3 || KIND == K_S3 || KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);
  constexpr bool xy = (AX != 2);
  constexpr int ZU = (LP * NQ) / NT;
  constexpr int ZC = (ZU >= 4) ? 4 : ZU;
  static_assert(ZU * NT == LP * NQ && ZU % ZC == 0, "z units");
  float2* rb2 = reinterpret_cast<float2*>(buf);
  const int lineA = 2 * (pair0 + lp);
  constexpr bool zt_inv = ZT && !fwd_in;  // inverse kinds: pre-processing and first stage done
  constexpr bool pr = PR && xy;
  static_assert(!pr || (PairR8<N>::ok && KIND != K_FILT && KIND != K_DERIV && KIND != K_DERIVT),
                "paired radix-8 stages");
  if constexpr (!xy && !ZT) {
    if constexpr (fwd_in) pair_stage<M, R1, 1, TPL, PP>(buf, sfft, lp, tj);
    else pair_pre<N>(buf, spre, lp, tj);
  }

  // ---------------- forward FFT + post ----------------
  if constexpr (fwd_in) {
    if constexpr (ZT) {
      static_assert(Cf::R3 == 1, "two-stage plan");
      pair_stage<M, 2 * Cf::R2, R1 / 2, TPL, PP>(buf, sfft, lp, tj);
    } else if constexpr (!pr) {
      pair_stage<M, Cf::R2, R1, TPL, PP>(buf, sfft, lp, tj);
      if constexpr (Cf::R3 > 1) pair_stage<M, Cf::R3, R1 * Cf::R2, TPL, PP>(buf, sfft, lp, tj);
    }
    if constexpr (xy && KIND != K_FILT && KIND != K_DERIV && KIND != K_DERIVT) {
      if constexpr (pr) pr_post_store<N, KIND, AX>(g, lineA, buf, sfft, spost, lp, tj, st);
      else pair_post_store<N, KIND, AX>(g, lineA, buf, spost, lp, tj, st);
      return;
    }
    if constexpr (KIND == K_DERIV) {
      pair_deriv<N, AX>(g, lineA, buf, spost, spre, lp, tj, mul);
    } else if constexpr (KIND == K_DERIVT) {
      pair_derivt<N, AX>(g, lineA, buf, spost, spre, lp, tj, mul);
    } else if constexpr (KIND == K_FILT) {
      pair_filt<N, AX>(g, lineA, buf, spost, spre, lp, tj, mul);
    } else {
      constexpr bool rows = !xy && !inv_out;  // z forward kinds: the z store reads position rows
      pair_post<N, KIND, AX, MulOp, rows>(g, lineA, buf, spost, lp, tj, mul);
      if constexpr (inv_out) pair_pre<N>(buf, spre, lp, tj);
    }
  }

  // ---------------- inverse FFT ----------------
  if constexpr (pr && inv_out) {
    pair_last_store<N, KIND, AX, StoreOp, 2 * Cf::R2, R1 / 2>(g, lineA, buf, sfft, lp, tj, st);
    return;
  } else if constexpr (zt_inv) {
    static_assert(Cf::R3 == 1, "two-stage plan");
    pair_stage<M, 2 * Cf::R2, R1 / 2, TPL, PP>(buf, sfft, lp, tj);
  } else if constexpr (inv_out) {
    pair_stage<M, R1, 1, TPL, PP>(buf, sfft, lp, tj);
    if constexpr (Cf::R3 > 1) pair_stage<M, Cf::R2, R1, TPL, PP>(buf, sfft, lp, tj);
    if constexpr (xy) {
      pair_last_store<N, KIND, AX>(g, lineA, buf, sfft, lp, tj, st);
      return;
    }
    pair_stage<M, Cf::RL, Cf::NSL, TPL, PP>(buf, sfft, lp, tj);
  }

  // ---------------- z store ----------------
  if constexpr (inv_out) {
    // Makhoul order, float4 per line: x_4a = slot a .im, x_4a+1 = slot M-1-a .re,
    // x_4a+2 = slot a .re, x_4a+3 = slot M-1-a .im (rows a, M-1-a: odd pitch, no conflicts)
#pragma unroll 1
    for (int c0 = 0; c0 < ZU; c0 += ZC) {
      float4 oa[ZC], ob[ZC];
#pragma unroll
      for (int c = 0; c < ZC; ++c) {
        const int u = tid + (c0 + c) * NT;
        const int a = u & (NQ - 1), q = u >> Cf::LOG2NQ;
        const PC sa = buf[a * PP + q], sb = buf[(M - 1 - a) * PP + q];
        oa[c] = make_float4(sa.im.x, sb.re.x, sa.re.x, sb.im.x);
        ob[c] = make_float4(sa.im.y, sb.re.y, sa.re.y, sb.im.y);
        if constexpr (KIND == K_S3 || KIND == K_DERIV) {
          oa[c].y = -oa[c].y; oa[c].w = -oa[c].w;
          ob[c].y = -ob[c].y; ob[c].w = -ob[c].w;
        }
      }
#pragma unroll
      for (int c = 0; c < ZC; ++c) {
        const int u = tid + (c0 + c) * NT;
        const int a = u & (NQ - 1), q = u >> Cf::LOG2NQ;
        const int la = 2 * (pair0 + q);
        const int i = la >> g.ly, j = la & (g.ny - 1);
        const long long idx = (long long)(la * N + 4 * a);
        st_q(st, i, j, 4 * a, idx, oa[c]);
        st_q(st, i, j + 1, 4 * a, idx + N, ob[c]);
      }
    }
  } else {
    // natural order from the position rows of pair_post: one position per unit,
    // consecutive lanes on consecutive rows (8-byte stride mod 128: no bank conflicts)
    constexpr int PU = (LP * N) / NT;
    constexpr int LOG2N = (N == 64) ? 6 : (N == 128) ? 7 : (N == 256) ? 8 : 9;
    static_assert((1 << LOG2N) == N && PU * NT == LP * N, "z position units");
#pragma unroll 4
    for (int c = 0; c < PU; ++c) {
      const int u = tid + c * NT;
      const int pos = u & (N - 1), q = u >> LOG2N;
      const float2 v = rb2[pos * PP + q];
      const int la = 2 * (pair0 + q);
      const int i = la >> g.ly, j = la & (g.ny - 1);
      const long long idx = (long long)(la * N + pos);
      st(i, j, pos, idx, v.x);
      st(i, j + 1, pos, idx + N, v.y);
    }
  }
}

template <int N, int KIND, int AX, class LoadOp, class StoreOp, class MulOp>
__global__ void __launch_bounds__(PairCfg<N>::NT) r2r_pair_kernel(Grid g, R2RTables<float> tb, LoadOp ld,
                                                                  StoreOp st, MulOp mul) {
  using Cf = PairCfg<N>;
  constexpr int M = Cf::M, LP = Cf::LP, PP = Cf::PP, NT = Cf::NT, TPL = Cf::TPL, NQ = Cf::NQ;
  constexpr int R1 = Cf::R1;
  constexpr bool fwd_in = (KIND == K_C2 || KIND == K_S2 || KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);
  constexpr bool inv_out = (KIND == K_C3 || KIND == K_S3 || KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);
  constexpr bool xy = (AX != 2);
  constexpr int ZU = (LP * NQ) / NT;  // z phases: (line pair, float4) units per thread
  constexpr int ZC = (ZU >= 4) ? 4 : ZU;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PC* buf = reinterpret_cast<PC*>(smem_raw);
  float4* sfft = reinterpret_cast<float4*>(buf + M * PP);
  float2* spost = reinterpret_cast<float2*>(sfft + M);
  float2* spre = spost + 2 * (M + 1);
  const int tid = threadIdx.x;
  const int lp = tid & (LP - 1), tj = tid >> Cf::LOG2LP;
  const int pair0 = blockIdx.x * LP;
  const int lineA = 2 * (pair0 + lp);
  pair_tables<N, fwd_in, inv_out>(tb, sfft, spost, spre, tid);
  __syncthreads();

  // ---------------- load ----------------
  if constexpr (xy && fwd_in) {
    // z_m = v_2m + i v_2m+1 of both lines straight into the first radix-R1 butterfly
    PC v[R1];
#pragma unroll
    for (int r = 0; r < R1; ++r) {
      const int m = tj + r * TPL;
      const int p0 = mk_pos<N>(2 * m), p1 = mk_pos<N>(2 * m + 1);
      int i, j, k;
      long long idx;
      xy_coords<AX>(g, lineA, p0, i, j, k, idx);
      float2 a = ld_ab<AX>(g, ld, i, j, k, idx);
      xy_coords<AX>(g, lineA, p1, i, j, k, idx);
      float2 b = ld_ab<AX>(g, ld, i, j, k, idx);
      if constexpr (KIND == K_S2 || KIND == K_DERIVT) {
        if (p0 & 1) a = neg2(a);
        if (p1 & 1) b = neg2(b);
      }
      v[r] = pmake(a, b);
    }
    PDft<R1>::run(v);
#pragma unroll
    for (int r = 0; r < R1; ++r) buf[(tj * R1 + r) * PP + lp] = v[r];
    __syncthreads();
  } else if constexpr (xy) {
    // inverse-only x/y kinds: the pre-processing reads its four reals per pair straight
    // from global memory (reversed for DST-III)
    constexpr int NP = (M / 2) / TPL;
    auto X = [&](int r) -> float2 {
      const int p = (KIND == K_S3) ? (N - 1 - r) : r;
      int i, j, k;
      long long idx;
      xy_coords<AX>(g, lineA, p, i, j, k, idx);
      return ld_ab<AX>(g, ld, i, j, k, idx);
    };
    PC z[NP][2];
    PC zmid = pmake(f2(0.f), f2(0.f));
#pragma unroll
    for (int b = 0; b < NP; ++b) {
      const int k = tj + b * TPL;
      const float2 xnk = (k == 0) ? f2(0.f) : X(N - k);
      pair_pre_one(spre, M, k, X(k), xnk, X(M - k), X(M + k), z[b][0], z[b][1]);
    }
    if (tj == 0) {
      const int k = M / 2;
      const PC U = pmake(X(k), neg2(X(N - k)));
      zmid = pcomb(spre[2 * k], U, spre[2 * k + 1], U);
    }
#pragma unroll
    for (int b = 0; b < NP; ++b) {
      const int k = tj + b * TPL;
      buf[k * PP + lp] = pswap(z[b][0]);
      if (k > 0) buf[(M - k) * PP + lp] = pswap(z[b][1]);
    }
    if (tj == 0) buf[(M / 2) * PP + lp] = pswap(zmid);
    __syncthreads();
  } else {
    // z: four consecutive elements of each line of a pair per unit (float4)
#pragma unroll 1
    for (int c0 = 0; c0 < ZU; c0 += ZC) {
      float4 xa[ZC], xb[ZC];
#pragma unroll
      for (int c = 0; c < ZC; ++c) {
        const int u = tid + (c0 + c) * NT;
        const int a = u & (NQ - 1), q = u >> Cf::LOG2NQ;
        const int la = 2 * (pair0 + q);
        const int i = la >> g.ly, j = la & (g.ny - 1);
        const long long idx = (long long)(la * N + 4 * a);
        xa[c] = ld_q(ld, i, j, 4 * a, idx);
        xb[c] = ld_q(ld, i, j + 1, 4 * a, idx + N);
      }
#pragma unroll
      for (int c = 0; c < ZC; ++c) {
        const int u = tid + (c0 + c) * NT;
        const int a = u & (NQ - 1), q = u >> Cf::LOG2NQ;
        float4 A = xa[c], B = xb[c];
        if constexpr (fwd_in) {
          if constexpr (KIND == K_S2 || KIND == K_DERIVT) {  // (-1)^p x_p
            A.y = -A.y; A.w = -A.w;
            B.y = -B.y; B.w = -B.w;
          }
          // z_a = (x_4a, x_4a+2), z_{M-1-a} = (x_4a+3, x_4a+1)
          buf[a * PP + q] = pmake(make_float2(A.x, B.x), make_float2(A.z, B.z));
          buf[(M - 1 - a) * PP + q] = pmake(make_float2(A.w, B.w), make_float2(A.y, B.y));
        } else if constexpr (KIND == K_S3) {
          // X_r = x_{N-1-r}: slot M-2a-2 = (x_4a+3, x_4a+2), slot M-2a-1 = (x_4a+1, x_4a)
          buf[(M - 2 * a - 2) * PP + q] = pmake(make_float2(A.w, B.w), make_float2(A.z, B.z));
          buf[(M - 2 * a - 1) * PP + q] = pmake(make_float2(A.y, B.y), make_float2(A.x, B.x));
        } else {
          buf[(2 * a) * PP + q] = pmake(make_float2(A.x, B.x), make_float2(A.y, B.y));
          buf[(2 * a + 1) * PP + q] = pmake(make_float2(A.z, B.z), make_float2(A.w, B.w));
        }
      }
    }
    __syncthreads();
  }

  pair_tail<N, KIND, AX>(g, pair0, lp, tj, tid, buf, sfft, spost, spre, st, mul);
}

}  // namespace swc
