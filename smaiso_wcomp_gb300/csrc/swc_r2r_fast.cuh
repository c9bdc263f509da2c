// swc_r2r_fast.cuh -- the r2r axis pass specialised at compile time on the line
// length N (64..512): same algorithm and data layout as r2r_pass_kernel
// (swc_r2r.cuh), but the radix plan, threads per line, lines per CTA and every
// shared-memory offset are constants, the whole pass is unrolled, the pre/post
// twiddles are applied to (k, M-k) pairs, and one shared buffer is reused by all
// phases (two barriers per exchange) so more CTAs fit on an SM.
#pragma once

#include "swc_r2r.cuh"

// Tuning constants (threads per CTA, loads in flight per thread); defaults measured on GB300.
#ifndef SWC_FAST_NT_F32
#define SWC_FAST_NT_F32 256
#endif
#ifndef SWC_FAST_NT_F64
#define SWC_FAST_NT_F64 128
#endif
#ifndef SWC_FAST_CH_F32
#define SWC_FAST_CH_F32 16
#endif
#ifndef SWC_FAST_CH_F64
#define SWC_FAST_CH_F64 8
#endif

namespace swc {

template <typename T, int N> struct FastCfg {
  static constexpr int M = N / 2;
  static constexpr int R1 = (M == 32) ? 8 : (M == 64) ? 8 : 16;   // largest radix first
  static constexpr int R2 = (M == 32) ? 4 : (M == 64) ? 8 : (M == 128) ? 8 : 16;
  static_assert(R1 * R2 == M, "two-stage plan");
  static constexpr int TPL = M / R1;                              // threads per line
  static constexpr int NT = (sizeof(T) == 8) ? SWC_FAST_NT_F64 : SWC_FAST_NT_F32;  // threads per CTA
  static constexpr int L = NT / TPL;                              // lines per CTA
  static constexpr int P = L + 1;                                 // complex row pitch
  static constexpr int ITERS = N / TPL;                           // load/store elements per thread
  static constexpr int CH = (sizeof(T) == 8) ? SWC_FAST_CH_F64 : SWC_FAST_CH_F32;  // loads in flight per chunk
  static constexpr int LOG2N = (N == 64) ? 6 : (N == 128) ? 7 : (N == 256) ? 8 : 9;
  static constexpr int LOG2L = (L == 8) ? 3 : (L == 16) ? 4 : (L == 32) ? 5 : 6;
  static_assert((1 << LOG2N) == N && (1 << LOG2L) == L, "powers of two");
  static constexpr size_t smem_bytes() { return (size_t)(M * P + 5 * M + 2) * 2 * sizeof(T); }
};

template <typename T, int N> inline bool fast_pass_supported(const Grid& g, int axis) {
  const long long nlines = g.ng / N;
  return nlines >= FastCfg<T, N>::L;
}

// real element r of tile line l, complex pitch P: component (r&1) of slot r>>1
template <int P> __device__ __forceinline__ int fridx(int r, int l) { return (((r >> 1) * P + l) << 1) + (r & 1); }

// Element `it` of thread `tid`: position p along the line, tile line le, coordinates
// and linear index (z tile: contiguous block of L rows; x/y: the thread's fixed line).
template <int N, int NT, int L, int LOG2N, int LOG2L, int TPL>
__device__ __forceinline__ void fast_elem(const Grid& g, int axis, long long line0, int tid, int it, int& p,
                                          int& le, int& i, int& j, int& k, long long& idx) {
  if (axis == 2) {
    const int e = tid + it * NT;
    p = e & (N - 1);
    le = e >> LOG2N;
    const int line = (int)line0 + le;
    i = line >> g.ly;
    j = line & (g.ny - 1);
    k = p;
    idx = (long long)(((int)line0 << LOG2N) + e);
  } else {
    le = tid & (L - 1);
    p = (tid >> LOG2L) + it * TPL;
    const int line = (int)(line0 + le);
    if (axis == 1) {
      i = line >> g.lz;
      k = line & (g.nz - 1);
      j = p;
      idx = (long long)((i << (g.ly + g.lz)) + (p << g.lz) + k);
    } else {
      j = line >> g.lz;
      k = line & (g.nz - 1);
      i = p;
      idx = (long long)((p << (g.ly + g.lz)) + line);
    }
  }
}

// Radix-R Stockham stage, all butterflies of this thread (compile-time geometry):
// read -> barrier -> write -> barrier (single buffer).
template <typename C, int M, int R, int NS, int TPL, int P>
__device__ __forceinline__ void fast_stage(C* buf, const C* tw, int l, int tj) {
  constexpr int NB = M / R;            // butterflies per line
  constexpr int PER = NB / TPL;        // butterflies per thread
  constexpr int STRIDE = M / R;
  C v[PER][R];
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int jb = tj + b * TPL;
#pragma unroll
    for (int r = 0; r < R; ++r) v[b][r] = buf[(jb + r * STRIDE) * P + l];
    if constexpr (NS > 1) {
      const int jj = jb & (NS - 1);
      constexpr int TSTEP = M / (NS * R);
#pragma unroll
      for (int r = 1; r < R; ++r) v[b][r] = cmul(v[b][r], tw[r * jj * TSTEP]);
    }
    Dft<R, C>::run(v[b]);
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int jb = tj + b * TPL;
    const int jj = jb & (NS - 1);
    const int base = (jb - jj) * R + jj;
#pragma unroll
    for (int r = 0; r < R; ++r) buf[(base + r * NS) * P + l] = v[b][r];
  }
  __syncthreads();
}

// DCT-II post-processing on (k, M-k) pairs: Z (complex, natural order, in buf) ->
// real output in natural order (reversed for DST-II), times the filter multiplier.
template <typename T, int N, int KIND, class MUL>
__device__ __forceinline__ void fast_post(const Grid& g, int axis, long long line, cx_t<T>* buf, const cx_t<T>* post,
                                          int l, int tj, const MUL& mul) {
  using Cf = FastCfg<T, N>;
  using C = cx_t<T>;
  constexpr int M = Cf::M, P = Cf::P, TPL = Cf::TPL;
  constexpr int NP = (M / 2) / TPL;  // pairs (k, M-k), k in [0, M/2), per thread
  T y[NP][4];
  T ymid[2] = {(T)0, (T)0};
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    const C zk = buf[k * P + l];
    const C zm = buf[((M - k) & (M - 1)) * P + l];  // k = 0: Z_M = Z_0
    const C u0 = cadd(cmul(post[2 * k], zk), cmulc(post[2 * k + 1], zm));
    const int km = M - k;  // k = 0: km = M (u_M from Z_0)
    const C u1 = cadd(cmul(post[2 * km], zm), cmulc(post[2 * km + 1], zk));
    y[b][0] = u0.x;   // Y_k
    y[b][1] = -u0.y;  // Y_{N-k}   (unused for k = 0)
    y[b][2] = u1.x;   // Y_{M-k}   (k = 0: Y_M)
    y[b][3] = -u1.y;  // Y_{M+k}   (unused for k = 0)
  }
  if (tj == 0) {  // k = M/2
    const C z = buf[(M / 2) * P + l];
    const C u = cadd(cmul(post[M], z), cmulc(post[M + 1], z));
    ymid[0] = u.x;
    ymid[1] = -u.y;
  }
  __syncthreads();
  T* rb = reinterpret_cast<T*>(buf);
  auto put = [&](int pos, T v) {
    if constexpr (KIND == K_FILT) {
      int i, j, kk;
      long long idx;
      line_coords(g, axis, line, pos, i, j, kk, idx);
      v *= mul(i, j, kk);
    }
    const int o = (KIND == K_S2) ? (N - 1 - pos) : pos;
    rb[fridx<P>(o, l)] = v;
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

// DCT-III pre-processing on (k, M-k) pairs: real input (natural order, in buf) ->
// (im, re)-swapped Z in buf, ready for the forward FFT stages.
template <typename T, int N>
__device__ __forceinline__ void fast_pre(cx_t<T>* buf, const cx_t<T>* pre, int l, int tj) {
  using Cf = FastCfg<T, N>;
  using C = cx_t<T>;
  constexpr int M = Cf::M, P = Cf::P, TPL = Cf::TPL;
  constexpr int NP = (M / 2) / TPL;
  const T* rb = reinterpret_cast<const T*>(buf);
  C z[NP][2];
  C zmid = cmake<C>((T)0, (T)0);
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    const T xk = rb[fridx<P>(k, l)];
    const T xnk = (k == 0) ? (T)0 : rb[fridx<P>(N - k, l)];
    const T xmk = rb[fridx<P>(M - k, l)];
    const T xmpk = rb[fridx<P>(M + k, l)];
    const C U = cmake<C>(xk, -xnk), Um = cmake<C>(xmk, -xmpk);
    z[b][0] = cadd(cmul(pre[2 * k], U), cmulc(pre[2 * k + 1], Um));  // Z_k
    const int km = (M - k) & (M - 1);                                 // unused for k = 0
    z[b][1] = cadd(cmul(pre[2 * km], Um), cmulc(pre[2 * km + 1], U)); // Z_{M-k}
  }
  if (tj == 0) {  // k = M/2
    const int k = M / 2;
    const C U = cmake<C>(rb[fridx<P>(k, l)], -rb[fridx<P>(N - k, l)]);
    zmid = cadd(cmul(pre[2 * k], U), cmulc(pre[2 * k + 1], U));
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    buf[k * P + l] = cswap(z[b][0]);
    if (k > 0) buf[(M - k) * P + l] = cswap(z[b][1]);
  }
  if (tj == 0) buf[(M / 2) * P + l] = cswap(zmid);
  __syncthreads();
}

// Coordinates of position p of line `line` of an x (AX = 0) or y (AX = 1) pass.
template <int AX>
__device__ __forceinline__ void xy_coords(const Grid& g, int line, int p, int& i, int& j, int& k, long long& idx) {
  if constexpr (AX == 1) {
    i = line >> g.lz;
    k = line & (g.nz - 1);
    j = p;
    idx = (long long)((i << (g.ly + g.lz)) + (p << g.lz) + k);
  } else {
    j = line >> g.lz;
    k = line & (g.nz - 1);
    i = p;
    idx = (long long)((p << (g.ly + g.lz)) + line);
  }
}

// Position along the line of real q of the Makhoul sequence v (v_q = x_p): p = 2q
// for q < N/2, p = 2(N-1-q)+1 otherwise. The same map places DCT-III outputs.
template <int N> __device__ __forceinline__ int mk_pos(int q) { return (q < N / 2) ? 2 * q : 2 * (N - 1 - q) + 1; }

// x/y forward kinds: DCT-II post-processing on (k, M-k) pairs with the outputs
// stored straight to global memory (consecutive lines are consecutive addresses).
template <typename T, int N, int KIND, int AX, class ST>
__device__ __forceinline__ void fast_post_store(const Grid& g, int line, const cx_t<T>* buf, const cx_t<T>* post,
                                                int l, int tj, const ST& st) {
  using Cf = FastCfg<T, N>;
  using C = cx_t<T>;
  constexpr int M = Cf::M, P = Cf::P, TPL = Cf::TPL;
  constexpr int NP = (M / 2) / TPL;
  auto put = [&](int pos, T v) {
    const int o = (KIND == K_S2) ? (N - 1 - pos) : pos;
    int i, j, k;
    long long idx;
    xy_coords<AX>(g, line, o, i, j, k, idx);
    st(i, j, k, idx, v);
  };
#pragma unroll
  for (int b = 0; b < NP; ++b) {
    const int k = tj + b * TPL;
    const C zk = buf[k * P + l];
    const C zm = buf[((M - k) & (M - 1)) * P + l];
    const C u0 = cadd(cmul(post[2 * k], zk), cmulc(post[2 * k + 1], zm));
    const int km = M - k;
    const C u1 = cadd(cmul(post[2 * km], zm), cmulc(post[2 * km + 1], zk));
    put(k, u0.x);
    put(M - k, u1.x);
    if (k > 0) {
      put(N - k, -u0.y);
      put(M + k, -u1.y);
    }
  }
  if (tj == 0) {
    const C z = buf[(M / 2) * P + l];
    const C u = cadd(cmul(post[M], z), cmulc(post[M + 1], z));
    put(M / 2, u.x);
    put(M + M / 2, -u.y);
  }
}

// x/y inverse kinds: the last radix-R2 stage with its outputs stored straight to
// global memory: slot m holds the (im, re)-swapped z_m, i.e. v_2m = .y, v_2m+1 = .x,
// and v_q lands at position mk_pos(q) (negated at odd positions for DST-III).
template <typename T, int N, int KIND, int AX, class ST>
__device__ __forceinline__ void fast_last_store(const Grid& g, int line, const cx_t<T>* buf, const cx_t<T>* tw, int l,
                                                int tj, const ST& st) {
  using Cf = FastCfg<T, N>;
  using C = cx_t<T>;
  constexpr int M = Cf::M, P = Cf::P, TPL = Cf::TPL, R = Cf::R2, NS = Cf::R1;
  constexpr int NB = M / R, PER = NB / TPL, STRIDE = M / R, TSTEP = M / (NS * R);
  C v[PER][R];
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int jb = tj + b * TPL;
#pragma unroll
    for (int r = 0; r < R; ++r) v[b][r] = buf[(jb + r * STRIDE) * P + l];
    const int jj = jb & (NS - 1);
#pragma unroll
    for (int r = 1; r < R; ++r) v[b][r] = cmul(v[b][r], tw[r * jj * TSTEP]);
    Dft<R, C>::run(v[b]);
  }
  auto put = [&](int q, T val) {
    const int pos = mk_pos<N>(q);
    if ((KIND == K_S3 || KIND == K_DERIV) && (pos & 1)) val = -val;
    int i, j, k;
    long long idx;
    xy_coords<AX>(g, line, pos, i, j, k, idx);
    st(i, j, k, idx, val);
  };
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int jb = tj + b * TPL;
    const int jj = jb & (NS - 1);
    const int base = (jb - jj) * R + jj;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int m = base + r * NS;
      put(2 * m, v[b][r].y);
      put(2 * m + 1, v[b][r].x);
    }
  }
}

template <typename T, int N, int KIND, int AX, class LoadOp, class StoreOp, class MulOp>
__global__ void __launch_bounds__(FastCfg<T, N>::NT) r2r_fast_kernel(Grid g, R2RTables<T> tb, LoadOp ld, StoreOp st,
                                                                     MulOp mul) {
  using Cf = FastCfg<T, N>;
  using C = cx_t<T>;
  constexpr int M = Cf::M, L = Cf::L, P = Cf::P, NT = Cf::NT, TPL = Cf::TPL, ITERS = Cf::ITERS, CH = Cf::CH;
  constexpr int R1 = Cf::R1, R2 = Cf::R2;
  constexpr bool fwd_in = (KIND == K_C2 || KIND == K_S2 || KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);
  constexpr bool inv_out = (KIND == K_C3 || KIND == K_S3 || KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);
  constexpr bool s2_in = (KIND == K_S2 || KIND == K_DERIVT);  // (-1)^p x_p on input
  constexpr bool xy = (AX != 2);  // x/y passes: global memory straight to/from registers
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  C* sfft = buf + M * P;
  C* spost = sfft + M;
  C* spre = spost + 2 * (M + 1);
  T* rb = reinterpret_cast<T*>(buf);
  const int tid = threadIdx.x;
  const long long line0 = (long long)blockIdx.x * L;
  const int l = tid & (L - 1), tj = tid >> Cf::LOG2L;
  const int my_line = (int)(line0 + l);

  for (int t = tid; t < M; t += NT) sfft[t] = __ldg(&tb.fft[t]);
  if constexpr (fwd_in)
    for (int t = tid; t < 2 * (M + 1); t += NT) spost[t] = __ldg(&tb.post[t]);
  if constexpr (inv_out)
    for (int t = tid; t < 2 * M; t += NT) spre[t] = __ldg(&tb.pre[t]);

  if constexpr (xy && fwd_in) {
    // ---- x/y forward: load the first radix-R1 butterfly's inputs straight into
    // registers (z_m = v_2m + i v_2m+1, m = tj + r TPL), DFT, one shared write ----
    C v[R1];
#pragma unroll
    for (int r = 0; r < R1; ++r) {
      const int m = tj + r * TPL;
      int i, j, k;
      long long idx;
      const int p0 = mk_pos<N>(2 * m), p1 = mk_pos<N>(2 * m + 1);
      xy_coords<AX>(g, my_line, p0, i, j, k, idx);
      T a = ld(i, j, k, idx);
      xy_coords<AX>(g, my_line, p1, i, j, k, idx);
      T b = ld(i, j, k, idx);
      if constexpr (s2_in) {
        if (p0 & 1) a = -a;
        if (p1 & 1) b = -b;
      }
      v[r] = cmake<C>(a, b);
    }
    Dft<R1, C>::run(v);
#pragma unroll
    for (int r = 0; r < R1; ++r) buf[(tj * R1 + r) * P + l] = v[r];
    __syncthreads();
  } else {
    // ---- load through shared memory: CH loads in flight per thread ----
#pragma unroll 1
    for (int c0 = 0; c0 < ITERS; c0 += CH) {
      T vals[CH];
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        int p, le, i, j, k;
        long long idx;
        fast_elem<N, NT, L, Cf::LOG2N, Cf::LOG2L, TPL>(g, AX, line0, tid, c0 + c, p, le, i, j, k, idx);
        vals[c] = ld(i, j, k, idx);
      }
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        int p, le, i, j, k;
        long long idx;
        fast_elem<N, NT, L, Cf::LOG2N, Cf::LOG2L, TPL>(g, AX, line0, tid, c0 + c, p, le, i, j, k, idx);
        T x = vals[c];
        if constexpr (fwd_in) {
          if (s2_in && (p & 1)) x = -x;
          const int q = (p & 1) ? (N - 1 - (p >> 1)) : (p >> 1);
          rb[fridx<P>(q, le)] = x;
        } else {
          rb[fridx<P>((KIND == K_S3) ? (N - 1 - p) : p, le)] = x;
        }
      }
    }
    __syncthreads();
    if constexpr (fwd_in) fast_stage<C, M, R1, 1, TPL, P>(buf, sfft, l, tj);
  }

  if constexpr (fwd_in) {
    fast_stage<C, M, R2, R1, TPL, P>(buf, sfft, l, tj);
    if constexpr (xy && KIND != K_FILT && KIND != K_DERIV && KIND != K_DERIVT) {
      fast_post_store<T, N, KIND, AX>(g, my_line, buf, spost, l, tj, st);
      return;
    }
    fast_post<T, N, (KIND == K_DERIV ? K_C2 : (KIND == K_DERIVT ? K_S2 : KIND)), MulOp>(g, AX, line0 + l, buf,
                                                                                        spost, l, tj, mul);
    if constexpr (KIND == K_DERIV) {
      // w_i = mul(i) u_{i+1} (w_{N-1} = 0), stored reversed as the DST-III input
      constexpr int PER = N / TPL;
      T w[PER];
#pragma unroll
      for (int b = 0; b < PER; ++b) {
        const int i = tj + b * TPL;
        w[b] = (T)0;
        if (i < N - 1) {
          int ii, jj, kk;
          long long idx;
          line_coords(g, AX, line0 + l, i, ii, jj, kk, idx);
          w[b] = mul(ii, jj, kk) * rb[fridx<P>(i + 1, l)];
        }
      }
      __syncthreads();
#pragma unroll
      for (int b = 0; b < PER; ++b) rb[fridx<P>(N - 1 - (tj + b * TPL), l)] = w[b];
      __syncthreads();
    }
    if constexpr (KIND == K_DERIVT) {
      // u_j = mul(j-1) z_{j-1} (u_0 = 0) from the DST-II output z, natural order (DCT-III input)
      constexpr int PER = N / TPL;
      T w[PER];
#pragma unroll
      for (int b = 0; b < PER; ++b) {
        const int j = tj + b * TPL;
        w[b] = (T)0;
        if (j >= 1) {
          int ii, jj, kk;
          long long idx;
          line_coords(g, AX, line0 + l, j - 1, ii, jj, kk, idx);
          w[b] = mul(ii, jj, kk) * rb[fridx<P>(j - 1, l)];
        }
      }
      __syncthreads();
#pragma unroll
      for (int b = 0; b < PER; ++b) rb[fridx<P>(tj + b * TPL, l)] = w[b];
      __syncthreads();
    }
  }
  if constexpr (inv_out) {
    fast_pre<T, N>(buf, spre, l, tj);
    fast_stage<C, M, R1, 1, TPL, P>(buf, sfft, l, tj);
    if constexpr (xy) {
      fast_last_store<T, N, KIND, AX>(g, my_line, buf, sfft, l, tj, st);
      return;
    }
    fast_stage<C, M, R2, R1, TPL, P>(buf, sfft, l, tj);
  }

  // ---- z store: batched shared reads, then global stores ----
#pragma unroll 1
  for (int c0 = 0; c0 < ITERS; c0 += CH) {
    T vals[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      int p, le, i, j, k;
      long long idx;
      fast_elem<N, NT, L, Cf::LOG2N, Cf::LOG2L, TPL>(g, AX, line0, tid, c0 + c, p, le, i, j, k, idx);
      if constexpr (inv_out) {
        const int q = (p & 1) ? (N - 1 - (p >> 1)) : (p >> 1);
        T y = rb[fridx<P>(q, le) ^ 1];
        if ((KIND == K_S3 || KIND == K_DERIV) && (p & 1)) y = -y;
        vals[c] = y;
      } else {
        vals[c] = rb[fridx<P>(p, le)];
      }
    }
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      int p, le, i, j, k;
      long long idx;
      fast_elem<N, NT, L, Cf::LOG2N, Cf::LOG2L, TPL>(g, AX, line0, tid, c0 + c, p, le, i, j, k, idx);
      st(i, j, k, idx, vals[c]);
    }
  }
}

}  // namespace swc
