// swc_r2r.cuh -- one axis pass of a 3D real-to-real transform (FFTW REDFT10/01,
// RODFT10/01 definitions) as an sm_103a kernel.
//
// A CTA stages L lines of length n along one axis in shared memory and transforms
// them with Makhoul's mapping onto an M = n/2 point complex FFT:
//   DCT-II : v = (x0, x2, ..., x3, x1), z_m = v_2m + i v_2m+1, Z = DFT_M(z),
//            u_k = c_k Z_k + d_k conj(Z_{M-k}),  Y_k = Re u_k, Y_{n-k} = -Im u_k
//   DCT-III: U_k = X_k - i X_{n-k}, Z_k = a_k U_k + b_k conj(U_{M-k}),
//            z = IDFT_M(Z) (unnormalised), y = inverse permutation of (Re z, Im z)
//   DST-II (x)_k = DCT-II((-1)^n x_n)_{n-1-k};  DST-III(x)_k = (-1)^k DCT-III(x reversed)_k
// with c, d, a, b tabulated per length (swc_tables.cu). The FFT is a Stockham
// autosort sequence of radix-16/8/4/2 stages, each thread holding one radix-R
// butterfly in registers; the inverse FFT is the forward one on (im, re)-swapped
// data, so only forward stages exist. Load and store functors fuse the pointwise
// work of the step into the first and last pass of each 3D transform.
#pragma once

#include "swc_common.cuh"

namespace swc {

// K_FILT: DCT-II, spectral multiplier, DCT-III along the axis (one CTA).
// K_DERIV: DCT-II, then w_i = mul(i) u_{i+1} (w_{n-1} = 0), then DST-III: the shifted
// spectral derivative of REF:1166-1250 along one axis in one pass.
// K_DERIVT: its transpose, DST-II, then u_j = mul(j-1) z_{j-1} (u_0 = 0), then DCT-III
// (with FFTW's definitions the transposes' mode-0 / last-mode weights drop out: the
// shift never reads z_{n-1} and writes u_0 = 0).
enum Kind { K_C2 = 0, K_C3 = 1, K_S2 = 2, K_S3 = 3, K_FILT = 4, K_DERIV = 5, K_DERIVT = 6 };

template <typename T> struct R2RTables {
  const cx_t<T>* fft;   // W_M^t = exp(-2 pi i t/M), t < M
  const cx_t<T>* post;  // DCT-II post-twiddles: post[2k] = c_k, post[2k+1] = d_k, k = 0..M
  const cx_t<T>* pre;   // DCT-III pre-twiddles : pre[2k] = a_k, pre[2k+1] = b_k, k < M
  int* status;          // device flag set to 1 when a pass's bounded wait runs out (or null)
  int max_polls = 1 << 22;  // bound of each wait of the TMA-fed pass (mbarrier polls)
  int wait_extra_tx = 0;    // test support: extra bytes each tile wait expects (0 = none)
  int rev = 0;              // TMA-fed pass: walk the tiles from the last one down
};

struct PassShape {
  int n, log2n;   // line length
  int axis;       // 0 = x (slowest), 1 = y, 2 = z (contiguous)
  int L, log2L;   // lines per CTA (power of two)
  int P;          // complex row pitch in shared memory (L + 1: staggers banks)
  int tpl;        // threads per line
  int nst;        // Stockham stages
  int radix[4];
  long long nlines;
};

// ---- register DFTs (forward, exp(-2 pi i/R)) ------------------------------------

// cos / sin of 2 pi k / 16, k = 0..7 (exact decimal expansions of sqrt-expressions).
#define SWC_C16_1 0.92387953251128675613
#define SWC_S16_1 0.38268343236508977173
#define SWC_R2H 0.70710678118654752440

template <int R, int K, typename C> __device__ __forceinline__ C twid(C v) {
  using T = decltype(C::x);
  constexpr int k16 = K * (16 / R);  // same angle on the 16-point circle
  if constexpr (k16 == 0) {
    return v;
  } else if constexpr (k16 == 4) {  // -i
    return cmake<C>(v.y, -v.x);
  } else if constexpr (k16 == 2) {  // (1 - i)/sqrt2
    return cmake<C>((T)SWC_R2H * (v.x + v.y), (T)SWC_R2H * (v.y - v.x));
  } else if constexpr (k16 == 6) {  // (-1 - i)/sqrt2
    return cmake<C>((T)SWC_R2H * (v.y - v.x), -(T)SWC_R2H * (v.x + v.y));
  } else {
    constexpr double cs[8] = {1.0, SWC_C16_1, SWC_R2H, SWC_S16_1, 0.0, -SWC_S16_1, -SWC_R2H, -SWC_C16_1};
    constexpr double sn[8] = {0.0, SWC_S16_1, SWC_R2H, SWC_C16_1, 1.0, SWC_C16_1, SWC_R2H, SWC_S16_1};
    const T c = (T)cs[k16], s = (T)sn[k16];
    // v * (c - i s)
    return cmake<C>(v.x * c + v.y * s, v.y * c - v.x * s);
  }
}

template <int R, typename C> struct Dft {
  template <int K> __device__ __forceinline__ static void combine(C* v, const C* e, const C* o) {
    if constexpr (K < R / 2) {
      const C t = twid<R, K>(o[K]);
      v[K] = cadd(e[K], t);
      v[K + R / 2] = csub(e[K], t);
      combine<K + 1>(v, e, o);
    }
  }
  __device__ __forceinline__ static void run(C* v) {
    C e[R / 2], o[R / 2];
#pragma unroll
    for (int i = 0; i < R / 2; ++i) { e[i] = v[2 * i]; o[i] = v[2 * i + 1]; }
    Dft<R / 2, C>::run(e);
    Dft<R / 2, C>::run(o);
    combine<0>(v, e, o);
  }
};
template <typename C> struct Dft<1, C> {
  __device__ __forceinline__ static void run(C*) {}
};

// One radix-R Stockham stage for butterfly jb of one line (complex rows of pitch P).
template <int R, typename C>
__device__ __forceinline__ void stockham_stage(const C* __restrict__ src, C* __restrict__ dst, int M, int Ns,
                                               int P, int l, int jb, const C* tw) {
  C v[R];
  const int stride = M / R;
#pragma unroll
  for (int r = 0; r < R; ++r) v[r] = src[(jb + r * stride) * P + l];
  const int jj = jb & (Ns - 1);
  if (Ns > 1) {
    const int tstep = M / (Ns * R);
#pragma unroll
    for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[r * jj * tstep]);
  }
  Dft<R, C>::run(v);
  const int base = (jb - jj) * R + jj;
#pragma unroll
  for (int r = 0; r < R; ++r) dst[(base + r * Ns) * P + l] = v[r];
}

// ---- geometry helpers ---------------------------------------------------------------

// Coordinates and linear index of element p of line `id` of a pass along `axis`.
__device__ __forceinline__ void line_coords(const Grid& g, int axis, long long id, int p, int& i, int& j, int& k,
                                            long long& idx) {
  if (axis == 2) {
    i = (int)(id >> g.ly);
    j = (int)(id & (g.ny - 1));
    k = p;
    idx = (id << g.lz) + p;
  } else if (axis == 1) {
    i = (int)(id >> g.lz);
    k = (int)(id & (g.nz - 1));
    j = p;
    idx = ((long long)i << (g.ly + g.lz)) + ((long long)p << g.lz) + k;
  } else {
    j = (int)(id >> g.lz);
    k = (int)(id & (g.nz - 1));
    i = p;
    idx = ((long long)p << (g.ly + g.lz)) + id;
  }
}

// real element r of line l in a complex-row buffer: component (r & 1) of slot (r >> 1)
__device__ __forceinline__ int ridx(int r, int l, int P) { return (((r >> 1) * P + l) << 1) + (r & 1); }

// Vector loads / stores for the FP32 two-line pass: 2 or 4 consecutive elements from
// an even / a multiple-of-4 index (float2/float4, or double2 pairs converted to FP32).
template <typename U> __device__ __forceinline__ float2 ld2v(const U* p, long long idx) {
  if constexpr (sizeof(U) == 4) {
    return *reinterpret_cast<const float2*>(p + idx);
  } else {
    const double2 d = *reinterpret_cast<const double2*>(p + idx);
    return make_float2((float)d.x, (float)d.y);
  }
}
template <typename U> __device__ __forceinline__ float4 ld4v(const U* p, long long idx) {
  if constexpr (sizeof(U) == 4) {
    return *reinterpret_cast<const float4*>(p + idx);
  } else {
    const double2 d0 = *reinterpret_cast<const double2*>(p + idx);
    const double2 d1 = *reinterpret_cast<const double2*>(p + idx + 2);
    return make_float4((float)d0.x, (float)d0.y, (float)d1.x, (float)d1.y);
  }
}
// The same loads through the read-only data path (ld.global.nc): for functors that also
// store, these loads may be scheduled ahead of the stores of earlier elements. Valid
// when every element is read before it is written and by the thread that writes it.
template <typename U> __device__ __forceinline__ float2 ld2g(const U* p, long long idx) {
  if constexpr (sizeof(U) == 4) {
    return __ldg(reinterpret_cast<const float2*>(p + idx));
  } else {
    const double2 d = __ldg(reinterpret_cast<const double2*>(p + idx));
    return make_float2((float)d.x, (float)d.y);
  }
}
template <typename U> __device__ __forceinline__ float4 ld4g(const U* p, long long idx) {
  if constexpr (sizeof(U) == 4) {
    return __ldg(reinterpret_cast<const float4*>(p + idx));
  } else {
    const double2 d0 = __ldg(reinterpret_cast<const double2*>(p + idx));
    const double2 d1 = __ldg(reinterpret_cast<const double2*>(p + idx + 2));
    return make_float4((float)d0.x, (float)d0.y, (float)d1.x, (float)d1.y);
  }
}
__device__ __forceinline__ double2 ld2dg(const double* p, long long idx) {
  return __ldg(reinterpret_cast<const double2*>(p + idx));
}
template <typename U> __device__ __forceinline__ void st2v(U* p, long long idx, float2 v) {
  if constexpr (sizeof(U) == 4) {
    *reinterpret_cast<float2*>(p + idx) = v;
  } else {
    *reinterpret_cast<double2*>(p + idx) = make_double2(v.x, v.y);
  }
}
template <typename U> __device__ __forceinline__ void st4v(U* p, long long idx, float4 v) {
  if constexpr (sizeof(U) == 4) {
    *reinterpret_cast<float4*>(p + idx) = v;
  } else {
    *reinterpret_cast<double2*>(p + idx) = make_double2(v.x, v.y);
    *reinterpret_cast<double2*>(p + idx + 2) = make_double2(v.z, v.w);
  }
}

// Plain load / store functors (with precision conversion); pair / quad are the vector
// forms used by the FP32 two-line pass.
template <typename T, typename U> struct LdPlain {
  const U* p;
  __device__ __forceinline__ T operator()(int, int, int, long long idx) const { return (T)p[idx]; }
  __device__ __forceinline__ float2 pair(int, int, int, long long idx) const { return ld2v(p, idx); }
  __device__ __forceinline__ float4 quad(int, int, int, long long idx) const { return ld4v(p, idx); }
};
template <typename T, typename U> struct StPlain {
  U* p;
  __device__ __forceinline__ void operator()(int, int, int, long long idx, T v) const { p[idx] = (U)v; }
  __device__ __forceinline__ void pair(int, int, int, long long idx, float2 v) const { st2v(p, idx, v); }
  __device__ __forceinline__ void quad(int, int, int, long long idx, float4 v) const { st4v(p, idx, v); }
};

// Identity multiplier for non-filter passes.
template <typename T> struct NoMul {
  __device__ __forceinline__ T operator()(int, int, int) const { return (T)1; }
};

// Plain FP32 load times a pointwise multiplier m(i, j, k) (a spectral multiplier on the
// input of an inverse pass). The TMA-fed z pass applies m as it reads the staged tile,
// so such a pass keeps the TMA pipeline; the direct passes use these forms.
template <class M> struct LdMul {
  const float* p;
  M m;
  __device__ __forceinline__ float operator()(int i, int j, int k, long long idx) const { return p[idx] * m(i, j, k); }
  __device__ __forceinline__ float2 pair(int i, int j, int k, long long idx) const {
    const float2 v = ld2v(p, idx);
    return make_float2(v.x * m(i, j, k), v.y * m(i, j, k + 1));
  }
  __device__ __forceinline__ float4 quad(int i, int j, int k, long long idx) const {
    const float4 v = ld4v(p, idx);
    return make_float4(v.x * m(i, j, k), v.y * m(i, j, k + 1), v.z * m(i, j, k + 2), v.w * m(i, j, k + 3));
  }
};

// ---- the pass kernel ------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ void run_stages(const PassShape& ps, cx_t<T>*& src, cx_t<T>*& dst, int l, int tj,
                                           const cx_t<T>* tw) {
  using C = cx_t<T>;
  const int M = ps.n >> 1;
  int Ns = 1;
  for (int s = 0; s < ps.nst; ++s) {
    const int R = ps.radix[s];
    const int nb = M / R;
    for (int jb = tj; jb < nb; jb += ps.tpl) {
      switch (R) {
        case 16: stockham_stage<16, C>(src, dst, M, Ns, ps.P, l, jb, tw); break;
        case 8: stockham_stage<8, C>(src, dst, M, Ns, ps.P, l, jb, tw); break;
        case 4: stockham_stage<4, C>(src, dst, M, Ns, ps.P, l, jb, tw); break;
        default: stockham_stage<2, C>(src, dst, M, Ns, ps.P, l, jb, tw); break;
      }
    }
    __syncthreads();
    C* t = src; src = dst; dst = t;
    Ns *= R;
  }
}

// DCT-III pre-processing: real input (natural order, `in` reals) -> swapped Z in `out`.
template <typename T>
__device__ __forceinline__ void dct3_pre(const PassShape& ps, const T* in, cx_t<T>* out, int l, int tj,
                                         const cx_t<T>* pre) {
  using C = cx_t<T>;
  const int n = ps.n, M = n >> 1, P = ps.P;
  for (int k = tj; k < M; k += ps.tpl) {
    const T xk = in[ridx(k, l, P)];
    const T xnk = (k == 0) ? (T)0 : in[ridx(n - k, l, P)];
    const T xmk = in[ridx(M - k, l, P)];
    const T xmpk = in[ridx(M + k, l, P)];
    const C a = pre[2 * k], b = pre[2 * k + 1];
    const C U = cmake<C>(xk, -xnk);
    const C Um = cmake<C>(xmk, -xmpk);
    const C Z = cadd(cmul(a, U), cmulc(b, Um));
    out[k * P + l] = cswap(Z);
  }
}

// DCT-II post-processing: Z in `in` -> real output (natural order) in `out`, with the
// output order reversed for DST-II and an optional spectral multiplier (filter pass).
template <typename T, int KIND, class MulOp>
__device__ __forceinline__ void dct2_post(const Grid& g, const PassShape& ps, long long id, const cx_t<T>* in, T* out,
                                          int l, int tj, const cx_t<T>* post, const MulOp& mul) {
  using C = cx_t<T>;
  const int n = ps.n, M = n >> 1, P = ps.P;
  for (int k = tj; k <= M; k += ps.tpl) {
    const C zk = in[(k & (M - 1)) * P + l];
    const C zm = in[((M - k) & (M - 1)) * P + l];
    const C c = post[2 * k], d = post[2 * k + 1];
    const C u = cadd(cmul(c, zk), cmulc(d, zm));
    T y0 = u.x;
    if constexpr (KIND == K_FILT) {
      int i, j, kk; long long idx;
      line_coords(g, ps.axis, id, k, i, j, kk, idx);
      y0 *= mul(i, j, kk);
    }
    const int p0 = (KIND == K_S2) ? (n - 1 - k) : k;
    out[ridx(p0, l, P)] = y0;
    if (k > 0 && k < M) {
      T y1 = -u.y;
      if constexpr (KIND == K_FILT) {
        int i, j, kk; long long idx;
        line_coords(g, ps.axis, id, n - k, i, j, kk, idx);
        y1 *= mul(i, j, kk);
      }
      const int p1 = (KIND == K_S2) ? (k - 1) : (n - k);
      out[ridx(p1, l, P)] = y1;
    }
  }
}

// Element `e` of a CTA's tile -> (position p along the line, tile line le). The z
// tile is L consecutive rows (contiguous memory): consecutive threads take
// consecutive positions. x/y tiles are n rows of L consecutive k: consecutive
// threads take consecutive lines (consecutive k). Both keep global accesses coalesced.
__device__ __forceinline__ void tile_elem(const PassShape& ps, int e, int& p, int& le) {
  if (ps.axis == 2) { p = e & (ps.n - 1); le = e >> ps.log2n; }
  else { le = e & (ps.L - 1); p = e >> ps.log2L; }
}

// Element `it` of thread `tid` (elements tid + it*threads of the tile): position p,
// tile line le, grid coordinates and linear index, computed affinely from the
// thread's fixed line (x/y passes) or the contiguous tile (z pass).
__device__ __forceinline__ void elem_coords(const Grid& g, const PassShape& ps, long long line0, int tid, int it,
                                            int& p, int& le, int& i, int& j, int& k, long long& idx) {
  if (ps.axis == 2) {
    const int e = tid + it * (ps.L * ps.tpl);
    p = e & (ps.n - 1);
    le = e >> ps.log2n;
    const long long line = line0 + le;
    i = (int)(line >> g.ly);
    j = (int)line & (g.ny - 1);
    k = p;
    idx = (line0 << ps.log2n) + e;
  } else {
    le = tid & (ps.L - 1);
    p = (tid >> ps.log2L) + it * ps.tpl;
    const int line = (int)(line0 + le);
    if (ps.axis == 1) {
      i = line >> g.lz;
      k = line & (g.nz - 1);
      j = p;
      idx = ((long long)i << (g.ly + g.lz)) + ((long long)(p << g.lz) + k);
    } else {
      j = line >> g.lz;
      k = line & (g.nz - 1);
      i = p;
      idx = ((long long)p << (g.ly + g.lz)) + line;
    }
  }
}

// Copy the twiddle tables a pass needs from global memory into shared memory.
template <typename T, int KIND>
__device__ __forceinline__ void stage_tables(const PassShape& ps, const R2RTables<T>& tb, cx_t<T>* sfft,
                                             cx_t<T>* spost, cx_t<T>* spre) {
  const int M = ps.n >> 1;
  for (int t = threadIdx.x; t < M; t += blockDim.x) sfft[t] = __ldg(&tb.fft[t]);
  if constexpr (KIND == K_C2 || KIND == K_S2 || KIND == K_FILT)
    for (int t = threadIdx.x; t < 2 * (M + 1); t += blockDim.x) spost[t] = __ldg(&tb.post[t]);
  if constexpr (KIND == K_C3 || KIND == K_S3 || KIND == K_FILT)
    for (int t = threadIdx.x; t < 2 * M; t += blockDim.x) spre[t] = __ldg(&tb.pre[t]);
}

// One axis pass. LoadOp: T(i, j, k, idx); StoreOp: void(i, j, k, idx, T).
// Every element of the array is loaded exactly once and stored exactly once, so
// load functors may also update other arrays at the same index.
// ITERS = elements per thread in the load/store phases (n*L/threads = 2*RMAX) when
// known at compile time: all of a thread's loads are then issued before any shared
// memory store, and all shared reads before any global store. ITERS = 0: runtime
// loop (short lines).
template <typename T, int KIND, int ITERS, class LoadOp, class StoreOp, class MulOp = NoMul<T>>
__global__ void __launch_bounds__(256) r2r_pass_kernel(Grid g, PassShape ps, R2RTables<T> tb, LoadOp ld,
                                                       StoreOp st, MulOp mul = MulOp()) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = ps.n, M = n >> 1, L = ps.L, P = ps.P;
  C* bufA = reinterpret_cast<C*>(smem_raw);
  C* bufB = bufA + M * P;
  C* sfft = bufB + M * P;        // M
  C* spost = sfft + M;           // 2(M+1)
  C* spre = spost + 2 * (M + 1);  // 2M
  const int tid = threadIdx.x, nt = blockDim.x;
  const long long line0 = (long long)blockIdx.x * L;
  const int l = tid & (L - 1);
  const int tj = tid >> ps.log2L;
  const long long my_line = line0 + l;
  constexpr bool fwd_in = (KIND == K_C2 || KIND == K_S2 || KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);

  stage_tables<T, ((KIND == K_DERIV || KIND == K_DERIVT) ? K_FILT : KIND)>(ps, tb, sfft, spost, spre);

  // ---- load: global -> bufA reals ----
  {
    T* ra = reinterpret_cast<T*>(bufA);
    auto place = [&](int p, int le, T x) {
      if constexpr (fwd_in) {
        if ((KIND == K_S2 || KIND == K_DERIVT) && (p & 1)) x = -x;
        const int q = (p & 1) ? (n - 1 - (p >> 1)) : (p >> 1);
        ra[ridx(q, le, P)] = x;
      } else {
        const int pos = (KIND == K_S3) ? (n - 1 - p) : p;
        ra[ridx(pos, le, P)] = x;
      }
    };
    if constexpr (ITERS > 0) {
      // chunks of CH loads in flight per thread, then their shared-memory stores
      constexpr int CH = (sizeof(T) == 8) ? 8 : 16;
#pragma unroll 1
      for (int c0 = 0; c0 < ITERS; c0 += CH) {
        T vals[CH];
#pragma unroll
        for (int c = 0; c < CH; ++c) {
          int p, le, i, j, k;
          long long idx;
          elem_coords(g, ps, line0, tid, c0 + c, p, le, i, j, k, idx);
          vals[c] = ld(i, j, k, idx);
        }
#pragma unroll
        for (int c = 0; c < CH; ++c) {
          int p, le;
          tile_elem(ps, tid + (c0 + c) * nt, p, le);
          place(p, le, vals[c]);
        }
      }    } else {
      const int iters = (n * L) / nt;
      for (int it = 0; it < iters; ++it) {
        int p, le, i, j, k;
        long long idx;
        tile_elem(ps, tid + it * nt, p, le);
        line_coords(g, ps.axis, line0 + le, p, i, j, k, idx);
        place(p, le, ld(i, j, k, idx));
      }
    }
  }
  __syncthreads();

  C* src = bufA;
  C* dst = bufB;
  T* res_real;   // natural-order real output
  bool swapped;  // output components are (im, re)-swapped (inverse FFT result)
  if constexpr (fwd_in) {
    run_stages<T>(ps, src, dst, l, tj, sfft);  // result in src
    dct2_post<T, (KIND == K_DERIV ? K_C2 : (KIND == K_DERIVT ? K_S2 : KIND)), MulOp>(
        g, ps, my_line, src, reinterpret_cast<T*>(dst), l, tj, spost, mul);
    __syncthreads();
    if constexpr (KIND == K_DERIV) {
      // w_i = mul(i) u_{i+1}, stored reversed (DST-III input), then the DST-III
      const T* u = reinterpret_cast<const T*>(dst);
      T* w = reinterpret_cast<T*>(src);
      for (int i = tj; i < n; i += ps.tpl) {
        T v = (T)0;
        if (i < n - 1) {
          int ii, jj, kk;
          long long idx;
          line_coords(g, ps.axis, my_line, i, ii, jj, kk, idx);
          v = mul(ii, jj, kk) * u[ridx(i + 1, l, P)];
        }
        w[ridx(n - 1 - i, l, P)] = v;
      }
      __syncthreads();
      dct3_pre<T>(ps, reinterpret_cast<const T*>(src), dst, l, tj, spre);
      __syncthreads();
      { C* t = src; src = dst; dst = t; }
      run_stages<T>(ps, src, dst, l, tj, sfft);
      res_real = reinterpret_cast<T*>(src);
      swapped = true;
    } else if constexpr (KIND == K_DERIVT) {
      // u_j = mul(j-1) z_{j-1} (u_0 = 0) from the DST-II output z, natural order (the
      // DCT-III input), then the DCT-III
      const T* z = reinterpret_cast<const T*>(dst);
      T* u = reinterpret_cast<T*>(src);
      for (int j = tj; j < n; j += ps.tpl) {
        T v = (T)0;
        if (j >= 1) {
          int ii, jj, kk;
          long long idx;
          line_coords(g, ps.axis, my_line, j - 1, ii, jj, kk, idx);
          v = mul(ii, jj, kk) * z[ridx(j - 1, l, P)];
        }
        u[ridx(j, l, P)] = v;
      }
      __syncthreads();
      dct3_pre<T>(ps, reinterpret_cast<const T*>(src), dst, l, tj, spre);
      __syncthreads();
      { C* t = src; src = dst; dst = t; }
      run_stages<T>(ps, src, dst, l, tj, sfft);
      res_real = reinterpret_cast<T*>(src);
      swapped = true;
    } else if constexpr (KIND == K_FILT) {
      // inverse DCT-III of the filtered spectrum, in the same CTA
      dct3_pre<T>(ps, reinterpret_cast<const T*>(dst), src, l, tj, spre);
      __syncthreads();
      run_stages<T>(ps, src, dst, l, tj, sfft);
      res_real = reinterpret_cast<T*>(src);
      swapped = true;
    } else {
      res_real = reinterpret_cast<T*>(dst);
      swapped = false;
    }
  } else {
    dct3_pre<T>(ps, reinterpret_cast<const T*>(src), dst, l, tj, spre);
    __syncthreads();
    { C* t = src; src = dst; dst = t; }
    run_stages<T>(ps, src, dst, l, tj, sfft);
    res_real = reinterpret_cast<T*>(src);
    swapped = true;
  }

  // ---- store: result -> global ----
  auto fetch = [&](int p, int le) -> T {
    if (swapped) {
      const int q = (p & 1) ? (n - 1 - (p >> 1)) : (p >> 1);
      T y = res_real[ridx(q, le, P) ^ 1];
      if ((KIND == K_S3 || KIND == K_DERIV) && (p & 1)) y = -y;
      return y;
    }
    return res_real[ridx(p, le, P)];
  };
  if constexpr (ITERS > 0) {
    constexpr int CH = (sizeof(T) == 8) ? 8 : 16;
#pragma unroll 1
    for (int c0 = 0; c0 < ITERS; c0 += CH) {
      T vals[CH];
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        int p, le;
        tile_elem(ps, tid + (c0 + c) * nt, p, le);
        vals[c] = fetch(p, le);
      }
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        int p, le, i, j, k;
        long long idx;
        elem_coords(g, ps, line0, tid, c0 + c, p, le, i, j, k, idx);
        st(i, j, k, idx, vals[c]);
      }
    }  } else {
    const int iters = (n * L) / nt;
    for (int it = 0; it < iters; ++it) {
      int p, le, i, j, k;
      long long idx;
      tile_elem(ps, tid + it * nt, p, le);
      line_coords(g, ps.axis, line0 + le, p, i, j, k, idx);
      st(i, j, k, idx, fetch(p, le));
    }
  }
}

// Shared-memory bytes of a pass: two complex buffers of M rows of pitch P, plus the
// FFT (M), DCT-II post (2(M+1)) and DCT-III pre (2M) twiddle tables.
inline size_t pass_smem_bytes(const PassShape& ps, size_t elem) {
  const size_t M = ps.n / 2;
  return (2 * M * ps.P + 5 * M + 2) * 2 * elem;
}

}  // namespace swc
