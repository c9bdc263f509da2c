// swc_r2r_tma.cuh -- the FP32 two-line r2r pass fed by the Tensor Memory Accelerator.
//
// Persistent CTAs walk tiles of 2 LP lines. Each tile arrives in shared memory by
// asynchronous copies -- a tiled tensor-map load (cp.async.bulk.tensor.3d) for x/y
// passes, whose tile is N rows of 2 LP adjacent lines; for z passes, whose 2 LP lines
// are one block of memory, one contiguous bulk copy (cp.async.bulk), or at N = 256 one
// bulk copy per line into padded rows (row staging, tma_issue_zrow) -- issued as soon as
// the previous tile has left the staging buffer, so the DRAM read of tile t+1 overlaps
// the transform and the stores of tile t. Completion is an
// mbarrier transaction count; every wait is bounded (tables' max_polls): a wait that
// runs out sets the tables' status flag and the CTA returns after one more bounded wait
// for its copy in flight. Test support: wait_extra_tx makes every wait expect more bytes
// than its copy delivers, so the wait runs out while the copy itself is a valid one; on
// the way out those extra bytes are credited (mbarrier.complete_tx), so the second wait
// ends when the valid copy has landed.
// Used for plain FP32 loads (LdPlain<float, float>, or times a multiplier applied to the
// staged tile: LdMul), any store/multiplier.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <type_traits>

#include "swc_r2r_pair.cuh"

namespace swc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Credit `bytes` of transaction count to the current phase, as landed copy bytes would.
__device__ __forceinline__ void mbar_complete_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.complete_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, int max_polls) {
  for (int it = 0; it < max_polls; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// tiled 3D tensor load into shared memory, completing on an mbarrier
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}
// contiguous bulk load (16-byte aligned addresses, size a multiple of 16 bytes)
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

template <int N> struct TmaCfg {
  using Cf = PairCfg<N>;
  static constexpr int LINES = 2 * Cf::LP;              // lines per tile
  static constexpr int TILE_BYTES = LINES * N * 4;      // bytes one tile copy delivers
  static constexpr int BOXN = (N < 256) ? N : 256;      // tensor box extent along the pass axis
  static constexpr int NBOX = N / BOXN;
  // Row staging of z tiles (zrow_kind): line l of the tile in row (l >> 1) + LP (l & 1)
  // of pitch N + 4 floats, so that lanes on consecutive line pairs read float4 a of
  // their lines from consecutive 16-byte bank groups.
  static constexpr bool ZROW = (N == 256 && Cf::R3 == 1 && LINES == 32);
  static constexpr int ZPITCH = N + 4;
  static constexpr int STAGE_BYTES = ZROW ? LINES * ZPITCH * 4 : TILE_BYTES;
  static_assert(TILE_BYTES < (1 << 20), "mbarrier transaction count");
  // staging tile + PC work buffer + tables + mbarrier
  static constexpr size_t smem_bytes() { return (size_t)STAGE_BYTES + Cf::smem_bytes() + 16; }
};

// x/y: a tile must not straddle rows of the array (nz a multiple of the tile's lines).
template <int N> inline bool tma_pass_supported(const Grid& g, int axis) {
  if (!pair_pass_supported<N>(g, axis)) return false;
  const long long nlines = g.ng / N;
  if (nlines % TmaCfg<N>::LINES) return false;
  return axis == 2 || (g.nz % TmaCfg<N>::LINES) == 0;
}

// one thread: expect the tile's bytes on the mbarrier and start its copy
template <int N, int AX>
__device__ __forceinline__ void tma_issue(const Grid& g, const CUtensorMap* map, const float* zsrc, int t,
                                          uint32_t sdst, uint32_t bar, int extra_tx) {
  using Tc = TmaCfg<N>;
  mbar_expect_tx(bar, Tc::TILE_BYTES + extra_tx);
  const int line0 = t * Tc::LINES;
  if constexpr (AX == 2) {
    bulk_load(sdst, zsrc + (size_t)line0 * N, Tc::TILE_BYTES, bar);
  } else {
    const int k0 = line0 & (g.nz - 1), o = line0 >> g.lz;  // o = i (y pass) or j (x pass)
#pragma unroll
    for (int b = 0; b < Tc::NBOX; ++b) {
      const uint32_t d = sdst + (uint32_t)(b * Tc::BOXN * Tc::LINES * 4);
      if constexpr (AX == 1) tma_load_3d(d, map, k0, b * Tc::BOXN, o, bar);
      else tma_load_3d(d, map, k0, o, b * Tc::BOXN, bar);
    }
  }
}

// one warp: the z tile in row staging, one line per lane (a contiguous bulk copy of N
// floats into row (l >> 1) + LP (l & 1)); lane 0 expects the tile's bytes first
template <int N>
__device__ __forceinline__ void tma_issue_zrow(const float* zsrc, int t, uint32_t sdst, uint32_t bar, int extra_tx,
                                               int lane) {
  using Tc = TmaCfg<N>;
  static_assert(Tc::ZROW, "row staging");
  if (lane == 0) mbar_expect_tx(bar, Tc::TILE_BYTES + extra_tx);
  __syncwarp();
  const uint32_t row = (uint32_t)((lane >> 1) + PairCfg<N>::LP * (lane & 1));
  bulk_load(sdst + row * (uint32_t)(Tc::ZPITCH * 4), zsrc + ((size_t)t * Tc::LINES + lane) * N, N * 4, bar);
}

// LMUL: a pointwise multiplier of the loaded values (LdMul); the z pass of the inverse
// cosine kind applies it as it reads the staged tile, the other forms take NoMul only.
// ZT: z pass with the row staging (tma_issue_zrow): each thread loads the inputs of its
// two first-stage butterflies straight from the staged tile -- the Makhoul-ordered
// elements (forward kinds) or the DCT-III pre-processed pairs (inverse kinds) -- and the
// line-pair re-layout of the z tile is not needed.
template <int N, int KIND, int AX, class StoreOp, class MulOp, class LMul, bool ZT = false>
__global__ void __launch_bounds__(PairCfg<N>::NT) r2r_tma_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                 const float* __restrict__ zsrc, Grid g,
                                                                 R2RTables<float> tb, StoreOp st, MulOp mul,
                                                                 LMul lmul, int ntiles) {
  using Cf = PairCfg<N>;
  using Tc = TmaCfg<N>;
  constexpr int M = Cf::M, LP = Cf::LP, PP = Cf::PP, NT = Cf::NT, TPL = Cf::TPL, NQ = Cf::NQ;
  constexpr int R1 = Cf::R1;
  constexpr bool fwd_in = (KIND == K_C2 || KIND == K_S2 || KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);
  constexpr bool inv_out = (KIND == K_C3 || KIND == K_S3 || KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);
  constexpr bool xy = (AX != 2);
  constexpr int ZU = (LP * NQ) / NT;
  constexpr bool load_mul = !std::is_same<LMul, NoMul<float>>::value;
  static_assert(!load_mul || (AX == 2 && KIND == K_C3), "load multiplier: z pass of the inverse cosine kind only");
  static_assert(!ZT || (AX == 2 && (fwd_in ? !load_mul : true) && Tc::ZROW && R1 % 2 == 0 && 2 * TPL * (R1 / 2) == M),
                "z row staging");
  // paired radix-8 stages next to the Makhoul steps: the plain kinds with plain stores (a
  // store functor that loads, StLpsiRhoL, runs slower inside the radix-16 last stage, 68 us
  // against 45; for the kinds with two transforms the paired middle measured no faster)
  constexpr bool PR = xy && PairR8<N>::ok && std::is_same<StoreOp, StPlain<float, float>>::value &&
                      !(KIND == K_FILT || KIND == K_DERIV || KIND == K_DERIVT);
  extern __shared__ __align__(128) unsigned char tma_smem[];
  const float* S = reinterpret_cast<const float*>(tma_smem);
  PC* buf = reinterpret_cast<PC*>(tma_smem + Tc::STAGE_BYTES);
  float4* sfft = reinterpret_cast<float4*>(buf + M * PP);
  float2* spost = reinterpret_cast<float2*>(sfft + M);
  float2* spre = spost + 2 * (M + 1);
  const uint32_t bar = smem_u32(spre + 2 * M);
  const uint32_t sdst = smem_u32(S);
  const int tid = threadIdx.x;
  const int lp = tid & (LP - 1), tj = tid >> Cf::LOG2LP;

  // tb.rev: the tiles in reverse order (for z and y passes, the i planes from the last
  // down), so that a pass can start on the planes the kernel before it touched last
  const bool rev = tb.rev != 0;
  auto tile_of = [ntiles, rev](int t) { return rev ? ntiles - 1 - t : t; };
  pair_tables<N, fwd_in, inv_out>(tb, sfft, spost, spre, tid);
  if (tid == 0) mbar_init(bar, 1);
  if constexpr (ZT) {
    __syncthreads();  // the barrier initialised before warp 0 starts the copies
    if (tid < 32 && (int)blockIdx.x < ntiles)
      tma_issue_zrow<N>(zsrc, tile_of(blockIdx.x), sdst, bar, tb.wait_extra_tx, tid);
  } else {
    if (tid == 0 && (int)blockIdx.x < ntiles)
      tma_issue<N, AX>(g, &tmap, zsrc, tile_of(blockIdx.x), sdst, bar, tb.wait_extra_tx);
  }
  __syncthreads();

  uint32_t parity = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x, parity ^= 1u) {
    const bool ok = mbar_wait_bounded(bar, parity, tb.max_polls);
    if (!__syncthreads_and(ok)) {
      if (tid == 0) {
        if (tb.status) atomicExch(tb.status, 1);
        // At most one copy is in flight (the next is issued only after this wait). The
        // bytes the wait expected beyond the copy's own (wait_extra_tx, the wait test;
        // 0 otherwise) are credited here, so the phase completes exactly when the real
        // copy's bytes have landed, and thread 0 -- which keeps the CTA and its shared
        // memory alive -- leaves only after that. A copy that still has not landed
        // after this second bounded wait is a failed copy: the status flag is already
        // set and the host reports SWC_ERR_CUDA for the pass.
        if (tb.wait_extra_tx > 0) mbar_complete_tx(bar, (uint32_t)tb.wait_extra_tx);
        mbar_wait_bounded(bar, parity, tb.max_polls);
      }
      return;
    }
    const int pair0 = tile_of(t) * LP;
    // ---- staging tile -> PC buffer ----
    if constexpr (ZT && fwd_in) {
      // First Stockham stage of radix R = R1/2 (2 TPL butterflies per line pair, elements
      // m = b + 2 TPL r), two butterflies per thread: b0 = tj and b1 = 2 TPL - 1 - tj. The
      // float4 a of a line holds z_a = (x_4a, x_4a+2) and z_(M-1-a) = (x_4a+3, x_4a+1)
      // (Makhoul order); for a = b + 2 TPL q (q < R/2), z_a is element q of butterfly b
      // and z_(M-1-a) element R-1-q of butterfly 2 TPL - 1 - b, so the 2 R/2 float4 per
      // line at a = b0 + 2 TPL q and a = b1 + 2 TPL q fill both butterflies.
      constexpr int R = R1 / 2, TB = 2 * TPL, ZP4 = Tc::ZPITCH / 4;
      const float4* S4 = reinterpret_cast<const float4*>(S);
      const int b0 = tj, b1 = TB - 1 - tj;
      PC v0[R], v1[R];
      auto quad = [&](int a, int par) -> float4 {  // float4 a of line 2 lp + par
        float4 x = S4[(lp + LP * par) * ZP4 + a];
        if constexpr (KIND == K_S2 || KIND == K_DERIVT) {  // (-1)^p x_p: odd positions 4a+1, 4a+3
          x.y = -x.y;
          x.w = -x.w;
        }
        return x;
      };
#pragma unroll
      for (int q = 0; q < R / 2; ++q) {
        const float4 A0 = quad(b0 + TB * q, 0), B0 = quad(b0 + TB * q, 1);
        const float4 A1 = quad(b1 + TB * q, 0), B1 = quad(b1 + TB * q, 1);
        v0[q] = pmake(make_float2(A0.x, B0.x), make_float2(A0.z, B0.z));
        v1[R - 1 - q] = pmake(make_float2(A0.w, B0.w), make_float2(A0.y, B0.y));
        v1[q] = pmake(make_float2(A1.x, B1.x), make_float2(A1.z, B1.z));
        v0[R - 1 - q] = pmake(make_float2(A1.w, B1.w), make_float2(A1.y, B1.y));
      }
      PDft<R>::run(v0);
      PDft<R>::run(v1);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        buf[(b0 * R + r) * PP + lp] = v0[r];
        buf[(b1 * R + r) * PP + lp] = v1[r];
      }
    } else if constexpr (ZT) {
      // Inverse kinds. The DCT-III pre-processing (pair_pre_one) maps the reals at k,
      // N-k, M-k, M+k to Z_k and Z_(M-k), and the first inverse-FFT stage of radix
      // R = R1/2 runs on (im, re)-swapped Z over butterflies b (elements b + 2 TPL r).
      // With b0 = tj, b1 = 2 TPL - tj (for tj = 0: b1 = TPL), both members of every
      // pair k = b + 2 TPL r (r < R/2) belong to this thread's two butterflies: the
      // partner M-k of a b0 element is element R-1-r of b1 and that of a b1 element is
      // element R-1-r of b0 -- except for tj = 0, whose b0 = 0 holds the pairs
      // (2 TPL r, M - 2 TPL r) and the middle mode M/2 (element R/2), and whose b1 = TPL
      // pairs with itself. The reals come straight from the staged rows (line 2 lp at
      // row lp, line 2 lp + 1 at row lp + LP); DST-III reads the line reversed; the load
      // multiplier scales them as they are read.
      constexpr int R = R1 / 2, TB = 2 * TPL, H = R / 2;
      const bool t0 = tj == 0;
      const int b0 = tj, b1 = t0 ? TPL : TB - tj;
      const int la = 2 * (pair0 + lp);
      const int li = la >> g.ly, lj = la & (g.ny - 1);
      auto X = [&](int pos) -> float2 {  // real element pos of lines A and B
        const int q = (KIND == K_S3) ? (N - 1 - pos) : pos;
        float a = S[lp * Tc::ZPITCH + q], b = S[(lp + LP) * Tc::ZPITCH + q];
        if constexpr (load_mul) {
          a *= lmul(li, lj, q);
          b *= lmul(li, lj + 1, q);
        }
        return make_float2(a, b);
      };
      auto pre = [&](int k, PC& z0, PC& z1) {  // k in [0, M/2): pswapped Z_k, Z_(M-k)
        const float2 xnk = X(k == 0 ? 0 : N - k);
        pair_pre_one(spre, M, k, X(k), k == 0 ? f2(0.f) : xnk, X(M - k), X(M + k), z0, z1);
        z0 = pswap(z0);
        z1 = pswap(z1);
      };
      PC v0[R], v1[R], A1[H], B1[H];
#pragma unroll
      for (int r = 0; r < H; ++r) {
        pre(b0 + TB * r, v0[r], A1[r]);
        pre(b1 + TB * r, v1[r], B1[r]);
      }
      PC mid;
      {
        const int k = M / 2;
        const PC U = pmake(X(k), neg2(X(N - k)));
        mid = pswap(pcomb(spre[2 * k], U, spre[2 * k + 1], U));
      }
      auto sel = [&](bool c, const PC& a, const PC& b) -> PC {
        return pmake(make_float2(c ? a.re.x : b.re.x, c ? a.re.y : b.re.y),
                     make_float2(c ? a.im.x : b.im.x, c ? a.im.y : b.im.y));
      };
#pragma unroll
      for (int r = 0; r < H; ++r) {
        // b0's upper elements R-1-r: partners of b1's pairs, or (tj = 0) of b0's own
        // pairs r+1 and, for r = H-1, the middle mode
        v0[R - 1 - r] = sel(t0, (r == H - 1) ? mid : A1[r + 1 < H ? r + 1 : 0], B1[r]);
        v1[R - 1 - r] = sel(t0, B1[r], A1[r]);
      }
      PDft<R>::run(v0);
      PDft<R>::run(v1);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        buf[(b0 * R + r) * PP + lp] = v0[r];
        buf[(b1 * R + r) * PP + lp] = v1[r];
      }
    } else if constexpr (xy && fwd_in) {
      // rows p of the tile hold the tile's lines side by side: (A, B) = one float2
      const float2* S2 = reinterpret_cast<const float2*>(S);
      PC v[R1];
#pragma unroll
      for (int r = 0; r < R1; ++r) {
        const int m = tj + r * TPL;
        const int p0 = mk_pos<N>(2 * m), p1 = mk_pos<N>(2 * m + 1);
        float2 a = S2[p0 * LP + lp], b = S2[p1 * LP + lp];
        if constexpr (KIND == K_S2 || KIND == K_DERIVT) {
          if (p0 & 1) a = neg2(a);
          if (p1 & 1) b = neg2(b);
        }
        v[r] = pmake(a, b);
      }
      PDft<R1>::run(v);
#pragma unroll
      for (int r = 0; r < R1; ++r) buf[(tj * R1 + r) * PP + lp] = v[r];
    } else if constexpr (xy && PR) {
      // inverse kinds, x/y: the pre-processing of the pairs of this thread's two radix-8
      // butterflies (pr_* in swc_r2r_pair.cuh) from the staged rows, and the first
      // inverse stage, in registers
      const float2* S2 = reinterpret_cast<const float2*>(S);
      auto X = [&](int r) -> float2 { return S2[((KIND == K_S3) ? (N - 1 - r) : r) * LP + lp]; };
      const bool t0 = tj == 0;
      const int b0 = tj, b1 = pr_b1(tj, TPL);
      auto one = [&](int k, PC& Zk, PC& Zm) {
        const float2 xnk = X(k == 0 ? 0 : N - k);
        PC z0, z1;
        pair_pre_one(spre, M, k, X(k), k == 0 ? f2(0.f) : xnk, X(M - k), X(M + k), z0, z1);
        Zk = pswap(z0);
        Zm = pswap(z1);
      };
      PC Zk0[4], Zm0[4], Zk1[4], Zm1[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        one(b0 + 16 * r, Zk0[r], Zm0[r]);
        one(b1 + 16 * r, Zk1[r], Zm1[r]);
      }
      PC mid;
      {
        const int k = M / 2;
        const PC U = pmake(X(k), neg2(X(N - k)));
        mid = pswap(pcomb(spre[2 * k], U, spre[2 * k + 1], U));
      }
      pr_first_inv<M, PP>(buf, t0, lp, b0, b1, Zk0, Zm0, Zk1, Zm1, mid);
    } else if constexpr (xy) {
      const float2* S2 = reinterpret_cast<const float2*>(S);
      constexpr int NP = (M / 2) / TPL;
      auto X = [&](int r) -> float2 { return S2[((KIND == K_S3) ? (N - 1 - r) : r) * LP + lp]; };
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
    } else {
      if constexpr (fwd_in) {
        // z: the tile is its 2 LP lines one after another; four elements per float4
        const float4* S4 = reinterpret_cast<const float4*>(S);
#pragma unroll 4
        for (int c = 0; c < ZU; ++c) {
          const int u = tid + c * NT;
          const int a = u & (NQ - 1), q = u >> Cf::LOG2NQ;
          float4 A = S4[(2 * q) * NQ + a], B = S4[(2 * q + 1) * NQ + a];
          if constexpr (KIND == K_S2 || KIND == K_DERIVT) {
            A.y = -A.y; A.w = -A.w;
            B.y = -B.y; B.w = -B.w;
          }
          buf[a * PP + q] = pmake(make_float2(A.x, B.x), make_float2(A.z, B.z));
          buf[(M - 1 - a) * PP + q] = pmake(make_float2(A.w, B.w), make_float2(A.y, B.y));
        }
      } else {
        // inverse kinds: one slot (two reals) per unit, consecutive lanes on consecutive
        // rows of the odd pitch; DST-III reads the line reversed
        const float2* S2 = reinterpret_cast<const float2*>(S);
        constexpr int SU = (LP * M) / NT;
        constexpr int LOG2M = (M == 32) ? 5 : (M == 64) ? 6 : (M == 128) ? 7 : 8;
        static_assert((1 << LOG2M) == M && SU * NT == LP * M, "z slot units");
#pragma unroll 4
        for (int c = 0; c < SU; ++c) {
          const int u = tid + c * NT;
          const int sl = u & (M - 1), q = u >> LOG2M;
          if constexpr (KIND == K_S3) {
            // slot s = (X_2s, X_2s+1) = (x_{N-1-2s}, x_{N-2-2s}) = swapped float2 M-1-s
            const float2 A = S2[(2 * q) * M + (M - 1 - sl)], B = S2[(2 * q + 1) * M + (M - 1 - sl)];
            buf[sl * PP + q] = pmake(make_float2(A.y, B.y), make_float2(A.x, B.x));
          } else {
            float2 A = S2[(2 * q) * M + sl], B = S2[(2 * q + 1) * M + sl];
            if constexpr (load_mul) {  // lines (i, j) and (i, j + 1), elements k = 2 sl, 2 sl + 1
              const int la = 2 * (pair0 + q);
              const int i = la >> g.ly, j = la & (g.ny - 1);
              A.x *= lmul(i, j, 2 * sl);
              A.y *= lmul(i, j, 2 * sl + 1);
              B.x *= lmul(i, j + 1, 2 * sl);
              B.y *= lmul(i, j + 1, 2 * sl + 1);
            }
            buf[sl * PP + q] = pmake(make_float2(A.x, B.x), make_float2(A.y, B.y));
          }
        }
      }
    }
    __syncthreads();  // the staging tile is free: start the next one
    if constexpr (ZT) {
      if (tid < 32 && t + (int)gridDim.x < ntiles)
        tma_issue_zrow<N>(zsrc, tile_of(t + gridDim.x), sdst, bar, tb.wait_extra_tx, tid);
    } else {
      if (tid == 0 && t + (int)gridDim.x < ntiles)
        tma_issue<N, AX>(g, &tmap, zsrc, tile_of(t + gridDim.x), sdst, bar, tb.wait_extra_tx);
    }
    pair_tail<N, KIND, AX, StoreOp, MulOp, ZT, PR>(g, pair0, lp, tj, tid, buf, sfft, spost, spre, st, mul);
  }
}

// ---- host side ----------------------------------------------------------------------

inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// Tensor map of an nx x ny x nz FP32 array for the x (AX = 0) or y (AX = 1) tiles.
template <int N, int AX> inline cudaError_t make_pass_map(const Grid& g, const float* base, CUtensorMap* map) {
  using Tc = TmaCfg<N>;
  auto enc = tensor_map_encoder();
  if (!enc) return cudaErrorNotSupported;
  const cuuint64_t dims[3] = {(cuuint64_t)g.nz, (cuuint64_t)g.ny, (cuuint64_t)g.nx};
  const cuuint64_t strides[2] = {(cuuint64_t)g.nz * 4, (cuuint64_t)g.ny * g.nz * 4};
  const cuuint32_t box[3] = {(cuuint32_t)Tc::LINES, AX == 1 ? (cuuint32_t)Tc::BOXN : 1u,
                             AX == 0 ? (cuuint32_t)Tc::BOXN : 1u};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int N, int KIND, int AX, class ST, class MUL, class LMUL, bool ZT>
cudaError_t launch_tma_map(const Grid& g, const R2RTables<float>& tb, cudaStream_t stream, const CUtensorMap& map,
                           const float* src, ST st, MUL mul, LMUL lmul) {
  using Tc = TmaCfg<N>;
  auto kern = r2r_tma_kernel<N, KIND, AX, ST, MUL, LMUL, ZT>;
  const size_t smem = Tc::smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, occ = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, PairCfg<N>::NT, smem)) != cudaSuccess) return e;
  const int ntiles = (int)((g.ng / N) / Tc::LINES);
  const int blocks = std::min(ntiles, std::max(occ, 1) * sms);
  kern<<<blocks, PairCfg<N>::NT, smem, stream>>>(map, src, g, tb, st, mul, lmul, ntiles);
  return cudaGetLastError();
}

// z passes take the row staging where the tile allows it (N = 256).
template <int N, int KIND> constexpr bool zt_kind() {
  return TmaCfg<N>::ZROW && (KIND == K_C2 || KIND == K_S2 || KIND == K_FILT || KIND == K_DERIV ||
                             KIND == K_DERIVT || KIND == K_C3 || KIND == K_S3);
}

template <int N, int KIND, int AX, class ST, class MUL, class LMUL = NoMul<float>>
cudaError_t launch_tma(const Grid& g, const R2RTables<float>& tb, cudaStream_t stream, const float* src, ST st,
                       MUL mul, LMUL lmul = LMUL()) {
  CUtensorMap map;
  std::memset(&map, 0, sizeof(map));
  if constexpr (AX == 2 && zt_kind<N, KIND>()) {
    return launch_tma_map<N, KIND, AX, ST, MUL, LMUL, true>(g, tb, stream, map, src, st, mul, lmul);
  } else {  // (an else branch, so that the row-staged kinds instantiate no second z kernel)
    if constexpr (AX != 2) {
      const cudaError_t e = make_pass_map<N, AX>(g, src, &map);
      if (e != cudaSuccess) return e;
    }
    return launch_tma_map<N, KIND, AX, ST, MUL, LMUL, false>(g, tb, stream, map, src, st, mul, lmul);
  }
}

}  // namespace swc
