// swc_adjoint_kernels.cuh -- kernels of the discrete adjoint of one time step
// (FP64 engine: T = double; mixed engine: the FP32 adjoint, T = float). Each kernel is
// the transpose of one forward stage of swc_step_impl.cuh;
// the comment of each names the forward expression (REF:line) it transposes.
//
// Transposes of the r2r kinds (per axis, FFTW definitions):
//   DCT-II^T  = DCT-III diag(2,1,...,1)      DCT-III^T = diag(1/2,1,...,1) DCT-II
//   DST-II^T  = DST-III diag(1,...,1,2)      DST-III^T = diag(1,...,1,1/2) DST-II
// so every transposed 3D transform is the other kind with a weight on mode 0 (or
// the last mode of a sine axis), folded into the load or store functor.
#pragma once

#include "swc_step_impl.cuh"

namespace swc {

// Weight of the transposes: for a cosine axis index 0, for a sine axis index n-1.
// sine[a] = 1 if axis a is a sine (DST) axis; w = 2 (load side) or 1/2 (store side).
template <typename T> struct AxisWeights {
  int sine[3];
  T w;
  __device__ __forceinline__ T at(const Grid& g, int i, int j, int k) const {
    T f = T(1.0);
    f *= (sine[0] ? (i == g.nx - 1) : (i == 0)) ? w : T(1.0);
    f *= (sine[1] ? (j == g.ny - 1) : (j == 0)) ? w : T(1.0);
    f *= (sine[2] ? (k == g.nz - 1) : (k == 0)) ? w : T(1.0);
    return f;
  }
};

// load x * weight (input side of DCT-II^T / DST-II^T), optionally times a second
// pointwise factor table (the Gaussian G of REF:1486)
template <typename T> struct LdW {
  Grid g;
  const T* p;
  AxisWeights<T> aw;
  __device__ __forceinline__ T operator()(int i, int j, int k, long long idx) const {
    return p[idx] * aw.at(g, i, j, k);
  }
  // vector forms for the FP32 two-line pass (z: k .. k+3; x/y: k, k+1)
  __device__ __forceinline__ float4 quad(int i, int j, int k, long long idx) const {
    const float4 v = ld4v(p, idx);
    return make_float4(v.x * (float)aw.at(g, i, j, k), v.y * (float)aw.at(g, i, j, k + 1),
                       v.z * (float)aw.at(g, i, j, k + 2), v.w * (float)aw.at(g, i, j, k + 3));
  }
  __device__ __forceinline__ float2 pair(int i, int j, int k, long long idx) const {
    const float2 v = ld2v(p, idx);
    return make_float2(v.x * (float)aw.at(g, i, j, k), v.y * (float)aw.at(g, i, j, k + 1));
  }
};

// store v * weight (output side of DCT-III^T / DST-III^T); acc: += instead of =
template <typename T> struct StW {
  Grid g;
  T* p;
  AxisWeights<T> aw;
  int acc;
  __device__ __forceinline__ void operator()(int i, int j, int k, long long idx, T v) const {
    const T y = v * aw.at(g, i, j, k);
    p[idx] = acc ? p[idx] + y : y;
  }
  __device__ __forceinline__ void pair(int i, int j, int k, long long idx, float2 v) const {
    float2 y = make_float2(v.x * (float)aw.at(g, i, j, k), v.y * (float)aw.at(g, i, j, k + 1));
    if (acc) {
      const float2 o = ld2v(p, idx);
      y.x += o.x;
      y.y += o.y;
    }
    st2v(p, idx, y);
  }
};

// Last pass of Delta_s(bar lapR) (normal phase, transpose of REF:1319-1342):
// rho_bar += L * y, L_bar += rho * y (Delta_s is symmetric).
template <typename T> struct StAdjLap {
  const T *L, *rho;
  T *brho, *bL;
  __device__ __forceinline__ void operator()(int, int, int, long long idx, T y) const {
    brho[idx] += L[idx] * y;
    bL[idx] += rho[idx] * y;
  }
  __device__ __forceinline__ void quad(int, int, int, long long idx, float4 y) const {
    const float4 l = ld4v(L, idx), r = ld4v(rho, idx), a = ld4v(brho, idx), b = ld4v(bL, idx);
    st4v(brho, idx, make_float4(a.x + l.x * y.x, a.y + l.y * y.y, a.z + l.z * y.z, a.w + l.w * y.w));
    st4v(bL, idx, make_float4(b.x + r.x * y.x, b.y + r.y * y.y, b.z + r.z * y.z, b.w + r.w * y.w));
  }
};

// parameter-gradient slots
enum { PG_ALPHA = 0, PG_BETA = 1, PG_GAMMA = 2, PG_NU = 3, PG_RHO0 = 4, PG_KP = 5, PG_COUNT = 8 };

// The pointwise adjoint kernels take four consecutive points of one z line per thread
// (every extent is a power of two >= 4) and move them with vector accesses (V4).
struct Pt4 {
  long long idx;  // the first of the four points
  int i, j, k;    // its coordinates; the others are (i, j, k + 1 .. k + 3)
};
__device__ __forceinline__ bool pt4(const Grid& g, Pt4& p) {
  p.idx = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  if (p.idx >= g.ng) return false;
  decompose(g, p.idx, p.i, p.j, p.k);
  return true;
}
static inline unsigned pt4_blocks(const Grid& g) { return (unsigned)((g.ng / 4 + 255) / 256); }

// Parameter-gradient cells: ceil(n^3 / 256) per slot after the PG_COUNT totals (the
// cells of blocks a kernel does not launch stay zero).
__device__ __forceinline__ size_t pg_cells(const Grid& g) { return (size_t)((g.ng + 255) / 256); }

// Block sums of v[0 .. NS) (in their own precision: the FP32 adjoint sums a block in
// FP32) added in FP64 to this block's own cell of the parameter slots slot[0 .. NS).
// Every thread of the block calls it, once per kernel. pg_reduce_kernel sums the cells
// in a fixed order, so the parameter gradients do not depend on the order in which
// blocks finish (no atomics).
template <typename V, int NS>
__device__ __forceinline__ void block_accum(const V (&v)[NS], const int (&slot)[NS], const Grid& g,
                                            double* pgrad) {
  __shared__ V shv[NS][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    V t = v[s];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) shv[s][w] = t;
  }
  __syncthreads();
  if ((int)threadIdx.x < NS) {
    const int s = threadIdx.x;
    V t = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += shv[s][q];
    pgrad[PG_COUNT + (size_t)slot[s] * pg_cells(g) + blockIdx.x] += (double)t;
  }
}

// pgrad[s] = sum over the nblk cells of slot s, in a fixed order (one block per slot,
// 256 threads).
static __global__ void __launch_bounds__(256) pg_reduce_kernel(double* pgrad, unsigned nblk) {
  __shared__ double sh[256];
  const int s = blockIdx.x;
  const double* cells = pgrad + PG_COUNT + (size_t)s * nblk;
  double t = 0;
  for (unsigned b = threadIdx.x; b < nblk; b += 256) t += cells[b];
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) pgrad[s] = sh[0];
}

template <typename T> struct AdjScalars {
  T ep, alpha, beta, gamma, zeta, kp, rho0, q02, dt, dtd2, rho_m, scale, nu, lam2nu;
};

// Transpose of the CN/AB2 update (REF:2185-2187) and of Nl_old <- Nl, psiq_old <- psiq.
//   Q' = (C1 Q - Qo/2 + h (3 Nl - Nlo)) / C2, Qo' = Q, Nlo' = Nl  (h = dt/2 scale)
template <typename T>
__global__ void __launch_bounds__(256) adj_cn_kernel(Grid g, const T* qx, const T* qy, const T* qz,
                                                     AdjScalars<T> s, int first, const T* Qold, const T* Qnew,
                                                     T* bQ, T* bQo, T* bNlo, T* bNlq, double* pgrad) {
  Pt4 p;
  T da[1] = {T(0.0)};
  if (pt4(g, p)) {
    const long long x = p.idx;
    V4<T> bq, nlo, qo, q0, q1, nl;
    bq.load(bQ, x);
    nlo.load(bNlo, x);
    qo.load(bQo, x);
    q0.load(Qold, x);
    q1.load(Qnew, x);
    const T qxy = qx[p.i] * qx[p.i] + qy[p.j] * qy[p.j];
    const T h = s.dtd2 * s.scale;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const T kz = qz[p.k + e];
      const T sq = s.q02 - (qxy + kz * kz);
      const T aLin = s.ep - s.alpha * (sq * sq);
      const T C1 = T(2.0) - s.dt * s.rho_m * aLin, C2 = T(1.5) - s.dt * s.rho_m * aLin;
      const T b = bq.v[e];
      {  // one reciprocal of C2 (FP64: rcp_f64's Newton-Raphson one)
        // REF:2170-2172: Nl_old = Nl at nLoop == 1; dC1/dalpha = dC2/dalpha = dt rho_m
        // sq^2  =>  dQ'/dalpha = dt rho_m sq^2 (Q - Q') / C2
        const T r = div_nr(T(1.0), C2), hb = h * r * b;
        T bnl = T(3.0) * hb + nlo.v[e];
        if (first) bnl -= hb;
        nl.v[e] = bnl;
        nlo.v[e] = first ? T(0.0) : -hb;
        bq.v[e] = C1 * r * b + qo.v[e];
        qo.v[e] = -T(0.5) * r * b;
        da[0] += b * s.dt * s.rho_m * sq * sq * (q0.v[e] - q1.v[e]) * r;
      }
    }
    nl.store(bNlq, x);
    nlo.store(bNlo, x);
    bq.store(bQ, x);
    qo.store(bQo, x);
  }
  const int slots[1] = {PG_ALPHA};
  block_accum(da, slots, g, pgrad);
}

// Transpose of dq = q . f-hat shifted (REF:2076-2078, subtracted from Nl-hat): f-hat_a
// at c receives -Vq_a[c+1] bar(Nlq) at c+1. Each output is stored times the input
// weights (wx, wy, wz) of the transposed transform it feeds.
template <typename T>
__global__ void __launch_bounds__(256) adj_dq_kernel(Grid g, const T* qx, const T* qy, const T* qz,
                                                     const T* bNlq, T* bfx, T* bfy, T* bfz, AxisWeights<T> wx,
                                                     AxisWeights<T> wy, AxisWeights<T> wz) {
  Pt4 p;
  if (!pt4(g, p)) return;
  const int i = p.i, j = p.j, k = p.k;
  const long long x = p.idx, sx = 1LL << (g.ly + g.lz), sy = g.nz;
  V4<T> f = V4<T>::zero();
  if (i + 1 < g.nx) {
    V4<T> n;
    n.load(bNlq, x + sx);
    const T q = -qx[i + 1];
#pragma unroll
    for (int e = 0; e < 4; ++e) f.v[e] = q * n.v[e] * wx.at(g, i, j, k + e);
  }
  f.store(bfx, x);
  f = V4<T>::zero();
  if (j + 1 < g.ny) {
    V4<T> n;
    n.load(bNlq, x + sy);
    const T q = -qy[j + 1];
#pragma unroll
    for (int e = 0; e < 4; ++e) f.v[e] = q * n.v[e] * wy.at(g, i, j, k + e);
  }
  f.store(bfy, x);
  {
    V4<T> n;
    n.load(bNlq, x);
    const T sh[4] = {n.v[1], n.v[2], n.v[3], (k + 4 < g.nz) ? bNlq[x + 4] : T(0.0)};
#pragma unroll
    for (int e = 0; e < 4; ++e)
      f.v[e] = (k + e + 1 < g.nz) ? -qz[k + e + 1] * sh[e] * wz.at(g, i, j, k + e) : T(0.0);
  }
  f.store(bfz, x);
}

// Transpose of the density update (REF:2121-2139) and of the real-space Nl
// (REF:2153-2160, grad.f handled by adj_dq_kernel):
//   S_rho = -v.grad rho - rho_in divv;  rho' = rho_in + dt (1.5 S_rho - 0.5 F);  F' = S_rho
//   Nl = -mu + c' (rho' - rho0 - kp A) psi - v.grad psi,  c' = kp zeta/(A + 0.001)
// rho_in: the density the forward step used (the relax reset rho0 + kp A, REF:1371,
// when relax is set). Outputs initialise the real-space cotangent buffers.
template <typename T> struct AdjNlArgs {
  const T *bNl, *psi, *A, *rho_in, *rho_new, *vx, *vy, *vz, *gpx, *gpy, *gpz, *grx, *gry, *grz, *divv;
  T *bR, *bF, *bmu, *bA, *bpsi, *bvx, *bvy, *bvz, *bgpx, *bgpy, *bgpz, *bgrx, *bgry, *bgrz, *bdivv;
  double* pgrad;
  AdjScalars<T> s;
  int relax;
};
template <typename T>
__global__ void __launch_bounds__(256) adj_nl_kernel(Grid g, AdjNlArgs<T> a) {
  Pt4 p;
  T acc[2] = {T(0.0), T(0.0)};  // kp, rho0
  if (pt4(g, p)) {
    const long long x = p.idx;
    const AdjScalars<T>& s = a.s;
    V4<T> b, brp, rin, o;
    {
      V4<T> psi, A, rn, bR, oA, op;
      b.load(a.bNl, x);
      psi.load(a.psi, x);
      A.load(a.A, x);
      rn.load(a.rho_new, x);
      bR.load(a.bR, x);
      if (a.relax) {
#pragma unroll
        for (int e = 0; e < 4; ++e) rin.v[e] = s.rho0 + s.kp * A.v[e];
      } else {
        rin.load(a.rho_in, x);
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const T den = A.v[e] + T(0.001);
        const T t2 = rn.v[e] - s.rho0 - s.kp * A.v[e];
        T cp, t2dd, t2d;  // kp zeta / den, t2 / den^2, t2 / den
        if constexpr (sizeof(T) == 8) {  // one Newton-Raphson reciprocal (rcp_f64)
          const T rd = rcp_f64(den);
          cp = s.kp * s.zeta * rd;
          t2d = t2 * rd;
          t2dd = t2d * rd;
        } else {
          cp = s.kp * s.zeta / den;
          t2dd = t2 / (den * den);
          t2d = t2 / den;
        }
        const T pb = psi.v[e] * b.v[e];
        brp.v[e] = bR.v[e] + cp * psi.v[e] * b.v[e];  // bar rho'
        o.v[e] = -b.v[e];
        oA.v[e] = pb * (-s.kp * s.zeta * t2dd - cp * s.kp);
        op.v[e] = cp * t2 * b.v[e];
        acc[0] += pb * (s.zeta * t2d - cp * A.v[e]);
        acc[1] += -b.v[e] * psi.v[e] * cp;
      }
      o.store(a.bmu, x);
      oA.store(a.bA, x);
      op.store(a.bpsi, x);
    }
    V4<T> bS;  // bar S_rho
    {
      V4<T> bF, dv;
      bF.load(a.bF, x);
      dv.load(a.divv, x);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        bS.v[e] = bF.v[e] + T(1.5) * s.dt * brp.v[e];
        o.v[e] = -rin.v[e] * bS.v[e];
        bF.v[e] = -T(0.5) * s.dt * brp.v[e];
        brp.v[e] = brp.v[e] - dv.v[e] * bS.v[e];  // bar rho_in (relax: folded into A later)
      }
      o.store(a.bdivv, x);
      bF.store(a.bF, x);
      brp.store(a.bR, x);
    }
    auto component = [&](const T* v_, const T* gp_, const T* gr_, T* bgp, T* bv, T* bgr) {
      V4<T> v, gp, gr, ov, og;
      v.load(v_, x);
      gp.load(gp_, x);
      gr.load(gr_, x);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        o.v[e] = -v.v[e] * b.v[e];
        ov.v[e] = -gp.v[e] * b.v[e] - gr.v[e] * bS.v[e];
        og.v[e] = -v.v[e] * bS.v[e];
      }
      o.store(bgp, x);
      ov.store(bv, x);
      og.store(bgr, x);
    };
    component(a.vx, a.gpx, a.grx, a.bgpx, a.bvx, a.bgrx);
    component(a.vy, a.gpy, a.gry, a.bgpy, a.bvy, a.bgry);
    component(a.vz, a.gpz, a.grz, a.bgpz, a.bvz, a.bgrz);
  }
  const int slots[2] = {PG_KP, PG_RHO0};
  block_accum(acc, slots, g, a.pgrad);
}

// Transpose of the Stokes solve, part 1 (REF:1581-1974 and the divergence REF:2076):
// at each output mode o and component a (where the forward computed it) form
//   bar dot_a(o)  = -(CM1/nu) CM2 bar vsol + (CM1/(lam+2nu)) CM2 G bar virr
//   bSdir_a(o)    =  (CM1/nu) bar vsol            (the S_a(o) term)
//   bfgp_a(o)     =  (CM1/(lam+2nu)) Vs bar virr   (the f-grad'(o + e_a) term)
// with bar vsol = bar v-hat_a, bar virr = bar v-hat_a + Vq_a[o_a+1] bar divv-hat(o + e_a);
// zero elsewhere. nu_bar += bar vsol (-vsol/nu) + bar virr (-2 virr/(lam + 2nu)).
// bar v-hat_a and bar divv-hat arrive without the output weights of the transposed
// transforms that made them (wv[a], wdq), which are applied here. Inputs and outputs are
// distinct arrays: the inputs take the read-only load path; FP32 forms 1/|q|^2 with the
// approximate reciprocal (rcp_pos), FP64 with the division.
template <typename T> struct AdjStokesArgs {
  const T *bvx, *bvy, *bvz, *bdq, *vsx_, *vsy_, *vsz_, *vix, *viy, *viz;
  T *bdotx, *bdoty, *bdotz, *bsx, *bsy, *bsz, *bgx, *bgy, *bgz;
  const T *vqx, *vqy, *vqz, *vsx, *vsy, *vsz, *gqx, *gqy, *gqz, *gsx, *gsy, *gsz;
  T scale, inv_nu, inv_lam2nu, nu, lam2nu;
  int block;
  AxisWeights<T> wvx, wvy, wvz, wdq;
  double* pgrad;
};
template <typename T>
__global__ void __launch_bounds__(256) adj_stokes1_kernel(Grid g, AdjStokesArgs<T> a) {
  Pt4 p;
  T dnu[1] = {T(0.0)};
  if (pt4(g, p)) {
    const int i = p.i, j = p.j, k = p.k;
    const long long x = p.idx, sx = 1LL << (g.ly + g.lz), sy = g.nz;
    const T qxi = a.vqx[i], qyj = a.vqy[j];
    V4<T> d = V4<T>::zero(), sd = V4<T>::zero(), fp = V4<T>::zero();
    if (i < g.nx - 1) {
      V4<T> bv, dq, vs, vi;
      bv.loadg(a.bvx, x);
      dq.loadg(a.bdq, x + sx);
      vs.loadg(a.vsx_, x);
      vi.loadg(a.vix, x);
      const T s_ = a.vsx[i], q1 = a.vqx[i + 1], gxy = a.gsx[i] * a.gqy[j];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const T qzk = a.vqz[k + e];
        const T inv = rcp_pos(s_ * s_ + qyj * qyj + qzk * qzk);
        const T CM1 = a.scale * inv, CM2 = s_ * inv, G = gxy * a.gqz[k + e];
        const T bvs = bv.v[e] * a.wvx.at(g, i, j, k + e);
        const T bvi = bvs + q1 * (dq.v[e] * a.wdq.at(g, i + 1, j, k + e));
        d.v[e] = -(CM1 * a.inv_nu) * CM2 * bvs + (CM1 * a.inv_lam2nu) * CM2 * G * bvi;
        sd.v[e] = (CM1 * a.inv_nu) * bvs;
        fp.v[e] = (CM1 * a.inv_lam2nu) * s_ * bvi;
        dnu[0] += bvs * (-vs.v[e] * a.inv_nu) + bvi * (-T(2.0) * vi.v[e] * a.inv_lam2nu);
      }
    }
    d.store(a.bdotx, x);
    sd.store(a.bsx, x);
    fp.store(a.bgx, x);
    V4<T> dy = V4<T>::zero(), sdy = V4<T>::zero(), fpy = V4<T>::zero();
    V4<T> dz = V4<T>::zero(), sdz = V4<T>::zero(), fpz = V4<T>::zero();
    if (j < g.ny - 1) {
      V4<T> bvy, dqy, vsy, viy, bvz, dqz, vsz, viz;
      bvy.loadg(a.bvy, x);
      dqy.loadg(a.bdq, x + sy);
      vsy.loadg(a.vsy_, x);
      viy.loadg(a.viy, x);
      bvz.loadg(a.bvz, x);
      dqz.loadg(a.bdq, x);
      vsz.loadg(a.vsz_, x);
      viz.loadg(a.viz, x);
      const T dq4 = (k + 4 < g.nz) ? a.bdq[x + 4] : T(0.0);
      const T dzs[4] = {dqz.v[1], dqz.v[2], dqz.v[3], dq4};  // bar divv-hat at k + e + 1
      const T sy_ = a.vsy[j], qy1 = a.vqy[j + 1];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (k + e >= g.nz - 1) continue;
        const T qzk = a.vqz[k + e];
        {
          const T inv = rcp_pos(qxi * qxi + sy_ * sy_ + qzk * qzk);
          const T CM1 = a.scale * inv, CM2 = sy_ * inv, G = a.gqx[i] * a.gsy[j] * a.gqz[k + e];
          const T bvs = bvy.v[e] * a.wvy.at(g, i, j, k + e);
          const T bvi = bvs + qy1 * (dqy.v[e] * a.wdq.at(g, i, j + 1, k + e));
          dy.v[e] = -(CM1 * a.inv_nu) * CM2 * bvs + (CM1 * a.inv_lam2nu) * CM2 * G * bvi;
          sdy.v[e] = (CM1 * a.inv_nu) * bvs;
          fpy.v[e] = (CM1 * a.inv_lam2nu) * sy_ * bvi;
          dnu[0] += bvs * (-vsy.v[e] * a.inv_nu) + bvi * (-T(2.0) * viy.v[e] * a.inv_lam2nu);
        }
        {
          const T s_ = a.vsz[k + e];
          const T inv = rcp_pos(qxi * qxi + qyj * qyj + s_ * s_);
          const T CM1 = a.scale * inv, CM2 = s_ * inv;
          const bool q1 = (k + e == 0) && (j > 0) && (i % a.block != 0);  // REF:1932
          const T G = q1 ? (a.gqx[i] * a.gsy[j] * a.gqz[k + e]) : (a.gqx[i] * a.gqy[j] * a.gsz[k + e]);
          const T bvs = bvz.v[e] * a.wvz.at(g, i, j, k + e);
          const T bvi = bvs + a.vqz[k + e + 1] * (dzs[e] * a.wdq.at(g, i, j, k + e + 1));
          dz.v[e] = -(CM1 * a.inv_nu) * CM2 * bvs + (CM1 * a.inv_lam2nu) * CM2 * G * bvi;
          sdz.v[e] = (CM1 * a.inv_nu) * bvs;
          fpz.v[e] = (CM1 * a.inv_lam2nu) * s_ * bvi;
          dnu[0] += bvs * (-vsz.v[e] * a.inv_nu) + bvi * (-T(2.0) * viz.v[e] * a.inv_lam2nu);
        }
      }
    }
    dy.store(a.bdoty, x);
    sdy.store(a.bsy, x);
    fpy.store(a.bgy, x);
    dz.store(a.bdotz, x);
    sdz.store(a.bsz, x);
    fpz.store(a.bgz, x);
  }
  const int slots[1] = {PG_NU};
  block_accum(dnu, slots, g, a.pgrad);
}

// Transpose of the Stokes solve, part 2: gather at each input mode p the terms of
// every output mode that read it (REF:1596-1624, 1775-1841 read patterns):
//   S_x(p): dot_x(p) w Vs_x[p_x]; dot_y(p_x+1, p_y-1, p_z) w Vq_x[p_x+1]; dot_z(p_x+1, p_y, p_z-1) w Vq_x[p_x+1]
//   S_y(p): dot_y(p) w Vs_y[p_y]; dot_x(p_x-1, p_y+1, p_z) w Vq_y[p_y+1]; dot_z(p_x, p_y+1, p_z-1) w Vq_y[p_y+1]
//   S_z(p): dot_z(p) w Vs_z[p_z]; dot_x(p_x-1, p_y, p_z+1) w Vq_z[p_z+1]; dot_y(p_x, p_y-1, p_z+1) w Vq_z[p_z+1]
//   fgrad'(p) = sum_a bfgp_a(p - e_a)
// bar dot and bfgp are zero outside each component's computed modes, so only the
// array bounds are tested. Then f-grad-hat_bar = fgrad'_bar, E-hat_bar = G fgrad'_bar
// (REF:1486). Each output is stored times the input weights of the transposed
// transform it feeds (ws[a] for S_a, w2 for f-grad-hat and E-hat).
template <typename T> struct AdjStokes2Args {
  const T *bdotx, *bdoty, *bdotz, *bsx, *bsy, *bsz, *bgx, *bgy, *bgz;
  T *bSx, *bSy, *bSz, *bfg, *bE;
  const T *vqx, *vqy, *vqz, *vsx, *vsy, *vsz, *gqx, *gqy, *gqz;
  AxisWeights<T> wsx, wsy, wsz, w2;
};
template <typename T>
__global__ void __launch_bounds__(256) adj_stokes2_kernel(Grid g, AdjStokes2Args<T> a) {
  Pt4 p;
  if (!pt4(g, p)) return;
  const int i = p.i, j = p.j, k = p.k;
  const long long x = p.idx, sx = 1LL << (g.ly + g.lz), sy = g.nz;
  // values at (., ., k - 1 .. k + 2) of a line starting at x: {v[x-1], q0, q1, q2}
  auto back1 = [&](const T* f, long long at, T (&o)[4]) {
    V4<T> q;
    q.load(f, at);
    o[0] = (k >= 1) ? f[at - 1] : T(0.0);
    o[1] = q.v[0];
    o[2] = q.v[1];
    o[3] = q.v[2];
  };
  // values at (., ., k + 1 .. k + 4) of a line starting at x: {q1, q2, q3, v[x+4]}
  auto fwd1 = [&](const T* f, long long at, T (&o)[4]) {
    V4<T> q;
    q.load(f, at);
    o[0] = q.v[1];
    o[1] = q.v[2];
    o[2] = q.v[3];
    o[3] = (k + 4 < g.nz) ? f[at + 4] : T(0.0);
  };
  V4<T> S, t;
  T sh[4];
  // S_x
  S.load(a.bsx, x);
  t.load(a.bdotx, x);
#pragma unroll
  for (int e = 0; e < 4; ++e) S.v[e] = S.v[e] + a.vsx[i] * t.v[e];
  if (i + 1 < g.nx) {
    const T q = a.vqx[i + 1];
    if (j >= 1) {
      t.load(a.bdoty, x + sx - sy);
#pragma unroll
      for (int e = 0; e < 4; ++e) S.v[e] += q * t.v[e];
    }
    back1(a.bdotz, x + sx, sh);
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (k + e >= 1) S.v[e] += q * sh[e];
  }
#pragma unroll
  for (int e = 0; e < 4; ++e) S.v[e] = S.v[e] * a.wsx.at(g, i, j, k + e);
  S.store(a.bSx, x);
  // S_y
  S.load(a.bsy, x);
  t.load(a.bdoty, x);
#pragma unroll
  for (int e = 0; e < 4; ++e) S.v[e] = S.v[e] + a.vsy[j] * t.v[e];
  if (j + 1 < g.ny) {
    const T q = a.vqy[j + 1];
    if (i >= 1) {
      t.load(a.bdotx, x - sx + sy);
#pragma unroll
      for (int e = 0; e < 4; ++e) S.v[e] += q * t.v[e];
    }
    back1(a.bdotz, x + sy, sh);
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (k + e >= 1) S.v[e] += q * sh[e];
  }
#pragma unroll
  for (int e = 0; e < 4; ++e) S.v[e] = S.v[e] * a.wsy.at(g, i, j, k + e);
  S.store(a.bSy, x);
  // S_z
  S.load(a.bsz, x);
  t.load(a.bdotz, x);
#pragma unroll
  for (int e = 0; e < 4; ++e) S.v[e] = S.v[e] + a.vsz[k + e] * t.v[e];
  {
    T sx4[4] = {T(0.0), T(0.0), T(0.0), T(0.0)}, sy4[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};
    if (i >= 1) fwd1(a.bdotx, x - sx, sx4);
    if (j >= 1) fwd1(a.bdoty, x - sy, sy4);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (k + e + 1 >= g.nz) continue;
      if (i >= 1) S.v[e] += a.vqz[k + e + 1] * sx4[e];
      if (j >= 1) S.v[e] += a.vqz[k + e + 1] * sy4[e];
    }
  }
#pragma unroll
  for (int e = 0; e < 4; ++e) S.v[e] = S.v[e] * a.wsz.at(g, i, j, k + e);
  S.store(a.bSz, x);
  // f-grad' and E
  V4<T> fg = V4<T>::zero();
  if (i >= 1) {
    t.load(a.bgx, x - sx);
#pragma unroll
    for (int e = 0; e < 4; ++e) fg.v[e] += t.v[e];
  }
  if (j >= 1) {
    t.load(a.bgy, x - sy);
#pragma unroll
    for (int e = 0; e < 4; ++e) fg.v[e] += t.v[e];
  }
  back1(a.bgz, x, sh);
#pragma unroll
  for (int e = 0; e < 4; ++e)
    if (k + e >= 1) fg.v[e] += sh[e];
  const T gxy = a.gqx[i] * a.gqy[j];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const T w = a.w2.at(g, i, j, k + e);
    t.v[e] = fg.v[e] * (gxy * a.gqz[k + e]) * w;
    fg.v[e] = fg.v[e] * w;
  }
  fg.store(a.bfg, x);
  t.store(a.bE, x);
}

// Transpose of S6 (REF:1385-1425) and of the relax reset (REF:1371-1374):
//   E = L^2/2, t = rho0 + kp A, fgrad = zeta/2 (rho^2 - t^2), mu1 = lapR + rho L,
//   S_a = mu1 gpsi_a + E grho_a, mu = lapR + rho P5, P5 = L - ep psi - beta psi^3 + gamma psi^5,
//   Erho = rho E, c = kp zeta (rho - t)/(A + 0.001), f_a = c gpsi_a;
//   relax: rho = rho0 + kp A and lapR = rho lapR_raw.
// bR enters holding bar rho_in from adj_nl_kernel and leaves holding the cotangent
// of the step's incoming density (zero in the relax phase, whose rho is reset).
template <typename T> struct AdjS6Args {
  const T *bfgrad, *bE, *bSx, *bSy, *bSz, *bfx, *bfy, *bfz, *bmu;
  const T *lapR, *rho_in, *L, *psi, *A, *gpx, *gpy, *gpz, *grx, *gry, *grz;
  T *bgpx, *bgpy, *bgpz, *bgrx, *bgry, *bgrz, *bA, *bpsi, *bR, *blapR, *bL;
  double* pgrad;
  AdjScalars<T> s;
  int relax;
  // Energy term of the loss, last step only (ew = lambda dx^3, 0 otherwise): the free
  // energy of REF:2214-2258 reads this step's L (stale, Q5) and A with the step's new
  // density rho_new, so L_bar += ew rho_new L and A_bar += -ew zeta kp (rho_new - rho_0 - kp A).
  const T* rho_new;
  T ew;
};
template <typename T>
__global__ void __launch_bounds__(256) adj_s6_kernel(Grid g, AdjS6Args<T> a) {
  Pt4 p;
  T acc[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};  // beta, gamma, rho0, kp
  if (pt4(g, p)) {
    const long long x = p.idx;
    const AdjScalars<T>& s = a.s;
    V4<T> A, L, rho, lraw, rden;  // rden = 1/(A + 0.001), A >= 0; inputs on the read-only path
    A.loadg(a.A, x);
#pragma unroll
    for (int e = 0; e < 4; ++e) rden.v[e] = rcp_pos(A.v[e] + T(0.001));
    L.loadg(a.L, x);
    lraw.loadg(a.lapR, x);
    if (a.relax) {
#pragma unroll
      for (int e = 0; e < 4; ++e) rho.v[e] = s.rho0 + s.kp * A.v[e];
    } else {
      rho.loadg(a.rho_in, x);
    }
    // bmu1 = bS . gpsi, bc = bf . gpsi, bEn = bS . grho + rho bEr, EbE = E bEr
    V4<T> bSx, bSy, bSz, bmu1, bc, bEn, EbE;
    bSx.loadg(a.bSx, x);
    bSy.loadg(a.bSy, x);
    bSz.loadg(a.bSz, x);
    {
      V4<T> bfx, bfy, bfz, gx, gy, gz, mu1, c;
      bfx.loadg(a.bfx, x);
      bfy.loadg(a.bfy, x);
      bfz.loadg(a.bfz, x);
      gx.loadg(a.gpx, x);
      gy.loadg(a.gpy, x);
      gz.loadg(a.gpz, x);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const T t = s.rho0 + s.kp * A.v[e];
        const T lapR = a.relax ? rho.v[e] * lraw.v[e] : lraw.v[e];
        mu1.v[e] = lapR + rho.v[e] * L.v[e];
        c.v[e] = s.kp * s.zeta * (rho.v[e] - t) * rden.v[e];
        bmu1.v[e] = bSx.v[e] * gx.v[e] + bSy.v[e] * gy.v[e] + bSz.v[e] * gz.v[e];
        bc.v[e] = bfx.v[e] * gx.v[e] + bfy.v[e] * gy.v[e] + bfz.v[e] * gz.v[e];
      }
      auto upd = [&](T* bg, const V4<T>& bS, const V4<T>& bf) {
        V4<T> o;
        o.load(bg, x);
#pragma unroll
        for (int e = 0; e < 4; ++e) o.v[e] += mu1.v[e] * bS.v[e] + c.v[e] * bf.v[e];
        o.store(bg, x);
      };
      upd(a.bgpx, bSx, bfx);
      upd(a.bgpy, bSy, bfy);
      upd(a.bgpz, bSz, bfz);
    }
    {
      V4<T> bEr, gx, gy, gz, E;
      bEr.loadg(a.bE, x);
      gx.loadg(a.grx, x);
      gy.loadg(a.gry, x);
      gz.loadg(a.grz, x);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        E.v[e] = T(0.5) * (L.v[e] * L.v[e]);
        bEn.v[e] = bSx.v[e] * gx.v[e] + bSy.v[e] * gy.v[e] + bSz.v[e] * gz.v[e] + rho.v[e] * bEr.v[e];
        EbE.v[e] = E.v[e] * bEr.v[e];
      }
      auto upd = [&](T* bg, const V4<T>& bS) {
        V4<T> o;
        o.load(bg, x);
#pragma unroll
        for (int e = 0; e < 4; ++e) o.v[e] += E.v[e] * bS.v[e];
        o.store(bg, x);
      };
      upd(a.bgrx, bSx);
      upd(a.bgry, bSy);
      upd(a.bgrz, bSz);
    }
    {
      V4<T> psi, bmu, bfg, oA, op, oR, ol, oL;
      psi.loadg(a.psi, x);
      bmu.loadg(a.bmu, x);
      bfg.loadg(a.bfgrad, x);
      oA.load(a.bA, x);
      op.load(a.bpsi, x);
      oR.load(a.bR, x);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const T Ae = A.v[e], Le = L.v[e], pe = psi.v[e], re = rho.v[e], bm = bmu.v[e], bf = bfg.v[e];
        const T t = s.rho0 + s.kp * Ae, rd = rden.v[e];
        const T p2 = pe * pe;
        const T P5 = Le - s.ep * pe - s.beta * (p2 * pe) + s.gamma * (p2 * p2 * pe);
        const T blap = bmu1.v[e] + bm;
        T brho = Le * bmu1.v[e] + P5 * bm + EbE.v[e] + s.zeta * re * bf + (s.kp * s.zeta * rd) * bc.v[e];
        oL.v[e] = re * bmu1.v[e] + re * bm + Le * bEn.v[e];
        op.v[e] += re * (-s.ep - T(3.0) * s.beta * p2 + T(5.0) * s.gamma * (p2 * p2)) * bm;
        const T bt = -s.zeta * t * bf - (s.kp * s.zeta * rd) * bc.v[e];
        T bA = s.kp * bt + bc.v[e] * (-s.kp * s.zeta * (re - t) * (rd * rd));
        T dkp = bt * Ae + bc.v[e] * s.zeta * (re - t) * rd, drho0 = bt;
        acc[0] += bm * re * (-(p2 * pe));
        acc[1] += bm * re * (p2 * p2 * pe);
        if (a.relax) {
          brho += lraw.v[e] * blap;
          ol.v[e] = re * blap;
          const T bri = brho + oR.v[e];  // every use of the reset density
          bA += s.kp * bri;
          dkp += Ae * bri;
          drho0 += bri;
          oR.v[e] = T(0.0);
        } else {
          ol.v[e] = blap;
          oR.v[e] += brho;
        }
        acc[2] += drho0;
        acc[3] += dkp;
        oA.v[e] += bA;
      }
      if (a.ew != T(0.0)) {
        V4<T> rn;
        rn.loadg(a.rho_new, x);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          oL.v[e] += a.ew * rn.v[e] * L.v[e];
          oA.v[e] += -a.ew * s.zeta * s.kp * (rn.v[e] - s.rho0 - s.kp * A.v[e]);
        }
      }
      oL.store(a.bL, x);
      op.store(a.bpsi, x);
      ol.store(a.blapR, x);
      oR.store(a.bR, x);
      oA.store(a.bA, x);
    }
  }
  const int slots[4] = {PG_BETA, PG_GAMMA, PG_RHO0, PG_KP};
  block_accum(acc, slots, g, a.pgrad);
}

// Energy term of the loss at the final state, E = dx^3 sum [rho e + zeta/2 d^2] with
// e = -ep/2 psi^2 + L^2/2 - beta/4 psi^4 + gamma/6 psi^6 and d = rho - rho_0 - kp A
// (REF:2214-2231; psi and rho after the last step, L and A of the last step). With
// w = lambda dx^3: psi_bar += w rho (-ep psi - beta psi^3 + gamma psi^5),
// rho_bar += w (e + zeta d), and the direct partials of beta, gamma, rho_0 and kp.
// (L_bar and A_bar enter in the last step's adj_s6_kernel.)
template <typename T>
__global__ void __launch_bounds__(256) adj_energy_final_kernel(Grid g, const T* psi, const double* rho, const T* L,
                                                               const T* A, T w, AdjScalars<T> s, T* bpsi, T* bR,
                                                               double* pgrad) {
  Pt4 p;
  T acc[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};  // beta, gamma, rho0, kp
  if (pt4(g, p)) {
    const long long x = p.idx;
    V4<T> ps, l, a, bp, br;
    ps.load(psi, x);
    l.load(L, x);
    a.load(A, x);
    bp.load(bpsi, x);
    br.load(bR, x);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const T r = (T)rho[x + e], pe = ps.v[e], p2 = pe * pe;
      const T en = -T(0.5) * s.ep * p2 + T(0.5) * (l.v[e] * l.v[e]) - T(0.25) * s.beta * (p2 * p2) +
                   (s.gamma / T(6.0)) * (p2 * p2 * p2);
      const T d = r - s.rho0 - s.kp * a.v[e];
      bp.v[e] += w * r * (-s.ep * pe - s.beta * (p2 * pe) + s.gamma * (p2 * p2 * pe));
      br.v[e] += w * (en + s.zeta * d);
      acc[0] += w * r * (-T(0.25) * (p2 * p2));
      acc[1] += w * r * ((p2 * p2 * p2) / T(6.0));
      acc[2] += -w * s.zeta * d;
      acc[3] += -w * s.zeta * d * a.v[e];
    }
    bp.store(bpsi, x);
    br.store(bR, x);
  }
  const int slots[4] = {PG_BETA, PG_GAMMA, PG_RHO0, PG_KP};
  block_accum(acc, slots, g, pgrad);
}

// bQ += Lambda(q) Y for the spectral multipliers of the forward (REF:1302 for
// dfDlapPsi, REF:1356 for the relax-phase Laplacian), and alpha_bar += Y dLambda/dalpha Q.
//   mode 0: Lambda = alpha (q0^2 - q^2);   mode 1: Lambda = -q^2 alpha (q0^2 - q^2)
// Y arrives without the output weights wy of the transposed transform that made it.
template <typename T>
__global__ void __launch_bounds__(256) adj_acc_spec_kernel(Grid g, const T* qx, const T* qy, const T* qz,
                                                           int mode, T alpha, T q02, AxisWeights<T> wy,
                                                           const T* Y, const T* Q, T* bQ, double* pgrad) {
  Pt4 p;
  T da[1] = {T(0.0)};
  if (pt4(g, p)) {
    const long long x = p.idx;
    V4<T> y, q, b;
    y.load(Y, x);
    q.load(Q, x);
    b.load(bQ, x);
    const T qxy = qx[p.i] * qx[p.i] + qy[p.j] * qy[p.j];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const T kz = qz[p.k + e];
      const T mq2 = qxy + kz * kz;
      const T dl = mode == 0 ? (q02 - mq2) : -mq2 * (q02 - mq2);  // dLambda/dalpha
      const T ye = y.v[e] * wy.at(g, p.i, p.j, p.k + e);
      b.v[e] += alpha * dl * ye;
      da[0] += ye * dl * q.v[e];
    }
    b.store(bQ, x);
  }
  const int slots[1] = {PG_ALPHA};
  block_accum(da, slots, g, pgrad);
}

// Transpose of A_raw = sqrt(q0^2 psi^2 + |grad psi|^2) (REF:1262-1266), applied to
// y = F(bar A) (the amplitude filter F of REF:1271-1288 is symmetric).
template <typename T>
__global__ void __launch_bounds__(256) adj_amp_kernel(Grid g, const T* y, const T* psi, const T* gx, const T* gy,
                                                      const T* gz, T q02, T* bpsi, T* bgx, T* bgy, T* bgz) {
  Pt4 p;
  if (!pt4(g, p)) return;
  const long long x = p.idx;
  V4<T> Y, P, X, G, Z, bp, bx, by, bz;
  Y.load(y, x);
  P.load(psi, x);
  X.load(gx, x);
  G.load(gy, x);
  Z.load(gz, x);
  bp.load(bpsi, x);
  bx.load(bgx, x);
  by.load(bgy, x);
  bz.load(bgz, x);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const T pe = P.v[e], ae = X.v[e], be = G.v[e], ce = Z.v[e];
    const T A = sqrt(q02 * (pe * pe) + (ae * ae) + (be * be) + (ce * ce));
    if (!(A > T(0.0))) continue;  // the square root is not differentiable at 0: no contribution
    const T sc = Y.v[e] / A;
    bp.v[e] += q02 * pe * sc;
    bx.v[e] += ae * sc;
    by.v[e] += be * sc;
    bz.v[e] += ce * sc;
  }
  bp.store(bpsi, x);
  bx.store(bgx, x);
  by.store(bgy, x);
  bz.store(bgz, x);
}

// End of step (11) of the adjoint: the transposed derivative passes of both gradient
// families summed into the cotangents of the step's input psi and rho.
template <typename T>
__global__ void __launch_bounds__(256) adj_gsum_kernel(Grid g, const T* px, const T* py, const T* pz, const T* rx,
                                                       const T* ry, const T* rz, T* bpsi, T* brho) {
  Pt4 p;
  if (!pt4(g, p)) return;
  const long long x = p.idx;
  V4<T> a, b, c, o;
  a.load(px, x);
  b.load(py, x);
  c.load(pz, x);
  o.load(bpsi, x);
#pragma unroll
  for (int e = 0; e < 4; ++e) o.v[e] += a.v[e] + b.v[e] + c.v[e];
  o.store(bpsi, x);
  a.load(rx, x);
  b.load(ry, x);
  c.load(rz, x);
  o.load(brho, x);
#pragma unroll
  for (int e = 0; e < 4; ++e) o.v[e] += a.v[e] + b.v[e] + c.v[e];
  o.store(brho, x);
}

// End of the adjoint step, the transpose of psi = DCT-III^3 psiq (REF:2194-2197):
// bQ += wq ypsi (ypsi without the output weights wq of its transposed transform).
template <typename T>
__global__ void __launch_bounds__(256) adj_fold_kernel(Grid g, const T* ypsi, AxisWeights<T> wq, T* bQ) {
  Pt4 p;
  if (!pt4(g, p)) return;
  const long long x = p.idx;
  V4<T> yp, q;
  yp.load(ypsi, x);
  q.load(bQ, x);
#pragma unroll
  for (int e = 0; e < 4; ++e) q.v[e] = q.v[e] + yp.v[e] * wq.at(g, p.i, p.j, p.k + e);
  q.store(bQ, x);
}

// out = a * x (+ b * y): small helper for the final dL/dpsi0 = scale C2^T (bQ + bQo).
template <typename T>
__global__ void __launch_bounds__(256) axpby_kernel(long long n, T a, const T* x, T b, const T* y,
                                                    T* out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) out[idx] = a * x[idx] + (y ? b * y[idx] : T(0.0));
}

}  // namespace swc
