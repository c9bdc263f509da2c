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

// accumulate (+=) a real-space result
template <typename T> struct StAcc {
  T* p;
  __device__ __forceinline__ void operator()(int, int, int, long long idx, T v) const { p[idx] += v; }
  __device__ __forceinline__ void pair(int, int, int, long long idx, float2 v) const {
    const float2 o = ld2v(p, idx);
    st2v(p, idx, make_float2(o.x + v.x, o.y + v.y));
  }
};

// Transpose of the shifted spectral derivative (REF:1190-1219): the forward wrote
// out[c] = -fac Vs[c] in[c+1]; here in_bar[c+1] += -fac Vs[c] y[c] (output weight
// of the transposed inverse transform applied first).
template <typename T> struct StAdjGrad {
  Grid g;
  T* target;
  const T* vs;
  T fac;
  int axis;
  long long shift;
  AxisWeights<T> aw;
  __device__ __forceinline__ void operator()(int i, int j, int k, long long idx, T v) const {
    const int c = axis == 0 ? i : (axis == 1 ? j : k);
    const int n = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
    if (c >= n - 1) return;
    target[idx + shift] += -fac * vs[c] * (v * aw.at(g, i, j, k));
  }
  // x/y passes of the FP32 two-line pass: elements (k, k+1); an even shift keeps the
  // shifted pair 8-byte aligned (one vector read-modify-write), shift 1 does not
  __device__ __forceinline__ void pair(int i, int j, int k, long long idx, float2 v) const {
    if (shift & 1) {
      (*this)(i, j, k, idx, v.x);
      (*this)(i, j, k + 1, idx + 1, v.y);
      return;
    }
    const int n = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
    const int c0 = axis == 0 ? i : (axis == 1 ? j : k), c1 = axis == 2 ? k + 1 : c0;
    const float a = (c0 < n - 1) ? -(float)fac * (float)vs[c0] * (v.x * (float)aw.at(g, i, j, k)) : 0.f;
    const float b = (c1 < n - 1) ? -(float)fac * (float)vs[c1] * (v.y * (float)aw.at(g, i, j, k + 1)) : 0.f;
    if (c0 >= n - 1 && c1 >= n - 1) return;
    const float2 o = ld2v(target, idx + shift);
    st2v(target, idx + shift, make_float2(o.x + a, o.y + b));
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

// Last pass of F(bar A) (F symmetric, REF:1271-1288), then the transpose of
// A_raw = sqrt(q0^2 psi^2 + |grad psi|^2) (REF:1262-1266).
template <typename T> struct StAdjAmp {
  const T *psi, *gx, *gy, *gz;
  T *bpsi, *bgx, *bgy, *bgz;
  T q02;
  __device__ __forceinline__ void operator()(int, int, int, long long idx, T y) const {
    const T p = psi[idx], a = gx[idx], b = gy[idx], c = gz[idx];
    const T A = sqrt(q02 * (p * p) + (a * a) + (b * b) + (c * c));
    if (!(A > 0)) return;  // the square root is not differentiable at 0: no contribution
    const T s = y / A;
    bpsi[idx] += q02 * p * s;
    bgx[idx] += a * s;
    bgy[idx] += b * s;
    bgz[idx] += c * s;
  }
  // z pass of the FP32 two-line pass: four consecutive elements with vector accesses
  __device__ __forceinline__ void quad(int, int, int, long long idx, float4 y) const {
    const float4 P = ld4v(psi, idx), X = ld4v(gx, idx), Y = ld4v(gy, idx), Z = ld4v(gz, idx);
    float4 bp = ld4v(bpsi, idx), bx = ld4v(bgx, idx), by = ld4v(bgy, idx), bz = ld4v(bgz, idx);
    const float q = (float)q02;
    auto one = [&](float p, float a, float b, float c, float yy, float& op, float& ox, float& oy, float& oz) {
      const float A = sqrtf(q * (p * p) + (a * a) + (b * b) + (c * c));
      if (!(A > 0.f)) return;
      const float s2 = yy / A;
      op += q * p * s2;
      ox += a * s2;
      oy += b * s2;
      oz += c * s2;
    };
    one(P.x, X.x, Y.x, Z.x, y.x, bp.x, bx.x, by.x, bz.x);
    one(P.y, X.y, Y.y, Z.y, y.y, bp.y, bx.y, by.y, bz.y);
    one(P.z, X.z, Y.z, Z.z, y.z, bp.z, bx.z, by.z, bz.z);
    one(P.w, X.w, Y.w, Z.w, y.w, bp.w, bx.w, by.w, bz.w);
    st4v(bpsi, idx, bp);
    st4v(bgx, idx, bx);
    st4v(bgy, idx, by);
    st4v(bgz, idx, bz);
  }
};

// parameter-gradient slots
enum { PG_ALPHA = 0, PG_BETA = 1, PG_GAMMA = 2, PG_NU = 3, PG_RHO0 = 4, PG_KP = 5, PG_COUNT = 8 };

// Block sum of v (in its own precision: the FP32 adjoint sums a block in FP32) added in
// FP64 to this block's own cell of parameter slot `slot` (all threads of the block must
// call). The cells sit after the PG_COUNT totals, gridDim.x per slot, and
// are summed in a fixed order by pg_reduce_kernel, so the parameter gradients do not
// depend on the order in which blocks finish (no atomics).
template <typename V> __device__ __forceinline__ void block_accum(V v, double* pgrad, int slot) {
  __shared__ V shv[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) shv[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    V t = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += shv[q];
    pgrad[PG_COUNT + (size_t)slot * gridDim.x + blockIdx.x] += (double)t;
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
                                                     T* bQ, T* bQo, T* bNlo, T* bNlq,
                                                     double* pgrad) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  T da = 0;
  if (idx < g.ng) {
    int i, j, k;
    decompose(g, idx, i, j, k);
    const T mq2 = qx[i] * qx[i] + qy[j] * qy[j] + qz[k] * qz[k];
    const T sq = s.q02 - mq2;
    const T aLin = s.ep - s.alpha * (sq * sq);
    const T C1 = T(2.0) - s.dt * s.rho_m * aLin, C2 = T(1.5) - s.dt * s.rho_m * aLin;
    const T h = s.dtd2 * s.scale;
    const T bq = bQ[idx];
    if constexpr (sizeof(T) == 8) {  // the FP64 adjoint keeps its divisions
      T bnl = T(3.0) * h / C2 * bq + bNlo[idx];
      if (first) bnl += -h / C2 * bq;  // REF:2170-2172: Nl_old = Nl at nLoop == 1
      bNlq[idx] = bnl;
      bNlo[idx] = first ? T(0.0) : -h / C2 * bq;
      const T bqo_next = bQo[idx];
      bQo[idx] = -T(0.5) / C2 * bq;
      bQ[idx] = C1 / C2 * bq + bqo_next;
      // dC1/dalpha = dC2/dalpha = dt rho_m sq^2  =>  dQ'/dalpha = dt rho_m sq^2 (Q - Q') / C2
      da = bq * s.dt * s.rho_m * sq * sq * (Qold[idx] - Qnew[idx]) / C2;
    } else {  // FP32: one reciprocal
      const T r = T(1.0) / C2, hb = h * r * bq;
      T bnl = T(3.0) * hb + bNlo[idx];
      if (first) bnl -= hb;
      bNlq[idx] = bnl;
      bNlo[idx] = first ? T(0.0) : -hb;
      const T bqo_next = bQo[idx];
      bQo[idx] = -T(0.5) * r * bq;
      bQ[idx] = C1 * r * bq + bqo_next;
      da = bq * s.dt * s.rho_m * sq * sq * (Qold[idx] - Qnew[idx]) * r;
    }
  }
  block_accum(da, pgrad, PG_ALPHA);
}

// Transpose of dq = q . f-hat shifted (REF:2076-2078, subtracted from Nl-hat): f-hat_a
// at c receives -Vq_a[c+1] bar(Nlq) at c+1.
template <typename T>
__global__ void __launch_bounds__(256) adj_dq_kernel(Grid g, const T* qx, const T* qy, const T* qz,
                                                     const T* bNlq, T* bfx, T* bfy, T* bfz) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.ng) return;
  int i, j, k;
  decompose(g, idx, i, j, k);
  const long long sx = 1LL << (g.ly + g.lz), sy = g.nz;
  bfx[idx] = (i + 1 < g.nx) ? -qx[i + 1] * bNlq[idx + sx] : T(0.0);
  bfy[idx] = (j + 1 < g.ny) ? -qy[j + 1] * bNlq[idx + sy] : T(0.0);
  bfz[idx] = (k + 1 < g.nz) ? -qz[k + 1] * bNlq[idx + 1] : T(0.0);
}

// Transpose of the density update (REF:2121-2139) and of the real-space Nl
// (REF:2153-2160, grad.f handled by adj_dq_kernel):
//   S_rho = -v.grad rho - rho_in divv;  rho' = rho_in + dt (T(1.5) S_rho - T(0.5) F);  F' = S_rho
//   Nl = -mu + c' (rho' - rho0 - kp A) psi - v.grad psi,  c' = kp zeta/(A + T(0.001))
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
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  T dkp = 0, drho0 = 0;
  if (idx < g.ng) {
    const T b = a.bNl[idx], psi = a.psi[idx], A = a.A[idx];
    const T rin = a.relax ? a.s.rho0 + a.s.kp * A : a.rho_in[idx];
    const T rn = a.rho_new[idx];
    const T den = A + T(0.001);
    const T cp = a.s.kp * a.s.zeta / den;
    const T t2 = rn - a.s.rho0 - a.s.kp * A;
    const T brp = a.bR[idx] + cp * psi * b;  // bar rho'
    a.bmu[idx] = -b;
    a.bA[idx] = psi * b * (-a.s.kp * a.s.zeta * t2 / (den * den) - cp * a.s.kp);
    a.bpsi[idx] = cp * t2 * b;
    const T vx = a.vx[idx], vy = a.vy[idx], vz = a.vz[idx];
    const T bS = a.bF[idx] + T(1.5) * a.s.dt * brp;  // bar S_rho
    a.bgpx[idx] = -vx * b;
    a.bgpy[idx] = -vy * b;
    a.bgpz[idx] = -vz * b;
    a.bvx[idx] = -a.gpx[idx] * b - a.grx[idx] * bS;
    a.bvy[idx] = -a.gpy[idx] * b - a.gry[idx] * bS;
    a.bvz[idx] = -a.gpz[idx] * b - a.grz[idx] * bS;
    a.bgrx[idx] = -vx * bS;
    a.bgry[idx] = -vy * bS;
    a.bgrz[idx] = -vz * bS;
    a.bdivv[idx] = -rin * bS;
    a.bR[idx] = brp - a.divv[idx] * bS;  // bar rho_in (relax: folded into A later)
    a.bF[idx] = -T(0.5) * a.s.dt * brp;
    dkp = b * psi * (a.s.zeta * t2 / den - cp * A);
    drho0 = -b * psi * cp;
  }
  block_accum(dkp, a.pgrad, PG_KP);
  block_accum(drho0, a.pgrad, PG_RHO0);
}

// Transpose of the Stokes solve, part 1 (REF:1581-1974 and the divergence REF:2076):
// at each output mode o and component a (where the forward computed it) form
//   bar dot_a(o)  = -(CM1/nu) CM2 bar vsol + (CM1/(lam+2nu)) CM2 G bar virr
//   bSdir_a(o)    =  (CM1/nu) bar vsol            (the S_a(o) term)
//   bfgp_a(o)     =  (CM1/(lam+2nu)) Vs bar virr   (the f-grad'(o + e_a) term)
// with bar vsol = bar v-hat_a, bar virr = bar v-hat_a + Vq_a[o_a+1] bar divv-hat(o + e_a);
// zero elsewhere. nu_bar += bar vsol (-vsol/nu) + bar virr (-2 virr/(lam + 2nu)).
template <typename T> struct AdjStokesArgs {
  const T *bvx, *bvy, *bvz, *bdq, *vsx_, *vsy_, *vsz_, *vix, *viy, *viz;
  T *bdotx, *bdoty, *bdotz, *bsx, *bsy, *bsz, *bgx, *bgy, *bgz;
  const T *vqx, *vqy, *vqz, *vsx, *vsy, *vsz, *gqx, *gqy, *gqz, *gsx, *gsy, *gsz;
  T scale, inv_nu, inv_lam2nu, nu, lam2nu;
  int block;
  double* pgrad;
};
template <typename T>
__global__ void __launch_bounds__(256) adj_stokes1_kernel(Grid g, AdjStokesArgs<T> a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  T dnu = 0;
  if (idx < g.ng) {
    int i, j, k;
    decompose(g, idx, i, j, k);
    const long long sx = 1LL << (g.ly + g.lz), sy = g.nz;
    const T qxi = a.vqx[i], qyj = a.vqy[j], qzk = a.vqz[k];
    T d = 0, sd = 0, fp = 0;
    if (i < g.nx - 1) {
      const T s_ = a.vsx[i];
      const T inv = T(1.0) / (s_ * s_ + qyj * qyj + qzk * qzk);
      const T CM1 = a.scale * inv, CM2 = s_ * inv, G = a.gsx[i] * a.gqy[j] * a.gqz[k];
      const T bvs = a.bvx[idx];
      const T bvi = bvs + a.vqx[i + 1] * a.bdq[idx + sx];
      d = -(CM1 * a.inv_nu) * CM2 * bvs + (CM1 * a.inv_lam2nu) * CM2 * G * bvi;
      sd = (CM1 * a.inv_nu) * bvs;
      fp = (CM1 * a.inv_lam2nu) * s_ * bvi;
      dnu += bvs * (-a.vsx_[idx] / a.nu) + bvi * (-T(2.0) * a.vix[idx] / a.lam2nu);
    }
    a.bdotx[idx] = d; a.bsx[idx] = sd; a.bgx[idx] = fp;
    T dy = 0, sdy = 0, fpy = 0, dz = 0, sdz = 0, fpz = 0;
    if (j < g.ny - 1 && k < g.nz - 1) {
      {
        const T s_ = a.vsy[j];
        const T inv = T(1.0) / (qxi * qxi + s_ * s_ + qzk * qzk);
        const T CM1 = a.scale * inv, CM2 = s_ * inv, G = a.gqx[i] * a.gsy[j] * a.gqz[k];
        const T bvs = a.bvy[idx];
        const T bvi = bvs + a.vqy[j + 1] * a.bdq[idx + sy];
        dy = -(CM1 * a.inv_nu) * CM2 * bvs + (CM1 * a.inv_lam2nu) * CM2 * G * bvi;
        sdy = (CM1 * a.inv_nu) * bvs;
        fpy = (CM1 * a.inv_lam2nu) * s_ * bvi;
        dnu += bvs * (-a.vsy_[idx] / a.nu) + bvi * (-T(2.0) * a.viy[idx] / a.lam2nu);
      }
      {
        const T s_ = a.vsz[k];
        const T inv = T(1.0) / (qxi * qxi + qyj * qyj + s_ * s_);
        const T CM1 = a.scale * inv, CM2 = s_ * inv;
        const bool q1 = (k == 0) && (j > 0) && (i % a.block != 0);  // REF:1932
        const T G = q1 ? (a.gqx[i] * a.gsy[j] * a.gqz[k]) : (a.gqx[i] * a.gqy[j] * a.gsz[k]);
        const T bvs = a.bvz[idx];
        const T bvi = bvs + a.vqz[k + 1] * a.bdq[idx + 1];
        dz = -(CM1 * a.inv_nu) * CM2 * bvs + (CM1 * a.inv_lam2nu) * CM2 * G * bvi;
        sdz = (CM1 * a.inv_nu) * bvs;
        fpz = (CM1 * a.inv_lam2nu) * s_ * bvi;
        dnu += bvs * (-a.vsz_[idx] / a.nu) + bvi * (-T(2.0) * a.viz[idx] / a.lam2nu);
      }
    }
    a.bdoty[idx] = dy; a.bsy[idx] = sdy; a.bgy[idx] = fpy;
    a.bdotz[idx] = dz; a.bsz[idx] = sdz; a.bgz[idx] = fpz;
  }
  block_accum(dnu, a.pgrad, PG_NU);
}

// Transpose of the Stokes solve, part 2: gather at each input mode p the terms of
// every output mode that read it (REF:1596-1624, 1775-1841 read patterns):
//   S_x(p): dot_x(p) w Vs_x[p_x]; dot_y(p_x+1, p_y-1, p_z) w Vq_x[p_x+1]; dot_z(p_x+1, p_y, p_z-1) w Vq_x[p_x+1]
//   S_y(p): dot_y(p) w Vs_y[p_y]; dot_x(p_x-1, p_y+1, p_z) w Vq_y[p_y+1]; dot_z(p_x, p_y+1, p_z-1) w Vq_y[p_y+1]
//   S_z(p): dot_z(p) w Vs_z[p_z]; dot_x(p_x-1, p_y, p_z+1) w Vq_z[p_z+1]; dot_y(p_x, p_y-1, p_z+1) w Vq_z[p_z+1]
//   fgrad'(p) = sum_a bfgp_a(p - e_a)
// bar dot and bfgp are zero outside each component's computed modes, so only the
// array bounds are tested. Then f-grad-hat_bar = fgrad'_bar, E-hat_bar = G fgrad'_bar (REF:1486).
template <typename T> struct AdjStokes2Args {
  const T *bdotx, *bdoty, *bdotz, *bsx, *bsy, *bsz, *bgx, *bgy, *bgz;
  T *bSx, *bSy, *bSz, *bfg, *bE;
  const T *vqx, *vqy, *vqz, *vsx, *vsy, *vsz, *gqx, *gqy, *gqz;
};
template <typename T>
__global__ void __launch_bounds__(256) adj_stokes2_kernel(Grid g, AdjStokes2Args<T> a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.ng) return;
  int i, j, k;
  decompose(g, idx, i, j, k);
  const long long sx = 1LL << (g.ly + g.lz), sy = g.nz;
  T Sx = a.bsx[idx] + a.vsx[i] * a.bdotx[idx];
  if (i + 1 < g.nx) {
    if (j >= 1) Sx += a.vqx[i + 1] * a.bdoty[idx + sx - sy];
    if (k >= 1) Sx += a.vqx[i + 1] * a.bdotz[idx + sx - 1];
  }
  T Sy = a.bsy[idx] + a.vsy[j] * a.bdoty[idx];
  if (j + 1 < g.ny) {
    if (i >= 1) Sy += a.vqy[j + 1] * a.bdotx[idx - sx + sy];
    if (k >= 1) Sy += a.vqy[j + 1] * a.bdotz[idx + sy - 1];
  }
  T Sz = a.bsz[idx] + a.vsz[k] * a.bdotz[idx];
  if (k + 1 < g.nz) {
    if (i >= 1) Sz += a.vqz[k + 1] * a.bdotx[idx - sx + 1];
    if (j >= 1) Sz += a.vqz[k + 1] * a.bdoty[idx - sy + 1];
  }
  a.bSx[idx] = Sx;
  a.bSy[idx] = Sy;
  a.bSz[idx] = Sz;
  T fg = 0;
  if (i >= 1) fg += a.bgx[idx - sx];
  if (j >= 1) fg += a.bgy[idx - sy];
  if (k >= 1) fg += a.bgz[idx - 1];
  a.bfg[idx] = fg;
  a.bE[idx] = fg * (a.gqx[i] * a.gqy[j] * a.gqz[k]);
}

// Transpose of S6 (REF:1385-1425) and of the relax reset (REF:1371-1374):
//   E = L^2/2, t = rho0 + kp A, fgrad = zeta/2 (rho^2 - t^2), mu1 = lapR + rho L,
//   S_a = mu1 gpsi_a + E grho_a, mu = lapR + rho P5, P5 = L - ep psi - beta psi^3 + gamma psi^5,
//   Erho = rho E, c = kp zeta (rho - t)/(A + T(0.001)), f_a = c gpsi_a;
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
};
template <typename T>
__global__ void __launch_bounds__(256) adj_s6_kernel(Grid g, AdjS6Args<T> a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  T dbeta = 0, dgamma = 0, drho0 = 0, dkp = 0;
  if (idx < g.ng) {
    const T A = a.A[idx], L = a.L[idx], psi = a.psi[idx];
    const T rho = a.relax ? a.s.rho0 + a.s.kp * A : a.rho_in[idx];
    const T lraw = a.lapR[idx];
    const T lapR = a.relax ? rho * lraw : lraw;
    const T gpx = a.gpx[idx], gpy = a.gpy[idx], gpz = a.gpz[idx];
    const T grx = a.grx[idx], gry = a.gry[idx], grz = a.grz[idx];
    const T E = T(0.5) * (L * L), t = a.s.rho0 + a.s.kp * A, den = A + T(0.001);
    const T mu1 = lapR + rho * L;
    const T c = a.s.kp * a.s.zeta * (rho - t) / den;
    const T p2 = psi * psi;
    const T P5 = L - a.s.ep * psi - a.s.beta * (p2 * psi) + a.s.gamma * (p2 * p2 * psi);
    const T bSx = a.bSx[idx], bSy = a.bSy[idx], bSz = a.bSz[idx];
    const T bfx = a.bfx[idx], bfy = a.bfy[idx], bfz = a.bfz[idx];
    const T bmu = a.bmu[idx], bfg = a.bfgrad[idx], bEr = a.bE[idx];
    const T bmu1 = bSx * gpx + bSy * gpy + bSz * gpz;
    a.bgpx[idx] += mu1 * bSx + c * bfx;
    a.bgpy[idx] += mu1 * bSy + c * bfy;
    a.bgpz[idx] += mu1 * bSz + c * bfz;
    const T bEn = bSx * grx + bSy * gry + bSz * grz + rho * bEr;
    a.bgrx[idx] += E * bSx;
    a.bgry[idx] += E * bSy;
    a.bgrz[idx] += E * bSz;
    const T bc = bfx * gpx + bfy * gpy + bfz * gpz;
    const T blap = bmu1 + bmu;
    T brho = L * bmu1 + P5 * bmu + E * bEr + a.s.zeta * rho * bfg + (a.s.kp * a.s.zeta / den) * bc;
    a.bL[idx] = rho * bmu1 + rho * bmu + L * bEn;
    a.bpsi[idx] += rho * (-a.s.ep - T(3.0) * a.s.beta * p2 + T(5.0) * a.s.gamma * (p2 * p2)) * bmu;
    const T bt = -a.s.zeta * t * bfg - (a.s.kp * a.s.zeta / den) * bc;
    T bA = a.s.kp * bt + bc * (-a.s.kp * a.s.zeta * (rho - t) / (den * den));
    dkp = bt * A + bc * a.s.zeta * (rho - t) / den;
    drho0 = bt;
    dbeta = bmu * rho * (-(p2 * psi));
    dgamma = bmu * rho * (p2 * p2 * psi);
    if (a.relax) {
      brho += lraw * blap;
      a.blapR[idx] = rho * blap;
      const T bri = brho + a.bR[idx];  // every use of the reset density
      bA += a.s.kp * bri;
      dkp += A * bri;
      drho0 += bri;
      a.bR[idx] = T(0.0);
    } else {
      a.blapR[idx] = blap;
      a.bR[idx] += brho;
    }
    a.bA[idx] += bA;
  }
  block_accum(dbeta, a.pgrad, PG_BETA);
  block_accum(dgamma, a.pgrad, PG_GAMMA);
  block_accum(drho0, a.pgrad, PG_RHO0);
  block_accum(dkp, a.pgrad, PG_KP);
}

// bQ += Lambda(q) Y for the spectral multipliers of the forward (REF:1302 for
// dfDlapPsi, REF:1356 for the relax-phase Laplacian), and alpha_bar += Y dLambda/dalpha Q.
//   mode 0: Lambda = alpha (q0^2 - q^2);   mode 1: Lambda = -q^2 alpha (q0^2 - q^2)
template <typename T>
__global__ void __launch_bounds__(256) adj_acc_spec_kernel(Grid g, const T* qx, const T* qy,
                                                           const T* qz, int mode, T alpha, T q02,
                                                           const T* Y, const T* Q, T* bQ,
                                                           double* pgrad) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  T da = 0;
  if (idx < g.ng) {
    int i, j, k;
    decompose(g, idx, i, j, k);
    const T mq2 = qx[i] * qx[i] + qy[j] * qy[j] + qz[k] * qz[k];
    const T dl = mode == 0 ? (q02 - mq2) : -mq2 * (q02 - mq2);  // dLambda/dalpha
    const T y = Y[idx];
    bQ[idx] += alpha * dl * y;
    da = y * dl * Q[idx];
  }
  block_accum(da, pgrad, PG_ALPHA);
}

// out = a * x (+ b * y): small helper for the final dL/dpsi0 = scale C2^T (bQ + bQo).
template <typename T>
__global__ void __launch_bounds__(256) axpby_kernel(long long n, T a, const T* x, T b, const T* y,
                                                    T* out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) out[idx] = a * x[idx] + (y ? b * y[idx] : T(0.0));
}

}  // namespace swc
