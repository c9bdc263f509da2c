// swc_adjoint_kernels.cuh -- kernels of the discrete adjoint of one time step
// (FP64). Each kernel is the transpose of one forward stage of swc_step_impl.cuh;
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
struct AxisWeights {
  int sine[3];
  double w;
  __device__ __forceinline__ double at(const Grid& g, int i, int j, int k) const {
    double f = 1.0;
    f *= (sine[0] ? (i == g.nx - 1) : (i == 0)) ? w : 1.0;
    f *= (sine[1] ? (j == g.ny - 1) : (j == 0)) ? w : 1.0;
    f *= (sine[2] ? (k == g.nz - 1) : (k == 0)) ? w : 1.0;
    return f;
  }
};

// load x * weight (input side of DCT-II^T / DST-II^T), optionally times a second
// pointwise factor table (the Gaussian G of REF:1486)
struct LdW {
  Grid g;
  const double* p;
  AxisWeights aw;
  __device__ __forceinline__ double operator()(int i, int j, int k, long long idx) const {
    return p[idx] * aw.at(g, i, j, k);
  }
};

// store v * weight (output side of DCT-III^T / DST-III^T); acc: += instead of =
struct StW {
  Grid g;
  double* p;
  AxisWeights aw;
  int acc;
  __device__ __forceinline__ void operator()(int i, int j, int k, long long idx, double v) const {
    const double y = v * aw.at(g, i, j, k);
    p[idx] = acc ? p[idx] + y : y;
  }
};

// accumulate (+=) a real-space result
struct StAcc {
  double* p;
  __device__ __forceinline__ void operator()(int, int, int, long long idx, double v) const { p[idx] += v; }
};

// Transpose of the shifted spectral derivative (REF:1190-1219): the forward wrote
// out[c] = -fac Vs[c] in[c+1]; here in_bar[c+1] += -fac Vs[c] y[c] (output weight
// of the transposed inverse transform applied first).
struct StAdjGrad {
  Grid g;
  double* target;
  const double* vs;
  double fac;
  int axis;
  long long shift;
  AxisWeights aw;
  __device__ __forceinline__ void operator()(int i, int j, int k, long long idx, double v) const {
    const int c = axis == 0 ? i : (axis == 1 ? j : k);
    const int n = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
    if (c >= n - 1) return;
    target[idx + shift] += -fac * vs[c] * (v * aw.at(g, i, j, k));
  }
};

// Last pass of Delta_s(bar lapR) (normal phase, transpose of REF:1319-1342):
// rho_bar += L * y, L_bar += rho * y (Delta_s is symmetric).
struct StAdjLap {
  const double *L, *rho;
  double *brho, *bL;
  __device__ __forceinline__ void operator()(int, int, int, long long idx, double y) const {
    brho[idx] += L[idx] * y;
    bL[idx] += rho[idx] * y;
  }
};

// Last pass of F(bar A) (F symmetric, REF:1271-1288), then the transpose of
// A_raw = sqrt(q0^2 psi^2 + |grad psi|^2) (REF:1262-1266).
struct StAdjAmp {
  const double *psi, *gx, *gy, *gz;
  double *bpsi, *bgx, *bgy, *bgz;
  double q02;
  __device__ __forceinline__ void operator()(int, int, int, long long idx, double y) const {
    const double p = psi[idx], a = gx[idx], b = gy[idx], c = gz[idx];
    const double A = sqrt(q02 * (p * p) + (a * a) + (b * b) + (c * c));
    if (!(A > 0)) return;  // the square root is not differentiable at 0: no contribution
    const double s = y / A;
    bpsi[idx] += q02 * p * s;
    bgx[idx] += a * s;
    bgy[idx] += b * s;
    bgz[idx] += c * s;
  }
};

// parameter-gradient slots
enum { PG_ALPHA = 0, PG_BETA = 1, PG_GAMMA = 2, PG_NU = 3, PG_RHO0 = 4, PG_KP = 5, PG_COUNT = 8 };

// Block sum of v added to this block's own cell of parameter slot `slot` (all threads of
// the block must call). The cells sit after the PG_COUNT totals, gridDim.x per slot, and
// are summed in a fixed order by pg_reduce_kernel, so the parameter gradients do not
// depend on the order in which blocks finish (no atomics).
__device__ __forceinline__ void block_accum(double v, double* pgrad, int slot) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    pgrad[PG_COUNT + (size_t)slot * gridDim.x + blockIdx.x] += t;
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

struct AdjScalars {
  double ep, alpha, beta, gamma, zeta, kp, rho0, q02, dt, dtd2, rho_m, scale, nu, lam2nu;
};

// Transpose of the CN/AB2 update (REF:2185-2187) and of Nl_old <- Nl, psiq_old <- psiq.
//   Q' = (C1 Q - Qo/2 + h (3 Nl - Nlo)) / C2, Qo' = Q, Nlo' = Nl  (h = dt/2 scale)
__global__ void __launch_bounds__(256) adj_cn_kernel(Grid g, const double* qx, const double* qy, const double* qz,
                                                     AdjScalars s, int first, const double* Qold, const double* Qnew,
                                                     double* bQ, double* bQo, double* bNlo, double* bNlq,
                                                     double* pgrad) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double da = 0;
  if (idx < g.ng) {
    int i, j, k;
    decompose(g, idx, i, j, k);
    const double mq2 = qx[i] * qx[i] + qy[j] * qy[j] + qz[k] * qz[k];
    const double sq = s.q02 - mq2;
    const double aLin = s.ep - s.alpha * (sq * sq);
    const double C1 = 2.0 - s.dt * s.rho_m * aLin, C2 = 1.5 - s.dt * s.rho_m * aLin;
    const double h = s.dtd2 * s.scale;
    const double bq = bQ[idx];
    double bnl = 3.0 * h / C2 * bq + bNlo[idx];
    if (first) bnl += -h / C2 * bq;  // REF:2170-2172: Nl_old = Nl at nLoop == 1
    bNlq[idx] = bnl;
    bNlo[idx] = first ? 0.0 : -h / C2 * bq;
    const double bqo_next = bQo[idx];
    bQo[idx] = -0.5 / C2 * bq;
    bQ[idx] = C1 / C2 * bq + bqo_next;
    // dC1/dalpha = dC2/dalpha = dt rho_m sq^2  =>  dQ'/dalpha = dt rho_m sq^2 (Q - Q') / C2
    da = bq * s.dt * s.rho_m * sq * sq * (Qold[idx] - Qnew[idx]) / C2;
  }
  block_accum(da, pgrad, PG_ALPHA);
}

// Transpose of dq = q . f-hat shifted (REF:2076-2078, subtracted from Nl-hat): f-hat_a
// at c receives -Vq_a[c+1] bar(Nlq) at c+1.
__global__ void __launch_bounds__(256) adj_dq_kernel(Grid g, const double* qx, const double* qy, const double* qz,
                                                     const double* bNlq, double* bfx, double* bfy, double* bfz) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.ng) return;
  int i, j, k;
  decompose(g, idx, i, j, k);
  const long long sx = 1LL << (g.ly + g.lz), sy = g.nz;
  bfx[idx] = (i + 1 < g.nx) ? -qx[i + 1] * bNlq[idx + sx] : 0.0;
  bfy[idx] = (j + 1 < g.ny) ? -qy[j + 1] * bNlq[idx + sy] : 0.0;
  bfz[idx] = (k + 1 < g.nz) ? -qz[k + 1] * bNlq[idx + 1] : 0.0;
}

// Transpose of the density update (REF:2121-2139) and of the real-space Nl
// (REF:2153-2160, grad.f handled by adj_dq_kernel):
//   S_rho = -v.grad rho - rho_in divv;  rho' = rho_in + dt (1.5 S_rho - 0.5 F);  F' = S_rho
//   Nl = -mu + c' (rho' - rho0 - kp A) psi - v.grad psi,  c' = kp zeta/(A + 0.001)
// rho_in: the density the forward step used (the relax reset rho0 + kp A, REF:1371,
// when relax is set). Outputs initialise the real-space cotangent buffers.
struct AdjNlArgs {
  const double *bNl, *psi, *A, *rho_in, *rho_new, *vx, *vy, *vz, *gpx, *gpy, *gpz, *grx, *gry, *grz, *divv;
  double *bR, *bF, *bmu, *bA, *bpsi, *bvx, *bvy, *bvz, *bgpx, *bgpy, *bgpz, *bgrx, *bgry, *bgrz, *bdivv;
  double* pgrad;
  AdjScalars s;
  int relax;
};
__global__ void __launch_bounds__(256) adj_nl_kernel(Grid g, AdjNlArgs a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double dkp = 0, drho0 = 0;
  if (idx < g.ng) {
    const double b = a.bNl[idx], psi = a.psi[idx], A = a.A[idx];
    const double rin = a.relax ? a.s.rho0 + a.s.kp * A : a.rho_in[idx];
    const double rn = a.rho_new[idx];
    const double den = A + 0.001;
    const double cp = a.s.kp * a.s.zeta / den;
    const double t2 = rn - a.s.rho0 - a.s.kp * A;
    const double brp = a.bR[idx] + cp * psi * b;  // bar rho'
    a.bmu[idx] = -b;
    a.bA[idx] = psi * b * (-a.s.kp * a.s.zeta * t2 / (den * den) - cp * a.s.kp);
    a.bpsi[idx] = cp * t2 * b;
    const double vx = a.vx[idx], vy = a.vy[idx], vz = a.vz[idx];
    const double bS = a.bF[idx] + 1.5 * a.s.dt * brp;  // bar S_rho
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
    a.bF[idx] = -0.5 * a.s.dt * brp;
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
struct AdjStokesArgs {
  const double *bvx, *bvy, *bvz, *bdq, *vsx_, *vsy_, *vsz_, *vix, *viy, *viz;
  double *bdotx, *bdoty, *bdotz, *bsx, *bsy, *bsz, *bgx, *bgy, *bgz;
  const double *vqx, *vqy, *vqz, *vsx, *vsy, *vsz, *gqx, *gqy, *gqz, *gsx, *gsy, *gsz;
  double scale, inv_nu, inv_lam2nu, nu, lam2nu;
  int block;
  double* pgrad;
};
__global__ void __launch_bounds__(256) adj_stokes1_kernel(Grid g, AdjStokesArgs a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double dnu = 0;
  if (idx < g.ng) {
    int i, j, k;
    decompose(g, idx, i, j, k);
    const long long sx = 1LL << (g.ly + g.lz), sy = g.nz;
    const double qxi = a.vqx[i], qyj = a.vqy[j], qzk = a.vqz[k];
    double d = 0, sd = 0, fp = 0;
    if (i < g.nx - 1) {
      const double s_ = a.vsx[i];
      const double inv = 1.0 / (s_ * s_ + qyj * qyj + qzk * qzk);
      const double CM1 = a.scale * inv, CM2 = s_ * inv, G = a.gsx[i] * a.gqy[j] * a.gqz[k];
      const double bvs = a.bvx[idx];
      const double bvi = bvs + a.vqx[i + 1] * a.bdq[idx + sx];
      d = -(CM1 * a.inv_nu) * CM2 * bvs + (CM1 * a.inv_lam2nu) * CM2 * G * bvi;
      sd = (CM1 * a.inv_nu) * bvs;
      fp = (CM1 * a.inv_lam2nu) * s_ * bvi;
      dnu += bvs * (-a.vsx_[idx] / a.nu) + bvi * (-2.0 * a.vix[idx] / a.lam2nu);
    }
    a.bdotx[idx] = d; a.bsx[idx] = sd; a.bgx[idx] = fp;
    double dy = 0, sdy = 0, fpy = 0, dz = 0, sdz = 0, fpz = 0;
    if (j < g.ny - 1 && k < g.nz - 1) {
      {
        const double s_ = a.vsy[j];
        const double inv = 1.0 / (qxi * qxi + s_ * s_ + qzk * qzk);
        const double CM1 = a.scale * inv, CM2 = s_ * inv, G = a.gqx[i] * a.gsy[j] * a.gqz[k];
        const double bvs = a.bvy[idx];
        const double bvi = bvs + a.vqy[j + 1] * a.bdq[idx + sy];
        dy = -(CM1 * a.inv_nu) * CM2 * bvs + (CM1 * a.inv_lam2nu) * CM2 * G * bvi;
        sdy = (CM1 * a.inv_nu) * bvs;
        fpy = (CM1 * a.inv_lam2nu) * s_ * bvi;
        dnu += bvs * (-a.vsy_[idx] / a.nu) + bvi * (-2.0 * a.viy[idx] / a.lam2nu);
      }
      {
        const double s_ = a.vsz[k];
        const double inv = 1.0 / (qxi * qxi + qyj * qyj + s_ * s_);
        const double CM1 = a.scale * inv, CM2 = s_ * inv;
        const bool q1 = (k == 0) && (j > 0) && (i % a.block != 0);  // REF:1932
        const double G = q1 ? (a.gqx[i] * a.gsy[j] * a.gqz[k]) : (a.gqx[i] * a.gqy[j] * a.gsz[k]);
        const double bvs = a.bvz[idx];
        const double bvi = bvs + a.vqz[k + 1] * a.bdq[idx + 1];
        dz = -(CM1 * a.inv_nu) * CM2 * bvs + (CM1 * a.inv_lam2nu) * CM2 * G * bvi;
        sdz = (CM1 * a.inv_nu) * bvs;
        fpz = (CM1 * a.inv_lam2nu) * s_ * bvi;
        dnu += bvs * (-a.vsz_[idx] / a.nu) + bvi * (-2.0 * a.viz[idx] / a.lam2nu);
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
struct AdjStokes2Args {
  const double *bdotx, *bdoty, *bdotz, *bsx, *bsy, *bsz, *bgx, *bgy, *bgz;
  double *bSx, *bSy, *bSz, *bfg, *bE;
  const double *vqx, *vqy, *vqz, *vsx, *vsy, *vsz, *gqx, *gqy, *gqz;
};
__global__ void __launch_bounds__(256) adj_stokes2_kernel(Grid g, AdjStokes2Args a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.ng) return;
  int i, j, k;
  decompose(g, idx, i, j, k);
  const long long sx = 1LL << (g.ly + g.lz), sy = g.nz;
  double Sx = a.bsx[idx] + a.vsx[i] * a.bdotx[idx];
  if (i + 1 < g.nx) {
    if (j >= 1) Sx += a.vqx[i + 1] * a.bdoty[idx + sx - sy];
    if (k >= 1) Sx += a.vqx[i + 1] * a.bdotz[idx + sx - 1];
  }
  double Sy = a.bsy[idx] + a.vsy[j] * a.bdoty[idx];
  if (j + 1 < g.ny) {
    if (i >= 1) Sy += a.vqy[j + 1] * a.bdotx[idx - sx + sy];
    if (k >= 1) Sy += a.vqy[j + 1] * a.bdotz[idx + sy - 1];
  }
  double Sz = a.bsz[idx] + a.vsz[k] * a.bdotz[idx];
  if (k + 1 < g.nz) {
    if (i >= 1) Sz += a.vqz[k + 1] * a.bdotx[idx - sx + 1];
    if (j >= 1) Sz += a.vqz[k + 1] * a.bdoty[idx - sy + 1];
  }
  a.bSx[idx] = Sx;
  a.bSy[idx] = Sy;
  a.bSz[idx] = Sz;
  double fg = 0;
  if (i >= 1) fg += a.bgx[idx - sx];
  if (j >= 1) fg += a.bgy[idx - sy];
  if (k >= 1) fg += a.bgz[idx - 1];
  a.bfg[idx] = fg;
  a.bE[idx] = fg * (a.gqx[i] * a.gqy[j] * a.gqz[k]);
}

// Transpose of S6 (REF:1385-1425) and of the relax reset (REF:1371-1374):
//   E = L^2/2, t = rho0 + kp A, fgrad = zeta/2 (rho^2 - t^2), mu1 = lapR + rho L,
//   S_a = mu1 gpsi_a + E grho_a, mu = lapR + rho P5, P5 = L - ep psi - beta psi^3 + gamma psi^5,
//   Erho = rho E, c = kp zeta (rho - t)/(A + 0.001), f_a = c gpsi_a;
//   relax: rho = rho0 + kp A and lapR = rho lapR_raw.
// bR enters holding bar rho_in from adj_nl_kernel and leaves holding the cotangent
// of the step's incoming density (zero in the relax phase, whose rho is reset).
struct AdjS6Args {
  const double *bfgrad, *bE, *bSx, *bSy, *bSz, *bfx, *bfy, *bfz, *bmu;
  const double *lapR, *rho_in, *L, *psi, *A, *gpx, *gpy, *gpz, *grx, *gry, *grz;
  double *bgpx, *bgpy, *bgpz, *bgrx, *bgry, *bgrz, *bA, *bpsi, *bR, *blapR, *bL;
  double* pgrad;
  AdjScalars s;
  int relax;
};
__global__ void __launch_bounds__(256) adj_s6_kernel(Grid g, AdjS6Args a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double dbeta = 0, dgamma = 0, drho0 = 0, dkp = 0;
  if (idx < g.ng) {
    const double A = a.A[idx], L = a.L[idx], psi = a.psi[idx];
    const double rho = a.relax ? a.s.rho0 + a.s.kp * A : a.rho_in[idx];
    const double lraw = a.lapR[idx];
    const double lapR = a.relax ? rho * lraw : lraw;
    const double gpx = a.gpx[idx], gpy = a.gpy[idx], gpz = a.gpz[idx];
    const double grx = a.grx[idx], gry = a.gry[idx], grz = a.grz[idx];
    const double E = 0.5 * (L * L), t = a.s.rho0 + a.s.kp * A, den = A + 0.001;
    const double mu1 = lapR + rho * L;
    const double c = a.s.kp * a.s.zeta * (rho - t) / den;
    const double p2 = psi * psi;
    const double P5 = L - a.s.ep * psi - a.s.beta * (p2 * psi) + a.s.gamma * (p2 * p2 * psi);
    const double bSx = a.bSx[idx], bSy = a.bSy[idx], bSz = a.bSz[idx];
    const double bfx = a.bfx[idx], bfy = a.bfy[idx], bfz = a.bfz[idx];
    const double bmu = a.bmu[idx], bfg = a.bfgrad[idx], bEr = a.bE[idx];
    const double bmu1 = bSx * gpx + bSy * gpy + bSz * gpz;
    a.bgpx[idx] += mu1 * bSx + c * bfx;
    a.bgpy[idx] += mu1 * bSy + c * bfy;
    a.bgpz[idx] += mu1 * bSz + c * bfz;
    const double bEn = bSx * grx + bSy * gry + bSz * grz + rho * bEr;
    a.bgrx[idx] += E * bSx;
    a.bgry[idx] += E * bSy;
    a.bgrz[idx] += E * bSz;
    const double bc = bfx * gpx + bfy * gpy + bfz * gpz;
    const double blap = bmu1 + bmu;
    double brho = L * bmu1 + P5 * bmu + E * bEr + a.s.zeta * rho * bfg + (a.s.kp * a.s.zeta / den) * bc;
    a.bL[idx] = rho * bmu1 + rho * bmu + L * bEn;
    a.bpsi[idx] += rho * (-a.s.ep - 3.0 * a.s.beta * p2 + 5.0 * a.s.gamma * (p2 * p2)) * bmu;
    const double bt = -a.s.zeta * t * bfg - (a.s.kp * a.s.zeta / den) * bc;
    double bA = a.s.kp * bt + bc * (-a.s.kp * a.s.zeta * (rho - t) / (den * den));
    dkp = bt * A + bc * a.s.zeta * (rho - t) / den;
    drho0 = bt;
    dbeta = bmu * rho * (-(p2 * psi));
    dgamma = bmu * rho * (p2 * p2 * psi);
    if (a.relax) {
      brho += lraw * blap;
      a.blapR[idx] = rho * blap;
      const double bri = brho + a.bR[idx];  // every use of the reset density
      bA += a.s.kp * bri;
      dkp += A * bri;
      drho0 += bri;
      a.bR[idx] = 0.0;
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
__global__ void __launch_bounds__(256) adj_acc_spec_kernel(Grid g, const double* qx, const double* qy,
                                                           const double* qz, int mode, double alpha, double q02,
                                                           const double* Y, const double* Q, double* bQ,
                                                           double* pgrad) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double da = 0;
  if (idx < g.ng) {
    int i, j, k;
    decompose(g, idx, i, j, k);
    const double mq2 = qx[i] * qx[i] + qy[j] * qy[j] + qz[k] * qz[k];
    const double dl = mode == 0 ? (q02 - mq2) : -mq2 * (q02 - mq2);  // dLambda/dalpha
    const double y = Y[idx];
    bQ[idx] += alpha * dl * y;
    da = y * dl * Q[idx];
  }
  block_accum(da, pgrad, PG_ALPHA);
}

// out = a * x (+ b * y): small helper for the final dL/dpsi0 = scale C2^T (bQ + bQo).
__global__ void __launch_bounds__(256) axpby_kernel(long long n, double a, const double* x, double b, const double* y,
                                                    double* out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) out[idx] = a * x[idx] + (y ? b * y[idx] : 0.0);
}

}  // namespace swc
