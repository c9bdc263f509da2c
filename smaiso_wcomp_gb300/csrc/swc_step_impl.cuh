// swc_step_impl.cuh -- the time step of smaiso-wcomp.cpp (loop body REF:1084-2198,
// diagnostics REF:2202-2262) as a sequence of sm_103a kernels, templated on the work
// precision T. The state that carries the scheme's stability and conservation --
// psiq, psiq_old (the CN/AB2 psi update), rho and its AB2 source f_rho -- is FP64 in
// both engines; the FP64 engine (T = double) computes everything else in FP64 too,
// the mixed engine (T = float) runs transforms and pointwise terms in FP32.
//
// Reorganisation relative to the reference (same mathematics, FP64 rounding only):
//  * v = vsol + virr is transformed once per component (REF:2093-2117 transforms
//    vsol and virr separately and only their sums enter REF:2128-2160); vsol alone
//    is transformed on the last step of a swc_step call, for output.
//  * grad.f (ampDgradpsi, REF:2078, 2090) enters Nl only, which is transformed back
//    by DCT-II (REF:2167); DCT-II^3 o DCT-III^3 = (1/scale) I, so the spectral
//    divergence is subtracted from the transformed Nl instead of transforming twice.
//  * the Gaussian factor exp(-1.57^2 2 |q|^2) (REF:1281, 1486, 1603...) is the product
//    of three per-axis tables; CM1/CM2 are recomputed from the wavenumbers instead
//    of being read from nine N^3 tables (REF:936-963).
//  * a forward transform, a spectral multiplier and an inverse transform along the
//    last axis are one "filter" pass (S3 amplitude filter, S5 Laplacian).
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <thread>
#include <vector>

#include "swc_engine.h"
#include "swc_r2r.cuh"
#include "swc_fpconv.h"
#include "swc_tables.cuh"

namespace swc {

#define SWC_CK(call)                                                                      \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return SWC_ERR_CUDA;                                                                \
    }                                                                                     \
  } while (0)

// ---------------------------------------------------------------------------------
// Load / store / multiplier functors fused into the transform passes
// ---------------------------------------------------------------------------------

// Multiplier of the derivative pass (shifted spectral derivative onto the sine grid
// of `axis`, REF:1166-1221): -c Vs[c_axis], c = 1/(2 n_axis); the pass itself applies
// the shift and the zero on the last mode.
// a / b of the FP64 terms by rcp_f64's Newton-Raphson reciprocal (1/b within an ulp,
// the quotient within 1.5 ulp of the division, in fewer FP64 operations on GB300's slow
// FP64 pipe); FP32 keeps the division.
template <typename T> __device__ __forceinline__ T div_nr(T a, T b) {
  if constexpr (sizeof(T) == 8) return a * rcp_f64(b);
  else return a / b;
}

template <typename T> struct MulDeriv {
  const T* vs;
  T c;
  int axis;
  __device__ __forceinline__ T operator()(int i, int j, int k) const {
    return -c * vs[axis == 0 ? i : (axis == 1 ? j : k)];
  }
};

// |psi| amplitude before filtering (REF:1262-1266).
template <typename T> struct LdAmp {
  const T *psi, *gx, *gy, *gz;
  T q02;
  __device__ __forceinline__ T operator()(int, int, int, long long idx) const {
    const T p = psi[idx], a = gx[idx], b = gy[idx], c = gz[idx];
    return sqrt(q02 * (p * p) + (a * a) + (b * b) + (c * c));
  }
  __device__ __forceinline__ float4 quad(int, int, int, long long idx) const {
    const float4 p = ld4v(psi, idx), a = ld4v(gx, idx), b = ld4v(gy, idx), c = ld4v(gz, idx);
    auto f = [&](float p_, float a_, float b_, float c_) {
      return sqrtf((float)q02 * (p_ * p_) + (a_ * a_) + (b_ * b_) + (c_ * c_));
    };
    return make_float4(f(p.x, a.x, b.x, c.x), f(p.y, a.y, b.y, c.y), f(p.z, a.z, b.z, c.z), f(p.w, a.w, b.w, c.w));
  }
};

// scale * exp(-1.57^2 * 2 * |q|^2) as a product of per-axis tables (REF:1280-1281).
template <typename T> struct MulGauss {
  const T *gx, *gy, *gz;
  T scale;
  __device__ __forceinline__ T operator()(int i, int j, int k) const { return scale * gx[i] * gy[j] * gz[k]; }
};

// One axis's factor of that product, times a constant: the filter pass along axis AX
// of the mixed engine's separable Gaussian (the three one-axis filter passes multiply
// out to MulGauss: the DCT-III DCT-II pairs give 2n per axis, 8 N^3 in all, which the
// scale of the last one cancels).
template <typename T, int AX> struct MulAxis {
  const T* g;
  T scale;
  __device__ __forceinline__ T operator()(int i, int j, int k) const {
    return scale * g[AX == 0 ? i : (AX == 1 ? j : k)];
  }
};

// -scale * |q|^2 (REF:1333-1334).
template <typename T> struct MulLap {
  const T *qx, *qy, *qz;
  T scale;
  __device__ __forceinline__ T operator()(int i, int j, int k) const {
    const T a = qx[i], b = qy[j], c = qz[k];
    return -scale * ((a * a) + (b * b) + (c * c));
  }
};

// FP64 engine: alpha (q0^2 - |q|^2) psiq (REF:1302), on the FP64 state.
template <typename T> struct LdLpsi {
  const double* psiq;
  const T *qx, *qy, *qz;
  T alpha, q02;
  __device__ __forceinline__ T operator()(int i, int j, int k, long long idx) const {
    const T a = qx[i], b = qy[j], c = qz[k];
    const T mq2 = (a * a) + (b * b) + (c * c);
    return alpha * (q02 - mq2) * (T)psiq[idx];
  }
};

// FP64 engine, relax phase: -|q|^2 alpha (q0^2 - |q|^2) psiq (REF:1356-1357).
template <typename T> struct LdRelaxLap {
  const double* psiq;
  const T *qx, *qy, *qz;
  T alpha, q02;
  __device__ __forceinline__ T operator()(int i, int j, int k, long long idx) const {
    const T a = qx[i], b = qy[j], c = qz[k];
    const T mq2 = (a * a) + (b * b) + (c * c);
    return -mq2 * alpha * (q02 - mq2) * (T)psiq[idx];
  }
};

// alpha (q0^2 - |q|^2) (REF:1302) and, RELAX, the relax phase's -|q|^2 alpha (q0^2 - |q|^2)
// (REF:1356-1357): the multipliers of the mixed engine's FP32 psiq copy (LdMul), which
// keep the first pass of these inverse transforms on the TMA pipeline.
template <int RELAX> struct LapMul {
  const float *qx, *qy, *qz;
  float alpha, q02;
  __device__ __forceinline__ float operator()(int i, int j, int k) const {
    const float mq2 = (qx[i] * qx[i] + qy[j] * qy[j]) + qz[k] * qz[k];
    const float m = alpha * (q02 - mq2);
    return RELAX ? -mq2 * m : m;
  }
};

// Last pass of dfDlapPsi in the mixed engine's normal phase: stores dfDlapPsi and
// rho * dfDlapPsi (REF:1321, with rho = rhof + off), so the Delta(rho L) transform
// starts with a plain TMA-fed pass. rhof is not written by the pass: its loads take
// the read-only path, so they need not wait for the stores issued before them.
struct StLpsiRhoL {
  float *lpsi, *rhoL;
  const float* rhof;
  float off;
  __device__ __forceinline__ void operator()(int, int, int, long long idx, float v) const {
    const float r = __ldg(rhof + idx);
    lpsi[idx] = v;
    rhoL[idx] = (r + off) * v;
  }
  __device__ __forceinline__ void pair(int, int, int, long long idx, float2 v) const {
    const float2 r = ld2g(rhof, idx);
    st2v(lpsi, idx, v);
    st2v(rhoL, idx, make_float2((r.x + off) * v.x, (r.y + off) * v.y));
  }
  __device__ __forceinline__ void quad(int, int, int, long long idx, float4 v) const {
    const float4 r = ld4g(rhof, idx);
    st4v(lpsi, idx, v);
    st4v(rhoL, idx, make_float4((r.x + off) * v.x, (r.y + off) * v.y, (r.z + off) * v.z, (r.w + off) * v.w));
  }
};

// FP64 engine: rho * dfDlapPsi (REF:1321).
template <typename T> struct LdRhoL {
  const double* rho;
  const T* lpsi;
  T off;
  __device__ __forceinline__ T operator()(int, int, int, long long idx) const {
    return ((T)rho[idx] + off) * lpsi[idx];
  }
};

// rho - c: the gradients (REF:1191-1219) never read mode 0, so a constant offset
// keeps them unchanged while the FP32 transform resolves the small variations.
template <typename T> struct LdOffset {
  const double* p;
  double c;
  __device__ __forceinline__ T operator()(int, int, int, long long idx) const { return (T)(p[idx] - c); }
  __device__ __forceinline__ float2 pair(int, int, int, long long idx) const {
    const double2 d = *reinterpret_cast<const double2*>(p + idx);
    return make_float2((float)(d.x - c), (float)(d.y - c));
  }
  __device__ __forceinline__ float4 quad(int, int, int, long long idx) const {
    const double2 d0 = *reinterpret_cast<const double2*>(p + idx);
    const double2 d1 = *reinterpret_cast<const double2*>(p + idx + 2);
    return make_float4((float)(d0.x - c), (float)(d0.y - c), (float)(d1.x - c), (float)(d1.y - c));
  }
};

// First pass of the Nl transform: density AB2 update (REF:2121-2139) and the real
// space Nl of REF:2153-2160 without the grad.f term (subtracted in spectral space).
template <typename T> struct LdNl {
  const T *vx, *vy, *vz, *grx, *gry, *grz, *divv, *mu, *amp, *psi, *gpx, *gpy, *gpz;
  double *rho, *frho;
  double dt, kp, zeta, rho0;
  __device__ __forceinline__ T operator()(int, int, int, long long idx) const {
    const T ux = vx[idx], uy = vy[idx], uz = vz[idx];
    const double r = rho[idx];
    const T srho = -ux * grx[idx] - uy * gry[idx] - uz * grz[idx] - (T)r * divv[idx];
    const double rn = r + dt * (1.5 * (double)srho - 0.5 * frho[idx]);
    rho[idx] = rn;
    frho[idx] = (double)srho;
    const T a = amp[idx];
    const T c = div_nr((T)kp * (T)zeta, a + (T)0.001) * ((T)rn - (T)rho0 - (T)kp * a) * psi[idx];
    return -mu[idx] + c - ux * gpx[idx] - uy * gpy[idx] - uz * gpz[idx];
  }
  // four consecutive elements with 16-byte loads / stores (FP32 fields, FP64 rho, f_rho);
  // each element is read, then written, by this thread only: read-only-path loads
  __device__ __forceinline__ float4 quad(int, int, int, long long idx) const {
    const float4 ux = ld4g(vx, idx), uy = ld4g(vy, idx), uz = ld4g(vz, idx);
    const float4 gx = ld4g(grx, idx), gy = ld4g(gry, idx), gz = ld4g(grz, idx), dv = ld4g(divv, idx);
    const float4 m = ld4g(mu, idx), am = ld4g(amp, idx), ps = ld4g(psi, idx);
    const float4 px = ld4g(gpx, idx), py = ld4g(gpy, idx), pz = ld4g(gpz, idx);
    const double2 r01 = ld2dg(rho, idx), r23 = ld2dg(rho, idx + 2);
    const double2 f01 = ld2dg(frho, idx), f23 = ld2dg(frho, idx + 2);
    double rn[4], sr[4];
    const float ux_[4] = {ux.x, ux.y, ux.z, ux.w}, uy_[4] = {uy.x, uy.y, uy.z, uy.w}, uz_[4] = {uz.x, uz.y, uz.z, uz.w};
    const float gx_[4] = {gx.x, gx.y, gx.z, gx.w}, gy_[4] = {gy.x, gy.y, gy.z, gy.w}, gz_[4] = {gz.x, gz.y, gz.z, gz.w};
    const float dv_[4] = {dv.x, dv.y, dv.z, dv.w}, m_[4] = {m.x, m.y, m.z, m.w}, am_[4] = {am.x, am.y, am.z, am.w};
    const float ps_[4] = {ps.x, ps.y, ps.z, ps.w}, px_[4] = {px.x, px.y, px.z, px.w};
    const float py_[4] = {py.x, py.y, py.z, py.w}, pz_[4] = {pz.x, pz.y, pz.z, pz.w};
    const double r_[4] = {r01.x, r01.y, r23.x, r23.y}, f_[4] = {f01.x, f01.y, f23.x, f23.y};
    float out[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float srho = -ux_[c] * gx_[c] - uy_[c] * gy_[c] - uz_[c] * gz_[c] - (float)r_[c] * dv_[c];
      rn[c] = r_[c] + dt * (1.5 * (double)srho - 0.5 * f_[c]);
      sr[c] = (double)srho;
      const float a = am_[c];
      const float cc = ((float)kp * (float)zeta / (a + 0.001f)) * ((float)rn[c] - (float)rho0 - (float)kp * a) * ps_[c];
      out[c] = -m_[c] + cc - ux_[c] * px_[c] - uy_[c] * py_[c] - uz_[c] * pz_[c];
    }
    *reinterpret_cast<double2*>(rho + idx) = make_double2(rn[0], rn[1]);
    *reinterpret_cast<double2*>(rho + idx + 2) = make_double2(rn[2], rn[3]);
    *reinterpret_cast<double2*>(frho + idx) = make_double2(sr[0], sr[1]);
    *reinterpret_cast<double2*>(frho + idx + 2) = make_double2(sr[2], sr[3]);
    return make_float4(out[0], out[1], out[2], out[3]);
  }
};

// Mixed engine, first pass of the Nl transform: the density AB2 update and Nl of LdNl
// with the FP32 terms in FP32 and FP64 only where the state is. rho_new = rho +
// (double) dt (1.5 s - 0.5 f_rho) is one FP64 add; f_rho is stored in FP32 (it is the
// FP32 source s of the previous step); the FP32 copy rhof = rho - off is refreshed from
// the FP64 sum, and rho = rhof + off is the FP32 density of the FP32 terms. The
// conversions run on the integer pipes (swc_fpconv.h): two FP64 adds per point remain.
struct LdNlMixed {
  const float *vx, *vy, *vz, *grx, *gry, *grz, *divv, *mu, *amp, *psi, *gpx, *gpy, *gpz;
  double* rho;
  float *frho, *rhof;
  double offd;
  float dt, kp, zeta, rho0, off;
  const float *mdfx, *mdfy, *mdfz;  // -grad.f in real space by component (REF:2078-2090, the
                                     // transposed-derivative passes): Nl += their sum
  __device__ __forceinline__ float point(float ux, float uy, float uz, float gx, float gy, float gz, float dv,
                                         float m, float a, float ps, float px, float py, float pz, float rf,
                                         float fp, double& r, float& s, float& rfn) const {
    s = -ux * gx - uy * gy - uz * gz - (rf + off) * dv;
    const float inc = dt * (1.5f * s - 0.5f * fp);
    r = r + widen_f32(inc);
    rfn = narrow_f64(r - offd);
    const float c = (kp * zeta / (a + 0.001f)) * ((rfn + off) - rho0 - kp * a) * ps;
    return -m + c - ux * px - uy * py - uz * pz;
  }
  __device__ __forceinline__ float operator()(int, int, int, long long idx) const {
    double r = rho[idx];
    float sr, rfn;
    const float out = point(vx[idx], vy[idx], vz[idx], grx[idx], gry[idx], grz[idx], divv[idx], mu[idx], amp[idx],
                            psi[idx], gpx[idx], gpy[idx], gpz[idx], rhof[idx], frho[idx], r, sr, rfn);
    rho[idx] = r;
    frho[idx] = sr;
    rhof[idx] = rfn;
    return out + ((mdfx[idx] + mdfy[idx]) + mdfz[idx]);
  }
  // four consecutive elements; each read, then written, by this thread only
  __device__ __forceinline__ float4 quad(int, int, int, long long idx) const {
    const float4 ux = ld4g(vx, idx), uy = ld4g(vy, idx), uz = ld4g(vz, idx);
    const float4 gx = ld4g(grx, idx), gy = ld4g(gry, idx), gz = ld4g(grz, idx), dv = ld4g(divv, idx);
    const float4 m = ld4g(mu, idx), am = ld4g(amp, idx), ps = ld4g(psi, idx);
    const float4 px = ld4g(gpx, idx), py = ld4g(gpy, idx), pz = ld4g(gpz, idx);
    const float4 rf = ld4g(rhof, idx), fp = ld4g(frho, idx);
    const double2 r01 = ld2dg(rho, idx), r23 = ld2dg(rho, idx + 2);
    double r[4] = {r01.x, r01.y, r23.x, r23.y};
    float sr[4], rfn[4], o[4];
    o[0] = point(ux.x, uy.x, uz.x, gx.x, gy.x, gz.x, dv.x, m.x, am.x, ps.x, px.x, py.x, pz.x, rf.x, fp.x, r[0], sr[0], rfn[0]);
    o[1] = point(ux.y, uy.y, uz.y, gx.y, gy.y, gz.y, dv.y, m.y, am.y, ps.y, px.y, py.y, pz.y, rf.y, fp.y, r[1], sr[1], rfn[1]);
    o[2] = point(ux.z, uy.z, uz.z, gx.z, gy.z, gz.z, dv.z, m.z, am.z, ps.z, px.z, py.z, pz.z, rf.z, fp.z, r[2], sr[2], rfn[2]);
    o[3] = point(ux.w, uy.w, uz.w, gx.w, gy.w, gz.w, dv.w, m.w, am.w, ps.w, px.w, py.w, pz.w, rf.w, fp.w, r[3], sr[3], rfn[3]);
    *reinterpret_cast<double2*>(rho + idx) = make_double2(r[0], r[1]);
    *reinterpret_cast<double2*>(rho + idx + 2) = make_double2(r[2], r[3]);
    st4v(frho, idx, make_float4(sr[0], sr[1], sr[2], sr[3]));
    st4v(rhof, idx, make_float4(rfn[0], rfn[1], rfn[2], rfn[3]));
    const float4 dx = ld4g(mdfx, idx), dy = ld4g(mdfy, idx), dz = ld4g(mdfz, idx);
    return make_float4(o[0] + ((dx.x + dy.x) + dz.x), o[1] + ((dx.y + dy.y) + dz.y), o[2] + ((dx.z + dy.z) + dz.z),
                       o[3] + ((dx.w + dy.w) + dz.w));
  }
};

// Last pass of the Nl transform: Nlq = DCT(Nl) - q.f, then the CN/AB2 update of psiq
// (REF:2170-2190), the FP64 engine's form: the reference's expression with C1, C2
// evaluated per mode (the mixed engine's increment form is LdNlUpdate below).
template <typename T> struct StNlUpdate {
  const T* dq;
  double *psiq, *psiq_old;
  T* nlq;
  const double *qx, *qy, *qz;
  double ep, alpha, q02, dt, rho_m, dtd2, scale;
  int first;
  __device__ __forceinline__ void operator()(int i, int j, int k, long long idx, T v) const {
    const T nl = v - dq[idx];
    const T nlo = first ? nl : nlq[idx];
    const double pq = psiq[idx], pqo = psiq_old[idx];
    const double src = dtd2 * scale * (3.0 * (double)nl - (double)nlo);
    const double a = qx[i], b = qy[j], c = qz[k];
    const double mq2 = a * a + b * b + c * c;
    const double s = q02 - mq2;
    const double aLin = ep - alpha * (s * s);
    const double C1 = (2.0 - dt * rho_m * aLin);
    const double C2 = (1.5 - dt * rho_m * aLin);
    const double pn = (C1 * pq - 0.5 * pqo + src) / C2;
    psiq_old[idx] = pq;
    psiq[idx] = pn;
    nlq[idx] = nl;
  }
  // elements idx, idx + 1 (x/y passes: (i, j, k), (i, j, k + 1)) with vector accesses;
  // each element is read, then written, by this thread only: read-only-path loads
  __device__ __forceinline__ void pair(int i, int j, int k, long long idx, float2 v) const {
    const float2 d = ld2g(dq, idx);
    const float nl0 = v.x - d.x, nl1 = v.y - d.y;
    float nlo0 = nl0, nlo1 = nl1;
    if (!first) {
      const float2 o = ld2g(nlq, idx);
      nlo0 = o.x;
      nlo1 = o.y;
    }
    const double2 pq = ld2dg(psiq, idx);
    const double2 pqo = ld2dg(psiq_old, idx);
    const double s0 = dtd2 * scale * (3.0 * (double)nl0 - (double)nlo0);
    const double s1 = dtd2 * scale * (3.0 * (double)nl1 - (double)nlo1);
    const double ab = qx[i] * qx[i] + qy[j] * qy[j];
    auto upd = [&](double cz, double p, double po, double src) {
      const double s = q02 - (ab + cz * cz);
      const double aLin = ep - alpha * (s * s);
      return div_nr((2.0 - dt * rho_m * aLin) * p - 0.5 * po + src, 1.5 - dt * rho_m * aLin);
    };
    const double pn0 = upd(qz[k], pq.x, pqo.x, s0);
    const double pn1 = upd(qz[k + 1], pq.y, pqo.y, s1);
    *reinterpret_cast<double2*>(psiq_old + idx) = pq;
    *reinterpret_cast<double2*>(psiq + idx) = make_double2(pn0, pn1);
    st2v(nlq, idx, make_float2(nl0, nl1));
  }
};

// Mixed engine: the CN/AB2 update of psiq (REF:2170-2190) in increment form, applied by
// nl_update_kernel before the first pass of psi = DCT-III^3 psiq_new (REF:2194-2197),
// which reads the FP32 copy psiqf. It reads the Nl transform's output nl_hat and Nl_old,
// psiq and psiq_old, writes the new psiq and psiqf. The increment (0.5 (psiq - psiq_old)
// + dt/2 scale (3 Nl - Nl_old))/C2, a small correction built from FP32 data, is formed in
// FP32 with 1/C2 evaluated in FP32 from the FP32 wavenumbers (C2 = 1.5 - dt rho_m
// (ep - alpha (q0^2 - |q|^2)^2), REF:957-958); FP64 holds the state: two FP64 adds per
// point (psiq - psiq_old, psiq + increment), conversions on the integer pipes. The k = 0
// mode and the modes near the q0 shell whose denominator differs from 1.5 by less than
// FP32 resolves (|1.5 - C2| < 8 eps_32 1.5) form the increment in FP64 with C2 evaluated
// in FP64.
struct LdNlUpdate {
  const float *nlw, *dq;
  const float* nlq;
  double *psiq, *psiq_old;
  const float *qxf, *qyf, *qzf;  // FP32 wavenumbers
  float q02f, epf, alphaf, dtrmf;
  float* psiqf;
  float srcs;  // dt/2 scale
  int first;
  Grid g;
  const double *qx, *qy, *qz;        // FP64 wavenumbers of the flagged modes' C2
  double ep, alpha, q02, dtrm, srcs_d;  // dtrm = dt rho_m, srcs_d = dt/2 scale
  __device__ __forceinline__ float point(float nl, float nlo, double pq, double pqo, float ic, double& pn,
                                         long long idx) const {
    if (ic < 0.0f) {  // flagged mode: FP64 increment, FP64 C2 (REF:957-958)
      const int k = (int)(idx & (g.nz - 1)), j = (int)((idx >> g.lz) & (g.ny - 1)), i = (int)(idx >> (g.ly + g.lz));
      const double s = q02 - (qx[i] * qx[i] + qy[j] * qy[j] + qz[k] * qz[k]);
      const double c2 = 1.5 - dtrm * (ep - alpha * (s * s));
      pn = pq + (0.5 * (pq - pqo) + srcs_d * (3.0 * (double)nl - (double)nlo)) / c2;
      return narrow_f64(pn);
    }
    const float inc = (0.5f * narrow_f64(pq - pqo) + srcs * (3.0f * nl - nlo)) * ic;
    pn = pq + widen_f32(inc);
    return narrow_f64(pn);
  }
  // 1/C2 of mode (i, j, k), negative for the modes that take the FP64 increment
  __device__ __forceinline__ float inv_c2(float mq2, bool zero_mode) const {
    const float s = q02f - mq2;
    const float damp = dtrmf * (epf - alphaf * (s * s));
    const float ic = 1.0f / (1.5f - damp);
    return (zero_mode || -damp < 8.0f * 1.1920928955078125e-7f * 1.5f) ? -ic : ic;
  }
  // four consecutive elements; each read, then written, by this thread only
  __device__ __forceinline__ float4 quad(int, int, int, long long idx) const {
    const float4 w = ld4g(nlw, idx);
    float4 ic;
    {
      const int k = (int)(idx & (g.nz - 1)), j = (int)((idx >> g.lz) & (g.ny - 1)), i = (int)(idx >> (g.ly + g.lz));
      const float qxy = qxf[i] * qxf[i] + qyf[j] * qyf[j];
      const float4 qz = ld4g(qzf, k);
      ic = make_float4(inv_c2(qxy + qz.x * qz.x, idx == 0), inv_c2(qxy + qz.y * qz.y, false),
                       inv_c2(qxy + qz.z * qz.z, false), inv_c2(qxy + qz.w * qz.w, false));
    }
    const float4 d = dq ? ld4g(dq, idx) : make_float4(0.f, 0.f, 0.f, 0.f);  // null (always): grad.f is in Nl
    const float nl[4] = {w.x - d.x, w.y - d.y, w.z - d.z, w.w - d.w};
    float nlo[4] = {nl[0], nl[1], nl[2], nl[3]};
    if (!first) {
      const float4 o = ld4g(nlq, idx);
      nlo[0] = o.x; nlo[1] = o.y; nlo[2] = o.z; nlo[3] = o.w;
    }
    const double2 p01 = ld2dg(psiq, idx), p23 = ld2dg(psiq, idx + 2);
    const double2 o01 = ld2dg(psiq_old, idx), o23 = ld2dg(psiq_old, idx + 2);
    double pn[4];
    float pf[4];
    pf[0] = point(nl[0], nlo[0], p01.x, o01.x, ic.x, pn[0], idx);
    pf[1] = point(nl[1], nlo[1], p01.y, o01.y, ic.y, pn[1], idx + 1);
    pf[2] = point(nl[2], nlo[2], p23.x, o23.x, ic.z, pn[2], idx + 2);
    pf[3] = point(nl[3], nlo[3], p23.y, o23.y, ic.w, pn[3], idx + 3);
    // the new psiq over psiq_old: the engine then exchanges the two buffers (and Nl-hat's
    // buffer with Nl_old's, Nl = Nl-hat here), so neither old value is copied
    *reinterpret_cast<double2*>(psiq_old + idx) = make_double2(pn[0], pn[1]);
    *reinterpret_cast<double2*>(psiq_old + idx + 2) = make_double2(pn[2], pn[3]);
    const float4 out = make_float4(pf[0], pf[1], pf[2], pf[3]);
    st4v(psiqf, idx, out);
    return out;
  }
};

// ---------------------------------------------------------------------------------
// Pointwise kernels
// ---------------------------------------------------------------------------------

// The mixed engine's CN/AB2 update (REF:2177-2190), four points per thread: the new psiq
// = psiq + FP32 increment into psiq_old's buffer, and its FP32 copy psiqf that the inverse
// transform then reads. The engine exchanges psiq_ with psiq_old_ and nlw_ with nlq_
// after the step (StepEngine::run_graph): psiq_old <- psiq and Nl_old <- Nl without copies.
static __global__ void __launch_bounds__(256) nl_update_kernel(long long n, LdNlUpdate lu) {
  const long long idx = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  if (idx < n) (void)lu.quad(0, 0, 0, idx);
}

// |psi, grad psi| (REF:1262-1266) of the mixed engine, four points per thread, ahead of
// the TMA-fed z pass that starts its transform: the 5-field streaming step runs at the
// HBM rate on its own, and the z pass, walking down the planes, starts on the ones
// still in L2.
static __global__ void __launch_bounds__(256) amp_kernel(long long n, LdAmp<float> la, float* out) {
  const long long idx = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  if (idx < n) st4v(out, idx, la.quad(0, 0, 0, idx));
}

__device__ __forceinline__ void decompose(const Grid& g, long long idx, int& i, int& j, int& k) {
  k = (int)(idx & (g.nz - 1));
  j = (int)((idx >> g.lz) & (g.ny - 1));
  i = (int)(idx >> (g.ly + g.lz));
}

// S5 relax tail + S6 (REF:1363-1425): stresses, chemical potential, forces.
template <typename T> struct S6Args {
  const T *lapR, *lpsi, *psi, *amp, *gpx, *gpy, *gpz, *grx, *gry, *grz;
  double* rho;
  T *fgrad, *ener, *Sx, *Sy, *Sz, *fx, *fy, *fz, *mu;
  double ep, beta, gamma, zeta, kp, rho0, amp_eq;
  int relax;
  T* rhof;      // mixed engine: FP32 copy rho - off (read; written in the relax phase); FP64: null
  double off;
  T rho0_t, kp_t, zeta_t, ep_t, beta_t, gamma_t, off_t;  // the coefficients in T, converted on the host
};

// FP64 -> FP32 copy (integer-pipe rounding), four elements per thread (n a multiple of 4).
static __global__ void __launch_bounds__(256) narrow_kernel(const double* src, float* dst, long long n) {
  const long long i = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= n) return;
  const double2 a = *reinterpret_cast<const double2*>(src + i), b = *reinterpret_cast<const double2*>(src + i + 2);
  *reinterpret_cast<float4*>(dst + i) = make_float4(narrow_f64(a.x), narrow_f64(a.y), narrow_f64(b.x), narrow_f64(b.y));
}

// FP32 -> FP64 copy, four elements per thread (n a multiple of 4).
static __global__ void __launch_bounds__(256) widen_kernel(const float* src, double* dst, long long n) {
  const long long i = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= n) return;
  const float4 v = *reinterpret_cast<const float4*>(src + i);
  *reinterpret_cast<double2*>(dst + i) = make_double2(v.x, v.y);
  *reinterpret_cast<double2*>(dst + i + 2) = make_double2(v.z, v.w);
}

// Mixed engine: the FP32 copies of the FP64 state, rhof = rho - off and psiqf = psiq,
// and the FP32 f_rho from its FP64 form (or zero; frhot null: left as it is).
static __global__ void __launch_bounds__(256) mixed_copies_kernel(long long n, const double* rho, const double* psiq,
                                                                  const double* frho, double off, float* rhof,
                                                                  float* psiqf, float* frhot) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    rhof[i] = narrow_f64(rho[i] - off);
    psiqf[i] = narrow_f64(psiq[i]);
    if (frhot) frhot[i] = frho ? narrow_f64(frho[i]) : 0.0f;
  }
}

// Four consecutive elements of a field (16-byte aligned): float4, or two double2.
template <typename T> struct V4 {
  T v[4];
  __device__ __forceinline__ static V4 zero() {
    V4 r;
    r.v[0] = r.v[1] = r.v[2] = r.v[3] = (T)0;
    return r;
  }
  __device__ __forceinline__ void load(const T* p, long long idx) {
    if constexpr (sizeof(T) == 4) {
      const float4 q = *reinterpret_cast<const float4*>(p + idx);
      v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
      const double2 q0 = *reinterpret_cast<const double2*>(p + idx);
      const double2 q1 = *reinterpret_cast<const double2*>(p + idx + 2);
      v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
    }
  }
  // the same through the read-only data path: for inputs the kernel does not write
  __device__ __forceinline__ void loadg(const T* p, long long idx) {
    if constexpr (sizeof(T) == 4) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(p + idx));
      v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
      const double2 q0 = __ldg(reinterpret_cast<const double2*>(p + idx));
      const double2 q1 = __ldg(reinterpret_cast<const double2*>(p + idx + 2));
      v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
    }
  }
  __device__ __forceinline__ void store(T* p, long long idx) const {
    if constexpr (sizeof(T) == 4) {
      *reinterpret_cast<float4*>(p + idx) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
      *reinterpret_cast<double2*>(p + idx) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2*>(p + idx + 2) = make_double2(v[2], v[3]);
    }
  }
};
template <typename T> __device__ __forceinline__ T ldg1(const T* p) { return __ldg(p); }
// 1/x for x a positive normal number (|q|^2 of a nonzero mode). FP32: __fdividef's
// approximate reciprocal (within 2 ulp), without the special-case path of the
// correctly rounded division; FP64: rcp_f64's Newton-Raphson reciprocal (within an ulp
// of the division, in fewer FP64 operations: csrc/swc_fpconv.h).
__device__ __forceinline__ float rcp_pos(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double rcp_pos(double x) { return rcp_f64(x); }

// Four consecutive points per thread (n^3 is a multiple of 4: every extent is >= 4).
// The mixed engine takes its FP32 density from rhof + off and touches the FP64 rho
// only in the relax phase, where it is reset.
template <typename T> __global__ void __launch_bounds__(256) s6_kernel(Grid g, S6Args<T> a) {
  constexpr bool mixed = sizeof(T) == 4;
  const long long idx = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  if (idx >= g.ng) return;
  V4<double> r;
  V4<T> rf;
  V4<T> A, lapR, L, P, gpx, gpy, gpz, grx, gry, grz;
  if constexpr (mixed) {
    if (!a.relax) rf.load(a.rhof, idx);
  } else {
    r.load(a.rho, idx);
  }
  A.load(a.amp, idx);
  lapR.load(a.lapR, idx);
  L.load(a.lpsi, idx);
  P.load(a.psi, idx);
  gpx.load(a.gpx, idx); gpy.load(a.gpy, idx); gpz.load(a.gpz, idx);
  grx.load(a.grx, idx); gry.load(a.gry, idx); grz.load(a.grz, idx);
  const T rho0 = a.rho0_t, kp = a.kp_t, zeta = a.zeta_t, ep = a.ep_t, beta = a.beta_t, gam = a.gamma_t;
  const T off = a.off_t;
  V4<T> fgrad, ener, Sx, Sy, Sz, fx, fy, fz, mu;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    T rr;
    if (a.relax) {
      // REF:1371-1374: rho reset to rho_0 + kp A during the relax phase
      // rho_1 + ((1 - rho_1)/Amp) A with (1 - rho_1)/Amp = kp evaluated once on the host
      if constexpr (mixed) {
        r.v[c] = a.rho0 + a.kp * widen_f32(A.v[c]);
        rf.v[c] = narrow_f64(r.v[c] - a.off);
        rr = rf.v[c] + off;
      } else {
        r.v[c] = a.rho0 + a.kp * (double)A.v[c];
        rr = (T)r.v[c];
      }
      lapR.v[c] = rr * lapR.v[c];
    } else {
      if constexpr (mixed) rr = rf.v[c] + off;
      else rr = (T)r.v[c];
    }
    const T Lc = L.v[c], p = P.v[c], Ac = A.v[c];
    const T E = (T)0.5 * (Lc * Lc);
    const T t = rho0 + kp * Ac;
    fgrad.v[c] = (T)0.5 * zeta * (rr * rr - t * t);
    const T mu1 = lapR.v[c] + rr * Lc;
    Sx.v[c] = mu1 * gpx.v[c] + E * grx.v[c];
    Sy.v[c] = mu1 * gpy.v[c] + E * gry.v[c];
    Sz.v[c] = mu1 * gpz.v[c] + E * grz.v[c];
    const T p2 = p * p;
    mu.v[c] = lapR.v[c] + rr * (Lc - ep * p - beta * (p2 * p) + gam * (p2 * p2 * p));
    ener.v[c] = rr * E;
    const T cc = div_nr(kp * zeta * (rr - rho0 - kp * Ac), Ac + (T)0.001);
    fx.v[c] = cc * gpx.v[c];
    fy.v[c] = cc * gpy.v[c];
    fz.v[c] = cc * gpz.v[c];
  }
  if (a.relax) {
    r.store(a.rho, idx);
    if constexpr (mixed) rf.store(a.rhof, idx);
  }
  fgrad.store(a.fgrad, idx);
  Sx.store(a.Sx, idx); Sy.store(a.Sy, idx); Sz.store(a.Sz, idx);
  mu.store(a.mu, idx);
  ener.store(a.ener, idx);
  fx.store(a.fx, idx); fy.store(a.fy, idx); fz.store(a.fz, idx);
}


// S8 + S9 (REF:1479-1974): Stokes solve on the three staggered grids, spectral.
template <typename T> struct StokesArgs {
  const T *Sx, *Sy, *Sz, *fgrad, *ener;
  T *vsolx, *vsoly, *vsolz, *virrx, *virry, *virrz;
  const T *vqx, *vqy, *vqz, *vsx, *vsy, *vsz;  // wavenumbers
  const T *gqx, *gqy, *gqz, *gsx, *gsy, *gsz;  // exp(-1.57^2 2 q^2) per axis
  T scale, inv_nu, inv_lam2nu;  // 1/nu, 1/(lambda + 2 nu)
  int block;  // x-slab size of the reference decomposition (REF:299)
  T *vsumx, *vsumy, *vsumz;  // v_sol + v_irr per component, the input of the S11 transforms
  int write_vsol;            // v_sol itself only when it is transformed for output
  int write_virr;            // v_irr itself: for the divergence kernel, or for the adjoint's tape
  T* divv;                   // stokes_kernel<T, true>: div v-hat of REF:2042-2076 (cosine grid)
};

// Four consecutive points along z per thread, with 32-bit indices (n^3 <= 2^30). The
// staggered neighbours at k-1 / k+1 come from the aligned 4-vector of the neighbouring
// row plus one scalar at its edge; every per-point expression is the one-point form.
//
// DIVV: the kernel also writes div v-hat (i, j, k) = qx v_irr,x(i-1, j, k) + qy
// v_irr,y(i, j-1, k) + qz v_irr,z(i, j, k-1) (REF:2042-2076). The three staggered points
// it reads share the point's own inputs: since Vs[n-1] = Vq[n] (and so gs[n-1] = gq[n],
// bit for bit: same expression), each has |q|^2 = |q(i,j,k)|^2, the Gaussian G(i,j,k),
// fg = fgrad + E G at (i,j,k), and the same q.S = D = qx Sx(i-1,j,k) + qy Sy(i,j-1,k) +
// qz Sz(i,j,k-1). With the reference's index ranges (v_x for i-1 < nx-1, v_y and v_z
// for j', k' < n-1, REF:1584, 1760-1812) and the rank-count quirk of v_z at k' = 0
// (REF:1932):
//   div v-hat = scale/((lambda + 2 nu) |q|^2) sum_valid q_a^2 (fg + D G_a / |q|^2).
// FP32: three 256-thread blocks per SM (80 registers; uncapped it takes 95 and runs
// two blocks, measured slower at 256^3: 172 us against 132 us per launch; capped at 64
// for four blocks it spills 68 bytes a thread and the 256^3 step is 6 us slower).
template <typename T, bool DIVV>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) stokes_kernel(Grid g, StokesArgs<T> a) {
  const int idx = 4 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (idx >= (int)g.ng) return;
  const int k0 = idx & (g.nz - 1), j = (idx >> g.lz) & (g.ny - 1), i = idx >> (g.ly + g.lz);
  const int sx = 1 << (g.ly + g.lz), sy = g.nz;
  const bool has_next = k0 + 4 < g.nz;  // k0 + 4 is in this row
  const bool ip = i > 0, jp = j > 0, kp = k0 != 0;
  // The inputs are read-only here: every load takes the read-only path, so none has to
  // wait for the output stores issued before it.
  V4<T> Sxc, Syc, Szc, qz, szv, gqz, gsz;
  Sxc.loadg(a.Sx, idx);
  Syc.loadg(a.Sy, idx);
  Szc.loadg(a.Sz, idx);
  qz.loadg(a.vqz, k0);
  szv.loadg(a.vsz, k0);
  gqz.loadg(a.gqz, k0);
  gsz.loadg(a.gsz, k0);
  const T qxi = a.vqx[i], qyj = a.vqy[j];
  // plane i-1, row j-1 and the point's own row: read by v_y, v_z and div v-hat
  V4<T> Sxm = V4<T>::zero(), Sym = V4<T>::zero(), F3, E3;
  if (ip) Sxm.loadg(a.Sx, idx - sx);
  if (jp) Sym.loadg(a.Sy, idx - sy);
  F3.loadg(a.fgrad, idx);
  E3.loadg(a.ener, idx);
  // v_x on the x-sine grid, i < nx-1 (REF:1581-1699)
  V4<T> vs, vi;
  if (i < g.nx - 1) {
    const T sxi = a.vsx[i];
    V4<T> Sy1 = V4<T>::zero(), Szn, F1, E1;
    if (jp) Sy1.loadg(a.Sy, idx + sx - sy);
    Szn.loadg(a.Sz, idx + sx);
    const T Szp = kp ? ldg1(a.Sz + idx + sx - 1) : (T)0;
    F1.loadg(a.fgrad, idx + sx);
    E1.loadg(a.ener, idx + sx);
    const T Gx = a.gqx[i + 1] * a.gqy[j], Gsx = a.gsx[i] * a.gqy[j];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const T Sz = (c == 0) ? Szp : Szn.v[c - 1];
      const T dot = sxi * Sxc.v[c] + qyj * Sy1.v[c] + qz.v[c] * Sz;
      const T mq2 = sxi * sxi + qyj * qyj + qz.v[c] * qz.v[c];
      const T inv = rcp_pos(mq2);
      const T CM1 = a.scale * inv, CM2 = sxi * inv;
      const T fg = F1.v[c] + E1.v[c] * (Gx * gqz.v[c]);
      vs.v[c] = (CM1 * a.inv_nu) * (Sxc.v[c] - CM2 * dot);
      vi.v[c] = (CM1 * a.inv_lam2nu) * (sxi * fg + CM2 * dot * (Gsx * gqz.v[c]));
    }
  } else {
    vs = V4<T>::zero();
    vi = V4<T>::zero();
  }
  if (a.write_vsol) vs.store(a.vsolx, idx);
  if (a.write_virr) vi.store(a.virrx, idx);
#pragma unroll
  for (int c = 0; c < 4; ++c) vs.v[c] = vs.v[c] + vi.v[c];
  vs.store(a.vsumx, idx);
  // v_y, v_z for j < ny-1, k < nz-1 (REF:1758-1974); other modes stay 0. Only the last
  // group of a row holds k = nz-1: its fourth results are computed from zero neighbours
  // and then cleared.
  V4<T> ys = V4<T>::zero(), yi = V4<T>::zero(), zs = V4<T>::zero(), zi = V4<T>::zero();
  if (j < g.ny - 1) {
    const T syj = a.vsy[j];
    V4<T> Sx2 = V4<T>::zero(), Szn2, F2, E2;
    if (ip) Sx2.loadg(a.Sx, idx - sx + sy);
    Szn2.loadg(a.Sz, idx + sy);
    const T Szp2 = kp ? ldg1(a.Sz + idx + sy - 1) : (T)0;
    F2.loadg(a.fgrad, idx + sy);
    E2.loadg(a.ener, idx + sy);
    // z: Sx[idx - sx + 1], Sy[idx - sy + 1], fgrad/ener[idx + 1] (k + 1 in the same row)
    T Sxn = (T)0, Syn = (T)0, Fn = (T)0, En = (T)0, gzn = (T)0;
    if (has_next) {
      if (ip) Sxn = ldg1(a.Sx + idx - sx + 4);
      if (jp) Syn = ldg1(a.Sy + idx - sy + 4);
      Fn = ldg1(a.fgrad + idx + 4);
      En = ldg1(a.ener + idx + 4);
      gzn = a.gqz[k0 + 4];
    }
    const T Gy = a.gqx[i] * a.gqy[j + 1], Gsy = a.gqx[i] * a.gsy[j], Gz = a.gqx[i] * a.gqy[j];
    // REF:1932: off the first slab of a rank, the k = 0, j > 0 modes use CM1y's filter
    const bool q1 = !kp && jp && (i % a.block) != 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const T szk = szv.v[c];
      {
        const T Sz = (c == 0) ? Szp2 : Szn2.v[c - 1];
        const T dot = qxi * Sx2.v[c] + syj * Syc.v[c] + qz.v[c] * Sz;
        const T mq2 = qxi * qxi + syj * syj + qz.v[c] * qz.v[c];
        const T inv = rcp_pos(mq2);
        const T CM1 = a.scale * inv, CM2 = syj * inv;
        const T fg = F2.v[c] + E2.v[c] * (Gy * gqz.v[c]);
        ys.v[c] = (CM1 * a.inv_nu) * (Syc.v[c] - CM2 * dot);
        yi.v[c] = (CM1 * a.inv_lam2nu) * (syj * fg + CM2 * dot * (Gsy * gqz.v[c]));
      }
      {
        const T Sx = (c < 3) ? Sxm.v[c + 1] : Sxn;
        const T Sy = (c < 3) ? Sym.v[c + 1] : Syn;
        const T dot = qxi * Sx + qyj * Sy + szk * Szc.v[c];
        const T mq2 = qxi * qxi + qyj * qyj + szk * szk;
        const T inv = rcp_pos(mq2);
        const T CM1 = a.scale * inv, CM2 = szk * inv;
        const T f1 = (c < 3) ? F3.v[c + 1] : Fn, e1 = (c < 3) ? E3.v[c + 1] : En;
        const T gz1 = (c < 3) ? gqz.v[c + 1] : gzn;
        const T fg = f1 + e1 * (Gz * gz1);
        const T G = (c == 0 && q1) ? (Gsy * gqz.v[c]) : (Gz * gsz.v[c]);
        zs.v[c] = (CM1 * a.inv_nu) * (Szc.v[c] - CM2 * dot);
        zi.v[c] = (CM1 * a.inv_lam2nu) * (szk * fg + CM2 * dot * G);
      }
    }
    if (!has_next) ys.v[3] = yi.v[3] = zs.v[3] = zi.v[3] = (T)0;
  }
  if (a.write_vsol) {
    ys.store(a.vsoly, idx);
    zs.store(a.vsolz, idx);
  }
  if (a.write_virr) {
    yi.store(a.virry, idx);
    zi.store(a.virrz, idx);
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    ys.v[c] = ys.v[c] + yi.v[c];
    zs.v[c] = zs.v[c] + zi.v[c];
  }
  ys.store(a.vsumy, idx);
  zs.store(a.vsumz, idx);
  if constexpr (DIVV) {
    V4<T> dv;
    const T szp = kp ? ldg1(a.Sz + idx - 1) : (T)0;  // Sz(i, j, k0 - 1)
    const T Gxy = a.gqx[i] * a.gqy[j];
    const T qx2 = qxi * qxi, qy2 = qyj * qyj;
    const bool off_first_slab = (i % a.block) != 0;
    const T Gz1 = (jp && off_first_slab) ? a.gqx[i] * a.gsy[j] * a.gqz[0] : (T)0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int k = k0 + c;
      const bool vx = ip, vy = jp && (k < g.nz - 1), vz = (k > 0) && (j < g.ny - 1);
      const T qzk = qz.v[c];
      const T qz2 = qzk * qzk;
      const T Szm = (c == 0) ? szp : Szc.v[c - 1];
      const T D = qxi * Sxm.v[c] + qyj * Sym.v[c] + qzk * Szm;
      const T inv = rcp_pos(qx2 + qy2 + qz2);
      const T G = Gxy * gqz.v[c];
      const T fg = F3.v[c] + E3.v[c] * G;
      const T t = D * inv;
      // v_z at k' = k - 1 = 0, j > 0, off a rank's first x slab: CM1y's filter
      // gqx[i] gsy[j] gqz[k'] (REF:1932) instead of G
      const T Gz = (k == 1 && jp && off_first_slab) ? Gz1 : G;
      const T w = fg + t * G;
      const T sum = (vx ? qx2 : (T)0) * w + (vy ? qy2 : (T)0) * w + (vz ? qz2 * (fg + t * Gz) : (T)0);
      // at i = j = k = 0 no term is valid (and |q|^2 = 0): the mode stays 0
      dv.v[c] = (vx || vy || vz) ? a.scale * a.inv_lam2nu * inv * sum : (T)0;
    }
    dv.store(a.divv, idx);
  }
}

// S10 (REF:2042-2079): div v and q.f on the cosine grid (q.f without `scale`).
template <typename T> struct DivArgs {
  const T *virrx, *virry, *virrz, *fx, *fy, *fz;
  T *divv, *dq;
  const T *vqx, *vqy, *vqz;
};
template <typename T> __global__ void __launch_bounds__(256) div_kernel(Grid g, DivArgs<T> a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.ng) return;
  int i, j, k;
  decompose(g, idx, i, j, k);
  const long long sx = 1LL << (g.ly + g.lz), sy = g.nz;
  const T vx = (i > 0) ? a.virrx[idx - sx] : (T)0, fx = (i > 0) ? a.fx[idx - sx] : (T)0;
  const T vy = (j > 0) ? a.virry[idx - sy] : (T)0, fy = (j > 0) ? a.fy[idx - sy] : (T)0;
  const T vz = (k > 0) ? a.virrz[idx - 1] : (T)0, fz = (k > 0) ? a.fz[idx - 1] : (T)0;
  const T qx = a.vqx[i], qy = a.vqy[j], qz = a.vqz[k];
  a.divv[idx] = qx * vx + qy * vy + qz * vz;
  a.dq[idx] = qx * fx + qy * fy + qz * fz;
}

// S15 (REF:2214-2231): per-block partial sums of |psi - psi_old|, |psi|, rho, the
// free energy density and the non-finite count; also rotates psi_old <- psi <- psi_new
// and writes the energy density field.
template <typename T> struct DiagArgs {
  const T *psi_new, *lpsi, *amp;
  T *psi, *psi_old, *energy;
  const double* rho;
  double* partial;  // 5 doubles per block
  double ep, beta, gamma, zeta, rho0, kp;
  const T* rhof;  // mixed engine: FP32 copy rho - off for the per-point terms (FP64: null)
  // the coefficients in T, converted on the host: -ep/2, beta/4, gamma/6, zeta/2, rho_0, kp, off
  T c_ep, c_beta, c_gamma, c_zeta, rho0_t, kp_t, off_t;
};
constexpr int kDiagThreads = 256;

// Kahan-compensated FP32 accumulation: sum + value, the lost low part kept in c.
__device__ __forceinline__ void kahan_add(float& sum, float& c, float v) {
  const float y = v - c;
  const float t = sum + y;
  c = (t - sum) - y;
  sum = t;
}

// FP64 engine: every per-point term and accumulation in FP64. Mixed engine: the
// per-point terms in FP32 (its psi, L and A are FP32) with compensated FP32 partial sums
// per thread (error <= 2 eps sum|x| over ~100 points), then FP64 across threads and
// blocks; the density sum (mass) stays FP64, rho being FP64 state; the non-finite count
// is an integer count (bit tests).
template <typename T> __global__ void __launch_bounds__(kDiagThreads) diag_kernel(Grid g, DiagArgs<T> a) {
  constexpr bool mixed = sizeof(T) == 4;
  __shared__ double sh[5][kDiagThreads / 32];
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0;
  float f0 = 0.f, k0 = 0.f, f1 = 0.f, k1 = 0.f, f3 = 0.f, k3 = 0.f;
  int nf = 0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < g.ng;
       idx += (long long)gridDim.x * blockDim.x) {
    const T pn = a.psi_new[idx], po = a.psi[idx], L = a.lpsi[idx], A = a.amp[idx];
    const double r = a.rho[idx];
    const T p2 = pn * pn;
    const T e = a.c_ep * p2 + (T)0.5 * (L * L) - a.c_beta * (p2 * p2) + a.c_gamma * (p2 * p2 * p2);
    if constexpr (mixed) {
      const T rr = a.rhof[idx] + a.off_t;
      const T d = rr - a.rho0_t - a.kp_t * A;
      kahan_add(f0, k0, fabsf(pn - po));
      kahan_add(f1, k1, fabsf(pn));
      s2 += r;
      kahan_add(f3, k3, rr * e + a.c_zeta * (d * d));
      const uint32_t pb = f32_bits(pn), rh = (uint32_t)__double2hiint(r);
      nf += (((pb >> 23) & 0xffu) == 0xffu) + (((rh >> 20) & 0x7ffu) == 0x7ffu);
    } else {
      s0 += (double)fabs(pn - po);
      s1 += (double)fabs(pn);
      s2 += r;
      const T d = (T)r - a.rho0_t - a.kp_t * A;
      s3 += (double)((T)r * e + a.c_zeta * (d * d));
      s4 += (double)(!isfinite(pn)) + (double)(!isfinite(r));
    }
    a.energy[idx] = (T)e;
    a.psi_old[idx] = po;
    a.psi[idx] = pn;
  }
  if constexpr (mixed) {
    s0 = (double)f0 - (double)k0;
    s1 = (double)f1 - (double)k1;
    s3 = (double)f3 - (double)k3;
    s4 = (double)nf;
  }
  double v[5] = {s0, s1, s2, s3, s4};
#pragma unroll
  for (int q = 0; q < 5; ++q)
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int q = 0; q < 5; ++q) sh[q][w] = v[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < 5; ++q) {
      double t = 0;
      for (int ww = 0; ww < kDiagThreads / 32; ++ww) t += sh[q][ww];
      a.partial[5 * blockIdx.x + q] = t;
    }
  }
}

// Deterministic final sum of the per-block partials (one block of 5 warps): warp q sums
// column q lane-strided, then by a fixed shuffle tree, so the result depends only on
// the partials and nblocks.
constexpr int kDiagFinalThreads = 160;
static __global__ void __launch_bounds__(kDiagFinalThreads) diag_final_kernel(const double* partial, int nblocks,
                                                                            double* out) {
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double t = 0;
  for (int b = lane; b < nblocks; b += 32) t += partial[5 * b + q];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) out[q] = t;
}

// ---------------------------------------------------------------------------------
// Engine
// ---------------------------------------------------------------------------------

template <typename T> struct DevTables {
  R2RTables<T> t[3];  // per axis
};

template <typename T> class StepEngine : public EngineBase {
 public:
  explicit StepEngine(const swc_params& p) : p_(p) {}
  ~StepEngine() override { release(); }

  int init();
  int set_state(const double* psi, const double* rho) override;
  int set_state_ic(const swc_ic& ic) override;
  int preloop(bool have_rho);  // the pre-loop from psi staged in frho_ (and rho_)
  int step(int nsteps) override;
  int step_async(int nsteps) override;
  int prepare() override;
  int sync() override;
  int diagnostics(swc_diag* out) override {
    *out = diag_;
    return SWC_OK;
  }
  int get_field(int field, double* dst) override;
  int get_field_async(int field, double* dst) override;
  int get_field_wait() override;
  int field_ptr(int field, void** ptr, int* elem_bytes) override;
  int get_step(int64_t* n) override {
    *n = nloop_;
    return SWC_OK;
  }
  int last_ms(double* ms) override {
    *ms = last_ms_;
    return SWC_OK;
  }
  int last_launches(int64_t* n) override {
    *n = last_launches_;
    return SWC_OK;
  }
  int save(const char* path) override;
  int load(const char* path) override;
  int backward(const double* dpsi, const double* drho, double energy_lambda, double* dpsi0, double* drho0,
               swc_grad* out) override {
    return backward_impl(dpsi, drho, energy_lambda, dpsi0, drho0, out);
  }

 private:
  // ---- adjoint support (checkpoints here; the adjoint itself in swc_adjoint_impl.cuh)
  int save_ckpt(size_t slot, bool with_psi = true);
  size_t ckpt_slot_bytes(bool with_psi = true) const;
  int restore_ckpt(size_t slot);
  int psi_from_state();  // psi = DCT-III^3 psiq with the step's own last three passes
  // FP64 engine: the FP64 adjoint (swc_adjoint_impl.cuh, in swc_step_fp64.cu); mixed
  // engine: the same adjoint in FP32 on the mixed trajectory (swc_step_mixed_adj.cu)
  int backward_impl(const double* dpsi, const double* drho, double energy_lambda, double* dpsi0, double* drho0,
                    swc_grad* out);
  double energy_w_ = 0.0;          // lambda dx^3 of the current swc_backward's energy term
  int record_tape(T* tp, int64_t n, bool alias = false);
  int host_to_field(const double* src, T* dst);
  int field_to_host(const T* src, double* dst);
  int stage_alloc();
  int adjoint_step(size_t slot, bool relax, bool first, bool last);
  int adjoint_alloc(size_t tape_fields);
  int tape_and_adjoint(int64_t n);                        // step n from the loaded state n-1
  int advance(int64_t from, int64_t k);                   // k plain steps from state `from`
  int reverse_binomial(int64_t l, int64_t n, size_t sl, size_t ff, int64_t nfree);
  int64_t fwd_steps_ = 0;          // forward steps rerun by the current swc_backward
  size_t engine_bytes_ = 0;        // device bytes of the engine's own arrays
  std::vector<double*> ckpt_;      // state at steps 0, K, 2K, ... (6 arrays each)
  std::vector<size_t> ckpt_bytes_; // allocated bytes of each slot
  std::vector<char> ckpt_psi_;     // the slot holds psi (else restore recomputes it)
  T* tape_ = nullptr;              // forward intermediates of one segment
  // binomial schedule: the tape step's fields read in place (the adjoint step that
  // consumes them runs next on the same stream) instead of copied into tape_
  const T* tape_alias_[32] = {};
  bool tape_alias_on_ = false;
  size_t tape_fields_ = 0;  // tape_ capacity in fields of n^3 values
  T* adj_ = nullptr;               // adjoint work arrays
  double* pgrad_ = nullptr;        // parameter-gradient totals, then per-block cells
  int* status_ = nullptr;          // set by a transform pass whose bounded wait ran out
  double* stage_ = nullptr;        // FP64 staging of FP32 fields for swc_get_field
  // swc_get_field_async: two FP64 snapshots of the field, each copied to the host on
  // copy_stream_ while the next steps run on stream_
  cudaStream_t copy_stream_ = nullptr;
  double* astage_[2] = {nullptr, nullptr};
  cudaEvent_t aready_[2] = {nullptr, nullptr}, adone_[2] = {nullptr, nullptr};
  bool apending_[2] = {false, false};
  int anext_ = 0;
  size_t pgrad_doubles() const { return 8 * (1 + (size_t)((g_.ng + 255) / 256)); }
  bool adj_valid_ = false;         // checkpoints describe the run since swc_set_state
  // launch one axis pass on stream_, data type U (T, or double for the FP64 pre-loop)
  template <typename U, int KIND, int AX, class LD, class ST, class MUL = NoMul<U>>
  int passU(LD ld, ST st, MUL mul = MUL());
  template <typename U, int KIND, int AX, class LD> int plane_order();
  template <int KIND, int AX, class LD, class ST, class MUL = NoMul<T>>
  int pass(LD ld, ST st, MUL mul = MUL()) {
    return passU<T, KIND, AX, LD, ST, MUL>(ld, st, mul);
  }
  template <typename U> R2RTables<U> tabs(int a) const {
    if constexpr (std::is_same<U, T>::value) return tab_.t[a];
    else return tabd_.t[a];
  }
  int enqueue_step(bool relax, bool first, bool diag);
  int enqueue_part_a(bool relax, bool first, bool diag);  // S1-S5
  int enqueue_part_b(bool relax, bool first, bool diag);  // S5 tail-S10 (swc_step_part_b.cuh)
  int enqueue_part_c(bool relax, bool first, bool diag);  // S11-S14 (swc_step_part_c.cuh)
  int inverse_velocity(int ax, T* in, T* out);             // (swc_step_part_c.cuh)
  int transform_vsol();                                    // (swc_step_part_c.cuh)
  // diag: the diagnostic variant (S15 reductions, psi_old <- psi rotation, energy field);
  // vsol: the Stokes kernel also writes v_sol (the last step of a swc_step call)
  // tape (swc_backward's one-step tape): the new psi goes to psi_new_, so psi_ keeps
  // the step's input psi, and no diagnostics run
  int run_graph(bool relax, bool first, bool diag, bool vsol, bool tape = false);
  int graph_of(bool relax, bool first, bool diag, bool vsol, bool tape, cudaGraphExec_t* out, int* key);
  // Mixed engine: after each step the CN update's ping-pong buffers change roles (the new
  // psiq is in psiq_old_'s buffer, the step's Nl-hat in nlw_'s); pp_ is the parity of the
  // assignment, part of the graph key (a captured graph holds the pointers).
  int pp_ = 0;
  void swap_pp() {
    if constexpr (!std::is_same<T, double>::value) {
      std::swap(psiq_, psiq_old_);
      std::swap(nlw_, nlq_);
      pp_ ^= 1;
    }
  }
  bool cap_vsol_ = false;  // vsol flag of the variant being captured
  bool cap_tape_ = false;  // tape flag of the variant being captured
  int64_t diag_step_ = -1;  // nLoop of the last step that ran the diagnostics
  int64_t pending_diag_ = -1;  // diagnostic step enqueued, its sums not yet read
  int check_step(int nsteps);
  int enqueue_steps(int nsteps);
  int finish_steps();
  void release();
  int field_src(int field, const void** src, bool* is_double);

  swc_params p_;
  Grid g_{};
  double amp_ = 0, kp_ = 0, rho_s_ = 0, rho_m_ = 0, dx_ = 0, scale_ = 0;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  std::vector<void*> allocs_;
  // tables
  DevTables<T> tab_{};
  DevTables<double> tabd_{};  // FP64 tables (same as tab_ when T = double)
  const T *vq_[3] = {}, *vs_[3] = {}, *gq_[3] = {}, *gs_[3] = {};
  const double* vqd_[3] = {};
  // state (FP64)
  double *psiq_ = nullptr, *psiq_old_ = nullptr, *rho_ = nullptr, *frho_ = nullptr;
  // work (T)
  T *nlq_ = nullptr, *psi_ = nullptr, *psi_new_ = nullptr, *psi_old_ = nullptr;
  T *gp_[3] = {}, *gr_[3] = {}, *amp_f_ = nullptr, *lpsi_ = nullptr, *lapR_ = nullptr, *mu_ = nullptr;
  T *fgrad_ = nullptr, *ener_ = nullptr, *S_[3] = {}, *f_[3] = {}, *vsol_[3] = {}, *virr_[3] = {};
  T *divv_ = nullptr, *dq_ = nullptr, *v_[3] = {}, *vsolr_[3] = {}, *energy_ = nullptr, *nlw_ = nullptr;
  double *partial_ = nullptr, *dsum_ = nullptr;
  // mixed engine: FP32 1/C2 per spectral mode, FP32 f_rho, and FP32 copies of the FP64
  // state kept where the state is written: rhof = rho - rho_off_, psiqf = psiq
  T *frhot_ = nullptr, *rhof_ = nullptr, *psiqf_ = nullptr;
  double rho_off_ = 0;  // (rho_0 + rho_s)/2 in the mixed engine, 0 in the FP64 engine
  int refresh_copies(int frho_mode);
  int diag_blocks_ = 0;
  std::map<int, cudaGraphExec_t> graphs_;
  std::map<int, int64_t> graph_kernels_;  // kernel nodes per captured variant
  int64_t last_launches_ = 0;
  int64_t launches_ = 0;  // running count while a variant is captured
  // plane order of the passes (plane_order): launches_ after the last pass, and whether
  // the last z or y pass walked its planes downward
  int64_t plane_mark_ = -1;
  bool plane_desc_ = false;
  bool have_state_ = false;
  bool have_vsol_ = false;
  bool vsol_pending_ = false;  // spectral v_sol of the last step not yet in real space
  int64_t nloop_ = 0;
  swc_diag diag_{};
  double last_ms_ = 0;
};

template <typename T> void StepEngine<T>::release() {
  // queued graphs may still run (e.g. after a watchdog timeout): drain before freeing
  if (stream_) cudaStreamSynchronize(stream_);
  if (copy_stream_) cudaStreamSynchronize(copy_stream_);
  cudaGetLastError();
  for (int b = 0; b < 2; ++b) {
    if (astage_[b]) cudaFree(astage_[b]);
    if (aready_[b]) cudaEventDestroy(aready_[b]);
    if (adone_[b]) cudaEventDestroy(adone_[b]);
    astage_[b] = nullptr;
    aready_[b] = adone_[b] = nullptr;
    apending_[b] = false;
  }
  if (copy_stream_) cudaStreamDestroy(copy_stream_);
  copy_stream_ = nullptr;
  for (double* c : ckpt_) cudaFree(c);
  ckpt_.clear();
  ckpt_bytes_.clear();
  ckpt_psi_.clear();
  if (tape_) cudaFree(tape_);
  if (adj_) cudaFree(adj_);
  if (pgrad_) cudaFree(pgrad_);
  if (stage_) cudaFree(stage_);
  tape_ = adj_ = nullptr;
  pgrad_ = stage_ = nullptr;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
  for (void* a : allocs_) cudaFree(a);
  allocs_.clear();
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
  if (stream_) cudaStreamDestroy(stream_);
  ev0_ = ev1_ = nullptr;
  stream_ = nullptr;
}

template <typename T> int StepEngine<T>::init() {
  SWC_CK(cudaSetDevice(p_.device));
  g_.nx = p_.nx; g_.ny = p_.ny; g_.nz = p_.nz;
  g_.lx = ilog2(p_.nx); g_.ly = ilog2(p_.ny); g_.lz = ilog2(p_.nz);
  g_.ng = (long long)p_.nx * p_.ny * p_.nz;
  // REF:250-272
  amp_ = std::sqrt((3 * p_.beta + std::sqrt(9 * p_.beta * p_.beta + 40 * p_.ep * p_.gamma)) / 5);
  kp_ = (1 - p_.rho_0) / amp_;
  rho_s_ = kp_ * amp_ + p_.rho_0;
  rho_m_ = rho_s_ / 2;
  rho_off_ = std::is_same<T, double>::value ? 0.0 : 0.5 * (p_.rho_0 + rho_s_);
  const double pi = 3.14159265358979323846;
  const int dims[3] = {p_.nx, p_.ny, p_.nz};
  double d[3];
  for (int a = 0; a < 3; ++a) d[a] = (dims[a] * 2.0 * pi / (p_.q0 * p_.nw)) / dims[a];
  dx_ = d[0];
  scale_ = 0.125 / ((double)p_.nx * p_.ny * p_.nz);
  SWC_CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  SWC_CK(cudaEventCreate(&ev0_));
  SWC_CK(cudaEventCreate(&ev1_));

  auto dalloc = [&](size_t bytes, void** out) -> int {
    void* ptr = nullptr;
    cudaError_t e = cudaMalloc(&ptr, bytes);
    if (e != cudaSuccess) {
      set_error("cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
      cudaGetLastError();
      return SWC_ERR_OOM;
    }
    allocs_.push_back(ptr);
    engine_bytes_ += bytes;
    *out = ptr;
    return SWC_OK;
  };
  auto upload = [&](const void* host, size_t bytes, const void** out) -> int {
    void* ptr;
    int rc = dalloc(bytes, &ptr);
    if (rc) return rc;
    // stream-ordered: the engine's stream is non-blocking (not ordered after the legacy stream)
    SWC_CK(cudaMemcpyAsync(ptr, host, bytes, cudaMemcpyHostToDevice, stream_));
    SWC_CK(cudaStreamSynchronize(stream_));
    *out = ptr;
    return SWC_OK;
  };
  // status flag of the transform passes' bounded waits (0 = fine)
  {
    int rc = dalloc(sizeof(int), (void**)&status_);
    if (rc) return rc;
    SWC_CK(cudaMemsetAsync(status_, 0, sizeof(int), stream_));
  }
  // wavenumbers REF:445-481 and Gaussian factors, per axis
  for (int a = 0; a < 3; ++a) {
    tab_.t[a].status = status_;
    tabd_.t[a].status = status_;
    const int n = dims[a];
    std::vector<double> vq(n), vs(n), gq(n), gs(n);
    for (int i = 0; i < n; ++i) {
      vq[i] = pi * (i) / (d[a] * n);
      vs[i] = pi * (i + 1) / (d[a] * n);
      gq[i] = std::exp(-1.57 * 1.57 * 2 * (vq[i] * vq[i]));
      gs[i] = std::exp(-1.57 * 1.57 * 2 * (vs[i] * vs[i]));
    }
    std::vector<T> tq(vq.begin(), vq.end()), ts(vs.begin(), vs.end()), tgq(gq.begin(), gq.end()),
        tgs(gs.begin(), gs.end());
    int rc;
    if ((rc = upload(tq.data(), n * sizeof(T), (const void**)&vq_[a]))) return rc;
    if ((rc = upload(ts.data(), n * sizeof(T), (const void**)&vs_[a]))) return rc;
    if ((rc = upload(tgq.data(), n * sizeof(T), (const void**)&gq_[a]))) return rc;
    if ((rc = upload(tgs.data(), n * sizeof(T), (const void**)&gs_[a]))) return rc;
    if ((rc = upload(vq.data(), n * sizeof(double), (const void**)&vqd_[a]))) return rc;
    HostTables<T> ht(n);
    if ((rc = upload(ht.fft.data(), ht.fft.size() * sizeof(T), (const void**)&tab_.t[a].fft))) return rc;
    if ((rc = upload(ht.post.data(), ht.post.size() * sizeof(T), (const void**)&tab_.t[a].post))) return rc;
    if ((rc = upload(ht.pre.data(), ht.pre.size() * sizeof(T), (const void**)&tab_.t[a].pre))) return rc;
    if constexpr (std::is_same<T, double>::value) {
      tabd_.t[a] = tab_.t[a];
    } else {
      HostTables<double> hd(n);
      if ((rc = upload(hd.fft.data(), hd.fft.size() * sizeof(double), (const void**)&tabd_.t[a].fft))) return rc;
      if ((rc = upload(hd.post.data(), hd.post.size() * sizeof(double), (const void**)&tabd_.t[a].post))) return rc;
      if ((rc = upload(hd.pre.data(), hd.pre.size() * sizeof(double), (const void**)&tabd_.t[a].pre))) return rc;
    }
  }
  const size_t nd = (size_t)g_.ng * sizeof(double), nt = (size_t)g_.ng * sizeof(T);
  int rc;
  double** dbufs[] = {&psiq_, &psiq_old_, &rho_, &frho_};
  for (double** b : dbufs)
    if ((rc = dalloc(nd, (void**)b))) return rc;
  T** tbufs[] = {&nlq_, &psi_, &psi_new_, &psi_old_, &gp_[0], &gp_[1], &gp_[2], &gr_[0], &gr_[1],
                 &gr_[2], &amp_f_, &lpsi_, &lapR_, &mu_, &fgrad_, &ener_, &S_[0], &S_[1], &S_[2], &f_[0],
                 &f_[1], &f_[2], &vsol_[0], &vsol_[1], &vsol_[2], &virr_[0], &virr_[1], &virr_[2], &divv_,
                 &dq_, &v_[0], &v_[1], &v_[2], &vsolr_[0], &vsolr_[1], &vsolr_[2], &energy_, &nlw_};
  for (T** b : tbufs) {
    if ((rc = dalloc(nt, (void**)b))) return rc;
    SWC_CK(cudaMemsetAsync(*b, 0, nt, stream_));
  }
  for (double** b : dbufs) SWC_CK(cudaMemsetAsync(*b, 0, nd, stream_));
  SWC_CK(cudaStreamSynchronize(stream_));
  if constexpr (!std::is_same<T, double>::value) {
    T** mbufs[] = {&frhot_, &rhof_, &psiqf_};
    for (T** b : mbufs) {
      if ((rc = dalloc(nt, (void**)b))) return rc;
      SWC_CK(cudaMemsetAsync(*b, 0, nt, stream_));
    }
    SWC_CK(cudaStreamSynchronize(stream_));
  }
  int sms = 0;
  SWC_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p_.device));
  diag_blocks_ = sms * 4;
  long long need = (g_.ng + kDiagThreads - 1) / kDiagThreads;
  if (need < diag_blocks_) diag_blocks_ = (int)need;
  if ((rc = dalloc(sizeof(double) * 5 * diag_blocks_, (void**)&partial_))) return rc;
  if ((rc = dalloc(sizeof(double) * 8, (void**)&dsum_))) return rc;
  return SWC_OK;
}

template <typename T>
template <typename U, int KIND, int AX, class LD, class ST, class MUL>
int StepEngine<T>::passU(LD ld, ST st, MUL mul) {
  R2RTables<U> tb = tabs<U>(AX);
  tb.rev = plane_order<U, KIND, AX, LD>();
  SWC_CK((launch_pass<U, KIND, AX, LD, ST, MUL>(g_, tb, stream_, ld, st, mul)));
  ++launches_;
  return SWC_OK;
}

// Tile order of the next pass (R2RTables::rev). z and y passes walk the field by i planes;
// each runs opposite to the plane-walking kernel before it, so that it starts on the
// planes that kernel touched last, which are still in L2 (a z pass after a y pass, a y
// pass after a z pass, a z pass after a pointwise kernel). x passes touch every i plane
// at each step of their walk (over j) and leave the order as it was; the pointwise
// kernels and the passes of the other forms walk upward. Only the TMA-fed form takes
// the order; the results do not depend on it.
template <typename T>
template <typename U, int KIND, int AX, class LD>
int StepEngine<T>::plane_order() {
  const bool chain = launches_ == plane_mark_;  // no other kernel since the last pass
  plane_mark_ = launches_ + 1;
  if (!chain) plane_desc_ = false;
  if constexpr (AX == 0) {
    return 0;
  } else {
    plane_desc_ = tma_fed_form<U, KIND, AX, LD>() && !plane_desc_;
    return plane_desc_ ? 1 : 0;
  }
}

#define SWC_TRY(x)         \
  do {                     \
    int rc_ = (x);         \
    if (rc_) return rc_;   \
  } while (0)

// The step is enqueued in three parts, each compiled in its own translation unit
// (parts B and C live in swc_step_part_b.cuh / swc_step_part_c.cuh) so the many pass
// instantiations build in parallel.
template <typename T> int StepEngine<T>::enqueue_step(bool relax, bool first, bool diag) {
  SWC_TRY(enqueue_part_a(relax, first, diag));
  SWC_TRY(enqueue_part_b(relax, first, diag));
  return enqueue_part_c(relax, first, diag);
}

// Part A: S1-S5 (gradients, amplitude filter, dfDlapPsi, lapR).
template <typename T> int StepEngine<T>::enqueue_part_a(bool relax, bool first, bool diag) {
  using LP = LdPlain<T, T>;
  using SP = StPlain<T, T>;

  // S1 + S2 (REF:1104-1250): rhoq = DCT(rho) and the six shifted spectral gradients
  // taken back to real space. With psiq = scale DCT-II^3 psi and the DCT-III/DCT-II pairs
  // of the two other axes cancelling (DCT-III DCT-II = 2n per axis), each gradient is
  // one pass along its own axis: d_a f = DST-III_a(-Vs_a shift_a(DCT-II_a f)) / (2 n_a),
  // for f = psi (REF:1190-1219) and f = rho (REF:1191-1219, where -scale Vs rhoq gives
  // the same 1/(2 n_a)). The mixed engine transforms rho - (rho_0 + rho_s)/2: the
  // gradients never read mode 0, and FP32 then resolves the small variations.
  {
    const T cx = (T)(1.0 / (2.0 * g_.nx)), cy = (T)(1.0 / (2.0 * g_.ny)), cz = (T)(1.0 / (2.0 * g_.nz));
    SWC_TRY((pass<K_DERIV, 2>(LP{psi_}, SP{gp_[2]}, MulDeriv<T>{vs_[2], cz, 2})));
    SWC_TRY((pass<K_DERIV, 1>(LP{psi_}, SP{gp_[1]}, MulDeriv<T>{vs_[1], cy, 1})));
    SWC_TRY((pass<K_DERIV, 0>(LP{psi_}, SP{gp_[0]}, MulDeriv<T>{vs_[0], cx, 0})));
    if constexpr (std::is_same<T, double>::value) {
      SWC_TRY((pass<K_DERIV, 2>(LdOffset<T>{rho_, 0.0}, SP{gr_[2]}, MulDeriv<T>{vs_[2], cz, 2})));
      SWC_TRY((pass<K_DERIV, 1>(LdOffset<T>{rho_, 0.0}, SP{gr_[1]}, MulDeriv<T>{vs_[1], cy, 1})));
      SWC_TRY((pass<K_DERIV, 0>(LdOffset<T>{rho_, 0.0}, SP{gr_[0]}, MulDeriv<T>{vs_[0], cx, 0})));
    } else {  // the FP32 copy rho - rho_off_, kept by the density update
      SWC_TRY((pass<K_DERIV, 2>(LP{rhof_}, SP{gr_[2]}, MulDeriv<T>{vs_[2], cz, 2})));
      SWC_TRY((pass<K_DERIV, 1>(LP{rhof_}, SP{gr_[1]}, MulDeriv<T>{vs_[1], cy, 1})));
      SWC_TRY((pass<K_DERIV, 0>(LP{rhof_}, SP{gr_[0]}, MulDeriv<T>{vs_[0], cx, 0})));
    }
  }
  // S3 (REF:1254-1289): amplitude, Gaussian filter
  if constexpr (std::is_same<T, float>::value) {
    amp_kernel<<<(unsigned)((g_.ng / 4 + 255) / 256), 256, 0, stream_>>>(
        g_.ng, LdAmp<float>{psi_, gp_[0], gp_[1], gp_[2], (float)(p_.q0 * p_.q0)}, amp_f_);
    SWC_CK(cudaGetLastError());
    ++launches_;
    // the Gaussian is a product of per-axis factors: three one-axis filter passes
    SWC_TRY((pass<K_FILT, 2>(LP{amp_f_}, SP{amp_f_}, MulAxis<T, 2>{gq_[2], (T)1})));
    SWC_TRY((pass<K_FILT, 1>(LP{amp_f_}, SP{amp_f_}, MulAxis<T, 1>{gq_[1], (T)1})));
    SWC_TRY((pass<K_FILT, 0>(LP{amp_f_}, SP{amp_f_}, MulAxis<T, 0>{gq_[0], (T)scale_})));
  } else {
    SWC_TRY((pass<K_C2, 2>(LdAmp<T>{psi_, gp_[0], gp_[1], gp_[2], (T)(p_.q0 * p_.q0)}, SP{amp_f_})));
    SWC_TRY((pass<K_C2, 1>(LP{amp_f_}, SP{amp_f_})));
    SWC_TRY((pass<K_FILT, 0>(LP{amp_f_}, SP{amp_f_}, MulGauss<T>{gq_[0], gq_[1], gq_[2], (T)scale_})));
    SWC_TRY((pass<K_C3, 1>(LP{amp_f_}, SP{amp_f_})));
    SWC_TRY((pass<K_C3, 2>(LP{amp_f_}, SP{amp_f_})));
  }
  // S4 (REF:1293-1308): dfDlapPsi
  const T alpha = (T)p_.alpha, q02 = (T)(p_.q0 * p_.q0);
  if constexpr (std::is_same<T, double>::value) {
    SWC_TRY((pass<K_C3, 2>(LdLpsi<T>{psiq_, vq_[0], vq_[1], vq_[2], alpha, q02}, SP{lpsi_})));
    SWC_TRY((pass<K_C3, 1>(LP{lpsi_}, SP{lpsi_})));
    SWC_TRY((pass<K_C3, 0>(LP{lpsi_}, SP{lpsi_})));
  } else {
    SWC_TRY((pass<K_C3, 2>(LdMul<LapMul<0>>{psiqf_, LapMul<0>{vq_[0], vq_[1], vq_[2], alpha, q02}}, SP{lpsi_})));
    SWC_TRY((pass<K_C3, 1>(LP{lpsi_}, SP{lpsi_})));
    if (relax) SWC_TRY((pass<K_C3, 0>(LP{lpsi_}, SP{lpsi_})));
    else SWC_TRY((pass<K_C3, 0>(LP{lpsi_}, StLpsiRhoL{lpsi_, lapR_, rhof_, (T)rho_off_})));
  }
  // S5 (REF:1312-1380)
  if (!relax) {
    if constexpr (std::is_same<T, double>::value)
      SWC_TRY((pass<K_C2, 2>(LdRhoL<T>{rho_, lpsi_, (T)0}, SP{lapR_})));
    else  // rho L written by the last pass of dfDlapPsi
      SWC_TRY((pass<K_C2, 2>(LP{lapR_}, SP{lapR_})));
    SWC_TRY((pass<K_C2, 1>(LP{lapR_}, SP{lapR_})));
    SWC_TRY((pass<K_FILT, 0>(LP{lapR_}, SP{lapR_}, MulLap<T>{vq_[0], vq_[1], vq_[2], (T)scale_})));
    SWC_TRY((pass<K_C3, 1>(LP{lapR_}, SP{lapR_})));
    SWC_TRY((pass<K_C3, 2>(LP{lapR_}, SP{lapR_})));
  } else {
    if constexpr (std::is_same<T, double>::value)
      SWC_TRY((pass<K_C3, 2>(LdRelaxLap<T>{psiq_, vq_[0], vq_[1], vq_[2], alpha, q02}, SP{lapR_})));
    else
      SWC_TRY((pass<K_C3, 2>(LdMul<LapMul<1>>{psiqf_, LapMul<1>{vq_[0], vq_[1], vq_[2], alpha, q02}}, SP{lapR_})));
    SWC_TRY((pass<K_C3, 1>(LP{lapR_}, SP{lapR_})));
    SWC_TRY((pass<K_C3, 0>(LP{lapR_}, SP{lapR_})));
  }
  return SWC_OK;
}

// The instantiated graph of one step variant, captured on first use.
template <typename T>
int StepEngine<T>::graph_of(bool relax, bool first, bool diag, bool vsol, bool tape, cudaGraphExec_t* out,
                            int* key_out) {
  vsol = vsol || diag || tape;
  const int key = (relax ? 1 : 0) | (first ? 2 : 0) | (diag ? 4 : 0) | (vsol ? 8 : 0) | (tape ? 16 : 0) | (pp_ << 5);
  auto it = graphs_.find(key);
  if (it == graphs_.end()) {
    cudaGraph_t graph = nullptr;
    SWC_CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeRelaxed));
    launches_ = 0;
    plane_mark_ = -1;
    cap_vsol_ = vsol;
    cap_tape_ = tape;
    int rc = enqueue_step(relax, first, diag);
    cap_tape_ = false;
    cudaError_t e = cudaStreamEndCapture(stream_, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) {
      set_error("cudaStreamEndCapture: %s", cudaGetErrorString(e));
      return SWC_ERR_CUDA;
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
      return SWC_ERR_CUDA;
    }
    it = graphs_.emplace(key, exec).first;
    graph_kernels_[key] = launches_;
  }
  *out = it->second;
  *key_out = key;
  return SWC_OK;
}

template <typename T> int StepEngine<T>::run_graph(bool relax, bool first, bool diag, bool vsol, bool tape) {
  cudaGraphExec_t exec;
  int key;
  SWC_TRY(graph_of(relax, first, diag, vsol, tape, &exec, &key));
  SWC_CK(cudaGraphLaunch(exec, stream_));
  last_launches_ += graph_kernels_[key];
  swap_pp();
  return SWC_OK;
}

// swc_prepare: capture every variant swc_step can launch (relax or normal phase, the
// first step, diagnostic step, v_sol written or not) without running any.
template <typename T> int StepEngine<T>::prepare() {
  if (!have_state_) {
    set_error("swc_prepare before swc_set_state");
    return SWC_ERR_STATE;
  }
  SWC_CK(cudaSetDevice(p_.device));
  cudaGraphExec_t exec;
  int key;
  // both assignments of the ping-pong buffers (the mixed engine alternates them)
  const int npp = std::is_same<T, double>::value ? 1 : 2;
  for (int q = 0; q < npp; ++q) {
    for (int relax = 0; relax < 2; ++relax)
      for (int first = 0; first < 2; ++first)
        for (int v = 0; v < 3; ++v) {
          const int rc = graph_of(relax, first, v == 2, v >= 1, false, &exec, &key);
          if (rc) {
            if (q) swap_pp();
            return rc;
          }
        }
    if (npp > 1) swap_pp();
  }
  return SWC_OK;
}

// psiq = scale * v (last pass of the pre-loop DCT, REF:982)
struct StScaleD {
  double* p;
  double s;
  __device__ __forceinline__ void operator()(int, int, int, long long idx, double v) const { p[idx] = s * v; }
};

// Mixed engine: rebuild the FP32 copies of the FP64 state, and f_rho: 0 zero (after
// swc_set_state), 1 from its FP64 form (after swc_load), 2 kept (checkpoint restore).
// No-op for the FP64 engine.
template <typename T> int StepEngine<T>::refresh_copies(int frho_mode) {
  if constexpr (!std::is_same<T, double>::value) {
    mixed_copies_kernel<<<1024, 256, 0, stream_>>>(g_.ng, rho_, psiq_, frho_mode == 1 ? frho_ : nullptr, rho_off_,
                                                  rhof_, psiqf_, frho_mode == 2 ? nullptr : frhot_);
    SWC_CK(cudaGetLastError());
  }
  (void)frho_mode;
  return SWC_OK;
}

template <typename T> int StepEngine<T>::set_state(const double* psi, const double* rho) {
  SWC_CK(cudaSetDevice(p_.device));
  const size_t nd = (size_t)g_.ng * sizeof(double);
  // psi staged in frho_, rho (or the reference's zero fill, REF:1053) in rho_
  SWC_CK(cudaMemcpyAsync(frho_, psi, nd, cudaMemcpyHostToDevice, stream_));
  if (rho) SWC_CK(cudaMemcpyAsync(rho_, rho, nd, cudaMemcpyHostToDevice, stream_));
  return preloop(rho != nullptr);
}

// The initial psi and rho written by the device generator into the same staging
// arrays: no host arrays, no host-to-device copy.
template <typename T> int StepEngine<T>::set_state_ic(const swc_ic& ic) {
  SWC_CK(cudaSetDevice(p_.device));
  SWC_TRY(ic_generate(p_, ic, frho_, rho_, stream_));
  const bool has_rho = ic.kind == SWC_IC_FLAT || ic.kind == SWC_IC_UNDULATED || ic.kind == SWC_IC_DISLOCATIONS;
  return preloop(has_rho);
}

template <typename T> int StepEngine<T>::preloop(bool have_rho) {
  const size_t nd = (size_t)g_.ng * sizeof(double), nt = (size_t)g_.ng * sizeof(T);
  // REF:968-982: psiq = scale * DCT(psi), in FP64 for both engines (psi staged in frho_)
  SWC_TRY((passU<double, K_C2, 2>(LdPlain<double, double>{frho_}, StPlain<double, double>{frho_})));
  SWC_TRY((passU<double, K_C2, 1>(LdPlain<double, double>{frho_}, StPlain<double, double>{frho_})));
  SWC_TRY((passU<double, K_C2, 0>(LdPlain<double, double>{frho_}, StScaleD{psiq_, scale_})));
  // REF:1052-1071 (+ caller's rho); f_rho, Nl_old and the work arrays start at zero
  if (!have_rho) SWC_CK(cudaMemsetAsync(rho_, 0, nd, stream_));
  SWC_CK(cudaMemsetAsync(frho_, 0, nd, stream_));
  SWC_CK(cudaMemcpyAsync(psiq_old_, psiq_, nd, cudaMemcpyDeviceToDevice, stream_));  // REF:1005
  T* zero[] = {nlq_, psi_old_, gp_[0], gp_[1], gp_[2], gr_[0], gr_[1], gr_[2], amp_f_, divv_, v_[0], v_[1], v_[2],
               vsolr_[0], vsolr_[1], vsolr_[2], energy_, lpsi_, mu_};
  for (T* z : zero) SWC_CK(cudaMemsetAsync(z, 0, nt, stream_));
  // REF:984-988: psi = iDCT(psiq)
  SWC_TRY((pass<K_C3, 2>(LdPlain<T, double>{psiq_}, StPlain<T, T>{psi_})));
  SWC_TRY((pass<K_C3, 1>(LdPlain<T, T>{psi_}, StPlain<T, T>{psi_})));
  SWC_TRY((pass<K_C3, 0>(LdPlain<T, T>{psi_}, StPlain<T, T>{psi_})));
  SWC_CK(cudaMemcpyAsync(psi_old_, psi_, nt, cudaMemcpyDeviceToDevice, stream_));  // REF:1010
  SWC_TRY(refresh_copies(0));
  if (p_.adjoint_ckpt != 0) SWC_TRY(save_ckpt(0));
  adj_valid_ = p_.adjoint_ckpt != 0;
  SWC_CK(cudaStreamSynchronize(stream_));
  nloop_ = 0;
  have_state_ = true;
  have_vsol_ = false;
  vsol_pending_ = false;
  std::memset(&diag_, 0, sizeof(diag_));
  diag_step_ = -1;
  pending_diag_ = -1;
  return SWC_OK;
}

// Checkpoint slot: psiq, psiq_old, rho (FP64), Nl_old, f_rho, psi (the engine's
// precision: FP64, or FP32 in the mixed engine), packed: ckpt_slot_bytes() each.
// Without psi (with_psi = false, the binomial schedule's snapshots after step 0): a
// state that a step wrote has psi = DCT-III^3 psiq from that step's last three passes,
// which restore_ckpt reruns on the restored psiq, bit for bit (step 0's psi comes from
// swc_set_state's own transform and is always kept).
template <typename T> size_t StepEngine<T>::ckpt_slot_bytes(bool with_psi) const {
  return (size_t)g_.ng * (3 * sizeof(double) + (with_psi ? 3 : 2) * sizeof(T));
}

template <typename T> int StepEngine<T>::save_ckpt(size_t slot, bool with_psi) {
  const size_t ng = (size_t)g_.ng;
  while (ckpt_.size() <= slot) {
    ckpt_.push_back(nullptr);
    ckpt_bytes_.push_back(0);
    ckpt_psi_.push_back(0);
  }
  const size_t need = ckpt_slot_bytes(with_psi);
  if (ckpt_bytes_[slot] < need) {
    if (ckpt_[slot]) cudaFree(ckpt_[slot]);
    ckpt_[slot] = nullptr;
    ckpt_bytes_[slot] = 0;
    double* c = nullptr;
    if (cudaMalloc(&c, need) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc for an adjoint checkpoint failed (%zu MB)", need >> 20);
      return SWC_ERR_OOM;
    }
    ckpt_[slot] = c;
    ckpt_bytes_[slot] = need;
  }
  ckpt_psi_[slot] = with_psi ? 1 : 0;
  char* c = reinterpret_cast<char*>(ckpt_[slot]);
  constexpr bool mixed = !std::is_same<T, double>::value;
  const void* src[6] = {psiq_, psiq_old_, rho_, nlq_, mixed ? (const void*)frhot_ : (const void*)frho_, psi_};
  const size_t sz[6] = {8, 8, 8, sizeof(T), sizeof(T), sizeof(T)};
  size_t off = 0;
  for (int q = 0; q < (with_psi ? 6 : 5); ++q) {
    SWC_CK(cudaMemcpyAsync(c + off, src[q], ng * sz[q], cudaMemcpyDeviceToDevice, stream_));
    off += ng * sz[q];
  }
  return SWC_OK;
}

template <typename T> int StepEngine<T>::restore_ckpt(size_t slot) {
  const size_t ng = (size_t)g_.ng;
  const char* c = reinterpret_cast<const char*>(ckpt_[slot]);
  constexpr bool mixed = !std::is_same<T, double>::value;
  void* dst[6] = {psiq_, psiq_old_, rho_, nlq_, mixed ? (void*)frhot_ : (void*)frho_, psi_};
  const size_t sz[6] = {8, 8, 8, sizeof(T), sizeof(T), sizeof(T)};
  const bool with_psi = ckpt_psi_[slot] != 0;
  size_t off = 0;
  for (int q = 0; q < (with_psi ? 6 : 5); ++q) {
    SWC_CK(cudaMemcpyAsync(dst[q], c + off, ng * sz[q], cudaMemcpyDeviceToDevice, stream_));
    off += ng * sz[q];
  }
  SWC_TRY(refresh_copies(2));  // the mixed engine's FP32 copies of rho and psiq (f_rho restored above)
  return with_psi ? SWC_OK : psi_from_state();
}

template <typename T> int StepEngine<T>::psi_from_state() {
  using LP = LdPlain<T, T>;
  using SP = StPlain<T, T>;
  if constexpr (std::is_same<T, double>::value) SWC_TRY((pass<K_C3, 2>(LdPlain<T, double>{psiq_}, SP{psi_})));
  else SWC_TRY((pass<K_C3, 2>(LP{psiqf_}, SP{psi_})));
  SWC_TRY((pass<K_C3, 1>(LP{psi_}, SP{psi_})));
  SWC_TRY((pass<K_C3, 0>(LP{psi_}, SP{psi_})));
  return SWC_OK;
}

template <typename T> int StepEngine<T>::check_step(int nsteps) {
  if (nsteps < 0) {
    set_error("nsteps must be >= 0");
    return SWC_ERR_BAD_PARAM;
  }
  if (!have_state_) {
    set_error("swc_step before swc_set_state");
    return SWC_ERR_STATE;
  }
  return SWC_OK;
}

// Enqueue nsteps graph launches on stream_ (host bookkeeping at enqueue time: the
// stream orders every later read of the fields after them).
template <typename T> int StepEngine<T>::enqueue_steps(int nsteps) {
  SWC_CK(cudaSetDevice(p_.device));
  last_launches_ = 0;
  for (int s = 0; s < nsteps; ++s) {
    const int64_t n = nloop_ + 1;  // nLoop after the increment at REF:1085
    const bool relax = !(n > p_.divv_switch || p_.load == 1);
    const bool last = s == nsteps - 1;
    // diagnostics: the call's last step, or every diag_interval steps (REF:2202: 50)
    const bool diag = p_.diag_interval > 0 ? (n % p_.diag_interval == 0) : last;
    SWC_TRY(run_graph(relax, n == 1, diag, last));
    if (diag) pending_diag_ = diag_step_ = n;
    nloop_ = n;
    if (p_.adjoint_ckpt > 0 && n % p_.adjoint_ckpt == 0) SWC_TRY(save_ckpt((size_t)(n / p_.adjoint_ckpt)));
  }
  have_vsol_ = true;
  vsol_pending_ = true;
  return SWC_OK;
}

// With the stream idle: the transform passes' wait status and the sums of the last
// diagnostic step enqueued since the previous check.
template <typename T> int StepEngine<T>::finish_steps() {
  double sums[5];
  int tma_status = 0;
  const int64_t diag_at = pending_diag_;
  if (diag_at >= 0) SWC_CK(cudaMemcpyAsync(sums, dsum_, sizeof(sums), cudaMemcpyDeviceToHost, stream_));
  SWC_CK(cudaMemcpyAsync(&tma_status, status_, sizeof(int), cudaMemcpyDeviceToHost, stream_));
  SWC_CK(cudaStreamSynchronize(stream_));
  pending_diag_ = -1;
  if (tma_status) {
    SWC_CK(cudaMemsetAsync(status_, 0, sizeof(int), stream_));
    SWC_CK(cudaStreamSynchronize(stream_));
    set_error("a tile copy of a transform pass did not complete in time (step %lld)", (long long)nloop_);
    return SWC_ERR_CUDA;
  }
  if (diag_at < 0) return SWC_OK;  // no diagnostic step since the last check
  // REF:2244-2258
  diag_.sum_abs_dpsi = sums[0];
  diag_.sum_abs_psi = sums[1];
  diag_.sum_rho = sums[2];
  diag_.sum_energy = sums[3];
  diag_.l1 = sums[0] / (p_.dt * sums[1]);
  diag_.mass = sums[2] * dx_ * dx_ * dx_;
  diag_.energy = sums[3] * dx_ * dx_ * dx_;
  diag_.step = diag_at;
  diag_.nonfinite = (int64_t)sums[4];
  if (diag_.nonfinite) {
    set_error("non-finite psi/rho after step %lld (%lld values)", (long long)diag_at, (long long)diag_.nonfinite);
    return SWC_ERR_NONFINITE;
  }
  return SWC_OK;
}

template <typename T> int StepEngine<T>::step(int nsteps) {
  SWC_TRY(check_step(nsteps));
  if (nsteps == 0) return SWC_OK;
  SWC_CK(cudaSetDevice(p_.device));
  SWC_CK(cudaEventRecord(ev0_, stream_));
  SWC_TRY(enqueue_steps(nsteps));
  SWC_CK(cudaEventRecord(ev1_, stream_));
  // host watchdog: poll the stream's last event, never spin on the device
  if (p_.watchdog_s > 0) {
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
      cudaError_t e = cudaEventQuery(ev1_);
      if (e == cudaSuccess) break;
      if (e != cudaErrorNotReady) {
        set_error("step failed: %s", cudaGetErrorString(e));
        return SWC_ERR_CUDA;
      }
      const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (el > p_.watchdog_s) {
        set_error("watchdog: swc_step exceeded %.3f s", p_.watchdog_s);
        return SWC_ERR_TIMEOUT;
      }
      std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
  } else {
    SWC_CK(cudaEventSynchronize(ev1_));
  }
  float ms = 0;
  SWC_CK(cudaEventElapsedTime(&ms, ev0_, ev1_));
  last_ms_ = ms;
  return finish_steps();
}

// swc_step_async: the steps are enqueued and the call returns; swc_sync (or the next
// swc_step) waits for them and reports their status and diagnostics.
template <typename T> int StepEngine<T>::step_async(int nsteps) {
  SWC_TRY(check_step(nsteps));
  if (nsteps == 0) return SWC_OK;
  return enqueue_steps(nsteps);
}

template <typename T> int StepEngine<T>::sync() {
  SWC_CK(cudaSetDevice(p_.device));
  return finish_steps();
}

template <typename T> int StepEngine<T>::field_src(int field, const void** src, bool* is_double) {
  *is_double = false;
  if ((field == SWC_F_VSOLX || field == SWC_F_VSOLY || field == SWC_F_VSOLZ) && vsol_pending_) {
    SWC_CK(cudaSetDevice(p_.device));
    SWC_TRY(transform_vsol());
    SWC_CK(cudaStreamSynchronize(stream_));
    vsol_pending_ = false;
  }
  switch (field) {
    case SWC_F_PSI: *src = psi_; break;
    case SWC_F_RHO: *src = rho_; *is_double = true; break;
    case SWC_F_AMP: *src = amp_f_; break;
    case SWC_F_DIVV: *src = divv_; break;
    case SWC_F_VX: *src = v_[0]; break;
    case SWC_F_VY: *src = v_[1]; break;
    case SWC_F_VZ: *src = v_[2]; break;
    case SWC_F_VSOLX: *src = vsolr_[0]; break;
    case SWC_F_VSOLY: *src = vsolr_[1]; break;
    case SWC_F_VSOLZ: *src = vsolr_[2]; break;
    case SWC_F_ENERGY:
      if (diag_step_ != nloop_) {
        set_error("the energy density is written at diagnostic steps only (last: step %lld, now %lld)",
                  (long long)diag_step_, (long long)nloop_);
        return SWC_ERR_STATE;
      }
      *src = energy_;
      break;
    case SWC_F_PSIQ: *src = psiq_; *is_double = true; break;
    case SWC_F_PSIQ_OLD: *src = psiq_old_; *is_double = true; break;
    case SWC_F_NLQ: *src = nlq_; break;
    case SWC_F_FRHO:  // the mixed engine keeps f_rho (an FP32 source term) in FP32
      if constexpr (std::is_same<T, double>::value) {
        *src = frho_;
        *is_double = true;
      } else {
        *src = frhot_;
        *is_double = false;
      }
      break;
    case SWC_F_LPSI: *src = lpsi_; break;
    case SWC_F_MU: *src = mu_; break;
    case SWC_F_GPSIX: *src = gp_[0]; break;
    case SWC_F_GPSIY: *src = gp_[1]; break;
    case SWC_F_GPSIZ: *src = gp_[2]; break;
    case SWC_F_GRHOX: *src = gr_[0]; break;
    case SWC_F_GRHOY: *src = gr_[1]; break;
    case SWC_F_GRHOZ: *src = gr_[2]; break;
    case SWC_F_PSI_OLD: *src = psi_old_; break;
    default:
      set_error("unknown field id %d", field);
      return SWC_ERR_BAD_PARAM;
  }
  return SWC_OK;
}

// The FP64 staging buffer of the mixed engine's host transfers (allocated on first use).
template <typename T> int StepEngine<T>::stage_alloc() {
  if (stage_) return SWC_OK;
  const size_t n = (size_t)g_.ng;
  if (cudaMalloc(&stage_, n * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    stage_ = nullptr;
    set_error("cudaMalloc of the %zu MB field staging buffer failed", (n * 8) >> 20);
    return SWC_ERR_OOM;
  }
  return SWC_OK;
}

template <typename T> int StepEngine<T>::get_field(int field, double* dst) {
  const void* src;
  bool is_d;
  SWC_TRY(field_src(field, &src, &is_d));
  SWC_CK(cudaSetDevice(p_.device));
  SWC_CK(cudaStreamSynchronize(stream_));
  const size_t n = (size_t)g_.ng;
  if (is_d || std::is_same<T, double>::value) {
    SWC_CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    SWC_CK(cudaStreamSynchronize(stream_));
  } else {
    // FP32 field: widened to FP64 on the device (staging buffer allocated on first use),
    // then one device-to-host copy straight into the caller's buffer
    SWC_TRY(stage_alloc());
    widen_kernel<<<(unsigned)((n / 4 + 255) / 256), 256, 0, stream_>>>(reinterpret_cast<const float*>(src), stage_,
                                                                       (long long)n);
    SWC_CK(cudaGetLastError());
    SWC_CK(cudaMemcpyAsync(dst, stage_, n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    SWC_CK(cudaStreamSynchronize(stream_));
  }
  return SWC_OK;
}

// Asynchronous read: the field is snapshotted in FP64 on stream_ (widened from FP32 in
// the mixed engine), and the snapshot is copied to dst on copy_stream_, so the copy
// overlaps the steps that follow. Two snapshot buffers alternate; a call first waits
// for the copy issued two calls before it (the buffer it reuses), so when it returns
// the destination of the call before last is complete. get_field_wait() completes all.
template <typename T> int StepEngine<T>::get_field_async(int field, double* dst) {
  const void* src;
  bool is_d;
  SWC_TRY(field_src(field, &src, &is_d));
  SWC_CK(cudaSetDevice(p_.device));
  const size_t n = (size_t)g_.ng;
  const int b = anext_;
  if (apending_[b]) {
    apending_[b] = false;
    SWC_CK(cudaEventSynchronize(adone_[b]));
  }
  if (!copy_stream_) SWC_CK(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking));
  if (!astage_[b]) {
    if (cudaMalloc(&astage_[b], n * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      astage_[b] = nullptr;
      set_error("cudaMalloc of the field snapshot failed (%zu MB)", (n * sizeof(double)) >> 20);
      return SWC_ERR_OOM;
    }
  }
  if (!aready_[b]) SWC_CK(cudaEventCreateWithFlags(&aready_[b], cudaEventDisableTiming));
  if (!adone_[b]) SWC_CK(cudaEventCreateWithFlags(&adone_[b], cudaEventDisableTiming));
  if (is_d || std::is_same<T, double>::value) {
    SWC_CK(cudaMemcpyAsync(astage_[b], src, n * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
  } else {
    widen_kernel<<<(unsigned)((n / 4 + 255) / 256), 256, 0, stream_>>>(reinterpret_cast<const float*>(src),
                                                                       astage_[b], (long long)n);
    SWC_CK(cudaGetLastError());
  }
  SWC_CK(cudaEventRecord(aready_[b], stream_));
  SWC_CK(cudaStreamWaitEvent(copy_stream_, aready_[b], 0));
  SWC_CK(cudaMemcpyAsync(dst, astage_[b], n * sizeof(double), cudaMemcpyDeviceToHost, copy_stream_));
  SWC_CK(cudaEventRecord(adone_[b], copy_stream_));
  apending_[b] = true;
  anext_ = b ^ 1;
  return SWC_OK;
}

template <typename T> int StepEngine<T>::get_field_wait() {
  SWC_CK(cudaSetDevice(p_.device));
  for (int b = 0; b < 2; ++b) {
    if (!apending_[b]) continue;
    apending_[b] = false;
    SWC_CK(cudaEventSynchronize(adone_[b]));
  }
  return SWC_OK;
}

template <typename T> int StepEngine<T>::field_ptr(int field, void** ptr, int* elem_bytes) {
  const void* src;
  bool is_d;
  SWC_TRY(field_src(field, &src, &is_d));
  *ptr = const_cast<void*>(src);
  *elem_bytes = is_d ? 8 : (int)sizeof(T);
  return SWC_OK;
}

// Checkpoint: header + psiq, psiq_old, rho, f_rho (FP64) + Nl_old, psi (T).
struct CkptHeader {
  char magic[8];
  int32_t version, nx, ny, nz, precision, elem;
  int64_t nloop;
};

template <typename T> int StepEngine<T>::save(const char* path) {
  if (!have_state_) {
    set_error("swc_save before swc_set_state");
    return SWC_ERR_STATE;
  }
  SWC_CK(cudaSetDevice(p_.device));
  SWC_CK(cudaStreamSynchronize(stream_));
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    set_error("cannot open %s for writing", path);
    return SWC_ERR_IO;
  }
  CkptHeader h{};
  std::memcpy(h.magic, "SWCCKPT1", 8);
  h.version = 1; h.nx = p_.nx; h.ny = p_.ny; h.nz = p_.nz; h.precision = p_.precision;
  h.elem = (int)sizeof(T); h.nloop = nloop_;
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
  const size_t n = (size_t)g_.ng;
  if constexpr (!std::is_same<T, double>::value) {  // the file holds f_rho in FP64 for both engines
    widen_kernel<<<(unsigned)((n / 4 + 255) / 256), 256, 0, stream_>>>(frhot_, frho_, (long long)n);
    SWC_CK(cudaGetLastError());
    SWC_CK(cudaStreamSynchronize(stream_));
  }
  std::vector<char> buf(n * sizeof(double));
  const void* dsrc[] = {psiq_, psiq_old_, rho_, frho_};
  for (const void* s : dsrc) {
    if (!ok) break;
    if (cudaMemcpyAsync(buf.data(), s, n * sizeof(double), cudaMemcpyDeviceToHost, stream_) != cudaSuccess ||
        cudaStreamSynchronize(stream_) != cudaSuccess)
      ok = false;
    else ok = std::fwrite(buf.data(), 1, n * sizeof(double), f) == n * sizeof(double);
  }
  const void* tsrc[] = {nlq_, psi_};
  for (const void* s : tsrc) {
    if (!ok) break;
    if (cudaMemcpyAsync(buf.data(), s, n * sizeof(T), cudaMemcpyDeviceToHost, stream_) != cudaSuccess ||
        cudaStreamSynchronize(stream_) != cudaSuccess)
      ok = false;
    else ok = std::fwrite(buf.data(), 1, n * sizeof(T), f) == n * sizeof(T);
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    set_error("writing checkpoint %s failed", path);
    return SWC_ERR_IO;
  }
  return SWC_OK;
}

template <typename T> int StepEngine<T>::load(const char* path) {
  SWC_CK(cudaSetDevice(p_.device));
  SWC_CK(cudaStreamSynchronize(stream_));
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    set_error("cannot open %s", path);
    return SWC_ERR_IO;
  }
  CkptHeader h{};
  bool ok = std::fread(&h, sizeof(h), 1, f) == 1;
  if (!ok || std::memcmp(h.magic, "SWCCKPT1", 8) != 0 || h.version != 1 || h.nx != p_.nx || h.ny != p_.ny ||
      h.nz != p_.nz || h.elem != (int)sizeof(T) || h.nloop < 0) {
    std::fclose(f);
    set_error("checkpoint %s does not match this context (grid/precision/format)", path);
    return SWC_ERR_IO;
  }
  const size_t n = (size_t)g_.ng;
  std::vector<char> buf(n * sizeof(double));
  double* ddst[] = {psiq_, psiq_old_, rho_, frho_};
  for (double* d : ddst) {
    if (!ok) break;
    ok = std::fread(buf.data(), 1, n * sizeof(double), f) == n * sizeof(double);
    if (ok) ok = cudaMemcpyAsync(d, buf.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream_) == cudaSuccess &&
                 cudaStreamSynchronize(stream_) == cudaSuccess;
  }
  T* tdst[] = {nlq_, psi_};
  for (T* d : tdst) {
    if (!ok) break;
    ok = std::fread(buf.data(), 1, n * sizeof(T), f) == n * sizeof(T);
    if (ok) ok = cudaMemcpyAsync(d, buf.data(), n * sizeof(T), cudaMemcpyHostToDevice, stream_) == cudaSuccess &&
                 cudaStreamSynchronize(stream_) == cudaSuccess;
  }
  std::fclose(f);
  if (!ok) {
    set_error("checkpoint %s is truncated or unreadable", path);
    return SWC_ERR_IO;
  }
  SWC_CK(cudaMemcpyAsync(psi_old_, psi_, n * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
  SWC_TRY(refresh_copies(1));
  SWC_CK(cudaStreamSynchronize(stream_));
  adj_valid_ = false;  // the checkpoints no longer describe this trajectory
  nloop_ = h.nloop;
  have_state_ = true;
  have_vsol_ = false;
  vsol_pending_ = false;
  std::memset(&diag_, 0, sizeof(diag_));
  diag_step_ = -1;
  pending_diag_ = -1;
  diag_.step = nloop_;
  return SWC_OK;
}

}  // namespace swc
