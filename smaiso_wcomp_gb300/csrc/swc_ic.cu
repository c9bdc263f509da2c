// swc_ic.cu -- initial conditions generated on the device (swc_ic_generate,
// swc_set_state_ic): the reference's own band state (smaiso-wcomp.cpp:571-590) with its
// layer perturbation, its two commented-out focal-conic states (:594-707), and the
// synthetic workload states -- flat and undulated smectic/isotropic interfaces and
// layer dislocations -- whose host form is smaiso_wcomp_gb300/ic.py. A 512x512x256
// state is written straight into device memory: no host arrays, no host-to-device
// copy.
//
// One thread per grid point, FP64. Counter-based noise: value(index) =
// f(SplitMix64(seed ^ index)), the integer hash of ic.py, so the uniform noise is bit
// for bit the host generator's and any subset of points can be regenerated alone.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "swc_common.cuh"
#include "swc_engine.h"

namespace swc {
namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// U[0,1) from the top 53 bits
__device__ __forceinline__ double uniform01(uint64_t seed, uint64_t index) {
  return (double)(splitmix64(seed ^ index) >> 11) * (1.0 / 9007199254740992.0);
}

struct IcArgs {
  Grid g;
  swc_ic ic;
  double amp;            // A (the model's Amp where ic.amp <= 0)
  double rho_0;          // the model's rho_0 (dislocations)
  double dx, dy, dz, lx, ly, lz, q0;
  double* psi;
  double* rho;           // may be null
};

__global__ void __launch_bounds__(256) ic_kernel(IcArgs a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= a.g.ng) return;
  const Grid& g = a.g;
  const int k = (int)(idx & (g.nz - 1)), j = (int)((idx >> g.lz) & (g.ny - 1)), i = (int)(idx >> (g.ly + g.lz));
  const swc_ic& c = a.ic;
  const double pi = 3.14159265358979323846;
  const double x = i * a.dx, y = j * a.dy, z = k * a.dz;
  double psi = 0.0, rho = 0.0;
  switch (c.kind) {
    case SWC_IC_BAND: {
      // REF:575-590: Amp cos(q0 k dz) stored at k2 = k + round(phi sin(Qi i dx)), band
      // Nz/2 - 8 < k < Nz/2 + 8; the point (i, j, k_out) holds the band value of k_out - shift
      const int shift = (int)round(c.phi * sin(c.qi * i * a.dx));
      const int ks = k - shift;
      if (ks > g.nz / 2 - 8 && ks < g.nz / 2 + 8) psi = a.amp * cos(a.q0 * ks * a.dz);
      break;
    }
    case SWC_IC_FLAT: {
      const double h = 0.5 * (1.0 + tanh((z - a.lz / 2) / c.xi));
      // the noise product and the sum rounded separately (no contraction), as the host
      // generator computes them: the uniform noise is bit for bit ic.py's
      psi = __dadd_rn(h * a.amp * cos(a.q0 * z), __dmul_rn(2.0 * uniform01(c.seed, (uint64_t)idx) - 1.0, c.noise));
      rho = c.rho_i + (c.rho_s - c.rho_i) * h;
      break;
    }
    case SWC_IC_UNDULATED: {
      const double z0 = a.lz / 2 + 2.0 * (2.0 * pi / a.q0) * sin(2 * pi * x / a.lx) * cos(2 * pi * y / a.ly);
      const double h = 0.5 * (1.0 + tanh((z - z0) / c.xi));
      // Box-Muller on the counter pair (2m, 2m + 1): cos for the even index, sin for the odd
      const uint64_t m2 = (uint64_t)idx & ~1ull;
      const double u1 = uniform01(c.seed, m2), u2 = uniform01(c.seed, m2 + 1);
      const double r = sqrt(-2.0 * log1p(-u1));
      const double gn = (idx & 1) ? r * sin(2.0 * pi * u2) : r * cos(2.0 * pi * u2);
      psi = __dadd_rn(h * a.amp * cos(a.q0 * z), __dmul_rn(gn, c.noise));
      rho = c.rho_i + (c.rho_s - c.rho_i) * h;
      break;
    }
    case SWC_IC_DISLOCATIONS: {
      double theta = 0.0;
      for (int q = 0; q < c.ncores; ++q) {
        const double xk = uniform01(c.seed, 2 * (uint64_t)q) * a.lx;
        const double zk = (0.15 + 0.45 * uniform01(c.seed, 2 * (uint64_t)q + 1)) * a.lz;
        theta += atan2(z - zk, x - xk);
      }
      const double h = 0.5 * (1.0 - tanh((z - 0.75 * a.lz) / c.xi));
      psi = h * a.amp * cos(a.q0 * z + theta);
      rho = a.rho_0 + (1.0 - a.rho_0) * h;
      break;
    }
    case SWC_IC_FOCAL_CONIC:
    case SWC_IC_FOCAL_CONICS: {
      // REF:594-639 (one conic) and REF:641-707 (two along x, the second ae + gap)
      const double mid = (double)(g.ny / 2);
      int i2 = i;
      double aE = c.ae, bE = c.ae;
      if (c.kind == SWC_IC_FOCAL_CONICS && i >= g.nx / 2) {
        i2 = i - g.nx / 2;
        aE = c.ae + c.gap;
        bE = c.ae + c.gap;
      }
      if (k < bE + 1) {
        const double xs = i2 - mid, ys = j - mid, zs = k;
        const double ds = sqrt(xs * xs + ys * ys);
        if (ds < mid) {
          const double ex = (ds - mid) / aE, ez = zs / bE;
          if (!(sqrt(ex * ex + ez * ez) > 1)) {
            const double w = (bE / aE) * (ds - mid);
            psi = a.amp * cos(a.q0 * a.dz * sqrt(w * w + zs * zs));
          }
        } else if (fabs(zs) < bE) {
          psi = a.amp * cos(a.q0 * zs * a.dz);
        }
      }
      break;
    }
    default:
      break;
  }
  a.psi[idx] = psi;
  if (a.rho) a.rho[idx] = rho;
}

}  // namespace

int ic_check(const swc_ic* ic) {
  if (!ic || ic->kind < SWC_IC_BAND || ic->kind > SWC_IC_FOCAL_CONICS) {
    set_error("unknown initial-condition kind");
    return SWC_ERR_BAD_PARAM;
  }
  if ((ic->kind == SWC_IC_FLAT || ic->kind == SWC_IC_UNDULATED || ic->kind == SWC_IC_DISLOCATIONS) &&
      !(ic->xi > 0)) {
    set_error("initial condition: xi must be > 0");
    return SWC_ERR_BAD_PARAM;
  }
  if (ic->kind == SWC_IC_DISLOCATIONS && (ic->ncores < 0 || ic->ncores > 4096)) {
    set_error("initial condition: ncores must be in [0, 4096]");
    return SWC_ERR_BAD_PARAM;
  }
  if ((ic->kind == SWC_IC_FOCAL_CONIC || ic->kind == SWC_IC_FOCAL_CONICS) && !(ic->ae > 0 && ic->ae + ic->gap > 0)) {
    set_error("initial condition: focal-conic size ae (and ae + gap) must be > 0");
    return SWC_ERR_BAD_PARAM;
  }
  return SWC_OK;
}

int ic_generate(const swc_params& p, const swc_ic& ic, double* psi, double* rho, cudaStream_t stream) {
  int rc = ic_check(&ic);
  if (rc) return rc;
  swc_derived d;
  swc_derive(&p, &d);
  IcArgs a;
  a.g = make_grid(p.nx, p.ny, p.nz);
  a.ic = ic;
  a.amp = ic.amp > 0 ? ic.amp : d.amp;
  a.rho_0 = p.rho_0;
  a.dx = d.dx; a.dy = d.dy; a.dz = d.dz;
  a.lx = d.lx; a.ly = d.ly; a.lz = d.lz;
  a.q0 = p.q0;
  a.psi = psi;
  a.rho = rho;
  ic_kernel<<<(unsigned)((a.g.ng + 255) / 256), 256, 0, stream>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("initial-condition kernel: %s", cudaGetErrorString(e));
    return SWC_ERR_CUDA;
  }
  return SWC_OK;
}

}  // namespace swc

extern "C" int swc_default_ic(const swc_params* p, int kind, swc_ic* ic) {
  using namespace swc;
  if (!p || !ic) {
    set_error("NULL argument");
    return SWC_ERR_BAD_PARAM;
  }
  *ic = swc_ic{};
  ic->kind = kind;
  ic->xi = 2.0;
  ic->rho_s = 1.0;
  switch (kind) {
    case SWC_IC_BAND:  // REF:281-283: Qi = 0.125/2, phi = 0 (the perturbation is off)
      ic->qi = 0.125 / 2;
      break;
    case SWC_IC_FLAT:
      ic->seed = 1001; ic->amp = 0.8; ic->noise = 1e-4; ic->rho_i = 0.9;
      break;
    case SWC_IC_UNDULATED:
      ic->seed = 1002; ic->amp = 0.8; ic->noise = 1e-3; ic->rho_i = 0.8;
      break;
    case SWC_IC_DISLOCATIONS:
      ic->seed = 1003; ic->amp = 0.8; ic->ncores = 16;
      break;
    case SWC_IC_FOCAL_CONIC:
    case SWC_IC_FOCAL_CONICS:
      ic->ae = 3.0 * p->nz / 8;
      break;
    default:
      set_error("unknown initial-condition kind %d", kind);
      return SWC_ERR_BAD_PARAM;
  }
  return SWC_OK;
}

extern "C" int swc_ic_generate(const swc_params* p, const swc_ic* ic, double* dev_psi, double* dev_rho,
                               void* stream) {
  using namespace swc;
  int rc = validate_params(p);
  if (rc) return rc;
  if (!ic || !dev_psi) {
    set_error("NULL initial condition or psi");
    return SWC_ERR_BAD_PARAM;
  }
  return ic_generate(*p, *ic, dev_psi, dev_rho, (cudaStream_t)stream);
}
