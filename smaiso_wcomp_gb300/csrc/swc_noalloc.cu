// swc_noalloc.cu -- swc_diagnostics_noalloc: the diagnostic reduction of the step
// (L1, mass, free energy) over caller-owned FP64 device fields, without allocating
// any device memory.
//
// Who needs it: callers that cannot call cudaMalloc/cudaFree at the point where they
// want the numbers -- a host code that gave this library a fixed device-memory budget
// and lets its own pool allocator own the rest of the card, a latency-critical loop
// that must not pay cudaFree's device-wide wait for outstanding work, or a job that
// may not change its device footprint after start-up on a GPU shared with others.
// The context API (swc_step + swc_diagnostics) allocates its reduction scratch with
// cudaMalloc when the context is created; this entry point uses a fixed array in the
// library image instead.
//
// Scratch: one FP64 partial sum of each of the five quantities per chunk of
// kNoAllocChunk grid points, in the file-scope array g_noalloc_scratch below
// (kNoAllocMaxChunks chunks = 160 KiB + 64 B). Every device that loads the library
// holds this array until the process exits. Grids above
// kNoAllocMaxChunks * kNoAllocChunk = 2^28 points are rejected.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>

#include "swc_engine.h"

namespace swc {
namespace {

constexpr int kNoAllocThreads = 256;
constexpr long long kNoAllocChunk = 65536;     // grid points per block
constexpr int kNoAllocMaxChunks = 4096;        // => at most 2^28 grid points
constexpr int kNoAllocMaxDevices = 64;

// [5 * kNoAllocMaxChunks] per-chunk partials, then 5 final sums (padded to 8).
static __device__ __align__(256) double g_noalloc_scratch[5 * kNoAllocMaxChunks + 8];

struct NoAllocArgs {
  const double *psi, *psi_old, *rho, *lpsi, *amp;
  long long ng;
  double ep, beta, gamma, zeta, rho0, kp;
};

// Same arithmetic as the context's diagnostic kernel (REF:2214-2231), one block per
// chunk; every block writes all five of its partials, so nothing needs clearing.
__global__ void __launch_bounds__(kNoAllocThreads) noalloc_partial_kernel(NoAllocArgs a, double* scratch) {
  __shared__ double sh[5][kNoAllocThreads / 32];
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0;
  const long long begin = (long long)blockIdx.x * kNoAllocChunk;
  long long end = begin + kNoAllocChunk;
  if (end > a.ng) end = a.ng;
  for (long long idx = begin + threadIdx.x; idx < end; idx += kNoAllocThreads) {
    const double pn = a.psi[idx], po = a.psi_old[idx], r = a.rho[idx], L = a.lpsi[idx], A = a.amp[idx];
    s0 += fabs(pn - po);
    s1 += fabs(pn);
    s2 += r;
    const double p2 = pn * pn;
    const double e = -0.5 * a.ep * p2 + 0.5 * (L * L) - 0.25 * a.beta * (p2 * p2) + (a.gamma / 6) * (p2 * p2 * p2);
    const double d = r - a.rho0 - a.kp * A;
    s3 += r * e + 0.5 * a.zeta * (d * d);
    s4 += (double)(!isfinite(pn)) + (double)(!isfinite(r));
  }
  double v[5] = {s0, s1, s2, s3, s4};
#pragma unroll
  for (int q = 0; q < 5; ++q)
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int q = 0; q < 5; ++q) sh[q][w] = v[q];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int q = 0; q < 5; ++q) {
      double t = 0;
      for (int ww = 0; ww < kNoAllocThreads / 32; ++ww) t += sh[q][ww];
      scratch[5 * blockIdx.x + q] = t;
    }
}

// Fixed-order sum of the nchunks partials into the five final slots.
__global__ void __launch_bounds__(32) noalloc_final_kernel(double* scratch, int nchunks) {
  const int q = threadIdx.x;
  if (q < 5) {
    double t = 0;
    for (int b = 0; b < nchunks; ++b) t += scratch[5 * b + q];
    scratch[5 * kNoAllocMaxChunks + q] = t;
  }
}

std::mutex g_setup_mu;
double* g_scratch_ptr[kNoAllocMaxDevices] = {};
CUcontext g_scratch_ctx[kNoAllocMaxDevices] = {};

// The driver context current on this thread (the device's primary context once the
// runtime has used the device); null if the driver entry point is unavailable.
CUcontext current_context() {
  static PFN_cuCtxGetCurrent_v4000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
  }();
  CUcontext c = nullptr;
  if (fn && fn(&c) != CUDA_SUCCESS) c = nullptr;
  return c;
}

// Set-up, with device `dev` current: the device address of the array in the module
// loaded into the device's current context. Looked up once per device, and again if
// that context has changed since (a cudaDeviceReset by the caller recreates the
// primary context, and with it the module and the array's address).
int scratch_for_current_device(int dev, double** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  const CUcontext ctx = current_context();
  if (!g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
    double* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      cudaGetLastError();
      g_scratch_ptr[dev] = nullptr;
      set_error("swc_diagnostics_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                cudaGetErrorString(e));
      return SWC_ERR_CUDA;
    }
    g_scratch_ptr[dev] = ptr;
    g_scratch_ctx[dev] = current_context();  // the lookup may have created the context
  }
  *out = g_scratch_ptr[dev];
  return SWC_OK;
}

// Makes p->device current for the call and puts the caller's device back on every
// return path.
struct DeviceScope {
  int prev = -1;
  bool changed = false;
  int enter(int dev) {
    if (dev < 0 || dev >= kNoAllocMaxDevices || cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      set_error("swc_diagnostics_noalloc: no usable CUDA device %d", dev);
      return SWC_ERR_NO_DEVICE;
    }
    if (prev != dev) {
      if (cudaSetDevice(dev) != cudaSuccess) {
        cudaGetLastError();
        set_error("swc_diagnostics_noalloc: cannot make device %d current", dev);
        return SWC_ERR_NO_DEVICE;
      }
      changed = true;
    }
    return SWC_OK;
  }
  ~DeviceScope() {
    if (changed) cudaSetDevice(prev);
  }
};

}  // namespace
}  // namespace swc

extern "C" int swc_diagnostics_noalloc(const swc_params* p, const double* psi, const double* psi_old,
                                       const double* rho, const double* lpsi, const double* amp, void* stream,
                                       swc_diag* out) {
  using namespace swc;
  int rc = validate_params(p);
  if (rc) return rc;
  const long long ng = (long long)p->nx * p->ny * p->nz;
  if (ng > (long long)kNoAllocMaxChunks * kNoAllocChunk) {
    set_error("swc_diagnostics_noalloc: %lld grid points exceed its fixed scratch (at most %lld points)", ng,
              (long long)kNoAllocMaxChunks * kNoAllocChunk);
    return SWC_ERR_BAD_PARAM;
  }
  if (!psi || !psi_old || !rho || !lpsi || !amp || !out) {
    set_error("swc_diagnostics_noalloc: NULL field or output");
    return SWC_ERR_BAD_PARAM;
  }
  DeviceScope scope;
  if ((rc = scope.enter(p->device))) return rc;
  double* scratch = nullptr;
  if ((rc = scratch_for_current_device(p->device, &scratch))) return rc;
  // REF:250-253, 267
  const double Amp = std::sqrt((3 * p->beta + std::sqrt(9 * p->beta * p->beta + 40 * p->ep * p->gamma)) / 5);
  const double kp = (1 - p->rho_0) / Amp;
  const double dx = (p->nx * 2.0 * 3.14159265358979323846 / (p->q0 * p->nw)) / p->nx;
  NoAllocArgs a{psi, psi_old, rho, lpsi, amp, ng, p->ep, p->beta, p->gamma, p->zeta, p->rho_0, kp};
  const int nchunks = (int)((ng + kNoAllocChunk - 1) / kNoAllocChunk);
  cudaStream_t s = (cudaStream_t)stream;
  noalloc_partial_kernel<<<nchunks, kNoAllocThreads, 0, s>>>(a, scratch);
  noalloc_final_kernel<<<1, 32, 0, s>>>(scratch, nchunks);
  double sums[5];
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sums, scratch + 5 * kNoAllocMaxChunks, sizeof(sums), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error("swc_diagnostics_noalloc: %s", cudaGetErrorString(e));
    return SWC_ERR_CUDA;
  }
  // REF:2244-2258
  out->sum_abs_dpsi = sums[0];
  out->sum_abs_psi = sums[1];
  out->sum_rho = sums[2];
  out->sum_energy = sums[3];
  out->l1 = sums[0] / (p->dt * sums[1]);
  out->mass = sums[2] * dx * dx * dx;
  out->energy = sums[3] * dx * dx * dx;
  out->step = -1;  // not tracked: the fields are the caller's
  out->nonfinite = (int64_t)sums[4];
  return SWC_OK;
}
