// swc_abi.cu -- the extern "C" entry points of include/swc.h (context API) and the
// shared parameter validation. Each call maps status codes, never lets a C++
// exception cross the boundary and records a message for swc_last_error().
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <new>
#include <string>

#include "swc_engine.h"

namespace swc {

// Independent FMA chains per thread (8 per thread, no memory traffic in the loop).
template <typename T> __global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) x[q] = (T)(threadIdx.x + q) * (T)1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = x[q] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) s += x[q];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T> static int fma_peak_t(double* tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    set_error("no CUDA device");
    return SWC_ERR_NO_DEVICE;
  }
  const int blocks = sms * 8, threads = 256;
  const int iters = sizeof(T) == 8 ? 4096 : 65536;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * (size_t)blocks * threads) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaMalloc failed");
    return SWC_ERR_OOM;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int w = 0; w < 2; ++w) fma_probe_kernel<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0);
    fma_probe_kernel<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) {
    set_error("FMA probe failed: %s", cudaGetErrorString(err));
    return SWC_ERR_CUDA;
  }
  *tflops = 2.0 * 8 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
  return SWC_OK;
}

int fma_peak(int precision, double* tflops) {
  return precision == SWC_PREC_FP64 ? fma_peak_t<double>(tflops) : fma_peak_t<float>(tflops);
}

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}
const char* get_error() { return g_last_error.c_str(); }

static bool pow2_in(int n, int lo, int hi) { return n >= lo && n <= hi && (n & (n - 1)) == 0; }

int validate_params(const swc_params* p) {
  if (!p) { set_error("params is NULL"); return SWC_ERR_BAD_PARAM; }
  if (!pow2_in(p->nx, 4, 1024) || !pow2_in(p->ny, 4, 1024) || !pow2_in(p->nz, 4, 1024)) {
    set_error("grid %dx%dx%d: each extent must be a power of two in [4, 1024]", p->nx, p->ny, p->nz);
    return SWC_ERR_BAD_PARAM;
  }
  if (p->nw < 1 || !(p->dt > 0) || !(p->q0 > 0) || !(p->nu > 0) || !(p->lambda + 2 * p->nu != 0)) {
    set_error("need nw >= 1, dt > 0, q0 > 0, nu > 0, lambda + 2 nu != 0");
    return SWC_ERR_BAD_PARAM;
  }
  const double disc = 9 * p->beta * p->beta + 40 * p->ep * p->gamma;
  if (!(disc >= 0) || !((3 * p->beta + std::sqrt(disc)) > 0)) {
    set_error("Amp = sqrt((3 beta + sqrt(9 beta^2 + 40 ep gamma))/5) is not real and positive");
    return SWC_ERR_BAD_PARAM;
  }
  if (p->ref_ranks < 1 || p->nx % p->ref_ranks != 0) {
    set_error("ref_ranks=%d must be >= 1 and divide nx=%d", p->ref_ranks, p->nx);
    return SWC_ERR_BAD_PARAM;
  }
  if (p->diag_interval < 0) {
    set_error("diag_interval must be >= 0");
    return SWC_ERR_BAD_PARAM;
  }
  if (p->adjoint_ckpt < -1) {
    set_error("adjoint_ckpt must be -1 (binomial), 0 or K > 0");
    return SWC_ERR_BAD_PARAM;
  }
  if (p->divv_switch < 0 || (p->precision != SWC_PREC_FP64 && p->precision != SWC_PREC_MIXED) || p->device < 0) {
    set_error("bad divv_switch / precision / device");
    return SWC_ERR_BAD_PARAM;
  }
  return SWC_OK;
}

}  // namespace swc

struct swc_ctx {
  swc::EngineBase* eng;
};

using swc::set_error;

#define SWC_GUARD(expr)                                   \
  try {                                                   \
    return (expr);                                        \
  } catch (const std::bad_alloc&) {                       \
    set_error("host allocation failed");                  \
    return SWC_ERR_OOM;                                   \
  } catch (...) {                                         \
    set_error("unexpected C++ exception");                \
    return SWC_ERR_CUDA;                                  \
  }

#define SWC_NEED_CTX(ctx)                                 \
  if (!(ctx) || !(ctx)->eng) {                            \
    set_error("null context");                            \
    return SWC_ERR_BAD_PARAM;                             \
  }

extern "C" {

int swc_abi_version(void) { return SWC_ABI_VERSION; }

const char* swc_strerror(int s) {
  switch (s) {
    case SWC_OK: return "ok";
    case SWC_ERR_BAD_PARAM: return "bad parameter";
    case SWC_ERR_OOM: return "out of memory";
    case SWC_ERR_CUDA: return "CUDA error";
    case SWC_ERR_NONFINITE: return "non-finite values in the state";
    case SWC_ERR_TIMEOUT: return "watchdog timeout";
    case SWC_ERR_STATE: return "call out of order";
    case SWC_ERR_IO: return "checkpoint I/O error";
    case SWC_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char* swc_last_error(void) { return swc::get_error(); }

int swc_default_params(swc_params* p, int nx, int ny, int nz) {
  if (!p) { set_error("params is NULL"); return SWC_ERR_BAD_PARAM; }
  p->nx = nx; p->ny = ny; p->nz = nz;
  p->nw = 8;          // :261
  p->dt = 0.001;      // :262
  p->alpha = 1.0;     // :241
  p->beta = 2.0;      // :240
  p->gamma = 1.0;     // :239
  p->ep = -0.001;     // :243 with argv[2] = 1
  p->q0 = 1.0;        // :244
  p->nu = 1.0;        // :249 (argv[1])
  p->lambda = 1.0;    // :256
  p->zeta = 1.0;      // :257
  p->rho_0 = 0.01;    // :251
  p->divv_switch = 50;  // :214
  p->load = 0;
  p->ref_ranks = 2;
  p->precision = SWC_PREC_FP64;
  p->device = 0;
  p->watchdog_s = 0.0;
  p->adjoint_ckpt = 0;
  p->adjoint_cap_gb = 0.0;
  p->adjoint_snapshots = 0;
  p->diag_interval = 0;
  return SWC_OK;
}

int swc_derive(const swc_params* p, swc_derived* o) {
  if (!p || !o) { set_error("NULL argument"); return SWC_ERR_BAD_PARAM; }
  const double pi = 3.14159265358979323846;
  o->amp = std::sqrt((3 * p->beta + std::sqrt(9 * p->beta * p->beta + 40 * p->ep * p->gamma)) / 5);
  o->kp = (1 - p->rho_0) / o->amp;
  o->rho_s = o->kp * o->amp + p->rho_0;
  o->rho_m = o->rho_s / 2;
  o->lx = p->nx * 2.0 * pi / (p->q0 * p->nw);
  o->ly = p->ny * 2.0 * pi / (p->q0 * p->nw);
  o->lz = p->nz * 2.0 * pi / (p->q0 * p->nw);
  o->dx = o->lx / p->nx; o->dy = o->ly / p->ny; o->dz = o->lz / p->nz;
  o->scale = 0.125 / ((double)p->nx * p->ny * p->nz);
  return SWC_OK;
}

int swc_create(const swc_params* p, swc_ctx** out) {
  SWC_GUARD(([&]() -> int {
    if (!out) { set_error("out is NULL"); return SWC_ERR_BAD_PARAM; }
    *out = nullptr;
    int rc = swc::validate_params(p);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= p->device) {
      cudaGetLastError();
      set_error("no CUDA device %d available", p->device);
      return SWC_ERR_NO_DEVICE;
    }
    swc::EngineBase* eng = nullptr;
    rc = (p->precision == SWC_PREC_FP64) ? swc::make_engine_fp64(*p, &eng) : swc::make_engine_mixed(*p, &eng);
    if (rc) return rc;
    *out = new swc_ctx{eng};
    return SWC_OK;
  }()));
}

int swc_destroy(swc_ctx* ctx) {
  if (!ctx) return SWC_OK;
  delete ctx->eng;
  delete ctx;
  return SWC_OK;
}

int swc_set_state(swc_ctx* ctx, const double* psi, const double* rho) {
  SWC_NEED_CTX(ctx);
  if (!psi) { set_error("psi is NULL"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->set_state(psi, rho));
}

int swc_set_state_ic(swc_ctx* ctx, const swc_ic* ic) {
  SWC_NEED_CTX(ctx);
  const int rc = swc::ic_check(ic);
  if (rc) return rc;
  SWC_GUARD(ctx->eng->set_state_ic(*ic));
}

int swc_step(swc_ctx* ctx, int nsteps) {
  SWC_NEED_CTX(ctx);
  SWC_GUARD(ctx->eng->step(nsteps));
}

int swc_prepare(swc_ctx* ctx) {
  SWC_NEED_CTX(ctx);
  SWC_GUARD(ctx->eng->prepare());
}

int swc_step_async(swc_ctx* ctx, int nsteps) {
  SWC_NEED_CTX(ctx);
  SWC_GUARD(ctx->eng->step_async(nsteps));
}

int swc_sync(swc_ctx* ctx) {
  SWC_NEED_CTX(ctx);
  SWC_GUARD(ctx->eng->sync());
}

int swc_diagnostics(swc_ctx* ctx, swc_diag* out) {
  SWC_NEED_CTX(ctx);
  if (!out) { set_error("out is NULL"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->diagnostics(out));
}

int swc_get_field(swc_ctx* ctx, int field, double* dst) {
  SWC_NEED_CTX(ctx);
  if (!dst) { set_error("dst is NULL"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->get_field(field, dst));
}

int swc_get_field_async(swc_ctx* ctx, int field, double* dst) {
  SWC_NEED_CTX(ctx);
  if (!dst) { set_error("dst is NULL"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->get_field_async(field, dst));
}

int swc_get_field_wait(swc_ctx* ctx) {
  SWC_NEED_CTX(ctx);
  SWC_GUARD(ctx->eng->get_field_wait());
}

int swc_field_device_ptr(swc_ctx* ctx, int field, void** dev_ptr, int* elem_bytes) {
  SWC_NEED_CTX(ctx);
  if (!dev_ptr || !elem_bytes) { set_error("NULL output"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->field_ptr(field, dev_ptr, elem_bytes));
}

int swc_get_step(swc_ctx* ctx, int64_t* nloop) {
  SWC_NEED_CTX(ctx);
  if (!nloop) { set_error("NULL output"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->get_step(nloop));
}

int swc_last_step_ms(swc_ctx* ctx, double* ms) {
  SWC_NEED_CTX(ctx);
  if (!ms) { set_error("NULL output"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->last_ms(ms));
}

int swc_last_step_launches(swc_ctx* ctx, int64_t* n) {
  SWC_NEED_CTX(ctx);
  if (!n) { set_error("NULL output"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->last_launches(n));
}

int swc_device_fma_peak(int precision, double* tflops) {
  if (!tflops || (precision != SWC_PREC_FP64 && precision != SWC_PREC_MIXED)) {
    set_error("bad argument");
    return SWC_ERR_BAD_PARAM;
  }
  return swc::fma_peak(precision, tflops);
}

int swc_backward(swc_ctx* ctx, const double* dL_dpsi, const double* dL_drho, double* dL_dpsi0, double* dL_drho0,
                 swc_grad* grad) {
  SWC_NEED_CTX(ctx);
  if (!grad) { set_error("grad is NULL"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->backward(dL_dpsi, dL_drho, 0.0, dL_dpsi0, dL_drho0, grad));
}

int swc_backward_energy(swc_ctx* ctx, double lambda, const double* dL_dpsi, const double* dL_drho,
                        double* dL_dpsi0, double* dL_drho0, swc_grad* grad) {
  SWC_NEED_CTX(ctx);
  if (!grad) { set_error("grad is NULL"); return SWC_ERR_BAD_PARAM; }
  if (!std::isfinite(lambda)) { set_error("lambda is not finite"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->backward(dL_dpsi, dL_drho, lambda, dL_dpsi0, dL_drho0, grad));
}

int swc_save(swc_ctx* ctx, const char* path) {
  SWC_NEED_CTX(ctx);
  if (!path) { set_error("path is NULL"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->save(path));
}

int swc_load(swc_ctx* ctx, const char* path) {
  SWC_NEED_CTX(ctx);
  if (!path) { set_error("path is NULL"); return SWC_ERR_BAD_PARAM; }
  SWC_GUARD(ctx->eng->load(path));
}

}  // extern "C"
