// swc_plan.cu -- r2r transform plans: the drop-in for fftw_mpi_plan_r2r_3d +
// fftw_execute (smaiso-wcomp.cpp:499-545) on one GPU. A 3D transform is three
// in-place axis passes (z, y, x); the plan owns only its twiddle tables.
#include <cstdint>
#include <cuda_runtime.h>

#include <new>
#include <vector>

#include "swc_engine.h"
#include "swc_r2r.cuh"
#include "swc_tables.cuh"

using namespace swc;

struct swc_r2r_plan {
  Grid g;
  int kind[3];
  int precision;
  int device;
  std::vector<void*> allocs;
  R2RTables<double> td[3];
  R2RTables<float> tf[3];
  int* status = nullptr;  // set by a pass whose bounded wait ran out; read by swc_r2r_execute_host
};

namespace {

template <typename T>
int upload_tables(swc_r2r_plan* p, int axis, int n, R2RTables<T>* out) {
  HostTables<T> ht(n);
  const std::vector<T>* src[3] = {&ht.fft, &ht.post, &ht.pre};
  const cx_t<T>** dst[3] = {&out->fft, &out->post, &out->pre};
  for (int q = 0; q < 3; ++q) {
    void* ptr = nullptr;
    const size_t bytes = src[q]->size() * sizeof(T);
    if (cudaMalloc(&ptr, bytes) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc for r2r tables failed");
      return SWC_ERR_OOM;
    }
    p->allocs.push_back(ptr);
    if (cudaMemcpy(ptr, src[q]->data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("uploading r2r tables failed");
      return SWC_ERR_CUDA;
    }
    *dst[q] = (const cx_t<T>*)ptr;
  }
  (void)axis;
  return SWC_OK;
}

template <typename T> cudaError_t run_axis(const swc_r2r_plan* p, int axis, T* data, cudaStream_t s) {
  const R2RTables<T>& tb = std::is_same<T, double>::value ? *(const R2RTables<T>*)&p->td[axis]
                                                          : *(const R2RTables<T>*)&p->tf[axis];
  // FFTW kind -> kernel kind: REDFT10 = DCT-II, REDFT01 = DCT-III, RODFT10 = DST-II, RODFT01 = DST-III
  const LdPlain<T, T> ld{data};
  const StPlain<T, T> st{data};
  switch (p->kind[axis] * 3 + axis) {
#define SWC_CASE(KD, K)                                                                              \
  case KD * 3 + 0: return launch_pass<T, K, 0>(p->g, tb, s, ld, st, NoMul<T>());                   \
  case KD * 3 + 1: return launch_pass<T, K, 1>(p->g, tb, s, ld, st, NoMul<T>());                   \
  case KD * 3 + 2: return launch_pass<T, K, 2>(p->g, tb, s, ld, st, NoMul<T>());
    SWC_CASE(SWC_REDFT10, K_C2)
    SWC_CASE(SWC_REDFT01, K_C3)
    SWC_CASE(SWC_RODFT10, K_S2)
    SWC_CASE(SWC_RODFT01, K_S3)
#undef SWC_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <typename T> int execute(const swc_r2r_plan* p, void* dev, cudaStream_t s) {
  for (int axis = 2; axis >= 0; --axis) {
    cudaError_t e = run_axis<T>(p, axis, (T*)dev, s);
    if (e != cudaSuccess) {
      set_error("r2r pass failed: %s", cudaGetErrorString(e));
      return SWC_ERR_CUDA;
    }
  }
  return SWC_OK;
}

}  // namespace

extern "C" {

int swc_r2r_plan_create(int nx, int ny, int nz, int kx, int ky, int kz, int precision, swc_r2r_plan** out) {
  if (!out) { set_error("out is NULL"); return SWC_ERR_BAD_PARAM; }
  *out = nullptr;
  const int dims[3] = {nx, ny, nz}, kinds[3] = {kx, ky, kz};
  for (int a = 0; a < 3; ++a) {
    if (!is_pow2(dims[a]) || dims[a] < 4 || dims[a] > 1024) {
      set_error("r2r extent %d: must be a power of two in [4, 1024]", dims[a]);
      return SWC_ERR_BAD_PARAM;
    }
    if (kinds[a] < SWC_REDFT10 || kinds[a] > SWC_RODFT01) {
      set_error("unknown r2r kind %d", kinds[a]);
      return SWC_ERR_BAD_PARAM;
    }
  }
  if (precision != SWC_PREC_FP64 && precision != SWC_PREC_MIXED) {
    set_error("precision must be SWC_PREC_FP64 or SWC_PREC_MIXED");
    return SWC_ERR_BAD_PARAM;
  }
  int dev = 0, ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    set_error("no CUDA device");
    return SWC_ERR_NO_DEVICE;
  }
  swc_r2r_plan* p = new (std::nothrow) swc_r2r_plan();
  if (!p) { set_error("host allocation failed"); return SWC_ERR_OOM; }
  p->g.nx = nx; p->g.ny = ny; p->g.nz = nz;
  p->g.lx = ilog2(nx); p->g.ly = ilog2(ny); p->g.lz = ilog2(nz);
  p->g.ng = (long long)nx * ny * nz;
  p->precision = precision;
  p->device = dev;
  {
    void* st = nullptr;  // status flag of the passes' bounded waits
    if (cudaMalloc(&st, sizeof(int)) != cudaSuccess || cudaMemset(st, 0, sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc for the plan status failed");
      swc_r2r_plan_destroy(p);
      return SWC_ERR_OOM;
    }
    p->allocs.push_back(st);
    p->status = (int*)st;
  }
  for (int a = 0; a < 3; ++a) {
    p->td[a].status = p->status;
    p->tf[a].status = p->status;
    p->kind[a] = kinds[a];
    p->tf[a].rev = a == 1;  // the y pass walks down the i planes the z pass before it left in L2
    const int rc = precision == SWC_PREC_FP64 ? upload_tables<double>(p, a, dims[a], &p->td[a])
                                              : upload_tables<float>(p, a, dims[a], &p->tf[a]);
    if (rc) { swc_r2r_plan_destroy(p); return rc; }
  }
  // the uploads ran on the legacy stream; execution may use any (non-blocking) stream
  if (cudaDeviceSynchronize() != cudaSuccess) {
    set_error("r2r plan: table upload failed");
    swc_r2r_plan_destroy(p);
    return SWC_ERR_CUDA;
  }
  *out = p;
  return SWC_OK;
}

int swc_r2r_plan_destroy(swc_r2r_plan* p) {
  if (!p) return SWC_OK;
  for (void* a : p->allocs) cudaFree(a);
  delete p;
  return SWC_OK;
}

int swc_r2r_execute(swc_r2r_plan* p, void* dev_inout, void* stream) {
  if (!p || !dev_inout) { set_error("NULL plan or buffer"); return SWC_ERR_BAD_PARAM; }
  if (reinterpret_cast<uintptr_t>(dev_inout) % 16 != 0) {  // the passes move 16-byte vectors
    set_error("device buffer must be 16-byte aligned");
    return SWC_ERR_BAD_PARAM;
  }
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWC_PREC_FP64 ? execute<double>(p, dev_inout, s) : execute<float>(p, dev_inout, s);
}

int swc_r2r_execute_axis(swc_r2r_plan* p, int axis, void* dev_inout, void* stream) {
  if (!p || !dev_inout || axis < 0 || axis > 2) { set_error("bad plan, buffer or axis"); return SWC_ERR_BAD_PARAM; }
  if (reinterpret_cast<uintptr_t>(dev_inout) % 16 != 0) {
    set_error("device buffer must be 16-byte aligned");
    return SWC_ERR_BAD_PARAM;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const cudaError_t e = p->precision == SWC_PREC_FP64 ? run_axis<double>(p, axis, (double*)dev_inout, s)
                                                      : run_axis<float>(p, axis, (float*)dev_inout, s);
  if (e != cudaSuccess) {
    set_error("r2r pass failed: %s", cudaGetErrorString(e));
    return SWC_ERR_CUDA;
  }
  return SWC_OK;
}

int swc_r2r_plan_set_wait_test(swc_r2r_plan* p, int extra_tx_bytes, int max_polls) {
  if (!p || extra_tx_bytes < 0 || extra_tx_bytes > 65536 || max_polls < 1 || max_polls > (1 << 22)) {
    set_error("bad plan or wait-test arguments");
    return SWC_ERR_BAD_PARAM;
  }
  for (int a = 0; a < 3; ++a) {
    p->tf[a].wait_extra_tx = p->td[a].wait_extra_tx = extra_tx_bytes;
    p->tf[a].max_polls = p->td[a].max_polls = max_polls;
  }
  return SWC_OK;
}

int swc_r2r_execute_host(swc_r2r_plan* p, const double* in, double* out) {
  if (!p || !in || !out) { set_error("NULL argument"); return SWC_ERR_BAD_PARAM; }
  const size_t n = (size_t)p->g.ng;
  const size_t elem = p->precision == SWC_PREC_FP64 ? sizeof(double) : sizeof(float);
  void* dev = nullptr;
  if (cudaMalloc(&dev, n * elem) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaMalloc for r2r data failed");
    return SWC_ERR_OOM;
  }
  int rc = SWC_OK;
  std::vector<float> tmp;
  if (elem == sizeof(double)) {
    if (cudaMemcpy(dev, in, n * elem, cudaMemcpyHostToDevice) != cudaSuccess) rc = SWC_ERR_CUDA;
  } else {
    tmp.assign(in, in + n);
    if (cudaMemcpy(dev, tmp.data(), n * elem, cudaMemcpyHostToDevice) != cudaSuccess) rc = SWC_ERR_CUDA;
  }
  if (!rc) rc = swc_r2r_execute(p, dev, nullptr);
  if (!rc) {
    if (elem == sizeof(double)) {
      if (cudaMemcpy(out, dev, n * elem, cudaMemcpyDeviceToHost) != cudaSuccess) rc = SWC_ERR_CUDA;
    } else {
      if (cudaMemcpy(tmp.data(), dev, n * elem, cudaMemcpyDeviceToHost) != cudaSuccess) rc = SWC_ERR_CUDA;
      else for (size_t i = 0; i < n; ++i) out[i] = tmp[i];
    }
  }
  if (rc == SWC_ERR_CUDA) set_error("r2r host execution: CUDA copy failed");
  cudaFree(dev);
  int st = 0;
  if (!rc && cudaMemcpy(&st, p->status, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && st) {
    cudaMemset(p->status, 0, sizeof(int));
    set_error("r2r host execution: a tile copy did not complete in time");
    rc = SWC_ERR_CUDA;
  }
  return rc;
}

}  // extern "C"
