// swc_engine.h -- host-side interface between the C ABI (swc_abi.cu) and the
// precision-specific step engines (swc_step_fp64.cu, swc_step_mixed.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/swc.h"

namespace swc {

// Thread-local message of the last failing call (read by swc_last_error()).
void set_error(const char* fmt, ...);
const char* get_error();

class EngineBase {
 public:
  virtual ~EngineBase() {}
  virtual int set_state(const double* psi, const double* rho) = 0;
  virtual int set_state_ic(const swc_ic& ic) = 0;
  virtual int step(int nsteps) = 0;
  virtual int step_async(int nsteps) = 0;
  virtual int prepare() = 0;
  virtual int sync() = 0;
  virtual int diagnostics(swc_diag* out) = 0;
  virtual int get_field(int field, double* dst) = 0;
  virtual int get_field_async(int field, double* dst) = 0;
  virtual int get_field_wait() = 0;
  virtual int field_ptr(int field, void** ptr, int* elem_bytes) = 0;
  virtual int get_step(int64_t* n) = 0;
  virtual int last_ms(double* ms) = 0;
  virtual int last_launches(int64_t* n) = 0;
  virtual int save(const char* path) = 0;
  virtual int load(const char* path) = 0;
  virtual int backward(const double* dpsi, const double* drho, double energy_lambda, double* dpsi0, double* drho0,
                       swc_grad* out) = 0;
};

// Device initial conditions (swc_ic.cu): psi and rho (may be null) as FP64 (i,j,k)
// arrays, enqueued on `stream`.
int ic_check(const swc_ic* ic);
int ic_generate(const swc_params& p, const swc_ic& ic, double* psi, double* rho, cudaStream_t stream);

// Dense FMA throughput probe of the current device (TFLOP/s, FMA = 2 flops).
int fma_peak(int precision, double* tflops);

// Validate parameters shared by every engine. Returns SWC_OK or SWC_ERR_BAD_PARAM.
int validate_params(const swc_params* p);

// Create an engine; returns status, *out owned by the caller.
int make_engine_fp64(const swc_params& p, EngineBase** out);
int make_engine_mixed(const swc_params& p, EngineBase** out);

}  // namespace swc
