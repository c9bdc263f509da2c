/*
 * swc.h -- C ABI of the GB300 (sm_103a) semi-implicit pseudo-spectral step of the
 * weakly compressible smectic-A / isotropic phase-field model (order parameter psi,
 * density rho, quasi-static velocity v).
 *
 * The reference (smaiso-wcomp.cpp) has no plugin or FFI surface: its time loop is
 * inline in main(). This header replaces the two internal boundaries of that loop:
 *
 *   1. the transform interface -- eight FFTW-MPI r2r plans executed in place on one
 *      N^3 buffer (smaiso-wcomp.cpp:499-545, fftw_execute at 969-2197), replaced by
 *      swc_r2r_plan_create / swc_r2r_execute*;
 *   2. the model state and the loop body -- the std::vector<double> fields in
 *      (i,j,k) k-fastest layout and one pass of `while (L1 > limL1)`
 *      (smaiso-wcomp.cpp:1081-2457), replaced by swc_create / swc_set_state /
 *      swc_step / swc_diagnostics / swc_get_field.
 *
 * Conventions
 *   - Every call returns an int status: SWC_OK (0) or a negative SWC_ERR_* code.
 *     No C++ exception crosses this boundary.  swc_last_error() gives a message.
 *   - Host buffers are owned by the caller and copied in/out; the context owns all
 *     device memory, its CUDA stream and its captured CUDA graphs.
 *   - A context is single-threaded (one stream); distinct contexts are independent.
 *   - Layout of every field: row-major (i,j,k) with k fastest,
 *     index = (i*ny + j)*nz + k (smaiso-wcomp.cpp:943).
 */
#ifndef SWC_H
#define SWC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWC_ABI_VERSION 4

/* ---- status codes ---------------------------------------------------------- */
enum {
  SWC_OK = 0,
  SWC_ERR_BAD_PARAM = -1,  /* invalid argument or unsupported grid */
  SWC_ERR_OOM = -2,        /* device or host allocation failed */
  SWC_ERR_CUDA = -3,       /* a CUDA runtime call failed */
  SWC_ERR_NONFINITE = -4,  /* NaN/Inf detected in the state after a step */
  SWC_ERR_TIMEOUT = -5,    /* host-side watchdog expired waiting for the stream */
  SWC_ERR_STATE = -6,      /* call out of order (e.g. swc_step before swc_set_state) */
  SWC_ERR_IO = -7,         /* checkpoint file could not be read or written */
  SWC_ERR_NO_DEVICE = -8   /* no usable CUDA device */
};

/* ---- precision of the step ---------------------------------------------- */
enum {
  SWC_PREC_FP64 = 0,  /* every transform and pointwise term in FP64 */
  SWC_PREC_MIXED = 1  /* FP32 transforms/pointwise; FP64 state, CN/AB2 update, reductions */
};

/* ---- r2r kinds: same definitions as FFTW's REDFT10/REDFT01/RODFT10/RODFT01 --- */
enum {
  SWC_REDFT10 = 0,  /* DCT-II : Y_k = 2 sum_n X_n cos(pi (n+1/2) k / N) */
  SWC_REDFT01 = 1,  /* DCT-III: Y_k = X_0 + 2 sum_{n>=1} X_n cos(pi n (k+1/2) / N) */
  SWC_RODFT10 = 2,  /* DST-II : Y_k = 2 sum_n X_n sin(pi (n+1/2)(k+1) / N) */
  SWC_RODFT01 = 3   /* DST-III: Y_k = (-1)^k X_{N-1} + 2 sum_{n<N-1} X_n sin(pi (n+1)(k+1/2) / N) */
};

/* ---- fields readable with swc_get_field ---------------------------------- */
enum {
  SWC_F_PSI = 0,       /* psi_local (real space) */
  SWC_F_RHO = 1,       /* rho_local */
  SWC_F_AMP = 2,       /* amp_local: filtered amplitude A */
  SWC_F_DIVV = 3,      /* divv_local (real space) */
  SWC_F_VX = 4,        /* vsolx + virrx (real space), "vx.dat" */
  SWC_F_VY = 5,
  SWC_F_VZ = 6,
  SWC_F_VSOLX = 7,     /* solenoidal part, "vsolx.dat" (last step of a swc_step call) */
  SWC_F_VSOLY = 8,
  SWC_F_VSOLZ = 9,
  SWC_F_ENERGY = 10,   /* energy density of the diagnostic, "energyMid.dat" source */
  SWC_F_PSIQ = 11,     /* psiq_local: scaled DCT-II of psi */
  SWC_F_PSIQ_OLD = 12, /* psiq_old_local */
  SWC_F_NLQ = 13,      /* Nl_local after its DCT-II (becomes Nl_old next step) */
  SWC_F_FRHO = 14,     /* f_rho_local: previous density source (AB2) */
  SWC_F_LPSI = 15,     /* dfDlapPsi_local = alpha (q0^2 + lap) psi */
  SWC_F_MU = 16,       /* mu_local */
  SWC_F_GPSIX = 17,    /* psiGrad{x,y,z}_local (real space) */
  SWC_F_GPSIY = 18,
  SWC_F_GPSIZ = 19,
  SWC_F_GRHOX = 20,    /* rhoD{x,y,z}_local (real space) */
  SWC_F_GRHOY = 21,
  SWC_F_GRHOZ = 22,
  SWC_F_PSI_OLD = 23,  /* psi_old_local at the last step of a swc_step call */
  SWC_F_COUNT = 24
};

/* ---- model and run parameters (smaiso-wcomp.cpp:206-278) ------------------ */
typedef struct swc_params {
  int nx, ny, nz;     /* grid (reference: 512^3, :218); powers of two, 8..1024 */
  int nw;             /* points per wavelength: dx = 2 pi / (q0 nw)  (:261, :267) */
  double dt;          /* time step (:262) */
  double alpha;       /* (:241) */
  double beta;        /* cubic coefficient (:240) */
  double gamma;       /* quintic coefficient (:239) */
  double ep;          /* epsilon, already signed: reference ep = -0.001*argv[2] (:243) */
  double q0;          /* smectic wavenumber (:244) */
  double nu;          /* shear viscosity, reference argv[1] (:249) */
  double lambda;      /* second viscosity (:256) */
  double zeta;        /* density penalty (:257) */
  double rho_0;       /* isotropic density (:251); kp = (1-rho_0)/Amp (:253) */
  int divv_switch;    /* relax-phase length in steps (:214, reference 50) */
  int load;           /* reference load flag: 1 skips the relax phase (:176, :1312) */
  int ref_ranks;      /* MPI rank count of the reference run reproduced (x slabs);
                         decides where the slab-start v_z filter applies (:1760-1804
                         vs :1932). Must divide nx. Reference needs an even count. */
  int precision;      /* SWC_PREC_FP64 or SWC_PREC_MIXED */
  int device;         /* CUDA device ordinal */
  double watchdog_s;  /* host watchdog per swc_step call in seconds (<=0: none) */
  int adjoint_ckpt;   /* 0: no adjoint. K > 0 (FP64 engine): swc_step keeps a state
                         checkpoint every K steps so swc_backward can recompute the
                         trajectory; device memory = (steps/K + 2) states of 3 N^3
                         doubles + 3 N^3 values + one segment tape of K x 24 N^3 values
                         (values: double in the FP64 engine, float in the mixed one,
                         whose adjoint runs in FP32).
                         -1: binomial checkpointing -- swc_step keeps only the initial
                         state and swc_backward reverses the trajectory with a binomial
                         recompute schedule over as many state snapshots as fit under
                         adjoint_cap_gb, with a one-step tape. */
  double adjoint_cap_gb; /* adjoint_ckpt = -1: device memory cap of the context during
                            swc_backward, in GB (1e9 B), engine arrays included; <= 0:
                            the device's free memory at the call less 1 GB. */
  int adjoint_snapshots; /* adjoint_ckpt = -1: at most this many snapshots (<= 0: as
                            many as fit under the cap) */
  int diag_interval;  /* when the diagnostics of :2202-2262 run: 0 = at the last step of
                         every swc_step call; K > 0 = at the steps with nLoop % K == 0
                         (the reference's cadence is K = 50, :2202), so a loop of
                         swc_step(ctx, 1) calls pays for them every K steps only. The
                         non-finite check and the energy-density field come with them. */
} swc_params;

/* Gradients returned by swc_backward: dL/d(coefficient) of the coefficients the
 * calibration loss is differentiated against. */
typedef struct swc_grad {
  double alpha;  /* d/d alpha   (REF:241) */
  double beta;   /* d/d beta    (REF:240) */
  double gamma;  /* d/d gamma   (REF:239) */
  double nu;     /* d/d nu      (REF:249) */
  double rho_0;  /* d/d rho_0   (REF:251; the density ratio rho_i/rho_s, rho_s = 1) */
  int64_t steps; /* steps differentiated (nLoop at the call) */
  int64_t forward_steps;  /* forward steps rerun by the call (recompute and tape) */
  int64_t snapshots;      /* state snapshot slots used (binomial mode; 0 otherwise) */
} swc_grad;

/* Diagnostics of the last diagnostic step (smaiso-wcomp.cpp:2202-2262; see
 * swc_params.diag_interval): by default the last step of the last swc_step call. */
typedef struct swc_diag {
  double l1;          /* sum|psi-psi_old| / (dt sum|psi|)        (:2246) */
  double mass;        /* sum rho * dx^3                          (:2252) */
  double energy;      /* free energy * dx^3                      (:2258) */
  double sum_abs_dpsi;
  double sum_abs_psi;
  double sum_rho;
  double sum_energy;
  int64_t step;       /* nLoop of the step they describe */
  int64_t nonfinite;  /* count of non-finite psi/rho values */
} swc_diag;

typedef struct swc_ctx swc_ctx;
typedef struct swc_r2r_plan swc_r2r_plan;

/* Library / error helpers. */
int swc_abi_version(void);
const char* swc_strerror(int status);
/* Message of the last failing call on this thread (empty string if none). */
const char* swc_last_error(void);

/* Fill *p with the reference's hard-coded values (smaiso-wcomp.cpp:206-278) for
 * a grid of nx x ny x nz, with nu = 1 and argv[2] = 1 (ep = -0.001). */
int swc_default_params(swc_params* p, int nx, int ny, int nz);

/* Derived constants exactly as the reference computes them (:239-272). */
typedef struct swc_derived {
  double amp;    /* Amp = sqrt((3 beta + sqrt(9 beta^2 + 40 ep gamma))/5) */
  double kp;     /* (1 - rho_0)/Amp */
  double rho_s;  /* kp Amp + rho_0 */
  double rho_m;  /* rho_s / 2 */
  double dx, dy, dz, lx, ly, lz;
  double scale;  /* 0.125/(nx ny nz) */
} swc_derived;
int swc_derive(const swc_params* p, swc_derived* out);

/* ---- the time loop (replaces smaiso-wcomp.cpp:968-2262) -------------------- */

/* Validate *p, allocate the device state and capture nothing yet. */
int swc_create(const swc_params* p, swc_ctx** out);
int swc_destroy(swc_ctx* ctx);

/* Copy the initial psi (and rho; NULL means the reference's zero fill, :1053)
 * from host memory and run the pre-loop (:968-1010): psiq = scale*DCT(psi),
 * psi = iDCT(psiq), psiq_old = psiq, step counter = 0. */
int swc_set_state(swc_ctx* ctx, const double* psi, const double* rho);

/* Advance nsteps time steps (each one loop body :1084-2198). The diagnostics of
 * :2202-2262 run at the last step of the call (swc_params.diag_interval = 0, the
 * default) or at every diag_interval-th step; the last step also keeps the solenoidal
 * velocity. Steps run as captured CUDA graphs on the context's stream; the call
 * returns after the stream is idle. Returns SWC_ERR_NONFINITE if the call's last
 * diagnostic step found NaN/Inf in psi or rho. */
int swc_step(swc_ctx* ctx, int nsteps);

/* Capture now the CUDA graphs of every step variant (relax / normal phase, first
 * step, diagnostic step, v_sol written or not), which swc_step otherwise captures on
 * first use, so that no later swc_step call pays for a capture (a loop timed or run
 * under a latency budget). Runs no step. Needs swc_set_state first. */
int swc_prepare(swc_ctx* ctx);

/* swc_step without the wait: the nsteps graph launches are enqueued on the context's
 * stream and the call returns, so the host can enqueue the next step (or a field
 * read, swc_get_field_async) while the device runs. The steps' status -- a transform
 * pass whose tile wait ran out, the diagnostics of the last diagnostic step enqueued
 * (swc_params.diag_interval) and its non-finite check -- is collected by the next
 * swc_sync or swc_step call. swc_get_field waits for the steps before reading. */
int swc_step_async(swc_ctx* ctx, int nsteps);

/* Wait for every step enqueued by swc_step_async and return their status
 * (SWC_ERR_NONFINITE, SWC_ERR_CUDA, ...); the diagnostics become readable. */
int swc_sync(swc_ctx* ctx);

/* Read the diagnostics of the last diagnostic step that swc_step or swc_sync collected. */
int swc_diagnostics(swc_ctx* ctx, swc_diag* out);

/* Copy one field (SWC_F_*) to host memory as nx*ny*nz doubles. Pinned (page-locked)
 * host memory gets a direct DMA copy; the mixed engine widens FP32 fields on the
 * device into a staging buffer it allocates on the first such call. The energy
 * density (SWC_F_ENERGY) exists after a diagnostic step only (else SWC_ERR_STATE). */
int swc_get_field(swc_ctx* ctx, int field, double* dst);

/* Asynchronous swc_get_field for a field read after every step (the loop's output,
 * REF:2273-2446, taken more often than the reference's every 500 steps): the field is
 * snapshotted in FP64 on the context's stream (widened from FP32 by the mixed engine)
 * and copied to dst on a second stream, so the copy overlaps the swc_step calls that
 * follow. dst must stay valid until the copy completes, and must be pinned host memory
 * for the copy to run asynchronously. Two snapshot buffers (2 * nx*ny*nz doubles,
 * allocated on the first call) alternate: a call first waits for the copy issued two
 * calls before it, so when it returns the destination of that earlier call holds
 * its field; swc_get_field_wait completes every pending copy. Errors of a copy are
 * returned by the call that waits for it. */
int swc_get_field_async(swc_ctx* ctx, int field, double* dst);
int swc_get_field_wait(swc_ctx* ctx);

/* Device pointer of a field in the context's own precision (8-byte elements for
 * FP64 fields, 4-byte for FP32 work fields of the mixed path); *elem_bytes tells
 * which. Valid until swc_destroy. */
int swc_field_device_ptr(swc_ctx* ctx, int field, void** dev_ptr, int* elem_bytes);

/* Step counter (nLoop of the reference). */
int swc_get_step(swc_ctx* ctx, int64_t* nloop);

/* Elapsed device time (ms) of the kernels of the last swc_step call, measured
 * with CUDA events on the context's stream. */
int swc_last_step_ms(swc_ctx* ctx, double* ms);

/* Number of kernels the last swc_step call launched (all steps of the call). */
int swc_last_step_launches(swc_ctx* ctx, int64_t* launches);

/* Dense FMA throughput of the current device in TFLOP/s (FMA = 2 flops) for
 * precision SWC_PREC_FP64 (double) or SWC_PREC_MIXED (float): independent FMA
 * chains on every SM, timed with CUDA events. Used as the roofline denominator of
 * the ALU-bound FP64 kernels. */
int swc_device_fma_peak(int precision, double* tflops);

/* Allocation-free variant of the diagnostic reduction. No counterpart in the
 * reference (its sums are plain loops, REF:2214-2231); same arithmetic as the
 * reduction behind swc_diagnostics, applied to caller-owned FP64 device fields of
 * nx*ny*nz doubles: psi (new), psi_old, rho, lpsi (dfDlapPsi) and amp, all on device
 * p->device. Geometry and coefficients come from *p (only dt, nw, q0, ep, beta, gamma,
 * zeta, rho_0 and device are read besides the grid). The call makes p->device current
 * while it runs and restores the caller's current device before it returns; `stream`
 * (a cudaStream_t, NULL = legacy default stream) must belong to that device. Result in
 * *out (step = -1); the call returns after the stream has finished the reduction.
 *
 * For callers that must not allocate device memory at this point: a host code that
 * gave this library a fixed device budget and lets its own allocator own the rest, a
 * latency-critical loop that cannot pay cudaFree's wait for all outstanding device
 * work, or a job that may not grow its device footprint on a shared GPU. It calls no
 * cudaMalloc/cudaFree and no allocating library routine: its scratch is a fixed
 * 160 KiB array inside the library, held by every device that loads the library until
 * the process exits. Limits and rules:
 *   - at most SWC_NOALLOC_MAX_POINTS grid points (SWC_ERR_BAD_PARAM beyond);
 *   - the first call on a device looks up the array's device address (set-up, once
 *     per device, with the device current; again after the device's context changed,
 *     e.g. after a cudaDeviceReset): make that first call before any stream capture;
 *   - every call shares the one array per device: calls that overlap on the GPU (on
 *     different streams or threads) race. Each call writes every scratch slot it
 *     reads, so no clearing is needed between calls. */
#define SWC_NOALLOC_MAX_POINTS (1LL << 28)
int swc_diagnostics_noalloc(const swc_params* p, const double* psi, const double* psi_old, const double* rho,
                            const double* lpsi, const double* amp, void* stream, swc_diag* out);

/* ---- initial conditions generated on the device (replaces smaiso-wcomp.cpp:556-722) */
enum {
  SWC_IC_BAND = 0,         /* REF:575-590: psi = Amp cos(q0 k dz) written at k2 = k + round(phi
                              sin(Qi i dx)) for Nz/2-8 < k < Nz/2+8, 0 elsewhere; rho = 0 */
  SWC_IC_FLAT = 1,         /* flat smectic/isotropic interface at Lz/2, layers parallel to it:
                              psi = h(z) A cos(q0 z) + U(-noise, noise), h = (1 + tanh((z - Lz/2)/xi))/2;
                              rho = rho_i + (rho_s - rho_i) h */
  SWC_IC_UNDULATED = 2,    /* the same with the interface at z0(x,y) = Lz/2 + 2 (2 pi/q0)
                              sin(2 pi x/Lx) cos(2 pi y/Ly) and Gaussian psi noise of sigma = noise;
                              rho = rho_i + (rho_s - rho_i) h */
  SWC_IC_DISLOCATIONS = 3, /* psi = h A cos(q0 z + sum_c atan2(z - z_c, x - x_c)): ncores edge
                              dislocations at seeded (x_c, z_c) below a flat interface at 3Lz/4,
                              h = (1 - tanh((z - 3Lz/4)/xi))/2; rho = rho_0 + (1 - rho_0) h */
  SWC_IC_FOCAL_CONIC = 4,  /* REF:594-639 (commented out in the reference): one focal conic of
                              size aE = bE = ae at the bottom of the box; rho = 0 */
  SWC_IC_FOCAL_CONICS = 5  /* REF:641-707 (commented out): two focal conics side by side along
                              x, the second of size ae + gap; rho = 0 */
};

/* Parameters of a device initial condition (swc_default_ic fills the defaults of a kind).
 * Noise and seeded positions come from SplitMix64(seed XOR linear index): uniform
 * U[0,1) = top 53 bits; Gaussian by Box-Muller on the index pair (2m, 2m+1). */
typedef struct swc_ic {
  int kind;         /* SWC_IC_* */
  int ncores;       /* DISLOCATIONS: number of cores */
  uint64_t seed;
  double amp;       /* IC amplitude A; <= 0: the model's Amp (REF:250), as BAND and the focal
                       conics use */
  double xi;        /* interface width */
  double noise;     /* FLAT: uniform half-width; UNDULATED: Gaussian sigma */
  double rho_s, rho_i;  /* FLAT, UNDULATED: densities of the smectic and isotropic sides */
  double phi, qi;   /* BAND: layer perturbation amplitude and wavenumber (REF:282-283, 584) */
  double ae, gap;   /* FOCAL_CONIC(S): size aE = bE (reference argv[3], REF:230-231) and the
                       second conic's extra size (REF:227) */
} swc_ic;

/* Defaults of an initial condition of `kind` for the grid of *p (the values of the
 * benchmark workloads for FLAT, UNDULATED and DISLOCATIONS; the reference's for BAND;
 * ae = 3 nz/8 for the focal conics). */
int swc_default_ic(const swc_params* p, int kind, swc_ic* ic);

/* Write the initial psi and rho (nx*ny*nz doubles each, (i,j,k) layout) of *ic into
 * caller-owned device memory (rho may be NULL), enqueued on `stream` (a cudaStream_t,
 * NULL = legacy default stream), on the current device. Allocates nothing. */
int swc_ic_generate(const swc_params* p, const swc_ic* ic, double* dev_psi, double* dev_rho, void* stream);

/* swc_set_state with the initial state generated on the device (no host arrays):
 * psi and rho of *ic, then the pre-loop (:968-1010). */
int swc_set_state_ic(swc_ctx* ctx, const swc_ic* ic);

/* ---- discrete adjoint of the time loop ------------------------------------
 * No counterpart in the reference. Differentiates L(psi(T), rho(T)) after the
 * swc_step calls made since swc_set_state (T = nLoop), given the host cotangents
 * dL_dpsi = dL/dpsi(T) and dL_drho = dL/drho(T) (either may be NULL = zero), by the
 * hand-written transpose of every stage of the step (transposed r2r transforms,
 * adjoint pointwise terms, transposed staggered Stokes solve, adjoint CN/AB2
 * update). Recomputes the trajectory segment by segment from the checkpoints kept
 * by swc_step (params.adjoint_ckpt). Outputs dL/dpsi0 and dL/drho0 with respect to
 * the arrays passed to swc_set_state (host, nx*ny*nz doubles, either may be NULL)
 * and the coefficient gradients in *grad. The FP64 engine differentiates in FP64, the
 * mixed engine in FP32 (on its own trajectory); the context's state is the state at
 * step T again when the call returns. Steps enqueued by swc_step_async are waited for
 * and their status returned first (as swc_sync). */
int swc_backward(swc_ctx* ctx, const double* dL_dpsi, const double* dL_drho, double* dL_dpsi0,
                 double* dL_drho0, swc_grad* grad);

/* swc_backward for a loss with the free-energy diagnostic of the last step added:
 * L = L_user(psi(T), rho(T)) + lambda * E(T), E(T) the energy of REF:2214-2258 at step
 * T = nLoop: dx^3 sum [rho (-ep/2 psi^2 + (dfDlapPsi)^2/2 - beta/4 psi^4 + gamma/6 psi^6)
 * + zeta/2 (rho - rho_0 - kp A)^2] with the new psi and rho of step T and the stale
 * dfDlapPsi (REF:2227) and the filtered amplitude A computed during step T (the value
 * swc_diagnostics reports for step T). dL_dpsi / dL_drho are the cotangents of L_user
 * (either may be NULL); lambda = 0 is swc_backward. The coefficient gradients include
 * E's direct dependence on beta, gamma, rho_0 and, through Amp and kp, on beta, gamma
 * and rho_0 (REF:250-253). No counterpart in the reference. */
int swc_backward_energy(swc_ctx* ctx, double lambda, const double* dL_dpsi, const double* dL_drho,
                        double* dL_dpsi0, double* dL_drho0, swc_grad* grad);

/* ---- full-state checkpoint (lossless; the reference's psi<rank>.dat text dump
 *      at :2334-2345 keeps only psi at 6 digits) ------------------------------ */
int swc_save(swc_ctx* ctx, const char* path);
int swc_load(swc_ctx* ctx, const char* path);

/* ---- r2r transforms (replaces fftw_mpi_plan_r2r_3d + fftw_execute,
 *      smaiso-wcomp.cpp:499-545) --------------------------------------------- */

/* Plan a 3D r2r transform of an nx x ny x nz array with one SWC_REDFT10/01,
 * SWC_RODFT10/01 kind per axis (kx along x = slowest index). precision selects
 * double (SWC_PREC_FP64) or float (SWC_PREC_MIXED) data. Unnormalised, like FFTW:
 * a forward/inverse pair multiplies by 2n per axis. */
int swc_r2r_plan_create(int nx, int ny, int nz, int kx, int ky, int kz, int precision,
                        swc_r2r_plan** out);
int swc_r2r_plan_destroy(swc_r2r_plan* plan);

/* In-place execution on device memory (double* or float* per the plan, 16-byte
 * aligned, as cudaMalloc returns; SWC_ERR_BAD_PARAM otherwise), enqueued on
 * `stream` (a cudaStream_t; NULL = legacy default stream). Allocates nothing. */
int swc_r2r_execute(swc_r2r_plan* plan, void* dev_inout, void* stream);

/* One axis pass of the plan (axis 0 = x, 1 = y, 2 = z), in place on device memory;
 * swc_r2r_execute is the passes z, y, x in turn. */
int swc_r2r_execute_axis(swc_r2r_plan* plan, int axis, void* dev_inout, void* stream);

/* Host convenience: copies in, transforms, copies out (out may equal in). The
 * data is double on the host for both precisions. */
int swc_r2r_execute_host(swc_r2r_plan* plan, const double* in, double* out);

/* Test support for the bounded waits of the FP32 TMA-fed passes (no counterpart in the
 * reference): every tile wait of this plan expects extra_tx_bytes (0..65536) more bytes
 * than its copy delivers, so it runs out after max_polls (1..2^22) mbarrier polls; the
 * CTA then sets the plan's status flag and returns, and the next swc_r2r_execute_host
 * reports SWC_ERR_CUDA. (0, 1 << 22) restores normal operation. */
int swc_r2r_plan_set_wait_test(swc_r2r_plan* plan, int extra_tx_bytes, int max_polls);

#ifdef __cplusplus
}
#endif
#endif /* SWC_H */
