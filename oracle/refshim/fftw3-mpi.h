/*
 * fftw3-mpi.h -- stand-in for FFTW3-MPI and the MPI-2 C++ bindings, wide enough to
 * compile smaiso-wcomp.cpp and to run it as P processes on one host.
 *
 * TEST INFRASTRUCTURE ONLY: it builds oracle/_ref/smaiso_wcomp_ref, whose outputs
 * pin the oracle's restatement of the time loop. Nothing in the product uses it.
 *
 * The reference includes <fftw3-mpi.h> only (smaiso-wcomp.cpp:36), which normally
 * pulls in <mpi.h> and <fftw3.h>; this header declares exactly the part of those
 * three APIs the file calls:
 *   - MPI::Init / Finalize, COMM_WORLD.Get_rank / Get_size / Send / Recv / Reduce /
 *     Bcast / Gather / Barrier, MPI::DOUBLE, MPI::SUM (:109, :293-297, :1122-1162,
 *     :1520-1564, :1730-1752, :1993-2035, :2237-2265, :2317-2332);
 *   - fftw_mpi_init, fftw_mpi_local_size_3d, fftw_mpi_plan_r2r_3d, fftw_execute,
 *     fftw_destroy_plan, fftw_cleanup with the REDFT10/01 and RODFT10/01 kinds
 *     (:294, :299, :499-545, :969-2197, :2483-2492).
 * The ranks are forked processes sharing one anonymous mapping: point-to-point
 * messages go through mailboxes (buffered sends, FIFO per source/destination/tag,
 * so the reference's even/odd send-receive orderings cannot deadlock), collectives
 * through a shared buffer and a process-shared barrier. A 3D r2r execution gathers
 * every rank's x slab into the shared buffer, transforms the whole array with the
 * oracle's r2r (swco_r2r3d, pinned to scipy golden vectors) and scatters it back:
 * the data layout and the unnormalised FFTW definitions are those of the plans
 * (x slabs, k fastest, output not transposed).
 *
 * The swc_ref_* hooks are called from the few lines the build recipe (oracle/Makefile,
 * target `ref`) substitutes into the source stream: grid size, step count, initial
 * psi, output directory, and two read-only probes of the loop's arrays.
 */
#ifndef SWC_REFSHIM_FFTW3_MPI_H
#define SWC_REFSHIM_FFTW3_MPI_H

#include <cstddef>
#include <string>

namespace MPI {

struct Datatype {
  int bytes;
};
struct Op {
  int code;
};
extern const Datatype DOUBLE;
extern const Op SUM;

class Intracomm {
 public:
  int Get_rank() const;
  int Get_size() const;
  void Send(const void* buf, int count, const Datatype& type, int dest, int tag) const;
  void Recv(void* buf, int count, const Datatype& type, int source, int tag) const;
  void Reduce(const void* sendbuf, void* recvbuf, int count, const Datatype& type, const Op& op,
              int root) const;
  void Bcast(void* buf, int count, const Datatype& type, int root) const;
  void Gather(const void* sendbuf, int sendcount, const Datatype& sendtype, void* recvbuf,
              int recvcount, const Datatype& recvtype, int root) const;
  void Barrier() const;
};

extern Intracomm COMM_WORLD;

void Init();
/* Ends the rank's process (after a barrier and a flush): the reference's main()
 * has no return statement after it. */
[[noreturn]] void Finalize();

}  // namespace MPI

/* FFTW kinds used by the reference; the values are the oracle's kind codes. */
typedef enum {
  FFTW_REDFT10 = 0,
  FFTW_REDFT01 = 1,
  FFTW_RODFT10 = 2,
  FFTW_RODFT01 = 3
} fftw_r2r_kind;

#define FFTW_MEASURE (0U)

typedef struct swc_ref_plan* fftw_plan;

void fftw_mpi_init();
ptrdiff_t fftw_mpi_local_size_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, const MPI::Intracomm& comm,
                                 ptrdiff_t* local_n0, ptrdiff_t* local_0_start);
fftw_plan fftw_mpi_plan_r2r_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double* in, double* out,
                               const MPI::Intracomm& comm, fftw_r2r_kind kind0, fftw_r2r_kind kind1,
                               fftw_r2r_kind kind2, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);
void fftw_cleanup();

/* ---- hooks behind the recipe's substitutions ------------------------------ */

/* Grid extent along axis 0 (x), 1 (y), 2 (z): SWC_REF_NX/NY/NZ. */
ptrdiff_t swc_ref_dim(int axis);
/* Output root replacing "/box" (:184, :198): SWC_REF_DIR. */
std::string swc_ref_box();
/* Step limit added to `while (L1 > limL1)` (:1081): SWC_REF_STEPS. */
long swc_ref_nsteps();
/* After the reference's own initial condition (:575-590): if SWC_REF_PSI0 names a
 * file of nx*ny*nz doubles in (i,j,k) order, the rank's slab of psi_local is read
 * from it instead. */
void swc_ref_initial_psi(double* psi_local, ptrdiff_t local_n0, ptrdiff_t local_0_start);

/* End of each loop pass: at the steps listed in SWC_REF_DUMP the 24 fields below are
 * written (each rank its slab, FP64, (i,j,k) order) to SWC_REF_DIR/dump/s<step>_<name>.bin. */
enum { SWC_REF_NFIELDS = 24 };
void swc_ref_after_step(int nloop, ptrdiff_t local_n0, ptrdiff_t local_0_start,
                        const double* const* fields, const double* const* vsol,
                        const double* const* virr);
/* After the diagnostics' broadcast (:2265): rank 0 appends the step's sums, full
 * precision, to SWC_REF_DIR/dump/diag.txt. */
void swc_ref_diag(int nloop, double l1, double sum_a, double sum_b, double mass, double energy);

/* The probes name the reference's own local variables (:345-436); the field order
 * is the C ABI's SWC_F_* order, with the velocity sums formed by the hook. */
#define SWC_REF_AFTER_STEP()                                                                       \
  do {                                                                                             \
    const double* swc_ref_f_[SWC_REF_NFIELDS] = {                                                  \
        psi_local.data(),      rho_local.data(),       amp_local.data(),      divv_local.data(),   \
        nullptr,               nullptr,                nullptr,               vsolx_local.data(),  \
        vsoly_local.data(),    vsolz_local.data(),     energy_local.data(),   psiq_local.data(),   \
        psiq_old_local.data(), Nl_local.data(),        f_rho_local.data(),    dfDlapPsi_local.data(), \
        mu_local.data(),       psiGradx_local.data(),  psiGrady_local.data(), psiGradz_local.data(), \
        rhoDx_local.data(),    rhoDy_local.data(),     rhoDz_local.data(),    psi_old_local.data()}; \
    const double* swc_ref_vs_[3] = {vsolx_local.data(), vsoly_local.data(), vsolz_local.data()};   \
    const double* swc_ref_vi_[3] = {virrx_local.data(), virry_local.data(), virrz_local.data()};   \
    swc_ref_after_step((int)nLoop, local_n0, local_0_start, swc_ref_f_, swc_ref_vs_, swc_ref_vi_);  \
  } while (0)

#define SWC_REF_DIAG() swc_ref_diag((int)nLoop, L1, sumA, sumB, rho_sum, energy)

#endif /* SWC_REFSHIM_FFTW3_MPI_H */
