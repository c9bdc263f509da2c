/*
 * refshim.cpp -- process-level MPI and FFTW-MPI stand-in behind fftw3-mpi.h.
 *
 * TEST INFRASTRUCTURE ONLY (builds oracle/_ref/smaiso_wcomp_ref, the reference run
 * that pins the oracle). The product never links it.
 *
 * main() here forks SWC_REF_RANKS processes; each runs the reference's main()
 * (renamed swc_ref_main by the recipe) as one MPI rank. They share one anonymous
 * mapping holding a process-shared mutex and condition variable, the mailboxes of
 * the point-to-point messages and one nx*ny*nz buffer used by the collectives and
 * by the 3D transforms. Every wait is bounded (SWC_REF_TIMEOUT_S, default 600 s):
 * a rank that waits longer reports where and exits non-zero, and the parent then
 * ends the other ranks it forked.
 */
#include "fftw3-mpi.h"

#include <fcntl.h>
#include <pthread.h>
#include <signal.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <sys/wait.h>
#include <time.h>
#include <unistd.h>

#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <iostream>
#include <set>
#include <vector>

extern "C" int swco_r2r3d(int nx, int ny, int nz, int kx, int ky, int kz, const double* in, double* out,
                          int direct);
int swc_ref_main(int argc, char* argv[]);

namespace {

constexpr int kMaxRanks = 64;
constexpr int kSlotsPerRank = 8;

struct MsgSlot {
  int used;
  int src, dst, tag;
  long seq;
  long bytes;
};

struct Shared {
  pthread_mutex_t mu;
  pthread_cond_t cv;
  int size;
  int bar_count;
  unsigned bar_gen;
  long seq;
  MsgSlot slot[kMaxRanks * kSlotsPerRank];
};

Shared* g_sh = nullptr;
char* g_msg = nullptr;       // slot data, g_msg_bytes each
long g_msg_bytes = 0;
double* g_buf = nullptr;     // nx*ny*nz doubles
int g_rank = -1;
int g_size = 0;
long g_dims[3] = {0, 0, 0};
double g_timeout_s = 600.0;
std::string g_dir;

[[noreturn]] void die(const char* what) {
  std::fprintf(stderr, "refshim rank %d: %s\n", g_rank, what);
  std::fflush(stderr);
  _exit(3);
}

long env_long(const char* name, long dflt) {
  const char* s = std::getenv(name);
  if (!s || !*s) return dflt;
  char* end = nullptr;
  const long v = std::strtol(s, &end, 10);
  if (!end || *end) {
    std::fprintf(stderr, "refshim: %s=%s is not an integer\n", name, s);
    std::exit(2);
  }
  return v;
}

void deadline(struct timespec* ts) {
  clock_gettime(CLOCK_MONOTONIC, ts);
  ts->tv_sec += (time_t)g_timeout_s;
}

// Wait on the shared condition with the mutex held; exits on timeout.
void wait_locked(const struct timespec& until, const char* where) {
  const int rc = pthread_cond_timedwait(&g_sh->cv, &g_sh->mu, &until);
  if (rc == ETIMEDOUT) {
    pthread_mutex_unlock(&g_sh->mu);
    char msg[160];
    std::snprintf(msg, sizeof msg, "timed out in %s", where);
    die(msg);
  }
}

void barrier(const char* where) {
  struct timespec until;
  deadline(&until);
  pthread_mutex_lock(&g_sh->mu);
  const unsigned gen = g_sh->bar_gen;
  if (++g_sh->bar_count == g_sh->size) {
    g_sh->bar_count = 0;
    g_sh->bar_gen++;
    pthread_cond_broadcast(&g_sh->cv);
  } else {
    while (gen == g_sh->bar_gen) wait_locked(until, where);
  }
  pthread_mutex_unlock(&g_sh->mu);
}

void check_peer(int peer, const char* op) {
  if (peer < 0 || peer >= g_size) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "%s addresses rank %d of %d (the reference's halo exchanges name a missing rank "
                  "only with one rank or an odd rank count)",
                  op, peer, g_size);
    die(msg);
  }
}

struct RefPlan {
  long n[3];
  int kind[3];
  double* in;
  double* out;
};

std::set<long>& dump_steps() {
  static std::set<long> steps;
  static bool parsed = false;
  if (!parsed) {
    parsed = true;
    const char* s = std::getenv("SWC_REF_DUMP");
    while (s && *s) {
      char* end = nullptr;
      const long v = std::strtol(s, &end, 10);
      if (end == s) break;
      steps.insert(v);
      s = (*end == ',') ? end + 1 : end;
    }
  }
  return steps;
}

const char* const kFieldNames[SWC_REF_NFIELDS] = {
    "psi",  "rho", "amp",  "divv",  "vx",    "vy",    "vz",    "vsolx",
    "vsoly", "vsolz", "energy", "psiq", "psiq_old", "nlq", "frho", "lpsi",
    "mu",   "gpsix", "gpsiy", "gpsiz", "grhox", "grhoy", "grhoz", "psi_old"};

void write_slab(const std::string& path, const double* data, long count, long offset) {
  const int fd = ::open(path.c_str(), O_CREAT | O_WRONLY, 0644);
  if (fd < 0) die("cannot open a dump file");
  const char* p = reinterpret_cast<const char*>(data);
  size_t left = (size_t)count * sizeof(double);
  off_t at = (off_t)offset * (off_t)sizeof(double);
  while (left > 0) {
    const ssize_t w = ::pwrite(fd, p, left, at);
    if (w <= 0) die("short write to a dump file");
    p += w;
    at += w;
    left -= (size_t)w;
  }
  ::close(fd);
}

}  // namespace

/* ---- MPI ------------------------------------------------------------------- */

namespace MPI {

const Datatype DOUBLE = {8};
const Op SUM = {0};
Intracomm COMM_WORLD;

void Init() {
  if (!g_sh) die("MPI::Init outside the forked ranks");
}

void Finalize() {
  barrier("MPI::Finalize");
  std::cout.flush();
  std::fflush(nullptr);
  std::exit(0);
}

int Intracomm::Get_rank() const { return g_rank; }
int Intracomm::Get_size() const { return g_size; }

void Intracomm::Send(const void* buf, int count, const Datatype& type, int dest, int tag) const {
  check_peer(dest, "Send");
  const long bytes = (long)count * type.bytes;
  if (bytes < 0 || bytes > g_msg_bytes) die("Send larger than one y-z slice");
  struct timespec until;
  deadline(&until);
  pthread_mutex_lock(&g_sh->mu);
  for (;;) {
    for (int s = 0; s < g_size * kSlotsPerRank; ++s) {
      MsgSlot& m = g_sh->slot[s];
      if (m.used) continue;
      std::memcpy(g_msg + (long)s * g_msg_bytes, buf, (size_t)bytes);
      m.src = g_rank;
      m.dst = dest;
      m.tag = tag;
      m.bytes = bytes;
      m.seq = g_sh->seq++;
      m.used = 1;
      pthread_cond_broadcast(&g_sh->cv);
      pthread_mutex_unlock(&g_sh->mu);
      return;
    }
    wait_locked(until, "Send (no free mailbox slot)");
  }
}

void Intracomm::Recv(void* buf, int count, const Datatype& type, int source, int tag) const {
  check_peer(source, "Recv");
  const long bytes = (long)count * type.bytes;
  struct timespec until;
  deadline(&until);
  pthread_mutex_lock(&g_sh->mu);
  for (;;) {
    int best = -1;
    for (int s = 0; s < g_size * kSlotsPerRank; ++s) {
      const MsgSlot& m = g_sh->slot[s];
      if (m.used && m.src == source && m.dst == g_rank && m.tag == tag &&
          (best < 0 || m.seq < g_sh->slot[best].seq))
        best = s;
    }
    if (best >= 0) {
      MsgSlot& m = g_sh->slot[best];
      if (m.bytes != bytes) {
        pthread_mutex_unlock(&g_sh->mu);
        die("Recv count differs from the matching Send");
      }
      std::memcpy(buf, g_msg + (long)best * g_msg_bytes, (size_t)bytes);
      m.used = 0;
      pthread_cond_broadcast(&g_sh->cv);
      pthread_mutex_unlock(&g_sh->mu);
      return;
    }
    wait_locked(until, "Recv");
  }
}

// Collectives stage through the shared buffer; their sums run in rank order.
void Intracomm::Reduce(const void* sendbuf, void* recvbuf, int count, const Datatype& type,
                       const Op& op, int root) const {
  if (type.bytes != 8 || op.code != SUM.code) die("Reduce supports MPI::DOUBLE with MPI::SUM");
  check_peer(root, "Reduce");
  std::memcpy(g_buf + (long)g_rank * count, sendbuf, sizeof(double) * (size_t)count);
  barrier("Reduce");
  if (g_rank == root) {
    double* out = static_cast<double*>(recvbuf);
    for (int e = 0; e < count; ++e) {
      double s = 0.0;
      for (int r = 0; r < g_size; ++r) s += g_buf[(long)r * count + e];
      out[e] = s;
    }
  }
  barrier("Reduce");
}

void Intracomm::Bcast(void* buf, int count, const Datatype& type, int root) const {
  check_peer(root, "Bcast");
  const size_t bytes = (size_t)count * (size_t)type.bytes;
  if (g_rank == root) std::memcpy(g_buf, buf, bytes);
  barrier("Bcast");
  if (g_rank != root) std::memcpy(buf, g_buf, bytes);
  barrier("Bcast");
}

void Intracomm::Gather(const void* sendbuf, int sendcount, const Datatype& sendtype, void* recvbuf,
                       int recvcount, const Datatype& recvtype, int root) const {
  check_peer(root, "Gather");
  const size_t sbytes = (size_t)sendcount * (size_t)sendtype.bytes;
  const size_t rbytes = (size_t)recvcount * (size_t)recvtype.bytes;
  if (sbytes != rbytes) die("Gather with different send and receive sizes");
  char* base = reinterpret_cast<char*>(g_buf);
  std::memcpy(base + (size_t)g_rank * sbytes, sendbuf, sbytes);
  barrier("Gather");
  if (g_rank == root) std::memcpy(recvbuf, base, sbytes * (size_t)g_size);
  barrier("Gather");
}

void Intracomm::Barrier() const { barrier("Barrier"); }

}  // namespace MPI

/* ---- FFTW-MPI -------------------------------------------------------------- */

void fftw_mpi_init() {}
void fftw_cleanup() {}

ptrdiff_t fftw_mpi_local_size_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, const MPI::Intracomm&,
                                 ptrdiff_t* local_n0, ptrdiff_t* local_0_start) {
  if (n0 != g_dims[0] || n1 != g_dims[1] || n2 != g_dims[2]) die("local_size_3d: grid mismatch");
  const ptrdiff_t block = n0 / g_size;
  *local_n0 = block;
  *local_0_start = block * g_rank;
  return block * n1 * n2;
}

fftw_plan fftw_mpi_plan_r2r_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double* in, double* out,
                               const MPI::Intracomm&, fftw_r2r_kind kind0, fftw_r2r_kind kind1,
                               fftw_r2r_kind kind2, unsigned) {
  RefPlan* p = new RefPlan;
  p->n[0] = n0;
  p->n[1] = n1;
  p->n[2] = n2;
  p->kind[0] = kind0;
  p->kind[1] = kind1;
  p->kind[2] = kind2;
  p->in = in;
  p->out = out;
  return reinterpret_cast<fftw_plan>(p);
}

void fftw_execute(const fftw_plan plan) {
  const RefPlan* p = reinterpret_cast<const RefPlan*>(plan);
  const long plane = p->n[1] * p->n[2];
  const long block = p->n[0] / g_size;
  const long slab = block * plane;
  double* mine = g_buf + (long)g_rank * slab;
  std::memcpy(mine, p->in, sizeof(double) * (size_t)slab);
  barrier("fftw_execute (gather)");
  if (g_rank == 0 && swco_r2r3d((int)p->n[0], (int)p->n[1], (int)p->n[2], p->kind[0], p->kind[1],
                                p->kind[2], g_buf, g_buf, 0) != 0)
    die("swco_r2r3d failed");
  barrier("fftw_execute (transform)");
  std::memcpy(p->out, mine, sizeof(double) * (size_t)slab);
  barrier("fftw_execute (scatter)");
}

void fftw_destroy_plan(fftw_plan plan) { delete reinterpret_cast<RefPlan*>(plan); }

/* ---- hooks ----------------------------------------------------------------- */

ptrdiff_t swc_ref_dim(int axis) { return (ptrdiff_t)g_dims[axis]; }

std::string swc_ref_box() { return g_dir; }

long swc_ref_nsteps() { return env_long("SWC_REF_STEPS", LONG_MAX); }

void swc_ref_initial_psi(double* psi_local, ptrdiff_t local_n0, ptrdiff_t local_0_start) {
  const char* path = std::getenv("SWC_REF_PSI0");
  if (!path || !*path) return;
  const long plane = g_dims[1] * g_dims[2];
  const int fd = ::open(path, O_RDONLY);
  if (fd < 0) die("cannot open SWC_REF_PSI0");
  char* p = reinterpret_cast<char*>(psi_local);
  size_t left = (size_t)(local_n0 * plane) * sizeof(double);
  off_t at = (off_t)(local_0_start * plane) * (off_t)sizeof(double);
  while (left > 0) {
    const ssize_t r = ::pread(fd, p, left, at);
    if (r <= 0) die("SWC_REF_PSI0 is shorter than nx*ny*nz doubles");
    p += r;
    at += r;
    left -= (size_t)r;
  }
  ::close(fd);
}

void swc_ref_after_step(int nloop, ptrdiff_t local_n0, ptrdiff_t local_0_start,
                        const double* const* fields, const double* const* vsol,
                        const double* const* virr) {
  if (!dump_steps().count(nloop)) return;
  const long plane = g_dims[1] * g_dims[2];
  const long count = local_n0 * plane;
  const long offset = local_0_start * plane;
  std::vector<double> sum((size_t)count);
  for (int f = 0; f < SWC_REF_NFIELDS; ++f) {
    const double* src = fields[f];
    if (!src) {  // v = v_sol + v_irr, the sum the reference writes to vx.dat (:2388-2396)
      const int c = f - 4;
      for (long e = 0; e < count; ++e) sum[(size_t)e] = vsol[c][e] + virr[c][e];
      src = sum.data();
    }
    write_slab(g_dir + "/dump/s" + std::to_string(nloop) + "_" + kFieldNames[f] + ".bin", src, count,
               offset);
  }
}

void swc_ref_diag(int nloop, double l1, double sum_a, double sum_b, double mass, double energy) {
  if (g_rank != 0) return;
  const std::string path = g_dir + "/dump/diag.txt";
  FILE* f = std::fopen(path.c_str(), "a");
  if (!f) die("cannot open diag.txt");
  std::fprintf(f, "%d %.17g %.17g %.17g %.17g %.17g\n", nloop, l1, sum_a, sum_b, mass, energy);
  std::fclose(f);
}

/* ---- launcher -------------------------------------------------------------- */

int main(int argc, char* argv[]) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s nu ep_arg aE load   (reference argv; env SWC_REF_*)\n", argv[0]);
    return 2;
  }
  g_dims[0] = env_long("SWC_REF_NX", 0);
  g_dims[1] = env_long("SWC_REF_NY", 0);
  g_dims[2] = env_long("SWC_REF_NZ", 0);
  g_size = (int)env_long("SWC_REF_RANKS", 2);
  g_timeout_s = (double)env_long("SWC_REF_TIMEOUT_S", 600);
  const char* dir = std::getenv("SWC_REF_DIR");
  if (g_dims[0] < 2 || g_dims[1] < 2 || g_dims[2] < 2 || !dir || !*dir) {
    std::fprintf(stderr, "refshim: set SWC_REF_NX, SWC_REF_NY, SWC_REF_NZ and SWC_REF_DIR\n");
    return 2;
  }
  if (g_size < 1 || g_size > kMaxRanks || g_dims[0] % g_size != 0) {
    std::fprintf(stderr, "refshim: SWC_REF_RANKS=%d must divide nx=%ld (at most %d)\n", g_size,
                 g_dims[0], kMaxRanks);
    return 2;
  }
  g_dir = dir;
  // The reference writes under <dir>/flatL-...-nu<argv1>-e0d<argv2>/ (:184-201).
  const std::string box = g_dir + "/flatL-rho100to1-zeta1-nw8-nu" + argv[1] + "-e0d" + argv[2];
  std::error_code ec;
  std::filesystem::create_directories(box + "/save", ec);
  std::filesystem::create_directories(g_dir + "/dump", ec);
  if (ec) {
    std::fprintf(stderr, "refshim: cannot create %s\n", box.c_str());
    return 2;
  }

  const long ng = g_dims[0] * g_dims[1] * g_dims[2];
  g_msg_bytes = g_dims[1] * g_dims[2] * (long)sizeof(double);
  const size_t head = (sizeof(Shared) + 4095) & ~(size_t)4095;
  const size_t msg = (size_t)g_msg_bytes * kMaxRanks * kSlotsPerRank;
  const size_t total = head + msg + (size_t)ng * sizeof(double);
  void* mem = mmap(nullptr, total, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
  if (mem == MAP_FAILED) {
    std::perror("refshim: mmap");
    return 2;
  }
  g_sh = static_cast<Shared*>(mem);
  g_msg = static_cast<char*>(mem) + head;
  g_buf = reinterpret_cast<double*>(static_cast<char*>(mem) + head + msg);
  pthread_mutexattr_t ma;
  pthread_mutexattr_init(&ma);
  pthread_mutexattr_setpshared(&ma, PTHREAD_PROCESS_SHARED);
  pthread_mutex_init(&g_sh->mu, &ma);
  pthread_condattr_t ca;
  pthread_condattr_init(&ca);
  pthread_condattr_setpshared(&ca, PTHREAD_PROCESS_SHARED);
  pthread_condattr_setclock(&ca, CLOCK_MONOTONIC);
  pthread_cond_init(&g_sh->cv, &ca);
  g_sh->size = g_size;

  std::cout.flush();
  std::fflush(nullptr);
  std::vector<pid_t> pids;
  for (int r = 0; r < g_size; ++r) {
    const pid_t pid = fork();
    if (pid < 0) {
      std::perror("refshim: fork");
      for (pid_t q : pids) kill(q, SIGTERM);
      return 2;
    }
    if (pid == 0) {
      g_rank = r;
      swc_ref_main(argc, argv);
      MPI::Finalize();
    }
    pids.push_back(pid);
  }
  // Reap the ranks; after the first failure, end the ranks still running (only
  // the processes forked above, by PID).
  std::set<pid_t> live(pids.begin(), pids.end());
  int failed = 0;
  while (!live.empty()) {
    int status = 0;
    const pid_t done = wait(&status);
    if (done < 0) break;
    live.erase(done);
    if (!WIFEXITED(status) || WEXITSTATUS(status) != 0) {
      if (!failed) std::fprintf(stderr, "refshim: a rank failed (status %d); stopping the others\n", status);
      failed = 1;
      for (pid_t q : live) kill(q, SIGTERM);
    }
  }
  return failed ? 1 : 0;
}
