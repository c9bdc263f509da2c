// swc_run.cpp -- C++ host driver with the reference's command line and outputs.
//
//   swc_run [options] nu ep_arg aE load
//
// Mirrors main() of smaiso-wcomp.cpp on one GPU through the C ABI (include/swc.h):
// positional arguments as REF:176, 230, 242, 249; the L1-driven loop REF:1081 with
// diagnostics every stepL1 = 50 steps (REF:2202-2265) and field output every
// stepSave = 10 diagnostics (REF:2271-2453); the same files in the same text layout
// (default ostream formatting, one value per line). Options replace the reference's
// compile-time constants:
//   --grid NX NY NZ   (REF:218, default 512 512 512)   --dt DT      (REF:262)
//   --nw NW           (REF:261)                       --rho0 R     (REF:251)
//   --divv-switch N   (REF:214)                       --ranks P    (x slabs of the reproduced run)
//   --step-l1 N       (REF:206)                       --step-save N (REF:207)
//   --max-steps N     (no reference counterpart: stop after N steps)
//   --out DIR         (REF:198-201, default ./flatL-rho100to1-zeta1-nw8-nu<nu>-e0d<ep>/)
//   --load-dir DIR    (REF:186-189: psi<rank>.dat read when load == 1, default <out>/save/)
//   --precision fp64|mixed
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <ctime>
#include <fstream>
#include <iostream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/swc.h"

namespace {

void die(const char* what, int rc) {
  std::fprintf(stderr, "swc_run: %s failed: %s (%s)\n", what, swc_strerror(rc), swc_last_error());
  std::exit(2);
}

void check(int rc, const char* what) {
  if (rc != SWC_OK) die(what, rc);
}

struct Opts {
  int nx = 512, ny = 512, nz = 512, nw = 8, ranks = 2, step_l1 = 50, step_save = 10, divv_switch = 50;
  long long max_steps = -1;
  double dt = 0.001, rho0 = 0.01;
  int precision = SWC_PREC_FP64;
  std::string out, load_dir;
  std::string nu_s, ep_s, ae_s, load_s;
};

Opts parse(int argc, char** argv) {
  Opts o;
  std::vector<std::string> pos;
  for (int a = 1; a < argc; ++a) {
    std::string s = argv[a];
    auto need = [&](int k) {
      if (a + k >= argc) {
        std::fprintf(stderr, "swc_run: %s needs %d value(s)\n", s.c_str(), k);
        std::exit(1);
      }
    };
    if (s == "--grid") { need(3); o.nx = std::atoi(argv[++a]); o.ny = std::atoi(argv[++a]); o.nz = std::atoi(argv[++a]); }
    else if (s == "--dt") { need(1); o.dt = std::atof(argv[++a]); }
    else if (s == "--nw") { need(1); o.nw = std::atoi(argv[++a]); }
    else if (s == "--rho0") { need(1); o.rho0 = std::atof(argv[++a]); }
    else if (s == "--divv-switch") { need(1); o.divv_switch = std::atoi(argv[++a]); }
    else if (s == "--ranks") { need(1); o.ranks = std::atoi(argv[++a]); }
    else if (s == "--step-l1") { need(1); o.step_l1 = std::atoi(argv[++a]); }
    else if (s == "--step-save") { need(1); o.step_save = std::atoi(argv[++a]); }
    else if (s == "--max-steps") { need(1); o.max_steps = std::atoll(argv[++a]); }
    else if (s == "--out") { need(1); o.out = argv[++a]; }
    else if (s == "--load-dir") { need(1); o.load_dir = argv[++a]; }
    else if (s == "--precision") {
      need(1);
      std::string v = argv[++a];
      o.precision = (v == "mixed") ? SWC_PREC_MIXED : SWC_PREC_FP64;
    } else pos.push_back(s);
  }
  if (pos.size() != 4) {
    std::fprintf(stderr, "usage: swc_run [options] nu ep_arg aE load\n");
    std::exit(1);
  }
  o.nu_s = pos[0]; o.ep_s = pos[1]; o.ae_s = pos[2]; o.load_s = pos[3];
  if (o.out.empty()) o.out = "flatL-rho100to1-zeta1-nw8-nu" + o.nu_s + "-e0d" + o.ep_s;
  if (o.out.back() != '/') o.out += "/";
  if (o.load_dir.empty()) o.load_dir = o.out + "save/";
  if (o.load_dir.back() != '/') o.load_dir += "/";
  return o;
}

void touch(const std::string& path) {
  std::ofstream f(path);
  if (!f.is_open()) {
    std::fprintf(stderr, "swc_run: cannot create %s\n", path.c_str());
    std::exit(3);
  }
}

// saveMid (REF:94-129): append the j = Ny/2 slice, i outer, k inner.
void save_mid(const std::string& path, const std::vector<double>& f, int nx, int ny, int nz) {
  std::ofstream out(path, std::ios_base::app);
  if (!out.is_open()) {
    std::fprintf(stderr, "swc_run: cannot append to %s\n", path.c_str());
    std::exit(3);
  }
  const int j = ny / 2;
  for (int i = 0; i < nx; ++i)
    for (int k = 0; k < nz; ++k) out << f[((size_t)i * ny + j) * nz + k] << "\n";
}

}  // namespace

int main(int argc, char** argv) {
  Opts o = parse(argc, argv);
  const int load = (int)std::atof(o.load_s.c_str());  // REF:176
  swc_params p;
  check(swc_default_params(&p, o.nx, o.ny, o.nz), "swc_default_params");
  p.nw = o.nw;
  p.dt = o.dt;
  p.ep = -0.001 * std::atof(o.ep_s.c_str());  // REF:242-243
  p.nu = std::atof(o.nu_s.c_str());           // REF:249
  p.rho_0 = o.rho0;
  p.divv_switch = o.divv_switch;
  p.load = load == 1 ? 1 : 0;
  p.ref_ranks = o.ranks;
  p.precision = o.precision;
  swc_derived d;
  check(swc_derive(&p, &d), "swc_derive");
  const double aE = std::atof(o.ae_s.c_str());
  const size_t ng = (size_t)o.nx * o.ny * o.nz;
  const int P = o.ranks, local_n0 = o.nx / (P > 0 ? P : 1);
  mkdir(o.out.c_str(), 0755);

  std::vector<double> psi(ng, 0.0);
  if (load != 1) {
    // REF:571-590 with phi = 0: Amp cos(q0 k dz) for Nz/2-8 < k < Nz/2+8
    for (int i = 0; i < o.nx; ++i)
      for (int j = 0; j < o.ny; ++j)
        for (int k = 0; k < o.nz; ++k)
          if ((k > o.nz / 2 - 8) && (k < o.nz / 2 + 8)) psi[((size_t)i * o.ny + j) * o.nz + k] = d.amp * std::cos(p.q0 * k * d.dz);
    for (int r = 0; r < P; ++r) touch(o.out + "psi" + std::to_string(r) + ".dat");  // REF:713-720
  } else {
    // REF:727-796: psi<rank>.dat holds the rank's x slab in (i,j,k) order
    for (int r = 0; r < P; ++r) {
      std::ifstream in(o.load_dir + "psi" + std::to_string(r) + ".dat");
      if (!in.is_open()) {
        std::fprintf(stderr, "swc_run: cannot read %spsi%d.dat\n", o.load_dir.c_str(), r);
        return 3;
      }
      const size_t base = (size_t)r * local_n0 * o.ny * o.nz;
      for (size_t t = 0; t < (size_t)local_n0 * o.ny * o.nz; ++t) in >> psi[base + t];
    }
  }
  {  // REF:801-919
    std::ofstream info(o.out + "info");
    info << "Nx: " << o.nx << "\n" << "Ny: " << o.ny << "\n" << "Nz: " << o.nz << "\n";
    info << "Points per wavelength (nw): " << o.nw << "\n" << "q0 (z direction): " << p.q0 << "\n";
    info << "epsilon: " << p.ep << "\n" << "beta: " << p.beta << "\n" << "gamma: " << p.gamma << "\n";
    info << "Viscosity (nu): " << p.nu << "\n" << "2nd Viscosity (lambda): " << p.lambda << "\n";
    info << "Density penalty (zeta): " << p.zeta << "\n" << "dx: " << d.dx << "\n" << "dt: " << p.dt << "\n";
    info << "stepL1: " << o.step_l1 << "\n" << "stepSave: " << o.step_save << "\n";
    info << "divv switch: " << o.divv_switch << "\n" << "Initial amp: " << d.amp << "\n";
    info << "kp: " << d.kp << "\n" << "rho_0: " << p.rho_0 << "\n";
    info << "Perturbation wavenumber Qx (flat): " << 0.125 / 2 << "\n";
    info << "Perturbation amplitude phi (flat): " << 0 << "\n";
    info << "Focal conic initial size (fc): " << aE << "\n";
  }
  const char* created[] = {"L1.dat", "mass.dat", "energy.dat", "psiMid.dat", "energyMid.dat", "vx.dat", "vy.dat",
                           "vz.dat", "vsolx.dat", "vsoly.dat", "vsolz.dat", "sx.dat", "sy.dat", "sz.dat",
                           "divv.dat", "rho.dat", "amp.dat", "surfPsi.dat"};
  for (const char* f : created) touch(o.out + f);

  swc_ctx* ctx = nullptr;
  check(swc_create(&p, &ctx), "swc_create");
  check(swc_set_state(ctx, psi.data(), nullptr), "swc_set_state");  // rho = 0 (REF:1053)

  std::cout << "Using 1 GPU (reproducing " << P << " x slabs)." << std::endl;
  const auto wall0 = std::chrono::system_clock::now();
  double L1 = 1.0;
  const double limL1 = std::pow(10.0, -6);
  int countSave = 0;
  long long nloop = 0;
  std::vector<double> surfZ((size_t)o.nx * o.ny, 0.0);  // persists between saves (REF:2278-2293)
  std::vector<double> f(ng);
  while (L1 > limL1 && (o.max_steps < 0 || nloop < o.max_steps)) {
    int n = o.step_l1;
    if (o.max_steps >= 0 && nloop + n > o.max_steps) n = (int)(o.max_steps - nloop);
    check(swc_step(ctx, n), "swc_step");
    nloop += n;
    if (n < o.step_l1) break;  // partial block: no diagnostic line, as the reference
    swc_diag dg;
    check(swc_diagnostics(ctx, &dg), "swc_diagnostics");
    L1 = dg.l1;
    { std::ofstream out(o.out + "L1.dat", std::ios_base::app); out << L1 << "\n"; }
    { std::ofstream out(o.out + "mass.dat", std::ios_base::app); out << dg.mass << "\n"; }
    { std::ofstream out(o.out + "energy.dat", std::ios_base::app); out << dg.energy << "\n"; }
    if (++countSave == o.step_save) {
      check(swc_get_field(ctx, SWC_F_RHO, f.data()), "swc_get_field(rho)");
      for (int i = 0; i < o.nx; ++i)
        for (int j = 0; j < o.ny; ++j)
          for (int k = o.nz - 1; k > -1; --k)
            if (f[((size_t)i * o.ny + j) * o.nz + k] > d.rho_s - 0.15) {
              surfZ[(size_t)i * o.ny + j] = k;
              break;
            }
      std::vector<double> psi_now(ng);
      check(swc_get_field(ctx, SWC_F_PSI, psi_now.data()), "swc_get_field(psi)");
      for (int r = 0; r < P; ++r) {  // REF:2334-2345, one file per reproduced rank
        std::ofstream out(o.out + "psi" + std::to_string(r) + ".dat");
        const size_t base = (size_t)r * local_n0 * o.ny * o.nz;
        for (size_t t = 0; t < (size_t)local_n0 * o.ny * o.nz; ++t) out << psi_now[base + t] << "\n";
      }
      save_mid(o.out + "psiMid.dat", psi_now, o.nx, o.ny, o.nz);
      {
        std::ofstream out(o.out + "surfPsi.dat", std::ios_base::app);
        for (size_t t = 0; t < surfZ.size(); ++t) out << surfZ[t] << "\n";
      }
      const struct { int field; const char* file; } mids[] = {
          {SWC_F_VX, "vx.dat"}, {SWC_F_VY, "vy.dat"}, {SWC_F_VZ, "vz.dat"}, {SWC_F_VSOLX, "vsolx.dat"},
          {SWC_F_VSOLY, "vsoly.dat"}, {SWC_F_VSOLZ, "vsolz.dat"}, {SWC_F_DIVV, "divv.dat"},
          {SWC_F_RHO, "rho.dat"}, {SWC_F_AMP, "amp.dat"}, {SWC_F_ENERGY, "energyMid.dat"}};
      for (const auto& m : mids) {
        check(swc_get_field(ctx, m.field, f.data()), "swc_get_field");
        save_mid(o.out + m.file, f, o.nx, o.ny, o.nz);
      }
      time_t now = time(0);
      std::cout << "The loop " << nloop << " local date and time is: " << ctime(&now) << std::endl;
      countSave = 0;
    }
  }
  const std::chrono::duration<double> wall = std::chrono::system_clock::now() - wall0;
  std::cout << "Finished " << nloop << " steps in " << wall.count() << " seconds [Wall Clock] " << std::endl;
  swc_destroy(ctx);
  return 0;
}
