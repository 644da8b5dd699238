// lbm_b200: command-line driver of the GB300 solver, with the command line and outputs of the
// reference's executables (lbm_v0 ... lbm_v3, src/common/driver.hpp and params.cpp), so that the
// reference's benchmark scripts run it unchanged:
//
//   lbm_b200 [--case poiseuille|cylinder] [--nx N] [--ny N] [--tau T] [--umax U] [--steps N]
//            [--out DIR] [--re R] [--diameter D] [--probe-every N] [--frame-every N]
//            [--frame-start N] [--bench [--warmup N] [--reps R]]
//
// --bench prints one line per timed repetition, "BENCH {json}", with the keys that
// bench/run_bench.py reads (version, nx, ny, steps, warmup, threads, time_s, mlups, real, ...,
// gpu, block, variant). Otherwise the Poiseuille case writes rho/ux/uy/vorticity/solid .npy files
// and meta.json to --out, and the cylinder case (inlet/outlet in x, Reynolds number --re) also
// writes probe.csv (u at 3 D behind the disc every --probe-every steps) and vorticity frames.
// Built twice: float, and double with -DLBM_REAL_DOUBLE (the reference's compile-time `real`).
#define LBM_B200_STANDALONE
#include <sys/stat.h>

#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "lbm_b200.hpp"

namespace {

using lbm::real;
const char* const kRealName = sizeof(real) == sizeof(double) ? "double" : "float";

struct Options {
  std::string case_name = "poiseuille";
  int nx = 64, ny = 34;
  real tau = real(0.9), u_max = real(0.05);
  int steps = 20000;
  std::string out = "output";
  double re = 100.0;
  int diameter = 40, probe_every = 50, frame_every = 0, frame_start = 0;
  bool bench = false;
  int warmup = 100, reps = 5;
};

Options parse(int argc, char** argv) {
  Options o;
  for (int a = 1; a < argc; ++a) {
    const std::string key = argv[a];
    if (key == "--bench") {
      o.bench = true;
      continue;
    }
    if (a + 1 >= argc) throw std::invalid_argument("missing value for " + key);
    const std::string v = argv[++a];
    if (key == "--case") o.case_name = v;
    else if (key == "--nx") o.nx = std::stoi(v);
    else if (key == "--ny") o.ny = std::stoi(v);
    else if (key == "--tau") o.tau = static_cast<real>(std::stod(v));
    else if (key == "--umax") o.u_max = static_cast<real>(std::stod(v));
    else if (key == "--steps") o.steps = std::stoi(v);
    else if (key == "--out") o.out = v;
    else if (key == "--warmup") o.warmup = std::stoi(v);
    else if (key == "--reps") o.reps = std::stoi(v);
    else if (key == "--re") o.re = std::stod(v);
    else if (key == "--diameter") o.diameter = std::stoi(v);
    else if (key == "--probe-every") o.probe_every = std::stoi(v);
    else if (key == "--frame-every") o.frame_every = std::stoi(v);
    else if (key == "--frame-start") o.frame_start = std::stoi(v);
    else throw std::invalid_argument("unknown option " + key);
  }
  if (o.nx < 1 || o.ny < 3) throw std::invalid_argument("grid too small");
  if (o.tau <= real(0.5)) throw std::invalid_argument("tau must be > 0.5 (positive viscosity)");
  if (o.steps < 0) throw std::invalid_argument("steps must be >= 0");
  if (o.warmup < 0 || o.reps < 1) throw std::invalid_argument("need warmup >= 0 and reps >= 1");
  if (o.re <= 0 || o.diameter < 2 || o.probe_every < 1 || o.frame_every < 0)
    throw std::invalid_argument("invalid cylinder parameters");
  return o;
}

lbm::Mask channel(int nx, int ny) {
  lbm::Mask m(static_cast<size_t>(nx) * ny, 0);
  for (int x = 0; x < nx; ++x) m[x] = m[static_cast<size_t>(ny - 1) * nx + x] = 1;
  return m;
}

lbm::Mask disc(int nx, int ny, double xc, double yc, double d) {
  lbm::Mask m(static_cast<size_t>(nx) * ny, 0);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const double dx = x - xc, dy = y - yc;
      m[static_cast<size_t>(y) * nx + x] = dx * dx + dy * dy <= 0.25 * d * d;
    }
  return m;
}

// F = 8 nu u_max / H^2 with nu = (tau - 1/2) / 3, in `real`.
real poiseuille_force(int h, real tau, real u_max) {
  const real nu = (tau - real(0.5)) / real(3);
  return real(8) * nu * u_max / (real(h) * real(h));
}

void mkdirs(const std::string& path) {
  std::string cur;
  for (size_t i = 0; i <= path.size(); ++i) {
    if (i == path.size() || path[i] == '/') {
      if (!cur.empty() && mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST)
        throw std::runtime_error("cannot create " + cur);
    }
    if (i < path.size()) cur += path[i];
  }
}

// NumPy .npy version 1.0, shape (ny, nx), little-endian data after a 64-byte-aligned header.
template <class T>
void write_npy(const std::string& path, const std::vector<T>& a, int ny, int nx, const char* descr) {
  if (a.size() != static_cast<size_t>(nx) * ny) throw std::invalid_argument("npy: bad size");
  std::string header = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': (" +
                       std::to_string(ny) + ", " + std::to_string(nx) + "), }";
  const size_t total = (10 + header.size() + 1 + 63) / 64 * 64;
  header.append(total - 10 - header.size() - 1, ' ');
  header += '\n';
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  const unsigned char pre[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  f.write(reinterpret_cast<const char*>(pre), 8);
  const uint16_t len = static_cast<uint16_t>(header.size());
  const unsigned char le[2] = {static_cast<unsigned char>(len & 0xff), static_cast<unsigned char>(len >> 8)};
  f.write(reinterpret_cast<const char*>(le), 2);
  f.write(header.data(), static_cast<std::streamsize>(header.size()));
  f.write(reinterpret_cast<const char*>(a.data()), static_cast<std::streamsize>(a.size() * sizeof(T)));
}

void write_field(const std::string& path, const std::vector<real>& a, int ny, int nx) {
  write_npy(path, a, ny, nx, sizeof(real) == 8 ? "<f8" : "<f4");
}

// Vorticity duy/dx - dux/dy, central differences, periodic in y; in x periodic or, for an open
// domain, one-sided on the two edge columns. Solid cells 0.
std::vector<real> vorticity(const std::vector<real>& ux, const std::vector<real>& uy,
                            const lbm::Mask& solid, int nx, int ny, bool periodic_x) {
  std::vector<real> w(ux.size(), real(0));
  for (int y = 0; y < ny; ++y) {
    const int yp = (y + 1) % ny, ym = (y + ny - 1) % ny;
    for (int x = 0; x < nx; ++x) {
      const size_t c = static_cast<size_t>(y) * nx + x;
      if (solid[c]) continue;
      int xp = (x + 1) % nx, xm = (x + nx - 1) % nx;
      real h = real(2);
      if (!periodic_x && x == 0) {
        xm = 0;
        h = real(1);
      }
      if (!periodic_x && x == nx - 1) {
        xp = nx - 1;
        h = real(1);
      }
      const real duy_dx = (uy[static_cast<size_t>(y) * nx + xp] - uy[static_cast<size_t>(y) * nx + xm]) / h;
      const real dux_dy = (ux[static_cast<size_t>(yp) * nx + x] - ux[static_cast<size_t>(ym) * nx + x]) / real(2);
      w[c] = duy_dx - dux_dy;
    }
  }
  return w;
}

void write_fields(const std::string& dir, const lbm::SolverB200& s, bool periodic_x) {
  std::vector<real> rho, ux, uy;
  s.macroscopic(rho, ux, uy);
  write_field(dir + "rho.npy", rho, s.ny(), s.nx());
  write_field(dir + "ux.npy", ux, s.ny(), s.nx());
  write_field(dir + "uy.npy", uy, s.ny(), s.nx());
  write_field(dir + "vorticity.npy", vorticity(ux, uy, s.solid(), s.nx(), s.ny(), periodic_x), s.ny(), s.nx());
  write_npy(dir + "solid.npy", s.solid(), s.ny(), s.nx(), "|u1");
}

std::string compiler() {
#ifdef __VERSION__
  return std::string("GNU ") + __VERSION__ + " + nvcc (sm_103a library)";
#else
  return "unknown";
#endif
}

int run_poiseuille(const Options& o) {
  const int h = o.ny - 2;
  const real force = poiseuille_force(h, o.tau, o.u_max);
  lbm::SolverB200 s(o.nx, o.ny, o.tau, force, real(0), channel(o.nx, o.ny));
  if (!o.bench)
    std::printf("case=%s nx=%d ny=%d tau=%g umax=%g steps=%d real=%s out=%s\n", o.case_name.c_str(),
                o.nx, o.ny, static_cast<double>(o.tau), static_cast<double>(o.u_max), o.steps,
                kRealName, o.out.c_str());
  s.init_equilibrium(real(1), real(0), real(0));
  if (o.bench) {
    s.run(o.warmup);
    for (int r = 0; r < o.reps; ++r) {
      const double t = s.timed_run(o.steps);
      const double mlups = static_cast<double>(o.nx) * o.ny * o.steps / t / 1e6;
      std::printf(
          "BENCH {\"version\": \"b200\", \"rep\": %d, \"nx\": %d, \"ny\": %d, \"steps\": %d, "
          "\"warmup\": %d, \"threads\": %d, \"time_s\": %.6f, \"mlups\": %.4f, \"real\": \"%s\", "
          "\"compiler\": \"%s\", \"flags\": \"-O2 -ffp-contract=off\", \"build_type\": \"Release\", %s}\n",
          r, o.nx, o.ny, o.steps, o.warmup, s.threads(), t, mlups, kRealName, compiler().c_str(),
          s.bench_info().c_str());
      std::fflush(stdout);
    }
    return 0;
  }
  const double m0 = s.total_mass();
  const double t = s.timed_run(o.steps);
  const double m1 = s.total_mass();
  std::printf("time=%.3f s  MLUPS=%.2f (indicative)  mass drift=%.3e\n", t,
              static_cast<double>(o.nx) * o.ny * o.steps / t / 1e6, (m1 - m0) / m0);
  mkdirs(o.out);
  const std::string dir = o.out + "/";
  write_fields(dir, s, true);
  std::ofstream meta(dir + "meta.json");
  meta << "{\"version\": \"b200\", \"case\": \"" << o.case_name << "\", \"nx\": " << o.nx
       << ", \"ny\": " << o.ny << ", \"tau\": " << static_cast<double>(o.tau)
       << ", \"umax\": " << static_cast<double>(o.u_max)
       << ", \"force_x\": " << static_cast<double>(force) << ", \"steps\": " << o.steps
       << ", \"real\": \"" << kRealName << "\"}\n";
  std::printf("fields written to %s\n", o.out.c_str());
  return 0;
}

int run_cylinder(const Options& o) {
  const double xc = 5.0 * o.diameter, yc = o.ny / 2 + 1;  // one cell above mid-height
  const int px = static_cast<int>(xc + 3.0 * o.diameter), py = static_cast<int>(yc);
  const double nu = static_cast<double>(o.u_max) * o.diameter / o.re;
  const real tau = static_cast<real>(0.5 + 3.0 * nu);
  lbm::SolverB200 s(o.nx, o.ny, tau, real(0), real(0), disc(o.nx, o.ny, xc, yc, o.diameter));
  std::printf("case=cylinder nx=%d ny=%d D=%d Re=%g u_in=%g -> tau=%.4f, Ma=%.3f, steps=%d real=%s out=%s\n",
              o.nx, o.ny, o.diameter, o.re, static_cast<double>(o.u_max), static_cast<double>(tau),
              std::sqrt(3.0) * static_cast<double>(o.u_max), o.steps, kRealName, o.out.c_str());
  s.set_inflow_outflow(o.u_max);
  s.init_equilibrium(real(1), o.u_max, real(0));
  mkdirs(o.out + "/frames");
  const std::string dir = o.out + "/";
  std::ofstream probe(dir + "probe.csv");
  probe << "step,ux,uy,rho\n";
  double seconds = 0.0;
  int n = 0, frames = 0;
  while (n < o.steps) {
    const int chunk = o.probe_every < o.steps - n ? o.probe_every : o.steps - n;
    seconds += s.timed_run(chunk);
    n += chunk;
    real f[9];
    s.populations_at(px, py, f);
    static const int cx[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1}, cy[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    real m0 = 0, mx = 0, my = 0;
    for (int i = 0; i < 9; ++i) {
      m0 += f[i];
      mx += cx[i] * f[i];
      my += cy[i] * f[i];
    }
    const real rho = real(1) + m0;
    probe << n << ',' << static_cast<double>(mx / rho) << ',' << static_cast<double>(my / rho) << ','
          << static_cast<double>(rho) << '\n';
    if (!std::isfinite(static_cast<double>(rho)))
      throw std::runtime_error("the simulation diverged (non-finite density at the probe)");
    if (o.frame_every > 0 && n >= o.frame_start && n % o.frame_every == 0) {
      std::vector<real> r, ux, uy;
      s.macroscopic(r, ux, uy);
      char name[64];
      std::snprintf(name, sizeof name, "frames/vort_%07d.npy", n);
      write_field(dir + name, vorticity(ux, uy, s.solid(), o.nx, o.ny, false), o.ny, o.nx);
      ++frames;
    }
  }
  std::printf("time=%.3f s  MLUPS=%.2f (indicative, without I/O)  frames=%d\n", seconds,
              static_cast<double>(o.nx) * o.ny * o.steps / seconds / 1e6, frames);
  write_fields(dir, s, false);
  std::ofstream meta(dir + "meta.json");
  meta << "{\"version\": \"b200\", \"case\": \"cylinder\", \"nx\": " << o.nx << ", \"ny\": " << o.ny
       << ", \"tau\": " << static_cast<double>(tau) << ", \"u_in\": " << static_cast<double>(o.u_max)
       << ", \"re\": " << o.re << ", \"diameter\": " << o.diameter << ", \"xc\": " << xc
       << ", \"yc\": " << yc << ", \"probe_x\": " << px << ", \"probe_y\": " << py
       << ", \"probe_every\": " << o.probe_every << ", \"frame_every\": " << o.frame_every
       << ", \"steps\": " << o.steps << ", \"real\": \"" << kRealName << "\"}\n";
  std::printf("probe, frames and fields written to %s\n", o.out.c_str());
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    const Options o = parse(argc, argv);
    if (o.case_name == "cylinder") return run_cylinder(o);
    if (o.case_name != "poiseuille") {
      std::fprintf(stderr, "unknown case '%s' (available: poiseuille, cylinder)\n", o.case_name.c_str());
      return 1;
    }
    return run_poiseuille(o);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
}
