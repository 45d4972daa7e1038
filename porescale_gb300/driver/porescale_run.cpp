// porescale_run -- the two-phase LBM driver of porescale on the C ABI.
//
// Runs in a directory prepared for the reference's coupled driver
// (LBM-LSM/lsm_lbm_static_alpha_beta_multipore.f): reads INPUT_PARAMETERS
// (S1:435-469), velocities19 (S1:508-524, checked against the built-in
// order) and ind (S1:532-539), then does what the reference's main program
// and majorityrule do for the fluid (S1:1413-1530, 3436-3992): initdistr or
// restart from iteration2, the two initialisation steps, itm-itms+1 blocks
// of itw steps, and after each block the iteration / iteration2 checkpoint
// and the check_state record (check_state_19 and one output.m row).  The
// lattice-spring half of the coupled program (lsm_step, calc_stress,
// calc_ab) is not part of this mode.
//
// With -m xx or -m yz it is instead the lattice-spring program of
// LSM2S/Cxxxx/XX_P.f or LSM2S/Cyzyz/YZ_P.f: their INPUT_PARAMETERS, the
// static solve, and their output files (run_lsm below).
//
// Options: -m lbm|xx|yz (default lbm), -p f64|f32|f16|bf16 (population
// storage, default f64, the reference's arithmetic) or f64|mixed (spring
// solve), -d DIR (run directory, default .), -q (quiet).
#include <sys/stat.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "porescale.h"

namespace {

struct Input {
  double cr2, rr0, rb0, B, sig, vir, vib, wet;
  int idir, itm, itw, its;
  double eps;
  int mtype, icon;
  double sat;
  int iipore, npores;
  double ee, lsize, bfr[3], bfb[3];
  int ncx, ncy, ncz;
  double Em, nu, rs, dt, dl;
};

std::string g_dir = ".";

std::string path(const std::string& f) { return g_dir + "/" + f; }

[[noreturn]] void die(const std::string& msg)
{
  std::fprintf(stderr, "porescale_run: %s\n", msg.c_str());
  std::exit(2);
}

// Fortran list-directed numbers: D exponents, trailing comments
double fnum(const std::string& tok)
{
  std::string t = tok;
  for (char& c : t)
    if (c == 'D' || c == 'd') c = 'E';
  char* end = nullptr;
  const double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str()) die("cannot read a number from '" + tok + "'");
  return v;
}

Input read_input()
{
  std::ifstream f(path("INPUT_PARAMETERS"));
  if (!f) die("INPUT_PARAMETERS not found in " + g_dir);
  std::vector<std::string> lines;
  std::string ln;
  while (std::getline(f, ln)) lines.push_back(ln);
  size_t k = 0;
  auto first = [&](int n) {  // the first n tokens of the next line
    if (k >= lines.size()) die("INPUT_PARAMETERS ends early");
    std::istringstream ss(lines[k++]);
    std::vector<double> v;
    std::string t;
    for (int i = 0; i < n; i++) {
      if (!(ss >> t)) die("INPUT_PARAMETERS line " + std::to_string(k) + " has too few values");
      v.push_back(fnum(t));
    }
    return v;
  };
  auto one = [&]() { return first(1)[0]; };
  Input in{};
  in.cr2 = one();
  in.rr0 = one();
  in.rb0 = one();
  in.B = one();
  in.sig = one();
  in.vir = one();
  in.vib = one();
  in.wet = one();
  in.idir = (int)one();
  in.itm = (int)one();
  in.itw = (int)one();
  in.its = (int)one();
  in.eps = one();
  in.mtype = (int)one();
  in.icon = (int)one();
  in.sat = one();
  in.iipore = (int)one();
  in.npores = (int)one();
  in.ee = one();
  in.lsize = one();
  auto b = first(3);
  for (int i = 0; i < 3; i++) in.bfr[i] = b[i];
  b = first(3);
  for (int i = 0; i < 3; i++) in.bfb[i] = b[i];
  in.ncx = (int)one();
  in.ncy = (int)one();
  in.ncz = (int)one();
  in.Em = one();
  in.nu = one();
  in.rs = one();
  in.dt = one();
  in.dl = one();
  return in;
}

// velocities19 must hold the D3Q19 order the library is built for
void check_velocities()
{
  std::ifstream f(path("velocities19"));
  if (!f) return;  // optional: the order is built in
  static const int cv[3][19] = {{0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0},
                                {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1},
                                {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 19; j++) {
      int v;
      if (!(f >> v)) die("velocities19 is truncated");
      if (v != cv[i][j]) die("velocities19 differs from the D3Q19 order this library implements");
    }
}

// ind: one line per (j, k), k outer, a leading blank then ncx digits
std::vector<int32_t> read_ind(int ncx, int ncy, int ncz)
{
  std::ifstream f(path("ind"));
  if (!f) die("ind not found in " + g_dir);
  std::vector<int32_t> ind((size_t)ncx * ncy * ncz);
  std::string ln;
  for (int k = 0; k < ncz; k++)
    for (int j = 0; j < ncy; j++) {
      if (!std::getline(f, ln)) die("ind has fewer than ncy*ncz lines");
      size_t p = ln.find_first_not_of(' ');
      if (p == std::string::npos || ln.size() < p + (size_t)ncx) die("short line in ind");
      for (int i = 0; i < ncx; i++) {
        const char c = ln[p + i];
        if (c < '0' || c > '9') die("non-digit in ind");
        ind[(size_t)i + (size_t)ncx * (j + (size_t)ncy * k)] = c - '0';
      }
    }
  return ind;
}

// Fortran E15.8: " 0.12345678E-03" with a leading 0.
std::string e15_8(double v)
{
  char buf[64];
  if (v == 0.0 || !std::isfinite(v)) {
    if (!std::isfinite(v)) std::snprintf(buf, sizeof buf, "%15s", std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
    else std::snprintf(buf, sizeof buf, "%15s", "0.00000000E+00");
    return buf;
  }
  int e = (int)std::floor(std::log10(std::fabs(v))) + 1;
  double m = std::fabs(v) / std::pow(10.0, e);
  // rounding to 8 digits may carry into the next decade
  double mr = std::round(m * 1e8) / 1e8;
  if (mr >= 1.0) {
    mr /= 10.0;
    e += 1;
  }
  std::snprintf(buf, sizeof buf, "%s0.%08.0fE%c%02d", v < 0 ? "-" : " ", mr * 1e8, e < 0 ? '-' : '+', std::abs(e));
  std::string s(buf);
  while (s.size() < 15) s = " " + s;
  return s;
}

void check(int rc, const char* what)
{
  if (rc == PS_OK) return;
  char buf[512];
  ps_last_error(buf, sizeof buf);
  die(std::string(what) + ": " + buf);
}

void write_state(const char* name, int it1, const std::vector<double>& fr, const std::vector<double>& fb)
{
  const std::string tmp = path(std::string(name) + ".tmp");
  FILE* f = std::fopen(tmp.c_str(), "w");
  if (!f) die("cannot write " + tmp);
  std::fprintf(f, "%12d\n", it1);
  for (const std::vector<double>* a : {&fr, &fb}) {
    for (size_t i = 0; i < a->size(); i++) std::fprintf(f, "%.17E%s", (*a)[i], (i % 4 == 3) ? "\n" : "  ");
    std::fprintf(f, "\n");
  }
  std::fflush(f);
  std::fclose(f);
  if (std::rename(tmp.c_str(), path(name).c_str()) != 0) die(std::string("cannot rename ") + name);
}

bool read_state(int& it1, std::vector<double>& fr, std::vector<double>& fb)
{
  std::ifstream f(path("iteration2"));
  if (!f) return false;
  std::string t;
  if (!(f >> t)) return false;
  it1 = (int)fnum(t);
  for (std::vector<double>* a : {&fr, &fb})
    for (double& v : *a) {
      if (!(f >> t)) die("iteration2 is truncated");
      v = fnum(t);
    }
  return true;
}

// ---- the lattice-spring driver (LSM2S/Cxxxx/XX_P.f, LSM2S/Cyzyz/YZ_P.f) ----
struct LsmInput {
  int ncx, ncy, ncz;
  double Em1, nu1, Em2, nu2, rs, dt, dl;
  int itm, its;
  double gstrain;
  int nthread, icon;
};

// INPUT_PARAMETERS of XX_P.f / YZ_P.f: one value per line (XX:364-382)
LsmInput read_lsm_input()
{
  std::ifstream f(path("INPUT_PARAMETERS"));
  if (!f) die("INPUT_PARAMETERS not found in " + g_dir);
  std::string ln;
  auto one = [&]() {
    if (!std::getline(f, ln)) die("INPUT_PARAMETERS ends early");
    std::istringstream ss(ln);
    std::string t;
    if (!(ss >> t)) die("empty line in INPUT_PARAMETERS");
    return fnum(t);
  };
  LsmInput in{};
  in.ncx = (int)one();
  in.ncy = (int)one();
  in.ncz = (int)one();
  in.Em1 = one();
  in.nu1 = one();
  in.Em2 = one();
  in.nu2 = one();
  in.rs = one();
  in.dt = one();
  in.dl = one();
  in.itm = (int)one();
  in.its = (int)one();
  in.gstrain = one();
  in.nthread = (int)one();
  in.icon = (int)one();
  return in;
}

// Static solve of the spring network with the imposed strain, then the
// reference program's output files: lsm_settings (XX:1316-1346), the
// LSM_coord / displ / velocity / force fields over the node grid (XX:1548-
// 1575; the static equilibrium has zero velocities and, to the solver's
// tolerance, zero net forces), iteration2 (positions, velocities,
// accelerations, XX:1599-1609) and the stress_tensor record appended by
// calc_stress (XX:1754, 1963-1994).
int run_lsm(int load, int prec, bool quiet)
{
  const LsmInput in = read_lsm_input();
  std::vector<int32_t> ind = read_ind(in.ncx, in.ncy, in.ncz);
  ps_lsm_params p{};
  // spring constants of the two solids (XX:411-414)
  p.alf1 = in.dl * in.Em1 / (5.0 - 10.0 * in.nu1);
  p.bet1 = in.dl * in.dl * in.dl * in.Em1 * (4 * in.nu1 - 1) / (20.0 * (2 * in.nu1 * in.nu1 + in.nu1 - 1));
  p.alf2 = in.dl * in.Em2 / (5.0 - 10.0 * in.nu2);
  p.bet2 = in.dl * in.dl * in.dl * in.Em2 * (4 * in.nu2 - 1) / (20.0 * (2 * in.nu2 * in.nu2 + in.nu2 - 1));
  p.gstrain = in.gstrain;
  p.load = load;
  p.precision = prec;
  void* h = nullptr;
  check(ps_lsm_create(&p, ind.data(), in.ncx, in.ncy, in.ncz, &h), "ps_lsm_create");
  ps_lsm_result r{};
  check(ps_lsm_solve(h, 1e-10, 2000000000, &r), "ps_lsm_solve");
  // reference node numbering: k-j-i over the node grid whose loaded axis has
  // planes 1..N+1 (plane N+1 tied to plane 1); a node exists when one of
  // its cubes is solid, no cube beyond the ends of the loaded axis
  const int pa = load == PS_LOAD_XSTRETCH ? 0 : 1;
  const int N[3] = {in.ncx, in.ncy, in.ncz};
  int M[3] = {in.ncx, in.ncy, in.ncz};
  M[pa] += 1;
  auto solid = [&](int x, int y, int z) {
    const int c[3] = {x, y, z};
    int w[3];
    for (int d = 0; d < 3; d++) {
      if (d == pa && (c[d] < 0 || c[d] >= N[d])) return false;
      w[d] = ((c[d] % N[d]) + N[d]) % N[d];
    }
    const int v = ind[(size_t)w[0] + (size_t)N[0] * (w[1] + (size_t)N[1] * w[2])];
    return v == 0 || v == 3;
  };
  std::vector<long long> num((size_t)M[0] * M[1] * M[2], 0);
  long long ns = 0;
  for (int z = 0; z < M[2]; z++)
    for (int y = 0; y < M[1]; y++)
      for (int x = 0; x < M[0]; x++) {
        bool e = false;
        for (int q = 0; q < 8 && !e; q++) e = solid(x - (q & 1), y - ((q >> 1) & 1), z - (q >> 2));
        if (e) num[(size_t)x + (size_t)M[0] * (y + (size_t)M[1] * z)] = ++ns;
      }
  std::vector<double> u((size_t)3 * ns);
  check(ps_lsm_get_disp(h, u.data()), "ps_lsm_get_disp");
  ps_lsm_info info{};
  check(ps_lsm_get_info(h, &info), "ps_lsm_get_info");
  {
    FILE* f = std::fopen(path("lsm_settings").c_str(), "w");
    std::fprintf(f, " Initial program settings\n Physical parameters\n");
    std::fprintf(f, " Young modulus Em1 of component solid 1 = %.16E\n Poissons ratio nu1 = %.16E\n", in.Em1, in.nu1);
    std::fprintf(f, " linear spring parameter alf = %.16E\n angular spring parameter bet = %.16E\n", p.alf1, p.bet1);
    std::fprintf(f, " Young modulus Em1 of component solid 2 = %.16E\n Poissons ratio nu2 = %.16E\n", in.Em2, in.nu2);
    std::fprintf(f, " linear spring parameter alf = %.16E\n angular spring parameter bet = %.16E\n", p.alf2, p.bet2);
    std::fprintf(f, " solid medium density rs = %.16E\n integration time step dt = %.16E\n", in.rs, in.dt);
    std::fprintf(f, " lattice unit step dl = %.16E\n Computational domain properties\n", in.dl);
    std::fprintf(f, " x unit cell size ncx = %d\n y unit cell size ncy = %d\n z unit cell size ncz = %d\n", in.ncx,
                 in.ncy, in.ncz);
    std::fprintf(f, " number of solid points ns = %lld\n static solve: conjugate gradient, %s\n", ns,
                 prec == PS_LSM_F64 ? "FP64" : "FP32 in FP64 refinement");
    std::fprintf(f, " iterations = %lld\n relative residual = %.6E\n", (long long)r.inner_iterations, r.relres);
    std::fclose(f);
  }
  {
    FILE* fc = std::fopen(path("LSM_coord_field").c_str(), "w");
    FILE* fd = std::fopen(path("LSM_displ_field").c_str(), "w");
    FILE* fv = std::fopen(path("LSM_velocity_field").c_str(), "w");
    FILE* ff = std::fopen(path("LSM_force_field").c_str(), "w");
    for (int k = 1; k <= in.ncz; k++)
      for (int j = 1; j <= in.ncy; j++)
        for (int i = 1; i <= in.ncx; i++) {
          const long long l = num[(size_t)(i - 1) + (size_t)M[0] * ((j - 1) + (size_t)M[1] * (k - 1))];
          if (l) {
            const double* ul = &u[(size_t)3 * (l - 1)];
            std::fprintf(fc, " %24.16E %24.16E %24.16E\n", i + ul[0], j + ul[1], k + ul[2]);
            std::fprintf(fd, " %24.16E %24.16E %24.16E\n", ul[0], ul[1], ul[2]);
          } else {
            std::fprintf(fc, " %12d %12d %12d\n", i, j, k);
            std::fprintf(fd, " %24.16E %24.16E %24.16E\n", 0.0, 0.0, 0.0);
          }
          std::fprintf(fv, " %24.16E %24.16E %24.16E\n", 0.0, 0.0, 0.0);
          std::fprintf(ff, " %24.16E %24.16E %24.16E\n", 0.0, 0.0, 0.0);
        }
    std::fclose(fc);
    std::fclose(fd);
    std::fclose(fv);
    std::fclose(ff);
  }
  {  // iteration2: positions (node coordinates + displacement), velocities, accelerations
    const std::string tmp = path("iteration2.tmp");
    FILE* f = std::fopen(tmp.c_str(), "w");
    std::vector<int> cx((size_t)ns), cy((size_t)ns), cz((size_t)ns);
    for (int z = 0; z < M[2]; z++)
      for (int y = 0; y < M[1]; y++)
        for (int x = 0; x < M[0]; x++) {
          const long long l = num[(size_t)x + (size_t)M[0] * (y + (size_t)M[1] * z)];
          if (l) {
            cx[l - 1] = x + 1;
            cy[l - 1] = y + 1;
            cz[l - 1] = z + 1;
          }
        }
    for (long long l = 0; l < ns; l++)
      std::fprintf(f, " %24.16E %24.16E %24.16E\n", cx[l] + u[3 * l], cy[l] + u[3 * l + 1], cz[l] + u[3 * l + 2]);
    for (int rep = 0; rep < 2; rep++)
      for (long long l = 0; l < ns; l++) std::fprintf(f, " %24.16E %24.16E %24.16E\n", 0.0, 0.0, 0.0);
    std::fclose(f);
    if (std::rename(tmp.c_str(), path("iteration2").c_str()) != 0) die("cannot rename iteration2");
  }
  {  // calc_stress record (XX:1963-1994 / YZ likewise)
    FILE* f = std::fopen(path("stress_tensor").c_str(), "a");
    const double Em = in.Em1, nu = in.nu1;
    std::fprintf(f, " Elastic medium properties\n Ypung modulus Em = %.16E\n Poisson ratio nu = %.16E\n", Em, nu);
    std::fprintf(f, " Stiffness coefficients\n C_xxxx = %.16E\n C_yyxx = %.16E\n C_xyxy = %.16E\n",
                 Em * (nu - 1.0) / (2.0 * nu * nu + nu - 1.0), Em * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)),
                 Em / (2.0 * (1.0 + nu)));
    std::fprintf(f, " Simulation parameters\n Cell volume vcell = %.16E\n", (double)in.ncx * in.ncy * in.ncz);
    std::fprintf(f, " Solid part volume(elementary cubes) rncub = %.16E\n", (double)r.ncube);
    std::fprintf(f, " Global strain = %.16E\n Simulation results\n averaged stress tensor over ALL the cell\n asigmap = \n",
                 r.strain);
    for (int c = 0; c < 3; c++)  // asigmap(1:3, c), Fortran column order
      std::fprintf(f, " %.16E %.16E %.16E\n", r.sigma[c] / r.ncube, r.sigma[3 + c] / r.ncube, r.sigma[6 + c] / r.ncube);
    std::fprintf(f, " Effective stiffness coefficients\n %s = %.16E\n", load == PS_LOAD_XSTRETCH ? "Exxxx" : "Eyzyz",
                 r.modulus);
    std::fclose(f);
  }
  if (!quiet)
    std::printf("%s = %.10e  (%lld iterations, relative residual %.3e)\n", load == PS_LOAD_XSTRETCH ? "Exxxx" : "Eyzyz",
                r.modulus, (long long)r.inner_iterations, r.relres);
  ps_lsm_destroy(h);
  return 0;
}

}  // namespace

int main(int argc, char** argv)
{
  int prec = PS_PREC_F64, lsm_load = -1;
  bool quiet = false;
  std::string pname = "f64";
  for (int a = 1; a < argc; a++) {
    const std::string s = argv[a];
    if (s == "-d" && a + 1 < argc) {
      g_dir = argv[++a];
    } else if (s == "-p" && a + 1 < argc) {
      pname = argv[++a];
    } else if (s == "-m" && a + 1 < argc) {
      const std::string m = argv[++a];
      if (m == "lbm") lsm_load = -1;
      else if (m == "xx") lsm_load = PS_LOAD_XSTRETCH;
      else if (m == "yz") lsm_load = PS_LOAD_YZSHEAR;
      else die("unknown mode " + m);
    } else if (s == "-q") {
      quiet = true;
    } else {
      die("usage: porescale_run [-d DIR] [-m lbm|xx|yz] [-p f64|f32|f16|bf16 (lbm) | f64|mixed (xx, yz)] [-q]");
    }
  }
  if (lsm_load >= 0) {
    const int lp = pname == "f64" ? PS_LSM_F64 : pname == "mixed" ? PS_LSM_MIXED : -1;
    if (lp < 0) die("unknown spring-solve precision " + pname);
    return run_lsm(lsm_load, lp, quiet);
  }
  prec = pname == "f64" ? PS_PREC_F64 : pname == "f32" ? PS_PREC_F32 : pname == "f16" ? PS_PREC_F16 : pname == "bf16" ? PS_PREC_BF16 : -1;
  if (prec < 0) die("unknown precision " + pname);
  const Input in = read_input();
  if (in.mtype != 0) die("mtype = 1 (interpolation rule) is not supported: the reference's own path is dead code");
  check_velocities();
  std::vector<int32_t> ind = read_ind(in.ncx, in.ncy, in.ncz);

  ps_lbm_params p{};
  p.cr2 = in.cr2;
  p.rr0 = in.rr0;
  p.rb0 = in.rb0;
  p.B = in.B;
  p.sig = in.sig;
  p.vir = in.vir;
  p.vib = in.vib;
  p.wet = in.wet;
  p.ee = in.ee;
  p.dt = in.dt;
  for (int i = 0; i < 3; i++) {
    p.bfr[i] = in.bfr[i];
    p.bfb[i] = in.bfb[i];
  }
  p.idir = in.idir;
  p.iipore = in.iipore;
  void* h = nullptr;
  check(ps_lbm_create(&p, ind.data(), in.ncx, in.ncy, in.ncz, prec, &h), "ps_lbm_create");
  ps_lbm_info info{};
  check(ps_lbm_get_info(h, &info), "ps_lbm_get_info");
  const long long nl = info.nl;
  std::vector<double> fr((size_t)19 * nl), fb((size_t)19 * nl);

  int itms = 1;
  if (in.icon == 1) {
    int it1 = 0;
    if (!read_state(it1, fr, fb)) die("icon = 1 but iteration2 is missing");
    check(ps_lbm_set_state(h, fr.data(), fb.data()), "ps_lbm_set_state");
    itms = it1 + 1;
  } else {
    check(ps_lbm_init_random(h, in.sat), "ps_lbm_init_random");
    FILE* f = std::fopen(path("output.m").c_str(), "w");
    const char* cols[] = {"1 - iteration", "2 - red  permeability", "3 - blue permeability",
                          "4 - red capillary number, volume average", "5 - blue capillary number, volume average",
                          "6 - red capillary number, phase average", "7 - blue capillary number, phase average",
                          "8 - capillary pressure P_r - P_b, phase average", "9 - capillary pressure P_red, phase average",
                          "10 - capillary pressure P_blue, phase average", "11 - saturation red = number of red/number",
                          "12 - saturation blue = number of blue/number"};
    for (const char* c : cols) std::fprintf(f, " %% %s\n", c);
    std::fprintf(f, " out = [\n");
    std::fclose(f);
    std::fclose(std::fopen(path("check_state_19").c_str(), "w"));
  }
  {  // settings_19, the LBM block (S1:1442-1488)
    FILE* f = std::fopen(path("settings_19").c_str(), "w");
    std::fprintf(f, " LBM settings\n Physical parameters\n iipore = %d\n npores = %d\n", in.iipore, in.npores);
    std::fprintf(f, " surface tension parameter sig = %.16E\n wettability parameter wet = %.16E\n", in.sig, in.wet);
    std::fprintf(f, " red fluid cinematic viscosity vir = %.16E\n blue fluid cinematic viscosity vib = %.16E\n", in.vir, in.vib);
    std::fprintf(f, " red fluid body force bfr = %.16E %.16E %.16E\n", in.bfr[0], in.bfr[1], in.bfr[2]);
    std::fprintf(f, " blue fluid body force bfb = %.16E %.16E %.16E\n", in.bfb[0], in.bfb[1], in.bfb[2]);
    std::fprintf(f, " Computational domain properties\n Unit cell size xyz = %d x %d x %d\n", in.ncx, in.ncy, in.ncz);
    std::fprintf(f, " number of liquid points nl = %lld\n simple propagation entries nps = %lld\n", (long long)info.nl,
                 (long long)info.nps);
    std::fprintf(f, " bounce-back boundary condition entries npb2 = %lld\n", (long long)info.npb2);
    std::fprintf(f, " bounce-back boundary condition entries npb4 = %lld\n", (long long)info.npb4);
    std::fprintf(f, " number of solid points ns = %lld\n", (long long)info.ns);
    std::fprintf(f, " Lattice Boltzmann algorithm parameters\n interface width parameter B = %.16E\n", in.B);
    std::fprintf(f, " direction of the body force idir = %d\n number of steps in the main loop itm = %d\n", in.idir, in.itm);
    std::fprintf(f, " number of steps in the inner loop itw = %d\n population storage = %s\n", in.itw,
                 prec == PS_PREC_F64 ? "f64" : prec == PS_PREC_F32 ? "f32" : prec == PS_PREC_F16 ? "f16" : "bf16");
    std::fclose(f);
  }
  check(ps_lbm_step(h, 2), "ps_lbm_step (initialisation)");  // S1:3454-3621
  ps_lbm_obs ob{};
  for (int it1 = itms; it1 <= in.itm; it1++) {
    check(ps_lbm_step(h, in.itw), "ps_lbm_step");
    check(ps_lbm_get_state(h, fr.data(), fb.data()), "ps_lbm_get_state");
    write_state("iteration", it1, fr, fb);  // the reference's two-file scheme (S1:3951-3961)
    write_state("iteration2", it1, fr, fb);
    std::remove(path("iteration").c_str());
    check(ps_lbm_observables(h, &ob), "ps_lbm_observables");
    // viscosities re-derived from the relaxation rates, as majorityrule does
    // before check_state (S1:3419-3420)
    const double svr = 1.0 / (3.0 * in.vir * in.dt + 0.5), svb = 1.0 / (3.0 * in.vib * in.dt + 0.5);
    const double vir = (1.0 / in.dt) * (1.0 / svr - 0.5) / 3.0, vib = (1.0 / in.dt) * (1.0 / svb - 0.5) / 3.0;
    const double sig = 0.03125 * in.sig;
    const int id = in.idir - 1;
    {  // check_state_19 block (S1:3244-3268)
      FILE* f = std::fopen(path("check_state_19").c_str(), "a");
      std::fprintf(f, " --------------------\n Iteration it1 = %d\n", it1);
      std::fprintf(f, " Reynolds number = %.16E\n", in.lsize * ob.bmt[2] / (ob.tmb * vir));
      std::fprintf(f, " total mass = %.16E\n mean flow velocity(seepage) = %.16E %.16E %.16E\n", ob.tm, ob.um[0],
                   ob.um[1], ob.um[2]);
      std::fprintf(f, " total red mass = %.16E\n red mass flux/t0 %.16E %.16E %.16E\n", ob.tmr, ob.Qr[0], ob.Qr[1], ob.Qr[2]);
      std::fprintf(f, " red number = %.16E\n red permeability %.16E\n", ob.nr, ob.permr);
      std::fprintf(f, " total blue mass = %.16E\n blue mass flux/t0 %.16E %.16E %.16E\n", ob.tmb, ob.Qb[0], ob.Qb[1],
                   ob.Qb[2]);
      std::fprintf(f, " blue number = %.16E\n blue permeability %.16E\n", ob.nb, ob.permb);
      if (ob.isneg) std::fprintf(f, " ATTENTION!!!, there are negative populations\n");
      std::fprintf(f, " --------------------\n");
      std::fclose(f);
    }
    {  // output.m row (S1:3274-3282, format 1X,I9,11(1X,E15.8),1X,';')
      FILE* f = std::fopen(path("output.m").c_str(), "a");
      const double cols[11] = {ob.permr,
                               ob.permb,
                               0.03125 * ob.Qr[id] * vir / sig,
                               0.03125 * ob.Qb[id] * vib / sig,
                               0.03125 * ob.umr[id] * vir * in.rr0 / (ob.nr * sig),
                               0.03125 * ob.umb[id] * vib * in.rb0 / (ob.nb * sig),
                               ob.Cpr - ob.Cpb,
                               ob.Cpr,
                               ob.Cpb,
                               ob.sat_r,
                               ob.sat_b};
      std::fprintf(f, " %9d", it1 * in.itw);
      for (double c : cols) std::fprintf(f, " %s", e15_8(c).c_str());
      std::fprintf(f, " ;\n");
      std::fclose(f);
    }
    if (!quiet)
      std::printf("it1 = %d  permr = %.6e  permb = %.6e  sat_r = %.4f\n", it1, ob.permr, ob.permb, ob.sat_r);
  }
  FILE* f = std::fopen(path("output.m").c_str(), "a");
  std::fprintf(f, " ];\n");
  std::fclose(f);
  ps_lbm_destroy(h);
  return 0;
}
