// lns3d_gpu: the reference program's implicit run (src/lns3d.f90 with the
// implicit drivers src/impdrv.f90 and src/impdrv3d.f90) as a host program
// over the C ABI of lns3d_gb300 -- what the Fortran host does with the
// iso_c_binding module, for machines without a Fortran compiler.
//
//   lns3d_gpu < deck.inp            (in the run directory, like lns3d)
//
// It keeps the reference's inputs and outputs:
//   deck on standard input, read as src/input.f90 reads it (one list-directed
//     read per statement, the rest of each line skipped);
//   grid.dat, metric.dat (src/gengrid.f90:17-80), mean.dat for linear runs
//     (src/genmean.f90:28-32), the restart output.R.N of the highest N present
//     (src/genini.f90, src/genini3d.f90), top.pot for the nonlinear Riemann
//     top (src/potential.f90:20-26);
//   writes the history output.h.N (one line per step: lstep, time, Delt, cfl,
//     totres of the step's last corrector, at full precision) and restart
//     files output.R.N every ntout steps and at the end
//     (src/impdrv.f90:430-466), with the reference's version numbering.
// Files are the gfortran layout (4-byte record markers), little-endian, or
// big-endian when GFORTRAN_CONVERT_UNIT=swap is set, as for the reference.
//
// Runs: complex single-mode (deck Lz != 0, linear = 1) on lns_ctx3d; linear
// 2D (Lz = 0, linear = 1) on lns_lin2d; nonlinear 2D (linear = 0) on
// lns_ctx2d; with the options those contexts support (they reject the
// others).  Sponges (ispg) are not set up here; impl = 2 restarts from a
// step count above zero are rejected (the contexts start the two-step
// scheme with backward Euler).
//
//   lns3d_gpu --echo-deck < deck.inp   prints the values read and stops.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../../include/lns3d_gb300.h"

namespace {

// ------------------------------------------------------------------ files
bool g_swap = false;

void swap_bytes(void* p, size_t es, size_t n) {
  unsigned char* b = (unsigned char*)p;
  for (size_t i = 0; i < n; ++i)
    for (size_t k = 0; k < es / 2; ++k) std::swap(b[i * es + k], b[i * es + es - 1 - k]);
}

[[noreturn]] void die(const std::string& msg) {
  std::fprintf(stderr, "lns3d_gpu: %s\n", msg.c_str());
  std::exit(1);
}

void check(int rc, const char* what) {
  if (rc != LNS_OK) die(std::string(what) + ": " + lns_last_error());
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) die(std::string(what) + ": " + cudaGetErrorString(e));
}

// the state stays on the device; it comes back only for restart files
struct DeviceState {
  double* v = nullptr;
  double* res = nullptr;
  size_t n = 0;
  explicit DeviceState(const std::vector<double>& host) : n(host.size()) {
    cuda_check(cudaMalloc(&v, sizeof(double) * n), "cudaMalloc");
    cuda_check(cudaMalloc(&res, sizeof(double)), "cudaMalloc");
    cuda_check(cudaMemcpy(v, host.data(), sizeof(double) * n, cudaMemcpyHostToDevice), "copy v in");
  }
  ~DeviceState() {
    cudaFree(v);
    cudaFree(res);
  }
  void fetch(std::vector<double>& host) const {
    cuda_check(cudaMemcpy(host.data(), v, sizeof(double) * n, cudaMemcpyDeviceToHost), "copy v out");
  }
  double residual() const {
    double r = 0.0;
    cuda_check(cudaMemcpy(&r, res, sizeof(double), cudaMemcpyDeviceToHost), "copy totres");
    return r;
  }
};

struct Record {
  std::vector<unsigned char> b;
  size_t pos = 0;
  template <typename T>
  void get(T* out, size_t n, size_t unit = sizeof(T)) {
    if (pos + n * sizeof(T) > b.size()) die("record too short");
    std::memcpy(out, b.data() + pos, n * sizeof(T));
    if (g_swap) swap_bytes(out, unit, n * sizeof(T) / unit);
    pos += n * sizeof(T);
  }
};

std::vector<Record> read_records(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) die("cannot open " + path);
  std::vector<Record> out;
  for (;;) {
    uint32_t n;
    if (std::fread(&n, 4, 1, f) != 1) break;
    if (g_swap) swap_bytes(&n, 4, 1);
    Record r;
    r.b.resize(n);
    uint32_t n2 = 0;
    if (std::fread(r.b.data(), 1, n, f) != n || std::fread(&n2, 4, 1, f) != 1) die("damaged record in " + path);
    if (g_swap) swap_bytes(&n2, 4, 1);
    if (n2 != n) die("damaged record in " + path);
    out.push_back(std::move(r));
  }
  std::fclose(f);
  return out;
}

struct Writer {
  std::vector<unsigned char> b;
  template <typename T>
  void put(const T* p, size_t n, size_t unit = sizeof(T)) {
    const size_t off = b.size();
    b.resize(off + n * sizeof(T));
    std::memcpy(b.data() + off, p, n * sizeof(T));
    if (g_swap) swap_bytes(b.data() + off, unit, n * sizeof(T) / unit);
  }
  void flush(FILE* f) {
    uint32_t n = (uint32_t)b.size(), m = n;
    if (g_swap) swap_bytes(&m, 4, 1);
    std::fwrite(&m, 4, 1, f);
    std::fwrite(b.data(), 1, b.size(), f);
    std::fwrite(&m, 4, 1, f);
    b.clear();
  }
};

bool exists(const std::string& p) {
  FILE* f = std::fopen(p.c_str(), "rb");
  if (f) std::fclose(f);
  return f != nullptr;
}

// src/getver.c igetver: the highest version N of base.ext.N present, 0 if none
int igetver(const std::string& base, const std::string& ext) {
  int best = 0;
  for (int v = 1; v < 100000; ++v) {
    if (exists(base + "." + ext + "." + std::to_string(v))) best = v;
    else if (v > best + 64) break;
  }
  return best;
}

// ------------------------------------------------------------------- deck
// list-directed reads: blanks or commas separate values; a read takes as
// many values as it has items, from further lines if needed; the rest of
// its last line is skipped
struct Deck {
  std::vector<std::string> lines;
  size_t li = 0;
  std::vector<std::string> toks;
  size_t ti = 0;
  void begin() {
    toks.clear();
    ti = 0;
  }
  std::string next() {
    while (ti >= toks.size()) {
      if (li >= lines.size()) die("deck ended early");
      std::string s = lines[li++];
      for (char& c : s)
        if (c == ',') c = ' ';
      std::istringstream is(s);
      toks.clear();
      ti = 0;
      std::string t;
      while (is >> t) toks.push_back(t);
    }
    return toks[ti++];
  }
  double real() {
    std::string t = next();
    for (char& c : t)
      if (c == 'd' || c == 'D') c = 'e';
    return std::strtod(t.c_str(), nullptr);
  }
  int integer() { return (int)std::strtol(next().c_str(), nullptr, 10); }
  bool logical() {
    std::string t = next();
    const char c = t[0] == '.' ? t[1] : t[0];
    return c == 't' || c == 'T';
  }
};

struct Input {
  double Ma, Re, Pref, Tref, Pr, dtmax, cflmax, eps_e, omega, x0, As, xs, xt, As2, xs2, xt2, theta, Lz;
  int mattyp, nstep, optx, opty, itout, ntout, ires, ispg, linear, impl, ilhs, niter, loctime;
  int top, wall, left, right, wallt, ibuff, idamp, Ns, Ns2, extrap;
  bool xper, yper, tflag, fflag, sflag;
  bool navier;
  double kz;
};

// src/input.f90:14-372
Input read_deck(Deck& d) {
  Input in{};
  d.begin(); in.Ma = d.real();
  d.begin(); in.mattyp = d.integer();
  d.begin(); in.Re = d.real();
  d.begin(); in.Pref = d.real(); in.Tref = d.real();
  in.navier = true;
  if (in.mattyp == 0 && in.Re == 0.0) {  // src/input.f90:40-44
    in.navier = false;
    in.Re = 1.0e99;
  }
  d.begin(); in.Pr = d.real();
  d.begin(); in.dtmax = d.real(); in.cflmax = d.real();
  d.begin(); in.nstep = d.integer();
  d.begin(); in.optx = d.integer(); in.opty = d.integer();
  d.begin(); in.xper = d.logical(); in.yper = d.logical();
  d.begin(); in.itout = d.integer(); in.ntout = d.integer();
  d.begin(); in.ires = d.integer();
  d.begin(); in.ispg = d.integer();
  d.begin(); in.linear = d.integer();
  d.begin(); in.impl = d.integer(); in.ilhs = d.integer(); in.niter = d.integer(); in.loctime = d.integer();
  d.begin(); in.top = d.integer(); in.wall = d.integer(); in.left = d.integer(); in.right = d.integer();
  in.wallt = d.integer();
  if (in.xper) in.left = in.right = -1;            // src/input.f90:115-120
  if (in.yper) in.wall = in.wallt = in.top = -1;   // src/input.f90:122-128
  d.begin(); in.eps_e = d.real(); in.ibuff = d.integer();
  d.begin(); in.omega = d.real(); in.x0 = d.real();
  d.begin(); in.idamp = d.integer();
  d.begin(); in.As = d.real(); in.Ns = d.integer(); in.xs = d.real(); in.xt = d.real();
  d.begin(); in.As2 = d.real(); in.Ns2 = d.integer(); in.xs2 = d.real(); in.xt2 = d.real();
  d.begin(); in.extrap = d.integer();
  d.begin(); in.theta = d.real();
  d.begin(); in.tflag = d.logical(); in.fflag = d.logical(); in.sflag = d.logical();
  d.begin(); in.Lz = d.real();
  in.kz = in.Lz != 0.0 ? 2.0 * 3.1415926535897932385e+0 / in.Lz : 0.0;   // src/input.f90:302-306
  return in;
}

void echo(const Input& in) {
  std::printf("Ma %.17g\nmattyp %d\nRe %.17g\nPref %.17g\nTref %.17g\nPr %.17g\ndtmax %.17g\ncflmax %.17g\n"
              "nstep %d\noptx %d\nopty %d\nxper %d\nyper %d\nitout %d\nntout %d\nires %d\nispg %d\nlinear %d\n"
              "impl %d\niLHS %d\nniter %d\nloctime %d\ntop %d\nwall %d\nleft %d\nright %d\nwallt %d\n"
              "eps_e %.17g\nibuff %d\nomega %.17g\nx0 %.17g\nidamp %d\nAs %.17g\nNs %d\nxs %.17g\nxt %.17g\n"
              "As2 %.17g\nNs2 %d\nxs2 %.17g\nxt2 %.17g\nextrap %d\ntheta %.17g\ntflag %d\nfflag %d\nsflag %d\n"
              "Lz %.17g\nkz %.17g\nnavier %d\n",
              in.Ma, in.mattyp, in.Re, in.Pref, in.Tref, in.Pr, in.dtmax, in.cflmax, in.nstep, in.optx, in.opty,
              in.xper, in.yper, in.itout, in.ntout, in.ires, in.ispg, in.linear, in.impl, in.ilhs, in.niter,
              in.loctime, in.top, in.wall, in.left, in.right, in.wallt, in.eps_e, in.ibuff, in.omega, in.x0,
              in.idamp, in.As, in.Ns, in.xs, in.xt, in.As2, in.Ns2, in.xs2, in.xt2, in.extrap, in.theta, in.tflag,
              in.fflag, in.sflag, in.Lz, in.kz, in.navier);
}

// ------------------------------------------------------------------ state
struct Header {
  int32_t lstep, nx, ny, nz, ndof;
  double time, Re, Ma, Pr, gamma, cv;
};

Header read_header(Record& r) {
  Header h{};
  r.get(&h.lstep, 1);
  r.get(&h.time, 1);
  r.get(&h.nx, 1);
  r.get(&h.ny, 1);
  r.get(&h.nz, 1);
  r.get(&h.ndof, 1);
  r.get(&h.Re, 1);
  r.get(&h.Ma, 1);
  r.get(&h.Pr, 1);
  r.get(&h.gamma, 1);
  r.get(&h.cv, 1);
  return h;
}

void write_restart(const std::string& path, const Header& h, const double* v, size_t nv) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) die("cannot write " + path);
  Writer w;
  w.put(&h.lstep, 1);
  w.put(&h.time, 1);
  w.put(&h.nx, 1);
  w.put(&h.ny, 1);
  w.put(&h.nz, 1);
  w.put(&h.ndof, 1);
  w.put(&h.Re, 1);
  w.put(&h.Ma, 1);
  w.put(&h.Pr, 1);
  w.put(&h.gamma, 1);
  w.put(&h.cv, 1);
  w.flush(f);
  w.put(v, nv, sizeof(double));
  w.flush(f);
  std::fclose(f);
}

}  // namespace

int main(int argc, char** argv) {
  const bool echo_only = argc > 1 && std::strcmp(argv[1], "--echo-deck") == 0;
  const char* conv = std::getenv("GFORTRAN_CONVERT_UNIT");
  g_swap = conv && std::strstr(conv, "swap");
  Deck deck;
  for (std::string line; std::getline(std::cin, line);) deck.lines.push_back(line);
  Input in = read_deck(deck);
  if (echo_only) {
    echo(in);
    return 0;
  }
  if (in.impl < 1 || in.impl > 3) die("impl must be 1, 2 or 3 for an implicit run");
  if (in.ispg != 0) die("sponges are not set up by this driver (ispg must be 0)");
  if (in.idamp != 0) die("the outflow damper is not supported (idamp must be 0)");
  if (in.mattyp != 0) die("constant viscosity only (mattyp 0)");

  // grid and metrics (src/gengrid.f90)
  auto grid = read_records("grid.dat");
  int32_t dims[3];
  grid[0].get(dims, 3);
  const int nx = dims[0], ny = dims[1];
  const size_t np = (size_t)nx * ny;
  std::vector<double> x(np), y(np);
  grid[1].get(x.data(), np);
  if (dims[2] > 1) grid[1].pos += (size_t)(dims[2] - 1) * np * 8;
  grid[1].get(y.data(), np);
  std::vector<double> metrics(10 * np);
  auto met = read_records("metric.dat");
  met[0].get(metrics.data(), 10 * np);
  const double dxi = 1.0 / (double)(nx - 1), deta = 1.0 / (double)(ny - 1);  // src/gengrid.f90:36,44

  // restart: the highest version of output.R (src/genini.f90)
  const std::string base = "output";
  const int iver0 = igetver(base, "R");
  const std::string rfile = base + ".R." + std::to_string(iver0);
  auto rst = read_records(rfile);
  Header h = read_header(rst[0]);
  if (h.nx != nx || h.ny != ny || h.ndof != 5) die("grid and data files are incompatible");
  if (in.impl == 2 && h.lstep > 0) die("impl = 2 restarts from lstep > 0 are not supported");
  const bool complex_run = in.kz != 0.0;
  std::vector<double> v(complex_run ? 10 * np : 5 * np);
  rst[1].get(v.data(), v.size());

  // history file (src/impdrv.f90:144-146)
  const std::string hfile = base + ".h." + std::to_string(igetver(base, "h") + 1);
  FILE* hist = std::fopen(hfile.c_str(), "w");
  if (!hist) die("cannot write " + hfile);

  int lstep = h.lstep;
  double time = h.time;
  const double gamma = 1.4, gamma1 = 0.4, cv = 716.5;  // src/init.f90:27-29
  Header out{0, nx, ny, 1, 5, 0.0, in.Re, in.Ma, in.Pr, gamma, cv};
  int iver = iver0;
  auto write_out = [&](const std::vector<double>& vv) {
    out.lstep = lstep;
    out.time = time;
    ++iver;
    while (exists(base + ".R." + std::to_string(iver))) ++iver;
    write_restart(base + ".R." + std::to_string(iver), out, vv.data(), vv.size());
    std::printf(" Wrote %s.R.%d at step = %d time = %.6e\n", base.c_str(), iver, lstep, time);
  };
  auto min_of = [](const std::vector<double>& a) {
    double m = a[0];
    for (double b : a) m = std::fmin(m, b);
    return m;
  };

  if (in.linear == 1) {
    // mean flow (src/genmean.f90)
    auto mean = read_records("mean.dat");
    read_header(mean[0]);
    std::vector<double> vm(5 * np);
    mean[1].get(vm.data(), vm.size());
    lns_params3d p{};
    p.nx = nx; p.ny = ny; p.dxi = dxi; p.deta = deta;
    p.Ma = in.Ma; p.Re = in.Re; p.Pr = in.Pr; p.gamma = gamma; p.gamma1 = gamma1;
    p.omega = complex_run ? in.omega : 0.0; p.beta = in.kz; p.alfa = 1.0;
    p.cflmax = in.cflmax; p.dtmax = in.dtmax; p.loctime = in.loctime;
    p.xper = in.xper; p.yper = in.yper; p.navier = in.navier;
    p.wall = in.wall; p.wallt = in.wallt; p.top = in.top; p.optx = in.optx; p.opty = in.opty;
    p.precision = LNS_FP64; p.impl = in.impl; p.ispg = 0; p.eps_e = in.eps_e;
    p.left = in.left; p.right = in.right;
    double cfl = 0.0;
    std::vector<double> dtl(np);
    if (complex_run) {
      // the eigenfunction planes read inflow.dat and the inflow namelist (src/gendist.f90)
      if (!in.xper && in.left == 4) die("the eigenfunction planes (left 4) are not set up by this driver");
      lns_ctx3d* c = nullptr;
      check(lns_ctx3d_create(&p, &c), "lns_ctx3d_create");
      check(lns_upload_metrics3d(c, metrics.data()), "lns_upload_metrics3d");
      // the forced top and the wave planes form their waves from x and x0 (wamp: ones)
      if (in.top == 1 || (!in.xper && (in.left == 1 || in.left == 5 || in.right == 5)))
        check(lns_upload_inflow3d(c, x.data(), nullptr, in.x0), "lns_upload_inflow3d");
      check(lns_upload_mean3d(c, vm.data(), &cfl), "lns_upload_mean3d");
      check(lns_get_field3d(c, 8, dtl.data()), "lns_get_field3d");
      const double delt = min_of(dtl);
      DeviceState dv(v);
      check(lns_itrbc3d_dev(c, dv.v, nullptr), "lns_itrbc3d_dev");  // src/impdrv3d.f90:125-126
      for (int istep = 1; istep <= in.nstep; ++istep) {
        check(lns_step3d_dev(c, dv.v, 1, in.niter, dv.res, nullptr), "lns_step3d_dev");
        time += delt;
        ++lstep;
        std::fprintf(hist, "%d %.17g %.17g %.17g %.17g\n", lstep, time, delt, cfl, dv.residual());
        if (lstep % in.ntout == 0 && istep != in.nstep) dv.fetch(v), write_out(v);
      }
      dv.fetch(v);
      lns_ctx3d_destroy(c);
    } else {
      lns_lin2d* c = nullptr;
      check(lns_lin2d_create(&p, &c), "lns_lin2d_create");
      check(lns_upload_metrics_lin2d(c, metrics.data()), "lns_upload_metrics_lin2d");
      check(lns_upload_mean_lin2d(c, vm.data(), &cfl), "lns_upload_mean_lin2d");
      check(lns_get_dtl_lin2d(c, dtl.data()), "lns_get_dtl_lin2d");
      const double delt = min_of(dtl);
      DeviceState dv(v);
      check(lns_itrbc_lin2d_dev(c, dv.v, nullptr), "lns_itrbc_lin2d_dev");  // src/impdrv.f90:160
      for (int istep = 1; istep <= in.nstep; ++istep) {
        check(lns_step_lin2d_dev(c, dv.v, 1, in.niter, dv.res, nullptr), "lns_step_lin2d_dev");
        time += delt;
        ++lstep;
        std::fprintf(hist, "%d %.17g %.17g %.17g %.17g\n", lstep, time, delt, cfl, dv.residual());
        if (lstep % in.ntout == 0 && istep != in.nstep) dv.fetch(v), write_out(v);
      }
      dv.fetch(v);
      lns_lin2d_destroy(c);
    }
  } else {
    if (complex_run) die("3D code must be linear");  // src/lns3d.f90:173
    // the Riemann planes read left.pot / right.pot and the &extras namelist's nbl
    if (!in.xper) die("a non-periodic xi direction of the nonlinear 2D step is not set up by this driver");
    lns_params2d p{};
    p.nx = nx; p.ny = ny; p.dxi = dxi; p.deta = deta;
    p.Ma = in.Ma; p.Re = in.Re; p.Pr = in.Pr; p.gamma = gamma; p.gamma1 = gamma1;
    p.alfa = 1.0; p.cflmax = in.cflmax; p.dtmax = in.dtmax; p.theta = in.theta;
    p.loctime = in.loctime; p.xper = in.xper; p.yper = in.yper; p.navier = in.navier;
    p.wall = in.wall; p.wallt = in.wallt; p.top = in.top; p.optx = in.optx; p.opty = in.opty;
    p.lhs_order = in.ilhs == 0 ? 2 : 4; p.impl = in.impl; p.ispg = 0; p.eps_e = in.eps_e;
    lns_ctx2d* c = nullptr;
    check(lns_ctx2d_create(&p, &c), "lns_ctx2d_create");
    check(lns_upload_metrics2d(c, metrics.data()), "lns_upload_metrics2d");
    // the top boundary normal (src/gengrid.f90:133-137) and top.pot
    std::vector<double> bnt(2 * (size_t)nx), pot(5 * (size_t)nx, 0.0);
    for (int i = 0; i < nx; ++i) {
      const size_t q = (size_t)i + (size_t)nx * (ny - 1);
      const double n1 = metrics[2 * np + q], n2 = metrics[3 * np + q];
      const double s = std::sqrt(n1 * n1 + n2 * n2);
      bnt[i] = n1 / s;
      bnt[nx + i] = n2 / s;
    }
    if (in.top == 0) {
      FILE* f = std::fopen("top.pot", "r");
      if (!f) die("Error in top.pot");
      for (int i = 0; i < nx; ++i)
        for (int k = 0; k < 5; ++k)
          if (std::fscanf(f, "%lf", &pot[5 * (size_t)i + k]) != 1) die("Error in top.pot");
      std::fclose(f);
    }
    check(lns_upload_top2d(c, bnt.data(), pot.data()), "lns_upload_top2d");
    std::vector<double> dtl(np);
    DeviceState dv(v);
    check(lns_itrbc2d_dev(c, dv.v, nullptr), "lns_itrbc2d_dev");  // src/impdrv.f90:160
    for (int istep = 1; istep <= in.nstep; ++istep) {
      check(lns_step2d_dev(c, dv.v, 1, in.niter, dv.res, nullptr), "lns_step2d_dev");
      check(lns_get_field2d(c, 6, dtl.data()), "lns_get_field2d");  // this step's set_time_step
      const double delt = min_of(dtl);
      time += delt;
      ++lstep;
      std::fprintf(hist, "%d %.17g %.17g %.17g %.17g\n", lstep, time, delt, 0.0, dv.residual());
      if (lstep % in.ntout == 0 && istep != in.nstep) dv.fetch(v), write_out(v);
    }
    dv.fetch(v);
    lns_ctx2d_destroy(c);
  }
  write_out(v);
  std::fclose(hist);
  return 0;
}
