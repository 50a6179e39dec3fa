#include "lbm.hpp"

#include "System.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>

namespace {
// The solver options that ./input.in's extension keys set (System.hpp), so the
// reference's own main(), which passes only the grid, tau, rho0 and u0, can
// select them too.  Keys the file does not set keep the constructor's defaults
// (the reference's profile, FP64 storage and arithmetic); a bad key or value
// throws.  No input.in: nothing changes.
void apply_input_extensions(cflbm_config &c) {
  System s("input.in");
  if (s.ext_error) throw std::runtime_error(s.error);
  for (const std::string &k : s.ext_keys) {
    if (k == "profile") c.profile = s.profile;
    else if (k == "storage") c.storage = s.storage;
    else if (k == "compute") c.compute = s.compute;
    else if (k == "rounding") c.rounding = s.rounding;
    else if (k == "geom") c.geom = s.geom;
    else if (k == "center") { c.cx = s.cx; c.cy = s.cy; c.cz = s.cz; }
    else if (k == "diam") c.diam = s.diam;
    else if (k == "wall_y") c.wall_y = s.wall_y;
    else if (k == "wall_z") c.wall_z = s.wall_z;
    else if (k == "perturb") c.perturb_amp = s.perturb;
    else if (k == "seed") c.seed = s.seed;
  }
}

// The reference's ghost widths: 2 in 2-D ("MPI Kokkos/lbm.hpp:19"), 3 in 3-D
// ("3D MPI+KOKKOS+MPIIO/lbm.hpp:22").
int ghost_of(int dim) { return dim == 2 ? 2 : 3; }
}  // namespace

LBM::LBM(MPI_Comm comm_, int sx, int sy, int sz, double &tau, double &rho0_, double &u0_)
    : glx(sx), gly(sy), glz(sz), rho0(rho0_), tau0(tau), u0(u0_), dim(3),
      ua(this, 0), va(this, 1), wa(this, 2), p(this, 3), f(this), usr(this), rho(this) {
  comm.comm = comm_;
  const int G = ghost_of(3);
  l_l[0] = sx;
  l_l[1] = sy;
  l_l[2] = sz;
  for (int d = 0; d < 3; ++d) {
    l_s[d] = G;
    l_e[d] = G + l_l[d];
  }
  lx = sx + 2 * G;
  ly = sy + 2 * G;
  lz = sz + 2 * G;
  x_hi = sx - 1;
  y_hi = sy - 1;
  z_hi = sz - 1;
  cflbm_config_default(&config);
  config.lattice = CFLBM_D3Q27;
  config.profile = CFLBM_PROFILE_REF3D;
  config.nx = sx;
  config.ny = sy;
  config.nz = sz;
  apply_input_extensions(config);
}

LBM::LBM(MPI_Comm comm_, int sx, int sy, double &tau, double &rho0_, double &u0_)
    : glx(sx), gly(sy), glz(1), rho0(rho0_), tau0(tau), u0(u0_), dim(2),
      ua(this, 0), va(this, 1), wa(this, 2), p(this, 3), f(this), usr(this), rho(this) {
  comm.comm = comm_;
  const int G = ghost_of(2);
  l_l[0] = sx;
  l_l[1] = sy;
  l_l[2] = 1;
  for (int d = 0; d < 3; ++d) {
    l_s[d] = G;
    l_e[d] = G + l_l[d];
  }
  lx = sx + 2 * G;
  ly = sy + 2 * G;
  lz = 1;
  x_hi = sx - 1;
  y_hi = sy - 1;
  cflbm_config_default(&config);
  config.lattice = CFLBM_D2Q9;
  config.profile = CFLBM_PROFILE_REF2D;
  config.nx = sx;
  config.ny = sy;
  config.nz = 1;
  apply_input_extensions(config);
}

LBM::LBM(int sx, int sy, double &tau, double &rho0_, double &u0_)
    : glx(sx + 1), gly(sy + 1), glz(1), rho0(rho0_), tau0(tau), u0(u0_), dim(2), serial(true),
      ua(this, 0), va(this, 1), wa(this, 2), p(this, 3), f(this), usr(this), rho(this) {
  const int G = ghost_of(2);
  l_l[0] = glx;
  l_l[1] = gly;
  l_l[2] = 1;
  for (int d = 0; d < 3; ++d) {
    l_s[d] = G;
    l_e[d] = G + l_l[d];
  }
  lx = sx + 5;
  ly = sy + 5;
  lz = 1;
  x_hi = glx - 1;
  y_hi = gly - 1;
  cflbm_config_default(&config);
  config.lattice = CFLBM_D2Q9;
  config.profile = CFLBM_PROFILE_REF2DS;
  config.nx = glx;
  config.ny = gly;
  config.nz = 1;
  apply_input_extensions(config);
}

LBM::~LBM() {
  if (h_) {
    try {
      flush_forces();
    } catch (...) {
    }
    cflbm_destroy(h_);
  }
}

void LBM::check(int rc, const char *what) {
  if (rc != CFLBM_OK)
    throw std::runtime_error(std::string(what) + ": " + cflbm_last_error());
}

void LBM::Initialize() {
  config.tau0 = tau0;
  config.u0 = u0;
  check(cflbm_create(&config, &h_), "cflbm_create");
  fetched_step_ = -1;
  pops_step_ = -1;
  solid_.clear();
}

void LBM::Collision() {
  if (++pending_ >= 1024) flush_forces();  // runs the queued steps first
}

void LBM::flush_steps() {
  if (pending_ > 0 && h_) {
    const int n = pending_;
    pending_ = 0;
    check(cflbm_step(h_, n), "cflbm_step");
  }
}

void LBM::Streaming() {}

void LBM::Update() {}

const std::vector<double> &LBM::field(int which) {
  flush_steps();
  cflbm_info info;
  check(cflbm_get_info(h_, &info), "cflbm_get_info");
  if (fetched_step_ != info.steps_done) {
    const size_t N = (size_t)glx * gly * glz;
    for (auto &v : f_) v.resize(N);
    check(cflbm_macros(h_, f_[0].data(), f_[1].data(), f_[2].data(), f_[3].data()),
          "cflbm_macros");
    fetched_step_ = info.steps_done;
  }
  return f_[which];
}

const std::vector<double> &LBM::populations() {
  flush_steps();
  cflbm_info info;
  check(cflbm_get_info(h_, &info), "cflbm_get_info");
  if (pops_step_ != info.steps_done) {
    pops_.resize((size_t)info.lattice * glx * gly * glz);
    check(cflbm_get_f_stream(h_, pops_.data()), "cflbm_get_f_stream");
    pops_step_ = info.steps_done;
  }
  return pops_;
}

const std::vector<uint8_t> &LBM::solid() {
  if (solid_.empty()) {
    if (!h_) throw std::runtime_error("LBM::usr before Initialize()");
    solid_.resize((size_t)glx * gly * glz);
    check(cflbm_get_solid(h_, solid_.data()), "cflbm_get_solid");
  }
  return solid_;
}

// "MPI Kokkos/lbm.cpp:398-407": every step appends "Cd Cl" (fixed, 17 digits)
// to test.dat.  Kept on the GPU and appended in bulk here.
void LBM::flush_forces() {
  flush_steps();
  if (dim != 2 || serial || !h_) return;  // the serial variant writes no test.dat
  cflbm_info info;
  check(cflbm_get_info(h_, &info), "cflbm_get_info");
  const int64_t todo = info.steps_done - forces_flushed_;
  if (todo <= 0) return;
  std::vector<double> hist(3 * (size_t)todo);
  int64_t n = 0;
  check(cflbm_force_history(h_, hist.data(), todo, &n), "cflbm_force_history");
  std::ofstream out("test.dat", std::ios::out | std::ios::app);
  for (int64_t k = 0; k < n; ++k)
    out << std::fixed << std::setprecision(17) << 2.0 * hist[3 * k] / u0 / u0 / 0.03125 / (glx - 1)
        << " " << 2.0 * hist[3 * k + 1] / u0 / u0 / 0.03125 / (glx - 1) << std::endl;
  forces_flushed_ = info.steps_done;
}

void LBM::MPIoutput(int n) {
  flush_forces();
  const std::string name = "output" + std::to_string(n) + ".plt";
  check(cflbm_write_tecplot(h_, name.c_str(), n), "cflbm_write_tecplot");
}

// The ASCII debugging dump ("MPI Kokkos/lbm.cpp:738-765", "3D.../lbm.cpp:741-771").
// 2-D: x, y, u, v, p per node; 3-D: the node's integer coordinates and
// population 1 as the reference's f holds it after Update: the post-stream,
// pre-collision value (the initial equilibrium at n = 0).
void LBM::Output(int n) {
  flush_forces();
  std::ofstream out;
  // The serial variant names its files output<n>.dat and writes x as
  // 4 (i - 2) / (lx - 5) ("Kokkos/lbm.cpp:219-243").
  const std::string name =
      "output" + std::to_string(n) + (serial ? "" : std::to_string(comm.me)) + ".dat";
  out << std::setiosflags(std::ios::fixed);
  out.open(name, std::ios::out);
  if (dim == 2 && serial) {
    const auto &u = field(0), &v = field(1), &pp = field(3);
    out << "variables=x,y,u,v,p" << std::endl;
    out << "zone I=" << lx - 4 << ",J=" << ly - 4 << std::endl;
    for (int j = 0; j < gly; ++j)
      for (int i = 0; i < glx; ++i) {
        const size_t c = (size_t)j * glx + i;
        out << std::setprecision(8) << std::setiosflags(std::ios::left)
            << 4 * (double)i / (lx - 5.0) << " " << (double)j / (ly - 5.0) << " " << u[c] << " "
            << v[c] << " " << pp[c] << std::endl;
      }
  } else if (dim == 2) {
    const auto &u = field(0), &v = field(1), &pp = field(3);
    out << "variables=x,y,u,v,p" << std::endl;
    out << "zone I=" << lx - 4 << ",J=" << ly - 4 << std::endl;
    for (int j = 0; j < gly; ++j)
      for (int i = 0; i < glx; ++i) {
        const size_t c = (size_t)j * glx + i;
        out << std::setprecision(8) << std::setiosflags(std::ios::left) << (i + x_lo) / (glx - 1.0)
            << " " << (j + y_lo) / (gly - 1.0) << " " << u[c] << " " << v[c] << " " << pp[c]
            << std::endl;
      }
  } else {
    const size_t N = (size_t)glx * gly * glz;
    const std::vector<double> &f = populations();
    out << "variables=x,y,z,f" << std::endl;
    out << "zone I=" << lx - 6 << ",J=" << ly - 6 << ",K=" << lz - 6 << std::endl;
    for (int k = 0; k < glz; ++k)
      for (int j = 0; j < gly; ++j)
        for (int i = 0; i < glx; ++i)
          out << std::setprecision(8) << std::setiosflags(std::ios::left) << x_lo + i << " "
              << y_lo + j << " " << z_lo + k << " " << f[N + ((size_t)k * gly + j) * glx + i]
              << std::endl;
  }
  if (comm.me == 0) {
    std::printf("\nThe result %d is writen\n\n============================\n", n);
  }
}

double HostField::operator()(int i, int j) const {
  LBM *o = owner_;
  const int G = o->l_s[0];
  const int x = i - G, y = j - G;
  if (x < 0 || x >= o->glx || y < 0 || y >= o->gly) return 0.0;
  return o->field(which_)[(size_t)y * o->glx + x];
}

double HostField::operator()(int i, int j, int k) const {
  LBM *o = owner_;
  const int G = o->l_s[0];
  const int x = i - G, y = j - G, z = k - G;
  if (x < 0 || x >= o->glx || y < 0 || y >= o->gly || z < 0 || z >= o->glz) return 0.0;
  return o->field(which_)[((size_t)z * o->gly + y) * o->glx + x];
}

const double *HostField::data() const { return owner_->field(which_).data(); }
size_t HostField::size() const { return owner_->field(which_).size(); }

double HostPops::operator()(int ii, int i, int j) const { return (*this)(ii, i, j, 0); }

double HostPops::operator()(int ii, int i, int j, int k) const {
  LBM *o = owner_;
  const int G = o->l_s[0];
  const int x = i - G, y = j - G, z = o->dim == 2 ? 0 : k - G;
  if (x < 0 || x >= o->glx || y < 0 || y >= o->gly || z < 0 || z >= o->glz) return 0.0;
  const size_t N = (size_t)o->glx * o->gly * o->glz;
  return o->populations()[(size_t)ii * N + ((size_t)z * o->gly + y) * o->glx + x];
}

int HostUsr::operator()(int i, int j) const { return (*this)(i, j, owner_->l_s[0]); }

int HostUsr::operator()(int i, int j, int k) const {
  LBM *o = owner_;
  const int G = o->l_s[0];
  const int x = i - G, y = j - G, z = o->dim == 2 ? 0 : k - G;
  if (x < 0 || x >= o->glx || y < 0 || y >= o->gly || z < 0 || z >= o->glz) return 1;
  return o->solid()[((size_t)z * o->gly + y) * o->glx + x] ? 0 : 1;
}

double HostRho::operator()(int, int) const { return owner_->rho0; }
double HostRho::operator()(int, int, int) const { return owner_->rho0; }
