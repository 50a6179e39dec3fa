// Drop-in replacement of the reference's LBM solver class on one GPU.
//
// Same class name, constructor arguments and method names as
//   3-D: "3D MPI+KOKKOS+MPIIO/lbm.hpp:106-233"
//        LBM(MPI_Comm, int sx, int sy, int sz, double &tau, double &rho0, double &u0)
//   2-D: "MPI Kokkos/lbm.hpp:64-128"
//        LBM(MPI_Comm, int sx, int sy, double &tau, double &rho0, double &u0)
//   2-D serial: "Kokkos/lbm.hpp:20-70"
//        LBM(int sx, int sy, double &tau, double &rho0, double &u0)
// so the reference's main() drives it unchanged.  All state lives on the GPU
// behind the C ABI (include/cflbm.h); the rank count is one, so
// setup_subdomain/pack/exchange/unpack do nothing.  Collision() accounts for one
// fused time step (collide + stream + boundaries + macroscopic update); the steps
// are queued and run together -- one cflbm_step call, replayed from CUDA graphs
// -- when a result is needed (MPIoutput, Output, the fields, test.dat, the
// handle) or every 1024 steps, so a main loop that steps one at a time runs as
// fast as one that asks for many steps.  Streaming() and Update() do nothing
// more; the 2-D per-step "Cd Cl" record of test.dat is kept on the GPU and
// appended in bulk.
//
// The constructors apply the solver options that ./input.in's extension keys
// set (System.hpp), so the reference's own main() selects them too; main()s
// that set `config` themselves override them before Initialize().
//
// ua/va/wa/p are host views of the macroscopic fields with the reference's
// ghost-inclusive indexing (ua(i,j,k) with i in [ghost, lx-ghost)); they are
// refreshed from the GPU on first access after a step.  f(ii,i,j,k) views the
// populations as the reference's f holds them after Update -- the post-stream,
// pre-collision state (cflbm_get_f_stream) -- usr(i,j,k) the solid mask (1 =
// fluid, 0 = solid, "3D MPI+KOKKOS+MPIIO/lbm.cpp:238") and rho(i,j,k) the
// density field, which the reference sets to rho0 in Initialize and never
// updates (lbm.cpp:237; the flow's density is 1 + 3p).  Ghost nodes read as 0
// (f, the macroscopic fields), 1 (usr) and rho0 (rho).
#ifndef CFLBM_HOST_LBM_HPP
#define CFLBM_HOST_LBM_HPP

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cflbm.h"

#include "mpi.h"  // the single-rank stand-in next to this header

struct LBM;

// Host view of one macroscopic field (reference indexing, ghosts read as 0).
class HostField {
 public:
  HostField(LBM *o, int which) : owner_(o), which_(which) {}
  double operator()(int i, int j) const;
  double operator()(int i, int j, int k) const;
  const double *data() const;
  size_t size() const;

 private:
  LBM *owner_;
  int which_;
};

// Host view of the populations (reference indexing f(ii, i, j[, k])).
class HostPops {
 public:
  explicit HostPops(LBM *o) : owner_(o) {}
  double operator()(int ii, int i, int j) const;
  double operator()(int ii, int i, int j, int k) const;

 private:
  LBM *owner_;
};

// Host view of the reference's usr (1 = fluid, 0 = solid) and rho (rho0).
class HostUsr {
 public:
  explicit HostUsr(LBM *o) : owner_(o) {}
  int operator()(int i, int j) const;
  int operator()(int i, int j, int k) const;

 private:
  LBM *owner_;
};
class HostRho {
 public:
  explicit HostRho(LBM *o) : owner_(o) {}
  double operator()(int, int) const;
  double operator()(int, int, int) const;

 private:
  LBM *owner_;
};

struct CommHelper {
  MPI_Comm comm = 0;
  int me = 0, nranks = 1;
  int rx = 1, ry = 1, rz = 1, px = 0, py = 0, pz = 0;
};

struct LBM {
  CommHelper comm;
  int glx, gly, glz;
  int lx, ly, lz;
  int l_s[3], l_e[3], l_l[3];
  int x_lo = 0, x_hi = 0, y_lo = 0, y_hi = 0, z_lo = 0, z_hi = 0;
  double rho0, mu = 0, cs2 = 1.0 / 3.0, tau0, u0;
  int dim;
  bool serial = false;  // the serial 2-D variant (its Output file name and coordinates)
  HostField ua, va, wa, p;
  HostPops f;
  HostUsr usr;
  HostRho rho;

  LBM(MPI_Comm comm_, int sx, int sy, int sz, double &tau, double &rho0_, double &u0_);
  LBM(MPI_Comm comm_, int sx, int sy, double &tau, double &rho0_, double &u0_);
  // The serial 2-D variant ("Kokkos/lbm.hpp:26"): LBM(sx, sy, tau, rho0, u0) with
  // lx = sx + 5, ly = sy + 5, i.e. (sx + 1) x (sy + 1) interior nodes.
  LBM(int sx, int sy, double &tau, double &rho0_, double &u0_);
  ~LBM();
  LBM(const LBM &) = delete;
  LBM &operator=(const LBM &) = delete;

  // Solver options beyond the reference's arguments (defaults: reference profile,
  // FP64 storage and arithmetic).  Set before Initialize().
  cflbm_config config;

  void Initialize();
  void Collision();
  void setup_subdomain() {}
  void pack() {}
  void exchange() {}
  void unpack() {}
  void Streaming();
  void Update();
  void MPIoutput(int n);
  void Output(int n);

  // The handle, with every queued step run.
  cflbm_handle *handle() {
    flush_steps();
    return h_;
  }
  const std::vector<double> &field(int which);
  // Post-stream populations of the last step, [ii][z][y][x] (cflbm_get_f_stream).
  const std::vector<double> &populations();
  // Interior solid mask, x fastest (cflbm_get_solid).
  const std::vector<uint8_t> &solid();

 private:
  void check(int rc, const char *what);
  void flush_forces();
  void flush_steps();
  cflbm_handle *h_ = nullptr;
  int pending_ = 0;  // steps accounted for by Collision() and not yet run
  std::vector<double> f_[4];
  int64_t fetched_step_ = -1;
  std::vector<double> pops_;
  int64_t pops_step_ = -1;
  std::vector<uint8_t> solid_;
  int64_t forces_flushed_ = 0;
  friend class HostField;
  friend class HostPops;
  friend class HostUsr;
  friend class HostRho;
};

#endif
