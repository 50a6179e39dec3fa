// Drop-in replacement of the reference's LBM solver class on one GPU.
//
// Same class name, constructor arguments and method names as
//   3-D: "3D MPI+KOKKOS+MPIIO/lbm.hpp:106-233"
//        LBM(MPI_Comm, int sx, int sy, int sz, double &tau, double &rho0, double &u0)
//   2-D: "MPI Kokkos/lbm.hpp:64-128"
//        LBM(MPI_Comm, int sx, int sy, double &tau, double &rho0, double &u0)
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
// ua/va/wa/p are host views of the macroscopic fields with the reference's
// ghost-inclusive indexing (ua(i,j,k) with i in [ghost, lx-ghost)); they are
// refreshed from the GPU on first access after a step.
#ifndef CFLBM_HOST_LBM_HPP
#define CFLBM_HOST_LBM_HPP

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cflbm.h"

#ifndef MPI_VERSION
typedef int MPI_Comm;
#ifndef MPI_COMM_WORLD
#define MPI_COMM_WORLD 0
#endif
#endif

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
  HostField ua, va, wa, p;

  LBM(MPI_Comm comm_, int sx, int sy, int sz, double &tau, double &rho0_, double &u0_);
  LBM(MPI_Comm comm_, int sx, int sy, double &tau, double &rho0_, double &u0_);
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

 private:
  void check(int rc, const char *what);
  void flush_forces();
  void flush_steps();
  cflbm_handle *h_ = nullptr;
  int pending_ = 0;  // steps accounted for by Collision() and not yet run
  std::vector<double> f_[4];
  int64_t fetched_step_ = -1;
  int64_t forces_flushed_ = 0;
  friend class HostField;
};

#endif
