// The reference's 3-D driver loop ("3D MPI+KOKKOS+MPIIO/main.cpp:6-51") on the
// GPU solver: System reads input.in, LBM steps, MPIoutput every `inter` steps
// and a "time=" line per output.  Extension keys in input.in (see System.hpp)
// select the lattice, profile, storage and arithmetic.
#include <chrono>
#include <cstdio>

#include "System.hpp"
#include "lbm.hpp"

int main() {
  System s1;
  if (!s1.ok) {
    std::fprintf(stderr, "%s\n", s1.error.c_str());
    return 2;
  }
  s1.Monitor();
  double tau = s1.tau, rho0 = s1.rho0, u0 = s1.u0;
  const bool d2 = s1.lattice == CFLBM_D2Q9;
  LBM *l1 = d2 ? new LBM(MPI_COMM_WORLD, s1.sx, s1.sy, tau, rho0, u0)
               : new LBM(MPI_COMM_WORLD, s1.sx, s1.sy, s1.sz, tau, rho0, u0);
  l1->config.profile = s1.profile;
  l1->config.storage = s1.storage;
  l1->config.compute = s1.compute;
  l1->config.geom = s1.geom;
  l1->config.cx = s1.cx;
  l1->config.cy = s1.cy;
  l1->config.cz = s1.cz;
  l1->config.diam = s1.diam;
  l1->config.wall_y = s1.wall_y;
  l1->config.wall_z = s1.wall_z;
  l1->config.perturb_amp = s1.perturb;
  l1->config.seed = s1.seed;
  try {
    l1->Initialize();
    l1->MPIoutput(0);
    l1->setup_subdomain();
    const auto start = std::chrono::steady_clock::now();
    for (int it = 1; it <= s1.Time; ++it) {
      l1->Collision();
      l1->pack();
      l1->exchange();
      l1->unpack();
      l1->Streaming();
      l1->Update();
      if (it % s1.inter == 0) {
        l1->MPIoutput(it / s1.inter);
        const double t =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        std::printf("time=%f\n", t);
      }
    }
  } catch (const std::exception &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    delete l1;
    return 1;
  }
  delete l1;
  return 0;
}
