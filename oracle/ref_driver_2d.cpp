// Driver for the reference's 2-D solver ("MPI Kokkos/lbm.cpp", single rank):
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py against oracle/shim into
// oracle/_ref/ref2d; never linked into the product.
//
// It replaces only the reference's main() ("MPI Kokkos/main.cpp:7-44"), whose
// grid, tau and step count are hard-coded, by one that takes them from argv and
// dumps the solver state in binary so tests can compare it with the oracle
// restatement and the GPU solver:
//
//   ref2d <outdir> <nx> <ny> <tau0> <u0> <steps>
//
// Writes into <outdir>: ran.i32 (lx*ly), f.f64 (9*lx*ly, post-stream, index
// (ii*lx+i)*ly+j), fpost.f64 (same after one more Collision()), u.f64, v.f64,
// p.f64 (lx*ly), test.dat (the reference's own per-step "Cd Cl" lines),
// output0.plt / output1.plt (the reference's MPIoutput before and after the run)
// and output00.dat / output10.dat (its ASCII Output, before and after).
#include <sys/stat.h>
#include <unistd.h>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "lbm.hpp"

template <class V>
static void dump(const char *name, const V &v) {
  std::FILE *fp = std::fopen(name, "wb");
  if (!fp) { std::perror(name); std::exit(2); }
  std::fwrite(v.data(), sizeof(*v.data()), v.size(), fp);
  std::fclose(fp);
}

int main(int argc, char **argv) {
  if (argc != 7) {
    std::fprintf(stderr, "usage: %s outdir nx ny tau0 u0 steps\n", argv[0]);
    return 2;
  }
  mkdir(argv[1], 0755);
  if (chdir(argv[1]) != 0) { std::perror("chdir"); return 2; }
  int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]);
  double tau = std::atof(argv[4]), u0 = std::atof(argv[5]), rho0 = 1.0;
  int steps = std::atoi(argv[6]);
  std::remove("test.dat");
  std::remove("output0.plt");
  std::remove("output1.plt");
  std::remove("output00.dat");
  std::remove("output10.dat");

  MPI_Init(&argc, &argv);
  Kokkos::initialize(argc, argv);
  {
    LBM l1(MPI_COMM_WORLD, nx, ny, tau, rho0, u0);
    l1.Initialize();
    dump("ran.i32", l1.ran);
    l1.MPIoutput(0);
    l1.Output(0);  // output00.dat: the initial state
    l1.setup_subdomain();
    for (int it = 1; it <= steps; ++it) {
      l1.Collision();
      l1.pack();
      l1.exchange();
      l1.unpack();
      l1.Streaming();
      l1.Update();
    }
    l1.MPIoutput(1);
    l1.Output(1);  // output10.dat: after the run
    dump("f.f64", l1.f);
    dump("u.f64", l1.ua);
    dump("v.f64", l1.va);
    dump("p.f64", l1.p);
    l1.Collision();
    dump("fpost.f64", l1.f);
    std::printf("lx=%d ly=%d\n", l1.lx, l1.ly);
  }
  Kokkos::finalize();
  MPI_Finalize();
  return 0;
}
