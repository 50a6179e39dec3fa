// Driver for the reference's serial 2-D solver ("Kokkos/lbm.cpp", one process):
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py against oracle/shim into
// oracle/_ref/ref2ds; never linked into the product.
//
// It replaces the reference's main() ("Kokkos/main.cpp:5-40"), which fixes the
// grid at 512 x 128 and the run length through System, by one that takes the
// run from argv:
//
//   ref2ds <outdir> <sx> <sy> <tau0> <u0> <steps>
//
// and writes ran.i32, f.f64 (9*lx*ly, index (ii*lx+i)*ly+j; lx = sx + 5,
// ly = sy + 5), fpost.f64, u.f64, v.f64, p.f64 and the reference's ASCII
// Output files output0.dat (initial state) and output1.dat (after the run).
#include <sys/stat.h>
#include <unistd.h>
#include <cstdio>
#include <cstdlib>
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
    std::fprintf(stderr, "usage: %s outdir sx sy tau0 u0 steps\n", argv[0]);
    return 2;
  }
  mkdir(argv[1], 0755);
  if (chdir(argv[1]) != 0) { std::perror("chdir"); return 2; }
  int sx = std::atoi(argv[2]), sy = std::atoi(argv[3]);
  double tau = std::atof(argv[4]), u0 = std::atof(argv[5]), rho0 = 1.0;
  int steps = std::atoi(argv[6]);
  std::remove("output0.dat");
  std::remove("output1.dat");
  Kokkos::initialize(argc, argv);
  {
    LBM l1(sx, sy, tau, rho0, u0);
    l1.Initialize();
    dump("ran.i32", l1.ran);
    l1.Output(0);
    for (int it = 1; it <= steps; ++it) {
      l1.Collision();
      l1.Streaming();
      l1.Update();
    }
    l1.Output(1);
    dump("f.f64", l1.f);
    dump("u.f64", l1.ua);
    dump("v.f64", l1.va);
    dump("p.f64", l1.p);
    l1.Collision();
    dump("fpost.f64", l1.f);
    std::printf("lx=%d ly=%d\n", l1.lx, l1.ly);
  }
  Kokkos::finalize();
  return 0;
}
