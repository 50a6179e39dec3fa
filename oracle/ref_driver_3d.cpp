// Driver for the reference's 3-D solver ("3D MPI+KOKKOS+MPIIO/lbm.cpp" and
// System.cpp, single rank): TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py
// against oracle/shim into oracle/_ref/ref3d; never linked into the product.
//
// It replaces the reference's main() ("3D MPI+KOKKOS+MPIIO/main.cpp:6-51"),
// whose step count comes from System's derived Time, by one that takes the run
// from argv.  pack()/exchange()/unpack() are not called: at one rank they only
// copy faces of f into host send buffers and never write f.
//
//   ref3d run    <outdir> <nx> <ny> <nz> <tau0> <u0> <steps>
//   ref3d system <dir>        (constructs System from <dir>/input.in, prints it)
//
// "run" writes ran.i32, f.f64 (27*lx*ly*lz, index ((ii*lx+i)*ly+j)*lz+k),
// fpost.f64, u.f64, v.f64, w.f64, p.f64, output0.plt and output1.plt (MPIoutput)
// and output00.dat and output10.dat (the ASCII Output) before and after the run.
#include <sys/stat.h>
#include <unistd.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "lbm.hpp"
#include "System.hpp"

template <class V>
static void dump(const char *name, const V &v) {
  std::FILE *fp = std::fopen(name, "wb");
  if (!fp) { std::perror(name); std::exit(2); }
  std::fwrite(v.data(), sizeof(*v.data()), v.size(), fp);
  std::fclose(fp);
}

int main(int argc, char **argv) {
  if (argc == 3 && std::strcmp(argv[1], "system") == 0) {
    if (chdir(argv[2]) != 0) { std::perror("chdir"); return 2; }
    System s1;
    std::printf("{\"sx\": %d, \"sy\": %d, \"sz\": %d, \"Time\": %d, \"inter\": %d, "
                "\"miu\": %.17g, \"u0\": %.17g, \"R\": %.17g, \"rho0\": %.17g, "
                "\"Ma\": %.17g, \"tau\": %.17g, \"Re\": %d}\n",
                s1.sx, s1.sy, s1.sz, s1.Time, s1.inter, s1.miu, s1.u0, s1.R, s1.rho0,
                s1.Ma, s1.tau, s1.Re);
    return 0;
  }
  if (argc != 9 || std::strcmp(argv[1], "run") != 0) {
    std::fprintf(stderr, "usage: %s run outdir nx ny nz tau0 u0 steps | system dir\n",
                 argv[0]);
    return 2;
  }
  mkdir(argv[2], 0755);
  if (chdir(argv[2]) != 0) { std::perror("chdir"); return 2; }
  int nx = std::atoi(argv[3]), ny = std::atoi(argv[4]), nz = std::atoi(argv[5]);
  double tau = std::atof(argv[6]), u0 = std::atof(argv[7]), rho0 = 1.0;
  int steps = std::atoi(argv[8]);
  std::remove("output0.plt");
  std::remove("output1.plt");
  std::remove("output00.dat");
  std::remove("output10.dat");

  MPI_Init(&argc, &argv);
  Kokkos::initialize(argc, argv);
  {
    LBM l1(MPI_COMM_WORLD, nx, ny, nz, tau, rho0, u0);
    l1.Initialize();
    dump("ran.i32", l1.ran);
    l1.MPIoutput(0);
    l1.Output(0);  // output00.dat: the initial state
    for (int it = 1; it <= steps; ++it) {
      l1.Collision();
      l1.Streaming();
      l1.Update();
    }
    l1.MPIoutput(1);
    l1.Output(1);  // output10.dat: after the run
    dump("f.f64", l1.f);
    dump("u.f64", l1.ua);
    dump("v.f64", l1.va);
    dump("w.f64", l1.wa);
    dump("p.f64", l1.p);
    l1.Collision();
    dump("fpost.f64", l1.f);
    std::printf("lx=%d ly=%d lz=%d\n", l1.lx, l1.ly, l1.lz);
  }
  Kokkos::finalize();
  MPI_Finalize();
  return 0;
}
