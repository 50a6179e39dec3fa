// CPU oracle for the cylinder-flow LBM hot path: TEST INFRASTRUCTURE ONLY.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
// library (oracle/liboracle.so, via ctypes).  The GPU product never links it.
//
// It is a plain FP64 C++/OpenMP restatement of the reference solver
// (Maccchiatooo/Cylinder-flow), organised pass-for-pass like the reference so
// that (a) its numbers can be pinned bit-for-bit against the reference's own
// sources compiled in oracle/_ref/ (see oracle/build.py), and (b) its timing is
// representative of the reference's CPU implementation: passes the reference
// runs as Kokkos parallel_for run here as OpenMP loops, and passes the reference
// runs as serial host loops (Update, the 2-D force sum) run serially here too.
//
// Three entry points:
//   oracle_ref2d_run    -- "MPI Kokkos/" D2Q9 solver at one rank, incl. Cd/Cl.
//   oracle_ref3d_run    -- "3D MPI+KOKKOS+MPIIO/" D3Q27 solver at one rank.
//   oracle_channel_run  -- the benchmark channel problems (equilibrium inlet,
//                          zero-gradient outlet, free-slip / periodic / no-slip
//                          walls, halfway bounce-back, optional Brinkman
//                          porosity), same collision and macroscopic model.
//
// Array layout inside the reference-profile runs is the reference's host layout
// (Kokkos LayoutRight): f(ii,i,j[,k]) at ((ii*lx+i)*ly+j)*lz+k, ghosts included,
// and out-of-range neighbour reads alias exactly as they do in the reference.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

struct Lattice {
  int Q, D;
  int e[27][3];
  double t[27];
  int bb[27];
};

// D2Q9: weights, velocities and bounce-back pairs of "Kokkos/lbm.cpp:57-95"
// (identical in "MPI Kokkos/lbm.cpp:52-90").  Order 0,E,N,W,S,NE,NW,SW,SE.
Lattice make_d2q9() {
  Lattice L{};
  L.Q = 9;
  L.D = 2;
  const int ex[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
  const int ey[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
  const int bb[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
  for (int i = 0; i < 9; ++i) {
    L.e[i][0] = ex[i];
    L.e[i][1] = ey[i];
    L.e[i][2] = 0;
    L.bb[i] = bb[i];
  }
  L.t[0] = 4.0 / 9.0;
  for (int i = 1; i < 5; ++i) L.t[i] = 1.0 / 9.0;
  for (int i = 5; i < 9; ++i) L.t[i] = 1.0 / 36.0;
  return L;
}

// D3Q27: "3D MPI+KOKKOS+MPIIO/lbm.cpp:55-218".  Directions come in +/- pairs,
// so bb(2k-1) = 2k.
Lattice make_d3q27() {
  Lattice L{};
  L.Q = 27;
  L.D = 3;
  const int E[27][3] = {{0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0},
                        {0, 0, 1},   {0, 0, -1},  {1, 1, 0},   {-1, -1, 0}, {1, -1, 0},
                        {-1, 1, 0},  {1, 0, 1},   {-1, 0, -1}, {1, 0, -1},  {-1, 0, 1},
                        {0, 1, 1},   {0, -1, -1}, {0, 1, -1},  {0, -1, 1},  {1, 1, 1},
                        {-1, -1, -1}, {1, -1, 1},  {-1, 1, -1}, {1, 1, -1},  {-1, -1, 1},
                        {1, -1, -1}, {-1, 1, 1}};
  for (int i = 0; i < 27; ++i) {
    for (int d = 0; d < 3; ++d) L.e[i][d] = E[i][d];
    L.bb[i] = (i == 0) ? 0 : ((i % 2 == 1) ? i + 1 : i - 1);
  }
  L.t[0] = 8.0 / 27.0;
  for (int i = 1; i <= 6; ++i) L.t[i] = 2.0 / 27.0;
  for (int i = 7; i <= 18; ++i) L.t[i] = 1.0 / 54.0;
  for (int i = 19; i <= 26; ++i) L.t[i] = 1.0 / 216.0;
  return L;
}

const Lattice &lat2() {
  static const Lattice L = make_d2q9();
  return L;
}
const Lattice &lat3() {
  static const Lattice L = make_d3q27();
  return L;
}

}  // namespace

extern "C" {

// Lattice tables, for tests: e (Q*3 ints), t (Q doubles), bb (Q ints).
int oracle_lattice(int Q, int *e, double *t, int *bb) {
  const Lattice *L = (Q == 9) ? &lat2() : (Q == 27) ? &lat3() : nullptr;
  if (!L) return 1;
  for (int i = 0; i < Q; ++i) {
    for (int d = 0; d < 3; ++d) e[3 * i + d] = L->e[i][d];
    t[i] = L->t[i];
    bb[i] = L->bb[i];
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Reference profile, 2-D: "MPI Kokkos/lbm.cpp" at one rank (x_lo = y_lo = 0,
// glx = nx, gly = ny, ghost = 2, lx = nx + 4, ly = ny + 4 per lbm.hpp:77-85).
//
// ran      : lx*ly ints, the reference's per-node draw (index i*ly+j).
// f_out    : 9*lx*ly post-stream populations after `steps` steps (or null).
// fpost_out: the same after one further Collision() (or null).
// u/v/p_out: lx*ly macroscopic fields after `steps` steps (or null).
// force_out: 2*steps doubles, the reduced (sum1, sum2) of each step (or null);
//            Cd = 2*sum1/u0/u0/0.03125/(nx-1) as written to test.dat.
// ---------------------------------------------------------------------------
int oracle_ref2d_run(int nx, int ny, double tau0, double u0, const int *ran, int steps,
                     double *f_out, double *fpost_out, double *u_out, double *v_out,
                     double *p_out, double *force_out, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  const Lattice &L = lat2();
  const int Q = 9;
  const int glx = nx, gly = ny;
  const int lx = nx + 4, ly = ny + 4;
  const long N = (long)lx * ly;
  std::vector<double> f(Q * N, 0.0), ft(Q * N, 0.0), ua(N, 0.0), va(N, 0.0), p(N, 0.0),
      fdx(N, 0.0), fdy(N, 0.0);
  std::vector<int> usr(N, 0);
  // Flat indexing without bounds checks, as Kokkos Views do: neighbour reads
  // that leave [0,lx) alias into the adjacent population exactly as in the
  // reference.
  auto F = [&](int ii, int i, int j) -> double & { return f[((long)ii * lx + i) * ly + j]; };
  auto FT = [&](int ii, int i, int j) -> double & { return ft[((long)ii * lx + i) * ly + j]; };
  auto A = [&](std::vector<double> &a, int i, int j) -> double & { return a[(long)i * ly + j]; };
  auto U = [&](int i, int j) -> int & { return usr[(long)i * ly + j]; };
  const auto &e = L.e;
  const auto &t = L.t;
  const auto &bb = L.bb;

  // Initialize: "MPI Kokkos/lbm.cpp:101-124".
#pragma omp parallel for collapse(2)
  for (int i = 0; i < lx; ++i)
    for (int j = 0; j < ly; ++j) {
      int lnx = i - 2, lny = j - 2;
      A(p, i, j) = 0.0;
      U(i, j) = (std::pow((lnx - 0.5 * (glx - 1)), 2) + std::pow((lny - 0.5 * (gly - 1)), 2) <=
                 std::pow(0.03125 * (glx - 1) / 2.0, 2))
                    ? 0
                    : 1;
      A(ua, i, j) = (u0 * 4.0 * lny * (gly - 1 - lny) / std::pow((gly - 1), 2)) * U(i, j) *
                    (0.9 + ran[(long)i * ly + j] * 0.002);
      A(va, i, j) = 0.0;
    }
#pragma omp parallel for collapse(2)
  for (int ii = 0; ii < Q; ++ii)
    for (int i = 0; i < lx; ++i)
      for (int j = 0; j < ly; ++j) {
        F(ii, i, j) = t[ii] * A(p, i, j) * 3.0 +
                      t[ii] * (3.0 * (e[ii][0] * A(ua, i, j) + e[ii][1] * A(va, i, j)) +
                               4.5 * std::pow(e[ii][0] * A(ua, i, j) + e[ii][1] * A(va, i, j), 2) -
                               1.5 * (std::pow(A(ua, i, j), 2) + std::pow(A(va, i, j), 2)));
      }

  auto collision = [&]() {
    // "MPI Kokkos/lbm.cpp:127-139".
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = 2; i < lx - 2; ++i)
        for (int j = 2; j < ly - 2; ++j) {
          double feq = t[ii] * A(p, i, j) * 3.0 +
                       t[ii] * (3.0 * (e[ii][0] * A(ua, i, j) + e[ii][1] * A(va, i, j)) +
                                4.5 * std::pow(e[ii][0] * A(ua, i, j) + e[ii][1] * A(va, i, j), 2) -
                                1.5 * (std::pow(A(ua, i, j), 2) + std::pow(A(va, i, j), 2)));
          F(ii, i, j) -= (F(ii, i, j) - feq) / (tau0 + 0.5);
        }
  };

  for (int it = 1; it <= steps; ++it) {
    const double t_step = omp_get_wtime();
    collision();
    // Streaming, "MPI Kokkos/lbm.cpp:313-418".  Inlet copy (:315-321).
    for (int j = 1; j < ly - 1; ++j) {
      F(1, 1, j) = F(1, 2, j);
      F(5, 1, j) = F(5, 2, j);
      F(8, 1, j) = F(8, 2, j);
    }
    // Outlet extrapolation along the population's own direction (:323-329).
    for (int j = 1; j < ly - 1; ++j) {
      F(3, lx - 2, j) = F(3, lx - 3, j);
      F(7, lx - 2, j) = F(7, lx - 3, j - 1);
      F(6, lx - 2, j) = F(6, lx - 3, j + 1);
    }
    // Wall rows (:331-345): the ghost row takes the opposite population two
    // rows in, shifted by twice the in-plane velocity.
    for (int i = 1; i < lx - 1; ++i) {
      F(2, i, 1) = F(4, i, 3);
      F(5, i, 1) = F(7, i + 2, 3);
      F(6, i, 1) = F(8, i - 2, 3);
    }
    for (int i = 1; i < lx - 1; ++i) {
      F(4, i, ly - 2) = F(2, i, ly - 4);
      F(7, i, ly - 2) = F(5, i - 2, ly - 4);
      F(8, i, ly - 2) = F(6, i + 2, ly - 4);
    }
    // Solid nodes next to fluid (:347-353).
    for (int ii = 0; ii < Q; ++ii)
      for (int i = 2; i < lx - 2; ++i)
        for (int j = 2; j < ly - 2; ++j)
          if (U(i, j) == 0 && U(i + e[ii][0], j + e[ii][1]) == 1)
            F(ii, i, j) = F(bb[ii], i + 2 * e[ii][0], j + 2 * e[ii][1]);
    // Momentum-exchange force, serial host loop (:356-377) and the two
    // parallel_reduce sums (:380-392), in (i, j) order.
    std::fill(fdx.begin(), fdx.end(), 0.0);
    std::fill(fdy.begin(), fdy.end(), 0.0);
    for (int i = 2; i < lx - 2; ++i)
      for (int j = 2; j < ly - 2; ++j)
        for (int ii = 0; ii < Q; ++ii)
          if (U(i, j) == 1 && U(i + e[ii][0], j + e[ii][1]) == 0) {
            A(fdx, i, j) += (F(ii, i, j) + F(bb[ii], i - e[bb[ii]][0], j - e[bb[ii]][1])) * e[ii][0];
            A(fdy, i, j) += (F(ii, i, j) + F(bb[ii], i - e[bb[ii]][0], j - e[bb[ii]][1])) * e[ii][1];
          }
    double resultd = 0.0, resultl = 0.0;
    for (int i = 2; i < lx - 2; ++i)
      for (int j = 2; j < ly - 2; ++j) resultd += A(fdx, i, j);
    for (int i = 2; i < lx - 2; ++i)
      for (int j = 2; j < ly - 2; ++j) resultl += A(fdy, i, j);
    if (force_out) {
      force_out[2 * (it - 1)] = resultd;
      force_out[2 * (it - 1) + 1] = resultl;
    }
    // Pull stream into ft, then copy back (:408-416).
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = 2; i < lx - 2; ++i)
        for (int j = 2; j < ly - 2; ++j) FT(ii, i, j) = F(ii, i - e[ii][0], j - e[ii][1]);
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = 2; i < lx - 2; ++i)
        for (int j = 2; j < ly - 2; ++j) F(ii, i, j) = FT(ii, i, j);
    // Update, serial host loop ("MPI Kokkos/lbm.cpp:420-457").
    std::fill(ua.begin(), ua.end(), 0.0);
    std::fill(va.begin(), va.end(), 0.0);
    std::fill(p.begin(), p.end(), 0.0);
    for (int i = 2; i < lx - 2; ++i)
      for (int j = 2; j < ly - 2; ++j) {
        for (int ii = 0; ii < Q; ++ii) {
          A(p, i, j) = A(p, i, j) + F(ii, i, j) / 3.0;
          A(ua, i, j) = A(ua, i, j) + F(ii, i, j) * e[ii][0];
          A(va, i, j) = A(va, i, j) + F(ii, i, j) * e[ii][1];
        }
        A(p, i, j) = A(p, i, j) * U(i, j);
        A(ua, i, j) = A(ua, i, j) * U(i, j);
        A(va, i, j) = A(va, i, j) * U(i, j);
        A(ua, 2, j) = (u0 * 4.0 * (j - 2) * (gly - 1 - (j - 2)) / std::pow((gly - 1), 2));
        A(va, 2, j) = 0.0;
        A(p, lx - 3, j) = 0.0;
      }
  }
  if (f_out) std::memcpy(f_out, f.data(), sizeof(double) * Q * N);
  if (u_out) std::memcpy(u_out, ua.data(), sizeof(double) * N);
  if (v_out) std::memcpy(v_out, va.data(), sizeof(double) * N);
  if (p_out) std::memcpy(p_out, p.data(), sizeof(double) * N);
  if (fpost_out) {
    collision();
    std::memcpy(fpost_out, f.data(), sizeof(double) * Q * N);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Reference profile, 2-D serial: "Kokkos/lbm.cpp" (one process; its LBM(sx, sy)
// builds lx = sx + 5, ly = sy + 5, lbm.hpp:26, so the interior is nx = sx + 1 by
// ny = sy + 1 nodes with two ghost layers on each side, lx = nx + 4).
//
// ran      : lx*ly ints, the reference's per-node draw (index i*ly+j).
// f_out    : 9*lx*ly post-stream populations after `steps` steps (or null).
// fpost_out: the same after one further Collision() (or null).
// u/v/p_out: lx*ly macroscopic fields after `steps` steps (or null).
// The variant computes no force.
// ---------------------------------------------------------------------------
int oracle_ref2ds_run(int nx, int ny, double tau0, double u0, const int *ran, int steps,
                      double *f_out, double *fpost_out, double *u_out, double *v_out,
                      double *p_out, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  const Lattice &L = lat2();
  const int Q = 9;
  const int lx = nx + 4, ly = ny + 4;
  const long N = (long)lx * ly;
  std::vector<double> f(Q * N, 0.0), ft(Q * N, 0.0), ua(N, 0.0), va(N, 0.0), p(N, 0.0);
  std::vector<int> usr(N, 0);
  auto F = [&](int ii, int i, int j) -> double & { return f[((long)ii * lx + i) * ly + j]; };
  auto FT = [&](int ii, int i, int j) -> double & { return ft[((long)ii * lx + i) * ly + j]; };
  auto A = [&](std::vector<double> &a, int i, int j) -> double & { return a[(long)i * ly + j]; };
  auto U = [&](int i, int j) -> int & { return usr[(long)i * ly + j]; };
  const auto &e = L.e;
  const auto &t = L.t;
  const auto &bb = L.bb;

  // Initialize: "Kokkos/lbm.cpp:105-133": a disk at (0.25 (lx - 5), 0.5 (ly - 1))
  // in box coordinates with r^2 = 0.01 (ly - 5)^2, Poiseuille u times
  // (1 + 0.001 ran), f = feq.
#pragma omp parallel for collapse(2)
  for (int i = 0; i < lx; ++i)
    for (int j = 0; j < ly; ++j) {
      A(p, i, j) = 0.0;
      U(i, j) = 1;
      if (std::pow((i - 0.25 * (lx - 5)), 2) + std::pow((j - 0.5 * (ly - 1)), 2) <=
          0.01 * (ly - 5) * (ly - 5))
        U(i, j) = 0;
      A(ua, i, j) = (u0 * 4.0 * (j - 2) * (ly - 3 - j) / std::pow((ly - 5), 2)) * U(i, j) *
                    (1.0 + ran[(long)i * ly + j] * 0.001);
      A(va, i, j) = 0.0;
    }
#pragma omp parallel for collapse(2)
  for (int ii = 0; ii < Q; ++ii)
    for (int i = 0; i < lx; ++i)
      for (int j = 0; j < ly; ++j) {
        F(ii, i, j) = t[ii] * A(p, i, j) * 3.0 +
                      t[ii] * (3.0 * (e[ii][0] * A(ua, i, j) + e[ii][1] * A(va, i, j)) +
                               4.5 * std::pow(e[ii][0] * A(ua, i, j) + e[ii][1] * A(va, i, j), 2) -
                               1.5 * (std::pow(A(ua, i, j), 2) + std::pow(A(va, i, j), 2)));
      }

  auto collision = [&]() {
    // "Kokkos/lbm.cpp:134-144".
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = 2; i < lx - 2; ++i)
        for (int j = 2; j < ly - 2; ++j) {
          double feq = t[ii] * A(p, i, j) * 3.0 +
                       t[ii] * (3.0 * (e[ii][0] * A(ua, i, j) + e[ii][1] * A(va, i, j)) +
                                4.5 * std::pow(e[ii][0] * A(ua, i, j) + e[ii][1] * A(va, i, j), 2) -
                                1.5 * (std::pow(A(ua, i, j), 2) + std::pow(A(va, i, j), 2)));
          F(ii, i, j) -= (F(ii, i, j) - feq) / (tau0 + 0.5);
        }
  };

  for (int it = 1; it <= steps; ++it) {
    collision();
    // Streaming, "Kokkos/lbm.cpp:145-186".  Inlet copy and outlet extrapolation
    // over j in [1, ly - 1) (:147-156).
    for (int j = 1; j < ly - 1; ++j) {
      F(1, 1, j) = F(1, 2, j);
      F(5, 1, j) = F(5, 2, j);
      F(8, 1, j) = F(8, 2, j);
      F(3, lx - 2, j) = F(3, lx - 3, j);
      F(7, lx - 2, j) = F(7, lx - 3, j - 1);
      F(6, lx - 2, j) = F(6, lx - 3, j + 1);
    }
    // Wall rows over i in [2, lx - 2) only (:158-168): the corners i = 1 and
    // i = lx - 2 of the ghost rows keep what the inlet/outlet pass left.
    for (int i = 2; i < lx - 2; ++i) {
      F(2, i, 1) = F(4, i, 3);
      F(5, i, 1) = F(7, i + 2, 3);
      F(6, i, 1) = F(8, i - 2, 3);
      F(4, i, ly - 2) = F(2, i, ly - 4);
      F(7, i, ly - 2) = F(5, i - 2, ly - 4);
      F(8, i, ly - 2) = F(6, i + 2, ly - 4);
    }
    // Solid nodes next to fluid, over the whole box (:170-176).
    for (int ii = 0; ii < Q; ++ii)
      for (int i = 0; i < lx; ++i)
        for (int j = 0; j < ly; ++j)
          if (U(i, j) == 0 && U(i + e[ii][0], j + e[ii][1]) == 1)
            F(ii, i, j) = F(bb[ii], i + 2 * e[ii][0], j + 2 * e[ii][1]);
    // Pull stream into ft over [1, lx - 1) x [1, ly - 1), copy back over the
    // interior (:177-186).
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = 1; i < lx - 1; ++i)
        for (int j = 1; j < ly - 1; ++j) FT(ii, i, j) = F(ii, i - e[ii][0], j - e[ii][1]);
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = 2; i < lx - 2; ++i)
        for (int j = 2; j < ly - 2; ++j) F(ii, i, j) = FT(ii, i, j);
    // Update, serial host loop ("Kokkos/lbm.cpp:188-217"), j outer.
    std::fill(ua.begin(), ua.end(), 0.0);
    std::fill(va.begin(), va.end(), 0.0);
    std::fill(p.begin(), p.end(), 0.0);
    for (int j = 2; j < ly - 2; ++j)
      for (int i = 2; i < lx - 2; ++i) {
        for (int ii = 0; ii < Q; ++ii) {
          A(p, i, j) = A(p, i, j) + F(ii, i, j) / 3.0;
          A(ua, i, j) = A(ua, i, j) + F(ii, i, j) * e[ii][0];
          A(va, i, j) = A(va, i, j) + F(ii, i, j) * e[ii][1];
        }
        A(ua, i, j) = A(ua, i, j) * U(i, j);
        A(va, i, j) = A(va, i, j) * U(i, j);
        A(p, i, j) = A(p, i, j) * U(i, j);
        A(ua, 2, j) = u0 * 4.0 * (j - 2) * (ly - 3 - j) / std::pow((ly - 5), 2);
        A(va, 2, j) = 0.0;
        A(p, lx - 3, j) = 0.0;
      }
  }
  if (f_out) std::memcpy(f_out, f.data(), sizeof(double) * Q * N);
  if (u_out) std::memcpy(u_out, ua.data(), sizeof(double) * N);
  if (v_out) std::memcpy(v_out, va.data(), sizeof(double) * N);
  if (p_out) std::memcpy(p_out, p.data(), sizeof(double) * N);
  if (fpost_out) {
    collision();
    std::memcpy(fpost_out, f.data(), sizeof(double) * Q * N);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Reference profile, 3-D: "3D MPI+KOKKOS+MPIIO/lbm.cpp" at one rank
// (ghost = 3, lx = nx + 6 ..., l_s = 3, l_e = 3 + n; lbm.hpp:146-219).
// Arguments as oracle_ref2d_run, arrays over lx*ly*lz (index (i*ly+j)*lz+k).
// ---------------------------------------------------------------------------
int oracle_ref3d_run(int nx, int ny, int nz, double tau0, double u0, const int *ran,
                     int steps, double *f_out, double *fpost_out, double *u_out,
                     double *v_out, double *w_out, double *p_out, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  const Lattice &L = lat3();
  const int Q = 27, G = 3;
  const int glx = nx, gly = ny, glz = nz;
  const int lx = nx + 2 * G, ly = ny + 2 * G, lz = nz + 2 * G;
  const int ls[3] = {G, G, G};
  const int le[3] = {G + nx, G + ny, G + nz};
  const long N = (long)lx * ly * lz;
  std::vector<double> f(Q * N, 0.0), ft(Q * N, 0.0), ua(N, 0.0), va(N, 0.0), wa(N, 0.0),
      p(N, 0.0);
  std::vector<int> usr(N, 0);
  auto F = [&](int ii, int i, int j, int k) -> double & {
    return f[(((long)ii * lx + i) * ly + j) * lz + k];
  };
  auto FT = [&](int ii, int i, int j, int k) -> double & {
    return ft[(((long)ii * lx + i) * ly + j) * lz + k];
  };
  auto A = [&](std::vector<double> &a, int i, int j, int k) -> double & {
    return a[((long)i * ly + j) * lz + k];
  };
  auto U = [&](int i, int j, int k) -> int & { return usr[((long)i * ly + j) * lz + k]; };
  const auto &e = L.e;
  const auto &t = L.t;
  const auto &bb = L.bb;

  // Initialize ("3D MPI+KOKKOS+MPIIO/lbm.cpp:231-254").  The sphere centre uses
  // integer division (glx - 1) / 8 in all three coordinates.
#pragma omp parallel for collapse(2)
  for (int i = 0; i < lx; ++i)
    for (int j = 0; j < ly; ++j)
      for (int k = 0; k < lz; ++k) {
        A(p, i, j, k) = 0;
        U(i, j, k) = (std::pow((i - G - (glx - 1) / 8), 2) + std::pow((j - G - (glx - 1) / 8), 2) +
                          std::pow((k - G - (glx - 1) / 8), 2) <=
                      std::pow(((glx - 1) / 64.0), 2))
                         ? 0
                         : 1;
        A(ua, i, j, k) = (u0 * 4.0 * (k - G) * (glz - 1 - (k - G)) / std::pow((glz - 1), 2)) *
                         U(i, j, k) * (1.0 + ran[((long)i * ly + j) * lz + k] * 0.001);
        A(va, i, j, k) = 0.0;
        A(wa, i, j, k) = 0.0;
      }
  auto feq_of = [&](int ii, int i, int j, int k) {
    double edu = e[ii][0] * A(ua, i, j, k) + e[ii][1] * A(va, i, j, k) + e[ii][2] * A(wa, i, j, k);
    double udu = std::pow(A(ua, i, j, k), 2) + std::pow(A(va, i, j, k), 2) +
                 std::pow(A(wa, i, j, k), 2);
    double eu2 = std::pow((e[ii][0] * A(ua, i, j, k) + e[ii][1] * A(va, i, j, k) +
                           e[ii][2] * A(wa, i, j, k)),
                          2);
    return t[ii] * A(p, i, j, k) * 3.0 + t[ii] * (3.0 * edu + 4.5 * eu2 - 1.5 * udu);
  };
#pragma omp parallel for collapse(2)
  for (int ii = 0; ii < Q; ++ii)
    for (int i = 0; i < lx; ++i)
      for (int j = 0; j < ly; ++j)
        for (int k = 0; k < lz; ++k) F(ii, i, j, k) = feq_of(ii, i, j, k);

  auto collision = [&]() {
    // "3D MPI+KOKKOS+MPIIO/lbm.cpp:257-272".
#pragma omp parallel for collapse(3)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = ls[0]; i < le[0]; ++i)
        for (int j = ls[1]; j < le[1]; ++j)
          for (int k = ls[2]; k < le[2]; ++k) {
            double feq = feq_of(ii, i, j, k);
            F(ii, i, j, k) -= (F(ii, i, j, k) - feq) / (tau0 + 0.5);
          }
  };

  for (int it = 1; it <= steps; ++it) {
    const double t_step = omp_get_wtime();
    collision();
    // Streaming ("3D MPI+KOKKOS+MPIIO/lbm.cpp:274-371"), face passes in the
    // reference's order: front (y lo), back (y hi), bottom (z lo), top (z hi),
    // inlet (x lo), outlet (x hi).
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = G - 1; i < lx - G + 1; ++i)
        for (int k = G - 1; k < lz - G + 1; ++k)
          if (e[ii][1] > 0)
            F(ii, i, ls[1] - 1, k) = F(bb[ii], i + 2 * e[ii][0], ls[1] + 1, k + 2 * e[ii][2]);
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = G - 1; i < lx - G + 1; ++i)
        for (int k = G - 1; k < lz - G + 1; ++k)
          if (e[ii][1] < 0)
            F(ii, i, le[1], k) = F(bb[ii], i + 2 * e[ii][0], le[1] - 2, k + 2 * e[ii][2]);
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = G - 1; i < lx - G + 1; ++i)
        for (int j = G - 1; j < ly - G + 1; ++j)
          if (e[ii][2] > 0)
            F(ii, i, j, ls[2] - 1) = F(bb[ii], i + 2 * e[ii][0], j + 2 * e[ii][1], ls[2] + 1);
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = G - 1; i < lx - G + 1; ++i)
        for (int j = G - 1; j < ly - G + 1; ++j)
          if (e[ii][2] < 0)
            F(ii, i, j, le[2]) = F(bb[ii], i + 2 * e[ii][0], j + 2 * e[ii][1], le[2] - 2);
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int j = G - 1; j < ly - G + 1; ++j)
        for (int k = G - 1; k < lz - G + 1; ++k)
          if (e[ii][0] > 0) F(ii, G - 1, j, k) = F(ii, G, j, k);
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int j = G - 1; j < ly - G + 1; ++j)
        for (int k = G - 1; k < lz - G + 1; ++k)
          if (e[ii][0] < 0)
            F(ii, le[0], j, k) = F(ii, le[0] + e[ii][0], j + e[ii][1], k + e[ii][2]);
    // Solid nodes next to fluid (:350-356).
#pragma omp parallel for collapse(2)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = G; i < lx - G; ++i)
        for (int j = G; j < ly - G; ++j)
          for (int k = G; k < lz - G; ++k)
            if (U(i, j, k) == 0 && U(i + e[ii][0], j + e[ii][1], k + e[ii][2]) == 1)
              F(ii, i, j, k) = F(bb[ii], i + 2 * e[ii][0], j + 2 * e[ii][1], k + 2 * e[ii][2]);
    // Pull stream and copy back (:359-369).
#pragma omp parallel for collapse(3)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = G; i < lx - G; ++i)
        for (int j = G; j < ly - G; ++j)
          for (int k = G; k < lz - G; ++k)
            FT(ii, i, j, k) = F(ii, i - e[ii][0], j - e[ii][1], k - e[ii][2]);
#pragma omp parallel for collapse(3)
    for (int ii = 0; ii < Q; ++ii)
      for (int i = G; i < lx - G; ++i)
        for (int j = G; j < ly - G; ++j)
          for (int k = G; k < lz - G; ++k) F(ii, i, j, k) = FT(ii, i, j, k);
    // Update, serial host loop (:374-417).
    std::fill(ua.begin(), ua.end(), 0.0);
    std::fill(va.begin(), va.end(), 0.0);
    std::fill(wa.begin(), wa.end(), 0.0);
    std::fill(p.begin(), p.end(), 0.0);
    for (int k = G; k < lz - G; ++k)
      for (int j = G; j < ly - G; ++j)
        for (int i = G; i < lx - G; ++i) {
          for (int ii = 0; ii < Q; ++ii) {
            A(p, i, j, k) = A(p, i, j, k) + F(ii, i, j, k) / 3.0;
            A(ua, i, j, k) = A(ua, i, j, k) + F(ii, i, j, k) * e[ii][0];
            A(va, i, j, k) = A(va, i, j, k) + F(ii, i, j, k) * e[ii][1];
            A(wa, i, j, k) = A(wa, i, j, k) + F(ii, i, j, k) * e[ii][2];
          }
          A(ua, i, j, k) = A(ua, i, j, k) * U(i, j, k);
          A(va, i, j, k) = A(va, i, j, k) * U(i, j, k);
          A(wa, i, j, k) = A(wa, i, j, k) * U(i, j, k);
          A(p, i, j, k) = A(p, i, j, k) * U(i, j, k);
          A(ua, G, j, k) = u0 * 4.0 * (k - G) * (glz - 1 - (k - G)) / std::pow((glz - 1), 2);
          A(va, G, j, k) = 0.0;
          A(wa, G, j, k) = 0.0;
          A(p, lx - G - 1, j, k) = 0.0;
        }
  }
  if (f_out) std::memcpy(f_out, f.data(), sizeof(double) * Q * N);
  if (u_out) std::memcpy(u_out, ua.data(), sizeof(double) * N);
  if (v_out) std::memcpy(v_out, va.data(), sizeof(double) * N);
  if (w_out) std::memcpy(w_out, wa.data(), sizeof(double) * N);
  if (p_out) std::memcpy(p_out, p.data(), sizeof(double) * N);
  if (fpost_out) {
    collision();
    std::memcpy(fpost_out, f.data(), sizeof(double) * Q * N);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Channel profile (the benchmark problems).  Same incompressible LBGK model and
// deviation storage as the reference (feq of "3D.../lbm.cpp:263-267", p = sum f/3,
// u = sum f e, macros zeroed in solids), with the boundary set the benchmark
// problems name instead of the reference's hard-wired one:
//   * inlet x = -1: equilibrium at rho = 1 (p = 0) and u = (u_in, 0, 0);
//   * outlet x = nx: zero gradient (copy of column nx-1);
//   * y and z walls: free-slip (specular), no-slip (halfway bounce-back) or
//     periodic, per face pair;
//   * solid cells: halfway bounce-back, f_i(x) <- f*_{bb(i)}(x) when x - e_i is
//     solid;
//   * optional Brinkman porosity alpha in [0,1] per cell: the equilibrium uses
//     (1 - alpha) u.
// Post-stream value of direction i at interior cell X (pull), source S = X - e_i:
//   1. z outside [0,nz): periodic -> wrap; free-slip -> i := mirror_z(i) and
//      S.z := X.z; no-slip -> result f*_{bb(i0)}(X).
//   2. y outside [0,ny): the same with y.
//   3. S.x < 0 -> result feq_i(p = 0, u_in); S.x >= nx -> S.x := nx - 1.
//   4. S solid -> result f*_{bb(i0)}(X);  else result f*_i(S).
// (i0 is the direction before any mirror.)  Force per step: momentum exchange
// over fluid->solid links, F += 2 f*_i(X) e_i, from the post-collision state.
// Perturbation: u_y += amp * (2 r - 1), r = splitmix64(seed + c * golden) / 2^64
// truncated to 53 bits, c = x + nx*(y + ny*z).
// Output arrays are interior-only, x fastest: f_post[(i*nz + z)*ny + y)*nx + x].
// ---------------------------------------------------------------------------
enum { WALL_FREESLIP = 0, WALL_NOSLIP = 1, WALL_PERIODIC = 2 };
enum { GEOM_NONE = 0, GEOM_CYLINDER = 1, GEOM_SPHERE = 2 };

struct oracle_channel_cfg {
  int Q, nx, ny, nz;
  double tau0, u_in;
  int wall_y, wall_z;
  int geom;
  double cx, cy, cz, diam;
  double amp;
  uint64_t seed;
  const double *alpha;  // nx*ny*nz Brinkman porosity or null
  const uint8_t *solid;  // nx*ny*nz explicit mask (1 = solid) or null -> geom
};

static inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

double oracle_perturbation(uint64_t seed, long cell, double amp) {
  uint64_t r = splitmix64(seed + (uint64_t)cell * 0x9E3779B97F4A7C15ULL);
  double u01 = (double)(r >> 11) * (1.0 / 9007199254740992.0);
  return amp * (2.0 * u01 - 1.0);
}

int oracle_channel_mask(const oracle_channel_cfg *c, uint8_t *mask) {
  const int nz = (c->Q == 9) ? 1 : c->nz;
  const double r2 = 0.25 * c->diam * c->diam;
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < c->ny; ++y)
      for (int x = 0; x < c->nx; ++x) {
        long idx = ((long)z * c->ny + y) * c->nx + x;
        uint8_t s = 0;
        if (c->solid) {
          s = c->solid[idx] ? 1 : 0;
        } else if (c->geom == GEOM_CYLINDER) {
          double dx = x - c->cx, dy = y - c->cy;
          s = (dx * dx + dy * dy <= r2) ? 1 : 0;
        } else if (c->geom == GEOM_SPHERE) {
          double dx = x - c->cx, dy = y - c->cy, dz = z - c->cz;
          s = (dx * dx + dy * dy + dz * dz <= r2) ? 1 : 0;
        }
        mask[idx] = s;
      }
  return 0;
}

int oracle_channel_run(const oracle_channel_cfg *c, int steps, double *fpost_out,
                       double *u_out, double *v_out, double *w_out, double *p_out,
                       double *force_out, int nthreads, double *step_seconds,
                       double *fstream_out) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  if (c->Q != 9 && c->Q != 27) return 1;
  const Lattice &L = (c->Q == 9) ? lat2() : lat3();
  const int Q = L.Q;
  const int nx = c->nx, ny = c->ny, nz = (Q == 9) ? 1 : c->nz;
  const long N = (long)nx * ny * nz;
  const double om_div = c->tau0 + 0.5;
  std::vector<double> f(Q * N), ft(Q * N), ua(N), va(N), wa(N), p(N);
  std::vector<uint8_t> solid(N);
  oracle_channel_mask(c, solid.data());
  const auto &e = L.e;
  const auto &t = L.t;
  const auto &bb = L.bb;
  auto cell = [&](int x, int y, int z) -> long { return ((long)z * ny + y) * nx + x; };
  int mir[3][27];
  for (int i = 0; i < Q; ++i)
    for (int d = 0; d < 3; ++d) {
      int want[3] = {e[i][0], e[i][1], e[i][2]};
      want[d] = -want[d];
      for (int k = 0; k < Q; ++k)
        if (e[k][0] == want[0] && e[k][1] == want[1] && e[k][2] == want[2]) mir[d][i] = k;
    }
  auto feq = [&](int ii, double pp, double u, double v, double w) {
    double edu = e[ii][0] * u + e[ii][1] * v + e[ii][2] * w;
    double udu = u * u + v * v + w * w;
    return t[ii] * pp * 3.0 + t[ii] * (3.0 * edu + 4.5 * edu * edu - 1.5 * udu);
  };
  double f_in[27];
  for (int ii = 0; ii < Q; ++ii) f_in[ii] = feq(ii, 0.0, c->u_in, 0.0, 0.0);

  // Initial state: p = 0, u = (u_in, perturbation, 0) in fluid, 0 in solids;
  // f = feq.
#pragma omp parallel for
  for (long n = 0; n < N; ++n) {
    double s = solid[n] ? 0.0 : 1.0;
    p[n] = 0.0;
    ua[n] = c->u_in * s;
    va[n] = oracle_perturbation(c->seed, n, c->amp) * s;
    wa[n] = 0.0;
    for (int ii = 0; ii < Q; ++ii) f[ii * N + n] = feq(ii, p[n], ua[n], va[n], wa[n]);
  }

  auto collision = [&]() {
#pragma omp parallel for
    for (long n = 0; n < N; ++n) {
      double a = c->alpha ? c->alpha[n] : 0.0;
      double u = (1.0 - a) * ua[n], v = (1.0 - a) * va[n], w = (1.0 - a) * wa[n];
      for (int ii = 0; ii < Q; ++ii) {
        double fe = feq(ii, p[n], u, v, w);
        f[ii * N + n] -= (f[ii * N + n] - fe) / om_div;
      }
    }
  };
  auto resolve = [&](int i0, int x, int y, int z, bool *hit) -> double {
    int i = i0;
    int sx = x - e[i][0], sy = y - e[i][1], sz = z - e[i][2];
    if (Q == 27 && (sz < 0 || sz >= nz)) {
      if (c->wall_z == WALL_PERIODIC) sz = (sz + nz) % nz;
      else if (c->wall_z == WALL_FREESLIP) { i = mir[2][i]; sz = z; }
      else return f[bb[i0] * N + cell(x, y, z)];
    }
    if (sy < 0 || sy >= ny) {
      if (c->wall_y == WALL_PERIODIC) sy = (sy + ny) % ny;
      else if (c->wall_y == WALL_FREESLIP) { i = mir[1][i]; sy = y; }
      else return f[bb[i0] * N + cell(x, y, z)];
    }
    if (sx < 0) return f_in[i];
    if (sx >= nx) sx = nx - 1;
    if (solid[cell(sx, sy, sz)]) {
      if (hit) *hit = true;
      return f[bb[i0] * N + cell(x, y, z)];
    }
    return f[i * N + cell(sx, sy, sz)];
  };

  for (int it = 1; it <= steps; ++it) {
    const double t_step = omp_get_wtime();
    collision();
    // Momentum exchange on fluid->solid links (post-collision state): every
    // pull of a fluid cell that bounces back off a solid source (after the
    // periodic/mirror mapping) carries 2 f*_{bb(i)}(X) e_{bb(i)} into the body.
    double Fx = 0.0, Fy = 0.0, Fz = 0.0;
    for (int z = 0; z < nz; ++z)
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
          long n = cell(x, y, z);
          if (solid[n]) continue;
          for (int ii = 1; ii < Q; ++ii) {
            bool hit = false;
            double v = resolve(ii, x, y, z, &hit);
            if (!hit) continue;
            double mom = 2.0 * v;
            Fx -= mom * e[ii][0];
            Fy -= mom * e[ii][1];
            Fz -= mom * e[ii][2];
          }
        }
    if (force_out) {
      force_out[3 * (it - 1)] = Fx;
      force_out[3 * (it - 1) + 1] = Fy;
      force_out[3 * (it - 1) + 2] = Fz;
    }
#pragma omp parallel for collapse(2)
    for (int z = 0; z < nz; ++z)
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
          long n = cell(x, y, z);
          for (int ii = 0; ii < Q; ++ii)
            ft[ii * N + n] = (ii == 0) ? f[n] : resolve(ii, x, y, z, nullptr);
        }
    std::swap(f, ft);
    // Update (reference form: p = sum f / 3, u = sum f e, zero in solids).
#pragma omp parallel for
    for (long n = 0; n < N; ++n) {
      double pp = 0.0, u = 0.0, v = 0.0, w = 0.0;
      for (int ii = 0; ii < Q; ++ii) {
        double fi = f[ii * N + n];
        pp = pp + fi / 3.0;
        u = u + fi * e[ii][0];
        v = v + fi * e[ii][1];
        w = w + fi * e[ii][2];
      }
      double s = solid[n] ? 0.0 : 1.0;
      p[n] = pp * s;
      ua[n] = u * s;
      va[n] = v * s;
      wa[n] = w * s;
    }
    if (step_seconds) step_seconds[it - 1] = omp_get_wtime() - t_step;
  }
  if (u_out) std::memcpy(u_out, ua.data(), sizeof(double) * N);
  if (v_out) std::memcpy(v_out, va.data(), sizeof(double) * N);
  if (w_out) std::memcpy(w_out, wa.data(), sizeof(double) * N);
  if (p_out) std::memcpy(p_out, p.data(), sizeof(double) * N);
  if (fstream_out) std::memcpy(fstream_out, f.data(), sizeof(double) * Q * N);
  if (fpost_out) {
    collision();
    std::memcpy(fpost_out, f.data(), sizeof(double) * Q * N);
  }
  return 0;
}

}  // extern "C"
