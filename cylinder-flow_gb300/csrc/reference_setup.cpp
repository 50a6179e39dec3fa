// Host-side geometry and initial fields of the solver profiles.
//
// The reference profiles reproduce the reference's initialisation formulas
// expression for expression (std::pow included), so the GPU starts from the
// same bits as the reference:
//   REF2D: "MPI Kokkos/lbm.cpp:101-113" at one rank (x_lo = y_lo = 0, ghost 2);
//   REF3D: "3D MPI+KOKKOS+MPIIO/lbm.cpp:231-242" at one rank (ghost 3);
//   REF2DS: "Kokkos/lbm.cpp:105-121", the serial variant (ghost 2).
// The per-node draw `ran` is the reference's Random_XorShift64_Pool field; when
// the caller does not pass one, a seeded stand-in in [0,100) is used.
#include <cmath>
#include <cstdint>
#include <vector>
#include "handle.hpp"

namespace cflbm {

static int32_t standin_ran(long long n) {
  return (int32_t)(splitmix64(5374857ULL + (unsigned long long)n * 0x9E3779B97F4A7C15ULL) % 100ULL);
}

int ref2d_setup(int nx, int ny, double u0, const int32_t *ran, RefSetup &o) {
  const int G = 2;
  const int glx = nx, gly = ny, lx = nx + 2 * G, ly = ny + 2 * G;
  const long long P = (long long)lx * ly;
  o.u.assign(P, 0.0);
  o.v.assign(P, 0.0);
  o.w.assign(P, 0.0);
  o.p.assign(P, 0.0);
  o.solid.assign((size_t)nx * ny, 0);
  o.inlet.assign(ny, 0.0);
  for (int i = 0; i < lx; ++i)
    for (int j = 0; j < ly; ++j) {
      const int lnx = i - 2, lny = j - 2;
      const int usr = (std::pow((lnx - 0.5 * (glx - 1)), 2) + std::pow((lny - 0.5 * (gly - 1)), 2) <=
                       std::pow(0.03125 * (glx - 1) / 2.0, 2))
                          ? 0
                          : 1;
      const long long rn = (long long)i * ly + j;  // the reference's layout
      const int r = ran ? ran[rn] : standin_ran(rn);
      const long long d = (long long)j * lx + i;    // ghosted box, x fastest
      o.u[d] = (u0 * 4.0 * lny * (gly - 1 - lny) / std::pow((gly - 1), 2)) * usr * (0.9 + r * 0.002);
      if (lnx >= 0 && lnx < nx && lny >= 0 && lny < ny)
        o.solid[(size_t)lny * nx + lnx] = usr ? 0 : 1;
    }
  // LBM::Update's inlet override ("MPI Kokkos/lbm.cpp:444-448").
  for (int y = 0; y < ny; ++y)
    o.inlet[y] = (u0 * 4.0 * y * (gly - 1 - y) / std::pow((gly - 1), 2));
  o.area = 0.03125 * (glx - 1);
  return 0;
}

int ref2ds_setup(int nx, int ny, double u0, const int32_t *ran, RefSetup &o) {
  // "Kokkos/lbm.cpp:105-121": the box of LBM(sx, sy) is lx = sx + 5 = nx + 4
  // (nx = sx + 1 interior nodes, ghost 2); a disk at (0.25 (lx - 5),
  // 0.5 (ly - 1)) in box coordinates with r^2 = 0.01 (ly - 5)^2; Poiseuille u
  // times (1 + 0.001 ran).
  const int G = 2;
  const int lx = nx + 2 * G, ly = ny + 2 * G;
  const long long P = (long long)lx * ly;
  o.u.assign(P, 0.0);
  o.v.assign(P, 0.0);
  o.w.assign(P, 0.0);
  o.p.assign(P, 0.0);
  o.solid.assign((size_t)nx * ny, 0);
  o.inlet.assign(ny, 0.0);
  for (int i = 0; i < lx; ++i)
    for (int j = 0; j < ly; ++j) {
      int usr = 1;
      if (std::pow((i - 0.25 * (lx - 5)), 2) + std::pow((j - 0.5 * (ly - 1)), 2) <=
          0.01 * (ly - 5) * (ly - 5))
        usr = 0;
      const long long rn = (long long)i * ly + j;  // the reference's layout
      const int r = ran ? ran[rn] : standin_ran(rn);
      const long long d = (long long)j * lx + i;    // ghosted box, x fastest
      o.u[d] = (u0 * 4.0 * (j - 2) * (ly - 3 - j) / std::pow((ly - 5), 2)) * usr * (1.0 + r * 0.001);
      const int lnx = i - G, lny = j - G;
      if (lnx >= 0 && lnx < nx && lny >= 0 && lny < ny)
        o.solid[(size_t)lny * nx + lnx] = usr ? 0 : 1;
    }
  // LBM::Update's inlet override ("Kokkos/lbm.cpp:213"), the same values as the
  // MPI variant's with ly - 5 = ny - 1.
  for (int y = 0; y < ny; ++y)
    o.inlet[y] = (u0 * 4.0 * y * (ny - 1 - y) / std::pow((ny - 1), 2));
  o.area = 0.2 * (ny - 1);  // the disk's diameter (the variant computes no force)
  return 0;
}

int ref3d_setup(int nx, int ny, int nz, double u0, const int32_t *ran, RefSetup &o) {
  const int G = 3;
  const int glx = nx, glz = nz;
  const int lx = nx + 2 * G, ly = ny + 2 * G, lz = nz + 2 * G;
  const long long P = (long long)lx * ly * lz;
  o.u.assign(P, 0.0);
  o.v.assign(P, 0.0);
  o.w.assign(P, 0.0);
  o.p.assign(P, 0.0);
  o.solid.assign((size_t)nx * ny * nz, 0);
  o.inlet.assign((size_t)ny * nz, 0.0);
  const int c = (glx - 1) / 8;
  for (int i = 0; i < lx; ++i)
    for (int j = 0; j < ly; ++j)
      for (int k = 0; k < lz; ++k) {
        const int usr = (std::pow((i - G - c), 2) + std::pow((j - G - c), 2) +
                             std::pow((k - G - c), 2) <=
                         std::pow(((glx - 1) / 64.0), 2))
                            ? 0
                            : 1;
        const long long rn = ((long long)i * ly + j) * lz + k;
        const int r = ran ? ran[rn] : standin_ran(rn);
        const long long d = ((long long)k * ly + j) * lx + i;
        o.u[d] = (u0 * 4.0 * (k - G) * (glz - 1 - (k - G)) / std::pow((glz - 1), 2)) * usr *
                 (1.0 + r * 0.001);
        const int x = i - G, y = j - G, z = k - G;
        if (x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz)
          o.solid[((size_t)z * ny + y) * nx + x] = usr ? 0 : 1;
      }
  // LBM::Update's inlet override ("3D MPI+KOKKOS+MPIIO/lbm.cpp:403-408").
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      o.inlet[(size_t)z * ny + y] = u0 * 4.0 * z * (glz - 1 - z) / std::pow((glz - 1), 2);
  const double D = 2.0 * ((glx - 1) / 64.0);
  o.area = M_PI * D * D / 4.0;
  return 0;
}

double channel_area(const cflbm_config &c) {
  const double D = c.diam > 0 ? c.diam : 1.0;
  if (c.geom == CFLBM_GEOM_SPHERE) return M_PI * D * D / 4.0;
  if (c.lattice == CFLBM_D3Q27) return D * c.nz;
  return D;
}

}  // namespace cflbm
