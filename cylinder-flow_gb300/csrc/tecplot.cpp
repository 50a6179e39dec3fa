// Tecplot binary (#!TDV112) writer with the reference's exact byte layout.
//
// 3-D: "3D MPI+KOKKOS+MPIIO/lbm.cpp:528-726" -- a 332-byte header (variables
//      x,y,z,u,v,w,p; zone "ZONE 001"; strand -1; solution time n; ordered zone
//      I,J,K = nx,ny,nz; min/max pairs with the coordinate ranges written as the
//      constants 0..4, 0..1, 0..1) followed by 7 FP64 blocks, x fastest.
// 2-D: "MPI Kokkos/lbm.cpp:548-726" -- a 276-byte header (x,y,u,v,p; parent
//      zone -1, strand -2; K = 1) followed by 5 FP64 blocks.
// Coordinates are x = 4 i/(nx-1), y = j/(ny-1), z = k/(nz-1)
// ("3D.../lbm.cpp:455-457").  The reference's single-rank MPI-IO write is one
// sequential write of the same bytes, which is what this does.
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>
#include "handle.hpp"

namespace cflbm {

namespace {
struct Buf {
  std::vector<unsigned char> b;
  void i32(int v) { raw(&v, 4); }
  void f32(float v) { raw(&v, 4); }
  void f64(double v) { raw(&v, 8); }
  void raw(const void *p, size_t n) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    b.insert(b.end(), c, c + n);
  }
};

void minmax(const double *a, size_t n, double &mn, double &mx) {
  mx = std::numeric_limits<double>::lowest();
  mn = std::numeric_limits<double>::max();
  for (size_t k = 0; k < n; ++k) {
    if (a[k] > mx) mx = a[k];
    if (a[k] < mn) mn = a[k];
  }
}
}  // namespace

int write_tecplot(const char *path, int dim, int nx, int ny, int nz, const double *u,
                  const double *v, const double *w, const double *p, int n) {
  const size_t N = (size_t)nx * ny * (dim == 3 ? nz : 1);
  Buf h;
  h.raw("#!TDV112", 8);
  h.i32(1);
  h.i32(0);
  h.i32(0);
  const char *names3[] = {"x", "y", "z", "u", "v", "w", "p"};
  const char *names2[] = {"x", "y", "u", "v", "p"};
  const int nv = dim == 3 ? 7 : 5;
  h.i32(nv);
  for (int k = 0; k < nv; ++k) {
    h.i32((int)(unsigned char)(dim == 3 ? names3[k] : names2[k])[0]);
    h.i32(0);
  }
  h.f32(299.0f);
  const char *zone = "ZONE 001";
  for (int k = 0; k < 8; ++k) h.i32((int)(unsigned char)zone[k]);
  h.i32(0);
  if (dim == 3) {
    h.i32(-1);  // strand id
  } else {
    h.i32(-1);  // parent zone
    h.i32(-2);  // strand id
  }
  h.f64((double)n);  // solution time
  if (dim == 3) h.i32(0);
  h.i32(-1);  // zone colour
  h.i32(0);   // zone type
  h.i32(0);   // var location
  h.i32(0);   // raw local
  h.i32(0);   // miscellaneous
  h.i32(nx);
  h.i32(ny);
  h.i32(dim == 3 ? nz : 1);
  h.i32(0);        // auxiliary
  h.f32(357.0f);   // end of header
  h.f32(299.0f);   // data section
  for (int k = 0; k < nv; ++k) h.i32(2);  // FP64 variables
  h.i32(0);   // passive
  h.i32(0);   // sharing
  h.i32(-1);  // zone number
  h.f64(0.0);
  h.f64(4.0);
  h.f64(0.0);
  h.f64(1.0);
  if (dim == 3) {
    h.f64(0.0);
    h.f64(1.0);
  }
  double mn, mx;
  minmax(u, N, mn, mx);
  h.f64(mn);
  h.f64(mx);
  minmax(v, N, mn, mx);
  h.f64(mn);
  h.f64(mx);
  if (dim == 3) {
    minmax(w, N, mn, mx);
    h.f64(mn);
    h.f64(mx);
  }
  minmax(p, N, mn, mx);
  h.f64(mn);
  h.f64(mx);
  const size_t expect = dim == 3 ? 332 : 276;
  if (h.b.size() != expect) return CFLBM_E_INVALID;

  std::FILE *fp = std::fopen(path, "wb");
  if (!fp) return CFLBM_E_IO;
  bool ok = std::fwrite(h.b.data(), 1, h.b.size(), fp) == h.b.size();
  std::vector<double> c(N);
  const int zz = dim == 3 ? nz : 1;
  // Coordinates.
  for (int axis = 0; axis < (dim == 3 ? 3 : 2) && ok; ++axis) {
    size_t q = 0;
    for (int k = 0; k < zz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i, ++q)
          c[q] = axis == 0 ? (double)4.0 * i / (nx - 1)
                           : axis == 1 ? (double)j / (ny - 1) : (double)k / (nz - 1);
    ok = std::fwrite(c.data(), sizeof(double), N, fp) == N;
  }
  const double *fields3[] = {u, v, w, p};
  const double *fields2[] = {u, v, p};
  for (int k = 0; k < (dim == 3 ? 4 : 3) && ok; ++k)
    ok = std::fwrite(dim == 3 ? fields3[k] : fields2[k], sizeof(double), N, fp) == N;
  if (std::fclose(fp) != 0) ok = false;
  return ok ? CFLBM_OK : CFLBM_E_IO;
}

}  // namespace cflbm
