// Boundary, bounce-back/force, initialisation and reduction kernels.
//
// These run on O(surface) work (ghost layers, fluid->solid links) except the
// initialisation, reduction and dump/restore kernels, which run once or on
// demand.  The hot per-step sweep is in sweep.cuh.
#include <cstdio>
#include "solver.cuh"

namespace cflbm {

namespace {

long long g_launches = 0;

// Runtime direction tables (boundary kernels index directions dynamically).
template <int Q> struct DT;
__constant__ signed char c_e9[9][2] = {{0, 0}, {1, 0},  {0, 1},   {-1, 0}, {0, -1},
                                        {1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
template <> struct DT<9> {
  __device__ static int ex(int i) { return c_e9[i][0]; }
  __device__ static int ey(int i) { return c_e9[i][1]; }
  __device__ static int ez(int) { return 0; }
};
__constant__ signed char c_e27[27][3] = {
    {0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},  {0, 0, 1},   {0, 0, -1},
    {1, 1, 0},  {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0},  {1, 0, 1},   {-1, 0, -1}, {1, 0, -1},
    {-1, 0, 1}, {0, 1, 1},   {0, -1, -1}, {0, 1, -1}, {0, -1, 1},  {1, 1, 1},   {-1, -1, -1},
    {1, -1, 1}, {-1, 1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, -1}, {-1, 1, 1}};
template <> struct DT<27> {
  __device__ static int ex(int i) { return c_e27[i][0]; }
  __device__ static int ey(int i) { return c_e27[i][1]; }
  __device__ static int ez(int i) { return c_e27[i][2]; }
};
template <int Q> __device__ int dopp(int i) { return Lat<Q>::opp(i); }
// D2Q9 opposite for a run-time index, without a table in local memory:
// 1<->3, 2<->4 (axes), 5<->7, 6<->8 (diagonals).
template <> __device__ int dopp<9>(int i) {
  return i == 0 ? 0 : (i <= 4 ? (i + 1) % 4 + 1 : (i - 3) % 4 + 5);
}
template <int Q> __device__ int dmirror(int i, int d) {
  int w0 = DT<Q>::ex(i), w1 = DT<Q>::ey(i), w2 = DT<Q>::ez(i);
  if (d == 1) w1 = -w1;
  if (d == 2) w2 = -w2;
  if (d == 0) w0 = -w0;
  for (int k = 0; k < Q; ++k)
    if (DT<Q>::ex(k) == w0 && DT<Q>::ey(k) == w1 && DT<Q>::ez(k) == w2) return k;
  return i;
}

// FP64 values of stored elements and back (Store<> codecs; L.fbase is the
// FP16 format's storage offset per population).
template <class ST> struct Dec;
template <> struct Dec<double> {
  template <int Q> __device__ static double get(double v, int, const Layout &) { return v; }
  template <int Q> __device__ static double put(double v, int, const Layout &) { return v; }
};
template <> struct Dec<float> {
  template <int Q> __device__ static double get(float v, int, const Layout &) {
    return (double)v;
  }
  template <int Q> __device__ static float put(double v, int, const Layout &) {
    return (float)v;
  }
};
template <> struct Dec<F16Dev> {
  template <int Q> __device__ static double get(__half v, int i, const Layout &L) {
    return __fma_rn((double)__half2float(v), 1.0 / F16_SCALE, (double)L.fbase[i]);
  }
  template <int Q> __device__ static __half put(double v, int i, const Layout &L) {
    return __double2half(__dmul_rn(__dsub_rn(v, (double)L.fbase[i]), (double)F16_SCALE));
  }
};

inline int blocks_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 65535LL * 8) b = 65535LL * 8;
  return (int)b;
}

// ---- channel-profile ghost fill ------------------------------------------------
// Post-stream value of direction i0 at interior cell X (pull from S = X - e_i0):
//   z out of range: periodic wrap, or free-slip mirror (i := mirror_z(i),
//   S.z := X.z), or no-slip (halfway bounce-back: f*_{opp(i0)}(X));
//   then the same for y; then S.x < 0 -> inlet equilibrium, S.x >= nx -> x := nx-1
//   (zero gradient); a solid source -> f*_{opp(i0)}(X).
template <int Q, class E>
__device__ E resolve_channel(const E *f, const FillArgs &a, int i0, int x, int y, int z) {
  const Layout &L = a.L;
  int i = i0;
  int sx = x - DT<Q>::ex(i0), sy = y - DT<Q>::ey(i0), sz = z - DT<Q>::ez(i0);
  if (Q == 27 && (sz < 0 || sz >= L.nz)) {
    if (a.wall_z == WALL_PERIODIC) sz = (sz + L.nz) % L.nz;
    else if (a.wall_z == WALL_FREESLIP) { i = dmirror<Q>(i, 2); sz = z; }
    else return f[dopp<Q>(i0) * L.S + L.idx(x, y, z)];
  }
  if (sy < 0 || sy >= L.ny) {
    if (a.wall_y == WALL_PERIODIC) sy = (sy + L.ny) % L.ny;
    else if (a.wall_y == WALL_FREESLIP) { i = dmirror<Q>(i, 1); sy = y; }
    else return f[dopp<Q>(i0) * L.S + L.idx(x, y, z)];
  }
  if (sx < 0) return static_cast<const E *>(a.f_in)[i];
  if (sx >= L.nx) sx = L.nx - 1;
  if (mask_solid(a.mask, a.nxw, L.ny, sx, sy, sz)) return f[dopp<Q>(i0) * L.S + L.idx(x, y, z)];
  return f[i * L.S + L.idx(sx, sy, sz)];
}

template <int Q, class ST>
__global__ void fill_channel_kernel(const FillArgs a) {
  using E = typename Store<ST>::elem;
  E *f = static_cast<E *>(a.f);
  const Layout &L = a.L;
  const bool d3 = (Q == 27);
  const long long zr = d3 ? (L.nz + 2) : 1;
  const long long nfx = (long long)(L.ny + 2) * zr;
  const long long nfy = (long long)L.nx * zr;
  const long long nfz = d3 ? (long long)L.nx * L.ny : 0;
  const long long total = 2 * (nfx + nfy + nfz);
  const int z0 = d3 ? -1 : 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    long long r = t;
    int sx, sy, sz;
    if (r < 2 * nfx) {
      const int side = (int)(r / nfx);
      r %= nfx;
      sx = side ? L.nx : -1;
      sy = (int)(r % (L.ny + 2)) - 1;
      sz = (int)(r / (L.ny + 2)) + z0;
    } else if ((r -= 2 * nfx) < 2 * nfy) {
      const int side = (int)(r / nfy);
      r %= nfy;
      sy = side ? L.ny : -1;
      sx = (int)(r % L.nx);
      sz = (int)(r / L.nx) + z0;
    } else {
      r -= 2 * nfy;
      const long long nfzd = nfz > 0 ? nfz : 1;
      const int side = (int)(r / nfzd);
      r %= nfzd;
      sz = side ? L.nz : -1;
      sx = (int)(r % L.nx);
      sy = (int)(r / L.nx);
    }
    const long long sidx = L.idx(sx, sy, sz);
    for (int i = 1; i < Q; ++i) {
      const int X = sx + DT<Q>::ex(i), Y = sy + DT<Q>::ey(i), Z = sz + DT<Q>::ez(i);
      if (!L.interior(X, Y, Z)) continue;
      f[i * L.S + sidx] = resolve_channel<Q, E>(f, a, i, X, Y, Z);
    }
  }
}

// ---- reference-profile face passes -------------------------------------------
// One pass of the reference's Streaming() boundary sequence over a face:
//   copy   (x low,  e_x > 0): f_i(-1, j, k)  = f_i(0, j, k)
//          ("3D MPI+KOKKOS+MPIIO/lbm.cpp:326-335", "MPI Kokkos/lbm.cpp:315-321")
//   extrap (x high, e_x < 0): f_i(nx, j, k) = f_i(nx-1, j+e_y, k+e_z)    (:338-347, :323-329)
//   bounce (wall, e_a pointing inward): the ghost layer takes the opposite
//          population two layers in, shifted by twice the in-plane velocity
//          (:278-324, :331-345).
// Tangential ranges cover the interior plus one ring, [-1, n+1), as the
// reference's [ghost-1, l-ghost+1).
// No cell a pass writes is read by the same pass (it writes layer -1 or n of its
// axis and reads layer 0, nx-1 or two layers in), so every (population, face
// cell) is an independent thread.  The values also go to the other buffer
// (a.f2): the ghost layers then carry the same values in both buffers, as in the
// reference's single array, and the sweep, which writes only the interior, needs
// no ghost copy.
template <int Q, class ST>
__global__ void face_op_kernel(const FillArgs a, const FaceOp op0, const FaceOp op1) {
  // Two passes of one axis in one launch (grid z: population of op0, then of
  // op1): the two faces of an axis write different layers and read neither's.
  const bool second = (int)blockIdx.z >= op0.ndir;
  const int kdir = (int)blockIdx.z - (second ? op0.ndir : 0);
  const int kind = second ? op1.kind : op0.kind, side = second ? op1.side : op0.side;
  using E = typename Store<ST>::elem;
  E *f = static_cast<E *>(a.f);
  E *f2 = static_cast<E *>(a.f2);
  const Layout &L = a.L;
  const bool d3 = (Q == 27);
  const int ax = op0.axis;
  const int nax = ax == 0 ? L.nx : (ax == 1 ? L.ny : L.nz);
  const int na = (ax == 0 ? L.ny : L.nx) + 2;               // first tangential axis
  const int nb = d3 ? (ax == 2 ? L.ny : L.nz) + 2 : 1;      // second tangential axis
  const int b0 = d3 ? -1 : 0;
  (void)nb;
  // (axis value, tangential a, tangential b) -> (x, y, z)
  auto cell = [&](int v, int ta, int tb) -> long long {
    const int x = ax == 0 ? v : ta;
    const int y = ax == 1 ? v : (ax == 0 ? ta : tb);
    const int z = d3 ? (ax == 2 ? v : tb) : 0;
    return L.idx(x, y, z);
  };
  // One thread per (population, face cell): grid x along the first tangential
  // axis, y the second, z the populations the pass writes (no index division).
  const int i = (int)(((second ? op1.dirs : op0.dirs) >> (5 * kdir)) & 31u);
  const int pa = blockIdx.x * blockDim.x + threadIdx.x - 1;
  const int pb = blockIdx.y + b0;
  if (pa >= na - 1) return;
  const int trim = second ? op1.trim : op0.trim;
  if (trim && (pa < 0 || pa >= na - 2)) return;  // the ghost ends of the range
  const int ex = DT<Q>::ex(i), ey = DT<Q>::ey(i), ez = DT<Q>::ez(i);
  const int ea = ax == 0 ? ex : (ax == 1 ? ey : ez);
  const int eta = ax == 0 ? ey : ex;                        // e along tangential a
  const int etb = ax == 2 ? ey : ez;                        // e along tangential b
  long long dst, src;
  int srcpop = i;
  if (kind == 0) {             // inlet copy (x axis)
    if (ea <= 0) return;
    dst = cell(-1, pa, pb);
    src = cell(0, pa, pb);
  } else if (kind == 1) {      // outlet extrapolation (x axis)
    if (ea >= 0) return;
    dst = cell(nax, pa, pb);
    src = cell(L.nx - 1, pa + eta, pb + etb);
  } else {                     // wall bounce
    if (side == 0 ? (ea <= 0) : (ea >= 0)) return;
    dst = cell(side == 0 ? -1 : nax, pa, pb);
    src = cell(side == 0 ? 1 : nax - 2, pa + 2 * eta, pb + 2 * etb);
    srcpop = dopp<Q>(i);
  }
  const E v = f[srcpop * L.S + src];
  f[i * L.S + dst] = v;
  if (f2) f2[i * L.S + dst] = v;
}

// Ghost layers of A copied into B: once, after the initial fields are written,
// so that both buffers start with the reference's initial ghost values.
template <int Q, class ST>
__global__ void ghost_copy_kernel(const Layout L, const void *src_, void *dst_) {
  using E = typename Store<ST>::elem;
  const E *src = static_cast<const E *>(src_);
  E *dst = static_cast<E *>(dst_);
  const long long cells = (long long)L.px * L.nyp * L.nzp;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < cells;
       t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % L.px) - L.xoff;
    const long long r = t / L.px;
    const int y = (int)(r % L.nyp) - L.G;
    const int z = (int)(r / L.nyp) - L.Gz;
    if (L.interior(x, y, z)) continue;
    const long long e = L.idx(x, y, z);
#pragma unroll 9
    for (int i = 0; i < Q; ++i) dst[i * L.S + e] = src[i * L.S + e];
  }
}

// ---- solid links: bounce-back fill + momentum-exchange force ----------------
// For link (s, k): s solid, X = s + e_k fluid.  Fill f_k(s) = f*_{opp(k)}(s +
// reach*e_k) (reach 1: halfway bounce-back; reach 2: the reference's usrbc,
// "3D.../lbm.cpp:350-356", "MPI Kokkos/lbm.cpp:347-353").  Force: the reference's
// momentum exchange ("MPI Kokkos/lbm.cpp:364-377") sums, over fluid X and
// direction ii = opp(k) pointing into the solid, (f_ii(X) + f_opp(ii)(X + e_ii))
// e_ii after the fill.  Reduced per block in FP64, then by the last block in
// block order (deterministic), into the force history slot of this step.
template <int Q, class ST>
__global__ void links_kernel(const LinkArgs a) {
  using E = typename Store<ST>::elem;
  E *f = static_cast<E *>(a.f);
  const Layout &L = a.L;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < a.n;
       t += (long long)gridDim.x * blockDim.x) {
    const int4 l = a.links[t];
    const int k = l.w, kb = dopp<Q>(k);
    const long long ok = L.off(DT<Q>::ex(k), DT<Q>::ey(k), DT<Q>::ez(k));
    const long long s = L.idx(l.x, l.y, l.z);
    const E v = f[kb * L.S + s + a.reach * ok];
    f[k * L.S + s] = v;
    const double m = Dec<ST>::template get<Q>(f[kb * L.S + s + ok], kb, L) +
                     Dec<ST>::template get<Q>(v, kb, L);
    fx += m * DT<Q>::ex(kb);
    fy += m * DT<Q>::ey(kb);
    fz += m * DT<Q>::ez(kb);
  }
  __shared__ double sh[3][32];
  for (int o = 16; o > 0; o >>= 1) {
    fx += __shfl_down_sync(0xffffffffu, fx, o);
    fy += __shfl_down_sync(0xffffffffu, fy, o);
    fz += __shfl_down_sync(0xffffffffu, fz, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sh[0][wid] = fx; sh[1][wid] = fy; sh[2][wid] = fz; }
  __syncthreads();
  __shared__ bool last;
  if (threadIdx.x == 0) {
    double bx = 0, by = 0, bz = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { bx += sh[0][w]; by += sh[1][w]; bz += sh[2][w]; }
    a.partials[3 * blockIdx.x] = bx;
    a.partials[3 * blockIdx.x + 1] = by;
    a.partials[3 * blockIdx.x + 2] = bz;
    __threadfence();
    last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double bx = 0, by = 0, bz = 0;
    const volatile double *p = a.partials;
    for (unsigned b = 0; b < gridDim.x; ++b) { bx += p[3 * b]; by += p[3 * b + 1]; bz += p[3 * b + 2]; }
    const long long st = *a.step;
    double *h = a.hist + 3 * (st % a.cap);
    h[0] = bx;
    h[1] = by;
    h[2] = bz;
    *a.step = st + 1;
    *a.counter = 0u;
  }
}

// ---- initialisation ---------------------------------------------------------------
// f = feq(p, u) over the whole ghosted box from host-computed macroscopic fields
// (reference profiles: "3D.../lbm.cpp:245-254", "MPI Kokkos/lbm.cpp:116-124").
template <int Q, class ST>
__global__ void init_macros_kernel(const Layout L, void *f_, const double *u, const double *v,
                                   const double *w, const double *p) {
  using E = typename Store<ST>::elem;
  E *f = static_cast<E *>(f_);
  const int lxp = L.nx + 2 * L.G, lyp = L.ny + 2 * L.G, lzp = L.nz + 2 * L.Gz;
  const long long total = (long long)lxp * lyp * lzp;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % lxp) - L.G;
    const int y = (int)((t / lxp) % lyp) - L.G;
    const int z = (int)(t / ((long long)lxp * lyp)) - L.Gz;
    const double uu = u[t], vv = v[t], ww = w[t], pp = p[t];
    const long long c = L.idx(x, y, z);
    for (int i = 0; i < Q; ++i) {
      const double edu = DT<Q>::ex(i) * uu + DT<Q>::ey(i) * vv + DT<Q>::ez(i) * ww;
      const double udu = uu * uu + vv * vv + ww * ww;
      const double feq =
          Lat<Q>::w(i) * pp * 3.0 + Lat<Q>::w(i) * (3.0 * edu + 4.5 * edu * edu - 1.5 * udu);
      f[i * L.S + c] = Dec<ST>::template put<Q>(feq, i, L);
    }
  }
}

// Channel profile: p = 0, u = (u_in, seeded perturbation, 0) in fluid, 0 in
// solids; f = feq.  Also records these as the step-0 macroscopic fields.
template <int Q, class ST>
__global__ void init_channel_kernel(const Layout L, void *f_, const uint32_t *mask, int nxw,
                                    double u_in, double amp, unsigned long long seed,
                                    const float *alpha, double omega,
                                    double *mu, double *mv, double *mw, double *mp) {
  using E = typename Store<ST>::elem;
  E *f = static_cast<E *>(f_);
  const long long total = (long long)L.nx * L.ny * L.nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % L.nx);
    const int y = (int)((t / L.nx) % L.ny);
    const int z = (int)(t / ((long long)L.nx * L.ny));
    const bool solid = mask_solid(mask, nxw, L.ny, x, y, z);
    const double uu = solid ? 0.0 : u_in;
    const double vv = solid ? 0.0 : perturbation(seed, t, amp);
    mu[t] = uu;
    mv[t] = vv;
    mw[t] = 0.0;
    mp[t] = 0.0;
    const long long c = L.idx(x, y, z);
    // The state is post-collision: the first collision relaxes f = feq(u) toward
    // feq((1 - alpha) u), the identity without porosity.
    const double s = alpha ? 1.0 - (double)alpha[t] : 1.0;
    for (int i = 0; i < Q; ++i) {
      const double edu = DT<Q>::ex(i) * uu + DT<Q>::ey(i) * vv;
      const double udu = uu * uu + vv * vv;
      const double f0 = Lat<Q>::w(i) * 0.0 * 3.0 +
                        Lat<Q>::w(i) * (3.0 * edu + 4.5 * edu * edu - 1.5 * udu);
      double fp = f0;
      if (alpha) {
        const double eb = s * edu, ub = s * s * udu;
        const double fb = Lat<Q>::w(i) * 0.0 * 3.0 +
                          Lat<Q>::w(i) * (3.0 * eb + 4.5 * eb * eb - 1.5 * ub);
        fp = f0 - (f0 - fb) * omega;
      }
      f[i * L.S + c] = Dec<ST>::template put<Q>(fp, i, L);
    }
  }
}

// ---- FP64 domain sums (mass = sum of rho over fluid, momentum) ------------------
template <int Q, class ST>
__global__ void reduce_mass_kernel(const ReduceArgs a) {
  using E = typename Store<ST>::elem;
  const E *f = static_cast<const E *>(a.f);
  const Layout &L = a.L;
  const long long total = (long long)L.nx * L.ny * L.nz;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % L.nx);
    const int y = (int)((t / L.nx) % L.ny);
    const int z = (int)(t / ((long long)L.nx * L.ny));
    if (mask_solid(a.mask, a.nxw, L.ny, x, y, z)) continue;
    const long long c = L.idx(x, y, z);
    double r = 1.0;
    for (int i = 0; i < Q; ++i) {
      const double fi = Dec<ST>::template get<Q>(f[i * L.S + c], i, L);
      r += fi;
      acc[1] += fi * DT<Q>::ex(i);
      acc[2] += fi * DT<Q>::ey(i);
      acc[3] += fi * DT<Q>::ez(i);
    }
    acc[0] += r;
  }
  __shared__ double sh[4][32];
  for (int o = 16; o > 0; o >>= 1)
    for (int q = 0; q < 4; ++q) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    for (int q = 0; q < 4; ++q) sh[q][wid] = acc[q];
  __syncthreads();
  __shared__ bool last;
  if (threadIdx.x == 0) {
    for (int q = 0; q < 4; ++q) {
      double b = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += sh[q][w];
      a.partials[4 * blockIdx.x + q] = b;
    }
    __threadfence();
    last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    const volatile double *p = a.partials;
    for (int q = 0; q < 4; ++q) {
      double s = 0.0;
      for (unsigned b = 0; b < gridDim.x; ++b) s += p[4 * b + q];
      a.out[q] = s;
    }
    *a.counter = 0u;
  }
}

// ---- dump / restore --------------------------------------------------------------
template <int Q, class ST>
__global__ void get_f_kernel(const Layout L, const void *f_, double *out) {
  using E = typename Store<ST>::elem;
  const E *f = static_cast<const E *>(f_);
  const long long N = (long long)L.nx * L.ny * L.nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N * Q;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / N);
    const long long n = t % N;
    const int x = (int)(n % L.nx);
    const int y = (int)((n / L.nx) % L.ny);
    const int z = (int)(n / ((long long)L.nx * L.ny));
    out[t] = Dec<ST>::template get<Q>(f[i * L.S + L.idx(x, y, z)], i, L);
  }
}

template <int Q, class ST>
__global__ void set_f_kernel(const Layout L, void *f_, const double *in) {
  using E = typename Store<ST>::elem;
  E *f = static_cast<E *>(f_);
  const long long N = (long long)L.nx * L.ny * L.nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N * Q;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / N);
    const long long n = t % N;
    const int x = (int)(n % L.nx);
    const int y = (int)((n / L.nx) % L.ny);
    const int z = (int)(n / ((long long)L.nx * L.ny));
    f[i * L.S + L.idx(x, y, z)] = Dec<ST>::template put<Q>(in[t], i, L);
  }
}

}  // namespace

long long launches() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
void count_launch(long long n) { __atomic_fetch_add(&g_launches, n, __ATOMIC_RELAXED); }

cudaError_t launch_sweep_q9(int store, int compute, const SweepArgs &a, cudaStream_t s);
cudaError_t launch_sweep_q27(int store, int compute, const SweepArgs &a, cudaStream_t s);

cudaError_t launch_sweep(int Q, int store, int compute, const SweepArgs &a, cudaStream_t s) {
  return Q == 9 ? launch_sweep_q9(store, compute, a, s) : launch_sweep_q27(store, compute, a, s);
}

cudaError_t launch_sweep_channel_q9(int store, int compute, const SweepArgs &a, cudaStream_t s,
                                     const SweepFork *fk);
cudaError_t launch_sweep_channel_q27(int store, int compute, const SweepArgs &a, cudaStream_t s,
                                      const SweepFork *fk);

cudaError_t launch_macros_channel_q9(int store, int compute, const SweepArgs &a, cudaStream_t s);
cudaError_t launch_macros_channel_q27(int store, int compute, const SweepArgs &a,
                                      cudaStream_t s);

cudaError_t launch_macros_channel(int Q, int store, int compute, const SweepArgs &a,
                                  cudaStream_t s) {
  return Q == 9 ? launch_macros_channel_q9(store, compute, a, s)
                : launch_macros_channel_q27(store, compute, a, s);
}

cudaError_t launch_stream_state_q9(int store, const SweepArgs &a, bool ref, double *out,
                                   cudaStream_t s);
cudaError_t launch_stream_state_q27(int store, const SweepArgs &a, bool ref, double *out,
                                    cudaStream_t s);
cudaError_t launch_stream_state(int Q, int store, const SweepArgs &a, bool ref, double *out,
                                cudaStream_t s) {
  return Q == 9 ? launch_stream_state_q9(store, a, ref, out, s)
                : launch_stream_state_q27(store, a, ref, out, s);
}

cudaError_t launch_sweep_channel(int Q, int store, int compute, const SweepArgs &a,
                                 cudaStream_t s, const SweepFork *fk) {
  return Q == 9 ? launch_sweep_channel_q9(store, compute, a, s, fk)
                : launch_sweep_channel_q27(store, compute, a, s, fk);
}

// Dispatch helper: run F<Q, ST> for the runtime (Q, store).
#define CFLBM_DISPATCH(Q, store, CALL)                                   \
  do {                                                                   \
    if ((Q) == 9) {                                                      \
      constexpr int QQ = 9;                                              \
      if ((store) == STORE_F64) { using ST = double; CALL; }             \
      else if ((store) == STORE_F32) { using ST = float; CALL; }         \
      else { using ST = F16Dev; CALL; }                                  \
    } else {                                                             \
      constexpr int QQ = 27;                                             \
      if ((store) == STORE_F64) { using ST = double; CALL; }             \
      else if ((store) == STORE_F32) { using ST = float; CALL; }         \
      else { using ST = F16Dev; CALL; }                                  \
    }                                                                    \
  } while (0)

cudaError_t launch_fill_channel(int Q, int store, const FillArgs &a, cudaStream_t s) {
  const bool d3 = Q == 27;
  const long long zr = d3 ? a.L.nz + 2 : 1;
  const long long total = 2 * ((a.L.ny + 2) * zr + (long long)a.L.nx * zr +
                               (d3 ? (long long)a.L.nx * a.L.ny : 0));
  const int blocks = blocks_for(total, 128);
  CFLBM_DISPATCH(Q, store, (fill_channel_kernel<QQ, ST><<<blocks, 128, 0, s>>>(a)));
  count_launch();
  return cudaGetLastError();
}

// The populations a pass writes: e along its axis positive (inlet copy, low wall)
// or negative (outlet extrapolation, high wall) -- 9 in D3Q27, 3 in D2Q9.
static void face_dirs(int Q, FaceOp &op) {
  op.ndir = 0;
  op.dirs = 0;
  for (int i = 1; i < Q; ++i) {
    const int e[3] = {Q == 27 ? Lat<27>::ex(i) : Lat<9>::ex(i),
                      Q == 27 ? Lat<27>::ey(i) : Lat<9>::ey(i),
                      Q == 27 ? Lat<27>::ez(i) : 0};
    const int ea = e[op.axis];
    const bool want = op.kind == 0 ? ea > 0 : (op.kind == 1 ? ea < 0 : (op.side == 0 ? ea > 0 : ea < 0));
    if (want && op.ndir < 9) op.dirs |= (unsigned long long)i << (5 * op.ndir++);
  }
}

cudaError_t launch_face_ops(int Q, int store, const FillArgs &a, FaceOp op0, FaceOp op1,
                            cudaStream_t s) {
  if (op0.axis != op1.axis) return cudaErrorInvalidValue;
  face_dirs(Q, op0);
  face_dirs(Q, op1);
  if (op0.ndir != op1.ndir || op0.ndir == 0) return cudaErrorInvalidValue;
  const int n[3] = {a.L.nx, a.L.ny, a.L.nz};
  const int ta = (op0.axis == 0) ? 1 : 0, tb = (op0.axis == 2) ? 1 : 2;
  const dim3 grid((unsigned)((n[ta] + 2 + 127) / 128), (unsigned)(Q == 27 ? n[tb] + 2 : 1),
                  (unsigned)(2 * op0.ndir));
  CFLBM_DISPATCH(Q, store, (face_op_kernel<QQ, ST><<<grid, 128, 0, s>>>(a, op0, op1)));
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_ghost_copy(int Q, int store, const Layout &L, const void *src, void *dst,
                              cudaStream_t s) {
  const int blocks = blocks_for((long long)L.px * L.nyp * L.nzp, 256);
  CFLBM_DISPATCH(Q, store, (ghost_copy_kernel<QQ, ST><<<blocks, 256, 0, s>>>(L, src, dst)));
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_links(int Q, int store, const LinkArgs &a, int blocks, cudaStream_t s) {
  CFLBM_DISPATCH(Q, store, (links_kernel<QQ, ST><<<blocks, 256, 0, s>>>(a)));
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_init_macros(int Q, int store, const Layout &L, void *f, const double *u,
                               const double *v, const double *w, const double *p,
                               cudaStream_t s) {
  const long long total =
      (long long)(L.nx + 2 * L.G) * (L.ny + 2 * L.G) * (L.nz + 2 * L.Gz);
  const int blocks = blocks_for(total, 256);
  CFLBM_DISPATCH(Q, store,
                 (init_macros_kernel<QQ, ST><<<blocks, 256, 0, s>>>(L, f, u, v, w, p)));
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_init_channel(int Q, int store, const Layout &L, void *f,
                                const uint32_t *mask, int nxw, double u_in, double amp,
                                unsigned long long seed, const float *alpha, double omega,
                                double *mu, double *mv, double *mw, double *mp, cudaStream_t s) {
  const int blocks = blocks_for((long long)L.nx * L.ny * L.nz, 256);
  CFLBM_DISPATCH(Q, store,
                 (init_channel_kernel<QQ, ST><<<blocks, 256, 0, s>>>(
                     L, f, mask, nxw, u_in, amp, seed, alpha, omega, mu, mv, mw, mp)));
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_reduce_mass(int Q, int store, const ReduceArgs &a, int blocks,
                               cudaStream_t s) {
  CFLBM_DISPATCH(Q, store, (reduce_mass_kernel<QQ, ST><<<blocks, 256, 0, s>>>(a)));
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_get_f(int Q, int store, const Layout &L, const void *f, double *out,
                         cudaStream_t s) {
  const int blocks = blocks_for((long long)L.nx * L.ny * L.nz * Q, 256);
  CFLBM_DISPATCH(Q, store, (get_f_kernel<QQ, ST><<<blocks, 256, 0, s>>>(L, f, out)));
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_set_f(int Q, int store, const Layout &L, void *f, const double *in,
                         cudaStream_t s) {
  const int blocks = blocks_for((long long)L.nx * L.ny * L.nz * Q, 256);
  CFLBM_DISPATCH(Q, store, (set_f_kernel<QQ, ST><<<blocks, 256, 0, s>>>(L, f, in)));
  count_launch();
  return cudaGetLastError();
}

}  // namespace cflbm
