// Discrete adjoint of the D2Q9 channel step (the differentiation form).
//
// Objective: J = mean over steps t0..t1 of the body force F_x (or F_y), where
// step t's force is the momentum exchange of state s_t, the post-collision
// field the t-th sweep reads.  Parameters: the per-cell Brinkman porosity
// alpha, the inlet speed u_in (inlet equilibrium and initial velocity) and the
// relaxation time tau = tau0 + 0.5 (omega = 1/tau).
//
// Forward: s_1 = C(feq(U0)), and s_{t+1} = C(g_{t+1}) with g_{t+1} = P s_t, P
// the boundary-resolving pull (plain shift, inlet equilibrium, zero-gradient
// outlet, free-slip mirror / no-slip / periodic y walls, halfway bounce-back on
// solids) and C the cellwise BGK collision toward feq(rho, (1 - alpha) u).
// With lambda_t = dJ/ds_t and mu^{t+1} = C'(g_{t+1})^T lambda_{t+1}:
//   lambda_t = P^T mu^{t+1} + c_t dF_t/ds_t       (c_t = 1/(t1-t0+1) in the window)
// The reverse sweep for state s_t is one fused kernel per cell X: gather
// lambda_{t+1}(X) from mu^{t+2} (a plain shift for regular cells; cells on the
// box faces or next to the body enumerate every neighbour (Y, i) whose pull
// source is X, i.e. bounce-back reverses into X's own opposite population),
// recompute g_{t+1}(X) = (P s_t)(X), and write mu^{t+1}(X) with the
// sensitivities of C and of the inlet pulls.  States come from checkpoints
// every K steps, recomputed one segment at a time into two alternating segment
// buffers: memory ceil(T/K) + 2K states.
// Sensitivity sums are deterministic: alpha per cell (arithmetic type within a
// segment, FP64 across segments), omega and u_in per block in FP64.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "handle.hpp"

namespace cflbm {
int record_error(int code, const char *msg);
}
using namespace cflbm;

namespace {

// D2Q9 velocities (0; +x, +y, -x, -y; diagonals 5..8), opposites and y mirrors
// as functions, usable with run-time indices in device code.
__host__ __device__ constexpr int AXf(int i) {
  return (i == 1 || i == 5 || i == 8) ? 1 : ((i == 3 || i == 6 || i == 7) ? -1 : 0);
}
__host__ __device__ constexpr int AYf(int i) {
  return (i == 2 || i == 5 || i == 6) ? 1 : ((i == 4 || i == 7 || i == 8) ? -1 : 0);
}
__host__ __device__ constexpr int AOPPf(int i) {
  return i == 0 ? 0 : (i < 5 ? (i + 1) % 4 + 1 : (i - 3) % 4 + 5);
}
__host__ __device__ constexpr int AMYf(int i) {
  return i == 2 ? 4 : i == 4 ? 2 : i == 5 ? 8 : i == 8 ? 5 : i == 6 ? 7 : i == 7 ? 6 : i;
}
__host__ __device__ constexpr double aw(int i) {
  return i == 0 ? 4.0 / 9.0 : (i < 5 ? 1.0 / 9.0 : 1.0 / 36.0);
}

constexpr int ABX = 32, ABY = 4, ANT = ABX * ABY;

constexpr int GMAX = 4;  // contributions per (cell, population) in the adjoint gather

struct AdjArgs {
  Layout L;                        // state layout
  const void *s;                   // s_t
  const void *mu_next;             // mu^{t+2}, dense [i][y][x]
  void *mu_out;                    // mu^{t+1}, dense (final gather: lambda_1)
  const uint32_t *mask;            // solid mask (bit-packed)
  int nxw;
  const int *aux;                  // per cell: AUX_SOLID, AUX_REGULAR or irregular entry r
  const long long *gat;            // per entry: 9 x GMAX dense mu indices (-1: none)
  const long long *pul;            // per entry: 9 pull sources, s element or -1 - inlet pop
  const unsigned *lkr;             // per entry: link bits (bit i: source of i is solid)
  const float *alpha;              // Brinkman porosity or null
  double omega;
  double u_in;
  double c_next;                   // objective weight of step t+1 (when seg is null)
  const int *seg;                  // device: index k of the segment being reversed
  const double *c_tab;             // objective weight of every step 0..T+1
  int K;                           // checkpoint spacing
  int q;                           // state s_t of this launch: t = k*K + 1 + q
  int obj_axis;                    // 0: F_x, 1: F_y
  void *g_alpha;                   // per cell, arithmetic type (segment accumulator)
  double *g_block;                 // per block: [0] omega, [1] u_in (FP64, owned)
};

enum { SRC_CELL = 0, SRC_INLET = 1 };
enum { AUX_SOLID = -2, AUX_REGULAR = -1 };

// Pull source of population i at fluid cell (x, y): the forward channel pull
// for D2Q9 (sweep.cuh, pull_resolved) with the configured y walls.  SRC_CELL:
// population j of (sx, sy) (bounce-back: the cell's own opposite population).
// SRC_INLET: inlet equilibrium population j.  lk: the cell's link bits.
int host_source(int nx, int ny, int wall_y, unsigned lk, int x, int y, int i, int &sx, int &sy,
                int &j) {
  if (i == 0) {
    sx = x; sy = y; j = 0;
    return SRC_CELL;
  }
  sx = x - AXf(i);
  sy = y - AYf(i);
  j = i;
  bool bb = false;
  if (sy < 0 || sy >= ny) {
    if (wall_y == WALL_PERIODIC) sy = sy < 0 ? sy + ny : sy - ny;
    else if (wall_y == WALL_FREESLIP) { j = AMYf(i); sy = y; }
    else bb = true;
  }
  if (bb || ((lk >> i) & 1u)) {
    sx = x; sy = y; j = AOPPf(i);
    return SRC_CELL;
  }
  if (sx < 0) return SRC_INLET;
  if (sx >= nx) sx = nx - 1;
  return SRC_CELL;
}

__device__ __forceinline__ double inlet_f(int j, double u) {
  const double e = AXf(j) * u;
  return aw(j) * (3.0 * e + 4.5 * e * e - 1.5 * u * u);
}
__device__ __forceinline__ double inlet_dfdu(int j, double u) {
  return aw(j) * (3.0 * AXf(j) + 9.0 * AXf(j) * AXf(j) * u - 3.0 * u);
}

// Block sums of two FP64 values; the result is valid in thread 0.
__device__ __forceinline__ void block_sum2(double v0, double v1, double (*sh)[ANT / 32],
                                           double &o0, double &o1) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v0 += __shfl_down_sync(0xffffffffu, v0, o);
    v1 += __shfl_down_sync(0xffffffffu, v1, o);
  }
  const int tid = threadIdx.y * ABX + threadIdx.x;
  if ((tid & 31) == 0) {
    sh[0][tid >> 5] = v0;
    sh[1][tid >> 5] = v1;
  }
  __syncthreads();
  o0 = o1 = 0.0;
  if (tid == 0)
    for (int w = 0; w < ANT / 32; ++w) {
      o0 += sh[0][w];
      o1 += sh[1][w];
    }
}

template <class A, bool FINAL>
__global__ void __launch_bounds__(ANT) adjoint_kernel(const AdjArgs a) {
  __shared__ double sh[2][ANT / 32];
  const int nx = a.L.nx, ny = a.L.ny;
  const int x = blockIdx.x * ABX + threadIdx.x;
  const int y = blockIdx.y * ABY + threadIdx.y;
  const bool in = x < nx && y < ny;
  const long long N = (long long)nx * ny;
  const long long cell = (long long)y * nx + x;
  const int aux = in ? a.aux[cell] : AUX_SOLID;
  const A *mu_n = static_cast<const A *>(a.mu_next);
  const A *s = static_cast<const A *>(a.s);
  A *ga = static_cast<A *>(a.g_alpha);
  double d_omega = 0.0, d_u = 0.0;

  // lambda_{t+1}(X) = (P^T mu^{t+2})(X) + c_{t+1} dF/ds_{t+1}(X), and (not FINAL)
  // g_{t+1}(X) = (P s_t)(X).  Regular cells: plain shifts.  Irregular cells (box
  // faces, next to the body): the host-built lists of contributing (Y, i) and of
  // pull sources.  Every load of a path is issued before any is used.
  A lam[9], g[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) lam[k] = g[k] = A(0);
  A al = A(0), gacc = A(0);
  int inl = 0;       // bit i: population i of g comes from the inlet
  long long pe[9];   // irregular: pull sources (inlet: -1 - population)
  if (aux == AUX_REGULAR) {
#pragma unroll
    for (int j = 0; j < 9; ++j) lam[j] = mu_n[j * N + cell + (long long)AYf(j) * nx + AXf(j)];
    if constexpr (!FINAL) {
      const long long c = a.L.idx(x, y, 0);
#pragma unroll
      for (int i = 0; i < 9; ++i) g[i] = s[i * a.L.S + c - a.L.off(AXf(i), AYf(i), 0)];
      if (a.alpha) al = A(a.alpha[cell]);
      gacc = ga[cell];
    }
  } else if (aux >= 0) {
    const long long *gt = a.gat + (long long)aux * 9 * GMAX;
    long long ge[9 * GMAX];
#pragma unroll
    for (int k = 0; k < 9 * GMAX; ++k) ge[k] = gt[k];
    const unsigned lk = a.lkr[aux];
    if constexpr (!FINAL) {
#pragma unroll
      for (int i = 0; i < 9; ++i) pe[i] = a.pul[(long long)aux * 9 + i];
    }
#pragma unroll
    for (int j = 0; j < 9; ++j)
#pragma unroll
      for (int m = 0; m < GMAX; ++m)
        if (ge[j * GMAX + m] >= 0) lam[j] += mu_n[ge[j * GMAX + m]];
    if constexpr (!FINAL) {
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        if (pe[i] >= 0) {
          g[i] = s[pe[i]];
        } else {
          g[i] = A(inlet_f((int)(-1 - pe[i]), a.u_in));
          inl |= 1 << i;
        }
      }
      if (a.alpha) al = A(a.alpha[cell]);
      gacc = ga[cell];
    }
    if (lk) {
      // The segment index lives on the device so one captured graph reverses any
      // full segment: a launch reads k and the weight of its step t + 1.
      const double c_next = a.seg ? a.c_tab[(long long)(*a.seg) * a.K + 2 + a.q] : a.c_next;
#pragma unroll
      for (int j = 1; j < 9; ++j)
        if ((lk >> AOPPf(j)) & 1u)
          lam[j] += A(c_next * 2.0 * (a.obj_axis == 0 ? AXf(j) : AYf(j)));
    }
  }
  if constexpr (FINAL) {
    if (in) {
#pragma unroll
      for (int k = 0; k < 9; ++k) static_cast<A *>(a.mu_out)[k * N + cell] = lam[k];
    }
    return;
  } else {
    A mu[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) mu[k] = A(0);
    if (aux != AUX_SOLID) {
      // ---- mu = C'(g)^T lambda and the collision sensitivities -------------------
      A rho3 = A(0), jx = A(0), jy = A(0);
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        rho3 += g[i];
        jx += g[i] * A(AXf(i));
        jy += g[i] * A(AYf(i));
      }
      const A one_a = A(1) - al;
      const A bx = one_a * jx, by = one_a * jy;
      const A om = A(a.omega);
      const A usq = bx * bx + by * by;
      A A0 = A(0), A1x = A(0), A1y = A(0), A2x = A(0), A2y = A(0), dom = A(0);
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        const A w = A(aw(k));
        const A eu = A(AXf(k)) * bx + A(AYf(k)) * by;
        const A feq = w * (rho3 + A(3) * eu + A(4.5) * eu * eu - A(1.5) * usq);
        dom += lam[k] * (feq - g[k]);
        const A lw = lam[k] * w;
        A0 += lw;
        A1x += lw * A(AXf(k));
        A1y += lw * A(AYf(k));
        A2x += lw * eu * A(AXf(k));
        A2y += lw * eu * A(AYf(k));
      }
      const A vx = A(3) * A1x + A(9) * A2x - A(3) * bx * A0;
      const A vy = A(3) * A1y + A(9) * A2y - A(3) * by * A0;
#pragma unroll
      for (int i = 0; i < 9; ++i)
        mu[i] = (A(1) - om) * lam[i] + om * (A0 + one_a * (vx * A(AXf(i)) + vy * A(AYf(i))));
      if (inl) {
#pragma unroll
        for (int i = 0; i < 9; ++i)
          if ((inl >> i) & 1)
            d_u += static_cast<double>(mu[i]) * inlet_dfdu((int)(-1 - pe[i]), a.u_in);
      }
      // d feq / d alpha, with d u_B / d alpha = -(jx, jy).
      const A dal = om * (-A(3) * (A1x * jx + A1y * jy) - A(9) * (A2x * jx + A2y * jy) +
                          A(3) * (bx * jx + by * jy) * A0);
      ga[cell] = gacc + dal;
      d_omega = static_cast<double>(dom);
    }
    if (in) {
#pragma unroll
      for (int k = 0; k < 9; ++k) static_cast<A *>(a.mu_out)[k * N + cell] = mu[k];
    }
    double so, su;
    block_sum2(d_omega, d_u, sh, so, su);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      double *gb = a.g_block + 2 * ((long long)blockIdx.y * gridDim.x + blockIdx.x);
      gb[0] += so;
      gb[1] += su;
    }
  }
}

// Sensitivities of the initial state s_1 = C(feq(U0)) through lambda_1:
// U0 = (u_in, v0) in fluid cells, U_B = (1 - alpha) U0, p = 0.
template <class A>
__global__ void __launch_bounds__(ANT) init_sens_kernel(const AdjArgs a, const A *lam1,
                                                        const double *v0, double *g_alpha64) {
  __shared__ double sh[2][ANT / 32];
  const int nx = a.L.nx, ny = a.L.ny;
  const int x = blockIdx.x * ABX + threadIdx.x;
  const int y = blockIdx.y * ABY + threadIdx.y;
  const long long N = (long long)nx * ny;
  const long long cell = (long long)y * nx + x;
  double gu = 0.0, gom = 0.0;
  if (x < nx && y < ny && !mask_solid(a.mask, a.nxw, ny, x, y, 0)) {
    const double al = a.alpha ? (double)a.alpha[cell] : 0.0;
    const double ux = a.u_in, uy = v0[cell];
    const double bx = (1.0 - al) * ux, by = (1.0 - al) * uy;
    const double om = a.omega;
    double gal = 0.0;
    for (int k = 0; k < 9; ++k) {
      const double w = aw(k), ex = AXf(k), ey = AYf(k);
      const double eu = ex * ux + ey * uy, eb = ex * bx + ey * by;
      const double f0 = w * (3.0 * eu + 4.5 * eu * eu - 1.5 * (ux * ux + uy * uy));
      const double fb = w * (3.0 * eb + 4.5 * eb * eb - 1.5 * (bx * bx + by * by));
      const double df0 = w * (3.0 * ex + 9.0 * eu * ex - 3.0 * ux);
      const double dfb = (1.0 - al) * w * (3.0 * ex + 9.0 * eb * ex - 3.0 * bx);
      const double l = (double)lam1[k * N + cell];
      gu += l * ((1.0 - om) * df0 + om * dfb);
      gom += l * (fb - f0);
      gal += l * om * w * (-3.0 * eu - 9.0 * eb * eu + 3.0 * (bx * ux + by * uy));
    }
    g_alpha64[cell] += gal;
  }
  double so, su;
  block_sum2(gom, gu, sh, so, su);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    double *gb = a.g_block + 2 * ((long long)blockIdx.y * gridDim.x + blockIdx.x);
    gb[0] += so;
    gb[1] += su;
  }
}

// End of a checkpoint segment: g64 += gA; gA = 0; the segment index steps back
// (every kernel that reads it precedes this one on the stream).
template <class A>
__global__ void flush_kernel(A *ga, double *g64, long long n, int *seg) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x) {
    g64[c] += static_cast<double>(ga[c]);
    ga[c] = A(0);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *seg -= 1;
}

// The recompute stream's segment index steps back after its segment.
__global__ void step_back_kernel(int *seg) { *seg -= 1; }

// seg_states[0] = checkpoint k = *seg (16-byte words; sizes are multiples of 16).
__global__ void checkpoint_copy_kernel(const uint4 *ck, const int *seg, long long words,
                                       uint4 *dst) {
  const uint4 *src = ck + (long long)(*seg) * words;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < words;
       c += (long long)gridDim.x * blockDim.x)
    dst[c] = src[c];
}

int afail(int code, const std::string &m) { return record_error(code, m.c_str()); }

#define ACK(call)                                                                         \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return afail(CFLBM_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

// Device scratch of one adjoint run, freed on return.
struct AdjScratch {
  std::vector<void *> ptrs;
  ~AdjScratch() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T **p, size_t n) {
    void *v = nullptr;
    cudaError_t e = cudaMalloc(&v, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) ptrs.push_back(v);
    *p = static_cast<T *>(v);
    return e;
  }
};

// The second stream of the reverse sweep and its fork/join events.
struct AdjStreams {
  cudaStream_t rec = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaError_t create() {
    cudaError_t e = cudaStreamCreateWithFlags(&rec, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    return e;
  }
  ~AdjStreams() {
    if (rec) cudaStreamSynchronize(rec);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (rec) cudaStreamDestroy(rec);
  }
};

// Host tables of the reverse sweep.  Every fluid cell X is classified from the
// forward pull itself: X is regular when its own pull is the plain shift
// (source X - e_i, population i, for every i) and the pulls that read X are
// exactly the 9 plain ones ((X + e_j, j) for every j).  For every other fluid
// cell (box faces, cells next to the body) the entry lists, per population j of
// X, the dense mu indices i*N + Y of every pull (Y, i) whose source is (X, j),
// and X's own 9 pull sources; lk holds its link bits (the momentum-exchange
// force reads them).
struct AdjTables {
  std::vector<int> aux;
  std::vector<long long> gat, pul;
  std::vector<unsigned> lkr;
};

int adjoint_tables(const cflbm_handle *h, const std::vector<uint8_t> &solid, AdjTables &t) {
  const int nx = h->L.nx, ny = h->L.ny, wall = h->cfg.wall_y;
  const long long N = (long long)nx * ny;
  std::vector<unsigned> lk((size_t)N, 0u);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      unsigned b = 0;
      for (int i = 1; i < 9; ++i) {
        int sx = x - AXf(i), sy = y - AYf(i);
        if (sy < 0 || sy >= ny) {
          if (wall == CFLBM_WALL_PERIODIC) sy = (sy + ny) % ny;
          else if (wall == CFLBM_WALL_FREESLIP) sy = y;
          else continue;
        }
        if (sx < 0) continue;
        if (sx >= nx) sx = nx - 1;
        if (solid[(size_t)sy * nx + sx]) b |= 1u << i;
      }
      lk[(size_t)y * nx + x] = b;
    }
  std::vector<uint8_t> plain((size_t)N, 0), bad((size_t)N, 0);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const size_t Y = (size_t)y * nx + x;
      if (solid[Y]) continue;
      for (int i = 0; i < 9; ++i) {
        int sx, sy, j;
        if (host_source(nx, ny, wall, lk[Y], x, y, i, sx, sy, j) == SRC_INLET) {
          bad[Y] = 1;
          continue;
        }
        const bool shift = sx == x - AXf(i) && sy == y - AYf(i) && j == i;
        if (!shift) bad[Y] = 1;
        const size_t X = (size_t)sy * nx + sx;
        if (shift) ++plain[X];
        else bad[X] = 1;
      }
    }
  t.aux.assign((size_t)N, AUX_REGULAR);
  long long nirr = 0;
  for (size_t c = 0; c < (size_t)N; ++c) {
    if (solid[c]) t.aux[c] = AUX_SOLID;
    else if (bad[c] || plain[c] != 9) t.aux[c] = (int)nirr++;
  }
  t.gat.assign((size_t)nirr * 9 * GMAX, -1);
  t.pul.assign((size_t)nirr * 9, 0);
  t.lkr.assign((size_t)nirr, 0u);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const size_t Y = (size_t)y * nx + x;
      if (solid[Y]) continue;
      const int rY = t.aux[Y];
      if (rY >= 0) t.lkr[rY] = lk[Y];
      for (int i = 0; i < 9; ++i) {
        int sx, sy, j;
        const int kind = host_source(nx, ny, wall, lk[Y], x, y, i, sx, sy, j);
        if (rY >= 0)
          t.pul[(size_t)rY * 9 + i] = kind == SRC_INLET ? -1 - j : j * h->L.S + h->L.idx(sx, sy, 0);
        if (kind == SRC_INLET) continue;
        const int rX = t.aux[(size_t)sy * nx + sx];
        if (rX < 0) continue;
        long long *slot = &t.gat[((size_t)rX * 9 + j) * GMAX];
        int m = 0;
        while (m < GMAX && slot[m] >= 0) ++m;
        if (m == GMAX)
          return afail(CFLBM_E_UNSUPPORTED, "cflbm_adjoint: more than 4 pulls read one population");
        slot[m] = (long long)i * N + (long long)Y;
      }
    }
  return CFLBM_OK;
}

template <class A>
int run_adjoint(cflbm_handle *h, const cflbm_adjoint_spec *sp, double *dJ_dalpha,
                cflbm_adjoint_result *res) {
  using clk = std::chrono::steady_clock;
  const Layout &L = h->L;
  const int nx = L.nx, ny = L.ny;
  const long long N = (long long)nx * ny;
  const int T = sp->steps, K = sp->checkpoint_every;
  const size_t sb = h->f_bytes;
  const int nck = (T + K - 1) / K;
  const dim3 blk(ABX, ABY), grd((nx + ABX - 1) / ABX, (ny + ABY - 1) / ABY);
  const long long nblk = (long long)grd.x * grd.y;
  cudaStream_t st = h->stream;

  AdjScratch sc;
  char *ck = nullptr, *seg = nullptr;
  A *mu0 = nullptr, *mu1 = nullptr, *ga = nullptr;
  double *ga64 = nullptr, *gblk = nullptr, *v0 = nullptr;
  int *aux = nullptr;
  long long *gat = nullptr, *pul = nullptr;
  unsigned *lkr = nullptr;
  double *scr_part = nullptr, *scr_hist = nullptr;
  unsigned *scr_cnt = nullptr;
  long long *scr_step = nullptr;
  ACK(sc.alloc(&ck, (size_t)nck * sb));
  ACK(sc.alloc(&seg, 2 * (size_t)K * sb));
  ACK(sc.alloc(&mu0, 9 * (size_t)N));
  ACK(sc.alloc(&mu1, 9 * (size_t)N));
  ACK(sc.alloc(&ga, N));
  ACK(sc.alloc(&ga64, N));
  ACK(sc.alloc(&gblk, 2 * nblk));
  ACK(sc.alloc(&v0, N));
  ACK(sc.alloc(&aux, N));
  ACK(sc.alloc(&scr_part, 3 * (size_t)(h->n_slow + 4)));
  ACK(sc.alloc(&scr_hist, 3));
  ACK(sc.alloc(&scr_cnt, 1));
  ACK(sc.alloc(&scr_step, 1));
  ACK(cudaMemsetAsync(mu1, 0, 9 * N * sizeof(A), st));
  ACK(cudaMemsetAsync(ga, 0, N * sizeof(A), st));
  ACK(cudaMemsetAsync(ga64, 0, N * 8, st));
  ACK(cudaMemsetAsync(gblk, 0, 2 * nblk * 8, st));
  ACK(cudaMemsetAsync(scr_cnt, 0, 4, st));
  ACK(cudaMemsetAsync(scr_step, 0, 8, st));
  long long n_irregular = 0;
  {
    std::vector<uint32_t> mw((size_t)h->nxw * ny);
    ACK(cudaMemcpyAsync(mw.data(), h->d_mask, mw.size() * 4, cudaMemcpyDeviceToHost, st));
    ACK(cudaStreamSynchronize(st));
    std::vector<uint8_t> solid(N);
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x)
        solid[(size_t)y * nx + x] = (mw[(size_t)y * h->nxw + (x >> 5)] >> (x & 31)) & 1u;
    AdjTables tb;
    int trc = adjoint_tables(h, solid, tb);
    if (trc) return trc;
    n_irregular = (long long)tb.lkr.size();
    ACK(sc.alloc(&gat, tb.gat.size()));
    ACK(sc.alloc(&pul, tb.pul.size()));
    ACK(sc.alloc(&lkr, tb.lkr.size()));
    std::vector<double> pv(N);
    for (long long n = 0; n < N; ++n)
      pv[n] = solid[n] ? 0.0 : perturbation(h->cfg.seed, n, h->cfg.perturb_amp);
    ACK(cudaMemcpyAsync(aux, tb.aux.data(), N * 4, cudaMemcpyHostToDevice, st));
    ACK(cudaMemcpyAsync(gat, tb.gat.data(), tb.gat.size() * 8, cudaMemcpyHostToDevice, st));
    ACK(cudaMemcpyAsync(pul, tb.pul.data(), tb.pul.size() * 8, cudaMemcpyHostToDevice, st));
    ACK(cudaMemcpyAsync(lkr, tb.lkr.data(), tb.lkr.size() * 4, cudaMemcpyHostToDevice, st));
    ACK(cudaMemcpyAsync(v0, pv.data(), N * 8, cudaMemcpyHostToDevice, st));
    ACK(cudaStreamSynchronize(st));
  }

  // ---- forward run, keeping s_1, s_{K+1}, s_{2K+1}, ... ---------------------------
  const auto t_f0 = clk::now();
  for (int k = 0; k < nck; ++k) {
    ACK(cudaMemcpyAsync(ck + (size_t)k * sb, h->fA, sb, cudaMemcpyDeviceToDevice, st));
    int rc = cflbm_step(h, std::min(K, T - k * K));
    if (rc) return rc;
  }
  ACK(cudaStreamSynchronize(st));
  const double t_forward = std::chrono::duration<double>(clk::now() - t_f0).count();
  std::vector<double> hist(3 * (size_t)T);
  int64_t nh = 0;
  int rc = cflbm_force_history(h, hist.data(), T, &nh);
  if (rc) return rc;
  if (nh != T) return afail(CFLBM_E_INVALID, "cflbm_adjoint: force history shorter than the run");
  const int t0 = sp->window_begin, t1 = sp->window_end;
  const double cw = 1.0 / (t1 - t0 + 1);
  double J = 0.0;
  for (int t = t0; t <= t1; ++t) J += cw * hist[3 * (size_t)(t - 1) + sp->objective];

  // ---- reverse sweep, one checkpoint segment at a time ----------------------------
  // Segment k holds states s_{kK+1} .. s_{kK+n}.  Recomputing it (copy
  // checkpoint k, n - 1 forward sweeps) and reversing it (adjoint kernels from
  // the top state down, then the flush) use one of two state buffers, k % 2.
  // Unit k reverses segment k on the main stream while a second stream
  // recomputes segment k - 1 into the other buffer; the unit joins at its end.
  // The segment indices the kernels read are device integers (one for each
  // stream's work, stepped by the stream's last kernel), so every interior unit
  // is the same launch sequence: it is captured as a CUDA graph per buffer and
  // mu parity and replayed.  The first unit (partial top segment, whose top
  // state s_T has lambda_{T+1} = 0) and the last (nothing left to recompute)
  // run as direct launches.
  const auto t_r0 = clk::now();
  int *d_seg = nullptr;  // [0]: segment being reversed, [1]: segment being recomputed
  double *c_tab = nullptr;
  ACK(sc.alloc(&d_seg, 2));
  ACK(sc.alloc(&c_tab, (size_t)T + 2));
  {
    std::vector<double> ct((size_t)T + 2, 0.0);
    for (int t = t0; t <= t1; ++t) ct[t] = cw;
    const int k_last[2] = {nck - 1, nck - 1};
    ACK(cudaMemcpyAsync(c_tab, ct.data(), ct.size() * 8, cudaMemcpyHostToDevice, st));
    ACK(cudaMemcpyAsync(d_seg, k_last, 8, cudaMemcpyHostToDevice, st));
    ACK(cudaStreamSynchronize(st));
  }
  AdjStreams rs;
  ACK(rs.create());
  cudaStream_t rec = rs.rec;
  AdjArgs aa{};
  aa.L = L;
  aa.mask = h->d_mask;
  aa.nxw = h->nxw;
  aa.aux = aux;
  aa.gat = gat;
  aa.pul = pul;
  aa.lkr = lkr;
  aa.alpha = h->d_alpha;
  aa.omega = h->omega;
  aa.u_in = h->cfg.u0;
  aa.obj_axis = sp->objective;
  aa.g_alpha = ga;
  aa.g_block = gblk;
  aa.seg = d_seg;
  aa.c_tab = c_tab;
  aa.K = K;
  A *mu_next = mu1, *mu_cur = mu0;
  const long long words = (long long)(sb / 16);
  const int copy_blocks = (int)std::min<long long>((words + 255) / 256, 4096);
  const int flush_blocks = (int)std::min<long long>((N + 255) / 256, 4096);
  char *buf[2] = {seg, seg + (size_t)K * sb};
  // Recompute one segment of n states into b (stream s).
  auto recompute = [&](cudaStream_t s, char *b, int n) -> int {
    checkpoint_copy_kernel<<<copy_blocks, 256, 0, s>>>(reinterpret_cast<const uint4 *>(ck),
                                                        d_seg + 1, words,
                                                        reinterpret_cast<uint4 *>(b));
    for (int q = 1; q < n; ++q) {
      SweepArgs sa = channel_args(h, b + (size_t)(q - 1) * sb, b + (size_t)q * sb, false);
      sa.partials = scr_part;
      sa.counter = scr_cnt;
      sa.hist = scr_hist;
      sa.step = scr_step;
      sa.cap = 1;
      ACK(launch_sweep_channel(9, h->cfg.storage, h->cfg.compute, sa, s));
    }
    step_back_kernel<<<1, 1, 0, s>>>(d_seg + 1);
    count_launch(2);
    ACK(cudaGetLastError());
    return CFLBM_OK;
  };
  // Reverse one segment of n states held in b (main stream).
  auto reverse = [&](char *b, int n, bool skip_top) -> int {
    for (int q = n - 1; q >= 0; --q) {
      if (skip_top && q == n - 1) continue;
      aa.s = b + (size_t)q * sb;
      aa.q = q;
      aa.mu_next = mu_next;
      aa.mu_out = mu_cur;
      adjoint_kernel<A, false><<<grd, blk, 0, st>>>(aa);
      count_launch(1);
      std::swap(mu_next, mu_cur);
    }
    flush_kernel<A><<<flush_blocks, 256, 0, st>>>(ga, ga64, N, d_seg);
    count_launch(1);
    ACK(cudaGetLastError());
    return CFLBM_OK;
  };
  // Unit k: reverse segment k (n states, buffer k % 2) while recomputing
  // segment k - 1 (K states, the other buffer) when k > 0.
  auto unit = [&](int k, int n, bool skip_top) -> int {
    ACK(cudaEventRecord(rs.fork, st));
    ACK(cudaStreamWaitEvent(rec, rs.fork, 0));
    if (k > 0) {
      const int rc2 = recompute(rec, buf[(k - 1) & 1], K);
      if (rc2) return rc2;
    }
    const int rc1 = reverse(buf[k & 1], n, skip_top);
    if (rc1) return rc1;
    ACK(cudaEventRecord(rs.join, rec));
    ACK(cudaStreamWaitEvent(st, rs.join, 0));
    return CFLBM_OK;
  };
  const int n_top = T - (nck - 1) * K;
  int urc = recompute(st, buf[(nck - 1) & 1], n_top);
  if (!urc) urc = unit(nck - 1, n_top, true);
  if (urc) return urc;
  cudaGraphExec_t gexec[4] = {nullptr, nullptr, nullptr, nullptr};
  struct GraphGuard {
    cudaGraphExec_t *g;
    ~GraphGuard() {
      for (int i = 0; i < 4; ++i)
        if (g[i]) cudaGraphExecDestroy(g[i]);
    }
  } guard{gexec};
  long long graph_launches = 0;
  for (int k = nck - 2; k >= 1; --k) {
    const int gi = (k & 1) * 2 + (mu_next == mu1 ? 0 : 1);
    if (!gexec[gi]) {
      const long long n0 = cflbm_launch_count();
      cudaGraph_t g = nullptr;
      ACK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      const int rcs = unit(k, K, false);
      const cudaError_t ec = cudaStreamEndCapture(st, &g);
      if (rcs) {
        if (g) cudaGraphDestroy(g);
        return rcs;
      }
      ACK(ec);
      const cudaError_t ei = cudaGraphInstantiate(&gexec[gi], g, 0);
      cudaGraphDestroy(g);
      ACK(ei);
      graph_launches = cflbm_launch_count() - n0;
      // Capture counted the launches and moved the host-side mu parity; this
      // first replay runs them.
      ACK(cudaGraphLaunch(gexec[gi], st));
    } else {
      ACK(cudaGraphLaunch(gexec[gi], st));
      count_launch(graph_launches);
      if (K & 1) std::swap(mu_next, mu_cur);
    }
  }
  if (nck >= 2) {
    urc = unit(0, K, false);
    if (urc) return urc;
  }
  // lambda_1 and the sensitivities of the initial state.
  aa.mu_next = mu_next;
  aa.mu_out = mu_cur;
  aa.seg = nullptr;
  aa.c_next = (1 >= t0 && 1 <= t1) ? cw : 0.0;
  adjoint_kernel<A, true><<<grd, blk, 0, st>>>(aa);
  init_sens_kernel<A><<<grd, blk, 0, st>>>(aa, mu_cur, v0, ga64);
  count_launch(2);
  ACK(cudaGetLastError());
  std::vector<double> hgb(2 * nblk);
  if (dJ_dalpha) ACK(cudaMemcpyAsync(dJ_dalpha, ga64, N * 8, cudaMemcpyDeviceToHost, st));
  ACK(cudaMemcpyAsync(hgb.data(), gblk, 2 * nblk * 8, cudaMemcpyDeviceToHost, st));
  ACK(cudaStreamSynchronize(st));
  const double t_reverse = std::chrono::duration<double>(clk::now() - t_r0).count();
  double somega = 0.0, su = 0.0;
  for (long long b = 0; b < nblk; ++b) {
    somega += hgb[2 * b];
    su += hgb[2 * b + 1];
  }
  std::memset(res, 0, sizeof(*res));
  res->J = J;
  res->dJ_du_in = su;
  res->dJ_dtau = -h->omega * h->omega * somega;
  res->seconds_forward = t_forward;
  res->seconds_reverse = t_reverse;
  res->device_bytes = (int64_t)((size_t)(nck + 2 * K) * sb + (2 * 9 + 1) * N * sizeof(A) +
                                N * (8 + 8 + 4) + n_irregular * (9 * GMAX * 8 + 9 * 8 + 4) +
                                2 * nblk * 8);
  return CFLBM_OK;
}

}  // namespace

extern "C" int cflbm_adjoint(cflbm_handle *h, const cflbm_adjoint_spec *sp, double *dJ_dalpha,
                             cflbm_adjoint_result *res) {
  if (!h || !sp || !res) return afail(CFLBM_E_INVALID, "cflbm_adjoint: null argument");
  if (h->Q != 9 || h->cfg.profile != CFLBM_PROFILE_CHANNEL)
    return afail(CFLBM_E_UNSUPPORTED, "cflbm_adjoint: the adjoint covers the D2Q9 channel profile");
  const bool f32 = h->cfg.storage == CFLBM_STORE_FP32 && h->cfg.compute == CFLBM_COMPUTE_FP32;
  const bool f64 = h->cfg.storage == CFLBM_STORE_FP64 && h->cfg.compute == CFLBM_COMPUTE_FP64;
  if (!f32 && !f64)
    return afail(CFLBM_E_UNSUPPORTED,
                 "cflbm_adjoint: storage/arithmetic must be FP32/FP32 or FP64/FP64");
  if (h->batched) return afail(CFLBM_E_INVALID, "cflbm_adjoint: batch instances are not supported");
  if (h->steps_done != 0) return afail(CFLBM_E_INVALID, "cflbm_adjoint: needs a fresh handle");
  if (h->L.nx < 3 || h->L.ny < 3)
    return afail(CFLBM_E_INVALID, "cflbm_adjoint: needs nx, ny >= 3");
  if (sp->steps < 1 || sp->checkpoint_every < 1 || sp->window_begin < 1 ||
      sp->window_end < sp->window_begin || sp->window_end > sp->steps ||
      (sp->objective != 0 && sp->objective != 1))
    return afail(CFLBM_E_INVALID, "cflbm_adjoint: bad spec (steps, checkpoint, window, objective)");
  if (h->hist_cap < sp->steps)
    return afail(CFLBM_E_INVALID, "cflbm_adjoint: force_history must hold every step of the run");
  cudaError_t e = cudaSetDevice(h->cfg.device);
  if (e != cudaSuccess) return afail(CFLBM_E_CUDA, cudaGetErrorString(e));
  return f32 ? run_adjoint<float>(h, sp, dJ_dalpha, res)
             : run_adjoint<double>(h, sp, dJ_dalpha, res);
}
