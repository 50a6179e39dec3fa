// Internal device-side declarations of the cylinder-flow solver.
//
// Data layout in HBM (two population buffers A/B, x fastest everywhere):
//   SOA : f[i][z + Gz][y + G][x + xoff]   one array per population
//   ROWS: f[z + Gz][y + G][i][x + xoff]   the Q rows of one (y, z) are adjacent
// with G ghost layers around the interior in x and y (and z in 3-D) and rows
// padded to `px` elements so every interior row starts on a 128-byte boundary.
// In both layouts population i of cell (x, y, z) sits at i*S + idx(x, y, z) and
// the pull source x - e_i is a constant offset, so each population is a pure
// shift and every element is read exactly once per sweep.  ROWS keeps the 2Q
// streams a warp touches within a few rows, i.e. a few DRAM pages and TLB
// entries, instead of 2Q arrays hundreds of megabytes apart.
// A holds the post-collision populations of the current step; the sweep pulls
// from A and writes the next post-collision state into B; the buffers swap.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "lattice.cuh"

namespace cflbm {

enum Profile { PROFILE_CHANNEL = 0, PROFILE_REF2D = 1, PROFILE_REF3D = 2, PROFILE_REF2DS = 3 };
enum Wall { WALL_FREESLIP = 0, WALL_NOSLIP = 1, WALL_PERIODIC = 2 };
enum StoreKind { STORE_F64 = 0, STORE_F32 = 1, STORE_F16 = 2 };
enum ComputeKind { COMPUTE_F64 = 0, COMPUTE_F32 = 1, COMPUTE_DF64 = 2 };
enum LayoutKind { LAYOUT_SOA = 0, LAYOUT_ROWS = 1 };

struct Layout {
  int nx, ny, nz;  // interior cells (nz = 1 in 2-D)
  int G, Gz;       // ghost layers in x/y and in z (0 in 2-D)
  int xoff;        // element offset of interior x = 0 inside a row
  int px;          // row pitch in elements
  int nyp, nzp;    // padded y and z extents
  long long S;     // elements between populations of one cell
  long long rs;    // elements between rows (y)
  long long zs;    // elements between planes (z)
  long long total; // elements per buffer
  float fbase[27]; // storage offset of each population (Store<F16Dev>; 0 otherwise)
  __host__ __device__ long long idx(int x, int y, int z) const {
    return (long long)(z + Gz) * zs + (long long)(y + G) * rs + (x + xoff);
  }
  __host__ __device__ long long off(int ex, int ey, int ez) const {
    return (long long)ex + rs * ey + zs * ez;
  }
  __host__ __device__ bool interior(int x, int y, int z) const {
    return x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz;
  }
};

__host__ __device__ inline bool mask_solid(const uint32_t *m, int nxw, int ny, int x, int y, int z) {
  return (m[((long long)z * ny + y) * nxw + (x >> 5)] >> (x & 31)) & 1u;
}

// Indices of the relaxation constants (their meaning: bgk_relax_v, sweep.cuh).
constexpr int RK_OMC = 0, RK_W = 1, RK_A = 5, RK_3 = 9, RK_LW = 13, RK_L3 = 14, RK_LA = 15,
              RK_M3 = 16, RK_N = 20;

struct SweepArgs {
  Layout L;
  const void *fa;        // post-collision state of this step (ghosts filled)
  void *fb;              // next post-collision state
  const uint32_t *mask;  // bit-packed interior solid mask
  int nxw;               // mask words per row
  float omega_f;
  double omega;
  // Relaxation constants (1 - omega and omega times the weight-class factors;
  // layout in sweep.cuh, RK_*): FP64, the conserving FP32 set, and the FP32
  // remainder rk - rkf for double-float arithmetic.
  double rk[RK_N];
  float rkf[RK_N];
  float rkl[RK_N];
  bool f16_sr;           // FP16 storage: stochastic rounding of stores (else nearest)
  // Per direction I, in elements: doff = I * S (the population's storage
  // offset) and poff = doff - L.off(e_I) (the plain pull's source), kernel
  // parameters so that no thread forms them with 64-bit products.
  long long doff[27];
  long long poff[27];
  int ref_override;      // reference profiles: inlet u at x = 0, p = 0 at x = nx-1
  const double *inlet_u; // ny*nz inlet velocity profile (reference profiles)
  const float *alpha;    // nx*ny*nz Brinkman porosity or null
  double *mu, *mv, *mw, *mp;  // macroscopic output (interior, x fastest) or null
  // Channel profile (boundaries resolved inside the sweep):
  int wall_y, wall_z;
  double f_in[27];       // inlet equilibrium populations (p = 0, u = (u_in, 0, 0))
  float f_in_f[27];      // the same in FP32 (FP32-arithmetic sweeps)
  float f_in_l[27];      // f_in - f_in_f in FP32 (double-float sweeps)
  const unsigned char *tile_slow;  // per warp tile (32 cells of a row): 1 = next to a solid
  const int *slow_tiles; // list of tiles next to solids (tile = (z*ny + y)*nxw + x/32)
  const int *tile_index; // per warp tile: its position in slow_tiles, -1 if not listed
  int n_slow;            // length of the list
  const long long *bcell_idx;  // boundary cells (fluid, solid links): storage index
  const unsigned *bcell_links; // and link word of each, in tile and x order
  int n_bcells;                // their number
  const unsigned *links_bits;  // per listed tile, 32 cells: bit i = source of i is solid,
                               // bit 31 = the cell is solid
  const long long *face_off;   // [16][Q] listed-tile pull offsets per face state
  const unsigned *face_bb;     // [16] directions bouncing back at a no-slip face
  double *partials;      // 3 doubles per block of the force kernel
  unsigned int *counter; // finished force blocks (self-resetting)
  double *hist;          // force history, 3 doubles per step
  long long *step;       // device step counter (history slot = step % cap)
  long long cap;
  int bnd_blocks;        // grid of the force launch (at most one block per SM)
  int sms;               // multiprocessors of the device
  int lines;             // 1: the interior runs the line-staged sweep (sweep_lines.cuh)
  unsigned *err;         // device error word of the handle (a bounded wait gave up)
};

struct FillArgs {
  Layout L;
  void *f;               // state being filled (in place)
  void *f2;              // the other buffer: face passes write their ghosts here too (or null)
  const uint32_t *mask;
  int nxw;
  int wall_y, wall_z;
  const void *f_in;      // inlet equilibrium, Q stored elements (channel profile)
};

struct FaceOp {
  int kind;  // 0 copy (inlet), 1 extrapolate (outlet), 2 bounce (wall)
  int axis;  // 0 x, 1 y, 2 z
  int side;  // 0 low, 1 high
  int trim;  // 1: the pass skips the two ghost ends of its tangential range
  int ndir;  // the populations the pass writes (filled by launch_face_ops),
  unsigned long long dirs;  // 5 bits each, the k-th at bit 5k
};

struct LinkArgs {
  Layout L;
  void *f;
  const int4 *links;     // (x, y, z, k): solid cell s, direction k, s + e_k fluid
  long long n;
  int reach;             // 1: halfway bounce-back, 2: the reference's s + 2 e_k rule
  double *partials;      // 3 doubles per block
  unsigned int *counter; // last-block detection, self-resetting
  double *hist;          // force history, 3 doubles per slot
  long long *step;       // device step counter (history slot = step % cap)
  long long cap;
};

struct ReduceArgs {
  Layout L;
  const void *f;
  const uint32_t *mask;
  int nxw;
  double *partials;      // 4 doubles per block
  unsigned int *counter;
  double *out;           // 4 doubles: mass, momentum x, y, z
};

// ---- launchers (defined in the .cu files, dispatch on lattice and storage) ----
cudaError_t launch_sweep(int Q, int store, int compute, const SweepArgs &a, cudaStream_t s);
// Fork/join of the two launches of a channel step: the force kernel runs on
// `side` while the sweep runs on the main stream (the force kernel only reads
// the state the sweep reads), joined before anything that follows.
struct SweepFork {
  cudaStream_t side;
  cudaEvent_t fork, join;
};
// u, v, w, p of the step that read a.fa (channel profile), into a.mu..a.mp.
cudaError_t launch_macros_channel(int Q, int store, int compute, const SweepArgs &a,
                                  cudaStream_t s);
cudaError_t launch_sweep_channel(int Q, int store, int compute, const SweepArgs &a,
                                 cudaStream_t s, const SweepFork *fk = nullptr);
// Post-stream populations of the step that read a.fa (FP64, dense [i][z][y][x]);
// ref: plain pull (reference profiles), else the channel's resolved pull.
cudaError_t launch_stream_state(int Q, int store, const SweepArgs &a, bool ref, double *out,
                                cudaStream_t s);
// Launch shape of the sweeps: blocks of 32 x 4 cells, one z plane per grid z
// (the solid-tile launch runs 4 listed warp tiles per block).
constexpr int SWEEP_BX = 32, SWEEP_BY = 4;
cudaError_t launch_fill_channel(int Q, int store, const FillArgs &a, cudaStream_t s);
// Two face passes of one axis (independent of each other) in one launch.
cudaError_t launch_face_ops(int Q, int store, const FillArgs &a, FaceOp op0, FaceOp op1,
                            cudaStream_t s);
cudaError_t launch_ghost_copy(int Q, int store, const Layout &L, const void *src, void *dst,
                              cudaStream_t s);
cudaError_t launch_links(int Q, int store, const LinkArgs &a, int blocks, cudaStream_t s);
cudaError_t launch_init_macros(int Q, int store, const Layout &L, void *f, const double *u,
                               const double *v, const double *w, const double *p,
                               cudaStream_t s);
cudaError_t launch_init_channel(int Q, int store, const Layout &L, void *f,
                                const uint32_t *mask, int nxw, double u_in, double amp,
                                unsigned long long seed, const float *alpha, double omega,
                                double *mu, double *mv, double *mw, double *mp, cudaStream_t s);
cudaError_t launch_reduce_mass(int Q, int store, const ReduceArgs &a, int blocks,
                               cudaStream_t s);
cudaError_t launch_get_f(int Q, int store, const Layout &L, const void *f, double *out,
                         cudaStream_t s);
cudaError_t launch_set_f(int Q, int store, const Layout &L, void *f, const double *in,
                         cudaStream_t s);
cudaError_t launch_fill_value(int Q, int store, const Layout &L, void *f, cudaStream_t s);

// Fill omega, omega_f and the relaxation constants rk/rkf/rkl of a sweep for
// lattice Q (any storage kind `store`: the codecs hand the arithmetic the
// populations themselves).
void set_relax(SweepArgs &a, int Q, int store, double omega);
// Fill doff/poff of a sweep from its layout a.L.
void set_offsets(SweepArgs &a, int Q);

// Line-staged sweep (lines.cu): whether it covers a handle's form, its one-time
// set-up (shared-memory opt-in) and its launch.
bool lines_supported(int Q, int store, int layout_rows, bool alpha, int nx);
cudaError_t lines_prepare();
cudaError_t launch_lines_f16_q27(const SweepArgs &a, int sms, cudaStream_t s);
cudaError_t launch_wait_timeout_probe(unsigned *err, long long polls, cudaStream_t s);

// Number of kernel launches issued through the launchers (all handles).
long long launches();
void count_launch(long long n = 1);

// Perturbation of the initial u_y: amp * (2 r - 1), r from splitmix64 of
// (seed + cell * golden ratio constant), 53 bits.
__host__ __device__ inline unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}
__host__ __device__ inline double perturbation(unsigned long long seed, long long cell,
                                               double amp) {
  unsigned long long r = splitmix64(seed + (unsigned long long)cell * 0x9E3779B97F4A7C15ULL);
  double u01 = (double)(r >> 11) * (1.0 / 9007199254740992.0);
  return amp * (2.0 * u01 - 1.0);
}

}  // namespace cflbm
