// Batched channels: many independent channel instances of uneven size and
// Reynolds number advanced together, one work-list launch per sweep kind per
// step over all instances, replayed from a captured CUDA graph, with the launch
// shape (tile height; one interior item per block or a persistent grid size)
// picked by a timing autotuner at creation.
//
// Each instance is an ordinary channel-profile handle (its own buffers, mask,
// solid-tile list, force history), so every per-instance result call of the C ABI
// works on cflbm_batch_handle(b, k).  The batch adds:
//   * a device table of per-instance sweep arguments, one per A/B parity and
//     macro flag;
//   * a work list of (instance, tile block) items for the interior launch, each
//     carrying its warp tiles' unlisted flags, and one for the solid-tile launch
//     (blocks of `by` listed tiles of one instance);
//   * the interior kernels (one item per block, or a persistent grid walking
//     contiguous ranges of items) and the persistent solid kernel, running the
//     same per-cell code as the single-channel sweep (channel2_cells,
//     pull_resolved, moments, finish_cell); the solid kernel reduces each
//     instance's body force into that instance's history, the last block of the
//     instance summing its partials in block order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#include "handle.hpp"
#include "sweep.cuh"

namespace cflbm {
int record_error(int code, const char *msg);
}

using namespace cflbm;

struct cflbm_batch {
  std::vector<cflbm_handle *> inst;
  int Q = 9, storage = 0, compute = 1;
  cudaStream_t stream = nullptr;
  int device = 0;
  SweepArgs *d_args = nullptr;       // [inst][parity][macros]
  int4 *d_work_fast[4] = {nullptr};  // per tile height candidate index
  int4 *d_work_solid[4] = {nullptr};
  int n_work_fast[4] = {0}, n_work_solid[4] = {0};
  int by = 4;            // tuned tile height
  int grid = 0;          // tuned persistent grid size
  int sms = 152;
  int graph_steps = 100;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // per parity
  int parity = 0;        // 0: every instance reads buf[0]
  long long steps_done = 0;
  long long cells = 0;
  double bytes_per_cell = 0;
  cudaEvent_t done = nullptr;
  cflbm::SweepFork fork{nullptr, nullptr, nullptr};  // solid-work kernel beside the fast one
  std::vector<double> tune_ms;  // timing of each candidate (for cflbm_batch_info)
};

namespace {

constexpr int BY_CANDIDATES[4] = {1, 2, 4, 8};

int bfail(int code, const std::string &msg) { return record_error(code, msg.c_str()); }

#define BCK(call)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return bfail(CFLBM_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));    \
  } while (0)

// Fast items (unlisted tiles) run two cells per thread with packed FP32x2
// arithmetic (channel2_cells: cells x and x + 32 of a row, items 64 cells wide);
// solid items (tiles next to a body or on a wall row) one cell per thread.
template <int Q, class ST, class A, int BY, bool SOLID>
__global__ void __launch_bounds__(32 * BY, SOLID ? 16 / BY + 1 : 24 / BY)
    batch_sweep_kernel(const SweepArgs *__restrict__ args, const int4 *__restrict__ work,
                       int n_work, int sel) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  __shared__ SweepArgs a;
  const int lane = threadIdx.x, wid = threadIdx.y, tid = wid * 32 + lane;
  // Each block takes a contiguous range of work items (items are ordered by
  // instance, then z, y, x), so the instance's arguments are staged in shared
  // memory only when the range crosses into the next instance.
  // The next item is loaded one iteration ahead, so an item's population loads
  // wait for nothing else.
  const int w0 = (int)((long long)blockIdx.x * n_work / gridDim.x);
  const int w1 = (int)((long long)(blockIdx.x + 1) * n_work / gridDim.x);
  int staged = -1;
  int4 wn = w0 < w1 ? work[w0] : make_int4(0, 0, 0, 0);
  for (int w = w0; w < w1; ++w) {
    // (instance, x pair | row flags << 16, y tile, z) for fast items,
    // (instance, 0, listed block, 0) for solid items
    const int4 wk = wn;
    if (w + 1 < w1) wn = work[w + 1];
    if (wk.x != staged) {     // block-uniform
      __syncthreads();
      const int *src = reinterpret_cast<const int *>(args + 4 * (long long)wk.x + sel);
      int *dst = reinterpret_cast<int *>(&a);
      for (int k = tid; k < (int)(sizeof(SweepArgs) / sizeof(int)); k += 32 * BY) dst[k] = src[k];
      __syncthreads();
      staged = wk.x;
    }
    const int nx = a.L.nx, ny = a.L.ny;
    int x = 0, y = 0, z = 0;
    bool active = false;
    long long t = 0;
    if constexpr (SOLID) {
      t = (long long)wk.z * BY + wid;
      active = t < a.n_slow;
      const int tile = active ? a.slow_tiles[t] : 0;
      const int row = tile / a.nxw;
      y = row % ny;
      z = row / ny;
      x = (tile % a.nxw) * 32 + lane;
    } else {
      // Bits 2r and 2r + 1 of the row flags: warp tiles 2 * pair and 2 * pair + 1
      // of row r of the item are unlisted (and inside the box).
      y = wk.z * BY + wid;
      z = wk.w;
      const int pair = wk.y & 0xffff;
      const unsigned rf = ((unsigned)wk.y >> 16) >> (2 * wid);
      const bool act0 = rf & 1u, act1 = (rf >> 1) & 1u;
      if (act0 || act1)  // warp-uniform
        channel2_cells<Q, ST, float2, false, false>(a, 64 * pair + lane, y, z, act0, act1);
      continue;
    }
    double Fx = 0.0, Fy = 0.0, Fz = 0.0;
    if (active) {  // warp-uniform
      const bool valid = x < nx;
      if (!valid) x = nx - 1;
      const long long S = a.L.S;
      const long long c = a.L.idx(x, y, z);
      const E *__restrict__ fa = static_cast<const E *>(a.fa);
      E *__restrict__ fb = static_cast<E *>(a.fb);
      A f[Q];
      bool solid_here = false;
      A Fxa = A(0), Fya = A(0), Fza = A(0);
      if constexpr (SOLID) {
        const unsigned links = a.links_bits[t * 32 + lane];
        solid_here = mask_solid(a.mask, a.nxw, ny, x, y, z);
        static_for(
            [&](auto ic) {
              constexpr int I = decltype(ic)::value;
              f[I] = pull_resolved<Q, ST, A, I>(fa, c, S, x, y, z, links, a);
            },
            std::make_integer_sequence<int, Q>{});
        if (valid && !solid_here) cell_force<Q, A, SF>(f, links, Fxa, Fya, Fza);
        Fx = f2d_bits(Fxa);
        Fy = f2d_bits(Fya);
        Fz = f2d_bits(Fza);
      } else {
        static_for(
            [&](auto ic) {
              constexpr int I = decltype(ic)::value;
              f[I] = pull_plain<Q, ST, A, I>(fa, c, S, x, a);
            },
            std::make_integer_sequence<int, Q>{});
      }
      A rho3, ux, uy, uz;
      moments<L, A, SF>(f, rho3, ux, uy, uz);
      if (solid_here) {
        rho3 = A(0); ux = A(0); uy = A(0); uz = A(0);
      }
      const long long cell = ((long long)z * ny + y) * nx + x;
      finish_cell<L, SF, A, E>(f, rho3, ux, uy, uz, cell, valid, fb, c, S, a);
    }
    if constexpr (SOLID) {
      __shared__ double sh[3][BY];
      __shared__ bool last;
      for (int o = 16; o > 0; o >>= 1) {
        Fx += __shfl_down_sync(0xffffffffu, Fx, o);
        Fy += __shfl_down_sync(0xffffffffu, Fy, o);
        Fz += __shfl_down_sync(0xffffffffu, Fz, o);
      }
      if (lane == 0) {
        sh[0][wid] = Fx;
        sh[1][wid] = Fy;
        sh[2][wid] = Fz;
      }
      __syncthreads();
      const int nblk = a.n_slow > 0 ? (a.n_slow + BY - 1) / BY : 1;
      if (tid == 0) {
        double bx = 0.0, byy = 0.0, bz = 0.0;
        for (int q = 0; q < BY; ++q) { bx += sh[0][q]; byy += sh[1][q]; bz += sh[2][q]; }
        a.partials[3 * wk.z] = bx;
        a.partials[3 * wk.z + 1] = byy;
        a.partials[3 * wk.z + 2] = bz;
        __threadfence();
        last = atomicAdd(a.counter, 1u) == (unsigned)(nblk - 1);
      }
      __syncthreads();
      if (last && tid == 0) {
        __threadfence();
        const volatile double *p = a.partials;
        double tx = 0.0, ty = 0.0, tz = 0.0;
        for (int k = 0; k < nblk; ++k) { tx += p[3 * k]; ty += p[3 * k + 1]; tz += p[3 * k + 2]; }
        const long long st = *a.step;
        double *h = a.hist + 3 * (st % a.cap);
        h[0] = tx;
        h[1] = ty;
        h[2] = tz;
        *a.step = st + 1;
        *a.counter = 0u;
      }
    }
  }
}

// Fast items, one per block: the block reads its item and its instance's
// arguments straight from global memory (cached in L1; no shared-memory staging
// and no barrier), and the hardware scheduler keeps the SMs full.  The launch
// is latency-bound, so it is held to 48 registers (40 warps per SM, no spill);
// measured on the 64-channel problem: 0.889 of the copy peak against 0.822 at
// 59 registers and 0.881 at 40 registers (a 24-byte spill).
template <int Q, class ST, int BY, int MINB = 40 / BY>
__global__ void __launch_bounds__(32 * BY, MINB)
    batch_fast_kernel(const SweepArgs *__restrict__ args, const int4 *__restrict__ work, int sel) {
  const int4 wk = work[blockIdx.x];  // (instance, x pair | row flags << 16, y tile, z)
  const SweepArgs &a = args[4 * (long long)wk.x + sel];
  const int wid = threadIdx.y;
  const unsigned rf = ((unsigned)wk.y >> 16) >> (2 * wid);
  const bool act0 = rf & 1u, act1 = (rf >> 1) & 1u;
  if (act0 || act1)  // warp-uniform
    channel2_cells<Q, ST, float2, false, false>(a, 64 * (wk.y & 0xffff) + threadIdx.x,
                                                wk.z * BY + wid, wk.w, act0, act1);
}

// grid > 0: persistent grids of `grid` blocks for both kinds of work; grid = 0:
// one fast item per block, and the solid work on 8 warps per SM.
template <int Q, class ST, int BY>
cudaError_t launch_batch_t(const cflbm_batch *b, int kind, int sel, int grid, cudaStream_t s) {
  const int ci = BY == 1 ? 0 : BY == 2 ? 1 : BY == 4 ? 2 : 3;
  dim3 block(32, BY, 1);
  if (kind == 0) {
    if (b->n_work_fast[ci] > 0) {
      if (grid > 0)
        batch_sweep_kernel<Q, ST, float, BY, false>
            <<<std::min(grid, b->n_work_fast[ci]), block, 0, s>>>(b->d_args, b->d_work_fast[ci],
                                                                  b->n_work_fast[ci], sel);
      else
        batch_fast_kernel<Q, ST, BY><<<b->n_work_fast[ci], block, 0, s>>>(
            b->d_args, b->d_work_fast[ci], sel);
    }
  } else {
    // Beside one-item-per-block interior launches: 8 solid warps per SM
    // (64-channel problem, tile height 2: 0.889 of the copy peak at 4 blocks
    // per SM against 0.769 at 2; tile height 4: 0.880 at 2 blocks per SM).
    const int g = grid > 0 ? grid : std::max(1, 8 / BY) * b->sms;
    batch_sweep_kernel<Q, ST, float, BY, true>
        <<<std::max(1, std::min(g, b->n_work_solid[ci])), block, 0, s>>>(
            b->d_args, b->d_work_solid[ci], b->n_work_solid[ci], sel);
  }
  count_launch();
  return cudaGetLastError();
}

template <int Q, class ST>
cudaError_t launch_batch_st(const cflbm_batch *b, int by, int kind, int sel, int grid,
                            cudaStream_t s) {
  switch (by) {
    case 1: return launch_batch_t<Q, ST, 1>(b, kind, sel, grid, s);
    case 2: return launch_batch_t<Q, ST, 2>(b, kind, sel, grid, s);
    case 4: return launch_batch_t<Q, ST, 4>(b, kind, sel, grid, s);
    default: return launch_batch_t<Q, ST, 8>(b, kind, sel, grid, s);
  }
}

cudaError_t launch_batch(const cflbm_batch *b, int by, int kind, int sel, int grid,
                         cudaStream_t s) {
  if (b->Q == 9) {
    if (b->storage == CFLBM_STORE_FP64) return launch_batch_st<9, double>(b, by, kind, sel, grid, s);
    if (b->storage == CFLBM_STORE_FP32) return launch_batch_st<9, float>(b, by, kind, sel, grid, s);
    return launch_batch_st<9, F16Dev>(b, by, kind, sel, grid, s);
  }
  if (b->storage == CFLBM_STORE_FP64) return launch_batch_st<27, double>(b, by, kind, sel, grid, s);
  if (b->storage == CFLBM_STORE_FP32) return launch_batch_st<27, float>(b, by, kind, sel, grid, s);
  return launch_batch_st<27, F16Dev>(b, by, kind, sel, grid, s);
}

// One batch step: both launches, reading buffer `parity` of every instance.  The
// solid-work kernel (tiles next to a body or on a wall row; latency-bound, with
// the force reduction) runs on the higher-priority side stream beside the fast
// kernel; the two write disjoint cells.
int batch_one_step(cflbm_batch *b, int by, int grid, bool macros, bool swap) {
  const int sel = b->parity * 2 + (macros ? 1 : 0);
  BCK(cudaEventRecord(b->fork.fork, b->stream));
  BCK(cudaStreamWaitEvent(b->fork.side, b->fork.fork, 0));
  BCK(launch_batch(b, by, 1, sel, grid, b->fork.side));
  BCK(cudaEventRecord(b->fork.join, b->fork.side));
  BCK(launch_batch(b, by, 0, sel, grid, b->stream));
  BCK(cudaStreamWaitEvent(b->stream, b->fork.join, 0));
  if (swap) {
    b->parity ^= 1;
    ++b->steps_done;
  }
  return CFLBM_OK;
}

void free_batch(cflbm_batch *b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto g : b->graph)
    if (g) cudaGraphExecDestroy(g);
  if (b->d_args) cudaFree(b->d_args);
  for (int k = 0; k < 4; ++k) {
    if (b->d_work_fast[k]) cudaFree(b->d_work_fast[k]);
    if (b->d_work_solid[k]) cudaFree(b->d_work_solid[k]);
  }
  if (b->done) cudaEventDestroy(b->done);
  if (b->fork.side) cudaStreamSynchronize(b->fork.side);
  if (b->fork.fork) cudaEventDestroy(b->fork.fork);
  if (b->fork.join) cudaEventDestroy(b->fork.join);
  if (b->fork.side) cudaStreamDestroy(b->fork.side);
  for (auto *h : b->inst) cflbm_destroy(h);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Make every instance handle's stream wait for the batch's work so far.
int publish(cflbm_batch *b) {
  BCK(cudaEventRecord(b->done, b->stream));
  for (auto *h : b->inst) BCK(cudaStreamWaitEvent(h->stream, b->done, 0));
  return CFLBM_OK;
}

}  // namespace

extern "C" {

int cflbm_batch_options_default(cflbm_batch_options *o) {
  if (!o) return bfail(CFLBM_E_INVALID, "options is NULL");
  std::memset(o, 0, sizeof(*o));
  o->graph_steps = 100;
  o->autotune = 1;
  o->tile_height = 4;
  o->blocks_per_sm = 8;
  return CFLBM_OK;
}

int cflbm_batch_create(const cflbm_config *cfgs, int n, const cflbm_batch_options *opt,
                       cflbm_batch **out) {
  if (!cfgs || n <= 0 || !out) return bfail(CFLBM_E_INVALID, "need configs, n > 0 and out");
  *out = nullptr;
  cflbm_batch_options o;
  if (opt) o = *opt; else cflbm_batch_options_default(&o);
  if (o.graph_steps < 2 || (o.graph_steps & 1))
    return bfail(CFLBM_E_INVALID, "graph_steps must be even and >= 2");
  for (int k = 0; k < n; ++k) {
    if (cfgs[k].profile != CFLBM_PROFILE_CHANNEL)
      return bfail(CFLBM_E_INVALID, "batched instances must use the CHANNEL profile");
    if (cfgs[k].lattice != cfgs[0].lattice || cfgs[k].storage != cfgs[0].storage ||
        cfgs[k].compute != CFLBM_COMPUTE_FP32 || cfgs[k].device != cfgs[0].device)
      return bfail(CFLBM_E_INVALID,
                   "batched instances need one lattice, one storage, FP32 arithmetic, one device");
  }
  std::unique_ptr<cflbm_batch, void (*)(cflbm_batch *)> bp(new cflbm_batch(), free_batch);
  cflbm_batch *b = bp.get();
  b->Q = cfgs[0].lattice;
  b->storage = cfgs[0].storage;
  b->device = cfgs[0].device;
  b->graph_steps = o.graph_steps;
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BCK(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
  {
    int lo = 0, hi = 0;
    BCK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    BCK(cudaStreamCreateWithPriority(&b->fork.side, cudaStreamNonBlocking, hi));
    BCK(cudaEventCreateWithFlags(&b->fork.fork, cudaEventDisableTiming));
    BCK(cudaEventCreateWithFlags(&b->fork.join, cudaEventDisableTiming));
  }
  int sms = 0;
  BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
  b->sms = sms;
  for (int k = 0; k < n; ++k) {
    cflbm_handle *h = nullptr;
    int rc = cflbm_create(&cfgs[k], &h);
    if (rc) return rc;
    h->batched = true;
    b->inst.push_back(h);
    b->cells += (long long)h->L.nx * h->L.ny * h->L.nz;
  }
  const int es = b->storage == CFLBM_STORE_FP64 ? 8 : b->storage == CFLBM_STORE_FP32 ? 4 : 2;
  b->bytes_per_cell = 2.0 * b->Q * es + 0.125;
  // Per-instance arguments: [parity][macros].
  std::vector<SweepArgs> args((size_t)n * 4);
  for (int k = 0; k < n; ++k) {
    cflbm_handle *h = b->inst[k];
    for (int par = 0; par < 2; ++par)
      for (int m = 0; m < 2; ++m)
        args[(size_t)k * 4 + par * 2 + m] =
            channel_args(h, h->buf[par], h->buf[par ^ 1], m == 1);
  }
  BCK(cudaMalloc(&b->d_args, args.size() * sizeof(SweepArgs)));
  BCK(cudaMemcpy(b->d_args, args.data(), args.size() * sizeof(SweepArgs), cudaMemcpyHostToDevice));
  // Per-tile listed flags of every instance, read back once.
  std::vector<std::vector<unsigned char>> slow(n);
  for (int k = 0; k < n; ++k) {
    const cflbm_handle *h = b->inst[k];
    slow[k].resize((size_t)h->nxw * h->L.ny * h->L.nz);
    BCK(cudaMemcpy(slow[k].data(), h->d_tile_slow, slow[k].size(), cudaMemcpyDeviceToHost));
  }
  // Work lists per tile-height candidate.
  for (int ci = 0; ci < 4; ++ci) {
    const int by = BY_CANDIDATES[ci];
    std::vector<int4> wf, ws;
    for (int k = 0; k < n; ++k) {
      const cflbm_handle *h = b->inst[k];
      const int gx = (h->nxw + 1) / 2, gy = (h->L.ny + by - 1) / by;  // 64-cell items
      const int nxw = h->nxw, ny = h->L.ny;
      // Items carry the unlisted flags of their warp tiles (two per row), so
      // the kernel reads no per-tile flag; items with no unlisted tile are left out.
      for (int z = 0; z < h->L.nz; ++z)
        for (int yb = 0; yb < gy; ++yb)
          for (int xb = 0; xb < gx; ++xb) {
            unsigned rf = 0;
            for (int r = 0; r < by; ++r) {
              const int y = yb * by + r;
              if (y >= ny) break;
              const size_t row = ((size_t)z * ny + y) * nxw;
              if (!slow[k][row + 2 * xb]) rf |= 1u << (2 * r);
              if (2 * xb + 1 < nxw && !slow[k][row + 2 * xb + 1]) rf |= 2u << (2 * r);
            }
            if (rf) wf.push_back(make_int4(k, xb | (int)(rf << 16), yb, z));
          }
      const int nb = (h->n_slow + by - 1) / by;
      for (int q = 0; q < std::max(nb, 1); ++q) ws.push_back(make_int4(k, 0, q, 0));  // .z = listed block
    }
    b->n_work_fast[ci] = (int)wf.size();
    b->n_work_solid[ci] = (int)ws.size();
    BCK(cudaMalloc(&b->d_work_fast[ci], wf.size() * sizeof(int4)));
    BCK(cudaMalloc(&b->d_work_solid[ci], ws.size() * sizeof(int4)));
    BCK(cudaMemcpy(b->d_work_fast[ci], wf.data(), wf.size() * sizeof(int4), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->d_work_solid[ci], ws.data(), ws.size() * sizeof(int4), cudaMemcpyHostToDevice));
  }
  // Launch shape: the autotuner times every (tile height, blocks per SM) pair on
  // the real state without advancing it (A -> B, no swap), then restores the
  // force-history counters.
  b->by = o.tile_height;
  b->grid = std::max(0, o.blocks_per_sm) * sms;
  if (o.autotune) {
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int ci = 0; ci < 4; ++ci)
      for (int bps : {0, 2, 3, 4, 6, 8, 12, 16}) {  // 0: one fast item per block
        const int by = BY_CANDIDATES[ci];
        if (32 * by * bps > 2048) continue;
        const int grid = bps * sms;
        int rc = batch_one_step(b, by, grid, false, false);
        if (rc) return rc;
        BCK(cudaEventRecord(e0, b->stream));
        for (int r = 0; r < 5 && rc == CFLBM_OK; ++r) rc = batch_one_step(b, by, grid, false, false);
        if (rc) return rc;
        BCK(cudaEventRecord(e1, b->stream));
        BCK(cudaEventSynchronize(e1));
        float ms = 0.f;
        BCK(cudaEventElapsedTime(&ms, e0, e1));
        b->tune_ms.push_back(ms / 5.0f);
        if (ms < best) {
          best = ms;
          b->by = by;
          b->grid = grid;
        }
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (auto *h : b->inst) {
      BCK(cudaMemsetAsync(h->d_step, 0, sizeof(long long), b->stream));
      BCK(cudaMemsetAsync(h->d_hist, 0, 3 * sizeof(double) * h->hist_cap, b->stream));
    }
    BCK(cudaStreamSynchronize(b->stream));
  }
  *out = bp.release();
  return CFLBM_OK;
}

int cflbm_batch_destroy(cflbm_batch *b) {
  free_batch(b);
  return CFLBM_OK;
}

int cflbm_batch_step(cflbm_batch *b, int nsteps) {
  if (!b || nsteps < 0) return bfail(CFLBM_E_INVALID, "bad arguments");
  BCK(cudaSetDevice(b->device));
  // Every instance handle's own stream must be idle-ordered before the batch
  // writes its buffers.
  for (auto *h : b->inst) {
    BCK(cudaEventRecord(h->ev_sync, h->stream));
    BCK(cudaStreamWaitEvent(b->stream, h->ev_sync, 0));
  }
  int left = nsteps;
  while (left > b->graph_steps) {
    if (!b->graph[b->parity]) {
      const int par = b->parity;
      cudaGraph_t g = nullptr;
      BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      int rc = CFLBM_OK;
      for (int s = 0; s < b->graph_steps && rc == CFLBM_OK; ++s)
        rc = batch_one_step(b, b->by, b->grid, false, true);
      cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      BCK(ec);
      cudaError_t ei = cudaGraphInstantiate(&b->graph[par], g, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(g);
      BCK(ei);
      b->parity = par;  // capture walked the parity through an even number of steps
      b->steps_done -= b->graph_steps;
    }
    BCK(cudaGraphLaunch(b->graph[b->parity], b->stream));
    count_launch(2LL * b->graph_steps);
    b->steps_done += b->graph_steps;
    left -= b->graph_steps;
  }
  for (int s = 0; s < left; ++s) {
    int rc = batch_one_step(b, b->by, b->grid, s == left - 1, true);
    if (rc) return rc;
  }
  // Keep the instance handles' host state in step with the device.
  for (auto *h : b->inst) {
    h->fA = h->buf[b->parity];
    h->fB = h->buf[b->parity ^ 1];
    h->steps_done = b->steps_done;
  }
  return publish(b);
}

int cflbm_batch_synchronize(cflbm_batch *b) {
  if (!b) return bfail(CFLBM_E_INVALID, "batch is NULL");
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamSynchronize(b->stream));
  return CFLBM_OK;
}

cflbm_handle *cflbm_batch_handle(cflbm_batch *b, int k) {
  if (!b || k < 0 || k >= (int)b->inst.size()) {
    bfail(CFLBM_E_INVALID, "instance index out of range");
    return nullptr;
  }
  return b->inst[k];
}

int cflbm_batch_get_info(cflbm_batch *b, cflbm_batch_info *info) {
  if (!b || !info) return bfail(CFLBM_E_INVALID, "bad arguments");
  std::memset(info, 0, sizeof(*info));
  info->instances = (int)b->inst.size();
  info->cells = b->cells;
  info->steps_done = b->steps_done;
  info->tile_height = b->by;
  info->grid_blocks = b->grid;
  info->graph_steps = b->graph_steps;
  info->bytes_per_cell_step = b->bytes_per_cell;
  info->tuned_candidates = (int)b->tune_ms.size();
  double best = 0;
  for (double t : b->tune_ms) best = (best == 0 || t < best) ? t : best;
  info->tuned_step_ms = best;
  return CFLBM_OK;
}

}  // extern "C"
