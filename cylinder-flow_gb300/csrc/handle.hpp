// Internal handle state and host-side helpers shared by the C ABI sources.
#pragma once
#include <algorithm>
#include <cstdint>
#include <string>
#include <thread>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/cflbm.h"
#include "solver.cuh"

struct cflbm_handle {
  cflbm_config cfg{};
  int Q = 9;
  cflbm::Layout L{};
  int nxw = 0;
  int esize = 8;
  cudaStream_t stream = nullptr;
  int sms = 1;  // multiprocessors of the device
  cflbm::SweepFork fork{nullptr, nullptr, nullptr};  // channel sweep: side stream + events
  void *fA = nullptr, *fB = nullptr;
  size_t f_bytes = 0;
  uint32_t *d_mask = nullptr;
  unsigned *d_links_bits = nullptr;  // link bits of the tiles next to solids
  unsigned char *d_tile_slow = nullptr;  // per warp tile: listed (face row or next to a solid)
  int *d_slow_tiles = nullptr;           // list of those tiles
  int *d_tile_index = nullptr;           // per warp tile: position in that list or -1
  long long *d_bcell_idx = nullptr;  // boundary cells (fluid, solid links): storage index
  unsigned *d_bcell_links = nullptr;  // and link word of each, in tile and x order
  int n_bcells = 0;                   // their number
  long long *d_face_off = nullptr;       // listed-tile pull offsets per face state
  unsigned *d_face_bb = nullptr;         // no-slip face bounce-back bits per face state
  // Channel profile: the steps do not write u, v, w, p; the fields of the last
  // step are formed on request from the state it read (fB after the step).
  bool macros_pending = false;
  int n_slow = 0;
  double f_in[27] = {0};        // inlet equilibrium (channel profile)
  int4 *d_links = nullptr;
  long long n_links = 0;
  long long n_solid = 0;
  double *d_mu = nullptr, *d_mv = nullptr, *d_mw = nullptr, *d_mp = nullptr;
  double *d_inlet = nullptr;
  float *d_alpha = nullptr;
  void *d_fin = nullptr;
  double *d_hist = nullptr;
  long long hist_cap = 0;
  long long *d_step = nullptr;
  double *d_partials = nullptr;
  int link_blocks = 1;
  int reduce_blocks = 1;
  unsigned int *d_counter = nullptr;   // links kernel
  unsigned int *d_counter2 = nullptr;  // mass kernel
  double *d_sums = nullptr;            // 4 doubles (mass, momentum)
  unsigned *d_err = nullptr;           // device error word (a bounded wait gave up)
  bool lines = false;                  // the interior runs the line-staged sweep
  long long steps_done = 0;
  double omega = 1.0;
  double area = 1.0;  // Cd/Cl reference area
  size_t device_bytes = 0;
  // Kernel timing (cflbm_set_timing): event pairs around sweeps / boundary phases.
  // CUDA graphs of GRAPH_STEPS steps, one per A/B parity (buf[0] = A at create).
  void *buf[2] = {nullptr, nullptr};
  cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
  long long launches_per_step = 0;
  bool timing = false;
  bool batched = false;            // owned and stepped by a cflbm_batch
  cudaEvent_t ev_sync = nullptr;   // orders this handle's stream before a batch step
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<size_t, size_t>> sweep_ev, bnd_ev;
};

namespace cflbm {

// Host-side set-up of the reference profiles (reference_setup.cpp).
struct RefSetup {
  std::vector<uint8_t> solid;  // interior mask, x fastest
  std::vector<double> u, v, w, p;  // ghosted box, x fastest
  std::vector<double> inlet;   // ny*nz inlet override profile
  double area = 1.0;
};
int ref2d_setup(int nx, int ny, double u0, const int32_t *ran, RefSetup &out);
int ref3d_setup(int nx, int ny, int nz, double u0, const int32_t *ran, RefSetup &out);
int ref2ds_setup(int nx, int ny, double u0, const int32_t *ran, RefSetup &out);

// Cd/Cl reference area of a channel's body (reference_setup.cpp).
double channel_area(const cflbm_config &c);

// Channel-sweep arguments of a handle (api.cu).
SweepArgs channel_args(const cflbm_handle *h, const void *fa, void *fb, bool write_macros);

// Tecplot binary writer (tecplot.cpp).
int write_tecplot(const char *path, int dim, int nx, int ny, int nz, const double *u,
                  const double *v, const double *w, const double *p, int n);

// Run body(r) for r in [0, n) on the host's cores (rows are independent).
template <class F>
void host_parallel_rows(long long n, F body) {
  const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  const long long nt = std::min<long long>(hw, std::max<long long>(1, n / 64));
  if (nt <= 1) {
    for (long long r = 0; r < n; ++r) body(r);
    return;
  }
  std::vector<std::thread> pool;
  for (long long t = 0; t < nt; ++t)
    pool.emplace_back([=, &body] {
      for (long long r = t; r < n; r += nt) body(r);
    });
  for (auto &th : pool) th.join();
}

}  // namespace cflbm
