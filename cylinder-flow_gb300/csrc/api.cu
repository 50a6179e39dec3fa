// C ABI of the solver (include/cflbm.h): handle life cycle and the step loop.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>
#include "handle.hpp"
#include "setup.cuh"

using namespace cflbm;

namespace {

// Steps per captured CUDA graph (even: A/B parity is preserved by a replay).
constexpr int GRAPH_STEPS = 64;

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define CK_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(CFLBM_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                  \
  } while (0)

int dev_alloc(cflbm_handle *h, void **p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(CFLBM_E_NOMEM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
  }
  h->device_bytes += bytes;
  return CFLBM_OK;
}

template <class T>
int dev_alloc_t(cflbm_handle *h, T **p, size_t count) {
  void *v = nullptr;
  int rc = dev_alloc(h, &v, count * sizeof(T));
  *p = static_cast<T *>(v);
  return rc;
}

void free_handle(cflbm_handle *h) {
  if (!h) return;
  if (h->cfg.device >= 0) cudaSetDevice(h->cfg.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  void *ptrs[] = {h->fA,    h->fB,     h->d_mask, h->d_links, h->d_mu,      h->d_mv,
                  h->d_links_bits, h->d_tile_slow, h->d_slow_tiles, h->d_tile_index,
                  h->d_face_off, h->d_face_bb, h->d_bcell_idx, h->d_bcell_links,
                  h->d_mw,  h->d_mp,   h->d_inlet, h->d_alpha, h->d_fin,    h->d_hist,
                  h->d_step, h->d_partials, h->d_counter, h->d_counter2, h->d_sums,
                  h->d_err};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  for (cudaGraphExec_t g : h->graph_exec)
    if (g) cudaGraphExecDestroy(g);
  if (h->ev_sync) cudaEventDestroy(h->ev_sync);
  if (h->fork.side) cudaStreamSynchronize(h->fork.side);
  if (h->fork.fork) cudaEventDestroy(h->fork.fork);
  if (h->fork.join) cudaEventDestroy(h->fork.join);
  if (h->fork.side) cudaStreamDestroy(h->fork.side);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int store_size(int storage) {
  return storage == CFLBM_STORE_FP64 ? 8 : storage == CFLBM_STORE_FP32 ? 4 : 2;
}

// Pack a host uint8 mask (x fastest) into 32-bit words per row.
std::vector<uint32_t> pack_mask(const std::vector<uint8_t> &solid, int nx, int ny, int nz,
                                int nxw) {
  std::vector<uint32_t> w((size_t)nxw * ny * nz, 0u);
  host_parallel_rows((long long)ny * nz, [&](long long r) {
    for (int x = 0; x < nx; ++x)
      if (solid[(size_t)r * nx + x]) w[(size_t)r * nxw + (x >> 5)] |= (1u << (x & 31));
  });
  return w;
}

template <int Q>
void build_links(const std::vector<uint8_t> &solid, int nx, int ny, int nz,
                 std::vector<int4> &links, long long &n_solid) {
  using L = Lat<Q>;
  // Rows in parallel, then concatenated in row order: the list order (z, y, x,
  // direction) fixes the order of the force sums over links.
  const long long rows = (long long)ny * nz;
  std::vector<std::vector<int4>> per(rows);
  std::vector<long long> nsol(rows, 0);
  host_parallel_rows(rows, [&](long long r) {
    const int y = (int)(r % ny), z = (int)(r / ny);
    for (int x = 0; x < nx; ++x) {
      if (!solid[(size_t)r * nx + x]) continue;
      ++nsol[r];
      for (int k = 1; k < Q; ++k) {
        const int X = x + L::ex(k), Y = y + L::ey(k), Z = z + L::ez(k);
        if (X < 0 || X >= nx || Y < 0 || Y >= ny || Z < 0 || Z >= nz) continue;
        if (solid[((size_t)Z * ny + Y) * nx + X]) continue;
        per[r].push_back(make_int4(x, y, z, k));
      }
    }
  });
  links.clear();
  n_solid = 0;
  size_t total = 0;
  for (long long r = 0; r < rows; ++r) total += per[r].size();
  links.reserve(total);
  for (long long r = 0; r < rows; ++r) {
    links.insert(links.end(), per[r].begin(), per[r].end());
    n_solid += nsol[r];
  }
}

// Pull tables of the listed tiles, one row per face state (bit 0: y = 0, bit 1:
// y = ny-1, bit 2: z = 0, bit 3: z = nz-1).  For every direction i: the source
// offset relative to the cell, population slot included, after the sweep's y/z
// face rules (periodic wrap; free-slip mirror: the same row and the mirrored
// population), and bit i of bb when a no-slip face bounces i back.  These are
// pull_resolved's face rules resolved once per state instead of per cell; the
// x rules (inlet, zero-gradient outlet) and solid links stay per cell.
template <int Q>
void face_tables(const Layout &Ly, int wall_y, int wall_z, std::vector<long long> &off,
                 std::vector<uint32_t> &bb) {
  using L = Lat<Q>;
  off.assign(16 * (size_t)Q, 0);
  bb.assign(16, 0u);
  for (int st = 0; st < 16; ++st)
    for (int i = 1; i < Q; ++i) {
      const int ex = L::ex(i), ey = L::ey(i), ez = L::ez(i);
      long long src = -Ly.off(ex, ey, ez);
      bool my = false, mz = false, b = false;
      if (ez != 0) {
        const bool out = ez > 0 ? (st & 4) : (st & 8);
        if (out && wall_z == CFLBM_WALL_PERIODIC) src += (ez > 0 ? 1LL : -1LL) * Ly.nz * Ly.zs;
        if (out && wall_z == CFLBM_WALL_FREESLIP) { mz = true; src += (long long)ez * Ly.zs; }
        if (out && wall_z == CFLBM_WALL_NOSLIP) b = true;
      }
      if (ey != 0) {
        const bool out = !b && (ey > 0 ? (st & 1) : (st & 2));
        if (out && wall_y == CFLBM_WALL_PERIODIC) src += (ey > 0 ? 1LL : -1LL) * Ly.ny * Ly.rs;
        if (out && wall_y == CFLBM_WALL_FREESLIP) { my = true; src += (long long)ey * Ly.rs; }
        if (out && wall_y == CFLBM_WALL_NOSLIP) b = true;
      }
      const int j = my ? (mz ? mirror<L>(mirror<L>(i, 1), 2) : mirror<L>(i, 1))
                       : (mz ? mirror<L>(i, 2) : i);
      off[(size_t)st * Q + i] = (long long)j * Ly.S + src;
      if (b) bb[st] |= 1u << i;
    }
}

// Equilibrium of the channel inlet (p = 0, u = (u_in, 0, 0)) in storage format
// (FP16: the deviation from the storage offset fbase, times F16_SCALE).
template <int Q>
std::vector<unsigned char> inlet_elements(double u_in, int storage, const float *fbase) {
  using L = Lat<Q>;
  std::vector<unsigned char> out((size_t)Q * store_size(storage));
  for (int i = 0; i < Q; ++i) {
    const double edu = L::ex(i) * u_in;
    const double feq = L::w(i) * 0.0 * 3.0 + L::w(i) * (3.0 * edu + 4.5 * edu * edu - 1.5 * u_in * u_in);
    if (storage == CFLBM_STORE_FP64) {
      std::memcpy(&out[8 * i], &feq, 8);
    } else if (storage == CFLBM_STORE_FP32) {
      const float v = (float)feq;
      std::memcpy(&out[4 * i], &v, 4);
    } else {
      const __half v = __double2half((feq - (double)fbase[i]) * (double)F16_SCALE);
      std::memcpy(&out[2 * i], &v, 2);
    }
  }
  return out;
}

// Storage offsets of the FP16 format: the free-stream equilibrium
// feq_i(rho = 1, u = (u_ref, 0, 0)) in deviation form, rounded to FP32
// (Store<F16Dev>); zero for the other formats.
template <int Q>
void storage_offsets(int storage, double u_ref, float *fbase) {
  using L = Lat<Q>;
  for (int i = 0; i < 27; ++i) fbase[i] = 0.0f;
  if (storage != CFLBM_STORE_FP16DEV) return;
  for (int i = 0; i < Q; ++i) {
    const double edu = L::ex(i) * u_ref;
    fbase[i] = (float)(L::w(i) * (3.0 * edu + 4.5 * edu * edu - 1.5 * u_ref * u_ref));
  }
}

int validate(const cflbm_config *c) {
  if (!c) return fail(CFLBM_E_INVALID, "config is NULL");
  if (c->lattice != CFLBM_D2Q9 && c->lattice != CFLBM_D3Q27)
    return fail(CFLBM_E_INVALID, "lattice must be 9 or 27, got %d", c->lattice);
  const int nz = c->lattice == CFLBM_D2Q9 ? 1 : c->nz;
  if (c->nx < 4 || c->ny < 4 || nz < 1 || (c->lattice == CFLBM_D3Q27 && nz < 4))
    return fail(CFLBM_E_INVALID, "grid %dx%dx%d too small", c->nx, c->ny, nz);
  if ((long long)c->nx * c->ny * nz > (1LL << 31))
    return fail(CFLBM_E_INVALID, "grid of %lld cells exceeds 2^31",
                (long long)c->nx * c->ny * nz);
  if (c->ny > 65535 * 4 || nz > 65535)
    return fail(CFLBM_E_INVALID, "ny or nz exceeds the launch grid limit");
  if (c->storage < 0 || c->storage > 2)
    return fail(CFLBM_E_INVALID, "storage %d unknown", c->storage);
  if (c->compute < 0 || c->compute > 2)
    return fail(CFLBM_E_INVALID, "compute %d unknown", c->compute);
  if (c->compute == CFLBM_COMPUTE_DF64 && c->storage != CFLBM_STORE_FP64)
    return fail(CFLBM_E_INVALID, "double-float arithmetic needs FP64 storage");
  if (c->profile < 0 || c->profile > 3)
    return fail(CFLBM_E_INVALID, "profile %d unknown", c->profile);
  if ((c->profile == CFLBM_PROFILE_REF2D || c->profile == CFLBM_PROFILE_REF2DS) &&
      c->lattice != CFLBM_D2Q9)
    return fail(CFLBM_E_INVALID, "REF2D/REF2DS profiles need the D2Q9 lattice");
  if (c->profile == CFLBM_PROFILE_REF3D && c->lattice != CFLBM_D3Q27)
    return fail(CFLBM_E_INVALID, "REF3D profile needs the D3Q27 lattice");
  if (c->wall_y < 0 || c->wall_y > 2 || c->wall_z < 0 || c->wall_z > 2)
    return fail(CFLBM_E_INVALID, "wall type out of range");
  if (!(c->tau0 > -0.5 + 1e-9) || !std::isfinite(c->tau0))
    return fail(CFLBM_E_INVALID, "tau0 = %g gives omega outside (0, 2)", c->tau0);
  if (!std::isfinite(c->u0)) return fail(CFLBM_E_INVALID, "u0 is not finite");
  if (c->force_history < 0) return fail(CFLBM_E_INVALID, "force_history < 0");
  if (c->layout != CFLBM_LAYOUT_SOA && c->layout != CFLBM_LAYOUT_ROWS)
    return fail(CFLBM_E_INVALID, "layout %d unknown", c->layout);
  if (c->rounding != CFLBM_ROUND_NEAREST && c->rounding != CFLBM_ROUND_STOCHASTIC)
    return fail(CFLBM_E_INVALID, "rounding %d unknown", c->rounding);
  return CFLBM_OK;
}

}  // namespace

extern "C" {

const char *cflbm_last_error(void) { return g_last_error.c_str(); }

int64_t cflbm_launch_count(void) { return (int64_t)launches(); }

int cflbm_config_default(cflbm_config *c) {
  if (!c) return fail(CFLBM_E_INVALID, "config is NULL");
  std::memset(c, 0, sizeof(*c));
  c->lattice = CFLBM_D2Q9;
  c->nx = 64;
  c->ny = 32;
  c->nz = 1;
  c->storage = CFLBM_STORE_FP64;
  c->compute = CFLBM_COMPUTE_FP64;
  c->profile = CFLBM_PROFILE_CHANNEL;
  c->wall_y = CFLBM_WALL_FREESLIP;
  c->wall_z = CFLBM_WALL_PERIODIC;
  c->tau0 = 0.03;
  c->u0 = 0.05;
  c->geom = CFLBM_GEOM_NONE;
  c->seed = 1234;
  c->layout = CFLBM_LAYOUT_ROWS;
  c->rounding = CFLBM_ROUND_STOCHASTIC;
  return CFLBM_OK;
}

int cflbm_create(const cflbm_config *cfg, cflbm_handle **out) {
  if (!out) return fail(CFLBM_E_INVALID, "out is NULL");
  *out = nullptr;
  int rc = validate(cfg);
  if (rc) return rc;
  std::unique_ptr<cflbm_handle, void (*)(cflbm_handle *)> hp(new cflbm_handle(), free_handle);
  cflbm_handle *h = hp.get();
  h->cfg = *cfg;
  h->cfg.solid = nullptr;
  h->cfg.alpha = nullptr;
  h->cfg.ref_ran = nullptr;
  h->Q = cfg->lattice;
  const int Q = h->Q;
  const bool d3 = Q == 27;
  const int nx = cfg->nx, ny = cfg->ny, nz = d3 ? cfg->nz : 1;
  h->cfg.nz = nz;
  CK_CUDA(cudaSetDevice(cfg->device));
  CK_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CK_CUDA(cudaEventCreateWithFlags(&h->ev_sync, cudaEventDisableTiming));
  CK_CUDA(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, cfg->device));
  if (cfg->profile == CFLBM_PROFILE_CHANNEL) {
    // Side stream of the channel step's force kernel, at the highest priority
    // so its blocks are scheduled ahead of the sweep's.
    int lo = 0, hi = 0;
    CK_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    CK_CUDA(cudaStreamCreateWithPriority(&h->fork.side, cudaStreamNonBlocking, hi));
    CK_CUDA(cudaEventCreateWithFlags(&h->fork.fork, cudaEventDisableTiming));
    CK_CUDA(cudaEventCreateWithFlags(&h->fork.join, cudaEventDisableTiming));
  }

  // Layout: ghosts as the profile needs them (the reference's 2 or 3 layers,
  // 1 for the channel), rows padded to 128 bytes with >= 4 spare elements past
  // the last ghost (the reference's wall pass reads two cells beyond the ring).
  const int es = store_size(cfg->storage);
  h->esize = es;
  const int G = cfg->profile == CFLBM_PROFILE_CHANNEL ? 1 : (cfg->profile == CFLBM_PROFILE_REF3D ? 3 : 2);
  const int align = 128 / es;
  Layout &L = h->L;
  L.nx = nx;
  L.ny = ny;
  L.nz = nz;
  L.G = G;
  L.Gz = d3 ? G : 0;
  L.xoff = align;
  // Row pitch: room for whole 32-cell warp tiles past the last interior cell, so
  // no lane of a partial last tile reads into the next row.
  const int nx_tiles = ((nx + 31) / 32) * 32;
  L.px = ((align + nx_tiles + G + 4 + align - 1) / align) * align;
  L.nyp = ny + 2 * G;
  L.nzp = nz + 2 * L.Gz;
  if (cfg->layout == CFLBM_LAYOUT_ROWS) {
    L.S = L.px;
    L.rs = (long long)Q * L.px;
  } else {
    L.S = (long long)L.px * L.nyp * L.nzp;
    L.rs = L.px;
  }
  L.zs = L.rs * L.nyp;
  L.total = (long long)Q * L.px * L.nyp * L.nzp;
  // FP16: the channel's free stream is the inlet's; the reference profiles'
  // Poiseuille inlet has no single stream velocity, so they store f itself.
  const double u_ref = cfg->profile == CFLBM_PROFILE_CHANNEL ? cfg->u0 : 0.0;
  if (d3) storage_offsets<27>(cfg->storage, u_ref, L.fbase);
  else storage_offsets<9>(cfg->storage, u_ref, L.fbase);
  h->nxw = (nx + 31) / 32;
  h->omega = 1.0 / (cfg->tau0 + 0.5);
  if (!(h->omega > 0.0 && h->omega < 2.0))
    return fail(CFLBM_E_INVALID, "omega = %g outside (0, 2)", h->omega);

  // Host-side geometry and initial fields.
  std::vector<uint8_t> solid;
  RefSetup ref;
  if (cfg->profile == CFLBM_PROFILE_REF2D) {
    ref2d_setup(nx, ny, cfg->u0, cfg->ref_ran, ref);
    solid = ref.solid;
    h->area = ref.area;
  } else if (cfg->profile == CFLBM_PROFILE_REF2DS) {
    ref2ds_setup(nx, ny, cfg->u0, cfg->ref_ran, ref);
    solid = ref.solid;
    h->area = ref.area;
  } else if (cfg->profile == CFLBM_PROFILE_REF3D) {
    ref3d_setup(nx, ny, nz, cfg->u0, cfg->ref_ran, ref);
    solid = ref.solid;
    h->area = ref.area;
  } else {
    // channel: the mask, links and listed tiles are built on the GPU below
    h->area = channel_area(h->cfg);
  }
  const bool chan = cfg->profile == CFLBM_PROFILE_CHANNEL;
  std::vector<int4> links;
  std::vector<uint32_t> mask;
  if (!chan) {
    if (d3) build_links<27>(solid, nx, ny, nz, links, h->n_solid);
    else build_links<9>(solid, nx, ny, nz, links, h->n_solid);
    h->n_links = (long long)links.size();
    mask = pack_mask(solid, nx, ny, nz, h->nxw);
  }

  // Device allocations.
  const size_t N = (size_t)nx * ny * nz;
  h->f_bytes = (size_t)L.total * es;
  if ((rc = dev_alloc(h, &h->fA, h->f_bytes))) return rc;
  if ((rc = dev_alloc(h, &h->fB, h->f_bytes))) return rc;
  h->buf[0] = h->fA;
  h->buf[1] = h->fB;
  CK_CUDA(cudaMemsetAsync(h->fA, 0, h->f_bytes, h->stream));
  CK_CUDA(cudaMemsetAsync(h->fB, 0, h->f_bytes, h->stream));
  if ((rc = dev_alloc_t(h, &h->d_mask, (size_t)h->nxw * ny * nz))) return rc;
  if (!chan)
    CK_CUDA(cudaMemcpyAsync(h->d_mask, mask.data(), mask.size() * 4, cudaMemcpyHostToDevice,
                            h->stream));
  if ((rc = dev_alloc_t(h, &h->d_links, links.size() + 1))) return rc;
  if (!links.empty())
    CK_CUDA(cudaMemcpyAsync(h->d_links, links.data(), links.size() * sizeof(int4),
                            cudaMemcpyHostToDevice, h->stream));
  if ((rc = dev_alloc_t(h, &h->d_mu, N))) return rc;
  if ((rc = dev_alloc_t(h, &h->d_mv, N))) return rc;
  if ((rc = dev_alloc_t(h, &h->d_mw, N))) return rc;
  if ((rc = dev_alloc_t(h, &h->d_mp, N))) return rc;
  h->hist_cap = cfg->force_history > 0 ? cfg->force_history : 65536;
  if ((rc = dev_alloc_t(h, &h->d_hist, 3 * (size_t)h->hist_cap))) return rc;
  CK_CUDA(cudaMemsetAsync(h->d_hist, 0, 3 * sizeof(double) * h->hist_cap, h->stream));
  if ((rc = dev_alloc_t(h, &h->d_step, 1))) return rc;
  CK_CUDA(cudaMemsetAsync(h->d_step, 0, sizeof(long long), h->stream));
  h->reduce_blocks = (int)std::min<long long>(std::max<long long>(((long long)N + 255) / 256, 1), 2048);
  if (chan) {
    // Mask, per-cell link bits, listed tiles and their link words on the GPU
    // (setup.cu); scratch: the link bits of every cell and an explicit mask's
    // bytes, freed before returning.
    SetupArgs sa{};
    sa.nx = nx;
    sa.ny = ny;
    sa.nz = nz;
    sa.nxw = h->nxw;
    sa.wall_y = cfg->wall_y;
    sa.wall_z = cfg->wall_z;
    sa.geom = cfg->geom;
    sa.cx = cfg->cx;
    sa.cy = cfg->cy;
    sa.cz = cfg->cz;
    sa.r2 = 0.25 * cfg->diam * cfg->diam;
    const size_t ntiles = (size_t)h->nxw * ny * nz;
    const int nchunks = setup_chunks(sa);
    // one scratch block: counters, chunk offsets + total, per-cell bits, input mask
    const size_t off_chunk = 64, off_bits = off_chunk + 4 * ((size_t)nchunks + 16);
    const size_t off_in = off_bits + 4 * N + 256;
    const size_t scratch_bytes = off_in + (cfg->solid ? N : 0);
    unsigned char *scratch = nullptr;
    CK_CUDA(cudaMalloc(&scratch, scratch_bytes));
    std::unique_ptr<unsigned char, cudaError_t (*)(void *)> scratch_guard(scratch, cudaFree);
    unsigned long long *counters = reinterpret_cast<unsigned long long *>(scratch);
    int *chunk = reinterpret_cast<int *>(scratch + off_chunk);
    int *d_total = chunk + nchunks;
    uint32_t *bits = reinterpret_cast<uint32_t *>(scratch + ((off_bits + 255) / 256) * 256);
    CK_CUDA(cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), h->stream));
    if (cfg->solid) {
      uint8_t *in = scratch + off_in;
      CK_CUDA(cudaMemcpyAsync(in, cfg->solid, N, cudaMemcpyHostToDevice, h->stream));
      sa.solid_in = in;
    }
    if ((rc = dev_alloc_t(h, &h->d_tile_slow, ntiles))) return rc;
    if ((rc = dev_alloc_t(h, &h->d_tile_index, ntiles))) return rc;
    CK_CUDA(launch_setup_mask_links(Q, sa, h->d_mask, bits, counters, h->stream));
    CK_CUDA(launch_setup_flags(sa, h->d_mask, bits, h->d_tile_slow, chunk, d_total, h->stream));
    unsigned long long cnt[2] = {0, 0};
    int total = 0;
    CK_CUDA(cudaMemcpyAsync(cnt, counters, sizeof(cnt), cudaMemcpyDeviceToHost, h->stream));
    CK_CUDA(cudaMemcpyAsync(&total, d_total, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK_CUDA(cudaStreamSynchronize(h->stream));
    h->n_solid = (long long)cnt[0];
    h->n_links = (long long)cnt[1];
    h->n_slow = total;
    if ((rc = dev_alloc_t(h, &h->d_slow_tiles, (size_t)total + 1))) return rc;
    if ((rc = dev_alloc_t(h, &h->d_links_bits, 32 * (size_t)total + 32))) return rc;
    CK_CUDA(launch_setup_list(sa, h->d_tile_slow, chunk, h->d_mask, bits, h->d_tile_index,
                              h->d_slow_tiles, h->d_links_bits, h->stream));
    // The force launch's cells: the fluid cells with solid links, one thread
    // each.  One warp per listed tile with such cells (about 9,000 of the
    // 17,000 listed tiles of the D3Q27 512x128x128 cylinder) left most lanes
    // idle and held its registers for 53 us per step beside the FP16 sweep.
    const int wch = bcell_chunks(total);
    unsigned char *wscr = nullptr;
    const size_t w_off = ((size_t)total + 256) / 256 * 256;
    CK_CUDA(cudaMalloc(&wscr, w_off + 4 * ((size_t)wch + 1)));
    std::unique_ptr<unsigned char, cudaError_t (*)(void *)> wscr_guard(wscr, cudaFree);
    int *wchunk = reinterpret_cast<int *>(wscr + w_off);
    int *wtot = wchunk + wch;
    CK_CUDA(launch_setup_bcell_count(total, h->d_links_bits, wscr, wchunk, wtot, h->stream));
    int nb = 0;
    CK_CUDA(cudaMemcpyAsync(&nb, wtot, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK_CUDA(cudaStreamSynchronize(h->stream));
    h->n_bcells = nb;
    if ((rc = dev_alloc_t(h, &h->d_bcell_idx, (size_t)nb + 1))) return rc;
    if ((rc = dev_alloc_t(h, &h->d_bcell_links, (size_t)nb + 1))) return rc;
    CK_CUDA(launch_setup_bcell_list(L, h->nxw, total, h->d_slow_tiles, h->d_links_bits, wscr,
                                    wchunk, h->d_bcell_idx, h->d_bcell_links, h->stream));
    std::vector<long long> foff;
    std::vector<uint32_t> fbb;
    if (d3) face_tables<27>(L, cfg->wall_y, cfg->wall_z, foff, fbb);
    else face_tables<9>(L, cfg->wall_y, cfg->wall_z, foff, fbb);
    if ((rc = dev_alloc_t(h, &h->d_face_off, foff.size()))) return rc;
    if ((rc = dev_alloc_t(h, &h->d_face_bb, fbb.size()))) return rc;
    CK_CUDA(cudaMemcpyAsync(h->d_face_off, foff.data(), foff.size() * sizeof(long long),
                            cudaMemcpyHostToDevice, h->stream));
    CK_CUDA(cudaMemcpyAsync(h->d_face_bb, fbb.data(), fbb.size() * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, h->stream));
    for (int i = 0; i < Q; ++i) {
      const int ex = d3 ? Lat<27>::ex(i) : Lat<9>::ex(i);
      const double w = d3 ? Lat<27>::w(i) : Lat<9>::w(i);
      const double edu = ex * cfg->u0;
      h->f_in[i] = w * 0.0 * 3.0 + w * (3.0 * edu + 4.5 * edu * edu - 1.5 * cfg->u0 * cfg->u0);
    }
    CK_CUDA(cudaStreamSynchronize(h->stream));  // host vectors die at scope end
  }
  h->link_blocks = (int)std::min<long long>(std::max<long long>((h->n_links + 255) / 256, 1), 1024);
  // Force partials: one per block of listed tiles, for any tile height >= 1.
  const size_t nparts = std::max<size_t>(4 * (size_t)std::max(h->link_blocks, h->reduce_blocks),
                                         3 * (size_t)std::max(h->n_slow, 1));
  if ((rc = dev_alloc_t(h, &h->d_partials, nparts))) return rc;
  if ((rc = dev_alloc_t(h, &h->d_counter, 1))) return rc;
  if ((rc = dev_alloc_t(h, &h->d_counter2, 1))) return rc;
  CK_CUDA(cudaMemsetAsync(h->d_counter, 0, sizeof(unsigned), h->stream));
  CK_CUDA(cudaMemsetAsync(h->d_counter2, 0, sizeof(unsigned), h->stream));
  if ((rc = dev_alloc_t(h, &h->d_sums, 4))) return rc;
  if ((rc = dev_alloc_t(h, &h->d_err, 1))) return rc;
  CK_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(unsigned), h->stream));
  // FP16 ROWS channel sweeps: the register-fed pair kernel; the line-staged
  // kernel (slower on GB300: 0.37 against 0.57 of the copy peak at 512x128x128)
  // when the environment variable CFLBM_FP16_SWEEP says "lines"
  const char *fp16_sweep = std::getenv("CFLBM_FP16_SWEEP");
  h->lines = cfg->profile == CFLBM_PROFILE_CHANNEL &&
             (fp16_sweep && std::strcmp(fp16_sweep, "lines") == 0) &&
             lines_supported(Q, cfg->storage, cfg->layout == CFLBM_LAYOUT_ROWS,
                             cfg->alpha != nullptr, nx);
  if (h->lines) CK_CUDA(lines_prepare());

  if (cfg->profile == CFLBM_PROFILE_CHANNEL) {
    std::vector<unsigned char> fin = d3 ? inlet_elements<27>(cfg->u0, cfg->storage, L.fbase)
                                        : inlet_elements<9>(cfg->u0, cfg->storage, L.fbase);
    if ((rc = dev_alloc(h, &h->d_fin, fin.size()))) return rc;
    CK_CUDA(cudaMemcpyAsync(h->d_fin, fin.data(), fin.size(), cudaMemcpyHostToDevice, h->stream));
    if (cfg->alpha) {
      std::vector<float> a(N);
      for (size_t n = 0; n < N; ++n) a[n] = (float)cfg->alpha[n];
      if ((rc = dev_alloc_t(h, &h->d_alpha, N))) return rc;
      CK_CUDA(cudaMemcpyAsync(h->d_alpha, a.data(), N * 4, cudaMemcpyHostToDevice, h->stream));
      CK_CUDA(cudaStreamSynchronize(h->stream));
    }
    CK_CUDA(launch_init_channel(Q, cfg->storage, L, h->fA, h->d_mask, h->nxw, cfg->u0,
                                cfg->perturb_amp, cfg->seed, h->d_alpha, h->omega, h->d_mu,
                                h->d_mv, h->d_mw, h->d_mp, h->stream));
  } else {
    if ((rc = dev_alloc_t(h, &h->d_inlet, ref.inlet.size()))) return rc;
    CK_CUDA(cudaMemcpyAsync(h->d_inlet, ref.inlet.data(), ref.inlet.size() * 8,
                            cudaMemcpyHostToDevice, h->stream));
    const size_t P = ref.u.size();
    double *du = nullptr, *dv = nullptr, *dw = nullptr, *dp = nullptr;
    CK_CUDA(cudaMalloc(&du, 4 * P * sizeof(double)));
    dv = du + P;
    dw = dv + P;
    dp = dw + P;
    cudaMemcpyAsync(du, ref.u.data(), P * 8, cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(dv, ref.v.data(), P * 8, cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(dw, ref.w.data(), P * 8, cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(dp, ref.p.data(), P * 8, cudaMemcpyHostToDevice, h->stream);
    cudaError_t e = launch_init_macros(Q, cfg->storage, L, h->fA, du, dv, dw, dp, h->stream);
    // Both buffers start with the same ghost layers; afterwards only the face
    // passes write ghosts, into both buffers.
    if (e == cudaSuccess) e = launch_ghost_copy(Q, cfg->storage, L, h->fA, h->fB, h->stream);
    // Step-0 macroscopic fields: the interior of the initial fields.
    std::vector<double> mu(N), mv(N), mw(N), mp(N);
    const int lxp = nx + 2 * G, lyp = ny + 2 * G;
    for (int z = 0; z < nz; ++z)
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
          const size_t d = ((size_t)(z + L.Gz) * lyp + (y + G)) * lxp + (x + G);
          const size_t n = ((size_t)z * ny + y) * nx + x;
          mu[n] = ref.u[d];
          mv[n] = ref.v[d];
          mw[n] = ref.w[d];
          mp[n] = ref.p[d];
        }
    cudaMemcpyAsync(h->d_mu, mu.data(), N * 8, cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(h->d_mv, mv.data(), N * 8, cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(h->d_mw, mw.data(), N * 8, cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(h->d_mp, mp.data(), N * 8, cudaMemcpyHostToDevice, h->stream);
    cudaError_t e2 = cudaStreamSynchronize(h->stream);
    cudaFree(du);
    CK_CUDA(e);
    CK_CUDA(e2);
  }
  CK_CUDA(cudaStreamSynchronize(h->stream));
  CK_CUDA(cudaGetLastError());
  *out = hp.release();
  return CFLBM_OK;
}

int cflbm_destroy(cflbm_handle *h) {
  free_handle(h);
  return CFLBM_OK;
}

// Record a timing event on the handle's stream (pool grows on demand).
static int record_event(cflbm_handle *h, size_t *idx) {
  if (h->ev_used == h->ev_pool.size()) {
    cudaEvent_t e;
    CK_CUDA(cudaEventCreate(&e));
    h->ev_pool.push_back(e);
  }
  *idx = h->ev_used++;
  CK_CUDA(cudaEventRecord(h->ev_pool[*idx], h->stream));
  return CFLBM_OK;
}

extern "C++" {
namespace cflbm {
void set_relax(SweepArgs &a, int Q, int, double omega) {
  a.omega = omega;
  a.omega_f = (float)omega;
  // per weight class c = |e|^2: weight, directions, directions with e_x != 0
  double w[4] = {};
  int n[4] = {}, m[4] = {};
  for (int k = 0; k < Q; ++k) {
    const int ex = Q == 27 ? Lat<27>::ex(k) : Lat<9>::ex(k);
    const int ey = Q == 27 ? Lat<27>::ey(k) : Lat<9>::ey(k);
    const int ez = Q == 27 ? Lat<27>::ez(k) : 0;
    const int c = ex * ex + ey * ey + ez * ez;
    w[c] = Q == 27 ? Lat<27>::w(k) : Lat<9>::w(k);
    ++n[c];
    m[c] += ex * ex;
  }
  const int NC = Q == 27 ? 4 : 3;
  double rk[RK_N] = {1.0 - omega};
  for (int c = 0; c < NC; ++c) {
    rk[RK_W + c] = omega * w[c];
    rk[RK_A + c] = 4.5 * omega * w[c];
    rk[RK_3 + c] = 3.0 * omega * w[c];
  }
  // FP32: Om = 1 - float(1 - omega) exactly; every class from Om, then the rest
  // class's Kw and the face class's K3, Ka recomputed so that the identities
  // hold exactly (the sums below are exact in FP64: few terms of 24-bit values
  // spanning < 32 binades) and split into FP32 pairs (hi + lo exact).
  float kf[RK_N] = {};
  kf[RK_OMC] = (float)(1.0 - omega);
  const double Om = 1.0 - (double)kf[RK_OMC];
  for (int c = 0; c < NC; ++c) {
    kf[RK_W + c] = (float)(Om * w[c]);
    kf[RK_A + c] = (float)(4.5 * Om * w[c]);
    kf[RK_3 + c] = (float)(3.0 * Om * w[c]);
  }
  double kw0 = Om, k31 = Om, ka1 = 1.5 * Om;
  for (int c = 1; c < NC; ++c) kw0 -= n[c] * (double)kf[RK_W + c];
  for (int c = 2; c < NC; ++c) {
    k31 -= m[c] * (double)kf[RK_3 + c];
    ka1 -= m[c] * (double)kf[RK_A + c];
  }
  k31 /= m[1];
  ka1 /= m[1];
  auto split = [&](double x, int hi, int lo) {
    kf[hi] = (float)x;
    kf[lo] = (float)(x - (double)kf[hi]);
  };
  split(kw0, RK_W, RK_LW);
  split(k31, RK_3 + 1, RK_L3);
  split(ka1, RK_A + 1, RK_LA);
  for (int c = 0; c < NC; ++c) {  // -2 K3 (exact)
    rk[RK_M3 + c] = -2.0 * rk[RK_3 + c];
    kf[RK_M3 + c] = -2.0f * kf[RK_3 + c];
  }
  for (int k = 0; k < RK_N; ++k) {
    a.rk[k] = rk[k];
    a.rkf[k] = kf[k];
    a.rkl[k] = (float)(rk[k] - (double)kf[k]);
  }
}

void set_offsets(SweepArgs &a, int Q) {
  for (int i = 0; i < 27; ++i) {
    a.doff[i] = a.poff[i] = 0;
    if (i >= Q) continue;
    const int ex = Q == 27 ? Lat<27>::ex(i) : Lat<9>::ex(i);
    const int ey = Q == 27 ? Lat<27>::ey(i) : Lat<9>::ey(i);
    const int ez = Q == 27 ? Lat<27>::ez(i) : 0;
    a.doff[i] = (long long)i * a.L.S;
    a.poff[i] = a.doff[i] - a.L.off(ex, ey, ez);
  }
}

// Arguments of the channel sweep of handle h reading fa and writing fb.
SweepArgs channel_args(const cflbm_handle *h, const void *fa, void *fb, bool write_macros) {
  SweepArgs sa{};
  sa.L = h->L;
  sa.fa = fa;
  sa.fb = fb;
  sa.mask = h->d_mask;
  sa.nxw = h->nxw;
  set_relax(sa, h->Q, h->cfg.storage, h->omega);
  set_offsets(sa, h->Q);
  sa.f16_sr = h->cfg.rounding == CFLBM_ROUND_STOCHASTIC;
  sa.alpha = h->d_alpha;
  if (write_macros) {
    sa.mu = h->d_mu;
    sa.mv = h->d_mv;
    sa.mw = h->d_mw;
    sa.mp = h->d_mp;
  }
  sa.wall_y = h->cfg.wall_y;
  sa.wall_z = h->cfg.wall_z;
  // Inlet populations in every arithmetic type.
  for (int i = 0; i < h->Q; ++i) {
    sa.f_in[i] = h->f_in[i];
    sa.f_in_f[i] = (float)h->f_in[i];
    sa.f_in_l[i] = (float)(h->f_in[i] - (double)sa.f_in_f[i]);
  }
  // Grid of the force launch beside the sweep: one boundary cell per thread,
  // at most one block per SM.
  const long long fthreads = SWEEP_BX * SWEEP_BY;
  sa.bnd_blocks = (int)std::max<long long>(
      1, std::min<long long>((h->n_bcells + fthreads - 1) / fthreads, (long long)h->sms));
  sa.tile_slow = h->d_tile_slow;
  sa.slow_tiles = h->d_slow_tiles;
  sa.tile_index = h->d_tile_index;
  sa.face_off = h->d_face_off;
  sa.face_bb = h->d_face_bb;
  sa.links_bits = h->d_links_bits;
  sa.n_slow = h->n_slow;
  sa.bcell_idx = h->d_bcell_idx;
  sa.bcell_links = h->d_bcell_links;
  sa.n_bcells = h->n_bcells;
  sa.partials = h->d_partials;
  sa.counter = h->d_counter;
  sa.hist = h->d_hist;
  sa.step = h->d_step;
  sa.cap = h->hist_cap;
  sa.sms = h->sms;
  sa.lines = h->lines ? 1 : 0;
  sa.err = h->d_err;
  return sa;
}
}  // namespace cflbm
}  // extern "C++"

static int one_step(cflbm_handle *h, bool write_macros) {
  size_t tb0 = 0, tb1 = 0, ts0 = 0, ts1 = 0;
  int trc;
  if (h->timing && h->cfg.profile != CFLBM_PROFILE_CHANNEL && (trc = record_event(h, &tb0)))
    return trc;
  const int Q = h->Q;
  const int st = h->cfg.storage;
  const Layout &L = h->L;
  FillArgs fa{};
  fa.L = L;
  fa.f = h->fA;
  fa.f2 = h->fB;  // face-pass ghosts go to both buffers (see face_op_kernel)
  fa.mask = h->d_mask;
  fa.nxw = h->nxw;
  fa.wall_y = h->cfg.wall_y;
  fa.wall_z = h->cfg.wall_z;
  fa.f_in = h->d_fin;
  const bool ref = h->cfg.profile != CFLBM_PROFILE_CHANNEL;
  if (!ref) {
    // u, v, w, p are formed on request (ensure_macros), not written every step.
    (void)write_macros;
    const SweepArgs sa = channel_args(h, h->fA, h->fB, false);
    if (h->timing && (trc = record_event(h, &ts0))) return trc;
    CK_CUDA(launch_sweep_channel(Q, st, h->cfg.compute, sa, h->stream, &h->fork));
    if (h->timing) {
      if ((trc = record_event(h, &ts1))) return trc;
      h->sweep_ev.push_back({ts0, ts1});
    }
    std::swap(h->fA, h->fB);
    ++h->steps_done;
    h->macros_pending = true;
    return CFLBM_OK;
  }
  if (h->cfg.profile == CFLBM_PROFILE_REF2D || h->cfg.profile == CFLBM_PROFILE_REF2DS) {
    // "MPI Kokkos/lbm.cpp:315-345": inlet, outlet, then the two wall rows.
    // Each pair (the two ends of one axis) writes and reads disjoint layers, so a
    // pair runs as one launch; the pairs keep the reference's order.  The serial
    // variant's wall rows ("Kokkos/lbm.cpp:158-168") leave out the two corner
    // nodes of each ghost row.
    const int trim = h->cfg.profile == CFLBM_PROFILE_REF2DS ? 1 : 0;
    const FaceOp ops[4] = {{0, 0, 0, 0}, {1, 0, 1, 0}, {2, 1, 0, trim}, {2, 1, 1, trim}};
    for (int k = 0; k < 4; k += 2)
      CK_CUDA(launch_face_ops(Q, st, fa, ops[k], ops[k + 1], h->stream));
  } else {
    // "3D MPI+KOKKOS+MPIIO/lbm.cpp:278-347": front, back, bottom, top, inlet, outlet.
    const FaceOp ops[6] = {{2, 1, 0}, {2, 1, 1}, {2, 2, 0}, {2, 2, 1}, {0, 0, 0}, {1, 0, 1}};
    for (int k = 0; k < 6; k += 2)
      CK_CUDA(launch_face_ops(Q, st, fa, ops[k], ops[k + 1], h->stream));
  }
  LinkArgs la{};
  la.L = L;
  la.f = h->fA;
  la.links = h->d_links;
  la.n = h->n_links;
  la.reach = ref ? 2 : 1;
  la.partials = h->d_partials;
  la.counter = h->d_counter;
  la.hist = h->d_hist;
  la.step = h->d_step;
  la.cap = h->hist_cap;
  CK_CUDA(launch_links(Q, st, la, h->link_blocks, h->stream));
  if (h->timing) {
    if ((trc = record_event(h, &tb1))) return trc;
    h->bnd_ev.push_back({tb0, tb1});
    if ((trc = record_event(h, &ts0))) return trc;
  }
  SweepArgs sa{};
  sa.L = L;
  sa.fa = h->fA;
  sa.fb = h->fB;
  sa.mask = h->d_mask;
  sa.nxw = h->nxw;
  set_relax(sa, Q, st, h->omega);
  set_offsets(sa, Q);
  sa.f16_sr = h->cfg.rounding == CFLBM_ROUND_STOCHASTIC;
  sa.ref_override = ref ? 1 : 0;
  sa.inlet_u = h->d_inlet;
  sa.alpha = h->d_alpha;
  if (write_macros) {
    sa.mu = h->d_mu;
    sa.mv = h->d_mv;
    sa.mw = h->d_mw;
    sa.mp = h->d_mp;
  }
  CK_CUDA(launch_sweep(Q, st, h->cfg.compute, sa, h->stream));
  if (h->timing) {
    if ((trc = record_event(h, &ts1))) return trc;
    h->sweep_ev.push_back({ts0, ts1});
  }
  std::swap(h->fA, h->fB);
  ++h->steps_done;
  return CFLBM_OK;
}

int cflbm_step(cflbm_handle *h, int nsteps) {
  if (!h) return fail(CFLBM_E_INVALID, "handle is NULL");
  if (nsteps < 0) return fail(CFLBM_E_INVALID, "nsteps < 0");
  if (h->batched)
    return fail(CFLBM_E_INVALID, "this handle belongs to a batch: step it with cflbm_batch_step");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  int left = nsteps;
  // Long calls replay a captured CUDA graph of GRAPH_STEPS steps (an even count,
  // so the A/B parity is unchanged), one graph per parity, captured on first use.
  // The last step always runs directly so it can write the macroscopic fields.
  while (!h->timing && left > GRAPH_STEPS) {
    const int par = h->fA == h->buf[0] ? 0 : 1;
    if (!h->graph_exec[par]) {
      cudaGraph_t g = nullptr;
      const long long n0 = launches();
      CK_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      int rc = CFLBM_OK;
      for (int s = 0; s < GRAPH_STEPS && rc == CFLBM_OK; ++s) rc = one_step(h, false);
      cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      CK_CUDA(ec);
      cudaError_t ei = cudaGraphInstantiate(&h->graph_exec[par], g, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(g);
      CK_CUDA(ei);
      h->launches_per_step = (launches() - n0) / GRAPH_STEPS;
      // Capture advanced the host-side step state (and counted the captured
      // launches) without running anything; this first replay runs them.
      CK_CUDA(cudaGraphLaunch(h->graph_exec[par], h->stream));
    } else {
      CK_CUDA(cudaGraphLaunch(h->graph_exec[par], h->stream));
      h->steps_done += GRAPH_STEPS;
      count_launch((long long)GRAPH_STEPS * h->launches_per_step);
    }
    left -= GRAPH_STEPS;
  }
  for (int s = 0; s < left; ++s) {
    int rc = one_step(h, s == left - 1);
    if (rc) return rc;
  }
  return CFLBM_OK;
}

// The device error word: a kernel whose bounded wait gave up recorded it.
static int check_device_error(cflbm_handle *h) {
  unsigned e = 0;
  CK_CUDA(cudaMemcpyAsync(&e, h->d_err, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
  CK_CUDA(cudaStreamSynchronize(h->stream));
  if (e) return fail(CFLBM_E_CUDA, "a sweep kernel's wait for its copies timed out (0x%08x)", e);
  return CFLBM_OK;
}

int cflbm_synchronize(cflbm_handle *h) {
  if (!h) return fail(CFLBM_E_INVALID, "handle is NULL");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  CK_CUDA(cudaStreamSynchronize(h->stream));
  CK_CUDA(cudaGetLastError());
  return check_device_error(h);
}

int cflbm_selftest_wait_timeout(cflbm_handle *h, int64_t polls) {
  if (!h) return fail(CFLBM_E_INVALID, "handle is NULL");
  if (polls < 1 || polls > (int64_t)1 << 22)
    return fail(CFLBM_E_INVALID, "polls = %lld outside [1, 2^22]", (long long)polls);
  CK_CUDA(cudaSetDevice(h->cfg.device));
  CK_CUDA(launch_wait_timeout_probe(h->d_err, (long long)polls, h->stream));
  return CFLBM_OK;
}

// Channel profile: forms u, v, w, p of the last step from the state that step
// read (fB after the step; intact until the next step), once per step.
static int ensure_macros(cflbm_handle *h) {
  if (!h->macros_pending) return CFLBM_OK;
  const SweepArgs sa = channel_args(h, h->fB, nullptr, true);
  CK_CUDA(launch_macros_channel(h->Q, h->cfg.storage, h->cfg.compute, sa, h->stream));
  h->macros_pending = false;
  return CFLBM_OK;
}

int cflbm_macros(cflbm_handle *h, double *u, double *v, double *w, double *p) {
  if (!h) return fail(CFLBM_E_INVALID, "handle is NULL");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  if (int rc = ensure_macros(h)) return rc;
  const size_t N = (size_t)h->L.nx * h->L.ny * h->L.nz;
  double *dst[4] = {u, v, w, p};
  double *src[4] = {h->d_mu, h->d_mv, h->d_mw, h->d_mp};
  for (int k = 0; k < 4; ++k)
    if (dst[k]) CK_CUDA(cudaMemcpyAsync(dst[k], src[k], N * 8, cudaMemcpyDeviceToHost, h->stream));
  CK_CUDA(cudaStreamSynchronize(h->stream));
  return CFLBM_OK;
}

int cflbm_macros_device(cflbm_handle *h, double *u, double *v, double *w, double *p) {
  if (!h) return fail(CFLBM_E_INVALID, "handle is NULL");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  if (int rc = ensure_macros(h)) return rc;
  const size_t N = (size_t)h->L.nx * h->L.ny * h->L.nz;
  double *dst[4] = {u, v, w, p};
  double *src[4] = {h->d_mu, h->d_mv, h->d_mw, h->d_mp};
  for (int k = 0; k < 4; ++k)
    if (dst[k]) CK_CUDA(cudaMemcpyAsync(dst[k], src[k], N * 8, cudaMemcpyDeviceToDevice, h->stream));
  return CFLBM_OK;
}

int cflbm_forces(cflbm_handle *h, double fxyz[3], double cd_cl[2]) {
  if (!h) return fail(CFLBM_E_INVALID, "handle is NULL");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  double F[3] = {0.0, 0.0, 0.0};
  if (h->steps_done > 0) {
    const long long slot = (h->steps_done - 1) % h->hist_cap;
    CK_CUDA(cudaMemcpyAsync(F, h->d_hist + 3 * slot, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                            h->stream));
  }
  CK_CUDA(cudaStreamSynchronize(h->stream));
  if (fxyz) {
    fxyz[0] = F[0];
    fxyz[1] = F[1];
    fxyz[2] = F[2];
  }
  if (cd_cl) {
    const double u0 = h->cfg.u0;
    if (h->cfg.profile == CFLBM_PROFILE_REF2D) {
      // The reference's own expression ("MPI Kokkos/lbm.cpp:404").
      cd_cl[0] = 2.0 * F[0] / u0 / u0 / 0.03125 / (h->L.nx - 1);
      cd_cl[1] = 2.0 * F[1] / u0 / u0 / 0.03125 / (h->L.nx - 1);
    } else {
      cd_cl[0] = 2.0 * F[0] / (u0 * u0 * h->area);
      cd_cl[1] = 2.0 * F[1] / (u0 * u0 * h->area);
    }
  }
  return CFLBM_OK;
}

int cflbm_forces_async(cflbm_handle *h, double fxyz[3]) {
  if (!h || !fxyz) return fail(CFLBM_E_INVALID, "bad arguments");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  if (h->steps_done == 0) {  // no step yet: zero, once earlier copies into fxyz are done
    CK_CUDA(cudaStreamSynchronize(h->stream));
    fxyz[0] = fxyz[1] = fxyz[2] = 0.0;
    return CFLBM_OK;
  }
  const long long slot = (h->steps_done - 1) % h->hist_cap;
  CK_CUDA(cudaMemcpyAsync(fxyz, h->d_hist + 3 * slot, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                          h->stream));
  return CFLBM_OK;
}

int cflbm_force_history(cflbm_handle *h, double *out, int64_t max_steps, int64_t *n_out) {
  if (!h || !out || max_steps < 0) return fail(CFLBM_E_INVALID, "bad arguments");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  const long long have = std::min<long long>(h->steps_done, h->hist_cap);
  const long long n = std::min<long long>(have, max_steps);
  // Oldest kept step first.
  const long long first = h->steps_done - n;
  for (long long k = 0; k < n;) {
    const long long slot = (first + k) % h->hist_cap;
    const long long run = std::min<long long>(n - k, h->hist_cap - slot);
    CK_CUDA(cudaMemcpyAsync(out + 3 * k, h->d_hist + 3 * slot, run * 3 * sizeof(double),
                            cudaMemcpyDeviceToHost, h->stream));
    k += run;
  }
  CK_CUDA(cudaStreamSynchronize(h->stream));
  if (n_out) *n_out = n;
  return CFLBM_OK;
}

int cflbm_mass(cflbm_handle *h, double *mass, double momentum[3]) {
  if (!h) return fail(CFLBM_E_INVALID, "handle is NULL");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  ReduceArgs ra{};
  ra.L = h->L;
  ra.f = h->fA;
  ra.mask = h->d_mask;
  ra.nxw = h->nxw;
  ra.partials = h->d_partials;
  ra.counter = h->d_counter2;
  ra.out = h->d_sums;
  CK_CUDA(launch_reduce_mass(h->Q, h->cfg.storage, ra, h->reduce_blocks, h->stream));
  double s[4];
  CK_CUDA(cudaMemcpyAsync(s, h->d_sums, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
  CK_CUDA(cudaStreamSynchronize(h->stream));
  if (int rc = check_device_error(h)) return rc;
  if (!std::isfinite(s[0])) return fail(CFLBM_E_NUMERIC, "mass is not finite (%g)", s[0]);
  if (mass) *mass = s[0];
  if (momentum) {
    momentum[0] = s[1];
    momentum[1] = s[2];
    momentum[2] = s[3];
  }
  return CFLBM_OK;
}

int cflbm_get_f(cflbm_handle *h, double *out) {
  if (!h || !out) return fail(CFLBM_E_INVALID, "bad arguments");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  const size_t n = (size_t)h->Q * h->L.nx * h->L.ny * h->L.nz;
  double *d = nullptr;
  CK_CUDA(cudaMalloc(&d, n * sizeof(double)));
  cudaError_t e = launch_get_f(h->Q, h->cfg.storage, h->L, h->fA, d, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, n * 8, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  CK_CUDA(e);
  return CFLBM_OK;
}

int cflbm_set_f(cflbm_handle *h, const double *in, int64_t steps_done) {
  if (!h || !in || steps_done < 0) return fail(CFLBM_E_INVALID, "bad arguments");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  const size_t n = (size_t)h->Q * h->L.nx * h->L.ny * h->L.nz;
  double *d = nullptr;
  CK_CUDA(cudaMalloc(&d, n * sizeof(double)));
  cudaError_t e = cudaMemcpyAsync(d, in, n * 8, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = launch_set_f(h->Q, h->cfg.storage, h->L, h->fA, d, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  CK_CUDA(e);
  h->steps_done = steps_done;
  h->macros_pending = false;
  long long st = steps_done;
  CK_CUDA(cudaMemcpy(h->d_step, &st, sizeof(st), cudaMemcpyHostToDevice));
  return CFLBM_OK;
}

int cflbm_get_f_stream(cflbm_handle *h, double *out) {
  if (!h || !out) return fail(CFLBM_E_INVALID, "bad arguments");
  if (h->steps_done == 0) return cflbm_get_f(h, out);  // f = feq, as after Initialize
  CK_CUDA(cudaSetDevice(h->cfg.device));
  const size_t n = (size_t)h->Q * h->L.nx * h->L.ny * h->L.nz;
  double *d = nullptr;
  CK_CUDA(cudaMalloc(&d, n * sizeof(double)));
  // fB: the state the last step pulled from (ghosts and solid nodes filled for
  // the reference profiles); intact until the next step.
  SweepArgs sa = channel_args(h, h->fB, nullptr, false);
  cudaError_t e = launch_stream_state(h->Q, h->cfg.storage, sa,
                                      h->cfg.profile != CFLBM_PROFILE_CHANNEL, d, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, n * 8, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  CK_CUDA(e);
  return CFLBM_OK;
}

int cflbm_get_solid(cflbm_handle *h, uint8_t *out) {
  if (!h || !out) return fail(CFLBM_E_INVALID, "bad arguments");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  const int nx = h->L.nx, ny = h->L.ny, nz = h->L.nz;
  std::vector<uint32_t> m((size_t)h->nxw * ny * nz);
  CK_CUDA(cudaMemcpyAsync(m.data(), h->d_mask, m.size() * 4, cudaMemcpyDeviceToHost, h->stream));
  CK_CUDA(cudaStreamSynchronize(h->stream));
  for (long long r = 0; r < (long long)ny * nz; ++r)
    for (int x = 0; x < nx; ++x)
      out[(size_t)r * nx + x] = (m[(size_t)r * h->nxw + (x >> 5)] >> (x & 31)) & 1u;
  return CFLBM_OK;
}

int cflbm_get_info(cflbm_handle *h, cflbm_info *info) {
  if (!h || !info) return fail(CFLBM_E_INVALID, "bad arguments");
  std::memset(info, 0, sizeof(*info));
  info->lattice = h->Q;
  info->nx = h->L.nx;
  info->ny = h->L.ny;
  info->nz = h->L.nz;
  info->storage = h->cfg.storage;
  info->compute = h->cfg.compute;
  info->profile = h->cfg.profile;
  info->ghost = h->L.G;
  info->pitch_x = h->L.px;
  info->pop_stride = h->L.S;
  info->layout = h->cfg.layout;
  info->steps_done = h->steps_done;
  info->n_links = h->n_links;
  info->n_solid = h->n_solid;
  info->omega = h->omega;
  info->bytes_per_cell_step = 2.0 * h->Q * h->esize + 0.125;
  info->device_bytes = h->device_bytes;
  return CFLBM_OK;
}

int cflbm_write_tecplot(cflbm_handle *h, const char *path, int n) {
  if (!h || !path) return fail(CFLBM_E_INVALID, "bad arguments");
  const size_t N = (size_t)h->L.nx * h->L.ny * h->L.nz;
  std::vector<double> u(N), v(N), w(N), p(N);
  int rc = cflbm_macros(h, u.data(), v.data(), w.data(), p.data());
  if (rc) return rc;
  rc = write_tecplot(path, h->Q == 27 ? 3 : 2, h->L.nx, h->L.ny, h->L.nz, u.data(), v.data(),
                     w.data(), p.data(), n);
  if (rc) return fail(rc, "writing %s failed", path);
  return CFLBM_OK;
}

int cflbm_get_stream(cflbm_handle *h, void **stream) {
  if (!h || !stream) return fail(CFLBM_E_INVALID, "bad arguments");
  *stream = (void *)h->stream;
  return CFLBM_OK;
}

int cflbm_set_timing(cflbm_handle *h, int enable) {
  if (!h) return fail(CFLBM_E_INVALID, "handle is NULL");
  h->timing = enable != 0;
  return CFLBM_OK;
}

int cflbm_get_timing(cflbm_handle *h, double ms[2], int64_t counts[2]) {
  if (!h || !ms || !counts) return fail(CFLBM_E_INVALID, "bad arguments");
  CK_CUDA(cudaSetDevice(h->cfg.device));
  CK_CUDA(cudaStreamSynchronize(h->stream));
  double tot[2] = {0.0, 0.0};
  const std::vector<std::pair<size_t, size_t>> *lists[2] = {&h->sweep_ev, &h->bnd_ev};
  for (int k = 0; k < 2; ++k)
    for (const auto &pr : *lists[k]) {
      float t = 0.f;
      CK_CUDA(cudaEventElapsedTime(&t, h->ev_pool[pr.first], h->ev_pool[pr.second]));
      tot[k] += t;
    }
  ms[0] = tot[0];
  ms[1] = tot[1];
  counts[0] = (int64_t)h->sweep_ev.size();
  counts[1] = (int64_t)h->bnd_ev.size();
  h->sweep_ev.clear();
  h->bnd_ev.clear();
  h->ev_used = 0;
  return CFLBM_OK;
}

int cflbm_write_tecplot_fields(const char *path, int dim, int nx, int ny, int nz,
                               const double *u, const double *v, const double *w,
                               const double *p, int n) {
  if (!path || !u || !v || !p || (dim == 3 && !w) || (dim != 2 && dim != 3) || nx < 2 ||
      ny < 2 || (dim == 3 && nz < 2))
    return fail(CFLBM_E_INVALID, "bad arguments");
  int rc = write_tecplot(path, dim, nx, ny, dim == 3 ? nz : 1, u, v, w, p, n);
  if (rc) return fail(rc, "writing %s failed", path);
  return CFLBM_OK;
}

}  // extern "C"

namespace cflbm {
// Error reporting for entry points defined in other translation units.
int record_error(int code, const char *msg) { return fail(code, "%s", msg); }
}  // namespace cflbm
