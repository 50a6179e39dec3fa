// Channel-profile set-up on the GPU: the bit-packed solid mask, the per-cell
// solid-link bits, the listed warp tiles (rows on a y/z face, or holding a
// solid cell or a cell with solid links) in tile order, and their link words.
//
// Host passes over every cell took 21-26 ms for a 8.4 M-cell grid on 16 host
// cores; here they are five launches over the grid and one read-back of three
// counts (the number of listed tiles sizes two buffers).  The list is ordered
// by tile, so the force sums over it run in tile order, as they always have.
// Link bits: bit i of cell X is set when the source of population i, X - e_i
// mapped onto the box as the sweep maps it (periodic wrap, free-slip mirror,
// no-slip wall, inlet, zero-gradient outlet), is a solid cell -- when the sweep
// bounces population i back.
#include "handle.hpp"
#include "setup.cuh"

namespace cflbm {
namespace {

constexpr int SETUP_THREADS = 256;
constexpr int TILES_PER_THREAD = 4;
constexpr int TILES_PER_CHUNK = SETUP_THREADS * TILES_PER_THREAD;

__device__ __forceinline__ bool geom_solid(const SetupArgs &s, int x, int y, int z) {
  if (s.geom != 1 && s.geom != 2) return false;
  // the host's expression order, no contraction: (dx dx + dy dy) (+ dz dz) <= r2
  const double dx = __dsub_rn((double)x, s.cx), dy = __dsub_rn((double)y, s.cy);
  double d = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  if (s.geom == 2) {
    const double dz = __dsub_rn((double)z, s.cz);
    d = __dadd_rn(d, __dmul_rn(dz, dz));
  }
  return d <= s.r2;
}

__device__ __forceinline__ bool is_solid(const uint32_t *mask, int nxw, int ny, int x, int y,
                                         int z) {
  return (mask[((long long)z * ny + y) * nxw + (x >> 5)] >> (x & 31)) & 1u;
}

// One thread per 32-cell mask word; counts the solid cells.
__global__ void mask_words_kernel(const SetupArgs s, uint32_t *mask,
                                  unsigned long long *counters) {
  const long long W = (long long)s.nxw * s.ny * s.nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < W;
       t += (long long)gridDim.x * blockDim.x) {
    const long long r = t / s.nxw;
    const int w = (int)(t % s.nxw);
    const int y = (int)(r % s.ny), z = (int)(r / s.ny);
    unsigned bits = 0u;
    for (int l = 0; l < 32; ++l) {
      const int x = 32 * w + l;
      if (x >= s.nx) break;
      const bool sol = s.solid_in ? s.solid_in[r * s.nx + x] != 0 : geom_solid(s, x, y, z);
      bits |= (sol ? 1u : 0u) << l;
    }
    mask[t] = bits;
    if (bits) atomicAdd(&counters[0], (unsigned long long)__popc(bits));
  }
}

// One thread per cell: bit i set when the source of population i, mapped onto
// the box as the sweep maps it, is solid; counts the reference-rule links
// (solid cell s, direction k, s + e_k a fluid cell of the box).
template <int Q>
__global__ void link_bits_kernel(const SetupArgs s, const uint32_t *mask, uint32_t *bits,
                                 unsigned long long *counters) {
  using L = Lat<Q>;
  const long long N = (long long)s.nx * s.ny * s.nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N;
       t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % s.nx);
    const int y = (int)((t / s.nx) % s.ny);
    const int z = (int)(t / ((long long)s.nx * s.ny));
    unsigned b = 0u;
#pragma unroll
    for (int i = 1; i < Q; ++i) {
      int sx = x - L::ex(i), sy = y - L::ey(i), sz = z - L::ez(i);
      if (Q == 27 && (sz < 0 || sz >= s.nz)) {
        if (s.wall_z == WALL_PERIODIC) sz = (sz + s.nz) % s.nz;
        else if (s.wall_z == WALL_FREESLIP) sz = z;
        else continue;  // no-slip wall, not the body
      }
      if (sy < 0 || sy >= s.ny) {
        if (s.wall_y == WALL_PERIODIC) sy = (sy + s.ny) % s.ny;
        else if (s.wall_y == WALL_FREESLIP) sy = y;
        else continue;
      }
      if (sx < 0) continue;  // inlet
      if (sx >= s.nx) sx = s.nx - 1;
      if (is_solid(mask, s.nxw, s.ny, sx, sy, sz)) b |= 1u << i;
    }
    bits[t] = b;
    if (is_solid(mask, s.nxw, s.ny, x, y, z)) {
      unsigned n = 0u;
#pragma unroll
      for (int k = 1; k < Q; ++k) {
        const int X = x + L::ex(k), Y = y + L::ey(k), Z = z + L::ez(k);
        if (X < 0 || X >= s.nx || Y < 0 || Y >= s.ny || Z < 0 || Z >= s.nz) continue;
        if (!is_solid(mask, s.nxw, s.ny, X, Y, Z)) ++n;
      }
      if (n) atomicAdd(&counters[1], (unsigned long long)n);
    }
  }
}

__device__ __forceinline__ bool tile_listed(const SetupArgs &s, const uint32_t *mask,
                                            const uint32_t *bits, long long t) {
  const long long r = t / s.nxw;
  const int w = (int)(t % s.nxw);
  const int y = (int)(r % s.ny), z = (int)(r / s.ny);
  if (y == 0 || y == s.ny - 1 || (s.nz > 1 && (z == 0 || z == s.nz - 1))) return true;
  if (mask[t]) return true;
  const int x1 = min(s.nx, 32 * w + 32);
  for (int x = 32 * w; x < x1; ++x)
    if (bits[r * s.nx + x]) return true;
  return false;
}

// Block-wide exclusive prefix sum of one int per thread (SETUP_THREADS).
__device__ __forceinline__ int block_exclusive_sum(int v, int *sh, int &total) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  int incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int n = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += n;
  }
  if (lane == 31) sh[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int ws = lane < SETUP_THREADS / 32 ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int n = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += n;
    }
    if (lane < SETUP_THREADS / 32) sh[lane] = ws;  // inclusive warp sums
  }
  __syncthreads();
  total = sh[SETUP_THREADS / 32 - 1];
  const int before = wid > 0 ? sh[wid - 1] : 0;
  __syncthreads();
  return before + incl - v;
}

// Per chunk of TILES_PER_CHUNK tiles: the listed flags and their count.
__global__ void tile_flags_kernel(const SetupArgs s, const uint32_t *mask, const uint32_t *bits,
                                  unsigned char *flag, int *chunk_count) {
  __shared__ int sh[SETUP_THREADS / 32];
  const long long T = (long long)s.nxw * s.ny * s.nz;
  const long long t0 = (long long)blockIdx.x * TILES_PER_CHUNK + threadIdx.x * TILES_PER_THREAD;
  int n = 0;
  for (int k = 0; k < TILES_PER_THREAD; ++k) {
    const long long t = t0 + k;
    if (t >= T) break;
    const bool f = tile_listed(s, mask, bits, t);
    flag[t] = f ? 1 : 0;
    n += f ? 1 : 0;
  }
  int total;
  (void)block_exclusive_sum(n, sh, total);
  if (threadIdx.x == 0) chunk_count[blockIdx.x] = total;
}

// One block: chunk counts -> exclusive offsets (in place); the total into *total.
__global__ void chunk_scan_kernel(int *chunk, int nchunks, int *total) {
  __shared__ int sh[SETUP_THREADS / 32];
  int carry = 0;
  for (int base = 0; base < nchunks; base += SETUP_THREADS) {
    const int c = base + (int)threadIdx.x;
    const int v = c < nchunks ? chunk[c] : 0;
    int sum;
    const int ex = block_exclusive_sum(v, sh, sum);
    if (c < nchunks) chunk[c] = carry + ex;
    carry += sum;
  }
  if (threadIdx.x == 0) *total = carry;
}

// Per chunk: the listed tiles' positions (tile order), the list and the link
// words (bit 31: solid cell).
__global__ void tile_list_kernel(const SetupArgs s, const unsigned char *flag,
                                 const int *chunk_off, const uint32_t *mask,
                                 const uint32_t *bits, int *tile_index, int *list,
                                 uint32_t *links_bits) {
  __shared__ int sh[SETUP_THREADS / 32];
  const long long T = (long long)s.nxw * s.ny * s.nz;
  const long long t0 = (long long)blockIdx.x * TILES_PER_CHUNK + threadIdx.x * TILES_PER_THREAD;
  int n = 0;
  for (int k = 0; k < TILES_PER_THREAD; ++k)
    if (t0 + k < T && flag[t0 + k]) ++n;
  int total;
  int pos = chunk_off[blockIdx.x] + block_exclusive_sum(n, sh, total);
  for (int k = 0; k < TILES_PER_THREAD; ++k) {
    const long long t = t0 + k;
    if (t >= T) break;
    if (!flag[t]) {
      tile_index[t] = -1;
      continue;
    }
    tile_index[t] = pos;
    list[pos] = (int)t;
    const long long r = t / s.nxw;
    const int w = (int)(t % s.nxw);
    const unsigned m = mask[t];
    for (int l = 0; l < 32; ++l) {
      const int x = 32 * w + l;
      links_bits[(long long)pos * 32 + l] =
          x < s.nx ? bits[r * s.nx + x] | (((m >> l) & 1u) << 31) : 0u;
    }
    ++pos;
  }
}

// One warp per listed tile t: cnt[t] = its fluid cells with solid links.
__global__ void bcell_count_kernel(int n_slow, const uint32_t *links_bits, unsigned char *cnt) {
  const long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= n_slow) return;  // warp-uniform
  const unsigned word = links_bits[t * 32 + lane];
  const unsigned b =
      __ballot_sync(0xffffffffu, (word & 0x7fffffffu) != 0u && !(word >> 31));
  if (lane == 0) cnt[t] = (unsigned char)__popc(b);
}

// Per chunk of TILES_PER_CHUNK tiles: the sum of their counts.
__global__ void bcell_chunk_kernel(int n, const unsigned char *cnt, int *chunk) {
  __shared__ int sh[SETUP_THREADS / 32];
  const long long t0 = (long long)blockIdx.x * TILES_PER_CHUNK + threadIdx.x * TILES_PER_THREAD;
  int c = 0;
  for (int k = 0; k < TILES_PER_THREAD; ++k)
    if (t0 + k < n) c += cnt[t0 + k];
  int total;
  (void)block_exclusive_sum(c, sh, total);
  if (threadIdx.x == 0) chunk[blockIdx.x] = total;
}

// Per chunk: its tiles' boundary cells at the chunk's offset, in tile and
// then x order: the storage index and the link word of each.
__global__ void bcell_list_kernel(const Layout L, int nxw, int n, const int *list,
                                  const uint32_t *links_bits, const unsigned char *cnt,
                                  const int *chunk, long long *cell, uint32_t *words) {
  __shared__ int sh[SETUP_THREADS / 32];
  const long long t0 = (long long)blockIdx.x * TILES_PER_CHUNK + threadIdx.x * TILES_PER_THREAD;
  int c = 0;
  for (int k = 0; k < TILES_PER_THREAD; ++k)
    if (t0 + k < n) c += cnt[t0 + k];
  int total;
  int pos = chunk[blockIdx.x] + block_exclusive_sum(c, sh, total);
  for (int k = 0; k < TILES_PER_THREAD; ++k) {
    const long long t = t0 + k;
    if (t >= n || !cnt[t]) continue;
    const int tile = list[t];
    const int row = tile / nxw;
    const long long c0 = L.idx((tile % nxw) * 32, row % L.ny, row / L.ny);
    for (int l = 0; l < 32; ++l) {
      const uint32_t w = links_bits[t * 32 + l];
      if ((w & 0x7fffffffu) && !(w >> 31)) {
        cell[pos] = c0 + l;
        words[pos] = w;
        ++pos;
      }
    }
  }
}

int grid_for(long long n) {
  long long b = (n + SETUP_THREADS - 1) / SETUP_THREADS;
  return (int)std::max<long long>(1, std::min<long long>(b, 65535LL * 16));
}

}  // namespace

int setup_chunks(const SetupArgs &s) {
  const long long T = (long long)s.nxw * s.ny * s.nz;
  return (int)((T + TILES_PER_CHUNK - 1) / TILES_PER_CHUNK);
}

cudaError_t launch_setup_mask_links(int Q, const SetupArgs &s, uint32_t *mask, uint32_t *bits,
                                    unsigned long long *counters, cudaStream_t st) {
  mask_words_kernel<<<grid_for((long long)s.nxw * s.ny * s.nz), SETUP_THREADS, 0, st>>>(
      s, mask, counters);
  const int g = grid_for((long long)s.nx * s.ny * s.nz);
  if (Q == 27) link_bits_kernel<27><<<g, SETUP_THREADS, 0, st>>>(s, mask, bits, counters);
  else link_bits_kernel<9><<<g, SETUP_THREADS, 0, st>>>(s, mask, bits, counters);
  count_launch(2);
  return cudaGetLastError();
}

cudaError_t launch_setup_flags(const SetupArgs &s, const uint32_t *mask, const uint32_t *bits,
                               unsigned char *flag, int *chunk, int *total, cudaStream_t st) {
  const int nchunks = setup_chunks(s);
  tile_flags_kernel<<<nchunks, SETUP_THREADS, 0, st>>>(s, mask, bits, flag, chunk);
  chunk_scan_kernel<<<1, SETUP_THREADS, 0, st>>>(chunk, nchunks, total);
  count_launch(2);
  return cudaGetLastError();
}

cudaError_t launch_setup_list(const SetupArgs &s, const unsigned char *flag, const int *chunk,
                              const uint32_t *mask, const uint32_t *bits, int *tile_index,
                              int *list, uint32_t *links_bits, cudaStream_t st) {
  tile_list_kernel<<<setup_chunks(s), SETUP_THREADS, 0, st>>>(s, flag, chunk, mask, bits,
                                                               tile_index, list, links_bits);
  count_launch();
  return cudaGetLastError();
}

int bcell_chunks(int n_slow) {
  return std::max(1, (n_slow + TILES_PER_CHUNK - 1) / TILES_PER_CHUNK);
}

cudaError_t launch_setup_bcell_count(int n_slow, const uint32_t *links_bits, unsigned char *cnt,
                                     int *chunk, int *total, cudaStream_t st) {
  const int nchunks = bcell_chunks(n_slow);
  if (n_slow > 0)
    bcell_count_kernel<<<(unsigned)((32LL * n_slow + SETUP_THREADS - 1) / SETUP_THREADS),
                         SETUP_THREADS, 0, st>>>(n_slow, links_bits, cnt);
  bcell_chunk_kernel<<<nchunks, SETUP_THREADS, 0, st>>>(n_slow, cnt, chunk);
  chunk_scan_kernel<<<1, SETUP_THREADS, 0, st>>>(chunk, nchunks, total);
  count_launch(n_slow > 0 ? 3 : 2);
  return cudaGetLastError();
}

cudaError_t launch_setup_bcell_list(const Layout &L, int nxw, int n_slow, const int *list,
                                    const uint32_t *links_bits, const unsigned char *cnt,
                                    const int *chunk, long long *cell, uint32_t *words,
                                    cudaStream_t st) {
  bcell_list_kernel<<<bcell_chunks(n_slow), SETUP_THREADS, 0, st>>>(L, nxw, n_slow, list,
                                                                   links_bits, cnt, chunk,
                                                                   cell, words);
  count_launch();
  return cudaGetLastError();
}

}  // namespace cflbm
