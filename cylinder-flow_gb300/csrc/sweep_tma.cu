// Channel interior sweep for FP16-deviation storage fed by the Tensor Memory
// Accelerator (FP32 collision, ROWS layout f[z][y][i][x]).
//
// With 2-byte populations a warp-wide load moves only 64 bytes, so the direct
// interior kernel cannot keep enough bytes in flight (it is latency-bound at
// about two thirds of the copy peak).  Here the loads are bulk tensor copies:
//   * a tile is 128 cells in x (four warp tiles) by BY rows of one z plane; the
//     host lists the tiles with at least one unlisted 32-cell row segment
//     (listed segments -- y/z faces, rows next to a body -- stay with the
//     resolving kernel, which runs beside this one);
//   * a producer warp issues, per tile, Q TMA loads (one per population: box
//     (128 + 2H) x BY rows, shifted by -e_i in y and z, H = 8 halo cells in x
//     so every box starts on a 16-byte boundary; rows of 288 bytes) into a
//     STAGES-deep ring of shared buffers, each completing an mbarrier;
//   * consumer warp (row, pair) reads cells x and x + 32 of its row at
//     compile-time shared offsets (inlet and outlet columns by select),
//     collides both with packed FP32x2 arithmetic (channel2 cell code) and
//     stores to global memory directly;
//   * persistent CTAs take tiles grid-stride, so at any moment all CTAs stream
//     one band of the box and the neighbour rows of the pulls stay in L2.
// Every mbarrier wait is bounded (about 2 s of SM clock); on expiry the thread
// sets the handle's error flag and stops taking work, and the producer waits
// (bounded) for the copies it has issued before the block exits.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <algorithm>
#include <vector>
#include "handle.hpp"
#include "sweep.cuh"

namespace cflbm {

namespace {

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and the error flag set) after ~2^32 SM clocks.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, int *err) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > (1LL << 32)) {
      atomicOr(err, 1);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, int c3, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
      "r"(smem_u32(bar))
      : "memory");
}

constexpr int TBX = 128;      // tile width (cells)
constexpr int TH = 8;         // x halo (cells): 16 bytes of FP16
constexpr int TBXL = TBX + 2 * TH;
constexpr int TBY = 4;        // tile rows
constexpr int TSTAGES = 3;
constexpr int TCONS = 2 * TBY;  // consumer warps: (row, pair of warp tiles)

template <int Q>
struct TmaGeom {
  static constexpr int POP = TBXL * TBY * 2;  // bytes of one population box
  static constexpr int STAGE = Q * POP;
  static constexpr size_t SMEM = (size_t)TSTAGES * STAGE + 2 * TSTAGES * sizeof(uint64_t);
  static_assert(POP % 128 == 0, "population boxes must stay 128-byte aligned");
};

template <int Q>
__global__ void __launch_bounds__(32 * (TCONS + 1))
    sweep_tma16_kernel(const SweepArgs a, const __grid_constant__ CUtensorMap tm,
                       const int4 *__restrict__ tiles, int n_tiles, int *err) {
  using L = Lat<Q>;
  using SF = Store<F16Dev>;
  using G = TmaGeom<Q>;
  using O = VA<float2>;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + TSTAGES * G::STAGE);
  uint64_t *empty = full + TSTAGES;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TSTAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], TCONS);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int gx = a.L.xoff, gy = a.L.G, gz = a.L.Gz;

  if (warp == TCONS) {
    // ---- producer ---------------------------------------------------------------
    if (lane != 0) return;
    int issued = 0;
    for (int n = blockIdx.x; n < n_tiles; n += gridDim.x, ++issued) {
      const int s = issued % TSTAGES, k = issued / TSTAGES;
      if (k > 0 && !mbar_wait(&empty[s], (k - 1) & 1, err)) break;
      if (*(volatile int *)err) break;
      const int4 t = tiles[n];  // (x0, y0, z, segment mask)
      unsigned char *in = smem + s * G::STAGE;
      mbar_expect_tx(&full[s], G::STAGE);
      static_for(
          [&](auto ic) {
            constexpr int I = decltype(ic)::value;
            tma_load_4d(in + I * G::POP, &tm, gx + t.x - TH, I, gy + t.y - L::ey(I),
                        gz + t.z - L::ez(I), &full[s]);
          },
          std::make_integer_sequence<int, Q>{});
    }
    // Copies still in flight (work abandoned after an error) must land before
    // the block's shared memory goes away.
    for (int m = std::max(0, issued - TSTAGES); m < issued; ++m)
      mbar_wait(&full[m % TSTAGES], (m / TSTAGES) & 1, err);
    return;
  }

  // ---- consumers: warp = (row ly, pair pr): cells x0 + 64 pr + lane and + 32 ----
  const int ly = warp >> 1, pr = warp & 1;
  const int nx = a.L.nx, ny = a.L.ny;
  const long long S = a.L.S;
  int done = 0;
  for (int n = blockIdx.x; n < n_tiles; n += gridDim.x, ++done) {
    const int s = done % TSTAGES, k = done / TSTAGES;
    if (!mbar_wait(&full[s], k & 1, err)) break;
    const int4 t = tiles[n];
    const bool act0 = (t.w >> (4 * ly + 2 * pr)) & 1;
    const bool act1 = (t.w >> (4 * ly + 2 * pr + 1)) & 1;
    if (act0 || act1) {  // warp-uniform
      const __half *in = reinterpret_cast<const __half *>(smem + s * G::STAGE) + ly * TBXL +
                         TH + 64 * pr + lane;
      const int x0 = t.x + 64 * pr + lane, x1 = x0 + 32;
      const int y = t.y + ly, z = t.z;
      const bool inlet0 = x0 == 0;
      const int out0 = x0 == nx - 1 ? 1 : 0, out1 = x1 == nx - 1 ? 1 : 0;
      float2 f[Q];
      static_for(
          [&](auto ic) {
            constexpr int I = decltype(ic)::value;
            constexpr int ex = L::ex(I);
            constexpr int base = I * TBY * TBXL - ex;
            float v0, v1;
            if constexpr (ex < 0) {  // zero gradient: the outlet column reads itself
              v0 = __half2float(in[base - out0]);
              v1 = __half2float(in[base + 32 - out1]);
            } else {
              v0 = __half2float(in[base]);
              v1 = __half2float(in[base + 32]);
            }
            if constexpr (ex > 0) v0 = inlet0 ? a.f_in_f[I] : v0;
            f[I] = make_float2(v0, v1);
          },
          std::make_integer_sequence<int, Q>{});
      // The stage may be refilled as soon as every consumer warp has its values.
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      const bool st0 = act0 && x0 < nx, st1 = act1 && x1 < nx;
      float2 rho3, ux, uy, uz;
      moments<L, float2, SF>(f, rho3, ux, uy, uz);
      const long long cell0 = ((long long)z * ny + y) * nx + x0;
      if (a.mu) {
        if (st0) {
          a.mu[cell0] = f2d_bits(ux.x);
          a.mv[cell0] = f2d_bits(uy.x);
          a.mw[cell0] = f2d_bits(uz.x);
          a.mp[cell0] = f2d_bits(__fmul_rn(rho3.x, 1.0f / 3.0f));
        }
        if (st1) {
          a.mu[cell0 + 32] = f2d_bits(ux.y);
          a.mv[cell0 + 32] = f2d_bits(uy.y);
          a.mw[cell0 + 32] = f2d_bits(uz.y);
          a.mp[cell0 + 32] = f2d_bits(__fmul_rn(rho3.y, 1.0f / 3.0f));
        }
      }
      if (a.alpha) {
        const float2 sb = make_float2(__fsub_rn(1.0f, st0 ? a.alpha[cell0] : 0.0f),
                                      __fsub_rn(1.0f, st1 ? a.alpha[cell0 + 32] : 0.0f));
        ux = O::mul(ux, sb);
        uy = O::mul(uy, sb);
        uz = O::mul(uz, sb);
      }
      bgk_relax_v<L, float2, SF>(f, rho3, ux, uy, uz, O::splat(a.omega_f));
      __half *q = static_cast<__half *>(a.fb) + a.L.idx(x0, y, z);
#pragma unroll
      for (int i = 0; i < Q; ++i) {
        if (st0) q[i * S] = __float2half_rn(f[i].x);
        if (st1) q[i * S + 32] = __float2half_rn(f[i].y);
      }
    } else {
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
    }
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

template <int Q>
cudaError_t tma_prepare(int *blocks_per_sm) {
  auto kern = sweep_tma16_kernel<Q>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)TmaGeom<Q>::SMEM);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kern, 32 * (TCONS + 1),
                                                       TmaGeom<Q>::SMEM);
}

}  // namespace

// Tiles and tensor maps of a channel handle with FP16 storage, FP32 collision
// and the ROWS layout; leaves h->tma false otherwise (the direct interior
// kernel then runs).  row_listed: per 32-cell row segment, 1 = listed.
int tma_setup(cflbm_handle *h, const std::vector<unsigned char> &row_listed) {
  h->tma = false;
  const cflbm_config &c = h->cfg;
  if (c.profile != CFLBM_PROFILE_CHANNEL || c.layout != CFLBM_LAYOUT_ROWS ||
      c.compute != CFLBM_COMPUTE_FP32 || c.storage != CFLBM_STORE_FP16DEV)
    return CFLBM_OK;
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return CFLBM_OK;
  const Layout &L = h->L;
  const int Q = h->Q, nz = L.nz, ny = L.ny, nxw = h->nxw;
  std::vector<int4> tiles;
  for (int z = 0; z < nz; ++z)
    for (int y0 = 0; y0 < ny; y0 += TBY)
      for (int x0 = 0; x0 < 32 * nxw; x0 += TBX) {
        int mask = 0;
        for (int r = 0; r < TBY && y0 + r < ny; ++r)
          for (int g = 0; g < TBX / 32; ++g) {
            const int w = x0 / 32 + g;
            if (w < nxw && !row_listed[((size_t)z * ny + (y0 + r)) * nxw + w])
              mask |= 1 << (4 * r + g);
          }
        if (mask) tiles.push_back(make_int4(x0, y0, z, mask));
      }
  int bps = 0;
  cudaError_t e = Q == 9 ? tma_prepare<9>(&bps) : tma_prepare<27>(&bps);
  if (e != cudaSuccess || bps < 1) {
    cudaGetLastError();
    return CFLBM_OK;
  }
  const cuuint64_t dims[4] = {(cuuint64_t)L.px, (cuuint64_t)Q, (cuuint64_t)L.nyp,
                              (cuuint64_t)L.nzp};
  const cuuint64_t strides[3] = {(cuuint64_t)L.px * 2, (cuuint64_t)L.rs * 2,
                                 (cuuint64_t)L.zs * 2};
  const cuuint32_t box[4] = {(cuuint32_t)TBXL, 1, (cuuint32_t)TBY, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  for (int b = 0; b < 2; ++b)
    if (enc(&h->tma_map[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 4, h->buf[b], dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return CFLBM_OK;
  if (!tiles.empty()) {
    if (cudaMalloc(&h->d_tma_tiles, tiles.size() * sizeof(int4)) != cudaSuccess)
      return record_error(CFLBM_E_NOMEM, "cudaMalloc of the TMA tile list failed");
    if (cudaMemcpy(h->d_tma_tiles, tiles.data(), tiles.size() * sizeof(int4),
                   cudaMemcpyHostToDevice) != cudaSuccess)
      return record_error(CFLBM_E_CUDA, "copy of the TMA tile list failed");
  }
  h->tma_tiles_n = (int)tiles.size();
  h->tma_grid = h->sms * bps;
  h->tma = true;
  return CFLBM_OK;
}

// The interior launch of a channel step through the TMA kernel (src: index of
// the buffer being read, 0 or 1).
cudaError_t launch_sweep_tma(const cflbm_handle *h, const SweepArgs &a, int src, cudaStream_t s) {
  if (h->tma_tiles_n == 0) return cudaSuccess;
  const int grid = std::max(1, std::min(h->tma_tiles_n, h->tma_grid));
  if (h->Q == 9)
    sweep_tma16_kernel<9><<<grid, 32 * (TCONS + 1), TmaGeom<9>::SMEM, s>>>(
        a, h->tma_map[src], h->d_tma_tiles, h->tma_tiles_n, h->d_err);
  else
    sweep_tma16_kernel<27><<<grid, 32 * (TCONS + 1), TmaGeom<27>::SMEM, s>>>(
        a, h->tma_map[src], h->d_tma_tiles, h->tma_tiles_n, h->d_err);
  count_launch(1);
  return cudaGetLastError();
}

}  // namespace cflbm
