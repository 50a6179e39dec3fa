// cflbm_domain_sums_noalloc: the FP64 domain-sum reduction (mass and momentum)
// for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- inside a host
// allocator callback or a custom memory pool that owns every device byte,
// during CUDA graph construction by a framework that forbids allocation, or in
// a process whose memory budget is fixed in advance -- but that already holds
// the populations in device memory and wants the conservation check.
// cflbm_mass() needs a handle, and creating a handle allocates.
//
// This entry point allocates nothing.  Its per-block partial sums and the
// completion counter live in one file-scope __device__ array of
// NOALLOC_SCRATCH_DOUBLES doubles (512 KiB plus the counter), which every GPU
// that loads this library holds until the process exits.  The array's name in
// host code is only a host-side stand-in, not a device address, so the first
// call on each device looks the device address up with cudaGetSymbolAddress
// (with that device current) and caches it; make that first call before any
// stream capture.  All calls share the array: the counter is cleared on the
// caller's stream before each launch, and calls that overlap on the GPU race.
#include <cstdio>
#include <mutex>
#include "handle.hpp"

namespace cflbm {
namespace {

// 16384 blocks x 4 partial sums, then the completion counter.
constexpr int NOALLOC_MAX_BLOCKS = 16384;
constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_CELLS_PER_THREAD = 32;
constexpr long long NOALLOC_CELLS_PER_BLOCK =
    (long long)NOALLOC_THREADS * NOALLOC_CELLS_PER_THREAD;
constexpr long long NOALLOC_MAX_CELLS = NOALLOC_MAX_BLOCKS * NOALLOC_CELLS_PER_BLOCK;
constexpr int NOALLOC_SCRATCH_DOUBLES = 4 * NOALLOC_MAX_BLOCKS + 32;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

template <int Q, class ST>
__device__ double decode(const typename Store<ST>::elem v, int i) {
  if constexpr (sizeof(typename Store<ST>::elem) == 2)
    return (double)__half2float(v) / (double)Lat<Q>::h_scale(i);
  else
    return (double)v;
}

// Same reduction as the handle's mass kernel (boundary.cu), over a dense
// [i][z][y][x] array: each block sums NOALLOC_CELLS_PER_BLOCK cells into four
// FP64 partials; the last block to finish adds the partials in block order.
template <int Q, class ST>
__global__ void __launch_bounds__(NOALLOC_THREADS)
    domain_sums_static_kernel(const typename Store<ST>::elem *f, const uint8_t *solid,
                              long long N, double *scratch, double *out) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const long long base = (long long)blockIdx.x * NOALLOC_CELLS_PER_BLOCK;
  for (int k = 0; k < NOALLOC_CELLS_PER_THREAD; ++k) {
    const long long n = base + (long long)k * NOALLOC_THREADS + threadIdx.x;
    if (n >= N) break;
    if (solid && solid[n]) continue;
    double r = 1.0;
    for (int i = 0; i < Q; ++i) {
      const double fi = decode<Q, ST>(f[(long long)i * N + n], i);
      r += fi;
      acc[1] += fi * Lat<Q>::ex(i);
      acc[2] += fi * Lat<Q>::ey(i);
      acc[3] += fi * Lat<Q>::ez(i);
    }
    acc[0] += r;
  }
  __shared__ double sh[4][NOALLOC_THREADS / 32];
  __shared__ bool last;
  for (int o = 16; o > 0; o >>= 1)
    for (int q = 0; q < 4; ++q) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    for (int q = 0; q < 4; ++q) sh[q][wid] = acc[q];
  __syncthreads();
  unsigned int *counter = reinterpret_cast<unsigned int *>(scratch + 4 * NOALLOC_MAX_BLOCKS);
  if (threadIdx.x == 0) {
    for (int q = 0; q < 4; ++q) {
      double b = 0.0;
      for (int w = 0; w < NOALLOC_THREADS / 32; ++w) b += sh[q][w];
      scratch[4 * blockIdx.x + q] = b;
    }
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {  // uniform per block: the whole last block adds the partials
    __threadfence();
    const volatile double *p = scratch;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += NOALLOC_THREADS)
      for (int q = 0; q < 4; ++q) s[q] += p[4 * b + q];
    for (int o = 16; o > 0; o >>= 1)
      for (int q = 0; q < 4; ++q) s[q] += __shfl_down_sync(0xffffffffu, s[q], o);
    __syncthreads();
    if (lane == 0)
      for (int q = 0; q < 4; ++q) sh[q][wid] = s[q];
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int q = 0; q < 4; ++q) {
        double t = 0.0;
        for (int w = 0; w < NOALLOC_THREADS / 32; ++w) t += sh[q][w];
        out[q] = t;
      }
      *counter = 0u;
    }
  }
}

// Device address of g_noalloc_scratch, looked up once per device.
std::mutex g_scratch_mu;
double *g_scratch_ptr[64] = {nullptr};

cudaError_t scratch_for_current_device(double **ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *ptr = g_scratch_ptr[dev];
  return cudaSuccess;
}

}  // namespace
}  // namespace cflbm

using namespace cflbm;

namespace cflbm {
int record_error(int code, const char *msg);  // api.cu: sets cflbm_last_error()
}

static int cflbm_noalloc_fail(int code, const char *msg) { return record_error(code, msg); }

extern "C" int cflbm_domain_sums_noalloc(int lattice, int storage, int nx, int ny, int nz,
                                         const void *d_f, const uint8_t *d_solid,
                                         double *d_out, void *stream) {
  if (lattice != 9 && lattice != 27)
    return cflbm_noalloc_fail(CFLBM_E_INVALID, "lattice must be 9 or 27");
  if (storage < 0 || storage > 2) return cflbm_noalloc_fail(CFLBM_E_INVALID, "unknown storage");
  if (!d_f || !d_out) return cflbm_noalloc_fail(CFLBM_E_INVALID, "d_f and d_out are required");
  if (nx < 1 || ny < 1 || nz < 1 || (lattice == 9 && nz != 1))
    return cflbm_noalloc_fail(CFLBM_E_INVALID, "bad grid size");
  const long long N = (long long)nx * ny * nz;
  if (N > NOALLOC_MAX_CELLS) {
    char msg[160];
    std::snprintf(msg, sizeof(msg),
                  "grid of %lld cells exceeds the %lld-cell limit of the static scratch",
                  N, NOALLOC_MAX_CELLS);
    return cflbm_noalloc_fail(CFLBM_E_INVALID, msg);
  }
  double *scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess) return cflbm_noalloc_fail(CFLBM_E_CUDA, cudaGetErrorString(e));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  e = cudaMemsetAsync(scratch + 4 * NOALLOC_MAX_BLOCKS, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return cflbm_noalloc_fail(CFLBM_E_CUDA, cudaGetErrorString(e));
  const int blocks = (int)((N + NOALLOC_CELLS_PER_BLOCK - 1) / NOALLOC_CELLS_PER_BLOCK);
#define CFLBM_NA_LAUNCH(QQ, ST)                                                              \
  domain_sums_static_kernel<QQ, ST><<<blocks, NOALLOC_THREADS, 0, s>>>(                       \
      static_cast<const typename Store<ST>::elem *>(d_f), d_solid, N, scratch, d_out)
  if (lattice == 9) {
    if (storage == CFLBM_STORE_FP64) CFLBM_NA_LAUNCH(9, double);
    else if (storage == CFLBM_STORE_FP32) CFLBM_NA_LAUNCH(9, float);
    else CFLBM_NA_LAUNCH(9, F16Dev);
  } else {
    if (storage == CFLBM_STORE_FP64) CFLBM_NA_LAUNCH(27, double);
    else if (storage == CFLBM_STORE_FP32) CFLBM_NA_LAUNCH(27, float);
    else CFLBM_NA_LAUNCH(27, F16Dev);
  }
#undef CFLBM_NA_LAUNCH
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return cflbm_noalloc_fail(CFLBM_E_CUDA, cudaGetErrorString(e));
  return CFLBM_OK;
}
