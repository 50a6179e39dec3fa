// Launcher of the line-staged channel sweep (sweep_lines.cuh): D3Q27, FP16
// deviation storage, ROWS layout.
#include <algorithm>
#include "sweep_lines.cuh"

namespace cflbm {

namespace {
// Bytes of one ring stage for a line of nx cells: the Q staged rows, the link
// words and positions of the line's tiles, rounded up to 128 bytes.
size_t stage_bytes(int nx, int elem) {
  const size_t nxw_pad = ((size_t)(nx + 31) / 32 + 3) / 4 * 4;
  const size_t b = (size_t)27 * lines_window(nx) * elem + nxw_pad * (32 * 4 + 4);
  return (b + 127) / 128 * 128;
}
// Ring depth and blocks per SM: two blocks per SM when two rings of two stages
// fit in 200 KB of shared memory, the deepest ring (up to 4 stages) that fits
// beside the other block.
void lines_shape(int nx, int elem, int &stages, int &per_sm, size_t &smem) {
  const size_t stage = stage_bytes(nx, elem);
  const size_t budget = 200u * 1024u;
  per_sm = (4 * stage <= budget) ? 2 : 1;
  stages = (int)std::min<size_t>(4, budget / per_sm / stage);
  smem = stage * (size_t)stages;
}
}  // namespace

bool lines_supported(int Q, int store, int layout_rows, bool alpha, int nx) {
  if (Q != 27 || store != STORE_F16 || !layout_rows || alpha) return false;
  int stages, per_sm;
  size_t smem;
  lines_shape(nx, 2, stages, per_sm, smem);
  return stages >= 2;
}

cudaError_t lines_prepare() {
  cudaError_t e = cudaFuncSetAttribute(sweep_lines_kernel<27, F16Dev, 2>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(sweep_lines_kernel<27, F16Dev, 2>,
                             cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  return e;
}

cudaError_t launch_lines_f16_q27(const SweepArgs &a, int sms, cudaStream_t s) {
  int stages, per_sm;
  size_t smem;
  lines_shape(a.L.nx, 2, stages, per_sm, smem);
  LinesArgs la{};
  la.stages = stages;
  la.window = lines_window(a.L.nx);
  la.nxw_pad = (a.nxw + 3) / 4 * 4;
  la.lines = (long long)a.L.ny * a.L.nz;
  la.stage_bytes = stage_bytes(a.L.nx, 2);
  la.err = a.err;
  const long long grid = std::min<long long>(la.lines, (long long)sms * per_sm);
  sweep_lines_kernel<27, F16Dev, 2><<<(unsigned)grid, LINES_THREADS + 32, smem, s>>>(a, la);
  return cudaGetLastError();
}

// Self-test of the bounded-wait error path: one thread waits on an mbarrier
// that nothing arrives on, gives up after `polls` polls and records
// LINES_TIMEOUT in *err, as a sweep's wait would.  No copy is in flight, so
// the kernel simply returns.
__global__ void wait_timeout_probe_kernel(unsigned *err, long long polls) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (!mbar_wait_bounded(&bar, 0u, polls)) atomicExch(err, LINES_TIMEOUT);
  }
}

cudaError_t launch_wait_timeout_probe(unsigned *err, long long polls, cudaStream_t s) {
  wait_timeout_probe_kernel<<<1, 32, 0, s>>>(err, polls);
  return cudaGetLastError();
}

}  // namespace cflbm
