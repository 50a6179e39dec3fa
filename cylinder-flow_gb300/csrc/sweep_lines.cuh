// Line-staged channel sweep: the rows a (y, z) line pulls from are copied into
// shared memory with 1-D bulk asynchronous copies (cp.async.bulk, completion on
// an mbarrier), so the bytes in flight no longer sit in registers.
//
// Why: with 2-byte populations a warp-wide load moves 64 bytes, and the
// register-fed two-cell kernel (sweep_channel2_kernel) cannot keep enough of
// them in flight to reach the copy bandwidth -- it is bound by latency, not by
// DRAM.  Here one thread of a block issues, per line, one bulk copy per
// population: the whole source row of that population (ROWS layout: the Q rows
// of a line are adjacent, each row is contiguous and starts on a 128-byte
// boundary), ~1 KB per copy for a 512-cell line, into a ring of stages; the
// block computes a line from shared memory while the next lines' copies fly.
//
// Which row: for line (y, z) and direction I the source is the row of
// population j of line (y - e_y, z - e_z) after the face rules of the line's
// face state (periodic wrap, free-slip mirror: face_off tables, the same the
// register-fed sweep uses), read at x - e_x; at a no-slip face (face_bb) the
// cell's own row of opp(I), unshifted (halfway bounce-back).  The x rules stay
// per cell: inlet equilibrium at x = 0 for e_x > 0, zero gradient at
// x = nx - 1 for e_x < 0.  Cells of a listed tile with solid links take the
// bounced population f*_opp(I)(X) from global memory (a few thousand cells per
// step); solid cells get p = u = 0.  The arithmetic is channel2_cells' (packed
// FP32x2, two cells per thread: x and x + 32 of a 64-cell warp span), so the
// states are bit-identical to the register-fed kernel's.
//
// One thread of the block waits for a stage's copies (bounded) and the block
// meets it at one barrier per line, which also orders the reads of the stage
// before its refill.  A wait that gives up records LINES_TIMEOUT in *a.err
// (read by the host at the next synchronising call), waits (bounded) for the
// copies the block has in flight, and returns.
#pragma once
#include "sweep.cuh"

namespace cflbm {

constexpr int LINES_THREADS = 256;           // two cells per thread: x and x + 32
constexpr int LINES_CELLS = 2 * LINES_THREADS;
constexpr unsigned LINES_TIMEOUT = 0x4C494E45u;  // error word ("LINE")
constexpr long long LINES_SPIN_LIMIT = 1LL << 22;  // try_wait polls (~seconds) before giving up

// Window of a row copied per line: elements [xoff - 8, xoff - 8 + lines_window)
// (16-byte aligned start, a multiple of 8 elements long), covering x - 1 ..
// nx of every pull.
__host__ __device__ inline int lines_window(int nx) { return ((nx + 16 + 7) / 8) * 8; }

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// true once the phase with the given parity has completed
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity) {
  for (long long k = 0; k < LINES_SPIN_LIMIT; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes,
                                              unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

struct LinesArgs {
  int stages;    // ring depth
  int window;    // lines_window(nx) elements per staged row
  long long lines;  // ny * nz
  unsigned *err;    // error word (0 = fine)
};

// Issue the Q bulk copies of line `ln` into stage buffer `buf` (one thread).
template <int Q, class E>
__device__ __forceinline__ void lines_issue(const SweepArgs &a, const LinesArgs &la, long long ln,
                                            E *buf, unsigned long long *bar,
                                            const long long *face_off, const unsigned *face_bb) {
  using L = Lat<Q>;
  const int ny = a.L.ny;
  const int y = (int)(ln % ny), z = (int)(ln / ny);
  const int st = face_state(y, z, ny, a.L.nz);
  const unsigned wbb = face_bb[st];
  const E *fa = static_cast<const E *>(a.fa);
  const long long line0 = a.L.idx(0, y, z) - a.L.xoff;  // element 0 of population 0's row
  const unsigned bytes = (unsigned)(la.window * sizeof(E));
  // order this block's earlier generic reads of the stage before the async writes
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect_tx(bar, bytes * Q);
#pragma unroll
  for (int I = 0; I < Q; ++I) {
    long long row;
    if (I == 0) row = line0;
    else if ((wbb >> I) & 1u) row = line0 + (long long)L::opp(I) * a.L.S;
    else row = line0 + face_off[st * Q + I] + L::ex(I);  // undo the table's x shift
    bulk_copy_g2s(buf + (size_t)I * la.window, fa + row + a.L.xoff - 8, bytes, bar);
  }
}

template <int Q, class ST, int MINB>
__global__ void __launch_bounds__(LINES_THREADS, MINB)
    sweep_lines_kernel(const SweepArgs a, const LinesArgs la) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  extern __shared__ __align__(128) unsigned char lines_smem[];
  __shared__ unsigned long long bars[4];
  __shared__ int failed;
  __shared__ long long s_off[16 * Q];  // the face-state tables, for the issuing thread
  __shared__ unsigned s_bb[16];
  E *ring = reinterpret_cast<E *>(lines_smem);
  const size_t stage_elems = (size_t)Q * la.window;
  const int tid = threadIdx.x, lane = tid & 31;
  const int nx = a.L.nx, ny = a.L.ny;
  for (int k = tid; k < 16 * Q; k += LINES_THREADS) s_off[k] = a.face_off[k];
  if (tid < 16) s_bb[tid] = a.face_bb[tid];
  if (tid == 0) {
    for (int s = 0; s < la.stages; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    failed = 0;
  }
  __syncthreads();
  // prologue: the first stages - 1 lines of this block
  if (tid == 0)
    for (int s = 0; s < la.stages - 1; ++s) {
      const long long ln = blockIdx.x + (long long)s * gridDim.x;
      if (ln < la.lines)
        lines_issue<Q, E>(a, la, ln, ring + s * stage_elems, &bars[s], s_off, s_bb);
    }
  // thread 0's bookkeeping for a clean exit after a failed wait: the stages
  // with copies in flight
  unsigned inflight = 0u;
  if (tid == 0)
    for (int k = 0; k < la.stages - 1; ++k)
      if (blockIdx.x + (long long)k * gridDim.x < la.lines) inflight |= 1u << k;
  int s = 0;
  unsigned pbits = 0u;  // bit k: parity of the next wait on stage k (thread 0)
  // One thread waits for a stage's copies; the block meets it at one barrier
  // per line, so no other warp spends issue slots polling the mbarrier.
  if (tid == 0 && blockIdx.x < la.lines) {
    if (mbar_wait_bounded(&bars[0], 0u)) {
      inflight &= ~1u;
      pbits ^= 1u;
    } else {
      failed = 1;
    }
  }
  __syncthreads();
  for (long long ln = blockIdx.x; ln < la.lines && !failed; ln += gridDim.x) {
    // refill the stage the previous line used with the line stages - 1 ahead
    // (every thread passed the barrier after finishing that line)
    if (tid == 0) {
      const long long nl = ln + (long long)(la.stages - 1) * gridDim.x;
      const int ns = (s + la.stages - 1) % la.stages;
      if (nl < la.lines) {
        lines_issue<Q, E>(a, la, nl, ring + ns * stage_elems, &bars[ns], s_off, s_bb);
        inflight |= 1u << ns;
      }
    }
    const E *buf = ring + s * stage_elems;
    const int y = (int)(ln % ny), z = (int)(ln / ny);
    const int st = face_state(y, z, ny, a.L.nz);
    const unsigned wbb = s_bb[st];
    const long long rowc = a.L.idx(0, y, z);  // cell x = 0, population 0
    for (int xb = 0; xb < nx; xb += LINES_CELLS) {
      // warp w takes the tiles 2w and 2w + 1 of this 512-cell block: cells x0
      // and x0 + 32, the pairs of the register-fed kernel (same rounding keys)
      const int x0 = xb + 64 * (tid >> 5) + lane, x1 = x0 + 32;
      if (xb + 64 * (tid >> 5) >= nx) continue;  // warp entirely past the line
      const bool st0 = x0 < nx, st1 = x1 < nx;
      // listed tiles of the warp's two 32-cell tiles (solid cells or links)
      const long long trow = ((long long)z * ny + y) * a.nxw;
      const int t0 = a.tile_index[trow + (x0 >> 5)];  // the warp's tile exists
      const int t1 = st1 ? a.tile_index[trow + (x1 >> 5)] : -1;
      const unsigned l0 = t0 >= 0 ? a.links_bits[(long long)t0 * SWEEP_BX + lane] : 0u;
      const unsigned l1 = t1 >= 0 ? a.links_bits[(long long)t1 * SWEEP_BX + lane] : 0u;
      const bool linked = __any_sync(0xffffffffu, ((l0 | l1) & 0x7FFFFFFFu) != 0u);
      float2 f[Q];
      static_for(
          [&](auto ic) {
            constexpr int I = decltype(ic)::value;
            constexpr int ex = L::ex(I);
            const int sx = ((wbb >> I) & 1u) ? 0 : ex;
            const E *row = buf + (size_t)I * la.window + 8;  // row[x'] = element of x'
            int xs0 = x0 - sx, xs1 = x1 - sx;
            if constexpr (ex < 0) {  // zero gradient: the outlet column repeats itself
              xs0 = (x0 == nx - 1 && sx != 0) ? x0 : xs0;
              xs1 = (x1 == nx - 1 && sx != 0) ? x1 : xs1;
            }
            const float b = ((wbb >> I) & 1u) ? a.L.fbase[L::opp(I)] : a.L.fbase[I];
            const float r0 = st0 ? PairCodec<ST>::raw(row[xs0]) : 0.0f;
            const float r1 = st1 ? PairCodec<ST>::raw(row[xs1]) : 0.0f;
            float2 v = PairCodec<ST>::dec(make_float2(r0, r1), make_float2(b, b));
            if constexpr (ex > 0) v.x = (x0 == 0 && sx != 0) ? a.f_in_f[I] : v.x;
            if constexpr (I > 0) {
              if (linked) {  // warp-uniform: bounce-back off solid sources
                const E *fa = static_cast<const E *>(a.fa);
                const long long ob = (long long)L::opp(I) * a.L.S + rowc;
                if ((l0 >> I) & 1u)
                  v.x = SF::template load<float, L>(fa + ob + x0, a.L.fbase[L::opp(I)]);
                if ((l1 >> I) & 1u)
                  v.y = SF::template load<float, L>(fa + ob + x1, a.L.fbase[L::opp(I)]);
              }
            }
            f[I] = v;
          },
          std::make_integer_sequence<int, Q>{});
      float2 rho3, ux, uy, uz;
      moments<L, float2, SF>(f, rho3, ux, uy, uz);
      if (l0 >> 31) { rho3.x = 0.0f; ux.x = 0.0f; uy.x = 0.0f; uz.x = 0.0f; }
      if (l1 >> 31) { rho3.y = 0.0f; ux.y = 0.0f; uy.y = 0.0f; uz.y = 0.0f; }
      bgk_relax_v<L, float2, SF>(f, rho3, ux, uy, uz, a);
      E *__restrict__ q = static_cast<E *>(a.fb) + rowc;
#pragma unroll
      for (int i = 0; i < Q; ++i)
        PairCodec<ST>::template put2<Q>(q + i * a.L.S + x0, q + i * a.L.S + x1, f[i],
                                        a.L.fbase[i], st0, st1,
                                        (unsigned)((ln * nx + x0) * Q + i));
    }
    // the next line's stage: thread 0 waits for its copies, then the barrier
    // (which also orders every read of stage s before its refill)
    const int s1 = s + 1 == la.stages ? 0 : s + 1;
    if (tid == 0 && ln + gridDim.x < la.lines) {
      if (mbar_wait_bounded(&bars[s1], (pbits >> s1) & 1u)) {
        inflight &= ~(1u << s1);
        pbits ^= 1u << s1;
      } else {
        failed = 1;
      }
    }
    __syncthreads();
    s = s1;
  }
  if (failed && tid == 0) {
    atomicExch(la.err, LINES_TIMEOUT);
    // let the copies this block issued land before its shared memory is released
    for (int k = 0; k < la.stages; ++k)
      if ((inflight >> k) & 1u) (void)mbar_wait_bounded(&bars[k], (pbits >> k) & 1u);
  }
}

}  // namespace cflbm
