// Line-staged channel sweep: the rows a (y, z) line pulls from are copied into
// shared memory with 1-D bulk asynchronous copies (cp.async.bulk, completion on
// an mbarrier), so the bytes in flight no longer sit in registers.
//
// Why: with 2-byte populations a warp-wide load moves 64 bytes, and the
// register-fed two-cell kernel (sweep_channel2_kernel) cannot keep enough of
// them in flight to reach the copy bandwidth -- it is bound by latency, not by
// DRAM.  Here the lanes of a producer warp issue, per line, one bulk copy per
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
// Measured on GB300 it is the slower of the two (0.31 against 0.59 of the copy
// peak at 512x128x128): it removes most of the load latency but executes about
// a third more instructions per cell, so it runs only on request
// (CFLBM_FP16_SWEEP=lines).
//
// A producer warp issues the copies (and the line's listed-tile positions and
// link words) into a ring of stages; eight consumer warps compute.  Stages are
// handed over with a full and an empty mbarrier each, so no block-wide barrier
// couples the warps.  Every wait is bounded; a wait that gives up records
// LINES_TIMEOUT in *a.err (read by the host at the next synchronising call);
// the producer then waits (bounded) for the copies it issued, and the block
// returns.
#pragma once
#include "sweep.cuh"

namespace cflbm {

constexpr int LINES_THREADS = 256;           // consumer threads, two cells each: x and x + 32
static_assert(SWEEP_BX == 32, "a tile is one warp of cells, its link words one 128-byte copy");
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
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity,
                                                  long long limit = LINES_SPIN_LIMIT) {
  for (long long k = 0; k < limit; ++k)
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
  int stages;       // ring depth
  int window;       // lines_window(nx) elements per staged row
  int nxw_pad;      // tiles of a line, rounded up to 4 (the stage's tile areas)
  long long lines;  // ny * nz
  size_t stage_bytes;  // bytes per stage: rows, then link words, then tile positions
  unsigned *err;    // error word (0 = fine)
};

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// The producer warp: for line ln into stage buffer `st` -- the line's tile
// positions (one per lane), the rows of every population and the link words
// of its listed tiles, all completing on `full`.
template <int Q, class E>
__device__ __forceinline__ void lines_produce(const SweepArgs &a, const LinesArgs &la, long long ln,
                                              unsigned char *st, unsigned long long *full,
                                              const long long *row_off) {
  const int lane = threadIdx.x & 31;
  const int ny = a.L.ny;
  const int y = (int)(ln % ny), z = (int)(ln / ny);
  const int fs = face_state(y, z, ny, a.L.nz);
  E *rows = reinterpret_cast<E *>(st);
  uint32_t *links = reinterpret_cast<uint32_t *>(st + (size_t)Q * la.window * sizeof(E));
  int *tiles = reinterpret_cast<int *>(links + (size_t)la.nxw_pad * 32);
  const long long trow = (long long)ln * a.nxw;
  // tile positions in the list (-1: not listed), and how many are listed
  int listed = 0;
  for (int w0 = 0; w0 < a.nxw; w0 += 32) {
    const int w = w0 + lane;
    const int t = w < a.nxw ? a.tile_index[trow + w] : -1;
    if (w < a.nxw) tiles[w] = t;
    listed += __popc(__ballot_sync(0xffffffffu, t >= 0));
  }
  const unsigned row_bytes = (unsigned)(la.window * sizeof(E));
  __syncwarp();
  if (lane == 0) {
    // order this block's earlier generic reads of the stage before the async writes
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(full, row_bytes * Q + 128u * (unsigned)listed);
  }
  __syncwarp();
  const E *fa = static_cast<const E *>(a.fa);
  const long long line0 = a.L.idx(0, y, z) - a.L.xoff;  // element 0 of population 0's row
  for (int I = lane; I < Q; I += 32)
    bulk_copy_g2s(rows + (size_t)I * la.window, fa + line0 + row_off[fs * Q + I] + a.L.xoff - 8,
                  row_bytes, full);
  for (int w = lane; w < a.nxw; w += 32) {
    const int t = tiles[w];
    if (t >= 0) bulk_copy_g2s(links + (size_t)w * 32, a.links_bits + (long long)t * SWEEP_BX, 128u, full);
  }
}

// Cells x0 and x0 + 32 of a staged line: pulls from the stage's rows (rows
// already chosen per face state by the producer), the per-cell x rules (inlet
// equilibrium at x = 0, zero gradient at x = nx - 1), and -- NOSLIP: the line
// lies on a no-slip face (wbb: its bounced directions, unshifted and decoded
// with the opposite's base); LINKED: a cell of the pair has solid links (their
// bounced populations from global memory; solid cells get p = u = 0).  The
// arithmetic is channel2_cells', so the states are bit-identical to the
// register-fed kernel's.
template <int Q, class ST, bool NOSLIP, bool LINKED>
__device__ __forceinline__ void lines_pair(const SweepArgs &a, const typename Store<ST>::elem *buf,
                                           int window, unsigned wbb, long long rowc, int x0,
                                           unsigned l0, unsigned l1, long long key) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  const int nx = a.L.nx;
  const int x1 = x0 + 32;
  const bool st0 = x0 < nx, st1 = x1 < nx;
  float2 f[Q];
  static_for(
      [&](auto ic) {
        constexpr int I = decltype(ic)::value;
        constexpr int ex = L::ex(I);
        const bool bbI = NOSLIP && ((wbb >> I) & 1u);
        const int sx = bbI ? 0 : ex;
        const E *row = buf + (size_t)I * window + 8;  // row[x'] = element of x'
        int xs0 = x0 - sx, xs1 = x1 - sx;
        if constexpr (ex < 0) {  // zero gradient: the outlet column repeats itself
          xs0 = (x0 == nx - 1 && !bbI) ? x0 : xs0;
          xs1 = (x1 == nx - 1 && !bbI) ? x1 : xs1;
        }
        const float b = bbI ? a.L.fbase[L::opp(I)] : a.L.fbase[I];
        const float r0 = st0 ? PairCodec<ST>::raw(row[xs0]) : 0.0f;
        const float r1 = st1 ? PairCodec<ST>::raw(row[xs1]) : 0.0f;
        float2 v = PairCodec<ST>::dec(make_float2(r0, r1), make_float2(b, b));
        if constexpr (ex > 0) v.x = (x0 == 0 && !bbI) ? a.f_in_f[I] : v.x;
        if constexpr (LINKED && I > 0) {  // bounce-back off solid sources
          const E *fa = static_cast<const E *>(a.fa);
          const long long ob = a.doff[L::opp(I)] + rowc;
          if ((l0 >> I) & 1u)
            v.x = SF::template load<float, L>(fa + ob + x0, a.L.fbase[L::opp(I)]);
          if ((l1 >> I) & 1u)
            v.y = SF::template load<float, L>(fa + ob + x1, a.L.fbase[L::opp(I)]);
        }
        f[I] = v;
      },
      std::make_integer_sequence<int, Q>{});
  float2 rho3, ux, uy, uz;
  moments<L, float2, SF>(f, rho3, ux, uy, uz);
  if constexpr (LINKED) {
    if (l0 >> 31) { rho3.x = 0.0f; ux.x = 0.0f; uy.x = 0.0f; uz.x = 0.0f; }
    if (l1 >> 31) { rho3.y = 0.0f; ux.y = 0.0f; uy.y = 0.0f; uz.y = 0.0f; }
  }
  bgk_relax_v<L, float2, SF>(f, rho3, ux, uy, uz, a);
  E *__restrict__ q = static_cast<E *>(a.fb) + rowc;
#pragma unroll
  for (int i = 0; i < Q; ++i)
    PairCodec<ST>::template put2<Q>(q + i * a.L.S + x0, q + i * a.L.S + x1, f[i],
                                    a.L.fbase[i], st0, st1, (unsigned)(key + i), a.f16_sr);
}

// Block: LINES_THREADS consumer threads (8 warps, two cells each per 512-cell
// block of a line) and one producer warp.  Stage s is handed over with two
// mbarriers: full[s] completes when the stage's copies have landed, empty[s]
// when every consumer warp is done with it.  No block-wide barrier in the loop:
// each warp waits only for the data it reads.
template <int Q, class ST, int MINB>
__global__ void __launch_bounds__(LINES_THREADS + 32, MINB)
    sweep_lines_kernel(const SweepArgs a, const LinesArgs la) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  extern __shared__ __align__(128) unsigned char lines_smem[];
  __shared__ unsigned long long full[4], empty[4];
  __shared__ volatile int failed;
  // per face state and direction: the source row relative to the line's
  // population-0 row (the face-state table's source without its x shift; at a
  // no-slip face the cell's own row of opp(I)), and the no-slip bits
  __shared__ long long s_row[16 * Q];
  __shared__ unsigned s_bb[16];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nx = a.L.nx, ny = a.L.ny;
  constexpr int NCW = LINES_THREADS / 32;  // consumer warps
  for (int k = tid; k < 16 * Q; k += blockDim.x) {
    const int fs = k / Q, I = k % Q;
    const unsigned bb = a.face_bb[fs];
    long long row = 0;
    if (I > 0)
      row = ((bb >> I) & 1u) ? (long long)L::opp(I) * a.L.S
                             : a.face_off[k] + (long long)L::ex(I);  // undo the table's x shift
    s_row[k] = row;
  }
  if (tid < 16) s_bb[tid] = a.face_bb[tid];
  if (tid == 0) {
    for (int s = 0; s < la.stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NCW);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    failed = 0;
  }
  __syncthreads();

  if (warp == NCW) {  // ---- producer ---------------------------------------
    int s = 0;
    unsigned epar = 0u;  // bit k: parity of the next empty-wait on stage k
    long long k = 0;
    for (long long ln = blockIdx.x; ln < la.lines; ln += gridDim.x, ++k) {
      if (k >= la.stages) {  // stage s is reused: every consumer warp released it
        bool ok = true;
        if (lane == 0) ok = mbar_wait_bounded(&empty[s], (epar >> s) & 1u);
        __syncwarp();
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok || failed) {
          if (lane == 0) failed = 1;
          break;
        }
        epar ^= 1u << s;
      }
      lines_produce<Q, E>(a, la, ln, lines_smem + (size_t)s * la.stage_bytes, &full[s], s_row);
      s = s + 1 == la.stages ? 0 : s + 1;
    }
    // Leave no copy in flight: wait (bounded) for every stage's last batch.
    if (lane == 0) {
      const long long issued = k;
      for (int q = 0; q < la.stages && q < issued; ++q) {
        const long long last = q + ((issued - 1 - q) / la.stages) * la.stages;  // batch index
        (void)mbar_wait_bounded(&full[q], (unsigned)((last / la.stages) & 1));
      }
      if (failed) atomicExch(la.err, LINES_TIMEOUT);
    }
    return;
  }

  // ---- consumers ----------------------------------------------------------
  int s = 0;
  unsigned fpar = 0u;  // bit k: parity of the next full-wait on stage k
  for (long long ln = blockIdx.x; ln < la.lines; ln += gridDim.x) {
    bool ok = true;
    if (lane == 0) ok = mbar_wait_bounded(&full[s], (fpar >> s) & 1u);
    __syncwarp();  // orders the stage's data, seen by lane 0's wait, before the warp's reads
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok || failed) {
      if (lane == 0) failed = 1;
      break;
    }
    fpar ^= 1u << s;
    const unsigned char *st = lines_smem + (size_t)s * la.stage_bytes;
    const E *buf = reinterpret_cast<const E *>(st);
    const uint32_t *slinks =
        reinterpret_cast<const uint32_t *>(st + (size_t)Q * la.window * sizeof(E));
    const int *stiles = reinterpret_cast<const int *>(slinks + (size_t)la.nxw_pad * 32);
    const int y = (int)(ln % ny), z = (int)(ln / ny);
    const int fst = face_state(y, z, ny, a.L.nz);
    const unsigned wbb = s_bb[fst];
    const long long rowc = a.L.idx(0, y, z);  // cell x = 0, population 0
    for (int xb = 0; xb < nx; xb += LINES_CELLS) {
      // warp w takes the tiles 2w and 2w + 1 of this 512-cell block: cells x0
      // and x0 + 32, the pairs of the register-fed kernel
      const int x0 = xb + 64 * warp + lane, x1 = x0 + 32;
      if (xb + 64 * warp >= nx) continue;  // warp entirely past the line
      const int w0 = x0 >> 5;
      const unsigned l0 = stiles[w0] >= 0 ? slinks[w0 * 32 + lane] : 0u;
      const unsigned l1 = (x1 < nx && stiles[w0 + 1] >= 0) ? slinks[(w0 + 1) * 32 + lane] : 0u;
      // solid links or solid cells in the pair
      const bool linked = __any_sync(0xffffffffu, (l0 | l1) != 0u);
      // warp-uniform: pairs off the no-slip faces (every line of the benchmark
      // channels) without solid links or cells take the lean instantiation
      const long long key = (ln * nx + x0) * Q;
      if (wbb || linked) lines_pair<Q, ST, true, true>(a, buf, la.window, wbb, rowc, x0, l0, l1, key);
      else lines_pair<Q, ST, false, false>(a, buf, la.window, 0u, rowc, x0, l0, l1, key);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    s = s + 1 == la.stages ? 0 : s + 1;
  }
}

}  // namespace cflbm
