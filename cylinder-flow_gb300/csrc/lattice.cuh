// Lattice tables and population storage formats, usable from host and device.
//
// Velocity order, weights and bounce-back pairs follow the reference exactly so
// that population index i means the same direction everywhere:
//   D2Q9  "Kokkos/lbm.cpp:57-95": 0, E, N, W, S, NE, NW, SW, SE;
//   D3Q27 "3D MPI+KOKKOS+MPIIO/lbm.cpp:55-218": rest, then +/- pairs (2k-1, 2k).
#pragma once
#include <cstdint>
#include <cuda_fp16.h>

namespace cflbm {

template <int Q> struct Lat;

template <> struct Lat<9> {
  static constexpr int Q = 9;
  static constexpr int D = 2;
  __host__ __device__ static constexpr int ex(int i) {
    constexpr int v[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    return v[i];
  }
  __host__ __device__ static constexpr int ey(int i) {
    constexpr int v[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    return v[i];
  }
  __host__ __device__ static constexpr int ez(int) { return 0; }
  __host__ __device__ static constexpr int opp(int i) {
    constexpr int v[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
    return v[i];
  }
  __host__ __device__ static constexpr double w(int i) {
    return i == 0 ? 4.0 / 9.0 : (i < 5 ? 1.0 / 9.0 : 1.0 / 36.0);
  }
  // The (i, opp(i)) pairs with i < opp(i).
  static constexpr int NPAIR = 4;
  __host__ __device__ static constexpr int pair(int k) {
    constexpr int v[4] = {1, 2, 5, 6};
    return v[k];
  }
  // Power-of-two scale close to 1/w_i: the FP16 format of the allocation-free
  // domain sums (noalloc.cu) stores f_i times it.
  __host__ __device__ static constexpr float h_scale(int i) {
    return i == 0 ? 2.0f : (i < 5 ? 8.0f : 32.0f);
  }
};

template <> struct Lat<27> {
  static constexpr int Q = 27;
  static constexpr int D = 3;
  __host__ __device__ static constexpr int ex(int i) {
    constexpr int v[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1,
                           -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
    return v[i];
  }
  __host__ __device__ static constexpr int ey(int i) {
    constexpr int v[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0,
                           0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1, -1, 1};
    return v[i];
  }
  __host__ __device__ static constexpr int ez(int i) {
    constexpr int v[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1,
                           1, 1, -1, -1, 1, 1, -1, 1, -1, -1, 1, -1, 1};
    return v[i];
  }
  __host__ __device__ static constexpr int opp(int i) {
    return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1);
  }
  __host__ __device__ static constexpr double w(int i) {
    return i == 0 ? 8.0 / 27.0 : (i <= 6 ? 2.0 / 27.0 : (i <= 18 ? 1.0 / 54.0 : 1.0 / 216.0));
  }
  static constexpr int NPAIR = 13;
  __host__ __device__ static constexpr int pair(int k) { return 2 * k + 1; }
  __host__ __device__ static constexpr float h_scale(int i) {
    return i == 0 ? 4.0f : (i <= 6 ? 16.0f : (i <= 18 ? 64.0f : 256.0f));
  }
};

// Direction with the component along axis d reversed (specular reflection).
template <class L>
__host__ __device__ constexpr int mirror(int i, int d) {
  int w0 = L::ex(i), w1 = L::ey(i), w2 = L::ez(i);
  if (d == 0) w0 = -w0;
  if (d == 1) w1 = -w1;
  if (d == 2) w2 = -w2;
  for (int k = 0; k < L::Q; ++k)
    if (L::ex(k) == w0 && L::ey(k) == w1 && L::ez(k) == w2) return k;
  return -1;
}

// ---- storage formats ---------------------------------------------------------
// Store<T>::load/store convert between the stored element and the arithmetic
// type A; FP16 deviation storage is described at Store<F16Dev>.
struct F16Dev {
  __half h;
};

template <class T> struct Store;

#if defined(__CUDACC__)

// double <-> float on the integer pipe.  On GB300 the F2F conversions run on
// the FP64 units (~0.5 T/s), which would cap an FP64-storage / FP32-arithmetic
// sweep at ~9 G cell updates/s; these take ~7 integer operations each.
//   f2d: exact for normal floats and zero; subnormal floats flush to zero;
//        infinities and NaNs are kept.
//   d2f: rounds the 29 dropped mantissa bits half up; |d| < 2^-126 flushes to
//        zero; |d| >= 2^128, infinities and NaNs become infinity.
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u;
  const unsigned ex = u & 0x7F800000u;
  unsigned hi = (((u >> 3) & 0x0FFFFFFFu) + (896u << 20)) | sign;
  unsigned lo = u << 29;
  if (ex == 0u) { hi = sign; lo = 0u; }
  if (ex == 0x7F800000u) hi |= 0x7FF00000u;
  return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ float d2f_bits(double d) {
  const unsigned hi = (unsigned)__double2hiint(d);
  const unsigned lo = (unsigned)__double2loint(d);
  const unsigned mag = hi & 0x7FFFFFFFu;
  unsigned t = __funnelshift_l(lo, hi, 3);  // exponent (low 9 bits) and 23 mantissa bits
  t = ((t - 0xC0000000u) & 0x7FFFFFFFu) + ((lo >> 28) & 1u);  // (896 << 23) mod 2^32
  if (mag < (897u << 20)) t = 0u;
  if (mag >= (1151u << 20)) t = 0x7F800000u;
  return __uint_as_float(t | (hi & 0x80000000u));
}

// Double-float number: the unevaluated sum hi + lo of two binary32 values,
// about 47 significant bits.  On GB300 the FP32 units run at ~70 times the
// FP64 units' rate, so a collision in this arithmetic is faster than in FP64
// at near-FP64 accuracy.  From FP64 storage, with integer operations and one
// FP32 subtraction (no FP64 unit): hi = d truncated to 24 significant bits,
// lo = the next 23 bits of d, formed as the float with hi's sign, exponent
// E - 23 and those bits as mantissa minus the same float with a zero mantissa
// (an exact subtraction); |d - (hi + lo)| < 2^-46 |d|.  |d| < 2^-100 loads as
// zero; |d| >= 2^128, infinities and NaNs load as NaN.  To FP64 storage:
// hi + lo with the exact integer conversions above and one FP64 addition.
// Only the channel and reference sweeps use it (compute = DF64).
struct df64 {
  float hi, lo;
  df64() = default;
  __device__ __forceinline__ df64(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ df64(float f) : hi(f), lo(0.0f) {}
  __device__ __forceinline__ df64(int i) : hi((float)i), lo(0.0f) {}
  __device__ __forceinline__ df64(double d) {
    const unsigned hw = (unsigned)__double2hiint(d), lw = (unsigned)__double2loint(d);
    const unsigned mag = hw & 0x7FFFFFFFu;
    // exponent (rebased by 1023 - 127 = 896, mod 2^32) and the top 23 mantissa bits
    const unsigned t = __funnelshift_l(lw, hw, 3) - 0xC0000000u;
    const unsigned hb = (t & 0x7FFFFFFFu) | (hw & 0x80000000u);
    const unsigned mg = (hb & 0xFF800000u) - (23u << 23);
    const unsigned lb = mg | ((lw >> 6) & 0x7FFFFFu);
    const bool tiny = mag < ((1023u - 100u) << 20);
    const bool big = mag >= (1151u << 20);
    hi = tiny ? 0.0f : (big ? __uint_as_float(0x7FC00000u) : __uint_as_float(hb));
    lo = tiny ? 0.0f : __fsub_rn(__uint_as_float(lb), __uint_as_float(mg));
  }
  __device__ __forceinline__ operator double() const {
    return __dadd_rn(f2d_bits(hi), f2d_bits(lo));
  }
};

// Storage codecs: load/store (global memory) and decode (an element already
// read, e.g. from shared memory) convert between the stored element and the
// arithmetic type A, so the arithmetic always sees the population itself.
// `base` is the storage offset of the population (Layout::fbase): 0 for FP64 and
// FP32; for FP16 deviation storage the equilibrium the format stores the
// deviation from, and `key` the element the FP16 store's rounding is keyed on
// (see Store<F16Dev>).
template <> struct Store<double> {
  using elem = double;
  template <class A>
  __device__ static A decode(elem v, float) {
    if constexpr (sizeof(A) == 4) return d2f_bits(v);
    else return static_cast<A>(v);
  }
  template <class A, class L>
  __device__ static A load(const elem *p, float) {
    if constexpr (sizeof(A) == 4) return d2f_bits(__ldg(p));
    else return static_cast<A>(__ldg(p));
  }
  template <class A, class L>
  __device__ static void store(elem *p, A v, float, unsigned, bool) {
    if constexpr (sizeof(A) == 4) *p = f2d_bits(v);
    else *p = static_cast<double>(v);
  }
};

template <> struct Store<float> {
  using elem = float;
  template <class A>
  __device__ static A decode(elem v, float) { return static_cast<A>(v); }
  template <class A, class L>
  __device__ static A load(const elem *p, float) { return static_cast<A>(__ldg(p)); }
  template <class A, class L>
  __device__ static void store(elem *p, A v, float, unsigned, bool) { *p = static_cast<float>(v); }
};

// FP16 deviation storage: binary16 of (f_i - base_i) * 2^12.  f_i is the
// reference's deviation form already (f_i - w_i rho0); base_i is the
// equilibrium of the free stream, feq_i(rho = 1, u = (u_ref, 0, 0)) (u_ref =
// the inlet speed of a channel, 0 for the reference profiles), so cells of the
// undisturbed stream store values near zero and keep binary16's relative
// precision on what differs from the free stream (the shifted-distribution
// idea of Lehmann et al., Phys. Rev. E 106, 015308, 2022, taken one step
// further).  One power of two for every direction: binary16 holds 2^-14..2^16
// normal, |f - base| stays below 0.1 in any flow the lattice can represent, so
// 2^12 keeps every value above 2^-24/2^12 normal down to 1.5e-8 with room to
// spare.  Decode: one FMA (the product by 2^-12 is exact).
//
// Encode (the sweeps' stores): round stochastically (default), or to nearest
// (cflbm_config::rounding); stochastic with sm_100-family hardware rounding,
// cvt.rs.f16x2.f32, fed with a hash of the value's FP32 bits and its element
// (key = cell * Q + i): runs stay deterministic, repeat and resume exactly, and
// every kernel and layout rounds a state alike.  cvt.rs rounds the upper half
// of its result with rbits[28:16] and the lower half with rbits[12:0], so a
// pair store gives each value the bits [28:16] of its own hash (byte_perm
// 0x3276 below) and a single store the same bits of the same hash.
// Drag error against FP64 arithmetic: D3Q27 768x384x384 sphere, Re 300, mean
// over steps 15,000-20,000: stochastic 1.3e-4, nearest 1.04e-3 (the steady
// part of round-to-nearest's error adds up over the run); D2Q9 400x100
// cylinder, periodic state, three perturbation seeds: stochastic 1.5e-4 ..
// 8.6e-4, nearest 4.6e-4 .. 6.5e-4.
constexpr float F16_SCALE = 4096.0f;
__device__ __forceinline__ unsigned f16_hash(float sv, unsigned key) {
  return (__float_as_uint(sv) ^ (key * 0x9E3779B1u)) * 0x85EBCA77u;
}
// binary16 of sv (scaled deviation) as the low 16 bits
__device__ __forceinline__ unsigned short f16_round(float sv, unsigned key, bool sr) {
  if (!sr) return __half_as_ushort(__float2half_rn(sv));
  unsigned d;
  asm("cvt.rs.f16x2.f32 %0, %1, %1, %2;" : "=r"(d) : "f"(sv), "r"(f16_hash(sv, key)));
  return (unsigned short)(d >> 16);
}
// binary16 of a (upper half) and b (lower half)
__device__ __forceinline__ unsigned f16_round2(float a, float b, unsigned ka, unsigned kb,
                                               bool sr) {
  unsigned d;
  if (!sr) {
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(a), "f"(b));
  } else {
    const unsigned r = __byte_perm(f16_hash(a, ka), f16_hash(b, kb), 0x3276);
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(a), "f"(b), "r"(r));
  }
  return d;
}
template <> struct Store<F16Dev> {
  using elem = __half;
  template <class A>
  __device__ static A decode(elem v, float base) {
    const float h = __half2float(v);
    if constexpr (sizeof(A) == 4) return __fmaf_rn(h, 1.0f / F16_SCALE, base);
    else return __fma_rn((double)h, 1.0 / F16_SCALE, (double)base);
  }
  template <class A, class L>
  __device__ static A load(const elem *p, float base) { return decode<A>(__ldg(p), base); }
  template <class A, class L>
  __device__ static void store(elem *p, A v, float base, unsigned key, bool sr) {
    float sv;
    if constexpr (sizeof(A) == 4) sv = __fmul_rn(__fsub_rn(v, base), F16_SCALE);
    else sv = __double2float_rn(__dmul_rn(__dsub_rn(static_cast<double>(v), (double)base),
                                          (double)F16_SCALE));
    *p = __ushort_as_half(f16_round(sv, key, sr));
  }
};
#endif  // __CUDACC__

}  // namespace cflbm
