// The fused collide-and-stream sweep: one pass over the interior per time step.
//
// For every interior cell X the kernels pull f_i(X) = f*_i(X - e_i) from the
// post-collision buffer A, form p = sum f / 3 and u = sum f e (the reference's
// LBM::Update, "3D MPI+KOKKOS+MPIIO/lbm.cpp:384-415"), zero them in solid cells,
// relax every population toward feq_i = t_i (3p + 3 e.u + 4.5 (e.u)^2 - 1.5 u^2)
// with rate omega = 1/(tau0 + 0.5) (the reference's LBM::Collision,
// lbm.cpp:257-272) and write the next post-collision state to B.  This replaces
// the reference's five passes (collision, stream1 into ft, stream2 copy-back,
// the host Update loop, the boundary passes) by one read and one write of every
// population.
//
// HBM traffic per cell update: Q loads + Q stores of the storage type (each
// population is a pure shift, so every element of A is read exactly once) plus
// 1/8 byte of solid mask.
//
// Kernels:
//   sweep_kernel          -- reference profiles: ghost layers and solid cells
//                            were filled by the boundary passes, so the pull is
//                            plain; applies the reference's inlet/outlet
//                            overrides of Update.
//   sweep_channel2_kernel -- channel profile, FP32 collision on FP32/FP16
//   sweep_channel_kernel     storage (two cells per thread, packed FP32x2) and
//                            the other forms (one cell per thread), over every
//                            warp tile: unlisted tiles pull plainly; listed
//                            tiles (y/z face rows, tiles next to solids) take
//                            their face rules from per-face-state offset tables
//                            and their solid links from per-cell link words, so
//                            the branch adds one select per direction, not the
//                            per-cell wall logic of pull_resolved.
//   channel_force_kernel  -- beside the sweep on a second stream: the body force
//                            from the populations the sweep bounces back.
//   macros_channel_kernel -- u, v, w, p on request.
#pragma once
#include <type_traits>
#include <utility>
#include "solver.cuh"

namespace cflbm {

template <class F, int... Is>
__device__ __forceinline__ void static_for(F &&f, std::integer_sequence<int, Is...>) {
  (f(std::integral_constant<int, Is>{}), ...);
}

// Collision arithmetic over V = float, double, float2 (two cells per thread,
// GB300's packed FFMA2/FADD2/FMUL2) or df64 (double-float, below).  Every operation is explicitly rounded, so
// the compiler neither contracts nor reorders: a cell gets the same bits from
// every kernel that collides it, scalar or packed.
template <class V> struct VA;
template <> struct VA<float> {
  using S = float;
  __device__ static float splat(float s) { return s; }
  __device__ static float add(float a, float b) { return __fadd_rn(a, b); }
  __device__ static float sub(float a, float b) { return __fsub_rn(a, b); }
  __device__ static float mul(float a, float b) { return __fmul_rn(a, b); }
  __device__ static float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
};
template <> struct VA<double> {
  using S = double;
  __device__ static double splat(double s) { return s; }
  __device__ static double add(double a, double b) { return __dadd_rn(a, b); }
  __device__ static double sub(double a, double b) { return __dsub_rn(a, b); }
  __device__ static double mul(double a, double b) { return __dmul_rn(a, b); }
  __device__ static double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
};
template <> struct VA<float2> {
  using S = float;
  __device__ static float2 splat(float s) { return make_float2(s, s); }
  __device__ static float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
  // a - b = fma(b, -1, a): the product is exact, so one rounding as in FADD.
  __device__ static float2 sub(float2 a, float2 b) {
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
  }
  __device__ static float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
  __device__ static float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
};

// Double-float arithmetic (df64, lattice.cuh)
// from published error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum
// and the FMA-based exact product (Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18, 1971; Joldes, Muller and
// Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017).
//   add: Dekker's double-word sum (their Algorithm 5, "sloppy"): TwoSum of the
//        high parts, the low parts added to its error, Fast2Sum -- 11
//        operations; error <= 2u^2 (|x| + |y|) (u = 2^-24), relative to the
//        operands, not the result, which is what a collision needs: every
//        population is compared to the field, not to itself;
//   mul: the exact product of the high parts plus the cross terms (the
//        lo*lo term, ~u^2 of the product, dropped), Fast2Sum -- 8 operations;
//        relative error <= 4u^2.
// T = float (the df64 arithmetic of one cell per thread).
template <class T> struct DWops {
  using O = VA<T>;
  __device__ static T neg(T a) { return O::sub(O::splat(0.0f), a); }
  __device__ static void two_sum(T a, T b, T &s, T &t) {
    s = O::add(a, b);
    const T ap = O::sub(s, b), bp = O::sub(s, ap);
    t = O::add(O::sub(a, ap), O::sub(b, bp));
  }
  __device__ static void fast_two_sum(T a, T b, T &s, T &t) {
    s = O::add(a, b);
    t = O::sub(b, O::sub(s, a));
  }
  __device__ static void add(T xh, T xl, T yh, T yl, T &zh, T &zl) {
    T sh, e;
    two_sum(xh, yh, sh, e);
    e = O::add(e, O::add(xl, yl));
    fast_two_sum(sh, e, zh, zl);
  }
  __device__ static void mul(T xh, T xl, T yh, T yl, T &zh, T &zl) {
    const T ch = O::mul(xh, yh);
    const T cl1 = O::fma(xh, yh, neg(ch));
    const T cl2 = O::fma(xl, yh, O::mul(xh, yl));
    fast_two_sum(ch, O::add(cl1, cl2), zh, zl);
  }
};
template <> __device__ __forceinline__ float DWops<float>::neg(float a) { return -a; }
template <> __device__ __forceinline__ float2 DWops<float2>::neg(float2 a) {
  return make_float2(-a.x, -a.y);
}

template <> struct VA<df64> {
  using S = double;
  using D = DWops<float>;
  __device__ static df64 splat(double s) {  // constants: folded at compile time
    const float h = (float)s;
    return df64(h, (float)(s - (double)h));
  }
  __device__ static df64 add(df64 x, df64 y) {
    df64 z;
    D::add(x.hi, x.lo, y.hi, y.lo, z.hi, z.lo);
    return z;
  }
  __device__ static df64 sub(df64 x, df64 y) { return add(x, df64(-y.hi, -y.lo)); }
  __device__ static df64 mul(df64 x, df64 y) {
    df64 z;
    D::mul(x.hi, x.lo, y.hi, y.lo, z.hi, z.lo);
    return z;
  }
  __device__ static df64 fma(df64 a, df64 b, df64 c) { return add(mul(a, b), c); }
};


// Index of the direction with velocity (ex, ey, ez), -1 if none; and the
// weight class of direction i (|e_i|^2: 0 rest, 1 axis, 2 face diagonal,
// 3 corner).
template <class L>
__host__ __device__ constexpr int dir_of(int ex, int ey, int ez) {
  for (int k = 0; k < L::Q; ++k)
    if (L::ex(k) == ex && L::ey(k) == ey && L::ez(k) == ez) return k;
  return -1;
}
template <class L>
__host__ __device__ constexpr int wclass(int i) {
  return L::ex(i) * L::ex(i) + L::ey(i) * L::ey(i) + L::ez(i) * L::ez(i);
}
// Pair index k (L::pair(k) = i) of direction i or of its opposite.
template <class L>
__host__ __device__ constexpr int pair_of(int i) {
  for (int k = 0; k < L::NPAIR; ++k)
    if (L::pair(k) == i || L::opp(L::pair(k)) == i) return k;
  return -1;
}

// Relaxation constants of a sweep (SweepArgs::rk, host-computed per handle):
//   rk[0]      = 1 - omega
//   rk[1 + c]  = omega w_c         (Kw, weight class c)
//   rk[5 + c]  = 4.5 omega w_c     (Ka)
//   rk[9 + c]  = 3 omega w_c       (K3)
//   rk[16 + c] = -6 omega w_c      (-2 K3)
// in FP64 (rk) and as the FP32 remainder rk - rkf (rkl), which with rkf forms
// the double-float constant.
// The FP32 set (rkf) is not rk rounded one by one: with Om = 1 - rkf[0] (exact)
// its values satisfy, as real numbers, the identities behind mass and momentum
// conservation of the collision,
//   sum_i Kw_i = Om,   sum_i K3_i e_ix^2 = Om,   sum_i Ka_i e_ix^2 = 1.5 Om,
// the rest class's Kw and the face class's K3 and Ka taking the remainder as a
// double-float pair (rkf[RK_W], rkf[RK_LW]), (rkf[RK_3 + 1], rkf[RK_L3]),
// (rkf[RK_A + 1], rkf[RK_LA]).  Constants rounded one by one miss these by a
// few 1e-8 per step -- a standing mass and momentum source that moves the
// period-averaged drag of the 400x100 channel by ~1e-3.
// (The RK_* indices are defined beside SweepArgs.)
template <class V> __device__ __forceinline__ V rconst(const SweepArgs &a, int k);
template <> __device__ __forceinline__ double rconst<double>(const SweepArgs &a, int k) {
  return a.rk[k];
}
template <> __device__ __forceinline__ float rconst<float>(const SweepArgs &a, int k) {
  return a.rkf[k];
}
template <> __device__ __forceinline__ float2 rconst<float2>(const SweepArgs &a, int k) {
  return make_float2(a.rkf[k], a.rkf[k]);
}
template <> __device__ __forceinline__ df64 rconst<df64>(const SweepArgs &a, int k) {
  return df64(a.rkf[k], a.rkl[k]);
}


template <class L, int k, class V>
__device__ __forceinline__ V pair_eu(V ux, V uy, V uz) {
  using O = VA<V>;
  using S = typename O::S;
  constexpr int i = L::pair(k);
  constexpr int ex = L::ex(i), ey = L::ey(i), ez = L::ez(i);
  if constexpr (ex != 0 && ey != 0 && ez != 0) {
    constexpr int kb = pair_of<L>(dir_of<L>(ex, ey, 0));
    static_assert(kb >= 0 && kb < k, "face diagonal precedes the corner");
    const V e = pair_eu<L, kb>(ux, uy, uz);
    const V b = L::ex(L::pair(kb)) == ex ? e : O::sub(O::splat(S(0)), e);
    return ez > 0 ? O::add(b, uz) : O::sub(b, uz);
  } else {
    constexpr int n = (ex != 0) + (ey != 0) + (ez != 0);
    if constexpr (n == 1) {
      return ex > 0 ? ux : ex < 0 ? O::sub(O::splat(S(0)), ux)
           : ey > 0 ? uy : ey < 0 ? O::sub(O::splat(S(0)), uy)
           : ez > 0 ? uz : O::sub(O::splat(S(0)), uz);
    } else {
      // two components (p, q): the positive one first
      constexpr bool hx = ex != 0, hy = ey != 0;
      constexpr int s1 = hx ? ex : ey, s2 = hx ? (hy ? ey : ez) : ez;
      const V p1 = hx ? ux : uy;
      const V p2 = hx ? (hy ? uy : uz) : uz;
      if constexpr (s1 > 0) return s2 > 0 ? O::add(p1, p2) : O::sub(p1, p2);
      else if constexpr (s2 > 0) return O::sub(p2, p1);
      else return O::sub(O::sub(O::splat(S(0)), p1), p2);
    }
  }
}

// The BGK relaxation over a getter and a putter: get(I) returns population I
// (a std::integral_constant index), put(I, v) receives its relaxed value, pair
// by pair, so a caller may hold every population in registers (bgk_relax_v) or
// fetch and store them one pair at a time.  Same operations in the same order
// either way.
template <class L, class V, class SF, class G, class Pt>
__device__ __forceinline__ void bgk_relax_each(G &&get, Pt &&put, V rho3, V ux, V uy, V uz,
                                               const SweepArgs &a) {
  using O = VA<V>;
  using S = typename O::S;
  const V omc = rconst<V>(a, RK_OMC);
  V usq;
  if constexpr (L::D == 3) usq = O::fma(ux, ux, O::fma(uy, uy, O::mul(uz, uz)));
  else usq = O::fma(ux, ux, O::mul(uy, uy));
  const V c0 = O::fma(O::splat(S(-1.5)), usq, rho3);
  constexpr int NC = L::D + 1;
  // FP32 arithmetic: the conserving constant pairs (rk layout above)
  constexpr bool kPairs = std::is_same_v<V, float> || std::is_same_v<V, float2>;
  V Ac[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) Ac[c] = O::mul(rconst<V>(a, RK_W + c), c0);
  if constexpr (kPairs) Ac[0] = O::fma(rconst<V>(a, RK_W), c0, O::mul(rconst<V>(a, RK_LW), c0));
  put(std::integral_constant<int, 0>{}, O::fma(omc, get(std::integral_constant<int, 0>{}), Ac[0]));
  static_for(
      [&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int i = L::pair(k), j = L::opp(L::pair(k));
        constexpr int c = wclass<L>(i);
        const V eu = pair_eu<L, k>(ux, uy, uz);
        V sp, sm;  // sym + asym, sym - asym
        if constexpr (!std::is_same_v<V, double>) {
          const V e2 = O::mul(eu, eu);
          V sym = O::fma(e2, rconst<V>(a, RK_A + c), Ac[c]);
          V asym = O::mul(rconst<V>(a, RK_3 + c), eu);
          if constexpr (kPairs && c == 1) {
            sym = O::fma(e2, rconst<V>(a, RK_LA), sym);
            asym = O::fma(rconst<V>(a, RK_L3), eu, asym);
          }
          sp = O::add(sym, asym);
          sm = O::sub(sym, asym);
        } else {
          // FP64: Horner in e.u, then the odd part's sign flip, 3 operations
          // for both (5 per pair instead of 7, 26 fewer per D3Q27 cell; a
          // double-float FMA costs more than the product and sum it replaces:
          // 7,683 against 7,764 M cell updates/s on 512x128x128, not used there)
          sp = O::fma(eu, O::fma(rconst<V>(a, RK_A + c), eu, rconst<V>(a, RK_3 + c)), Ac[c]);
          sm = O::fma(rconst<V>(a, RK_M3 + c), eu, sp);
        }
        put(std::integral_constant<int, i>{},
            O::fma(omc, get(std::integral_constant<int, i>{}), sp));
        put(std::integral_constant<int, j>{},
            O::fma(omc, get(std::integral_constant<int, j>{}), sm));
      },
      std::make_integer_sequence<int, L::NPAIR>{});
}

// BGK relaxation toward the incompressible equilibrium
//   feq_i = w_i (3p + 3 e_i.u + 4.5 (e_i.u)^2 - 1.5 |u|^2)
// ("3D MPI+KOKKOS+MPIIO/lbm.cpp:257-272"), f <- (1 - omega) f + omega feq, with
// omega and the weight folded into per-class constants (rconst) and written per
// +/- pair: the pair shares e.u, (e.u)^2 and the even part of feq; the odd part
// flips sign.  Per cell and pair k of class c:
//   c0 = rho3 - 1.5 |u|^2,  A_c = Kw_c c0,
//   sym = Ka_c (e.u)^2 + A_c,  asym = K3_c e.u,
//   f_i = (1 - omega) f_i + (sym + asym),  f_opp(i) = (1 - omega) f_opp(i) + (sym - asym).
// In FP64 arithmetic sym + asym = A_c + e.u (K3_c + Ka_c e.u) and
// sym - asym = (sym + asym) - 2 K3_c e.u (both near A_c: no cancellation).
// The corner directions' e.u reuse the face diagonals' (e_x u_x + e_y u_y).
// D3Q27 in FP64: 84 operations per cell (110 with sym and asym apart, 151
// unfolded).
template <class L, class V, class SF>
__device__ __forceinline__ void bgk_relax_v(V *f, V rho3, V ux, V uy, V uz, const SweepArgs &a) {
  bgk_relax_each<L, V, SF>([&](auto ic) { return f[decltype(ic)::value]; },
                           [&](auto ic, V v) { f[decltype(ic)::value] = v; }, rho3, ux, uy, uz,
                           a);
}

template <class L, class A, class SF>
__device__ __forceinline__ void bgk_relax(A *f, A rho3, A ux, A uy, A uz, const SweepArgs &a) {
  bgk_relax_v<L, A, SF>(f, rho3, ux, uy, uz, a);
}

// Moments in deviation form: rho3 = 3p = sum f, u = sum f e, as a three-level
// cascade over the 3 x 3 x 3 cube of velocities -- per (e_x, e_y) line the sum
// and the difference along z, then along y, then along x -- 49 additions for
// D3Q27 (14 for D2Q9) instead of 66 (18) with pair sums.
template <class L, class V, class G>
__device__ __forceinline__ void moments_get(G &&get, V &rho3, V &ux, V &uy, V &uz) {
  using O = VA<V>;
  using S = typename O::S;
  if constexpr (L::D == 3) {
    V s0[3][3], s1[3][3];
    static_for(
        [&](auto kc) {
          constexpr int k = decltype(kc)::value, a = k / 3, b = k % 3;
          const V lo = get(std::integral_constant<int, dir_of<L>(a - 1, b - 1, -1)>{});
          const V mid = get(std::integral_constant<int, dir_of<L>(a - 1, b - 1, 0)>{});
          const V hi = get(std::integral_constant<int, dir_of<L>(a - 1, b - 1, 1)>{});
          s0[a][b] = O::add(O::add(lo, hi), mid);
          s1[a][b] = O::sub(hi, lo);
        },
        std::make_integer_sequence<int, 9>{});
    V t00[3], t01[3], t10[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      t00[a] = O::add(O::add(s0[a][0], s0[a][2]), s0[a][1]);
      t01[a] = O::sub(s0[a][2], s0[a][0]);
      t10[a] = O::add(O::add(s1[a][0], s1[a][2]), s1[a][1]);
    }
    rho3 = O::add(O::add(t00[0], t00[2]), t00[1]);
    ux = O::sub(t00[2], t00[0]);
    uy = O::add(O::add(t01[0], t01[2]), t01[1]);
    uz = O::add(O::add(t10[0], t10[2]), t10[1]);
  } else {
    V s0[3], s1[3];
    static_for(
        [&](auto ac) {
          constexpr int a = decltype(ac)::value;
          const V lo = get(std::integral_constant<int, dir_of<L>(a - 1, -1, 0)>{});
          const V mid = get(std::integral_constant<int, dir_of<L>(a - 1, 0, 0)>{});
          const V hi = get(std::integral_constant<int, dir_of<L>(a - 1, 1, 0)>{});
          s0[a] = O::add(O::add(lo, hi), mid);
          s1[a] = O::sub(hi, lo);
        },
        std::make_integer_sequence<int, 3>{});
    rho3 = O::add(O::add(s0[0], s0[2]), s0[1]);
    ux = O::sub(s0[2], s0[0]);
    uy = O::add(O::add(s1[0], s1[2]), s1[1]);
    uz = O::splat(S(0));
  }
}
template <class L, class V, class SF>
__device__ __forceinline__ void moments(const V *f, V &rho3, V &ux, V &uy, V &uz) {
  moments_get<L, V>([&](auto ic) { return f[decltype(ic)::value]; }, rho3, ux, uy, uz);
}

// Macros out (when requested), Brinkman damping of the equilibrium velocity,
// relaxation, store: the common tail of every sweep.
// u, v, w and p = rho3 / 3 of one cell into the FP64 macroscopic fields.
template <class A>
__device__ __forceinline__ void store_macros(const SweepArgs &a, long long cell, A rho3, A ux,
                                             A uy, A uz) {
  if constexpr (sizeof(A) == 4) {
    a.mu[cell] = f2d_bits(ux);
    a.mv[cell] = f2d_bits(uy);
    a.mw[cell] = f2d_bits(uz);
    a.mp[cell] = f2d_bits(__fmul_rn(rho3, 1.0f / 3.0f));
  } else {
    a.mu[cell] = ux;
    a.mv[cell] = uy;
    a.mw[cell] = uz;
    a.mp[cell] = __ddiv_rn(rho3, 3.0);
  }
}

template <class L, class SF, class A, class E>
__device__ __forceinline__ void finish_cell(A *f, A rho3, A ux, A uy, A uz, long long cell,
                                            bool store, E *__restrict__ fb, long long c,
                                            long long S, const SweepArgs &a) {
  if (a.mu && store) store_macros<A>(a, cell, rho3, ux, uy, uz);
  if (a.alpha) {
    const A s = VA<A>::sub(A(1), static_cast<A>(a.alpha[cell]));
    ux = VA<A>::mul(ux, s);
    uy = VA<A>::mul(uy, s);
    uz = VA<A>::mul(uz, s);
  }
  bgk_relax<L, A, SF>(f, rho3, ux, uy, uz, a);
  if (store) {
#pragma unroll
    for (int i = 0; i < L::Q; ++i)
      SF::template store<A, L>(fb + i * S + c, f[i], a.L.fbase[i], (unsigned)(cell * L::Q + i),
                               a.f16_sr);
  }
}

// ---- reference profiles --------------------------------------------------------
template <int Q, class ST, class A, int MINB>
__global__ void __launch_bounds__(SWEEP_BX * SWEEP_BY, MINB) sweep_kernel(const SweepArgs a) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  const int x = blockIdx.x * SWEEP_BX + threadIdx.x;
  const int y = blockIdx.y * SWEEP_BY + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= a.L.nx || y >= a.L.ny) return;
  const long long S = a.L.S;
  const long long c = a.L.idx(x, y, z);
  const E *__restrict__ fa = static_cast<const E *>(a.fa);
  E *__restrict__ fb = static_cast<E *>(a.fb);

  A f[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i)
    f[i] = SF::template load<A, L>(fa + i * S + c - a.L.off(L::ex(i), L::ey(i), L::ez(i)),
                                   a.L.fbase[i]);

  A rho3, ux, uy, uz;
  moments<L, A, SF>(f, rho3, ux, uy, uz);
  const long long cell = ((long long)z * a.L.ny + y) * a.L.nx + x;
  if (mask_solid(a.mask, a.nxw, a.L.ny, x, y, z)) {
    rho3 = A(0); ux = A(0); uy = A(0); uz = A(0);
  }
  if (a.ref_override) {
    if (x == 0) {
      ux = static_cast<A>(a.inlet_u[(long long)z * a.L.ny + y]);
      uy = A(0);
      uz = A(0);
    }
    if (x == a.L.nx - 1) rho3 = A(0);
  }
  finish_cell<L, SF, A, E>(f, rho3, ux, uy, uz, cell, true, fb, c, S, a);
}

template <int Q, class ST, class A, int MINB>
cudaError_t launch_sweep_t(const SweepArgs &a, cudaStream_t s) {
  dim3 block(SWEEP_BX, SWEEP_BY, 1);
  dim3 grid((a.L.nx + SWEEP_BX - 1) / SWEEP_BX, (a.L.ny + SWEEP_BY - 1) / SWEEP_BY, a.L.nz);
  sweep_kernel<Q, ST, A, MINB><<<grid, block, 0, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

// ---- channel profile -------------------------------------------------------------
// Compile-time data of direction I: velocity, opposite and the specular
// mirrors in y, z and both.
template <int Q, int I> struct DirC {
  using L = Lat<Q>;
  static constexpr int ex = L::ex(I), ey = L::ey(I), ez = L::ez(I), opp = L::opp(I);
  static constexpr int my = mirror<L>(I, 1), mz = mirror<L>(I, 2);
  static constexpr int myz = mirror<L>(mirror<L>(I, 1), 2);
};


// Inlet equilibrium population in the arithmetic type (no FP64 conversion in
// FP32 sweeps; f_in_f + f_in_l for double-float).
template <class A>
__device__ __forceinline__ A inlet_pop(const SweepArgs &a, int i) {
  if constexpr (std::is_same<A, df64>::value) return df64(a.f_in_f[i], a.f_in_l[i]);
  else if constexpr (sizeof(A) == 8) return a.f_in[i];
  else return a.f_in_f[i];
}

// Two cells per thread: the pair arithmetic type P (float2) and its per-cell
// component type C (float).
template <class P> struct PairT;
template <> struct PairT<float2> {
  using C = float;
  __device__ static float2 make(float a, float b) { return make_float2(a, b); }
  __device__ static float x(float2 p) { return p.x; }
  __device__ static float y(float2 p) { return p.y; }
  __device__ static double to_double(float c) { return f2d_bits(c); }
  __device__ static float third(float c) { return __fmul_rn(c, 1.0f / 3.0f); }
};

// Storage codec of a cell pair on FP32x2 (the two-cell kernels): raw() takes
// an element as loaded (FP64 converted to FP32; FP16 kept as its bits) and
// dec() forms the pair's FP32 values -- for FP16 one mixed-precision FMA per
// value, h 2^-12 + b; the encode applies the FP16 format's offset and scale to
// the pair in one packed FMA -- the same values as Store<>::load/store per cell
// (the product with a power of two is exact, so fma(v, 2^12, -2^12 b) is
// 2^12 (v - b) rounded once).  `key` is the first value's element (cell * Q +
// i); the second cell lies 32 cells further.
template <class ST> struct PairCodec;
template <> struct PairCodec<double> {
  __device__ static float raw(double e) { return d2f_bits(e); }
  __device__ static float2 dec(float2 r, float2) { return r; }
  template <int Q>
  __device__ static void put2(double *p0, double *p1, float2 v, float, bool s0, bool s1,
                              unsigned, bool) {
    if (s0) *p0 = f2d_bits(v.x);
    if (s1) *p1 = f2d_bits(v.y);
  }
};
template <> struct PairCodec<float> {
  __device__ static float raw(float e) { return e; }
  __device__ static float2 dec(float2 r, float2) { return r; }
  template <int Q>
  __device__ static void put2(float *p0, float *p1, float2 v, float, bool s0, bool s1,
                              unsigned, bool) {
    if (s0) *p0 = v.x;
    if (s1) *p1 = v.y;
  }
};
template <> struct PairCodec<F16Dev> {
  // raw: the binary16 bits, unconverted; dec: one mixed-precision FMA per value
  // (fma.rn.f32.f16, sm_100 family: binary16 operands, FP32 addend and result),
  // h * 2^-12 + b rounded once -- the FP32 value of h times 2^-12 is exact, so
  // this equals converting h and one FP32 FMA
  __device__ static float raw(__half e) { return __uint_as_float((unsigned)__half_as_ushort(e)); }
  __device__ static float2 dec(float2 r, float2 b) {
    const unsigned short h0 = (unsigned short)__float_as_uint(r.x);
    const unsigned short h1 = (unsigned short)__float_as_uint(r.y);
    const unsigned short s = 0x0C00;  // 2^-12 = 1 / F16_SCALE in binary16
    float d0, d1;
    asm("fma.rn.f32.f16 %0, %1, %2, %3;" : "=f"(d0) : "h"(h0), "h"(s), "f"(b.x));
    asm("fma.rn.f32.f16 %0, %1, %2, %3;" : "=f"(d1) : "h"(h1), "h"(s), "f"(b.y));
    return make_float2(d0, d1);
  }
  template <int Q>
  __device__ static void put2(__half *p0, __half *p1, float2 v, float b, bool s0, bool s1,
                              unsigned key, bool sr) {
    const float nb = -F16_SCALE * b;
    const float2 sv = __ffma2_rn(v, make_float2(F16_SCALE, F16_SCALE), make_float2(nb, nb));
    const unsigned d = f16_round2(sv.x, sv.y, key, key + 32u * Q, sr);
    if (s0) *p0 = __ushort_as_half((unsigned short)(d >> 16));
    if (s1) *p1 = __ushort_as_half((unsigned short)(d & 0xFFFFu));
  }
};

// Post-stream population I of cell X (offset c) for rows away from the y/z
// faces and cells away from solids: the plain pull, with the inlet column
// taking the inlet equilibrium and the outlet column repeating itself (zero
// gradient).  Branch-free: the load is always issued (at x = 0 it reads the
// ghost column) so all Q loads of a cell can be in flight together.
template <int Q, class ST, class A, int I>
__device__ __forceinline__ A pull_plain(const typename Store<ST>::elem *__restrict__ fa,
                                        long long c, long long S, int x, const SweepArgs &a) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using Dd = DirC<Q, I>;
  long long src = c - a.L.off(Dd::ex, Dd::ey, Dd::ez);
  if constexpr (Dd::ex < 0) src += (x == a.L.nx - 1) ? Dd::ex : 0;
  A v = SF::template load<A, L>(fa + I * S + src, a.L.fbase[I]);
  if constexpr (Dd::ex > 0) v = (x == 0) ? inlet_pop<A>(a, I) : v;
  return v;
}

// Post-stream population I of cell X for any cell: the source S = X - e_I is
// mapped onto the box --
//   z face: periodic -> wrap; free-slip -> mirror (population mirror_z(I),
//           S.z = X.z); no-slip -> halfway bounce-back f*_{opp(I)}(X);
//   y face: the same;
//   x < 0:  inlet equilibrium; x >= nx: zero gradient (S.x = nx - 1);
//   solid S (bit I of `links`): halfway bounce-back f*_{opp(I)}(X).
// Written with selects on the address and population, so the load is
// unconditional and independent of the other directions' loads.
template <int Q, class ST, class A, int I>
__device__ __forceinline__ A pull_resolved(const typename Store<ST>::elem *__restrict__ fa,
                                           long long c, long long S, int x, int y, int z,
                                           unsigned links, const SweepArgs &a) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using Dd = DirC<Q, I>;
  if constexpr (I == 0) {
    return SF::template load<A, L>(fa + c, a.L.fbase[0]);
  } else {
    long long src = c - a.L.off(Dd::ex, Dd::ey, Dd::ez);
    bool my = false, mz = false, bb = false;
    if constexpr (Dd::ez != 0) {
      const bool out = Dd::ez > 0 ? (z == 0) : (z == a.L.nz - 1);
      const bool per = out && a.wall_z == WALL_PERIODIC;
      mz = out && a.wall_z == WALL_FREESLIP;
      bb = out && a.wall_z == WALL_NOSLIP;
      src += per ? (Dd::ez > 0 ? 1LL : -1LL) * a.L.nz * a.L.zs : 0LL;
      src += mz ? (long long)Dd::ez * a.L.zs : 0LL;
    }
    if constexpr (Dd::ey != 0) {
      const bool out = !bb && (Dd::ey > 0 ? (y == 0) : (y == a.L.ny - 1));
      const bool per = out && a.wall_y == WALL_PERIODIC;
      my = out && a.wall_y == WALL_FREESLIP;
      bb = bb || (out && a.wall_y == WALL_NOSLIP);
      src += per ? (Dd::ey > 0 ? 1LL : -1LL) * a.L.ny * a.L.rs : 0LL;
      src += my ? (long long)Dd::ey * a.L.rs : 0LL;
    }
    bb = bb || ((links >> I) & 1u);
    const int j = my ? (mz ? Dd::myz : Dd::my) : (mz ? Dd::mz : I);
    if constexpr (Dd::ex < 0) src += (x == a.L.nx - 1) ? Dd::ex : 0;  // zero gradient
    // a mirror j of I has I's |e| and e_x, hence I's storage offset; the
    // bounced population is opp(I) and decodes with its own
    const long long addr = bb ? (long long)Dd::opp * S + c : (long long)j * S + src;
    A v = SF::template load<A, L>(fa + addr, bb ? a.L.fbase[Dd::opp] : a.L.fbase[I]);
    if constexpr (Dd::ex > 0) v = (!bb && x == 0) ? inlet_pop<A>(a, j) : v;
    return v;
  }
}

// Face state of a row: bit 0 y = 0, bit 1 y = ny-1, bit 2 z = 0, bit 3 z = nz-1.
__device__ __forceinline__ int face_state(int y, int z, int ny, int nz) {
  return (y == 0 ? 1 : 0) | (y == ny - 1 ? 2 : 0) | (z == 0 ? 4 : 0) | (z == nz - 1 ? 8 : 0);
}

// Post-stream population I of a cell of a listed tile, from the face-state
// tables (off = a.face_off[state * Q + I], wbb = the no-slip face bit of I): the
// same source as pull_resolved.  Solid link (bit I of `links`) or no-slip face:
// halfway bounce-back f*_{opp(I)}(X); otherwise the table's source with the
// per-cell x rules (inlet equilibrium at x = 0, zero gradient at x = nx-1).  A
// mirrored population has the same |e| and e_x as I, so I's storage offset
// and inlet value apply.
template <int Q, class ST, class A, int I>
__device__ __forceinline__ A pull_listed(const typename Store<ST>::elem *__restrict__ fa,
                                         long long c, long long S, int x, long long off,
                                         bool wbb, unsigned links, const SweepArgs &a) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using Dd = DirC<Q, I>;
  if constexpr (I == 0) {
    return SF::template load<A, L>(fa + c, a.L.fbase[0]);
  } else {
    const bool bb = wbb || ((links >> I) & 1u);
    long long src = c + off;
    if constexpr (Dd::ex < 0) src += (x == a.L.nx - 1) ? Dd::ex : 0;  // zero gradient
    A v = SF::template load<A, L>(fa + (bb ? (long long)Dd::opp * S + c : src),
                                  bb ? a.L.fbase[Dd::opp] : a.L.fbase[I]);
    if constexpr (Dd::ex > 0) v = (!bb && x == 0) ? inlet_pop<A>(a, I) : v;
    return v;
  }
}

// Force of one cell's solid bounce-backs, summed in the arithmetic type (at most
// Q - 1 terms): each adds 2 f*_{opp(I)}(X) e_{opp(I)} = -2 v_I e_I.
template <int Q, class A, class SF>
__device__ __forceinline__ void cell_force(const A *f, unsigned links, A &fx, A &fy, A &fz) {
  static_for(
      [&](auto ic) {
        constexpr int I = decltype(ic)::value;
        if constexpr (I > 0) {
          using O = VA<A>;
          const A m = ((links >> I) & 1u)
                          ? O::mul(A(2.0), f[I]) : A(0);
          if constexpr (Lat<Q>::ex(I) != 0) fx = Lat<Q>::ex(I) > 0 ? O::sub(fx, m) : O::add(fx, m);
          if constexpr (Lat<Q>::ey(I) != 0) fy = Lat<Q>::ey(I) > 0 ? O::sub(fy, m) : O::add(fy, m);
          if constexpr (Lat<Q>::ez(I) != 0) fz = Lat<Q>::ez(I) > 0 ? O::sub(fz, m) : O::add(fz, m);
        }
      },
      std::make_integer_sequence<int, Q>{});
}

// One cell of a listed tile in the arithmetic type A: the pull through the
// face-state tables and the link word (bit 31: a solid cell, whose p and u are
// zero), moments, BGK and the store; x >= nx loads the last column and stores
// nothing.
template <int Q, class ST, class A>
__device__ __forceinline__ void channel_listed_cell(const SweepArgs &a, int x, int y, int z,
                                                    unsigned links) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  const int nx = a.L.nx, ny = a.L.ny;
  const bool valid = x < nx;
  if (!valid) x = nx - 1;
  const long long S = a.L.S;
  const long long c = a.L.idx(x, y, z);
  const E *__restrict__ fa = static_cast<const E *>(a.fa);
  const int st = face_state(y, z, ny, a.L.nz);
  const long long *__restrict__ offs = a.face_off + st * Q;
  const unsigned wbb = a.face_bb[st];
  A f[Q];
  static_for(
      [&](auto ic) {
        constexpr int I = decltype(ic)::value;
        f[I] = pull_listed<Q, ST, A, I>(fa, c, S, x, offs[I], (wbb >> I) & 1u, links, a);
      },
      std::make_integer_sequence<int, Q>{});
  A rho3, ux, uy, uz;
  moments<L, A, SF>(f, rho3, ux, uy, uz);
  if (links >> 31) {
    rho3 = A(0); ux = A(0); uy = A(0); uz = A(0);
  }
  const long long cell = ((long long)z * ny + y) * nx + x;
  finish_cell<L, SF, A, E>(f, rho3, ux, uy, uz, cell, valid, static_cast<E *>(a.fb), c, S, a);
}

// Interior channel sweep with two cells per thread and packed FP32x2
// arithmetic: a warp takes the two warp tiles 2b and 2b + 1 of a row, so a thread
// owns cells x and x + 32, whose loads and stores share their address (the
// second is an immediate 32 elements further).  Moments and BGK run once on
// the pair type P = float2 with GB300's packed FFMA2/FADD2/FMUL2, halving the
// arithmetic instructions of the issue-bound FP32-collision forms.  (A
// double-float pair type needs ~250 registers for two cells' 27 populations;
// at 2-3 blocks per SM it ran at 2.9-3.9 G cell updates/s against 7.5 for one
// cell per thread at 5 blocks per SM, D3Q27 512x128x128.)  A pair holding a listed
// tile pulls through pull_pair_listed (face-state tables and link words), or,
// with LISTED1 in the kernel, takes its two cells one after the other through
// channel_listed_cell (the same values: lane for lane the packed operations
// are the scalar ones).
// POFF: the source offset from the kernel-parameter table a.poff (when `a` is a
// kernel parameter); otherwise formed from the layout strides (when `a` sits in
// global or shared memory, as in the batch, where the table would be a load).
template <int Q, class ST, class P, int I, bool POFF = true>
__device__ __forceinline__ P pull_pair(const typename Store<ST>::elem *__restrict__ p,
                                       const typename Store<ST>::elem *__restrict__ pm0,
                                       const typename Store<ST>::elem *__restrict__ pm1,
                                       long long S, long long rs, long long zs, bool act0,
                                       bool act1, bool inlet0, const SweepArgs &a) {
  using Dd = DirC<Q, I>;
  using PC = PairCodec<ST>;
  long long off;
  if constexpr (POFF) off = a.poff[I];
  else off = I * S - (Dd::ex + Dd::ey * rs + Dd::ez * zs);
  float r0 = 0.0f, r1 = 0.0f;
  if constexpr (Dd::ex < 0) {  // the outlet column repeats itself (pm = p - 1 there)
    if (act0) r0 = PC::raw(__ldg(pm0 + off));
    if (act1) r1 = PC::raw(__ldg(pm1 + off));
  } else {
    if (act0) r0 = PC::raw(__ldg(p + off));
    if (act1) r1 = PC::raw(__ldg(p + off + 32));
  }
  const float b = a.L.fbase[I];
  float2 v = PC::dec(make_float2(r0, r1), make_float2(b, b));
  if constexpr (Dd::ex > 0) v.x = inlet0 ? a.f_in_f[I] : v.x;
  return v;
}

// The pair pull of a listed tile pair: pull_listed for cells x0 and x0 + 32
// (l0 / l1 their link words), both loads issued.
template <int Q, class ST, class P, int I>
__device__ __forceinline__ P pull_pair_listed(const typename Store<ST>::elem *__restrict__ p,
                                              long long S, long long off, bool wbb,
                                              unsigned l0, unsigned l1, bool act1,
                                              bool out0, bool out1, bool inlet0,
                                              const SweepArgs &a) {
  using Dd = DirC<Q, I>;
  using PC = PairCodec<ST>;
  if constexpr (I == 0) {
    const float b = a.L.fbase[0];
    return PC::dec(make_float2(PC::raw(__ldg(p)), act1 ? PC::raw(__ldg(p + 32)) : 0.0f),
                   make_float2(b, b));
  } else {
    const bool bb0 = wbb || ((l0 >> I) & 1u), bb1 = wbb || ((l1 >> I) & 1u);
    long long s0 = off, s1 = off + 32;
    if constexpr (Dd::ex < 0) {  // zero gradient at the outlet column
      s0 += out0 ? Dd::ex : 0;
      s1 += out1 ? Dd::ex : 0;
    }
    constexpr long long OS = Dd::opp;
    const float b0 = bb0 ? a.L.fbase[Dd::opp] : a.L.fbase[I];
    const float b1 = bb1 ? a.L.fbase[Dd::opp] : a.L.fbase[I];
    const float r0 = PC::raw(__ldg(p + (bb0 ? a.doff[OS] : s0)));
    const float r1 = act1 ? PC::raw(__ldg(p + (bb1 ? a.doff[OS] + 32 : s1))) : 0.0f;
    float2 v = PC::dec(make_float2(r0, r1), make_float2(b0, b1));
    if constexpr (Dd::ex > 0) v.x = (!bb0 && inlet0) ? a.f_in_f[I] : v.x;
    return v;
  }
}

// Cells x0 and x0 + 32 of row (y, z) (x0 = 32 * even warp tile + lane); act0 /
// act1: the two warp tiles are unlisted (warp-uniform).
// LISTED: the pair holds a listed tile; both cells pull through the face-state
// tables and their link words l0 / l1 (bit 31: solid cell), act0 = true and
// act1 = the second tile exists.
template <int Q, class ST, class P, bool LISTED = false, bool POFF = true>
__device__ __forceinline__ void channel2_cells(const SweepArgs &a, int x0, int y, int z,
                                               bool act0, bool act1, unsigned l0 = 0u,
                                               unsigned l1 = 0u) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  using O = VA<P>;
  using T = PairT<P>;
  using C = typename T::C;
  const int nx = a.L.nx, ny = a.L.ny;
  const int x1 = x0 + 32;
  const bool st0 = act0 && x0 < nx, st1 = act1 && x1 < nx;
  const long long S = a.L.S;
  const long long c = a.L.idx(x0, y, z);
  const E *__restrict__ fa = static_cast<const E *>(a.fa);
  const E *__restrict__ p = fa + c;
  const E *__restrict__ pm0 = p - (x0 == nx - 1 ? 1 : 0);
  const E *__restrict__ pm1 = p + 32 - (x1 == nx - 1 ? 1 : 0);
  const bool inlet0 = x0 == 0;
  P f[Q];
  if constexpr (LISTED) {
    const int st = face_state(y, z, ny, a.L.nz);
    const long long *__restrict__ offs = a.face_off + st * Q;
    const unsigned wbb = a.face_bb[st];
    static_for(
        [&](auto ic) {
          constexpr int I = decltype(ic)::value;
          f[I] = pull_pair_listed<Q, ST, P, I>(p, S, offs[I], (wbb >> I) & 1u, l0, l1, act1,
                                               x0 == nx - 1, x1 == nx - 1, inlet0, a);
        },
        std::make_integer_sequence<int, Q>{});
  } else {
    static_for(
        [&](auto ic) {
          constexpr int I = decltype(ic)::value;
          f[I] = pull_pair<Q, ST, P, I, POFF>(p, pm0, pm1, S, a.L.rs, a.L.zs, act0, act1,
                                              inlet0, a);
        },
        std::make_integer_sequence<int, Q>{});
  }
  P rho3, ux, uy, uz;
  moments<L, P, SF>(f, rho3, ux, uy, uz);
  if constexpr (LISTED) {  // solid cells: p = u = 0
    const C z0 = C(0.0f);
    if (l0 >> 31) {
      rho3 = T::make(z0, T::y(rho3)); ux = T::make(z0, T::y(ux));
      uy = T::make(z0, T::y(uy)); uz = T::make(z0, T::y(uz));
    }
    if (l1 >> 31) {
      rho3 = T::make(T::x(rho3), z0); ux = T::make(T::x(ux), z0);
      uy = T::make(T::x(uy), z0); uz = T::make(T::x(uz), z0);
    }
  }
  const long long cell0 = ((long long)z * ny + y) * nx + x0;
  if (a.mu) {
    if (st0) {
      a.mu[cell0] = T::to_double(T::x(ux));
      a.mv[cell0] = T::to_double(T::x(uy));
      a.mw[cell0] = T::to_double(T::x(uz));
      a.mp[cell0] = T::to_double(T::third(T::x(rho3)));
    }
    if (st1) {
      a.mu[cell0 + 32] = T::to_double(T::y(ux));
      a.mv[cell0 + 32] = T::to_double(T::y(uy));
      a.mw[cell0 + 32] = T::to_double(T::y(uz));
      a.mp[cell0 + 32] = T::to_double(T::third(T::y(rho3)));
    }
  }
  if (a.alpha) {
    const P sb = T::make(C(__fsub_rn(1.0f, st0 ? a.alpha[cell0] : 0.0f)),
                         C(__fsub_rn(1.0f, st1 ? a.alpha[cell0 + 32] : 0.0f)));
    ux = O::mul(ux, sb);
    uy = O::mul(uy, sb);
    uz = O::mul(uz, sb);
  }
  bgk_relax_v<L, P, SF>(f, rho3, ux, uy, uz, a);
  E *__restrict__ q = static_cast<E *>(a.fb) + c;
#pragma unroll
  for (int i = 0; i < L::Q; ++i)
    PairCodec<ST>::template put2<Q>(q + i * S, q + i * S + 32, f[i], a.L.fbase[i], st0, st1,
                                    (unsigned)(cell0 * Q + i), a.f16_sr);
}

template <int Q, class ST, class P, int MINB, bool LISTED1 = false>
__global__ void __launch_bounds__(SWEEP_BX * SWEEP_BY, MINB)
    sweep_channel2_kernel(const SweepArgs a) {
  const int ny = a.L.ny;
  const int y = blockIdx.y * SWEEP_BY + threadIdx.y, z = blockIdx.z;
  if (y >= ny) return;
  const int w0 = 2 * blockIdx.x;
  const long long trow = ((long long)z * ny + y) * a.nxw;
  const bool has1 = w0 + 1 < a.nxw;
  const int t0 = a.tile_index[trow + w0];
  const int t1 = has1 ? a.tile_index[trow + w0 + 1] : -1;
  const int x0 = 32 * w0 + threadIdx.x;
  // A listed pair returns from its own inlined code: with the packed listed
  // and plain bodies in an if / else the FP16 kernel spilled 196 bytes, in
  // this form 60.
  if (t0 >= 0 || t1 >= 0) {  // warp-uniform
    const unsigned l0 = t0 >= 0 ? a.links_bits[(long long)t0 * SWEEP_BX + threadIdx.x] : 0u;
    const unsigned l1 = t1 >= 0 ? a.links_bits[(long long)t1 * SWEEP_BX + threadIdx.x] : 0u;
    if constexpr (LISTED1) {
#pragma unroll 1
      for (int h = 0; h < (has1 ? 2 : 1); ++h)
        channel_listed_cell<Q, ST, typename PairT<P>::C>(a, x0 + 32 * h, y, z, h ? l1 : l0);
    } else {
      channel2_cells<Q, ST, P, true>(a, x0, y, z, true, has1, l0, l1);
    }
    return;
  }
  channel2_cells<Q, ST, P>(a, x0, y, z, true, has1);
}

// Channel sweep, one cell per thread, one warp tile per warp, over the whole
// box: unlisted tiles pull plainly, listed tiles through the face-state tables
// and their link words (solid cells zeroed).  The tile's listed position is
// warp-uniform, so is the branch.
template <int Q, class ST, class A, int MINB>
__global__ void __launch_bounds__(SWEEP_BX * SWEEP_BY, MINB) sweep_channel_kernel(const SweepArgs a) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  const int nx = a.L.nx, ny = a.L.ny;
  const int lane = threadIdx.x;
  const int y = blockIdx.y * SWEEP_BY + threadIdx.y, z = blockIdx.z;
  if (y >= ny) return;
  const int t = a.tile_index[((long long)z * ny + y) * a.nxw + blockIdx.x];
  int x = blockIdx.x * SWEEP_BX + lane;
  const bool valid = x < nx;
  if (!valid) x = nx - 1;
  const long long S = a.L.S;
  const long long c = a.L.idx(x, y, z);
  const E *__restrict__ fa = static_cast<const E *>(a.fa);
  E *__restrict__ fb = static_cast<E *>(a.fb);
  A f[Q];
  bool solid_here = false;
  if (t >= 0) {
    const unsigned links = a.links_bits[(long long)t * SWEEP_BX + lane];
    solid_here = links >> 31;
    const int st = face_state(y, z, ny, a.L.nz);
    const long long *__restrict__ offs = a.face_off + st * Q;
    const unsigned wbb = a.face_bb[st];
    static_for(
        [&](auto ic) {
          constexpr int I = decltype(ic)::value;
          f[I] = pull_listed<Q, ST, A, I>(fa, c, S, x, offs[I], (wbb >> I) & 1u, links, a);
        },
        std::make_integer_sequence<int, Q>{});
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

// Sums per-thread FP64 force partials of a small grid: warp shuffles, per
// block into partials[blockIdx.x], then over blocks, in block order, by the last
// block to finish, into the force-history slot of this step.
__device__ __forceinline__ void force_to_history(const SweepArgs &a, double dx, double dy,
                                                 double dz) {
  constexpr int NW = SWEEP_BY;
  const int lane = threadIdx.x, wid = threadIdx.y;
  const int tid = wid * SWEEP_BX + lane;
  __shared__ double sh[3][NW];
  __shared__ bool last;
  for (int o = 16; o > 0; o >>= 1) {
    dx += __shfl_down_sync(0xffffffffu, dx, o);
    dy += __shfl_down_sync(0xffffffffu, dy, o);
    dz += __shfl_down_sync(0xffffffffu, dz, o);
  }
  if (lane == 0) {
    sh[0][wid] = dx;
    sh[1][wid] = dy;
    sh[2][wid] = dz;
  }
  __syncthreads();
  if (tid == 0) {
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int w = 0; w < NW; ++w) { bx += sh[0][w]; by += sh[1][w]; bz += sh[2][w]; }
    a.partials[3 * blockIdx.x] = bx;
    a.partials[3 * blockIdx.x + 1] = by;
    a.partials[3 * blockIdx.x + 2] = bz;
    __threadfence();
    last = atomicAdd(a.counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    const volatile double *p = a.partials;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (unsigned k = tid; k < gridDim.x; k += SWEEP_BX * SWEEP_BY) {
      s0 += p[3 * k];
      s1 += p[3 * k + 1];
      s2 += p[3 * k + 2];
    }
    for (int o = 16; o > 0; o >>= 1) {
      s0 += __shfl_down_sync(0xffffffffu, s0, o);
      s1 += __shfl_down_sync(0xffffffffu, s1, o);
      s2 += __shfl_down_sync(0xffffffffu, s2, o);
    }
    __syncthreads();
    if (lane == 0) {
      sh[0][wid] = s0;
      sh[1][wid] = s1;
      sh[2][wid] = s2;
    }
    __syncthreads();
    if (tid == 0) {
      double tx = 0.0, ty = 0.0, tz = 0.0;
      for (int w = 0; w < NW; ++w) { tx += sh[0][w]; ty += sh[1][w]; tz += sh[2][w]; }
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

// Momentum-exchange force on the solids for this step, beside the sweep on a
// second stream: a small grid (at most one block per SM) strides over the
// boundary cells (fluid cells with solid links; the set-up's list, in tile and
// x order), one cell per thread, and reads the populations the sweep bounces
// back (f*_{opp(I)}(X) from the state it pulls from); per cell the sum runs in
// the arithmetic type, over cells in FP64.
template <int Q, class ST, class A, int MINB>
__global__ void __launch_bounds__(SWEEP_BX * SWEEP_BY, MINB) channel_force_kernel(const SweepArgs a) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  const long long S = a.L.S;
  const E *__restrict__ fa = static_cast<const E *>(a.fa);
  const long long stride = (long long)gridDim.x * SWEEP_BX * SWEEP_BY;
  double dx = 0.0, dy = 0.0, dz = 0.0;
  for (long long k = (long long)blockIdx.x * SWEEP_BX * SWEEP_BY + threadIdx.y * SWEEP_BX +
                     threadIdx.x;
       k < a.n_bcells; k += stride) {
    const unsigned links = a.bcell_links[k];
    const long long c = a.bcell_idx[k];
    A f[Q];
    static_for(
        [&](auto ic) {
          constexpr int I = decltype(ic)::value;
          f[I] = ((links >> I) & 1u)
                     ? SF::template load<A, L>(fa + (long long)DirC<Q, I>::opp * S + c,
                                               a.L.fbase[DirC<Q, I>::opp])
                     : A(0);
        },
        std::make_integer_sequence<int, Q>{});
    A Fx = A(0), Fy = A(0), Fz = A(0);
    cell_force<Q, A, SF>(f, links, Fx, Fy, Fz);
    if constexpr (sizeof(A) == 4) {
      dx += f2d_bits(Fx);
      dy += f2d_bits(Fy);
      dz += f2d_bits(Fz);
    } else {
      dx += Fx;
      dy += Fy;
      dz += Fz;
    }
  }
  force_to_history(a, dx, dy, dz);
}

// Macroscopic fields of the step that read a.fa, formed on request instead of
// in every step: the step's pull (the resolved pull, which equals the plain one
// away from faces and solids), its moments and its solid rule, one cell per
// thread, written as the sweep writes them.  Reads the Q populations of every
// cell once and writes 4 doubles per cell.
template <int Q, class ST, class A>
__global__ void __launch_bounds__(SWEEP_BX * SWEEP_BY) macros_channel_kernel(const SweepArgs a) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  const int nx = a.L.nx, ny = a.L.ny;
  const int lane = threadIdx.x;
  const int y = blockIdx.y * SWEEP_BY + threadIdx.y, z = blockIdx.z;
  if (y >= ny) return;
  const long long tile = ((long long)z * ny + y) * a.nxw + blockIdx.x;
  const int t = a.tile_index[tile];
  int x = blockIdx.x * SWEEP_BX + lane;
  const bool valid = x < nx;
  if (!valid) x = nx - 1;
  const unsigned links = t >= 0 ? a.links_bits[(long long)t * SWEEP_BX + lane] : 0u;
  const bool solid_here = t >= 0 && mask_solid(a.mask, a.nxw, ny, x, y, z);
  const long long S = a.L.S;
  const long long c = a.L.idx(x, y, z);
  const E *__restrict__ fa = static_cast<const E *>(a.fa);
  A f[Q];
  static_for(
      [&](auto ic) {
        constexpr int I = decltype(ic)::value;
        f[I] = pull_resolved<Q, ST, A, I>(fa, c, S, x, y, z, links, a);
      },
      std::make_integer_sequence<int, Q>{});
  A rho3, ux, uy, uz;
  moments<L, A, SF>(f, rho3, ux, uy, uz);
  if (solid_here) {
    rho3 = A(0); ux = A(0); uy = A(0); uz = A(0);
  }
  if (valid) store_macros<A>(a, ((long long)z * ny + y) * nx + x, rho3, ux, uy, uz);
}

// The post-stream (pre-collision) populations of the step that read a.fa, in
// FP64, dense [i][z][y][x] into out: what the reference's f holds after its
// Streaming() and Update().  Channel profile: the step's resolved pull;
// reference profiles: the plain pull from the ghost-filled state.
template <int Q, class ST, bool REF>
__global__ void __launch_bounds__(SWEEP_BX * SWEEP_BY) stream_state_kernel(const SweepArgs a,
                                                                           double *out) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  const int nx = a.L.nx, ny = a.L.ny;
  const int lane = threadIdx.x;
  const int y = blockIdx.y * SWEEP_BY + threadIdx.y, z = blockIdx.z;
  const int x = blockIdx.x * SWEEP_BX + lane;
  if (y >= ny || x >= nx) return;
  const long long S = a.L.S;
  const long long c = a.L.idx(x, y, z);
  const E *__restrict__ fa = static_cast<const E *>(a.fa);
  const long long N = (long long)nx * ny * a.L.nz;
  const long long cell = ((long long)z * ny + y) * nx + x;
  unsigned links = 0u;
  if constexpr (!REF) {
    const int t = a.tile_index[((long long)z * ny + y) * a.nxw + blockIdx.x];
    links = t >= 0 ? a.links_bits[(long long)t * SWEEP_BX + lane] : 0u;
  }
  static_for(
      [&](auto ic) {
        constexpr int I = decltype(ic)::value;
        double v;
        if constexpr (REF)
          v = SF::template load<double, L>(fa + I * S + c - a.L.off(L::ex(I), L::ey(I), L::ez(I)),
                                           a.L.fbase[I]);
        else
          v = pull_resolved<Q, ST, double, I>(fa, c, S, x, y, z, links, a);
        out[(long long)I * N + cell] = v;
      },
      std::make_integer_sequence<int, Q>{});
}

template <int Q, class ST>
cudaError_t launch_stream_state_t(const SweepArgs &a, bool ref, double *out, cudaStream_t s) {
  dim3 block(SWEEP_BX, SWEEP_BY, 1);
  dim3 grid((a.L.nx + SWEEP_BX - 1) / SWEEP_BX, (a.L.ny + SWEEP_BY - 1) / SWEEP_BY, a.L.nz);
  if (ref) stream_state_kernel<Q, ST, true><<<grid, block, 0, s>>>(a, out);
  else stream_state_kernel<Q, ST, false><<<grid, block, 0, s>>>(a, out);
  count_launch();
  return cudaGetLastError();
}

template <int Q, class ST, class A>
cudaError_t launch_macros_channel_t(const SweepArgs &a, cudaStream_t s) {
  dim3 block(SWEEP_BX, SWEEP_BY, 1);
  dim3 grid((a.L.nx + SWEEP_BX - 1) / SWEEP_BX, (a.L.ny + SWEEP_BY - 1) / SWEEP_BY, a.L.nz);
  macros_channel_kernel<Q, ST, A><<<grid, block, 0, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

// The interior launch: FP32 collision on FP32 or FP16 storage takes the packed
// two-cells-per-thread kernel; the others the one-cell kernel.
template <int Q, class ST, class A, int MINB_FAST>
void launch_interior(const SweepArgs &a, dim3 grid, dim3 block, cudaStream_t s) {
  if constexpr (Q == 27 && sizeof(A) == 4 && std::is_same<ST, F16Dev>::value) {
    if (a.lines) {  // FP16, ROWS layout: the line-staged sweep
      (void)launch_lines_f16_q27(a, a.sms, s);
      return;
    }
  }
  if constexpr (sizeof(A) == 4 && !std::is_same<ST, double>::value) {
    // Blocks per SM, measured on the D3Q27 bench step with packed listed
    // pairs: FP32 storage 0.850 / 0.908 / 0.937 of the copy peak at 4 / 5 / 6
    // per SM (7 and 8 spill more); FP16 0.613 / 0.636 / 0.632.  D2Q9 on grids
    // of 2^20 cells and more: 10 per SM (48 registers; 8192x1024: FP32 storage
    // 0.982 against 0.946 at 6, FP16 0.729 against 0.659); smaller D2Q9 grids
    // are bound by per-thread latency (640x160 FP32: 6.1 us per step at 6
    // against 6.6 at 10).
    dim3 g2((a.nxw + 1) / 2, grid.y, grid.z);
    if constexpr (Q == 9) {
      if ((long long)a.L.nx * a.L.ny * a.L.nz >= (1LL << 20)) {
        sweep_channel2_kernel<Q, ST, float2, 10><<<g2, block, 0, s>>>(a);
        return;
      }
    }
    // Listed pairs: packed (both cells at once) or one cell after the other
    // (LISTED1; fewer live registers).  One cell at a time, measured on the
    // channel steps: FP16 D3Q27 39.5 against 37.5 G cell updates/s on
    // 512x128x128 and 47.4 against 45.3 on 768x384x384 (5 per SM; 37.9 / 46.4
    // at 6), FP32 D2Q9 400x100 6.66 against 6.46 (5 per SM); FP32 D3Q27 the
    // same either way (31.0 / 32.2 at 6 per SM); the wide D2Q9 grids 1-2 %
    // slower (8192x1024: FP16 129.5 against 130.8, FP32 91.4 against 93.3).
    if constexpr (Q == 27 && std::is_same<ST, float>::value)
      sweep_channel2_kernel<Q, ST, float2, 6><<<g2, block, 0, s>>>(a);
    else
      sweep_channel2_kernel<Q, ST, float2, 5, true><<<g2, block, 0, s>>>(a);
  } else {
    sweep_channel_kernel<Q, ST, A, MINB_FAST><<<grid, block, 0, s>>>(a);
  }
}

template <int Q, class ST, class A, int MINB_FAST, int MINB_SLOW>
cudaError_t launch_sweep_channel_t(const SweepArgs &a, cudaStream_t s, const SweepFork *fk) {
  dim3 block(SWEEP_BX, SWEEP_BY, 1);
  dim3 grid((a.L.nx + SWEEP_BX - 1) / SWEEP_BX, (a.L.ny + SWEEP_BY - 1) / SWEEP_BY, a.L.nz);
  const int sb = a.bnd_blocks;
  if (fk && fk->side) {
    // The force launch goes first on the (higher-priority) side stream, so its
    // latency-bound blocks overlap the sweep's streaming.
    cudaError_t e = cudaEventRecord(fk->fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(fk->side, fk->fork, 0);
    if (e != cudaSuccess) return e;
    channel_force_kernel<Q, ST, A, MINB_SLOW><<<sb > 0 ? sb : 1, block, 0, fk->side>>>(a);
    e = cudaEventRecord(fk->join, fk->side);
    if (e != cudaSuccess) return e;
    launch_interior<Q, ST, A, MINB_FAST>(a, grid, block, s);
    e = cudaStreamWaitEvent(s, fk->join, 0);
    if (e != cudaSuccess) return e;
  } else {
    launch_interior<Q, ST, A, MINB_FAST>(a, grid, block, s);
    channel_force_kernel<Q, ST, A, MINB_SLOW><<<sb > 0 ? sb : 1, block, 0, s>>>(a);
  }
  count_launch(2);
  return cudaGetLastError();
}

}  // namespace cflbm
