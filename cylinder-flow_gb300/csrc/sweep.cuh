// The fused collide-and-stream sweep: one pass over the interior per time step.
//
// For every interior cell x the kernel pulls f_i from x - e_i in the
// post-collision buffer A (ghost layers and the populations of solid cells that
// face fluid have been filled beforehand, so the pull needs no boundary logic),
// forms p = sum f / 3 and u = sum f e (the reference's LBM::Update,
// "3D MPI+KOKKOS+MPIIO/lbm.cpp:384-415"), zeroes them in solid cells, applies the
// reference profiles' inlet/outlet overrides, relaxes every population toward
// feq_i = t_i (3p + 3 e.u + 4.5 (e.u)^2 - 1.5 u^2) with rate omega (the
// reference's LBM::Collision, lbm.cpp:257-272, where omega = 1/(tau0+0.5)), and
// writes the result to B.  This replaces the reference's five separate passes
// (collision, stream1 into ft, stream2 copy-back, the host Update loop) by one
// read and one write of every population.
//
// HBM traffic per cell update: Q loads + Q stores of the storage type (no reuse
// is needed: in the SoA layout each population is a pure shift, so every
// element of A is read exactly once per sweep) plus 1/8 byte of solid mask.
#pragma once
#include "solver.cuh"

namespace cflbm {

template <int Q, class ST, class A, int MINB>
__global__ void __launch_bounds__(128, MINB) sweep_kernel(const SweepArgs a) {
  using L = Lat<Q>;
  using SF = Store<ST>;
  using E = typename SF::elem;
  const int x = blockIdx.x * 32 + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= a.L.nx || y >= a.L.ny) return;
  const long long S = a.L.S;
  const long long c = a.L.idx(x, y, z);
  const long long row = a.L.px;
  const long long plane = (long long)a.L.px * a.L.nyp;
  const E *__restrict__ fa = static_cast<const E *>(a.fa);
  E *__restrict__ fb = static_cast<E *>(a.fb);

  A f[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const long long o = L::ex(i) + L::ey(i) * row + L::ez(i) * plane;
    f[i] = SF::template load<A, L>(fa + i * S + c - o, i);
  }

  // Moments (deviation form: rho3 = 3p = sum f, u = sum f e).
  A rho3 = f[0], ux = A(0), uy = A(0), uz = A(0);
#pragma unroll
  for (int k = 0; k < L::NPAIR; ++k) {
    const int i = L::pair(k), j = L::opp(L::pair(k));
    const A s = f[i] + f[j];
    const A d = f[i] - f[j];
    rho3 += s;
    if (L::ex(i) > 0) ux += d; else if (L::ex(i) < 0) ux -= d;
    if (L::ey(i) > 0) uy += d; else if (L::ey(i) < 0) uy -= d;
    if (L::ez(i) > 0) uz += d; else if (L::ez(i) < 0) uz -= d;
  }
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
  if (a.mu) {
    a.mu[cell] = static_cast<double>(ux);
    a.mv[cell] = static_cast<double>(uy);
    a.mw[cell] = static_cast<double>(uz);
    a.mp[cell] = static_cast<double>(rho3) / 3.0;
  }
  if (a.alpha) {
    const A s = A(1) - static_cast<A>(a.alpha[cell]);
    ux *= s;
    uy *= s;
    uz *= s;
  }

  // BGK relaxation, written per +/- pair: the pair shares (e.u)^2 and the
  // even part of feq; the odd part flips sign.
  A om;
  if constexpr (sizeof(A) == 8) om = a.omega; else om = a.omega_f;
  const A c0 = rho3 - A(1.5) * (ux * ux + uy * uy + uz * uz);
  f[0] = f[0] + om * (A(L::w(0)) * c0 - f[0]);
#pragma unroll
  for (int k = 0; k < L::NPAIR; ++k) {
    const int i = L::pair(k), j = L::opp(L::pair(k));
    A eu = A(0);
    if (L::ex(i) > 0) eu += ux; else if (L::ex(i) < 0) eu -= ux;
    if (L::ey(i) > 0) eu += uy; else if (L::ey(i) < 0) eu -= uy;
    if (L::ez(i) > 0) eu += uz; else if (L::ez(i) < 0) eu -= uz;
    const A sym = A(L::w(i)) * (c0 + A(4.5) * eu * eu);
    const A asym = A(3.0 * L::w(i)) * eu;
    f[i] = f[i] + om * ((sym + asym) - f[i]);
    f[j] = f[j] + om * ((sym - asym) - f[j]);
  }

#pragma unroll
  for (int i = 0; i < Q; ++i) SF::template store<A, L>(fb + i * S + c, f[i], i);
}

template <int Q, class ST, class A, int MINB>
cudaError_t launch_sweep_t(const SweepArgs &a, cudaStream_t s) {
  dim3 block(32, 4, 1);
  dim3 grid((a.L.nx + 31) / 32, (a.L.ny + 3) / 4, a.L.nz);
  sweep_kernel<Q, ST, A, MINB><<<grid, block, 0, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

}  // namespace cflbm
