// Drop-in replacement of the reference's System class
// ("3D MPI+KOKKOS+MPIIO/System.hpp:7-20", System.cpp:5-41).
//
// System() reads ./input.in exactly as the reference does -- the first nine
// numbers, whitespace separated: rho0 R Re / u0 Time inter / nx ny nz -- and
// derives cs2, cs, Ma, miu, tau = u0*R/Re/cs2 and then OVERRIDES Time and inter
// with (2R)^2/miu and Time/10, as the reference does (System.cpp:19-22).
//
// Extension (ignored by the reference, which stops after nine numbers): after
// the "=============" separator, lines of the form "cflbm.<key> <value>" set
// solver options: lattice (9|27), profile (ref2d|ref3d|channel), storage
// (fp64|fp32|fp16dev), compute (fp64|fp32|df64), steps (overrides the derived Time),
// inter, geom (none|cylinder|sphere), center (cx cy cz), diam, wall_y, wall_z
// (freeslip|noslip|periodic), perturb (amplitude), seed, rounding
// (stochastic|nearest: FP16 stores).  An unknown key or value sets ok = false
// and names it in `error`.
#ifndef CFLBM_HOST_SYSTEM_HPP
#define CFLBM_HOST_SYSTEM_HPP
#include <cstdint>
#include <string>
#include <vector>

class System {
 public:
  System();                             // reads ./input.in
  explicit System(const std::string &path);
  void Monitor();

  int sx, sy, sz;
  int Time, inter;
  double miu, u0, R, rho0, Ma, tau;
  int Re;
  double cs2, cs;

  // Extension options (defaults reproduce the reference's 3-D run).
  int lattice = 27;
  int profile = 2;  // CFLBM_PROFILE_REF3D
  int storage = 0;
  int compute = 0;
  int rounding = 1;  // CFLBM_ROUND_STOCHASTIC
  int geom = 0;
  double cx = 0, cy = 0, cz = 0, diam = 0;
  int wall_y = 0, wall_z = 2;
  double perturb = 0.0;
  uint64_t seed = 1234;
  bool ok = false;  // input.in was found and parsed
  std::string error;  // why not (an unreadable file, a bad extension key or value)
  bool ext_error = false;             // `error` is about an extension key
  std::vector<std::string> ext_keys;  // the extension keys the file set, in order

 private:
  void read(const std::string &path);
};
#endif
