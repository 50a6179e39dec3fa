// Kokkos-subset shim (random numbers): TEST INFRASTRUCTURE ONLY.
//
// Random_XorShift64_Pool<> hands out xorshift64* generator states.  The
// reference draws one integer per grid node with state.urand(100) inside a
// parallel_for.  Real Kokkos gives each thread its own state, so the field the
// reference draws is already thread-schedule dependent; this shim keeps ONE
// state behind a lock so a run is reproducible for a fixed thread count.  The
// oracle drivers dump the drawn field ("ran") so every other implementation is
// seeded from exactly the values the reference used.
#pragma once
#include <cstdint>
#include <mutex>
#include <memory>
#include "Kokkos_Core.hpp"

namespace Kokkos {

template <class Gen, class Scalar> struct rand;

template <class Device = void>
class Random_XorShift64 {
 public:
  explicit Random_XorShift64(uint64_t *s) : s_(s) {}
  uint64_t urand64() {
    uint64_t x = *s_;
    x ^= x >> 12;
    x ^= x << 25;
    x ^= x >> 27;
    *s_ = x;
    return x * 2685821657736338717ULL;
  }
  uint32_t urand() { return static_cast<uint32_t>(urand64() >> 32); }
  uint32_t urand(uint32_t range) { return static_cast<uint32_t>((urand64() >> 32) % range); }
  double drand() { return (urand64() >> 11) * (1.0 / 9007199254740992.0); }

 private:
  uint64_t *s_;
};

template <class Device = void>
class Random_XorShift64_Pool {
 public:
  using generator_type = Random_XorShift64<Device>;
  explicit Random_XorShift64_Pool(uint64_t seed)
      : st_(std::make_shared<State>()) {
    st_->s = seed ? seed * 0x9E3779B97F4A7C15ULL : 0x9E3779B97F4A7C15ULL;
  }
  generator_type get_state() const {
    st_->m.lock();
    return generator_type(&st_->s);
  }
  void free_state(const generator_type &) const { st_->m.unlock(); }

 private:
  struct State {
    std::mutex m;
    uint64_t s;
  };
  std::shared_ptr<State> st_;
};

template <class D>
struct rand<Random_XorShift64<D>, double> {
  static double draw(Random_XorShift64<D> &g) { return g.drand(); }
};

}  // namespace Kokkos
