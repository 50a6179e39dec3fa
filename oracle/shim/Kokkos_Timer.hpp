// Kokkos-subset shim (timer): TEST INFRASTRUCTURE ONLY.
#pragma once
#include <chrono>

namespace Kokkos {
class Timer {
 public:
  Timer() : t0_(std::chrono::steady_clock::now()) {}
  void reset() { t0_ = std::chrono::steady_clock::now(); }
  double seconds() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
  }

 private:
  std::chrono::steady_clock::time_point t0_;
};
}  // namespace Kokkos
