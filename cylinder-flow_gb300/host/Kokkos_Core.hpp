// Kokkos_Core.hpp -- what the reference's drivers take from Kokkos when they run
// on the drop-in classes: Kokkos::initialize and Kokkos::finalize
// ("3D MPI+KOKKOS+MPIIO/main.cpp:11,48").  The drop-in's state lives on the GPU
// behind the C ABI (include/cflbm.h), so there is no Kokkos execution space to
// start; both calls do nothing.  Put this directory first on the include path
// (-I .../host) in place of a Kokkos installation.
#ifndef CFLBM_HOST_KOKKOS_CORE_HPP
#define CFLBM_HOST_KOKKOS_CORE_HPP

namespace Kokkos {
inline void initialize(int &argc, char *argv[]) {
  (void)argc;
  (void)argv;
}
inline void initialize() {}
inline void finalize() {}
}  // namespace Kokkos

#endif
