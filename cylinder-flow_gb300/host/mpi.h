/* mpi.h -- the single-rank subset of MPI that the reference's drivers call,
 * for building them unmodified against the drop-in classes (lbm.hpp,
 * System.hpp) on one GPU.
 *
 * The reference's 3-D main ("3D MPI+KOKKOS+MPIIO/main.cpp:1-51") calls
 * MPI_Init, MPI_Comm_rank, MPI_Barrier, MPI_Wtime and MPI_Finalize on
 * MPI_COMM_WORLD; at one rank these are bookkeeping only: rank 0 of 1, a
 * barrier that returns at once, a monotonic wall clock.  Put this directory
 * first on the include path (-I .../host) in place of an MPI installation.
 */
#ifndef CFLBM_HOST_MPI_H
#define CFLBM_HOST_MPI_H

#include <stdio.h>
#include <time.h>

#define MPI_VERSION 3
#define MPI_SUCCESS 0

typedef int MPI_Comm;
#define MPI_COMM_WORLD ((MPI_Comm)0)

static inline int MPI_Init(int *argc, char ***argv) {
  (void)argc;
  (void)argv;
  return MPI_SUCCESS;
}
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm comm, int *rank) {
  (void)comm;
  *rank = 0;
  return MPI_SUCCESS;
}
static inline int MPI_Comm_size(MPI_Comm comm, int *size) {
  (void)comm;
  *size = 1;
  return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm comm) {
  (void)comm;
  return MPI_SUCCESS;
}
static inline double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#endif
