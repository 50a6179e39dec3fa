/* Single-rank MPI stub: TEST INFRASTRUCTURE ONLY.
 *
 * The reference's MPI variants ("MPI Kokkos/", "3D MPI+KOKKOS+MPIIO/") call a
 * small part of MPI: communicator size/rank, Barrier, Allgather, Reduce,
 * blocking Send/Recv, and MPI-IO (File_open/seek/write, a Fortran-order
 * subarray file view and File_write_all).  No MPI library is installed here, so
 * this header implements those calls for exactly one rank, which is the
 * configuration the GPU solver replaces: every neighbour is -1, collectives are
 * copies, and the subarray view of rank 0 covers the whole global array, so a
 * collective write is a sequential write at the view's displacement.
 * Anything that would need a second rank aborts with a message. */
#ifndef CFLBM_ORACLE_MPI_STUB_H
#define CFLBM_ORACLE_MPI_STUB_H

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <vector>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef int MPI_Request;
struct MPI_Status { int MPI_SOURCE, MPI_TAG, MPI_ERROR; };
typedef std::FILE *MPI_File;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_REAL 5
#define MPI_DOUBLE 8
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_INFO_NULL 0
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 4
#define MPI_SEEK_SET 0
#define MPI_ORDER_FORTRAN 57
#define MPI_ORDER_C 56
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

namespace cflbm_mpi_stub {
struct TypeInfo {
  size_t bytes;     /* size of one element of this type */
  bool full_array;  /* derived type covering a whole global array */
};
inline std::vector<TypeInfo> &types() {
  static std::vector<TypeInfo> t = [] {
    std::vector<TypeInfo> v(16, TypeInfo{0, true});
    v[MPI_CHAR] = {1, true};
    v[MPI_INT] = {4, true};
    v[MPI_REAL] = {4, true};
    v[MPI_DOUBLE] = {8, true};
    return v;
  }();
  return t;
}
inline size_t type_bytes(MPI_Datatype t) { return types().at(t).bytes; }
[[noreturn]] inline void die(const char *what) {
  std::fprintf(stderr, "single-rank MPI stub: %s needs more than one rank\n", what);
  std::abort();
}
}  // namespace cflbm_mpi_stub

inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline double MPI_Wtime() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
inline int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int, MPI_Datatype,
                         MPI_Comm) {
  std::memcpy(r, s, sc * cflbm_mpi_stub::type_bytes(st));
  return 0;
}
inline int MPI_Reduce(const void *s, void *r, int c, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  std::memcpy(r, s, c * cflbm_mpi_stub::type_bytes(t));
  return 0;
}
inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) {
  cflbm_mpi_stub::die("MPI_Send");
}
inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
  cflbm_mpi_stub::die("MPI_Recv");
}
inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
  cflbm_mpi_stub::die("MPI_Isend");
}
inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
  cflbm_mpi_stub::die("MPI_Irecv");
}

inline int MPI_Type_create_subarray(int ndims, const int *sizes, const int *subsizes,
                                    const int *starts, int, MPI_Datatype old,
                                    MPI_Datatype *out) {
  bool full = true;
  for (int d = 0; d < ndims; ++d)
    if (subsizes[d] != sizes[d] || starts[d] != 0) full = false;
  if (!full) cflbm_mpi_stub::die("a partial subarray file view");
  cflbm_mpi_stub::types().push_back({cflbm_mpi_stub::type_bytes(old), true});
  *out = static_cast<MPI_Datatype>(cflbm_mpi_stub::types().size() - 1);
  return 0;
}
inline int MPI_Type_contiguous(int, MPI_Datatype old, MPI_Datatype *out) {
  cflbm_mpi_stub::types().push_back({cflbm_mpi_stub::type_bytes(old), true});
  *out = static_cast<MPI_Datatype>(cflbm_mpi_stub::types().size() - 1);
  return 0;
}
inline int MPI_Type_commit(MPI_Datatype *) { return 0; }

/* MPI_File_open does not truncate an existing file; neither does the stub. */
inline int MPI_File_open(MPI_Comm, const char *name, int, MPI_Info, MPI_File *fh) {
  std::FILE *f = std::fopen(name, "r+b");
  if (!f) f = std::fopen(name, "w+b");
  if (!f) return 1;
  *fh = f;
  return 0;
}
inline int MPI_File_close(MPI_File *fh) {
  std::fclose(*fh);
  *fh = nullptr;
  return 0;
}
inline int MPI_File_seek(MPI_File fh, MPI_Offset off, int) {
  return std::fseek(fh, static_cast<long>(off), SEEK_SET);
}
inline int MPI_File_write(MPI_File fh, const void *buf, int count, MPI_Datatype t,
                          MPI_Status *) {
  size_t b = cflbm_mpi_stub::type_bytes(t);
  return std::fwrite(buf, b, count, fh) == static_cast<size_t>(count) ? 0 : 1;
}
inline int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype, MPI_Datatype,
                             const char *, MPI_Info) {
  return std::fseek(fh, static_cast<long>(disp), SEEK_SET);
}
inline int MPI_File_write_all(MPI_File fh, const void *buf, int count, MPI_Datatype t,
                              MPI_Status *s) {
  return MPI_File_write(fh, buf, count, t, s);
}

#endif
