// Channel-profile set-up on the GPU (setup.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "solver.cuh"

namespace cflbm {

struct SetupArgs {
  int nx, ny, nz, nxw;
  int wall_y, wall_z;
  int geom;                 // enum cflbm_geom (1 cylinder, 2 sphere)
  double cx, cy, cz, r2;    // body centre, squared radius
  const uint8_t *solid_in;  // device copy of an explicit nx*ny*nz mask, or null
};

// Tile chunks of the listing passes (the length of the chunk array).
int setup_chunks(const SetupArgs &s);
// Mask words (counters[0] += solid cells) and per-cell link bits
// (counters[1] += the reference-rule links of solid cells).
cudaError_t launch_setup_mask_links(int Q, const SetupArgs &s, uint32_t *mask, uint32_t *bits,
                                    unsigned long long *counters, cudaStream_t st);
// Per-tile listed flags, per-chunk offsets into the list, the list's length.
cudaError_t launch_setup_flags(const SetupArgs &s, const uint32_t *mask, const uint32_t *bits,
                               unsigned char *flag, int *chunk, int *total, cudaStream_t st);
// Tile positions, the list and its link words.
cudaError_t launch_setup_list(const SetupArgs &s, const unsigned char *flag, const int *chunk,
                              const uint32_t *mask, const uint32_t *bits, int *tile_index,
                              int *list, uint32_t *links_bits, cudaStream_t st);

// The boundary cells (fluid cells with solid links) of the listed tiles, in
// tile and then x order, for the force launch: per listed tile its count
// (cnt: n_slow bytes; chunk: bcell_chunks(n_slow) + 1 ints; their number into
// *total), then the storage index and link word of each.
int bcell_chunks(int n_slow);
cudaError_t launch_setup_bcell_count(int n_slow, const uint32_t *links_bits, unsigned char *cnt,
                                     int *chunk, int *total, cudaStream_t st);
cudaError_t launch_setup_bcell_list(const Layout &L, int nxw, int n_slow, const int *list,
                                    const uint32_t *links_bits, const unsigned char *cnt,
                                    const int *chunk, long long *cell, uint32_t *words,
                                    cudaStream_t st);

}  // namespace cflbm
