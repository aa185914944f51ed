// Kernel launchers (defined in wk_kernels.cu, called by the host runtime).
#pragma once

#include <cuda_runtime.h>

#include "wk_internal.h"

namespace wk {
namespace dev {

constexpr int kRowsPerBlock = 1024;   // input rows per probe/compact block
constexpr int kThreads = 256;

// rows of output per k2u write tile for a given output width (multiple of 32)
int k2u_tile_rows(int out_cols);

// Pass 1 of k2u: probe key hist[r][scol] -> deg[r], off[r]; per-block sums.
void launch_k2u_probe(const int32_t *hist, int64_t R, int C, int scol, uint32_t dir, PredView pv,
                      uint32_t *deg, uint32_t *off, unsigned long long *blk_sum, unsigned int *blk_nz,
                      int *err, cudaStream_t st);

// Pass 1 of k2k/k2c: probe + membership of the end value; ballot masks and per-block counts.
// ecol >= 0: end is column ecol (k2k); ecol < 0: end is the constant `end_const` (k2c).
void launch_filter_probe(const int32_t *hist, int64_t R, int C, int scol, int ecol, int32_t end_const,
                         uint32_t dir, PredView pv, uint32_t *mask, unsigned long long *blk_sum,
                         unsigned int *blk_nz, int *err, cudaStream_t st);

// Exclusive scan of the per-block sums in place; totals[0] = sum, totals[1] = nz;
// if cz_pos != nullptr also writes cz_pos[nz] = sum (sentinel).
void launch_scan_blocks(unsigned long long *blk_sum, unsigned int *blk_nz, int64_t nblk,
                        unsigned long long *totals, unsigned long long *cz_pos, cudaStream_t st);

// Pass 2 of k2u: compact rows with deg > 0 and record the first compacted row of every tile.
void launch_k2u_compact(const uint32_t *deg, const uint32_t *off, int64_t R,
                        const unsigned long long *blk_sum, const unsigned int *blk_nz,
                        int32_t *cz_row, unsigned long long *cz_pos, uint32_t *cz_off,
                        int32_t *tile_k0, int tile_rows, cudaStream_t st);

// Pass 3 of k2u: write output tiles row || neighbour, coalesced.
void launch_k2u_write(const int32_t *hist, int C, const int32_t *edges, const int32_t *cz_row,
                      const unsigned long long *cz_pos, const uint32_t *cz_off, int64_t nz,
                      const int32_t *tile_k0, int64_t ntiles, int tile_rows, int64_t R_out,
                      int32_t *out, cudaStream_t st);

// Pass 2 of k2k/k2c: copy the flagged rows in order.
void launch_filter_write(const int32_t *hist, int64_t R, int C, const uint32_t *mask,
                         const unsigned int *blk_nz, int32_t *out, cudaStream_t st);

// Copy an adjacency list (index or constant start) into a one-column table.
void launch_copy_list(const int32_t *src, int64_t n, int32_t *dst, cudaStream_t st);

}  // namespace dev
}  // namespace wk
