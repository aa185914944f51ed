// Kernel launchers (defined in wk_kernels.cu, called by the host runtime).
#pragma once

#include <cuda_runtime.h>

#include "wk_internal.h"

namespace wk {
namespace dev {

constexpr int kRowsPerBlock = 1024;   // input rows per CTA of every op kernel
constexpr int kThreads = 256;

constexpr int kSliceRows = 8192;      // k2u output rows per expansion CTA (a multiple of 4)
constexpr int kPlanTileShift = 13;    // input blocks per k2u plan CTA: 8192
constexpr int kGroupShift = 8;        // input blocks per k2u group sum: 256

// k2u pass 1: probe hist[r][scol] -> deg[r], off[r]; per-block output counts
// blk_sum[b]; group_sums[2g] += output rows and group_sums[2g + 1] += slices
// of the blocks of group g (256 blocks; zeroed before the launch); err bit 0:
// overflow chain longer than the segment's overflow area, bit 1: a block's
// count reached 2^31.
// func (the direction is functional, PredView::func): deg receives each row's
// neighbour as int32 (-1 when there is none) for launch_k2u_expand_func; err
// bit 3 when a row's list had more than one entry (an index key), which the
// functional expansion cannot write.
void launch_k2u_count(const int32_t *hist, int64_t R, int C, int scol, uint32_t dir, PredView pv, uint32_t *deg, uint32_t *off, unsigned long long *blk_sum, unsigned long long *group_sums,
                      int *err, bool func, cudaStream_t st);

// k2u pass 2 of a functional direction (2 <= C + 1 <= 8): the matched rows
// with their neighbour appended, compacted in order; one CTA per non-empty block.
void launch_k2u_expand_func(const int32_t *hist, int64_t R, int C, const int32_t *nbr,
                            const unsigned long long *blk_sum, const unsigned long long *bp,
                            const unsigned long long *sp, unsigned long long slices, int32_t *out, cudaStream_t st);

// k2u plan: bp[b] = the block's output prefix, sp[b] = its first slice
// (nblk + 1 entries each); totals[0] = output rows, totals[2] = slices, the
// expansion's CTA count.  One CTA per 8192 blocks; the last one to finish
// zeroes the group sums and *plan_done (both must be zero at launch).
void launch_k2u_plan(const unsigned long long *blk_sum, int64_t nblk, unsigned long long *group_sums,
                     unsigned int *plan_done, unsigned long long *bp, unsigned long long *sp, unsigned long long *totals,
                     cudaStream_t st);

// k2u pass 2: one CTA per slice writes its rows (row || neighbour) of its
// block's output; out holds totals[0] rows of C + 1 columns and is 16 B aligned.
void launch_k2u_expand(const int32_t *hist, int64_t R, int C, const int32_t *edges, const uint32_t *deg,
                       const uint32_t *off, const unsigned long long *blk_sum, const unsigned long long *bp,
                       const unsigned long long *sp, unsigned long long slices, int32_t *out, cudaStream_t st);

// k2k/k2c pass 1: probe + membership of the end value; per-row ballot masks,
// per-block kept-row counts, flags cleared; totals[0] += adjacency entries a
// linear scan touches, totals[1] += kept rows.
// ecol >= 0: end is column ecol (k2k); ecol < 0: end is the constant `end_const` (k2c).
void launch_filter_probe(const int32_t *hist, int64_t R, int C, int scol, int ecol, int32_t end_const,
                         uint32_t dir, PredView pv, uint32_t *mask, unsigned int *blk_nz,
                         unsigned long long *flags, unsigned long long *totals, int *err, cudaStream_t st);

// k2k/k2c pass 2: copy the kept rows in order (out holds up to R rows of C columns).
void launch_filter_write(const int32_t *hist, int64_t R, int C, const uint32_t *mask, const unsigned int *blk_nz,
                         unsigned long long *flags, int32_t *out, cudaStream_t st);

// Copy an adjacency list (index or constant start) into a one-column table.
void launch_copy_list(const int32_t *src, int64_t n, int32_t *dst, cudaStream_t st);

}  // namespace dev
}  // namespace wk
