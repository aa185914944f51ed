// Kernel launchers (defined in wk_kernels.cu, called by the host runtime).
#pragma once

#include <cuda_runtime.h>

#include "wk_internal.h"

namespace wk {
namespace dev {

constexpr int kRowsPerBlock = 1024;   // input rows per CTA of every op kernel
constexpr int kThreads = 256;

constexpr int kSliceRows = 8192;      // k2u output rows per expansion CTA (a multiple of 4)
constexpr int kGroupShift = 8;        // input blocks per k2u group sum: 256

// The groups' exclusive prefixes of output rows and slices (entry n = the op's
// totals), added up by the host from the count kernel's group sums and passed
// to the expansion by value, for ops of up to kTableGroups groups (67M input
// rows); n = 0 for a larger op, whose expansion scans the group sums itself.
constexpr int kTableGroups = 256;
struct GroupTable {
    unsigned long long out[kTableGroups + 1];
    unsigned int sl[kTableGroups + 1];
    int n;
};

// k2u pass 1: probe hist[r][scol] -> deg[r], off[r]; per-block output counts
// blk_sum[b]; group_sums[2g] += output rows and group_sums[2g + 1] += slices
// of the blocks of group g (256 blocks; zero at launch), so the op's totals
// are the sums over its groups.  clear[0 .. nclear) is set to zero (the
// other of two alternating sums buffers, for the next op).  err bit 0:
// overflow chain longer than the segment's overflow area, bit 1: a block's
// count reached 2^31.
// func (the direction is functional, PredView::func): deg receives each row's
// neighbour as int32 (-1 when there is none) for launch_k2u_expand_func; err
// bit 3 when a row's list had more than one entry (an index key), which the
// functional expansion cannot write.
// sms: the device's SM count (two input blocks per CTA once an op has 16 per SM).
void launch_k2u_count(const int32_t *hist, int64_t R, int C, int scol, uint32_t dir, PredView pv, uint32_t *deg,
                      uint32_t *off, unsigned long long *blk_sum, unsigned long long *group_sums, int *err, bool func,
                      unsigned long long *clear, int64_t nclear, int sms, cudaStream_t st);

// The op's error word and group sums (n words from src) for the host: a
// one-CTA kernel, stream-ordered behind the count, copies them into
// dst[2 .. 2 + n) of pinned, device-mapped host memory and then writes seq
// into dst[0], so a host that sees seq there reads the op's totals without a
// device-to-host copy or a stream synchronisation.
struct Publish {
    const unsigned long long *src;
    unsigned long long *dst;
    long long n;
    unsigned long long seq;
};
void launch_publish(const Publish &pub, cudaStream_t st);

// Load every k2u count and expansion kernel on the current device (they load
// lazily, at first launch, otherwise); returns a cudaError_t.
int preload_k2u_kernels();

// k2u pass 2 of a functional direction (2 <= C + 1 <= 8): the matched rows
// with their neighbour appended, compacted in order; one CTA per non-empty
// block (slices = the op's total from the group sums).
void launch_k2u_expand_func(const int32_t *hist, int64_t R, int C, const int32_t *nbr,
                            const unsigned long long *blk_sum, const unsigned long long *group_sums,
                            const GroupTable &gt, unsigned long long slices, int32_t *out, cudaStream_t st);
// k2u pass 2: one CTA per slice (slices = the op's total from the group sums)
// finds its block from blk_sum and the group sums and writes its rows
// (row || neighbour) of the block's output; out holds the op's output rows
// of C + 1 columns and is 16 B aligned.
void launch_k2u_expand(const int32_t *hist, int64_t R, int C, const int32_t *edges, const uint32_t *deg,
                       const uint32_t *off, const unsigned long long *blk_sum, const unsigned long long *group_sums,
                       const GroupTable &gt, unsigned long long slices, int32_t *out, cudaStream_t st);

// k2k/k2c pass 1: probe + membership of the end value; per-row ballot masks,
// per-block kept-row counts, each added into its group's sum (group_sums[2 g],
// 2^kGroupShift blocks a group, zero on entry); totals[0] += adjacency entries
// a linear scan touches, totals[1] += kept rows.  The nclear words at `clear`
// (the other sums buffer) are zeroed.
// ecol >= 0: end is column ecol (k2k); ecol < 0: end is the constant `end_const` (k2c).
void launch_filter_probe(const int32_t *hist, int64_t R, int C, int scol, int ecol, int32_t end_const,
                         uint32_t dir, PredView pv, uint32_t *mask, unsigned int *blk_nz,
                         unsigned long long *group_sums, unsigned long long *clear, int64_t nclear,
                         unsigned long long *totals, int *err, cudaStream_t st);

// k2k/k2c pass 2: copy the kept rows in order (out holds up to R rows of C columns).
void launch_filter_write(const int32_t *hist, int64_t R, int C, const uint32_t *mask, const unsigned int *blk_nz,
                         const unsigned long long *group_sums, int32_t *out, cudaStream_t st);

// Copy an adjacency list (index or constant start) into a one-column table.
void launch_copy_list(const int32_t *src, int64_t n, int32_t *dst, cudaStream_t st);

}  // namespace dev
}  // namespace wk
