// bucket.cuh — most-significant-bucket front end of the key sort.
//
// GB300 counterpart of the sample sort's partitioning (src/ext_mem.rs
// phases 1-3: splitters drawn from a sample, every record distributed to its
// partition) fused with the packed-key seed sort (src/pack.rs:241-321):
//   1. every key carries a 16-bit bucket id in the bits above it: its top
//      key bits, or its rank among sampled splitter keys (binary search), or
//      the bucket a small learned CDF model predicts, checked against the two
//      neighbouring splitters and corrected;
//   2. two stable onesweep passes on the bucket id make every bucket
//      contiguous (histogram, scan and scatter with shared-memory staging);
//   3. one thread block sorts each bucket on the remaining key bits in shared
//      memory (an on-chip LSD radix sort; 24 B of HBM traffic per record for
//      all its passes), buckets too large for shared memory by the global sort.
#pragma once

#include "common.cuh"

namespace capssa {
namespace bucket {

constexpr int kBucketBits = 16;
constexpr uint32_t kBuckets = 1u << kBucketBits;
constexpr uint32_t kCap = 8192;  // largest bucket one block sorts on chip

// Sort keys/vals (n pairs, vals already set) stably by key bits [0, low_bits)
// within each bucket; bucket b occupies [start[b], start[b+1]).  Buckets of
// more than kCap records are sorted by the global radix sort.  The result
// stays in (keys, vals).  (t1k, t1v) and (t2k, t2v) are scratch pairs of n
// entries each.
capssa_status sort_buckets(Ctx &c, uint64_t *keys, uint32_t *vals, uint64_t *t1k, uint32_t *t1v,
                           uint64_t *t2k, uint32_t *t2v, uint32_t n, const uint32_t *d_start,
                           const uint32_t *h_start, int low_bits);

// start[b] = first index whose bucket id (key >> shift, kBucketBits wide) is
// >= b, for b = 0..kBuckets (start[kBuckets] = n), from keys sorted by id.
capssa_status bucket_starts(Ctx &c, const uint64_t *keys, uint32_t n, int shift,
                            uint32_t *d_start);

}  // namespace bucket
}  // namespace capssa
