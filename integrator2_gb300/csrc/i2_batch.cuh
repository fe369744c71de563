// i2_batch.cuh -- flattened walks over the segments of a batch (one segment = the pairs of one
// class of one mesh).
//
// A batched stage kernel treats the work items of all segments (pairs, listed pairs or queued
// cells, counted on the device by earlier kernels) as one index space.  Each block first reads
// every segment's item count and builds their prefix sums in shared memory; a worker (thread,
// warp or block) w of W then takes the global items w, w + W, ... and finds each item's segment
// by binary search over the prefix sums.  So one launch per stage covers every segment, however
// many there are and however uneven their sizes, with no host synchronisation.
#pragma once

#include "i2_engine.h"

namespace i2 {

// segments one stage launch walks (the prefix sums take 8 bytes of shared memory each); larger
// batches are walked in chunks of this many segments
constexpr int kBatchSegChunk = 2048;

// prefix[s] = items of segments before s, prefix[nseg] = all items; every thread of the block
// must call it
template <class Count>
__device__ long long seg_prefix(const BatchSeg *__restrict__ segs, int nseg, long long *prefix, Count count)
{
    for (int s = threadIdx.x; s < nseg; s += blockDim.x) prefix[s + 1] = count(segs[s]);
    if (threadIdx.x == 0) prefix[0] = 0;
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        long long carry = 0;
        for (int base = 1; base <= nseg; base += 32) {
            const int i = base + lane;
            long long v = i <= nseg ? prefix[i] : 0;
            for (int off = 1; off < 32; off <<= 1) {
                const long long u = __shfl_up_sync(0xffffffffu, v, off);
                if (lane >= off) v += u;
            }
            if (i <= nseg) prefix[i] = v + carry;
            carry += __shfl_sync(0xffffffffu, v, 31);
        }
    }
    __syncthreads();
    return prefix[nseg];
}

// the segment of global item g (prefix[seg] <= g < prefix[seg + 1])
__device__ __forceinline__ int seg_find(const long long *prefix, int nseg, long long g)
{
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ bool seg_adjacent(const BatchSeg &S) { return S.A.n > 0 && (S.cls == kEdge || S.cls == kVertex); }

} // namespace i2
