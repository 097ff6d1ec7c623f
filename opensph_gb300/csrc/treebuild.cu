// treebuild.cu — k-d tree of the Barnes-Hut gravity (compiled with -fmad=false).
//
// Replaces KdTree::buildTree as BarnesHut::build runs it (core/objects/finders/KdTree.inl.h:44-160,
// core/gravity/BarnesHut.cpp:50-84). The split rule is the reference's, element for element: the dimension of
// largest extent of the split box (singular dimensions skipped), the box centre as split position, the
// two-pointer partition around it, the sliding midpoint (the extreme element, first occurrence, moved to the
// empty side) and, after more than five consecutive slides, std::nth_element at the middle. Leaf membership,
// the order of the particles inside each leaf and the leaf boxes are therefore the reference's.
//
// The two-pointer partition swaps, for k = 0 .. K-1, the k-th element above the split position counted from
// the left with the k-th element below it counted from the right, where K is the number of such pairs that
// are out of order; this is what a block scan (ranks) and a binary search (K, the predicate is monotone)
// compute in parallel.
//
// Layout: the particles in tree order as 32-byte elements (order keys of x, y and z, and the particle index:
// elems[k] = {orderKey(r[i][0..2]), i} with i = idx[k]), so that every pass over a segment reads contiguous
// memory on the integer pipe and a swap of the partition moves one sector per side; idx (KdTree::idxs) is
// written from them at the end.
//
// Two phases, with no host round trip between levels:
//   1. segments of more than SUBTREE_MAX elements, level by level over all of them at once, a chunk of
//      R1_CHUNK elements per CTA: statistics of the three candidate dimensions -> per segment the split
//      dimension and the chunk offsets -> ranks of the elements above / below the split -> K, sliding
//      midpoint, nth_element and the children -> the K swaps. The host launches as many levels as the
//      previous build used plus two (then, only if large segments remain, four more at a time after reading
//      their count); the kernels read the segment and chunk counts from device memory, so levels without work
//      end at once.
//   2. every other segment (the children of at most SUBTREE_MAX elements, and whatever phase 1 left over) is
//      split down to its leaves by one warp, depth first, on a copy of its idx and keys in shared memory.
// A counting sort by level then lists the nodes level by level for the walks; one copy to the host returns the
// node, leaf and level counts, and the moments are formed bottom-up (gravity.cu) after it, while the host goes on.

#include <algorithm>
#include <cfloat>
#include <cmath>

#include "tree.cuh"

namespace sphgpu {

namespace {

// 128-thread blocks, so that a block fits where one block of the concurrently running pair loop retired
constexpr uint32_t R1_CHUNK = 2048;    // elements per CTA in phase 1
constexpr int R1_THREADS = 128;
constexpr int R1_PER_THREAD = int(R1_CHUNK) / R1_THREADS;
constexpr int SWAP_THREADS = 512;      // the swaps of a chunk, four per thread
constexpr uint32_t SUBTREE_MAX = 512;  // segments up to this size are split to their leaves by one warp
constexpr int R2_WARPS = 4;            // warps per CTA of the subtree kernel
constexpr int R2_STACK = 36;           // pending segments per warp

__device__ __forceinline__ int argMax3(const double s[3]) {
    int m = 0;
    if (s[1] > s[m]) {
        m = 1;
    }
    if (s[2] > s[m]) {
        m = 2;
    }
    return m;
}

__device__ __forceinline__ double coord(const dbl4* __restrict__ r, uint32_t i, int dim) {
    return __ldg(reinterpret_cast<const double*>(r) + 4 * size_t(i) + dim);
}

// the double of an order key (the inverse of orderKey; -0 was mapped to the key of +0)
__device__ __forceinline__ double keyValue(unsigned long long k) {
    return doubleUnflip(k);
}

// ---------------------------------------------------------------------------------------------------------
// libstdc++'s introselect (std::nth_element: __introselect with __move_median_to_first,
// __unguarded_partition, __heap_select and __insertion_sort, libstdc++ bits/stl_algo.h and stl_heap.h, GPL-3.0
// with the GCC runtime library exception), replayed step by step for the rare nth_element split of
// KdTree::buildTree, whose resulting order of equal-to-median elements is only defined by these steps.
// Single thread; the keys of the moved elements are recomputed by the caller.
// ---------------------------------------------------------------------------------------------------------

struct NthCtx {
    uint32_t* a;
    const dbl4* r;
    int dim;
    __device__ __forceinline__ bool less(uint32_t x, uint32_t y) const {
        return coord(r, x, dim) < coord(r, y, dim);
    }
};

__device__ void pushHeap(NthCtx& c, long first, long hole, long top, uint32_t value) {
    long parent = (hole - 1) / 2;
    while (hole > top && c.less(c.a[first + parent], value)) {
        c.a[first + hole] = c.a[first + parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    c.a[first + hole] = value;
}

__device__ void adjustHeap(NthCtx& c, long first, long hole, long len, uint32_t value) {
    const long top = hole;
    long second = hole;
    while (second < (len - 1) / 2) {
        second = 2 * (second + 1);
        if (c.less(c.a[first + second], c.a[first + second - 1])) {
            second--;
        }
        c.a[first + hole] = c.a[first + second];
        hole = second;
    }
    if ((len & 1) == 0 && second == (len - 2) / 2) {
        second = 2 * (second + 1);
        c.a[first + hole] = c.a[first + second - 1];
        hole = second - 1;
    }
    pushHeap(c, first, hole, top, value);
}

__device__ void heapSelect(NthCtx& c, long first, long middle, long last) {
    const long len = middle - first;
    if (len >= 2) {
        long parent = (len - 2) / 2;
        while (true) {
            adjustHeap(c, first, parent, len, c.a[first + parent]);
            if (parent == 0) {
                break;
            }
            parent--;
        }
    }
    for (long i = middle; i < last; ++i) {
        if (c.less(c.a[i], c.a[first])) {
            const uint32_t value = c.a[i];
            c.a[i] = c.a[first];
            adjustHeap(c, first, 0, len, value);
        }
    }
}

__device__ __forceinline__ void iterSwap(uint32_t* a, long x, long y) {
    const uint32_t t = a[x];
    a[x] = a[y];
    a[y] = t;
}

__device__ void moveMedianToFirst(NthCtx& c, long result, long x, long y, long z) {
    if (c.less(c.a[x], c.a[y])) {
        if (c.less(c.a[y], c.a[z])) {
            iterSwap(c.a, result, y);
        } else if (c.less(c.a[x], c.a[z])) {
            iterSwap(c.a, result, z);
        } else {
            iterSwap(c.a, result, x);
        }
    } else if (c.less(c.a[x], c.a[z])) {
        iterSwap(c.a, result, x);
    } else if (c.less(c.a[y], c.a[z])) {
        iterSwap(c.a, result, z);
    } else {
        iterSwap(c.a, result, y);
    }
}

__device__ long unguardedPartition(NthCtx& c, long first, long last, long pivot) {
    while (true) {
        while (c.less(c.a[first], c.a[pivot])) {
            ++first;
        }
        --last;
        while (c.less(c.a[pivot], c.a[last])) {
            --last;
        }
        if (!(first < last)) {
            return first;
        }
        iterSwap(c.a, first, last);
        ++first;
    }
}

__device__ void insertionSort(NthCtx& c, long first, long last) {
    if (first == last) {
        return;
    }
    for (long i = first + 1; i != last; ++i) {
        if (c.less(c.a[i], c.a[first])) {
            const uint32_t val = c.a[i];
            for (long k = i; k > first; --k) {
                c.a[k] = c.a[k - 1];
            }
            c.a[first] = val;
        } else {
            const uint32_t val = c.a[i];
            long last2 = i, next = i - 1;
            while (c.less(val, c.a[next])) {
                c.a[last2] = c.a[next];
                last2 = next;
                --next;
            }
            c.a[last2] = val;
        }
    }
}

__device__ void nthElement(NthCtx& c, long first, long nth, long last) {
    if (first == last || nth == last) {
        return;
    }
    long n = last - first;
    int lg = 0;
    while (n > 1) {
        n >>= 1;
        ++lg;
    }
    int depth = 2 * lg;
    while (last - first > 3) {
        if (depth == 0) {
            heapSelect(c, first, nth + 1, last);
            iterSwap(c.a, first, nth);
            return;
        }
        --depth;
        const long mid = first + (last - first) / 2;
        moveMedianToFirst(c, first, first + 1, mid, last - 1);
        const long cut = unguardedPartition(c, first + 1, last, first);
        if (cut <= nth) {
            first = cut;
        } else {
            last = cut;
        }
    }
    insertionSort(c, first, last);
}

// ---------------------------------------------------------------------------------------------------------
// shared pieces
// ---------------------------------------------------------------------------------------------------------

__device__ __forceinline__ bool betterArg(unsigned long long v, uint32_t p, unsigned long long bv, uint32_t bp,
    bool isMax) {
    return isMax ? (v > bv || (v == bv && p < bp)) : (v < bv || (v == bv && p < bp));
}

__device__ __forceinline__ void warpArgExtreme(unsigned long long& val, uint32_t& pos, bool isMax) {
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long ov = __shfl_xor_sync(0xffffffffu, val, off);
        const uint32_t op = __shfl_xor_sync(0xffffffffu, pos, off);
        if (betterArg(ov, op, val, pos, isMax)) {
            val = ov;
            pos = op;
        }
    }
}

// split dimension of a segment: the largest extent of its box, skipping singular dimensions (all keys equal);
// degenerated when every extent is zero (KdTree::buildTree's loop over the dimensions)
__device__ __forceinline__ int splitDimension(const BhSegment& sg, const bool nonSingular[3], bool& degenerated) {
    double boxSize[3];
    for (int d = 0; d < 3; ++d) {
        boxSize[d] = sg.hi[d] - sg.lo[d];
    }
    int splitIdx = argMax3(boxSize);
    degenerated = false;
    for (int dim = 0; dim < 3; ++dim) {
        if (!nonSingular[splitIdx]) {
            boxSize[splitIdx] = 0.;
            splitIdx = argMax3(boxSize);
            if (boxSize[0] == 0. && boxSize[1] == 0. && boxSize[2] == 0.) {
                degenerated = true;
                break;
            }
        } else {
            break;
        }
    }
    return splitIdx;
}

// Inner node `node` gets two children: node ids, parent/level links and the child segments. Returns false (with
// the error word set) when the node pool is exhausted.
__device__ bool makeChildren(BhNodeGeom* geom, uint32_t* counters, uint32_t nodeCapacity, uint32_t* devError,
    const BhSegment& sg, uint32_t n1, int d, double cut, bool sliding, BhSegment& l, BhSegment& r) {
    const uint32_t child = atomicAdd(&counters[C_NODES], 2u);
    if (child + 2 > nodeCapacity) {
        atomicOr(devError, uint32_t(DEV_ERR_NODE_CAPACITY));
        return false;
    }
    BhNodeGeom& g = geom[sg.node];
    g.left = int32_t(child);
    g.right = int32_t(child + 1);
    g.from = sg.from;
    g.to = sg.to;
    const int lvl = g.level;
    geom[child].parent = sg.node;
    geom[child].level = lvl + 1;
    geom[child + 1].parent = sg.node;
    geom[child + 1].level = lvl + 1;
    atomicMax(&counters[C_DEPTH], uint32_t(lvl + 2));
    const uint32_t next = sliding ? sg.sliding + 1 : 0;
    l = sg;
    r = sg;
    l.to = n1;
    l.node = int32_t(child);
    l.sliding = next;
    l.hi[d] = cut;
    r.from = n1;
    r.node = int32_t(child + 1);
    r.sliding = next;
    r.lo[d] = cut;
    return true;
}

// ---------------------------------------------------------------------------------------------------------
// root
// ---------------------------------------------------------------------------------------------------------

__global__ void resetBoundsKernel(unsigned long long* b) {
    if (threadIdx.x < 3) {
        b[threadIdx.x] = ~0ull;
        b[3 + threadIdx.x] = 0ull;
    }
}

__global__ void boundsKernel(const dbl4* __restrict__ r, uint32_t n, unsigned long long* b) {
    unsigned long long mn[3] = { ~0ull, ~0ull, ~0ull }, mx[3] = { 0, 0, 0 };
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dbl4 p = r[i];
        const unsigned long long f[3] = { doubleFlip(p.x), doubleFlip(p.y), doubleFlip(p.z) };
        for (int k = 0; k < 3; ++k) {
            mn[k] = min(mn[k], f[k]);
            mx[k] = max(mx[k], f[k]);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
            mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
        }
    }
    // the warps' extremes combined in the block, one atomic per block and coordinate (a few hundred blocks: the
    // atomics on six words were the kernel's time with one per warp)
    __shared__ unsigned long long sMn[32][3], sMx[32][3];
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            sMn[w][k] = mn[k];
            sMx[w][k] = mx[k];
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        unsigned long long a = sMn[0][k], c = sMx[0][k];
        for (int q = 1; q < nw; ++q) {
            a = min(a, sMn[q][k]);
            c = max(c, sMx[q][k]);
        }
        atomicMin(&b[k], a);
        atomicMax(&b[3 + k], c);
    }
}

__device__ __forceinline__ TreeElem makeElem(const dbl4* __restrict__ r, uint32_t i) {
    const dbl4 p = r[i];
    TreeElem e;
    e.key[0] = orderKey(p.x);
    e.key[1] = orderKey(p.y);
    e.key[2] = orderKey(p.z);
    e.idx = i;
    e.pad = 0;
    return e;
}

__device__ __forceinline__ void swapElements(TreeElem* elems, uint32_t a, uint32_t b) {
    const TreeElem x = elems[a], y = elems[b];
    elems[a] = y;
    elems[b] = x;
}

// std::nth_element of the segment [from, to) by coordinate d (KdTree::buildTree's fallback), on the particle
// indices copied to scratch; the elements are then rebuilt from the positions
__device__ void nthElementSegment(const dbl4* __restrict__ r, TreeElem* elems, uint32_t* scratch, uint32_t from,
    uint32_t to, uint32_t nth, int d) {
    for (uint32_t k = from; k < to; ++k) {
        scratch[k] = elems[k].idx;
    }
    NthCtx ctx{ scratch, r, d };
    nthElement(ctx, long(from), long(nth), long(to));
    for (uint32_t k = from; k < to; ++k) {
        elems[k] = makeElem(r, scratch[k]);
    }
}

// Phase-1 arrays of one level parity (segments, their chunks and the per-chunk results); the level after next
// reuses them.
struct LevelBufs {
    BhSegment* seg;        // segments of the level
    BhChunk* chunks;       // chunks of the level, contiguous per segment
    BhChunkStats* stats;   // per chunk
    uint32_t* offB;        // per chunk: elements above the split before the chunk, within its segment
    uint32_t* offS;
    uint32_t* done;        // per segment's first chunk: chunks done in the statistics [0] and rank [cap] passes
};

// queues a phase-1 segment (more than SUBTREE_MAX elements) with its chunks into the level buffers `b` of
// parity q, or a smaller one into the phase-2 queue
__device__ void pushSegment(const BhSegment& sg, LevelBufs b, int q, uint32_t* counters, uint32_t chunkCapacity,
    uint32_t segCapacity, BhSegment* queue, uint32_t* devError) {
    const uint32_t len = sg.to - sg.from;
    if (len <= SUBTREE_MAX) {
        const uint32_t slot = atomicAdd(&counters[C_QUEUE], 1u);
        if (slot < segCapacity) {
            queue[slot] = sg;
        } else {
            atomicOr(devError, uint32_t(DEV_ERR_SEGMENT_CAPACITY));
        }
        return;
    }
    const uint32_t slot = atomicAdd(&counters[C_SEGS + q], 1u);
    const uint32_t nc = (len + R1_CHUNK - 1) / R1_CHUNK;
    const uint32_t c0 = atomicAdd(&counters[C_CHUNKS + q], nc);
    if (slot >= segCapacity || c0 + nc > chunkCapacity) {
        atomicOr(devError, uint32_t(DEV_ERR_SEGMENT_CAPACITY));
        // the segment still gets its leaves, by one warp in phase 2
        const uint32_t qs = atomicAdd(&counters[C_QUEUE], 1u);
        if (qs < segCapacity) {
            queue[qs] = sg;
        }
        return;
    }
    b.seg[slot] = sg;
    for (uint32_t k = 0; k < nc; ++k) {
        b.chunks[c0 + k].seg = slot;
        b.chunks[c0 + k].index = k;
        b.chunks[c0 + k].first = c0;
        b.chunks[c0 + k].count = nc;
    }
    b.done[c0] = 0;
    b.done[chunkCapacity + c0] = 0;
}

// the elements of the particles in index order, and the root segment (box = bounding box of all points, as
// KdTree::buildImpl) in the phase-1 buffers or, for a small set, in the phase-2 queue
__global__ void rootKernel(const dbl4* __restrict__ r, uint32_t n, TreeElem* elems, LevelBufs b0, BhSegment* queue,
    BhNodeGeom* geom, uint32_t* counters, uint32_t chunkCapacity, uint32_t segCapacity,
    const unsigned long long* bounds, uint32_t* devError) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        elems[i] = makeElem(r, i);
    }
    if (i == 0) {
        BhSegment s;
        s.from = 0;
        s.to = n;
        s.node = 0;
        s.sliding = 0;
        for (int k = 0; k < 3; ++k) {
            s.lo[k] = doubleUnflip(bounds[k]);
            s.hi[k] = doubleUnflip(bounds[3 + k]);
        }
        geom[0].parent = -1;
        geom[0].level = 0;
        for (int k = 0; k < C_WORDS; ++k) {
            counters[k] = 0;
        }
        counters[C_NODES] = 1;
        counters[C_DEPTH] = 1;
        pushSegment(s, b0, 0, counters, chunkCapacity, segCapacity, queue, devError);
    }
}

// ---------------------------------------------------------------------------------------------------------
// phase 1: segments of more than SUBTREE_MAX elements, three launches per level. The CTA that completes the
// last chunk of a segment in a pass (an atomic count per segment after a memory fence; nothing waits) does that
// segment's per-segment step: the split decision after the statistics, the partition count K, the sliding
// midpoint or nth_element and the children after the ranks.
// ---------------------------------------------------------------------------------------------------------

// exclusive prefix sum over the R1_THREADS threads of a block
__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) {
            x += y;
        }
    }
    if (lane == 31) {
        sh[warp] = x;
    }
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) {
        before += sh[w];
    }
    __syncthreads();
    return before + x - v;
}

// true in every thread of the CTA that completed the last chunk of segment `first` in pass `pass`
__device__ __forceinline__ bool lastChunkOfSegment(uint32_t* done, uint32_t first, uint32_t count, bool* flag) {
    __threadfence(); // this thread's results of the pass before the count
    __syncthreads();
    if (threadIdx.x == 0) {
        *flag = atomicAdd(&done[first], 1u) == count - 1;
        if (*flag) {
            __threadfence();
        }
    }
    __syncthreads();
    return *flag;
}

// Pass 1: per chunk and candidate dimension, the elements above / below the box centre and the extremes (first
// position); the segment's last CTA decides the split dimension and mode and the chunk offsets. Also clears the
// counters of the level after this one's successor (same parity as the level before).
__global__ void __launch_bounds__(R1_THREADS) statsDecideKernel(const TreeElem* __restrict__ elems, LevelBufs b,
    uint32_t* counters, int parity, uint32_t chunkCapacity, BhSegWork* work) {
    __shared__ uint32_t shCnt[R1_THREADS / 32][6];
    __shared__ unsigned long long shV[R1_THREADS / 32][6];
    __shared__ uint32_t shP[R1_THREADS / 32][6];
    __shared__ bool shLast;
    const uint32_t nChunks = min(counters[C_CHUNKS + parity], chunkCapacity);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counters[C_SEGS + 1 - parity] = 0;
        counters[C_CHUNKS + 1 - parity] = 0;
        if (nChunks > 0) {
            counters[C_R1_LEVELS]++;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t c = blockIdx.x; c < nChunks; c += gridDim.x) {
        const BhChunk ch = b.chunks[c];
        const BhSegment sg = b.seg[ch.seg];
        const uint32_t from = sg.from + ch.index * R1_CHUNK;
        const uint32_t to = min(sg.to, from + R1_CHUNK);
        unsigned long long center[3];
        for (int d = 0; d < 3; ++d) {
            center[d] = orderKey(0.5 * (sg.lo[d] + sg.hi[d]));
        }
        uint32_t nb[3] = { 0, 0, 0 }, ns[3] = { 0, 0, 0 };
        unsigned long long mnv[3] = { ~0ull, ~0ull, ~0ull }, mxv[3] = { 0ull, 0ull, 0ull };
        uint32_t mnp[3] = { 0xffffffffu, 0xffffffffu, 0xffffffffu }, mxp[3] = { 0xffffffffu, 0xffffffffu, 0xffffffffu };
#pragma unroll 4
        for (int j = 0; j < R1_PER_THREAD; ++j) {
            const uint32_t k = from + uint32_t(j * R1_THREADS) + threadIdx.x;
            if (k < to) {
                const ulonglong2 k01 = *reinterpret_cast<const ulonglong2*>(&elems[k].key[0]);
                const unsigned long long xs[3] = { k01.x, k01.y, elems[k].key[2] };
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const unsigned long long x = xs[d];
                    nb[d] += x > center[d] ? 1u : 0u;
                    ns[d] += x < center[d] ? 1u : 0u;
                    if (betterArg(x, k, mnv[d], mnp[d], false)) {
                        mnv[d] = x;
                        mnp[d] = k;
                    }
                    if (betterArg(x, k, mxv[d], mxp[d], true)) {
                        mxv[d] = x;
                        mxp[d] = k;
                    }
                }
            }
        }
        for (int d = 0; d < 3; ++d) {
            nb[d] = __reduce_add_sync(0xffffffffu, nb[d]);
            ns[d] = __reduce_add_sync(0xffffffffu, ns[d]);
            warpArgExtreme(mnv[d], mnp[d], false);
            warpArgExtreme(mxv[d], mxp[d], true);
        }
        if (lane == 0) {
            for (int d = 0; d < 3; ++d) {
                shCnt[warp][d] = nb[d];
                shCnt[warp][3 + d] = ns[d];
                shV[warp][d] = mnv[d];
                shP[warp][d] = mnp[d];
                shV[warp][3 + d] = mxv[d];
                shP[warp][3 + d] = mxp[d];
            }
        }
        __syncthreads();
        if (warp == 0) {
            constexpr int W = R1_THREADS / 32;
            BhChunkStats out;
            for (int d = 0; d < 3; ++d) {
                uint32_t cb = lane < W ? shCnt[lane][d] : 0u, cs = lane < W ? shCnt[lane][3 + d] : 0u;
                unsigned long long v0 = lane < W ? shV[lane][d] : ~0ull, v1 = lane < W ? shV[lane][3 + d] : 0ull;
                uint32_t p0 = lane < W ? shP[lane][d] : 0xffffffffu, p1 = lane < W ? shP[lane][3 + d] : 0xffffffffu;
                cb = __reduce_add_sync(0xffffffffu, cb);
                cs = __reduce_add_sync(0xffffffffu, cs);
                warpArgExtreme(v0, p0, false);
                warpArgExtreme(v1, p1, true);
                out.nb[d] = cb;
                out.ns[d] = cs;
                out.diff[d] = 0;
                out.minv[d] = v0;
                out.minp[d] = p0;
                out.maxv[d] = v1;
                out.maxp[d] = p1;
            }
            out.pad = 0;
            if (lane == 0) {
                b.stats[c] = out;
            }
        }
        if (!lastChunkOfSegment(b.done, ch.first, ch.count, &shLast) || warp != 0) {
            continue;
        }
        // the segment's decision (warp 0 of the last CTA; the other chunks' statistics are read through L2)
        mnv[0] = mnv[1] = mnv[2] = ~0ull;
        mxv[0] = mxv[1] = mxv[2] = 0ull;
        mnp[0] = mnp[1] = mnp[2] = mxp[0] = mxp[1] = mxp[2] = 0xffffffffu;
        for (uint32_t k = lane; k < ch.count; k += 32) {
            const BhChunkStats* st = &b.stats[ch.first + k];
            for (int d = 0; d < 3; ++d) {
                const unsigned long long v0 = __ldcg(&st->minv[d]), v1 = __ldcg(&st->maxv[d]);
                const uint32_t p0 = __ldcg(&st->minp[d]), p1 = __ldcg(&st->maxp[d]);
                if (betterArg(v0, p0, mnv[d], mnp[d], false)) {
                    mnv[d] = v0;
                    mnp[d] = p0;
                }
                if (betterArg(v1, p1, mxv[d], mxp[d], true)) {
                    mxv[d] = v1;
                    mxp[d] = p1;
                }
            }
        }
        bool nonSingular[3];
        for (int d = 0; d < 3; ++d) {
            warpArgExtreme(mnv[d], mnp[d], false);
            warpArgExtreme(mxv[d], mxp[d], true);
            nonSingular[d] = mnv[d] != mxv[d];
        }
        bool degenerated;
        const int splitIdx = splitDimension(sg, nonSingular, degenerated);
        uint32_t ob = 0, os = 0;
        for (uint32_t k0 = 0; k0 < ch.count; k0 += 32) {
            const uint32_t k = k0 + lane;
            uint32_t cb = 0, cs = 0;
            if (k < ch.count) {
                cb = __ldcg(&b.stats[ch.first + k].nb[splitIdx]);
                cs = __ldcg(&b.stats[ch.first + k].ns[splitIdx]);
            }
            uint32_t xb = cb, xs = cs;
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t yb = __shfl_up_sync(0xffffffffu, xb, off), ys = __shfl_up_sync(0xffffffffu, xs, off);
                if (lane >= off) {
                    xb += yb;
                    xs += ys;
                }
            }
            if (k < ch.count) {
                b.offB[ch.first + k] = ob + xb - cb;
                b.offS[ch.first + k] = os + xs - cs;
            }
            ob += __shfl_sync(0xffffffffu, xb, 31);
            os += __shfl_sync(0xffffffffu, xs, 31);
        }
        if (lane == 0) {
            BhSegWork w;
            w.splitIdx = splitIdx;
            w.mode = degenerated ? 2 : (sg.sliding <= 5 ? 0 : 1);
            w.nB = ob;
            w.nS = os;
            w.minv = mnv[splitIdx];
            w.minp = mnp[splitIdx];
            w.maxv = mxv[splitIdx];
            w.maxp = mxp[splitIdx];
            w.K = 0;
            w.pad = 0;
            work[ch.seg] = w;
        }
    }
}

// The segment's pair count K of the two-pointer partition (one warp: a 32-ary search of the monotone predicate
// posB[k] >= posS[nS - 1 - k], one probe per lane and round), then, in lane 0, the sliding midpoint or
// nth_element and the children: those of more than SUBTREE_MAX elements, with their chunks, into the next
// level's buffers, the others into the phase-2 queue.
__device__ void finishSegment(const dbl4* __restrict__ r, TreeElem* elems, const uint32_t* __restrict__ posB,
    uint32_t* posScratch, const BhSegment& sg, uint32_t segSlot, BhSegWork* work, LevelBufs next, int nextParity,
    uint32_t* counters, uint32_t chunkCapacity, uint32_t segCapacity, BhSegment* queue, BhNodeGeom* geom,
    uint32_t nodeCapacity, uint32_t* devError, const uint32_t* __restrict__ posS) {
    const int lane = threadIdx.x & 31;
    BhSegWork w = work[segSlot];
    const uint32_t from = sg.from, to = sg.to;
    uint32_t K = 0;
    if (w.mode == 0) {
        const uint32_t nS = w.nS;
        uint32_t lo = 0, hi = min(w.nB, nS);
        while (hi > lo) {
            const uint32_t span = hi - lo;
            if (span <= 32u) {
                const uint32_t k = lo + uint32_t(lane);
                const bool pred = uint32_t(lane) < span && __ldcg(&posB[from + k]) >= __ldcg(&posS[from + nS - 1 - k]);
                const unsigned m = __ballot_sync(0xffffffffu, pred);
                lo = m ? lo + uint32_t(__ffs(m) - 1) : hi;
                break;
            }
            // lanes probe lo + j span / 32; the first true probe bounds the answer from above, the last false one
            // from below
            const uint32_t k = lo + uint32_t((unsigned long long)span * uint32_t(lane) / 32u);
            const bool pred = __ldcg(&posB[from + k]) >= __ldcg(&posS[from + nS - 1 - k]);
            const unsigned m = __ballot_sync(0xffffffffu, pred);
            const int j = m ? __ffs(m) - 1 : 32;
            if (j == 0) {
                hi = lo;
                break;
            }
            const uint32_t newLo = lo + uint32_t((unsigned long long)span * uint32_t(j - 1) / 32u) + 1u;
            const uint32_t newHi = j < 32 ? lo + uint32_t((unsigned long long)span * uint32_t(j) / 32u) : hi;
            lo = newLo;
            hi = newHi;
        }
        K = lo;
    }
    if (lane != 0) {
        return;
    }
    const int d = w.splitIdx;
    double splitPosition = 0.5 * (sg.lo[d] + sg.hi[d]);
    uint32_t n1;
    bool sliding = false;
    double cut;
    if (w.mode == 0) {
        const uint32_t nB = w.nB, nS = w.nS;
        n1 = K < nB ? __ldcg(&posB[from + K]) : to;
        if (K >= 1) {
            n1 = min(n1, __ldcg(&posS[from + nS - K]));
        }
        if (n1 == from || n1 == to) {
            // sliding midpoint (then K = 0): the extreme element to the empty side
            const bool isMax = (n1 == to);
            const uint32_t dst = isMax ? to - 1 : from;
            const uint32_t src = isMax ? w.maxp : w.minp;
            splitPosition = coord(r, elems[src].idx, d);
            swapElements(elems, dst, src);
            n1 = isMax ? to - 1 : from + 1;
            sliding = true;
        }
        cut = splitPosition;
    } else {
        n1 = (from + to) >> 1;
        if (w.mode == 1) {
            // the rank scratch of this segment is not used in this mode
            nthElementSegment(r, elems, posScratch, from, to, n1, d);
        }
        cut = coord(r, elems[n1].idx, d);
    }
    work[segSlot].K = K;
    BhSegment left, right;
    if (!makeChildren(geom, counters, nodeCapacity, devError, sg, n1, d, cut, sliding, left, right)) {
        return;
    }
    pushSegment(left, next, nextParity, counters, chunkCapacity, segCapacity, queue, devError);
    pushSegment(right, next, nextParity, counters, chunkCapacity, segCapacity, queue, devError);
}

// Pass 2: positions of the elements above (posB) and below (posS) the split position, in segment order
// (R1_PER_THREAD consecutive elements per thread, one block scan of their packed counts per chunk); the
// segment's last CTA finishes the segment.
__global__ void __launch_bounds__(R1_THREADS) ranksFinishKernel(const dbl4* __restrict__ r, TreeElem* elems,
    LevelBufs b, LevelBufs next, uint32_t* counters, int parity, uint32_t chunkCapacity, uint32_t segCapacity,
    BhSegWork* work, uint32_t* posB, uint32_t* posS, BhSegment* queue, BhNodeGeom* geom, uint32_t nodeCapacity,
    uint32_t* devError) {
    __shared__ uint32_t shScan[R1_THREADS / 32];
    __shared__ bool shLast;
    const uint32_t nChunks = min(counters[C_CHUNKS + parity], chunkCapacity);
    for (uint32_t c = blockIdx.x; c < nChunks; c += gridDim.x) {
        const BhChunk ch = b.chunks[c];
        const BhSegment sg = b.seg[ch.seg];
        const int mode = work[ch.seg].mode;
        if (mode == 0) {
            const int d = work[ch.seg].splitIdx;
            const unsigned long long split = orderKey(0.5 * (sg.lo[d] + sg.hi[d]));
            const uint32_t from = sg.from + ch.index * R1_CHUNK;
            const uint32_t to = min(sg.to, from + R1_CHUNK);
            const uint32_t k0 = from + threadIdx.x * R1_PER_THREAD;
            uint32_t flagsB = 0, flagsS = 0;
#pragma unroll
            for (int j = 0; j < R1_PER_THREAD; ++j) {
                const uint32_t k = k0 + j;
                if (k < to) {
                    const unsigned long long x = elems[k].key[d];
                    flagsB |= (x > split ? 1u : 0u) << j;
                    flagsS |= (x < split ? 1u : 0u) << j;
                }
            }
            // counts of at most R1_CHUNK fit 16 bits each
            const uint32_t packed = (uint32_t(__popc(flagsB)) << 16) | uint32_t(__popc(flagsS));
            const uint32_t pre = blockExclusiveScan(packed, shScan);
            uint32_t rb = sg.from + b.offB[c] + (pre >> 16), rs = sg.from + b.offS[c] + (pre & 0xffffu);
#pragma unroll
            for (int j = 0; j < R1_PER_THREAD; ++j) {
                if (flagsB & (1u << j)) {
                    posB[rb++] = k0 + j;
                }
                if (flagsS & (1u << j)) {
                    posS[rs++] = k0 + j;
                }
            }
        }
        if (lastChunkOfSegment(b.done + chunkCapacity, ch.first, ch.count, &shLast) && threadIdx.x < 32) {
            finishSegment(r, elems, posB, posB, sg, ch.seg, work, next, 1 - parity, counters, chunkCapacity,
                segCapacity, queue, geom, nodeCapacity, devError, posS);
        }
        __syncthreads();
    }
}

// Pass 3: the K swaps of each segment's two-pointer partition, four per thread
__global__ void __launch_bounds__(SWAP_THREADS) chunkSwapKernel(TreeElem* elems, const uint32_t* __restrict__ posB,
    const uint32_t* __restrict__ posS, LevelBufs b, const uint32_t* __restrict__ counters, int parity,
    uint32_t chunkCapacity, const BhSegWork* __restrict__ work) {
    const uint32_t nChunks = min(counters[C_CHUNKS + parity], chunkCapacity);
    for (uint32_t c = blockIdx.x; c < nChunks; c += gridDim.x) {
        const BhChunk ch = b.chunks[c];
        const BhSegWork w = work[ch.seg];
        const uint32_t from = b.seg[ch.seg].from;
        const uint32_t k0 = ch.index * R1_CHUNK;
        const uint32_t k1 = min(w.K, k0 + R1_CHUNK);
        for (uint32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
            swapElements(elems, posB[from + k], posS[from + w.nS - 1 - k]);
        }
    }
}

// segments still in the phase-1 buffers after the last launched level go to the phase-2 queue
__global__ void flushKernel(LevelBufs b, uint32_t* counters, int parity, BhSegment* queue, uint32_t segCapacity,
    uint32_t* devError) {
    const uint32_t nIn = min(counters[C_SEGS + parity], segCapacity);
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < nIn; s += gridDim.x * blockDim.x) {
        const uint32_t slot = atomicAdd(&counters[C_QUEUE], 1u);
        if (slot < segCapacity) {
            queue[slot] = b.seg[s];
        } else {
            atomicOr(devError, uint32_t(DEV_ERR_SEGMENT_CAPACITY));
        }
    }
}

// ---------------------------------------------------------------------------------------------------------
// phase 2: one warp splits a segment down to its leaves, depth first
// ---------------------------------------------------------------------------------------------------------

// the elements [base, base + len) of a subtree: idx, keys of the three dimensions and the rank scratch, indexed
// from 0 (shared-memory copies, or the global arrays offset by base)
template <typename Pos>
struct SubView {
    uint32_t* idx;
    unsigned long long* key[3];
    Pos* posB;
    Pos* posS;
    uint32_t base;
};

template <typename Pos>
__device__ __forceinline__ void swapSub(const SubView<Pos>& a, uint32_t x, uint32_t y) {
    const uint32_t t = a.idx[x];
    a.idx[x] = a.idx[y];
    a.idx[y] = t;
    for (int d = 0; d < 3; ++d) {
        const unsigned long long k = a.key[d][x];
        a.key[d][x] = a.key[d][y];
        a.key[d][y] = k;
    }
}

// One split (or the leaf) of segment sg by the calling warp. Returns true, with the children in l and rr (valid in
// lane 0 only), when the segment was split.
template <typename Pos>
__device__ bool warpSplit(const dbl4* __restrict__ r, const SubView<Pos>& a, const BhSegment& sg, BhNodeGeom* geom,
    uint32_t* counters, uint32_t* leaves, uint32_t leafSize, uint32_t nodeCapacity, uint32_t* devError, BhSegment& l,
    BhSegment& rr) {
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const uint32_t from = sg.from - a.base, to = sg.to - a.base;
    const int node = sg.node;
    if (sg.to - sg.from <= leafSize) {
        // KdTree::addLeaf: tight box of the leaf's points, as the extreme order keys (integer minima, exact in any
        // order; a coordinate of -0 is returned as +0, which no difference or comparison of the box tells apart)
        unsigned long long lo[3] = { ~0ull, ~0ull, ~0ull }, hi[3] = { 0ull, 0ull, 0ull };
        for (uint32_t k = from + lane; k < to; k += 32) {
            for (int d = 0; d < 3; ++d) {
                const unsigned long long x = a.key[d][k];
                lo[d] = min(lo[d], x);
                hi[d] = max(hi[d], x);
            }
        }
        for (int d = 0; d < 3; ++d) {
            for (int off = 16; off > 0; off >>= 1) {
                lo[d] = min(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
                hi[d] = max(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
            }
        }
        if (lane == 0) {
            BhNodeGeom& g = geom[node];
            for (int d = 0; d < 3; ++d) {
                g.lo[d] = keyValue(lo[d]);
                g.hi[d] = keyValue(hi[d]);
            }
            g.left = -1;
            g.right = -1;
            g.from = sg.from;
            g.to = sg.to;
            const uint32_t slot = atomicAdd(&counters[C_LEAVES], 1u);
            leaves[slot] = uint32_t(node);
        }
        return false;
    }
    // singular dimensions: every key equal to the last element's
    bool diff[3] = { false, false, false };
    {
        const unsigned long long last[3] = { a.key[0][to - 1], a.key[1][to - 1], a.key[2][to - 1] };
        for (uint32_t k = from + lane; k < to; k += 32) {
            for (int d = 0; d < 3; ++d) {
                diff[d] = diff[d] || (a.key[d][k] != last[d]);
            }
        }
    }
    bool nonSingular[3];
    for (int d = 0; d < 3; ++d) {
        nonSingular[d] = __any_sync(0xffffffffu, diff[d]);
    }
    bool degenerated;
    const int splitIdx = splitDimension(sg, nonSingular, degenerated);
    double splitPosition = 0.5 * (sg.lo[splitIdx] + sg.hi[splitIdx]);
    uint32_t n1;
    bool sliding = false;
    double cut;
    const unsigned long long* kd = a.key[splitIdx];
    if (sg.sliding <= 5 && !degenerated) {
        const unsigned long long splitKey = orderKey(splitPosition);
        uint32_t nB = 0, nS = 0;
        for (uint32_t k0 = from; k0 < to; k0 += 32) {
            const uint32_t k = k0 + lane;
            bool isB = false, isS = false;
            if (k < to) {
                const unsigned long long x = kd[k];
                isB = x > splitKey;
                isS = x < splitKey;
            }
            const unsigned mB = __ballot_sync(0xffffffffu, isB), mS = __ballot_sync(0xffffffffu, isS);
            if (isB) {
                a.posB[from + nB + __popc(mB & below)] = Pos(k);
            }
            if (isS) {
                a.posS[from + nS + __popc(mS & below)] = Pos(k);
            }
            nB += __popc(mB);
            nS += __popc(mS);
        }
        __syncwarp();
        const uint32_t m = min(nB, nS);
        uint32_t cntLocal = 0;
        for (uint32_t k = lane; k < m; k += 32) {
            cntLocal += (a.posB[from + k] < a.posS[from + nS - 1 - k]) ? 1u : 0u;
        }
        const uint32_t K = __reduce_add_sync(0xffffffffu, cntLocal);
        uint32_t n1b = K < nB ? a.posB[from + K] : to;
        if (K >= 1) {
            n1b = min(n1b, a.posS[from + nS - K]);
        }
        for (uint32_t k = lane; k < K; k += 32) {
            swapSub(a, a.posB[from + k], a.posS[from + nS - 1 - k]);
        }
        __syncwarp();
        n1 = n1b;
        if (n1 == from || n1 == to) {
            // sliding midpoint: the extreme element (first occurrence) to the empty side
            const bool isMax = (n1 == to);
            unsigned long long val = isMax ? 0ull : ~0ull;
            uint32_t pos = 0xffffffffu;
            for (uint32_t k = from + lane; k < to; k += 32) {
                const unsigned long long x = kd[k];
                if (betterArg(x, k, val, pos, isMax)) {
                    val = x;
                    pos = k;
                }
            }
            warpArgExtreme(val, pos, isMax);
            splitPosition = coord(r, a.idx[pos], splitIdx);
            __syncwarp();
            if (lane == 0) {
                swapSub(a, isMax ? to - 1 : from, pos);
            }
            __syncwarp();
            n1 = isMax ? to - 1 : from + 1;
            sliding = true;
        }
        cut = splitPosition;
    } else {
        n1 = (from + to) >> 1;
        if (!degenerated) {
            if (lane == 0) {
                NthCtx c{ a.idx, r, splitIdx };
                nthElement(c, long(from), long(n1), long(to));
            }
            __syncwarp();
            for (uint32_t k = from + lane; k < to; k += 32) {
                const dbl4 p = r[a.idx[k]];
                a.key[0][k] = orderKey(p.x);
                a.key[1][k] = orderKey(p.y);
                a.key[2][k] = orderKey(p.z);
            }
        }
        __syncwarp();
        cut = coord(r, a.idx[n1], splitIdx);
    }
    int ok = 0;
    if (lane == 0) {
        ok = makeChildren(geom, counters, nodeCapacity, devError, sg, n1 + a.base, splitIdx, cut, sliding, l, rr) ? 1
                                                                                                                  : 0;
    }
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// shared memory of one warp of subtreeKernel
// (18.7 KB: three CTAs of four warps fit the shared memory of an SM)
struct SubtreeShared {
    uint32_t idx[SUBTREE_MAX];
    unsigned long long key[3][SUBTREE_MAX];
    uint16_t posB[SUBTREE_MAX];
    uint16_t posS[SUBTREE_MAX];
    BhSegment stack[R2_STACK];
};
static_assert(SUBTREE_MAX <= 65536, "subtree positions are 16-bit");

// the segment `top` split down to its leaves, depth first, by the calling warp (stack in shared memory)
template <typename Pos>
__device__ void splitSubtree(const dbl4* __restrict__ r, const SubView<Pos>& a, const BhSegment& top,
    BhSegment* stack, BhNodeGeom* geom, uint32_t* counters, uint32_t* leaves, uint32_t leafSize,
    uint32_t nodeCapacity, uint32_t* devError) {
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        stack[0] = top;
    }
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
        const BhSegment sg = stack[--sp];
        __syncwarp();
        // with the stack full, the segment becomes a leaf (flagged as an error): every node keeps a valid state
        const bool full = sp + 2 > R2_STACK;
        if (full && lane == 0) {
            atomicOr(devError, uint32_t(DEV_ERR_SEGMENT_CAPACITY));
        }
        BhSegment l, rr;
        if (warpSplit(r, a, sg, geom, counters, leaves, full ? 0xffffffffu : leafSize, nodeCapacity, devError, l,
                rr)) {
            if (lane == 0) {
                stack[sp] = rr;
                stack[sp + 1] = l;
            }
            sp += 2;
        }
        __syncwarp();
    }
}

// idx receives the final permutation; keys (3 x n) is the scratch of segments too large for shared memory
__global__ void __launch_bounds__(R2_WARPS * 32) subtreeKernel(const dbl4* __restrict__ r, uint32_t n,
    const TreeElem* __restrict__ elems, uint32_t* idx, unsigned long long* keys, uint32_t* posBg, uint32_t* posSg,
    const BhSegment* __restrict__ queue, uint32_t* counters, BhNodeGeom* geom, uint32_t* leaves, uint32_t leafSize,
    uint32_t nodeCapacity, uint32_t segCapacity, uint32_t* devError) {
    extern __shared__ __align__(16) unsigned char smem[];
    SubtreeShared& sh = reinterpret_cast<SubtreeShared*>(smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const uint32_t nQueue = min(counters[C_QUEUE], segCapacity);
    for (;;) {
        uint32_t q = 0;
        if (lane == 0) {
            q = atomicAdd(&counters[C_TAKEN], 1u);
        }
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= nQueue) {
            break;
        }
        const BhSegment top = queue[q];
        const uint32_t len = top.to - top.from;
        if (len <= SUBTREE_MAX) {
            for (uint32_t k = lane; k < len; k += 32) {
                const TreeElem e = elems[top.from + k];
                sh.idx[k] = e.idx;
                for (int d = 0; d < 3; ++d) {
                    sh.key[d][k] = e.key[d];
                }
            }
            SubView<uint16_t> a;
            a.base = top.from;
            a.idx = sh.idx;
            for (int d = 0; d < 3; ++d) {
                a.key[d] = sh.key[d];
            }
            a.posB = sh.posB;
            a.posS = sh.posS;
            __syncwarp();
            splitSubtree(r, a, top, sh.stack, geom, counters, leaves, leafSize, nodeCapacity, devError);
            for (uint32_t k = lane; k < len; k += 32) {
                idx[top.from + k] = sh.idx[k];
            }
        } else {
            // a segment that phase 1 left over: the same splits on global copies
            for (uint32_t k = lane; k < len; k += 32) {
                const TreeElem e = elems[top.from + k];
                idx[top.from + k] = e.idx;
                for (int d = 0; d < 3; ++d) {
                    keys[size_t(d) * n + top.from + k] = e.key[d];
                }
            }
            SubView<uint32_t> a;
            a.base = top.from;
            a.idx = idx + top.from;
            for (int d = 0; d < 3; ++d) {
                a.key[d] = keys + size_t(d) * n + top.from;
            }
            a.posB = posBg + top.from;
            a.posS = posSg + top.from;
            __syncwarp();
            splitSubtree(r, a, top, sh.stack, geom, counters, leaves, leafSize, nodeCapacity, devError);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------------------------------
// nodes by level (counting sort) for the level-by-level list phase of the mixed walk
// ---------------------------------------------------------------------------------------------------------

// nodes per level: a shared-memory histogram per tile of blockDim nodes, one global atomic per level and tile
__global__ void levelCountKernel(const BhNodeGeom* __restrict__ geom, const uint32_t* __restrict__ counters,
    uint32_t nodeCapacity, uint32_t* levelCount, uint32_t* devError) {
    __shared__ uint32_t hist[TREE_MAX_LEVELS];
    const uint32_t nn = min(counters[C_NODES], nodeCapacity);
    const uint32_t depth = min(counters[C_DEPTH], TREE_MAX_LEVELS);
    for (uint32_t t0 = blockIdx.x * blockDim.x; t0 < nn; t0 += gridDim.x * blockDim.x) {
        for (uint32_t l = threadIdx.x; l < depth; l += blockDim.x) {
            hist[l] = 0;
        }
        __syncthreads();
        const uint32_t id = t0 + threadIdx.x;
        if (id < nn) {
            const int lvl = geom[id].level;
            if (lvl < 0 || uint32_t(lvl) >= depth) {
                atomicOr(devError, uint32_t(DEV_ERR_NODE_CAPACITY));
            } else {
                atomicAdd(&hist[lvl], 1u);
            }
        }
        __syncthreads();
        for (uint32_t l = threadIdx.x; l < depth; l += blockDim.x) {
            if (hist[l]) {
                atomicAdd(&levelCount[l], hist[l]);
            }
        }
        __syncthreads();
    }
}

// exclusive scan of the level counts (one warp, TREE_MAX_LEVELS / 32 consecutive levels per lane)
__global__ void levelScanKernel(const uint32_t* __restrict__ levelCount, uint32_t* levelFirst, uint32_t* cursor) {
    constexpr int PER = int(TREE_MAX_LEVELS) / 32;
    const int lane = threadIdx.x;
    uint32_t local = 0;
    for (int k = 0; k < PER; ++k) {
        local += levelCount[lane * PER + k];
    }
    uint32_t x = local;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) {
            x += y;
        }
    }
    uint32_t run = x - local;
    for (int k = 0; k < PER; ++k) {
        levelFirst[lane * PER + k] = run;
        cursor[lane * PER + k] = 0;
        run += levelCount[lane * PER + k];
    }
}

// node ids by level: per tile, ranks within the tile's level bins in shared memory and one global cursor
// advance per level and tile
__global__ void levelScatterKernel(const BhNodeGeom* __restrict__ geom, const uint32_t* __restrict__ counters,
    uint32_t nodeCapacity, const uint32_t* __restrict__ levelFirst, uint32_t* cursor, uint32_t* levelNodes) {
    __shared__ uint32_t hist[TREE_MAX_LEVELS];
    __shared__ uint32_t base[TREE_MAX_LEVELS];
    const uint32_t nn = min(counters[C_NODES], nodeCapacity);
    const uint32_t depth = min(counters[C_DEPTH], TREE_MAX_LEVELS);
    for (uint32_t t0 = blockIdx.x * blockDim.x; t0 < nn; t0 += gridDim.x * blockDim.x) {
        for (uint32_t l = threadIdx.x; l < depth; l += blockDim.x) {
            hist[l] = 0;
        }
        __syncthreads();
        const uint32_t id = t0 + threadIdx.x;
        int lvl = -1;
        uint32_t local = 0;
        if (id < nn) {
            lvl = geom[id].level;
            if (lvl >= 0 && uint32_t(lvl) < depth) {
                local = atomicAdd(&hist[lvl], 1u);
            } else {
                lvl = -1;
            }
        }
        __syncthreads();
        for (uint32_t l = threadIdx.x; l < depth; l += blockDim.x) {
            if (hist[l]) {
                base[l] = levelFirst[l] + atomicAdd(&cursor[l], hist[l]);
            }
        }
        __syncthreads();
        if (lvl >= 0) {
            levelNodes[base[lvl] + local] = id;
        }
        __syncthreads();
    }
}

int residentGrid(const void* kernel, int threads, size_t shared) {
    int perSm = 0, sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, threads, shared);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::max(1, perSm * sms);
}

} // namespace

cudaError_t treeBuildAllocate(Tree& t, uint32_t n) {
    const uint32_t nn = n > 0 ? n : 1;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) {
            e = cudaMalloc(p, bytes > 0 ? bytes : 16);
        }
    };
    alloc((void**)&t.elems, size_t(nn) * sizeof(TreeElem));
    alloc((void**)&t.subtree_keys, 3 * size_t(nn) * sizeof(unsigned long long));
    alloc((void**)&t.queue, size_t(t.seg_capacity) * sizeof(BhSegment));
    alloc((void**)&t.level_count, TREE_MAX_LEVELS * sizeof(uint32_t));
    alloc((void**)&t.level_first_dev, TREE_MAX_LEVELS * sizeof(uint32_t));
    alloc((void**)&t.level_cursor, TREE_MAX_LEVELS * sizeof(uint32_t));
    alloc((void**)&t.level_nodes, size_t(t.node_capacity) * sizeof(uint32_t));
    // phase-1 buffers of two level parities
    t.chunk_capacity = treeChunkCapacity(nn);
    const size_t cc2 = 2 * size_t(t.chunk_capacity);
    alloc((void**)&t.chunks, cc2 * sizeof(BhChunk));
    alloc((void**)&t.chunk_stats, cc2 * sizeof(BhChunkStats));
    alloc((void**)&t.chunk_off_b, cc2 * sizeof(uint32_t));
    alloc((void**)&t.chunk_off_s, cc2 * sizeof(uint32_t));
    alloc((void**)&t.chunk_done, 2 * cc2 * sizeof(uint32_t));
    alloc((void**)&t.work, size_t(t.seg_capacity) * sizeof(BhSegWork));
    if (e == cudaSuccess) {
        e = cudaMallocHost((void**)&t.info_host, (C_WORDS + TREE_MAX_LEVELS) * sizeof(uint32_t));
    }
    return e;
}

void treeBuildFree(Tree& t) {
    void* ptrs[] = { t.elems, t.subtree_keys, t.queue, t.level_count, t.level_first_dev, t.level_cursor, t.level_nodes,
        t.chunks, t.chunk_stats, t.chunk_off_b, t.chunk_off_s, t.chunk_done, t.work };
    for (void* p : ptrs) {
        if (p) {
            cudaFree(p);
        }
    }
    if (t.info_host) {
        cudaFreeHost(t.info_host);
    }
}

// chunks of one phase-1 level: each segment has more than SUBTREE_MAX elements, so a level holds fewer than
// n / SUBTREE_MAX segments and at most n / R1_CHUNK + (segments) chunks
uint32_t treeChunkCapacity(uint32_t n) {
    const uint32_t nn = n > 0 ? n : 1;
    return nn / R1_CHUNK + nn / SUBTREE_MAX + 64;
}

namespace {

LevelBufs levelBufs(const Tree& t, int parity) {
    const size_t off = size_t(parity) * t.chunk_capacity;
    LevelBufs b;
    b.seg = t.seg[parity];
    b.chunks = t.chunks + off;
    b.stats = t.chunk_stats + off;
    b.offB = t.chunk_off_b + off;
    b.offS = t.chunk_off_s + off;
    b.done = t.chunk_done + 2 * off;
    return b;
}

} // namespace

cudaError_t treeBuild(const DState& s, Tree& t, const Physics& ph, uint32_t* devError, cudaStream_t st) {
    const uint32_t n = s.n;
    t.built = false;
    t.level_first.clear();
    if (n == 0) {
        t.node_count = 0;
        t.leaf_count = 0;
        t.built = true;
        return cudaSuccess;
    }
    static int gridC = 0, gridR2 = 0, gridSwap = 0;
    const size_t r2Shared = R2_WARPS * sizeof(SubtreeShared);
    if (gridC == 0) {
        gridC = std::min(residentGrid(reinterpret_cast<const void*>(statsDecideKernel), R1_THREADS, 0),
            residentGrid(reinterpret_cast<const void*>(ranksFinishKernel), R1_THREADS, 0));
        gridSwap = residentGrid(reinterpret_cast<const void*>(chunkSwapKernel), SWAP_THREADS, 0);
        cudaFuncSetAttribute(subtreeKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(r2Shared));
        gridR2 = residentGrid(reinterpret_cast<const void*>(subtreeKernel), R2_WARPS * 32, r2Shared);
    }
    t.launches = 0;
    auto launched = [&](uint32_t k) { t.launches += k; };
    const uint32_t cc = t.chunk_capacity;
    resetBoundsKernel<<<1, 32, 0, st>>>(t.bbox);
    boundsKernel<<<std::min(ceilDiv(n, 256), 152 * 2), 256, 0, st>>>(s.r, n, t.bbox);
    rootKernel<<<ceilDiv(n, 256), 256, 0, st>>>(s.r, n, t.elems, levelBufs(t, 0), t.queue, t.geom, t.counters, cc,
        t.seg_capacity, t.bbox, devError);
    cudaMemsetAsync(t.level_count, 0, TREE_MAX_LEVELS * sizeof(uint32_t), st);
    launched(3);
    // phase 1: the previous build's level count plus two (a first build: from the size)
    uint32_t levels = t.r1_levels + 2;
    if (t.r1_levels == 0) {
        levels = 2;
        for (uint32_t m = n; m > SUBTREE_MAX; m >>= 1) {
            ++levels;
        }
    }
    if (n <= SUBTREE_MAX) {
        levels = 0;
    }
    auto launchLevel = [&](uint32_t level) {
        const int p = int(level & 1u);
        const LevelBufs b = levelBufs(t, p), next = levelBufs(t, 1 - p);
        statsDecideKernel<<<gridC, R1_THREADS, 0, st>>>(t.elems, b, t.counters, p, cc, t.work);
        ranksFinishKernel<<<gridC, R1_THREADS, 0, st>>>(s.r, t.elems, b, next, t.counters, p, cc, t.seg_capacity,
            t.work, t.scratch_b, t.scratch_s, t.queue, t.geom, t.node_capacity, devError);
        chunkSwapKernel<<<gridSwap, SWAP_THREADS, 0, st>>>(t.elems, t.scratch_b, t.scratch_s, b, t.counters, p, cc,
            t.work);
        launched(3);
    };
    for (uint32_t level = 0; level < levels; ++level) {
        launchLevel(level);
    }
    // a deeper tree than the last one (a first build, a more concentrated distribution): more levels while large
    // segments remain (one host read per batch; the one-warp splits of the queue would take them otherwise)
    for (int batch = 0; levels > 0 && batch < 64; ++batch) {
        cudaMemcpyAsync(t.info_host, t.counters + C_SEGS + (levels & 1u), sizeof(uint32_t), cudaMemcpyDeviceToHost,
            st);
        if (cudaStreamSynchronize(st) != cudaSuccess || t.info_host[0] == 0) {
            break;
        }
        for (uint32_t k = 0; k < 4; ++k) {
            launchLevel(levels++);
        }
    }
    const uint32_t gridSeg = std::max(1, std::min(ceilDiv(n / SUBTREE_MAX + 1, 256), 152 * 8));
    flushKernel<<<gridSeg, 256, 0, st>>>(levelBufs(t, int(levels & 1u)), t.counters, int(levels & 1u), t.queue,
        t.seg_capacity, devError);
    // phase 2
    subtreeKernel<<<gridR2, R2_WARPS * 32, r2Shared, st>>>(s.r, n, t.elems, t.idx, t.subtree_keys, t.scratch_b,
        t.scratch_s, t.queue,
        t.counters, t.geom, t.leaves, ph.leaf_size, t.node_capacity, t.seg_capacity, devError);
    // nodes by level
    const int gridNodes = std::min(ceilDiv(t.node_capacity, 256), 152 * 8);
    levelCountKernel<<<gridNodes, 256, 0, st>>>(t.geom, t.counters, t.node_capacity, t.level_count, devError);
    levelScanKernel<<<1, 32, 0, st>>>(t.level_count, t.level_first_dev, t.level_cursor);
    levelScatterKernel<<<gridNodes, 256, 0, st>>>(t.geom, t.counters, t.node_capacity, t.level_first_dev,
        t.level_cursor, t.level_nodes);
    launched(5);
    // the counts to the host (the walk launches its level passes from them), before the moments: the host returns
    // while the moments are formed, so that work queued on other streams next (the SPH pair loop) overlaps them
    cudaMemcpyAsync(t.info_host, t.counters, C_WORDS * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(t.info_host + C_WORDS, t.level_count, TREE_MAX_LEVELS * sizeof(uint32_t), cudaMemcpyDeviceToHost,
        st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        return e;
    }
    // moments, bottom-up, and the walks' FP32 node records, sized on the device
    t.mixed_moments = ph.precision == SPHGPU_PRECISION_MIXED;
    launchMomentsDev(s, t, ph, t.mixed_moments, st);
    launchPrepareWalkDev(s, t, ph, st);
    launched(3);
    const uint32_t* info = t.info_host;
    t.node_count = std::min(info[C_NODES], t.node_capacity);
    t.leaf_count = std::min(info[C_LEAVES], n);
    t.r1_levels = info[C_R1_LEVELS];
    const uint32_t depth = std::min(info[C_DEPTH], TREE_MAX_LEVELS);
    uint32_t run = 0;
    for (uint32_t l = 0; l < depth; ++l) {
        t.level_first.push_back(run);
        run += info[C_WORDS + l];
    }
    t.level_first.push_back(run);
    t.built = true;
    return cudaGetLastError();
}

} // namespace sphgpu
