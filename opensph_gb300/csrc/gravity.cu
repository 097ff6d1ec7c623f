// gravity.cu — Barnes-Hut self-gravity in FP64 (compiled with -fmad=false).
//
// Replaces BarnesHut::build / evalSelfGravity / evalAcceleration (core/gravity/BarnesHut.cpp:50-175,
// 212-489) with the k-d tree of KdTree::buildTree (core/objects/finders/KdTree.inl.h:44-160) and the
// moments of core/gravity/Moments.h.
//
// Build: level-synchronous. Every segment (tree node still to split) of a level is processed by one CTA,
// which reproduces the reference partition exactly: the two-pointer partition of the reference around the
// box centre is equivalent to pairing the k-th element above the split (from the left) with the k-th
// element below it (from the right) while they are out of order, which a CTA computes with block scans;
// the sliding-midpoint steps (single extreme element moved to one side) are arg-min/arg-max reductions
// with the reference's first-occurrence tie rule; after more than five consecutive slides the reference's
// std::nth_element is replayed by one thread (libstdc++ introselect). Leaf membership and the order of the
// particles inside each leaf are therefore identical to the reference's, and so are the leaf boxes and
// centres of mass. Moments are then formed bottom-up in one launch (momentsUpKernel).
//
// Walk: one warp per leaf replays the reference's dual walk along the leaf's root path: at each ancestor
// the pending check-list entries are classified against that ancestor's box with the reference's
// sphere-box test (core/objects/geometry/Sphere.h:70-116), so every leaf receives exactly the reference's
// particle list and node list. Each lane owns one particle of the leaf (leaf size <= 32) and evaluates the
// exact softened pair terms and octupole expansions as soon as the warp classifies them.

#include <algorithm>

#include "tree.cuh"

namespace sphgpu {

namespace {

// 128 threads per block, so that a block of each build kernel fits in the registers the concurrent pair loop
// (main stream) leaves free on an SM: the build then starts its blocks at once instead of waiting for pair
// blocks to retire
constexpr int BUILD_THREADS = 128;
constexpr int MAX_PATH = 512;

struct PosView {
    const dbl4* r;
    __device__ __forceinline__ double val(uint32_t i, int dim) const {
        return __ldg(reinterpret_cast<const double*>(r) + 4 * size_t(i) + dim);
    }
    // orderKey of the coordinate: the build compares keys (integer pipe) instead of doubles (slow FP64 pipe)
    __device__ __forceinline__ unsigned long long key(uint32_t i, int dim) const {
        return orderKey(val(i, dim));
    }
};

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

// ---------------------------------------------------------------------------------------------------------
// libstdc++ introselect, replayed for the rare nth_element split of KdTree::buildTree (single thread)
// ---------------------------------------------------------------------------------------------------------

struct NthCtx {
    uint32_t* a;
    PosView pv;
    int dim;
    __device__ __forceinline__ bool less(uint32_t x, uint32_t y) const {
        return pv.val(x, dim) < pv.val(y, dim);
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
// build
// ---------------------------------------------------------------------------------------------------------

__global__ void initRootKernel(uint32_t n, uint32_t* idx, BhSegment* seg, BhNodeGeom* geom, uint32_t* counters,
    const unsigned long long* bounds) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        idx[i] = i;
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
        seg[0] = s;
        geom[0].parent = -1;
        geom[0].level = 0;
        counters[0] = 1;
        counters[1] = 0;
        counters[2] = 0;
        counters[3] = 0;
        counters[4] = 0;
    }
}

__global__ void boundsOnlyKernel(const dbl4* __restrict__ r, uint32_t n, unsigned long long* b) {
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
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            atomicMin(&b[k], mn[k]);
            atomicMax(&b[3 + k], mx[k]);
        }
    }
}

__global__ void resetBounds6(unsigned long long* b) {
    if (threadIdx.x < 3) {
        b[threadIdx.x] = ~0ull;
        b[3 + threadIdx.x] = 0ull;
    }
}

// block-wide helpers (BUILD_THREADS threads)
__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t& total, uint32_t* sh) {
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
    if (warp == 0) {
        uint32_t w = lane < (BUILD_THREADS / 32) ? sh[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) {
                w += y;
            }
        }
        if (lane < (BUILD_THREADS / 32)) {
            sh[lane] = w;
        }
    }
    __syncthreads();
    const uint32_t warpOffset = warp > 0 ? sh[warp - 1] : 0;
    total = sh[BUILD_THREADS / 32 - 1];
    __syncthreads();
    return warpOffset + x - v;
}

__device__ __forceinline__ uint32_t blockSum(uint32_t v, uint32_t* sh) {
    uint32_t total;
    blockExclusiveScan(v, total, sh);
    return total;
}

__device__ __forceinline__ bool blockAny(bool v, int* sh) {
    const int r = __syncthreads_or(v ? 1 : 0);
    (void)sh;
    return r != 0;
}

// (key, position) lexicographic minimum (maximum) across the block, the first occurrence on ties
__device__ void blockArgExtreme(unsigned long long& val, uint32_t& pos, bool isMax, unsigned long long* shv,
    uint32_t* shp) {
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long ov = __shfl_xor_sync(0xffffffffu, val, off);
        const uint32_t op = __shfl_xor_sync(0xffffffffu, pos, off);
        const bool better = isMax ? (ov > val || (ov == val && op < pos)) : (ov < val || (ov == val && op < pos));
        if (better) {
            val = ov;
            pos = op;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        shv[warp] = val;
        shp[warp] = pos;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < BUILD_THREADS / 32; ++w) {
            const unsigned long long ov = shv[w];
            const uint32_t op = shp[w];
            const bool better =
                isMax ? (ov > shv[0] || (ov == shv[0] && op < shp[0])) : (ov < shv[0] || (ov == shv[0] && op < shp[0]));
            if (better) {
                shv[0] = ov;
                shp[0] = op;
            }
        }
    }
    __syncthreads();
    val = shv[0];
    pos = shp[0];
    __syncthreads();
}

__global__ void __launch_bounds__(BUILD_THREADS) splitLevelKernel(PosView pv, uint32_t* idx, uint32_t* posB,
    uint32_t* posS, const BhSegment* segIn, uint32_t nIn, BhSegment* segOut, BhNodeGeom* geom, uint32_t* counters,
    uint32_t* leaves, uint32_t leafSize, uint32_t nodeCapacity, uint32_t segCapacity, uint32_t* devError,
    uint32_t minSize, uint32_t maxSize) {
    __shared__ uint32_t shScan[32];
    __shared__ unsigned long long shV[32];
    __shared__ uint32_t shP[32];
    __shared__ int shAny[4];
    __shared__ uint32_t shNode[2];
    for (uint32_t sidx = blockIdx.x; sidx < nIn; sidx += gridDim.x) {
        const BhSegment sg = segIn[sidx];
        const uint32_t from = sg.from, to = sg.to;
        const int node = sg.node;
        if (to - from > maxSize || to - from <= minSize) {
            continue; // large segments: the multi-CTA pipeline below; small ones: splitWarpKernel
        }
        if (to - from <= leafSize) {
            // KdTree::addLeaf: tight box of the leaf's points
            double lo[3] = { DBL_MAX, DBL_MAX, DBL_MAX }, hi[3] = { -DBL_MAX, -DBL_MAX, -DBL_MAX };
            if (threadIdx.x == 0) {
                for (uint32_t k = from; k < to; ++k) {
                    const uint32_t i = idx[k];
                    for (int d = 0; d < 3; ++d) {
                        const double x = pv.val(i, d);
                        lo[d] = fmin(lo[d], x);
                        hi[d] = fmax(hi[d], x);
                    }
                }
                BhNodeGeom& g = geom[node];
                for (int d = 0; d < 3; ++d) {
                    g.lo[d] = lo[d];
                    g.hi[d] = hi[d];
                }
                g.left = -1;
                g.right = -1;
                g.from = from;
                g.to = to;
                const uint32_t slot = atomicAdd(&counters[2], 1u);
                leaves[slot] = uint32_t(node);
            }
            __syncthreads();
            continue;
        }
        // split by the dimension of largest extent of the (split) box
        double boxSize[3];
        for (int d = 0; d < 3; ++d) {
            boxSize[d] = sg.hi[d] - sg.lo[d];
        }
        int splitIdx = argMax3(boxSize);
        // singularity of each dimension: all values equal to the last one
        bool diff[3] = { false, false, false };
        {
            const uint32_t il = idx[to - 1];
            const unsigned long long last[3] = { pv.key(il, 0), pv.key(il, 1), pv.key(il, 2) };
            for (uint32_t k = from + threadIdx.x; k < to; k += BUILD_THREADS) {
                const uint32_t i = idx[k];
                for (int d = 0; d < 3; ++d) {
                    diff[d] = diff[d] || (pv.key(i, d) != last[d]);
                }
            }
        }
        bool nonSingular[3];
        for (int d = 0; d < 3; ++d) {
            nonSingular[d] = blockAny(diff[d], shAny);
        }
        bool degenerated = false;
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
        double splitPosition = 0.5 * (sg.lo[splitIdx] + sg.hi[splitIdx]);
        uint32_t n1;
        bool sliding = false;
        double lo1[3], hi1[3], lo2[3], hi2[3];
        for (int d = 0; d < 3; ++d) {
            lo1[d] = lo2[d] = sg.lo[d];
            hi1[d] = hi2[d] = sg.hi[d];
        }
        if (sg.sliding <= 5 && !degenerated) {
            // ranks of the elements above (B) and below (S) the split position, left to right
            const unsigned long long splitKey = orderKey(splitPosition);
            uint32_t baseB = 0, baseS = 0;
            for (uint32_t k0 = from; k0 < to; k0 += BUILD_THREADS) {
                const uint32_t k = k0 + threadIdx.x;
                bool isB = false, isS = false;
                if (k < to) {
                    const unsigned long long x = pv.key(idx[k], splitIdx);
                    isB = x > splitKey;
                    isS = x < splitKey;
                }
                uint32_t totB, totS;
                const uint32_t rb = blockExclusiveScan(isB ? 1u : 0u, totB, shScan);
                const uint32_t rs = blockExclusiveScan(isS ? 1u : 0u, totS, shScan);
                if (isB) {
                    posB[from + baseB + rb] = k;
                }
                if (isS) {
                    posS[from + baseS + rs] = k;
                }
                baseB += totB;
                baseS += totS;
            }
            __syncthreads();
            const uint32_t nB = baseB, nS = baseS;
            // K = number of (k-th B from the left, k-th S from the right) pairs that are out of order
            const uint32_t m = min(nB, nS);
            uint32_t cntLocal = 0;
            for (uint32_t k = threadIdx.x; k < m; k += BUILD_THREADS) {
                cntLocal += (posB[from + k] < posS[from + nS - 1 - k]) ? 1u : 0u;
            }
            const uint32_t K = blockSum(cntLocal, shScan);
            // the two-pointer partition swaps exactly these pairs
            for (uint32_t k = threadIdx.x; k < K; k += BUILD_THREADS) {
                const uint32_t a = posB[from + k], b = posS[from + nS - 1 - k];
                const uint32_t t = idx[a];
                idx[a] = idx[b];
                idx[b] = t;
            }
            __syncthreads();
            uint32_t n1b = K < nB ? posB[from + K] : to;
            if (K >= 1) {
                n1b = min(n1b, posS[from + nS - K]);
            }
            n1 = n1b;
            if (n1 == from || n1 == to) {
                // sliding midpoint: move the extreme element (first occurrence) to the empty side
                const bool isMax = (n1 == to);
                unsigned long long val = isMax ? 0ull : ~0ull;
                uint32_t pos = 0xffffffffu;
                for (uint32_t k = from + threadIdx.x; k < to; k += BUILD_THREADS) {
                    const unsigned long long x = pv.key(idx[k], splitIdx);
                    const bool better = isMax ? (x > val || (x == val && k < pos)) : (x < val || (x == val && k < pos));
                    if (better) {
                        val = x;
                        pos = k;
                    }
                }
                blockArgExtreme(val, pos, isMax, shV, shP);
                // the extreme coordinate itself (its key was formed from it)
                const double extreme = pv.val(idx[pos], splitIdx);
                __syncthreads();
                if (threadIdx.x == 0) {
                    const uint32_t dst = isMax ? to - 1 : from;
                    const uint32_t t = idx[dst];
                    idx[dst] = idx[pos];
                    idx[pos] = t;
                }
                __syncthreads();
                splitPosition = extreme;
                n1 = isMax ? to - 1 : from + 1;
                sliding = true;
            }
            hi1[splitIdx] = splitPosition;
            lo2[splitIdx] = splitPosition;
        } else {
            n1 = (from + to) >> 1;
            if (!degenerated && threadIdx.x == 0) {
                NthCtx c{ idx, pv, splitIdx };
                nthElement(c, long(from), long(n1), long(to));
            }
            __syncthreads();
            const double x = pv.val(idx[n1], splitIdx);
            hi1[splitIdx] = x;
            lo2[splitIdx] = x;
        }
        // inner node with two children; allocate ids and push the child segments of the next level
        if (threadIdx.x == 0) {
            uint32_t child = atomicAdd(&counters[0], 2u);
            uint32_t slot = atomicAdd(&counters[1], 2u);
            if (child + 2 > nodeCapacity || slot + 2 > segCapacity) {
                atomicOr(devError, child + 2 > nodeCapacity ? uint32_t(DEV_ERR_NODE_CAPACITY)
                                                            : uint32_t(DEV_ERR_SEGMENT_CAPACITY));
                child = 0xffffffffu;
            }
            shNode[0] = child;
            shNode[1] = slot;
        }
        __syncthreads();
        const uint32_t child = shNode[0], slot = shNode[1];
        if (threadIdx.x == 0 && child != 0xffffffffu) {
            BhNodeGeom& g = geom[node];
            g.left = int32_t(child);
            g.right = int32_t(child + 1);
            g.from = from;
            g.to = to;
            const int lvl = g.level;
            geom[child].parent = node;
            geom[child].level = lvl + 1;
            geom[child + 1].parent = node;
            geom[child + 1].level = lvl + 1;
            const uint32_t next = sliding ? sg.sliding + 1 : 0;
            BhSegment l, r;
            l.from = from;
            l.to = n1;
            l.node = int32_t(child);
            l.sliding = next;
            r.from = n1;
            r.to = to;
            r.node = int32_t(child + 1);
            r.sliding = next;
            for (int d = 0; d < 3; ++d) {
                l.lo[d] = lo1[d];
                l.hi[d] = hi1[d];
                r.lo[d] = lo2[d];
                r.hi[d] = hi2[d];
            }
            segOut[slot] = l;
            segOut[slot + 1] = r;
            atomicMax(&counters[4], max(n1 - from, to - n1));
        }
        __syncthreads();
    }
}

// The same split for segments of at most WARP_SEGMENT elements (the deep levels, tens of thousands of small
// segments): one warp per segment, warp ballots and shuffles instead of block scans and barriers. The
// partition, the sliding-midpoint moves and the child segments are identical to splitLevelKernel's.
constexpr uint32_t WARP_SEGMENT = 1024;
constexpr int SPLIT_WARP_THREADS = 128;

__device__ __forceinline__ void warpArgExtreme(unsigned long long& val, uint32_t& pos, bool isMax) {
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long ov = __shfl_xor_sync(0xffffffffu, val, off);
        const uint32_t op = __shfl_xor_sync(0xffffffffu, pos, off);
        const bool better = isMax ? (ov > val || (ov == val && op < pos)) : (ov < val || (ov == val && op < pos));
        if (better) {
            val = ov;
            pos = op;
        }
    }
}

// nInDev: when not null, the segment count of the level is read from the device (batched deep levels)
__global__ void __launch_bounds__(SPLIT_WARP_THREADS) splitWarpKernel(PosView pv, uint32_t* idx, uint32_t* posB,
    uint32_t* posS, const BhSegment* segIn, uint32_t nIn, const uint32_t* nInDev, BhSegment* segOut,
    BhNodeGeom* geom, uint32_t* counters, uint32_t* leaves, uint32_t leafSize, uint32_t nodeCapacity,
    uint32_t segCapacity, uint32_t* devError, uint32_t maxSize) {
    if (nInDev) {
        nIn = *nInDev;
    }
    const int lane = threadIdx.x & 31;
    const uint32_t warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nWarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned below = (1u << lane) - 1u;
    for (uint32_t sidx = warpGlobal; sidx < nIn; sidx += nWarps) {
        const BhSegment sg = segIn[sidx];
        const uint32_t from = sg.from, to = sg.to;
        const int node = sg.node;
        if (to - from > maxSize) {
            continue;
        }
        if (to - from <= leafSize) {
            // KdTree::addLeaf: tight box of the leaf's points (min / max are exact in any order)
            double lo[3] = { DBL_MAX, DBL_MAX, DBL_MAX }, hi[3] = { -DBL_MAX, -DBL_MAX, -DBL_MAX };
            for (uint32_t k = from + lane; k < to; k += 32) {
                const dbl4 p = pv.r[idx[k]];
                const double x[3] = { p.x, p.y, p.z };
                for (int d = 0; d < 3; ++d) {
                    lo[d] = fmin(lo[d], x[d]);
                    hi[d] = fmax(hi[d], x[d]);
                }
            }
            for (int off = 16; off > 0; off >>= 1) {
                for (int d = 0; d < 3; ++d) {
                    lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
                    hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
                }
            }
            if (lane == 0) {
                BhNodeGeom& g = geom[node];
                for (int d = 0; d < 3; ++d) {
                    g.lo[d] = lo[d];
                    g.hi[d] = hi[d];
                }
                g.left = -1;
                g.right = -1;
                g.from = from;
                g.to = to;
                const uint32_t slot = atomicAdd(&counters[2], 1u);
                leaves[slot] = uint32_t(node);
            }
            continue;
        }
        double boxSize[3];
        for (int d = 0; d < 3; ++d) {
            boxSize[d] = sg.hi[d] - sg.lo[d];
        }
        int splitIdx = argMax3(boxSize);
        bool diff[3] = { false, false, false };
        {
            const uint32_t il = idx[to - 1];
            const dbl4 pl = pv.r[il];
            const unsigned long long last[3] = { orderKey(pl.x), orderKey(pl.y), orderKey(pl.z) };
            for (uint32_t k = from + lane; k < to; k += 32) {
                const dbl4 p = pv.r[idx[k]];
                const unsigned long long x[3] = { orderKey(p.x), orderKey(p.y), orderKey(p.z) };
                for (int d = 0; d < 3; ++d) {
                    diff[d] = diff[d] || (x[d] != last[d]);
                }
            }
        }
        bool nonSingular[3];
        for (int d = 0; d < 3; ++d) {
            nonSingular[d] = __any_sync(0xffffffffu, diff[d]);
        }
        bool degenerated = false;
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
        double splitPosition = 0.5 * (sg.lo[splitIdx] + sg.hi[splitIdx]);
        uint32_t n1;
        bool sliding = false;
        double lo1[3], hi1[3], lo2[3], hi2[3];
        for (int d = 0; d < 3; ++d) {
            lo1[d] = lo2[d] = sg.lo[d];
            hi1[d] = hi2[d] = sg.hi[d];
        }
        if (sg.sliding <= 5 && !degenerated) {
            const unsigned long long splitKey = orderKey(splitPosition);
            uint32_t nB = 0, nS = 0;
            for (uint32_t k0 = from; k0 < to; k0 += 32) {
                const uint32_t k = k0 + lane;
                bool isB = false, isS = false;
                if (k < to) {
                    const unsigned long long x = pv.key(idx[k], splitIdx);
                    isB = x > splitKey;
                    isS = x < splitKey;
                }
                const unsigned mB = __ballot_sync(0xffffffffu, isB), mS = __ballot_sync(0xffffffffu, isS);
                if (isB) {
                    posB[from + nB + __popc(mB & below)] = k;
                }
                if (isS) {
                    posS[from + nS + __popc(mS & below)] = k;
                }
                nB += __popc(mB);
                nS += __popc(mS);
            }
            __syncwarp();
            const uint32_t m = min(nB, nS);
            uint32_t cntLocal = 0;
            for (uint32_t k = lane; k < m; k += 32) {
                cntLocal += (posB[from + k] < posS[from + nS - 1 - k]) ? 1u : 0u;
            }
            const uint32_t K = __reduce_add_sync(0xffffffffu, cntLocal);
            for (uint32_t k = lane; k < K; k += 32) {
                const uint32_t a = posB[from + k], b = posS[from + nS - 1 - k];
                const uint32_t t = idx[a];
                idx[a] = idx[b];
                idx[b] = t;
            }
            __syncwarp();
            uint32_t n1b = K < nB ? posB[from + K] : to;
            if (K >= 1) {
                n1b = min(n1b, posS[from + nS - K]);
            }
            n1 = n1b;
            if (n1 == from || n1 == to) {
                const bool isMax = (n1 == to);
                unsigned long long val = isMax ? 0ull : ~0ull;
                uint32_t pos = 0xffffffffu;
                for (uint32_t k = from + lane; k < to; k += 32) {
                    const unsigned long long x = pv.key(idx[k], splitIdx);
                    const bool better = isMax ? (x > val || (x == val && k < pos)) : (x < val || (x == val && k < pos));
                    if (better) {
                        val = x;
                        pos = k;
                    }
                }
                warpArgExtreme(val, pos, isMax);
                const double extreme = pv.val(idx[pos], splitIdx);
                __syncwarp();
                if (lane == 0) {
                    const uint32_t dst = isMax ? to - 1 : from;
                    const uint32_t t = idx[dst];
                    idx[dst] = idx[pos];
                    idx[pos] = t;
                }
                __syncwarp();
                splitPosition = extreme;
                n1 = isMax ? to - 1 : from + 1;
                sliding = true;
            }
            hi1[splitIdx] = splitPosition;
            lo2[splitIdx] = splitPosition;
        } else {
            n1 = (from + to) >> 1;
            if (!degenerated && lane == 0) {
                NthCtx c{ idx, pv, splitIdx };
                nthElement(c, long(from), long(n1), long(to));
            }
            __syncwarp();
            const double x = pv.val(idx[n1], splitIdx);
            hi1[splitIdx] = x;
            lo2[splitIdx] = x;
        }
        if (lane == 0) {
            uint32_t child = atomicAdd(&counters[0], 2u);
            const uint32_t slot = atomicAdd(&counters[1], 2u);
            if (child + 2 > nodeCapacity || slot + 2 > segCapacity) {
                atomicOr(devError, child + 2 > nodeCapacity ? uint32_t(DEV_ERR_NODE_CAPACITY)
                                                            : uint32_t(DEV_ERR_SEGMENT_CAPACITY));
                child = 0xffffffffu;
            }
            if (child != 0xffffffffu) {
                BhNodeGeom& g = geom[node];
                g.left = int32_t(child);
                g.right = int32_t(child + 1);
                g.from = from;
                g.to = to;
                const int lvl = g.level;
                geom[child].parent = node;
                geom[child].level = lvl + 1;
                geom[child + 1].parent = node;
                geom[child + 1].level = lvl + 1;
                const uint32_t next = sliding ? sg.sliding + 1 : 0;
                BhSegment l, r;
                l.from = from;
                l.to = n1;
                l.node = int32_t(child);
                l.sliding = next;
                r.from = n1;
                r.to = to;
                r.node = int32_t(child + 1);
                r.sliding = next;
                for (int d = 0; d < 3; ++d) {
                    l.lo[d] = lo1[d];
                    l.hi[d] = hi1[d];
                    r.lo[d] = lo2[d];
                    r.hi[d] = hi2[d];
                }
                segOut[slot] = l;
                segOut[slot + 1] = r;
                atomicMax(&counters[4], max(n1 - from, to - n1));
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------------------------------
// multi-CTA split of large segments (same partition as splitLevelKernel, spread over chunks of CHUNK
// elements): A chunk statistics for the three candidate dimensions -> B per-segment decision and chunk
// offsets -> E global ranks of the elements above / below the split -> F pair count K, sliding midpoint,
// nth_element, child segments -> G the K swaps of the two-pointer partition.
// ---------------------------------------------------------------------------------------------------------

__global__ void chunkListKernel(const BhSegment* __restrict__ segIn, uint32_t nIn, uint32_t maxSize,
    uint32_t* counters, BhChunk* chunks, BhSegWork* work, uint32_t chunkCapacity, uint32_t* devError) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < nIn; s += gridDim.x * blockDim.x) {
        const uint32_t len = segIn[s].to - segIn[s].from;
        if (len <= maxSize) {
            continue;
        }
        const uint32_t nc = (len + BH_CHUNK - 1) / BH_CHUNK;
        const uint32_t c0 = atomicAdd(&counters[3], nc);
        if (c0 + nc > chunkCapacity) {
            atomicOr(devError, uint32_t(DEV_ERR_SEGMENT_CAPACITY));
            continue;
        }
        for (uint32_t k = 0; k < nc; ++k) {
            chunks[c0 + k].seg = s;
            chunks[c0 + k].index = k;
            chunks[c0 + k].first = c0;
            chunks[c0 + k].count = nc;
        }
    }
    (void)work;
}

__device__ __forceinline__ bool betterArg(unsigned long long v, uint32_t p, unsigned long long bv, uint32_t bp,
    bool isMax) {
    return isMax ? (v > bv || (v == bv && p < bp)) : (v < bv || (v == bv && p < bp));
}

// End of a batched deep level: the node count at the start of the next level and its segment count go to
// levelInfo[next] (2 words each), and the per-level counters are cleared. One thread.
__global__ void levelEndKernel(uint32_t* counters, uint32_t* levelInfo, uint32_t next) {
    levelInfo[2 * next] = counters[0];
    levelInfo[2 * next + 1] = counters[1];
    counters[1] = 0;
    counters[4] = 0;
}

__global__ void setWordKernel(uint32_t* p, uint32_t v) {
    *p = v;
}

__global__ void __launch_bounds__(BUILD_THREADS) chunkStatsKernel(PosView pv, const uint32_t* __restrict__ idx,
    const BhSegment* __restrict__ segIn, const BhChunk* __restrict__ chunks, BhChunkStats* stats) {
    __shared__ uint32_t shScan[32];
    __shared__ unsigned long long shV[32];
    __shared__ uint32_t shP[32];
    const BhChunk ch = chunks[blockIdx.x];
    const BhSegment sg = segIn[ch.seg];
    const uint32_t from = sg.from + ch.index * BH_CHUNK;
    const uint32_t to = min(sg.to, from + BH_CHUNK);
    unsigned long long center[3], last[3];
    const uint32_t il = idx[sg.to - 1];
    for (int d = 0; d < 3; ++d) {
        center[d] = orderKey(0.5 * (sg.lo[d] + sg.hi[d]));
        last[d] = pv.key(il, d);
    }
    uint32_t nb[3] = { 0, 0, 0 }, ns[3] = { 0, 0, 0 };
    bool diff[3] = { false, false, false };
    unsigned long long mnv[3] = { ~0ull, ~0ull, ~0ull }, mxv[3] = { 0ull, 0ull, 0ull };
    uint32_t mnp[3] = { 0xffffffffu, 0xffffffffu, 0xffffffffu }, mxp[3] = { 0xffffffffu, 0xffffffffu, 0xffffffffu };
    for (uint32_t k = from + threadIdx.x; k < to; k += BUILD_THREADS) {
        const dbl4 p = pv.r[idx[k]];
        const unsigned long long x[3] = { orderKey(p.x), orderKey(p.y), orderKey(p.z) };
        for (int d = 0; d < 3; ++d) {
            nb[d] += x[d] > center[d] ? 1u : 0u;
            ns[d] += x[d] < center[d] ? 1u : 0u;
            diff[d] = diff[d] || (x[d] != last[d]);
            if (betterArg(x[d], k, mnv[d], mnp[d], false)) {
                mnv[d] = x[d];
                mnp[d] = k;
            }
            if (betterArg(x[d], k, mxv[d], mxp[d], true)) {
                mxv[d] = x[d];
                mxp[d] = k;
            }
        }
    }
    BhChunkStats out;
    for (int d = 0; d < 3; ++d) {
        out.nb[d] = blockSum(nb[d], shScan);
        out.ns[d] = blockSum(ns[d], shScan);
        out.diff[d] = __syncthreads_or(diff[d] ? 1 : 0) ? 1u : 0u;
        unsigned long long v = mnv[d];
        uint32_t q = mnp[d];
        blockArgExtreme(v, q, false, shV, shP);
        out.minv[d] = v;
        out.minp[d] = q;
        v = mxv[d];
        q = mxp[d];
        blockArgExtreme(v, q, true, shV, shP);
        out.maxv[d] = v;
        out.maxp[d] = q;
    }
    if (threadIdx.x == 0) {
        stats[blockIdx.x] = out;
    }
}

// one warp per large segment (the warp of its first chunk): split dimension and mode, chunk offsets of the
// elements above / below the box centre (warp scan), extremes of the split coordinate
__global__ void segDecideKernel(const BhSegment* __restrict__ segIn, const BhChunk* __restrict__ chunks,
    uint32_t nChunks, const BhChunkStats* __restrict__ stats, uint32_t* chunkOffB, uint32_t* chunkOffS,
    BhSegWork* work) {
    const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nChunks || chunks[c].index != 0) {
        return;
    }
    const BhChunk ch = chunks[c];
    const BhSegment sg = segIn[ch.seg];
    bool anyDiff[3] = { false, false, false };
    for (uint32_t k = lane; k < ch.count; k += 32) {
        for (int d = 0; d < 3; ++d) {
            anyDiff[d] = anyDiff[d] || stats[ch.first + k].diff[d] != 0;
        }
    }
    bool nonSingular[3];
    for (int d = 0; d < 3; ++d) {
        nonSingular[d] = __any_sync(0xffffffffu, anyDiff[d]);
    }
    double boxSize[3];
    for (int d = 0; d < 3; ++d) {
        boxSize[d] = sg.hi[d] - sg.lo[d];
    }
    int splitIdx = argMax3(boxSize);
    bool degenerated = false;
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
    uint32_t ob = 0, os = 0;
    unsigned long long mnv = ~0ull, mxv = 0ull;
    uint32_t mnp = 0xffffffffu, mxp = 0xffffffffu;
    for (uint32_t k0 = 0; k0 < ch.count; k0 += 32) {
        const uint32_t k = k0 + lane;
        uint32_t nb = 0, ns = 0;
        if (k < ch.count) {
            const BhChunkStats& st = stats[ch.first + k];
            nb = st.nb[splitIdx];
            ns = st.ns[splitIdx];
            if (betterArg(st.minv[splitIdx], st.minp[splitIdx], mnv, mnp, false)) {
                mnv = st.minv[splitIdx];
                mnp = st.minp[splitIdx];
            }
            if (betterArg(st.maxv[splitIdx], st.maxp[splitIdx], mxv, mxp, true)) {
                mxv = st.maxv[splitIdx];
                mxp = st.maxp[splitIdx];
            }
        }
        // inclusive scans of the counts across the lanes
        uint32_t xb = nb, xs = ns;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t yb = __shfl_up_sync(0xffffffffu, xb, off), ys = __shfl_up_sync(0xffffffffu, xs, off);
            if (lane >= off) {
                xb += yb;
                xs += ys;
            }
        }
        if (k < ch.count) {
            chunkOffB[ch.first + k] = ob + xb - nb;
            chunkOffS[ch.first + k] = os + xs - ns;
        }
        ob += __shfl_sync(0xffffffffu, xb, 31);
        os += __shfl_sync(0xffffffffu, xs, 31);
    }
    warpArgExtreme(mnv, mnp, false);
    warpArgExtreme(mxv, mxp, true);
    if (lane == 0) {
        BhSegWork w;
        w.splitIdx = splitIdx;
        w.mode = degenerated ? 2 : (sg.sliding <= 5 ? 0 : 1);
        w.nB = ob;
        w.nS = os;
        w.minv = mnv;
        w.minp = mnp;
        w.maxv = mxv;
        w.maxp = mxp;
        w.K = 0;
        work[ch.seg] = w;
    }
}

__global__ void __launch_bounds__(BUILD_THREADS) chunkRanksKernel(PosView pv, const uint32_t* __restrict__ idx,
    const BhSegment* __restrict__ segIn, const BhChunk* __restrict__ chunks, const uint32_t* __restrict__ chunkOffB,
    const uint32_t* __restrict__ chunkOffS, const BhSegWork* __restrict__ work, uint32_t* posB, uint32_t* posS) {
    __shared__ uint32_t shScan[32];
    const BhChunk ch = chunks[blockIdx.x];
    const BhSegment sg = segIn[ch.seg];
    const BhSegWork w = work[ch.seg];
    if (w.mode != 0) {
        return;
    }
    const int d = w.splitIdx;
    const unsigned long long split = orderKey(0.5 * (sg.lo[d] + sg.hi[d]));
    const uint32_t from = sg.from + ch.index * BH_CHUNK;
    const uint32_t to = min(sg.to, from + BH_CHUNK);
    uint32_t baseB = sg.from + chunkOffB[blockIdx.x], baseS = sg.from + chunkOffS[blockIdx.x];
    for (uint32_t k0 = from; k0 < to; k0 += BUILD_THREADS) {
        const uint32_t k = k0 + threadIdx.x;
        bool isB = false, isS = false;
        if (k < to) {
            const unsigned long long x = pv.key(idx[k], d);
            isB = x > split;
            isS = x < split;
        }
        uint32_t totB, totS;
        const uint32_t rb = blockExclusiveScan(isB ? 1u : 0u, totB, shScan);
        const uint32_t rs = blockExclusiveScan(isS ? 1u : 0u, totS, shScan);
        if (isB) {
            posB[baseB + rb] = k;
        }
        if (isS) {
            posS[baseS + rs] = k;
        }
        baseB += totB;
        baseS += totS;
    }
}

// one thread per large segment: the pair count K of the two-pointer partition, the split and the children
__global__ void segFinishKernel(PosView pv, uint32_t* idx, const uint32_t* __restrict__ posB,
    const uint32_t* __restrict__ posS, const BhSegment* __restrict__ segIn, const BhChunk* __restrict__ chunks,
    uint32_t nChunks, BhSegWork* work, BhSegment* segOut, BhNodeGeom* geom, uint32_t* counters,
    uint32_t nodeCapacity, uint32_t segCapacity, uint32_t* devError) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nChunks || chunks[c].index != 0) {
        return;
    }
    const uint32_t s = chunks[c].seg;
    const BhSegment sg = segIn[s];
    BhSegWork w = work[s];
    const uint32_t from = sg.from, to = sg.to;
    const int d = w.splitIdx;
    double splitPosition = 0.5 * (sg.lo[d] + sg.hi[d]);
    uint32_t n1;
    bool sliding = false;
    double cut;
    if (w.mode == 0) {
        const uint32_t nB = w.nB, nS = w.nS;
        // first k with posB[k] >= posS[nS - 1 - k] (the predicate is monotone in k)
        uint32_t lo = 0, hi = min(nB, nS);
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (posB[from + mid] < posS[from + nS - 1 - mid]) {
                lo = mid + 1;
            } else {
                hi = mid;
            }
        }
        const uint32_t K = lo;
        w.K = K;
        n1 = K < nB ? posB[from + K] : to;
        if (K >= 1) {
            n1 = min(n1, posS[from + nS - K]);
        }
        if (n1 == from || n1 == to) {
            const bool isMax = (n1 == to);
            const uint32_t dst = isMax ? to - 1 : from;
            const uint32_t src = isMax ? w.maxp : w.minp;
            splitPosition = pv.val(idx[src], d);
            const uint32_t t = idx[dst];
            idx[dst] = idx[src];
            idx[src] = t;
            n1 = isMax ? to - 1 : from + 1;
            sliding = true;
        }
        cut = splitPosition;
    } else {
        w.K = 0;
        n1 = (from + to) >> 1;
        if (w.mode == 1) {
            NthCtx ctx{ idx, pv, d };
            nthElement(ctx, long(from), long(n1), long(to));
        }
        cut = pv.val(idx[n1], d);
    }
    work[s] = w;
    uint32_t child = atomicAdd(&counters[0], 2u);
    const uint32_t slot = atomicAdd(&counters[1], 2u);
    if (child + 2 > nodeCapacity || slot + 2 > segCapacity) {
        atomicOr(devError, child + 2 > nodeCapacity ? uint32_t(DEV_ERR_NODE_CAPACITY) : uint32_t(DEV_ERR_SEGMENT_CAPACITY));
        return;
    }
    BhNodeGeom& g = geom[sg.node];
    g.left = int32_t(child);
    g.right = int32_t(child + 1);
    g.from = from;
    g.to = to;
    const int lvl = g.level;
    geom[child].parent = sg.node;
    geom[child].level = lvl + 1;
    geom[child + 1].parent = sg.node;
    geom[child + 1].level = lvl + 1;
    const uint32_t next = sliding ? sg.sliding + 1 : 0;
    BhSegment l = sg, r = sg;
    l.to = n1;
    l.node = int32_t(child);
    l.sliding = next;
    l.hi[d] = cut;
    r.from = n1;
    r.node = int32_t(child + 1);
    r.sliding = next;
    r.lo[d] = cut;
    segOut[slot] = l;
    segOut[slot + 1] = r;
    atomicMax(&counters[4], max(n1 - from, to - n1));
}

__global__ void chunkSwapKernel(uint32_t* idx, const uint32_t* __restrict__ posB, const uint32_t* __restrict__ posS,
    const BhSegment* __restrict__ segIn, const BhChunk* __restrict__ chunks, const BhSegWork* __restrict__ work) {
    const BhChunk ch = chunks[blockIdx.x];
    const BhSegWork w = work[ch.seg];
    const uint32_t from = segIn[ch.seg].from;
    const uint32_t k0 = ch.index * BH_CHUNK;
    const uint32_t k1 = min(w.K, k0 + BH_CHUNK);
    for (uint32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const uint32_t a = posB[from + k], b = posS[from + w.nS - 1 - k];
        const uint32_t t = idx[a];
        idx[a] = idx[b];
        idx[b] = t;
    }
}

// BarnesHut::buildLeaf (core/gravity/BarnesHut.cpp:376-437), geometry part: mass, centre of mass and opening
// radius of the leaf in FP64, summed in the leaf's particle order (the walk's decisions depend on these bits).
// Returns false for a single-particle leaf (no moments beyond the mass).
__device__ bool buildLeafGeom(const dbl4* __restrict__ r, const double* __restrict__ m, double G,
    const uint32_t* __restrict__ idx, double thetaInv, BhNodeGeom& g, double& m0) {
    const uint32_t cnt = g.to - g.from;
    if (cnt == 1) {
        const uint32_t i = idx[g.from];
        const dbl4 p = r[i];
        g.com[0] = p.x;
        g.com[1] = p.y;
        g.com[2] = p.z;
        m0 = G * m[i];
        g.r_open = 0.;
        return false;
    }
    double cx = 0., cy = 0., cz = 0., mLeaf = 0.;
    for (uint32_t k = g.from; k < g.to; ++k) {
        const uint32_t i = idx[k];
        const dbl4 p = r[i];
        const double mi = G * m[i];
        cx += mi * p.x;
        cy += mi * p.y;
        cz += mi * p.z;
        mLeaf += mi;
    }
    cx /= mLeaf;
    cy /= mLeaf;
    cz /= mLeaf;
    g.com[0] = cx;
    g.com[1] = cy;
    g.com[2] = cz;
    const double rmx = fmax(cx - g.lo[0], g.hi[0] - cx), rmy = fmax(cy - g.lo[1], g.hi[1] - cy),
                 rmz = fmax(cz - g.lo[2], g.hi[2] - cz);
    g.r_open = 2. / sqrt(3.) * thetaInv * sqrt(rmx * rmx + rmy * rmy + rmz * rmz);
    m0 = mLeaf;
    return true;
}

// reduced (traceless) multipoles from the raw second and third moments (computeReducedMultipole,
// core/gravity/Moments.h:90-111)
template <typename T>
__device__ __forceinline__ void reduceMoments(const T M2[6], const T M3[10], T q2[6], T q3[10]) {
    const T tr = M2[0] + M2[3] + M2[5];
    for (int a = 0; a < 3; ++a) {
        for (int b = a; b < 3; ++b) {
            q2[i2(a, b)] = M2[i2(a, b)] + (a == b ? tr : T(0)) * T(-1. / 3.);
        }
    }
    T T1[3];
    for (int k = 0; k < 3; ++k) {
        T1[k] = M3[i3(0, 0, k)] + M3[i3(1, 1, k)] + M3[i3(2, 2, k)];
    }
    for (int a = 0; a < 3; ++a) {
        for (int b = a; b < 3; ++b) {
            for (int c = b; c < 3; ++c) {
                const T perm = (a == b ? T1[c] : T(0)) + (b == c ? T1[a] : T(0)) + (c == a ? T1[b] : T(0));
                q3[i3(a, b, c)] = M3[i3(a, b, c)] + perm * T(-1. / 5.);
            }
        }
    }
}

// moments of a leaf about its centre of mass: T = double for the FP64 walk, float for the mixed walk (the
// separations are formed in FP64 and rounded once)
template <typename T>
__device__ void leafMoments(const dbl4* __restrict__ r, const double* __restrict__ m, double G,
    const uint32_t* __restrict__ idx, const BhNodeGeom& g, T q2[6], T q3[10]) {
    T M2[6] = { 0, 0, 0, 0, 0, 0 }, M3[10] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0 };
    for (uint32_t k = g.from; k < g.to; ++k) {
        const uint32_t i = idx[k];
        const dbl4 p = r[i];
        const T mi = T(G * m[i]);
        const T d[3] = { T(p.x - g.com[0]), T(p.y - g.com[1]), T(p.z - g.com[2]) };
        for (int a = 0; a < 3; ++a) {
            for (int b = a; b < 3; ++b) {
                M2[i2(a, b)] += (d[a] * d[b]) * mi;
                for (int c = b; c < 3; ++c) {
                    M3[i3(a, b, c)] += (d[a] * d[b] * d[c]) * mi;
                }
            }
        }
    }
    reduceMoments(M2, M3, q2, q3);
}

// BarnesHut::buildLeaf with FP64 moments, one thread per leaf
__device__ void buildLeaf(const dbl4* __restrict__ r, const double* __restrict__ m, double G,
    const uint32_t* __restrict__ idx, double thetaInv, BhNodeGeom& g, BhNodeMoments& mo) {
    for (int k = 0; k < 6; ++k) {
        mo.q2[k] = 0.;
    }
    for (int k = 0; k < 10; ++k) {
        mo.q3[k] = 0.;
    }
    mo.pad = 0.;
    if (buildLeafGeom(r, m, G, idx, thetaInv, g, mo.m0)) {
        leafMoments(r, m, G, idx, g, mo.q2, mo.q3);
    }
}

// parallelAxisTheorem for orders 2 and 3 (core/gravity/Moments.h:182-295): the child's moments (mass Q,
// reduced cq2, cq3) moved by d = child centre - new centre, accumulated into (q2, q3)
template <typename T>
__device__ void shiftAdd(T Q, const T cq2[6], const T cq3[10], const T d[3], T q2[6], T q3[10]) {
    const T dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    T Qd[3];
    for (int k = 0; k < 3; ++k) {
        Qd[k] = cq2[i2(k, 0)] * d[0] + cq2[i2(k, 1)] * d[1] + cq2[i2(k, 2)] * d[2];
    }
    for (int a = 0; a < 3; ++a) {
        for (int b = a; b < 3; ++b) {
            const T f2 = d[a] * d[b] + (a == b ? dd : T(0)) * T(-1. / 3.);
            q2[i2(a, b)] += cq2[i2(a, b)] + f2 * Q;
            for (int cc = b; cc < 3; ++cc) {
                const T perm = (a == b ? d[cc] : T(0)) + (b == cc ? d[a] : T(0)) + (cc == a ? d[b] : T(0));
                const T f3 = d[a] * d[b] * d[cc] + perm * dd * T(-1. / 5.);
                const T pq = cq2[i2(a, b)] * d[cc] + cq2[i2(b, cc)] * d[a] + cq2[i2(cc, a)] * d[b];
                const T t2 = (a == b ? Qd[cc] : T(0)) + (a == cc ? Qd[b] : T(0)) + (b == cc ? Qd[a] : T(0));
                q3[i3(a, b, cc)] += cq3[i3(a, b, cc)] + f3 * Q + pq + T(-2. / 5.) * t2;
            }
        }
    }
}

// BarnesHut::buildInner (core/gravity/BarnesHut.cpp:439-489), geometry part: box, mass, centre of mass and
// opening radius from the two children (FP64). Returns false for a massless node.
__device__ bool buildInnerGeom(double thetaInv, BhNodeGeom& g, const BhNodeGeom& gl, const BhNodeGeom& gr, double ml,
    double mr, double& m0) {
    for (int d = 0; d < 3; ++d) {
        g.lo[d] = fmin(gl.lo[d], gr.lo[d]);
        g.hi[d] = fmax(gl.hi[d], gr.hi[d]);
    }
    const double mt = ml + mr;
    if (mt == 0.) {
        m0 = 0.;
        g.com[0] = g.com[1] = g.com[2] = 0.;
        g.r_open = 0.;
        return false;
    }
    for (int d = 0; d < 3; ++d) {
        g.com[d] = (ml * gl.com[d] + mr * gr.com[d]) / mt;
    }
    const double rmx = fmax(g.com[0] - g.lo[0], g.hi[0] - g.com[0]);
    const double rmy = fmax(g.com[1] - g.lo[1], g.hi[1] - g.com[1]);
    const double rmz = fmax(g.com[2] - g.lo[2], g.hi[2] - g.com[2]);
    g.r_open = 2. / sqrt(3.) * thetaInv * sqrt(rmx * rmx + rmy * rmy + rmz * rmz);
    m0 = mt;
    return true;
}

// BarnesHut::buildInner with FP64 moments (left child first)
__device__ void buildInner(double thetaInv, BhNodeGeom& g, const BhNodeGeom& gl, const BhNodeGeom& gr,
    const BhNodeMoments& ml, const BhNodeMoments& mr, BhNodeMoments& mo) {
    for (int k = 0; k < 6; ++k) {
        mo.q2[k] = 0.;
    }
    for (int k = 0; k < 10; ++k) {
        mo.q3[k] = 0.;
    }
    mo.pad = 0.;
    if (!buildInnerGeom(thetaInv, g, gl, gr, ml.m0, mr.m0, mo.m0)) {
        return;
    }
    const double dl[3] = { gl.com[0] - g.com[0], gl.com[1] - g.com[1], gl.com[2] - g.com[2] };
    shiftAdd(ml.m0, ml.q2, ml.q3, dl, mo.q2, mo.q3);
    const double dr[3] = { gr.com[0] - g.com[0], gr.com[1] - g.com[1], gr.com[2] - g.com[2] };
    shiftAdd(mr.m0, mr.q2, mr.q3, dr, mo.q2, mo.q3);
}

// loads that bypass L1 (the sibling subtree was written by another SM during this launch)
template <typename T>
__device__ __forceinline__ T loadCG(const T* p) {
    static_assert(sizeof(T) % 8 == 0, "8-byte multiple");
    T out;
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(p);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&out);
    for (size_t k = 0; k < sizeof(T) / 8; ++k) {
        dst[k] = __ldcg(src + k);
    }
    return out;
}

// FP32 reduced moments of a node in the mixed walk's node record (groups NF_MOM .. NF_MOM + 3)
__device__ __forceinline__ void writeMomentsF(float* nodef, int node, const float q2[6], const float q3[10]) {
    float4* o = reinterpret_cast<float4*>(nodef) + size_t(node) * NODEF4 + NF_MOM;
    o[0] = make_float4(q2[0], q2[1], q2[2], q2[3]);
    o[1] = make_float4(q2[4], q2[5], q3[0], q3[1]);
    o[2] = make_float4(q3[2], q3[3], q3[4], q3[5]);
    o[3] = make_float4(q3[6], q3[7], q3[8], q3[9]);
}

__device__ __forceinline__ void readMomentsF(const float* nodef, int node, float q2[6], float q3[10]) {
    const float4* o = reinterpret_cast<const float4*>(nodef) + size_t(node) * NODEF4 + NF_MOM;
    const float4 a = __ldcg(o), b = __ldcg(o + 1), c = __ldcg(o + 2), d = __ldcg(o + 3);
    q2[0] = a.x, q2[1] = a.y, q2[2] = a.z, q2[3] = a.w, q2[4] = b.x, q2[5] = b.y;
    q3[0] = b.z, q3[1] = b.w, q3[2] = c.x, q3[3] = c.y, q3[4] = c.z, q3[5] = c.w;
    q3[6] = d.x, q3[7] = d.y, q3[8] = d.z, q3[9] = d.w;
}

// All moments in one launch, bottom-up: one thread per leaf forms the leaf's moments, then climbs; at each
// inner node the thread that arrives second (atomic counter per node) forms the node from its two finished
// children, the first one stops. Nothing waits, so the launch always completes; every node gets the same
// values in any arrival order (children combined left then right). Mixed: the geometry (mass, centre of
// mass, opening radius, box) is formed in FP64 exactly as for the FP64 walk, so both walks take the same
// decisions, while the reduced moments, which the mixed walk evaluates in FP32, are formed in FP32 directly
// into its node records.
template <bool Mixed>
__global__ void momentsUpKernel(const dbl4* __restrict__ r, const double* __restrict__ m, double G,
    const uint32_t* __restrict__ idx, double thetaInv, BhNodeGeom* geom, BhNodeMoments* mom, float* nodef,
    const uint32_t* __restrict__ leaves, uint32_t nLeaves, uint32_t* visits) {
    const uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= nLeaves) {
        return;
    }
    const int node = int(leaves[li]);
    int parent;
    {
        BhNodeGeom g = geom[node];
        if (Mixed) {
            double m0;
            float q2[6] = { 0, 0, 0, 0, 0, 0 }, q3[10] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0 };
            if (buildLeafGeom(r, m, G, idx, thetaInv, g, m0)) {
                leafMoments(r, m, G, idx, g, q2, q3);
            }
            mom[node].m0 = m0;
            writeMomentsF(nodef, node, q2, q3);
        } else {
            BhNodeMoments mo;
            buildLeaf(r, m, G, idx, thetaInv, g, mo);
            mom[node] = mo;
        }
        geom[node] = g;
        parent = g.parent;
    }
    while (parent >= 0) {
        __threadfence();
        if (atomicAdd(&visits[parent], 1u) == 0) {
            return;
        }
        __threadfence();
        BhNodeGeom g = loadCG(&geom[parent]);
        const BhNodeGeom gl = loadCG(&geom[g.left]);
        const BhNodeGeom gr = loadCG(&geom[g.right]);
        if (Mixed) {
            const double ml = __ldcg(&mom[g.left].m0), mr = __ldcg(&mom[g.right].m0);
            double m0;
            float q2[6] = { 0, 0, 0, 0, 0, 0 }, q3[10] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0 };
            if (buildInnerGeom(thetaInv, g, gl, gr, ml, mr, m0)) {
                float cq2[6], cq3[10];
                readMomentsF(nodef, g.left, cq2, cq3);
                const float dl[3] = { float(gl.com[0] - g.com[0]), float(gl.com[1] - g.com[1]),
                    float(gl.com[2] - g.com[2]) };
                shiftAdd(float(ml), cq2, cq3, dl, q2, q3);
                readMomentsF(nodef, g.right, cq2, cq3);
                const float dr[3] = { float(gr.com[0] - g.com[0]), float(gr.com[1] - g.com[1]),
                    float(gr.com[2] - g.com[2]) };
                shiftAdd(float(mr), cq2, cq3, dr, q2, q3);
            }
            mom[parent].m0 = m0;
            writeMomentsF(nodef, parent, q2, q3);
        } else {
            const BhNodeMoments ml = loadCG(&mom[g.left]);
            const BhNodeMoments mr = loadCG(&mom[g.right]);
            BhNodeMoments mo;
            buildInner(thetaInv, g, gl, gr, ml, mr, mo);
            mom[parent] = mo;
        }
        geom[parent] = g;
        parent = g.parent;
    }
}

// ---------------------------------------------------------------------------------------------------------
// walk: one warp per leaf
// ---------------------------------------------------------------------------------------------------------

constexpr int WALK_THREADS = 128;

__global__ void __launch_bounds__(WALK_THREADS) walkKernel(const dbl4* __restrict__ r,
    const double* __restrict__ m, double G, const uint32_t* __restrict__ idx, const BhNodeGeom* __restrict__ geom,
    const BhNodeMoments* __restrict__ mom, const float* __restrict__ nodef, const uint32_t* __restrict__ leaves,
    uint32_t nLeaves, const double* __restrict__ lut, int kernelRadius, int order, int32_t* scratch,
    uint32_t listCap, dbl4* agrav, unsigned long long* stats, uint32_t* devError) {
    __shared__ int32_t pathSh[WALK_THREADS / 32][MAX_PATH];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const uint32_t warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nWarps = (gridDim.x * blockDim.x) >> 5;
    int32_t* listA = scratch + size_t(warpGlobal) * 2 * listCap;
    int32_t* listB = listA + listCap;
    int32_t* path = pathSh[wib];
    unsigned long long nApprox = 0, nExact = 0, nPn = 0, nPp = 0;
    (void)nWarps;

    // leaves are taken from a shared counter (stats[4]) so that warps that drew cheap leaves take more
    for (;;) {
        uint32_t li = 0;
        if (lane == 0) {
            li = uint32_t(atomicAdd(&stats[4], 1ull));
        }
        li = __shfl_sync(0xffffffffu, li, 0);
        if (li >= nLeaves) {
            break;
        }
        const int leaf = int(leaves[li]);
        const BhNodeGeom lg = geom[leaf];
        const uint32_t cnt = lg.to - lg.from;
        // root path (path[0] = root ... path[depth] = leaf)
        int depth = 0;
        if (lane == 0) {
            int d = 0, nd = leaf;
            while (geom[nd].parent >= 0 && d < MAX_PATH - 1) {
                nd = geom[nd].parent;
                ++d;
            }
            depth = d;
            nd = leaf;
            for (int k = d; k >= 0; --k) {
                path[k] = nd;
                nd = geom[nd].parent;
            }
            if (d >= MAX_PATH - 1) {
                atomicOr(devError, uint32_t(DEV_ERR_WALK_CAPACITY));
            }
        }
        depth = __shfl_sync(0xffffffffu, depth, 0);
        __syncwarp();
        const bool active = uint32_t(lane) < cnt;
        const float4* nf = reinterpret_cast<const float4*>(nodef);
        float lh[3], ll[3];
        {
            const float4 a = nodeGroup(nf, leaf, NF_COM_HI), b = nodeGroup(nf, leaf, NF_COM_LO);
            lh[0] = a.x, lh[1] = a.y, lh[2] = a.z;
            ll[0] = b.x, ll[1] = b.y, ll[2] = b.z;
        }
        uint32_t pi = 0;
        dbl4 ri = mkd4(0., 0., 0., 1.);
        if (active) {
            pi = idx[lg.from + lane];
            ri = r[pi];
        }
        double ax = 0., ay = 0., az = 0.;
        int32_t* cur = listA;
        int32_t* nxt = listB;
        uint32_t ncur = 0, nnxt = 0;
        bool overflow = false;
        for (int k = 1; k <= depth && !overflow; ++k) {
            const int ev = path[k];
            const int par = path[k - 1];
            const BhNodeGeom& pg = geom[par];
            const int sib = pg.left == ev ? pg.right : pg.left;
            WalkFrame fr;
            setFrame(fr, nf, ev, k == depth, lh, ll);
            if (lane == 0) {
                cur[ncur] = sib;
            }
            ncur += 1;
            __syncwarp();
            uint32_t pos = 0;
            while (pos < ncur) {
                const uint32_t batch = min(32u, ncur - pos);
                const uint32_t e = pos + lane;
                int node = -1, cls = CL_KEEP;
                if (uint32_t(lane) < batch) {
                    node = cur[e];
                    cls = classifyEntry(node, geom, nf, fr, lh, ll);
                }
                const unsigned mKeep = __ballot_sync(0xffffffffu, uint32_t(lane) < batch && cls == CL_KEEP);
                const unsigned mOpen = __ballot_sync(0xffffffffu, cls == CL_OPEN);
                const unsigned mPart = __ballot_sync(0xffffffffu, cls == CL_PARTICLES);
                const unsigned mNode = __ballot_sync(0xffffffffu, cls == CL_NODE);
                const unsigned below = (1u << lane) - 1u;
                const uint32_t nOpen = __popc(mOpen), nKeep = __popc(mKeep);
                if (ncur + 2 * nOpen > listCap || nnxt + nKeep > listCap) {
                    overflow = true;
                    break;
                }
                if (cls == CL_KEEP && uint32_t(lane) < batch) {
                    nxt[nnxt + __popc(mKeep & below)] = node;
                }
                if (cls == CL_OPEN) {
                    const uint32_t slot = ncur + 2 * __popc(mOpen & below);
                    cur[slot] = geom[node].left;
                    cur[slot + 1] = geom[node].right;
                }
                pos += batch;
                ncur += 2 * nOpen;
                nnxt += nKeep;
                __syncwarp();
                // exact pair terms with every particle of the listed leaves
                unsigned mp = mPart;
                while (mp) {
                    const int src = __ffs(mp) - 1;
                    mp &= mp - 1;
                    const int pn = __shfl_sync(0xffffffffu, node, src);
                    const uint32_t f0 = geom[pn].from, f1 = geom[pn].to;
                    nExact += 1;
                    nPp += uint64_t(cnt) * (f1 - f0);
                    for (uint32_t t = f0; t < f1; ++t) {
                        const uint32_t j = idx[t];
                        const dbl4 rj = r[j];
                        const double mj = G * m[j];
                        if (active) {
                            double gx, gy, gz;
                            gravGrad(rj.x - ri.x, rj.y - ri.y, rj.z - ri.z, 0.5 * (rj.w + ri.w), lut, kernelRadius,
                                gx, gy, gz);
                            ax += mj * gx;
                            ay += mj * gy;
                            az += mj * gz;
                        }
                    }
                }
                // multipole expansions
                unsigned mn = mNode;
                while (mn) {
                    const int src = __ffs(mn) - 1;
                    mn &= mn - 1;
                    const int nn = __shfl_sync(0xffffffffu, node, src);
                    nApprox += 1;
                    nPn += cnt;
                    if (active) {
                        const BhNodeGeom& ng = geom[nn];
                        evalMultipole(ri.x - ng.com[0], ri.y - ng.com[1], ri.z - ng.com[2], mom[nn], order, ax, ay, az);
                    }
                }
            }
            // the kept entries are the check list of the next ancestor
            int32_t* t = cur;
            cur = nxt;
            nxt = t;
            ncur = nnxt;
            nnxt = 0;
        }
        if (overflow) {
            if (lane == 0) {
                atomicOr(devError, uint32_t(DEV_ERR_WALK_CAPACITY));
            }
            continue;
        }
        // intra-leaf pairs
        nPp += uint64_t(cnt) * (cnt - 1);
        for (uint32_t t = lg.from; t < lg.to; ++t) {
            const uint32_t j = idx[t];
            const dbl4 rj = r[j];
            const double mj = G * m[j];
            if (active && j != pi) {
                double gx, gy, gz;
                gravGrad(rj.x - ri.x, rj.y - ri.y, rj.z - ri.z, 0.5 * (rj.w + ri.w), lut, kernelRadius, gx, gy, gz);
                ax += mj * gx;
                ay += mj * gy;
                az += mj * gz;
            }
        }
        if (active) {
            agrav[pi] = mkd4(ax, ay, az, 0.);
        }
    }
    if (lane == 0) {
        atomicAdd(&stats[0], nApprox);
        atomicAdd(&stats[1], nExact);
        atomicAdd(&stats[2], nPn);
        atomicAdd(&stats[3], nPp);
    }
}

// BarnesHut::evalImpl / evalExact (core/gravity/BarnesHut.cpp:118-175, 364-374): one thread per point
__global__ void pointsKernel(const dbl4* __restrict__ r, const double* __restrict__ m, double G,
    const uint32_t* __restrict__ idx, const BhNodeGeom* __restrict__ geom, const BhNodeMoments* __restrict__ mom,
    const double* __restrict__ lut, int kernelRadius, int order, double thetaInv, const dbl4* pts, dbl4* acc,
    uint32_t np) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) {
        return;
    }
    const dbl4 p = pts[k];
    const double thetaSqr = 1. / (thetaInv * thetaInv);
    double ax = 0., ay = 0., az = 0.;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int id = stack[--sp];
        const BhNodeGeom& g = geom[id];
        const double sx = g.hi[0] - g.lo[0], sy = g.hi[1] - g.lo[1], sz = g.hi[2] - g.lo[2];
        const double boxSizeSqr = sx * sx + sy * sy + sz * sz;
        const double cx = 0.5 * (g.lo[0] + g.hi[0]) - p.x, cy = 0.5 * (g.lo[1] + g.hi[1]) - p.y,
                     cz = 0.5 * (g.lo[2] + g.hi[2]) - p.z;
        const double boxDistSqr = cx * cx + cy * cy + cz * cz;
        const bool contains = !(p.x < g.lo[0] || p.x > g.hi[0] || p.y < g.lo[1] || p.y > g.hi[1] || p.z < g.lo[2] ||
                                p.z > g.hi[2]);
        if (!contains && boxSizeSqr > 0. && boxSizeSqr / (boxDistSqr + SPH_EPS) < thetaSqr) {
            evalMultipole(p.x - g.com[0], p.y - g.com[1], p.z - g.com[2], mom[id], order, ax, ay, az);
        } else if (g.left < 0) {
            for (uint32_t t = g.from; t < g.to; ++t) {
                const uint32_t i = idx[t];
                const dbl4 ri = r[i];
                double gx, gy, gz;
                gravGrad(ri.x - p.x, ri.y - p.y, ri.z - p.z, ri.w, lut, kernelRadius, gx, gy, gz);
                const double mi = G * m[i];
                ax += mi * gx;
                ay += mi * gy;
                az += mi * gz;
            }
        } else if (sp + 2 <= 128) {
            stack[sp++] = g.right;
            stack[sp++] = g.left;
        }
    }
    acc[k] = mkd4(ax, ay, az, 0.);
}

} // namespace

cudaError_t treeAllocate(Tree& t, uint32_t n, uint32_t leafSize) {
    const uint32_t nn = n > 0 ? n : 1;
    t.node_capacity = 2 * nn + 8;
    t.seg_capacity = nn + 8;
    // one check-list pair per resident warp: at most 64 warps on each of the 152 SMs, never more warps than
    // particles (a leaf holds at least one)
    t.walk_warps = std::min<uint32_t>(152u * 64u, (nn + 3) & ~3u);
    t.walk_capacity = 4096;
    (void)leafSize;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) {
            e = cudaMalloc(p, bytes > 0 ? bytes : 16);
        }
    };
    alloc((void**)&t.idx, nn * sizeof(uint32_t));
    alloc((void**)&t.scratch_b, nn * sizeof(uint32_t));
    alloc((void**)&t.scratch_s, nn * sizeof(uint32_t));
    alloc((void**)&t.geom, size_t(t.node_capacity) * sizeof(BhNodeGeom));
    alloc((void**)&t.mom, size_t(t.node_capacity) * sizeof(BhNodeMoments));
    alloc((void**)&t.seg[0], size_t(t.seg_capacity) * sizeof(BhSegment));
    alloc((void**)&t.seg[1], size_t(t.seg_capacity) * sizeof(BhSegment));
    alloc((void**)&t.counters, 8 * sizeof(uint32_t));
    alloc((void**)&t.level_info, 64 * sizeof(uint32_t));
    alloc((void**)&t.leaves, nn * sizeof(uint32_t));
    alloc((void**)&t.visits, size_t(t.node_capacity) * sizeof(uint32_t));
    alloc((void**)&t.walk_scratch, size_t(t.walk_warps) * 2 * t.walk_capacity * sizeof(int32_t));
    alloc((void**)&t.stats, 8 * sizeof(unsigned long long)); // 4 interaction counters, [4] next leaf of the walk
    alloc((void**)&t.bbox, 8 * sizeof(unsigned long long));
    alloc((void**)&t.nodef, size_t(t.node_capacity) * NODEF * sizeof(float));
    t.chunk_capacity = 2 * nn / BH_CHUNK + 64;
    alloc((void**)&t.chunks, size_t(t.chunk_capacity) * sizeof(BhChunk));
    alloc((void**)&t.chunk_stats, size_t(t.chunk_capacity) * sizeof(BhChunkStats));
    alloc((void**)&t.chunk_off_b, size_t(t.chunk_capacity) * sizeof(uint32_t));
    alloc((void**)&t.chunk_off_s, size_t(t.chunk_capacity) * sizeof(uint32_t));
    alloc((void**)&t.work, size_t(t.seg_capacity) * sizeof(BhSegWork));
    alloc((void**)&t.pf, nn * sizeof(float4));
    alloc((void**)&t.mf, nn * sizeof(float));
    if (e == cudaSuccess) {
        e = cudaMallocHost((void**)&t.counters_host, 8 * sizeof(uint32_t));
    }
    if (e == cudaSuccess) {
        e = cudaMallocHost((void**)&t.level_host, 64 * sizeof(uint32_t));
    }
    return e;
}

void treeFree(Tree& t) {
    void* ptrs[] = { t.idx, t.scratch_b, t.scratch_s, t.geom, t.mom, t.seg[0], t.seg[1], t.counters, t.leaves, t.visits,
        t.walk_scratch, t.nl_pool, t.nl_kept[0], t.nl_kept[1], t.nl_meta, t.nl_counters, t.nl_defer, t.stats, t.bbox,
        t.nodef, t.pf, t.mf, t.chunks, t.chunk_stats, t.chunk_off_b, t.chunk_off_s, t.work, t.level_info };
    for (void* p : ptrs) {
        if (p) {
            cudaFree(p);
        }
    }
    if (t.counters_host) {
        cudaFreeHost(t.counters_host);
    }
    if (t.nl_host) {
        cudaFreeHost(t.nl_host);
    }
    if (t.level_host) {
        cudaFreeHost(t.level_host);
    }
    t = Tree();
}

namespace {

void launchMoments(const DState& s, Tree& t, const Physics& ph, bool mixed, cudaStream_t st) {
    cudaMemsetAsync(t.visits, 0, size_t(t.node_count) * sizeof(uint32_t), st);
    if (t.leaf_count == 0) {
        return;
    }
    if (mixed) {
        momentsUpKernel<true><<<ceilDiv(t.leaf_count, 128), 128, 0, st>>>(s.r, s.m, ph.G, t.idx, ph.theta_inv, t.geom,
            t.mom, t.nodef, t.leaves, t.leaf_count, t.visits);
    } else {
        momentsUpKernel<false><<<ceilDiv(t.leaf_count, 128), 128, 0, st>>>(s.r, s.m, ph.G, t.idx, ph.theta_inv,
            t.geom, t.mom, t.nodef, t.leaves, t.leaf_count, t.visits);
    }
}

} // namespace

void treeEnsureFp64Moments(const DState& s, Tree& t, const Physics& ph, cudaStream_t st) {
    if (t.built && t.mixed_moments) {
        launchMoments(s, t, ph, false, st);
        t.mixed_moments = false;
    }
}

cudaError_t treeBuild(const DState& s, Tree& t, const Physics& ph, uint32_t* devError, cudaStream_t st) {
    const uint32_t n = s.n;
    t.built = false;
    t.level_start.clear();
    if (n == 0) {
        t.node_count = 0;
        t.leaf_count = 0;
        t.built = true;
        return cudaSuccess;
    }
    // root box = bounding box of all points (KdTree::buildImpl)
    t.launches = 3;
    resetBounds6<<<1, 32, 0, st>>>(t.bbox);
    boundsOnlyKernel<<<min(ceilDiv(n, 256), 152 * 8), 256, 0, st>>>(s.r, n, t.bbox);
    initRootKernel<<<ceilDiv(n, 256), 256, 0, st>>>(n, t.idx, t.seg[0], t.geom, t.counters, t.bbox);
    const PosView pv{ s.r };
    uint32_t nIn = 1;
    int cur = 0;
    t.level_start.push_back(0);
    t.level_start.push_back(1);
    // the largest segment of a level, known on the host (the root at level 0, then bounded by halving)
    uint32_t maxSeg = n;
    for (int level = 0; nIn > 0; ++level) {
        const int grid = int(min(nIn, 152u * 16u));
        const bool big = maxSeg > BH_SMALL_SEGMENT;
        uint32_t nChunks = 0;
        if (big) {
            cudaMemsetAsync(t.counters + 3, 0, sizeof(uint32_t), st);
            chunkListKernel<<<ceilDiv(nIn, 256), 256, 0, st>>>(t.seg[cur], nIn, BH_SMALL_SEGMENT, t.counters,
                t.chunks, t.work, t.chunk_capacity, devError);
            t.launches++;
        }
        if (maxSeg > WARP_SEGMENT) {
            splitLevelKernel<<<grid, BUILD_THREADS, 0, st>>>(pv, t.idx, t.scratch_b, t.scratch_s, t.seg[cur], nIn,
                t.seg[1 - cur], t.geom, t.counters, t.leaves, ph.leaf_size, t.node_capacity, t.seg_capacity, devError,
                WARP_SEGMENT, BH_SMALL_SEGMENT);
            t.launches++;
        }
        const uint32_t warpBlocks = min(uint32_t(ceilDiv(nIn, SPLIT_WARP_THREADS / 32)), 152u * 64u * 32u / SPLIT_WARP_THREADS);
        splitWarpKernel<<<warpBlocks, SPLIT_WARP_THREADS, 0, st>>>(pv, t.idx, t.scratch_b, t.scratch_s, t.seg[cur],
            nIn, nullptr, t.seg[1 - cur], t.geom, t.counters, t.leaves, ph.leaf_size, t.node_capacity,
            t.seg_capacity, devError, WARP_SEGMENT);
        t.launches++;
        if (big) {
            cudaMemcpyAsync(t.counters_host, t.counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
            cudaError_t e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                return e;
            }
            nChunks = min(t.counters_host[3], t.chunk_capacity);
        }
        if (nChunks > 0) {
            chunkStatsKernel<<<nChunks, BUILD_THREADS, 0, st>>>(pv, t.idx, t.seg[cur], t.chunks, t.chunk_stats);
            segDecideKernel<<<ceilDiv(nChunks, 4), 128, 0, st>>>(t.seg[cur], t.chunks, nChunks, t.chunk_stats,
                t.chunk_off_b, t.chunk_off_s, t.work);
            chunkRanksKernel<<<nChunks, BUILD_THREADS, 0, st>>>(pv, t.idx, t.seg[cur], t.chunks, t.chunk_off_b,
                t.chunk_off_s, t.work, t.scratch_b, t.scratch_s);
            segFinishKernel<<<ceilDiv(nChunks, 128), 128, 0, st>>>(pv, t.idx, t.scratch_b, t.scratch_s, t.seg[cur],
                t.chunks, nChunks, t.work, t.seg[1 - cur], t.geom, t.counters, t.node_capacity, t.seg_capacity,
                devError);
            chunkSwapKernel<<<nChunks, BUILD_THREADS, 0, st>>>(t.idx, t.scratch_b, t.scratch_s, t.seg[cur], t.chunks,
                t.work);
            t.launches += 5;
        }
        cudaMemcpyAsync(t.counters_host, t.counters, 5 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        cudaMemsetAsync(t.counters + 1, 0, sizeof(uint32_t), st);
        cudaMemsetAsync(t.counters + 4, 0, sizeof(uint32_t), st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            return e;
        }
        nIn = t.counters_host[1];
        maxSeg = t.counters_host[4];
        t.node_count = t.counters_host[0];
        t.leaf_count = t.counters_host[2];
        if (nIn > 0) {
            t.level_start.push_back(t.node_count);
        }
        cur = 1 - cur;
        if (level > 100000) {
            break;
        }
        if (nIn > 0 && maxSeg <= WARP_SEGMENT) {
            // every remaining segment is split by warps (segments only shrink): LEVEL_BATCH levels per host
            // round trip, the segment counts read by the kernels from levelInfo
            constexpr uint32_t LEVEL_BATCH = 8;
            setWordKernel<<<1, 1, 0, st>>>(t.level_info + 1, nIn);
            t.launches++;
            while (nIn > 0) {
                for (uint32_t b = 0; b < LEVEL_BATCH; ++b) {
                    splitWarpKernel<<<152u * 64u * 32u / SPLIT_WARP_THREADS, SPLIT_WARP_THREADS, 0, st>>>(pv, t.idx, t.scratch_b, t.scratch_s,
                        t.seg[cur], 0, t.level_info + 2 * b + 1, t.seg[1 - cur], t.geom, t.counters, t.leaves,
                        ph.leaf_size, t.node_capacity, t.seg_capacity, devError, WARP_SEGMENT);
                    levelEndKernel<<<1, 1, 0, st>>>(t.counters, t.level_info, b + 1);
                    cur = 1 - cur;
                }
                t.launches += 2 * LEVEL_BATCH;
                cudaMemcpyAsync(t.level_host, t.level_info, 2 * (LEVEL_BATCH + 1) * sizeof(uint32_t),
                    cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(t.counters_host, t.counters, 5 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
                // the next batch starts from the last level's segment count
                cudaMemcpyAsync(t.level_info + 1, t.level_info + 2 * LEVEL_BATCH + 1, sizeof(uint32_t),
                    cudaMemcpyDeviceToDevice, st);
                e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) {
                    return e;
                }
                for (uint32_t b = 1; b <= LEVEL_BATCH; ++b) {
                    if (t.level_host[2 * b + 1] > 0) {
                        t.level_start.push_back(t.level_host[2 * b]);
                    }
                }
                nIn = t.level_host[2 * LEVEL_BATCH + 1];
                t.node_count = t.counters_host[0];
                t.leaf_count = t.counters_host[2];
                level += int(LEVEL_BATCH);
                if (level > 100000) {
                    break;
                }
            }
        }
    }
    // moments, bottom-up in one launch
    t.mixed_moments = ph.precision == SPHGPU_PRECISION_MIXED;
    launchMoments(s, t, ph, t.mixed_moments, st);
    // FP32 node records of the walks (classification geometry; for the mixed walk also the evaluation data)
    launchPrepareWalk(s, t, ph, st);
    t.launches += 2;
    t.built = true;
    return cudaGetLastError();
}

void launchGravityWalk(const DState& s, Tree& t, const Physics& ph, const double* lut, uint32_t* devError,
    cudaStream_t st) {
    cudaMemsetAsync(t.stats, 0, 5 * sizeof(unsigned long long), st);
    if (s.n == 0) {
        return;
    }
    cudaMemsetAsync(s.agrav, 0, size_t(s.n) * sizeof(dbl4), st);
    if (ph.leaf_size > 32) {
        // one warp owns a leaf: larger leaves are not supported by this walk
        return;
    }
    static int residentBlocks = 0;
    if (residentBlocks == 0) {
        int perSm = 0, sms = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, walkKernel, WALK_THREADS, 0);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
        residentBlocks = std::max(1, perSm * sms);
    }
    const int blocks = std::max(1, std::min(residentBlocks, int(t.walk_warps / (WALK_THREADS / 32))));
    walkKernel<<<blocks, WALK_THREADS, 0, st>>>(s.r, s.m, ph.G, t.idx, t.geom, t.mom, t.nodef, t.leaves,
        t.leaf_count, lut,
        ph.kernel_radius,
        ph.multipole_order, t.walk_scratch, t.walk_capacity, s.agrav, t.stats, devError);
}

void launchGravityPoints(const DState& s, const Tree& t, const Physics& ph, const double* lut, const dbl4* points,
    dbl4* acc, uint32_t npoints, cudaStream_t st) {
    if (npoints == 0 || s.n == 0) {
        return;
    }
    pointsKernel<<<ceilDiv(npoints, 128), 128, 0, st>>>(s.r, s.m, ph.G, t.idx, t.geom, t.mom, lut, ph.kernel_radius,
        ph.multipole_order, ph.theta_inv, points, acc, npoints);
}

} // namespace sphgpu
