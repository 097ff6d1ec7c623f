// gravity32.cu — mixed-precision Barnes-Hut walk: FP64 tree, moments and walk decisions, FP32 evaluation.
//
// The tree, its FP64 moments and the classification of every check-list entry (the sphere-box test of the
// reference's dual walk, core/gravity/BarnesHut.cpp:212-312) are exactly those of the FP64 path, so each
// leaf gets the reference's particle list and node list. Only the evaluation of those interactions runs
// in FP32: particle positions are stored relative to the centre of mass of their leaf, node and leaf
// centres as unevaluated float pairs (hi + lo), so every separation entering the FP32 kernels is formed
// from small numbers without cancellation; sums use Kahan compensation; the result is written in FP64.

#include <algorithm>
#include <cfloat>

#include "tree.cuh"

namespace sphgpu {

namespace {

constexpr int WALK_THREADS_F = 128;

__device__ __forceinline__ void splitF(double x, float& hi, float& lo) {
    hi = float(x);
    lo = float(x - double(hi));
}

__device__ void prepareNode(const BhNodeGeom* __restrict__ geom, const BhNodeMoments* __restrict__ mom, uint32_t id,
    float* __restrict__ nodef, bool moments) {
    const BhNodeGeom& g = geom[id];
    const BhNodeMoments& mo = mom[id];
    float4* o = reinterpret_cast<float4*>(nodef) + size_t(id) * NODEF4;
    float ch[3], cl[3];
    for (int d = 0; d < 3; ++d) {
        splitF(g.com[d], ch[d], cl[d]);
    }
    float ro = float(g.r_open);
    if (g.r_open > 0. && !(ro > 0.f)) {
        ro = FLT_MIN;
    }
    o[NF_COM_HI] = make_float4(ch[0], ch[1], ch[2], float(mo.m0));
    o[NF_COM_LO] = make_float4(cl[0], cl[1], cl[2], g.left < 0 ? -ro : ro);
    if (moments) {
        // the reduced moments, rounded from FP64 (a tree built with FP32 moments already holds them)
        float q[16];
        for (int k = 0; k < 6; ++k) {
            q[k] = float(mo.q2[k]);
        }
        for (int k = 0; k < 10; ++k) {
            q[6 + k] = float(mo.q3[k]);
        }
        for (int k = 0; k < 4; ++k) {
            o[NF_MOM + k] = make_float4(q[4 * k], q[4 * k + 1], q[4 * k + 2], q[4 * k + 3]);
        }
    }
    float bh[2][3], bl[2][3];
    for (int d = 0; d < 3; ++d) {
        splitF(g.lo[d], bh[0][d], bl[0][d]);
        splitF(g.hi[d], bh[1][d], bl[1][d]);
    }
    o[NF_BOX] = make_float4(bh[0][0], bh[0][1], bh[0][2], 0.f);
    o[NF_BOX + 1] = make_float4(bl[0][0], bl[0][1], bl[0][2], 0.f);
    o[NF_BOX + 2] = make_float4(bh[1][0], bh[1][1], bh[1][2], 0.f);
    o[NF_BOX + 3] = make_float4(bl[1][0], bl[1][1], bl[1][2], 0.f);
    // (the leaves' particle inputs of the mixed walk, pf and mf, are written by the mixed moments' leaf pass)
}

__global__ void prepareMixedKernel(const BhNodeGeom* __restrict__ geom, const BhNodeMoments* __restrict__ mom,
    const uint32_t* __restrict__ nodeCountDev, uint32_t nodeCapacity, float* __restrict__ nodef, bool moments) {
    const uint32_t nodeCount = min(*nodeCountDev, nodeCapacity);
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < nodeCount; id += gridDim.x * blockDim.x) {
        prepareNode(geom, mom, id, nodef, moments);
    }
}

struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// GravityLutKernel::grad in FP32 (radius 0: point masses), accumulated as m (gx, gy, gz) into (bx, by, bz).
// h is the pair's symmetrised smoothing length; rad2 the squared kernel radius (0: every pair is a point
// pair). The point-mass branch is taken when |r| >= radius h, tested as |r|^2 >= radius^2 h^2 so that the
// far pairs need no reciprocal of h; inside the kernel the LUT index is clamped to the table, so the rounding
// of the test at the boundary (where the LUT equals the point-mass value) reads no entry past the last.
__device__ __forceinline__ void gravAccF(float rx, float ry, float rz, float h, float m, const float* __restrict__ lut,
    float rad2, float& bx, float& by, float& bz) {
    const float d2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
    float g;
    if (d2 >= rad2 * (h * h)) {
        const float inv = rsqrtf(d2);
        g = inv * inv * inv;
    } else {
        const float hInv = __fdividef(1.f, h); // (the fast reciprocal: 2 ulp, far below the interpolation error)
        const float hInv2 = hInv * hInv;
        const float floatIdx = float(LUT_ENTRIES / 4) * (d2 * hInv2);
        const int idx1 = min(int(floatIdx), LUT_ENTRIES - 1);
        const float ratio = floatIdx - float(idx1);
        const float g0 = __ldg(lut + idx1), g1 = __ldg(lut + idx1 + 1);
        g = fmaf(g1 - g0, ratio, g0) * (hInv2 * hInv);
    }
    const float mg = m * g;
    bx = fmaf(mg, rx, bx);
    by = fmaf(mg, ry, by);
    bz = fmaf(mg, rz, bz);
}

// evaluateGravity (core/gravity/Moments.h:336-360) in FP32, accumulated into (bx, by, bz); (x, y, z) = com - r_i
// (the reference's dr = r_i - com, negated), m0 = c0.w, the traceless quadrupole and octupole in c2..c5
// (layout of the node record). The reference's terms g1 m0 x + g3 Q0q x + g2 Q1 + g4 Q0o x + g3 s / 2 (with
// g1 = |x|^-3, g2 = -3 |x|^-5, g3 = 15 |x|^-7, g4 = -105 |x|^-9, Q1 = q2 . x, Q0q = x . Q1 / 2, s = q3 : x x,
// Q0o = x . s / 6) are evaluated on the unit vector u = x / |x|:
//   a = |x|^-2 [ (m0 + 7.5 |x|^-2 u.q2.u - 17.5 |x|^-3 q3:uuu) u - 3 |x|^-2 q2.u + 7.5 |x|^-3 q3:uu ],
// so that no intermediate is a high power of 1/|x| (|x|^-9 is below the FP32 normal range at the separations of
// kilometre-sized bodies; every factor here is of the order of m0).
__device__ __forceinline__ void accMultipoleF(float x, float y, float z, float m0, const float4& c2, const float4& c3,
    const float4& c4, const float4& c5, int order, float& bx, float& by, float& bz) {
    const float d2 = fmaf(z, z, fmaf(y, y, x * x));
    const float inv = rsqrtf(d2);
    const float t = inv * inv;
    const float ux = x * inv, uy = y * inv, uz = z * inv;
    float A = m0, cx = 0.f, cy = 0.f, cz = 0.f;
    if (order >= 2) {
        const float qxx = c2.x, qxy = c2.y, qxz = c2.z, qyy = c2.w, qyz = c3.x, qzz = c3.y;
        const float Px = fmaf(qxz, uz, fmaf(qxy, uy, qxx * ux));
        const float Py = fmaf(qyz, uz, fmaf(qyy, uy, qxy * ux));
        const float Pz = fmaf(qzz, uz, fmaf(qyz, uy, qxz * ux));
        const float t2 = -3.f * t;
        A = fmaf(-2.5f * t2, fmaf(Pz, uz, fmaf(Py, uy, Px * ux)), A);
        cx = t2 * Px;
        cy = t2 * Py;
        cz = t2 * Pz;
        if (order >= 3) {
            // xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz
            const float q0 = c3.z, q1 = c3.w, q2 = c4.x, q3 = c4.y, q4 = c4.z, q5 = c4.w, q6 = c5.x, q7 = c5.y,
                        q8 = c5.z, q9 = c5.w;
            const float t3 = t * inv;
            const float ux2 = ux + ux, uy2 = uy + uy;
            const float xx = ux * ux, yy = uy * uy, zz = uz * uz, xy2 = ux2 * uy, xz2 = ux2 * uz, yz2 = uy2 * uz;
            // s_i = q_ijk u_j u_k
            const float sx = fmaf(q4, yz2, fmaf(q2, xz2, fmaf(q1, xy2, fmaf(q5, zz, fmaf(q3, yy, q0 * xx)))));
            const float sy = fmaf(q7, yz2, fmaf(q4, xz2, fmaf(q3, xy2, fmaf(q8, zz, fmaf(q6, yy, q1 * xx)))));
            const float sz = fmaf(q8, yz2, fmaf(q5, xz2, fmaf(q4, xy2, fmaf(q9, zz, fmaf(q7, yy, q2 * xx)))));
            const float o3 = 7.5f * t3;
            A = fmaf(-17.5f * t3, fmaf(sz, uz, fmaf(sy, uy, sx * ux)), A);
            cx = fmaf(o3, sx, cx);
            cy = fmaf(o3, sy, cy);
            cz = fmaf(o3, sz, cz);
        }
    }
    bx = fmaf(t, fmaf(A, ux, cx), bx);
    by = fmaf(t, fmaf(A, uy, cy), by);
    bz = fmaf(t, fmaf(A, uz, cz), bz);
}

// Leaves hold at most 32 particles. A leaf of cnt <= 16 particles splits its warp into g = min(32 / cnt, 4)
// lane groups of cnt lanes (lane = particle of the leaf); the groups share the leaf's walk and take turns
// over its interactions (group q evaluates the q-th, (q + g)-th, ... node of each batch and every g-th
// particle of each particle list), and their partial sums are added to group 0 in group order at the end.
constexpr uint32_t MAX_GROUPS = 4;

// ---- two-phase walk ----------------------------------------------------------------------------------------
//
// The dual walk of the reference (BarnesHut::evalNode, core/gravity/BarnesHut.cpp:212-312) classifies, at each
// node ev on a leaf's path, the check list it inherits from ev's parent (plus ev's sibling) against ev's box:
// entries that cannot be decided for all of ev are kept for ev's children. The classification at ev does not
// depend on the leaf below it, so it is done once per node: phase 1 (listLevelKernel, one launch per tree
// level, a warp per node) builds every node's node list N(ev), particle-list list P(ev) and kept list K(ev);
// phase 2 (evalListsKernel, a warp per leaf) evaluates, for the particles of a leaf, the N and P lists of all
// its ancestors and the pairs inside the leaf. The interaction lists are those of the per-leaf walk.


__global__ void flagErrorKernel(uint32_t* devError, uint32_t bit) {
    atomicOr(devError, bit);
}

// Two passes per level: the first (deferPass == 0) runs every node of the level with
// small per-warp staging lists and many warps; a node whose lists outgrow them is appended to the defer list and
// left to the second pass (deferPass == 1), which runs only the deferred nodes with large staging lists. A node
// that outgrows those too is a capacity error.
constexpr uint32_t LIST_POOL_CHUNK = 512;
constexpr uint32_t LIST_KEPT_CHUNK = 256;

__global__ void __launch_bounds__(128, 8) listLevelKernel(const BhNodeGeom* __restrict__ geom,
    const float* __restrict__ nodef, const uint32_t* __restrict__ levelNodes, uint32_t first, uint32_t last,
    int deferPass, uint32_t* __restrict__ defer, uint32_t scratchWarps,
    int32_t* scratch, uint32_t cap, int32_t* __restrict__ pool, uint32_t poolCap,
    const int32_t* __restrict__ keptIn, int32_t* __restrict__ keptOut, uint32_t keptCap, uint32_t* __restrict__ meta,
    uint32_t* __restrict__ counters, int parity) {
    __shared__ WalkFrame frameSh[4];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const uint32_t warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    // the first launch of a level clears the kept-pool and deferred-node counters of the next level (the other
    // parity), which no launch of this level uses
    if (!deferPass && blockIdx.x == 0 && threadIdx.x == 0) {
        counters[1 + (1 - parity)] = 0;
        counters[6 + (1 - parity)] = 0;
    }
    // the warps that have staging lists in the scratch (the grid is rounded up to whole blocks)
    const uint32_t nWarps = min((gridDim.x * blockDim.x) >> 5, scratchWarps);
    if (warpGlobal >= nWarps) {
        return;
    }
    int32_t* cur = scratch + size_t(warpGlobal) * 4 * cap;
    int32_t* kept = cur + cap;
    int32_t* lN = kept + cap;
    int32_t* lP = lN + cap;
    const float4* nf = reinterpret_cast<const float4*>(nodef);
    // counters[6 + parity]: the number of deferred nodes of this level
    const uint32_t total = deferPass ? min(counters[6 + parity], last - first) : last - first;
    // the warp's current chunks of the list pool and of the kept pool: a node's lists take their space
    // from them, and a chunk is reserved with one atomic when the next node's lists do not fit (one returning
    // atomic per node was about 0.1 ms of the list phase); the counters add up the reserved chunks
    // (kept in shared memory: position and end of the pool chunk, of the kept chunk)
    __shared__ uint32_t chunkSh[4][4];
    uint32_t* ch = chunkSh[wib];
    if (lane < 4) {
        ch[lane] = 0;
    }
    __syncwarp();
    for (uint32_t k = warpGlobal; k < total; k += nWarps) {
        const uint32_t ev = deferPass ? defer[k] : levelNodes[first + k];
        const BhNodeGeom& eg = geom[ev];
        const int par = eg.parent;
        const int pl = geom[par].left;
        const int sib = pl == int(ev) ? geom[par].right : pl;
        const uint32_t kIn = meta[size_t(par) * NL_META + 5];
        const uint32_t kOff = meta[size_t(par) * NL_META + 4];
        bool overflow = kIn + 1 > cap;
        uint32_t ncur = 0;
        if (!overflow) {
            for (uint32_t e = lane; e < kIn; e += 32) {
                cur[e] = keptIn[kOff + e];
            }
            ncur = kIn + 1;
            if (lane == 0) {
                cur[kIn] = sib;
            }
        }
        // the box of ev relative to its own centre of mass (the classification frame of the per-leaf walk
        // used the leaf's centre; any frame gives the same FP64-guarded decisions)
        float lh[3], ll[3];
        {
            const float4 a = nodeGroup(nf, int(ev), NF_COM_HI), b = nodeGroup(nf, int(ev), NF_COM_LO);
            lh[0] = a.x, lh[1] = a.y, lh[2] = a.z;
            ll[0] = b.x, ll[1] = b.y, ll[2] = b.z;
        }
        WalkFrame& fr = frameSh[wib];
        if (lane == 0) {
            setFrame(fr, nf, int(ev), eg.left < 0, lh, ll);
        }
        __syncwarp();
        uint32_t nK = 0, nN = 0, nP = 0;
        uint32_t pos = 0;
        while (pos < ncur && !overflow) {
            const uint32_t batch = min(32u, ncur - pos);
            int node = -1, cls = CL_KEEP;
            if (uint32_t(lane) < batch) {
                node = cur[pos + lane];
                cls = classifyEntry(node, geom, nf, fr, lh, ll);
            }
            const bool valid = uint32_t(lane) < batch;
            const unsigned mKeep = __ballot_sync(0xffffffffu, valid && cls == CL_KEEP);
            const unsigned mOpen = __ballot_sync(0xffffffffu, valid && cls == CL_OPEN);
            const unsigned mPart = __ballot_sync(0xffffffffu, valid && cls == CL_PARTICLES);
            const unsigned mNode = __ballot_sync(0xffffffffu, valid && cls == CL_NODE);
            const unsigned below = (1u << lane) - 1u;
            if (ncur + 2 * __popc(mOpen) > cap || nK + __popc(mKeep) > cap || nN + __popc(mNode) > cap ||
                nP + __popc(mPart) > cap) {
                overflow = true;
                break;
            }
            if (valid) {
                if (cls == CL_KEEP) {
                    kept[nK + __popc(mKeep & below)] = node;
                } else if (cls == CL_NODE) {
                    lN[nN + __popc(mNode & below)] = node;
                } else if (cls == CL_PARTICLES) {
                    lP[nP + __popc(mPart & below)] = node;
                } else {
                    const uint32_t slot = ncur + 2 * __popc(mOpen & below);
                    const int2 ch = *reinterpret_cast<const int2*>(&geom[node].left);
                    cur[slot] = ch.x;
                    cur[slot + 1] = ch.y;
                }
            }
            pos += batch;
            ncur += 2 * __popc(mOpen);
            nK += __popc(mKeep);
            nN += __popc(mNode);
            nP += __popc(mPart);
            __syncwarp();
        }
        if (overflow && !deferPass) {
            if (lane == 0) {
                defer[atomicAdd(&counters[6 + parity], 1u)] = ev;
            }
            __syncwarp();
            continue;
        }
        // space in the pools: the counters keep counting past the capacities, so that the host can grow the
        // pools to the need and build the lists again
        uint32_t base = 0, kbase = 0;
        if (lane == 0 && !overflow) {
            const uint32_t need = nN + nP;
            if (ch[0] + need > ch[1]) {
                const uint32_t size = max(need, LIST_POOL_CHUNK);
                ch[0] = atomicAdd(&counters[0], size);
                ch[1] = ch[0] + size;
            }
            base = ch[0];
            ch[0] += need;
            if (nK) {
                if (ch[2] + nK > ch[3]) {
                    const uint32_t size = max(nK, LIST_KEPT_CHUNK);
                    ch[2] = atomicAdd(&counters[1 + parity], size);
                    ch[3] = ch[2] + size;
                    atomicMax(&counters[3], ch[3]);
                }
                kbase = ch[2];
                ch[2] += nK;
            }
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        kbase = __shfl_sync(0xffffffffu, kbase, 0);
        if (overflow || base + nN + nP > poolCap || kbase + nK > keptCap) {
            if (lane == 0) {
                if (overflow) {
                    atomicOr(&counters[5], 1u); // the staging lists were too short
                }
                uint32_t* m = meta + size_t(ev) * NL_META;
                m[0] = m[1] = m[2] = m[3] = m[4] = m[5] = 0;
            }
            continue;
        }
        for (uint32_t e = lane; e < nN; e += 32) {
            pool[base + e] = lN[e];
        }
        for (uint32_t e = lane; e < nP; e += 32) {
            pool[base + nN + e] = lP[e];
        }
        for (uint32_t e = lane; e < nK; e += 32) {
            keptOut[kbase + e] = kept[e];
        }
        if (lane == 0) {
            uint32_t* m = meta + size_t(ev) * NL_META;
            m[0] = base;
            m[1] = nN;
            m[2] = base + nN;
            m[3] = nP;
            m[4] = kbase;
            m[5] = nK;
        }
        __syncwarp();
    }
}

// The same classification with a CTA per node, for the levels with few nodes (the top of the tree, whose
// inherited lists are long): each round classifies LB_THREADS queue entries, and block-wide prefix sums over the
// warps' ballots place the outputs and the opened children in queue order. The queue is processed in order
// whatever the round size (children are appended behind every entry of the round), so the lists are those of
// listLevelKernel. Per-CTA staging of cap entries per list; outgrowing it is a capacity error.
constexpr int LB_THREADS = 256;
constexpr int LB_WARPS = LB_THREADS / 32;

__global__ void __launch_bounds__(LB_THREADS, 4) listBlockKernel(const BhNodeGeom* __restrict__ geom,
    const float* __restrict__ nodef, const uint32_t* __restrict__ levelNodes, uint32_t first, uint32_t last,
    int32_t* scratch, uint32_t cap,
    int32_t* __restrict__ pool, uint32_t poolCap, const int32_t* __restrict__ keptIn, int32_t* __restrict__ keptOut,
    uint32_t keptCap, uint32_t* __restrict__ meta, uint32_t* __restrict__ counters, int parity) {
    __shared__ WalkFrame fr;
    __shared__ uint32_t warpCnt[LB_WARPS][4]; // per warp of a round: kept, opened, particle lists, nodes
    __shared__ uint32_t baseSh[2];
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int w = tid >> 5;
    // (as listLevelKernel's first launch: the next level's kept-pool and deferred-node counters)
    if (blockIdx.x == 0 && tid == 0) {
        counters[1 + (1 - parity)] = 0;
        counters[6 + (1 - parity)] = 0;
    }
    int32_t* cur = scratch + size_t(blockIdx.x) * 4 * cap;
    int32_t* kept = cur + cap;
    int32_t* lN = kept + cap;
    int32_t* lP = lN + cap;
    const float4* nf = reinterpret_cast<const float4*>(nodef);
    for (uint32_t e = first + blockIdx.x; e < last; e += gridDim.x) {
        const uint32_t ev = levelNodes[e];
        const BhNodeGeom& eg = geom[ev];
        const int par = eg.parent;
        const int pl = geom[par].left;
        const int sib = pl == int(ev) ? geom[par].right : pl;
        const uint32_t kIn = meta[size_t(par) * NL_META + 5];
        const uint32_t kOff = meta[size_t(par) * NL_META + 4];
        bool overflow = kIn + 1 > cap;
        uint32_t ncur = 0;
        if (!overflow) {
            for (uint32_t e = tid; e < kIn; e += LB_THREADS) {
                cur[e] = keptIn[kOff + e];
            }
            ncur = kIn + 1;
            if (tid == 0) {
                cur[kIn] = sib;
            }
        }
        float lh[3], ll[3];
        {
            const float4 a = nodeGroup(nf, int(ev), NF_COM_HI), b = nodeGroup(nf, int(ev), NF_COM_LO);
            lh[0] = a.x, lh[1] = a.y, lh[2] = a.z;
            ll[0] = b.x, ll[1] = b.y, ll[2] = b.z;
        }
        if (tid == 0) {
            setFrame(fr, nf, int(ev), eg.left < 0, lh, ll);
        }
        __syncthreads();
        uint32_t nK = 0, nN = 0, nP = 0;
        uint32_t pos = 0;
        while (pos < ncur && !overflow) {
            const uint32_t batch = min(uint32_t(LB_THREADS), ncur - pos);
            const bool valid = uint32_t(tid) < batch;
            int node = -1, cls = CL_KEEP;
            if (valid) {
                node = cur[pos + tid];
                cls = classifyEntry(node, geom, nf, fr, lh, ll);
            }
            const unsigned mKeep = __ballot_sync(0xffffffffu, valid && cls == CL_KEEP);
            const unsigned mOpen = __ballot_sync(0xffffffffu, valid && cls == CL_OPEN);
            const unsigned mPart = __ballot_sync(0xffffffffu, valid && cls == CL_PARTICLES);
            const unsigned mNode = __ballot_sync(0xffffffffu, valid && cls == CL_NODE);
            if (lane == 0) {
                warpCnt[w][0] = __popc(mKeep);
                warpCnt[w][1] = __popc(mOpen);
                warpCnt[w][2] = __popc(mPart);
                warpCnt[w][3] = __popc(mNode);
            }
            __syncthreads();
            uint32_t pre[4] = { 0, 0, 0, 0 }, tot[4] = { 0, 0, 0, 0 };
            for (int q = 0; q < LB_WARPS; ++q) {
                for (int c = 0; c < 4; ++c) {
                    const uint32_t v = warpCnt[q][c];
                    pre[c] += q < w ? v : 0u;
                    tot[c] += v;
                }
            }
            const bool full = ncur + 2 * tot[1] > cap || nK + tot[0] > cap || nN + tot[3] > cap || nP + tot[2] > cap;
            if (!full && valid) {
                const unsigned below = (1u << lane) - 1u;
                if (cls == CL_KEEP) {
                    kept[nK + pre[0] + __popc(mKeep & below)] = node;
                } else if (cls == CL_NODE) {
                    lN[nN + pre[3] + __popc(mNode & below)] = node;
                } else if (cls == CL_PARTICLES) {
                    lP[nP + pre[2] + __popc(mPart & below)] = node;
                } else {
                    const uint32_t slot = ncur + 2 * (pre[1] + __popc(mOpen & below));
                    const int2 ch = *reinterpret_cast<const int2*>(&geom[node].left);
                    cur[slot] = ch.x;
                    cur[slot + 1] = ch.y;
                }
            }
            __syncthreads();
            if (full) {
                overflow = true;
                break;
            }
            pos += batch;
            ncur += 2 * tot[1];
            nK += tot[0];
            nN += tot[3];
            nP += tot[2];
        }
        if (tid == 0) {
            uint32_t base = 0, kbase = 0;
            if (!overflow) {
                base = atomicAdd(&counters[0], nN + nP);
                kbase = nK ? atomicAdd(&counters[1 + parity], nK) : 0u;
                atomicMax(&counters[3], kbase + nK);
            }
            baseSh[0] = base;
            baseSh[1] = kbase;
        }
        __syncthreads();
        const uint32_t base = baseSh[0], kbase = baseSh[1];
        if (overflow || base + nN + nP > poolCap || kbase + nK > keptCap) {
            if (tid == 0) {
                if (overflow) {
                    atomicOr(&counters[5], 1u); // the staging lists were too short
                }
                uint32_t* m = meta + size_t(ev) * NL_META;
                m[0] = m[1] = m[2] = m[3] = m[4] = m[5] = 0;
            }
        } else {
            for (uint32_t e = tid; e < nN; e += LB_THREADS) {
                pool[base + e] = lN[e];
            }
            for (uint32_t e = tid; e < nP; e += LB_THREADS) {
                pool[base + nN + e] = lP[e];
            }
            for (uint32_t e = tid; e < nK; e += LB_THREADS) {
                keptOut[kbase + e] = kept[e];
            }
            if (tid == 0) {
                uint32_t* m = meta + size_t(ev) * NL_META;
                m[0] = base;
                m[1] = nN;
                m[2] = base + nN;
                m[3] = nP;
                m[4] = kbase;
                m[5] = nK;
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(WALK_THREADS_F, 7) evalListsKernel(const uint32_t* __restrict__ idx,
    const BhNodeGeom* __restrict__ geom, const float* __restrict__ nodef, const float4* __restrict__ pf,
    const float* __restrict__ mf, const uint32_t* __restrict__ leaves, uint32_t nLeaves,
    const float* __restrict__ lut, int kernelRadius, int order, const int32_t* __restrict__ pool,
    const uint32_t* __restrict__ meta, dbl4* agrav, unsigned long long* stats) {
    constexpr int W = WALK_THREADS_F / 32;
    __shared__ int32_t pathSh[W][MAX_PATH_F];
    // per warp: the node records of one batch of a node list ([record group][entry]), the source leaves of one
    // batch of a particle list (centre relative to the leaf's hi centre + lo centre, particle range), and the
    // particles of one source leaf
    __shared__ float4 recSh[W][6][32];
    __shared__ float4 srcSh[W][2][32];
    __shared__ float4 partSh[W][32];
    __shared__ float massSh[W][32];
    // interaction counters of the warp: node lists, particle lists, particle-node and particle-particle evaluations
    __shared__ unsigned long long countSh[W][4];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    int32_t* path = pathSh[wib];
    const float4* nf = reinterpret_cast<const float4*>(nodef);
    const float rad2 = float(kernelRadius) * float(kernelRadius);
    const int nRec = order >= 3 ? 6 : (order == 2 ? 4 : 2);
    unsigned long long* wc = countSh[wib];
    if (lane < 4) {
        wc[lane] = 0;
    }
    __syncwarp();
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
        const uint32_t from = geom[leaf].from, to = geom[leaf].to;
        const uint32_t cnt = to - from;
        // the root path, path[0] = root ... path[depth] = leaf, in one climb from the leaf's level
        int depth = 0;
        if (lane == 0) {
            depth = min(geom[leaf].level, MAX_PATH_F - 1);
            int nd = leaf;
            for (int k = depth; k >= 0; --k) {
                path[k] = nd;
                nd = geom[nd].parent;
            }
        }
        depth = __shfl_sync(0xffffffffu, depth, 0);
        __syncwarp();
        // (leaves hold at most 32 particles: the configuration refuses larger leaf sizes)
        const uint32_t g = cnt == 0 ? 1u : max(1u, min(32u / cnt, MAX_GROUPS));
        const uint32_t grp = cnt == 0 ? 0u : uint32_t(lane) / cnt;
        const uint32_t pid = uint32_t(lane) - grp * cnt;
        const bool inGroup = grp < g && cnt > 0;
        float4 di = make_float4(0.f, 0.f, 0.f, 0.f);
        if (inGroup) {
            di = pf[from + pid];
        }
        // the particle relative to the hi part of its leaf's centre: separations from a node centre c (hi + lo)
        // are formed as (c.hi - leaf.hi) + (c.lo - pl), pl = leaf.lo + (r_i - leaf centre)
        float lh[3], pl[3];
        {
            const float4 a = nodeGroup(nf, leaf, NF_COM_HI), b = nodeGroup(nf, leaf, NF_COM_LO);
            lh[0] = a.x, lh[1] = a.y, lh[2] = a.z;
            pl[0] = b.x + di.x, pl[1] = b.y + di.y, pl[2] = b.z + di.z;
        }
        KahanF ax, ay, az;
        // the leaf's list lengths and source particles (the same in every lane)
        uint32_t leafN = 0, leafP = 0, leafSrc = 0;
        for (int k = 1; k <= depth; ++k) {
            const uint32_t* m = meta + size_t(path[k]) * NL_META;
            const uint32_t nOff = m[0], nLen = m[1], pOff = m[2], pLen = m[3];
            leafN += nLen;
            leafP += pLen;
            // particle lists of this level, then its nodes, 32 entries at a time
            for (uint32_t c = 0; c < pLen; c += 32) {
                const uint32_t batch = min(32u, pLen - c);
                if (uint32_t(lane) < batch) {
                    const int pn = pool[pOff + c + lane];
                    const float4 a = nodeGroup(nf, pn, NF_COM_HI), b = nodeGroup(nf, pn, NF_COM_LO);
                    const uint2 range = *reinterpret_cast<const uint2*>(&geom[pn].from);
                    srcSh[wib][0][lane] = make_float4(a.x - lh[0], a.y - lh[1], a.z - lh[2], b.x);
                    srcSh[wib][1][lane] = make_float4(b.y, b.z, __uint_as_float(range.x), __uint_as_float(range.y));
                }
                __syncwarp();
                float bx = 0.f, by = 0.f, bz = 0.f;
                for (uint32_t q = 0; q < batch; ++q) {
                    const float4 s0 = srcSh[wib][0][q], s1 = srcSh[wib][1][q];
                    // separation of the source leaf's centre from particle i
                    const float ox = s0.x + (s0.w - pl[0]);
                    const float oy = s0.y + (s1.x - pl[1]);
                    const float oz = s0.z + (s1.y - pl[2]);
                    const uint32_t r0 = __float_as_uint(s1.z), r1 = __float_as_uint(s1.w);
                    leafSrc += r1 - r0;
                    for (uint32_t base = r0; base < r1; base += 32) {
                        const uint32_t ns = min(32u, r1 - base);
                        if (uint32_t(lane) < ns) {
                            partSh[wib][lane] = pf[base + lane];
                            massSh[wib][lane] = mf[base + lane];
                        }
                        __syncwarp();
                        if (inGroup) {
#pragma unroll 2
                            for (uint32_t t = grp; t < ns; t += g) {
                                const float4 dj = partSh[wib][t];
                                gravAccF(ox + dj.x, oy + dj.y, oz + dj.z, dj.w + di.w, massSh[wib][t], lut, rad2, bx,
                                    by, bz);
                            }
                        }
                        __syncwarp();
                    }
                }
                if (inGroup) {
                    ax.add(bx);
                    ay.add(by);
                    az.add(bz);
                }
            }
            for (uint32_t c = 0; c < nLen; c += 32) {
                const uint32_t batch = min(32u, nLen - c);
                if (uint32_t(lane) < batch) {
                    const int nn = pool[nOff + c + lane];
                    // record groups 0..5: centre hi, centre lo, reduced moments
#pragma unroll
                    for (int r = 0; r < 6; ++r) {
                        if (r < nRec) {
                            recSh[wib][r][lane] = nodeGroup(nf, nn, r);
                        }
                    }
                }
                __syncwarp();
                float bx = 0.f, by = 0.f, bz = 0.f;
                // rounds of g nodes, node q of a round to lane group q
                for (uint32_t q0 = 0; q0 < batch; q0 += g) {
                    const uint32_t q = q0 + grp;
                    if (inGroup && q < batch) {
                        const float4 c0 = recSh[wib][0][q], c1 = recSh[wib][1][q];
                        const float4 c2 = recSh[wib][2][q], c3 = recSh[wib][3][q];
                        const float4 c4 = recSh[wib][4][q], c5 = recSh[wib][5][q];
                        accMultipoleF((c0.x - lh[0]) + (c1.x - pl[0]), (c0.y - lh[1]) + (c1.y - pl[1]),
                            (c0.z - lh[2]) + (c1.z - pl[2]), c0.w, c2, c3, c4, c5, order, bx, by, bz);
                    }
                }
                __syncwarp();
                if (inGroup) {
                    ax.add(bx);
                    ay.add(by);
                    az.add(bz);
                }
            }
        }
        if (lane == 0) {
            wc[0] += leafN;
            wc[1] += leafP;
            wc[2] += uint64_t(cnt) * leafN;
            wc[3] += uint64_t(cnt) * (leafSrc + cnt - 1);
        }
        // pairs inside the leaf
        if (inGroup) {
            float sx = 0.f, sy = 0.f, sz = 0.f;
            for (uint32_t t = from + grp; t < to; t += g) {
                const float4 dj = pf[t];
                if (t != from + pid) {
                    gravAccF(dj.x - di.x, dj.y - di.y, dj.z - di.z, dj.w + di.w, mf[t], lut, rad2, sx, sy, sz);
                }
            }
            ax.add(sx);
            ay.add(sy);
            az.add(sz);
        }
        // partial sums of groups 1 .. g-1 into group 0, in group order
        for (uint32_t q = 1; q < g; ++q) {
            const int srcLane = grp == 0 ? lane + int(q * cnt) : lane;
            const float xs = __shfl_sync(0xffffffffu, ax.s, srcLane), xc = __shfl_sync(0xffffffffu, ax.c, srcLane);
            const float ys = __shfl_sync(0xffffffffu, ay.s, srcLane), yc = __shfl_sync(0xffffffffu, ay.c, srcLane);
            const float zs = __shfl_sync(0xffffffffu, az.s, srcLane), zc = __shfl_sync(0xffffffffu, az.c, srcLane);
            if (grp == 0) {
                ax.add(xs);
                ax.add(-xc);
                ay.add(ys);
                ay.add(-yc);
                az.add(zs);
                az.add(-zc);
            }
        }
        if (grp == 0 && uint32_t(lane) < cnt) {
            const uint32_t pi = idx[from + pid];
            agrav[pi] = mkd4(double(ax.s) - double(ax.c), double(ay.s) - double(ay.c), double(az.s) - double(az.c), 0.);
        }
        __syncwarp();
    }
    __syncwarp();
    if (lane < 4) {
        atomicAdd(&stats[lane], wc[lane]);
    }
}



} // namespace

void launchPrepareWalkDev(const DState& s, Tree& t, const Physics& ph, cudaStream_t st) {
    if (s.n == 0) {
        return;
    }
    // the node count is read on the device (counters[C_NODES]); at most 2 n nodes
    const int blocks = std::max(1, std::min(ceilDiv(t.node_capacity, 128), 152 * 16));
    prepareMixedKernel<<<blocks, 128, 0, st>>>(t.geom, t.mom, t.counters + C_NODES, t.node_capacity, t.nodef,
        !t.mixed_moments);
    (void)ph;
}

// walk phase 1 for both precisions: the node, particle-list and kept lists of every node, level by level
void launchWalkLists(const DState& s, Tree& t, uint32_t* devError, cudaStream_t st) {
    if (!t.nl_meta) {
        cudaMalloc(&t.nl_meta, size_t(t.node_capacity) * NL_META * sizeof(uint32_t));
        cudaMalloc(&t.nl_counters, 8 * sizeof(uint32_t));
        cudaMallocHost(&t.nl_host, 8 * sizeof(uint32_t));
    }
    if (!t.nl_defer) {
        cudaMalloc(&t.nl_defer, size_t(t.node_capacity) * sizeof(uint32_t));
    }
    uint32_t poolNeed = std::max<uint32_t>(1u << 20, 64u * t.node_count);
    uint32_t keptNeed = std::max<uint32_t>(1u << 20, 32u * t.node_count);
    // level l holds the nodes level_nodes[level_first[l] .. level_first[l + 1])
    const uint32_t levels = t.level_first.empty() ? 0u : uint32_t(t.level_first.size() - 1);
    // the lists of all levels; when a pool overflowed, grow it to twice the counted need (the count misses what
    // the children of the nodes that did not fit would have added), and when a node's lists outgrew the staging,
    // the staging four times, and build them again
    bool fits = false;
    for (int attempt = 0; attempt < 8 && !fits; ++attempt) {
        // per-warp staging of one node's lists in the walk scratch: 4 lists of NL_STAGE entries in the first pass
        // of a level, of NL_STAGE_DEFER entries (the scratch of walk_defer_factor warps) in the pass over the nodes
        // deferred by the first and on the levels of few nodes
        const size_t scratchEntries = size_t(t.walk_warps) * 2 * t.walk_capacity;
        const uint32_t NL_STAGE = t.walk_capacity;
        const uint32_t NL_STAGE_DEFER = uint32_t(std::min<size_t>(size_t(t.walk_defer_factor) * t.walk_capacity,
            scratchEntries / 4));
        const uint32_t listWarps = std::max(1u, uint32_t(scratchEntries / (4 * size_t(NL_STAGE))));
        const uint32_t deferWarps = std::max(1u, uint32_t(scratchEntries / (4 * size_t(NL_STAGE_DEFER))));
        if (t.nl_capacity < poolNeed) {
            cudaFree(t.nl_pool);
            cudaMalloc(&t.nl_pool, size_t(poolNeed) * sizeof(int32_t));
            t.nl_capacity = poolNeed;
        }
        if (t.nl_kept_capacity < keptNeed) {
            cudaFree(t.nl_kept[0]);
            cudaFree(t.nl_kept[1]);
            cudaMalloc(&t.nl_kept[0], size_t(keptNeed) * sizeof(int32_t));
            cudaMalloc(&t.nl_kept[1], size_t(keptNeed) * sizeof(int32_t));
            t.nl_kept_capacity = keptNeed;
        }
        cudaMemsetAsync(t.nl_counters, 0, 8 * sizeof(uint32_t), st);
        cudaMemsetAsync(t.nl_meta, 0, NL_META * sizeof(uint32_t), st); // the root: nothing kept
        for (uint32_t level = 1; level < levels; ++level) {
            const uint32_t first = t.level_first[level];
            const uint32_t last = t.level_first[level + 1];
            if (last <= first) {
                // (no launch to clear the next level's counters: both parities' are cleared here)
                cudaMemsetAsync(t.nl_counters + 1, 0, 2 * sizeof(uint32_t), st);
                cudaMemsetAsync(t.nl_counters + 6, 0, 2 * sizeof(uint32_t), st);
                continue;
            }
            // (this level's kept-pool and deferred-node counters, counters[1 + parity] and counters[6 + parity],
            // were cleared by the previous level's first launch, or by the clearing of all counters above)
            const int parity = int(level & 1u);
            if (last - first <= deferWarps) {
                // few nodes: a CTA per node with the large staging lists
                listBlockKernel<<<last - first, LB_THREADS, 0, st>>>(t.geom, t.nodef, t.level_nodes, first, last,
                    t.walk_scratch,
                    NL_STAGE_DEFER, t.nl_pool, t.nl_capacity, t.nl_kept[1 - parity], t.nl_kept[parity],
                    t.nl_kept_capacity, t.nl_meta, t.nl_counters, parity);
                t.walk_launches++;
                continue;
            }
            const uint32_t warps = std::min(last - first, listWarps);
            listLevelKernel<<<ceilDiv(warps, 4), 128, 0, st>>>(t.geom, t.nodef, t.level_nodes, first, last, 0,
                t.nl_defer, warps,
                t.walk_scratch, NL_STAGE, t.nl_pool, t.nl_capacity, t.nl_kept[1 - parity], t.nl_kept[parity],
                t.nl_kept_capacity, t.nl_meta, t.nl_counters, parity);
            const uint32_t dWarps = std::min(last - first, deferWarps);
            listLevelKernel<<<ceilDiv(dWarps, 4), 128, 0, st>>>(t.geom, t.nodef, t.level_nodes, first, last, 1,
                t.nl_defer, dWarps,
                t.walk_scratch, NL_STAGE_DEFER, t.nl_pool, t.nl_capacity, t.nl_kept[1 - parity], t.nl_kept[parity],
                t.nl_kept_capacity, t.nl_meta, t.nl_counters, parity);
            t.walk_launches += 2;
        }
        cudaMemcpyAsync(t.nl_host, t.nl_counters, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) {
            return;
        }
        const uint32_t usedPool = t.nl_host[0], usedKept = t.nl_host[3];
        const bool staged = t.nl_host[5] == 0;
        fits = staged && usedPool <= t.nl_capacity && usedKept <= t.nl_kept_capacity;
        poolNeed = std::max(poolNeed, 2 * usedPool);
        keptNeed = std::max(keptNeed, 2 * usedKept);
        if (!staged) {
            // longer staging for the few nodes whose lists outgrew it: fewer warps share the scratch, and only when
            // one warp holds all of it, a larger scratch
            if (size_t(t.walk_defer_factor) * 4 * t.walk_capacity <= scratchEntries / 4) {
                t.walk_defer_factor *= 4;
            } else if (treeGrowWalkScratch(t, 4 * t.walk_capacity) != cudaSuccess) {
                break;
            }
        }
    }
    if (!fits) {
        flagErrorKernel<<<1, 1, 0, st>>>(devError, uint32_t(DEV_ERR_WALK_CAPACITY));
    }
    (void)s;
}

void launchGravityWalkMixed(const DState& s, Tree& t, const Physics& ph, const float* lutF, uint32_t* devError,
    cudaStream_t st, cudaEvent_t evalStart, cudaEvent_t evalEnd) {
    cudaMemsetAsync(t.stats, 0, 5 * sizeof(unsigned long long), st);
    t.walk_launches = 0;
    if (s.n == 0 || t.node_count == 0) {
        return;
    }
    launchWalkLists(s, t, devError, st);
    static int residentBlocks = 0;
    if (residentBlocks == 0) {
        int perSm = 0, sms = 0;
        // the staging buffers of eight resident blocks need most of the unified L1 / shared memory
        cudaFuncSetAttribute(evalListsKernel, cudaFuncAttributePreferredSharedMemoryCarveout,
            int(cudaSharedmemCarveoutMaxShared));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, evalListsKernel, WALK_THREADS_F, 0);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
        residentBlocks = std::max(1, perSm * sms);
    }
    const int blocks = std::max(1, std::min(residentBlocks, int(t.walk_warps / (WALK_THREADS_F / 32))));
    if (evalStart) {
        cudaEventRecord(evalStart, st);
    }
    evalListsKernel<<<blocks, WALK_THREADS_F, 0, st>>>(t.idx, t.geom, t.nodef, t.pf, t.mf, t.leaves, t.leaf_count,
        lutF, ph.kernel_radius, ph.multipole_order, t.nl_pool, t.nl_meta, s.agrav, t.stats);
    if (evalEnd) {
        cudaEventRecord(evalEnd, st);
    }
    t.walk_launches++;
}

} // namespace sphgpu
