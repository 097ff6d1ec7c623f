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
constexpr int MAX_PATH_F = 512;

__device__ __forceinline__ void splitF(double x, float& hi, float& lo) {
    hi = float(x);
    lo = float(x - double(hi));
}

__global__ void prepareMixedKernel(const dbl4* __restrict__ r, const double* __restrict__ m, double G,
    const uint32_t* __restrict__ idx, const BhNodeGeom* __restrict__ geom, const BhNodeMoments* __restrict__ mom,
    uint32_t nodeCount, float* __restrict__ nodef, float4* __restrict__ pf, float* __restrict__ mf, bool moments) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nodeCount) {
        return;
    }
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
    if (g.left < 0) {
        for (uint32_t k = g.from; k < g.to; ++k) {
            const uint32_t i = idx[k];
            const dbl4 p = r[i];
            pf[k] = make_float4(float(p.x - g.com[0]), float(p.y - g.com[1]), float(p.z - g.com[2]), float(p.w));
            mf[k] = float(G * m[i]);
        }
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

// GravityLutKernel::grad in FP32 (radius 0: point masses)
__device__ __forceinline__ void gravGradF(float rx, float ry, float rz, float h, const float* __restrict__ lut,
    int kernelRadius, float& gx, float& gy, float& gz) {
    const float d2 = rx * rx + ry * ry + rz * rz;
    const float hInv = 1.f / h;
    const float qSqr = d2 * (hInv * hInv);
    const float rad = float(kernelRadius);
    if (qSqr >= rad * rad) {
        const float inv = rsqrtf(d2);
        const float inv3 = inv * inv * inv;
        gx = rx * inv3;
        gy = ry * inv3;
        gz = rz * inv3;
        return;
    }
    const float floatIdx = float(LUT_ENTRIES / 4) * qSqr;
    const int idx1 = min(int(floatIdx), LUT_ENTRIES - 1);
    const float ratio = floatIdx - float(idx1);
    const float g0 = __ldg(lut + idx1), g1 = __ldg(lut + idx1 + 1);
    const float g = (g0 + (g1 - g0) * ratio) * (hInv * hInv * hInv);
    gx = rx * g;
    gy = ry * g;
    gz = rz * g;
}

// evaluateGravity (core/gravity/Moments.h:336-360) in FP32 at dr = r_i - com; m0 = c0.w, the traceless
// quadrupole and octupole in c2..c5 (layout of the node record)
__device__ __forceinline__ void evalMultipoleF(float drx, float dry, float drz, float m0, const float4& c2,
    const float4& c3, const float4& c4, const float4& c5, int order, float& ax, float& ay, float& az) {
    const float d2 = drx * drx + dry * dry + drz * drz;
    const float inv = rsqrtf(d2);
    const float invDistSqr = inv * inv;
    const float g0 = -inv;
    const float g1 = -invDistSqr * g0;
    const float g2 = -3.f * invDistSqr * g1;
    const float g3 = -5.f * invDistSqr * g2;
    const float g4 = -7.f * invDistSqr * g3;
    const float x = -drx, y = -dry, z = -drz;
    float rx = g1 * x * m0, ry = g1 * y * m0, rz = g1 * z * m0;
    if (order >= 2) {
        const float qxx = c2.x, qxy = c2.y, qxz = c2.z, qyy = c2.w, qyz = c3.x, qzz = c3.y;
        const float Q1x = qxx * x + qxy * y + qxz * z;
        const float Q1y = qxy * x + qyy * y + qyz * z;
        const float Q1z = qxz * x + qyz * y + qzz * z;
        const float Q0 = 0.5f * (Q1x * x + Q1y * y + Q1z * z);
        rx += g3 * x * Q0 + g2 * Q1x;
        ry += g3 * y * Q0 + g2 * Q1y;
        rz += g3 * z * Q0 + g2 * Q1z;
    }
    if (order >= 3) {
        // xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz
        const float q0 = c3.z, q1 = c3.w, q2 = c4.x, q3 = c4.y, q4 = c4.z, q5 = c4.w, q6 = c5.x, q7 = c5.y,
                    q8 = c5.z, q9 = c5.w;
        const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
        // s_i = q_ijk x_j x_k
        const float sx = q0 * xx + q3 * yy + q5 * zz + 2.f * (q1 * xy + q2 * xz + q4 * yz);
        const float sy = q1 * xx + q6 * yy + q8 * zz + 2.f * (q3 * xy + q4 * xz + q7 * yz);
        const float sz = q2 * xx + q7 * yy + q9 * zz + 2.f * (q4 * xy + q5 * xz + q8 * yz);
        const float Q0 = (sx * x + sy * y + sz * z) * (1.f / 6.f);
        rx += g4 * x * Q0 + g3 * (0.5f * sx);
        ry += g4 * y * Q0 + g3 * (0.5f * sy);
        rz += g4 * z * Q0 + g3 * (0.5f * sz);
    }
    ax += rx;
    ay += ry;
    az += rz;
}

// Leaves hold at most 32 particles. A leaf of cnt <= 16 particles splits its warp into g = min(32 / cnt, 4)
// lane groups of cnt lanes (lane = particle of the leaf); the groups share the leaf's walk and take turns
// over its interactions (group q evaluates the q-th, (q + g)-th, ... node of each batch and every g-th
// particle of each particle list), and their partial sums are added to group 0 in group order at the end.
constexpr uint32_t MAX_GROUPS = 4;

__global__ void __launch_bounds__(WALK_THREADS_F, 12) walkMixedKernel(const uint32_t* __restrict__ idx,
    const BhNodeGeom* __restrict__ geom, const float* __restrict__ nodef, const float4* __restrict__ pf,
    const float* __restrict__ mf, const uint32_t* __restrict__ leaves, uint32_t nLeaves, const float* __restrict__ lut,
    int kernelRadius, int order, int32_t* scratch, uint32_t listCap, dbl4* agrav, unsigned long long* stats,
    uint32_t* devError) {
    __shared__ int32_t pathSh[WALK_THREADS_F / 32][MAX_PATH_F];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const uint32_t warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nWarps = (gridDim.x * blockDim.x) >> 5;
    int32_t* listA = scratch + size_t(warpGlobal) * 2 * listCap;
    int32_t* listB = listA + listCap;
    int32_t* path = pathSh[wib];
    const float4* nf = reinterpret_cast<const float4*>(nodef);
    // interaction counters of the warp (approximated nodes, particle lists, particle-node and particle-particle
    // evaluations), kept in shared memory to leave the registers to the walk
    __shared__ unsigned long long countSh[WALK_THREADS_F / 32][4];
    __shared__ WalkFrame frameSh[WALK_THREADS_F / 32];
    unsigned long long* wc = countSh[wib];
    if (lane < 4) {
        wc[lane] = 0;
    }
    __syncwarp();

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
        const uint32_t from = geom[leaf].from, to = geom[leaf].to;
        const uint32_t cnt = to - from;
        int depth = 0;
        if (lane == 0) {
            int d = 0, nd = leaf;
            while (geom[nd].parent >= 0 && d < MAX_PATH_F - 1) {
                nd = geom[nd].parent;
                ++d;
            }
            depth = d;
            nd = leaf;
            for (int k = d; k >= 0; --k) {
                path[k] = nd;
                nd = geom[nd].parent;
            }
            if (d >= MAX_PATH_F - 1) {
                atomicOr(devError, uint32_t(DEV_ERR_WALK_CAPACITY));
            }
        }
        depth = __shfl_sync(0xffffffffu, depth, 0);
        __syncwarp();
        const uint32_t g = cnt == 0 ? 1u : min(32u / cnt, MAX_GROUPS);
        const uint32_t grp = cnt == 0 ? 0u : uint32_t(lane) / cnt;
        const uint32_t pid = uint32_t(lane) - grp * cnt;
        const bool inGroup = grp < g && cnt > 0;
        float lh[3], ll[3];
        {
            const float4 a = nodeGroup(nf, leaf, NF_COM_HI), b = nodeGroup(nf, leaf, NF_COM_LO);
            lh[0] = a.x, lh[1] = a.y, lh[2] = a.z;
            ll[0] = b.x, ll[1] = b.y, ll[2] = b.z;
        }
        float4 di = make_float4(0.f, 0.f, 0.f, 1.f);
        if (inGroup) {
            di = pf[from + pid];
        }
        KahanF ax, ay, az;
        int32_t* cur = listA;
        int32_t* nxt = listB;
        uint32_t ncur = 0, nnxt = 0;
        bool overflow = false;
        for (int k = 1; k <= depth && !overflow; ++k) {
            const int ev = path[k];
            const int par = path[k - 1];
            const int pl = geom[par].left;
            const int sib = pl == ev ? geom[par].right : pl;
            // the frame is the same for the whole warp: kept in shared memory, not in 8 registers per lane
            WalkFrame& fr = frameSh[wib];
            if (lane == 0) {
                setFrame(fr, nf, ev, k == depth, lh, ll);
            }
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
                    const int2 ch = *reinterpret_cast<const int2*>(&geom[node].left);
                    cur[slot] = ch.x;
                    cur[slot + 1] = ch.y;
                }
                pos += batch;
                ncur += 2 * nOpen;
                nnxt += nKeep;
                __syncwarp();
                // plain FP32 partial sums over this batch's interactions, added to the compensated totals once
                float bx = 0.f, by = 0.f, bz = 0.f;
                // particle lists: every particle of the listed leaves, split over the lane groups
                unsigned mp = mPart;
                while (mp) {
                    const int src = __ffs(mp) - 1;
                    mp &= mp - 1;
                    const int pn = __shfl_sync(0xffffffffu, node, src);
                    const float4 a = nodeGroup(nf, pn, NF_COM_HI), b = nodeGroup(nf, pn, NF_COM_LO);
                    const float Dx = (a.x - lh[0]) + (b.x - ll[0]);
                    const float Dy = (a.y - lh[1]) + (b.y - ll[1]);
                    const float Dz = (a.z - lh[2]) + (b.z - ll[2]);
                    const uint2 range = *reinterpret_cast<const uint2*>(&geom[pn].from);
                    if (lane == 0) {
                        wc[1] += 1;
                        wc[3] += uint64_t(cnt) * (range.y - range.x);
                    }
                    if (inGroup) {
#pragma unroll 2
                        for (uint32_t t = range.x + grp; t < range.y; t += g) {
                            const float4 dj = pf[t];
                            const float mj = mf[t];
                            float gx, gy, gz;
                            gravGradF((Dx + dj.x) - di.x, (Dy + dj.y) - di.y, (Dz + dj.z) - di.z, 0.5f * (dj.w + di.w),
                                lut, kernelRadius, gx, gy, gz);
                            bx += mj * gx;
                            by += mj * gy;
                            bz += mj * gz;
                        }
                    }
                }
                // multipole expansions: rounds of g nodes, node q of a round to lane group q
                unsigned mn = mNode;
                if (lane == 0) {
                    const uint32_t nNodes = __popc(mNode);
                    wc[0] += nNodes;
                    wc[2] += uint64_t(cnt) * nNodes;
                }
                while (mn) {
                    int mysrc = -1;
                    for (uint32_t q = 0; q < g && mn; ++q) {
                        const int b = __ffs(mn) - 1;
                        mn &= mn - 1;
                        if (q == grp) {
                            mysrc = b;
                        }
                    }
                    const int nn = __shfl_sync(0xffffffffu, node, mysrc < 0 ? 0 : mysrc);
                    if (inGroup && mysrc >= 0) {
                        const float4 c0 = nodeGroup(nf, nn, NF_COM_HI), c1 = nodeGroup(nf, nn, NF_COM_LO);
                        const float4 c2 = nodeGroup(nf, nn, NF_MOM), c3 = nodeGroup(nf, nn, NF_MOM + 1);
                        const float4 c4 = nodeGroup(nf, nn, NF_MOM + 2), c5 = nodeGroup(nf, nn, NF_MOM + 3);
                        const float Dx = (c0.x - lh[0]) + (c1.x - ll[0]);
                        const float Dy = (c0.y - lh[1]) + (c1.y - ll[1]);
                        const float Dz = (c0.z - lh[2]) + (c1.z - ll[2]);
                        evalMultipoleF(di.x - Dx, di.y - Dy, di.z - Dz, c0.w, c2, c3, c4, c5, order, bx, by, bz);
                    }
                }
                if (inGroup) {
                    ax.add(bx);
                    ay.add(by);
                    az.add(bz);
                }
            }
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
        // pairs inside the leaf
        if (lane == 0) {
            wc[3] += uint64_t(cnt) * (cnt - 1);
        }
        if (inGroup) {
            float sx = 0.f, sy = 0.f, sz = 0.f;
            for (uint32_t t = from + grp; t < to; t += g) {
                const float4 dj = pf[t];
                const float mj = mf[t];
                if (t != from + pid) {
                    float gx, gy, gz;
                    gravGradF(dj.x - di.x, dj.y - di.y, dj.z - di.z, 0.5f * (dj.w + di.w), lut, kernelRadius, gx, gy,
                        gz);
                    sx += mj * gx;
                    sy += mj * gy;
                    sz += mj * gz;
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
    }
    __syncwarp();
    if (lane < 4) {
        atomicAdd(&stats[lane], wc[lane]);
    }
}

} // namespace

void launchPrepareWalk(const DState& s, Tree& t, const Physics& ph, cudaStream_t st) {
    if (s.n == 0 || t.node_count == 0) {
        return;
    }
    prepareMixedKernel<<<ceilDiv(t.node_count, 128), 128, 0, st>>>(s.r, s.m, ph.G, t.idx, t.geom, t.mom,
        t.node_count, t.nodef, t.pf, t.mf, !t.mixed_moments);
}

void launchGravityWalkMixed(const DState& s, Tree& t, const Physics& ph, const float* lutF, uint32_t* devError,
    cudaStream_t st) {
    cudaMemsetAsync(t.stats, 0, 5 * sizeof(unsigned long long), st);
    if (s.n == 0 || t.node_count == 0) {
        return;
    }
    static int residentBlocks = 0;
    if (residentBlocks == 0) {
        int perSm = 0, sms = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, walkMixedKernel, WALK_THREADS_F, 0);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
        residentBlocks = std::max(1, perSm * sms);
    }
    const int blocks = std::max(1, std::min(residentBlocks, int(t.walk_warps / (WALK_THREADS_F / 32))));
    walkMixedKernel<<<blocks, WALK_THREADS_F, 0, st>>>(t.idx, t.geom, t.nodef, t.pf, t.mf, t.leaves, t.leaf_count,
        lutF, ph.kernel_radius, ph.multipole_order, t.walk_scratch, t.walk_capacity, s.agrav, t.stats, devError);
}

} // namespace sphgpu
