// gravity32.cu — mixed-precision Barnes-Hut walk: FP64 tree, moments and walk decisions, FP32 evaluation.
//
// The tree, its FP64 moments and the classification of every check-list entry (the sphere-box test of the
// reference's dual walk, core/gravity/BarnesHut.cpp:212-312) are exactly those of the FP64 path, so each
// leaf gets the reference's particle list and node list. Only the evaluation of those interactions runs
// in FP32: particle positions are stored relative to the centre of mass of their leaf, node and leaf
// centres as unevaluated float pairs (hi + lo), so every separation entering the FP32 kernels is formed
// from small numbers without cancellation; sums use Kahan compensation; the result is written in FP64.

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
    uint32_t nodeCount, float* __restrict__ nodef, float4* __restrict__ pf, float* __restrict__ mf) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nodeCount) {
        return;
    }
    const BhNodeGeom& g = geom[id];
    const BhNodeMoments& mo = mom[id];
    float* o = nodef + size_t(id) * NODEF;
    for (int d = 0; d < 3; ++d) {
        splitF(g.com[d], o[d], o[3 + d]);
    }
    o[6] = float(mo.m0);
    for (int k = 0; k < 6; ++k) {
        o[7 + k] = float(mo.q2[k]);
    }
    for (int k = 0; k < 10; ++k) {
        o[13 + k] = float(mo.q3[k]);
    }
    o[NODEF_ROPEN] = float(g.r_open);
    o[NODEF_ZERO] = g.r_open == 0. ? 1.f : 0.f;
    for (int d = 0; d < 3; ++d) {
        splitF(g.lo[d], o[NODEF_BOX + d], o[NODEF_BOX + 3 + d]);
        splitF(g.hi[d], o[NODEF_BOX + 6 + d], o[NODEF_BOX + 9 + d]);
    }
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

// evaluateGravity (core/gravity/Moments.h:336-360) in FP32 at dr = r_i - com
__device__ __forceinline__ void evalMultipoleF(float drx, float dry, float drz, const float* __restrict__ o,
    int order, float& ax, float& ay, float& az) {
    const float d2 = drx * drx + dry * dry + drz * drz;
    const float inv = rsqrtf(d2);
    const float invDistSqr = inv * inv;
    const float g0 = -inv;
    const float g1 = -invDistSqr * g0;
    const float g2 = -3.f * invDistSqr * g1;
    const float g3 = -5.f * invDistSqr * g2;
    const float g4 = -7.f * invDistSqr * g3;
    const float x = -drx, y = -dry, z = -drz;
    const float m0 = o[6];
    float rx = g1 * x * m0, ry = g1 * y * m0, rz = g1 * z * m0;
    if (order >= 2) {
        const float qxx = o[7], qxy = o[8], qxz = o[9], qyy = o[10], qyz = o[11], qzz = o[12];
        const float Q1x = qxx * x + qxy * y + qxz * z;
        const float Q1y = qxy * x + qyy * y + qyz * z;
        const float Q1z = qxz * x + qyz * y + qzz * z;
        const float Q0 = 0.5f * (Q1x * x + Q1y * y + Q1z * z);
        rx += g3 * x * Q0 + g2 * Q1x;
        ry += g3 * y * Q0 + g2 * Q1y;
        rz += g3 * z * Q0 + g2 * Q1z;
    }
    if (order >= 3) {
        const float* q = o + 13; // xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz
        const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
        // s_i = q_ijk x_j x_k
        const float sx = q[0] * xx + q[3] * yy + q[5] * zz + 2.f * (q[1] * xy + q[2] * xz + q[4] * yz);
        const float sy = q[1] * xx + q[6] * yy + q[8] * zz + 2.f * (q[3] * xy + q[4] * xz + q[7] * yz);
        const float sz = q[2] * xx + q[7] * yy + q[9] * zz + 2.f * (q[4] * xy + q[5] * xz + q[8] * yz);
        const float Q0 = (sx * x + sy * y + sz * z) * (1.f / 6.f);
        rx += g4 * x * Q0 + g3 * (0.5f * sx);
        ry += g4 * y * Q0 + g3 * (0.5f * sy);
        rz += g4 * z * Q0 + g3 * (0.5f * sz);
    }
    ax += rx;
    ay += ry;
    az += rz;
}

__global__ void __launch_bounds__(WALK_THREADS_F, 6) walkMixedKernel(const uint32_t* __restrict__ idx,
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
    unsigned long long nApprox = 0, nExact = 0, nPn = 0, nPp = 0;

    for (uint32_t li = warpGlobal; li < nLeaves; li += nWarps) {
        const int leaf = int(leaves[li]);
        const BhNodeGeom lg = geom[leaf];
        const uint32_t cnt = lg.to - lg.from;
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
        const bool active = uint32_t(lane) < cnt;
        const float* lf = nodef + size_t(leaf) * NODEF;
        const float lhx = lf[0], lhy = lf[1], lhz = lf[2], llx = lf[3], lly = lf[4], llz = lf[5];
        float4 di = make_float4(0.f, 0.f, 0.f, 1.f);
        uint32_t pi = 0;
        if (active) {
            di = pf[lg.from + lane];
            pi = idx[lg.from + lane];
        }
        KahanF ax, ay, az;
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
            for (int d = 0; d < 3; ++d) {
                fr.lh[d] = lf[d];
                fr.ll[d] = lf[3 + d];
            }
            setFrame(fr, geom[ev], nodef + size_t(ev) * NODEF, k == depth);
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
                    cls = classifyEntry(node, geom, nodef, fr);
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
                unsigned mp = mPart;
                while (mp) {
                    const int src = __ffs(mp) - 1;
                    mp &= mp - 1;
                    const int pn = __shfl_sync(0xffffffffu, node, src);
                    const float* pfn = nodef + size_t(pn) * NODEF;
                    const float Dx = (pfn[0] - lhx) + (pfn[3] - llx);
                    const float Dy = (pfn[1] - lhy) + (pfn[4] - lly);
                    const float Dz = (pfn[2] - lhz) + (pfn[5] - llz);
                    const uint32_t f0 = geom[pn].from, f1 = geom[pn].to;
                    nExact += 1;
                    nPp += uint64_t(cnt) * (f1 - f0);
                    float sx = 0.f, sy = 0.f, sz = 0.f;
                    for (uint32_t t = f0; t < f1; ++t) {
                        const float4 dj = pf[t];
                        const float mj = mf[t];
                        float gx, gy, gz;
                        gravGradF((Dx + dj.x) - di.x, (Dy + dj.y) - di.y, (Dz + dj.z) - di.z, 0.5f * (dj.w + di.w), lut,
                            kernelRadius, gx, gy, gz);
                        sx += mj * gx;
                        sy += mj * gy;
                        sz += mj * gz;
                    }
                    if (active) {
                        ax.add(sx);
                        ay.add(sy);
                        az.add(sz);
                    }
                }
                unsigned mn = mNode;
                while (mn) {
                    const int src = __ffs(mn) - 1;
                    mn &= mn - 1;
                    const int nn = __shfl_sync(0xffffffffu, node, src);
                    const float* o = nodef + size_t(nn) * NODEF;
                    const float Dx = (o[0] - lhx) + (o[3] - llx);
                    const float Dy = (o[1] - lhy) + (o[4] - lly);
                    const float Dz = (o[2] - lhz) + (o[5] - llz);
                    nApprox += 1;
                    nPn += cnt;
                    float sx = 0.f, sy = 0.f, sz = 0.f;
                    evalMultipoleF(di.x - Dx, di.y - Dy, di.z - Dz, o, order, sx, sy, sz);
                    if (active) {
                        ax.add(sx);
                        ay.add(sy);
                        az.add(sz);
                    }
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
        nPp += uint64_t(cnt) * (cnt - 1);
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (uint32_t t = lg.from; t < lg.to; ++t) {
            const float4 dj = pf[t];
            const float mj = mf[t];
            if (t != lg.from + uint32_t(lane)) {
                float gx, gy, gz;
                gravGradF(dj.x - di.x, dj.y - di.y, dj.z - di.z, 0.5f * (dj.w + di.w), lut, kernelRadius, gx, gy, gz);
                sx += mj * gx;
                sy += mj * gy;
                sz += mj * gz;
            }
        }
        if (active) {
            ax.add(sx);
            ay.add(sy);
            az.add(sz);
            agrav[pi] = mkd4(double(ax.s) - double(ax.c), double(ay.s) - double(ay.c), double(az.s) - double(az.c), 0.);
        }
    }
    if (lane == 0) {
        atomicAdd(&stats[0], nApprox);
        atomicAdd(&stats[1], nExact);
        atomicAdd(&stats[2], nPn);
        atomicAdd(&stats[3], nPp);
    }
}

} // namespace

void launchPrepareWalk(const DState& s, Tree& t, const Physics& ph, cudaStream_t st) {
    if (s.n == 0 || t.node_count == 0) {
        return;
    }
    prepareMixedKernel<<<ceilDiv(t.node_count, 128), 128, 0, st>>>(s.r, s.m, ph.G, t.idx, t.geom, t.mom,
        t.node_count, t.nodef, t.pf, t.mf);
}

void launchGravityWalkMixed(const DState& s, Tree& t, const Physics& ph, const float* lutF, uint32_t* devError,
    cudaStream_t st) {
    cudaMemsetAsync(t.stats, 0, 4 * sizeof(unsigned long long), st);
    if (s.n == 0 || t.node_count == 0) {
        return;
    }
    launchPrepareWalk(s, t, ph, st);
    const int blocks = int(t.walk_warps / (WALK_THREADS_F / 32));
    walkMixedKernel<<<blocks, WALK_THREADS_F, 0, st>>>(t.idx, t.geom, t.nodef, t.pf, t.mf, t.leaves, t.leaf_count,
        lutF, ph.kernel_radius, ph.multipole_order, t.walk_scratch, t.walk_capacity, s.agrav, t.stats, devError);
}

} // namespace sphgpu
