// walk64.cu — phase 2 of the FP64 Barnes-Hut walk (the plain FP64 path): for every leaf, the interaction lists of
// its ancestors, built once per node by the list phase shared with the mixed walk (gravity32.cu: the reference's
// dual-walk classification, core/gravity/BarnesHut.cpp:212-312, decided exactly as the reference decides it), and
// the pairs inside the leaf, evaluated in FP64.
//
// The evaluation is the reference's mathematics in FP64 with a different grouping of the operations:
//   * multipoles (evaluateGravity, core/gravity/Moments.h:336-360): the same monopole, quadrupole and octupole
//     terms, regrouped around the unit separation u = x / |x| and the ten distinct octupole components, with one
//     reciprocal square root for all powers of 1 / |x|;
//   * pairs (GravityLutKernel::grad, core/sph/kernel/GravityKernel.h:69-80 with symmetrized h): the reference's
//     arithmetic in its order, explicitly rounded, with 1 / |r|^3 from one reciprocal square root; a pair farther
//     than the kernel support by a relative margin of 1e-10 takes the point-mass branch directly, without the
//     reference's division by h (whose own test would choose the same branch);
//   * sums in FP64.
// Every term differs from the reference's in the last bits only (the results agree to about 1e-15 of the
// acceleration scale). The translation unit is compiled with contraction allowed; what must be the reference's
// arithmetic to the bit (node geometry, moments, the sphere-box tests) lives in the units compiled without it.
//
// Work layout: a warp per leaf, taken from a global counter, a lane per particle of the leaf. Each particle sums
// its terms in one fixed order (the particle lists and node lists of its ancestors from the root down, then the
// pairs inside its leaf) whatever the lane layout. Splitting a small leaf's sources among several lane groups
// would run about 1.3x faster but reorders the sums, and a last-bit change in the accelerations is enough to
// change which hard-sphere collisions the N-body solver finds within a step: the collision sequences of the
// reference's N-body runs are reproduced with the fixed order and not without it.
//
// A tree of few leaves (fewer than the resident warps) leaves most of the FP64 units idle with a warp per leaf:
// there, outside the N-body solver, each leaf is taken by S <= 8 warps ("slices"): slice s evaluates the source
// particles s, s + S, s + 2 S, ... of every source leaf and of the leaf itself, and the nodes at positions s,
// s + S, ... of the node lists in the fixed order above, into its own partial sums, which a second kernel adds
// in slice order. The result is deterministic for a given tree; it differs from the single-slice order in the
// last bits.
#include <algorithm>

#include "tree.cuh"

namespace sphgpu {
namespace {

constexpr int WALK64_THREADS = 128;

// evaluateGravity at x = com - r_i (the reference's dr = r_i - com, negated), added into b
__device__ __forceinline__ void multipoleAcc64(double x, double y, double z, const BhNodeMoments& mo, int order,
    double& bx, double& by, double& bz) {
    const double inv = rsqrt(fma(z, z, fma(y, y, x * x)));
    const double t = inv * inv;
    const double ux = x * inv, uy = y * inv, uz = z * inv;
    double A = mo.m0, cx = 0., cy = 0., cz = 0.;
    if (order >= 2) {
        // quadrupole: 15 Q0 x / |x|^7 - 3 Q1 / |x|^5 with Q1 = q2 x, Q0 = x.Q1 / 2
        const double qxx = mo.q2[0], qxy = mo.q2[1], qxz = mo.q2[2], qyy = mo.q2[3], qyz = mo.q2[4], qzz = mo.q2[5];
        const double Px = fma(qxz, uz, fma(qxy, uy, qxx * ux));
        const double Py = fma(qyz, uz, fma(qyy, uy, qxy * ux));
        const double Pz = fma(qzz, uz, fma(qyz, uy, qxz * ux));
        const double t2 = -3. * t;
        A = fma(-2.5 * t2, fma(Pz, uz, fma(Py, uy, Px * ux)), A);
        cx = t2 * Px;
        cy = t2 * Py;
        cz = t2 * Pz;
        if (order >= 3) {
            // octupole: -105 Q0 x / |x|^9 + 15 Q1 / |x|^7 with Q1_i = q3_ijk x_j x_k / 2, Q0 = x.Q1 / 3;
            // components xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz
            const double* q = mo.q3;
            const double t3 = t * inv;
            const double ux2 = ux + ux, uy2 = uy + uy;
            const double xx = ux * ux, yy = uy * uy, zz = uz * uz, xy2 = ux2 * uy, xz2 = ux2 * uz, yz2 = uy2 * uz;
            const double sx = fma(q[4], yz2, fma(q[2], xz2, fma(q[1], xy2, fma(q[5], zz, fma(q[3], yy, q[0] * xx)))));
            const double sy = fma(q[7], yz2, fma(q[4], xz2, fma(q[3], xy2, fma(q[8], zz, fma(q[6], yy, q[1] * xx)))));
            const double sz = fma(q[8], yz2, fma(q[5], xz2, fma(q[4], xy2, fma(q[9], zz, fma(q[7], yy, q[2] * xx)))));
            const double o3 = 7.5 * t3;
            A = fma(-17.5 * t3, fma(sz, uz, fma(sy, uy, sx * ux)), A);
            cx = fma(o3, sx, cx);
            cy = fma(o3, sy, cy);
            cz = fma(o3, sz, cz);
        }
    }
    bx = fma(t, fma(A, ux, cx), bx);
    by = fma(t, fma(A, uy, cy), by);
    bz = fma(t, fma(A, uz, cz), bz);
}

// m * grad of the gravity kernel at separation r = r_j - r_i with the symmetrized h, added into b. The products
// and sums are explicitly rounded in the reference's order (m * (r / |r|^3), the LUT branch m * ((h^-3 r) g)),
// with one reciprocal square root for 1 / |r|, so that a pair's term does not depend on contraction.
__device__ __forceinline__ void pairAcc64(double rx, double ry, double rz, double h, double m,
    const double* __restrict__ lut, double rad, double& bx, double& by, double& bz) {
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
    const double hr = h * rad;
    double gx, gy, gz;
    // farther than the support by a relative 1e-10: the reference's own test below takes the same branch
    bool far = r2 > (hr * hr) * (1. + 1.e-10);
    if (!far) {
        const double hInv = __drcp_rn(h);
        const double sx = __dmul_rn(rx, hInv), sy = __dmul_rn(ry, hInv), sz = __dmul_rn(rz, hInv);
        const double qSqr = __dadd_rn(__dadd_rn(__dmul_rn(sx, sx), __dmul_rn(sy, sy)), __dmul_rn(sz, sz));
        if (__dadd_rn(qSqr, SPH_EPS) >= __dmul_rn(rad, rad)) {
            far = true;
        } else {
            const double floatIdx = __dmul_rn(double(LUT_ENTRIES) * (1. / (2. * 2.)), qSqr);
            const int idx1 = int(floatIdx);
            const double ratio = __dsub_rn(floatIdx, double(idx1));
            const double l = __dadd_rn(__dmul_rn(__ldg(lut + idx1), __dsub_rn(1., ratio)),
                __dmul_rn(__ldg(lut + idx1 + 1), ratio));
            const double h3 = __dmul_rn(__dmul_rn(hInv, hInv), hInv);
            gx = __dmul_rn(__dmul_rn(h3, rx), l);
            gy = __dmul_rn(__dmul_rn(h3, ry), l);
            gz = __dmul_rn(__dmul_rn(h3, rz), l);
        }
    }
    if (far) {
        const double inv = rsqrt(r2);
        const double inv3 = __dmul_rn(__dmul_rn(inv, inv), inv);
        gx = __dmul_rn(rx, inv3);
        gy = __dmul_rn(ry, inv3);
        gz = __dmul_rn(rz, inv3);
    }
    bx = __dadd_rn(bx, __dmul_rn(m, gx));
    by = __dadd_rn(by, __dmul_rn(m, gy));
    bz = __dadd_rn(bz, __dmul_rn(m, gz));
}

__global__ void __launch_bounds__(WALK64_THREADS, 6) evalLists64Kernel(const dbl4* __restrict__ r,
    const double* __restrict__ m, double G, const uint32_t* __restrict__ idx, const BhNodeGeom* __restrict__ geom,
    const BhNodeMoments* __restrict__ mom, const uint32_t* __restrict__ leaves, uint32_t nLeaves,
    const double* __restrict__ lut, int kernelRadius, int order, const int32_t* __restrict__ pool,
    const uint32_t* __restrict__ meta, dbl4* agrav, unsigned long long* stats, uint32_t slices, dbl4* part,
    uint32_t n) {
    constexpr int W = WALK64_THREADS / 32;
    __shared__ int32_t pathSh[W][MAX_PATH_F];
    __shared__ unsigned long long countSh[W][4];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    int32_t* path = pathSh[wib];
    unsigned long long* wc = countSh[wib];
    const double rad = double(kernelRadius);
    if (lane < 4) {
        wc[lane] = 0;
    }
    __syncwarp();
    for (;;) {
        uint32_t item = 0;
        if (lane == 0) {
            item = uint32_t(atomicAdd(&stats[4], 1ull));
        }
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nLeaves * slices) {
            break;
        }
        const uint32_t li = item / slices, sl = item - li * slices;
        const int leaf = int(leaves[li]);
        const uint32_t from = geom[leaf].from, to = geom[leaf].to;
        const uint32_t cnt = to - from;
        // the root path, path[0] = root ... path[depth] = leaf
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
        const bool active = uint32_t(lane) < cnt;
        dbl4 ri = mkd4(0., 0., 0., 1.);
        if (active) {
            ri = r[idx[from + lane]];
        }
        double ax = 0., ay = 0., az = 0.;
        uint32_t leafN = 0, leafP = 0, leafSrc = 0;
        // the slice whose turn the next node is
        uint32_t turn = 0;
        for (int k = 1; k <= depth; ++k) {
            const uint32_t* mt = meta + size_t(path[k]) * NL_META;
            const uint32_t nOff = mt[0], nLen = mt[1], pOff = mt[2], pLen = mt[3];
            leafN += nLen;
            leafP += pLen;
            for (uint32_t c = 0; c < pLen; ++c) {
                const int pn = pool[pOff + c];
                const uint32_t f0 = geom[pn].from, f1 = geom[pn].to;
                leafSrc += f1 - f0;
                if (active) {
                    for (uint32_t t = f0 + sl; t < f1; t += slices) {
                        const uint32_t j = idx[t];
                        const dbl4 rj = r[j];
                        pairAcc64(rj.x - ri.x, rj.y - ri.y, rj.z - ri.z, 0.5 * (rj.w + ri.w), G * m[j], lut, rad, ax,
                            ay, az);
                    }
                }
            }
            for (uint32_t c = 0; c < nLen; ++c) {
                const bool mine = turn == sl;
                turn = turn + 1 == slices ? 0u : turn + 1;
                if (active && mine) {
                    const int nn = pool[nOff + c];
                    const BhNodeGeom& ng = geom[nn];
                    multipoleAcc64(ng.com[0] - ri.x, ng.com[1] - ri.y, ng.com[2] - ri.z, mom[nn], order, ax, ay, az);
                }
            }
        }
        // pairs inside the leaf
        if (active) {
            for (uint32_t t = from + sl; t < to; t += slices) {
                if (t != from + uint32_t(lane)) {
                    const uint32_t j = idx[t];
                    const dbl4 rj = r[j];
                    pairAcc64(rj.x - ri.x, rj.y - ri.y, rj.z - ri.z, 0.5 * (rj.w + ri.w), G * m[j], lut, rad, ax, ay,
                        az);
                }
            }
        }
        if (lane == 0 && sl == 0) {
            wc[0] += leafN;
            wc[1] += leafP;
            wc[2] += uint64_t(cnt) * leafN;
            wc[3] += uint64_t(cnt) * (leafSrc + cnt - 1);
        }
        if (active) {
            if (slices == 1) {
                agrav[idx[from + lane]] = mkd4(ax, ay, az, 0.);
            } else {
                part[size_t(sl) * n + from + lane] = mkd4(ax, ay, az, 0.);
            }
        }
        __syncwarp();
    }
    __syncwarp();
    if (lane < 4) {
        atomicAdd(&stats[lane], wc[lane]);
    }
}

// the partial sums of the slices, added in slice order, into the accelerations (tree slot k = particle idx[k])
__global__ void addSlicesKernel(const dbl4* __restrict__ part, uint32_t n, uint32_t slices,
    const uint32_t* __restrict__ idx, dbl4* agrav) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) {
        return;
    }
    dbl4 a = part[k];
    for (uint32_t sl = 1; sl < slices; ++sl) {
        const dbl4 b = part[size_t(sl) * n + k];
        a.x += b.x;
        a.y += b.y;
        a.z += b.z;
    }
    agrav[idx[k]] = mkd4(a.x, a.y, a.z, 0.);
}

} // namespace

void launchGravityWalk(const DState& s, Tree& t, const Physics& ph, const double* lut, uint32_t* devError,
    cudaStream_t st, cudaEvent_t evalStart, cudaEvent_t evalEnd) {
    cudaMemsetAsync(t.stats, 0, 5 * sizeof(unsigned long long), st);
    t.walk_launches = 0;
    if (s.n == 0 || t.node_count == 0) {
        return;
    }
    cudaMemsetAsync(s.agrav, 0, size_t(s.n) * sizeof(dbl4), st);
    if (ph.leaf_size > 32) {
        return;
    }
    launchWalkLists(s, t, devError, st);
    static int residentBlocks = 0;
    if (residentBlocks == 0) {
        int perSm = 0, sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, evalLists64Kernel, WALK64_THREADS, 0);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        residentBlocks = std::max(1, perSm * sms);
    }
    // slices per leaf: enough warps to fill the resident ones (never for the N-body solver, whose collision
    // sequences need the single fixed order)
    uint32_t slices = 1;
    if (!ph.nbody && t.leaf_count > 0) {
        const uint32_t residentWarps = uint32_t(residentBlocks) * (WALK64_THREADS / 32);
        slices = std::min(8u, std::max(1u, residentWarps / t.leaf_count));
        if (slices > 1 && t.slice_capacity < size_t(slices) * s.n) {
            if (t.slice_part) {
                cudaFree(t.slice_part);
            }
            t.slice_capacity = 0;
            if (cudaMalloc(&t.slice_part, size_t(slices) * s.n * sizeof(dbl4)) == cudaSuccess) {
                t.slice_capacity = size_t(slices) * s.n;
            } else {
                t.slice_part = nullptr;
                cudaGetLastError();
                slices = 1;
            }
        }
    }
    const int blocks =
        std::max(1, std::min(residentBlocks, ceilDiv(t.leaf_count * slices, WALK64_THREADS / 32)));
    if (evalStart) {
        cudaEventRecord(evalStart, st);
    }
    evalLists64Kernel<<<blocks, WALK64_THREADS, 0, st>>>(s.r, s.m, ph.G, t.idx, t.geom, t.mom, t.leaves,
        t.leaf_count, lut, ph.kernel_radius, ph.multipole_order, t.nl_pool, t.nl_meta, s.agrav, t.stats, slices,
        t.slice_part, s.n);
    t.walk_launches++;
    if (slices > 1) {
        addSlicesKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(t.slice_part, s.n, slices, t.idx, s.agrav);
        t.walk_launches++;
    }
    if (evalEnd) {
        cudaEventRecord(evalEnd, st);
    }
}

} // namespace sphgpu
