// gravity.cu — Barnes-Hut self-gravity in FP64 (compiled with -fmad=false).
//
// Replaces BarnesHut::build (moments) / evalSelfGravity / evalAcceleration (core/gravity/BarnesHut.cpp:50-175,
// 212-489) with the moments of core/gravity/Moments.h over the k-d tree of treebuild.cu. Moments are formed
// bottom-up in one launch (momentsUpKernel).
//
// Walk: the interaction lists of every node come from the list phase shared with the mixed walk (gravity32.cu:
// the reference's dual-walk classification, core/gravity/BarnesHut.cpp:212-312 with Sphere::intersectsBox,
// core/objects/geometry/Sphere.h:70-116, done once per node level by level, FP32-guarded with FP64 decisions at
// the margin), so every leaf receives exactly the reference's particle list and node list; walk64.cu evaluates
// them in FP64, a warp per leaf and a lane per particle.

#include <algorithm>

#include "tree.cuh"

namespace sphgpu {

namespace {


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

// the mixed walk's leaf: FP32 moments about the centre of mass (as leafMoments<float>, only for a leaf with mass)
// and, for every particle of the leaf, the evaluation inputs of the mixed walk: the position relative to the
// centre of mass with half the smoothing length (pf) and G m (mf), from the same FP64 differences
__device__ void leafMomentsMixed(const dbl4* __restrict__ r, const double* __restrict__ m, double G,
    const uint32_t* __restrict__ idx, const BhNodeGeom& g, bool massive, float q2[6], float q3[10], float4* pf,
    float* mf) {
    float M2[6] = { 0, 0, 0, 0, 0, 0 }, M3[10] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0 };
    for (uint32_t k = g.from; k < g.to; ++k) {
        const uint32_t i = idx[k];
        const dbl4 p = r[i];
        const float mi = float(G * m[i]);
        const float d[3] = { float(p.x - g.com[0]), float(p.y - g.com[1]), float(p.z - g.com[2]) };
        pf[k] = make_float4(d[0], d[1], d[2], 0.5f * float(p.w));
        mf[k] = mi;
        if (massive) {
            for (int a = 0; a < 3; ++a) {
                for (int b = a; b < 3; ++b) {
                    M2[i2(a, b)] += (d[a] * d[b]) * mi;
                    for (int c = b; c < 3; ++c) {
                        M3[i3(a, b, c)] += (d[a] * d[b] * d[c]) * mi;
                    }
                }
            }
        }
    }
    if (massive) {
        reduceMoments(M2, M3, q2, q3);
    }
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
__device__ void momentsUpLeaf(const dbl4* __restrict__ r, const double* __restrict__ m, double G,
    const uint32_t* __restrict__ idx, double thetaInv, BhNodeGeom* geom, BhNodeMoments* mom, float* nodef, int node,
    uint32_t* visits, float4* pf, float* mf) {
    int parent;
    {
        BhNodeGeom g = geom[node];
        if (Mixed) {
            double m0;
            float q2[6] = { 0, 0, 0, 0, 0, 0 }, q3[10] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0 };
            const bool massive = buildLeafGeom(r, m, G, idx, thetaInv, g, m0);
            leafMomentsMixed(r, m, G, idx, g, massive, q2, q3, pf, mf);
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

template <bool Mixed>
__global__ void momentsUpKernel(const dbl4* __restrict__ r, const double* __restrict__ m, double G,
    const uint32_t* __restrict__ idx, double thetaInv, BhNodeGeom* geom, BhNodeMoments* mom, float* nodef,
    const uint32_t* __restrict__ leaves, const uint32_t* __restrict__ leafCount, uint32_t maxLeaves,
    uint32_t* visits, float4* pf, float* mf) {
    const uint32_t nLeaves = min(*leafCount, maxLeaves);
    for (uint32_t li = blockIdx.x * blockDim.x + threadIdx.x; li < nLeaves; li += gridDim.x * blockDim.x) {
        momentsUpLeaf<Mixed>(r, m, G, idx, thetaInv, geom, mom, nodef, int(leaves[li]), visits, pf, mf);
    }
}

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

// BruteForceGravity::evalSelfGravity for listed particles (core/gravity/BruteForceGravity.h:38-58, evalImpl
// :110-129): a_i = G sum_{j != i} m_j grad(r_j - r_i) with the symmetrised smoothing length, in FP64 and in index
// order, as the reference sums it. One thread per target; the sources in tiles staged in shared memory.
constexpr int DIRECT_THREADS = 128;

__global__ void __launch_bounds__(DIRECT_THREADS) directKernel(const dbl4* __restrict__ r,
    const double* __restrict__ m, double G, uint32_t n, const uint32_t* __restrict__ targets, uint32_t nt,
    const double* __restrict__ lut, int kernelRadius, dbl4* acc) {
    __shared__ dbl4 shR[DIRECT_THREADS];
    __shared__ double shM[DIRECT_THREADS];
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = k < nt;
    const uint32_t i = valid ? targets[k] : 0u;
    const dbl4 ri = valid && i < n ? r[i] : mkd4(0., 0., 0., 0.);
    double ax = 0., ay = 0., az = 0.;
    for (uint32_t base = 0; base < n; base += DIRECT_THREADS) {
        const uint32_t j = base + threadIdx.x;
        if (j < n) {
            shR[threadIdx.x] = r[j];
            shM[threadIdx.x] = m[j];
        }
        __syncthreads();
        const uint32_t cnt = min(uint32_t(DIRECT_THREADS), n - base);
        if (valid) {
            for (uint32_t t = 0; t < cnt; ++t) {
                if (base + t == i) {
                    continue;
                }
                const dbl4 rj = shR[t];
                double gx, gy, gz;
                gravGrad(rj.x - ri.x, rj.y - ri.y, rj.z - ri.z, 0.5 * (rj.w + ri.w), lut, kernelRadius, gx, gy, gz);
                const double mj = shM[t];
                ax += mj * gx;
                ay += mj * gy;
                az += mj * gz;
            }
        }
        __syncthreads();
    }
    if (valid) {
        acc[k] = mkd4(G * ax, G * ay, G * az, 0.);
    }
}

// BarnesHut::evalAttractors (core/gravity/BarnesHut.cpp:100-125), attractor-particle part: thread i subtracts
// (G M_a) grad W(r_i - x_a, (h_i + R_a) / 2) of each attractor in order from dv_i (all four components: the
// reference scales the whole separation Vector); each block sums (G m_i) grad W per attractor in thread order
// into partial[block][a][3].
constexpr int ATT_THREADS = 256;

__device__ __forceinline__ void gravGrad4(const double r[4], double h, const double* __restrict__ lut,
    int kernelRadius, double g[4]) {
    const double hInv = 1. / h;
    const double sx = r[0] * hInv, sy = r[1] * hInv, sz = r[2] * hInv;
    const double qSqr = sx * sx + sy * sy + sz * sz;
    const double rad = double(kernelRadius);
    if (qSqr + SPH_EPS >= rad * rad) {
        const double len = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        const double l3 = len * len * len;
        for (int c = 0; c < 4; ++c) {
            g[c] = r[c] / l3;
        }
        return;
    }
    const double floatIdx = (double(LUT_ENTRIES) * (1. / (2. * 2.))) * qSqr;
    const int idx1 = int(floatIdx);
    const double ratio = floatIdx - double(idx1);
    const double gr = __ldg(lut + idx1) * (1. - ratio) + __ldg(lut + idx1 + 1) * ratio;
    const double h3 = hInv * hInv * hInv;
    for (int c = 0; c < 4; ++c) {
        g[c] = (h3 * r[c]) * gr;
    }
}

__global__ void __launch_bounds__(ATT_THREADS) attractorParticlesKernel(const dbl4* __restrict__ r,
    const double* __restrict__ m, double G, uint32_t n, const double* __restrict__ att, uint32_t count,
    const double* __restrict__ lut, int kernelRadius, dbl4* dv, double* partial) {
    __shared__ double sh[3][ATT_THREADS];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    dbl4 ri = mkd4(0., 0., 0., 0.), d = mkd4(0., 0., 0., 0.);
    double mi = 0.;
    if (valid) {
        ri = r[i];
        d = dv[i];
        mi = G * m[i];
    }
    for (uint32_t a = 0; a < count; ++a) {
        const double* xa = att + 5 * a;
        double f[4] = { 0., 0., 0., 0. };
        if (valid) {
            const double sep[4] = { ri.x - xa[0], ri.y - xa[1], ri.z - xa[2], ri.w - xa[3] };
            gravGrad4(sep, 0.5 * (ri.w + xa[3]), lut, kernelRadius, f);
            const double gm = G * xa[4];
            d.x -= gm * f[0];
            d.y -= gm * f[1];
            d.z -= gm * f[2];
            d.w -= gm * f[3];
        }
        for (int c = 0; c < 3; ++c) {
            sh[c][threadIdx.x] = mi * f[c];
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            double acc = 0.;
            for (int t = 0; t < ATT_THREADS; ++t) {
                acc += sh[threadIdx.x][t];
            }
            partial[(size_t(blockIdx.x) * count + a) * 3 + threadIdx.x] = acc;
        }
        __syncthreads();
    }
    if (valid) {
        dv[i] = d;
    }
}

// the attractors' accelerations: block partial sums in block order, then the attractor-attractor terms of each
// pair i < j in order (f = G grad W(x_i - x_j, (R_i + R_j) / 2), acc_i -= M_j f, acc_j += M_i f). One thread.
__global__ void attractorFinishKernel(const double* __restrict__ partial, uint32_t blocks, const double* __restrict__ att,
    uint32_t count, double G, const double* __restrict__ lut, int kernelRadius, double* acc) {
    for (uint32_t a = 0; a < count; ++a) {
        for (int c = 0; c < 3; ++c) {
            double s = acc[3 * a + c];
            for (uint32_t b = 0; b < blocks; ++b) {
                s += partial[(size_t(b) * count + a) * 3 + c];
            }
            acc[3 * a + c] = s;
        }
    }
    for (uint32_t i = 0; i < count; ++i) {
        for (uint32_t j = i + 1; j < count; ++j) {
            const double* xi = att + 5 * i;
            const double* xj = att + 5 * j;
            const double sep[4] = { xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2], xi[3] - xj[3] };
            double g[4];
            gravGrad4(sep, 0.5 * (xi[3] + xj[3]), lut, kernelRadius, g);
            for (int c = 0; c < 3; ++c) {
                const double f = G * g[c];
                acc[3 * i + c] -= xj[4] * f;
                acc[3 * j + c] += xi[4] * f;
            }
        }
    }
}

} // namespace

void launchGravityAttractors(const DState& s, const Physics& ph, const double* lut, const double* att, uint32_t count,
    dbl4* dv, double* partial, double* acc, cudaStream_t st) {
    const uint32_t blocks = s.n ? uint32_t(ceilDiv(s.n, ATT_THREADS)) : 0u;
    if (blocks && count) {
        attractorParticlesKernel<<<blocks, ATT_THREADS, 0, st>>>(s.r, s.m, ph.G, s.n, att, count, lut,
            ph.kernel_radius, dv, partial);
    }
    attractorFinishKernel<<<1, 1, 0, st>>>(partial, blocks, att, count, ph.G, lut, ph.kernel_radius, acc);
}

uint32_t gravityAttractorPartials(uint32_t n, uint32_t count) {
    return (n ? uint32_t(ceilDiv(n, ATT_THREADS)) : 0u) * count * 3u;
}

void launchGravityDirect(const DState& s, const Physics& ph, const double* lut, const uint32_t* targets, uint32_t nt,
    dbl4* acc, cudaStream_t st) {
    if (nt == 0) {
        return;
    }
    directKernel<<<ceilDiv(nt, DIRECT_THREADS), DIRECT_THREADS, 0, st>>>(s.r, s.m, ph.G, s.n, targets, nt, lut,
        ph.kernel_radius, acc);
}

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
    alloc((void**)&t.counters, C_WORDS * sizeof(uint32_t));
    alloc((void**)&t.leaves, nn * sizeof(uint32_t));
    alloc((void**)&t.visits, size_t(t.node_capacity) * sizeof(uint32_t));
    alloc((void**)&t.walk_scratch, size_t(t.walk_warps) * 2 * t.walk_capacity * sizeof(int32_t));
    alloc((void**)&t.stats, 8 * sizeof(unsigned long long)); // 4 interaction counters, [4] next leaf of the walk
    alloc((void**)&t.bbox, 8 * sizeof(unsigned long long));
    alloc((void**)&t.nodef, size_t(t.node_capacity) * NODEF * sizeof(float));
    alloc((void**)&t.pf, nn * sizeof(float4));
    alloc((void**)&t.mf, nn * sizeof(float));
    if (e == cudaSuccess) {
        e = treeBuildAllocate(t, nn);
    }
    return e;
}

cudaError_t treeGrowWalkScratch(Tree& t, uint32_t capacity) {
    if (capacity <= t.walk_capacity) {
        return cudaSuccess;
    }
    cudaFree(t.walk_scratch);
    t.walk_scratch = nullptr;
    t.walk_capacity = capacity;
    return cudaMalloc((void**)&t.walk_scratch, size_t(t.walk_warps) * 2 * t.walk_capacity * sizeof(int32_t));
}

void treeFree(Tree& t) {
    void* ptrs[] = { t.idx, t.scratch_b, t.scratch_s, t.geom, t.mom, t.seg[0], t.seg[1], t.counters, t.leaves, t.visits,
        t.walk_scratch, t.nl_pool, t.nl_kept[0], t.nl_kept[1], t.nl_meta, t.nl_counters, t.nl_defer, t.stats, t.bbox,
        t.nodef, t.pf, t.mf, t.slice_part };
    for (void* p : ptrs) {
        if (p) {
            cudaFree(p);
        }
    }
    if (t.nl_host) {
        cudaFreeHost(t.nl_host);
    }
    treeBuildFree(t);
    t = Tree();
}

void launchMomentsDev(const DState& s, Tree& t, const Physics& ph, bool mixed, cudaStream_t st) {
    cudaMemsetAsync(t.visits, 0, size_t(t.node_capacity) * sizeof(uint32_t), st);
    static int grid = 0;
    if (grid == 0) {
        int perSm = 0, sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, momentsUpKernel<false>, 128, 0);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = std::max(1, perSm * sms);
    }
    // the leaf count is read on the device (counters[C_LEAVES]); at most one leaf per particle
    const int blocks = std::max(1, std::min(grid, ceilDiv(s.n, 128)));
    if (mixed) {
        momentsUpKernel<true><<<blocks, 128, 0, st>>>(s.r, s.m, ph.G, t.idx, ph.theta_inv, t.geom, t.mom, t.nodef,
            t.leaves, t.counters + C_LEAVES, s.n, t.visits, t.pf, t.mf);
    } else {
        momentsUpKernel<false><<<blocks, 128, 0, st>>>(s.r, s.m, ph.G, t.idx, ph.theta_inv, t.geom, t.mom, t.nodef,
            t.leaves, t.counters + C_LEAVES, s.n, t.visits, t.pf, t.mf);
    }
}

void treeEnsureFp64Moments(const DState& s, Tree& t, const Physics& ph, cudaStream_t st) {
    if (t.built && t.mixed_moments) {
        launchMomentsDev(s, t, ph, false, st);
        t.mixed_moments = false;
    }
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
