// tree.cuh — Barnes-Hut helpers shared by the FP64 and mixed-precision tree walks: symmetric tensor
// indexing, the sphere-box classification of the dual walk, the softened gravity kernel and the
// multipole evaluation.
#pragma once

#include "state.h"

namespace sphgpu {
namespace {

// symmetric tensor index helpers: rank 2 {xx xy xz yy yz zz}, rank 3 {xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz}
__device__ __forceinline__ int i2(int a, int b) {
    const int lo = min(a, b), hi = max(a, b);
    return lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
}
__device__ __forceinline__ int i3(int a, int b, int c) {
    int x = a, y = b, z = c, t;
    if (x > y) {
        t = x;
        x = y;
        y = t;
    }
    if (y > z) {
        t = y;
        y = z;
        z = t;
    }
    if (x > y) {
        t = x;
        x = y;
        y = t;
    }
    // index of the sorted triple in {000 001 002 011 012 022 111 112 122 222}
    if (x == 0) {
        return y == 0 ? z : (y == 1 ? 2 + z : 5);
    }
    if (x == 1) {
        return y == 1 ? 5 + z : 8;
    }
    return 9;
}

// ---------------------------------------------------------------------------------------------------------
// evaluation helpers
// ---------------------------------------------------------------------------------------------------------

// GravityLutKernel::grad (core/sph/kernel/GravityKernel.h:69-80) of LutKernel<3>(GravityKernel<CubicSpline>)
__device__ __forceinline__ void gravGrad(double rx, double ry, double rz, double h, const double* __restrict__ lut,
    int kernelRadius, double& gx, double& gy, double& gz) {
    const double hInv = 1. / h;
    const double sx = rx * hInv, sy = ry * hInv, sz = rz * hInv;
    const double qSqr = sx * sx + sy * sy + sz * sz;
    const double rad = double(kernelRadius);
    if (qSqr + SPH_EPS >= rad * rad) {
        const double len = sqrt(rx * rx + ry * ry + rz * rz);
        const double l3 = len * len * len;
        gx = rx / l3;
        gy = ry / l3;
        gz = rz / l3;
        return;
    }
    const double floatIdx = (double(LUT_ENTRIES) * (1. / (2. * 2.))) * qSqr;
    const int idx1 = int(floatIdx);
    const double ratio = floatIdx - double(idx1);
    const double g = __ldg(lut + idx1) * (1. - ratio) + __ldg(lut + idx1 + 1) * ratio;
    const double h3 = hInv * hInv * hInv;
    gx = (h3 * rx) * g;
    gy = (h3 * ry) * g;
    gz = (h3 * rz) * g;
}

// evaluateGravity (core/gravity/Moments.h:336-360) at dr = r_i - com, accumulated into a
__device__ __forceinline__ void evalMultipole(double drx, double dry, double drz, const BhNodeMoments& mo, int order,
    double& ax, double& ay, double& az) {
    const double invDistSqr = 1. / (drx * drx + dry * dry + drz * drz);
    double gamma[5];
    gamma[0] = -sqrt(invDistSqr);
    for (int i = 1; i < 5; ++i) {
        gamma[i] = -(2. * i - 1.) * invDistSqr * gamma[i - 1];
    }
    const double x[3] = { -drx, -dry, -drz };
    double a[3] = { 0., 0., 0. };
    if (order >= 3) {
        double Q1[3], Q0 = 0.;
        for (int i = 0; i < 3; ++i) {
            double s = 0.;
            for (int j = 0; j < 3; ++j) {
                for (int k = 0; k < 3; ++k) {
                    s += mo.q3[i3(i, j, k)] * x[j] * x[k];
                }
            }
            Q1[i] = s * 0.5;
            Q0 += s * x[i];
        }
        Q0 *= 1. / 6.;
        for (int i = 0; i < 3; ++i) {
            a[i] += gamma[4] * x[i] * Q0 + gamma[3] * Q1[i];
        }
    }
    if (order >= 2) {
        double Q1[3], Q0 = 0.;
        for (int i = 0; i < 3; ++i) {
            Q1[i] = mo.q2[i2(i, 0)] * x[0] + mo.q2[i2(i, 1)] * x[1] + mo.q2[i2(i, 2)] * x[2];
            Q0 += Q1[i] * x[i];
        }
        Q0 *= 0.5;
        for (int i = 0; i < 3; ++i) {
            a[i] += gamma[3] * x[i] * Q0 + gamma[2] * Q1[i];
        }
    }
    for (int i = 0; i < 3; ++i) {
        a[i] += gamma[1] * x[i] * mo.m0;
    }
    ax += a[0];
    ay += a[1];
    az += a[2];
}

// Sphere::intersectsBox (core/objects/geometry/Sphere.h:70-116): 0 box outside, 1 intersection, 2 box inside the
// sphere. Every product and sum is an explicitly rounded intrinsic, never contracted into a fused multiply-add
// whatever the translation unit's flags, so that the decisions at the margin are the reference's (its squared
// lengths sum x, y, z left to right).
__device__ __forceinline__ double sqrLength3(double x, double y, double z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

__device__ int intersectsBox(const double p[3], double rad, const double lo[3], const double hi[3]) {
    double lft[3], rgt[3];
    for (int d = 0; d < 3; ++d) {
        lft[d] = fmax(__dsub_rn(lo[d], p[d]), 0.);
        rgt[d] = fmax(__dsub_rn(p[d], hi[d]), 0.);
    }
    const double rSqr = __dmul_rn(rad, rad);
    const double distSqr = __dsub_rn(__dsub_rn(rSqr, sqrLength3(lft[0], lft[1], lft[2])),
        sqrLength3(rgt[0], rgt[1], rgt[2]));
    if (!(distSqr > 0.)) {
        return 0;
    }
    const double sx = __dsub_rn(hi[0], lo[0]), sy = __dsub_rn(hi[1], lo[1]), sz = __dsub_rn(hi[2], lo[2]);
    const double vx[8] = { lo[0], __dadd_rn(lo[0], sx), lo[0], lo[0], hi[0], __dsub_rn(hi[0], sx), hi[0], hi[0] };
    const double vy[8] = { lo[1], lo[1], __dadd_rn(lo[1], sy), lo[1], hi[1], hi[1], __dsub_rn(hi[1], sy), hi[1] };
    const double vz[8] = { lo[2], lo[2], lo[2], __dadd_rn(lo[2], sz), hi[2], hi[2], hi[2], __dsub_rn(hi[2], sz) };
    for (int k = 0; k < 8; ++k) {
        const double d2 = sqrLength3(__dsub_rn(vx[k], p[0]), __dsub_rn(vy[k], p[1]), __dsub_rn(vz[k], p[2]));
        if (!(d2 < rSqr)) {
            return 1;
        }
    }
    return 2;
}

enum : int { CL_KEEP = 0, CL_PARTICLES = 1, CL_NODE = 2, CL_OPEN = 3 };

// Per-node FP32 record shared by both walks, 40 floats (160 B) in float4 groups so that every group is one
// vector load:
//   [0] com hi x, y, z, M0           [1] com lo x, y, z, signed r_open
//   [2] q2 xx xy xz yy  [3] q2 yz zz, q3 xxx xxy  [4] q3 xxz xyy xyz xzz  [5] q3 yyy yyz yzz zzz
//   [6] box lower corner hi  [7] box lower corner lo  [8] box upper corner hi  [9] box upper corner lo
// Centres and corners are unevaluated float pairs (hi + lo) of the FP64 values. The signed r_open is
// -r_open for leaves and +r_open for inner nodes; it is (either signed) zero exactly when the FP64 r_open is
// zero (a tiny positive r_open is stored as the smallest normal float).
// walk lists, per node: N offset, N length, P offset, P length, kept offset, kept length
constexpr int NL_META = 6;
constexpr int MAX_PATH_F = 512;

constexpr int NODEF = 40;
constexpr int NODEF4 = NODEF / 4;
constexpr int NF_COM_HI = 0;
constexpr int NF_COM_LO = 1;
constexpr int NF_MOM = 2;
constexpr int NF_BOX = 6;

__device__ __forceinline__ float4 nodeGroup(const float4* __restrict__ nf, int node, int group) {
    return __ldg(nf + size_t(node) * NODEF4 + group);
}

// Sphere::intersectsBox evaluated in FP32 on coordinates relative to the walking leaf's centre of mass,
// with a guard band: returns the reference's answer (0 outside, 1 intersection, 2 inside) whenever the FP32
// values are further from every decision threshold than their error bound, and -1 otherwise (the caller
// then decides in FP64). The inputs are FP64 quantities rounded once to FP32 (relative error <= 2^-24 of
// their magnitude) and every decision compares sums of a few squares of such values, so an error bound of
// 1e-5 of the largest squared magnitude involved is conservative by two orders of magnitude.
__device__ __forceinline__ int intersectsBoxGuarded(const float p[3], float rad, const float lo[3], const float hi[3]) {
    float l2 = 0.f, r2 = 0.f, pm = 0.f, em = 0.f;
    for (int d = 0; d < 3; ++d) {
        const float lft = fmaxf(lo[d] - p[d], 0.f);
        const float rgt = fmaxf(p[d] - hi[d], 0.f);
        l2 += lft * lft;
        r2 += rgt * rgt;
        pm = fmaxf(pm, fabsf(p[d]));
        em = fmaxf(em, fmaxf(fabsf(lo[d]), fabsf(hi[d])));
    }
    const float rSqr = rad * rad;
    const float s = pm + em;
    const float delta = 1.e-5f * (rSqr + 3.f * s * s);
    const float dist = rSqr - l2 - r2;
    if (dist < -delta) {
        return 0;
    }
    if (dist <= delta) {
        return -1;
    }
    bool ambiguous = false;
    for (int k = 0; k < 8; ++k) {
        const float vx = (k & 1) ? hi[0] : lo[0];
        const float vy = (k & 2) ? hi[1] : lo[1];
        const float vz = (k & 4) ? hi[2] : lo[2];
        const float dx = vx - p[0], dy = vy - p[1], dz = vz - p[2];
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 >= rSqr + delta) {
            return 1;
        }
        ambiguous = ambiguous || (d2 > rSqr - delta);
    }
    return ambiguous ? -1 : 2;
}

// The evaluated node (an ancestor of the walking leaf, or the leaf itself) of one level of the dual walk:
// its box relative to the leaf centre of mass in FP32; the FP64 box is read from the node only for the rare
// classifications that the guarded FP32 test leaves undecided.
struct WalkFrame {
    float elof[3], ehif[3];
    int ev;
    bool evLeaf;
};

// lh / ll: the leaf centre of mass as hi + lo floats
__device__ __forceinline__ void setFrame(WalkFrame& f, const float4* __restrict__ nf, int ev, bool evLeaf,
    const float lh[3], const float ll[3]) {
    const float4 lo_h = nodeGroup(nf, ev, NF_BOX), lo_l = nodeGroup(nf, ev, NF_BOX + 1);
    const float4 hi_h = nodeGroup(nf, ev, NF_BOX + 2), hi_l = nodeGroup(nf, ev, NF_BOX + 3);
    f.elof[0] = (lo_h.x - lh[0]) + (lo_l.x - ll[0]);
    f.elof[1] = (lo_h.y - lh[1]) + (lo_l.y - ll[1]);
    f.elof[2] = (lo_h.z - lh[2]) + (lo_l.z - ll[2]);
    f.ehif[0] = (hi_h.x - lh[0]) + (hi_l.x - ll[0]);
    f.ehif[1] = (hi_h.y - lh[1]) + (hi_l.y - ll[1]);
    f.ehif[2] = (hi_h.z - lh[2]) + (hi_l.z - ll[2]);
    f.ev = ev;
    f.evLeaf = evLeaf;
}

// FP64 sphere-box test of a node's opening sphere against the evaluated node's box, for the classifications
// the FP32 test leaves undecided (rare; kept out of line so that it adds no registers to the walk loops)
__device__ __noinline__ int intersectsNodeBox(const BhNodeGeom* __restrict__ geom, int node, int ev) {
    const BhNodeGeom& ng = geom[node];
    const BhNodeGeom& eg = geom[ev];
    return intersectsBox(ng.com, ng.r_open, eg.lo, eg.hi);
}

// Classification of one check-list entry against the evaluated node (BarnesHut::evalNode,
// core/gravity/BarnesHut.cpp:233-276): FP32 guarded test first, FP64 test only when it is undecided.
__device__ __forceinline__ int classifyEntry(int node, const BhNodeGeom* __restrict__ geom,
    const float4* __restrict__ nf, const WalkFrame& f, const float lh[3], const float ll[3]) {
    const float4 a = nodeGroup(nf, node, NF_COM_HI), b = nodeGroup(nf, node, NF_COM_LO);
    const float ro = fabsf(b.w);
    const bool leaf = signbit(b.w);
    if (ro == 0.f) {
        return CL_PARTICLES;
    }
    const float p[3] = { (a.x - lh[0]) + (b.x - ll[0]), (a.y - lh[1]) + (b.y - ll[1]), (a.z - lh[2]) + (b.z - ll[2]) };
    int res = intersectsBoxGuarded(p, ro, f.elof, f.ehif);
    if (res < 0) {
        res = intersectsNodeBox(geom, node, f.ev);
    }
    if (res == 2 || (f.evLeaf && res != 0)) {
        return leaf ? CL_PARTICLES : CL_OPEN;
    }
    return res == 0 ? CL_NODE : CL_KEEP;
}

} // namespace
} // namespace sphgpu
