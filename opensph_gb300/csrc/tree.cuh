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

// Sphere::intersectsBox: 0 box outside, 1 intersection, 2 box inside the sphere
__device__ int intersectsBox(const double p[3], double rad, const double lo[3], const double hi[3]) {
    double l2 = 0., r2 = 0.;
    for (int d = 0; d < 3; ++d) {
        const double lft = fmax(lo[d] - p[d], 0.);
        const double rgt = fmax(p[d] - hi[d], 0.);
        l2 = d == 0 ? lft * lft : l2 + lft * lft;
        r2 = d == 0 ? rgt * rgt : r2 + rgt * rgt;
    }
    const double rSqr = rad * rad;
    const double distSqr = rSqr - l2 - r2;
    if (!(distSqr > 0.)) {
        return 0;
    }
    const double sx = hi[0] - lo[0], sy = hi[1] - lo[1], sz = hi[2] - lo[2];
    const double vx[8] = { lo[0], lo[0] + sx, lo[0] + 0., lo[0] + 0., hi[0], hi[0] - sx, hi[0] - 0., hi[0] - 0. };
    const double vy[8] = { lo[1], lo[1] + 0., lo[1] + sy, lo[1] + 0., hi[1], hi[1] - 0., hi[1] - sy, hi[1] - 0. };
    const double vz[8] = { lo[2], lo[2] + 0., lo[2] + 0., lo[2] + sz, hi[2], hi[2] - 0., hi[2] - 0., hi[2] - sz };
    for (int k = 0; k < 8; ++k) {
        const double dx = vx[k] - p[0], dy = vy[k] - p[1], dz = vz[k] - p[2];
        if (!(dx * dx + dy * dy + dz * dz < rSqr)) {
            return 1;
        }
    }
    return 2;
}

enum : int { CL_KEEP = 0, CL_PARTICLES = 1, CL_NODE = 2, CL_OPEN = 3 };

// per-node FP32 record shared by both walks: com hi[3], com lo[3], m0, q2[6], q3[10], r_open, r_open == 0,
// box lower corner hi[3] + lo[3], box upper corner hi[3] + lo[3] (40 floats)
constexpr int NODEF = 40;
constexpr int NODEF_ROPEN = 23;
constexpr int NODEF_ZERO = 24;
constexpr int NODEF_BOX = 25;

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

// Classification of one check-list entry against the evaluated node (BarnesHut::evalNode,
// core/gravity/BarnesHut.cpp:233-276): FP32 guarded test first, FP64 test only when it is undecided.
struct WalkFrame {
    double elo[3], ehi[3];   // evaluated node box (FP64)
    float elof[3], ehif[3];  // the same relative to the leaf centre of mass (FP32)
    float lh[3], ll[3];      // leaf centre of mass as hi + lo floats
    bool evLeaf;
};

__device__ __forceinline__ int classifyEntry(int node, const BhNodeGeom* __restrict__ geom,
    const float* __restrict__ nodef, const WalkFrame& f) {
    const float* o = nodef + size_t(node) * NODEF;
    const BhNodeGeom& ng = geom[node];
    if (o[NODEF_ZERO] != 0.f) {
        return CL_PARTICLES;
    }
    const float p[3] = { (o[0] - f.lh[0]) + (o[3] - f.ll[0]), (o[1] - f.lh[1]) + (o[4] - f.ll[1]),
        (o[2] - f.lh[2]) + (o[5] - f.ll[2]) };
    int res = intersectsBoxGuarded(p, o[NODEF_ROPEN], f.elof, f.ehif);
    if (res < 0) {
        res = intersectsBox(ng.com, ng.r_open, f.elo, f.ehi);
    }
    if (res == 2 || (f.evLeaf && res != 0)) {
        return ng.left < 0 ? CL_PARTICLES : CL_OPEN;
    }
    return res == 0 ? CL_NODE : CL_KEEP;
}

// The evaluated node's box relative to the leaf centre, formed from hi + lo float pairs (no FP64 arithmetic);
// the FP64 box is loaded for the rare undecided classifications.
__device__ __forceinline__ void setFrame(WalkFrame& f, const BhNodeGeom& ev, const float* __restrict__ evf,
    bool evLeaf) {
    const float* b = evf + NODEF_BOX;
    for (int d = 0; d < 3; ++d) {
        f.elo[d] = ev.lo[d];
        f.ehi[d] = ev.hi[d];
        f.elof[d] = (b[d] - f.lh[d]) + (b[3 + d] - f.ll[d]);
        f.ehif[d] = (b[6 + d] - f.lh[d]) + (b[9 + d] - f.ll[d]);
    }
    f.evLeaf = evLeaf;
}


} // namespace
} // namespace sphgpu
