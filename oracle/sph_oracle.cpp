// sph_oracle.cpp — CPU oracle of OpenSPH's per-step hot path (TEST INFRASTRUCTURE, NOT THE PRODUCT).
//
// Plain C++ restatement of the reference algorithms that the GPU library replaces. Each function cites the
// reference file:line it follows. Arithmetic is written term by term in the reference's evaluation order
// and compiled without FP contraction (-ffp-contract=off), so every per-pair and per-particle term is the
// IEEE-identical value the reference computes; sums over neighbours are taken in gather form (each particle
// sums over all of its neighbours, the AsymmetricSolver form the reference proves equivalent,
// core/sph/solvers/test/Solvers.cpp:178-216), so totals differ from the reference's scatter order only by
// summation order. The Barnes-Hut k-d tree reproduces the reference partition exactly (Hoare partition with
// the same comparisons, the same sliding-midpoint rule and std::nth_element fallback).

#include "sph_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <thread>
#include <vector>

namespace {

// core/math/MathUtils.h:26-38: EPS and LARGE are float literals widened to double.
const double EPS = double(1.e-12f);
const double LARGE = double(1.e20f);
const double INFTY = std::numeric_limits<double>::max();
const double PI = 3.14159265358979323846264338327950288419716939937510;

int gThreads = 0;

int threadCount() {
    if (gThreads > 0) {
        return gThreads;
    }
    const unsigned hc = std::thread::hardware_concurrency();
    return hc ? int(hc) : 1;
}

void parallelFor(uint64_t n, const std::function<void(uint64_t, uint64_t)>& body, uint64_t grain = 64) {
    const int nt = threadCount();
    if (nt <= 1 || n <= grain) {
        body(0, n);
        return;
    }
    // dynamic chunks so that irregular work (tree walk, neighbour counts) balances
    const uint64_t chunk = std::max<uint64_t>(grain, n / (uint64_t(nt) * 16));
    std::atomic<uint64_t> next{ 0 };
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) {
        pool.emplace_back([&] {
            for (;;) {
                const uint64_t from = next.fetch_add(chunk);
                if (from >= n) {
                    return;
                }
                body(from, std::min(n, from + chunk));
            }
        });
    }
    for (auto& th : pool) {
        th.join();
    }
}

// ---------------------------------------------------------------------------------------------------------
// Small vector type with the reference's 4th (smoothing length) component
// ---------------------------------------------------------------------------------------------------------

struct V4 {
    double x, y, z, h;
};

inline V4 load4(const double* a, uint64_t i) {
    return V4{ a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3] };
}
inline void store4(double* a, uint64_t i, const V4& v) {
    a[4 * i] = v.x;
    a[4 * i + 1] = v.y;
    a[4 * i + 2] = v.z;
    a[4 * i + 3] = v.h;
}
inline V4 sub(const V4& a, const V4& b) {
    return V4{ a.x - b.x, a.y - b.y, a.z - b.z, a.h - b.h };
}
// core/objects/geometry/Vector.h:587-590 (dot on x, y, z, evaluated left to right)
inline double dot3(const V4& a, const V4& b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
inline double sqrLen(const V4& a) {
    return dot3(a, a);
}
inline V4 scale(const V4& a, double s) {
    return V4{ a.x * s, a.y * s, a.z * s, a.h * s };
}
inline V4 vmax(const V4& a, const V4& b) {
    return V4{ std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z), std::max(a.h, b.h) };
}
inline V4 vmin(const V4& a, const V4& b) {
    return V4{ std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z), std::min(a.h, b.h) };
}
inline double comp(const V4& a, int k) {
    return k == 0 ? a.x : (k == 1 ? a.y : (k == 2 ? a.z : a.h));
}
inline void setComp(V4& a, int k, double v) {
    (k == 0 ? a.x : (k == 1 ? a.y : (k == 2 ? a.z : a.h))) = v;
}

// ---------------------------------------------------------------------------------------------------------
// Kernels: LutKernel<3> of CubicSpline<3> and of GravityKernel<CubicSpline<3>>
// ---------------------------------------------------------------------------------------------------------

// core/sph/kernel/Kernel.h:150-188 (CubicSpline<3>, normalisation 1/pi)
double cubicValue(double qSqr) {
    const double norm = 1. / PI;
    const double q = std::sqrt(qSqr);
    if (q < 1.) {
        const double a = 2. - q, b = 1. - q;
        return norm * (0.25 * (a * a * a) - (b * b * b));
    }
    if (q < 2.) {
        const double a = 2. - q;
        return norm * (0.25 * (a * a * a));
    }
    return 0.;
}
double cubicGrad(double qSqr) {
    const double norm = 1. / PI;
    const double q = std::sqrt(qSqr);
    if (q == 0.) {
        return -3. * norm;
    }
    if (q < 1.) {
        const double a = 2. - q, b = 1. - q;
        return (1. / q) * norm * (-0.75 * (a * a) + 3. * (b * b));
    }
    if (q < 2.) {
        const double a = 2. - q;
        return (1. / q) * norm * (-0.75 * (a * a));
    }
    return 0.;
}
// core/sph/kernel/GravityKernel.h:84-118 (GravityKernel<CubicSpline<3>>)
double gravValue(double qSqr) {
    const double q = std::sqrt(qSqr);
    if (q < 1.) {
        const double q2 = q * q;
        return 2. / 3. * qSqr - 3. / 10. * (q2 * q2) + 1. / 10. * ((q2 * q2) * q) - 7. / 5.;
    }
    const double q2 = q * q;
    return 4. / 3. * qSqr - (q * q * q) + 3. / 10. * (qSqr * qSqr) - 1. / 30. * ((q2 * q2) * q) - 8. / 5. +
           1. / (15. * q);
}
double gravGrad(double qSqr) {
    const double q = std::sqrt(qSqr);
    if (q == 0.) {
        return 4. / 3.;
    }
    if (q < 1.) {
        return 1. / q * (4. / 3. * q - 6. / 5. * (q * q * q) + 1. / 2. * (qSqr * qSqr));
    }
    return 1. / q *
           (8. / 3. * q - 3. * qSqr + 6. / 5. * (q * q * q) - 1. / 6. * (qSqr * qSqr) - 1. / (15. * qSqr));
}

// core/sph/kernel/Kernel.h:51-145: 40,000 intervals in q^2 over [0, radius^2], linear interpolation
struct Lut {
    static const int NEntries = 40000;
    std::vector<double> values, grads;
    double rad = 0., qSqrToIdx = 0.;

    template <typename FV, typename FG>
    void init(double radius, FV fv, FG fg) {
        rad = radius;
        const double radInvSqr = 1. / (rad * rad);
        qSqrToIdx = double(NEntries) * radInvSqr;
        values.resize(NEntries + 1);
        grads.resize(NEntries + 1);
        for (int i = 0; i < NEntries + 1; ++i) {
            const double qSqr = double(i) / qSqrToIdx;
            values[i] = fv(qSqr);
            grads[i] = fg(qSqr);
        }
    }
    double value(double qSqr) const {
        if (qSqr >= rad * rad) {
            return 0.;
        }
        const double floatIdx = qSqrToIdx * qSqr;
        const int idx1 = int(floatIdx);
        const double ratio = floatIdx - double(idx1);
        return values[idx1] * (1. - ratio) + values[idx1 + 1] * ratio;
    }
    double grad(double qSqr) const {
        if (qSqr >= rad * rad) {
            return 0.;
        }
        const double floatIdx = qSqrToIdx * qSqr;
        const int idx1 = int(floatIdx);
        const double ratio = floatIdx - double(idx1);
        return grads[idx1] * (1. - ratio) + grads[idx1 + 1] * ratio;
    }
};

const Lut& sphLut() {
    static const Lut lut = [] {
        Lut l;
        l.init(2., cubicValue, cubicGrad);
        return l;
    }();
    return lut;
}
const Lut& gravLut() {
    static const Lut lut = [] {
        Lut l;
        l.init(2., gravValue, gravGrad);
        return l;
    }();
    return lut;
}

// Kernel::grad (core/sph/kernel/Kernel.h:32-36) on x, y, z: r * h^-5 * W'(q^2)/q
inline V4 sphGrad(const V4& r, double h) {
    const double hInv = 1. / h;
    const double h2 = hInv * hInv;
    const double h5 = (h2 * h2) * hInv;
    const double g = sphLut().grad(sqrLen(r) * (hInv * hInv));
    return V4{ (r.x * h5) * g, (r.y * h5) * g, (r.z * h5) * g, 0. };
}

// LutKernel<3> of SolidSphereKernel (core/sph/kernel/GravityKernel.h:121-136): gradImpl = 1, radius 2
const Lut& solidLut() {
    static const Lut lut = [] {
        Lut l;
        l.init(
            2., [](double) { return 0.; }, [](double) { return 1.; });
        return l;
    }();
    return lut;
}

// GravityLutKernel::grad (core/sph/kernel/GravityKernel.h:69-80); kernelRadius 0 = point masses, 2 = the
// gravity kernel of the cubic spline, -2 = the solid-sphere kernel (radius 2)
inline V4 gravGradV(const V4& r, double h, int kernelRadius) {
    const double hInv = 1. / h;
    const V4 rh{ r.x * hInv, r.y * hInv, r.z * hInv, 0. };
    const double qSqr = sqrLen(rh);
    const double rad = double(kernelRadius < 0 ? -kernelRadius : kernelRadius);
    if (qSqr + EPS >= rad * rad) {
        const double len = std::sqrt(sqrLen(r));
        const double l3 = len * len * len;
        return V4{ r.x / l3, r.y / l3, r.z / l3, 0. };
    }
    const double g = (kernelRadius < 0 ? solidLut() : gravLut()).grad(qSqr);
    const double h3 = hInv * hInv * hInv;
    return V4{ (h3 * r.x) * g, (h3 * r.y) * g, (h3 * r.z) * g, 0. };
}

// ---------------------------------------------------------------------------------------------------------
// Materials: EOS, von Mises, Grady-Kipp
// ---------------------------------------------------------------------------------------------------------

// TillotsonEos::evaluate (core/physics/Eos.cpp:198-238), IdealGasEos::evaluate (:42-45)
void eosEval(const sphgpu_material& mt, double rho, double u, double& p, double& cs) {
    if (mt.eos == SPHGPU_EOS_IDEAL_GAS) {
        const double gamma = mt.adiabatic_index;
        p = (gamma - 1.) * u * rho;
        cs = std::sqrt(gamma * p / rho);
        return;
    }
    const double rho0 = mt.density, A = mt.bulk_modulus, B = mt.tillotson_nonlinear_b;
    const double a = mt.tillotson_small_a, b = mt.tillotson_small_b;
    const double alpha = mt.tillotson_alpha, beta = mt.tillotson_beta;
    const double u0 = mt.tillotson_sublimation, uiv = mt.tillotson_energy_iv, ucv = mt.tillotson_energy_cv;

    const double eta = rho / rho0;
    const double mu = eta - 1.;
    const double denom = u / (u0 * eta * eta) + 1.;
    const double pc = (a + b / denom) * rho * u + A * mu + B * mu * mu;
    double dpdu = a * rho + b * rho / (denom * denom);
    double dpdrho = a * u + b * u * (3. * denom - 2.) / (denom * denom) + A / rho0 + 2. * B * mu / rho0;
    const double csc = dpdrho + dpdu * pc / (rho * rho);

    const double rhoExp = rho0 / rho - 1.;
    const double betaExp = std::exp(-std::min(beta * rhoExp, 70.));
    const double alphaExp = std::exp(-std::min(alpha * (rhoExp * rhoExp), 70.));
    const double pe = a * rho * u + (b * rho * u / denom + A * mu * betaExp) * alphaExp;
    dpdu = a * rho + alphaExp * b * rho / (denom * denom);
    dpdrho = a * u + alphaExp * (b * u * (3. * denom - 2.) / (denom * denom)) +
             alphaExp * (b * u * rho / denom) * rho0 * (2. * alpha * rhoExp) / (rho * rho) +
             alphaExp * A * betaExp * (1. / rho0 + rho0 * mu / (rho * rho) * (2. * alpha * rhoExp + beta));
    double cse = dpdrho + dpdu * pe / (rho * rho);
    cse = std::max(cse, 0.);

    double pp = pc, cc = csc;
    if (rho <= rho0 && u > ucv) {
        pp = pe;
        cc = cse;
    } else if (rho <= rho0 && u > uiv && u <= ucv) {
        pp = ((u - uiv) * pe + (ucv - u) * pc) / (ucv - uiv);
        cc = ((u - uiv) * cse + (ucv - u) * csc) / (ucv - uiv);
    }
    cc = std::max(cc, 0.25 * A / rho0);
    p = pp;
    cs = std::sqrt(cc);
}

// traceless tensor {xx, yy, xy, xz, yz}; ddot (core/objects/geometry/TracelessTensor.h:388-390)
inline double ddotTT(const double* a, const double* b) {
    const double azz = -a[0] - a[1], bzz = -b[0] - b[1];
    const double d = a[0] * b[0] + a[1] * b[1] + azz * bzz;
    const double o = a[2] * b[2] + a[3] * b[3] + a[4] * b[4];
    return d + 2. * o;
}

// VonMisesRheology::initialize (core/physics/Rheology.cpp:36-83)
void vonMises(const sphgpu_material& mt, double u, double Dval, bool hasD, double& p, double* S, double& reduce) {
    const double d = hasD ? Dval * Dval * Dval : 0.;
    if (p < 0.) {
        p = (1. - d) * p;
    }
    const double unorm = u / mt.melt_energy;
    double Y = unorm < 1.e-5 ? mt.elasticity_limit : mt.elasticity_limit * std::max(1. - unorm, 0.);
    Y = (1. - d) * Y;
    if (Y < EPS) {
        reduce = 0.;
        for (int k = 0; k < 5; ++k) {
            S[k] = 0.;
        }
        return;
    }
    const double J2 = 0.5 * ddotTT(S, S) + 1.e-15;
    const double red = std::min(Y / std::sqrt(3. * J2), 1.);
    reduce = red;
    for (int k = 0; k < 5; ++k) {
        S[k] = S[k] * red;
    }
}

// sqrtApprox (core/math/MathUtils.h:42-62): one Newton step of the float inverse square root
double sqrtApprox(double f) {
    if (f == 0.) {
        return 0.;
    }
    int32_t i;
    const float x2 = float(f) * 0.5f;
    float y = float(f);
    std::memcpy(&i, &y, sizeof(float));
    i = 0x5f3759df - (i >> 1);
    std::memcpy(&y, &i, sizeof(float));
    const double inv = double(y * (1.5f - (x2 * y * y)));
    return 1. / inv;
}

// findEigenvalues (core/objects/geometry/SymmetricTensor.h:377-398) of {xx, yy, zz, xy, xz, yz}
void eigenvalues(const double* t, double sig[3]) {
    const double dx = t[0], dy = t[1], dz = t[2], ox = t[3], oy = t[4], oz = t[5];
    const double mx = std::max(dx, ox), my = std::max(dy, oy), mz = std::max(dz, oz);
    const double n = sqrtApprox(mx * mx + my * my + mz * mz);
    if (n < 1.e-12) {
        sig[0] = sig[1] = sig[2] = 0.;
        return;
    }
    const double inv1 = dx * 1. + dy * 1. + dz * 1.;
    const double inv2 = (ox * ox + oy * oy + oz * oz) - (dy * dz + dz * dx + dx * dy);
    const double inv3 = dx * dy * dz + 2 * ox * oy * oz - ((ox * ox) * dz + (oy * oy) * dy + (oz * oz) * dx);
    const double p = -inv1 / n;
    const double q = -inv2 / (n * n);
    const double r = -inv3 / (n * n * n);
    const double a = q - p * p / 3.;
    const double b = (2. * (p * p * p) - 9. * p * q + 27. * r) / 27.;
    const double aCub = (a * a * a) / 27.;
    if (0.25 * b * b + aCub >= 0.) {
        sig[0] = sig[1] = sig[2] = 0.;
        return;
    }
    const double t1 = 2. * std::sqrt(-a / 3.);
    const double phi = std::acos(-0.5 * b / std::sqrt(-aCub));
    const double v0 = phi / 3., v1 = (phi + 2 * PI) / 3., v2 = (phi + 4 * PI) / 3.;
    const double p3 = p / 3.;
    sig[0] = (t1 * std::cos(v0) - p3) * n;
    sig[1] = (t1 * std::cos(v1) - p3) * n;
    sig[2] = (t1 * std::cos(v2) - p3) * n;
}

// ScalarGradyKippModel::integrate (core/physics/Damage.cpp:128-170)
double gradyKipp(const sphgpu_material& mt, const double* S, double p, double D, double epsMin, double mZero,
    double growth, uint32_t nFlaws, double dDcur) {
    if (D >= mt.damage_range[1]) {
        return LARGE;
    }
    const double sigma[6] = { S[0] - p, S[1] - p, (-S[0] - S[1]) - p, S[2], S[3], S[4] };
    double sig[3];
    eigenvalues(sigma, sig);
    const double sigMax = std::max(std::max(sig[0], sig[1]), sig[2]);
    const double youngRed = std::max((1. - D * D * D) * mt.young_modulus, 1.e-20);
    const double strain = sigMax / youngRed;
    const double ratio = strain / epsMin;
    if (ratio <= 1.) {
        return dDcur;
    }
    return growth * std::cbrt(std::min(std::pow(ratio, mZero), double(nFlaws)));
}

// ---------------------------------------------------------------------------------------------------------
// Neighbour pairs (uniform grid, exact FP64 test of SymmetricSolver::loop)
// ---------------------------------------------------------------------------------------------------------

struct Neighbours {
    std::vector<uint64_t> start; // CSR over particles, all neighbours of each particle (both orientations)
    std::vector<uint32_t> idx;
};

inline bool interacts(const V4& ri, const V4& rj) {
    const double hbar = 0.5 * (ri.h + rj.h);
    const double rad = 2. * hbar;
    return sqrLen(sub(ri, rj)) < rad * rad;
}

Neighbours findNeighbours(uint64_t n, const double* r) {
    Neighbours out;
    out.start.assign(n + 1, 0);
    if (n == 0) {
        return out;
    }
    double hmax = 0.;
    V4 lo{ INFTY, INFTY, INFTY, 0 }, hi{ -INFTY, -INFTY, -INFTY, 0 };
    for (uint64_t i = 0; i < n; ++i) {
        const V4 p = load4(r, i);
        hmax = std::max(hmax, p.h);
        lo = vmin(lo, p);
        hi = vmax(hi, p);
    }
    const double cell = std::max(2. * hmax, 1e-300);
    int dims[3];
    for (int k = 0; k < 3; ++k) {
        const double ext = comp(hi, k) - comp(lo, k);
        dims[k] = std::max(1, std::min(1024, int(ext / cell) + 1));
    }
    auto cellOf = [&](const V4& p, int k) {
        int c = int((comp(p, k) - comp(lo, k)) / cell);
        return std::min(std::max(c, 0), dims[k] - 1);
    };
    const uint64_t ncell = uint64_t(dims[0]) * dims[1] * dims[2];
    std::vector<uint32_t> cellStart(ncell + 1, 0), sorted(n);
    std::vector<uint64_t> key(n);
    for (uint64_t i = 0; i < n; ++i) {
        const V4 p = load4(r, i);
        key[i] = (uint64_t(cellOf(p, 2)) * dims[1] + cellOf(p, 1)) * dims[0] + cellOf(p, 0);
        cellStart[key[i] + 1]++;
    }
    for (uint64_t c = 0; c < ncell; ++c) {
        cellStart[c + 1] += cellStart[c];
    }
    {
        std::vector<uint32_t> fill(cellStart.begin(), cellStart.end() - 1);
        for (uint64_t i = 0; i < n; ++i) {
            sorted[fill[key[i]]++] = uint32_t(i);
        }
    }
    std::vector<std::vector<uint32_t>> lists(n);
    parallelFor(n, [&](uint64_t from, uint64_t to) {
        for (uint64_t i = from; i < to; ++i) {
            const V4 ri = load4(r, i);
            const int cx = cellOf(ri, 0), cy = cellOf(ri, 1), cz = cellOf(ri, 2);
            for (int z = std::max(cz - 1, 0); z <= std::min(cz + 1, dims[2] - 1); ++z) {
                for (int y = std::max(cy - 1, 0); y <= std::min(cy + 1, dims[1] - 1); ++y) {
                    for (int x = std::max(cx - 1, 0); x <= std::min(cx + 1, dims[0] - 1); ++x) {
                        const uint64_t c = (uint64_t(z) * dims[1] + y) * dims[0] + x;
                        for (uint32_t s = cellStart[c]; s < cellStart[c + 1]; ++s) {
                            const uint32_t j = sorted[s];
                            if (j != i && interacts(ri, load4(r, j))) {
                                lists[i].push_back(j);
                            }
                        }
                    }
                }
            }
            std::sort(lists[i].begin(), lists[i].end());
        }
    });
    for (uint64_t i = 0; i < n; ++i) {
        out.start[i + 1] = out.start[i] + lists[i].size();
    }
    out.idx.resize(out.start[n]);
    for (uint64_t i = 0; i < n; ++i) {
        std::copy(lists[i].begin(), lists[i].end(), out.idx.begin() + out.start[i]);
    }
    return out;
}

// ---------------------------------------------------------------------------------------------------------
// Barnes-Hut: k-d tree (core/objects/finders/KdTree.inl.h:11-260), moments (core/gravity/Moments.h),
// dual tree walk (core/gravity/BarnesHut.cpp:86-362)
// ---------------------------------------------------------------------------------------------------------

struct Box {
    V4 lo{ INFTY, INFTY, INFTY, INFTY };
    V4 hi{ -INFTY, -INFTY, -INFTY, -INFTY };
    void extend(const V4& v) {
        hi = vmax(hi, v);
        lo = vmin(lo, v);
    }
    void extend(const Box& b) {
        hi = vmax(hi, b.hi);
        lo = vmin(lo, b.lo);
    }
    bool empty() const {
        return lo.x > hi.x; // default-constructed box (core/objects/geometry/Box.h)
    }
    V4 size() const {
        return sub(hi, lo);
    }
};

// symmetric rank-2: xx xy xz yy yz zz ; rank-3: xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz
inline int i2(int a, int b) {
    static const int t[3][3] = { { 0, 1, 2 }, { 1, 3, 4 }, { 2, 4, 5 } };
    return t[a][b];
}
// index of the symmetric rank-3 component (a, b, c) in {xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz}
static const int kI3[3][3][3] = { { { 0, 1, 2 }, { 1, 3, 4 }, { 2, 4, 5 } },
    { { 1, 3, 4 }, { 3, 6, 7 }, { 4, 7, 8 } },
    { { 2, 4, 5 }, { 4, 7, 8 }, { 5, 8, 9 } } };
inline int i3(int a, int b, int c) {
    return kI3[a][b][c];
}

struct BhNode {
    bool leaf = false;
    uint32_t from = 0, to = 0;
    int left = -1, right = -1;
    Box box;
    V4 com{ 0, 0, 0, 0 };
    double rOpen = 0.;
    double m0 = 0.;
    double q2[6] = { 0 };
    double q3[10] = { 0 };
};

// the kernel selector of BarnesHutTree / gravGradV for a configuration (GravityKernelEnum)
inline int kernelRadiusOf(const sphgpu_config& cfg) {
    switch (cfg.gravity_kernel) {
    case SPHGPU_GRAVITY_KERNEL_POINT_PARTICLES:
        return 0;
    case SPHGPU_GRAVITY_KERNEL_SOLID_SPHERES:
        return -2;
    default:
        return 2;
    }
}

struct BarnesHutTree {
    const double* r = nullptr;
    std::vector<double> m; // premultiplied by G
    std::vector<uint32_t> idxs;
    std::vector<BhNode> nodes;
    uint32_t leafSize = 25;
    double thetaInv = 2.;
    int order = 3;
    int kernelRadius = 2;
    std::atomic<uint64_t> nApprox{ 0 }, nExact{ 0 };

    V4 pt(uint32_t i) const {
        return load4(r, i);
    }
    double val(uint32_t k, int dim) const {
        return comp(pt(idxs[k]), dim);
    }

    // KdTree::isSingular (core/objects/finders/KdTree.inl.h:284-291)
    bool isSingular(uint32_t from, uint32_t to, int dim) const {
        for (uint32_t i = from; i < to; ++i) {
            if (val(i, dim) != val(to - 1, dim)) {
                return false;
            }
        }
        return true;
    }

    static int argMax(const V4& v) {
        int m = 0;
        if (v.y > comp(v, m)) {
            m = 1;
        }
        if (v.z > comp(v, m)) {
            m = 2;
        }
        return m;
    }

    // KdTree::buildTree (core/objects/finders/KdTree.inl.h:44-160), returns the node index
    int buildTree(uint32_t from, uint32_t to, const Box& box, uint32_t slidingCnt) {
        const int index = int(nodes.size());
        nodes.emplace_back();
        if (to - from <= leafSize) {
            BhNode& node = nodes[index];
            node.leaf = true;
            node.from = from;
            node.to = to;
            for (uint32_t i = from; i < to; ++i) {
                node.box.extend(pt(idxs[i]));
            }
            return index;
        }
        V4 boxSize = box.size();
        int splitIdx = argMax(boxSize);
        bool slidingMidpoint = false, degenerated = false;
        for (int dim = 0; dim < 3; ++dim) {
            if (isSingular(from, to, splitIdx)) {
                setComp(boxSize, splitIdx, 0.);
                splitIdx = argMax(boxSize);
                if (boxSize.x == 0. && boxSize.y == 0. && boxSize.z == 0.) {
                    degenerated = true;
                    break;
                }
            } else {
                break;
            }
        }
        const V4 center{ 0.5 * (box.lo.x + box.hi.x), 0.5 * (box.lo.y + box.hi.y), 0.5 * (box.lo.z + box.hi.z), 0 };
        double splitPosition = comp(center, splitIdx);
        int64_t n1 = from, n2 = int64_t(to) - 1;
        Box box1 = box, box2 = box;
        if (slidingCnt <= 5 && !degenerated) {
            for (;; std::swap(idxs[n1], idxs[n2])) {
                for (; n1 < int64_t(to) && val(uint32_t(n1), splitIdx) <= splitPosition; ++n1)
                    ;
                for (; n2 >= int64_t(from) && val(uint32_t(n2), splitIdx) >= splitPosition; --n2)
                    ;
                if (n1 >= n2) {
                    break;
                }
            }
            if (n1 == int64_t(from)) {
                uint32_t idx = from;
                splitPosition = val(from, splitIdx);
                for (uint32_t i = from + 1; i < to; ++i) {
                    const double x1 = val(i, splitIdx);
                    if (x1 < splitPosition) {
                        idx = i;
                        splitPosition = x1;
                    }
                }
                std::swap(idxs[from], idxs[idx]);
                n1++;
                slidingMidpoint = true;
            } else if (n1 == int64_t(to)) {
                uint32_t idx = from;
                splitPosition = val(from, splitIdx);
                for (uint32_t i = from + 1; i < to; ++i) {
                    const double x2 = val(i, splitIdx);
                    if (x2 > splitPosition) {
                        idx = i;
                        splitPosition = x2;
                    }
                }
                std::swap(idxs[to - 1], idxs[idx]);
                n1--;
                slidingMidpoint = true;
            }
            setComp(box1.hi, splitIdx, splitPosition);
            setComp(box2.lo, splitIdx, splitPosition);
        } else {
            n1 = (int64_t(from) + int64_t(to)) >> 1;
            if (!degenerated) {
                const double* rr = r;
                const int dim = splitIdx;
                std::nth_element(idxs.begin() + from, idxs.begin() + n1, idxs.begin() + to,
                    [rr, dim](uint32_t i1, uint32_t i2) { return rr[4 * i1 + dim] < rr[4 * i2 + dim]; });
            }
            const double x = val(uint32_t(n1), splitIdx);
            setComp(box1.hi, splitIdx, x);
            setComp(box2.lo, splitIdx, x);
        }
        const uint32_t next = slidingMidpoint ? slidingCnt + 1 : 0;
        // the reference builds the right subtree first under the sequential scheduler; the partition of
        // the two halves is independent, so the order does not change the tree
        const int right = buildTree(uint32_t(n1), to, box2, next);
        const int left = buildTree(from, uint32_t(n1), box1, next);
        nodes[index].left = left;
        nodes[index].right = right;
        return index;
    }

    // BarnesHut::buildLeaf (core/gravity/BarnesHut.cpp:376-437)
    void buildLeaf(BhNode& leaf) {
        const uint32_t cnt = leaf.to - leaf.from;
        if (cnt == 0) {
            leaf.rOpen = 0.;
            return;
        }
        if (cnt == 1) {
            const uint32_t i = idxs[leaf.from];
            leaf.com = pt(i);
            leaf.m0 = m[i];
            leaf.rOpen = 0.;
            return;
        }
        V4 com{ 0, 0, 0, 0 };
        double mLeaf = 0.;
        for (uint32_t k = leaf.from; k < leaf.to; ++k) {
            const uint32_t i = idxs[k];
            const V4 p = pt(i);
            com = V4{ com.x + m[i] * p.x, com.y + m[i] * p.y, com.z + m[i] * p.z, com.h + m[i] * p.h };
            mLeaf += m[i];
        }
        com = V4{ com.x / mLeaf, com.y / mLeaf, com.z / mLeaf, com.h / mLeaf };
        leaf.com = com;
        const V4 rMax = vmax(sub(com, leaf.box.lo), sub(leaf.box.hi, com));
        leaf.rOpen = 2. / std::sqrt(3.) * thetaInv * std::sqrt(sqrLen(rMax));
        double M2[6] = { 0 }, M3[10] = { 0 };
        for (uint32_t k = leaf.from; k < leaf.to; ++k) {
            const uint32_t i = idxs[k];
            const V4 p = pt(i);
            const double d[3] = { p.x - com.x, p.y - com.y, p.z - com.z };
            for (int a = 0; a < 3; ++a) {
                for (int b = a; b < 3; ++b) {
                    M2[i2(a, b)] += (d[a] * d[b]) * m[i];
                    for (int c = b; c < 3; ++c) {
                        M3[i3(a, b, c)] += (d[a] * d[b] * d[c]) * m[i];
                    }
                }
            }
        }
        // computeReducedMultipole<2,3> (core/gravity/Moments.h:90-111)
        const double tr = M2[0] + M2[3] + M2[5];
        for (int a = 0; a < 3; ++a) {
            for (int b = a; b < 3; ++b) {
                leaf.q2[i2(a, b)] = M2[i2(a, b)] + (a == b ? tr : 0.) * (-1. / 3.);
            }
        }
        double T1[3];
        for (int k = 0; k < 3; ++k) {
            T1[k] = M3[i3(0, 0, k)] + M3[i3(1, 1, k)] + M3[i3(2, 2, k)];
        }
        for (int a = 0; a < 3; ++a) {
            for (int b = a; b < 3; ++b) {
                for (int c = b; c < 3; ++c) {
                    const double perm =
                        (a == b ? T1[c] : 0.) + (b == c ? T1[a] : 0.) + (c == a ? T1[b] : 0.);
                    leaf.q3[i3(a, b, c)] = M3[i3(a, b, c)] + perm * (-1. / 5.);
                }
            }
        }
        leaf.m0 = mLeaf;
    }

    // parallelAxisTheorem for orders 2 and 3 (core/gravity/Moments.h:182-295), accumulated into (q2, q3)
    static void shiftAdd(const BhNode& c, const double d[3], double q2[6], double q3[10]) {
        const double Q = c.m0;
        const double dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double Qd[3];
        for (int k = 0; k < 3; ++k) {
            Qd[k] = c.q2[i2(k, 0)] * d[0] + c.q2[i2(k, 1)] * d[1] + c.q2[i2(k, 2)] * d[2];
        }
        for (int a = 0; a < 3; ++a) {
            for (int b = a; b < 3; ++b) {
                const double f2 = d[a] * d[b] + (a == b ? dd : 0.) * (-1. / 3.);
                q2[i2(a, b)] += c.q2[i2(a, b)] + f2 * Q;
                for (int cc = b; cc < 3; ++cc) {
                    const double perm = (a == b ? d[cc] : 0.) + (b == cc ? d[a] : 0.) + (cc == a ? d[b] : 0.);
                    const double f3 = d[a] * d[b] * d[cc] + perm * dd * (-1. / 5.);
                    const double pq = c.q2[i2(a, b)] * d[cc] + c.q2[i2(b, cc)] * d[a] + c.q2[i2(cc, a)] * d[b];
                    const double t2 = (a == b ? Qd[cc] : 0.) + (a == cc ? Qd[b] : 0.) + (b == cc ? Qd[a] : 0.);
                    q3[i3(a, b, cc)] += c.q3[i3(a, b, cc)] + f3 * Q + pq + (-2. / 5.) * t2;
                }
            }
        }
    }

    // BarnesHut::buildInner (core/gravity/BarnesHut.cpp:439-489)
    void buildInner(BhNode& node, const BhNode& l, const BhNode& rr) {
        node.box = Box();
        node.box.extend(l.box);
        node.box.extend(rr.box);
        const double ml = l.m0, mr = rr.m0;
        if (ml + mr == 0.) {
            node.rOpen = 0.;
            return;
        }
        const double mt = ml + mr;
        node.com = V4{ (ml * l.com.x + mr * rr.com.x) / mt, (ml * l.com.y + mr * rr.com.y) / mt,
            (ml * l.com.z + mr * rr.com.z) / mt, (ml * l.com.h + mr * rr.com.h) / mt };
        const V4 rMax = vmax(sub(node.com, node.box.lo), sub(node.box.hi, node.com));
        node.rOpen = 2. / std::sqrt(3.) * thetaInv * std::sqrt(sqrLen(rMax));
        node.m0 = mt;
        std::fill(node.q2, node.q2 + 6, 0.);
        std::fill(node.q3, node.q3 + 10, 0.);
        const double dl[3] = { l.com.x - node.com.x, l.com.y - node.com.y, l.com.z - node.com.z };
        shiftAdd(l, dl, node.q2, node.q3);
        const double dr[3] = { rr.com.x - node.com.x, rr.com.y - node.com.y, rr.com.z - node.com.z };
        shiftAdd(rr, dr, node.q2, node.q3);
    }

    void buildMoments(int idx) {
        BhNode& node = nodes[idx];
        if (node.leaf) {
            buildLeaf(node);
            return;
        }
        buildMoments(node.left);
        buildMoments(node.right);
        buildInner(nodes[idx], nodes[nodes[idx].left], nodes[nodes[idx].right]);
    }

    void build(uint64_t n, const double* pos, const double* mass, double G) {
        r = pos;
        m.resize(n);
        for (uint64_t i = 0; i < n; ++i) {
            m[i] = G * mass[i];
        }
        idxs.resize(n);
        for (uint64_t i = 0; i < n; ++i) {
            idxs[i] = uint32_t(i);
        }
        nodes.clear();
        nodes.reserve(2 * n / std::max(1u, leafSize) + 16);
        if (n == 0) {
            return;
        }
        Box entire;
        for (uint64_t i = 0; i < n; ++i) {
            entire.extend(pt(uint32_t(i)));
        }
        buildTree(0, uint32_t(n), entire, 0);
        buildMoments(0);
    }

    // evaluateGravity (core/gravity/Moments.h:336-360) for dr = r_i - com
    V4 evalMultipole(const V4& dr, const BhNode& node) const {
        const double invDistSqr = 1. / sqrLen(dr);
        double gamma[5];
        gamma[0] = -std::sqrt(invDistSqr);
        for (int i = 1; i < 5; ++i) {
            gamma[i] = -(2. * i - 1.) * invDistSqr * gamma[i - 1];
        }
        const double x[3] = { -dr.x, -dr.y, -dr.z };
        double a[3] = { 0, 0, 0 };
        if (order >= 3) {
            double Q1[3] = { 0, 0, 0 };
            double Q0 = 0.;
            for (int i = 0; i < 3; ++i) {
                double s = 0.;
                for (int j = 0; j < 3; ++j) {
                    for (int k = 0; k < 3; ++k) {
                        s += node.q3[i3(i, j, k)] * x[j] * x[k];
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
                Q1[i] = node.q2[i2(i, 0)] * x[0] + node.q2[i2(i, 1)] * x[1] + node.q2[i2(i, 2)] * x[2];
                Q0 += Q1[i] * x[i];
            }
            Q0 *= 0.5;
            for (int i = 0; i < 3; ++i) {
                a[i] += gamma[3] * x[i] * Q0 + gamma[2] * Q1[i];
            }
        }
        for (int i = 0; i < 3; ++i) {
            a[i] += gamma[1] * x[i] * node.m0;
        }
        return V4{ a[0], a[1], a[2], 0. };
    }

    // Sphere::intersectsBox (core/objects/geometry/Sphere.h:70-116): 0 outside, 1 intersection, 2 inside
    static int intersects(const V4& p, double rad, const Box& box) {
        const V4 leftOf = vmax(sub(box.lo, p), V4{ 0, 0, 0, 0 });
        const V4 rightOf = vmax(sub(p, box.hi), V4{ 0, 0, 0, 0 });
        const double rSqr = rad * rad;
        const double distSqr = rSqr - sqrLen(leftOf) - sqrLen(rightOf);
        if (!(distSqr > 0.)) {
            return 0;
        }
        const V4 s = box.size();
        const V4 verts[8] = {
            box.lo,
            V4{ box.lo.x + s.x, box.lo.y + 0., box.lo.z + 0., 0 },
            V4{ box.lo.x + 0., box.lo.y + s.y, box.lo.z + 0., 0 },
            V4{ box.lo.x + 0., box.lo.y + 0., box.lo.z + s.z, 0 },
            box.hi,
            V4{ box.hi.x - s.x, box.hi.y - 0., box.hi.z - 0., 0 },
            V4{ box.hi.x - 0., box.hi.y - s.y, box.hi.z - 0., 0 },
            V4{ box.hi.x - 0., box.hi.y - 0., box.hi.z - s.z, 0 },
        };
        for (const V4& v : verts) {
            if (!(sqrLen(sub(v, p)) < rSqr)) {
                return 1;
            }
        }
        return 2;
    }

    // BarnesHut::evalParticleList + evalNodeList (core/gravity/BarnesHut.cpp:314-362), gather form
    void evalLeaf(const BhNode& leaf, const std::vector<int>& plist, const std::vector<int>& nlist, double* dv) {
        for (uint32_t a = leaf.from; a < leaf.to; ++a) {
            const uint32_t i = idxs[a];
            const V4 ri = pt(i);
            double acc[3] = { 0, 0, 0 };
            for (int pidx : plist) {
                const BhNode& other = nodes[pidx];
                for (uint32_t b = other.from; b < other.to; ++b) {
                    const uint32_t j = idxs[b];
                    const V4 rj = pt(j);
                    const V4 g = gravGradV(sub(rj, ri), 0.5 * (rj.h + ri.h), kernelRadius);
                    acc[0] += m[j] * g.x;
                    acc[1] += m[j] * g.y;
                    acc[2] += m[j] * g.z;
                }
            }
            for (uint32_t b = leaf.from; b < leaf.to; ++b) {
                if (b == a) {
                    continue;
                }
                const uint32_t j = idxs[b];
                const V4 rj = pt(j);
                const V4 g = gravGradV(sub(rj, ri), 0.5 * (rj.h + ri.h), kernelRadius);
                acc[0] += m[j] * g.x;
                acc[1] += m[j] * g.y;
                acc[2] += m[j] * g.z;
            }
            for (int nidx : nlist) {
                const V4 g = evalMultipole(sub(ri, nodes[nidx].com), nodes[nidx]);
                acc[0] += g.x;
                acc[1] += g.y;
                acc[2] += g.z;
            }
            dv[4 * i] += acc[0];
            dv[4 * i + 1] += acc[1];
            dv[4 * i + 2] += acc[2];
        }
        nExact += plist.size();
        nApprox += nlist.size();
    }

    // BarnesHut::evalNode (core/gravity/BarnesHut.cpp:212-312)
    void evalNode(int evalIdx, std::vector<int> check, std::vector<int> plist, std::vector<int> nlist, double* dv) {
        const BhNode& ev = nodes[evalIdx];
        if (ev.box.empty()) {
            return;
        }
        std::vector<int> keep;
        for (size_t k = 0; k < check.size(); ++k) {
            const int idx = check[k];
            const BhNode& node = nodes[idx];
            if (node.rOpen == 0.) {
                plist.push_back(idx);
                continue;
            }
            const int res = intersects(node.com, node.rOpen, ev.box);
            if (res == 2 || (ev.leaf && res != 0)) {
                if (node.leaf) {
                    plist.push_back(idx);
                } else {
                    check.push_back(node.left);
                    check.push_back(node.right);
                }
                continue;
            } else if (res == 0) {
                nlist.push_back(idx);
                continue;
            }
            keep.push_back(idx);
        }
        if (ev.leaf) {
            evalLeaf(ev, plist, nlist, dv);
            return;
        }
        std::vector<int> checkL = keep;
        checkL.push_back(ev.right);
        evalNode(ev.left, std::move(checkL), plist, nlist, dv);
        keep.push_back(ev.left);
        evalNode(ev.right, std::move(keep), std::move(plist), std::move(nlist), dv);
    }

    void evalSelfGravity(double* dv) {
        if (nodes.empty()) {
            return;
        }
        // expand the walk to a set of independent subtrees, then evaluate those in parallel
        struct Task {
            int node;
            std::vector<int> check, plist, nlist;
        };
        std::vector<Task> tasks{ Task{ 0, {}, {}, {} } };
        for (int level = 0; level < 12; ++level) {
            std::vector<Task> next;
            bool expanded = false;
            for (Task& t : tasks) {
                const BhNode& ev = nodes[t.node];
                if (ev.leaf || ev.box.empty()) {
                    next.push_back(std::move(t));
                    continue;
                }
                expanded = true;
                std::vector<int> check = t.check, keep;
                for (size_t k = 0; k < check.size(); ++k) {
                    const int idx = check[k];
                    const BhNode& node = nodes[idx];
                    if (node.rOpen == 0.) {
                        t.plist.push_back(idx);
                        continue;
                    }
                    const int res = intersects(node.com, node.rOpen, ev.box);
                    if (res == 2) {
                        if (node.leaf) {
                            t.plist.push_back(idx);
                        } else {
                            check.push_back(node.left);
                            check.push_back(node.right);
                        }
                        continue;
                    } else if (res == 0) {
                        t.nlist.push_back(idx);
                        continue;
                    }
                    keep.push_back(idx);
                }
                Task l{ ev.left, keep, t.plist, t.nlist };
                l.check.push_back(ev.right);
                Task r{ ev.right, keep, t.plist, t.nlist };
                r.check.push_back(ev.left);
                next.push_back(std::move(l));
                next.push_back(std::move(r));
            }
            tasks.swap(next);
            if (!expanded) {
                break;
            }
        }
        parallelFor(
            tasks.size(),
            [&](uint64_t from, uint64_t to) {
                for (uint64_t k = from; k < to; ++k) {
                    evalNode(tasks[k].node, tasks[k].check, tasks[k].plist, tasks[k].nlist, dv);
                }
            },
            1);
    }

    // BarnesHut::evalImpl / evalExact (core/gravity/BarnesHut.cpp:118-175, :364-374)
    V4 evalPoint(const V4& r0) const {
        double f[3] = { 0, 0, 0 };
        const double thetaSqr = 1. / (thetaInv * thetaInv);
        std::vector<int> stack{ 0 };
        while (!stack.empty()) {
            const int idx = stack.back();
            stack.pop_back();
            const BhNode& node = nodes[idx];
            if (node.box.empty()) {
                continue;
            }
            const V4 s = node.box.size();
            const double boxSizeSqr = sqrLen(s);
            const V4 c{ 0.5 * (node.box.lo.x + node.box.hi.x), 0.5 * (node.box.lo.y + node.box.hi.y),
                0.5 * (node.box.lo.z + node.box.hi.z), 0 };
            const double boxDistSqr = sqrLen(sub(c, r0));
            const bool contains = !(r0.x < node.box.lo.x || r0.x > node.box.hi.x || r0.y < node.box.lo.y ||
                                    r0.y > node.box.hi.y || r0.z < node.box.lo.z || r0.z > node.box.hi.z);
            if (!contains && boxSizeSqr > 0. && boxSizeSqr / (boxDistSqr + EPS) < thetaSqr) {
                const V4 g = evalMultipole(sub(r0, node.com), node);
                f[0] += g.x;
                f[1] += g.y;
                f[2] += g.z;
            } else if (node.leaf) {
                for (uint32_t k = node.from; k < node.to; ++k) {
                    const uint32_t i = idxs[k];
                    const V4 ri = pt(i);
                    const V4 g = gravGradV(sub(ri, r0), ri.h, kernelRadius);
                    f[0] += m[i] * g.x;
                    f[1] += m[i] * g.y;
                    f[2] += m[i] * g.z;
                }
            } else {
                stack.push_back(node.right);
                stack.push_back(node.left);
            }
        }
        return V4{ f[0], f[1], f[2], 0 };
    }
};

// ---------------------------------------------------------------------------------------------------------
// Solver: SymmetricSolver::integrate with GravitySolver::loop (core/sph/solvers/SymmetricSolver.cpp:58-141,
// core/sph/solvers/GravitySolver.cpp:64-91) in gather form
// ---------------------------------------------------------------------------------------------------------

struct Flags {
    bool solid, gravity, adaptive, sumOnlyUndamaged;
};

Flags flagsOf(const sphgpu_config& cfg, const ora_state& s) {
    Flags f;
    f.solid = (cfg.forces & SPHGPU_FORCE_SOLID_STRESS) != 0 && s.S != nullptr;
    f.gravity = (cfg.forces & SPHGPU_FORCE_SELF_GRAVITY) != 0;
    f.adaptive = cfg.adaptive_smoothing_length != 0;
    f.sumOnlyUndamaged = f.solid && cfg.sum_only_undamaged && s.reduce != nullptr;
    return f;
}

const sphgpu_material& matOf(const sphgpu_config& cfg, const ora_state& s, uint64_t i) {
    const uint32_t k = s.mat ? s.mat[i] : 0;
    return cfg.materials[k < cfg.material_count ? k : 0];
}

bool hasRheology(const sphgpu_material& mt) {
    return mt.yielding != SPHGPU_YIELDING_NONE;
}

// CachedGravity (core/gravity/CachedGravity.h:45-63): the run time of the current step and the accelerations
// of the last evaluation, reused while the run time is less than the recomputation period after it and the
// particle count is unchanged (reset at the start of every run)
struct GravityCache {
    double runTime = 0.;
    double tLast = -INFINITY;
    uint64_t n = 0;
    std::vector<double> acc;
};
GravityCache gCache;

// BarnesHut::evalSelfGravity into acc (4n, zeroed), through the cache for a positive recomputation period
void selfGravity(const sphgpu_config& cfg, uint64_t n, const double* r, const double* m, std::vector<double>& acc) {
    const double period = cfg.gravity_recomputation_period;
    if (period > 0. && gCache.n == n && gCache.runTime - gCache.tLast < period) {
        acc = gCache.acc;
        return;
    }
    BarnesHutTree bh;
    bh.leafSize = cfg.gravity_leaf_size;
    bh.thetaInv = 1. / cfg.gravity_opening_angle;
    bh.order = cfg.gravity_multipole_order;
    bh.kernelRadius = kernelRadiusOf(cfg);
    bh.build(n, r, m, cfg.gravity_constant);
    bh.evalSelfGravity(acc.data());
    if (period > 0.) {
        gCache.acc = acc;
        gCache.n = n;
        gCache.tLast = gCache.runTime;
    }
}

void integrate(const sphgpu_config& cfg, ora_state& s) {
    const uint64_t n = s.n;
    const Flags fl = flagsOf(cfg, s);
    // materials initialize (core/sph/Materials.cpp:47-58, 74-79)
    parallelFor(n, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; ++i) {
            const sphgpu_material& mt = matOf(cfg, s, i);
            eosEval(mt, s.rho[i], s.u[i], s.p[i], s.cs[i]);
            if (fl.solid && hasRheology(mt)) {
                vonMises(mt, s.u[i], s.D ? s.D[i] : 0., s.D != nullptr && mt.damage != SPHGPU_DAMAGE_NONE,
                    s.p[i], s.S + 5 * i, s.reduce[i]);
            }
        }
    });
    // equations initialize: AdaptiveSmoothingLength clamps h (core/sph/equations/EquationTerm.cpp:356-364)
    if (fl.adaptive) {
        for (uint64_t i = 0; i < n; ++i) {
            const double h = s.r[4 * i + 3];
            s.r[4 * i + 3] = std::max(cfg.smoothing_length_range[0], std::min(h, cfg.smoothing_length_range[1]));
        }
    }
    // gravity into the acceleration buffer (GravitySolver::loop)
    std::vector<double> acc(4 * n, 0.);
    if (fl.gravity) {
        selfGravity(cfg, n, s.r, s.m, acc);
    }
    // pair loop
    const Neighbours nb = findNeighbours(n, s.r);
    const double alpha = cfg.av_alpha, beta = cfg.av_beta;
    // CorrectionTensor (core/sph/equations/Derivative.cpp:36-74), a PRECOMPUTE derivative of the
    // AsymmetricSolver: C_i = (sum_j m_j / rho_j sym((r_j - r_i) x grad W_ij))^-1, identity when the sum is null
    // or its determinant is at most 0.01
    const bool corrected = fl.solid && cfg.correction_tensor != 0;
    std::vector<double> corr;
    if (corrected) {
        corr.assign(6 * n, 0.);
        parallelFor(n, [&](uint64_t a, uint64_t b) {
            for (uint64_t i = a; i < b; ++i) {
                const V4 ri = load4(s.r, i);
                double c[6] = { 0, 0, 0, 0, 0, 0 };
                for (uint64_t k = nb.start[i]; k < nb.start[i + 1]; ++k) {
                    const uint32_t j = nb.idx[k];
                    if (fl.sumOnlyUndamaged && (s.flag[i] != s.flag[j] || s.reduce[i] == 0. || s.reduce[j] == 0.)) {
                        continue;
                    }
                    const V4 rj = load4(s.r, j);
                    const V4 grad = sphGrad(sub(ri, rj), 0.5 * (ri.h + rj.h));
                    const V4 e = sub(rj, ri);
                    const double f = s.m[j] / s.rho[j];
                    c[0] += f * (e.x * grad.x);
                    c[1] += f * (e.y * grad.y);
                    c[2] += f * (e.z * grad.z);
                    c[3] += f * (0.5 * (e.x * grad.y + e.y * grad.x));
                    c[4] += f * (0.5 * (e.x * grad.z + e.z * grad.x));
                    c[5] += f * (0.5 * (e.y * grad.z + e.z * grad.y));
                }
                const bool isNull = c[0] == 0. && c[1] == 0. && c[2] == 0. && c[3] == 0. && c[4] == 0. && c[5] == 0.;
                const double det = c[0] * c[1] * c[2] + 2. * c[3] * c[4] * c[5] -
                                   (c[3] * c[3] * c[2] + c[4] * c[4] * c[1] + c[5] * c[5] * c[0]);
                double* out = corr.data() + 6 * i;
                double* dst = s.corr ? s.corr + 6 * i : nullptr;
                if (isNull || !(det > 0.01)) {
                    out[0] = out[1] = out[2] = 1.;
                    out[3] = out[4] = out[5] = 0.;
                } else {
                    out[0] = (c[1] * c[2] - c[5] * c[5]) / det;
                    out[1] = (c[2] * c[0] - c[4] * c[4]) / det;
                    out[2] = (c[0] * c[1] - c[3] * c[3]) / det;
                    out[3] = (c[4] * c[5] - c[2] * c[3]) / det;
                    out[4] = (c[5] * c[3] - c[1] * c[4]) / det;
                    out[5] = (c[3] * c[4] - c[0] * c[5]) / det;
                }
                if (dst) {
                    std::copy(out, out + 6, dst);
                }
            }
        });
    }
    parallelFor(n, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; ++i) {
            const V4 ri = load4(s.r, i), vi = load4(s.v, i);
            const double rhoi = s.rho[i], pi = s.p[i], csi = s.cs[i];
            double ax = acc[4 * i], ay = acc[4 * i + 1], az = acc[4 * i + 2];
            double du = 0., divv = 0.;
            double gv[6] = { 0, 0, 0, 0, 0, 0 };
            uint32_t cnt = 0;
            for (uint64_t k = nb.start[i]; k < nb.start[i + 1]; ++k) {
                const uint32_t j = nb.idx[k];
                const V4 rj = load4(s.r, j), vj = load4(s.v, j);
                const double hbar = 0.5 * (ri.h + rj.h);
                const V4 grad = sphGrad(sub(ri, rj), hbar);
                const double mj = s.m[j], rhoj = s.rho[j];
                cnt++;
                // VelocityDivergence<CenterDensityDiscr> (DerivativeHelpers.h:292-361)
                const V4 dvji = sub(vj, vi);
                divv += mj / rhoi * dot3(dvji, grad);
                // PressureGradient<StandardForceDiscr> (EquationTerm.cpp:12-66)
                {
                    const double pr = pi / (rhoi * rhoi) + s.p[j] / (rhoj * rhoj);
                    ax += mj * -(pr * grad.x);
                    ay += mj * -(pr * grad.y);
                    az += mj * -(pr * grad.z);
                }
                // StandardAV (core/sph/equations/av/Standard.h:63-83)
                {
                    const V4 dvij = sub(vi, vj);
                    const V4 drij = sub(ri, rj);
                    const double dvdr = dot3(dvij, drij);
                    double av = 0.;
                    if (!(dvdr >= 0.)) {
                        const double rhobar = 0.5 * (rhoi + rhoj);
                        const double csbar = 0.5 * (csi + s.cs[j]);
                        const double mu = hbar * dvdr / (sqrLen(drij) + 1.e-2 * (hbar * hbar));
                        av = 1. / rhobar * (-alpha * csbar * mu + beta * (mu * mu));
                    }
                    ax += mj * -(av * grad.x);
                    ay += mj * -(av * grad.y);
                    az += mj * -(av * grad.z);
                    du += mj * (0.5 * av * dot3(dvij, grad));
                }
                if (fl.solid) {
                    const bool undamaged = !fl.sumOnlyUndamaged ||
                                           (s.flag[i] == s.flag[j] && s.reduce[i] != 0. && s.reduce[j] != 0.);
                    if (undamaged) {
                        // VelocityGradient (DerivativeHelpers.h:347-361, SymmetricTensor.h:362-368), with the
                        // corrected gradient C_i grad W when the correction tensor is on (DerivativeHelpers.h:100-104)
                        V4 cg = grad;
                        if (corrected) {
                            const double* C = corr.data() + 6 * i;
                            cg.x = C[0] * grad.x + C[3] * grad.y + C[4] * grad.z;
                            cg.y = C[3] * grad.x + C[1] * grad.y + C[5] * grad.z;
                            cg.z = C[4] * grad.x + C[5] * grad.y + C[2] * grad.z;
                        }
                        const double f = mj / rhoi;
                        const double o0 = 0.5 * (dvji.x * cg.y + dvji.y * cg.x);
                        const double o1 = 0.5 * (dvji.x * cg.z + dvji.z * cg.x);
                        const double o2 = 0.5 * (dvji.y * cg.z + dvji.z * cg.y);
                        gv[0] += f * (dvji.x * cg.x);
                        gv[1] += f * (dvji.y * cg.y);
                        gv[2] += f * (dvji.z * cg.z);
                        gv[3] += f * o0;
                        gv[4] += f * o1;
                        gv[5] += f * o2;
                        // StressDivergence<StandardForceDiscr> (EquationTerm.cpp:114-140)
                        const double* Si = s.S + 5 * i;
                        const double* Sj = s.S + 5 * j;
                        const double ri2 = rhoi * rhoi, rj2 = rhoj * rhoj;
                        double t[5];
                        for (int c = 0; c < 5; ++c) {
                            t[c] = Si[c] / ri2 + Sj[c] / rj2;
                        }
                        const double tzz = -t[0] - t[1];
                        const double fx = t[0] * grad.x + t[2] * grad.y + t[3] * grad.z;
                        const double fy = t[2] * grad.x + t[1] * grad.y + t[4] * grad.z;
                        const double fz = t[3] * grad.x + t[4] * grad.y + tzz * grad.z;
                        ax += mj * fx;
                        ay += mj * fy;
                        az += mj * fz;
                    }
                }
            }
            s.dv[4 * i] = ax;
            s.dv[4 * i + 1] = ay;
            s.dv[4 * i + 2] = az;
            s.du[i] = du;
            s.divv[i] = divv;
            if (s.ncnt) {
                s.ncnt[i] = cnt;
            }
            if (fl.solid && s.gradv) {
                for (int c = 0; c < 6; ++c) {
                    s.gradv[6 * i + c] = gv[c];
                }
            }
            s.drho[i] = 0.;
            if (s.dS) {
                for (int c = 0; c < 5; ++c) {
                    s.dS[5 * i + c] = 0.;
                }
            }
            if (s.dD) {
                s.dD[i] = 0.;
            }
        }
    });
    // equations finalize, reverse order of getStandardEquations (core/sph/equations/EquationTerm.h:293-297)
    parallelFor(n, [&](uint64_t a, uint64_t b) {
        for (uint64_t i = a; i < b; ++i) {
            const sphgpu_material& mt = matOf(cfg, s, i);
            // AdaptiveSmoothingLength / ConstSmoothingLength (EquationTerm.cpp:366-391, 427-434)
            if (fl.adaptive) {
                const double h = s.r[4 * i + 3];
                s.v[4 * i + 3] = h > 2. * cfg.smoothing_length_range[0] ? h / 3. * s.divv[i] : 0.;
            } else {
                s.v[4 * i + 3] = 0.;
            }
            s.dv[4 * i + 3] = 0.;
            // ContinuityEquation (EquationTerm.cpp:289-316)
            s.drho[i] += -s.rho[i] * s.divv[i];
            // SolidStressForce (EquationTerm.cpp:177-203)
            if (fl.solid && hasRheology(mt)) {
                const double* g = s.gradv + 6 * i;
                const double* S = s.S + 5 * i;
                const double Szz = -S[0] - S[1];
                const double dd = S[0] * g[0] + S[1] * g[1] + Szz * g[2];
                const double oo = S[2] * g[3] + S[3] * g[4] + S[4] * g[5];
                s.du[i] += 1. / s.rho[i] * (dd + 2. * oo);
                const double tr3 = (g[0] * 1. + g[1] * 1. + g[2] * 1.) / 3.;
                const double twoMu = 2. * mt.shear_modulus;
                double* dS = s.dS + 5 * i;
                dS[0] += twoMu * (g[0] - tr3);
                dS[1] += twoMu * (g[1] - tr3);
                dS[2] += twoMu * g[3];
                dS[3] += twoMu * g[4];
                dS[4] += twoMu * g[5];
            }
            // PressureForce (EquationTerm.cpp:90-99)
            s.du[i] -= s.p[i] / s.rho[i] * s.divv[i];
            // material finalize: ScalarGradyKippModel::integrate (core/physics/Damage.cpp:128-170)
            if (fl.solid && hasRheology(mt) && mt.damage == SPHGPU_DAMAGE_SCALAR_GRADY_KIPP && s.D) {
                s.dD[i] = gradyKipp(mt, s.S + 5 * i, s.p[i], s.D[i], s.eps_min[i], s.m_zero[i], s.growth[i],
                    s.n_flaws[i], s.dD[i]);
            }
        }
    });
}

// ---------------------------------------------------------------------------------------------------------
// Time stepping (core/timestepping/TimeStepping.cpp:82-391) and the Courant criterion (TimeStepCriterion.cpp:
// 315-356)
// ---------------------------------------------------------------------------------------------------------

// clampWithDerivative (core/objects/wrappers/Interval.h:159-162); returns true if the range is bounded
inline void clampDeriv(double& x, double& dx, const double range[2]) {
    if (range[0] == -INFTY && range[1] == INFTY) {
        return;
    }
    const bool zero = (x >= range[1] && dx > 0.) || (x <= range[0] && dx < 0.);
    x = std::max(range[0], std::min(x, range[1]));
    if (zero) {
        dx = 0.;
    }
}

struct FirstOrder {
    double* x;
    double* dx;
    int comps;
    int range; // 0 density, 1 energy, 2 damage, -1 unbounded
};

std::vector<FirstOrder> firstOrder(const sphgpu_config& cfg, ora_state& s) {
    std::vector<FirstOrder> q{ { s.rho, s.drho, 1, 0 }, { s.u, s.du, 1, 1 } };
    const Flags fl = flagsOf(cfg, s);
    if (fl.solid) {
        q.push_back({ s.S, s.dS, 5, -1 });
    }
    if (fl.solid && s.D) {
        q.push_back({ s.D, s.dD, 1, 2 });
    }
    return q;
}

const double* rangeOf(const sphgpu_material& mt, int k) {
    return k == 0 ? mt.density_range : (k == 1 ? mt.energy_range : mt.damage_range);
}

// MultiCriterion::compute (core/timestepping/TimeStepCriterion.cpp:331-389) over the criteria of the settings:
// CourantCriterion (:294-329), DerivativeCriterion with the minimal step (:139-206), AccelerationCriterion
// (:212-246), DivergenceCriterion (:252-288); each capped by the maximal step, then the smoothing by max_change
// against the previous step.
double criterionStep(const sphgpu_config& cfg, const ora_state& s, double lastStep) {
    const uint32_t crit = cfg.timestep_criteria ? cfg.timestep_criteria : uint32_t(SPHGPU_CRITERION_COURANT);
    const bool solid = (cfg.forces & SPHGPU_FORCE_SOLID_STRESS) != 0;
    auto capped = [&](double step) { return step > cfg.max_timestep ? cfg.max_timestep : step; };
    double minStep = INFTY;
    if (crit & SPHGPU_CRITERION_COURANT) {
        double m = INFTY;
        for (uint64_t i = 0; i < s.n; ++i) {
            if (s.cs[i] > 0.) {
                m = std::min(m, cfg.courant_number * s.r[4 * i + 3] / s.cs[i]);
            }
        }
        minStep = std::min(minStep, capped(m));
    }
    bool anyDamage = false;
    for (uint32_t k = 0; k < cfg.material_count; ++k) {
        anyDamage = anyDamage ||
                    (cfg.materials[k].yielding != SPHGPU_YIELDING_NONE && cfg.materials[k].damage != SPHGPU_DAMAGE_NONE);
    }
    if (crit & SPHGPU_CRITERION_DERIVATIVES) {
        const double f = cfg.derivative_factor;
        double m = INFTY;
        auto add = [&](double v, double dv, double minValue) {
            const double av = std::abs(v), adv = std::abs(dv);
            if (std::abs(av) < 2. * minValue) {
                return;
            }
            m = std::min(m, f * (av + minValue) / (adv + EPS));
        };
        for (uint64_t i = 0; i < s.n; ++i) {
            const sphgpu_material& mt = cfg.materials[cfg.material_count > 1 ? s.mat[i] : 0];
            add(s.rho[i], s.drho[i], mt.density_min);
            add(s.u[i], s.du[i], mt.energy_min);
            if (solid && s.S) {
                const double* S = s.S;
                const double* dS = s.dS;
                const uint64_t n = s.n;
                // TracelessTensor components xx, yy, zz, xy, xz, yz (getComponents, TracelessTensor.h:393)
                const double sv[6] = { S[i], S[n + i], -S[i] - S[n + i], S[2 * n + i], S[3 * n + i], S[4 * n + i] };
                const double dsv[6] = { dS[i], dS[n + i], -dS[i] - dS[n + i], dS[2 * n + i], dS[3 * n + i],
                    dS[4 * n + i] };
                for (int c = 0; c < 6; ++c) {
                    add(sv[c], dsv[c], mt.stress_min);
                }
            }
            // DAMAGE is a first-order quantity of the whole storage when any material has a fracture model
            if (solid && anyDamage && s.D && s.dD) {
                add(s.D[i], s.dD[i], mt.damage_min);
            }
        }
        minStep = std::min(minStep, capped(m));
    }
    if (crit & SPHGPU_CRITERION_ACCELERATION) {
        double m = INFTY;
        for (uint64_t i = 0; i < s.n; ++i) {
            const double ax = s.dv[4 * i], ay = s.dv[4 * i + 1], az = s.dv[4 * i + 2];
            const double a2 = ax * ax + ay * ay + az * az;
            if (a2 > EPS) {
                const double h = s.r[4 * i + 3];
                m = std::min(m, cfg.derivative_factor * std::sqrt(std::sqrt(h * h / a2)));
            }
        }
        minStep = std::min(minStep, capped(m));
    }
    if (crit & SPHGPU_CRITERION_DIVERGENCE) {
        double m = INFTY;
        for (uint64_t i = 0; i < s.n; ++i) {
            const double dv = std::abs(s.divv[i]);
            if (dv > EPS) {
                m = std::min(m, cfg.divergence_factor / dv);
            }
        }
        minStep = std::min(minStep, capped(m));
    }
    if (cfg.max_change > 0. && cfg.max_change < INFTY) {
        minStep = std::min(minStep, lastStep * (1. + cfg.max_change));
    }
    return minStep;
}

void stepPC(const sphgpu_config& cfg, ora_state& s, double dt) {
    const uint64_t n = s.n;
    const double dt2 = 0.5 * (dt * dt);
    std::vector<FirstOrder> fo = firstOrder(cfg, s);
    // makePredictions (TimeStepping.cpp:286-300)
    for (uint64_t i = 0; i < n; ++i) {
        for (int k = 0; k < 4; ++k) {
            double& r = s.r[4 * i + k];
            double& v = s.v[4 * i + k];
            const double a = s.dv[4 * i + k];
            r += v * dt + a * dt2;
            v += a * dt;
        }
        for (const FirstOrder& q : fo) {
            for (int c = 0; c < q.comps; ++c) {
                q.x[q.comps * i + c] += q.dx[q.comps * i + c] * dt;
            }
            if (q.range >= 0) {
                clampDeriv(q.x[i], q.dx[i], rangeOf(matOf(cfg, s, i), q.range));
            }
        }
    }
    // save the predicted derivatives, then evaluate the derivatives at the predicted state
    std::vector<double> pdv(s.dv, s.dv + 4 * n);
    std::vector<std::vector<double>> pdx;
    for (const FirstOrder& q : fo) {
        pdx.emplace_back(q.dx, q.dx + q.comps * n);
    }
    integrate(cfg, s);
    // makeCorrections (TimeStepping.cpp:302-322)
    const double a = 1. / 3., b = 0.5;
    for (uint64_t i = 0; i < n; ++i) {
        for (int k = 0; k < 4; ++k) {
            const double diff = pdv[4 * i + k] - s.dv[4 * i + k];
            s.r[4 * i + k] -= a * diff * dt2;
            s.v[4 * i + k] -= b * diff * dt;
        }
        for (size_t qi = 0; qi < fo.size(); ++qi) {
            const FirstOrder& q = fo[qi];
            for (int c = 0; c < q.comps; ++c) {
                const uint64_t e = q.comps * i + c;
                q.x[e] -= 0.5 * (pdx[qi][e] - q.dx[e]) * dt;
            }
            if (q.range >= 0) {
                clampDeriv(q.x[i], q.dx[i], rangeOf(matOf(cfg, s, i), q.range));
            }
        }
    }
}

void stepLF(const sphgpu_config& cfg, ora_state& s, double dt) {
    const uint64_t n = s.n;
    std::vector<FirstOrder> fo = firstOrder(cfg, s);
    for (uint64_t i = 0; i < 4 * n; ++i) {
        s.r[i] += s.v[i] * 0.5 * dt;
    }
    integrate(cfg, s);
    for (uint64_t i = 0; i < n; ++i) {
        for (const FirstOrder& q : fo) {
            for (int c = 0; c < q.comps; ++c) {
                q.x[q.comps * i + c] += q.dx[q.comps * i + c] * dt;
            }
            if (q.range >= 0) {
                clampDeriv(q.x[i], q.dx[i], rangeOf(matOf(cfg, s, i), q.range));
            }
        }
    }
    for (uint64_t i = 0; i < 4 * n; ++i) {
        s.v[i] += s.dv[i] * dt;
    }
    for (uint64_t i = 0; i < 4 * n; ++i) {
        s.r[i] += s.v[i] * 0.5 * dt;
    }
}

bool validConfig(const sphgpu_config* cfg, const ora_state* s) {
    return cfg && s && cfg->materials && cfg->material_count > 0 && s->r && s->v && s->dv && s->m && s->rho &&
           s->drho && s->u && s->du && s->p && s->cs && s->divv;
}

} // namespace

extern "C" {

void ora_set_threads(int threads) {
    gThreads = threads;
}

double ora_sph_kernel_value(double qsqr) {
    return sphLut().value(qsqr);
}
double ora_sph_kernel_grad(double qsqr) {
    return sphLut().grad(qsqr);
}
double ora_gravity_kernel_grad(double qsqr) {
    return gravLut().grad(qsqr);
}

int ora_eos(const sphgpu_material* mat, uint64_t n, const double* rho, const double* u, double* p, double* cs) {
    if (!mat || (n && (!rho || !u || !p || !cs))) {
        return SPHGPU_ERR_ARGUMENT;
    }
    for (uint64_t i = 0; i < n; ++i) {
        eosEval(*mat, rho[i], u[i], p[i], cs[i]);
    }
    return SPHGPU_OK;
}

int ora_pairs(uint64_t n, const double* r, uint32_t* pi, uint32_t* pj, uint64_t capacity, uint64_t* npairs) {
    if (!npairs || (n && !r)) {
        return SPHGPU_ERR_ARGUMENT;
    }
    const Neighbours nb = findNeighbours(n, r);
    uint64_t cnt = 0;
    for (uint64_t i = 0; i < n; ++i) {
        for (uint64_t k = nb.start[i]; k < nb.start[i + 1]; ++k) {
            const uint32_t j = nb.idx[k];
            if (j > i) {
                if (cnt < capacity) {
                    pi[cnt] = uint32_t(i);
                    pj[cnt] = j;
                }
                cnt++;
            }
        }
    }
    *npairs = cnt;
    return cnt > capacity ? SPHGPU_ERR_CAPACITY : SPHGPU_OK;
}

int ora_gravity_bh(uint64_t n, const double* r, const double* m, double G, double theta, int order,
    uint32_t leaf_size, int kernel_radius, double* dv, uint64_t* stats) {
    if (!dv || (n && (!r || !m)) || theta <= 0. || leaf_size == 0) {
        return SPHGPU_ERR_ARGUMENT;
    }
    BarnesHutTree bh;
    bh.leafSize = leaf_size;
    bh.thetaInv = 1. / theta;
    bh.order = order;
    bh.kernelRadius = kernel_radius;
    bh.build(n, r, m, G);
    bh.evalSelfGravity(dv);
    if (stats) {
        stats[0] = bh.nApprox;
        stats[1] = bh.nExact;
        stats[2] = bh.nodes.size();
    }
    return SPHGPU_OK;
}

int ora_gravity_points(uint64_t n, const double* r, const double* m, double G, double theta, int order,
    uint32_t leaf_size, int kernel_radius, uint64_t npoints, const double* points, double* acc) {
    if ((n && (!r || !m)) || (npoints && (!points || !acc)) || theta <= 0. || leaf_size == 0) {
        return SPHGPU_ERR_ARGUMENT;
    }
    BarnesHutTree bh;
    bh.leafSize = leaf_size;
    bh.thetaInv = 1. / theta;
    bh.order = order;
    bh.kernelRadius = kernel_radius;
    bh.build(n, r, m, G);
    for (uint64_t k = 0; k < npoints; ++k) {
        const V4 a = n ? bh.evalPoint(load4(points, k)) : V4{ 0, 0, 0, 0 };
        store4(acc, k, a);
    }
    return SPHGPU_OK;
}

// BruteForceGravity::evalImpl (core/gravity/BruteForceGravity.h:110-129)
int ora_gravity_direct(uint64_t n, const double* r, const double* m, double G, int kernel_radius,
    uint64_t ntargets, const uint32_t* idx, double* acc) {
    if ((n && (!r || !m)) || (ntargets && !acc)) {
        return SPHGPU_ERR_ARGUMENT;
    }
    parallelFor(ntargets, [&](uint64_t a, uint64_t b) {
        for (uint64_t t = a; t < b; ++t) {
            const uint64_t i = idx ? idx[t] : t;
            const V4 ri = load4(r, i);
            double f[3] = { 0, 0, 0 };
            for (uint64_t j = 0; j < n; ++j) {
                if (j == i) {
                    continue;
                }
                const V4 rj = load4(r, j);
                const V4 g = gravGradV(sub(rj, ri), 0.5 * (rj.h + ri.h), kernel_radius);
                const double mj = G * m[j];
                f[0] += mj * g.x;
                f[1] += mj * g.y;
                f[2] += mj * g.z;
            }
            store4(acc, t, V4{ f[0], f[1], f[2], 0 });
        }
    });
    return SPHGPU_OK;
}

// BarnesHut::evalAttractors (core/gravity/BarnesHut.cpp:100-125): for each attractor a (in order) and particle i
// (in index order), f = grad W(r_i - x_a, (h_i + R_a) / 2), dv_i -= (G M_a) f and acc_a += (G m_i) f; then for
// each attractor pair i < j, f = G grad W(x_i - x_j, (R_i + R_j) / 2), acc_i -= M_j f and acc_j += M_i f.
// att: 5 doubles per attractor (x, y, z, radius, mass); dv: 4 per particle and acc: 3 per attractor, in/out.
// GravityLutKernel::grad keeping the fourth component of the separation (the reference scales the whole Vector,
// so a difference of smoothing lengths or radii yields a non-zero h component)
V4 gravGradV4(const V4& r, double h, int kernelRadius) {
    const double hInv = 1. / h;
    const V4 rh{ r.x * hInv, r.y * hInv, r.z * hInv, 0. };
    const double qSqr = sqrLen(rh);
    const double rad = double(kernelRadius < 0 ? -kernelRadius : kernelRadius);
    if (qSqr + EPS >= rad * rad) {
        const double len = std::sqrt(sqrLen(r));
        const double l3 = len * len * len;
        return V4{ r.x / l3, r.y / l3, r.z / l3, r.h / l3 };
    }
    const double g = (kernelRadius < 0 ? solidLut() : gravLut()).grad(qSqr);
    const double h3 = hInv * hInv * hInv;
    return V4{ (h3 * r.x) * g, (h3 * r.y) * g, (h3 * r.z) * g, (h3 * r.h) * g };
}

int ora_gravity_attractors(uint64_t n, const double* r, const double* m, double G, int kernel_radius,
    uint64_t count, const double* att, double* dv, double* acc) {
    if ((n && (!r || !m || !dv)) || (count && (!att || !acc))) {
        return SPHGPU_ERR_ARGUMENT;
    }
    for (uint64_t a = 0; a < count; ++a) {
        const V4 xa{ att[5 * a], att[5 * a + 1], att[5 * a + 2], att[5 * a + 3] };
        const double gm = G * att[5 * a + 4];
        for (uint64_t i = 0; i < n; ++i) {
            const V4 ri = load4(r, i);
            const V4 f = gravGradV4(sub(ri, xa), 0.5 * (ri.h + xa.h), kernel_radius);
            dv[4 * i] -= gm * f.x;
            dv[4 * i + 1] -= gm * f.y;
            dv[4 * i + 2] -= gm * f.z;
            dv[4 * i + 3] -= gm * f.h;
            const double mi = G * m[i];
            acc[3 * a] += mi * f.x;
            acc[3 * a + 1] += mi * f.y;
            acc[3 * a + 2] += mi * f.z;
        }
    }
    for (uint64_t i = 0; i < count; ++i) {
        for (uint64_t j = i + 1; j < count; ++j) {
            const V4 xi{ att[5 * i], att[5 * i + 1], att[5 * i + 2], att[5 * i + 3] };
            const V4 xj{ att[5 * j], att[5 * j + 1], att[5 * j + 2], att[5 * j + 3] };
            const V4 g = gravGradV(sub(xi, xj), 0.5 * (xi.h + xj.h), kernel_radius);
            const double f[3] = { G * g.x, G * g.y, G * g.z };
            for (int c = 0; c < 3; ++c) {
                acc[3 * i + c] -= att[5 * j + 4] * f[c];
                acc[3 * j + c] += att[5 * i + 4] * f[c];
            }
        }
    }
    return SPHGPU_OK;
}

int ora_integrate(const sphgpu_config* cfg, ora_state* s) {
    if (!validConfig(cfg, s)) {
        return SPHGPU_ERR_ARGUMENT;
    }
    gCache = GravityCache();
    integrate(*cfg, *s);
    return SPHGPU_OK;
}

int ora_run(const sphgpu_config* cfg, ora_state* s, uint32_t nsteps, double* dt, double* dts) {
    if (!validConfig(cfg, s) || !dt) {
        return SPHGPU_ERR_ARGUMENT;
    }
    gCache = GravityCache();
    for (uint32_t k = 0; k < nsteps; ++k) {
        if (dts) {
            dts[k] = *dt;
        }
        if (cfg->integrator == SPHGPU_INTEGRATOR_LEAP_FROG) {
            stepLF(*cfg, *s, *dt);
        } else {
            stepPC(*cfg, *s, *dt);
        }
        gCache.runTime += *dt;
        *dt = criterionStep(*cfg, *s, *dt);
    }
    return SPHGPU_OK;
}

int ora_totals(const ora_state* s, double out[9]) {
    if (!s || !out) {
        return SPHGPU_ERR_ARGUMENT;
    }
    std::fill(out, out + 9, 0.);
    for (uint64_t i = 0; i < s->n; ++i) {
        const V4 r = load4(s->r, i), v = load4(s->v, i);
        const double m = s->m[i];
        out[0] += m * v.x;
        out[1] += m * v.y;
        out[2] += m * v.z;
        out[3] += m * (r.y * v.z - r.z * v.y);
        out[4] += m * (r.z * v.x - r.x * v.z);
        out[5] += m * (r.x * v.y - r.y * v.x);
        out[6] += 0.5 * m * dot3(v, v);
        out[7] += m * s->u[i];
        out[8] += m;
    }
    return SPHGPU_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------------------------------------
// Frozen-list model of the adjoint workload, in forward-mode dual numbers (tangent-linear reference)
// ---------------------------------------------------------------------------------------------------------

namespace {

struct Dual {
    double v = 0., d = 0.;
    Dual() = default;
    Dual(double a, double b = 0.) : v(a), d(b) {}
};
inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dual operator/(Dual a, Dual b) { return Dual(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)); }
inline Dual sqrtD(Dual a) {
    const double s = std::sqrt(a.v);
    return Dual(s, a.d / (2. * s));
}

// LutKernel<3> gradient table as a piecewise-linear function of q^2, with its derivative
inline Dual lutGradD(Dual q2) {
    const Lut& lut = sphLut();
    if (q2.v >= 4.) {
        return Dual(0., 0.);
    }
    const double f = lut.qSqrToIdx * q2.v;
    const int i1 = int(f);
    const double ratio = f - double(i1);
    const double g0 = lut.grads[i1], g1 = lut.grads[i1 + 1];
    return Dual(g0 * (1. - ratio) + g1 * ratio, (g1 - g0) * lut.qSqrToIdx * q2.d);
}

struct FrozenModel {
    const ora_frozen_params& p;
    uint64_t n;
    const double* m;
    std::vector<Dual> r, v, rho, u; // r, v: 3 per particle
    std::vector<double> h;
    Dual alpha;
    Neighbours nb;

    void rebuild() {
        std::vector<double> pos(4 * n);
        for (uint64_t i = 0; i < n; ++i) {
            for (int k = 0; k < 3; ++k) {
                pos[4 * i + k] = r[3 * i + k].v;
            }
            pos[4 * i + 3] = h[i];
        }
        nb = findNeighbours(n, pos.data());
    }

    void step() {
        const double dt = p.dt, gamma = p.gamma, beta = p.beta;
        std::vector<Dual> rp(3 * n), pr(n), cs(n);
        for (uint64_t i = 0; i < n; ++i) {
            for (int k = 0; k < 3; ++k) {
                rp[3 * i + k] = r[3 * i + k] + v[3 * i + k] * Dual(0.5 * dt);
            }
            pr[i] = Dual(gamma - 1.) * u[i] * rho[i];
            cs[i] = sqrtD(Dual(gamma) * pr[i] / rho[i]);
        }
        std::vector<Dual> nv(3 * n), nr(3 * n), nrho(n), nu(n);
        parallelFor(n, [&](uint64_t a, uint64_t b) {
            for (uint64_t i = a; i < b; ++i) {
                Dual ax, ay, az, divv, heat;
                const Dual Pi_ = pr[i] / (rho[i] * rho[i]);
                for (uint64_t kk = nb.start[i]; kk < nb.start[i + 1]; ++kk) {
                    const uint32_t j = nb.idx[kk];
                    const double hbar = 0.5 * (h[i] + h[j]);
                    const Dual dx = rp[3 * i] - rp[3 * j], dy = rp[3 * i + 1] - rp[3 * j + 1],
                               dz = rp[3 * i + 2] - rp[3 * j + 2];
                    const Dual s = dx * dx + dy * dy + dz * dz;
                    const double hInv = 1. / hbar;
                    const double h5 = hInv * hInv * hInv * hInv * hInv;
                    const Dual F = Dual(h5) * lutGradD(s * Dual(hInv * hInv));
                    const Dual gx = dx * F, gy = dy * F, gz = dz * F;
                    const double mj = m[j];
                    const Dual vjx = v[3 * j] - v[3 * i], vjy = v[3 * j + 1] - v[3 * i + 1],
                               vjz = v[3 * j + 2] - v[3 * i + 2];
                    divv = divv + Dual(mj) / rho[i] * (vjx * gx + vjy * gy + vjz * gz);
                    const Dual Pj = pr[j] / (rho[j] * rho[j]);
                    Dual coef = -(Pi_ + Pj);
                    const Dual wd = -(vjx * dx + vjy * dy + vjz * dz);
                    if (wd.v < 0.) {
                        const Dual D = s + Dual(1.e-2 * hbar * hbar);
                        const Dual mu = Dual(hbar) * wd / D;
                        const Dual rb = Dual(0.5) * (rho[i] + rho[j]);
                        const Dual cb = Dual(0.5) * (cs[i] + cs[j]);
                        const Dual Pi = (-alpha * cb * mu + Dual(beta) * mu * mu) / rb;
                        coef = coef - Pi;
                        heat = heat + Dual(mj) * Dual(0.5) * Pi * -(vjx * gx + vjy * gy + vjz * gz);
                    }
                    ax = ax + Dual(mj) * coef * gx;
                    ay = ay + Dual(mj) * coef * gy;
                    az = az + Dual(mj) * coef * gz;
                }
                const Dual drho = -rho[i] * divv;
                const Dual du = heat - pr[i] / rho[i] * divv;
                nrho[i] = rho[i] + drho * Dual(dt);
                nu[i] = u[i] + du * Dual(dt);
                const Dual acc[3] = { ax, ay, az };
                for (int k = 0; k < 3; ++k) {
                    nv[3 * i + k] = v[3 * i + k] + acc[k] * Dual(dt);
                    nr[3 * i + k] = rp[3 * i + k] + nv[3 * i + k] * Dual(0.5 * dt);
                }
            }
        });
        r.swap(nr);
        v.swap(nv);
        rho.swap(nrho);
        u.swap(nu);
    }
};

} // namespace

extern "C" int ora_frozen_loss(const ora_frozen_params* prm, uint64_t n, const double* r, const double* v,
    const double* m, const double* rho, const double* u, const double* tr, const double* tv, const double* trho,
    const double* tu, double talpha, double* loss, double* dloss) {
    if (!prm || !r || !v || !m || !rho || !u || !loss || prm->rebuild_every == 0) {
        return SPHGPU_ERR_ARGUMENT;
    }
    FrozenModel fm{ *prm, n, m };
    fm.r.resize(3 * n);
    fm.v.resize(3 * n);
    fm.rho.resize(n);
    fm.u.resize(n);
    fm.h.resize(n);
    for (uint64_t i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) {
            fm.r[3 * i + k] = Dual(r[4 * i + k], tr ? tr[4 * i + k] : 0.);
            fm.v[3 * i + k] = Dual(v[4 * i + k], tv ? tv[4 * i + k] : 0.);
        }
        fm.h[i] = r[4 * i + 3];
        fm.rho[i] = Dual(rho[i], trho ? trho[i] : 0.);
        fm.u[i] = Dual(u[i], tu ? tu[i] : 0.);
    }
    fm.alpha = Dual(prm->alpha, talpha);
    for (uint32_t s = 0; s < prm->steps; ++s) {
        if (s % prm->rebuild_every == 0) {
            fm.rebuild();
        }
        fm.step();
    }
    Dual L;
    for (uint64_t i = 0; i < std::min<uint64_t>(prm->n_target, n); ++i) {
        for (int k = 0; k < 3; ++k) {
            L = L + fm.v[3 * i + k] * fm.v[3 * i + k];
        }
    }
    *loss = L.v;
    if (dloss) {
        *dloss = L.d;
    }
    return SPHGPU_OK;
}

// ---------------------------------------------------------------------------------------------------------
// HardSphereSolver (core/gravity/NBodySolver.cpp:17-597) with the handlers of core/gravity/Collision.h.
// The collision loop keeps the reference's own data structures: an ordered set of records with the order
// (time, -overlap, i, j) and an index -> record multimap (CollisionSet, NBodySolver.cpp:213-327).
// Deterministic choices where the reference depends on its k-d tree traversal order or on std::sort's order
// of equal keys: rank ties are broken by index; of several overlapping neighbours the record smallest in the
// record order is taken (the reference returns the first one its traversal meets) and every neighbour found
// by the first-pass search writes its search radius. Searches that the reference might resolve differently
// are counted as "ambiguous" so that fixtures can be checked to contain none.
// ---------------------------------------------------------------------------------------------------------

#include <map>
#include <set>
#include <unordered_map>

namespace {

// Constants::gravity (core/physics/Constants.h:32)
const double G_PHYS = 6.67408e-11;

inline V4 add4(const V4& a, const V4& b) {
    return V4{ a.x + b.x, a.y + b.y, a.z + b.z, a.h + b.h };
}
inline V4 div4(const V4& a, double f) {
    return V4{ a.x / f, a.y / f, a.z / f, a.h / f };
}
inline V4 cross3(const V4& a, const V4& b) {
    return V4{ a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0. };
}
inline double pow3(double x) {
    return x * x * x;
}
// weightedAverage (core/gravity/Collision.h:81-85)
inline V4 weightedAverage(const V4& a, double wa, const V4& b, double wb) {
    return div4(add4(scale(a, wa), scale(b, wb)), wa + wb);
}

struct SymT {
    double d[3], o[3];
};
// Rigid::sphereInertia (core/physics/Functions.h:61-63)
inline SymT sphereInertia(double m, double r) {
    const double k = 0.4 * m * (r * r);
    return SymT{ { 1. * k, 1. * k, 1. * k }, { 0. * k, 0. * k, 0. * k } };
}
// SymmetricTensor * Vector (core/objects/geometry/SymmetricTensor.h:102-107)
inline V4 symMul(const SymT& t, const V4& v) {
    return V4{ t.d[0] * v.x + t.o[0] * v.y + t.o[1] * v.z, t.o[0] * v.x + t.d[1] * v.y + t.o[2] * v.z,
        t.o[1] * v.x + t.o[2] * v.y + t.d[2] * v.z, 0. };
}
// SymmetricTensor::determinant / inverse (SymmetricTensor.h:193-231)
inline SymT symInverse(const SymT& t) {
    const double det = t.d[0] * t.d[1] * t.d[2] + 2. * t.o[0] * t.o[1] * t.o[2] -
                       ((t.o[0] * t.o[0]) * t.d[2] + (t.o[1] * t.o[1]) * t.d[1] + (t.o[2] * t.o[2]) * t.d[0]);
    SymT r;
    r.d[0] = (t.d[1] * t.d[2] - t.o[2] * t.o[2]) / det;
    r.d[1] = (t.d[2] * t.d[0] - t.o[1] * t.o[1]) / det;
    r.d[2] = (t.d[0] * t.d[1] - t.o[0] * t.o[0]) / det;
    r.o[0] = (t.o[1] * t.o[2] - t.d[2] * t.o[0]) / det;
    r.o[1] = (t.o[2] * t.o[0] - t.d[1] * t.o[1]) / det;
    r.o[2] = (t.o[0] * t.o[1] - t.d[0] * t.o[2]) / det;
    return r;
}

// areParticlesBound (Collision.h:86-91)
inline bool particlesBound(double mSum, double hSum, const V4& dv, double limit) {
    const double vEscSqr = 2. * G_PHYS * mSum / hSum;
    return sqrLen(dv) * limit < vEscSqr;
}

struct NbParts {
    std::vector<V4> r, v, dv, w;
    std::vector<double> m;
    std::vector<char> removed;
};

struct MergerO {
    double h, m;
    V4 r, v, w;
};
// MergingCollisionHandler::collide without the inertia tensor (Collision.h:160-215)
MergerO mergerOf(const NbParts& P, uint32_t i, uint32_t j) {
    const V4 &ri = P.r[i], &rj = P.r[j], &vi = P.v[i], &vj = P.v[j];
    const double mi = P.m[i], mj = P.m[j];
    MergerO g;
    g.h = std::cbrt(pow3(ri.h) + pow3(rj.h));
    g.m = mi + mj;
    g.r = weightedAverage(ri, mi, rj, mj);
    g.v = weightedAverage(vi, mi, vj, mj);
    V4 L = add4(scale(cross3(sub(ri, g.r), sub(vi, g.v)), mi), scale(cross3(sub(rj, g.r), sub(vj, g.v)), mj));
    L = add4(L, symMul(sphereInertia(mi, ri.h), P.w[i]));
    L = add4(L, symMul(sphereInertia(mj, rj.h), P.w[j]));
    g.w = symMul(symInverse(sphereInertia(g.m, g.h)), L);
    return g;
}

enum { NB_NONE = 0, NB_BOUNCE = 1, NB_MERGER = 2 };

// MergingCollisionHandler::collide + acceptMerge (Collision.h:160-261)
int mergeCollide(NbParts& P, uint32_t i, uint32_t j, double bounceLimit, double rotationLimit) {
    const MergerO g = mergerOf(P, i, j);
    if (!particlesBound(P.m[i] + P.m[j], P.r[i].h + P.r[j].h, sub(P.v[i], P.v[j]), bounceLimit)) {
        return NB_NONE;
    }
    const double omegaCritSqr = G_PHYS * (P.m[i] + P.m[j]) / pow3(g.h);
    if (sqrLen(g.w) * rotationLimit > omegaCritSqr) {
        return NB_NONE;
    }
    P.m[i] = g.m;
    P.r[i] = V4{ g.r.x, g.r.y, g.r.z, g.h };
    P.v[i] = V4{ g.v.x, g.v.y, g.v.z, 0. };
    P.w[i] = g.w;
    P.removed[j] = 1;
    return NB_MERGER;
}

// ElasticBounceHandler::reflect (Collision.h:316-326)
inline V4 reflect(const V4& v, const V4& vCom, const V4& dir, double rn, double rt) {
    const V4 vRel = sub(v, vCom);
    const double proj = dot3(vRel, dir);
    const V4 vT = sub(vRel, scale(dir, proj));
    const V4 vN = scale(dir, proj);
    return add4(sub(scale(vT, rt), scale(vN, rn)), vCom);
}

// ElasticBounceHandler::collide (Collision.h:301-313)
int bounceCollide(NbParts& P, uint32_t i, uint32_t j, double rn, double rt) {
    const V4 d = sub(P.r[i], P.r[j]);
    const V4 dr = div4(d, std::sqrt(sqrLen(d)));
    const V4 ndr{ -dr.x, -dr.y, -dr.z, -dr.h };
    const V4 vCom = weightedAverage(P.v[i], P.m[i], P.v[j], P.m[j]);
    const V4 vi = reflect(P.v[i], vCom, ndr, rn, rt);
    const V4 vj = reflect(P.v[j], vCom, dr, rn, rt);
    P.v[i] = V4{ vi.x, vi.y, vi.z, 0. };
    P.v[j] = V4{ vj.x, vj.y, vj.z, 0. };
    return NB_BOUNCE;
}

// Factory::getCollisionHandler (core/system/Factory.cpp:415-429)
int collisionHandler(NbParts& P, const sphgpu_config& c, uint32_t i, uint32_t j) {
    switch (c.collision_handler) {
    case SPHGPU_COLLISION_PERFECT_MERGING:
        return mergeCollide(P, i, j, 0., 0.);
    case SPHGPU_COLLISION_ELASTIC_BOUNCE:
        return bounceCollide(P, i, j, c.restitution_normal, c.restitution_tangent);
    default: {
        const int res = mergeCollide(P, i, j, c.bounce_merge_limit, c.rotation_merge_limit);
        return res != NB_NONE ? res : bounceCollide(P, i, j, c.restitution_normal, c.restitution_tangent);
    }
    }
}

// RepelHandler::handle before the follow-up handler (Collision.h:443-467)
void repel(NbParts& P, uint32_t i, uint32_t j) {
    const V4 d = sub(P.r[i], P.r[j]);
    const double dist = std::sqrt(sqrLen(d));
    V4 dir = div4(d, dist);
    dir.h = 0.;
    const double x1 = (P.r[i].h + P.r[j].h - dist) / (1. + P.m[i] / P.m[j]);
    const double x2 = P.m[i] / P.m[j] * x1;
    P.r[i] = add4(P.r[i], scale(dir, x1));
    P.r[j] = sub(P.r[j], scale(dir, x2));
}

// Factory::getOverlapHandler (core/system/Factory.cpp:431-450): IOverlapHandler::handle
void overlapHandle(NbParts& P, const sphgpu_config& c, uint32_t i, uint32_t j) {
    const double rn = c.restitution_normal, rt = c.restitution_tangent;
    switch (c.overlap_handler) {
    case SPHGPU_OVERLAP_FORCE_MERGE:
        mergeCollide(P, i, j, 0., 0.);
        break;
    case SPHGPU_OVERLAP_REPEL:
        repel(P, i, j);
        bounceCollide(P, i, j, rn, rt);
        break;
    case SPHGPU_OVERLAP_REPEL_OR_MERGE:
        repel(P, i, j);
        if (mergeCollide(P, i, j, c.bounce_merge_limit, c.rotation_merge_limit) == NB_NONE) {
            bounceCollide(P, i, j, rn, rt);
        }
        break;
    case SPHGPU_OVERLAP_INTERNAL_BOUNCE:
        bounceCollide(P, i, j, rn, rt);
        break;
    case SPHGPU_OVERLAP_PASS_OR_MERGE:
        mergeCollide(P, i, j, c.bounce_merge_limit, c.rotation_merge_limit);
        break;
    default:
        break;
    }
}

// IOverlapHandler::overlaps (Collision.h:379-381, 404-406, 439-442, 494-499, 537-560)
bool overlapHandled(const NbParts& P, const sphgpu_config& c, uint32_t i, uint32_t j) {
    switch (c.overlap_handler) {
    case SPHGPU_OVERLAP_NONE:
        return false;
    case SPHGPU_OVERLAP_INTERNAL_BOUNCE:
        return dot3(sub(P.r[i], P.r[j]), sub(P.v[i], P.v[j])) < 0.;
    case SPHGPU_OVERLAP_PASS_OR_MERGE: {
        if (!particlesBound(P.m[i] + P.m[j], P.r[i].h + P.r[j].h, sub(P.v[i], P.v[j]), c.bounce_merge_limit)) {
            return false;
        }
        const MergerO g = mergerOf(P, i, j);
        const double omegaCritSqr = G_PHYS * (P.m[i] + P.m[j]) / pow3(g.h);
        return !(sqrLen(g.w) * c.rotation_merge_limit > omegaCritSqr);
    }
    default:
        return true;
    }
}

// HardSphereSolver::checkCollision (NBodySolver.cpp:565-597); +inf when there is no collision in [0, dt]
double checkCollision(const V4& r1, const V4& v1, const V4& r2, const V4& v2, double dt) {
    const V4 dr = sub(r1, r2);
    const V4 dv = sub(v1, v2);
    const double dvdr = dot3(dv, dr);
    if (dvdr >= 0.) {
        return INFINITY;
    }
    const V4 drPerp = sub(dr, div4(scale(dv, dvdr), sqrLen(dv)));
    const double hs = r1.h + r2.h;
    if (sqrLen(drPerp) <= hs * hs) {
        const double dv2 = sqrLen(dv);
        const double det = 1. - (sqrLen(dr) - hs * hs) / (dvdr * dvdr) * dv2;
        const double sqrtDet = std::sqrt(std::max(0., det));
        const double root = det > 1. ? 1. + sqrtDet : 1. - sqrtDet;
        const double tColl = -dvdr / dv2 * root;
        if (tColl <= dt) {
            return tColl;
        }
    }
    return INFINITY;
}

// CollisionRecord (NBodySolver.cpp:165-211)
struct NbRec {
    double t, nov; // time, minus the overlap
    uint32_t i, j;
    bool operator<(const NbRec& o) const {
        if (t != o.t) {
            return t < o.t;
        }
        if (nov != o.nov) {
            return nov < o.nov;
        }
        if (i != o.i) {
            return i < o.i;
        }
        return j < o.j;
    }
    bool operator==(const NbRec& o) const {
        return t == o.t && nov == o.nov && i == o.i && j == o.j;
    }
};

// CollisionSet (NBodySolver.cpp:213-327)
struct NbCollisionSet {
    std::set<NbRec> records;
    std::multimap<uint32_t, NbRec> byIndex;

    void insert(const NbRec& r) {
        if (!records.insert(r).second) {
            return;
        }
        byIndex.insert({ r.i, r });
        byIndex.insert({ r.j, r });
    }
    void eraseIndexEntry(uint32_t idx, const NbRec& r) {
        auto range = byIndex.equal_range(idx);
        for (auto it = range.first; it != range.second; ++it) {
            if (it->second == r) {
                byIndex.erase(it);
                return;
            }
        }
    }
    void removeByCollision(const NbRec& r) {
        eraseIndexEntry(r.i, r);
        eraseIndexEntry(r.j, r);
        records.erase(r);
    }
    void removeByIndex(uint32_t idx, std::set<uint32_t>& invalid) {
        invalid.insert(idx);
        std::vector<NbRec> mine;
        auto range = byIndex.equal_range(idx);
        for (auto it = range.first; it != range.second; ++it) {
            mine.push_back(it->second);
        }
        for (const NbRec& r : mine) {
            const uint32_t other = r.i == idx ? r.j : r.i;
            invalid.insert(other);
            records.erase(r);
            eraseIndexEntry(other, r);
            eraseIndexEntry(idx, r);
        }
    }
};

struct NbCand {
    double t = INFINITY, nov = 0.;
    uint32_t j = 0;
    bool less(const NbCand& o) const {
        if (t != o.t) {
            return t < o.t;
        }
        if (nov != o.nov) {
            return nov < o.nov;
        }
        return j < o.j;
    }
};

// HardSphereSolver::collide (NBodySolver.cpp:329-484) on the host state
struct NbCollider {
    const sphgpu_config& cfg;
    NbParts& P;
    uint32_t n;
    double dt;
    std::vector<double> s;       // h + |v| dt
    std::vector<std::atomic<int64_t>> writer; // searchRadii writer (the largest index)
    std::vector<double> srad;
    std::vector<uint32_t> bounces;
    // dense grid of the positions at the start of the call (cell edge 2 max(mean s, max s / 8), grown until it
    // has at most max(4 n, 4096) cells), plus the particles moved since
    double cell = 1., lo[3] = { 0, 0, 0 };
    int64_t dims[3] = { 1, 1, 1 };
    std::vector<uint32_t> cellStart, order;
    std::vector<uint32_t> moved;
    std::vector<char> isMoved;
    // indices removed by the previous call: the reference clears its `removed` set only after the first
    // pass (NBodySolver.cpp:367-396), so the first-pass searches skip these indices of the new numbering
    const std::vector<uint32_t>* prevRemoved = nullptr;
    std::atomic<uint64_t> ambiguous{ 0 };
    uint64_t stats[4] = { 0, 0, 0, 0 };

    NbCollider(const sphgpu_config& c, NbParts& p, uint32_t count, double interval)
        : cfg(c), P(p), n(count), dt(interval), writer(count) {}

    int64_t coord(double x, int k) const {
        const double c = std::floor((x - lo[k]) / cell);
        if (!(c > 0.)) {
            return 0;
        }
        return c >= double(dims[k] - 1) ? dims[k] - 1 : int64_t(c);
    }
    uint64_t cellIndex(int64_t x, int64_t y, int64_t z) const {
        return (uint64_t(z) * uint64_t(dims[1]) + uint64_t(y)) * uint64_t(dims[0]) + uint64_t(x);
    }
    void buildGrid() {
        double smax = 0., ssum = 0., hi[3] = { -INFINITY, -INFINITY, -INFINITY };
        lo[0] = lo[1] = lo[2] = INFINITY;
        for (uint32_t i = 0; i < n; ++i) {
            smax = std::max(smax, s[i]);
            ssum += s[i];
            const double x[3] = { P.r[i].x, P.r[i].y, P.r[i].z };
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], x[k]);
                hi[k] = std::max(hi[k], x[k]);
            }
        }
        cell = 2. * std::max(ssum / double(n), 0.125 * smax) * 1.0001;
        if (!(cell > 0.)) {
            cell = 1.;
        }
        const double capacity = std::max(4. * double(n), 4096.);
        for (;;) {
            double total = 1.;
            for (int k = 0; k < 3; ++k) {
                dims[k] = int64_t(std::floor((hi[k] - lo[k]) / cell)) + 1;
                total *= double(dims[k]);
            }
            if (total <= capacity) {
                break;
            }
            cell *= 1.25;
        }
        const size_t ncell = size_t(dims[0] * dims[1] * dims[2]);
        std::vector<uint64_t> key(n);
        cellStart.assign(ncell + 1, 0);
        for (uint32_t i = 0; i < n; ++i) {
            key[i] = cellIndex(coord(P.r[i].x, 0), coord(P.r[i].y, 1), coord(P.r[i].z, 2));
            cellStart[key[i] + 1]++;
        }
        for (size_t c = 0; c < ncell; ++c) {
            cellStart[c + 1] += cellStart[c];
        }
        order.resize(n);
        std::vector<uint32_t> fill(cellStart.begin(), cellStart.end() - 1);
        for (uint32_t i = 0; i < n; ++i) {
            order[fill[key[i]]++] = i;
        }
    }
    // every particle j != i with |r_j - r_i|^2 < radius^2, deduplicated, in index order: the cells of the box
    // [r_i - R', r_i + R'] (R' = radius widened by 1e-9 against rounding) and the moved particles
    void within(uint32_t i, double radius, std::vector<uint32_t>& out) const {
        out.clear();
        const V4 ri = P.r[i];
        const double radiusSqr = radius * radius;
        int64_t c0[3], c1[3];
        const double x[3] = { ri.x, ri.y, ri.z };
        for (int k = 0; k < 3; ++k) {
            const double w = radius * (1. + 1e-9) + 1e-9 * (std::fabs(x[k]) + std::fabs(lo[k]));
            c0[k] = coord(x[k] - w, k);
            c1[k] = coord(x[k] + w, k);
        }
        auto consider = [&](uint32_t j) {
            if (j != i && sqrLen(sub(P.r[j], ri)) < radiusSqr) {
                out.push_back(j);
            }
        };
        for (int64_t z = c0[2]; z <= c1[2]; ++z) {
            for (int64_t y = c0[1]; y <= c1[1]; ++y) {
                for (int64_t xx = c0[0]; xx <= c1[0]; ++xx) {
                    const uint64_t c = cellIndex(xx, y, z);
                    for (uint32_t q = cellStart[c]; q < cellStart[c + 1]; ++q) {
                        consider(order[q]);
                    }
                }
            }
        }
        for (uint32_t j : moved) {
            consider(j);
        }
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }
    void writeRadius(uint32_t j, int64_t i) {
        int64_t cur = writer[j].load(std::memory_order_relaxed);
        while (cur < i && !writer[j].compare_exchange_weak(cur, i, std::memory_order_relaxed)) {
        }
    }
    bool rankLess(uint32_t j, uint32_t i) const {
        return s[j] < s[i] || (s[j] == s[i] && j < i);
    }

    // findClosestCollision (NBodySolver.cpp:509-563); first: FIND_LOWER_RANK over [0, dt], else USE_RADII
    NbCand find(uint32_t i, bool first, double lower, double size) {
        thread_local std::vector<uint32_t> found, neighs;
        neighs.clear();
        if (first) {
            within(i, 2. * s[i], found);
            for (uint32_t j : found) {
                if (rankLess(j, i)) {
                    neighs.push_back(j);
                }
            }
        } else if (srad[i] > 0.) {
            within(i, 2. * srad[i], neighs);
        }
        NbCand best;
        uint32_t overlapsHandled = 0;
        for (uint32_t j : neighs) {
            if (first) {
                writeRadius(j, i);
                writeRadius(i, i);
            }
            if (P.removed[j] || bounces[j] > cfg.max_bounces) {
                continue;
            }
            if (first && prevRemoved && std::binary_search(prevRemoved->begin(), prevRemoved->end(), j)) {
                continue;
            }
            const V4 r1 = add4(P.r[i], scale(P.v[i], lower));
            const V4 r2 = add4(P.r[j], scale(P.v[j], lower));
            const double hs = P.r[i].h + P.r[j].h;
            const double overlapValue = 1. - sqrLen(sub(r1, r2)) / (hs * hs);
            NbCand c;
            c.j = j;
            if (overlapValue > cfg.allowed_overlap * cfg.allowed_overlap) {
                if (!overlapHandled(P, cfg, i, j)) {
                    continue;
                }
                ++overlapsHandled;
                c.t = lower;
                c.nov = -overlapValue;
            } else {
                const double t = checkCollision(r1, P.v[i], r2, P.v[j], size);
                if (!(t < INFINITY)) {
                    continue;
                }
                c.t = t + lower;
            }
            if (c.less(best)) {
                best = c;
            }
        }
        // the reference returns the first overlap its traversal meets (and, in the first pass, stops writing
        // search radii there): with more than one overlap, or an overlap among several first-pass
        // neighbours, its result may differ from this one
        if (overlapsHandled > 1 || (first && overlapsHandled > 0 && neighs.size() > 1)) {
            ambiguous.fetch_add(1, std::memory_order_relaxed);
        }
        return best;
    }

    void run() {
        if (cfg.collision_handler == SPHGPU_COLLISION_NONE || n == 0) {
            return;
        }
        s.resize(n);
        for (uint32_t i = 0; i < n; ++i) {
            s[i] = P.r[i].h + std::sqrt(sqrLen(P.v[i])) * dt;
        }
        for (uint32_t i = 0; i < n; ++i) {
            writer[i].store(-1, std::memory_order_relaxed);
        }
        bounces.assign(n, 0);
        isMoved.assign(n, 0);
        P.removed.assign(n, 0);
        buildGrid();
        // the first pass is independent per particle (parallel like the reference's parallelFor)
        std::vector<NbCand> first(n);
        parallelFor(n, [&](uint64_t a, uint64_t b) {
            for (uint64_t i = a; i < b; ++i) {
                first[i] = find(uint32_t(i), true, 0., dt);
            }
        });
        NbCollisionSet set;
        for (uint32_t i = 0; i < n; ++i) {
            if (first[i].t < INFINITY) {
                set.insert(NbRec{ first[i].t, first[i].nov, i, first[i].j });
            }
        }
        srad.assign(n, 0.);
        for (uint32_t i = 0; i < n; ++i) {
            const int64_t w = writer[i].load(std::memory_order_relaxed);
            srad[i] = w >= 0 ? s[size_t(w)] : 0.;
        }
        while (!set.records.empty()) {
            const NbRec col = *set.records.begin();
            const uint32_t i = col.i, j = col.j;
            const double t = col.t;
            P.r[i] = add4(P.r[i], scale(P.v[i], t));
            P.r[j] = add4(P.r[j], scale(P.v[j], t));
            int result;
            if (col.nov < 0.) {
                overlapHandle(P, cfg, i, j);
                result = NB_BOUNCE;
                stats[3]++;
            } else {
                result = collisionHandler(P, cfg, i, j);
                stats[0]++;
                if (result == NB_MERGER) {
                    stats[1]++;
                } else if (result == NB_BOUNCE) {
                    stats[2]++;
                }
            }
            P.r[i] = sub(P.r[i], scale(P.v[i], t));
            P.r[j] = sub(P.r[j], scale(P.v[j], t));
            if (result == NB_NONE) {
                set.removeByCollision(col);
                continue;
            }
            std::set<uint32_t> invalid;
            set.removeByIndex(i, invalid);
            set.removeByIndex(j, invalid);
            bounces[i]++;
            bounces[j]++;
            for (uint32_t q : { i, j }) {
                if (!isMoved[q]) {
                    isMoved[q] = 1;
                    moved.push_back(q);
                }
            }
            const double lower = t + EPS;
            if (!(lower > dt)) {
                for (uint32_t idx : invalid) {
                    if (P.removed[idx] || bounces[idx] > cfg.max_bounces) {
                        continue;
                    }
                    const NbCand c = find(idx, false, lower, dt - lower);
                    if (!(c.t < INFINITY)) {
                        continue;
                    }
                    if ((idx == i && c.j == j) || (c.j == i && idx == j)) {
                        continue;
                    }
                    set.insert(NbRec{ c.t, c.nov, idx, c.j });
                }
            }
        }
    }
};

// Storage::remove of the merged particles, keeping the order of the others
void nbCompact(NbParts& P, uint32_t& n) {
    uint32_t k = 0;
    for (uint32_t i = 0; i < n; ++i) {
        if (!P.removed[i]) {
            P.r[k] = P.r[i];
            P.v[k] = P.v[i];
            P.dv[k] = P.dv[i];
            P.w[k] = P.w[i];
            P.m[k] = P.m[i];
            ++k;
        }
    }
    n = k;
}

} // namespace

namespace {

NbParts nbLoad(const ora_nbody_state& st) {
    NbParts P;
    P.r.resize(st.n);
    P.v.resize(st.n);
    P.dv.resize(st.n);
    P.w.resize(st.n);
    P.m.assign(st.m, st.m + st.n);
    for (uint32_t i = 0; i < st.n; ++i) {
        P.r[i] = load4(st.r, i);
        P.v[i] = load4(st.v, i);
        P.dv[i] = st.dv ? load4(st.dv, i) : V4{ 0, 0, 0, 0 };
        P.w[i] = st.w ? load4(st.w, i) : V4{ 0, 0, 0, 0 };
    }
    P.removed.assign(st.n, 0);
    return P;
}

void nbStore(const NbParts& P, uint32_t n, ora_nbody_state& st) {
    st.n = n;
    for (uint32_t i = 0; i < n; ++i) {
        store4(st.r, i, P.r[i]);
        store4(st.v, i, P.v[i]);
        if (st.dv) {
            store4(st.dv, i, P.dv[i]);
        }
        if (st.w) {
            store4(st.w, i, P.w[i]);
        }
        st.m[i] = P.m[i];
    }
}

void nbCollide(const sphgpu_config& cfg, NbParts& P, uint32_t& n, double dt, uint64_t stats[4], uint64_t* ambiguous,
    std::vector<uint32_t>& prevRemoved, uint32_t* origin = nullptr) {
    NbCollider c(cfg, P, n, dt);
    c.prevRemoved = &prevRemoved;
    c.run();
    if (cfg.collision_handler != SPHGPU_COLLISION_NONE && n > 0) {
        prevRemoved.clear();
        for (uint32_t i = 0; i < n; ++i) {
            if (P.removed[i]) {
                prevRemoved.push_back(i);
            }
        }
    }
    if (origin) {
        uint32_t k = 0;
        for (uint32_t i = 0; i < n; ++i) {
            if (P.removed.empty() || !P.removed[i]) {
                origin[k++] = i;
            }
        }
    }
    for (int k = 0; k < 4; ++k) {
        stats[k] += c.stats[k];
    }
    if (ambiguous) {
        *ambiguous += c.ambiguous.load();
    }
    if (cfg.collision_handler != SPHGPU_COLLISION_NONE && n > 0) {
        nbCompact(P, n);
    }
}

// HardSphereSolver::integrate (NBodySolver.cpp:97-117): dv = self-gravity, v.h = dv.h = 0
void nbIntegrate(const sphgpu_config& cfg, NbParts& P, uint32_t n) {
    std::vector<double> r(4 * size_t(n)), acc(4 * size_t(n), 0.);
    for (uint32_t i = 0; i < n; ++i) {
        store4(r.data(), i, P.r[i]);
    }
    if ((cfg.forces & SPHGPU_FORCE_SELF_GRAVITY) && n > 0) {
        selfGravity(cfg, n, r.data(), P.m.data(), acc);
    }
    for (uint32_t i = 0; i < n; ++i) {
        const V4 a = load4(acc.data(), i);
        P.dv[i] = V4{ a.x, a.y, a.z, 0. };
        P.v[i].h = 0.;
    }
}

// leap-frog drift (core/timestepping/TimeStepping.cpp:358-361, 385-388)
void nbDrift(NbParts& P, uint32_t n, double dt) {
    for (uint32_t i = 0; i < n; ++i) {
        const V4 v = P.v[i];
        P.r[i].x += v.x * 0.5 * dt;
        P.r[i].y += v.y * 0.5 * dt;
        P.r[i].z += v.z * 0.5 * dt;
        P.r[i].h += v.h * 0.5 * dt;
    }
}

bool nbValid(const sphgpu_config* cfg, const ora_nbody_state* st) {
    return cfg && st && cfg->solver_type == SPHGPU_SOLVER_NBODY_HARD_SPHERE && (st->n == 0 || (st->r && st->v && st->m));
}

} // namespace

extern "C" {

int ora_nbody_collide(const sphgpu_config* cfg, ora_nbody_state* st, double dt, uint64_t stats[4],
    uint64_t* ambiguous, uint32_t* origin, uint32_t* prev_removed, uint32_t* prev_count) {
    if (!nbValid(cfg, st) || !stats) {
        return SPHGPU_ERR_ARGUMENT;
    }
    NbParts P = nbLoad(*st);
    uint32_t n = st->n;
    std::vector<uint32_t> prev;
    if (prev_removed && prev_count) {
        prev.assign(prev_removed, prev_removed + *prev_count);
    }
    nbCollide(*cfg, P, n, dt, stats, ambiguous, prev, origin);
    if (prev_removed && prev_count) {
        std::copy(prev.begin(), prev.end(), prev_removed);
        *prev_count = uint32_t(prev.size());
    }
    nbStore(P, n, *st);
    return SPHGPU_OK;
}

int ora_nbody_integrate(const sphgpu_config* cfg, ora_nbody_state* st) {
    if (!nbValid(cfg, st) || !st->dv) {
        return SPHGPU_ERR_ARGUMENT;
    }
    NbParts P = nbLoad(*st);
    gCache = GravityCache();
    nbIntegrate(*cfg, P, st->n);
    nbStore(P, st->n, *st);
    return SPHGPU_OK;
}

// LeapFrog::stepParticles with HardSphereSolver (core/timestepping/TimeStepping.cpp:352-391) and, with the
// ACCELERATION bit, MultiCriterion of AccelerationCriterion (core/timestepping/TimeStepCriterion.cpp:221-257,
// 389-420); without criteria the step stays fixed
int ora_nbody_run(const sphgpu_config* cfg, ora_nbody_state* st, uint32_t nsteps, double* dt, double* dts,
    uint64_t stats[4], uint64_t* ambiguous, uint32_t* counts) {
    if (!nbValid(cfg, st) || !st->dv || !dt || !stats) {
        return SPHGPU_ERR_ARGUMENT;
    }
    NbParts P = nbLoad(*st);
    uint32_t n = st->n;
    std::vector<uint32_t> prev;
    const double maxChange = cfg->max_change > 0. ? cfg->max_change : INFTY;
    gCache = GravityCache();
    for (uint32_t k = 0; k < nsteps; ++k) {
        const double h = *dt;
        if (dts) {
            dts[k] = h;
        }
        nbCollide(*cfg, P, n, 0.5 * h, stats, ambiguous, prev);
        nbDrift(P, n, h);
        nbIntegrate(*cfg, P, n);
        for (uint32_t i = 0; i < n; ++i) {
            P.v[i].x += P.dv[i].x * h;
            P.v[i].y += P.dv[i].y * h;
            P.v[i].z += P.dv[i].z * h;
            P.v[i].h += P.dv[i].h * h;
        }
        nbCollide(*cfg, P, n, 0.5 * h, stats, ambiguous, prev);
        nbDrift(P, n, h);
        gCache.runTime += h;
        if (cfg->timestep_criteria & SPHGPU_CRITERION_ACCELERATION) {
            double minStep = INFTY;
            for (uint32_t i = 0; i < n; ++i) {
                const double a2 = sqrLen(P.dv[i]);
                if (a2 > EPS) {
                    minStep = std::min(minStep, cfg->derivative_factor * std::sqrt(std::sqrt(P.r[i].h * P.r[i].h / a2)));
                }
            }
            if (minStep > cfg->max_timestep) {
                minStep = cfg->max_timestep;
            }
            if (maxChange < INFTY) {
                const double lim = h * (1. + maxChange);
                if (minStep > lim) {
                    minStep = lim;
                }
            }
            *dt = minStep;
        }
        if (counts) {
            counts[k] = n;
        }
    }
    nbStore(P, n, *st);
    return SPHGPU_OK;
}

} // extern "C"
