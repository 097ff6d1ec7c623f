// adjoint.cu — hand-written reverse mode of the hydrodynamic step over frozen neighbour lists.
//
// The differentiated model (no counterpart in the reference, which has no differentiation): ideal gas
// (IdealGasEos, core/physics/Eos.cpp:42-45), ContinuityEquation + PressureForce + StandardAV
// (core/sph/equations/EquationTerm.cpp:42-99, 289-316; core/sph/equations/av/Standard.h:63-83) with the
// cubic-spline LUT kernel (core/sph/kernel/Kernel.h:51-188), leap-frog (core/timestepping/TimeStepping.cpp:
// 352-391) with a fixed time step and constant smoothing lengths. The neighbour list of every particle (all
// j != i with |r_i - r_j| < 2 * 0.5 (h_i + h_j), sorted by j) is rebuilt every `rebuild_every` steps from
// the state at that step and held fixed in between, which makes each step a smooth function of the state
// except at the AV switch v_ij . r_ij < 0. Loss = sum over particles [0, n_target) of |v|^2 at the end.
//
// One step from (r, v, rho, u):
//   r' = r + v dt/2, p = (gamma - 1) u rho, c = sqrt(gamma p / rho), P = p / rho^2        (prepare kernel)
//   pair sums over the frozen list: divv, a, heat; then rho+ = rho - rho divv dt,
//   u+ = u + (heat - p / rho divv) dt, v+ = v + a dt, r+ = r' + v+ dt/2                  (pair kernel)
//
// Forward: ping-pong state, a checkpoint of (r, v, rho, u) at the first step of every segment of
// `checkpoint_every` steps; the states of the last segment are kept, so its reverse needs no recomputation.
// Backward: segments in reverse; each is recomputed from its checkpoint keeping the state entering every
// step (and its velocity divergence), then its steps are reversed. The reverse of the pair sums is a gather:
// particle k sums, over its neighbours j, the adjoint of both ordered pairs (k, j) and (j, k). Both are
// linear in the adjoint seeds of their first particle, so their contributions to k combine into one vector
// through the shared pair quantities (separation, kernel gradient and its derivative, AV factor), evaluated
// once per neighbour. No atomics; results are deterministic.
//
// Precision: SPHGPU_PRECISION_FP64 evaluates every pair term in FP64 in the expression order of the oracle's
// restatement (this unit is compiled without FMA contraction), so the FP64 forward loss is bit-identical to
// it. SPHGPU_PRECISION_MIXED evaluates the pair terms in FP32 from hi + lo float pairs of the drifted
// positions and velocities (neighbour differences keep FP64-level relative accuracy) with compensated FP32
// sums; the per-particle update and its adjoint, the state and the checkpoints stay FP64.

#include <cub/device/device_scan.cuh>
#include <cub/device/device_segmented_sort.cuh>

#include <algorithm>
#include <cstring>
#include <type_traits>

#include "state.h"

namespace sphgpu {

namespace {

constexpr int ADJ_THREADS = 128;
constexpr int ADJ_PREP_THREADS = 256;
constexpr int RED_THREADS = 256;

struct StepParams {
    double dt, gamma, alpha, beta;
    uint32_t n;
};

// particle state entering a step (FP64)
struct StateView {
    const dbl4* r;
    const dbl4* v;
    const double* rho;
    const double* u;
};
struct StateOut {
    dbl4* r;
    dbl4* v;
    double* rho;
    double* u;
};

// adjoint of a state: 8 component arrays of n doubles (r x y z, v x y z, rho, u)
struct Adj {
    double* a[8];
};

// pair-loop records of one step. FP64: q0 = (r', h), q1 = (v, m), q2 = (rho, P, c, p),
// q3 = (abar, divvbar), q4 = heatbar. Mixed: f0 = (r' hi, h), f1 = (r' lo, m), f2 = (v hi, rho),
// f3 = (v lo, P), f4 = (abar, c), f5 = (divvbar, heatbar).
struct Records {
    dbl4 *q0, *q1, *q2, *q3;
    double* q4;
    float4 *f0, *f1, *f2, *f3, *f4;
    float2* f5;
};

struct ListView {
    const uint32_t* start;
    const uint32_t* idx;
};

// LutKernel gradient table as a piecewise-linear function of q^2 (core/sph/kernel/Kernel.h:92-104): value and
// slope with respect to q^2
__device__ __forceinline__ void lutEval(const double* __restrict__ lut, double q2, double& L, double& dL) {
    if (q2 >= 4.) {
        L = 0.;
        dL = 0.;
        return;
    }
    const double scale = double(LUT_ENTRIES) * 0.25; // entries / radius^2
    const double f = scale * q2;
    const int i1 = min(int(f), LUT_ENTRIES - 1);
    const double ratio = f - double(i1);
    const double g0 = __ldg(lut + i1), g1 = __ldg(lut + i1 + 1);
    L = g0 * (1. - ratio) + g1 * ratio;
    dL = (g1 - g0) * scale;
}

__device__ __forceinline__ void lutEval(const float* __restrict__ lut, float q2, float& L, float& dL) {
    if (q2 >= 4.f) {
        L = 0.f;
        dL = 0.f;
        return;
    }
    const float scale = float(LUT_ENTRIES) * 0.25f;
    const float f = scale * q2;
    const int i1 = min(int(f), LUT_ENTRIES - 1);
    const float ratio = f - float(i1);
    const float g0 = __ldg(lut + i1), g1 = __ldg(lut + i1 + 1);
    L = g0 * (1.f - ratio) + g1 * ratio;
    dL = (g1 - g0) * scale;
}

// running sum: plain in FP64, Kahan-compensated in FP32
template <typename T>
struct CSum {
    T s = T(0);
    __device__ __forceinline__ void add(T x) { s += x; }
    __device__ __forceinline__ double value() const { return double(s); }
};
template <>
struct CSum<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return double(s) - double(c); }
};

__device__ __forceinline__ void splitF(double x, float& hi, float& lo) {
    hi = float(x);
    lo = float(x - double(hi));
}

// own particle as seen by the pair loop
template <typename T>
struct Own {
    T x[3], xl[3], v[3], vl[3];
    T h, m, rho, P, c;
    T ab[3], divvb, heatb;
};

// neighbour j relative to the own particle: d = r'_own - r'_j, w = v_own - v_j
template <typename T>
struct Nb {
    T d[3], w[3];
    T h, m, rho, P, c;
    T ab[3], divvb, heatb;
};

template <bool Mixed>
using Real = std::conditional_t<Mixed, float, double>;

template <bool Mixed, bool Seeds>
__device__ __forceinline__ Own<Real<Mixed>> loadOwn(const Records& R, uint32_t i) {
    Own<Real<Mixed>> o;
    if constexpr (Mixed) {
        const float4 a = R.f0[i], b = R.f1[i], c = R.f2[i], d = R.f3[i], e = R.f4[i];
        o.x[0] = a.x, o.x[1] = a.y, o.x[2] = a.z, o.h = a.w;
        o.xl[0] = b.x, o.xl[1] = b.y, o.xl[2] = b.z, o.m = b.w;
        o.v[0] = c.x, o.v[1] = c.y, o.v[2] = c.z, o.rho = c.w;
        o.vl[0] = d.x, o.vl[1] = d.y, o.vl[2] = d.z, o.P = d.w;
        o.c = e.w;
        if constexpr (Seeds) {
            const float2 f = R.f5[i];
            o.ab[0] = e.x, o.ab[1] = e.y, o.ab[2] = e.z;
            o.divvb = f.x, o.heatb = f.y;
        }
    } else {
        const dbl4 a = R.q0[i], b = R.q1[i], c = R.q2[i];
        o.x[0] = a.x, o.x[1] = a.y, o.x[2] = a.z, o.h = a.w;
        o.v[0] = b.x, o.v[1] = b.y, o.v[2] = b.z, o.m = b.w;
        o.rho = c.x, o.P = c.y, o.c = c.z;
        if constexpr (Seeds) {
            const dbl4 d = R.q3[i];
            o.ab[0] = d.x, o.ab[1] = d.y, o.ab[2] = d.z, o.divvb = d.w;
            o.heatb = R.q4[i];
        }
    }
    return o;
}

template <bool Mixed, bool Seeds>
__device__ __forceinline__ Nb<Real<Mixed>> loadNb(const Records& R, const Own<Real<Mixed>>& o, uint32_t j) {
    Nb<Real<Mixed>> n;
    if constexpr (Mixed) {
        const float4 a = R.f0[j], b = R.f1[j], c = R.f2[j], d = R.f3[j], e = R.f4[j];
        // the hi differences of neighbours are exact or nearly so; the lo parts restore the FP64 residue
        n.d[0] = (o.x[0] - a.x) + (o.xl[0] - b.x);
        n.d[1] = (o.x[1] - a.y) + (o.xl[1] - b.y);
        n.d[2] = (o.x[2] - a.z) + (o.xl[2] - b.z);
        n.w[0] = (o.v[0] - c.x) + (o.vl[0] - d.x);
        n.w[1] = (o.v[1] - c.y) + (o.vl[1] - d.y);
        n.w[2] = (o.v[2] - c.z) + (o.vl[2] - d.z);
        n.h = a.w, n.m = b.w, n.rho = c.w, n.P = d.w, n.c = e.w;
        if constexpr (Seeds) {
            const float2 f = R.f5[j];
            n.ab[0] = e.x, n.ab[1] = e.y, n.ab[2] = e.z;
            n.divvb = f.x, n.heatb = f.y;
        }
    } else {
        const dbl4 a = R.q0[j], b = R.q1[j], c = R.q2[j];
        n.d[0] = o.x[0] - a.x;
        n.d[1] = o.x[1] - a.y;
        n.d[2] = o.x[2] - a.z;
        n.w[0] = o.v[0] - b.x;
        n.w[1] = o.v[1] - b.y;
        n.w[2] = o.v[2] - b.z;
        n.h = a.w, n.m = b.w, n.rho = c.x, n.P = c.y, n.c = c.z;
        if constexpr (Seeds) {
            const dbl4 d = R.q3[j];
            n.ab[0] = d.x, n.ab[1] = d.y, n.ab[2] = d.z, n.divvb = d.w;
            n.heatb = R.q4[j];
        }
    }
    return n;
}

// ---- neighbour lists ----------------------------------------------------------------------------------

__global__ void gatherPositions(uint32_t n, const dbl4* __restrict__ r, const uint32_t* __restrict__ perm,
    dbl4* rs) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) {
        rs[s] = r[perm[s]];
    }
}

// the interaction test of the pair loop (core/sph/solvers/SymmetricSolver.cpp:126-130)
__device__ __forceinline__ bool closePair(const dbl4& a, const dbl4& b) {
    const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    const double hbar = 0.5 * (a.w + b.w);
    const double rad = 2. * hbar;
    return dx * dx + dy * dy + dz * dz < rad * rad;
}

// Fill = false: count[i] = neighbours of i; Fill = true: write them from start[i] (cell order, sorted later)
template <bool Fill>
__global__ void listKernel(uint32_t n, const dbl4* __restrict__ rs, const uint32_t* __restrict__ perm,
    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ cstart, const uint32_t* __restrict__ cend,
    const GridInfo* __restrict__ g, uint32_t* count, const uint32_t* __restrict__ start, uint32_t* idx) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) {
        return;
    }
    const uint32_t i = perm[s];
    const dbl4 ri = rs[s];
    const int dx = g->dims[0], dy = g->dims[1], dz = g->dims[2];
    const uint32_t key = keys[s];
    const int cx = int(key % uint32_t(dx)), cy = int((key / uint32_t(dx)) % uint32_t(dy)),
              cz = int(key / (uint32_t(dx) * uint32_t(dy)));
    uint32_t c = 0;
    uint32_t out = 0;
    if (Fill) {
        out = start[i];
    }
    for (int z = max(cz - 1, 0); z <= min(cz + 1, dz - 1); ++z) {
        for (int y = max(cy - 1, 0); y <= min(cy + 1, dy - 1); ++y) {
            for (int x = max(cx - 1, 0); x <= min(cx + 1, dx - 1); ++x) {
                const uint32_t cell = (uint32_t(z) * uint32_t(dy) + uint32_t(y)) * uint32_t(dx) + uint32_t(x);
                const uint32_t e = cend[cell];
                for (uint32_t t = cstart[cell]; t < e; ++t) {
                    if (t == s || !closePair(ri, rs[t])) {
                        continue;
                    }
                    if (Fill) {
                        idx[out++] = perm[t];
                    }
                    ++c;
                }
            }
        }
    }
    if (!Fill) {
        count[i] = c;
    }
}

// ---- prepare: drift, EOS and the pair-loop records (plus the adjoint seeds in the reverse pass) -----------

template <bool Mixed, bool Seeds>
__global__ void prepareKernel(StepParams prm, StateView s, const double* __restrict__ m, Adj in, Records R,
    StateOut keep, StateOut ckpt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= prm.n) {
        return;
    }
    const dbl4 r = s.r[i], v = s.v[i];
    const double rho = s.rho[i], u = s.u[i], mi = m[i];
    if (keep.r) {
        keep.r[i] = r;
        keep.v[i] = v;
        keep.rho[i] = rho;
        keep.u[i] = u;
    }
    if (ckpt.r) {
        ckpt.r[i] = r;
        ckpt.v[i] = v;
        ckpt.rho[i] = rho;
        ckpt.u[i] = u;
    }
    const double hdt = 0.5 * prm.dt;
    const double rp[3] = { r.x + v.x * hdt, r.y + v.y * hdt, r.z + v.z * hdt };
    const double p = (prm.gamma - 1.) * u * rho;
    const double c = sqrt(prm.gamma * p / rho);
    const double P = p / (rho * rho);
    double ab[3] = { 0., 0., 0. }, divvb = 0., heatb = 0.;
    if constexpr (Seeds) {
        // adjoint of r+ = r' + v+ dt/2, v+ = v + a dt, rho+ = rho + drho dt, u+ = u + du dt with
        // drho = -rho divv, du = heat - p / rho divv
        const double dt = prm.dt;
        const double drhob = in.a[6][i] * dt, dub = in.a[7][i] * dt;
        for (int k = 0; k < 3; ++k) {
            ab[k] = (in.a[3 + k][i] + in.a[k][i] * hdt) * dt;
        }
        divvb = -rho * drhob - p / rho * dub;
        heatb = dub;
    }
    if constexpr (Mixed) {
        float xh[3], xl[3], vh[3], vl[3];
        const double vv[3] = { v.x, v.y, v.z };
        for (int k = 0; k < 3; ++k) {
            splitF(rp[k], xh[k], xl[k]);
            splitF(vv[k], vh[k], vl[k]);
        }
        R.f0[i] = make_float4(xh[0], xh[1], xh[2], float(r.w));
        R.f1[i] = make_float4(xl[0], xl[1], xl[2], float(mi));
        R.f2[i] = make_float4(vh[0], vh[1], vh[2], float(rho));
        R.f3[i] = make_float4(vl[0], vl[1], vl[2], float(P));
        R.f4[i] = make_float4(float(ab[0]), float(ab[1]), float(ab[2]), float(c));
        if constexpr (Seeds) {
            R.f5[i] = make_float2(float(divvb), float(heatb));
        }
    } else {
        R.q0[i] = mkd4(rp[0], rp[1], rp[2], r.w);
        R.q1[i] = mkd4(v.x, v.y, v.z, mi);
        R.q2[i] = mkd4(rho, P, c, p);
        if constexpr (Seeds) {
            R.q3[i] = mkd4(ab[0], ab[1], ab[2], divvb);
            R.q4[i] = heatb;
        }
    }
}

// ---- forward pair sums + update ---------------------------------------------------------------------------

template <bool Mixed>
__global__ void __launch_bounds__(ADJ_THREADS) forwardPairKernel(StepParams prm, ListView L, Records R,
    const double* __restrict__ lut_d, const float* __restrict__ lut_f, StateView s, StateOut out,
    double* divvOut) {
    using T = Real<Mixed>;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= prm.n) {
        return;
    }
    const T* lut;
    if constexpr (Mixed) {
        lut = lut_f;
    } else {
        lut = lut_d;
    }
    const Own<T> o = loadOwn<Mixed, false>(R, i);
    const T alpha = T(prm.alpha), beta = T(prm.beta);
    CSum<T> ax, ay, az, dv, ht;
    const uint32_t e1 = L.start[i + 1];
    for (uint32_t e = L.start[i]; e < e1; ++e) {
        const uint32_t j = L.idx[e];
        const Nb<T> q = loadNb<Mixed, false>(R, o, j);
        // the terms in the expression order of the oracle's restatement (bit-identical in FP64)
        const T hbar = T(0.5) * (o.h + q.h);
        const T dx = q.d[0], dy = q.d[1], dz = q.d[2];
        const T s2 = dx * dx + dy * dy + dz * dz;
        const T hInv = T(1) / hbar;
        const T h5 = hInv * hInv * hInv * hInv * hInv;
        T Lv, dLv;
        lutEval(lut, s2 * (hInv * hInv), Lv, dLv);
        const T F = h5 * Lv;
        const T gx = dx * F, gy = dy * F, gz = dz * F;
        const T vjx = -q.w[0], vjy = -q.w[1], vjz = -q.w[2];
        const T Tq = vjx * gx + vjy * gy + vjz * gz;
        dv.add(q.m / o.rho * Tq);
        T coef = -(o.P + q.P);
        const T wd = -(vjx * dx + vjy * dy + vjz * dz);
        if (wd < T(0)) {
            const T D = s2 + T(1.e-2) * hbar * hbar;
            const T mu = hbar * wd / D;
            const T rb = T(0.5) * (o.rho + q.rho);
            const T cb = T(0.5) * (o.c + q.c);
            const T Pav = (-alpha * cb * mu + beta * mu * mu) / rb;
            coef = coef - Pav;
            ht.add(q.m * T(0.5) * Pav * -Tq);
        }
        ax.add(q.m * coef * gx);
        ay.add(q.m * coef * gy);
        az.add(q.m * coef * gz);
    }
    // FP64 update (leap-frog kick + drift, continuity, energy)
    const double dt = prm.dt, hdt = 0.5 * prm.dt;
    const dbl4 r = s.r[i], v = s.v[i];
    const double rho = s.rho[i], u = s.u[i];
    const double rp[3] = { r.x + v.x * hdt, r.y + v.y * hdt, r.z + v.z * hdt };
    const double p = (prm.gamma - 1.) * u * rho;
    const double divv = dv.value(), heat = ht.value();
    const double drho = -rho * divv;
    const double du = heat - p / rho * divv;
    out.rho[i] = rho + drho * dt;
    out.u[i] = u + du * dt;
    const double nv[3] = { v.x + ax.value() * dt, v.y + ay.value() * dt, v.z + az.value() * dt };
    out.v[i] = mkd4(nv[0], nv[1], nv[2], v.w);
    out.r[i] = mkd4(rp[0] + nv[0] * hdt, rp[1] + nv[1] * hdt, rp[2] + nv[2] * hdt, r.w);
    if (divvOut) {
        divvOut[i] = divv;
    }
}

// ---- reverse of one step ------------------------------------------------------------------------------

template <bool Mixed>
__global__ void __launch_bounds__(ADJ_THREADS) backwardPairKernel(StepParams prm, ListView L, Records R,
    const double* __restrict__ lut_d, const float* __restrict__ lut_f, StateView s,
    const double* __restrict__ divvIn, Adj in, Adj out, double* alphaAcc) {
    using T = Real<Mixed>;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= prm.n) {
        return;
    }
    const T* lut;
    if constexpr (Mixed) {
        lut = lut_f;
    } else {
        lut = lut_d;
    }
    const Own<T> o = loadOwn<Mixed, true>(R, k);
    const T alpha = T(prm.alpha), beta = T(prm.beta);
    CSum<T> rpb[3], vb[3], rhob, Pb, cb, alb;
    const uint32_t e1 = L.start[k + 1];
    for (uint32_t e = L.start[k]; e < e1; ++e) {
        const uint32_t j = L.idx[e];
        const Nb<T> q = loadNb<Mixed, true>(R, o, j);
        const T hbar = T(0.5) * (o.h + q.h);
        const T s2 = q.d[0] * q.d[0] + q.d[1] * q.d[1] + q.d[2] * q.d[2];
        const T hInv = T(1) / hbar;
        const T hInv2 = hInv * hInv;
        const T h5 = hInv2 * hInv2 * hInv;
        T Lv, dLv;
        lutEval(lut, s2 * hInv2, Lv, dLv);
        const T F = h5 * Lv;
        const T Fp = h5 * dLv * hInv2; // dF / d(s2)
        const T g[3] = { q.d[0] * F, q.d[1] * F, q.d[2] * F };
        const T wg = q.w[0] * g[0] + q.w[1] * g[1] + q.w[2] * g[2];
        const T wd = q.w[0] * q.d[0] + q.w[1] * q.d[1] + q.w[2] * q.d[2];
        const T akg = o.ab[0] * g[0] + o.ab[1] * g[1] + o.ab[2] * g[2];
        const T ajg = q.ab[0] * g[0] + q.ab[1] * g[1] + q.ab[2] * g[2];
        const bool av = wd < T(0);
        T Pav = T(0), D = T(1), mu = T(0), rb = T(1), cbar = T(0);
        if (av) {
            D = s2 + T(1.e-2) * hbar * hbar;
            mu = hbar * wd / D;
            rb = T(0.5) * (o.rho + q.rho);
            cbar = T(0.5) * (o.c + q.c);
            Pav = (-alpha * cbar * mu + beta * mu * mu) / rb;
        }
        // ordered pairs (k, j) with k's seeds and (j, k) with j's seeds, combined in k's frame
        // (d = r'_k - r'_j, w = v_k - v_j, g = grad W at d); G is the adjoint of g, Wb that of w
        const T cds = o.divvb * q.m / o.rho + q.divvb * o.m / q.rho;
        const T H = T(0.5) * (o.heatb * q.m + q.heatb * o.m);
        const T Ck = q.m * (-(o.P + q.P) - Pav);
        const T Cj = o.m * (-(q.P + o.P) - Pav);
        const T wcoef = H * Pav - cds;
        T G[3], Wb[3];
        for (int c = 0; c < 3; ++c) {
            G[c] = wcoef * q.w[c] + Ck * o.ab[c] - Cj * q.ab[c];
            Wb[c] = wcoef * g[c];
        }
        const T Pbk = -q.m * akg + o.heatb * q.m * T(0.5) * wg;
        const T Pbj = o.m * ajg + q.heatb * o.m * T(0.5) * wg;
        rhob.add(o.divvb * q.m * wg / (o.rho * o.rho));
        Pb.add(-q.m * akg + o.m * ajg);
        T dcoef = T(2) * (G[0] * q.d[0] + G[1] * q.d[1] + G[2] * q.d[2]) * Fp;
        T db[3] = { F * G[0], F * G[1], F * G[2] };
        if (av) {
            const T PavB = Pbk + Pbj;
            const T mub = PavB * (-alpha * cbar + T(2) * beta * mu) / rb;
            const T wdb = mub * hbar / D;
            const T Db = -mub * mu / D;
            dcoef += T(2) * Db;
            for (int c = 0; c < 3; ++c) {
                Wb[c] += wdb * q.d[c];
                db[c] += wdb * q.w[c];
            }
            rhob.add(T(-0.5) * PavB * Pav / rb);
            cb.add(T(-0.5) * PavB * alpha * mu / rb);
            alb.add(-Pbk * cbar * mu / rb);
        }
        for (int c = 0; c < 3; ++c) {
            rpb[c].add(db[c] + dcoef * q.d[c]);
            vb[c].add(Wb[c]);
        }
    }
    // per-particle parts in FP64: kick + drift, continuity, energy, P = p / rho^2, sound speed, EOS, first drift
    const double dt = prm.dt, hdt = 0.5 * prm.dt, gamma = prm.gamma;
    const double rho = s.rho[k], u = s.u[k], divv = divvIn[k];
    const double p = (gamma - 1.) * u * rho;
    const double c = sqrt(gamma * p / rho);
    const double drhob = in.a[6][k] * dt, dub = in.a[7][k] * dt;
    double rpB[3], vB[3];
    for (int q = 0; q < 3; ++q) {
        const double rbo = in.a[q][k];
        rpB[q] = rpb[q].value() + rbo;
        vB[q] = vb[q].value() + in.a[3 + q][k] + rbo * hdt;
    }
    double rhoB = rhob.value() + in.a[6][k] - divv * drhob + p / (rho * rho) * divv * dub;
    const double PB = Pb.value(), cB = cb.value();
    double pB = -divv / rho * dub + PB / (rho * rho);
    rhoB -= 2. * p * PB / (rho * rho * rho);
    if (c > 0.) {
        pB += cB * gamma / (2. * c * rho);
        rhoB -= cB * gamma * p / (2. * c * rho * rho);
    }
    const double uB = in.a[7][k] + pB * (gamma - 1.) * rho;
    rhoB += pB * (gamma - 1.) * u;
    for (int q = 0; q < 3; ++q) {
        out.a[q][k] = rpB[q];
        out.a[3 + q][k] = vB[q] + rpB[q] * hdt;
    }
    out.a[6][k] = rhoB;
    out.a[7][k] = uB;
    alphaAcc[k] += alb.value();
}

// adjoint of the loss: dL/dv = 2 v for the targets, scaled by the loss adjoint
__global__ void lossSeedKernel(uint32_t n, uint32_t nTarget, const dbl4* __restrict__ v, double scale, Adj out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const dbl4 vi = v[i];
    const double f = i < nTarget ? 2. * scale : 0.;
    out.a[0][i] = 0.;
    out.a[1][i] = 0.;
    out.a[2][i] = 0.;
    out.a[3][i] = f * vi.x;
    out.a[4][i] = f * vi.y;
    out.a[5][i] = f * vi.z;
    out.a[6][i] = 0.;
    out.a[7][i] = 0.;
}

// block-ordered sums (deterministic): part[b] = (sum of |v|^2 over targets, sum of acc) over block b
__global__ void __launch_bounds__(RED_THREADS) reducePartKernel(uint32_t n, uint32_t nTarget,
    const dbl4* __restrict__ v, const double* __restrict__ acc, double* part) {
    __shared__ double sh[2][RED_THREADS];
    const uint32_t i = blockIdx.x * RED_THREADS + threadIdx.x;
    double l = 0., a = 0.;
    if (i < n) {
        if (v && i < nTarget) {
            const dbl4 vi = v[i];
            l = vi.x * vi.x + vi.y * vi.y + vi.z * vi.z;
        }
        if (acc) {
            a = acc[i];
        }
    }
    sh[0][threadIdx.x] = l;
    sh[1][threadIdx.x] = a;
    __syncthreads();
    for (int off = RED_THREADS / 2; off > 0; off >>= 1) {
        if (int(threadIdx.x) < off) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + off];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + off];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = sh[0][0];
        part[2 * blockIdx.x + 1] = sh[1][0];
    }
}

__global__ void reduceFinalKernel(uint32_t blocks, const double* __restrict__ part, double* out) {
    if (threadIdx.x < 2) {
        double acc = 0.;
        for (uint32_t b = 0; b < blocks; ++b) {
            acc += part[2 * b + threadIdx.x];
        }
        out[threadIdx.x] = acc;
    }
}

// SoA adjoint -> the host layout of r and v (4 doubles per particle; the 4th, h, is held constant: 0)
__global__ void packGradKernel(uint32_t n, Adj a, double* gr, double* gv) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    gr[4 * i] = a.a[0][i];
    gr[4 * i + 1] = a.a[1][i];
    gr[4 * i + 2] = a.a[2][i];
    gr[4 * i + 3] = 0.;
    gv[4 * i] = a.a[3][i];
    gv[4 * i + 1] = a.a[4][i];
    gv[4 * i + 2] = a.a[5][i];
    gv[4 * i + 3] = 0.;
}

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count * sizeof(T), 16));
}

} // namespace

// ---- host orchestration -------------------------------------------------------------------------------

struct AdjointState {
    sphgpu_adjoint_config cfg{};
    uint32_t n = 0;
    uint32_t segments = 0;
    uint32_t seg_steps = 0;   // steps held by the segment buffers
    bool mixed = false;
    // frozen neighbour list (CSR, sorted by neighbour index)
    uint32_t* count = nullptr;
    uint32_t* start = nullptr;
    uint32_t* list = nullptr;
    uint32_t* list_tmp = nullptr;
    uint64_t list_capacity = 0;
    void* scan_temp = nullptr;
    size_t scan_bytes = 0;
    void* sort_temp = nullptr;
    size_t sort_bytes = 0;
    int64_t list_id = -1;     // rebuild interval the list in memory belongs to
    uint64_t list_entries = 0;
    // ping-pong state
    dbl4* r[2] = { nullptr, nullptr };
    dbl4* v[2] = { nullptr, nullptr };
    double* rho[2] = { nullptr, nullptr };
    double* u[2] = { nullptr, nullptr };
    // states entering each step of one segment, and their velocity divergence
    dbl4* seg_r = nullptr;
    dbl4* seg_v = nullptr;
    double* seg_rho = nullptr;
    double* seg_u = nullptr;
    double* seg_divv = nullptr;
    int64_t seg_kept = -1;    // segment whose states are in the segment buffers
    // checkpoints: state at the first step of each segment
    dbl4* ck_r = nullptr;
    dbl4* ck_v = nullptr;
    double* ck_rho = nullptr;
    double* ck_u = nullptr;
    dbl4* final_v = nullptr;
    Records rec{};
    double* adj[2][8] = {};
    int adj_cur = 0;
    double* alpha_acc = nullptr;
    double* part = nullptr;
    double* result = nullptr;
    double* host_result = nullptr; // pinned
    double* grad_stage = nullptr;  // 8n: packed r and v gradients
    bool forward_done = false;
    bool backward_done = false;
    unsigned long long launches = 0;
};

namespace {

void freeAll(AdjointState* a) {
    void* ptrs[] = { a->count, a->start, a->list, a->list_tmp, a->scan_temp, a->sort_temp, a->r[0], a->r[1], a->v[0],
        a->v[1], a->rho[0], a->rho[1], a->u[0], a->u[1], a->seg_r, a->seg_v, a->seg_rho, a->seg_u, a->seg_divv,
        a->ck_r, a->ck_v, a->ck_rho, a->ck_u, a->final_v, a->rec.q0, a->rec.q1, a->rec.q2, a->rec.q3, a->rec.q4,
        a->rec.f0, a->rec.f1, a->rec.f2, a->rec.f3, a->rec.f4, a->rec.f5, a->alpha_acc, a->part, a->result,
        a->grad_stage };
    for (void* p : ptrs) {
        if (p) {
            cudaFree(p);
        }
    }
    for (auto& set : a->adj) {
        for (double* p : set) {
            if (p) {
                cudaFree(p);
            }
        }
    }
    if (a->host_result) {
        cudaFreeHost(a->host_result);
    }
}

StepParams stepParams(const AdjointState* a) {
    StepParams p;
    p.dt = a->cfg.dt;
    p.gamma = a->cfg.gamma;
    p.alpha = a->cfg.alpha;
    p.beta = a->cfg.beta;
    p.n = a->n;
    return p;
}

Adj adjSet(AdjointState* a, int which) {
    Adj x;
    for (int k = 0; k < 8; ++k) {
        x.a[k] = a->adj[which][k];
    }
    return x;
}

StateView view(const AdjointState* a, int b) {
    return StateView{ a->r[b], a->v[b], a->rho[b], a->u[b] };
}
StateOut outView(AdjointState* a, int b) {
    return StateOut{ a->r[b], a->v[b], a->rho[b], a->u[b] };
}
StateOut segSlot(AdjointState* a, uint32_t q) {
    const size_t o = size_t(q) * a->n;
    return StateOut{ a->seg_r + o, a->seg_v + o, a->seg_rho + o, a->seg_u + o };
}
StateOut ckSlot(AdjointState* a, uint32_t c) {
    const size_t o = size_t(c) * a->n;
    return StateOut{ a->ck_r + o, a->ck_v + o, a->ck_rho + o, a->ck_u + o };
}

cudaError_t growList(AdjointState* a, uint64_t total) {
    if (a->list) {
        cudaFree(a->list);
        a->list = nullptr;
    }
    if (a->list_tmp) {
        cudaFree(a->list_tmp);
        a->list_tmp = nullptr;
    }
    a->list_capacity = total + total / 4 + 1024;
    cudaError_t e = dalloc(&a->list, a->list_capacity);
    if (e == cudaSuccess) {
        e = dalloc(&a->list_tmp, a->list_capacity);
    }
    if (e != cudaSuccess) {
        a->list_capacity = 0;
    }
    return e;
}

// Builds the frozen lists from positions r with the handle's neighbour grid (its cell-sorted position copy
// is overwritten).
cudaError_t buildList(AdjointState* a, const DState& s0, Grid& grid, const Physics& ph, const dbl4* r,
    cudaStream_t st) {
    const uint32_t n = a->n;
    DState s = s0;
    s.r = const_cast<dbl4*>(r);
    launchGridBuild(s, grid, ph, st);
    a->launches += grid.launches;
    const uint32_t blocks = ceilDiv(n, 128);
    gatherPositions<<<ceilDiv(n, 256), 256, 0, st>>>(n, r, grid.perm, grid.rs);
    listKernel<false><<<blocks, 128, 0, st>>>(n, grid.rs, grid.perm, grid.keys_sorted, grid.cell_start,
        grid.cell_end, grid.info, a->count, nullptr, nullptr);
    a->launches += 2;
    cudaError_t e = cudaMemsetAsync(a->count + n, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) {
        return e;
    }
    size_t bytes = a->scan_bytes;
    e = cub::DeviceScan::ExclusiveSum(a->scan_temp, bytes, a->count, a->start, int(n + 1), st);
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(a->host_result, a->start + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) {
        return e;
    }
    uint32_t total = 0;
    std::memcpy(&total, a->host_result, sizeof(uint32_t));
    if (uint64_t(total) > a->list_capacity) {
        e = growList(a, total);
        if (e != cudaSuccess) {
            return e;
        }
    }
    size_t need = 0;
    e = cub::DeviceSegmentedSort::SortKeys(nullptr, need, a->list_tmp, a->list, int(total), int(n), a->start,
        a->start + 1, st);
    if (e == cudaSuccess && need > a->sort_bytes) {
        if (a->sort_temp) {
            cudaFree(a->sort_temp);
            a->sort_temp = nullptr;
        }
        a->sort_bytes = 0;
        e = cudaMalloc(&a->sort_temp, need);
        if (e == cudaSuccess) {
            a->sort_bytes = need;
        }
    }
    if (e != cudaSuccess) {
        return e;
    }
    listKernel<true><<<blocks, 128, 0, st>>>(n, grid.rs, grid.perm, grid.keys_sorted, grid.cell_start,
        grid.cell_end, grid.info, nullptr, a->start, a->list_tmp);
    a->launches += 1;
    bytes = a->sort_bytes;
    e = cub::DeviceSegmentedSort::SortKeys(a->sort_temp, bytes, a->list_tmp, a->list, int(total), int(n), a->start,
        a->start + 1, st);
    a->list_entries = total;
    if (e != cudaSuccess) {
        return e;
    }
    return cudaGetLastError();
}

// one forward step from ping-pong buffer `from` into the other; keep / ck (may be empty) receive the entering
// state, divvOut (may be null) the velocity divergence
void forwardStep(AdjointState* a, const DState& s, const double* lut, const float* lutf, int from, StateOut keep,
    StateOut ck, double* divvOut, cudaStream_t st) {
    const uint32_t n = a->n;
    const StepParams prm = stepParams(a);
    const Adj none{};
    const ListView L{ a->start, a->list };
    if (a->mixed) {
        prepareKernel<true, false><<<ceilDiv(n, ADJ_PREP_THREADS), ADJ_PREP_THREADS, 0, st>>>(prm, view(a, from),
            s.m, none, a->rec, keep, ck);
        forwardPairKernel<true><<<ceilDiv(n, ADJ_THREADS), ADJ_THREADS, 0, st>>>(prm, L, a->rec, lut, lutf,
            view(a, from), outView(a, 1 - from), divvOut);
    } else {
        prepareKernel<false, false><<<ceilDiv(n, ADJ_PREP_THREADS), ADJ_PREP_THREADS, 0, st>>>(prm, view(a, from),
            s.m, none, a->rec, keep, ck);
        forwardPairKernel<false><<<ceilDiv(n, ADJ_THREADS), ADJ_THREADS, 0, st>>>(prm, L, a->rec, lut, lutf,
            view(a, from), outView(a, 1 - from), divvOut);
    }
    a->launches += 2;
}

// reverse of step q of the segment in the segment buffers: adjoint set adj_cur -> the other set
void backwardStep(AdjointState* a, const DState& s, const double* lut, const float* lutf, uint32_t q,
    cudaStream_t st) {
    const uint32_t n = a->n;
    const StepParams prm = stepParams(a);
    const size_t o = size_t(q) * n;
    const StateView sv{ a->seg_r + o, a->seg_v + o, a->seg_rho + o, a->seg_u + o };
    const Adj in = adjSet(a, a->adj_cur), out = adjSet(a, 1 - a->adj_cur);
    const ListView L{ a->start, a->list };
    const StateOut none{};
    if (a->mixed) {
        prepareKernel<true, true><<<ceilDiv(n, ADJ_PREP_THREADS), ADJ_PREP_THREADS, 0, st>>>(prm, sv, s.m, in,
            a->rec, none, none);
        backwardPairKernel<true><<<ceilDiv(n, ADJ_THREADS), ADJ_THREADS, 0, st>>>(prm, L, a->rec, lut, lutf, sv,
            a->seg_divv + o, in, out, a->alpha_acc);
    } else {
        prepareKernel<false, true><<<ceilDiv(n, ADJ_PREP_THREADS), ADJ_PREP_THREADS, 0, st>>>(prm, sv, s.m, in,
            a->rec, none, none);
        backwardPairKernel<false><<<ceilDiv(n, ADJ_THREADS), ADJ_THREADS, 0, st>>>(prm, L, a->rec, lut, lutf, sv,
            a->seg_divv + o, in, out, a->alpha_acc);
    }
    a->launches += 2;
    a->adj_cur = 1 - a->adj_cur;
}

cudaError_t copyState(AdjointState* a, int to, const dbl4* r, const dbl4* v, const double* rho, const double* u,
    cudaStream_t st) {
    const uint32_t n = a->n;
    cudaError_t e = cudaMemcpyAsync(a->r[to], r, n * sizeof(dbl4), cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(a->v[to], v, n * sizeof(dbl4), cudaMemcpyDeviceToDevice, st);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(a->rho[to], rho, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(a->u[to], u, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
    }
    return e;
}

// (sum |v|^2 over the targets, sum of acc) into host_result[0..1]
cudaError_t reduceToHost(AdjointState* a, const dbl4* v, const double* acc, cudaStream_t st) {
    const uint32_t n = a->n;
    const uint32_t blocks = std::max<uint32_t>(ceilDiv(n, RED_THREADS), 1);
    const uint32_t nt = std::min(a->cfg.n_target, n);
    reducePartKernel<<<blocks, RED_THREADS, 0, st>>>(n, nt, v, acc, a->part);
    reduceFinalKernel<<<1, 32, 0, st>>>(blocks, a->part, a->result);
    a->launches += 2;
    cudaError_t e = cudaMemcpyAsync(a->host_result, a->result, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(st);
    }
    return e;
}

} // namespace

void adjointFree(AdjointState* a) {
    if (a) {
        freeAll(a);
        delete a;
    }
}

cudaError_t adjointConfigure(AdjointState*& a, uint32_t n, const sphgpu_adjoint_config& cfg) {
    const uint32_t segments = cfg.steps == 0 ? 0 : (cfg.steps + cfg.checkpoint_every - 1) / cfg.checkpoint_every;
    const uint32_t segSteps = std::max<uint32_t>(std::min(cfg.checkpoint_every, cfg.steps), 1);
    const bool mixed = cfg.precision == SPHGPU_PRECISION_MIXED;
    if (a && a->n == n && a->segments == segments && a->seg_steps == segSteps && a->mixed == mixed) {
        a->cfg = cfg;
        a->list_id = -1;
        a->seg_kept = -1;
        a->forward_done = false;
        a->backward_done = false;
        return cudaSuccess;
    }
    adjointFree(a);
    a = new AdjointState();
    a->cfg = cfg;
    a->n = n;
    a->segments = segments;
    a->seg_steps = segSteps;
    a->mixed = mixed;
    const size_t nn = std::max<uint32_t>(n, 1);
    const size_t nck = std::max<uint32_t>(segments, 1);
    cudaError_t e = cudaSuccess;
    auto A = [&](auto** p, size_t count) {
        if (e == cudaSuccess) {
            e = dalloc(p, count);
        }
    };
    A(&a->count, nn + 1);
    A(&a->start, nn + 1);
    for (int b = 0; b < 2; ++b) {
        A(&a->r[b], nn);
        A(&a->v[b], nn);
        A(&a->rho[b], nn);
        A(&a->u[b], nn);
        for (int c = 0; c < 8; ++c) {
            A(&a->adj[b][c], nn);
        }
    }
    A(&a->seg_r, nn * segSteps);
    A(&a->seg_v, nn * segSteps);
    A(&a->seg_rho, nn * segSteps);
    A(&a->seg_u, nn * segSteps);
    A(&a->seg_divv, nn * segSteps);
    A(&a->ck_r, nn * nck);
    A(&a->ck_v, nn * nck);
    A(&a->ck_rho, nn * nck);
    A(&a->ck_u, nn * nck);
    A(&a->final_v, nn);
    if (mixed) {
        A(&a->rec.f0, nn);
        A(&a->rec.f1, nn);
        A(&a->rec.f2, nn);
        A(&a->rec.f3, nn);
        A(&a->rec.f4, nn);
        A(&a->rec.f5, nn);
    } else {
        A(&a->rec.q0, nn);
        A(&a->rec.q1, nn);
        A(&a->rec.q2, nn);
        A(&a->rec.q3, nn);
        A(&a->rec.q4, nn);
    }
    A(&a->alpha_acc, nn);
    A(&a->part, 2 * (nn / RED_THREADS + 2));
    A(&a->result, 2);
    A(&a->grad_stage, 8 * nn);
    if (e == cudaSuccess) {
        e = cudaMallocHost(reinterpret_cast<void**>(&a->host_result), 4 * sizeof(double));
    }
    if (e == cudaSuccess) {
        e = cub::DeviceScan::ExclusiveSum(nullptr, a->scan_bytes, a->count, a->start, int(nn + 1));
    }
    if (e == cudaSuccess) {
        e = cudaMalloc(&a->scan_temp, std::max<size_t>(a->scan_bytes, 16));
    }
    if (e != cudaSuccess) {
        adjointFree(a);
        a = nullptr;
    }
    return e;
}

cudaError_t adjointForward(AdjointState* a, const DState& s, Grid& grid, const Physics& ph, const double* lut,
    const float* lutf, double* loss, cudaStream_t st) {
    const uint32_t n = a->n;
    const sphgpu_adjoint_config& cfg = a->cfg;
    a->forward_done = false;
    a->backward_done = false;
    cudaError_t e = copyState(a, 0, s.r, s.v, s.rho, s.u, st);
    if (e != cudaSuccess) {
        return e;
    }
    int cur = 0;
    const uint32_t K = cfg.checkpoint_every, R = cfg.rebuild_every;
    const int64_t last = int64_t(a->segments) - 1;
    for (uint32_t t = 0; t < cfg.steps; ++t) {
        const uint32_t seg = t / K, q = t % K;
        if (t % R == 0) {
            e = buildList(a, s, grid, ph, a->r[cur], st);
            if (e != cudaSuccess) {
                return e;
            }
            a->list_id = t / R;
        }
        const bool keep = int64_t(seg) == last;
        forwardStep(a, s, lut, lutf, cur, keep ? segSlot(a, q) : StateOut{}, q == 0 ? ckSlot(a, seg) : StateOut{},
            keep ? a->seg_divv + size_t(q) * n : nullptr, st);
        cur = 1 - cur;
    }
    a->seg_kept = last;
    e = cudaMemcpyAsync(a->final_v, a->v[cur], std::max<uint32_t>(n, 1) * sizeof(dbl4), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
        return e;
    }
    e = reduceToHost(a, a->final_v, nullptr, st);
    if (e != cudaSuccess) {
        return e;
    }
    *loss = a->host_result[0];
    a->forward_done = true;
    return cudaGetLastError();
}

cudaError_t adjointBackward(AdjointState* a, const DState& s, Grid& grid, const Physics& ph, const double* lut,
    const float* lutf, double lossBar, double* alphaBar, cudaStream_t st) {
    const uint32_t n = a->n;
    const sphgpu_adjoint_config& cfg = a->cfg;
    const uint32_t K = cfg.checkpoint_every, R = cfg.rebuild_every;
    a->backward_done = false;
    a->adj_cur = 0;
    const uint32_t nt = std::min(cfg.n_target, n);
    lossSeedKernel<<<std::max<uint32_t>(ceilDiv(n, 256), 1), 256, 0, st>>>(n, nt, a->final_v, lossBar,
        adjSet(a, 0));
    a->launches += 1;
    cudaError_t e = cudaMemsetAsync(a->alpha_acc, 0, std::max<uint32_t>(n, 1) * sizeof(double), st);
    if (e != cudaSuccess) {
        return e;
    }
    for (int64_t seg = int64_t(a->segments) - 1; seg >= 0; --seg) {
        const uint32_t s0 = uint32_t(seg) * K;
        const uint32_t len = std::min(K, cfg.steps - s0);
        const int64_t need = s0 / R;
        if (need != a->list_id) {
            // the rebuild step need * R starts a segment, since the checkpoint interval divides R
            e = buildList(a, s, grid, ph, ckSlot(a, uint32_t(need * R / K)).r, st);
            if (e != cudaSuccess) {
                return e;
            }
            a->list_id = need;
        }
        if (a->seg_kept != seg) {
            const StateOut c = ckSlot(a, uint32_t(seg));
            e = copyState(a, 0, c.r, c.v, c.rho, c.u, st);
            if (e != cudaSuccess) {
                return e;
            }
            int cur = 0;
            for (uint32_t q = 0; q < len; ++q) {
                forwardStep(a, s, lut, lutf, cur, segSlot(a, q), StateOut{}, a->seg_divv + size_t(q) * n, st);
                cur = 1 - cur;
            }
            a->seg_kept = seg;
        }
        for (int64_t q = int64_t(len) - 1; q >= 0; --q) {
            backwardStep(a, s, lut, lutf, uint32_t(q), st);
        }
    }
    e = reduceToHost(a, nullptr, a->alpha_acc, st);
    if (e != cudaSuccess) {
        return e;
    }
    *alphaBar = a->host_result[1];
    a->backward_done = true;
    return cudaGetLastError();
}

cudaError_t adjointGradients(AdjointState* a, double* gr, double* gv, double* grho, double* gu, cudaStream_t st) {
    const uint32_t n = a->n;
    const Adj g = adjSet(a, a->adj_cur);
    cudaError_t e = cudaSuccess;
    if (n > 0 && (gr || gv)) {
        packGradKernel<<<ceilDiv(n, 256), 256, 0, st>>>(n, g, a->grad_stage, a->grad_stage + 4 * size_t(n));
        a->launches += 1;
        if (gr) {
            e = cudaMemcpyAsync(gr, a->grad_stage, 4 * size_t(n) * sizeof(double), cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess && gv) {
            e = cudaMemcpyAsync(gv, a->grad_stage + 4 * size_t(n), 4 * size_t(n) * sizeof(double),
                cudaMemcpyDeviceToHost, st);
        }
    }
    if (e == cudaSuccess && grho && n > 0) {
        e = cudaMemcpyAsync(grho, g.a[6], n * sizeof(double), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess && gu && n > 0) {
        e = cudaMemcpyAsync(gu, g.a[7], n * sizeof(double), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(st);
    }
    return e;
}

bool adjointForwardDone(const AdjointState* a) {
    return a && a->forward_done;
}

bool adjointBackwardDone(const AdjointState* a) {
    return a && a->backward_done;
}

uint64_t adjointListEntries(const AdjointState* a) {
    return a ? a->list_entries : 0;
}

unsigned long long adjointTakeLaunches(AdjointState* a) {
    if (!a) {
        return 0;
    }
    const unsigned long long l = a->launches;
    a->launches = 0;
    return l;
}

} // namespace sphgpu
