// sph32.cu — mixed-precision SPH pair loop (FP32 pair terms, compensated accumulation, FP64 finalize).
//
// Same derivative set as sph64.cu (SymmetricSolver::loop with VelocityDivergence, VelocityGradient,
// PressureGradient, StressDivergence, StandardAV and NeighborCountTerm, core/sph/solvers/SymmetricSolver.cpp:
// 109-141), evaluated with FP32 arithmetic on inputs prepared so that no large absolute value enters a
// difference: positions are stored relative to the origin of their own grid cell (the pair separation is
// then rel_i - rel_j - offset * cell, exact to FP32 rounding of a cell-sized quantity), velocities as
// unevaluated float pairs hi + lo (the separation of two nearby velocities is exact in the hi part by the
// Sterbenz lemma, so the FP32 difference keeps ~1e-14 relative accuracy of the FP64 inputs). Sums over
// neighbours use Kahan compensation. Material updates, finalize and integrator stay FP64.

#include <algorithm>

#include "physics.cuh"

namespace sphgpu {

namespace {

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const {
        return double(s) - double(c);
    }
};

__device__ __forceinline__ float lutGradF(const float* __restrict__ lut, float qSqr) {
    if (qSqr >= 4.f) {
        return 0.f;
    }
    const float floatIdx = float(LUT_ENTRIES / 4) * qSqr;
    const int idx1 = min(int(floatIdx), LUT_ENTRIES - 1);
    const float ratio = floatIdx - float(idx1);
    const float g0 = __ldg(lut + idx1), g1 = __ldg(lut + idx1 + 1);
    return g0 + (g1 - g0) * ratio;
}

// The pair loop runs in three kernels. neighboursMixedKernel tests the candidates of the cells around a particle
// (one float4 load and a distance test each) and writes the interacting ones, in cell order, to a per-particle
// neighbour list (sorted index | coarse-cell offset << 27, laid out [slot][particle] so that a warp's writes and
// reads of one slot are contiguous); it holds few registers and runs at high occupancy. pairSumMixedKernel then evaluates the pair terms
// from the lists and finalizes the particle. A particle with more than NB_CAP neighbours is left to
// pairSumMixedOverflowKernel, which scans its cells again (rare: a queue of such particles is filled by the first
// kernel). Each particle visits its neighbours in cell order, so the sums are those of a direct loop over the cells.
constexpr int PAIR_THREADS = 128;
constexpr uint32_t NB_INDEX_BITS = 27;
constexpr uint32_t NB_INDEX_MASK = (1u << NB_INDEX_BITS) - 1u;

// the cells of a particle's pair stencil (span cells on each side) in key order (x fastest, then y, then z),
// calling f(t, off) for every candidate t != si, off = the coarse-cell offset (ox + 1) + 3 (oy + 1) + 9 (oz + 1)
// of t's cell against si's
template <typename F>
__device__ __forceinline__ void forEachCandidate(const Grid& g, uint32_t si, F&& f) {
    const GridInfo* gi = g.info;
    const int dxc = gi->dims[0], dyc = gi->dims[1], dzc = gi->dims[2];
    const int span = gi->span, shift = gi->shift;
    const uint32_t key = g.keys_sorted[si];
    const int cx = int(key % uint32_t(dxc)), cy = int((key / uint32_t(dxc)) % uint32_t(dyc)),
              cz = int(key / (uint32_t(dxc) * uint32_t(dyc)));
    for (int z = max(cz - span, 0); z <= min(cz + span, dzc - 1); ++z) {
        const int oz = (z >> shift) - (cz >> shift);
        for (int y = max(cy - span, 0); y <= min(cy + span, dyc - 1); ++y) {
            const int oy = (y >> shift) - (cy >> shift);
            for (int x = max(cx - span, 0); x <= min(cx + span, dxc - 1); ++x) {
                const int ox = (x >> shift) - (cx >> shift);
                const int off = (ox + 1) + 3 * (oy + 1) + 9 * (oz + 1);
                const uint32_t c = (uint32_t(z) * uint32_t(dyc) + uint32_t(y)) * uint32_t(dxc) + uint32_t(x);
                const uint32_t te = g.cell_end[c];
                for (uint32_t t = g.cell_start[c]; t < te; ++t) {
                    if (t != si) {
                        f(t, off);
                    }
                }
            }
        }
    }
}

// the pair test of candidate t in cell offset off against particle i (pi0: cell-relative position and h)
__device__ __forceinline__ bool interactsMixed(const Grid& g, const float4& pi0, float cellf, uint32_t t, int off) {
    const float sx = float(off % 3 - 1) * cellf, sy = float((off / 3) % 3 - 1) * cellf, sz = float(off / 9 - 1) * cellf;
    const float4 pj0 = g.mx0[t];
    const float drx = (pi0.x - pj0.x) - sx, dry = (pi0.y - pj0.y) - sy, drz = (pi0.z - pj0.z) - sz;
    const float d2 = drx * drx + dry * dry + drz * drz;
    const float rad = 2.f * (0.5f * (pi0.w + pj0.w));
    return d2 < rad * rad;
}

// CorrectionTensor::evalNeighs (core/sph/equations/Derivative.cpp:36-74) in mixed precision: the sum of
// m_j / rho_j sym((r_j - r_i) x grad W_ij) in FP32 with compensation, its determinant and inverse in FP64; the
// result is written in FP64 (particle order, the quantity) and FP32 (cell order, for the pair loop).
__global__ void __launch_bounds__(128) correctionMixedKernel(DState s, Grid g, Physics ph,
    const float* __restrict__ lut) {
    const uint32_t n = s.n;
    const uint32_t si = blockIdx.x * blockDim.x + threadIdx.x;
    if (si >= n) {
        return;
    }
    const GridInfo* gi = g.info;
    const float4 pi0 = g.mx0[si], pi3 = g.mx3[si];
    const float cellf = float(gi->ccell);
    Kahan c[6];
    forEachCandidate(g, si, [&](uint32_t t, int off) {
        const float sx = float(off % 3 - 1) * cellf, sy = float((off / 3) % 3 - 1) * cellf,
                    sz = float(off / 9 - 1) * cellf;
        const float4 pj0 = g.mx0[t];
        const float drx = (pi0.x - pj0.x) - sx, dry = (pi0.y - pj0.y) - sy, drz = (pi0.z - pj0.z) - sz;
        const float d2 = drx * drx + dry * dry + drz * drz;
        const float hbar = 0.5f * (pi0.w + pj0.w);
        const float rad = 2.f * hbar;
        if (!(d2 < rad * rad)) {
            return;
        }
        const float4 pj3 = g.mx3[t];
        if (ph.sum_only_undamaged &&
            !(__float_as_uint(pi3.w) == __float_as_uint(pj3.w) && pi3.z != 0.f && pj3.z != 0.f)) {
            return;
        }
        const float4 pj1 = g.mx1[t], pj2 = g.mx2[t];
        const float hInv = 1.f / hbar;
        const float h2 = hInv * hInv;
        const float gl = lutGradF(lut, d2 * h2) * (h2 * h2 * hInv);
        const float gx = drx * gl, gy = dry * gl, gz = drz * gl;
        const float f = pj1.w / pj2.w;
        c[0].add(f * (-drx * gx));
        c[1].add(f * (-dry * gy));
        c[2].add(f * (-drz * gz));
        c[3].add(f * (-0.5f * (drx * gy + dry * gx)));
        c[4].add(f * (-0.5f * (drx * gz + drz * gx)));
        c[5].add(f * (-0.5f * (dry * gz + drz * gy)));
    });
    double cd[6];
    for (int k = 0; k < 6; ++k) {
        cd[k] = c[k].value();
    }
    const bool isNull = cd[0] == 0. && cd[1] == 0. && cd[2] == 0. && cd[3] == 0. && cd[4] == 0. && cd[5] == 0.;
    const double det = cd[0] * cd[1] * cd[2] + 2. * cd[3] * cd[4] * cd[5] -
                       (cd[3] * cd[3] * cd[2] + cd[4] * cd[4] * cd[1] + cd[5] * cd[5] * cd[0]);
    double inv[6] = { 1., 1., 1., 0., 0., 0. };
    if (!isNull && det > 0.01) {
        inv[0] = (cd[1] * cd[2] - cd[5] * cd[5]) / det;
        inv[1] = (cd[2] * cd[0] - cd[4] * cd[4]) / det;
        inv[2] = (cd[0] * cd[1] - cd[3] * cd[3]) / det;
        inv[3] = (cd[4] * cd[5] - cd[2] * cd[3]) / det;
        inv[4] = (cd[5] * cd[3] - cd[1] * cd[4]) / det;
        inv[5] = (cd[3] * cd[4] - cd[0] * cd[5]) / det;
    }
    const uint32_t i = g.perm[si];
    for (int k = 0; k < 6; ++k) {
        s.corr[k * n + i] = inv[k];
        g.mxC[k * n + si] = float(inv[k]);
    }
}

// The candidates are visited row by row: a row's cells have consecutive keys, so the particles of any run of
// them are one contiguous range (first[] of the fine grid), and a candidate's coarse x offset follows from its
// position against the first positions of the coarse cell's fine cells. Rows and cells farther from the particle
// than h_i + h_max (with a 1e-4 margin over the FP32 rounding) are skipped: on the fine grid of h_max cells this
// leaves about a third of the candidates of the 27 coarse cells. Candidates are loaded four at a time ahead of
// their tests. The neighbours come out in key order (x fastest, then y, then z), the order of forEachCandidate.
__global__ void __launch_bounds__(PAIR_THREADS) neighboursMixedKernel(Grid g, uint32_t n) {
    const uint32_t si = blockIdx.x * blockDim.x + threadIdx.x;
    if (si >= n) {
        return;
    }
    const GridInfo* gi = g.info;
    const float4 pi0 = g.mx0[si];
    const float cellf = float(gi->cell), ccellf = float(gi->ccell);
    const int dxc = gi->dims[0], dyc = gi->dims[1], dzc = gi->dims[2];
    const int span = gi->span, shift = gi->shift;
    const uint32_t key = g.keys_sorted[si];
    const int cx = int(key % uint32_t(dxc)), cy = int((key / uint32_t(dxc)) % uint32_t(dyc)),
              cz = int(key / (uint32_t(dxc) * uint32_t(dyc)));
    const int ccx = cx >> shift, ccy = cy >> shift, ccz = cz >> shift;
    // the particle's position in its own cell
    const float fx = pi0.x - float(cx - (ccx << shift)) * cellf;
    const float fy = pi0.y - float(cy - (ccy << shift)) * cellf;
    const float fz = pi0.z - float(cz - (ccz << shift)) * cellf;
    const float reach = (pi0.w + float(gi->hmax)) * 1.0001f;
    const float reach2 = reach * reach;
    // distance from the particle to the slab of the cell at offset d along one axis
    auto gap = [&](int d, float f) {
        return d > 0 ? float(d) * cellf - f : (d < 0 ? f - float(d + 1) * cellf : 0.f);
    };
    uint32_t c = 0;
    for (int dz = -span; dz <= span; ++dz) {
        const int z = cz + dz;
        const float gz = gap(dz, fz);
        if (z < 0 || z >= dzc || gz > reach) {
            continue;
        }
        const int ocz = (z >> shift) - ccz;
        for (int dy = -span; dy <= span; ++dy) {
            const int y = cy + dy;
            const float gy = gap(dy, fy);
            const float gyz = gy * gy + gz * gz;
            if (y < 0 || y >= dyc || gyz > reach2) {
                continue;
            }
            // the cells of the row within reach
            const float xr = sqrtf(reach2 - gyz);
            const int left = xr >= fx ? min(span, int((xr - fx) / cellf) + 1) : 0;
            const int right = min(span, int((xr + fx) / cellf));
            const int xlo = max(cx - left, 0), xhi = min(cx + right, dxc - 1);
            const uint32_t rowBase = (uint32_t(z) * uint32_t(dyc) + uint32_t(y)) * uint32_t(dxc);
            const uint32_t lo = g.cell_first[rowBase + uint32_t(xlo)], hi = g.cell_first[rowBase + uint32_t(xhi) + 1];
            // positions below b1 are in the coarse cell to the left, from b2 in the one to the right
            const int cb0 = min(max(ccx << shift, xlo), xhi + 1), cb1 = min(max((ccx + 1) << shift, xlo), xhi + 1);
            const uint32_t b1 = g.cell_first[rowBase + uint32_t(cb0)], b2 = g.cell_first[rowBase + uint32_t(cb1)];
            const int ocy = (y >> shift) - ccy;
            const float sy = float(ocy) * ccellf, sz = float(ocz) * ccellf;
            const uint32_t offYZ = uint32_t(3 * (ocy + 1) + 9 * (ocz + 1));
            // (the separation and the radius 2 h_bar = h_i + h_j, rounded as in the pair terms)
            auto test = [&](const float4& pj0, uint32_t t) {
                const float sx = t < b1 ? -ccellf : (t < b2 ? 0.f : ccellf);
                const float drx = (pi0.x - pj0.x) - sx, dry = (pi0.y - pj0.y) - sy, drz = (pi0.z - pj0.z) - sz;
                const float d2 = drx * drx + dry * dry + drz * drz;
                const float rad = pi0.w + pj0.w;
                if (d2 < rad * rad && t != si) {
                    if (c < uint32_t(NB_CAP)) {
                        const uint32_t off = offYZ + uint32_t(t >= b1) + uint32_t(t >= b2);
                        g.nb[size_t(c) * n + si] = t | (off << NB_INDEX_BITS);
                    }
                    ++c;
                }
            };
            uint32_t t = lo;
            for (; t + 4 <= hi; t += 4) {
                const float4 q0 = g.mx0[t], q1 = g.mx0[t + 1], q2 = g.mx0[t + 2], q3 = g.mx0[t + 3];
                test(q0, t);
                test(q1, t + 1);
                test(q2, t + 2);
                test(q3, t + 3);
            }
            for (; t < hi; ++t) {
                test(g.mx0[t], t);
            }
        }
    }
    g.nb_count[si] = c;
    if (c > uint32_t(NB_CAP)) {
        g.nb_over[atomicAdd(g.nb_over_count, 1u)] = si;
    }
}

// particle i's side of the pair terms, and its sums
struct MixedSelf {
    float4 p0, p1, p2, p3;
    float S[5];
    float C[6];
    float rhoInv;
};

// compensated: the acceleration, energy and density (velocity divergence) rates; the velocity gradient, which
// enters only the stress and damage rates, is summed plainly
struct MixedSums {
    Kahan ax, ay, az, du, divv;
    float gv[6] = { 0.f, 0.f, 0.f, 0.f, 0.f, 0.f };
    uint32_t cnt = 0;
};

template <bool Solid>
__device__ __forceinline__ void loadSelfMixed(const Grid& g, const Physics& ph, uint32_t n, uint32_t si, MixedSelf& me) {
    me.p0 = g.mx0[si];
    me.p1 = g.mx1[si];
    me.p2 = g.mx2[si];
    me.p3 = g.mx3[si];
    for (int c = 0; c < 5; ++c) {
        me.S[c] = Solid ? g.mxS[c * n + si] : 0.f;
    }
    // strain-rate correction tensor of the velocity gradient (identity without it)
    const bool corr = Solid && ph.correction;
    for (int k = 0; k < 6; ++k) {
        me.C[k] = corr ? g.mxC[k * n + si] : (k < 3 ? 1.f : 0.f);
    }
    me.rhoInv = 1.f / me.p2.w;
}

// the pair terms of neighbour t (cell offset off) of particle i, added into the sums
template <bool Solid>
__device__ __forceinline__ void pairTermMixed(const Grid& g, const Physics& ph, const float* __restrict__ lut,
    uint32_t n, float cellf, const MixedSelf& me, uint32_t t, int off, MixedSums& a) {
    const float4 &pi0 = me.p0, &pi1 = me.p1, &pi2 = me.p2, &pi3 = me.p3;
    const float sx = float(off % 3 - 1) * cellf, sy = float((off / 3) % 3 - 1) * cellf, sz = float(off / 9 - 1) * cellf;
    const float4 pj0 = g.mx0[t];
    const float drx = (pi0.x - pj0.x) - sx, dry = (pi0.y - pj0.y) - sy, drz = (pi0.z - pj0.z) - sz;
    const float d2 = drx * drx + dry * dry + drz * drz;
    const float hbar = 0.5f * (pi0.w + pj0.w);
    const float4 pj1 = g.mx1[t], pj2 = g.mx2[t], pj3 = g.mx3[t];
    // (fast divisions: an error of about 2 ulp, below the rounding of the FP32 pair terms themselves)
    const float hInv = __fdividef(1.f, hbar);
    const float h2 = hInv * hInv;
    const float gl = lutGradF(lut, d2 * h2) * (h2 * h2 * hInv);
    const float gx = drx * gl, gy = dry * gl, gz = drz * gl;
    a.cnt++;
    const float mj = pj1.w, rhoj = pj2.w;
    const float dvx = (pj1.x - pi1.x) + (pj2.x - pi2.x);
    const float dvy = (pj1.y - pi1.y) + (pj2.y - pi2.y);
    const float dvz = (pj1.z - pi1.z) + (pj2.z - pi2.z);
    const float mr = mj * me.rhoInv;
    a.divv.add(mr * (dvx * gx + dvy * gy + dvz * gz));
    float fx = -(pi3.x + pj3.x), fy = fx, fz = fx;
    fx *= gx;
    fy *= gy;
    fz *= gz;
    const float dvdr = -(dvx * drx + dvy * dry + dvz * drz);
    if (dvdr < 0.f) {
        const float rhobar = 0.5f * (pi2.w + rhoj);
        const float csbar = 0.5f * (pi3.y + pj3.y);
        const float mu = __fdividef(hbar * dvdr, d2 + 1.e-2f * (hbar * hbar));
        const float av = __fdividef(-float(ph.av_alpha) * csbar * mu + float(ph.av_beta) * (mu * mu), rhobar);
        fx -= av * gx;
        fy -= av * gy;
        fz -= av * gz;
        a.du.add(mj * (0.5f * av * -(dvx * gx + dvy * gy + dvz * gz)));
    }
    if (Solid) {
        const bool undamaged = !ph.sum_only_undamaged ||
                               (__float_as_uint(pi3.w) == __float_as_uint(pj3.w) && pi3.z != 0.f && pj3.z != 0.f);
        if (undamaged) {
            float hx = gx, hy = gy, hz = gz;
            if (ph.correction) {
                hx = me.C[0] * gx + me.C[3] * gy + me.C[4] * gz;
                hy = me.C[3] * gx + me.C[1] * gy + me.C[5] * gz;
                hz = me.C[4] * gx + me.C[5] * gy + me.C[2] * gz;
            }
            a.gv[0] += mr * (dvx * hx);
            a.gv[1] += mr * (dvy * hy);
            a.gv[2] += mr * (dvz * hz);
            a.gv[3] += mr * (0.5f * (dvx * hy + dvy * hx));
            a.gv[4] += mr * (0.5f * (dvx * hz + dvz * hx));
            a.gv[5] += mr * (0.5f * (dvy * hz + dvz * hy));
            float tt[5];
            for (int k = 0; k < 5; ++k) {
                tt[k] = me.S[k] + g.mxS[k * n + t];
            }
            const float tzz = -tt[0] - tt[1];
            fx += tt[0] * gx + tt[2] * gy + tt[3] * gz;
            fy += tt[2] * gx + tt[1] * gy + tt[4] * gz;
            fz += tt[3] * gx + tt[4] * gy + tzz * gz;
        }
    }
    a.ax.add(mj * fx);
    a.ay.add(mj * fy);
    a.az.add(mj * fz);
}

// FP64 finalize of particle i (sorted position si) with its sums and the gravity acceleration
template <bool Solid>
__device__ __forceinline__ void finishMixed(const DState& s, const Grid& g, const Physics& ph,
    const MaterialD* __restrict__ mats, uint32_t si, const MixedSums& a) {
    const uint32_t n = s.n;
    const uint32_t i = g.perm[si];
    double gax = 0., gay = 0., gaz = 0.;
    if (ph.gravity) {
        const dbl4 ag = s.agrav[i];
        gax = ag.x;
        gay = ag.y;
        gaz = ag.z;
    }
    const dbl4 ri = g.rs[si];
    const double rhoi = g.rhos[si], pri = g.ps[si];
    double Si[5] = { 0, 0, 0, 0, 0 };
    double gvd[6];
    for (int c = 0; c < 6; ++c) {
        gvd[c] = double(a.gv[c]);
    }
    if (Solid) {
        for (int c = 0; c < 5; ++c) {
            Si[c] = g.Ss[c * n + si];
        }
    }
    finalizeParticle<Solid, true>(s, ph, mats, i, ri, rhoi, pri, Si, gax + a.ax.value(), gay + a.ay.value(),
        gaz + a.az.value(), a.du.value(), a.divv.value(), gvd, a.cnt);
}

template <bool Solid>
__global__ void __launch_bounds__(PAIR_THREADS, 8) pairSumMixedKernel(DState s, Grid g, Physics ph,
    const MaterialD* __restrict__ mats, const float* __restrict__ lut) {
    const uint32_t n = s.n;
    const uint32_t si = blockIdx.x * blockDim.x + threadIdx.x;
    if (si >= n) {
        return;
    }
    const uint32_t total = g.nb_count[si];
    if (total > uint32_t(NB_CAP)) {
        return; // pairSumMixedOverflowKernel
    }
    const float cellf = float(g.info->ccell);
    MixedSelf me;
    loadSelfMixed<Solid>(g, ph, n, si, me);
    MixedSums a;
    for (uint32_t q = 0; q < total; ++q) {
        const uint32_t e = g.nb[size_t(q) * n + si];
        pairTermMixed<Solid>(g, ph, lut, n, cellf, me, e & NB_INDEX_MASK, int(e >> NB_INDEX_BITS), a);
    }
    finishMixed<Solid>(s, g, ph, mats, si, a);
}

template <bool Solid>
__global__ void __launch_bounds__(PAIR_THREADS) pairSumMixedOverflowKernel(DState s, Grid g, Physics ph,
    const MaterialD* __restrict__ mats, const float* __restrict__ lut) {
    const uint32_t n = s.n;
    const uint32_t count = min(*g.nb_over_count, n);
    const float cellf = float(g.info->ccell);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const uint32_t si = g.nb_over[k];
        MixedSelf me;
        loadSelfMixed<Solid>(g, ph, n, si, me);
        MixedSums a;
        forEachCandidate(g, si, [&](uint32_t t, int off) {
            if (interactsMixed(g, me.p0, cellf, t, off)) {
                pairTermMixed<Solid>(g, ph, lut, n, cellf, me, t, off, a);
            }
        });
        finishMixed<Solid>(s, g, ph, mats, si, a);
    }
}

} // namespace

void launchCorrectionMixed(const DState& s, const Grid& g, const Physics& ph, const float* lut, cudaStream_t st) {
    if (s.n) {
        correctionMixedKernel<<<ceilDiv(s.n, 128), 128, 0, st>>>(s, g, ph, lut);
    }
}

void launchPairSumMixed(const DState& s, const Grid& g, const Physics& ph, const MaterialD* mats, const float* lut,
    cudaStream_t st) {
    if (!s.n) {
        return;
    }
    cudaMemsetAsync(g.nb_over_count, 0, sizeof(uint32_t), st);
    neighboursMixedKernel<<<ceilDiv(s.n, PAIR_THREADS), PAIR_THREADS, 0, st>>>(g, s.n);
    // the overflow pass runs on a small fixed grid over the particles queued by the first kernel (usually none)
    const int overBlocks = std::min(ceilDiv(s.n, PAIR_THREADS), 152);
    if (ph.solid) {
        pairSumMixedKernel<true><<<ceilDiv(s.n, PAIR_THREADS), PAIR_THREADS, 0, st>>>(s, g, ph, mats, lut);
        pairSumMixedOverflowKernel<true><<<overBlocks, PAIR_THREADS, 0, st>>>(s, g, ph, mats, lut);
    } else {
        pairSumMixedKernel<false><<<ceilDiv(s.n, PAIR_THREADS), PAIR_THREADS, 0, st>>>(s, g, ph, mats, lut);
        pairSumMixedOverflowKernel<false><<<overBlocks, PAIR_THREADS, 0, st>>>(s, g, ph, mats, lut);
    }
}

} // namespace sphgpu
