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
    const float cellf = float(gi->cell);
    Kahan c[6];
    const int dxc = gi->dims[0], dyc = gi->dims[1], dzc = gi->dims[2];
    const uint32_t key = g.keys_sorted[si];
    const int cx = int(key % uint32_t(dxc)), cy = int((key / uint32_t(dxc)) % uint32_t(dyc)),
              cz = int(key / (uint32_t(dxc) * uint32_t(dyc)));
    for (int off = 0; off < 27; ++off) {
        const int ox = off % 3 - 1, oy = (off / 3) % 3 - 1, oz = off / 9 - 1;
        const int x = cx + ox, y = cy + oy, z = cz + oz;
        if (x < 0 || x >= dxc || y < 0 || y >= dyc || z < 0 || z >= dzc) {
            continue;
        }
        const uint32_t cell = (uint32_t(z) * uint32_t(dyc) + uint32_t(y)) * uint32_t(dxc) + uint32_t(x);
        const uint32_t te = g.cell_end[cell];
        const float sx = float(ox) * cellf, sy = float(oy) * cellf, sz = float(oz) * cellf;
        for (uint32_t t = g.cell_start[cell]; t < te; ++t) {
            if (t == si) {
                continue;
            }
            const float4 pj0 = g.mx0[t];
            const float drx = (pi0.x - pj0.x) - sx, dry = (pi0.y - pj0.y) - sy, drz = (pi0.z - pj0.z) - sz;
            const float d2 = drx * drx + dry * dry + drz * drz;
            const float hbar = 0.5f * (pi0.w + pj0.w);
            const float rad = 2.f * hbar;
            if (!(d2 < rad * rad)) {
                continue;
            }
            const float4 pj3 = g.mx3[t];
            if (ph.sum_only_undamaged &&
                !(__float_as_uint(pi3.w) == __float_as_uint(pj3.w) && pi3.z != 0.f && pj3.z != 0.f)) {
                continue;
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
        }
    }
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

// Candidates of the 27 cells are first tested (cheap: one float4 load and a distance test per candidate,
// every lane busy) and the interacting ones queued per lane in shared memory; the pair terms are then
// evaluated from the queues, when any lane's queue is full and at the end. The pair terms thus run with
// nearly all lanes active instead of only the ~15 % of lanes whose candidate interacts. Each lane still
// visits its neighbours in cell order, so the sums are the same as a direct loop's.
constexpr int PAIR_THREADS = 128;
constexpr int PAIR_QUEUE = 32;

template <bool Solid>
__global__ void __launch_bounds__(PAIR_THREADS) pairSumMixedKernel(DState s, Grid g, Physics ph,
    const MaterialD* __restrict__ mats, const float* __restrict__ lut) {
    __shared__ uint32_t queueT[PAIR_QUEUE][PAIR_THREADS];
    __shared__ uint8_t queueOff[PAIR_QUEUE][PAIR_THREADS];
    const uint32_t n = s.n;
    const uint32_t si = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = si < n;
    const uint32_t sv = valid ? si : n - 1;
    const GridInfo* gi = g.info;
    const float4 pi0 = g.mx0[sv], pi1 = g.mx1[sv], pi2 = g.mx2[sv], pi3 = g.mx3[sv];
    const float cellf = float(gi->cell);
    float Sif[5] = { 0, 0, 0, 0, 0 };
    if (Solid) {
        for (int c = 0; c < 5; ++c) {
            Sif[c] = g.mxS[c * n + sv];
        }
    }
    const float rhoiInv = 1.f / pi2.w;
    const float alpha = float(ph.av_alpha), beta = float(ph.av_beta);
    Kahan ax, ay, az, du, divv;
    Kahan gv[6];
    // strain-rate correction tensor of the velocity gradient (identity without it)
    float Ci[6] = { 1.f, 1.f, 1.f, 0.f, 0.f, 0.f };
    if (Solid && ph.correction) {
        for (int k = 0; k < 6; ++k) {
            Ci[k] = g.mxC[k * n + sv];
        }
    }
    uint32_t cnt = 0;
    const int dxc = gi->dims[0], dyc = gi->dims[1], dzc = gi->dims[2];
    const uint32_t key = g.keys_sorted[sv];
    const int cx = int(key % uint32_t(dxc)), cy = int((key / uint32_t(dxc)) % uint32_t(dyc)),
              cz = int(key / (uint32_t(dxc) * uint32_t(dyc)));

    // pair terms of the queued neighbours (the loop is warp-uniform; each lane stops at its own count)
    auto flush = [&](uint32_t nq) {
        const uint32_t nmax = __reduce_max_sync(0xffffffffu, nq);
        for (uint32_t q = 0; q < nmax; ++q) {
            if (q >= nq) {
                continue;
            }
            const uint32_t t = queueT[q][threadIdx.x];
            const int off = queueOff[q][threadIdx.x];
            const float sx = float(off % 3 - 1) * cellf, sy = float((off / 3) % 3 - 1) * cellf,
                        sz = float(off / 9 - 1) * cellf;
            const float4 pj0 = g.mx0[t];
            const float drx = (pi0.x - pj0.x) - sx, dry = (pi0.y - pj0.y) - sy, drz = (pi0.z - pj0.z) - sz;
            const float d2 = drx * drx + dry * dry + drz * drz;
            const float hbar = 0.5f * (pi0.w + pj0.w);
            const float4 pj1 = g.mx1[t], pj2 = g.mx2[t], pj3 = g.mx3[t];
            const float hInv = 1.f / hbar;
            const float h2 = hInv * hInv;
            const float gl = lutGradF(lut, d2 * h2) * (h2 * h2 * hInv);
            const float gx = drx * gl, gy = dry * gl, gz = drz * gl;
            cnt++;
            const float mj = pj1.w, rhoj = pj2.w;
            const float dvx = (pj1.x - pi1.x) + (pj2.x - pi2.x);
            const float dvy = (pj1.y - pi1.y) + (pj2.y - pi2.y);
            const float dvz = (pj1.z - pi1.z) + (pj2.z - pi2.z);
            const float mr = mj * rhoiInv;
            divv.add(mr * (dvx * gx + dvy * gy + dvz * gz));
            float fx = -(pi3.x + pj3.x), fy = fx, fz = fx;
            fx *= gx;
            fy *= gy;
            fz *= gz;
            const float dvdr = -(dvx * drx + dvy * dry + dvz * drz);
            if (dvdr < 0.f) {
                const float rhobar = 0.5f * (pi2.w + rhoj);
                const float csbar = 0.5f * (pi3.y + pj3.y);
                const float mu = hbar * dvdr / (d2 + 1.e-2f * (hbar * hbar));
                const float av = (-alpha * csbar * mu + beta * (mu * mu)) / rhobar;
                fx -= av * gx;
                fy -= av * gy;
                fz -= av * gz;
                du.add(mj * (0.5f * av * -(dvx * gx + dvy * gy + dvz * gz)));
            }
            if (Solid) {
                const bool undamaged = !ph.sum_only_undamaged ||
                                       (__float_as_uint(pi3.w) == __float_as_uint(pj3.w) && pi3.z != 0.f &&
                                           pj3.z != 0.f);
                if (undamaged) {
                    float hx = gx, hy = gy, hz = gz;
                    if (ph.correction) {
                        hx = Ci[0] * gx + Ci[3] * gy + Ci[4] * gz;
                        hy = Ci[3] * gx + Ci[1] * gy + Ci[5] * gz;
                        hz = Ci[4] * gx + Ci[5] * gy + Ci[2] * gz;
                    }
                    gv[0].add(mr * (dvx * hx));
                    gv[1].add(mr * (dvy * hy));
                    gv[2].add(mr * (dvz * hz));
                    gv[3].add(mr * (0.5f * (dvx * hy + dvy * hx)));
                    gv[4].add(mr * (0.5f * (dvx * hz + dvz * hx)));
                    gv[5].add(mr * (0.5f * (dvy * hz + dvz * hy)));
                    float tt[5];
                    for (int k = 0; k < 5; ++k) {
                        tt[k] = Sif[k] + g.mxS[k * n + t];
                    }
                    const float tzz = -tt[0] - tt[1];
                    fx += tt[0] * gx + tt[2] * gy + tt[3] * gz;
                    fy += tt[2] * gx + tt[1] * gy + tt[4] * gz;
                    fz += tt[3] * gx + tt[4] * gy + tzz * gz;
                }
            }
            ax.add(mj * fx);
            ay.add(mj * fy);
            az.add(mj * fz);
        }
    };

    uint32_t nq = 0;
    // the particle range of neighbour cell off (empty outside the grid); the next cell's range is loaded while the
    // current cell's candidates are tested
    auto cellRange = [&](int off, uint32_t& tb, uint32_t& te) {
        const int x = cx + off % 3 - 1, y = cy + (off / 3) % 3 - 1, z = cz + off / 9 - 1;
        tb = 0;
        te = 0;
        if (valid && x >= 0 && x < dxc && y >= 0 && y < dyc && z >= 0 && z < dzc) {
            const uint32_t c = (uint32_t(z) * uint32_t(dyc) + uint32_t(y)) * uint32_t(dxc) + uint32_t(x);
            tb = g.cell_start[c];
            te = g.cell_end[c];
        }
    };
    uint32_t nextB, nextE;
    cellRange(0, nextB, nextE);
    for (int off = 0; off < 27; ++off) {
        const int ox = off % 3 - 1, oy = (off / 3) % 3 - 1, oz = off / 9 - 1;
        const uint32_t tb = nextB, te = nextE;
        if (off + 1 < 27) {
            cellRange(off + 1, nextB, nextE);
        }
        const uint32_t len = te - tb;
        const uint32_t lmax = __reduce_max_sync(0xffffffffu, len);
        const float sx = float(ox) * cellf, sy = float(oy) * cellf, sz = float(oz) * cellf;
        for (uint32_t k = 0; k < lmax; ++k) {
            const uint32_t t = tb + k;
            bool pass = false;
            if (k < len && t != si) {
                const float4 pj0 = g.mx0[t];
                const float drx = (pi0.x - pj0.x) - sx, dry = (pi0.y - pj0.y) - sy, drz = (pi0.z - pj0.z) - sz;
                const float d2 = drx * drx + dry * dry + drz * drz;
                const float rad = 2.f * (0.5f * (pi0.w + pj0.w));
                pass = d2 < rad * rad;
            }
            if (pass) {
                queueT[nq][threadIdx.x] = t;
                queueOff[nq][threadIdx.x] = uint8_t(off);
                ++nq;
            }
            if (__any_sync(0xffffffffu, nq == PAIR_QUEUE)) {
                flush(nq);
                nq = 0;
            }
        }
    }
    flush(nq);
    if (!valid) {
        return;
    }
    const uint32_t i = g.perm[si];
    double gax = 0., gay = 0., gaz = 0.;
    if (ph.gravity) {
        const dbl4 a = s.agrav[i];
        gax = a.x;
        gay = a.y;
        gaz = a.z;
    }
    const dbl4 ri = g.rs[si];
    const double rhoi = g.rhos[si], pri = g.ps[si];
    double Si[5] = { 0, 0, 0, 0, 0 };
    double gvd[6];
    for (int c = 0; c < 6; ++c) {
        gvd[c] = gv[c].value();
    }
    if (Solid) {
        for (int c = 0; c < 5; ++c) {
            Si[c] = g.Ss[c * n + si];
        }
    }
    finalizeParticle<Solid>(s, ph, mats, i, ri, rhoi, pri, Si, gax + ax.value(), gay + ay.value(), gaz + az.value(),
        du.value(), divv.value(), gvd, cnt);
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
    if (ph.solid) {
        pairSumMixedKernel<true><<<ceilDiv(s.n, PAIR_THREADS), PAIR_THREADS, 0, st>>>(s, g, ph, mats, lut);
    } else {
        pairSumMixedKernel<false><<<ceilDiv(s.n, PAIR_THREADS), PAIR_THREADS, 0, st>>>(s, g, ph, mats, lut);
    }
}

} // namespace sphgpu
