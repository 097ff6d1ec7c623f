// sph64.cu — FP64 SPH derivative loop, material models and integrators (compiled with -fmad=false).
//
// Replaces, for one GPU:
//   SymmetricSolver::loop + DerivativeHolder::evalSymmetric (core/sph/solvers/SymmetricSolver.cpp:109-141)
//     with its terms: VelocityDivergence / VelocityGradient (core/sph/equations/DerivativeHelpers.h:292-361),
//     PressureGradient, StressDivergence (core/sph/equations/EquationTerm.cpp:12-140), StandardAV
//     (core/sph/equations/av/Standard.h:63-83), NeighborCountTerm (core/sph/equations/HelperTerms.h:16-63)
//   EquationHolder::finalize (EquationTerm.cpp:90-99, 177-203, 289-316, 366-391, 427-434)
//   EosMaterial / SolidMaterial initialize + finalize (core/sph/Materials.cpp:47-81): TillotsonEos,
//     IdealGasEos (core/physics/Eos.cpp:42-45, 198-238), VonMisesRheology (core/physics/Rheology.cpp:36-83),
//     ScalarGradyKippModel::integrate (core/physics/Damage.cpp:128-170)
//   PredictorCorrector / LeapFrog (core/timestepping/TimeStepping.cpp:82-391), CourantCriterion
//     (core/timestepping/TimeStepCriterion.cpp:315-356)
//
// The pair loop is a gather: one thread per particle (in cell-sorted order) sums the contributions of all
// of its neighbours. Each per-pair term is the same IEEE expression the reference evaluates for that pair
// (this file is compiled without FMA contraction), so results differ from the reference's sequential
// scatter only by the order of the sums. No atomics: the results are bit-reproducible run to run.

#include "physics.cuh"

namespace sphgpu {

namespace {

// ------------------------------------------------------------------------------------------------------
// kernels
// ------------------------------------------------------------------------------------------------------

__global__ void materialsInitKernel(DState s, Physics ph, const MaterialD* __restrict__ mats) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < s.n) {
        if (ph.precision == SPHGPU_PRECISION_MIXED) {
            materialInit<true>(s, ph, mats, i);
        } else {
            materialInit<false>(s, ph, mats, i);
        }
    }
}

// LutKernel<3>::gradImpl (core/sph/kernel/Kernel.h:129-144)
__device__ __forceinline__ double lutGrad(const double* __restrict__ lut, double qSqr) {
    if (qSqr >= 4.) {
        return 0.;
    }
    const double floatIdx = (double(LUT_ENTRIES) * (1. / (2. * 2.))) * qSqr;
    const int idx1 = int(floatIdx);
    const double ratio = floatIdx - double(idx1);
    return __ldg(lut + idx1) * (1. - ratio) + __ldg(lut + idx1 + 1) * ratio;
}

__device__ __forceinline__ bool interacts64(const dbl4& a, const dbl4& b) {
    const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    const double d2 = dx * dx + dy * dy + dz * dz;
    const double rad = 2. * (0.5 * (a.w + b.w));
    return d2 < rad * rad;
}

// Inverse of the correction-tensor sum, or the identity when the sum is null or nearly singular
// (CorrectionTensor::evalNeighs, core/sph/equations/Derivative.cpp:59-72; SymmetricTensor::determinant /
// inverse, core/objects/geometry/SymmetricTensor.h:193-231). c: xx, yy, zz, xy, xz, yz.
__device__ __forceinline__ void invertCorrection(double c[6]) {
    const bool isNull = c[0] == 0. && c[1] == 0. && c[2] == 0. && c[3] == 0. && c[4] == 0. && c[5] == 0.;
    const double det = c[0] * c[1] * c[2] + 2. * c[3] * c[4] * c[5] - (c[3] * c[3] * c[2] + c[4] * c[4] * c[1] +
                                                                         c[5] * c[5] * c[0]);
    if (isNull || !(det > 0.01)) {
        c[0] = c[1] = c[2] = 1.;
        c[3] = c[4] = c[5] = 0.;
        return;
    }
    const double d0 = c[1] * c[2] - c[5] * c[5];
    const double d1 = c[2] * c[0] - c[4] * c[4];
    const double d2 = c[0] * c[1] - c[3] * c[3];
    const double o0 = c[4] * c[5] - c[2] * c[3];
    const double o1 = c[5] * c[3] - c[1] * c[4];
    const double o2 = c[3] * c[4] - c[0] * c[5];
    c[0] = d0 / det;
    c[1] = d1 / det;
    c[2] = d2 / det;
    c[3] = o0 / det;
    c[4] = o1 / det;
    c[5] = o2 / det;
}

// CorrectionTensor::evalNeighs (core/sph/equations/Derivative.cpp:36-74): C_i = (sum_j m_j / rho_j
// sym((r_j - r_i) x grad W_ij))^-1 over the pairs the velocity gradient sums (the SUM_ONLY_UNDAMAGED filter)
__global__ void __launch_bounds__(128) correction64Kernel(DState s, Grid g, Physics ph,
    const double* __restrict__ lut) {
    const uint32_t n = s.n;
    const uint32_t si = blockIdx.x * blockDim.x + threadIdx.x;
    if (si >= n) {
        return;
    }
    const GridInfo* gi = g.info;
    const uint32_t i = g.perm[si];
    const dbl4 ri = g.rs[si];
    const double redi = g.reduces[si];
    const uint32_t flagi = g.flags[si];
    double c[6] = { 0, 0, 0, 0, 0, 0 };
    const int dxc = gi->dims[0], dyc = gi->dims[1], dzc = gi->dims[2];
    const uint32_t key = g.keys_sorted[si];
    const int cx = int(key % uint32_t(dxc)), cy = int((key / uint32_t(dxc)) % uint32_t(dyc)),
              cz = int(key / (uint32_t(dxc) * uint32_t(dyc)));
    for (int z = max(cz - 1, 0); z <= min(cz + 1, dzc - 1); ++z) {
        for (int y = max(cy - 1, 0); y <= min(cy + 1, dyc - 1); ++y) {
            const uint32_t rowBase = (uint32_t(z) * uint32_t(dyc) + uint32_t(y)) * uint32_t(dxc);
            const uint32_t c0 = rowBase + uint32_t(max(cx - 1, 0));
            const uint32_t c1 = rowBase + uint32_t(min(cx + 1, dxc - 1));
            uint32_t tb = 0xffffffffu, tEnd = 0;
            for (uint32_t cc = c0; cc <= c1; ++cc) {
                const uint32_t cs0 = g.cell_start[cc], ce0 = g.cell_end[cc];
                if (ce0 > cs0) {
                    tb = min(tb, cs0);
                    tEnd = max(tEnd, ce0);
                }
            }
            for (uint32_t t = tb; t < tEnd; ++t) {
                if (t == si) {
                    continue;
                }
                const dbl4 rj = g.rs[t];
                if (!interacts64(ri, rj)) {
                    continue;
                }
                if (ph.sum_only_undamaged && (flagi != g.flags[t] || redi == 0. || g.reduces[t] == 0.)) {
                    continue;
                }
                const double hbar = 0.5 * (ri.w + rj.w);
                const double drx = ri.x - rj.x, dry = ri.y - rj.y, drz = ri.z - rj.z;
                const double hInv = 1. / hbar;
                const double h2 = hInv * hInv;
                const double h5 = (h2 * h2) * hInv;
                const double gl = lutGrad(lut, (drx * drx + dry * dry + drz * drz) * (hInv * hInv));
                const double gx = (drx * h5) * gl, gy = (dry * h5) * gl, gz = (drz * h5) * gl;
                const double ex = rj.x - ri.x, ey = rj.y - ri.y, ez = rj.z - ri.z;
                const double f = g.ms[t] / g.rhos[t];
                c[0] += f * (ex * gx);
                c[1] += f * (ey * gy);
                c[2] += f * (ez * gz);
                c[3] += f * (0.5 * (ex * gy + ey * gx));
                c[4] += f * (0.5 * (ex * gz + ez * gx));
                c[5] += f * (0.5 * (ey * gz + ez * gy));
            }
        }
    }
    invertCorrection(c);
    for (int k = 0; k < 6; ++k) {
        s.corr[k * n + i] = c[k];
    }
}

// Gather form: a thread per particle sums its terms over the candidates of the 27 cells around it, then
// finalizes the particle. With few particles (fewer than about a thread per SM thread slot at S = 1), 2^shift = S
// consecutive lanes of a warp share a particle: lane s of the group takes the candidates s, s + S, ... of every
// row range, and the groups' partial sums are added by a fixed pairwise tree of shuffles (deterministic; the
// order of the sums differs from the single-thread order in the last bits only) before lane 0 finalizes.
template <bool Solid>
__global__ void __launch_bounds__(128) pairSum64Kernel(DState s, Grid g, Physics ph,
    const MaterialD* __restrict__ mats, const double* __restrict__ lut, uint32_t shift) {
    const uint32_t n = s.n;
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t slices = 1u << shift;
    const uint32_t si = gt >> shift;
    const uint32_t sl = gt & (slices - 1u);
    // (the lanes of a group share si: a group returns as a whole)
    if (si >= n) {
        return;
    }
    const GridInfo* gi = g.info;
    const uint32_t i = g.perm[si];
    const dbl4 ri = g.rs[si];
    const dbl4 vi = g.vs[si];
    const double rhoi = g.rhos[si], pri = g.ps[si], csi = g.css[si];
    double Si[5] = { 0, 0, 0, 0, 0 };
    double redi = 0.;
    uint32_t flagi = 0;
    if (Solid) {
        for (int c = 0; c < 5; ++c) {
            Si[c] = g.Ss[c * n + si];
        }
        redi = g.reduces[si];
        flagi = g.flags[si];
    }
    double ax = 0., ay = 0., az = 0.;
    if (ph.gravity && sl == 0) {
        const dbl4 a = s.agrav[i];
        ax = a.x;
        ay = a.y;
        az = a.z;
    }
    double du = 0., divv = 0.;
    double gv[6] = { 0, 0, 0, 0, 0, 0 };
    uint32_t cnt = 0;
    const double alpha = ph.av_alpha, beta = ph.av_beta;
    // strain-rate correction tensor of the velocity gradient (identity without it)
    double Ci[6] = { 1., 1., 1., 0., 0., 0. };
    if (Solid && ph.correction) {
        for (int k = 0; k < 6; ++k) {
            Ci[k] = s.corr[k * n + i];
        }
    }
    const int dxc = gi->dims[0], dyc = gi->dims[1], dzc = gi->dims[2];
    const uint32_t key = g.keys_sorted[si];
    const int cx = int(key % uint32_t(dxc)), cy = int((key / uint32_t(dxc)) % uint32_t(dyc)),
              cz = int(key / (uint32_t(dxc) * uint32_t(dyc)));
    const double rhoi2 = rhoi * rhoi;
    for (int z = max(cz - 1, 0); z <= min(cz + 1, dzc - 1); ++z) {
        for (int y = max(cy - 1, 0); y <= min(cy + 1, dyc - 1); ++y) {
            const uint32_t rowBase = (uint32_t(z) * uint32_t(dyc) + uint32_t(y)) * uint32_t(dxc);
            const uint32_t c0 = rowBase + uint32_t(max(cx - 1, 0));
            const uint32_t c1 = rowBase + uint32_t(min(cx + 1, dxc - 1));
            // the cells of one x-row have consecutive keys, so their particles form one contiguous range
            // of the cell-sorted order
            uint32_t tb = 0xffffffffu, tEnd = 0;
            for (uint32_t c = c0; c <= c1; ++c) {
                const uint32_t cs0 = g.cell_start[c], ce0 = g.cell_end[c];
                if (ce0 > cs0) {
                    tb = min(tb, cs0);
                    tEnd = max(tEnd, ce0);
                }
            }
            for (uint32_t t = tb + sl; t < tEnd; t += slices) {
                if (t == si) {
                    continue;
                }
                const dbl4 rj = g.rs[t];
                if (!interacts64(ri, rj)) {
                    continue;
                }
                const dbl4 vj = g.vs[t];
                const double mj = g.ms[t], rhoj = g.rhos[t];
                // symmetrized kernel gradient at hbar (core/sph/kernel/Kernel.h:32-36, 640-644)
                const double hbar = 0.5 * (ri.w + rj.w);
                const double drx = ri.x - rj.x, dry = ri.y - rj.y, drz = ri.z - rj.z;
                const double hInv = 1. / hbar;
                const double h2 = hInv * hInv;
                const double h5 = (h2 * h2) * hInv;
                const double gl = lutGrad(lut, (drx * drx + dry * dry + drz * drz) * (hInv * hInv));
                const double gx = (drx * h5) * gl, gy = (dry * h5) * gl, gz = (drz * h5) * gl;
                cnt++;
                // velocity divergence (CenterDensityDiscr)
                const double dvx = vj.x - vi.x, dvy = vj.y - vi.y, dvz = vj.z - vi.z;
                divv += mj / rhoi * (dvx * gx + dvy * gy + dvz * gz);
                // pressure gradient (StandardForceDiscr)
                {
                    const double pr = pri / rhoi2 + g.ps[t] / (rhoj * rhoj);
                    ax += mj * -(pr * gx);
                    ay += mj * -(pr * gy);
                    az += mj * -(pr * gz);
                }
                // standard artificial viscosity
                {
                    const double ux = vi.x - vj.x, uy = vi.y - vj.y, uz = vi.z - vj.z;
                    const double dvdr = ux * drx + uy * dry + uz * drz;
                    if (!(dvdr >= 0.)) {
                        const double rhobar = 0.5 * (rhoi + rhoj);
                        const double csbar = 0.5 * (csi + g.css[t]);
                        const double mu =
                            hbar * dvdr / ((drx * drx + dry * dry + drz * drz) + 1.e-2 * (hbar * hbar));
                        const double av = 1. / rhobar * (-alpha * csbar * mu + beta * (mu * mu));
                        ax += mj * -(av * gx);
                        ay += mj * -(av * gy);
                        az += mj * -(av * gz);
                        du += mj * (0.5 * av * (ux * gx + uy * gy + uz * gz));
                    }
                }
                if (Solid) {
                    const bool undamaged =
                        !ph.sum_only_undamaged || (flagi == g.flags[t] && redi != 0. && g.reduces[t] != 0.);
                    if (undamaged) {
                        const double f = mj / rhoi;
                        // C_i grad W (SymmetricTensor::operator*(Vector), SymmetricTensor.h:102-107)
                        double hx = gx, hy = gy, hz = gz;
                        if (ph.correction) {
                            hx = Ci[0] * gx + Ci[3] * gy + Ci[4] * gz;
                            hy = Ci[3] * gx + Ci[1] * gy + Ci[5] * gz;
                            hz = Ci[4] * gx + Ci[5] * gy + Ci[2] * gz;
                        }
                        gv[0] += f * (dvx * hx);
                        gv[1] += f * (dvy * hy);
                        gv[2] += f * (dvz * hz);
                        gv[3] += f * (0.5 * (dvx * hy + dvy * hx));
                        gv[4] += f * (0.5 * (dvx * hz + dvz * hx));
                        gv[5] += f * (0.5 * (dvy * hz + dvz * hy));
                        const double rhoj2 = rhoj * rhoj;
                        double tt[5];
                        for (int c = 0; c < 5; ++c) {
                            tt[c] = Si[c] / rhoi2 + g.Ss[c * n + t] / rhoj2;
                        }
                        const double tzz = -tt[0] - tt[1];
                        ax += mj * (tt[0] * gx + tt[2] * gy + tt[3] * gz);
                        ay += mj * (tt[2] * gx + tt[1] * gy + tt[4] * gz);
                        az += mj * (tt[3] * gx + tt[4] * gy + tzz * gz);
                    }
                }
            }
        }
    }
    if (slices > 1) {
        const uint32_t lane = threadIdx.x & 31u;
        const unsigned mask = ((slices == 32u ? 0u : (1u << slices)) - 1u) << (lane & ~(slices - 1u));
        for (uint32_t off = slices >> 1; off > 0; off >>= 1) {
            ax += __shfl_down_sync(mask, ax, off, int(slices));
            ay += __shfl_down_sync(mask, ay, off, int(slices));
            az += __shfl_down_sync(mask, az, off, int(slices));
            du += __shfl_down_sync(mask, du, off, int(slices));
            divv += __shfl_down_sync(mask, divv, off, int(slices));
            cnt += __shfl_down_sync(mask, cnt, off, int(slices));
            if (Solid) {
                for (int c = 0; c < 6; ++c) {
                    gv[c] += __shfl_down_sync(mask, gv[c], off, int(slices));
                }
            }
        }
        if (sl != 0) {
            return;
        }
    }
    finalizeParticle<Solid>(s, ph, mats, i, ri, rhoi, pri, Si, ax, ay, az, du, divv, gv, cnt);
}

// The mixed-precision path's integrator keeps its state and arithmetic in FP64 but forms the updates with fused
// multiply-adds (this unit is otherwise compiled without contraction, so that the FP64 path's updates are the
// reference's products and sums): fewer FP64 operations on a part whose FP64 rate is 1/64 of its FP32 rate,
// results that differ from the FP64 path's in the last bits.
__device__ __forceinline__ double updFma(double x, double dx, double k) {
    return __fma_rn(dx, k, x);
}

// PredictorCorrector::makePredictions (TimeStepping.cpp:286-300) + materials initialize at the prediction
__global__ void predictKernel(DState s, Physics ph, const MaterialD* __restrict__ mats, const double* __restrict__ dtp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = s.n;
    if (i >= n) {
        return;
    }
    const bool fast = ph.precision == SPHGPU_PRECISION_MIXED;
    const double dt = *dtp;
    const double dt2 = 0.5 * (dt * dt);
    dbl4 r = s.r[i], v = s.v[i];
    const dbl4 a = s.dv[i];
    if (fast) {
        r.x = updFma(updFma(r.x, v.x, dt), a.x, dt2);
        r.y = updFma(updFma(r.y, v.y, dt), a.y, dt2);
        r.z = updFma(updFma(r.z, v.z, dt), a.z, dt2);
        r.w = updFma(updFma(r.w, v.w, dt), a.w, dt2);
        v.x = updFma(v.x, a.x, dt);
        v.y = updFma(v.y, a.y, dt);
        v.z = updFma(v.z, a.z, dt);
        v.w = updFma(v.w, a.w, dt);
    } else {
        r.x += v.x * dt + a.x * dt2;
        r.y += v.y * dt + a.y * dt2;
        r.z += v.z * dt + a.z * dt2;
        r.w += v.w * dt + a.w * dt2;
        v.x += a.x * dt;
        v.y += a.y * dt;
        v.z += a.z * dt;
        v.w += a.w * dt;
    }
    s.r[i] = r;
    s.v[i] = v;
    const MaterialD& mt = mats[ph.nmat > 1 ? s.mat[i] : 0];
    double rho = s.rho[i], drho = s.drho[i];
    rho = fast ? updFma(rho, drho, dt) : rho + drho * dt;
    clampDeriv(rho, drho, mt.rho_lo, mt.rho_hi);
    s.rho[i] = rho;
    s.drho[i] = drho;
    double u = s.u[i], du = s.du[i];
    u = fast ? updFma(u, du, dt) : u + du * dt;
    clampDeriv(u, du, mt.u_lo, mt.u_hi);
    s.u[i] = u;
    s.du[i] = du;
    if (ph.solid) {
        for (int c = 0; c < 5; ++c) {
            const double S = s.S[c * n + i], dS = s.dS[c * n + i];
            s.S[c * n + i] = fast ? updFma(S, dS, dt) : S + dS * dt;
        }
        if (ph.damage) {
            double D = s.D[i], dD = s.dD[i];
            D = fast ? updFma(D, dD, dt) : D + dD * dt;
            clampDeriv(D, dD, mt.d_lo, mt.d_hi);
            s.D[i] = D;
            s.dD[i] = dD;
        }
    }
    clampSmoothingLength(s, ph, i);
}

__device__ __forceinline__ void blockMinToGlobal(double local, double* out) {
    __shared__ double red[32];
    for (int off = 16; off > 0; off >>= 1) {
        local = fmin(local, __shfl_xor_sync(0xffffffffu, local, off));
    }
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = local;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : DBL_MAX;
        for (int off = 16; off > 0; off >>= 1) {
            v = fmin(v, __shfl_xor_sync(0xffffffffu, v, off));
        }
        if (threadIdx.x == 0 && v < DBL_MAX) {
            atomicMinPos(out, v);
        }
    }
}

// The per-particle candidates of MultiCriterion::compute (core/timestepping/TimeStepCriterion.cpp:139-389) on the
// state after the step: CourantCriterion C h / c_s (c_s > 0); DerivativeCriterion f (|x| + x_min) / (|dx| + EPS)
// for every component of the first-order quantities (density, energy, deviatoric stress with its zz component
// -xx - yy, damage) whose |x| >= 2 x_min; AccelerationCriterion f (h^2 / |dv|^2)^(1/4) for |dv|^2 > EPS;
// DivergenceCriterion f_div / |div v| for |div v| > EPS. The global minimum of these, capped by the maximal
// step, is the minimum over the criteria the reference forms.
__device__ __forceinline__ double derivStep(double factor, double x, double dx, double xmin, double cur) {
    const double ax = fabs(x);
    if (ax < 2. * xmin) {
        return cur;
    }
    return fmin(cur, factor * (ax + xmin) / (fabs(dx) + SPH_EPS));
}

__device__ __forceinline__ double criteriaStep(const DState& s, const Physics& ph, const MaterialD& mt, uint32_t i,
    const dbl4& r, double rho, double drho, double u, double du, const double* S, const double* dS, double D,
    double dD) {
    double local = DBL_MAX;
    if (ph.criteria & SPHGPU_CRITERION_COURANT) {
        const double cs = s.cs[i];
        if (cs > 0.) {
            local = ph.courant * r.w / cs;
        }
    }
    if (ph.criteria & SPHGPU_CRITERION_DERIVATIVES) {
        const double f = ph.derivative_factor;
        local = derivStep(f, rho, drho, mt.rho_min, local);
        local = derivStep(f, u, du, mt.u_min, local);
        if (ph.solid) {
            // TracelessTensor components xx, yy, zz = -xx - yy, xy, xz, yz
            const double sv[6] = { S[0], S[1], -S[0] - S[1], S[2], S[3], S[4] };
            const double dsv[6] = { dS[0], dS[1], -dS[0] - dS[1], dS[2], dS[3], dS[4] };
            for (int c = 0; c < 6; ++c) {
                local = derivStep(f, sv[c], dsv[c], mt.s_min, local);
            }
            if (ph.damage) {
                local = derivStep(f, D, dD, mt.d_min, local);
            }
        }
    }
    if (ph.criteria & SPHGPU_CRITERION_ACCELERATION) {
        const dbl4 a = s.dv[i];
        const double a2 = a.x * a.x + a.y * a.y + a.z * a.z;
        if (a2 > SPH_EPS) {
            local = fmin(local, ph.derivative_factor * sqrt(sqrt(r.w * r.w / a2)));
        }
    }
    if (ph.criteria & SPHGPU_CRITERION_DIVERGENCE) {
        const double dv = fabs(s.divv[i]);
        if (dv > SPH_EPS) {
            local = fmin(local, ph.divergence_factor / dv);
        }
    }
    return local;
}

// PredictorCorrector::makeCorrections (TimeStepping.cpp:302-322) + the time-step criteria partial minimum
__global__ void correctKernel(DState s, Physics ph, const MaterialD* __restrict__ mats, const double* __restrict__ dtp,
    double* dtMin) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = s.n;
    double local = DBL_MAX;
    if (i < n) {
        const bool fast = ph.precision == SPHGPU_PRECISION_MIXED;
        const double dt = *dtp;
        const double dt2 = 0.5 * (dt * dt);
        const double ca = 1. / 3., cb = 0.5;
        // (mixed path) x - c (px - dx) dt as fma(px - dx, -c dt, x)
        const double kr = -(ca * dt2), kv = -(cb * dt), kh = -(0.5 * dt);
        dbl4 r = s.r[i], v = s.v[i];
        const dbl4 pa = s.pdv[i], a = s.dv[i];
        if (fast) {
            const double ex = pa.x - a.x, ey = pa.y - a.y, ez = pa.z - a.z, ew = pa.w - a.w;
            r.x = updFma(r.x, ex, kr);
            r.y = updFma(r.y, ey, kr);
            r.z = updFma(r.z, ez, kr);
            r.w = updFma(r.w, ew, kr);
            v.x = updFma(v.x, ex, kv);
            v.y = updFma(v.y, ey, kv);
            v.z = updFma(v.z, ez, kv);
            v.w = updFma(v.w, ew, kv);
        } else {
            r.x -= ca * (pa.x - a.x) * dt2;
            r.y -= ca * (pa.y - a.y) * dt2;
            r.z -= ca * (pa.z - a.z) * dt2;
            r.w -= ca * (pa.w - a.w) * dt2;
            v.x -= cb * (pa.x - a.x) * dt;
            v.y -= cb * (pa.y - a.y) * dt;
            v.z -= cb * (pa.z - a.z) * dt;
            v.w -= cb * (pa.w - a.w) * dt;
        }
        s.r[i] = r;
        s.v[i] = v;
        const MaterialD& mt = mats[ph.nmat > 1 ? s.mat[i] : 0];
        double rho = s.rho[i], drho = s.drho[i];
        rho = fast ? updFma(rho, s.pdrho[i] - drho, kh) : rho - 0.5 * (s.pdrho[i] - drho) * dt;
        clampDeriv(rho, drho, mt.rho_lo, mt.rho_hi);
        s.rho[i] = rho;
        s.drho[i] = drho;
        double u = s.u[i], du = s.du[i];
        u = fast ? updFma(u, s.pdu[i] - du, kh) : u - 0.5 * (s.pdu[i] - du) * dt;
        clampDeriv(u, du, mt.u_lo, mt.u_hi);
        s.u[i] = u;
        s.du[i] = du;
        double S[5] = { 0, 0, 0, 0, 0 }, dS[5] = { 0, 0, 0, 0, 0 }, D = 0., dD = 0.;
        if (ph.solid) {
            for (int c = 0; c < 5; ++c) {
                dS[c] = s.dS[c * n + i];
                const double Sc = s.S[c * n + i], pdS = s.pdS[c * n + i];
                S[c] = fast ? updFma(Sc, pdS - dS[c], kh) : Sc - 0.5 * (pdS - dS[c]) * dt;
                s.S[c * n + i] = S[c];
            }
            if (ph.damage) {
                D = s.D[i];
                dD = s.dD[i];
                D = fast ? updFma(D, s.pdD[i] - dD, kh) : D - 0.5 * (s.pdD[i] - dD) * dt;
                clampDeriv(D, dD, mt.d_lo, mt.d_hi);
                s.D[i] = D;
                s.dD[i] = dD;
            }
        }
        local = criteriaStep(s, ph, mt, i, r, rho, drho, u, du, S, dS, D, dD);
    }
    blockMinToGlobal(local, dtMin);
}

// LeapFrog::stepParticles first drift (TimeStepping.cpp:356-362) + materials initialize
__global__ void leapFrogDriftKernel(DState s, Physics ph, const MaterialD* __restrict__ mats, const double* __restrict__ dtp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) {
        return;
    }
    const double dt = *dtp;
    dbl4 r = s.r[i];
    const dbl4 v = s.v[i];
    r.x += v.x * 0.5 * dt;
    r.y += v.y * 0.5 * dt;
    r.z += v.z * 0.5 * dt;
    r.w += v.w * 0.5 * dt;
    s.r[i] = r;
    clampSmoothingLength(s, ph, i);
    (void)mats;
}

// AdaptiveSmoothingLength::initialize alone (ISolver::integrate on a state set by the caller)
__global__ void clampHKernel(DState s, Physics ph) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < s.n) {
        clampSmoothingLength(s, ph, i);
    }
}

// LeapFrog: first-order Euler update, kick, second drift (TimeStepping.cpp:367-388) + Courant minimum
__global__ void leapFrogKickKernel(DState s, Physics ph, const MaterialD* __restrict__ mats,
    const double* __restrict__ dtp, double* dtMin) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = s.n;
    double local = DBL_MAX;
    if (i < n) {
        const double dt = *dtp;
        const MaterialD& mt = mats[ph.nmat > 1 ? s.mat[i] : 0];
        double rho = s.rho[i], drho = s.drho[i];
        rho += drho * dt;
        clampDeriv(rho, drho, mt.rho_lo, mt.rho_hi);
        s.rho[i] = rho;
        s.drho[i] = drho;
        double u = s.u[i], du = s.du[i];
        u += du * dt;
        clampDeriv(u, du, mt.u_lo, mt.u_hi);
        s.u[i] = u;
        s.du[i] = du;
        double S[5] = { 0, 0, 0, 0, 0 }, dS[5] = { 0, 0, 0, 0, 0 }, D = 0., dD = 0.;
        if (ph.solid) {
            for (int c = 0; c < 5; ++c) {
                dS[c] = s.dS[c * n + i];
                S[c] = s.S[c * n + i] + dS[c] * dt;
                s.S[c * n + i] = S[c];
            }
            if (ph.damage) {
                D = s.D[i];
                dD = s.dD[i];
                D += dD * dt;
                clampDeriv(D, dD, mt.d_lo, mt.d_hi);
                s.D[i] = D;
                s.dD[i] = dD;
            }
        }
        dbl4 v = s.v[i];
        const dbl4 a = s.dv[i];
        v.x += a.x * dt;
        v.y += a.y * dt;
        v.z += a.z * dt;
        v.w += a.w * dt;
        dbl4 r = s.r[i];
        r.x += v.x * 0.5 * dt;
        r.y += v.y * 0.5 * dt;
        r.z += v.z * 0.5 * dt;
        r.w += v.w * 0.5 * dt;
        s.v[i] = v;
        s.r[i] = r;
        local = criteriaStep(s, ph, mt, i, r, rho, drho, u, du, S, dS, D, dD);
    }
    blockMinToGlobal(local, dtMin);
}

// end of a step: the run time advances by the step just taken; with criteria, the next step is the minimum
// capped by the maximal step, then limited to (1 + maxChange) times the previous step (MultiCriterion::
// compute's smoothing, off for maxChange >= DBL_MAX)
__global__ void stepEndKernel(double* dt, double* dtMin, double maxDt, double maxChange, double* time, int criterion) {
    *time += *dt;
    if (!criterion) {
        return;
    }
    double m = *dtMin;
    m = m > maxDt ? maxDt : m;
    if (maxChange < DBL_MAX) {
        const double lim = *dt * (1. + maxChange);
        if (m > lim) {
            m = lim;
        }
    }
    *dt = m;
    *dtMin = DBL_MAX;
}

// Neumaier-compensated block partial sums of the conserved totals, then one block adds the partials in a
// fixed order: deterministic for a fixed grid
constexpr int TOT_BLOCKS = 256;
constexpr int TOT_THREADS = 256;

__device__ __forceinline__ void kahanAdd(double& sum, double& c, double x) {
    const double t = sum + x;
    if (fabs(sum) >= fabs(x)) {
        c += (sum - t) + x;
    } else {
        c += (x - t) + sum;
    }
    sum = t;
}

// omega: frame frequency about z (TotalMomentum / TotalAngularMomentum(omega), core/physics/Integrals.cpp:24-62):
// the momenta use v + omega x r; the kinetic energy uses v alone, as TotalEnergy does
__global__ void totalsKernel(DState s, double omega, double* partial) {
    double sum[9], comp[9];
    for (int k = 0; k < 9; ++k) {
        sum[k] = 0.;
        comp[k] = 0.;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
        const dbl4 r = s.r[i], v = s.v[i];
        const double m = s.m[i];
        const double wx = v.x - omega * r.y, wy = v.y + omega * r.x, wz = v.z;
        kahanAdd(sum[0], comp[0], m * wx);
        kahanAdd(sum[1], comp[1], m * wy);
        kahanAdd(sum[2], comp[2], m * wz);
        kahanAdd(sum[3], comp[3], m * (r.y * wz - r.z * wy));
        kahanAdd(sum[4], comp[4], m * (r.z * wx - r.x * wz));
        kahanAdd(sum[5], comp[5], m * (r.x * wy - r.y * wx));
        kahanAdd(sum[6], comp[6], 0.5 * m * (v.x * v.x + v.y * v.y + v.z * v.z));
        kahanAdd(sum[7], comp[7], m * s.u[i]);
        kahanAdd(sum[8], comp[8], m);
    }
    __shared__ double sh[9][TOT_THREADS];
    for (int k = 0; k < 9; ++k) {
        sh[k][threadIdx.x] = sum[k] + comp[k];
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        double acc = 0., c = 0.;
        for (int t = 0; t < TOT_THREADS; ++t) {
            kahanAdd(acc, c, sh[threadIdx.x][t]);
        }
        partial[blockIdx.x * 9 + threadIdx.x] = acc + c;
    }
}

__global__ void totalsFinish(const double* partial, double* out) {
    if (threadIdx.x < 9) {
        double acc = 0., c = 0.;
        for (int b = 0; b < TOT_BLOCKS; ++b) {
            kahanAdd(acc, c, partial[b * 9 + threadIdx.x]);
        }
        out[threadIdx.x] = acc + c;
    }
}

__device__ __forceinline__ bool finite4(const dbl4& a) {
    return isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(a.w);
}

__global__ void checkFiniteKernel(DState s, unsigned long long* firstBad) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
        bool ok = finite4(s.r[i]) && finite4(s.v[i]) && finite4(s.dv[i]) && isfinite(s.m[i]);
        if (s.rho) {
            ok = ok && isfinite(s.rho[i]) && isfinite(s.u[i]) && isfinite(s.drho[i]) && isfinite(s.du[i]) &&
                 isfinite(s.p[i]) && isfinite(s.cs[i]);
        }
        if (s.omega) {
            ok = ok && finite4(s.omega[i]);
        }
        if (s.S) {
            for (int c = 0; c < 5; ++c) {
                ok = ok && isfinite(s.S[c * s.n + i]) && isfinite(s.dS[c * s.n + i]);
            }
        }
        if (s.D) {
            ok = ok && isfinite(s.D[i]) && isfinite(s.dD[i]);
        }
        if (!ok) {
            atomicMin(firstBad, (unsigned long long)i);
        }
    }
}

} // namespace

void launchMaterialsInit(const DState& s, const Physics& ph, const MaterialD* mats, cudaStream_t st) {
    if (s.n) {
        materialsInitKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, ph, mats);
    }
}

bool launchClampH(const DState& s, const Physics& ph, cudaStream_t st) {
    if (s.n && ph.adaptive_h) {
        clampHKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, ph);
        return true;
    }
    return false;
}

void launchPairSum64(const DState& s, const Grid& g, const Physics& ph, const MaterialD* mats, const double* lut,
    cudaStream_t st) {
    if (!s.n) {
        return;
    }
    // lanes per particle: a power of two up to 8, while the threads stay within about 1,024 per SM
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        sms = std::max(sms, 1);
    }
    uint32_t shift = 0;
    while (shift < 3 && (size_t(s.n) << (shift + 1)) <= size_t(sms) * 1024) {
        ++shift;
    }
    const int blocks = int((((size_t(s.n) << shift) + 127) / 128));
    if (ph.solid) {
        pairSum64Kernel<true><<<blocks, 128, 0, st>>>(s, g, ph, mats, lut, shift);
    } else {
        pairSum64Kernel<false><<<blocks, 128, 0, st>>>(s, g, ph, mats, lut, shift);
    }
}

void launchPredict(const DState& s, const Physics& ph, const MaterialD* mats, const double* dt, cudaStream_t st) {
    if (s.n) {
        predictKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, ph, mats, dt);
    }
}

void launchCorrect(const DState& s, const Physics& ph, const MaterialD* mats, const double* dt, double* dtMin,
    cudaStream_t st) {
    if (s.n) {
        correctKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, ph, mats, dt, dtMin);
    }
}

void launchLeapFrogDriftInit(const DState& s, const Physics& ph, const MaterialD* mats, const double* dt,
    cudaStream_t st) {
    if (s.n) {
        leapFrogDriftKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, ph, mats, dt);
    }
}

void launchLeapFrogKick(const DState& s, const Physics& ph, const MaterialD* mats, const double* dt, double* dtMin,
    cudaStream_t st) {
    if (s.n) {
        leapFrogKickKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, ph, mats, dt, dtMin);
    }
}

void launchStepEnd(double* dt, double* dtMin, double maxDt, double maxChange, double* time, bool criterion,
    cudaStream_t st) {
    stepEndKernel<<<1, 1, 0, st>>>(dt, dtMin, maxDt, maxChange, time, criterion ? 1 : 0);
}

void launchTotals(const DState& s, double omega, double* partial, double* out, cudaStream_t st) {
    totalsKernel<<<TOT_BLOCKS, TOT_THREADS, 0, st>>>(s, omega, partial);
    totalsFinish<<<1, 32, 0, st>>>(partial, out);
}

// dv = a_gravity + a_sph for pair loops that ran concurrently with the walk (GravitySolver::loop puts the gravity
// term into the accumulator before the pair terms; here it is added to their sum)
__global__ void addGravityKernel(DState s) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) {
        return;
    }
    const dbl4 a = s.agrav[i], d = s.dv[i];
    s.dv[i] = mkd4(a.x + d.x, a.y + d.y, a.z + d.z, d.w);
}

void launchAddGravity(const DState& s, cudaStream_t st) {
    if (s.n) {
        addGravityKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(s);
    }
}

void launchCorrection64(const DState& s, const Grid& g, const Physics& ph, const double* lut, cudaStream_t st) {
    if (s.n) {
        correction64Kernel<<<ceilDiv(s.n, 128), 128, 0, st>>>(s, g, ph, lut);
    }
}

void launchCheckFinite(const DState& s, unsigned long long* firstBad, cudaStream_t st) {
    if (s.n) {
        checkFiniteKernel<<<min(ceilDiv(s.n, 256), 152 * 8), 256, 0, st>>>(s, firstBad);
    }
}

} // namespace sphgpu
