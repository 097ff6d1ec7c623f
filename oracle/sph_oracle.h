/* sph_oracle.h — CPU oracle of OpenSPH's per-step hot path (TEST INFRASTRUCTURE, NOT THE PRODUCT).
 *
 * A plain C++ restatement of the reference algorithms, used only by tests/, by __graft_entry__.smoke() and
 * by bench.py's CPU-baseline leg to check and time the GPU library. Its settings and state layouts are the
 * public structs of include/sphgpu.h so both sides read the same inputs. Its results are pinned against
 * golden vectors produced by the reference itself (tests/golden/, made by tests/golden/make_golden.py from
 * oracle/ref_driver.cpp).
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include "../include/sphgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Host particle state. Arrays are owned by the caller; optional arrays may be NULL when the physics of the
 * run does not use them (solid arrays without SOLID_STRESS, damage arrays without a fracture model). */
typedef struct {
    uint32_t n;
    double* r;       /* 4n: x, y, z, h */
    double* v;       /* 4n */
    double* dv;      /* 4n */
    double* m;
    double* rho;
    double* drho;
    double* u;
    double* du;
    double* p;
    double* cs;
    double* divv;
    uint32_t* ncnt;
    uint32_t* flag;
    uint32_t* mat;
    double* S;       /* 5n: xx, yy, xy, xz, yz */
    double* dS;      /* 5n */
    double* gradv;   /* 6n: xx, yy, zz, xy, xz, yz */
    double* reduce;
    double* D;
    double* dD;
    double* eps_min;
    double* m_zero;
    double* growth;
    uint32_t* n_flaws;
    double* corr;    /* 6n, optional: strain-rate correction tensor (xx, yy, zz, xy, xz, yz) */
} ora_state;

/* Number of worker threads used by the parallel loops (0 = hardware concurrency). */
void ora_set_threads(int threads);

/* LUT kernels (core/sph/kernel/Kernel.h:51-188, core/sph/kernel/GravityKernel.h:35-120). */
double ora_sph_kernel_value(double qsqr);
double ora_sph_kernel_grad(double qsqr);
double ora_gravity_kernel_grad(double qsqr);

/* EosMaterial::initialize for one material (core/sph/Materials.cpp:47-58). */
int ora_eos(const sphgpu_material* mat, uint64_t n, const double* rho, const double* u, double* p, double* cs);

/* Interacting pair set of SymmetricSolver::loop (i < j, sorted by (i, j)). */
int ora_pairs(uint64_t n, const double* r, uint32_t* pi, uint32_t* pj, uint64_t capacity, uint64_t* npairs);

/* BarnesHut::build + evalSelfGravity, adding into dv (4n). kernel_radius 0 selects point masses (the
 * default-constructed kernel), 2 the SPH gravity kernel of the cubic spline. stats: approx, exact, nodes. */
int ora_gravity_bh(uint64_t n, const double* r, const double* m, double G, double theta, int order,
    uint32_t leaf_size, int kernel_radius, double* dv, uint64_t* stats);
/* BarnesHut::evalAcceleration at npoints points after building on the n particles. */
int ora_gravity_points(uint64_t n, const double* r, const double* m, double G, double theta, int order,
    uint32_t leaf_size, int kernel_radius, uint64_t npoints, const double* points, double* acc);
/* BruteForceGravity::evalSelfGravity restricted to the targets listed in idx (all if idx is NULL). */
/* BarnesHut::evalAttractors (core/gravity/BarnesHut.cpp:100-125): att 5 doubles per attractor (x, y, z, radius,
 * mass); dv (4 per particle) and acc (3 per attractor) are updated in place. */
int ora_gravity_attractors(uint64_t n, const double* r, const double* m, double G, int kernel_radius,
    uint64_t count, const double* att, double* dv, double* acc);
int ora_gravity_direct(uint64_t n, const double* r, const double* m, double G, int kernel_radius,
    uint64_t ntargets, const uint32_t* idx, double* acc);

/* ISolver::integrate on the state (highest derivatives are overwritten). */
int ora_integrate(const sphgpu_config* cfg, ora_state* s);
/* nsteps of ITimeStepping::step with the Courant criterion; *dt is the step to use first and receives the
 * next one; dts (nsteps entries, may be NULL) receives the step used by each step. */
int ora_run(const sphgpu_config* cfg, ora_state* s, uint32_t nsteps, double* dt, double* dts);
/* Conserved totals, same layout as sphgpu_totals. */
int ora_totals(const ora_state* s, double out[9]);

/* Frozen-list hydrodynamic model of the adjoint workload: ideal gas, ContinuityEquation + PressureForce +
 * StandardAV, leap-frog with a fixed time step, constant h, neighbour lists rebuilt every rebuild_every
 * steps and held fixed in between. Loss = sum over particles [0, n_target) of |v|^2 after `steps` steps.
 * With tangent inputs (any may be NULL = zero) it also returns the directional derivative of the loss
 * (forward-mode, dual numbers): the FP64 tangent-linear reference of the GPU adjoint. */
typedef struct {
    uint32_t steps;
    uint32_t rebuild_every;
    uint32_t n_target;
    uint32_t reserved;
    double dt;
    double gamma;
    double alpha;
    double beta;
} ora_frozen_params;

int ora_frozen_loss(const ora_frozen_params* prm, uint64_t n, const double* r, const double* v, const double* m,
    const double* rho, const double* u, const double* tr, const double* tv, const double* trho, const double* tu,
    double talpha, double* loss, double* dloss);

/* HardSphereSolver state (core/gravity/NBodySolver.cpp): r (4n: x, y, z, radius), v, dv (4n), m, angular
 * frequency w (4n, may be NULL = 0). Merged particles are removed in place, keeping the order of the others;
 * n is updated. */
typedef struct {
    uint32_t n;
    double* r;
    double* v;
    double* dv;
    double* m;
    double* w;
} ora_nbody_state;

/* HardSphereSolver::collide over [0, dt); stats (collisions, mergers, bounces, overlaps) are ADDED to;
 * ambiguous (may be NULL) is increased by the number of searches whose result may depend on the reference's
 * k-d tree traversal order; origin (n entries, may be NULL) receives the index before the call of each
 * particle kept. prev_removed / prev_count (n entries and a count, may be NULL): in, the indices the previous
 * call removed, which the first-pass searches skip as the reference's solver does; out, those of this call. */
int ora_nbody_collide(const sphgpu_config* cfg, ora_nbody_state* s, double dt, uint64_t stats[4],
    uint64_t* ambiguous, uint32_t* origin, uint32_t* prev_removed, uint32_t* prev_count);
/* HardSphereSolver::integrate: dv = self-gravity (Barnes-Hut), v.h = dv.h = 0. */
int ora_nbody_integrate(const sphgpu_config* cfg, ora_nbody_state* s);
/* nsteps leap-frog steps of the N-body solver; *dt is the first step and receives the next one; dts and
 * counts (particle count after each step) have nsteps entries and may be NULL. */
int ora_nbody_run(const sphgpu_config* cfg, ora_nbody_state* s, uint32_t nsteps, double* dt, double* dts,
    uint64_t stats[4], uint64_t* ambiguous, uint32_t* counts);

#ifdef __cplusplus
}
#endif

#endif
