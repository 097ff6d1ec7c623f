// nbody.cu — HardSphereSolver (core/gravity/NBodySolver.h:24-140, core/gravity/NBodySolver.cpp:17-597) and the
// collision / overlap handlers of core/gravity/Collision.h on the GPU.
//
// ISolver::integrate is the Barnes-Hut walk of gravity.cu / gravity32.cu (dv = a_gravity, h derivatives zeroed,
// NBodySolver.cpp:97-117). ISolver::collide (NBodySolver.cpp:329-484) is split into
//   1. a data-parallel first pass: search radius s_i = h_i + |v_i| dt, a uniform grid of cell edge
//      2 max(mean s, max s / 8) of which each particle scans the cells of its own search box, and per particle
//      the earliest collision or overlap with its lower-rank neighbours
//      (findClosestCollision with FIND_LOWER_RANK, NBodySolver.cpp:509-563; rank = order by s, ties by index);
//   2. a stable sort of the found records by the reference's order (time, -overlap, i, j);
//   3. one CTA that resolves the records in time order exactly as the reference's loop does: advance the
//      pair to the collision time, apply the handler, rewind with the new velocities, invalidate every
//      pending record that involves either particle and re-search the particles of the invalidated records
//      over [t + EPS, dt) (USE_RADII, radius 2 searchRadii); new records go into a binary heap in shared
//      memory, invalidation is lazy (a record holds the versions of its two particles);
//   4. a stable compaction of the merged-away particles (Storage::remove keeps the order of the others).
// Every arithmetic expression of the reference (checkCollision, the handlers, Vector / SymmetricTensor
// helpers) is restated with the same operation order, without FMA contraction (this unit is compiled with
// -fmad=false). The only library function whose last bit may differ from the host's is cbrt (the radius of a
// merger). Where the reference's result depends on its k-d tree traversal order (several overlapping
// neighbours of one particle: the reference takes the first it visits), this implementation takes the record
// that is smallest in the reference's own record order (largest overlap, then lowest index).

#include <algorithm>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "state.h"

namespace sphgpu {

namespace {

// Constants::gravity (core/physics/Constants.h:32): the merge criteria use it whatever the gravity constant
constexpr double G_PHYS = 6.67408e-11;

// CollisionRecord (NBodySolver.cpp:165-211) plus the bookkeeping of this implementation
struct CollRec {
    double t;        // collision time within the step (interval lower bound for overlaps); +inf: none
    double nov;      // minus the overlap value (0 for collisions)
    uint32_t i, j;   // i: the particle whose search produced the record
    uint32_t vi, vj; // versions of i and j when the record was made
    int32_t next_i;  // next (older) record in the list of particle i
    int32_t next_j;  // next record in the list of particle j
    uint32_t dead;   // rejected by the handler (CollisionResult::NONE): removed alone
    uint32_t pad;
};

// record order of the reference: (time, -overlap, i, j)
__device__ __forceinline__ bool recLess(double ta, double nova, uint32_t ia, uint32_t ja, double tb, double novb,
    uint32_t ib, uint32_t jb) {
    if (ta != tb) {
        return ta < tb;
    }
    if (nova != novb) {
        return nova < novb;
    }
    if (ia != ib) {
        return ia < ib;
    }
    return ja < jb;
}

// counters (device, 16 x u64)
enum {
    CNT_COLLISIONS = 0, // cumulative over the call
    CNT_MERGERS = 1,
    CNT_BOUNCES = 2,
    CNT_OVERLAPS = 3,
    CNT_RECORDS = 4,    // first-pass records
    CNT_REMOVED = 5,    // particles removed by this call
    CNT_ERROR = 6,      // capacity error bits
    CNT_EVENTS = 7,     // records processed
    CNT_CYCLES_LEAD = 8,   // SM cycles of the event loop in its serial part (selection, handler, invalidation)
    CNT_CYCLES_SEARCH = 9, // in the re-searches
    CNT_CYCLES_INSERT = 10, // in the insertion of new records
    CNT_COUNT = 16
};
enum : unsigned long long {
    COLL_ERR_POOL = 1,    // record pool exhausted
    COLL_ERR_HEAP = 2,    // heap of new records exhausted
    COLL_ERR_INVALID = 4, // too many invalidated particles for one collision
    COLL_ERR_EXTRA = 8    // moved-particle lists exhausted
};

enum Result { RES_NONE = 0, RES_BOUNCE = 1, RES_MERGER = 2 };

// ---- Vector and SymmetricTensor arithmetic of the reference (core/objects/geometry/Vector.h,
// ---- SymmetricTensor.h), four components where the reference's operators act on four
__device__ __forceinline__ dbl4 add4(const dbl4& a, const dbl4& b) {
    return mkd4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ dbl4 sub4(const dbl4& a, const dbl4& b) {
    return mkd4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__device__ __forceinline__ dbl4 mul4(const dbl4& a, double f) {
    return mkd4(a.x * f, a.y * f, a.z * f, a.w * f);
}
__device__ __forceinline__ dbl4 div4(const dbl4& a, double f) {
    return mkd4(a.x / f, a.y / f, a.z / f, a.w / f);
}
// dot and getSqrLength use x, y, z only (Vector.h:566-589)
__device__ __forceinline__ double dot3(const dbl4& a, const dbl4& b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
__device__ __forceinline__ double len2(const dbl4& a) {
    return dot3(a, a);
}
__device__ __forceinline__ dbl4 cross3(const dbl4& a, const dbl4& b) {
    return mkd4(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.);
}
__device__ __forceinline__ double pow3(double x) {
    return x * x * x;
}
// weightedAverage (Collision.h:81-85)
__device__ __forceinline__ dbl4 weightedAverage(const dbl4& a, double wa, const dbl4& b, double wb) {
    return div4(add4(mul4(a, wa), mul4(b, wb)), wa + wb);
}

struct Sym {
    double d[3], o[3]; // diagonal, off-diagonal xy xz yz
};
// Rigid::sphereInertia (core/physics/Functions.h:61-63): identity * (0.4 m r^2)
__device__ __forceinline__ Sym sphereInertia(double m, double r) {
    const double k = 0.4 * m * (r * r);
    return Sym{ { 1. * k, 1. * k, 1. * k }, { 0. * k, 0. * k, 0. * k } };
}
// SymmetricTensor * Vector (SymmetricTensor.h:102-107)
__device__ __forceinline__ dbl4 symMul(const Sym& t, const dbl4& v) {
    return mkd4(t.d[0] * v.x + t.o[0] * v.y + t.o[1] * v.z, t.o[0] * v.x + t.d[1] * v.y + t.o[2] * v.z,
        t.o[1] * v.x + t.o[2] * v.y + t.d[2] * v.z, 0.);
}
// SymmetricTensor::inverse (SymmetricTensor.h:193-231)
__device__ __forceinline__ Sym symInverse(const Sym& t) {
    const double det = t.d[0] * t.d[1] * t.d[2] + 2. * t.o[0] * t.o[1] * t.o[2] -
                       ((t.o[0] * t.o[0]) * t.d[2] + (t.o[1] * t.o[1]) * t.d[1] + (t.o[2] * t.o[2]) * t.d[0]);
    Sym r;
    r.d[0] = (t.d[1] * t.d[2] - t.o[2] * t.o[2]) / det;
    r.d[1] = (t.d[2] * t.d[0] - t.o[1] * t.o[1]) / det;
    r.d[2] = (t.d[0] * t.d[1] - t.o[0] * t.o[0]) / det;
    r.o[0] = (t.o[1] * t.o[2] - t.d[2] * t.o[0]) / det;
    r.o[1] = (t.o[2] * t.o[0] - t.d[1] * t.o[1]) / det;
    r.o[2] = (t.o[0] * t.o[1] - t.d[0] * t.o[2]) / det;
    return r;
}

// areParticlesBound (Collision.h:86-91)
__device__ __forceinline__ bool particlesBound(double mSum, double hSum, const dbl4& dv, double limit) {
    const double vEscSqr = 2. * G_PHYS * mSum / hSum;
    const double vRelSqr = len2(dv);
    return vRelSqr * limit < vEscSqr;
}

// The would-be merger of i and j (MergingCollisionHandler::collide without the inertia tensor,
// Collision.h:160-215); its acceptance (acceptMerge, :249-261) is tested in mergeCollide
struct Merger {
    double h, m;
    dbl4 r, v, w;
};
__device__ Merger mergerOf(const dbl4& ri, const dbl4& vi, double mi, const dbl4& wi, const dbl4& rj,
    const dbl4& vj, double mj, const dbl4& wj) {
    Merger g;
    g.h = cbrt(pow3(ri.w) + pow3(rj.w));
    g.m = mi + mj;
    g.r = weightedAverage(ri, mi, rj, mj);
    g.v = weightedAverage(vi, mi, vj, mj);
    dbl4 L = add4(mul4(cross3(sub4(ri, g.r), sub4(vi, g.v)), mi), mul4(cross3(sub4(rj, g.r), sub4(vj, g.v)), mj));
    L = add4(L, symMul(sphereInertia(mi, ri.w), wi));
    L = add4(L, symMul(sphereInertia(mj, rj.w), wj));
    g.w = symMul(symInverse(sphereInertia(g.m, g.h)), L);
    return g;
}
// The two particles of a collision, copied out of the state arrays for the handlers and written back after
// them (the handlers' arithmetic on the copies is the same as on the arrays)
struct PairState {
    dbl4 ri, rj, vi, vj, wi, wj;
    double mi, mj;
    uint32_t removedJ;
};

// MergingCollisionHandler::collide (Collision.h:160-243). acceptMerge tests boundness first and needs the merger
// only for the rotation limit, so the merger is formed after that test (it has no side effects).
__device__ int mergeCollide(PairState& S, double bounceLimit, double rotationLimit) {
    if (!particlesBound(S.mi + S.mj, S.ri.w + S.rj.w, sub4(S.vi, S.vj), bounceLimit)) {
        return RES_NONE;
    }
    const Merger g = mergerOf(S.ri, S.vi, S.mi, S.wi, S.rj, S.vj, S.mj, S.wj);
    const double omegaCritSqr = G_PHYS * (S.mi + S.mj) / pow3(g.h);
    if (len2(g.w) * rotationLimit > omegaCritSqr) {
        return RES_NONE;
    }
    S.mi = g.m;
    S.ri = mkd4(g.r.x, g.r.y, g.r.z, g.h);
    S.vi = mkd4(g.v.x, g.v.y, g.v.z, 0.);
    S.wi = g.w;
    S.removedJ = 1;
    return RES_MERGER;
}

// ElasticBounceHandler::reflect (Collision.h:316-326)
__device__ __forceinline__ dbl4 reflect(const dbl4& v, const dbl4& vCom, const dbl4& dir, double rn, double rt) {
    const dbl4 vRel = sub4(v, vCom);
    const double proj = dot3(vRel, dir);
    const dbl4 vT = sub4(vRel, mul4(dir, proj));
    const dbl4 vN = mul4(dir, proj);
    return add4(sub4(mul4(vT, rt), mul4(vN, rn)), vCom);
}

// ElasticBounceHandler::collide (Collision.h:301-313)
__device__ int bounceCollide(PairState& S, double rn, double rt) {
    const dbl4 d = sub4(S.ri, S.rj);
    const dbl4 dr = div4(d, sqrt(len2(d)));
    const dbl4 ndr = mkd4(-dr.x, -dr.y, -dr.z, -dr.w);
    const dbl4 vCom = weightedAverage(S.vi, S.mi, S.vj, S.mj);
    const dbl4 vi = reflect(S.vi, vCom, ndr, rn, rt);
    const dbl4 vj = reflect(S.vj, vCom, dr, rn, rt);
    S.vi = mkd4(vi.x, vi.y, vi.z, 0.);
    S.vj = mkd4(vj.x, vj.y, vj.z, 0.);
    return RES_BOUNCE;
}

// the collision handler of Factory::getCollisionHandler (core/system/Factory.cpp:415-429)
__device__ int collisionHandler(PairState& S, const CollideParams& p) {
    switch (p.handler) {
    case SPHGPU_COLLISION_PERFECT_MERGING:
        return mergeCollide(S, 0., 0.);
    case SPHGPU_COLLISION_ELASTIC_BOUNCE:
        return bounceCollide(S, p.rest_n, p.rest_t);
    default: { // MERGE_OR_BOUNCE: FallbackHandler<MergingCollisionHandler, ElasticBounceHandler>
        const int res = mergeCollide(S, p.bounce_limit, p.rotation_limit);
        return res != RES_NONE ? res : bounceCollide(S, p.rest_n, p.rest_t);
    }
    }
}

// RepelHandler::handle before its follow-up handler (Collision.h:443-467)
__device__ void repel(PairState& S) {
    const dbl4 d = sub4(S.ri, S.rj);
    const double dist = sqrt(len2(d));
    dbl4 dir = div4(d, dist);
    dir.w = 0.;
    const double x1 = (S.ri.w + S.rj.w - dist) / (1. + S.mi / S.mj);
    const double x2 = S.mi / S.mj * x1;
    S.ri = add4(S.ri, mul4(dir, x1));
    S.rj = sub4(S.rj, mul4(dir, x2));
}

// IOverlapHandler::handle of Factory::getOverlapHandler (core/system/Factory.cpp:431-450, Collision.h:372-567)
__device__ void overlapHandle(PairState& S, const CollideParams& p) {
    switch (p.overlap) {
    case SPHGPU_OVERLAP_FORCE_MERGE:
        mergeCollide(S, 0., 0.);
        break;
    case SPHGPU_OVERLAP_REPEL:
        repel(S);
        bounceCollide(S, p.rest_n, p.rest_t);
        break;
    case SPHGPU_OVERLAP_REPEL_OR_MERGE:
        repel(S);
        if (mergeCollide(S, p.bounce_limit, p.rotation_limit) == RES_NONE) {
            bounceCollide(S, p.rest_n, p.rest_t);
        }
        break;
    case SPHGPU_OVERLAP_INTERNAL_BOUNCE:
        bounceCollide(S, p.rest_n, p.rest_t);
        break;
    case SPHGPU_OVERLAP_PASS_OR_MERGE:
        mergeCollide(S, p.bounce_limit, p.rotation_limit);
        break;
    default:
        break;
    }
}

// IOverlapHandler::overlaps (Collision.h:379-381, 404-406, 439-442, 494-499, 537-560)
__device__ bool overlapHandled(const CollideParams& p, const dbl4& ri, const dbl4& vi, double mi, const dbl4& wi,
    const dbl4& rj, const dbl4& vj, double mj, const dbl4& wj) {
    switch (p.overlap) {
    case SPHGPU_OVERLAP_NONE:
        return false;
    case SPHGPU_OVERLAP_INTERNAL_BOUNCE:
        return dot3(sub4(ri, rj), sub4(vi, vj)) < 0.;
    case SPHGPU_OVERLAP_PASS_OR_MERGE: {
        if (!particlesBound(mi + mj, ri.w + rj.w, sub4(vi, vj), p.bounce_limit)) {
            return false;
        }
        const Merger g = mergerOf(ri, vi, mi, wi, rj, vj, mj, wj);
        const double omegaCritSqr = G_PHYS * (mi + mj) / pow3(g.h);
        return !(len2(g.w) * p.rotation_limit > omegaCritSqr);
    }
    default:
        return true;
    }
}

// HardSphereSolver::checkCollision (NBodySolver.cpp:565-597): time of contact within [0, dt], or +inf
__device__ double checkCollision(const dbl4& r1, const dbl4& v1, const dbl4& r2, const dbl4& v2, double dt) {
    const dbl4 dr = sub4(r1, r2);
    const dbl4 dv = sub4(v1, v2);
    const double dvdr = dot3(dv, dr);
    if (dvdr >= 0.) {
        return INFINITY;
    }
    const double dvl = len2(dv);
    const dbl4 drPerp = sub4(dr, div4(mul4(dv, dvdr), dvl));
    const double hs = r1.w + r2.w;
    if (len2(drPerp) <= hs * hs) {
        const double dv2 = len2(dv);
        const double det = 1. - (len2(dr) - hs * hs) / (dvdr * dvdr) * dv2;
        const double sqrtDet = sqrt(fmax(0., det));
        const double root = det > 1. ? 1. + sqrtDet : 1. - sqrtDet;
        const double tColl = -dvdr / dv2 * root;
        if (tColl <= dt) {
            return tColl;
        }
    }
    return INFINITY;
}

// One candidate of findClosestCollision (NBodySolver.cpp:530-562) for the interval [lower, lower + size]:
// the record key (time, -overlap) or time = +inf when the pair neither overlaps (with the overlap handled)
// nor collides in the interval.
struct Cand {
    double t, nov;
    uint32_t j;
};
__device__ __forceinline__ bool candLess(const Cand& a, const Cand& b) {
    if (a.t != b.t) {
        return a.t < b.t;
    }
    if (a.nov != b.nov) {
        return a.nov < b.nov;
    }
    return a.j < b.j;
}
__device__ Cand evalPair(const CollideParams& p, uint32_t j, const dbl4& ri, const dbl4& vi, double mi,
    const dbl4& wi, const dbl4& rj, const dbl4& vj, double mj, const dbl4& wj, double lower, double size) {
    Cand c{ INFINITY, 0., j };
    const dbl4 r1 = add4(ri, mul4(vi, lower));
    const dbl4 r2 = add4(rj, mul4(vj, lower));
    const double hs = ri.w + rj.w;
    {
        // Conservative FP32 rejection of the common case: the surfaces are further apart than the relative
        // motion can close within the interval, |r1 - r2| > (h_i + h_j + |v_i - v_j| size)(1 + 1e-4). Such a
        // pair neither overlaps nor touches before lower + size, so the FP64 test below would find nothing
        // either; the differences are formed in FP64 first, so the FP32 error is relative (~1e-7).
        const float dx = float(r1.x - r2.x), dy = float(r1.y - r2.y), dz = float(r1.z - r2.z);
        const float ux = float(vi.x - vj.x), uy = float(vi.y - vj.y), uz = float(vi.z - vj.z);
        const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
        const float reach = (float(hs) + sqrtf(ux * ux + uy * uy + uz * uz) * float(size)) * 1.0001f;
        if (dist > reach) {
            return c;
        }
    }
    const double overlapValue = 1. - len2(sub4(r1, r2)) / (hs * hs);
    if (overlapValue > p.allowed * p.allowed) {
        if (overlapHandled(p, ri, vi, mi, wi, rj, vj, mj, wj)) {
            c.t = lower;
            c.nov = -overlapValue;
        }
        return c;
    }
    const double t = checkCollision(r1, vi, r2, vj, size);
    if (t < INFINITY) {
        c.t = t + lower;
    }
    return c;
}

__device__ __forceinline__ int nbCellCoord(double x, double lo, double inv, int dim) {
    int c = int((x - lo) * inv);
    return min(max(c, 0), dim - 1);
}

// the cells of the box [x - R, x + R] along one axis, R widened by 1e-9 (relative to R and to the coordinates)
// so that rounding in x -/+ R cannot drop the cell of a particle closer than R
__device__ __forceinline__ void cellSpan(double x, double R, double lo, double inv, int dim, int& c0, int& c1) {
    const double w = R * (1. + 1e-9) + 1e-9 * (fabs(x) + fabs(lo));
    c0 = nbCellCoord(x - w, lo, inv, dim);
    c1 = nbCellCoord(x + w, lo, inv, dim);
}

__device__ __forceinline__ uint32_t nbCellKey(const GridInfo& gi, const dbl4& p) {
    const int cx = nbCellCoord(p.x, gi.lo[0], gi.inv_cell, gi.dims[0]);
    const int cy = nbCellCoord(p.y, gi.lo[1], gi.inv_cell, gi.dims[1]);
    const int cz = nbCellCoord(p.z, gi.lo[2], gi.inv_cell, gi.dims[2]);
    return (uint32_t(cz) * uint32_t(gi.dims[1]) + uint32_t(cy)) * uint32_t(gi.dims[0]) + uint32_t(cx);
}

// ---- 1. first pass -----------------------------------------------------------------------------------------

// search radius r_H + |v| dt (NBodySolver.cpp:348-351, 515-517) and the per-call bookkeeping
__global__ void prepareKernel(DState s, Collide c, const double* __restrict__ dtp, double factor) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) {
        return;
    }
    const double dt = factor * *dtp;
    const dbl4 r = s.r[i], v = s.v[i];
    c.s[i] = r.w + sqrt(len2(v)) * dt;
    c.writer[i] = -1;
    c.ver[i] = 0;
    c.bounces[i] = 0;
    c.removed[i] = 0;
    c.head[i] = -1;
}

// cell-sorted copies for the first pass: FP64 positions, FP32 positions relative to the origin of the particle's
// cell with the search radius, and the bit patterns of the search radii (non-negative doubles order like their
// bit patterns)
__global__ void gatherKernel(DState s, Grid g, Collide c) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= s.n) {
        return;
    }
    const GridInfo gi = *g.info;
    const uint32_t i = g.perm[k];
    const uint32_t key = g.keys_sorted[k];
    const uint32_t cx = key % uint32_t(gi.dims[0]);
    const uint32_t cy = (key / uint32_t(gi.dims[0])) % uint32_t(gi.dims[1]);
    const uint32_t cz = key / (uint32_t(gi.dims[0]) * uint32_t(gi.dims[1]));
    const dbl4 r = s.r[i];
    const double si = c.s[i];
    c.rs[k] = r;
    c.posf[k] = make_float4(float(r.x - (gi.lo[0] + double(cx) * gi.cell)), float(r.y - (gi.lo[1] + double(cy) * gi.cell)),
        float(r.z - (gi.lo[2] + double(cz) * gi.cell)), float(2. * si));
    c.sbits[k] = static_cast<unsigned long long>(__double_as_longlong(si));
    const dbl4 v = s.v[i];
    c.velf[k] = make_float4(float(v.x), float(v.y), float(v.z), float(r.w));
    c.moved_cell[i] = int32_t(key);
}

// findClosestCollision(i, FIND_LOWER_RANK, [0, dt]) of every particle (NBodySolver.cpp:367-374, 509-563): the
// neighbours j of lower rank with |r_j - r_i|^2 < (2 s_i)^2 (KdTree::find, core/objects/finders/KdTree.inl.h:
// 316-391, rank by s as in buildWithRank's comparator, :348-351); every neighbour found records i as a
// writer of its search radius (searchRadii[i] = searchRadii[j] = s_i, the largest index writing last).
// The distance test runs on the FP32 cell-relative copies with a margin that bounds their rounding
// (1e-6 of the radius plus 2e-5 of the cell edge); only candidates within the margin of the sphere are tested
// again in FP64, so the neighbour set is exactly the FP64 one.
__global__ void __launch_bounds__(128, 4) detectKernel(DState s, Grid g, Collide c, CollideParams p,
    const double* __restrict__ dtp, double factor) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= s.n) {
        return;
    }
    const GridInfo gi = *g.info;
    const uint32_t i = g.perm[k];
    const double dt = factor * *dtp;
    const dbl4 ri = c.rs[k];
    const float4 pi = c.posf[k];
    const unsigned long long sbi = c.sbits[k];
    const double radius = 2. * __longlong_as_double(static_cast<long long>(sbi));
    const double radiusSqr = radius * radius;
    const float slack = float(radius) * 1e-6f + float(gi.cell) * 2e-5f;
    const float4 vfi = c.velf[k];
    const float vabsi = sqrtf(vfi.x * vfi.x + vfi.y * vfi.y + vfi.z * vfi.z);
    const float dtf = float(dt);
    const float rOut = float(radius) + slack;
    const float rIn = float(radius) - slack;
    const float rOut2 = rOut * rOut;
    const float rIn2 = rIn > 0.f ? rIn * rIn : -1.f;
    const uint32_t key = g.keys_sorted[k];
    const int cx = int(key % uint32_t(gi.dims[0]));
    const int cy = int((key / uint32_t(gi.dims[0])) % uint32_t(gi.dims[1]));
    const int cz = int(key / (uint32_t(gi.dims[0]) * uint32_t(gi.dims[1])));
    const float cellf = float(gi.cell);
    int x0, x1, y0, y1, z0, z1;
    cellSpan(ri.x, radius, gi.lo[0], gi.inv_cell, gi.dims[0], x0, x1);
    cellSpan(ri.y, radius, gi.lo[1], gi.inv_cell, gi.dims[1], y0, y1);
    cellSpan(ri.z, radius, gi.lo[2], gi.inv_cell, gi.dims[2], z0, z1);
    Cand best{ INFINITY, 0., 0u };
    bool any = false;
    dbl4 vi, wi;
    double mi = 0.;
    bool own = false;
    for (int z = z0; z <= z1; ++z) {
        const float oz = float(z - cz) * cellf - pi.z;
        for (int y = y0; y <= y1; ++y) {
            const float oy = float(y - cy) * cellf - pi.y;
            for (int x = x0; x <= x1; ++x) {
                const float ox = float(x - cx) * cellf - pi.x;
                const uint32_t cell = (uint32_t(z) * uint32_t(gi.dims[1]) + uint32_t(y)) * uint32_t(gi.dims[0]) +
                                      uint32_t(x);
                const uint32_t end = g.cell_end[cell];
                for (uint32_t q = g.cell_start[cell]; q < end; ++q) {
                    if (q == k) {
                        continue;
                    }
                    const float4 pj = c.posf[q];
                    const float dx = pj.x + ox, dy = pj.y + oy, dz = pj.z + oz;
                    const float d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 > rOut2) {
                        continue;
                    }
                    const unsigned long long sbj = c.sbits[q];
                    const uint32_t j = g.perm[q];
                    if (!(sbj < sbi || (sbj == sbi && j < i))) {
                        continue;
                    }
                    dbl4 rj;
                    if (d2 >= rIn2) {
                        rj = c.rs[q];
                        if (!(len2(sub4(rj, ri)) < radiusSqr)) {
                            continue;
                        }
                    }
                    any = true;
                    atomicMax(&c.writer[j], int32_t(i));
                    if (c.prev_removed[j]) {
                        // the reference's `removed` set still holds the previous call's indices during the
                        // first pass (it is cleared after it, NBodySolver.cpp:367-396)
                        continue;
                    }
                    {
                        // the FP32 rejection of evalPair on the cell-sorted copies (no FP64 work for pairs
                        // whose surfaces are further apart than their relative motion can close in dt); the
                        // distance is bounded below by the copies' rounding slack, the velocity difference
                        // widened by 1e-6 of the speeds
                        const float4 vfj = c.velf[q];
                        const float ux = vfi.x - vfj.x, uy = vfi.y - vfj.y, uz = vfi.z - vfj.z;
                        const float vabsj = sqrtf(vfj.x * vfj.x + vfj.y * vfj.y + vfj.z * vfj.z);
                        const float du = sqrtf(ux * ux + uy * uy + uz * uz);
                        const float dist = sqrtf(d2) * (1.f - 1e-6f) - slack;
                        const float reach = (vfi.w + vfj.w + du * dtf) * 1.0001f + 1e-6f * (vabsi + vabsj) * dtf;
                        if (dist > reach) {
                            continue;
                        }
                    }
                    if (!own) {
                        vi = s.v[i];
                        wi = s.omega[i];
                        mi = s.m[i];
                        own = true;
                    }
                    rj = c.rs[q];
                    const Cand cd = evalPair(p, j, ri, vi, mi, wi, rj, s.v[j], s.m[j], s.omega[j], 0., dt);
                    if (candLess(cd, best)) {
                        best = cd;
                    }
                }
            }
        }
    }
    if (any) {
        atomicMax(&c.writer[i], int32_t(i));
    }
    CollRec rec;
    rec.t = best.t;
    rec.nov = best.t < INFINITY ? best.nov : 0.;
    rec.i = i;
    rec.j = best.j;
    rec.vi = 0;
    rec.vj = 0;
    rec.next_i = -1;
    rec.next_j = -1;
    rec.dead = 0;
    rec.pad = 0;
    static_cast<CollRec*>(c.pool)[i] = rec;
    c.valid[i] = best.t < INFINITY ? 1u : 0u;
}

// ---- 2. order of the first-pass records ----------------------------------------------------------------------

// key of the stable radix passes: 0 -> -overlap, 1 -> time
__global__ void recordKeysKernel(const CollRec* __restrict__ pool, const uint32_t* __restrict__ order, uint32_t n,
    int which, unsigned long long* keys) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        const CollRec& r = pool[order[k]];
        keys[k] = orderKey(which == 0 ? r.nov : r.t);
    }
}

// the first-pass records enter the per-particle record lists (order within the lists is irrelevant: all of
// them carry version 0)
__global__ void linkKernel(CollRec* pool, const uint32_t* __restrict__ order, uint32_t n, int32_t* head) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        const uint32_t id = order[k];
        CollRec& r = pool[id];
        r.next_i = atomicExch(&head[r.i], int32_t(id));
        r.next_j = atomicExch(&head[r.j], int32_t(id));
    }
}

// ---- 3. the collision loop (NBodySolver.cpp:401-477) ------------------------------------------------------------

constexpr int EV_THREADS = 256;
constexpr int EV_WARPS = EV_THREADS / 32;
constexpr int HEAP_CAP = 3072; // records made by re-searches and not yet processed
constexpr int INV_CAP = 256;   // particles of the records invalidated by one collision

struct HeapEnt {
    double t, nov;
    uint32_t i, j;
    uint32_t rec, pad;
};

struct EvShared {
    HeapEnt heap[HEAP_CAP];
    uint32_t inv[INV_CAP];
    Cand res[INV_CAP];
    uint32_t invCount;
    uint32_t heapSize;
    uint32_t evI, evJ;
    int done;
    int search;
    double lower, size;
};

struct EvArgs {
    CollRec* pool;
    uint32_t poolCapacity;
    const uint32_t* order; // first-pass records in processing order
    uint32_t nrec;
    int32_t* head;
    uint32_t* ver;
    uint32_t* bounces;
    const int32_t* writer;
    const double* srad;    // search radius of each particle (s of the writer)
    int32_t* movedCell;
    int32_t* extraHead;
    int32_t* extra;
    uint32_t extraCapacity;
    uint32_t* removed;
    unsigned long long* counters;
};

__device__ __forceinline__ bool heapLess(const HeapEnt& a, const HeapEnt& b) {
    return recLess(a.t, a.nov, a.i, a.j, b.t, b.nov, b.i, b.j);
}

__device__ void heapPush(EvShared& sh, const HeapEnt& e) {
    uint32_t k = sh.heapSize++;
    while (k > 0) {
        const uint32_t parent = (k - 1) / 2;
        if (!heapLess(e, sh.heap[parent])) {
            break;
        }
        sh.heap[k] = sh.heap[parent];
        k = parent;
    }
    sh.heap[k] = e;
}

__device__ void heapPop(EvShared& sh) {
    const uint32_t n = --sh.heapSize;
    if (n == 0) {
        return;
    }
    const HeapEnt last = sh.heap[n];
    uint32_t k = 0;
    while (true) {
        uint32_t c = 2 * k + 1;
        if (c >= n) {
            break;
        }
        if (c + 1 < n && heapLess(sh.heap[c + 1], sh.heap[c])) {
            ++c;
        }
        if (!heapLess(sh.heap[c], last)) {
            break;
        }
        sh.heap[k] = sh.heap[c];
        k = c;
    }
    sh.heap[k] = last;
}

__device__ __forceinline__ bool recValid(const CollRec& r, const uint32_t* ver) {
    return !r.dead && r.vi == ver[r.i] && r.vj == ver[r.j];
}

// FlatSet insertion of the invalidated indices (CollisionSet::removeByIndex, NBodySolver.cpp:265-280)
__device__ __forceinline__ bool invAdd(EvShared& sh, uint32_t x) {
    for (uint32_t k = 0; k < sh.invCount; ++k) {
        if (sh.inv[k] == x) {
            return true;
        }
    }
    if (sh.invCount >= INV_CAP) {
        return false;
    }
    sh.inv[sh.invCount++] = x;
    return true;
}

// the pending records of particle q that are still valid contribute both their particles
__device__ bool collectPartners(EvShared& sh, const EvArgs& a, uint32_t q) {
    int32_t id = a.head[q];
    const uint32_t vq = a.ver[q];
    while (id >= 0) {
        const CollRec& r = a.pool[id];
        const bool isI = r.i == q;
        if ((isI ? r.vi : r.vj) != vq) {
            break; // this and every older record of q were made before q's last collision
        }
        if (recValid(r, a.ver)) {
            if (!invAdd(sh, r.i) || !invAdd(sh, r.j)) {
                return false;
            }
        }
        id = isI ? r.next_i : r.next_j;
    }
    return true;
}

// a particle moved by a handler is listed in the cell of its new position as well
__device__ bool listMoved(const EvArgs& a, const GridInfo& gi, const dbl4& r, uint32_t q, uint32_t& extraUsed) {
    const int32_t cell = int32_t(nbCellKey(gi, r));
    if (cell == a.movedCell[q]) {
        return true;
    }
    if (extraUsed >= a.extraCapacity) {
        return false;
    }
    const uint32_t e = extraUsed++;
    a.extra[3 * e + 0] = int32_t(q);
    a.extra[3 * e + 1] = a.extraHead[cell];
    a.extra[3 * e + 2] = cell;
    a.extraHead[cell] = int32_t(e);
    a.movedCell[q] = cell;
    return true;
}

__device__ __forceinline__ void candShflMin(Cand& c) {
    for (int off = 16; off > 0; off >>= 1) {
        Cand o;
        o.t = __shfl_xor_sync(0xffffffffu, c.t, off);
        o.nov = __shfl_xor_sync(0xffffffffu, c.nov, off);
        o.j = __shfl_xor_sync(0xffffffffu, c.j, off);
        if (candLess(o, c)) {
            c = o;
        }
    }
}

// one warp: findClosestCollision(idx, USE_RADII, [lower, lower + size]) (NBodySolver.cpp:509-563) with
// findAll(idx, 2 searchRadii[idx]) over the current positions: the grid cells around idx hold the particles at
// their positions at the start of the call, the moved-particle lists those a handler moved since.
__device__ Cand researchWarp(const DState& s, const Grid& g, const GridInfo& gi, const EvArgs& a,
    const CollideParams& p, uint32_t idx, double lower, double size) {
    const int lane = threadIdx.x & 31;
    Cand best{ INFINITY, 0., 0u };
    const double sr = a.srad[idx];
    if (!(sr > 0.)) {
        return best;
    }
    const double radius = 2. * sr;
    const double radiusSqr = radius * radius;
    const dbl4 ri = s.r[idx], vi = s.v[idx], wi = s.omega[idx];
    const double mi = s.m[idx];
    int x0, x1, y0, y1, z0, z1;
    cellSpan(ri.x, radius, gi.lo[0], gi.inv_cell, gi.dims[0], x0, x1);
    cellSpan(ri.y, radius, gi.lo[1], gi.inv_cell, gi.dims[1], y0, y1);
    cellSpan(ri.z, radius, gi.lo[2], gi.inv_cell, gi.dims[2], z0, z1);
    auto consider = [&](uint32_t j, const dbl4& rj) {
        if (j == idx) {
            return;
        }
        if (!(len2(sub4(rj, ri)) < radiusSqr)) {
            return;
        }
        if (a.removed[j] || a.bounces[j] > p.max_bounces) {
            return;
        }
        const Cand cd = evalPair(p, j, ri, vi, mi, wi, rj, s.v[j], s.m[j], s.omega[j], lower, size);
        if (candLess(cd, best)) {
            best = cd;
        }
    };
    // the lanes take the cells of the box (a cell holds a few particles; the latency of the cell ranges is
    // paid once per 32 cells instead of once per cell); within a cell the next particle's index and position
    // are loaded while the current one is evaluated
    const int nx = x1 - x0 + 1, ny = y1 - y0 + 1;
    const int ncell = nx * ny * (z1 - z0 + 1);
    for (int b = lane; b < ncell; b += 32) {
        const int x = x0 + b % nx;
        const int y = y0 + (b / nx) % ny;
        const int z = z0 + b / (nx * ny);
        const uint32_t cell = (uint32_t(z) * uint32_t(gi.dims[1]) + uint32_t(y)) * uint32_t(gi.dims[0]) + uint32_t(x);
        const uint32_t end = g.cell_end[cell];
        uint32_t q = g.cell_start[cell];
        uint32_t jn = 0;
        dbl4 rn = mkd4(0., 0., 0., 0.);
        if (q < end) {
            jn = g.perm[q];
            rn = s.r[jn];
        }
        while (q < end) {
            const uint32_t j = jn;
            const dbl4 rj = rn;
            if (++q < end) {
                jn = g.perm[q];
                rn = s.r[jn];
            }
            consider(j, rj);
        }
        for (int32_t e = a.extraHead[cell]; e >= 0; e = a.extra[3 * e + 1]) {
            const uint32_t j = uint32_t(a.extra[3 * e]);
            consider(j, s.r[j]);
        }
    }
    candShflMin(best);
    return best;
}

__global__ void __launch_bounds__(EV_THREADS, 1) eventKernel(DState s, Grid g, EvArgs a, CollideParams p,
    const double* __restrict__ dtp, double factor) {
    extern __shared__ __align__(16) unsigned char smem[];
    EvShared& sh = *reinterpret_cast<EvShared*>(smem);
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const GridInfo gi = *g.info;
    const double dt = factor * *dtp;
    // leader-only state
    uint32_t cursor = 0, poolNext = s.n, extraUsed = 0, removedCount = 0;
    unsigned long long nColl = 0, nMerge = 0, nBounce = 0, nOverlap = 0, nEvents = 0, err = 0;
    if (tid == 0) {
        sh.heapSize = 0;
    }
    __syncthreads();
    long long tLead = 0, tSearch = 0, tInsert = 0, t0 = clock64();
    while (true) {
        if (tid == 0) {
            sh.done = 1;
            sh.search = 0;
            // the first record in the reference's order among the pending ones (CollisionSet::top)
            while (cursor < a.nrec && !recValid(a.pool[a.order[cursor]], a.ver)) {
                ++cursor;
            }
            while (sh.heapSize > 0 && !recValid(a.pool[sh.heap[0].rec], a.ver)) {
                heapPop(sh);
            }
            int32_t id = -1;
            if (cursor < a.nrec) {
                id = int32_t(a.order[cursor]);
            }
            if (sh.heapSize > 0) {
                const HeapEnt& h = sh.heap[0];
                const CollRec& rc = a.pool[id >= 0 ? id : 0];
                if (id < 0 || recLess(h.t, h.nov, h.i, h.j, rc.t, rc.nov, rc.i, rc.j)) {
                    id = int32_t(h.rec);
                    heapPop(sh);
                } else {
                    ++cursor;
                }
            } else if (id >= 0) {
                ++cursor;
            }
            if (id >= 0 && err == 0) {
                sh.done = 0;
                ++nEvents;
                CollRec& rec = a.pool[id];
                const uint32_t i = rec.i, j = rec.j;
                const double tColl = rec.t;
                // advance the pair to the collision, resolve it, move back along the new velocities
                PairState S{ s.r[i], s.r[j], s.v[i], s.v[j], s.omega[i], s.omega[j], s.m[i], s.m[j], a.removed[j] };
                S.ri = add4(S.ri, mul4(S.vi, tColl));
                S.rj = add4(S.rj, mul4(S.vj, tColl));
                int result;
                if (rec.nov < 0.) {
                    const uint32_t before = S.removedJ;
                    overlapHandle(S, p);
                    removedCount += S.removedJ - before;
                    result = RES_BOUNCE;
                    ++nOverlap;
                } else {
                    result = collisionHandler(S, p);
                    ++nColl;
                    if (result == RES_MERGER) {
                        ++nMerge;
                        ++removedCount;
                    } else if (result == RES_BOUNCE) {
                        ++nBounce;
                    }
                }
                S.ri = sub4(S.ri, mul4(S.vi, tColl));
                S.rj = sub4(S.rj, mul4(S.vj, tColl));
                s.r[i] = S.ri;
                s.r[j] = S.rj;
                s.v[i] = S.vi;
                s.v[j] = S.vj;
                s.omega[i] = S.wi;
                s.omega[j] = S.wj;
                s.m[i] = S.mi;
                s.m[j] = S.mj;
                a.removed[j] = S.removedJ;
                if (result == RES_NONE) {
                    rec.dead = 1;
                } else {
                    // every pending record of i or j is removed; their particles are searched again
                    sh.invCount = 0;
                    invAdd(sh, i);
                    invAdd(sh, j);
                    if (!collectPartners(sh, a, i) || !collectPartners(sh, a, j)) {
                        err |= COLL_ERR_INVALID;
                    }
                    a.ver[i] += 1;
                    a.ver[j] += 1;
                    a.bounces[i] += 1;
                    a.bounces[j] += 1;
                    if (!listMoved(a, gi, S.ri, i, extraUsed) ||
                        (!S.removedJ && !listMoved(a, gi, S.rj, j, extraUsed))) {
                        err |= COLL_ERR_EXTRA;
                    }
                    sh.evI = i;
                    sh.evJ = j;
                    sh.lower = tColl + SPH_EPS;
                    sh.size = dt - sh.lower;
                    sh.search = (err == 0 && !(sh.lower > dt)) ? 1 : 0;
                }
            }
        }
        __syncthreads();
        if (tid == 0) {
            const long long t1 = clock64();
            tLead += t1 - t0;
            t0 = t1;
        }
        if (sh.done) {
            break;
        }
        if (sh.search) {
            for (uint32_t k = warp; k < sh.invCount; k += EV_WARPS) {
                const uint32_t idx = sh.inv[k];
                Cand c{ INFINITY, 0., 0u };
                if (!a.removed[idx] && a.bounces[idx] <= p.max_bounces) {
                    c = researchWarp(s, g, gi, a, p, idx, sh.lower, sh.size);
                }
                if (lane == 0) {
                    sh.res[k] = c;
                }
            }
        }
        __syncthreads();
        if (tid == 0) {
            const long long t1 = clock64();
            tSearch += t1 - t0;
            t0 = t1;
        }
        if (tid == 0 && sh.search) {
            for (uint32_t k = 0; k < sh.invCount; ++k) {
                const Cand c = sh.res[k];
                if (!(c.t < INFINITY)) {
                    continue;
                }
                const uint32_t idx = sh.inv[k];
                if ((idx == sh.evI && c.j == sh.evJ) || (c.j == sh.evI && idx == sh.evJ)) {
                    continue; // the same pair is not processed twice in a row
                }
                if (poolNext >= a.poolCapacity) {
                    err |= COLL_ERR_POOL;
                    break;
                }
                if (sh.heapSize >= HEAP_CAP) {
                    err |= COLL_ERR_HEAP;
                    break;
                }
                const uint32_t id = poolNext++;
                CollRec r;
                r.t = c.t;
                r.nov = c.nov;
                r.i = idx;
                r.j = c.j;
                r.vi = a.ver[idx];
                r.vj = a.ver[c.j];
                r.next_i = a.head[idx];
                r.next_j = a.head[c.j];
                r.dead = 0;
                r.pad = 0;
                a.pool[id] = r;
                a.head[idx] = int32_t(id);
                a.head[c.j] = int32_t(id);
                heapPush(sh, HeapEnt{ r.t, r.nov, r.i, r.j, id, 0u });
            }
        }
        __syncthreads();
        if (tid == 0) {
            const long long t1 = clock64();
            tInsert += t1 - t0;
            t0 = t1;
        }
    }
    if (tid == 0) {
        // the moved-particle lists start empty in the next call
        for (uint32_t e = 0; e < extraUsed; ++e) {
            a.extraHead[a.extra[3 * e + 2]] = -1;
        }
        a.counters[CNT_COLLISIONS] = nColl;
        a.counters[CNT_MERGERS] = nMerge;
        a.counters[CNT_BOUNCES] = nBounce;
        a.counters[CNT_OVERLAPS] = nOverlap;
        a.counters[CNT_REMOVED] = removedCount;
        a.counters[CNT_ERROR] = err;
        a.counters[CNT_EVENTS] = nEvents;
        a.counters[CNT_CYCLES_LEAD] = (unsigned long long)tLead;
        a.counters[CNT_CYCLES_SEARCH] = (unsigned long long)tSearch;
        a.counters[CNT_CYCLES_INSERT] = (unsigned long long)tInsert;
    }
}

// searchRadii (NBodySolver.cpp:355-356, 532-534): the s of the last particle whose first-pass search found this
// one, or 0
__global__ void searchRadiiKernel(uint32_t n, const int32_t* __restrict__ writer, const double* __restrict__ sr,
    double* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int32_t w = writer[i];
        out[i] = w >= 0 ? sr[w] : 0.;
    }
}

// ---- 4. Storage::remove of the merged particles, keeping the order of the others ------------------------------

__global__ void keepFlagsKernel(uint32_t n, const uint32_t* __restrict__ removed, uint32_t* keep) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        keep[i] = removed[i] ? 0u : 1u;
    }
}

__global__ void compactKernel(DState s, Collide c, const uint32_t* __restrict__ offset) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n || c.removed[i]) {
        return;
    }
    const uint32_t d = offset[i];
    c.tmp_r[d] = s.r[i];
    c.tmp_v[d] = s.v[i];
    c.tmp_dv[d] = s.dv[i];
    c.tmp_w[d] = s.omega[i];
    c.tmp_m[d] = s.m[i];
    c.tmp_origin[d] = s.origin[i];
}

__global__ void iotaKernel(uint32_t* a, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        a[i] = i;
    }
}

// ---- integrator pieces (LeapFrog::stepParticles, core/timestepping/TimeStepping.cpp:352-391) ---------------------

// drift r += v dt / 2; with the criterion: AccelerationCriterion::compute (core/timestepping/
// TimeStepCriterion.cpp:221-257), factor (h^2 / |dv|^2)^(1/4) where |dv|^2 > EPS
__global__ void driftKernel(DState s, Physics ph, const double* __restrict__ dtp, double* dtMin, int criterion) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double local = DBL_MAX;
    if (i < s.n) {
        const double dt = *dtp;
        const dbl4 v = s.v[i];
        dbl4 r = s.r[i];
        r.x += v.x * 0.5 * dt;
        r.y += v.y * 0.5 * dt;
        r.z += v.z * 0.5 * dt;
        r.w += v.w * 0.5 * dt;
        s.r[i] = r;
        if (criterion) {
            const dbl4 a = s.dv[i];
            const double a2 = len2(a);
            if (a2 > SPH_EPS) {
                local = ph.derivative_factor * sqrt(sqrt(r.w * r.w / a2));
            }
        }
    }
    if (criterion) {
        for (int off = 16; off > 0; off >>= 1) {
            local = fmin(local, __shfl_xor_sync(0xffffffffu, local, off));
        }
        if ((threadIdx.x & 31) == 0 && local < DBL_MAX) {
            atomicMinPos(dtMin, local);
        }
    }
}

// HardSphereSolver::integrate (NBodySolver.cpp:97-117): dv = a_gravity with dv.h = v.h = 0; with kick, the
// leap-frog kick v += dv dt follows
__global__ void integrateKernel(DState s, int gravity, const double* __restrict__ dtp, int kick) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) {
        return;
    }
    const dbl4 a = gravity ? s.agrav[i] : mkd4(0., 0., 0., 0.);
    const dbl4 dv = mkd4(a.x, a.y, a.z, 0.);
    s.dv[i] = dv;
    dbl4 v = s.v[i];
    v.w = 0.;
    if (kick) {
        const double dt = *dtp;
        v.x += dv.x * dt;
        v.y += dv.y * dt;
        v.z += dv.z * dt;
        v.w += dv.w * dt;
    }
    s.v[i] = v;
}

} // namespace

namespace {

__global__ void scatterValidKernel(uint32_t n, const uint32_t* __restrict__ valid, const uint32_t* __restrict__ offset,
    uint32_t* order, int* count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && valid[i]) {
        order[offset[i]] = i;
    }
    if (i == n - 1) {
        *count = int(offset[i] + valid[i]);
    }
}

} // namespace

cudaError_t collideAllocate(Collide& c, uint32_t n, uint32_t cellCapacity, uint32_t records) {
    const size_t nn = n > 0 ? n : 1;
    c.capacity = uint32_t(nn);
    c.pool_capacity = uint32_t(nn + (records > 0 ? size_t(records) : std::max<size_t>(nn, size_t(1) << 16)));
    c.extra_capacity = uint32_t(std::max<size_t>(2 * nn, size_t(1) << 16));
    cudaError_t e = cudaSuccess;
    auto A = [&](auto** p, size_t count) {
        if (e == cudaSuccess) {
            e = cudaMalloc((void**)p, count * sizeof(**p));
        }
    };
    A(&c.s, nn);
    A(&c.srad, nn);
    A(&c.nsel, 1);
    A(&c.writer, nn);
    A(&c.ver, nn);
    A(&c.bounces, nn);
    A(&c.removed, nn);
    A(&c.prev_removed, nn);
    A(&c.head, nn);
    A(&c.moved_cell, nn);
    if (e == cudaSuccess) {
        e = cudaMalloc(&c.pool, size_t(c.pool_capacity) * sizeof(CollRec));
    }
    A(&c.valid, nn);
    A(&c.order_a, nn);
    A(&c.order_b, nn);
    A(&c.key_a, nn);
    A(&c.key_b, nn);
    A(&c.extra_head, std::max<size_t>(cellCapacity, 1));
    A(&c.extra, 3 * size_t(c.extra_capacity));
    A(&c.counters, CNT_COUNT);
    A(&c.scan, nn);
    A(&c.rs, nn);
    A(&c.posf, nn);
    A(&c.sbits, nn);
    A(&c.velf, nn);
    if (e == cudaSuccess) {
        e = cudaMallocHost((void**)&c.counters_host, CNT_COUNT * sizeof(unsigned long long));
    }
    if (e != cudaSuccess) {
        return e;
    }
    size_t sortBytes = 0, scanBytes = 0;
    e = cub::DeviceRadixSort::SortPairs(nullptr, sortBytes, c.key_a, c.key_b, c.order_a, c.order_b, int(nn));
    if (e == cudaSuccess) {
        e = cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, c.valid, c.scan, int(nn));
    }
    if (e != cudaSuccess) {
        return e;
    }
    c.temp_bytes = std::max(sortBytes, scanBytes);
    e = cudaMalloc(&c.temp, c.temp_bytes > 0 ? c.temp_bytes : 16);
    if (e == cudaSuccess) {
        e = cudaMemset(c.extra_head, 0xff, std::max<size_t>(cellCapacity, 1) * sizeof(int32_t));
    }
    if (e == cudaSuccess) {
        e = cudaMemset(c.prev_removed, 0, nn * sizeof(uint32_t));
    }
    if (e == cudaSuccess) {
        e = cudaFuncSetAttribute(eventKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(EvShared)));
    }
    return e;
}

void collideFree(Collide& c) {
    void* ptrs[] = { c.s, c.srad, c.nsel, c.writer, c.ver, c.bounces, c.removed, c.prev_removed, c.head, c.moved_cell, c.pool,
        c.valid, c.order_a, c.order_b, c.key_a, c.key_b, c.extra_head, c.extra, c.counters, c.temp, c.scan, c.rs,
        c.posf, c.sbits, c.velf };
    for (void* p : ptrs) {
        if (p) {
            cudaFree(p);
        }
    }
    if (c.counters_host) {
        cudaFreeHost(c.counters_host);
    }
    c = Collide();
}

int nbodyCollide(DState& s, Grid& g, Collide& c, const CollideParams& p, const double* dt, double factor,
    uint32_t* capacityError, cudaStream_t st) {
    c.launches = 0;
    *capacityError = 0;
    const uint32_t n = s.n;
    if (p.handler == SPHGPU_COLLISION_NONE || n == 0) {
        return SPHGPU_OK; // HardSphereSolver::collide ignores all collisions without a handler
    }
    const int blocks = ceilDiv(n, 256);
    prepareKernel<<<blocks, 256, 0, st>>>(s, c, dt, factor);
    launchGridBuildRadius(s.r, c.s, n, g, st);
    gatherKernel<<<blocks, 256, 0, st>>>(s, g, c);
    detectKernel<<<ceilDiv(n, 128), 128, 0, st>>>(s, g, c, p, dt, factor);
    c.launches += 3 + g.launches;
    size_t bytes = c.temp_bytes;
    cudaError_t e = cub::DeviceScan::ExclusiveSum(c.temp, bytes, c.valid, c.scan, int(n), st);
    if (e != cudaSuccess) {
        return SPHGPU_ERR_CUDA;
    }
    scatterValidKernel<<<blocks, 256, 0, st>>>(n, c.valid, c.scan, c.order_a, c.nsel);
    c.launches += 1;
    e = cudaMemcpyAsync(c.counters_host, c.nsel, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) {
        return SPHGPU_ERR_CUDA;
    }
    const uint32_t nrec = uint32_t(*reinterpret_cast<int*>(c.counters_host));
    if (nrec == 0) {
        std::swap(c.removed, c.prev_removed); // nothing removed by this call
        return SPHGPU_OK;
    }
    // stable radix passes: (i) is the order of the scatter, then -overlap, then time
    CollRec* pool = static_cast<CollRec*>(c.pool);
    const int rb = ceilDiv(nrec, 256);
    recordKeysKernel<<<rb, 256, 0, st>>>(pool, c.order_a, nrec, 0, c.key_a);
    bytes = c.temp_bytes;
    e = cub::DeviceRadixSort::SortPairs(c.temp, bytes, c.key_a, c.key_b, c.order_a, c.order_b, int(nrec), 0, 64, st);
    recordKeysKernel<<<rb, 256, 0, st>>>(pool, c.order_b, nrec, 1, c.key_a);
    bytes = c.temp_bytes;
    if (e == cudaSuccess) {
        e = cub::DeviceRadixSort::SortPairs(c.temp, bytes, c.key_a, c.key_b, c.order_b, c.order_a, int(nrec), 0, 64,
            st);
    }
    if (e != cudaSuccess) {
        return SPHGPU_ERR_CUDA;
    }
    linkKernel<<<rb, 256, 0, st>>>(pool, c.order_a, nrec, c.head);
    searchRadiiKernel<<<blocks, 256, 0, st>>>(n, c.writer, c.s, c.srad);
    EvArgs a;
    a.pool = pool;
    a.poolCapacity = c.pool_capacity;
    a.order = c.order_a;
    a.nrec = nrec;
    a.head = c.head;
    a.ver = c.ver;
    a.bounces = c.bounces;
    a.writer = c.writer;
    a.srad = c.srad;
    a.movedCell = c.moved_cell;
    a.extraHead = c.extra_head;
    a.extra = c.extra;
    a.extraCapacity = c.extra_capacity;
    a.removed = c.removed;
    a.counters = c.counters;
    eventKernel<<<1, EV_THREADS, sizeof(EvShared), st>>>(s, g, a, p, dt, factor);
    c.launches += 5;
    e = cudaMemcpyAsync(c.counters_host, c.counters, CNT_COUNT * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
        st);
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) {
        return SPHGPU_ERR_CUDA;
    }
    const unsigned long long* cnt = c.counters_host;
    // When a work list ran out, the loop stopped after the collisions it had processed: those stay applied and
    // are counted, and the particles they merged away are removed below, so the state stays consistent (mass and
    // momentum conserved); the collisions left in the interval are not processed.
    const bool overflow = cnt[CNT_ERROR] != 0;
    if (overflow) {
        *capacityError = uint32_t(cnt[CNT_ERROR]);
    }
    for (int k = 0; k < 4; ++k) {
        c.totals[k] += cnt[k];
    }
    c.profile[0] += cnt[CNT_EVENTS];
    c.profile[1] += cnt[CNT_CYCLES_LEAD];
    c.profile[2] += cnt[CNT_CYCLES_SEARCH];
    c.profile[3] += cnt[CNT_CYCLES_INSERT];
    const uint32_t removed = uint32_t(cnt[CNT_REMOVED]);
    if (removed > 0) {
        keepFlagsKernel<<<blocks, 256, 0, st>>>(n, c.removed, c.valid);
        bytes = c.temp_bytes;
        e = cub::DeviceScan::ExclusiveSum(c.temp, bytes, c.valid, c.scan, int(n), st);
        if (e != cudaSuccess) {
            return SPHGPU_ERR_CUDA;
        }
        compactKernel<<<blocks, 256, 0, st>>>(s, c, c.scan);
        c.launches += 2;
        std::swap(s.r, c.tmp_r);
        std::swap(s.v, c.tmp_v);
        std::swap(s.dv, c.tmp_dv);
        std::swap(s.omega, c.tmp_w);
        std::swap(s.m, c.tmp_m);
        std::swap(s.origin, c.tmp_origin);
        s.n = n - removed;
    }
    std::swap(c.removed, c.prev_removed);
    return overflow ? SPHGPU_ERR_CAPACITY : SPHGPU_OK;
}

void launchIota(uint32_t* a, uint32_t n, cudaStream_t st) {
    if (n) {
        iotaKernel<<<ceilDiv(n, 256), 256, 0, st>>>(a, n);
    }
}

void launchNbodyDrift(const DState& s, const Physics& ph, const double* dt, double* dtMin, bool criterion,
    cudaStream_t st) {
    if (s.n) {
        driftKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, ph, dt, dtMin, criterion ? 1 : 0);
    }
}

void launchNbodyIntegrate(const DState& s, bool gravity, const double* dt, bool kick, cudaStream_t st) {
    if (s.n) {
        integrateKernel<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, gravity ? 1 : 0, dt, kick ? 1 : 0);
    }
}

} // namespace sphgpu
