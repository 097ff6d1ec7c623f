// state.h — device state of one sphgpu handle and the launchers of each translation unit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "common.cuh"

namespace sphgpu {

// Particle state in HBM, in the reference's storage order. Vector quantities keep the reference layout
// {x, y, z, h} (one 32-byte dbl4 per particle); tensors are stored component-major (SoA, component c
// of particle i at [c * n + i]) so that a thread-per-particle kernel reads them coalesced.
struct DState {
    uint32_t n;
    dbl4* r;
    dbl4* v;
    dbl4* dv;
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
    double* S;      // 5 x n: xx, yy, xy, xz, yz
    double* dS;     // 5 x n
    double* gradv;  // 6 x n: xx, yy, zz, xy, xz, yz
    double* reduce;
    double* D;
    double* dD;
    double* eps_min;
    double* m_zero;
    double* growth;
    uint32_t* n_flaws;
    // derivatives saved by the predictor (PredictorCorrector::predictions)
    dbl4* pdv;
    double* pdrho;
    double* pdu;
    double* pdS;
    double* pdD;
    // self-gravity acceleration of the current evaluation
    dbl4* agrav;
    // strain-rate correction tensor (6 x n: xx, yy, zz, xy, xz, yz), with the correction tensor only
    double* corr;
    // N-body solver: angular frequency {x, y, z, 0} (QuantityId::ANGULAR_FREQUENCY)
    dbl4* omega;
    // N-body solver: index of each particle at the last sphgpu_take_removed / position upload
    uint32_t* origin;
};

// Physics switches and constants of one handle
struct Physics {
    int solid;           // SOLID_STRESS with a stress tensor
    int damage;          // any material with a fracture model
    int gravity;
    int adaptive_h;
    int sum_only_undamaged;
    int integrator;
    int precision;
    int multipole_order;
    int kernel_radius;   // 0: point masses, 2: gravity kernel of the cubic spline
    uint32_t leaf_size;
    uint32_t nmat;
    double h_lo, h_hi;
    double av_alpha, av_beta;
    double G;
    double theta_inv;
    double courant;
    double max_dt;
    uint32_t criteria;        // SPHGPU_CRITERION_* bits
    double derivative_factor; // derivative and acceleration criteria
    double divergence_factor;
    double max_change;        // relative growth limit of the step (off when >= DBL_MAX)
    int correction;           // strain-rate correction tensor applied to the velocity gradient
    int nbody;                // HardSphereSolver instead of the SPH solver
};

// HardSphereSolver collision settings (core/gravity/NBodySolver.cpp:29-44, core/gravity/Collision.h)
struct CollideParams {
    int handler;              // SPHGPU_COLLISION_*
    int overlap;              // SPHGPU_OVERLAP_*
    double rest_n, rest_t;    // coefficients of restitution
    double allowed;           // allowed overlap ratio
    double bounce_limit;      // merge limit on the relative speed (in escape speeds squared)
    double rotation_limit;    // merge limit on the spin of the merger
    uint32_t max_bounces;
    uint32_t pad;
};

// Device work space of HardSphereSolver::collide (nbody.cu)
struct Collide {
    uint32_t capacity = 0;       // particles
    uint32_t pool_capacity = 0;  // collision records: one per particle for the first pass + later ones
    uint32_t extra_capacity = 0; // entries of the moved-particle cell lists
    double* s = nullptr;         // search radius h + |v| dt
    double* srad = nullptr;      // searchRadii of the reference: s of the writer, 0 without one
    int* nsel = nullptr;         // device: first-pass record count
    int32_t* writer = nullptr;   // highest index of the particles whose first-pass search found this one
    uint32_t* ver = nullptr;     // per particle: number of processed collisions that involved it
    uint32_t* bounces = nullptr;
    uint32_t* removed = nullptr;
    uint32_t* prev_removed = nullptr; // flags of the indices removed by the previous call
    int32_t* head = nullptr;     // per particle: newest record that involves it
    int32_t* moved_cell = nullptr; // per particle: cell it is listed in last
    void* pool = nullptr;        // collision records
    uint32_t* valid = nullptr;   // first-pass record flags
    uint32_t* order_a = nullptr;
    uint32_t* order_b = nullptr;
    unsigned long long* key_a = nullptr;
    unsigned long long* key_b = nullptr;
    int32_t* extra_head = nullptr; // per grid cell
    int32_t* extra = nullptr;      // 3 ints per entry: particle, next, cell
    unsigned long long* counters = nullptr; // device, see nbody.cu
    unsigned long long* counters_host = nullptr; // pinned mirror
    void* temp = nullptr;
    size_t temp_bytes = 0;
    uint32_t* scan = nullptr;    // compaction offsets
    dbl4* rs = nullptr;          // cell-sorted positions (first pass)
    float4* posf = nullptr;      // cell-sorted FP32 positions relative to the cell origin, 2 s
    unsigned long long* sbits = nullptr; // cell-sorted bit patterns of s
    float4* velf = nullptr;      // cell-sorted FP32 velocity and radius h
    // compaction targets, swapped with the state arrays (allocated and freed with the state arrays)
    dbl4* tmp_r = nullptr;
    dbl4* tmp_v = nullptr;
    dbl4* tmp_dv = nullptr;
    dbl4* tmp_w = nullptr;
    double* tmp_m = nullptr;
    uint32_t* tmp_origin = nullptr;
    uint32_t launches = 0;
    unsigned long long totals[4] = { 0, 0, 0, 0 }; // collisions, mergers, bounces, overlaps (host copy)
    // records processed by the event loop and its SM cycles in the serial part, the re-searches, the insertions
    unsigned long long profile[4] = { 0, 0, 0, 0 };
};

// Neighbour grid buffers (cell-sorted copies of the pair-loop inputs)
// neighbour-list slots per particle of the mixed pair loop (a particle with more evaluates the rest by a second
// scan of its cells), and the particle count up to which the lists' 27-bit indices reach
constexpr int NB_CAP = 128;
constexpr uint32_t NB_MAX_PARTICLES = 1u << 27;

struct Grid {
    uint32_t cell_capacity = 0;
    GridInfo* info = nullptr;          // device
    unsigned long long* bounds = nullptr; // device: flipped min x,y,z, max x,y,z, max h
    uint32_t* keys = nullptr;
    uint32_t* keys_sorted = nullptr;
    uint32_t* perm_in = nullptr;
    uint32_t* perm = nullptr;          // sorted position -> particle index
    uint32_t* cell_start = nullptr;
    uint32_t* cell_end = nullptr;
    void* sort_temp = nullptr;
    size_t sort_temp_bytes = 0;
    // cell-sorted copies
    dbl4* rs = nullptr;
    dbl4* vs = nullptr;
    double* ms = nullptr;
    double* rhos = nullptr;
    double* ps = nullptr;
    double* css = nullptr;
    double* Ss = nullptr;      // 5 x n
    double* reduces = nullptr;
    uint32_t* flags = nullptr;
    // mixed-precision copies (cell-sorted): positions relative to the particle's own cell origin, velocities
    // as unevaluated float pairs (hi + lo) so that neighbour differences keep FP64-level accuracy
    float4* mx0 = nullptr;     // x - cell_x, y - cell_y, z - cell_z, h
    float4* mx1 = nullptr;     // vx_hi, vy_hi, vz_hi, m
    float4* mx2 = nullptr;     // vx_lo, vy_lo, vz_lo, rho
    float4* mx3 = nullptr;     // p / rho^2, cs, stress reducing, flag (bit pattern)
    float* mxS = nullptr;      // 5 x n: S / rho^2
    float* mxC = nullptr;      // 6 x n: correction tensor (mixed path, cell-sorted)
    // mixed pair loop: the interacting neighbours of each particle (NB_CAP x n, [slot][particle], sorted index |
    // cell offset << 27) and their number (which may exceed NB_CAP)
    uint32_t* nb = nullptr;
    uint32_t* nb_count = nullptr;
    uint32_t* nb_over = nullptr;       // particles (sorted positions) with more than NB_CAP neighbours
    uint32_t* nb_over_count = nullptr; // device: their number
    uint32_t* cell_first = nullptr;    // fine grids: first sorted position of each cell key (cell_capacity + 1)
    uint32_t launches = 0;     // own kernels launched by the last build / gather (library sort excluded)
};

// Barnes-Hut tree buffers
struct BhNodeGeom {
    double lo[3];
    double hi[3];
    double com[3];
    double r_open;
    int32_t left, right;    // children (-1 for leaves)
    uint32_t from, to;      // particle range in the index permutation (leaves)
    int32_t parent;
    int32_t level;
};

struct BhNodeMoments {
    double m0;
    double q2[6];  // xx xy xz yy yz zz
    double q3[10]; // xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz
    double pad;
};

struct BhSegment {
    uint32_t from, to;
    int32_t node;
    uint32_t sliding;
    double lo[3], hi[3];
};

// k-d tree build: deepest level of a node (the level lists of the mixed walk), and the device counters of the
// build (Tree::counters)
constexpr uint32_t TREE_MAX_LEVELS = 512;
enum : int {
    C_NODES = 0,
    C_LEAVES = 1,
    C_QUEUE = 2,     // segments in the queue of the per-warp subtree splits
    C_TAKEN = 3,     // queue entries taken
    C_R1_LEVELS = 4, // levels of the multi-CTA phase that had segments
    C_DEPTH = 5,     // deepest node level + 1
    C_SEGS = 6,      // [6], [7]: multi-CTA segment counts of two consecutive levels (by parity)
    C_CHUNKS = 8,    // [8], [9]: chunk counts of two consecutive levels (by parity)
    C_WORDS = 16
};

struct BhChunk {
    uint32_t seg;    // segment index in the level's list
    uint32_t index;  // chunk index within the segment
    uint32_t first;  // slot of the segment's first chunk
    uint32_t count;  // chunks of the segment
};

struct BhChunkStats {
    uint32_t nb[3], ns[3];  // elements above / below the box centre, per dimension
    uint32_t diff[3];       // any element differs from the segment's last one, per dimension
    uint32_t pad;
    unsigned long long minv[3], maxv[3]; // orderKey of the extremes
    uint32_t minp[3], maxp[3]; // first positions of the extremes
};

struct BhSegWork {
    int32_t splitIdx;
    int32_t mode;      // 0 two-pointer partition, 1 nth_element, 2 degenerate box
    uint32_t nB, nS, K;
    uint32_t minp, maxp;
    uint32_t pad;
    unsigned long long minv, maxv; // orderKey of the extremes
};

// One particle of the k-d tree build: the order keys of its coordinates and its index, one 32-byte sector, so
// that a swap of the partition moves one sector per side
struct alignas(32) TreeElem {
    unsigned long long key[3];
    uint32_t idx;
    uint32_t pad;
};

struct Tree {
    uint32_t node_capacity = 0;
    uint32_t seg_capacity = 0;
    uint32_t* idx = nullptr;          // permutation of particles (KdTree::idxs)
    TreeElem* elems = nullptr;        // build: order keys of x, y, z and the particle index, in tree order
    unsigned long long* subtree_keys = nullptr; // build: keys (3 x n) of segments split by one warp in global memory
    uint32_t* scratch_b = nullptr;    // positions of elements above the split (per segment)
    uint32_t* scratch_s = nullptr;    // positions of elements below the split
    BhNodeGeom* geom = nullptr;
    BhNodeMoments* mom = nullptr;
    BhSegment* seg[2] = { nullptr, nullptr }; // multi-CTA phase: segments of two consecutive levels
    BhSegment* queue = nullptr;       // segments split to their leaves by one warp each
    uint32_t* counters = nullptr;     // device: C_NODES ...
    uint32_t* info_host = nullptr;    // pinned: the counters and the level counts after a build
    uint32_t* level_count = nullptr;  // device: nodes per level
    uint32_t* level_first_dev = nullptr; // device: first entry of each level in level_nodes
    uint32_t* level_cursor = nullptr; // device: scatter cursors
    uint32_t* level_nodes = nullptr;  // device: node ids ordered by level
    std::vector<uint32_t> level_first; // host: first entry of each level in level_nodes (+ the total)
    uint32_t r1_levels = 0;           // multi-CTA levels the last build used
    uint32_t* leaves = nullptr;       // leaf node ids
    uint32_t* visits = nullptr;       // per node: children finished (bottom-up moments)
    int32_t* walk_scratch = nullptr;  // per-warp checklists
    // mixed walk in two phases: the interaction lists of every node, built once per node level by level, and
    // the per-leaf evaluation over the lists of the leaf's ancestors
    int32_t* nl_pool = nullptr;       // node (N) and particle-list (P) entries of all nodes
    uint32_t nl_capacity = 0;
    int32_t* nl_kept[2] = { nullptr, nullptr }; // kept (undecided) lists of two consecutive levels
    uint32_t nl_kept_capacity = 0;
    uint32_t* nl_meta = nullptr;      // per node: N offset, N length, P offset, P length, kept offset, kept length
    uint32_t* nl_counters = nullptr;  // device: [0] pool entries reserved, [1], [2] kept entries reserved (by level
                                      // parity), [3] end of the kept entries, [5] a node's lists outgrew the
                                      // staging, [6], [7] deferred nodes (by level parity)
    uint32_t* nl_host = nullptr;      // pinned mirror of nl_counters
    uint32_t* nl_defer = nullptr;     // nodes of a level whose lists outgrew the first pass's staging
    uint32_t walk_launches = 0;       // kernels launched by the last mixed walk
    uint32_t walk_warps = 0;
    uint32_t walk_capacity = 0;       // entries per list per warp
    uint32_t walk_defer_factor = 4;   // staging of a deferred node: the scratch of this many warps
    unsigned long long* stats = nullptr; // device: approx, exact
    unsigned long long* bbox = nullptr;  // device: flipped bounding box of the root
    float* nodef = nullptr;           // mixed walk: FP32 evaluation record per node (28 floats)
    float4* pf = nullptr;             // mixed walk: particle position relative to its leaf's centre of mass, h
    float* mf = nullptr;              // mixed walk: G * m in tree order
    dbl4* slice_part = nullptr;       // FP64 walk of few leaves: partial sums per slice (slices x n, tree order)
    size_t slice_capacity = 0;
    uint32_t chunk_capacity = 0;
    BhChunk* chunks = nullptr;
    BhChunkStats* chunk_stats = nullptr;
    uint32_t* chunk_off_b = nullptr;
    uint32_t* chunk_off_s = nullptr;
    uint32_t* chunk_done = nullptr;   // per segment's first chunk: chunks finished in the two passes of a level
    BhSegWork* work = nullptr;
    uint32_t node_count = 0;
    uint32_t leaf_count = 0;
    uint32_t launches = 0;            // kernels launched by the last build
    bool built = false;
    bool mixed_moments = false;       // reduced moments only in FP32 (node records), not in mom
};

// ---- launchers (grid.cu) ----
// fine: cells of h_max for the mixed pair loop (needs the grid's cell_first array)
void launchGridBuild(const DState& s, Grid& g, const Physics& ph, cudaStream_t st, bool fine = false);
void launchGatherSorted(const DState& s, Grid& g, const Physics& ph, cudaStream_t st);
// copies: the cell-sorted copies of the SPH pair loops (not needed by the collision search)
cudaError_t gridAllocate(Grid& g, uint32_t n, bool solid, bool correction = false, bool copies = true,
    bool neighbourLists = false);
void gridFree(Grid& g);
void launchCountPairs(const DState& s, const Grid& g, unsigned long long* count, cudaStream_t st);
// the directed pairs (i, j), j != i, |r_j - r_i| < 2 h_i (pi NULL: count only)
void launchRadiusPairs(const DState& s, const Grid& g, uint32_t* pi, uint32_t* pj, unsigned long long* count,
    unsigned long long capacity, cudaStream_t st);
// particles within radius of pos on the grid of the last build (unordered; count may exceed capacity)
void launchFindBall(const Grid& g, uint32_t n, const dbl4& pos, double radius, uint32_t* idx, double* d2,
    unsigned long long* count, unsigned long long capacity, cudaStream_t st);
void launchListPairs(const DState& s, const Grid& g, uint32_t* pi, uint32_t* pj, unsigned long long* count,
    unsigned long long capacity, cudaStream_t st);

// grid over the positions r: radius NULL -> cell edge >= 2 max h (27-cell stencil of the pair loops), or max h
// with fine (the mixed pair loop); else the collision grid, cell edge 2 max(mean radius, max radius / 8),
// searched over each particle's own cell box
void launchGridBuildRadius(const dbl4* r, const double* radius, uint32_t n, Grid& g, cudaStream_t st,
    bool fine = false);

// ---- launchers (sph64.cu) ----
void launchMaterialsInit(const DState& s, const Physics& ph, const MaterialD* mats, cudaStream_t st);
// the smoothing-length clamp of adaptive h alone; returns whether a kernel was launched
bool launchClampH(const DState& s, const Physics& ph, cudaStream_t st);
void launchPairSum64(const DState& s, const Grid& g, const Physics& ph, const MaterialD* mats,
    const double* lut_grad, cudaStream_t st);
void launchPredict(const DState& s, const Physics& ph, const MaterialD* mats, const double* dt, cudaStream_t st);
void launchCorrect(const DState& s, const Physics& ph, const MaterialD* mats, const double* dt, double* dt_min,
    cudaStream_t st);
void launchLeapFrogDriftInit(const DState& s, const Physics& ph, const MaterialD* mats, const double* dt,
    cudaStream_t st);
void launchLeapFrogKick(const DState& s, const Physics& ph, const MaterialD* mats, const double* dt,
    double* dt_min, cudaStream_t st);
// end of a step: time += dt; with criterion, dt = the criteria minimum capped by max_dt and max_change
void launchStepEnd(double* dt, double* dt_min, double max_dt, double max_change, double* time, bool criterion,
    cudaStream_t st);
void launchTotals(const DState& s, double omega, double* partial, double* out, cudaStream_t st);
void launchCheckFinite(const DState& s, unsigned long long* first_bad, cudaStream_t st);
void launchAddGravity(const DState& s, cudaStream_t st);
void launchPairSumMixed(const DState& s, const Grid& g, const Physics& ph, const MaterialD* mats,
    const float* lut_grad_f, cudaStream_t st);
// CorrectionTensor (core/sph/equations/Derivative.cpp:36-74) of every particle, before the pair loop
void launchCorrection64(const DState& s, const Grid& g, const Physics& ph, const double* lut_grad, cudaStream_t st);
void launchCorrectionMixed(const DState& s, const Grid& g, const Physics& ph, const float* lut_grad_f,
    cudaStream_t st);

// ---- launchers (gravity.cu) ----
cudaError_t treeAllocate(Tree& t, uint32_t n, uint32_t leaf_size);
void treeFree(Tree& t);
// reallocates the per-warp check lists of the walks with `capacity` entries per list (no-op when not larger)
cudaError_t treeGrowWalkScratch(Tree& t, uint32_t capacity);
cudaError_t treeBuild(const DState& s, Tree& t, const Physics& ph, uint32_t* dev_error, cudaStream_t st);
// (treebuild.cu) the build's own buffers, and the chunk capacity of the multi-CTA phase for n particles
cudaError_t treeBuildAllocate(Tree& t, uint32_t n);
void treeBuildFree(Tree& t);
uint32_t treeChunkCapacity(uint32_t n);
// (gravity.cu, gravity32.cu) moments and FP32 node records of a tree whose node and leaf counts are on the device
void launchMomentsDev(const DState& s, Tree& t, const Physics& ph, bool mixed, cudaStream_t st);
void launchPrepareWalkDev(const DState& s, Tree& t, const Physics& ph, cudaStream_t st);
// forms the FP64 moments of a tree built with FP32 moments (for the FP64 point evaluation)
void treeEnsureFp64Moments(const DState& s, Tree& t, const Physics& ph, cudaStream_t st);
// evalStart / evalEnd (or null): events recorded around the walk's evaluation kernel
void launchGravityWalk(const DState& s, Tree& t, const Physics& ph, const double* lut_grad, uint32_t* dev_error,
    cudaStream_t st, cudaEvent_t evalStart = nullptr, cudaEvent_t evalEnd = nullptr);
// (gravity32.cu) walk phase 1, shared by both walks: the interaction lists of every node, level by level
void launchWalkLists(const DState& s, Tree& t, uint32_t* dev_error, cudaStream_t st);
void launchGravityWalkMixed(const DState& s, Tree& t, const Physics& ph, const float* lut_grad_f,
    uint32_t* dev_error, cudaStream_t st, cudaEvent_t evalStart = nullptr, cudaEvent_t evalEnd = nullptr);
// BarnesHut::evalAttractors on the device: att (5 doubles per attractor), dv (particles, in/out), acc (3 doubles per
// attractor, in/out), partial (gravityAttractorPartials(n, count) doubles of scratch)
void launchGravityAttractors(const DState& s, const Physics& ph, const double* lut, const double* att, uint32_t count,
    dbl4* dv, double* partial, double* acc, cudaStream_t st);
uint32_t gravityAttractorPartials(uint32_t n, uint32_t count);
// BruteForceGravity for the listed particles (device arrays), FP64
void launchGravityDirect(const DState& s, const Physics& ph, const double* lut, const uint32_t* targets, uint32_t nt,
    dbl4* acc, cudaStream_t st);
void launchGravityPoints(const DState& s, const Tree& t, const Physics& ph, const double* lut_grad,
    const dbl4* points, dbl4* acc, uint32_t npoints, cudaStream_t st);

// ---- HardSphereSolver (nbody.cu) ----
// records: collision records beyond one per particle (0 = max(n, 65,536))
cudaError_t collideAllocate(Collide& c, uint32_t n, uint32_t cell_capacity, uint32_t records);
void collideFree(Collide& c);
// HardSphereSolver::collide over [0, factor * (*dt)); compacts the state when particles merged (s.n shrinks).
// Synchronises the stream. Returns SPHGPU_OK or an error status (capacity bits in *capacity_error).
int nbodyCollide(DState& s, Grid& g, Collide& c, const CollideParams& p, const double* dt, double factor,
    uint32_t* capacity_error, cudaStream_t st);
// a[i] = i for i < n
void launchIota(uint32_t* a, uint32_t n, cudaStream_t st);
// leap-frog drift r += v dt / 2; with criteria, the acceleration time-step minimum into dt_min
void launchNbodyDrift(const DState& s, const Physics& ph, const double* dt, double* dt_min, bool criterion,
    cudaStream_t st);
// HardSphereSolver::integrate: dv = a_gravity (0 without gravity), v.h = dv.h = 0; with kick, then v += dv dt
void launchNbodyIntegrate(const DState& s, bool gravity, const double* dt, bool kick, cudaStream_t st);

// ---- adjoint of the frozen-list hydrodynamic step (adjoint.cu) ----
struct AdjointState;
cudaError_t adjointConfigure(AdjointState*& a, uint32_t n, const sphgpu_adjoint_config& cfg);
void adjointFree(AdjointState* a);
cudaError_t adjointForward(AdjointState* a, const DState& s, Grid& grid, const Physics& ph, const double* lut,
    const float* lutf, double* loss, cudaStream_t st);
cudaError_t adjointBackward(AdjointState* a, const DState& s, Grid& grid, const Physics& ph, const double* lut,
    const float* lutf, double lossBar, double* alphaBar, cudaStream_t st);
cudaError_t adjointGradients(AdjointState* a, double* gr, double* gv, double* grho, double* gu, cudaStream_t st);
bool adjointForwardDone(const AdjointState* a);
bool adjointBackwardDone(const AdjointState* a);
uint64_t adjointListEntries(const AdjointState* a);
unsigned long long adjointTakeLaunches(AdjointState* a);

} // namespace sphgpu
