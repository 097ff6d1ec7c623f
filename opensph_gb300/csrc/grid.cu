// grid.cu — neighbour search: cell-sorted uniform grid (replaces ISymmetricFinder / KdTree::findLowerRank,
// core/objects/finders/KdTree.inl.h:316-391, NeighborFinder.cpp:11-25).
//
// Each step: device reduction of the bounding box and max h -> grid of cells of edge >= 2 h_max (the
// kernel support; h_max for the mixed pair loop's fine grid) -> cell key per particle -> radix sort of (key,
// index) -> per-cell [start, end) ranges (and, for the fine grid, the first position of every cell key) ->
// cell-sorted copies of the pair-loop inputs. The pair loops then scan the 27 cells around each particle (the
// cells within two of it on the fine grid).
// The interacting pair set is decided by the exact FP64 test of SymmetricSolver::loop
// (core/sph/solvers/SymmetricSolver.cpp:126-130): |r_i - r_j|^2 < (2 * 0.5 (h_i + h_j))^2, evaluated
// with round-to-nearest multiplies and adds (no FMA), i.e. bit-identically to the reference.

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>

#include "state.h"

namespace sphgpu {

namespace {

__global__ void resetBounds(unsigned long long* b) {
    if (threadIdx.x < 3) {
        b[threadIdx.x] = ~0ull;     // min slots (flipped order)
        b[3 + threadIdx.x] = 0ull;  // max slots
    }
    if (threadIdx.x == 6) {
        b[6] = 0ull;                // max h
    }
    if (threadIdx.x == 7) {
        b[7] = 0ull;                // sum of the radii (a double), for the mean-based cell of the collision grid
    }
}

// bounding box of the positions and the maximum of h (rad == nullptr) or of rad
__global__ void boundsKernel(const dbl4* __restrict__ r, const double* __restrict__ rad, uint32_t n,
    unsigned long long* b) {
    unsigned long long mn[3] = { ~0ull, ~0ull, ~0ull }, mx[3] = { 0, 0, 0 }, hm = 0;
    double sum = 0.;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dbl4 p = r[i];
        const unsigned long long fx = doubleFlip(p.x), fy = doubleFlip(p.y), fz = doubleFlip(p.z);
        mn[0] = min(mn[0], fx);
        mn[1] = min(mn[1], fy);
        mn[2] = min(mn[2], fz);
        mx[0] = max(mx[0], fx);
        mx[1] = max(mx[1], fy);
        mx[2] = max(mx[2], fz);
        hm = max(hm, doubleFlip(rad ? rad[i] : p.w));
        sum += rad ? rad[i] : 0.;
    }
    for (int off = 16; off > 0; off >>= 1) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
            mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
        }
        hm = max(hm, __shfl_xor_sync(0xffffffffu, hm, off));
        sum += __shfl_xor_sync(0xffffffffu, sum, off);
    }
    // the warps' values combined in the block, one atomic per block and word (a few hundred blocks: the atomics
    // on these words were the kernel's time with one per warp)
    __shared__ unsigned long long sMn[32][3], sMx[32][3], sHm[32];
    __shared__ double sSum[32];
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            sMn[w][k] = mn[k];
            sMx[w][k] = mx[k];
        }
        sHm[w] = hm;
        sSum[w] = sum;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        unsigned long long a = sMn[0][k], c = sMx[0][k];
        for (int q = 1; q < nw; ++q) {
            a = min(a, sMn[q][k]);
            c = max(c, sMx[q][k]);
        }
        atomicMin(&b[k], a);
        atomicMax(&b[3 + k], c);
    } else if (threadIdx.x == 3) {
        unsigned long long a = sHm[0];
        double t = sSum[0];
        for (int q = 1; q < nw; ++q) {
            a = max(a, sHm[q]);
            t += sSum[q];
        }
        atomicMax(&b[6], a);
        if (rad) {
            atomicAdd(reinterpret_cast<double*>(&b[7]), t);
        }
    }
}

// meanCell: cell edge 2 max(mean radius, max radius / 8) (the collision search scans the cells of each
// particle's own search box); fine: cell edge h_max (the 5 x 5 x 5 stencil of the mixed pair loop, coarse cells of
// 2 x 2 x 2 fine cells); else 2 h_max (the 27-cell stencil of the SPH pair loops)
__global__ void gridSetupKernel(const unsigned long long* b, uint32_t capacity, uint32_t n, int meanCell, int fine,
    GridInfo* g) {
    if (threadIdx.x != 0 || blockIdx.x != 0) {
        return;
    }
    double lo[3], ext[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = n ? doubleUnflip(b[k]) : 0.;
        const double hi = n ? doubleUnflip(b[3 + k]) : 0.;
        ext[k] = hi - lo[k];
    }
    const double hmax = n ? doubleUnflip(b[6]) : 0.;
    // cell edge: kernel support 2 h_max, widened by 1e-4 so that rounding in the cell index can never
    // separate two interacting particles by more than one cell
    const double support = 2. * hmax * 1.0001;
    double cell = fine ? 0.5 * support : support;
    if (meanCell && n) {
        const double mean = __longlong_as_double(static_cast<long long>(b[7])) / double(n);
        cell = 2. * fmax(mean, 0.125 * hmax) * 1.0001;
    }
    const double extMax = fmax(fmax(ext[0], ext[1]), ext[2]);
    if (!(cell > 0.)) {
        cell = extMax > 0. ? extMax : 1.;
    }
    int dims[3];
    for (int it = 0; it < 64; ++it) {
        unsigned long long total = 1;
        for (int k = 0; k < 3; ++k) {
            const double d = floor(ext[k] / cell) + 1.;
            dims[k] = d > 1.e6 ? 1000000 : int(d);
            total *= (unsigned long long)dims[k];
        }
        if (total <= capacity) {
            break;
        }
        cell *= 1.25;
    }
    for (int k = 0; k < 3; ++k) {
        g->lo[k] = lo[k];
        g->dims[k] = dims[k];
        g->lo_f[k] = float(lo[k]);
    }
    g->cell = cell;
    g->inv_cell = 1. / cell;
    g->hmax = hmax;
    // a fine grid that had to be coarsened to fit the cell capacity to 2 h_max or more is an ordinary grid
    const bool isFine = fine && !meanCell && cell < support;
    g->span = isFine ? 2 : 1;
    g->shift = isFine ? 1 : 0;
    g->ccell = isFine ? 2. * cell : cell;
    g->ncells = uint32_t(dims[0]) * uint32_t(dims[1]) * uint32_t(dims[2]);
}

__device__ __forceinline__ int cellCoord(double x, double lo, double inv, int dim) {
    int c = int((x - lo) * inv);
    return min(max(c, 0), dim - 1);
}

__global__ void keysKernel(const dbl4* __restrict__ r, uint32_t n, const GridInfo* __restrict__ g,
    uint32_t* __restrict__ keys, uint32_t* __restrict__ perm) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const dbl4 p = r[i];
    const double inv = g->inv_cell;
    const int cx = cellCoord(p.x, g->lo[0], inv, g->dims[0]);
    const int cy = cellCoord(p.y, g->lo[1], inv, g->dims[1]);
    const int cz = cellCoord(p.z, g->lo[2], inv, g->dims[2]);
    keys[i] = (uint32_t(cz) * uint32_t(g->dims[1]) + uint32_t(cy)) * uint32_t(g->dims[0]) + uint32_t(cx);
    perm[i] = i;
}

__global__ void clearCells(uint32_t* start, uint32_t* end, const GridInfo* __restrict__ g) {
    const uint32_t nc = g->ncells;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        start[c] = 0;
        end[c] = 0;
    }
}

__global__ void cellRanges(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* start, uint32_t* end) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) {
        return;
    }
    const uint32_t k = keys[s];
    if (s == 0 || keys[s - 1] != k) {
        start[k] = s;
    }
    if (s == n - 1 || keys[s + 1] != k) {
        end[k] = s + 1;
    }
}

// first[c] = the first sorted position whose cell key is at least c, for c = 0 .. ncells (first[ncells] = n): the
// particles of the consecutive cells c0 .. c1 are the positions first[c0] .. first[c1 + 1]
__global__ void cellFirstKernel(const uint32_t* __restrict__ keys, uint32_t n, const GridInfo* __restrict__ g,
    uint32_t capacity, uint32_t* first) {
    const uint32_t nc = min(g->ncells, capacity);
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c <= nc; c += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (keys[mid] < c) {
                lo = mid + 1;
            } else {
                hi = mid;
            }
        }
        first[c] = lo;
    }
}

__global__ void gatherSorted(DState st, const uint32_t* __restrict__ perm, dbl4* rs, dbl4* vs, double* ms,
    double* rhos, double* ps, double* css, double* Ss, double* reduces, uint32_t* flags, int solid) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = st.n;
    if (s >= n) {
        return;
    }
    const uint32_t i = perm[s];
    rs[s] = st.r[i];
    vs[s] = st.v[i];
    ms[s] = st.m[i];
    rhos[s] = st.rho[i];
    ps[s] = st.p[i];
    css[s] = st.cs[i];
    if (solid) {
        for (int c = 0; c < 5; ++c) {
            Ss[c * n + s] = st.S[c * n + i];
        }
        reduces[s] = st.reduce[i];
        flags[s] = st.flag[i];
    }
}

__device__ __forceinline__ void splitFloat(double x, float& hi, float& lo) {
    hi = float(x);
    lo = float(x - double(hi));
}

// mixed-precision packing of the pair-loop inputs (cell-relative FP32 positions, hi/lo FP32 velocities)
__global__ void gatherSortedMixed(DState st, const uint32_t* __restrict__ perm, const uint32_t* __restrict__ keys,
    const GridInfo* __restrict__ g, float4* mx0, float4* mx1, float4* mx2, float4* mx3, float* mxS, int solid) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = st.n;
    if (s >= n) {
        return;
    }
    const uint32_t i = perm[s];
    const uint32_t key = keys[s];
    const uint32_t dx = uint32_t(g->dims[0]), dy = uint32_t(g->dims[1]);
    const int sh = g->shift;
    // the origin of the particle's coarse cell
    const double cx = double((key % dx) >> sh), cy = double(((key / dx) % dy) >> sh),
                 cz = double((key / (dx * dy)) >> sh);
    const dbl4 p = st.r[i];
    const dbl4 v = st.v[i];
    const double rho = st.rho[i];
    mx0[s] = make_float4(float(p.x - (g->lo[0] + cx * g->ccell)), float(p.y - (g->lo[1] + cy * g->ccell)),
        float(p.z - (g->lo[2] + cz * g->ccell)), float(p.w));
    float hx, lx, hy, ly, hz, lz;
    splitFloat(v.x, hx, lx);
    splitFloat(v.y, hy, ly);
    splitFloat(v.z, hz, lz);
    mx1[s] = make_float4(hx, hy, hz, float(st.m[i]));
    mx2[s] = make_float4(lx, ly, lz, float(rho));
    // (the FP32 records take S / rho^2 and p / rho^2 from one FP64 reciprocal: the FP64 pipe runs at 1/64 of the
    // FP32 rate on this part; the products round to the quotients' floats or to a neighbouring one)
    const double invRho2 = 1. / (rho * rho);
    float red = 0.f, flg = 0.f;
    if (solid) {
        red = float(st.reduce[i]);
        flg = __uint_as_float(st.flag[i]);
        for (int c = 0; c < 5; ++c) {
            mxS[c * n + s] = float(st.S[c * n + i] * invRho2);
        }
    }
    mx3[s] = make_float4(float(st.p[i] * invRho2), float(st.cs[i]), red, flg);
}

// exact FP64 interaction test of SymmetricSolver::loop, no FMA contraction
__device__ __forceinline__ bool interacts(const dbl4& a, const dbl4& b) {
    const double dx = __dsub_rn(a.x, b.x), dy = __dsub_rn(a.y, b.y), dz = __dsub_rn(a.z, b.z);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    const double hbar = __dmul_rn(0.5, __dadd_rn(a.w, b.w));
    const double rad = __dmul_rn(2., hbar);
    return d2 < __dmul_rn(rad, rad);
}

// the query of findAll(i, 2 h_i) (KdTree::find, core/objects/finders/KdTree.inl.h:316-391): |r_j - r_i|^2 <
// (2 h_i)^2 in FP64
__device__ __forceinline__ bool withinTwoH(const dbl4& a, const dbl4& b) {
    const double dx = __dsub_rn(b.x, a.x), dy = __dsub_rn(b.y, a.y), dz = __dsub_rn(b.z, a.z);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    const double rad = __dmul_rn(2., a.w);
    return d2 < __dmul_rn(rad, rad);
}

// Directed = false: the unordered interacting pairs (i < j, 2 h_bar); true: the directed pairs (i, j), j != i, of
// every particle's ball of radius 2 h_i (the cell edge is at least 2 max h, so 27 cells hold either set)
template <bool List, bool Directed = false>
__global__ void pairsKernel(uint32_t n, const dbl4* __restrict__ rs, const uint32_t* __restrict__ perm,
    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ cstart, const uint32_t* __restrict__ cend,
    const GridInfo* __restrict__ g, uint32_t* pi, uint32_t* pj, unsigned long long* count,
    unsigned long long capacity) {
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
    for (int z = max(cz - 1, 0); z <= min(cz + 1, dz - 1); ++z) {
        for (int y = max(cy - 1, 0); y <= min(cy + 1, dy - 1); ++y) {
            for (int x = max(cx - 1, 0); x <= min(cx + 1, dx - 1); ++x) {
                const uint32_t c = (uint32_t(z) * uint32_t(dy) + uint32_t(y)) * uint32_t(dx) + uint32_t(x);
                const uint32_t e = cend[c];
                for (uint32_t t = cstart[c]; t < e; ++t) {
                    const uint32_t j = perm[t];
                    if (Directed ? (j == i || !withinTwoH(ri, rs[t])) : (j <= i || !interacts(ri, rs[t]))) {
                        continue;
                    }
                    const unsigned long long slot = atomicAdd(count, 1ull);
                    if (List && slot < capacity) {
                        pi[slot] = i;
                        pj[slot] = j;
                    }
                }
            }
        }
    }
}

} // namespace

cudaError_t gridAllocate(Grid& g, uint32_t n, bool solid, bool correction, bool copies, bool neighbourLists) {
    const uint32_t nn = n > 0 ? n : 1;
    g.cell_capacity = max(1u << 12, min(4u * nn, 1u << 26));
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) {
            e = cudaMalloc(p, bytes > 0 ? bytes : 16);
        }
    };
    alloc((void**)&g.info, sizeof(GridInfo));
    alloc((void**)&g.bounds, 8 * sizeof(unsigned long long));
    alloc((void**)&g.keys, nn * sizeof(uint32_t));
    alloc((void**)&g.keys_sorted, nn * sizeof(uint32_t));
    alloc((void**)&g.perm_in, nn * sizeof(uint32_t));
    alloc((void**)&g.perm, nn * sizeof(uint32_t));
    alloc((void**)&g.cell_start, size_t(g.cell_capacity) * sizeof(uint32_t));
    alloc((void**)&g.cell_end, size_t(g.cell_capacity) * sizeof(uint32_t));
    if (copies) {
        alloc((void**)&g.rs, nn * sizeof(dbl4));
        alloc((void**)&g.vs, nn * sizeof(dbl4));
        alloc((void**)&g.ms, nn * sizeof(double));
        alloc((void**)&g.rhos, nn * sizeof(double));
        alloc((void**)&g.ps, nn * sizeof(double));
        alloc((void**)&g.css, nn * sizeof(double));
        alloc((void**)&g.mx0, nn * sizeof(float4));
        alloc((void**)&g.mx1, nn * sizeof(float4));
        alloc((void**)&g.mx2, nn * sizeof(float4));
        alloc((void**)&g.mx3, nn * sizeof(float4));
    }
    if (solid) {
        alloc((void**)&g.Ss, 5 * size_t(nn) * sizeof(double));
        alloc((void**)&g.reduces, nn * sizeof(double));
        alloc((void**)&g.flags, nn * sizeof(uint32_t));
        alloc((void**)&g.mxS, 5 * size_t(nn) * sizeof(float));
    }
    if (correction) {
        alloc((void**)&g.mxC, 6 * size_t(nn) * sizeof(float));
    }
    if (neighbourLists) {
        alloc((void**)&g.nb, size_t(NB_CAP) * nn * sizeof(uint32_t));
        alloc((void**)&g.nb_count, nn * sizeof(uint32_t));
        alloc((void**)&g.nb_over, nn * sizeof(uint32_t));
        alloc((void**)&g.nb_over_count, sizeof(uint32_t));
        alloc((void**)&g.cell_first, (size_t(g.cell_capacity) + 1) * sizeof(uint32_t));
    }
    if (e != cudaSuccess) {
        return e;
    }
    g.sort_temp_bytes = 0;
    e = cub::DeviceRadixSort::SortPairs(nullptr, g.sort_temp_bytes, g.keys, g.keys_sorted, g.perm_in, g.perm,
        int(nn), 0, 32);
    if (e != cudaSuccess) {
        return e;
    }
    return cudaMalloc(&g.sort_temp, g.sort_temp_bytes > 0 ? g.sort_temp_bytes : 16);
}

void gridFree(Grid& g) {
    void* ptrs[] = { g.info, g.bounds, g.keys, g.keys_sorted, g.perm_in, g.perm, g.cell_start, g.cell_end,
        g.sort_temp, g.rs, g.vs, g.ms, g.rhos, g.ps, g.css, g.Ss, g.reduces, g.flags, g.mx0, g.mx1, g.mx2, g.mx3,
        g.mxS, g.mxC, g.nb, g.nb_count, g.nb_over, g.nb_over_count, g.cell_first };
    for (void* p : ptrs) {
        if (p) {
            cudaFree(p);
        }
    }
    g = Grid();
}

void launchGridBuild(const DState& s, Grid& g, const Physics& ph, cudaStream_t st, bool fine) {
    (void)ph;
    launchGridBuildRadius(s.r, nullptr, s.n, g, st, fine && g.cell_first != nullptr);
}

void launchGridBuildRadius(const dbl4* r, const double* radius, uint32_t n, Grid& g, cudaStream_t st, bool fine) {
    const int meanCell = radius ? 1 : 0;
    g.launches = n > 0 ? 6 : 2;
    resetBounds<<<1, 32, 0, st>>>(g.bounds);
    if (n > 0) {
        const int blocks = min(ceilDiv(n, 256), 152 * 2);
        boundsKernel<<<blocks, 256, 0, st>>>(r, radius, n, g.bounds);
    }
    gridSetupKernel<<<1, 1, 0, st>>>(g.bounds, g.cell_capacity, n, meanCell, fine ? 1 : 0, g.info);
    if (n == 0) {
        return;
    }
    keysKernel<<<ceilDiv(n, 256), 256, 0, st>>>(r, n, g.info, g.keys, g.perm_in);
    int bits = 1;
    while ((1u << bits) < g.cell_capacity && bits < 32) {
        ++bits;
    }
    size_t temp = g.sort_temp_bytes;
    cub::DeviceRadixSort::SortPairs(g.sort_temp, temp, g.keys, g.keys_sorted, g.perm_in, g.perm, int(n), 0, bits,
        st);
    clearCells<<<152 * 4, 256, 0, st>>>(g.cell_start, g.cell_end, g.info);
    cellRanges<<<ceilDiv(n, 256), 256, 0, st>>>(g.keys_sorted, n, g.cell_start, g.cell_end);
    if (fine) {
        cellFirstKernel<<<std::min(ceilDiv(g.cell_capacity + 1, 256), 152 * 16), 256, 0, st>>>(g.keys_sorted, n,
            g.info, g.cell_capacity, g.cell_first);
        g.launches += 1;
    }
}

void launchGatherSorted(const DState& s, Grid& g, const Physics& ph, cudaStream_t st) {
    if (s.n == 0) {
        return;
    }
    g.launches = ph.precision == SPHGPU_PRECISION_MIXED ? 2 : 1;
    if (ph.precision == SPHGPU_PRECISION_MIXED) {
        gatherSortedMixed<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, g.perm, g.keys_sorted, g.info, g.mx0, g.mx1, g.mx2,
            g.mx3, g.mxS, ph.solid);
    }
    gatherSorted<<<ceilDiv(s.n, 256), 256, 0, st>>>(s, g.perm, g.rs, g.vs, g.ms, g.rhos, g.ps, g.css, g.Ss,
        g.reduces, g.flags, ph.solid);
}

// ISymmetricFinder::findAll(const Vector& pos, radius) (core/objects/finders/NeighborFinder.h:112-117) on the grid:
// every particle j with |r_j - pos|^2 < radius^2 (xyz, FP64, the test of KdTree::find), from the cells that the
// ball's bounding box overlaps. Output slots are taken atomically (unordered); count keeps counting past capacity.
__global__ void findBallKernel(const dbl4* __restrict__ rs, const uint32_t* __restrict__ perm,
    const uint32_t* __restrict__ cellStart, const uint32_t* __restrict__ cellEnd, const GridInfo* __restrict__ info,
    dbl4 pos, double radius, uint32_t* outIdx, double* outD2, unsigned long long* count, unsigned long long capacity) {
    const GridInfo gi = *info;
    int c0[3], c1[3];
    const double p[3] = { pos.x, pos.y, pos.z };
    for (int d = 0; d < 3; ++d) {
        const double a = floor((p[d] - radius - gi.lo[d]) * gi.inv_cell);
        const double b = floor((p[d] + radius - gi.lo[d]) * gi.inv_cell);
        c0[d] = int(fmax(0., fmin(a, double(gi.dims[d] - 1))));
        c1[d] = int(fmax(0., fmin(b, double(gi.dims[d] - 1))));
    }
    const uint32_t nx = uint32_t(c1[0] - c0[0] + 1), ny = uint32_t(c1[1] - c0[1] + 1), nz = uint32_t(c1[2] - c0[2] + 1);
    const unsigned long long total = (unsigned long long)nx * ny * nz;
    const double r2 = radius * radius;
    for (unsigned long long t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const uint32_t x = c0[0] + uint32_t(t % nx), y = c0[1] + uint32_t((t / nx) % ny),
                       z = c0[2] + uint32_t(t / (unsigned long long)(nx * ny));
        const uint32_t c = (z * uint32_t(gi.dims[1]) + y) * uint32_t(gi.dims[0]) + x;
        for (uint32_t k = cellStart[c]; k < cellEnd[c]; ++k) {
            const dbl4 q = rs[k];
            const double dx = q.x - pos.x, dy = q.y - pos.y, dz = q.z - pos.z;
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < r2) {
                const unsigned long long slot = atomicAdd(count, 1ull);
                if (slot < capacity) {
                    outIdx[slot] = perm[k];
                    outD2[slot] = d2;
                }
            }
        }
    }
}

void launchFindBall(const Grid& g, uint32_t n, const dbl4& pos, double radius, uint32_t* idx, double* d2,
    unsigned long long* count, unsigned long long capacity, cudaStream_t st) {
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
    if (n == 0) {
        return;
    }
    findBallKernel<<<152, 128, 0, st>>>(g.rs, g.perm, g.cell_start, g.cell_end, g.info, pos, radius, idx, d2, count,
        capacity);
}

void launchRadiusPairs(const DState& s, const Grid& g, uint32_t* pi, uint32_t* pj, unsigned long long* count,
    unsigned long long capacity, cudaStream_t st) {
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
    if (s.n == 0) {
        return;
    }
    if (pi) {
        pairsKernel<true, true><<<ceilDiv(s.n, 128), 128, 0, st>>>(s.n, g.rs, g.perm, g.keys_sorted, g.cell_start,
            g.cell_end, g.info, pi, pj, count, capacity);
    } else {
        pairsKernel<false, true><<<ceilDiv(s.n, 128), 128, 0, st>>>(s.n, g.rs, g.perm, g.keys_sorted, g.cell_start,
            g.cell_end, g.info, nullptr, nullptr, count, 0);
    }
}

void launchCountPairs(const DState& s, const Grid& g, unsigned long long* count, cudaStream_t st) {
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
    if (s.n == 0) {
        return;
    }
    pairsKernel<false><<<ceilDiv(s.n, 128), 128, 0, st>>>(s.n, g.rs, g.perm, g.keys_sorted, g.cell_start,
        g.cell_end, g.info, nullptr, nullptr, count, 0);
}

void launchListPairs(const DState& s, const Grid& g, uint32_t* pi, uint32_t* pj, unsigned long long* count,
    unsigned long long capacity, cudaStream_t st) {
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
    if (s.n == 0) {
        return;
    }
    pairsKernel<true><<<ceilDiv(s.n, 128), 128, 0, st>>>(s.n, g.rs, g.perm, g.keys_sorted, g.cell_start,
        g.cell_end, g.info, pi, pj, count, capacity);
}

} // namespace sphgpu
