// grid.cu -- multi-level uniform-grid spatial hash over the valid points of an
// organised cloud, with exact k-nearest-neighbour and radius queries; the
// PCL-style StatisticalOutlierRemoval and the metric (millimetre-sigma)
// Gaussian filter.
//
// Neither filter exists in the reference tree (PCL is linked but never
// included, PhaseShiftGrayCode3D/PCL114_Release_x64.props:17-18); SOR follows
// PCL's documented StatisticalOutlierRemoval algorithm: mean distance to the k
// nearest neighbours, threshold mean + std_mul * stddev, keep d <= threshold.
//
// Build (no host synchronisation): a trimmed mean of adjacent-pixel spacing
// (the plain mean on the pixel-ray path) sets the finest cell c on the device; the finest level (cell c) is
// counting-sorted into a power-of-two hash table of (offset, count) pairs, the
// coarse level (cell >= 16c) into a dense grid over the bounding box.
//
// SOR on a cloud with pixel rays (the organised cloud of the calibrated size):
//   window pass: one thread per pixel walks its 15x15 window in a spiral with
//            a max-heap of the k + 1 nearest, certified exact by a bound on
//            the distance to every point seen along another pixel's ray;
//   far search: one warp per remaining point searches rings of coarse cells
//            around its own until the next ring lies beyond the (k + 1)-th
//            distance held;
//   hard search: the few points still open (far-isolated outliers) take one
//            CTA each over the coarse level's occupied cells.
// Without pixel rays the first two passes are replaced by the tile search:
// one CTA per 16x8 pixel tile gathers the finest-level points of the tile's
// cell box (dilated by TILE_DILATE cells) into shared memory; every thread
// scans the same candidate list and is exact once it holds k + 1 candidates
// within its distance to the box boundary.  A visited point's finest cell is
// re-derived from its coordinates, so hash collisions never count a point
// twice.  Every path sums the same k + 1 roots in fixed point, so a query's
// mean distance has the same bits whichever path settles it.
//
// The metric Gaussian: a window pass with the same ray bound; the queries it
// cannot certify take the grid path (27 cells of side 3 sigma, 64-bit
// fixed-point sums), whose build is skipped on the device when none are left.
// The SOR statistics are summed in a fixed order: both filters are
// deterministic.

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <utility>

#include "zim_tiles.cuh"

namespace {

constexpr int GB = 256;          // threads for pixel-parallel kernels
constexpr int KNN_MAX_K1 = 64;   // k + 1 <= 64
constexpr int SCAN_B = 1024;
constexpr int MAX_LEVELS = 2;    // finest + one coarse level
constexpr int FINE_RINGS = 2;    // phase-1 fallback rings on the finest level
constexpr int P2_WARPS = 4;      // phase-2 warps per CTA
constexpr int RING_MAX = 6;      // phase-2 rings of dense cells before the hard list
// md marker of a deferred query whose bound on the (k + 1)-th squared distance
// is handed on in the bound array (md = -1: no bound)
constexpr float MD_BOUND = -3.f;
constexpr int TILE_X = 16, TILE_Y = 8, TILE_T = TILE_X * TILE_Y;
// the window passes' tiles (SOR window, metric Gaussian window, per-tile ray
// distances): taller tiles stage less halo per query
constexpr int WT_X = 16, WT_Y = 16, WT_T = WT_X * WT_Y;
constexpr int TILE_DILATE = 2;        // cells added around a tile's box
constexpr int TILE_MAX_CELLS = 1024;  // gathered box of cells per tile
constexpr int TILE_MAX_CAND = 1536;   // gathered points per tile (a surface tile gathers ~800)
constexpr int COARSE_MULT = 16;       // coarse level cell = 16 x finest
constexpr long long DENSE_MAX = 1 << 18;  // cells of the dense coarse level (caps its scans and sweeps)

struct GridStats {
    double sp_sum, sp_cnt;    // spacing pass 1
    double sp2_sum, sp2_cnt;  // spacing pass 2 (trimmed)
    double n_valid;
    double md_sum, md_sq;     // SOR statistics (fixed-order sums)
    float cell[MAX_LEVELS], inv_cell[MAX_LEVELS];
    int max_ring[MAX_LEVELS];
    int bbox_min[3], bbox_max[3];  // order-preserving float bits
    float org[3];                  // coarse (dense) level: origin and dimensions
    int dims[3];
    float amax;                    // largest |coordinate| of the bounding box
    double thr;                    // SOR threshold, and the largest float <= it
    float thr_f;
    int keep_all;
    unsigned ray_dev_bits;         // largest distance of a point from its pixel ray (float bits)
    unsigned n_deferred, n_occ, p2_next, n_hard;
    unsigned n_pending;            // metric Gaussian: queries the window pass left to the grid
};

__device__ __forceinline__ int fbits(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float bitsf(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ unsigned hash3(int x, int y, int z, unsigned tmask) {
    return ((unsigned)x * 73856093u ^ (unsigned)y * 19349663u ^ (unsigned)z * 83492791u) & tmask;
}

// Deterministic block reduction (fixed shuffle tree); result valid in thread 0.
template <typename T, typename Op>
__device__ __forceinline__ T block_reduce(T v, Op op, T ident) {
    __shared__ T ws[32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int off = 16; off; off >>= 1) v = op(v, __shfl_down_sync(0xffffffffu, v, off));
    if (lane == 0) ws[w] = v;
    __syncthreads();
    T r = ident;
    if (w == 0) {
        r = lane < (int)(blockDim.x >> 5) ? ws[lane] : ident;
        for (int off = 16; off; off >>= 1) r = op(r, __shfl_down_sync(0xffffffffu, r, off));
    }
    __syncthreads();
    return r;
}
struct Add { template <typename T> __device__ T operator()(T a, T b) const { return a + b; } };
struct Min { __device__ int operator()(int a, int b) const { return a < b ? a : b; } };
struct Max { __device__ int operator()(int a, int b) const { return a > b ? a : b; } };

// The build kernels take a gate: when it points to 0 the grid is not needed
// (no query is left for it) and every block returns at once.
__device__ __forceinline__ bool gated_off(const unsigned* gate) { return gate && *gate == 0u; }

__global__ void stats_init_kernel(GridStats* s) {
    s->sp_sum = s->sp_cnt = s->sp2_sum = s->sp2_cnt = 0;
    s->md_sum = s->md_sq = s->n_valid = 0;
    s->n_deferred = s->n_occ = s->p2_next = s->n_hard = s->n_pending = 0;
    s->ray_dev_bits = 0u;
    for (int a = 0; a < 3; a++) { s->bbox_min[a] = INT_MAX; s->bbox_max[a] = INT_MIN; }
}

// Blocks of the spacing passes (grid-stride).  Each block writes its partial
// sums; spacing_total_kernel adds them in a fixed order, so the cell size does
// not depend on the order blocks finish in.
constexpr int SPACING_BLOCKS = 1024;

// pass 1: mean spacing of horizontally adjacent valid pixels, bbox, count, and
// (rays != 0) the largest distance of a point from its pixel ray.  Counts are
// integers (exact); a thread's spacings add in FP32 (they only set the cell
// size) and go to FP64 once, for the fixed-order totals.
__global__ void spacing1_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, int rows, int cols,
                                int rays, zt::RayParams rp, GridStats* s, double* __restrict__ part,
                                const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    float df = 0.f;
    unsigned ci = 0u, nvi = 0u, dev = 0u;
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
    // blocks over rows, threads over a row's pixels (no index division), four
    // pixels of a thread at a time with their loads issued together (the same
    // pixels in the same order as one at a time)
    constexpr int U = 4;
    for (int y = blockIdx.x; y < rows; y += gridDim.x) {
        const size_t r0 = (size_t)y * cols;
        for (int xb = threadIdx.x; xb < cols; xb += U * blockDim.x) {
            bool m[U], mr[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int x = xb + u * (int)blockDim.x;
                m[u] = x < cols && mask[r0 + x];
                mr[u] = x + 1 < cols && mask[r0 + x + 1];
            }
            float p[U][3], q[U][3];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const size_t i = r0 + xb + u * blockDim.x;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    p[u][a] = m[u] ? xyz[3 * i + a] : 0.f;
                    q[u][a] = m[u] && mr[u] ? xyz[3 * i + 3 + a] : 0.f;
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (!m[u]) continue;
                const int x = xb + u * (int)blockDim.x;
                nvi++;
                for (int a = 0; a < 3; a++) {
                    mn[a] = min(mn[a], fbits(p[u][a]));
                    mx[a] = max(mx[a], fbits(p[u][a]));
                }
                if (rays) {
                    float ax, ay, az;
                    zt::ray_dir(rp, x, y, ax, ay, az);
                    const float d = zt::ray_dev(p[u][0], p[u][1], p[u][2], ax, ay, az);
                    dev = max(dev, __float_as_uint(d == d ? d : INFINITY));  // NaN counts as unbounded
                }
                if (mr[u]) {
                    float dx = q[u][0] - p[u][0], dy = q[u][1] - p[u][1], dz = q[u][2] - p[u][2];
                    df += sqrtf(dx * dx + dy * dy + dz * dz);
                    ci++;
                }
            }
        }
    }
    double d = block_reduce((double)df, Add(), 0.0);
    double c = block_reduce((double)ci, Add(), 0.0);
    double nv = block_reduce((double)nvi, Add(), 0.0);
    if (rays) {  // uniform
        dev = __reduce_max_sync(0xffffffffu, dev);
        if ((threadIdx.x & 31) == 0 && dev) atomicMax(&s->ray_dev_bits, dev);
    }
    for (int a = 0; a < 3; a++) {
        mn[a] = block_reduce(mn[a], Min(), INT_MAX);
        mx[a] = block_reduce(mx[a], Max(), INT_MIN);
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = d;
        part[3 * blockIdx.x + 1] = c;
        part[3 * blockIdx.x + 2] = nv;
        for (int a = 0; a < 3; a++) {
            if (mn[a] != INT_MAX) atomicMin(&s->bbox_min[a], mn[a]);
            if (mx[a] != INT_MIN) atomicMax(&s->bbox_max[a], mx[a]);
        }
    }
}

// pass 2: mean spacing over pairs closer than 3x the pass-1 mean
__global__ void spacing2_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, int rows, int cols,
                                const GridStats* __restrict__ s, double* __restrict__ part,
                                const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    const double m1 = s->sp_cnt > 0 ? s->sp_sum / s->sp_cnt : 0.0;
    const float cut = (float)(3.0 * m1);  // the pass only sets the cell size
    float df = 0.f;
    unsigned ci = 0u;
    for (int y = blockIdx.x; y < rows; y += gridDim.x)
        for (int x = threadIdx.x; x + 1 < cols; x += blockDim.x) {
            const size_t i = (size_t)y * cols + x;
            if (!(mask[i] && mask[i + 1])) continue;
            float dx = xyz[3 * i + 3] - xyz[3 * i], dy = xyz[3 * i + 4] - xyz[3 * i + 1],
                  dz = xyz[3 * i + 5] - xyz[3 * i + 2];
            float v = sqrtf(dx * dx + dy * dy + dz * dz);
            if (v <= cut) { df += v; ci++; }
        }
    double d = block_reduce((double)df, Add(), 0.0);
    double c = block_reduce((double)ci, Add(), 0.0);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = d;
        part[3 * blockIdx.x + 1] = c;
        part[3 * blockIdx.x + 2] = 0.0;
    }
}

// Fixed-order total of the spacing passes' block partials (one block of
// SPACING_BLOCKS threads).  pass 1 sets the mean spacing and the valid count,
// pass 2 the trimmed mean spacing.
__global__ void spacing_total_kernel(const double* __restrict__ part, int nblk, int pass, GridStats* s,
                                     const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    const int t = threadIdx.x;
    double d = t < nblk ? part[3 * t] : 0.0, c = t < nblk ? part[3 * t + 1] : 0.0;
    double nv = t < nblk ? part[3 * t + 2] : 0.0;
    d = block_reduce(d, Add(), 0.0);
    c = block_reduce(c, Add(), 0.0);
    nv = block_reduce(nv, Add(), 0.0);
    if (t == 0) {
        if (pass == 1) {
            s->sp_sum = d;
            s->sp_cnt = c;
            s->n_valid = nv;
        } else {
            s->sp2_sum = d;
            s->sp2_cnt = c;
        }
    }
}

// Finest cell = fixed_cell if > 0, else factor * (trimmed) mean spacing (a
// hashed level).  The coarse level is a dense grid over the bounding box with
// cells of COARSE_MULT finest cells, enlarged until it has at most DENSE_MAX
// cells.  The cell sizes only affect speed, never the result.
__global__ void cell_kernel(GridStats* s, float fixed_cell, float factor, int levels, const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    float cell = fixed_cell;
    if (!(cell > 0.f)) {
        // the trimmed mean spacing (pass 2) where it ran, else pass 1's mean
        double sp = s->sp2_cnt > 0 ? s->sp2_sum / s->sp2_cnt : (s->sp_cnt > 0 ? s->sp_sum / s->sp_cnt : 1.0);
        cell = (float)(factor * sp);
    }
    float ext = 0.f, e[3] = {0.f, 0.f, 0.f}, amax = 0.f;
    for (int a = 0; a < 3; a++)
        if (s->bbox_max[a] >= s->bbox_min[a]) {
            e[a] = bitsf(s->bbox_max[a]) - bitsf(s->bbox_min[a]);
            ext = fmaxf(ext, e[a]);
            s->org[a] = bitsf(s->bbox_min[a]);
            amax = fmaxf(amax, fmaxf(fabsf(bitsf(s->bbox_min[a])), fabsf(bitsf(s->bbox_max[a]))));
        } else {
            s->org[a] = 0.f;
        }
    s->amax = amax;
    cell = fmaxf(cell, ext * 1e-5f);
    cell = fmaxf(cell, 1e-6f);
    s->cell[0] = cell;
    s->inv_cell[0] = 1.0f / cell;
    s->max_ring[0] = (int)ceilf(ext / cell) + 2;
    if (levels > 1) {
        float c = cell * (float)COARSE_MULT;
        for (;;) {
            long long v = 1;
            for (int a = 0; a < 3; a++) {
                s->dims[a] = (int)floorf(e[a] / c) + 1;
                v *= s->dims[a];
            }
            if (v <= DENSE_MAX) break;
            c *= 1.26f;
        }
        s->cell[1] = c;
        s->inv_cell[1] = 1.0f / c;
        s->max_ring[1] = (int)ceilf(ext / c) + 2;
    }
}

// Squared distance with one fixed rounding sequence, so the same pair of
// points gives the same value at every call site of the kNN search.
__device__ __forceinline__ float sqdist(float dx, float dy, float dz) { return fmaf(dz, dz, fmaf(dy, dy, dx * dx)); }

// Hardware square root (PTX sqrt.approx.f32, relative error below 2^-22): one
// instruction, the same at every call site, so every search path rounds alike.
__device__ __forceinline__ float root_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Order-independent sum of the k + 1 nearest distances: each root, scaled by
// 2^(23 - e) with root(largest squared distance) < 2^e, is truncated to an
// integer below 2^23 and the integers are added exactly (at most 64 of them:
// below 2^29), so every search path and every visiting order gives the same
// bits.  The truncation is one FMA rounded toward zero onto 2^23, whose
// mantissa then holds the integer: no 64-bit conversion (FP64 pipe) per root.
// The roots are root_approx's; e leaves 2^-19 of room above the largest, more
// than the approximation's error, so no smaller entry's root reaches 2^e.
// Roots below 2^(e - 23), a 2^-22 fraction of the largest, count as 0.
__device__ __forceinline__ int root_exponent(float d2max) {
    int e;
    frexpf(root_approx(d2max) * 1.000002f, &e);
    return min(max(e, -60), 100);  // keeps 2^(23 - e) and 2^(e - 23) normal
}
__device__ __forceinline__ float root_scale(int e) { return __uint_as_float((unsigned)(150 - e) << 23); }
__device__ __forceinline__ unsigned root_fixed(float d2, float scale) {
    return __float_as_uint(__fmaf_rz(root_approx(d2), scale, 8388608.f)) - 0x4B000000u;
}
// (sum / k) 2^(e - 23), one float division
__device__ __forceinline__ float fixed_mean(unsigned sum, int e, int k) {
    return __fdiv_rn(__uint2float_rn(sum), (float)k) * __uint_as_float((unsigned)(104 + e) << 23);
}

__device__ __forceinline__ void cell_of(float x, float y, float z, float ic, int& cx, int& cy, int& cz) {
    cx = __float2int_rd(x * ic);
    cy = __float2int_rd(y * ic);
    cz = __float2int_rd(z * ic);
}

// Table slot of a point: hashed cell on the finest level, dense cell index on
// the coarse level.
__device__ __forceinline__ unsigned grid_slot(const GridStats* __restrict__ s, int level, unsigned tmask, float x,
                                              float y, float z) {
    if (level == 0) {
        int cx, cy, cz;
        cell_of(x, y, z, s->inv_cell[0], cx, cy, cz);
        return hash3(cx, cy, cz, tmask);
    }
    const float ic = s->inv_cell[1];
    int ix = min(max(__float2int_rd((x - s->org[0]) * ic), 0), s->dims[0] - 1);
    int iy = min(max(__float2int_rd((y - s->org[1]) * ic), 0), s->dims[1] - 1);
    int iz = min(max(__float2int_rd((z - s->org[2]) * ic), 0), s->dims[2] - 1);
    return ((unsigned)iz * (unsigned)s->dims[1] + (unsigned)iy) * (unsigned)s->dims[0] + (unsigned)ix;
}

// Neighbouring pixels mostly share a cell, so the lanes of a warp that hit the
// same slot add to it once (the lowest such lane).
// The table kernels stride over the points with a grid sized to the GPU, not
// to the cloud: a gated-off launch then costs a few waves of empty blocks.
__global__ void hash_count_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                  const GridStats* __restrict__ s, int level, unsigned tmask,
                                  unsigned* __restrict__ counts, const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    for (size_t b = (size_t)blockIdx.x * blockDim.x; b < n; b += (size_t)gridDim.x * blockDim.x) {
        const size_t i = b + threadIdx.x;
        const bool v = i < n && mask[i];
        const unsigned h = v ? grid_slot(s, level, tmask, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]) : 0xffffffffu;
        const unsigned grp = __match_any_sync(0xffffffffu, h);
        if (v && (threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&counts[h], (unsigned)__popc(grp));
    }
}

__global__ void zero_kernel(unsigned* __restrict__ p, size_t n, const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = 0u;
}

__device__ __forceinline__ unsigned block_scan_incl(unsigned v, unsigned* ws) {
    unsigned x = v;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int off = 1; off < 32; off <<= 1) {
        unsigned t = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += t;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        unsigned y = ws[lane];
        for (int off = 1; off < 32; off <<= 1) {
            unsigned t = __shfl_up_sync(0xffffffffu, y, off);
            if (lane >= off) y += t;
        }
        ws[lane] = y;
    }
    __syncthreads();
    return x + (w ? ws[w - 1] : 0u);
}

// exclusive scan of the counts into tab[].x (per-block part), block totals
__global__ void scan_blocks_kernel(const unsigned* __restrict__ counts, uint2* __restrict__ tab, size_t n,
                                   unsigned* __restrict__ block_tot, const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    __shared__ unsigned ws[32];
    const size_t nb = (n + SCAN_B - 1) / SCAN_B;
    for (size_t b = blockIdx.x; b < nb; b += gridDim.x) {
        const size_t i = b * SCAN_B + threadIdx.x;
        const unsigned v = i < n ? counts[i] : 0u;
        const unsigned incl = block_scan_incl(v, ws);
        if (i < n) tab[i] = make_uint2(incl - v, v);
        if (threadIdx.x == SCAN_B - 1) block_tot[b] = incl;
        __syncthreads();  // ws is reused by the next chunk
    }
}

__global__ void scan_totals_kernel(unsigned* __restrict__ tot, int nb, const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    __shared__ unsigned carry;
    __shared__ unsigned ws[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += SCAN_B) {
        int i = base + threadIdx.x;
        unsigned v = i < nb ? tot[i] : 0u;
        unsigned incl = block_scan_incl(v, ws);
        unsigned c = carry;
        if (i < nb) tot[i] = c + incl - v;
        __syncthreads();
        if (threadIdx.x == SCAN_B - 1) carry = c + incl;
        __syncthreads();
    }
}

__global__ void scan_add_kernel(uint2* __restrict__ tab, size_t n, const unsigned* __restrict__ tot,
                                const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    const size_t nb = (n + SCAN_B - 1) / SCAN_B;
    for (size_t b = blockIdx.x; b < nb; b += gridDim.x) {
        const size_t i = b * SCAN_B + threadIdx.x;
        if (i < n) tab[i].x += tot[b];
    }
}

__global__ void hash_scatter_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                    const GridStats* __restrict__ s, int level, unsigned tmask,
                                    const uint2* __restrict__ tab, unsigned* __restrict__ fill,
                                    float4* __restrict__ pts, const unsigned* __restrict__ gate) {
    if (gated_off(gate)) return;
    for (size_t b = (size_t)blockIdx.x * blockDim.x; b < n; b += (size_t)gridDim.x * blockDim.x) {
        const size_t i = b + threadIdx.x;
        const bool v = i < n && mask[i];
        float x = 0.f, y = 0.f, z = 0.f;
        unsigned h = 0xffffffffu;
        if (v) {
            x = xyz[3 * i]; y = xyz[3 * i + 1]; z = xyz[3 * i + 2];
            h = grid_slot(s, level, tmask, x, y, z);
        }
        // one atomic per slot and warp; lanes take consecutive places in lane order
        const unsigned grp = __match_any_sync(0xffffffffu, h);
        const int lane = threadIdx.x & 31, leader = __ffs(grp) - 1;
        unsigned base = 0;
        if (v && lane == leader) base = atomicAdd(&fill[h], (unsigned)__popc(grp));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (v) {
            const unsigned pos = tab[h].x + base + (unsigned)__popc(grp & ((1u << lane) - 1u));
            pts[pos] = make_float4(x, y, z, __int_as_float((int)i));
        }
    }
}

// Sorts each bucket by pixel index, so bucket contents no longer depend on the
// order of the scatter's atomics.
__global__ void bucket_sort_kernel(const uint2* __restrict__ tab, unsigned T, float4* __restrict__ pts) {
    unsigned h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= T) return;
    const uint2 e = tab[h];
    for (unsigned a = e.x + 1; a < e.x + e.y; a++) {
        float4 v = pts[a];
        int key = __float_as_int(v.w);
        unsigned b = a;
        while (b > e.x && __float_as_int(pts[b - 1].w) > key) {
            pts[b] = pts[b - 1];
            b--;
        }
        pts[b] = v;
    }
}

struct Level {
    const uint2* tab;  // (offset, count) per bucket
    const float4* pts;
    unsigned tmask;
};

__device__ __forceinline__ uint2 bucket(const Level& g, int x, int y, int z) {
    return __ldg(g.tab + hash3(x, y, z, g.tmask));
}

// Visits the points of all cells at Chebyshev distance exactly r from (cx, cy, cz).
template <typename F>
__device__ __forceinline__ void visit_ring(const Level& g, float ic, int cx, int cy, int cz, int r, F&& fn) {
    for (int dz = -r; dz <= r; dz++)
        for (int dy = -r; dy <= r; dy++) {
            const bool full = (r == 0 || dz == -r || dz == r || dy == -r || dy == r);
            const int step = full ? 1 : 2 * r;
            for (int dx = -r; dx <= r; dx += step) {
                int x = cx + dx, y = cy + dy, z = cz + dz;
                uint2 b = bucket(g, x, y, z);
                for (unsigned t = b.x; t < b.x + b.y; t++) {
                    float4 p = __ldg(g.pts + t);
                    int px, py, pz;
                    cell_of(p.x, p.y, p.z, ic, px, py, pz);
                    if (px != x || py != y || pz != z) continue;
                    fn(p);
                }
            }
        }
}

// Pixel offsets within WIN_R of the centre, ordered by length.
constexpr int WIN_R = 4;
constexpr int WIN_W = TILE_X + 2 * WIN_R, WIN_H = TILE_Y + 2 * WIN_R;
constexpr int WIN_N = (2 * WIN_R + 1) * (2 * WIN_R + 1) - 1;
__constant__ signed char c_spiral[WIN_N][2] = {
    {0, -1}, {-1, 0}, {1, 0}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}, {0, -2}, {-2, 0},
    {2, 0}, {0, 2}, {-1, -2}, {1, -2}, {-2, -1}, {2, -1}, {-2, 1}, {2, 1}, {-1, 2}, {1, 2},
    {-2, -2}, {2, -2}, {-2, 2}, {2, 2}, {0, -3}, {-3, 0}, {3, 0}, {0, 3}, {-1, -3}, {1, -3},
    {-3, -1}, {3, -1}, {-3, 1}, {3, 1}, {-1, 3}, {1, 3}, {-2, -3}, {2, -3}, {-3, -2}, {3, -2},
    {-3, 2}, {3, 2}, {-2, 3}, {2, 3}, {0, -4}, {-4, 0}, {4, 0}, {0, 4}, {-1, -4}, {1, -4},
    {-4, -1}, {4, -1}, {-4, 1}, {4, 1}, {-1, 4}, {1, 4}, {-3, -3}, {3, -3}, {-3, 3}, {3, 3},
    {-2, -4}, {2, -4}, {-4, -2}, {4, -2}, {-4, 2}, {4, 2}, {-2, 4}, {2, 4}, {-3, -4}, {3, -4},
    {-4, -3}, {4, -3}, {-4, 3}, {4, 3}, {-3, 4}, {3, 4}, {-4, -4}, {4, -4}, {-4, 4}, {4, 4}};
static_assert(WIN_W * WIN_H <= TILE_MAX_CAND, "pixel window staged in the candidate buffer");
static_assert(TILE_MAX_CELLS <= 8 * TILE_T, "cell scan: eight cells per thread");

constexpr int SV_CAP = 128;  // survivors per warp query (k + 1 <= 64 of them kept)

// Phase 1: one CTA per 16 x 8 pixel tile on the finest level.
//  - Window bound: the query and its k nearest valid pixels (in pixel
//    distance, within WIN_R) are k + 1 real points, so the largest of their
//    squared distances, tau0, bounds the (k + 1)-th nearest squared distance.
//  - Box: the tile's points, minus depth outliers (a trimmed mean of their z
//    cells), span a box of cells; the CTA gathers every point of that box
//    dilated by TILE_DILATE cells into shared memory, sorted by cell.  All
//    points within distance g of a query lie in the box, g being the query's
//    distance to the box boundary.
//  - Each in-box query scans only the cells its ball of squared radius
//    min(tau0, g^2) touches; holding k + 1 candidates within that ball, it is
//    exact.  The warp does this one query at a time, lanes over candidates.
// Queries the box cannot settle search the finest-level cells that hold the
// ball of radius sqrt(tau0) (up to FINE_RINGS rings).  Unresolved queries are
// appended to the deferred list with md = -1.  (Clouds with pixel rays skip
// this phase: the window passes take every query.)
__global__ void __launch_bounds__(TILE_T) sor_knn_tile_kernel(const float* __restrict__ xyz,
                                                              const uint8_t* __restrict__ mask, int rows, int cols,
                                                              int k, Level g, GridStats* s, float* __restrict__ md_out,
                                                              unsigned* __restrict__ deferred) {
    extern __shared__ float4 tile_smem[];
    float4* cand = tile_smem;                  // TILE_MAX_CAND
    __shared__ int s_off[TILE_MAX_CELLS + 1];  // candidate offset of each box cell
    __shared__ float s_sv[TILE_T / 32 * SV_CAP];  // per-warp survivor lists
    __shared__ int s_nsv[TILE_T / 32];
    __shared__ unsigned s_ws[32];
    __shared__ int s_box[6];
    __shared__ float s_zc;
    __shared__ unsigned s_total;
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * TILE_X, y0 = blockIdx.y * TILE_Y;
    const int x = x0 + (tid % TILE_X), y = y0 + (tid / TILE_X);
    const bool in = x < cols && y < rows;
    const size_t i = in ? (size_t)y * cols + x : 0;
    const bool active = in && mask[i] && s->n_valid > k;
    if (in && !active) md_out[i] = 0.f;
    if (!__syncthreads_or(active)) return;  // the whole CTA leaves together
    const float ic = s->inv_cell[0], cell = s->cell[0];
    float qx = 0.f, qy = 0.f, qz = 0.f;
    int c[3] = {0, 0, 0};
    if (active) {
        qx = xyz[3 * i]; qy = xyz[3 * i + 1]; qz = xyz[3 * i + 2];
        cell_of(qx, qy, qz, ic, c[0], c[1], c[2]);
    }
    // window bound tau0 from the pixel neighbourhood (staged in cand; w = 0 marks invalid)
    for (int t = tid; t < WIN_W * WIN_H; t += TILE_T) {
        const int wx = x0 - WIN_R + t % WIN_W, wy = y0 - WIN_R + t / WIN_W;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (wx >= 0 && wx < cols && wy >= 0 && wy < rows) {
            const size_t j = (size_t)wy * cols + wx;
            if (mask[j]) v = make_float4(xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], 1.f);
        }
        cand[t] = v;
    }
    __syncthreads();
    float tau0 = INFINITY;
    if (active) {
        const int wc = (tid / TILE_X + WIN_R) * WIN_W + tid % TILE_X + WIN_R;
        int found = 0;
        float m = 0.f;
        for (int o = 0; o < WIN_N && found < k; o++) {
            const float4 p = cand[wc + c_spiral[o][1] * WIN_W + c_spiral[o][0]];
            if (p.w == 0.f) continue;
            const float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
            m = fmaxf(m, sqdist(dx, dy, dz));
            found++;
        }
        if (found == k) tau0 = m;
    }
    __syncthreads();
    // trimmed mean of the z cells: mean, then mean of those within 8 cells of it
    float n1 = block_reduce(active ? 1.f : 0.f, Add(), 0.f);
    float z1 = block_reduce(active ? (float)c[2] : 0.f, Add(), 0.f);
    if (tid == 0) s_zc = n1 > 0 ? z1 / n1 : 0.f;
    __syncthreads();
    bool near1 = active && fabsf((float)c[2] - s_zc) <= 8.f;
    float n2 = block_reduce(near1 ? 1.f : 0.f, Add(), 0.f);
    float z2 = block_reduce(near1 ? (float)c[2] : 0.f, Add(), 0.f);
    __syncthreads();
    if (tid == 0) s_zc = n2 > 0 ? z2 / n2 : s_zc;
    __syncthreads();
    const bool inbox = active && fabsf((float)c[2] - s_zc) <= 4.f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int lo = block_reduce(inbox ? c[a] : INT_MAX, Min(), INT_MAX);
        int hi = block_reduce(inbox ? c[a] : INT_MIN, Max(), INT_MIN);
        if (tid == 0) { s_box[a] = lo; s_box[3 + a] = hi; }
    }
    __syncthreads();
    const bool any = s_box[0] != INT_MAX;
    const int lo0 = s_box[0] - TILE_DILATE, lo1 = s_box[1] - TILE_DILATE, lo2 = s_box[2] - TILE_DILATE;
    const long long ex = any ? (long long)s_box[3] - s_box[0] + 1 + 2 * TILE_DILATE : 0;
    const long long ey = any ? (long long)s_box[4] - s_box[1] + 1 + 2 * TILE_DILATE : 0;
    const long long ez = any ? (long long)s_box[5] - s_box[2] + 1 + 2 * TILE_DILATE : 0;
    const long long V = ex * ey * ez;
    bool fast = any && V <= TILE_MAX_CELLS;  // uniform over the CTA
    if (fast) {
        // counting sort of the box's points by cell: count, scan, place
        for (int t = tid; t < V; t += TILE_T) {
            const int ix = lo0 + (int)(t % ex), iy = lo1 + (int)((t / ex) % ey), iz = lo2 + (int)(t / (ex * ey));
            const uint2 b = bucket(g, ix, iy, iz);
            int n_in = 0;
            for (unsigned u = b.x; u < b.x + b.y; u++) {
                const float4 p = __ldg(g.pts + u);
                int px, py, pz;
                cell_of(p.x, p.y, p.z, ic, px, py, pz);
                n_in += (px == ix && py == iy && pz == iz);
            }
            s_off[t] = n_in;
        }
        __syncthreads();
        unsigned v8[8], own = 0;
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int t = tid * 8 + u;
            v8[u] = t < V ? (unsigned)s_off[t] : 0u;
            own += v8[u];
        }
        const unsigned incl = block_scan_incl(own, s_ws);
        unsigned run = incl - own;
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int t = tid * 8 + u;
            if (t < V) s_off[t] = (int)run;
            run += v8[u];
        }
        if (tid == TILE_T - 1) {
            s_total = incl;
            s_off[V] = (int)incl;
        }
        __syncthreads();
        fast = s_total <= (unsigned)TILE_MAX_CAND;
        if (fast) {
            for (int t = tid; t < V; t += TILE_T) {
                const int ix = lo0 + (int)(t % ex), iy = lo1 + (int)((t / ex) % ey), iz = lo2 + (int)(t / (ex * ey));
                const uint2 b = bucket(g, ix, iy, iz);
                int pos = s_off[t];
                for (unsigned u = b.x; u < b.x + b.y; u++) {
                    const float4 p = __ldg(g.pts + u);
                    int px, py, pz;
                    cell_of(p.x, p.y, p.z, ic, px, py, pz);
                    if (px == ix && py == iy && pz == iz) cand[pos++] = p;
                }
            }
        }
        __syncthreads();
    }
    const int K1 = k + 1;
    const bool fq = active && fast && inbox;
    // margin for the float rounding of the cell mapping (|p| * 2^-23 << 1e-3 cell)
    const float margin = fmaxf(1e-3f * cell, 4e-7f * fmaxf(fabsf(qx), fmaxf(fabsf(qy), fabsf(qz))));
    float thr = -1.f;
    int bx0 = INT_MAX, by0 = INT_MAX, bz0 = INT_MAX, bx1 = INT_MIN, by1 = INT_MIN, bz1 = INT_MIN;
    if (fq) {
        float gmin = fminf(fminf(qx - lo0 * cell, (lo0 + ex) * cell - qx),
                           fminf(fminf(qy - lo1 * cell, (lo1 + ey) * cell - qy),
                                 fminf(qz - lo2 * cell, (lo2 + ez) * cell - qz)));
        gmin = fmaxf(gmin - margin, 0.f);
        // every point with d2 <= thr lies in the cells the ball of radius R touches
        thr = fminf(tau0, gmin * gmin);
        const float R = sqrtf(thr) + margin;
        bx0 = max(lo0, __float2int_rd((qx - R) * ic)); bx1 = min(lo0 + (int)ex - 1, __float2int_rd((qx + R) * ic));
        by0 = max(lo1, __float2int_rd((qy - R) * ic)); by1 = min(lo1 + (int)ey - 1, __float2int_rd((qy + R) * ic));
        bz0 = max(lo2, __float2int_rd((qz - R) * ic)); bz1 = min(lo2 + (int)ez - 1, __float2int_rd((qz + R) * ic));
    }
    // Warp-cooperative selection, one query at a time: the lanes split the
    // query's candidate cells, keep the squared distances within its bound in
    // the warp's survivor list, then drop the largest until k + 1 remain and
    // sum their roots in fixed point (the same bits on every path).
    //  - fast queries read the cell-sorted box in shared memory (consecutive
    //    lanes, consecutive candidates);
    //  - the others (and fast queries the box could not settle) search the
    //    rings of finest cells that hold the ball of their window bound tau0,
    //    one cell per lane from the global table;
    //  - what neither settles is deferred to the far search with md = -1.
    const unsigned full = 0xffffffffu;
    const int lane = tid & 31, wid = tid >> 5;
    float* sv = s_sv + wid * SV_CAP;
    bool done = false;
    // rings that hold every point within sqrt(tau0) of the query (|floor a - floor b| <= ceil |a - b|)
    int rr = INT_MAX;
    if (active && tau0 < INFINITY) rr = (int)ceilf((sqrtf(tau0) + margin) * ic);
    for (int pass = 0; pass < 2; pass++) {
        unsigned todo = __ballot_sync(full, pass == 0 ? fq : (active && !done && rr <= FINE_RINGS));
        while (todo) {
            const int q = __ffs(todo) - 1;
            todo &= todo - 1;
            const float Qx = __shfl_sync(full, qx, q), Qy = __shfl_sync(full, qy, q), Qz = __shfl_sync(full, qz, q);
            const float T = __shfl_sync(full, pass == 0 ? thr : tau0, q);
            int nsv = 0;
            if (pass == 0) {
                const int X0 = __shfl_sync(full, bx0, q), X1 = __shfl_sync(full, bx1, q);
                const int Y0 = __shfl_sync(full, by0, q), Y1 = __shfl_sync(full, by1, q);
                const int Z0 = __shfl_sync(full, bz0, q), Z1 = __shfl_sync(full, bz1, q);
                for (int iz = Z0; iz <= Z1; iz++)
                    for (int iy = Y0; iy <= Y1; iy++) {
                        const int row = (int)(((long long)(iz - lo2) * ey + (iy - lo1)) * ex) - lo0;
                        const int j0 = s_off[row + X0], j1 = s_off[row + X1 + 1];
                        for (int jb = j0; jb < j1; jb += 32) {
                            const int j = jb + lane;
                            float d2 = INFINITY;
                            if (j < j1) {
                                const float4 p = cand[j];
                                d2 = sqdist(p.x - Qx, p.y - Qy, p.z - Qz);
                            }
                            const bool keep = d2 <= T;
                            const unsigned b = __ballot_sync(full, keep);
                            const int pos = nsv + __popc(b & ((1u << lane) - 1u));
                            if (keep && pos < SV_CAP) sv[pos] = d2;
                            nsv += __popc(b);
                        }
                    }
            } else {
                const int C0 = __shfl_sync(full, c[0], q), C1 = __shfl_sync(full, c[1], q);
                const int C2 = __shfl_sync(full, c[2], q), R = __shfl_sync(full, rr, q);
                const int side = 2 * R + 1, ncell = side * side * side;
                if (lane == 0) s_nsv[wid] = 0;
                __syncwarp();
                for (int t = lane; t < ncell; t += 32) {
                    const int cx = C0 - R + t % side, cy = C1 - R + (t / side) % side, cz = C2 - R + t / (side * side);
                    const uint2 b = bucket(g, cx, cy, cz);
                    for (unsigned u = b.x; u < b.x + b.y; u++) {
                        const float4 p = __ldg(g.pts + u);
                        int px, py, pz;
                        cell_of(p.x, p.y, p.z, ic, px, py, pz);
                        if (px != cx || py != cy || pz != cz) continue;
                        const float d2 = sqdist(p.x - Qx, p.y - Qy, p.z - Qz);
                        if (d2 > T) continue;
                        const int pos = atomicAdd(&s_nsv[wid], 1);
                        if (pos < SV_CAP) sv[pos] = d2;
                    }
                }
                __syncwarp();
                nsv = s_nsv[wid];
            }
            __syncwarp();
            if (nsv < K1 || nsv > SV_CAP) continue;  // warp-uniform: not settled here
            // keys: squared-distance bits + 1 (non-negative floats order as unsigned); 0 = empty
            unsigned key[SV_CAP / 32];
#pragma unroll
            for (int r = 0; r < SV_CAP / 32; r++) {
                const int idx = lane + 32 * r;
                key[r] = idx < nsv ? __float_as_uint(sv[idx]) + 1u : 0u;
            }
            for (int m = nsv - K1; m > 0; m--) {
                unsigned lm = 0;
#pragma unroll
                for (int r = 0; r < SV_CAP / 32; r++) lm = max(lm, key[r]);
                const unsigned wm = __reduce_max_sync(full, lm);
                const unsigned own = __ballot_sync(full, lm == wm);
                if (lane == __ffs(own) - 1) {
                    bool gone = false;
#pragma unroll
                    for (int r = 0; r < SV_CAP / 32; r++)
                        if (!gone && key[r] == wm) { key[r] = 0u; gone = true; }
                }
            }
            unsigned lm = 0;
#pragma unroll
            for (int r = 0; r < SV_CAP / 32; r++) lm = max(lm, key[r]);
            const float vmax = __uint_as_float(__reduce_max_sync(full, lm) - 1u);
            const int e = root_exponent(vmax);
            const float sc = root_scale(e);
            unsigned part = 0;
#pragma unroll
            for (int r = 0; r < SV_CAP / 32; r++)
                if (key[r]) part += root_fixed(__uint_as_float(key[r] - 1u), sc);
            part = __reduce_add_sync(full, part);
            if (lane == q) {
                md_out[i] = fixed_mean(part, e, k);
                done = true;
            }
        }
    }
    if (active && !done) {
        md_out[i] = -1.f;
        const unsigned slot = atomicAdd(&s->n_deferred, 1u);
        deferred[slot] = (unsigned)i;
    }
}

// ------------------------------------------------ window fast path (SOR) ----
//
// An organised cloud from one camera keeps its neighbours close in the image:
// a point p seen along the ray of pixel b, and a query q near the ray of pixel
// a, satisfy |p - q| >= |q| sin(angle(a, b)) - dev(q) - dev(p), where dev is a
// point's distance from its own pixel ray.  For every pixel b outside the
// (2 WR + 1)^2 window around a, |b - a| >= WR + 1 pixels, and with the pinhole
// rays a = (u - cx, v - cy, f), |a x b| >= f |b - a| and |b| <= |a| + |b - a|,
// so sin(angle) >= f (WR + 1) / (|a| (|a| + WR + 1)).  A query whose k + 1
// nearest points inside its window lie within
//     |q| f (WR + 1) / (|a| (|a| + WR + 1)) - dev(q) - max dev
// has the same k + 1 nearest points in the whole cloud: its mean distance is
// exact from the window alone.  Inside the window the same bound holds with the
// largest dev of the block's staged points in place of the cloud's (points
// averaged across a depth edge lie far off their rays, but only near it), so
// the spiral stops at the radius that local bound gives and the cloud-wide
// maximum only has to clear the window's edge.  Queries the bounds do not
// certify go to the deferred list (md = -1) for the grid searches.

using zt::RayParams;
using zt::ray_dir;
using zt::ray_dev;
constexpr int WR = zt::SPIRAL_R;  // window half-size of the fast path
constexpr int WW = WT_X + 2 * WR, WH = WT_Y + 2 * WR;
constexpr int WN = zt::SPIRAL_N;
constexpr int WR2MAX = 2 * WR * WR;

// The window's pixel offsets ordered by length, then row, then column, as
// staged-tile offsets with their squared length, and per squared radius the
// number of offsets within it: a walk's stop radius becomes a loop limit.
struct WinSpiral {
    int ent[WN];             // (dy * WW + dx) & 0xffff | (dx^2 + dy^2) << 16
    short upto[WR2MAX + 1];  // offsets of squared length <= i
    constexpr WinSpiral() : ent(), upto() {
        int n = 0;
        for (int l = 1; l <= WR2MAX; l++)
            for (int dy = -WR; dy <= WR; dy++)
                for (int dx = -WR; dx <= WR; dx++)
                    if (dx * dx + dy * dy == l) ent[n++] = ((dy * WW + dx) & 0xffff) | (l << 16);
        int c = 0;
        for (int i = 0; i <= WR2MAX; i++) {
            while (c < WN && (ent[c] >> 16) <= i) c++;
            upto[i] = (short)c;
        }
    }
};
__constant__ WinSpiral c_win = WinSpiral();
constexpr WinSpiral k_win{};  // the same table at compile time
// tile offset of spiral entry O as a compile-time constant
template <int O>
__device__ __forceinline__ int win_off_c() {
    constexpr int v = (int)(short)(k_win.ent[O] & 0xffff);
    return v;
}
__device__ __forceinline__ int win_off(int o) { return (int)(short)(c_win.ent[o] & 0xffff); }
__device__ __forceinline__ int win_len2(int o) { return c_win.ent[o] >> 16; }
// offsets whose squared length is at most r2 (r2 >= 0 or +inf)
__device__ __forceinline__ int win_upto(float r2) { return r2 < (float)WR2MAX ? c_win.upto[(int)r2] : WN; }

// Per-thread max-heap of the K1 smallest squared distances seen so far, in
// column tid of a [K1][WT_T] shared array (conflict-free): the root is the
// current K1-th smallest, and a nearer point replaces it with one sift-down.
template <int KC>  // the heap size at compile time (0: K1)
struct WinHeap {
    float* L;
    int K1_;
    __device__ __forceinline__ int size() const { return KC ? KC : K1_; }
    __device__ __forceinline__ float& at(int j) { return L[j * WT_T]; }
    // places v at j, moving larger children up
    __device__ __forceinline__ void sift(int j, float v) {
        const int K1 = size();
#pragma unroll
        for (int lev = 0; lev < 6; lev++) {  // a heap of at most 64 entries is 6 levels deep
            int c = 2 * j + 1;
            if (c >= K1) break;
            float cv = at(c);
            if (c + 1 < K1) {
                const float c2 = at(c + 1);
                if (c2 > cv) {
                    cv = c2;
                    c++;
                }
            }
            if (!(cv > v)) break;
            at(j) = cv;
            j = c;
        }
        at(j) = v;
    }
    __device__ __forceinline__ void build() {
        for (int j = size() / 2 - 1; j >= 0; j--) sift(j, at(j));
    }
};

// A query the window pass cannot settle goes straight to the deferred list
// (md = -1) for the grid searches.
__device__ __forceinline__ void defer_query(GridStats* s, unsigned* deferred, float* md_out, size_t i) {
    md_out[i] = -1.f;
    deferred[atomicAdd(&s->n_deferred, 1u)] = (unsigned)i;
}

// The same with an upper bound on its (k + 1)-th smallest squared distance
// (md = MD_BOUND, the bound in `bound`): the grid searches start from it.
__device__ __forceinline__ void defer_query_bound(GridStats* s, unsigned* deferred, float* md_out, float* bound,
                                                  size_t i, float b) {
    bound[i] = b;
    md_out[i] = MD_BOUND;
    deferred[atomicAdd(&s->n_deferred, 1u)] = (unsigned)i;
}

// The heap's first K1T - 1 distances (heap slots K1T - 2 down to 0) from the
// first K1T - 1 spiral offsets, invalid pixels as +inf.
template <int K1T, int... O>
__device__ __forceinline__ void fill_first(WinHeap<K1T>& heap, const float4* W, int wc, float4 q,
                                           std::integer_sequence<int, O...>) {
    auto d2 = [&](const float4 p) { return p.w == 0.f ? INFINITY : sqdist(p.x - q.x, p.y - q.y, p.z - q.z); };
    ((heap.at(K1T - 2 - O) = d2(W[wc + win_off_c<O>()])), ...);
}

// K1T: k + 1 at compile time (0: from k)
template <int K1T>
__global__ void __launch_bounds__(WT_T) sor_window_kernel(const float* __restrict__ xyz,
                                                            const uint8_t* __restrict__ mask, int rows, int cols,
                                                            int k, RayParams rp, GridStats* __restrict__ s,
                                                            float* __restrict__ md_out,
                                                            unsigned* __restrict__ deferred,
                                                            float* __restrict__ bound) {
    extern __shared__ float4 win_smem[];
    float4* W = win_smem;                                      // WW x WH window, w = 1 valid
    float* Ls = reinterpret_cast<float*>(win_smem + WW * WH);  // (k + 1) x WT_T heaps
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * WT_X, y0 = blockIdx.y * WT_Y;
    __shared__ unsigned warp_dev[WT_T / 32];
    unsigned tdev = 0u;  // largest dev of this thread's staged points (float bits, >= 0)
#pragma unroll
    for (int t = tid; t < WW * WH; t += WT_T) {
        const int wx = x0 - WR + t % WW, wy = y0 - WR + t / WW;
        // invalid and off-image pixels: NaN coordinates (their squared distance
        // never passes a comparison), w = 0
        const float nan = __int_as_float(0x7fc00000);
        float4 v = make_float4(nan, nan, nan, 0.f);
        if (wx >= 0 && wx < cols && wy >= 0 && wy < rows) {
            const size_t j = (size_t)wy * cols + wx;
            if (mask[j]) {
                v = make_float4(xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], 1.f);
                float ax, ay, az;
                ray_dir(rp, wx, wy, ax, ay, az);
                const float d = ray_dev(v.x, v.y, v.z, ax, ay, az);
                tdev = max(tdev, __float_as_uint(d == d ? d : INFINITY));  // NaN counts as unbounded
            }
        }
        W[t] = v;
    }
    tdev = __reduce_max_sync(0xffffffffu, tdev);
    if ((tid & 31) == 0) warp_dev[tid >> 5] = tdev;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < WT_T / 32; j++) tdev = max(tdev, warp_dev[j]);
    const int tx = tid % WT_X, ty = tid / WT_X;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= cols || y >= rows) return;  // no block-wide synchronisation below
    const size_t i = (size_t)y * cols + x;
    if (!mask[i] || !(s->n_valid > k)) {
        md_out[i] = 0.f;
        return;
    }
    const int wc = (ty + WR) * WW + tx + WR;
    const float4 q = W[wc];
    const int K1 = K1T ? K1T : k + 1;
    // the query and its first k valid window pixels in spiral order fill the
    // heap; its root (their largest distance) is the first bound.  They fill
    // it from the last slot backwards: the spiral meets pixels roughly by
    // increasing distance, so the array is close to descending -- close to a
    // max-heap already -- and the build sifts little.  (Only the multiset of
    // the heap's values matters: the root is its maximum, a replacement drops
    // the maximum, and the mean distance is an order-free fixed-point sum.)
    WinHeap<K1T> heap{Ls + tid, K1};
    heap.at(K1 - 1) = 0.f;
    int o = 0;
    if constexpr (K1T > 0) {
        // k known at compile time: the first k spiral offsets fill the heap
        // straight from constant tile offsets, an invalid pixel as +inf (the
        // largest value: the first valid distance to come replaces it, and a
        // heap still holding one at the end means fewer than k + 1 points)
        fill_first<K1T>(heap, W, wc, q, std::make_integer_sequence<int, K1T - 1>{});
        o = K1T - 1;
    } else {
        int cnt = 1;
        for (; o < WN && cnt < K1; o++) {
            const float4 p = W[wc + win_off(o)];
            if (p.w == 0.f) continue;
            heap.at(K1 - 1 - cnt++) = sqdist(p.x - q.x, p.y - q.y, p.z - q.z);
        }
        if (cnt < K1) {
            defer_query(s, deferred, md_out, i);
            return;
        }
    }
    heap.build();
    float thr = heap.at(0);
    // bound(r) = C r / (an + r): no point of a pixel at distance >= r from the
    // query's lies nearer than bound(r) - dev (slack: float rounding, 1e-5 |q|)
    float ax, ay, az;
    ray_dir(rp, x, y, ax, ay, az);
    const float an = sqrtf(fmaf(ax, ax, fmaf(ay, ay, az * az)));
    const float qn = sqrtf(fmaf(q.x, q.x, fmaf(q.y, q.y, q.z * q.z)));
    const float C = qn * rp.f / an;
    const float dev_q = ray_dev(q.x, q.y, q.z, ax, ay, az) + 1e-5f * qn;
    const float dev = dev_q + __uint_as_float(tdev);                    // window pixels
    const float dev_out = dev_q + __uint_as_float(s->ray_dev_bits);     // pixels outside it
    // squared pixel distance beyond which every window point is farther than
    // sqrt(thr): C r / (an + r) > sqrt(thr) + dev  <=>  r > (sqrt(thr) + dev) an / (C - sqrt(thr) - dev).
    // Approximate arithmetic: the stop only ends the walk; the exact
    // certificate below decides whether the window result stands.
    auto stop_r2 = [&](float thr) {
        const float sd = root_approx(thr) + dev;
        if (!(C > sd)) return INFINITY;
        const float r = __fdividef(sd * an, C - sd);
        return r * r;
    };
    // the spiral runs by increasing length: once past the stop distance, the
    // rest of the window (and everything outside it) is provably farther
    int lim = win_upto(stop_r2(thr));
    for (; o < lim; o++) {
        const float4 p = W[wc + win_off(o)];
        const float d2 = sqdist(p.x - q.x, p.y - q.y, p.z - q.z);
        if (d2 < thr) {  // false for an invalid pixel (NaN)
            heap.sift(0, d2);
            thr = heap.at(0);
            lim = win_upto(stop_r2(thr));
        }
    }
    if (!(thr < INFINITY)) {  // fewer than k + 1 points in the whole window
        defer_query(s, deferred, md_out, i);
        return;
    }
    // every window offset not visited is at least as long as offset o
    const float rbreak = o < WN ? fminf(sqrtf((float)win_len2(o)), (float)(WR + 1)) : (float)(WR + 1);
    const float kth = thr;
    // certificate: every window pixel not visited is at least rbreak away, and
    // every pixel outside the window at least WR + 1
    const float rk = sqrtf(kth), ro = (float)(WR + 1);
    const bool ok = C * rbreak / (an + rbreak) - dev > rk && C * ro / (an + ro) - dev_out > rk;
    if (!ok) {
        // the heap holds k + 1 distances of cloud points (the query's own 0
        // among them): its root bounds the (k + 1)-th smallest from above
        defer_query_bound(s, deferred, md_out, bound, i, kth);
        return;
    }
    const int e = root_exponent(kth);
    const float sc = root_scale(e);
    unsigned sum = 0;
#pragma unroll
    for (int j = 0; j < (K1T ? K1T : 64); j++) {
        if (j >= K1) break;
        sum += root_fixed(heap.at(j), sc);
    }
    md_out[i] = fixed_mean(sum, e, k);
}

constexpr int FW_CAP = 256;  // far search: list entries per warp (8 per lane)

// Smallest list value v with at least K entries <= v (entries: lane j holds
// keys[r] for r < 8, 0xffffffff = empty; keys are non-negative float bits).
__device__ __forceinline__ unsigned warp_kth_key(const unsigned (&keys)[FW_CAP / 32], int K) {
    unsigned lo = 0u, hi = 0x7f800000u;  // +inf bits
    while (lo < hi) {
        const unsigned mid = lo + ((hi - lo) >> 1);
        int c = 0;
#pragma unroll
        for (int r = 0; r < FW_CAP / 32; r++) c += keys[r] <= mid;
        c = __reduce_add_sync(0xffffffffu, c);
        if (c >= K) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// Occupied cells of the coarse (dense) level: (cell index, offset, count).
__global__ void occupied_cells_kernel(const uint2* __restrict__ tab, GridStats* s, uint4* __restrict__ occ) {
    const unsigned used = (unsigned)s->dims[0] * (unsigned)s->dims[1] * (unsigned)s->dims[2];
    unsigned h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= used) return;
    const uint2 e = tab[h];
    if (e.y == 0) return;
    occ[atomicAdd(&s->n_occ, 1u)] = make_uint4(h, e.x, e.y, 0u);
}

// Squared distance from q to a coarse cell's cube, the cube grown by a margin
// that covers the float rounding of the cell mapping.
__device__ __forceinline__ float cell_box_d2(unsigned idx, const GridStats* __restrict__ s, float qx, float qy,
                                             float qz, float margin) {
    const unsigned nx = (unsigned)s->dims[0], ny = (unsigned)s->dims[1];
    const float c = s->cell[1];
    const float lx = s->org[0] + (float)(idx % nx) * c - margin;
    const float ly = s->org[1] + (float)((idx / nx) % ny) * c - margin;
    const float lz = s->org[2] + (float)(idx / (nx * ny)) * c - margin;
    const float w = c + 2.f * margin;
    float ex = fmaxf(fmaxf(lx - qx, qx - (lx + w)), 0.f);
    float ey = fmaxf(fmaxf(ly - qy, qy - (ly + w)), 0.f);
    float ez = fmaxf(fmaxf(lz - qz, qz - (lz + w)), 0.f);
    return ex * ex + ey * ey + ez * ez;
}

// Phase 2: one warp per deferred point on the coarse (dense) level, ring by
// ring of cells around the query's cell: ring r holds every cell at Chebyshev
// distance r, all at least (r - 1) cells away.  The warp keeps the squared
// distances within the bound (the (k + 1)-th smallest held) in its list and
// stops once the next ring lies beyond the bound.  Queries still open after RING_MAX rings, or whose ties overflow the
// list, go to the hard list (md = MD_BOUND with a valid bound in the bound
// array, or -1).  Work is handed out through an atomic counter.
__global__ void __launch_bounds__(P2_WARPS * 32) sor_knn_far_kernel(const float* __restrict__ xyz, int k,
                                                                     GridStats* s,
                                                                     const uint2* __restrict__ tab1,
                                                                     const float4* __restrict__ pts,
                                                                     const unsigned* __restrict__ deferred,
                                                                     float* __restrict__ md_out,
                                                                     float* __restrict__ bound,
                                                                     unsigned* __restrict__ hard) {
    __shared__ float lst[P2_WARPS][FW_CAP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int K1 = k + 1;
    float* lw = lst[w];
    const unsigned nd = s->n_deferred;
    for (;;) {
        unsigned item = 0;
        if (lane == 0) item = atomicAdd(&s->p2_next, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nd) break;
        const unsigned i = deferred[item];
        const float qx = xyz[3 * i], qy = xyz[3 * i + 1], qz = xyz[3 * i + 2];
        // the cell mapping (x - org) * inv_cell and the cube corners org + i * cell
        // round by a few ulps of the largest coordinate
        const float margin = 1e-4f * s->cell[1] + 4e-6f * s->amax;
        bool done = false;
        float thr = md_out[i] == MD_BOUND ? bound[i] : INFINITY;
        float fmd = 0.f;
        bool ring_done = false;
        {
            int n = 0;
            bool overflow = false;
            auto tighten = [&]() {
                __syncwarp();
                unsigned keys[FW_CAP / 32];
#pragma unroll
                for (int q = 0; q < FW_CAP / 32; q++) {
                    const int e = lane + 32 * q;
                    keys[q] = e < n ? __float_as_uint(lw[e]) : 0xffffffffu;
                }
                const unsigned kk = warp_kth_key(keys, K1);
                thr = fminf(thr, __uint_as_float(kk));
                __syncwarp();
                int m = 0;
#pragma unroll
                for (int q = 0; q < FW_CAP / 32; q++) {
                    const bool kp = keys[q] <= __float_as_uint(thr);
                    const unsigned bb = __ballot_sync(0xffffffffu, kp);
                    if (kp) lw[m + __popc(bb & ((1u << lane) - 1u))] = __uint_as_float(keys[q]);
                    m += __popc(bb);
                }
                n = m;
                __syncwarp();
            };
            const float c1 = s->cell[1], ic1 = s->inv_cell[1];
            const int nx = s->dims[0], ny = s->dims[1], nz = s->dims[2];
            const int qcx = min(max(__float2int_rd((qx - s->org[0]) * ic1), 0), nx - 1);
            const int qcy = min(max(__float2int_rd((qy - s->org[1]) * ic1), 0), ny - 1);
            const int qcz = min(max(__float2int_rd((qz - s->org[2]) * ic1), 0), nz - 1);
            for (int r = 0; r <= RING_MAX && !overflow; r++) {
                if (r >= 1 && thr < INFINITY) {
                    const float gap = (float)(r - 1) * c1 - margin;
                    if (gap > 0.f && gap * gap > thr) {
                        done = n >= K1;
                        break;
                    }
                }
                const int side = 2 * r + 1, ncell = side * side * side;
                for (int t0 = 0; t0 < ncell && !overflow; t0 += 32) {
                    const int t = t0 + lane;
                    bool take = false;
                    uint2 e = make_uint2(0u, 0u);
                    if (t < ncell) {
                        const int dx = t % side - r, dy = (t / side) % side - r, dz = t / (side * side) - r;
                        const int cheb = max(abs(dx), max(abs(dy), abs(dz)));
                        const int ix = qcx + dx, iy = qcy + dy, iz = qcz + dz;
                        if (cheb == r && ix >= 0 && ix < nx && iy >= 0 && iy < ny && iz >= 0 && iz < nz) {
                            const unsigned idx = ((unsigned)iz * (unsigned)ny + (unsigned)iy) * (unsigned)nx + (unsigned)ix;
                            e = __ldg(tab1 + idx);
                            take = e.y > 0u && cell_box_d2(idx, s, qx, qy, qz, margin) <= thr;
                        }
                    }
                    unsigned m = __ballot_sync(0xffffffffu, take);
                    while (m && !overflow) {
                        const int b = __ffs(m) - 1;
                        m &= m - 1;
                        const unsigned first = __shfl_sync(0xffffffffu, e.x, b);
                        const unsigned end = first + __shfl_sync(0xffffffffu, e.y, b);
                        // 128 points a step: four loads in flight per lane
                        for (unsigned u0 = first; u0 < end; u0 += 128) {
                            if (n > FW_CAP - 128) {
                                tighten();
                                if (n > FW_CAP - 128) {  // too many ties to hold
                                    overflow = true;
                                    break;
                                }
                            }
                            float d2[4];
#pragma unroll
                            for (int r = 0; r < 4; r++) {
                                const unsigned u = u0 + 32u * r + lane;
                                d2[r] = INFINITY;
                                if (u < end) {
                                    const float4 p = __ldg(pts + u);
                                    d2[r] = sqdist(p.x - qx, p.y - qy, p.z - qz);
                                }
                            }
#pragma unroll
                            for (int r = 0; r < 4; r++) {
                                const bool keep = d2[r] < INFINITY && d2[r] <= thr;
                                const unsigned bb = __ballot_sync(0xffffffffu, keep);
                                if (keep) lw[n + __popc(bb & ((1u << lane) - 1u))] = d2[r];
                                n += __popc(bb);
                            }
                            if (thr == INFINITY && n >= 2 * K1) tighten();
                        }
                    }
                }
            }
            if (done) {
                __syncwarp();
                unsigned keys[FW_CAP / 32];
#pragma unroll
                for (int q = 0; q < FW_CAP / 32; q++) {
                    const int e2 = lane + 32 * q;
                    keys[q] = e2 < n ? __float_as_uint(lw[e2]) : 0xffffffffu;
                }
                const unsigned kk = warp_kth_key(keys, K1);
                const float kv = __uint_as_float(kk);
                const int ee = root_exponent(kv);
                const float sc = root_scale(ee);
                unsigned part = 0;
                int below = 0;
#pragma unroll
                for (int q = 0; q < FW_CAP / 32; q++)
                    if (keys[q] < kk) {
                        part += root_fixed(__uint_as_float(keys[q]), sc);
                        below++;
                    }
                part = __reduce_add_sync(0xffffffffu, part);
                below = __reduce_add_sync(0xffffffffu, below);
                part += (unsigned)(K1 - below) * root_fixed(kv, sc);
                fmd = fixed_mean(part, ee, k);
                ring_done = true;
            }
        }
        if (lane == 0) {
            if (ring_done) {
                md_out[i] = fmd;
            } else {
                // a finite bound is valid: the second pass's, or a (k + 1)-th smallest held
                hard[atomicAdd(&s->n_hard, 1u)] = i;
                md_out[i] = thr < INFINITY ? MD_BOUND : -1.f;
                bound[i] = thr;
            }
        }
        __syncwarp();
    }
}

// Farthest point of a coarse cell's cube (grown by the margin) from q, squared.
__device__ __forceinline__ float cell_far_d2(unsigned idx, const GridStats* __restrict__ s, float qx, float qy,
                                             float qz, float margin) {
    const unsigned nx = (unsigned)s->dims[0], ny = (unsigned)s->dims[1];
    const float c = s->cell[1];
    const float lx = s->org[0] + (float)(idx % nx) * c - margin;
    const float ly = s->org[1] + (float)((idx / nx) % ny) * c - margin;
    const float lz = s->org[2] + (float)(idx / (nx * ny)) * c - margin;
    const float w = c + 2.f * margin;
    const float ex = fmaxf(fabsf(qx - lx), fabsf(lx + w - qx));
    const float ey = fmaxf(fabsf(qy - ly), fabsf(ly + w - qy));
    const float ez = fmaxf(fabsf(qz - lz), fabsf(lz + w - qz));
    return ex * ex + ey * ey + ez * ez;
}

// Phase 3: one CTA per hard query over the coarse level's occupied cells.  The
// bound starts at the farthest corner of the nearest-cornered cell holding
// K1 points (or the query's own bound).  Warps take cells one at a time and
// skip those whose cube lies beyond the CTA's bound; each keeps in its list
// the distances below its bound and counts those equal to it, and a list of K1
// or more entries tightens the bound to their K1-th smallest, shared through
// an atomic minimum.  Lists then hold every point below the final bound, plus
// the counted ties: one warp selects the K1 smallest from them.
constexpr int HARD_T = 1024, HARD_W = HARD_T / 32;
__global__ void __launch_bounds__(HARD_T) sor_hard_kernel(const float* __restrict__ xyz, int k,
                                                          const GridStats* __restrict__ s,
                                                          const uint4* __restrict__ occ,
                                                          const float4* __restrict__ pts,
                                                          const unsigned* __restrict__ hard,
                                                          float* __restrict__ md_out,
                                                          const float* __restrict__ bound,
                                                          uint32_t* __restrict__ err) {
    __shared__ float hl[HARD_W][FW_CAP];
    __shared__ unsigned s_thr, s_next, s_ties;
    __shared__ unsigned s_wmin[HARD_W];
    __shared__ int s_n[HARD_W];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int K1 = k + 1;
    const unsigned nh = s->n_hard, nocc = s->n_occ;
    const float margin = 1e-4f * s->cell[1] + 4e-6f * s->amax;
    float* lw = hl[w];
    for (unsigned item = blockIdx.x; item < nh; item += gridDim.x) {
        const unsigned i = hard[item];
        const float qx = xyz[3 * i], qy = xyz[3 * i + 1], qz = xyz[3 * i + 2];
        const float own = md_out[i] == MD_BOUND ? bound[i] : INFINITY;
        // a cell of K1 points lies wholly within its farthest corner
        unsigned fb = 0x7f800000u;  // +inf bits; non-negative floats order as unsigned
        for (unsigned j = tid; j < nocc; j += HARD_T) {
            const uint4 o = __ldg(occ + j);
            if (o.z >= (unsigned)K1) fb = min(fb, __float_as_uint(cell_far_d2(o.x, s, qx, qy, qz, margin) * 1.00001f));
        }
        fb = __reduce_min_sync(0xffffffffu, fb);
        if (lane == 0) s_wmin[w] = fb;
        if (tid == 0) {
            s_next = 0u;
            s_ties = 0u;
        }
        __syncthreads();
        if (tid == 0) {
            unsigned m = __float_as_uint(own);
            for (int j = 0; j < HARD_W; j++) m = min(m, s_wmin[j]);
            s_thr = m;
        }
        __syncthreads();
        float thr = __uint_as_float(s_thr);
        int n = 0;      // list entries (all below thr)
        unsigned tie = 0u;  // points at exactly thr
        auto tighten = [&]() {
            __syncwarp();
            unsigned keys[FW_CAP / 32];
#pragma unroll
            for (int q = 0; q < FW_CAP / 32; q++) {
                const int e = lane + 32 * q;
                keys[q] = e < n ? __float_as_uint(lw[e]) : 0xffffffffu;
            }
            if (n < K1) return;  // warp-uniform; the K1-th is thr itself or unknown
            const unsigned kk = warp_kth_key(keys, K1);  // below thr
            thr = __uint_as_float(kk);
            int m = 0;
            unsigned t = 0u;
            __syncwarp();
#pragma unroll
            for (int q = 0; q < FW_CAP / 32; q++) {
                const bool kp = keys[q] < kk;
                const unsigned bb = __ballot_sync(0xffffffffu, kp);
                if (kp) lw[m + __popc(bb & ((1u << lane) - 1u))] = __uint_as_float(keys[q]);
                m += __popc(bb);
                t += __popc(__ballot_sync(0xffffffffu, keys[q] == kk));
            }
            n = m;
            tie = t;
            if (lane == 0) atomicMin(&s_thr, kk);
            __syncwarp();
        };
        for (;;) {
            unsigned j = 0;
            if (lane == 0) j = atomicAdd(&s_next, 1u);
            j = __shfl_sync(0xffffffffu, j, 0);
            if (j >= nocc) break;
            const float shared_thr = __uint_as_float(*(volatile unsigned*)&s_thr);
            if (shared_thr < thr) {  // another warp's bound: entries at or above it go
                thr = shared_thr;
                int m = 0;
                __syncwarp();
                for (int q0 = 0; q0 < n; q0 += 32) {
                    const int e = q0 + lane;
                    const float v = e < n ? lw[e] : INFINITY;
                    const bool kp = v < thr;
                    const unsigned bb = __ballot_sync(0xffffffffu, kp);
                    __syncwarp();
                    if (kp) lw[m + __popc(bb & ((1u << lane) - 1u))] = v;
                    m += __popc(bb);
                }
                n = m;
                tie = 0u;
                __syncwarp();
            }
            const uint4 o = __ldg(occ + j);
            if (cell_box_d2(o.x, s, qx, qy, qz, margin) > thr) continue;
            const unsigned end = o.y + o.z;
            for (unsigned u0 = o.y; u0 < end; u0 += 128) {
                if (n > FW_CAP - 128) tighten();  // n < K1 after it: room for 128
                float d2[4];
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    const unsigned u = u0 + 32u * r + lane;
                    d2[r] = __int_as_float(0x7fffffff);  // NaN: neither below nor equal to the bound
                    if (u < end) {
                        const float4 p = __ldg(pts + u);
                        d2[r] = sqdist(p.x - qx, p.y - qy, p.z - qz);
                    }
                }
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    const bool kp = d2[r] < thr;
                    const unsigned bb = __ballot_sync(0xffffffffu, kp);
                    if (kp) lw[n + __popc(bb & ((1u << lane) - 1u))] = d2[r];
                    n += __popc(bb);
                    tie += __popc(__ballot_sync(0xffffffffu, d2[r] == thr));
                }
                if (n >= 2 * K1 && !(thr < INFINITY)) tighten();
            }
            if (n >= K1) tighten();
        }
        __syncthreads();
        // final bound: entries below it stay; entries equal to it and the
        // ties of the warps that hold it are counted
        const float fin = __uint_as_float(s_thr);
        {
            unsigned t = thr == fin ? tie : 0u;
            int m = 0;
            __syncwarp();
            for (int q0 = 0; q0 < n; q0 += 32) {
                const int e = q0 + lane;
                const float v = e < n ? lw[e] : __int_as_float(0x7fffffff);
                const bool kp = v < fin;
                const unsigned bb = __ballot_sync(0xffffffffu, kp);
                t += __popc(__ballot_sync(0xffffffffu, v == fin));
                __syncwarp();
                if (kp) lw[m + __popc(bb & ((1u << lane) - 1u))] = v;
                m += __popc(bb);
            }
            if (lane == 0) {
                s_n[w] = m;
                atomicAdd(&s_ties, t);
            }
        }
        __syncthreads();
        if (w == 0) {
            // the K1-th smallest of the lists' entries and the ties (at fin):
            // binary search on the key bits
            const unsigned ties = s_ties;
            int total = 0;
            for (int v = 0; v < HARD_W; v++) total += s_n[v];
            unsigned lo = 0u, hi = __float_as_uint(fin);
            if (!(fin < INFINITY) || total + (int)ties < K1) {
                if (lane == 0) {
                    atomicOr(err, 0x10u);  // fewer than k + 1 points reachable
                    md_out[i] = 0.f;
                }
            } else {
                if (total >= K1) {
                    while (lo < hi) {
                        const unsigned mid = lo + ((hi - lo) >> 1);
                        int c = 0;
                        for (int v = 0; v < HARD_W; v++)
                            for (int e = lane; e < s_n[v]; e += 32) c += __float_as_uint(hl[v][e]) <= mid;
                        c = __reduce_add_sync(0xffffffffu, c);
                        if (c >= K1) hi = mid;
                        else lo = mid + 1u;
                    }
                }
                const unsigned kk = hi;  // the K1-th (fin when fewer than K1 entries lie below it)
                const float kv = __uint_as_float(kk);
                const int ee = root_exponent(kv);
                const float sc = root_scale(ee);
                unsigned part = 0u;
                int below = 0;
                for (int v = 0; v < HARD_W; v++)
                    for (int e = lane; e < s_n[v]; e += 32) {
                        const unsigned key = __float_as_uint(hl[v][e]);
                        if (key < kk) {
                            part += root_fixed(hl[v][e], sc);
                            below++;
                        }
                    }
                part = __reduce_add_sync(0xffffffffu, part);
                below = __reduce_add_sync(0xffffffffu, below);
                part += (unsigned)(K1 - below) * root_fixed(kv, sc);
                if (lane == 0) md_out[i] = fixed_mean(part, ee, k);
            }
        }
        __syncthreads();  // the lists are reused by the next query
    }
}

// Per-block sums of the mean distances (valid pixels, grid-stride over a fixed
// number of blocks, so each thread's share is fixed), then a fixed-order total.
// FP64 runs at a small fraction of the FP32 rate: two double adds per point.
// A thread's terms add in FP32 with a compensation term (Neumaier: the sum is
// exact to ~2^-24 of its size, like a double sum of these few terms) and go to
// FP64 once; no FP64 operation per point.
__device__ __forceinline__ void comp_add(float& sum, float& comp, float x) {
    const float t = sum + x;
    comp += fabsf(sum) >= fabsf(x) ? (sum - t) + x : (x - t) + sum;
    sum = t;
}

__global__ void sor_partial_kernel(const uint8_t* __restrict__ mask, const float* __restrict__ md, size_t n,
                                   double* __restrict__ part) {
    float as = 0.f, ac = 0.f, bs = 0.f, bc = 0.f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (!mask[i]) continue;
        const float m = md[i];
        comp_add(as, ac, m);
        comp_add(bs, bc, m * m);  // PCL: float square, double sum
    }
    double a = block_reduce((double)as + (double)ac, Add(), 0.0);
    double b = block_reduce((double)bs + (double)bc, Add(), 0.0);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

// Totals, then the threshold mean + std_mul * stddev once; the classifier
// compares the float mean distances with thr_f, the largest float <= thr, which
// decides exactly as (double)md > thr.
__global__ void sor_stats_kernel(const double* __restrict__ part, int nb, int k, double std_mul, GridStats* s) {
    double a = 0, b = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    a = block_reduce(a, Add(), 0.0);
    b = block_reduce(b, Add(), 0.0);
    if (threadIdx.x == 0) {
        s->md_sum = a;
        s->md_sq = b;
        const double nv = s->n_valid;
        s->keep_all = nv <= k;  // too few points for a k-neighbourhood: nothing is removed
        if (!s->keep_all) {
            const double mean = a / nv;
            const double var = (b - a * a / nv) / (nv - 1);
            s->thr = mean + std_mul * sqrt(var);
            s->thr_f = __double2float_rd(s->thr);
        }
    }
}

__global__ void sor_classify_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                    const GridStats* __restrict__ s, const float* __restrict__ md,
                                    uint8_t* __restrict__ mask_out, float* __restrict__ xyz_out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool keep = mask[i] && (s->keep_all || !(md[i] > s->thr_f));
    mask_out[i] = keep ? 1 : 0;
    if (xyz_out) {
        xyz_out[3 * i] = keep ? xyz[3 * i] : 0.f;
        xyz_out[3 * i + 1] = keep ? xyz[3 * i + 1] : 0.f;
        xyz_out[3 * i + 2] = keep ? xyz[3 * i + 2] : 0.f;
    }
}

// Radius-3-sigma Gaussian: out = p + sum w (q - p) / sum w over the 27 cells of
// side 3 sigma around p; buckets are index-sorted, so the FP32 sums are
// deterministic.
// Metric Gaussian by the window fast path: the points within r of a query,
// summed row by row over the disk of its window out to the pixel distance
// beyond which the ray bound puts every point farther than r (see
// sor_window_kernel); the others are marked -2 in `pending` for
// metric_gaussian_kernel.
constexpr int WRG = WR;
constexpr int GW = WT_X + 2 * WRG, GH = WT_Y + 2 * WRG;

__global__ void __launch_bounds__(WT_T) mg_window_kernel(const float* __restrict__ xyz,
                                                           const uint8_t* __restrict__ mask, int rows, int cols,
                                                           float r, float inv2s2, RayParams rp,
                                                           GridStats* __restrict__ s,
                                                           const unsigned* __restrict__ tile_dev,
                                                           float* __restrict__ pending, float* __restrict__ out) {
    __shared__ float4 W[GW * GH];
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * WT_X, y0 = blockIdx.y * WT_Y;
#pragma unroll
    for (int t = tid; t < GW * GH; t += WT_T) {
        const int wx = x0 - WRG + t % GW, wy = y0 - WRG + t / GW;
        // invalid and off-image pixels are NaN: their distance test fails
        const float nan = __int_as_float(0x7fc00000);
        float4 v = make_float4(nan, nan, nan, 0.f);
        if (wx >= 0 && wx < cols && wy >= 0 && wy < rows) {
            const size_t j = (size_t)wy * cols + wx;
            if (mask[j]) v = make_float4(xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], 1.f);
        }
        W[t] = v;
    }
    __syncthreads();
    const int tx = tid % WT_X, ty = tid / WT_X;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= cols || y >= rows) return;
    const size_t i = (size_t)y * cols + x;
    const float4 q = W[(ty + WRG) * GW + tx + WRG];
    if (!mask[i]) {  // invalid points pass through
        out[3 * i] = xyz[3 * i];
        out[3 * i + 1] = xyz[3 * i + 1];
        out[3 * i + 2] = xyz[3 * i + 2];
        pending[i] = 0.f;
        return;
    }
    float ax, ay, az;
    ray_dir(rp, x, y, ax, ay, az);
    const float an = sqrtf(fmaf(ax, ax, fmaf(ay, ay, az * az)));
    const float qn = sqrtf(fmaf(q.x, q.x, fmaf(q.y, q.y, q.z * q.z)));
    const float C = qn * rp.f / an;
    // the window's pixels are the 3 x 3 tiles around this one (halo 7 < 8):
    // their points lie within the largest of those tiles' ray distances;
    // pixels outside the window within the largest of all
    unsigned td = 0u;
    for (int by = max(0, (int)blockIdx.y - 1); by <= min((int)gridDim.y - 1, (int)blockIdx.y + 1); by++)
        for (int bx = max(0, (int)blockIdx.x - 1); bx <= min((int)gridDim.x - 1, (int)blockIdx.x + 1); bx++)
            td = max(td, tile_dev[(size_t)by * gridDim.x + bx]);
    const float dev_q = ray_dev(q.x, q.y, q.z, ax, ay, az) + 1e-5f * qn;
    const float dev = dev_q + __uint_as_float(td);
    const float dev_out = dev_q + __uint_as_float(s->ray_dev_bits);
    // window pixels farther than rs from the query hold no point within r,
    // and neither does any pixel outside the window (at least WRG + 1 away)
    const float sd = r + dev;
    const float rs = C > sd ? sd * an / (C - sd) : INFINITY;
    const float ro = (float)(WRG + 1);
    if (!(rs < ro) || !(C * ro / (an + ro) - dev_out > r)) {
        pending[i] = -2.f;
        atomicAdd(&s->n_pending, 1u);  // the grid gets built
        return;
    }
    const float r2 = r * r;
    const int wc = (ty + WRG) * GW + tx + WRG;
    // The disk of pixels within rs, row by row (the query itself included:
    // offset 0, weight exactly 1); w = 2^(d2 kq), kq = -log2(e) / (2 s^2)
    const float kq = -1.44269504088896341f * inv2s2;
    float sx = 0.f, sy = 0.f, sz = 0.f, sw = 0.f;
    const int R2 = (int)(rs * rs);  // offsets with dx^2 + dy^2 <= R2 (< (WRG + 1)^2)
#pragma unroll 1
    for (int dy = -WRG; dy <= WRG; dy++) {
        const int rem = R2 - dy * dy;
        if (rem < 0) continue;
        // exact floor of the root: a root of a non-square below 64 lies at
        // least 0.06 from an integer, far beyond the float error
        const int w = min((int)sqrtf((float)rem), WRG);
        const float4* row = W + wc + dy * GW;
#pragma unroll 2
        for (int dx = -w; dx <= w; dx++) {
            const float4 p = row[dx];
            const float ex = p.x - q.x, ey = p.y - q.y, ez = p.z - q.z;
            const float d2 = sqdist(ex, ey, ez);
            if (!(d2 <= r2)) continue;  // also every invalid pixel (NaN)
            float wt;
            asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(wt) : "f"(d2 * kq));
            sx = fmaf(wt, ex, sx); sy = fmaf(wt, ey, sy); sz = fmaf(wt, ez, sz);
            sw += wt;
        }
    }
    const float iw = 1.0f / sw;
    out[3 * i] = q.x + sx * iw;
    out[3 * i + 1] = q.y + sy * iw;
    out[3 * i + 2] = q.z + sz * iw;
    pending[i] = 0.f;
}

__device__ __forceinline__ void metric_gaussian_point(const float* __restrict__ xyz, const uint8_t* __restrict__ mask,
                                                      size_t i, float r2, float inv2s2, const Level& g,
                                                      const GridStats* __restrict__ s,
                                                      const float* __restrict__ pending, float* __restrict__ out) {
    if (pending && pending[i] != -2.f) return;  // settled by the window pass
    const float qx = xyz[3 * i], qy = xyz[3 * i + 1], qz = xyz[3 * i + 2];
    if (!mask[i]) {
        out[3 * i] = qx; out[3 * i + 1] = qy; out[3 * i + 2] = qz;
        return;
    }
    const float ic = s->inv_cell[0];
    int cx, cy, cz;
    cell_of(qx, qy, qz, ic, cx, cy, cz);
    // fixed-point sums (each term rounded on its own): the result does not
    // depend on the order the buckets list their points in
    const float r = sqrtf(r2), sc = 1099511627776.0f / r;  // 2^40 / r
    long long sx = 0, sy = 0, sz = 0, sw = 0;
    auto acc = [&](const float4& p) {
        float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
        float d2 = sqdist(dx, dy, dz);
        if (d2 > r2) return;
        float w = __expf(-d2 * inv2s2);
        sx += __float2ll_rn(w * dx * sc);
        sy += __float2ll_rn(w * dy * sc);
        sz += __float2ll_rn(w * dz * sc);
        sw += __float2ll_rn(w * 1099511627776.0f);
    };
    visit_ring(g, ic, cx, cy, cz, 0, acc);
    visit_ring(g, ic, cx, cy, cz, 1, acc);
    const double k = (double)r / (double)sw;  // (S / 2^40 * r) / (W / 2^40)
    out[3 * i] = (float)((double)qx + (double)sx * k);
    out[3 * i + 1] = (float)((double)qy + (double)sy * k);
    out[3 * i + 2] = (float)((double)qz + (double)sz * k);
}

// Grid-stride over the points (a grid sized to the GPU: when the window pass
// left nothing, the launch costs a few waves of blocks that return at once).
__global__ void metric_gaussian_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                       float r2, float inv2s2, Level g, const GridStats* __restrict__ s,
                                       const float* __restrict__ pending, float* __restrict__ out) {
    if (pending && s->n_pending == 0u) return;  // the window pass settled every query
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        metric_gaussian_point(xyz, mask, i, r2, inv2s2, g, s, pending, out);
}

unsigned table_size(size_t want) {
    unsigned t = 1024;
    while (t < want && t < (1u << 30)) t <<= 1;
    return t;
}

// level tables: about 4 points per bucket on the hashed finest level; the
// coarse level is a dense grid of at most DENSE_MAX cells
unsigned level_table(size_t n, int l) { return l == 0 ? table_size(n / 4) : (unsigned)DENSE_MAX; }

struct GridScratch {
    GridStats* stats;
    int levels;
    unsigned tsize[MAX_LEVELS];
    uint2* tab[MAX_LEVELS];
    float4* pts[MAX_LEVELS];
    unsigned* counts;  // shared by the levels' builds
    unsigned* tot;
    float* md;
    unsigned* deferred;
    unsigned* hard;  // phase-3 queries
    float* bound;    // per pixel: a deferred query's bound (md = MD_BOUND)
    double* part;
    uint4* occ;  // occupied coarse cells: (cell index, offset, count, 0)
};

// block partials: the spacing passes' (3 per block), then the SOR statistics' (2 per block)
size_t part_bytes(size_t n) {
    const size_t sor = ((n + GB - 1) / GB) * 2 * sizeof(double), sp = (size_t)SPACING_BLOCKS * 3 * sizeof(double);
    return sor > sp ? sor : sp;
}

size_t grid_bytes(size_t n, int levels) {
    size_t b = zim_align256(sizeof(GridStats)) + zim_align256(n * 4) * 4 + zim_align256(part_bytes(n)) +
               zim_align256((size_t)level_table(n, levels - 1) * sizeof(uint4));
    unsigned tmax = 1024;
    for (int l = 0; l < levels; l++) {
        unsigned t = level_table(n, l);
        tmax = t > tmax ? t : tmax;
        b += zim_align256((size_t)t * 8) + zim_align256(n * 16);
    }
    b += zim_align256((size_t)tmax * 4) + zim_align256(((tmax + SCAN_B - 1) / SCAN_B) * 4);
    return b + 4096;
}

zim_status carve_grid(zim_ctx* ctx, size_t n, int levels, GridScratch& G) {
    G.levels = levels;
    G.stats = (GridStats*)zim_scratch_take(ctx, sizeof(GridStats));
    unsigned tmax = 1024;
    for (int l = 0; l < levels; l++) {
        G.tsize[l] = level_table(n, l);
        tmax = G.tsize[l] > tmax ? G.tsize[l] : tmax;
        G.tab[l] = (uint2*)zim_scratch_take(ctx, (size_t)G.tsize[l] * 8);
        G.pts[l] = (float4*)zim_scratch_take(ctx, n * 16);
        if (!G.tab[l] || !G.pts[l]) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "grid scratch carve");
    }
    G.counts = (unsigned*)zim_scratch_take(ctx, (size_t)tmax * 4);
    G.tot = (unsigned*)zim_scratch_take(ctx, ((tmax + SCAN_B - 1) / SCAN_B) * 4);
    G.md = (float*)zim_scratch_take(ctx, n * 4);
    G.deferred = (unsigned*)zim_scratch_take(ctx, n * 4);
    G.hard = (unsigned*)zim_scratch_take(ctx, n * 4);
    G.bound = (float*)zim_scratch_take(ctx, n * 4);
    G.part = (double*)zim_scratch_take(ctx, part_bytes(n));
    G.occ = (uint4*)zim_scratch_take(ctx, (size_t)G.tsize[levels - 1] * sizeof(uint4));
    if (!G.stats || !G.counts || !G.tot || !G.md || !G.deferred || !G.hard || !G.bound || !G.part || !G.occ)
        return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "grid scratch carve");
    return ZIM_OK;
}

// Per 16x8 pixel tile (the window passes' tiles) the largest distance of a
// valid point from its pixel ray (float bits; NaN counts as unbounded), and the
// largest of all into ray_dev_bits.
__global__ void __launch_bounds__(WT_T) tile_ray_dev_kernel(const float* __restrict__ xyz,
                                                              const uint8_t* __restrict__ mask, int rows, int cols,
                                                              zt::RayParams rp, GridStats* s,
                                                              unsigned* __restrict__ tile_dev) {
    __shared__ unsigned wmax[WT_T / 32];
    const int x = blockIdx.x * WT_X + (int)threadIdx.x % WT_X, y = blockIdx.y * WT_Y + (int)threadIdx.x / WT_X;
    unsigned dev = 0u;
    if (x < cols && y < rows) {
        const size_t i = (size_t)y * cols + x;
        if (mask[i]) {
            float ax, ay, az;
            zt::ray_dir(rp, x, y, ax, ay, az);
            const float d = zt::ray_dev(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], ax, ay, az);
            dev = __float_as_uint(d == d ? d : INFINITY);
        }
    }
    dev = __reduce_max_sync(0xffffffffu, dev);
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = dev;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 1; j < WT_T / 32; j++) dev = max(dev, wmax[j]);
        tile_dev[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = dev;
        if (dev) atomicMax(&s->ray_dev_bits, dev);
    }
}

// The grid's statistics (spacing, bounding box, cell sizes; with pixel rays
// also the largest distance of a point from its ray, ray_dev_bits).
// init = false: the stats were zeroed already (and may hold counts); gate as
// for the build kernels.
zim_status grid_stats(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, float fixed_cell,
                      float factor, const RayParams* rays, GridScratch& G, cudaStream_t st, bool init = true,
                      const unsigned* gate = nullptr) {
    size_t n = (size_t)rows * cols;
    unsigned nblk = (unsigned)((n + GB - 1) / GB);
    if (init) {
        stats_init_kernel<<<1, 1, 0, st>>>(G.stats);
        ctx->launches += 1;
    }
    const unsigned sblk = nblk < (unsigned)SPACING_BLOCKS ? nblk : (unsigned)SPACING_BLOCKS;
    spacing1_kernel<<<sblk, GB, 0, st>>>(xyz, mask, rows, cols, rays ? 1 : 0, rays ? *rays : RayParams{}, G.stats,
                                         G.part, gate);
    spacing_total_kernel<<<1, SPACING_BLOCKS, 0, st>>>(G.part, (int)sblk, 1, G.stats, gate);
    // the trimmed spacing sets the cell; with pixel rays the window passes
    // settle nearly every query and the grid serves only the few deferred
    // ones, so the plain mean of pass 1 sets it (the cell size only affects
    // speed, never a result)
    if (!(fixed_cell > 0.f) && !rays) {
        spacing2_kernel<<<sblk, GB, 0, st>>>(xyz, mask, rows, cols, G.stats, G.part, gate);
        spacing_total_kernel<<<1, SPACING_BLOCKS, 0, st>>>(G.part, (int)sblk, 2, G.stats, gate);
        ctx->launches += 2;
    }
    cell_kernel<<<1, 1, 0, st>>>(G.stats, fixed_cell, factor, G.levels, gate);
    ctx->launches += 3;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

// The levels' tables from first_level up (counting sort of the points by
// slot); gate as for the table kernels (null: always built).
zim_status grid_tables(zim_ctx* ctx, const float* xyz, const uint8_t* mask, size_t n, bool sort_buckets,
                       GridScratch& G, cudaStream_t st, int first_level = 0, const unsigned* gate = nullptr) {
    // grids sized to the GPU (the kernels stride): 8 blocks of 256 per SM,
    // 2 of the scans' 1024
    const unsigned sms = (unsigned)(ctx->sm_count > 0 ? ctx->sm_count : 152);
    const unsigned nblk = (unsigned)std::min<size_t>((n + GB - 1) / GB, 8 * sms);
    for (int l = first_level; l < G.levels; l++) {
        const unsigned T = G.tsize[l], nb = (T + SCAN_B - 1) / SCAN_B;
        const unsigned tblk = std::min((T + GB - 1) / GB, 8 * sms), sblk = std::min(nb, 2 * sms);
        zero_kernel<<<tblk, GB, 0, st>>>(G.counts, T, gate);
        hash_count_kernel<<<nblk, GB, 0, st>>>(xyz, mask, n, G.stats, l, T - 1, G.counts, gate);
        scan_blocks_kernel<<<sblk, SCAN_B, 0, st>>>(G.counts, G.tab[l], T, G.tot, gate);
        scan_totals_kernel<<<1, SCAN_B, 0, st>>>(G.tot, (int)nb, gate);
        scan_add_kernel<<<sblk, SCAN_B, 0, st>>>(G.tab[l], T, G.tot, gate);
        zero_kernel<<<tblk, GB, 0, st>>>(G.counts, T, gate);
        hash_scatter_kernel<<<nblk, GB, 0, st>>>(xyz, mask, n, G.stats, l, T - 1, G.tab[l], G.counts, G.pts[l],
                                                  gate);
        ctx->launches += 7;
        if (sort_buckets) {
            bucket_sort_kernel<<<(T + GB - 1) / GB, GB, 0, st>>>(G.tab[l], T, G.pts[l]);
            ctx->launches += 1;
        }
    }
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

// Statistics and tables (levels from first_level up).
zim_status build_grid(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, float fixed_cell,
                      float factor, bool sort_buckets, const RayParams* rays, GridScratch& G, cudaStream_t st,
                      int first_level = 0) {
    zim_status s = grid_stats(ctx, xyz, mask, rows, cols, fixed_cell, factor, rays, G, st);
    if (s) return s;
    return grid_tables(ctx, xyz, mask, (size_t)rows * cols, sort_buckets, G, st, first_level);
}

}  // namespace

size_t zim_grid_scratch_bytes(size_t n) { return grid_bytes(n, MAX_LEVELS); }

zim_status zim_sor_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, int mean_k,
                          double std_mul, float* xyz_out, uint8_t* mask_out, float* mean_dist,
                          const zim_ray_model& rays, cudaStream_t st) {
    size_t n = (size_t)rows * cols;
    GridScratch G;
    zim_status s = carve_grid(ctx, n, MAX_LEVELS, G);
    if (s) return s;
    // finest cell ~ 3.5 x spacing: the (k+1)-th neighbour of a surface point
    // lies within one ring for ~98% of points at k = 30
    float factor = 3.5f * sqrtf(fmaxf(1.0f, (float)mean_k / 30.0f));
    const RayParams rpw = zt::ray_params(rays);
    // with pixel rays the window passes and the coarse level settle every
    // query: the finest level (the tile search's) is not built
    s = build_grid(ctx, xyz, mask, rows, cols, 0.f, factor, false, rays.valid ? &rpw : nullptr, G, st,
                   rays.valid ? 1 : 0);
    if (s) return s;
    const Level fine{G.tab[0], G.pts[0], G.tsize[0] - 1};
    float* md = mean_dist ? mean_dist : G.md;
    occupied_cells_kernel<<<(unsigned)((DENSE_MAX + GB - 1) / GB), GB, 0, st>>>(G.tab[1], G.stats, G.occ);
    dim3 tgrid((cols + TILE_X - 1) / TILE_X, (rows + TILE_Y - 1) / TILE_Y);
    const int window = rays.valid ? 1 : 0;
    if (window) {
        const RayParams rp = rpw;
        const dim3 wgrid((cols + WT_X - 1) / WT_X, (rows + WT_Y - 1) / WT_Y);
        const size_t wsm = (size_t)WW * WH * sizeof(float4) + (size_t)(mean_k + 1) * WT_T * 4;
        // k = 30 and 50 (the configurations') with a compile-time heap size
        auto kern = mean_k == 30 ? sor_window_kernel<31> : mean_k == 50 ? sor_window_kernel<51> : sor_window_kernel<0>;
        ZIM_CUDA_TRY(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm));
        kern<<<wgrid, WT_T, wsm, st>>>(xyz, mask, rows, cols, mean_k, rp, G.stats, md, G.deferred, G.bound);
        ctx->launches += 1;
    } else {
        // without pixel rays every query starts on the finest grid level
        const size_t tsm = (size_t)TILE_MAX_CAND * sizeof(float4);
        // dynamic + static shared memory exceeds the default 48 KB (attribute is per device: set it every call)
        ZIM_CUDA_TRY(ctx, cudaFuncSetAttribute(sor_knn_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
        sor_knn_tile_kernel<<<tgrid, TILE_T, tsm, st>>>(xyz, mask, rows, cols, mean_k, fine, G.stats, md, G.deferred);
        ctx->launches += 1;
    }
    // enough warps in flight to cover the latency of the point scans
    const unsigned sms = (unsigned)(ctx->sm_count > 0 ? ctx->sm_count : 152);
    sor_knn_far_kernel<<<8 * sms, P2_WARPS * 32, 0, st>>>(xyz, mean_k, G.stats, G.tab[1], G.pts[1], G.deferred, md,
                                                          G.bound, G.hard);
    // a few hard queries per cloud: one CTA each
    sor_hard_kernel<<<2 * sms, HARD_T, 0, st>>>(xyz, mean_k, G.stats, G.occ, G.pts[1], G.hard, md, G.bound,
                                                ctx->d_error);
    ctx->launches += 3;
    const unsigned nblk = (unsigned)((n + GB - 1) / GB);
    const unsigned pblk = nblk < (unsigned)SPACING_BLOCKS ? nblk : (unsigned)SPACING_BLOCKS;
    sor_partial_kernel<<<pblk, GB, 0, st>>>(mask, md, n, G.part);
    sor_stats_kernel<<<1, 1024, 0, st>>>(G.part, (int)pblk, mean_k, std_mul, G.stats);
    sor_classify_kernel<<<nblk, GB, 0, st>>>(xyz, mask, n, G.stats, md, mask_out, xyz_out);
    ctx->launches += 3;
    static_assert(sizeof(GridStats) <= 256, "stats snapshot buffer");
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_sor_stats, G.stats, sizeof(GridStats), cudaMemcpyDeviceToDevice, st));
    ctx->have_sor_stats = true;
    ctx->last_sor_std_mul = std_mul;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

zim_status zim_metric_gaussian_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                                      double sigma, float* out, const zim_ray_model& rays, cudaStream_t st) {
    size_t n = (size_t)rows * cols;
    GridScratch G;
    zim_status s = carve_grid(ctx, n, 1, G);
    if (s) return s;
    const float rad = (float)(3.0 * sigma);
    const RayParams rpw = zt::ray_params(rays);
    if (rays.valid) {
        // the window pass needs only the largest ray distance; the grid's
        // statistics wait for the window pass's verdict
        stats_init_kernel<<<1, 1, 0, st>>>(G.stats);
        dim3 tgrid((cols + WT_X - 1) / WT_X, (rows + WT_Y - 1) / WT_Y);
        tile_ray_dev_kernel<<<tgrid, WT_T, 0, st>>>(xyz, mask, rows, cols, rpw, G.stats,
                                                      reinterpret_cast<unsigned*>(G.bound));
        ctx->launches += 2;
    } else {
        s = grid_stats(ctx, xyz, mask, rows, cols, rad, 1.0f, nullptr, G, st);
        if (s) return s;
    }
    Level g{G.tab[0], G.pts[0], G.tsize[0] - 1};
    const float inv2s2 = (float)(1.0 / (2.0 * sigma * sigma));
    float* pending = nullptr;
    if (rays.valid) {
        const RayParams rp = rpw;
        dim3 tgrid((cols + WT_X - 1) / WT_X, (rows + WT_Y - 1) / WT_Y);
        pending = G.md;
        // G.bound holds the per-tile ray distances (one word per tile)
        mg_window_kernel<<<tgrid, WT_T, 0, st>>>(xyz, mask, rows, cols, rad, inv2s2, rp, G.stats,
                                                   reinterpret_cast<const unsigned*>(G.bound), pending, out);
        ctx->launches += 1;
    }
    // the grid only for the queries the window pass left (launched, and
    // skipped on the device when there are none)
    if (pending) {
        s = grid_stats(ctx, xyz, mask, rows, cols, rad, 1.0f, nullptr, G, st, false, &G.stats->n_pending);
        if (s) return s;
    }
    s = grid_tables(ctx, xyz, mask, n, false, G, st, 0, pending ? &G.stats->n_pending : nullptr);
    if (s) return s;
    const unsigned mblk = (unsigned)std::min<size_t>((n + GB - 1) / GB, 8 * (ctx->sm_count > 0 ? ctx->sm_count : 152));
    metric_gaussian_kernel<<<mblk, GB, 0, st>>>(xyz, mask, n, rad * rad, inv2s2, g, G.stats,
                                                                        pending, out);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_filter_sor(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                                             int mean_k, double std_mul, uint8_t* mask_out, float* mean_dist,
                                             void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!xyz || !mask || !mask_out || rows <= 0 || cols <= 0) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    if (mean_k < 1 || mean_k + 1 > KNN_MAX_K1) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "mean_k must be in [1, 63]");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    zim_status s = zim_scratch_reserve(ctx, zim_grid_scratch_bytes((size_t)rows * cols));
    if (s) return s;
    zim_scratch_reset(ctx);
    // a cloud of the calibrated rectified size: its pixels' rays as the window hint
    const zim_ray_model rays = rows == ctx->rect_h && cols == ctx->rect_w ? zim_rays_of(ctx, true, 0, 0)
                                                                          : zim_ray_model{};
    return zim_sor_launch(ctx, xyz, mask, rows, cols, mean_k, std_mul, nullptr, mask_out, mean_dist, rays,
                          zim_stream(stream));
}

extern "C" ZIM_API zim_status zim_filter_sor_stats(zim_ctx* ctx, zim_sor_stats* out) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!out || !ctx->have_sor_stats) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "no SOR run on this context");
    GridStats h;
    ZIM_CUDA_TRY(ctx, cudaDeviceSynchronize());
    ZIM_CUDA_TRY(ctx, cudaMemcpy(&h, ctx->d_sor_stats, sizeof h, cudaMemcpyDeviceToHost));
    const double nv = h.n_valid;
    out->n_valid = nv;
    out->mean = nv > 0 ? h.md_sum / nv : 0.0;
    out->stddev = nv > 1 ? sqrt((h.md_sq - h.md_sum * h.md_sum / nv) / (nv - 1)) : 0.0;
    out->threshold = out->mean + ctx->last_sor_std_mul * out->stddev;
    out->n_far_search = h.n_deferred;
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_filter_metric_gaussian(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows,
                                                         int cols, double sigma, float* out, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!xyz || !mask || !out || rows <= 0 || cols <= 0 || !(sigma > 0))
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    zim_status s = zim_scratch_reserve(ctx, zim_grid_scratch_bytes((size_t)rows * cols));
    if (s) return s;
    zim_scratch_reset(ctx);
    const zim_ray_model rays = rows == ctx->rect_h && cols == ctx->rect_w ? zim_rays_of(ctx, true, 0, 0)
                                                                          : zim_ray_model{};
    return zim_metric_gaussian_launch(ctx, xyz, mask, rows, cols, sigma, out, rays, zim_stream(stream));
}
