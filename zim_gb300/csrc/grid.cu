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
// sets the finest cell on the device; levels with cells c, 4c, 16c, 64c are
// counting-sorted into power-of-two hash tables of (offset, count) pairs.
// A kNN query visits Chebyshev rings of cells around its own cell and stops
// once it holds k + 1 candidates and the (k + 1)-th distance is within the
// ring's guaranteed radius r * cell, so the result is exact.
//   phase 1: one thread per point, finest level, rings <= 2 (almost all points);
//   phase 2: one warp per remaining point (isolated outliers), coarser levels,
//            the lanes splitting each ring's cells, cells farther than the
//            current (k + 1)-th distance pruned, the lanes' sorted lists merged
//            after each ring.
// A visited point's cell is re-derived from its coordinates, so hash
// collisions never count a point twice.  Both filters are deterministic: the
// SOR statistics are summed in a fixed order, and the Gaussian's buckets are
// sorted by pixel index before they are summed.
#include <cfloat>
#include <climits>
#include <cmath>

#include "zim_internal.cuh"

namespace {

constexpr int GB = 256;          // threads for pixel-parallel kernels
constexpr int KNN_THREADS = 128; // phase-1 CTA
constexpr int KNN_MAX_K1 = 64;   // k + 1 <= 64
constexpr int SCAN_B = 1024;
constexpr int MAX_LEVELS = 4;
constexpr int FINE_RINGS = 2;    // phase 1 rings on the finest level
constexpr int COARSE_RINGS = 4;  // phase 2 rings per level before going coarser
constexpr int P2_WARPS = 4;      // phase-2 warps per CTA

struct GridStats {
    double sp_sum, sp_cnt;    // spacing pass 1
    double sp2_sum, sp2_cnt;  // spacing pass 2 (trimmed)
    double n_valid;
    double md_sum, md_sq;     // SOR statistics (fixed-order sums)
    float cell[MAX_LEVELS], inv_cell[MAX_LEVELS];
    int max_ring[MAX_LEVELS];
    int bbox_min[3], bbox_max[3];  // order-preserving float bits
    unsigned n_deferred;
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
__device__ T block_reduce(T v, Op op, T ident) {
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

__global__ void stats_init_kernel(GridStats* s) {
    s->sp_sum = s->sp_cnt = s->sp2_sum = s->sp2_cnt = 0;
    s->md_sum = s->md_sq = s->n_valid = 0;
    s->n_deferred = 0;
    for (int a = 0; a < 3; a++) { s->bbox_min[a] = INT_MAX; s->bbox_max[a] = INT_MIN; }
}

// pass 1: mean spacing of horizontally adjacent valid pixels, bbox, count
__global__ void spacing1_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, int rows, int cols,
                                GridStats* s) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t n = (size_t)rows * cols;
    double d = 0, c = 0, nv = 0;
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
    if (i < n && mask[i]) {
        nv = 1;
        float p[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        for (int a = 0; a < 3; a++) mn[a] = mx[a] = fbits(p[a]);
        if ((i % cols) + 1 < (size_t)cols && mask[i + 1]) {
            float dx = xyz[3 * i + 3] - p[0], dy = xyz[3 * i + 4] - p[1], dz = xyz[3 * i + 5] - p[2];
            d = sqrtf(dx * dx + dy * dy + dz * dz);
            c = 1;
        }
    }
    d = block_reduce(d, Add(), 0.0);
    c = block_reduce(c, Add(), 0.0);
    nv = block_reduce(nv, Add(), 0.0);
    for (int a = 0; a < 3; a++) {
        mn[a] = block_reduce(mn[a], Min(), INT_MAX);
        mx[a] = block_reduce(mx[a], Max(), INT_MIN);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&s->sp_sum, d);
        atomicAdd(&s->sp_cnt, c);
        atomicAdd(&s->n_valid, nv);  // integer-valued: exact in any order
        for (int a = 0; a < 3; a++) {
            if (mn[a] != INT_MAX) atomicMin(&s->bbox_min[a], mn[a]);
            if (mx[a] != INT_MIN) atomicMax(&s->bbox_max[a], mx[a]);
        }
    }
}

// pass 2: mean spacing over pairs closer than 3x the pass-1 mean
__global__ void spacing2_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, int rows, int cols,
                                GridStats* s) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t n = (size_t)rows * cols;
    const double m1 = s->sp_cnt > 0 ? s->sp_sum / s->sp_cnt : 0.0;
    double d = 0, c = 0;
    if (i < n && mask[i] && (i % cols) + 1 < (size_t)cols && mask[i + 1]) {
        float dx = xyz[3 * i + 3] - xyz[3 * i], dy = xyz[3 * i + 4] - xyz[3 * i + 1], dz = xyz[3 * i + 5] - xyz[3 * i + 2];
        float v = sqrtf(dx * dx + dy * dy + dz * dz);
        if (v <= 3.0 * m1) { d = v; c = 1; }
    }
    d = block_reduce(d, Add(), 0.0);
    c = block_reduce(c, Add(), 0.0);
    if (threadIdx.x == 0) {
        atomicAdd(&s->sp2_sum, d);
        atomicAdd(&s->sp2_cnt, c);
    }
}

// finest cell = fixed_cell if > 0, else factor * trimmed mean spacing; level l
// has cell * 4^l.  The cell size only affects speed, never the result.
__global__ void cell_kernel(GridStats* s, float fixed_cell, float factor, int levels) {
    float cell = fixed_cell;
    if (!(cell > 0.f)) {
        double sp = s->sp2_cnt > 0 ? s->sp2_sum / s->sp2_cnt : 1.0;
        cell = (float)(factor * sp);
    }
    float ext = 0.f;
    for (int a = 0; a < 3; a++)
        if (s->bbox_max[a] >= s->bbox_min[a]) ext = fmaxf(ext, bitsf(s->bbox_max[a]) - bitsf(s->bbox_min[a]));
    cell = fmaxf(cell, ext * 1e-5f);
    cell = fmaxf(cell, 1e-6f);
    for (int l = 0; l < MAX_LEVELS; l++) {
        float c = l < levels ? cell * (float)(1 << (2 * l)) : cell;
        s->cell[l] = c;
        s->inv_cell[l] = 1.0f / c;
        s->max_ring[l] = (int)ceilf(ext / c) + 2;
    }
}

__device__ __forceinline__ void cell_of(float x, float y, float z, float ic, int& cx, int& cy, int& cz) {
    cx = __float2int_rd(x * ic);
    cy = __float2int_rd(y * ic);
    cz = __float2int_rd(z * ic);
}

__global__ void hash_count_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                  const GridStats* __restrict__ s, int level, unsigned tmask,
                                  unsigned* __restrict__ counts) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i]) return;
    int cx, cy, cz;
    cell_of(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], s->inv_cell[level], cx, cy, cz);
    atomicAdd(&counts[hash3(cx, cy, cz, tmask)], 1u);
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
                                   unsigned* __restrict__ block_tot) {
    __shared__ unsigned ws[32];
    size_t i = (size_t)blockIdx.x * SCAN_B + threadIdx.x;
    unsigned v = i < n ? counts[i] : 0u;
    unsigned incl = block_scan_incl(v, ws);
    if (i < n) tab[i] = make_uint2(incl - v, v);
    if (threadIdx.x == SCAN_B - 1) block_tot[blockIdx.x] = incl;
}

__global__ void scan_totals_kernel(unsigned* __restrict__ tot, int nb) {
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

__global__ void scan_add_kernel(uint2* __restrict__ tab, size_t n, const unsigned* __restrict__ tot) {
    size_t i = (size_t)blockIdx.x * SCAN_B + threadIdx.x;
    if (i < n) tab[i].x += tot[blockIdx.x];
}

__global__ void hash_scatter_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                    const GridStats* __restrict__ s, int level, unsigned tmask,
                                    const uint2* __restrict__ tab, unsigned* __restrict__ fill,
                                    float4* __restrict__ pts) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i]) return;
    float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    int cx, cy, cz;
    cell_of(x, y, z, s->inv_cell[level], cx, cy, cz);
    unsigned h = hash3(cx, cy, cz, tmask);
    unsigned pos = tab[h].x + atomicAdd(&fill[h], 1u);
    pts[pos] = make_float4(x, y, z, __int_as_float((int)i));
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
struct Levels {
    Level l[MAX_LEVELS];
    int n;
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

// Phase 1: one thread per point on the finest level.  Points not resolved
// within FINE_RINGS rings are appended to the deferred list (md = -1).
__global__ void __launch_bounds__(KNN_THREADS) sor_knn_fine_kernel(const float* __restrict__ xyz,
                                                                   const uint8_t* __restrict__ mask, size_t n, int k,
                                                                   Level g, GridStats* s, float* __restrict__ md_out,
                                                                   unsigned* __restrict__ deferred) {
    __shared__ float L[KNN_MAX_K1][KNN_THREADS];
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!mask[i] || s->n_valid <= k) {
        md_out[i] = 0.f;
        return;
    }
    const int K1 = k + 1, tid = threadIdx.x;
    const float qx = xyz[3 * i], qy = xyz[3 * i + 1], qz = xyz[3 * i + 2];
    int cnt = 0;
    auto ins = [&](const float4& p) {
        float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
        float d2 = dx * dx + dy * dy + dz * dz;
        int j;
        if (cnt < K1) j = cnt++;
        else if (d2 < L[K1 - 1][tid]) j = K1 - 1;
        else return;
        while (j > 0 && L[j - 1][tid] > d2) {
            L[j][tid] = L[j - 1][tid];
            j--;
        }
        L[j][tid] = d2;
    };
    const float ic = s->inv_cell[0], cell = s->cell[0];
    int cx, cy, cz;
    cell_of(qx, qy, qz, ic, cx, cy, cz);
    for (int r = 0; r <= FINE_RINGS; r++) {
        visit_ring(g, ic, cx, cy, cz, r, ins);
        float gr = r * cell;
        if (cnt >= K1 && L[K1 - 1][tid] <= gr * gr) {
            float sum = 0.f;
            for (int j = 1; j < K1; j++) sum += sqrtf(L[j][tid]);
            md_out[i] = sum / (float)k;
            return;
        }
    }
    md_out[i] = -1.f;
    unsigned slot = atomicAdd(&s->n_deferred, 1u);
    deferred[slot] = (unsigned)i;
}

// Cell t (0 <= t < 24 r^2 + 2) of the Chebyshev ring r around the origin.
__device__ __forceinline__ void ring_cell(int r, int t, int& dx, int& dy, int& dz) {
    if (r == 0) { dx = dy = dz = 0; return; }
    const int side = 2 * r + 1, face = side * side;
    if (t < 2 * face) {
        dz = t < face ? -r : r;
        int q = t < face ? t : t - face;
        dy = q / side - r;
        dx = q % side - r;
        return;
    }
    t -= 2 * face;
    const int per = 8 * r;
    dz = t / per - (r - 1);
    int p = t % per;
    if (p < side) { dx = p - r; dy = -r; return; }
    p -= side;
    if (p < side) { dx = p - r; dy = r; return; }
    p -= side;
    dy = (p >> 1) - (r - 1);
    dx = (p & 1) ? r : -r;
}

// Phase 2: one warp per deferred point, coarser levels.  Each lane keeps a
// sorted list of its K1 best; after every ring the lists are merged to find
// the (k+1)-th distance (termination and pruning bound) and the mean.
__global__ void __launch_bounds__(P2_WARPS * 32) sor_knn_coarse_kernel(const float* __restrict__ xyz, int k, Levels lv,
                                                                        const GridStats* __restrict__ s,
                                                                        const unsigned* __restrict__ deferred,
                                                                        float* __restrict__ md_out,
                                                                        uint32_t* __restrict__ err) {
    __shared__ float L[P2_WARPS][KNN_MAX_K1][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int K1 = k + 1;
    const unsigned nd = s->n_deferred;
    for (unsigned item = blockIdx.x * P2_WARPS + w; item < nd; item += gridDim.x * P2_WARPS) {
        const unsigned i = deferred[item];
        const float qx = xyz[3 * i], qy = xyz[3 * i + 1], qz = xyz[3 * i + 2];
        bool done = false;
        float md = 0.f;
        for (int l = (lv.n > 1 ? 1 : 0); l < lv.n && !done; l++) {
            const Level& g = lv.l[l];
            const float ic = s->inv_cell[l], cell = s->cell[l];
            int cx, cy, cz;
            cell_of(qx, qy, qz, ic, cx, cy, cz);
            int cnt = 0;
            float bound = INFINITY;  // current (k+1)-th squared distance over the warp
            const int rmax = (l == lv.n - 1) ? s->max_ring[l] : COARSE_RINGS;
            for (int r = 0; r <= rmax && !done; r++) {
                const int ncell = r == 0 ? 1 : 24 * r * r + 2;
                for (int t = lane; t < ncell; t += 32) {
                    int dx, dy, dz;
                    ring_cell(r, t, dx, dy, dz);
                    const int x = cx + dx, y = cy + dy, z = cz + dz;
                    // squared distance from q to the cell box (pruning), slightly shrunk
                    float ex = fmaxf(fmaxf(x * cell - qx, qx - (x + 1) * cell), 0.f);
                    float ey = fmaxf(fmaxf(y * cell - qy, qy - (y + 1) * cell), 0.f);
                    float ez = fmaxf(fmaxf(z * cell - qz, qz - (z + 1) * cell), 0.f);
                    float bd = fmaxf(sqrtf(ex * ex + ey * ey + ez * ez) - 1e-4f * cell, 0.f);
                    if (bd * bd > bound) continue;
                    uint2 b = bucket(g, x, y, z);
                    for (unsigned u = b.x; u < b.x + b.y; u++) {
                        float4 p = __ldg(g.pts + u);
                        int px, py, pz;
                        cell_of(p.x, p.y, p.z, ic, px, py, pz);
                        if (px != x || py != y || pz != z) continue;
                        float ddx = p.x - qx, ddy = p.y - qy, ddz = p.z - qz;
                        float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                        int j;
                        if (cnt < K1) j = cnt++;
                        else if (d2 < L[w][K1 - 1][lane]) j = K1 - 1;
                        else continue;
                        while (j > 0 && L[w][j - 1][lane] > d2) {
                            L[w][j][lane] = L[w][j - 1][lane];
                            j--;
                        }
                        L[w][j][lane] = d2;
                    }
                }
                __syncwarp();
                // merge: the K1 smallest over all lanes, in order
                int head = 0;
                float kth = INFINITY, sum = 0.f;
                for (int round = 0; round < K1; round++) {
                    float v = head < cnt ? L[w][head][lane] : INFINITY;
                    int who = lane;
                    for (int off = 16; off; off >>= 1) {
                        float ov = __shfl_xor_sync(0xffffffffu, v, off);
                        int ow = __shfl_xor_sync(0xffffffffu, who, off);
                        if (ov < v || (ov == v && ow < who)) { v = ov; who = ow; }
                    }
                    if (lane == who) head++;
                    if (round > 0) sum += sqrtf(v);
                    if (round == K1 - 1) kth = v;
                }
                bound = kth;
                const float gr = r * cell;
                if (kth <= gr * gr) {
                    done = true;
                    md = sum / (float)k;
                }
                __syncwarp();
            }
        }
        if (!done && lane == 0) atomicOr(err, 0x10u);  // fewer than k+1 points reachable
        if (lane == 0) md_out[i] = md;
    }
}

// Per-block sums of the mean distances (valid pixels), then a fixed-order total.
__global__ void sor_partial_kernel(const uint8_t* __restrict__ mask, const float* __restrict__ md, size_t n,
                                   double* __restrict__ part) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0, b = 0;
    if (i < n && mask[i]) {
        float m = md[i];
        a = m;
        b = (double)(m * m);  // PCL: float square, double sum
    }
    a = block_reduce(a, Add(), 0.0);
    b = block_reduce(b, Add(), 0.0);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

__global__ void sor_stats_kernel(const double* __restrict__ part, int nb, GridStats* s) {
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
    }
}

__global__ void sor_classify_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n, int k,
                                    double std_mul, const GridStats* __restrict__ s, const float* __restrict__ md,
                                    uint8_t* __restrict__ mask_out, float* __restrict__ xyz_out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double nv = s->n_valid;
    bool keep = false;
    if (mask[i]) {
        if (nv <= k) keep = true;  // too few points for a k-neighbourhood: nothing is removed
        else {
            double mean = s->md_sum / nv;
            double var = (s->md_sq - s->md_sum * s->md_sum / nv) / (nv - 1);
            double thr = mean + std_mul * sqrt(var);
            keep = !((double)md[i] > thr);
        }
    }
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
__global__ void metric_gaussian_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                       float r2, float inv2s2, Level g, const GridStats* __restrict__ s,
                                       float* __restrict__ out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float qx = xyz[3 * i], qy = xyz[3 * i + 1], qz = xyz[3 * i + 2];
    if (!mask[i]) {
        out[3 * i] = qx; out[3 * i + 1] = qy; out[3 * i + 2] = qz;
        return;
    }
    const float ic = s->inv_cell[0];
    int cx, cy, cz;
    cell_of(qx, qy, qz, ic, cx, cy, cz);
    float sx = 0.f, sy = 0.f, sz = 0.f, sw = 0.f;
    auto acc = [&](const float4& p) {
        float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
        float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 > r2) return;
        float w = __expf(-d2 * inv2s2);
        sx = fmaf(w, dx, sx); sy = fmaf(w, dy, sy); sz = fmaf(w, dz, sz);
        sw += w;
    };
    visit_ring(g, ic, cx, cy, cz, 0, acc);
    visit_ring(g, ic, cx, cy, cz, 1, acc);
    float iw = 1.0f / sw;
    out[3 * i] = qx + sx * iw;
    out[3 * i + 1] = qy + sy * iw;
    out[3 * i + 2] = qz + sz * iw;
}

unsigned table_size(size_t want) {
    unsigned t = 1024;
    while (t < want && t < (1u << 30)) t <<= 1;
    return t;
}

// level l tables: about 4 points per bucket on the finest level, 16x fewer per level
unsigned level_table(size_t n, int l) { return table_size((n / 4) >> (4 * l)); }

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
    double* part;
};

size_t grid_bytes(size_t n, int levels) {
    size_t b = zim_align256(sizeof(GridStats)) + zim_align256(n * 4) * 2 + zim_align256(((n + GB - 1) / GB) * 16);
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
    G.part = (double*)zim_scratch_take(ctx, ((n + GB - 1) / GB) * 16);
    if (!G.stats || !G.counts || !G.tot || !G.md || !G.deferred || !G.part)
        return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "grid scratch carve");
    return ZIM_OK;
}

zim_status build_grid(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, float fixed_cell,
                      float factor, bool sort_buckets, GridScratch& G, cudaStream_t st) {
    size_t n = (size_t)rows * cols;
    unsigned nblk = (unsigned)((n + GB - 1) / GB);
    stats_init_kernel<<<1, 1, 0, st>>>(G.stats);
    spacing1_kernel<<<nblk, GB, 0, st>>>(xyz, mask, rows, cols, G.stats);
    spacing2_kernel<<<nblk, GB, 0, st>>>(xyz, mask, rows, cols, G.stats);
    cell_kernel<<<1, 1, 0, st>>>(G.stats, fixed_cell, factor, G.levels);
    ctx->launches += 4;
    for (int l = 0; l < G.levels; l++) {
        const unsigned T = G.tsize[l], nb = (T + SCAN_B - 1) / SCAN_B;
        ZIM_CUDA_TRY(ctx, cudaMemsetAsync(G.counts, 0, (size_t)T * 4, st));
        hash_count_kernel<<<nblk, GB, 0, st>>>(xyz, mask, n, G.stats, l, T - 1, G.counts);
        scan_blocks_kernel<<<nb, SCAN_B, 0, st>>>(G.counts, G.tab[l], T, G.tot);
        scan_totals_kernel<<<1, SCAN_B, 0, st>>>(G.tot, (int)nb);
        scan_add_kernel<<<nb, SCAN_B, 0, st>>>(G.tab[l], T, G.tot);
        ZIM_CUDA_TRY(ctx, cudaMemsetAsync(G.counts, 0, (size_t)T * 4, st));
        hash_scatter_kernel<<<nblk, GB, 0, st>>>(xyz, mask, n, G.stats, l, T - 1, G.tab[l], G.counts, G.pts[l]);
        ctx->launches += 5;
        if (sort_buckets) {
            bucket_sort_kernel<<<(T + GB - 1) / GB, GB, 0, st>>>(G.tab[l], T, G.pts[l]);
            ctx->launches += 1;
        }
    }
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

}  // namespace

size_t zim_grid_scratch_bytes(size_t n) { return grid_bytes(n, MAX_LEVELS); }

zim_status zim_sor_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, int mean_k,
                          double std_mul, float* xyz_out, uint8_t* mask_out, float* mean_dist, cudaStream_t st) {
    size_t n = (size_t)rows * cols;
    GridScratch G;
    zim_status s = carve_grid(ctx, n, MAX_LEVELS, G);
    if (s) return s;
    // finest cell ~ 3.5 x spacing: the (k+1)-th neighbour of a surface point
    // lies within one ring for ~98% of points at k = 30
    float factor = 3.5f * sqrtf(fmaxf(1.0f, (float)mean_k / 30.0f));
    s = build_grid(ctx, xyz, mask, rows, cols, 0.f, factor, false, G, st);
    if (s) return s;
    Levels lv;
    lv.n = G.levels;
    for (int l = 0; l < G.levels; l++) lv.l[l] = Level{G.tab[l], G.pts[l], G.tsize[l] - 1};
    float* md = mean_dist ? mean_dist : G.md;
    sor_knn_fine_kernel<<<(unsigned)((n + KNN_THREADS - 1) / KNN_THREADS), KNN_THREADS, 0, st>>>(
        xyz, mask, n, mean_k, lv.l[0], G.stats, md, G.deferred);
    sor_knn_coarse_kernel<<<(unsigned)(2 * (ctx->sm_count > 0 ? ctx->sm_count : 152)), P2_WARPS * 32, 0, st>>>(
        xyz, mean_k, lv, G.stats, G.deferred, md, ctx->d_error);
    const unsigned nblk = (unsigned)((n + GB - 1) / GB);
    sor_partial_kernel<<<nblk, GB, 0, st>>>(mask, md, n, G.part);
    sor_stats_kernel<<<1, 1024, 0, st>>>(G.part, (int)nblk, G.stats);
    sor_classify_kernel<<<nblk, GB, 0, st>>>(xyz, mask, n, mean_k, std_mul, G.stats, md, mask_out, xyz_out);
    ctx->launches += 5;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

zim_status zim_metric_gaussian_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                                      double sigma, float* out, cudaStream_t st) {
    size_t n = (size_t)rows * cols;
    GridScratch G;
    zim_status s = carve_grid(ctx, n, 1, G);
    if (s) return s;
    const float rad = (float)(3.0 * sigma);
    s = build_grid(ctx, xyz, mask, rows, cols, rad, 1.0f, true, G, st);
    if (s) return s;
    Level g{G.tab[0], G.pts[0], G.tsize[0] - 1};
    metric_gaussian_kernel<<<(unsigned)((n + GB - 1) / GB), GB, 0, st>>>(
        xyz, mask, n, rad * rad, (float)(1.0 / (2.0 * sigma * sigma)), g, G.stats, out);
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
    return zim_sor_launch(ctx, xyz, mask, rows, cols, mean_k, std_mul, nullptr, mask_out, mean_dist, zim_stream(stream));
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
    return zim_metric_gaussian_launch(ctx, xyz, mask, rows, cols, sigma, out, zim_stream(stream));
}
