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
// sets the finest cell on the device; up to four levels with cells
// c, 4c, 16c, 64c are counting-sorted into power-of-two hash tables (count,
// exclusive scan, scatter).  A kNN query visits Chebyshev rings of cells around
// its cell and stops once it holds k + 1 candidates and the (k + 1)-th
// distance is within the ring's guaranteed radius r * cell, so the result is
// exact; a query that is not done after a few rings restarts one level
// coarser, which bounds the work of isolated outliers.  A visited point's cell
// is re-derived from its coordinates, so hash collisions never count a point
// twice.  Both filters are deterministic: the SOR statistics are summed in a
// fixed order and the Gaussian accumulates in 64-bit fixed point.
#include <cfloat>
#include <climits>
#include <cmath>

#include "zim_internal.cuh"

namespace {

constexpr int GB = 256;         // threads for pixel-parallel kernels
constexpr int KNN_THREADS = 128;
constexpr int KNN_MAX_K1 = 64;  // k + 1 <= 64
constexpr int SCAN_B = 1024;
constexpr int MAX_LEVELS = 4;
constexpr int LEVEL_RINGS = 3;  // rings tried on a level before going coarser

struct GridStats {
    double sp_sum, sp_cnt;    // spacing pass 1
    double sp2_sum, sp2_cnt;  // spacing pass 2 (trimmed)
    double n_valid;
    double md_sum, md_sq;     // SOR statistics (fixed-order sums)
    float cell[MAX_LEVELS], inv_cell[MAX_LEVELS];
    int max_ring[MAX_LEVELS];
    int bbox_min[3], bbox_max[3];  // order-preserving float bits
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
template <typename T>
__device__ T block_sum(T v) {
    __shared__ T ws[32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int off = 16; off; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) ws[w] = v;
    __syncthreads();
    T r = 0;
    if (w == 0) {
        r = lane < (int)(blockDim.x >> 5) ? ws[lane] : (T)0;
        for (int off = 16; off; off >>= 1) r += __shfl_down_sync(0xffffffffu, r, off);
    }
    __syncthreads();
    return r;
}

__global__ void stats_init_kernel(GridStats* s) {
    s->sp_sum = s->sp_cnt = s->sp2_sum = s->sp2_cnt = 0;
    s->md_sum = s->md_sq = s->n_valid = 0;
    for (int a = 0; a < 3; a++) { s->bbox_min[a] = INT_MAX; s->bbox_max[a] = INT_MIN; }
}

// pass 1: mean spacing of horizontally adjacent valid pixels, bbox, count
__global__ void spacing1_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, int rows, int cols,
                                GridStats* s) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t n = (size_t)rows * cols;
    double d = 0, c = 0, nv = 0;
    if (i < n && mask[i]) {
        nv = 1;
        float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
        atomicMin(&s->bbox_min[0], fbits(px)); atomicMax(&s->bbox_max[0], fbits(px));
        atomicMin(&s->bbox_min[1], fbits(py)); atomicMax(&s->bbox_max[1], fbits(py));
        atomicMin(&s->bbox_min[2], fbits(pz)); atomicMax(&s->bbox_max[2], fbits(pz));
        if ((i % cols) + 1 < (size_t)cols && mask[i + 1]) {
            float dx = xyz[3 * i + 3] - px, dy = xyz[3 * i + 4] - py, dz = xyz[3 * i + 5] - pz;
            d = sqrtf(dx * dx + dy * dy + dz * dz);
            c = 1;
        }
    }
    d = block_sum(d);
    c = block_sum(c);
    nv = block_sum(nv);
    if (threadIdx.x == 0) {
        atomicAdd(&s->sp_sum, d);
        atomicAdd(&s->sp_cnt, c);
        atomicAdd(&s->n_valid, nv);  // integer-valued: exact in any order
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
    d = block_sum(d);
    c = block_sum(c);
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

// exclusive scan, three phases
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

__global__ void scan_blocks_kernel(const unsigned* __restrict__ in, unsigned* __restrict__ out, size_t n,
                                   unsigned* __restrict__ block_tot) {
    __shared__ unsigned ws[32];
    size_t i = (size_t)blockIdx.x * SCAN_B + threadIdx.x;
    unsigned v = i < n ? in[i] : 0u;
    unsigned incl = block_scan_incl(v, ws);
    if (i < n) out[i] = incl - v;
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

__global__ void scan_add_kernel(unsigned* __restrict__ out, size_t n, const unsigned* __restrict__ tot) {
    size_t i = (size_t)blockIdx.x * SCAN_B + threadIdx.x;
    if (i < n) out[i] += tot[blockIdx.x];
}

__global__ void hash_scatter_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                    const GridStats* __restrict__ s, int level, unsigned tmask,
                                    const unsigned* __restrict__ off, unsigned* __restrict__ fill,
                                    float4* __restrict__ pts) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i]) return;
    float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    int cx, cy, cz;
    cell_of(x, y, z, s->inv_cell[level], cx, cy, cz);
    unsigned h = hash3(cx, cy, cz, tmask);
    unsigned pos = off[h] + atomicAdd(&fill[h], 1u);
    pts[pos] = make_float4(x, y, z, __int_as_float((int)i));
}

struct Level {
    const unsigned* off;  // exclusive offsets; bucket h spans [off[h], off[h] + cnt[h])
    const unsigned* cnt;
    const float4* pts;
    unsigned tmask;
};
struct Levels {
    Level l[MAX_LEVELS];
    int n;
};

// Visits the points of all cells at Chebyshev distance exactly r from (cx, cy, cz).
template <typename F>
__device__ __forceinline__ void visit_ring(const Level& g, float ic, int cx, int cy, int cz, int r, F&& fn) {
    for (int dz = -r; dz <= r; dz++)
        for (int dy = -r; dy <= r; dy++) {
            const bool full = (r == 0 || dz == -r || dz == r || dy == -r || dy == r);
            const int step = full ? 1 : 2 * r;
            for (int dx = -r; dx <= r; dx += step) {
                int x = cx + dx, y = cy + dy, z = cz + dz;
                unsigned h = hash3(x, y, z, g.tmask);
                unsigned b = __ldg(g.off + h), e = b + __ldg(g.cnt + h);
                for (unsigned t = b; t < e; t++) {
                    float4 p = __ldg(g.pts + t);
                    int px, py, pz;
                    cell_of(p.x, p.y, p.z, ic, px, py, pz);
                    if (px != x || py != y || pz != z) continue;
                    fn(p);
                }
            }
        }
}

__global__ void __launch_bounds__(KNN_THREADS) sor_knn_kernel(const float* __restrict__ xyz,
                                                              const uint8_t* __restrict__ mask, size_t n, int k,
                                                              Levels lv, const GridStats* __restrict__ s,
                                                              float* __restrict__ md_out, double* __restrict__ part,
                                                              uint32_t* __restrict__ err) {
    __shared__ float L[KNN_MAX_K1][KNN_THREADS];
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int K1 = k + 1;
    const int tid = threadIdx.x;
    double md = 0.0, md2 = 0.0;
    if (i < n && mask[i] && s->n_valid > k) {
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
        bool done = false;
        for (int l = 0; l < lv.n && !done; l++) {
            cnt = 0;
            const float ic = s->inv_cell[l], cell = s->cell[l];
            int cx, cy, cz;
            cell_of(qx, qy, qz, ic, cx, cy, cz);
            const int rmax = (l == lv.n - 1) ? s->max_ring[l] : LEVEL_RINGS;
            for (int r = 0; r <= rmax; r++) {
                visit_ring(lv.l[l], ic, cx, cy, cz, r, ins);
                float gr = r * cell;
                if (cnt >= K1 && L[K1 - 1][tid] <= gr * gr) { done = true; break; }
            }
        }
        if (!done && cnt < K1) atomicOr(err, 0x10u);  // fewer than k+1 points reachable
        float sum = 0.f;
        for (int j = 1; j < min(cnt, K1); j++) sum += sqrtf(L[j][tid]);
        float m = sum / (float)k;
        md_out[i] = m;
        md = m;
        md2 = (double)(m * m);  // PCL: float square, double sum
    } else if (i < n) {
        md_out[i] = 0.f;
    }
    md = block_sum(md);
    md2 = block_sum(md2);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = md;
        part[2 * blockIdx.x + 1] = md2;
    }
}

// Sums the per-block partials in a fixed order (one CTA).
__global__ void sor_stats_kernel(const double* __restrict__ part, int nb, GridStats* s) {
    double a = 0, b = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    a = block_sum(a);
    b = block_sum(b);
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

// Radius-3-sigma Gaussian: out = p + sum w (q - p) / sum w, accumulated in
// 64-bit fixed point (scale fx) so the result does not depend on the order in
// which the hash buckets hold the neighbours.
__global__ void metric_gaussian_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                       float r2, float inv2s2, double fx, Level g, const GridStats* __restrict__ s,
                                       float* __restrict__ out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float qx = xyz[3 * i], qy = xyz[3 * i + 1], qz = xyz[3 * i + 2];
    if (!mask[i]) {
        out[3 * i] = qx; out[3 * i + 1] = qy; out[3 * i + 2] = qz;
        return;
    }
    const float ic = s->inv_cell[0];
    const float ffx = (float)fx;
    int cx, cy, cz;
    cell_of(qx, qy, qz, ic, cx, cy, cz);
    long long sx = 0, sy = 0, sz = 0, sw = 0;
    auto acc = [&](const float4& p) {
        float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
        float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 > r2) return;
        float w = __expf(-d2 * inv2s2);
        float wf = w * ffx;
        sx += __float2ll_rn(wf * dx);
        sy += __float2ll_rn(wf * dy);
        sz += __float2ll_rn(wf * dz);
        sw += __float2ll_rn(wf);
    };
    visit_ring(g, ic, cx, cy, cz, 0, acc);
    visit_ring(g, ic, cx, cy, cz, 1, acc);
    double iw = 1.0 / (double)sw;
    out[3 * i] = qx + (float)((double)sx * iw);
    out[3 * i + 1] = qy + (float)((double)sy * iw);
    out[3 * i + 2] = qz + (float)((double)sz * iw);
}

unsigned table_size(size_t n) {
    unsigned t = 1024;
    while (t < n && t < (1u << 30)) t <<= 1;
    return t;
}

struct GridScratch {
    GridStats* stats;
    int levels;
    unsigned tsize[MAX_LEVELS];
    unsigned* counts[MAX_LEVELS];
    unsigned* off[MAX_LEVELS];
    float4* pts[MAX_LEVELS];
    unsigned* tot;
    float* md;
    double* part;
};

size_t grid_bytes(size_t n, int levels) {
    size_t b = zim_align256(sizeof(GridStats)) + zim_align256(n * 4) + zim_align256(((n + KNN_THREADS - 1) / KNN_THREADS) * 16);
    size_t tmax = 0;
    for (int l = 0; l < levels; l++) {
        unsigned t = table_size(n >> (2 * l));
        tmax = t > tmax ? t : tmax;
        b += 2 * zim_align256((size_t)t * 4) + zim_align256(n * 16);
    }
    b += zim_align256(((tmax + SCAN_B - 1) / SCAN_B) * 4);
    return b + 2048;
}

zim_status carve_grid(zim_ctx* ctx, size_t n, int levels, GridScratch& G) {
    G.levels = levels;
    G.stats = (GridStats*)zim_scratch_take(ctx, sizeof(GridStats));
    unsigned tmax = 0;
    for (int l = 0; l < levels; l++) {
        G.tsize[l] = table_size(n >> (2 * l));
        tmax = G.tsize[l] > tmax ? G.tsize[l] : tmax;
        G.counts[l] = (unsigned*)zim_scratch_take(ctx, (size_t)G.tsize[l] * 4);
        G.off[l] = (unsigned*)zim_scratch_take(ctx, (size_t)G.tsize[l] * 4);
        G.pts[l] = (float4*)zim_scratch_take(ctx, n * 16);
        if (!G.counts[l] || !G.off[l] || !G.pts[l]) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "grid scratch carve");
    }
    G.tot = (unsigned*)zim_scratch_take(ctx, ((tmax + SCAN_B - 1) / SCAN_B) * 4);
    G.md = (float*)zim_scratch_take(ctx, n * 4);
    G.part = (double*)zim_scratch_take(ctx, ((n + KNN_THREADS - 1) / KNN_THREADS) * 16);
    if (!G.stats || !G.tot || !G.md || !G.part) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "grid scratch carve");
    return ZIM_OK;
}

zim_status build_grid(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, float fixed_cell,
                      float factor, GridScratch& G, cudaStream_t st) {
    size_t n = (size_t)rows * cols;
    unsigned nblk = (unsigned)((n + GB - 1) / GB);
    stats_init_kernel<<<1, 1, 0, st>>>(G.stats);
    spacing1_kernel<<<nblk, GB, 0, st>>>(xyz, mask, rows, cols, G.stats);
    spacing2_kernel<<<nblk, GB, 0, st>>>(xyz, mask, rows, cols, G.stats);
    cell_kernel<<<1, 1, 0, st>>>(G.stats, fixed_cell, factor, G.levels);
    ctx->launches += 4;
    for (int l = 0; l < G.levels; l++) {
        const unsigned T = G.tsize[l], nb = (T + SCAN_B - 1) / SCAN_B;
        ZIM_CUDA_TRY(ctx, cudaMemsetAsync(G.counts[l], 0, (size_t)T * 4, st));
        hash_count_kernel<<<nblk, GB, 0, st>>>(xyz, mask, n, G.stats, l, T - 1, G.counts[l]);
        scan_blocks_kernel<<<nb, SCAN_B, 0, st>>>(G.counts[l], G.off[l], T, G.tot);
        scan_totals_kernel<<<1, SCAN_B, 0, st>>>(G.tot, (int)nb);
        scan_add_kernel<<<nb, SCAN_B, 0, st>>>(G.off[l], T, G.tot);
        ZIM_CUDA_TRY(ctx, cudaMemsetAsync(G.counts[l], 0, (size_t)T * 4, st));
        hash_scatter_kernel<<<nblk, GB, 0, st>>>(xyz, mask, n, G.stats, l, T - 1, G.off[l], G.counts[l], G.pts[l]);
        ctx->launches += 5;
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
    // usually lies within one ring for k <= 50
    float factor = 3.5f * sqrtf(fmaxf(1.0f, (float)mean_k / 30.0f));
    s = build_grid(ctx, xyz, mask, rows, cols, 0.f, factor, G, st);
    if (s) return s;
    Levels lv;
    lv.n = G.levels;
    for (int l = 0; l < G.levels; l++) lv.l[l] = Level{G.off[l], G.counts[l], G.pts[l], G.tsize[l] - 1};
    float* md = mean_dist ? mean_dist : G.md;
    unsigned nblk = (unsigned)((n + KNN_THREADS - 1) / KNN_THREADS);
    sor_knn_kernel<<<nblk, KNN_THREADS, 0, st>>>(xyz, mask, n, mean_k, lv, G.stats, md, G.part, ctx->d_error);
    sor_stats_kernel<<<1, 1024, 0, st>>>(G.part, (int)nblk, G.stats);
    sor_classify_kernel<<<(unsigned)((n + GB - 1) / GB), GB, 0, st>>>(xyz, mask, n, mean_k, std_mul, G.stats, md,
                                                                      mask_out, xyz_out);
    ctx->launches += 3;
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
    s = build_grid(ctx, xyz, mask, rows, cols, rad, 1.0f, G, st);
    if (s) return s;
    Level g{G.off[0], G.counts[0], G.pts[0], G.tsize[0] - 1};
    // fixed-point scale: |w (q - p)| <= rad per term, ~1e4 terms stay below 2^62
    const double fx = std::ldexp(1.0, 40) / fmax(1.0, (double)rad);
    metric_gaussian_kernel<<<(unsigned)((n + GB - 1) / GB), GB, 0, st>>>(
        xyz, mask, n, rad * rad, (float)(1.0 / (2.0 * sigma * sigma)), fx, g, G.stats, out);
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
