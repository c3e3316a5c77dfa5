// batch.cu -- the batched path: many stereo pairs of uneven size, encoding and
// calibration through persistent per-stage kernels that drain device work
// queues, captured once as a CUDA graph.
//
// No counterpart in the reference (one pair per call:
// PhaseShiftGrayCode3D/src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:397-480,
// JSLAB_PhaseEpipolarReconstructor_V2_GPU.cu:352-480).  Per pair the stages
// compute exactly what zim_reconstruct_pair computes (the same device code,
// zim_tiles.cuh); what changes is the schedule:
//   stage 1  decode:          item = (pair, camera, band of 8-row tile rows)
//   stage 1b post-smooth of the decoded phase (same items), when configured
//   stage 2  rectify + match: item = (pair, band of rectified rows); the right
//            row is rectified straight into shared memory and each left pixel
//            is rectified in registers, so no rectified phase reaches HBM
//   stage 3  median + reprojection, stage 4 pixel Gaussian, stage 5 radius
//            outlier filter: item = (pair, band of 8-row tile rows)
//   stage 6  the grid filters (SOR -> MLS -> metric Gaussian) of the pairs
//            that turn them on: whole-cloud searches, run per pair on a few
//            lanes (a stream and a scratch context each; the largest pairs
//            first, each to the least-loaded lane), so one pair's
//            latency-bound passes overlap another's kernels
// A persistent CTA takes items from its stage's queue (one atomic per item)
// until the queue is empty, so small and large pairs share the GPU and no
// per-pair launch or tail is paid.  Items are ordered largest pair first.
// Stage order is kept by kernel boundaries (no inter-CTA waits) and, for the
// lanes, by graph edges from the last pixel stage and back to the stream.
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "zim_tiles.cuh"

namespace {

constexpr int BT = 256;  // threads per persistent CTA (one 32 x 8 tile)
static_assert(BT == zt::DX * zt::DY && BT == zt::RX * zt::RY, "tile shape");

enum { Q_DECODE, Q_SMOOTH, Q_MATCH, Q_REPROJ, Q_PXG, Q_ROR, NQ };

struct PairDev {
    zt::DecodeParams dp;
    zt::ReprojParams rp;
    int sample_type;
    const void* frames[2];
    const float* map[2][2];
    int rows, cols, rw, rh;
    int post_smooth, pha_f;
    float grad_threshold;
    int32_t* order[2];
    float* res[2];
    int32_t* sk[2];  // post-smoothed taps (16 x cycles, residual), when post_smooth
    float* sr[2];
    float* disp_raw;
    float* disp_out;
    float* x_rep;  // reprojection output
    uint8_t* m_rep;
    float* x_pxg;  // pixel Gaussian output (mask written only if it updates the mask)
    uint8_t* m_pxg;
    const float* x_ror_in;
    const uint8_t* m_ror_in;
    float* x_ror;
    uint8_t* m_ror;
    float pxg_w00, pxg_w01, pxg_w11;
    float ror_r2;
    int ror_min_nb, ror_hw;
};

struct Queues {
    const int4* items[NQ];
    int n[NQ];
};

// One item index per CTA: thread 0 takes it, everyone reads it.  The caller's
// trailing __syncthreads keeps the next write behind every read.
__device__ __forceinline__ int next_item(unsigned* counter, int* s_item) {
    if (threadIdx.x == 0) *s_item = (int)atomicAdd(counter, 1u);
    __syncthreads();
    return *s_item;
}

__global__ void __launch_bounds__(BT) batch_decode_kernel(const PairDev* __restrict__ pairs, const int4* __restrict__ items,
                                                          int n_items, unsigned* __restrict__ counter) {
    __shared__ zt::DecodeSmem sm;
    __shared__ zt::DecodeParams dp;
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int it = next_item(counter, &s_item);
        if (it >= n_items) break;
        const int4 w = items[it];  // pair, camera, first tile row, tile rows
        const PairDev& P = pairs[w.x];
        {
            const int* src = reinterpret_cast<const int*>(&P.dp);
            int* dst = reinterpret_cast<int*>(&dp);
            for (int k = tid; k < (int)(sizeof(zt::DecodeParams) / 4); k += BT) dst[k] = __ldg(src + k);
        }
        __syncthreads();
        const int tiles_x = (P.cols + zt::DX - 1) / zt::DX;
        const void* fr = P.frames[w.y];
        int32_t* ord = P.order[w.y];
        float* res = P.res[w.y];
        for (int ty = w.z; ty < w.z + w.w; ty++)
            for (int tx = 0; tx < tiles_x; tx++) {
                if (P.sample_type == ZIM_SAMPLE_U8)
                    zt::decode_tile<uint8_t>((const uint8_t*)fr, dp, tx, ty, tid, sm, ord, res, nullptr, nullptr);
                else
                    zt::decode_tile<uint16_t>((const uint16_t*)fr, dp, tx, ty, tid, sm, ord, res, nullptr, nullptr);
            }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(BT) batch_smooth_kernel(const PairDev* __restrict__ pairs,
                                                          const int4* __restrict__ items, int n_items,
                                                          unsigned* __restrict__ counter) {
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int it = next_item(counter, &s_item);
        if (it >= n_items) break;
        const int4 w = items[it];  // pair, camera, first tile row, tile rows
        const PairDev& P = pairs[w.x];
        const int tiles_x = (P.cols + zt::DX - 1) / zt::DX;
        for (int ty = w.z; ty < w.z + w.w; ty++)
            for (int tx = 0; tx < tiles_x; tx++) {
                const int x = tx * zt::DX + tid % zt::DX, y = ty * zt::DY + tid / zt::DX;
                if (x >= P.cols || y >= P.rows) continue;
                if (P.post_smooth == 2)
                    zt::smooth_pixel_hdr(P.order[w.y], P.res[w.y], P.rows, P.cols, x, y, P.sk[w.y], P.sr[w.y]);
                else
                    zt::smooth_pixel(P.order[w.y], P.res[w.y], P.rows, P.cols, x, y, P.sk[w.y], P.sr[w.y]);
            }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(BT) batch_match_kernel(const PairDev* __restrict__ pairs, const int4* __restrict__ items,
                                                         int n_items, unsigned* __restrict__ counter, int max_cols) {
    extern __shared__ int4 smem_raw[];
    int* s_ord = reinterpret_cast<int*>(smem_raw);
    int* s_base = s_ord + max_cols;
    float* s_res = reinterpret_cast<float*>(s_base + max_cols);
    int* s_lo = reinterpret_cast<int*>(s_res + max_cols);
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int it = next_item(counter, &s_item);
        if (it >= n_items) break;
        const int4 w = items[it];  // pair, first rectified row, rows
        const PairDev& P = pairs[w.x];
        const int cols = P.rw, pha_f = P.pha_f;
        int* s_hi = s_lo + (pha_f + 1);
        int* s_bad = s_hi + (pha_f + 1);
        for (int row = w.y; row < w.y + w.z; row++) {
            const size_t ro = (size_t)row * cols;
            for (int k = tid; k <= pha_f; k += BT) {
                s_lo[k] = INT_MAX;
                s_hi[k] = -1;
                s_bad[k] = 0;
            }
            for (int j = tid; j < cols; j += BT) {
                int32_t b, o;
                float r;
                if (P.post_smooth == 1 || P.post_smooth == 2)
                    zt::rectify_pixel_smoothed(P.sk[1], P.sr[1], P.order[1], P.rows, P.cols,
                                               __ldg(P.map[1][0] + ro + j), __ldg(P.map[1][1] + ro + j), b, r, o);
                else
                    zt::rectify_pixel(P.order[1], P.res[1], P.rows, P.cols, __ldg(P.map[1][0] + ro + j),
                                      __ldg(P.map[1][1] + ro + j), P.post_smooth, b, r, o);
                s_ord[j] = o;
                s_base[j] = b;
                s_res[j] = r;
            }
            __syncthreads();
            zt::match_spans(s_ord, cols, pha_f, s_lo, s_hi, tid, BT);
            __syncthreads();
            zt::match_spans_check(s_ord, s_base, s_res, cols, pha_f, s_hi, s_bad, tid, BT);
            __syncthreads();
            for (int j = tid; j < cols; j += BT) {
                int32_t bL, kL;
                float rL;
                if (P.post_smooth == 1 || P.post_smooth == 2)
                    zt::rectify_pixel_smoothed(P.sk[0], P.sr[0], P.order[0], P.rows, P.cols,
                                               __ldg(P.map[0][0] + ro + j), __ldg(P.map[0][1] + ro + j), bL, rL, kL);
                else
                    zt::rectify_pixel(P.order[0], P.res[0], P.rows, P.cols, __ldg(P.map[0][0] + ro + j),
                                      __ldg(P.map[0][1] + ro + j), P.post_smooth, bL, rL, kL);
                float d;
                int best;
                zt::match_pixel(j, kL, bL, rL, s_ord, s_base, s_res, s_lo, s_hi, s_bad, cols, pha_f, P.grad_threshold,
                                d, best);
                P.disp_raw[ro + j] = d;
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(BT) batch_reproject_kernel(const PairDev* __restrict__ pairs,
                                                             const int4* __restrict__ items, int n_items,
                                                             unsigned* __restrict__ counter) {
    __shared__ zt::MedianSmem sm;
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int it = next_item(counter, &s_item);
        if (it >= n_items) break;
        const int4 w = items[it];  // pair, first tile row, tile rows
        const PairDev& P = pairs[w.x];
        const int tiles_x = (P.rw + zt::MTX - 1) / zt::MTX;
        for (int ty = w.y; ty < w.y + w.z; ty++)
            for (int tx = 0; tx < tiles_x; tx++)
                zt::median_reproject_tile(P.disp_raw, P.rh, P.rw, P.rp, tx, ty, tid, sm, P.disp_out, P.x_rep, P.m_rep);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(BT) batch_pxg_kernel(const PairDev* __restrict__ pairs,
                                                       const int4* __restrict__ items, int n_items,
                                                       unsigned* __restrict__ counter) {
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int it = next_item(counter, &s_item);
        if (it >= n_items) break;
        const int4 w = items[it];
        const PairDev& P = pairs[w.x];
        const int tiles_x = (P.rw + zt::RX - 1) / zt::RX;
        for (int ty = w.y; ty < w.y + w.z; ty++)
            for (int tx = 0; tx < tiles_x; tx++) {
                const int x = tx * zt::RX + tid % zt::RX, y = ty * zt::RY + tid / zt::RX;
                if (x >= P.rw || y >= P.rh) continue;
                zt::px_gaussian_pixel(P.x_rep, P.m_rep, P.rh, P.rw, x, y, P.pxg_w00, P.pxg_w01, P.pxg_w11, P.x_pxg,
                                      P.m_pxg);
            }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(BT) batch_ror_kernel(const PairDev* __restrict__ pairs,
                                                       const int4* __restrict__ items, int n_items,
                                                       unsigned* __restrict__ counter) {
    extern __shared__ float4 ror_smem[];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        const int it = next_item(counter, &s_item);
        if (it >= n_items) break;
        const int4 w = items[it];
        const PairDev& P = pairs[w.x];
        const int tiles_x = (P.rw + zt::RX - 1) / zt::RX;
        for (int ty = w.y; ty < w.y + w.z; ty++)
            for (int tx = 0; tx < tiles_x; tx++)
                zt::ror_tile(P.x_ror_in, P.m_ror_in, P.rh, P.rw, tx, ty, tid, P.ror_r2, P.ror_min_nb, P.ror_hw,
                             ror_smem, P.x_ror, P.m_ror);
        __syncthreads();
    }
}

}  // namespace

struct zim_batch {
    zim_ctx* ctx = nullptr;
    int device = 0;  // the context's device, kept so that destruction never reads the context
    std::vector<zim_rect_state> calibs;
    std::vector<zim_batch_pair> pairs;
    zim_recon_config rcfg{};
    bool use_pxg = false, use_ror = false;
    zim_batch_tuning tuning{4, 4, 4, 4};
    bool tuned = false;
    // device state of the submission
    void* d_mem = nullptr;  // intermediates + descriptors + queues, one allocation
    size_t d_bytes = 0;
    PairDev* d_pairs = nullptr;
    unsigned* d_counters = nullptr;
    Queues q{};
    int max_cols = 0, max_pha_f = 0;
    size_t match_smem = 0;
    size_t ror_smem = 0;
    int grid[NQ] = {0, 0, 0, 0, 0, 0};
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // host layout of the intermediates (for resubmission with another tuning)
    std::vector<PairDev> host_pairs;
    std::vector<char> tma;  // per pair: decoded by the bulk-copy kernel, not the queue
    size_t items_off = 0;
    // grid filters: per pair the resolved config and its buffers (x_in / m_in:
    // the pixel stages' output; x1, x2: intermediate clouds; mls_tmp: MLS
    // ping-pong for three or more passes)
    struct GridRoute {
        bool on = false;
        const float* x_in = nullptr;
        const uint8_t* m_in = nullptr;
        float *x1 = nullptr, *x2 = nullptr, *mls_tmp = nullptr;
    };
    std::vector<zim_recon_config> filt;
    std::vector<GridRoute> groute;
    static constexpr int MAX_LANES = 6;
    int n_lanes = 0;
    zim_ctx* lane_ctx[MAX_LANES] = {};
    cudaStream_t lane_stream[MAX_LANES] = {};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[MAX_LANES] = {};
    unsigned long long lane_launches = 0;  // grid-filter kernels per graph replay
};

namespace {

void release_submission(zim_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    cudaFree(b->d_mem);
    b->d_mem = nullptr;
    b->d_bytes = 0;
}

int occupancy(const void* fn, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, BT, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

// Builds the work items for a tuning (largest pair first) into host vectors.
void build_items(const zim_batch* b, const zim_batch_tuning& t, std::vector<int4> (&items)[NQ]) {
    std::vector<int> order(b->pairs.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        return (size_t)b->pairs[a].rows * b->pairs[a].cols > (size_t)b->pairs[c].rows * b->pairs[c].cols;
    });
    for (int q = 0; q < NQ; q++) items[q].clear();
    for (int pi : order) {
        const zim_batch_pair& p = b->pairs[pi];
        const zim_rect_state& C = b->calibs[p.calib];
        const int trows = (p.rows + zt::DY - 1) / zt::DY;
        const bool tma = (size_t)pi < b->tma.size() && b->tma[pi];
        for (int cam = 0; cam < 2; cam++)
            for (int r = 0; r < trows; r += t.decode_rows) {
                const int4 it = make_int4(pi, cam, r, std::min(t.decode_rows, trows - r));
                if (!tma) items[Q_DECODE].push_back(it);
                if (p.decode.post_smooth) items[Q_SMOOTH].push_back(it);  // modes 1 and 2
            }
        for (int r = 0; r < C.rect_h; r += t.match_rows)
            items[Q_MATCH].push_back(make_int4(pi, r, std::min(t.match_rows, C.rect_h - r), 0));
        const int rtrows = (C.rect_h + zt::RY - 1) / zt::RY;
        for (int r = 0; r < rtrows; r += t.filter_rows) {
            const int4 it = make_int4(pi, r, std::min(t.filter_rows, rtrows - r), 0);
            items[Q_REPROJ].push_back(it);
            if (b->use_pxg) items[Q_PXG].push_back(it);
            if (b->use_ror) items[Q_ROR].push_back(it);
        }
    }
}

// One pair's grid filters on a lane: SOR -> MLS -> metric Gaussian as the
// whole-pair path chains them (the same launch functions, the same inputs),
// the last writer of xyz / mask writing the pair's outputs.
zim_status lane_filters(zim_batch* b, int pi, zim_ctx* lctx, cudaStream_t st) {
    const zim_batch_pair& p = b->pairs[pi];
    const zim_recon_config& r = b->filt[pi];
    const zim_batch::GridRoute& g = b->groute[pi];
    const zim_rect_state& C = b->calibs[p.calib];
    const int RH = C.rect_h, RW = C.rect_w;
    const zim_ray_model rays = zim_rays_from(C.Q, C.R1, b->rcfg.use_rectified_coords != 0, 0, 0);
    const int last = r.use_metric_gaussian ? 2 : (r.use_mls ? 1 : 0);
    const float* cx = g.x_in;
    const uint8_t* cm = g.m_in;
    zim_scratch_reset(lctx);
    if (r.use_sor) {
        float* ox = last == 0 ? p.xyz : g.x1;
        zim_status s = zim_sor_launch(lctx, cx, cm, RH, RW, r.sor_mean_k, r.sor_std_mul, ox, p.mask, nullptr, rays, st);
        if (s) return s;
        zim_scratch_reset(lctx);
        cx = ox;
        cm = p.mask;
    }
    if (r.use_mls) {
        float* ox = last == 1 ? p.xyz : (cx == g.x1 ? g.x2 : g.x1);
        zim_status s = zim_mls_launch(lctx, cx, cm, RH, RW, r.mls_window_size, r.mls_spatial_sigma,
                                      r.mls_polynomial_order, r.mls_max_radius, r.mls_iterations, ox, g.mls_tmp, rays,
                                      st);
        if (s) return s;
        cx = ox;
    }
    if (r.use_metric_gaussian) {
        zim_status s = zim_metric_gaussian_launch(lctx, cx, cm, RH, RW, r.metric_gaussian_sigma, p.xyz, rays, st);
        if (s) return s;
        zim_scratch_reset(lctx);
    }
    return ZIM_OK;
}

// Lanes for the grid filters: n contexts on the batch's device (scratch
// reserved for the largest filtered cloud), a stream and a join event each.
zim_status setup_lanes(zim_batch* b, int n, size_t scratch) {
    zim_ctx* ctx = b->ctx;
    for (int l = 0; l < n; l++) {
        if (!b->lane_ctx[l]) {
            zim_status s = zim_create(ctx->device, &b->lane_ctx[l]);
            if (s) return zim_fail(ctx, s, "lane context creation failed");
            ZIM_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&b->lane_stream[l], cudaStreamNonBlocking));
            ZIM_CUDA_TRY(ctx, cudaEventCreateWithFlags(&b->join_ev[l], cudaEventDisableTiming));
        }
        zim_status s = zim_scratch_reserve(b->lane_ctx[l], scratch);
        if (s) return zim_fail(ctx, s, "lane scratch: %s", zim_last_error(b->lane_ctx[l]));
    }
    if (!b->fork_ev) ZIM_CUDA_TRY(ctx, cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
    b->n_lanes = n;
    return ZIM_OK;
}

void free_lanes(zim_batch* b) {
    for (int l = 0; l < zim_batch::MAX_LANES; l++) {
        if (b->lane_ctx[l]) zim_destroy(b->lane_ctx[l]);
        if (b->lane_stream[l]) cudaStreamDestroy(b->lane_stream[l]);
        if (b->join_ev[l]) cudaEventDestroy(b->join_ev[l]);
        b->lane_ctx[l] = nullptr;
        b->lane_stream[l] = nullptr;
        b->join_ev[l] = nullptr;
    }
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    b->fork_ev = nullptr;
    b->n_lanes = 0;
}

zim_status capture(zim_batch* b) {
    zim_ctx* ctx = b->ctx;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 152;
    const int want = std::max(1, b->tuning.ctas_per_sm);
    b->grid[Q_DECODE] = sms * std::min(want, occupancy((const void*)batch_decode_kernel, 0));
    b->grid[Q_SMOOTH] = sms * std::min(want, occupancy((const void*)batch_smooth_kernel, 0));
    b->grid[Q_MATCH] = sms * std::min(want, occupancy((const void*)batch_match_kernel, b->match_smem));
    b->grid[Q_REPROJ] = sms * std::min(want, occupancy((const void*)batch_reproject_kernel, 0));
    b->grid[Q_PXG] = sms * std::min(want, occupancy((const void*)batch_pxg_kernel, 0));
    b->grid[Q_ROR] = sms * std::min(want, occupancy((const void*)batch_ror_kernel, b->ror_smem));
    cudaStream_t s = b->cap_stream;
    ZIM_CUDA_TRY(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(b->d_counters, 0, NQ * sizeof(unsigned), s);
    const Queues& q = b->q;
    // pairs the bulk-copy decode takes (its own launch per camera; the same
    // arithmetic as the queue's tiles)
    for (size_t pi = 0; pi < b->tma.size(); pi++)
        if (b->tma[pi]) {
            const PairDev& D = b->host_pairs[pi];
            for (int c = 0; c < 2; c++)
                if (!zim_decode_tma_launch(ctx, D.frames[c], D.sample_type, D.dp, D.order[c], D.res[c], s)) {
                    cudaGraph_t g = nullptr;
                    cudaStreamEndCapture(s, &g);
                    if (g) cudaGraphDestroy(g);
                    return zim_fail(ctx, ZIM_ERR_CUDA, "batch decode copy path unavailable");
                }
        }
    if (q.n[Q_DECODE])
        batch_decode_kernel<<<std::min(b->grid[Q_DECODE], q.n[Q_DECODE]), BT, 0, s>>>(
            b->d_pairs, q.items[Q_DECODE], q.n[Q_DECODE], b->d_counters + Q_DECODE);
    if (q.n[Q_SMOOTH])
        batch_smooth_kernel<<<std::min(b->grid[Q_SMOOTH], q.n[Q_SMOOTH]), BT, 0, s>>>(
            b->d_pairs, q.items[Q_SMOOTH], q.n[Q_SMOOTH], b->d_counters + Q_SMOOTH);
    if (q.n[Q_MATCH])
        batch_match_kernel<<<std::min(b->grid[Q_MATCH], q.n[Q_MATCH]), BT, b->match_smem, s>>>(
            b->d_pairs, q.items[Q_MATCH], q.n[Q_MATCH], b->d_counters + Q_MATCH, b->max_cols);
    if (q.n[Q_REPROJ])
        batch_reproject_kernel<<<std::min(b->grid[Q_REPROJ], q.n[Q_REPROJ]), BT, 0, s>>>(
            b->d_pairs, q.items[Q_REPROJ], q.n[Q_REPROJ], b->d_counters + Q_REPROJ);
    if (q.n[Q_PXG])
        batch_pxg_kernel<<<std::min(b->grid[Q_PXG], q.n[Q_PXG]), BT, 0, s>>>(b->d_pairs, q.items[Q_PXG], q.n[Q_PXG],
                                                                            b->d_counters + Q_PXG);
    if (q.n[Q_ROR])
        batch_ror_kernel<<<std::min(b->grid[Q_ROR], q.n[Q_ROR]), BT, b->ror_smem, s>>>(
            b->d_pairs, q.items[Q_ROR], q.n[Q_ROR], b->d_counters + Q_ROR);
    cudaError_t le = cudaGetLastError();
    // the grid filters: the lanes fork from the capture after the pixel stages
    // and join back before its end
    zim_status fs = ZIM_OK;
    b->lane_launches = 0;
    if (le == cudaSuccess && b->n_lanes > 0) {
        unsigned long long l0 = 0;
        for (int l = 0; l < b->n_lanes; l++) l0 += b->lane_ctx[l]->launches;
        le = cudaEventRecord(b->fork_ev, s);
        for (int l = 0; le == cudaSuccess && l < b->n_lanes; l++) le = cudaStreamWaitEvent(b->lane_stream[l], b->fork_ev, 0);
        // largest cost first, each pair to the lane with the least work so far
        // (cost ~ rectified pixels, weighted by the filters the pair runs)
        std::vector<std::pair<double, int>> order;
        for (size_t pi = 0; pi < b->groute.size(); pi++)
            if (b->groute[pi].on) {
                const zim_recon_config& f = b->filt[pi];
                const zim_rect_state& C = b->calibs[b->pairs[pi].calib];
                const double w = (f.use_sor ? 1.0 : 0.0) + (f.use_mls ? 1.3 * std::max(1, f.mls_iterations) : 0.0) +
                                 (f.use_metric_gaussian ? 0.4 : 0.0);
                order.push_back({-w * C.rect_w * (double)C.rect_h, (int)pi});
            }
        std::sort(order.begin(), order.end());
        double load[zim_batch::MAX_LANES] = {};
        for (size_t k = 0; le == cudaSuccess && fs == ZIM_OK && k < order.size(); k++) {
            int lane = 0;
            for (int l = 1; l < b->n_lanes; l++)
                if (load[l] < load[lane]) lane = l;
            load[lane] -= order[k].first;
            fs = lane_filters(b, order[k].second, b->lane_ctx[lane], b->lane_stream[lane]);
        }
        for (int l = 0; le == cudaSuccess && l < b->n_lanes; l++) {
            le = cudaEventRecord(b->join_ev[l], b->lane_stream[l]);
            if (le == cudaSuccess) le = cudaStreamWaitEvent(s, b->join_ev[l], 0);
        }
        unsigned long long l1 = 0;
        for (int l = 0; l < b->n_lanes; l++) l1 += b->lane_ctx[l]->launches;
        b->lane_launches = l1 - l0;
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (le != cudaSuccess || e != cudaSuccess || fs != ZIM_OK) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (fs != ZIM_OK) {
            const zim_ctx* lc = nullptr;
            for (int l = 0; l < b->n_lanes; l++)
                if (b->lane_ctx[l] && !b->lane_ctx[l]->last_error.empty()) lc = b->lane_ctx[l];
            return zim_fail(ctx, fs, "batch grid filters: %s", lc ? lc->last_error.c_str() : "failed");
        }
        return zim_fail(ctx, ZIM_ERR_CUDA, "batch graph capture failed: %s",
                        cudaGetErrorString(le != cudaSuccess ? le : e));
    }
    b->graph = g;
    ZIM_CUDA_TRY(ctx, cudaGraphInstantiate(&b->exec, g, 0));
    return ZIM_OK;
}

// Rebuilds the work queues for b->tuning (same pairs, same buffers) and recaptures.
zim_status requeue(zim_batch* b) {
    zim_ctx* ctx = b->ctx;
    std::vector<int4> items[NQ];
    build_items(b, b->tuning, items);
    size_t need = 0;
    for (int q = 0; q < NQ; q++) need += zim_align256(items[q].size() * sizeof(int4) + 16);
    if (b->items_off + need > b->d_bytes) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "batch item space");
    char* base = (char*)b->d_mem + b->items_off;
    ZIM_CUDA_TRY(ctx, cudaDeviceSynchronize());
    for (int q = 0; q < NQ; q++) {
        if (!items[q].empty())
            ZIM_CUDA_TRY(ctx, cudaMemcpy(base, items[q].data(), items[q].size() * sizeof(int4), cudaMemcpyHostToDevice));
        b->q.items[q] = (const int4*)base;
        b->q.n[q] = (int)items[q].size();
        base += zim_align256(items[q].size() * sizeof(int4) + 16);
    }
    return capture(b);
}

// Upper bound of the item space over the tunings the autotuner tries (1-row bands).
size_t max_item_bytes(const zim_batch* b) {
    size_t n[NQ] = {0, 0, 0, 0, 0, 0};
    for (const zim_batch_pair& p : b->pairs) {
        const zim_rect_state& C = b->calibs[p.calib];
        n[Q_DECODE] += 2 * (size_t)((p.rows + zt::DY - 1) / zt::DY);
        n[Q_SMOOTH] += 2 * (size_t)((p.rows + zt::DY - 1) / zt::DY);
        n[Q_MATCH] += (size_t)C.rect_h;
        const size_t rt = (C.rect_h + zt::RY - 1) / zt::RY;
        n[Q_REPROJ] += rt;
        n[Q_PXG] += rt;
        n[Q_ROR] += rt;
    }
    size_t s = 0;
    for (int q = 0; q < NQ; q++) s += zim_align256(n[q] * sizeof(int4) + 16);
    return s;
}

bool tuning_ok(const zim_batch_tuning& t) {
    return t.decode_rows >= 1 && t.decode_rows <= 1024 && t.match_rows >= 1 && t.match_rows <= 1024 &&
           t.filter_rows >= 1 && t.filter_rows <= 1024 && t.ctas_per_sm >= 1 && t.ctas_per_sm <= 32;
}

}  // namespace

extern "C" ZIM_API zim_status zim_batch_create(zim_ctx* ctx, const zim_stereo_calib* calibs, int n_calibs,
                                               int use_full_left, zim_batch** out) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!calibs || n_calibs < 1 || !out) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    *out = nullptr;
    zim_batch* b = new zim_batch;
    b->ctx = ctx;
    b->device = ctx->device;
    for (int i = 0; i < n_calibs; i++) {
        zim_rect_state st;
        zim_status s = zim_rect_build(ctx, &calibs[i], use_full_left, st);
        if (s) {
            zim_batch_destroy(b);
            return s;
        }
        b->calibs.push_back(st);
    }
    if (cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        zim_batch_destroy(b);
        return zim_fail(ctx, ZIM_ERR_CUDA, "stream creation failed");
    }
    *out = b;
    return ZIM_OK;
}

// Destruction reads nothing of the batch's context, which a garbage-collected
// host language may already have destroyed (the reverse order of creation is
// not guaranteed there).  It cannot report errors, so it clears those its own
// calls leave behind rather than let a later call of the thread report them.
extern "C" ZIM_API void zim_batch_destroy(zim_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    cudaDeviceSynchronize();
    release_submission(b);
    free_lanes(b);
    for (zim_rect_state& st : b->calibs) zim_rect_free(st);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    delete b;
    cudaGetLastError();
}

extern "C" ZIM_API zim_status zim_batch_rect_size(const zim_batch* b, int calib, int* rw, int* rh) {
    if (!b || calib < 0 || calib >= (int)b->calibs.size()) return ZIM_ERR_INVALID_ARG;
    if (rw) *rw = b->calibs[calib].rect_w;
    if (rh) *rh = b->calibs[calib].rect_h;
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_batch_submit(zim_batch* b, const zim_batch_pair* pairs, int n_pairs,
                                               const zim_recon_config* rcfg, const zim_batch_tuning* tuning) {
    if (!b) return ZIM_ERR_INVALID_ARG;
    zim_ctx* ctx = b->ctx;
    if (!pairs || n_pairs < 1 || !rcfg) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    if (rcfg->reproject_model != 0)
        return zim_fail(ctx, ZIM_ERR_UNSUPPORTED, "the batch reprojects through each calibration's Q matrix");
    if (rcfg->use_ror && (rcfg->radius_window_size < 0 || rcfg->radius_window_size > ZIM_MAX_ROR_WINDOW))
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "radius_window_size must be in [0, %d]", ZIM_MAX_ROR_WINDOW);
    if (tuning && !tuning_ok(*tuning)) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad tuning");
    int max_cols = 1, max_pha = 0;
    for (int i = 0; i < n_pairs; i++) {
        const zim_batch_pair& p = pairs[i];
        if (p.calib < 0 || p.calib >= (int)b->calibs.size())
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pair %d: bad calibration index", i);
        const zim_rect_state& C = b->calibs[p.calib];
        if (p.rows != C.src_h || p.cols != C.src_w)
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pair %d: image %dx%d differs from its calibration's %dx%d", i,
                            p.cols, p.rows, C.src_w, C.src_h);
        zim_status s = zim_decode_validate(&p.decode);
        if (s) return zim_fail(ctx, s, "pair %d: invalid decode config", i);
        if (p.sample_type != ZIM_SAMPLE_U8 && p.sample_type != ZIM_SAMPLE_U16)
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pair %d: bad sample type", i);
        if (!p.frames[0] || !p.frames[1] || !p.xyz || !p.mask)
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pair %d: null frames or outputs", i);
        if (C.rect_w > ZIM_MAX_MATCH_COLS) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pair %d: rectified width", i);
        const zim_recon_config& f = p.filters ? *p.filters : *rcfg;
        if (f.use_sor && (f.sor_mean_k < 1 || f.sor_mean_k > 63))
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pair %d: sor_mean_k must be in [1, 63]", i);
        if (f.use_mls && (f.mls_window_size < 0 || f.mls_window_size > 64 || !(f.mls_spatial_sigma > 0)))
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pair %d: bad MLS parameter", i);
        if (f.use_metric_gaussian && !(f.metric_gaussian_sigma > 0))
            return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pair %d: metric_gaussian_sigma must be positive", i);
        const int pf = p.pha_f > 0 ? p.pha_f : zim_decode_max_order(&p.decode);
        if (pf < 0 || pf > ZIM_MAX_ORDER) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "pair %d: pha_f out of range", i);
        max_cols = std::max(max_cols, C.rect_w);
        max_pha = std::max(max_pha, pf);
    }
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    ZIM_CUDA_TRY(ctx, cudaDeviceSynchronize());
    release_submission(b);
    b->pairs.assign(pairs, pairs + n_pairs);
    b->rcfg = *rcfg;
    // the grid filters of each pair (copied: the caller's configs need not outlive the call)
    b->filt.assign(n_pairs, *rcfg);
    b->groute.assign(n_pairs, zim_batch::GridRoute{});
    size_t lane_scratch = 0;
    int n_filtered = 0;
    for (int i = 0; i < n_pairs; i++) {
        if (b->pairs[i].filters) b->filt[i] = *b->pairs[i].filters;
        b->pairs[i].filters = nullptr;
        const zim_recon_config& f = b->filt[i];
        b->groute[i].on = f.use_sor || f.use_mls || f.use_metric_gaussian;
        if (b->groute[i].on) {
            const zim_rect_state& C = b->calibs[b->pairs[i].calib];
            lane_scratch = std::max(lane_scratch, zim_grid_scratch_bytes((size_t)C.rect_w * C.rect_h) + 4096);
            n_filtered++;
        }
    }
    b->use_pxg = rcfg->use_px_gaussian != 0;
    b->use_ror = rcfg->use_ror != 0;
    if (tuning) b->tuning = *tuning;
    b->max_cols = max_cols;
    b->max_pha_f = max_pha;
    b->match_smem = (size_t)max_cols * 12 + (size_t)(max_pha + 1) * 12;
    ZIM_CUDA_TRY(ctx, cudaFuncSetAttribute(batch_match_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)b->match_smem));
    b->ror_smem = b->use_ror ? zt::ror_smem_bytes(rcfg->radius_window_size / 2) : 0;
    if (b->use_ror)
        ZIM_CUDA_TRY(ctx, cudaFuncSetAttribute(batch_ror_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)b->ror_smem));

    // memory plan: descriptors, counters, per-pair intermediates, items
    const bool pxg_mask = b->use_pxg && rcfg->px_gaussian_updates_mask;
    size_t bytes = zim_align256(sizeof(PairDev) * n_pairs) + 256;
    for (const zim_batch_pair& p : b->pairs) {
        const zim_rect_state& C = b->calibs[p.calib];
        const size_t src = (size_t)p.rows * p.cols, dst = (size_t)C.rect_w * C.rect_h;
        bytes += 2 * (zim_align256(src * 4) * (p.decode.post_smooth ? 4 : 2)) + zim_align256(dst * 4);
        bytes += 2 * (zim_align256(dst * 12) + zim_align256(dst));  // two intermediate clouds at most
    }
    for (int i = 0; i < n_pairs; i++)
        if (b->groute[i].on) {  // the pixel stages' cloud + mask, two filter clouds, MLS ping-pong
            const zim_rect_state& C = b->calibs[b->pairs[i].calib];
            const size_t dst = (size_t)C.rect_w * C.rect_h;
            bytes += 4 * zim_align256(dst * 12) + zim_align256(dst);
        }
    b->items_off = bytes;
    bytes += max_item_bytes(b) + 4096;
    if (cudaMalloc(&b->d_mem, bytes) != cudaSuccess) {
        cudaGetLastError();
        return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "batch allocation of %zu bytes failed", bytes);
    }
    b->d_bytes = bytes;
    char* cur = (char*)b->d_mem;
    auto take = [&](size_t n) {
        char* p = cur;
        cur += zim_align256(n);
        return (void*)p;
    };
    b->d_pairs = (PairDev*)take(sizeof(PairDev) * n_pairs);
    b->d_counters = (unsigned*)take(NQ * sizeof(unsigned));
    float w00, w01, w11;
    zt::px_gaussian_weights(w00, w01, w11);
    b->host_pairs.assign(n_pairs, PairDev{});
    for (int i = 0; i < n_pairs; i++) {
        const zim_batch_pair& p = b->pairs[i];
        const zim_rect_state& C = b->calibs[p.calib];
        PairDev& D = b->host_pairs[i];
        std::memset(&D, 0, sizeof D);
        zt::decode_params(&p.decode, p.rows, p.cols, D.dp);
        zt::reproj_params(C.Q, C.R1, rcfg, D.rp);
        D.sample_type = p.sample_type;
        D.rows = p.rows; D.cols = p.cols; D.rw = C.rect_w; D.rh = C.rect_h;
        D.post_smooth = p.decode.enable_hdr ? (p.decode.post_smooth ? 2 : 3) : (p.decode.post_smooth ? 1 : 0);
        D.pha_f = p.pha_f > 0 ? p.pha_f : zim_decode_max_order(&p.decode);
        D.grad_threshold = (float)rcfg->grad_threshold;
        const size_t src = (size_t)p.rows * p.cols, dst = (size_t)C.rect_w * C.rect_h;
        for (int c = 0; c < 2; c++) {
            D.frames[c] = p.frames[c];
            D.map[c][0] = C.d_map[c][0];
            D.map[c][1] = C.d_map[c][1];
            D.order[c] = (int32_t*)take(src * 4);
            D.res[c] = (float*)take(src * 4);
            if (p.decode.post_smooth) {
                D.sk[c] = (int32_t*)take(src * 4);
                D.sr[c] = (float*)take(src * 4);
            }
        }
        D.disp_raw = (float*)take(dst * 4);
        D.disp_out = p.disp;
        // stage routing: the last writer of xyz / mask writes the caller's
        // buffers; with grid filters the pixel stages end in intermediates (the
        // mask too when SOR rewrites it) and the filters write the outputs
        zim_batch::GridRoute& G = b->groute[i];
        float* out_x = p.xyz;
        uint8_t* out_m = p.mask;
        if (G.on) {
            out_x = (float*)take(dst * 12);
            if (b->filt[i].use_sor) out_m = (uint8_t*)take(dst);
            G.x1 = (float*)take(dst * 12);
            G.x2 = (float*)take(dst * 12);
            G.mls_tmp = (float*)take(dst * 12);
            G.x_in = out_x;
            G.m_in = out_m;
        }
        float* xbuf[2] = {(float*)take(dst * 12), (float*)take(dst * 12)};
        uint8_t* mbuf[2] = {(uint8_t*)take(dst), (uint8_t*)take(dst)};
        const bool last_rep = !b->use_pxg && !b->use_ror;
        D.x_rep = last_rep ? out_x : xbuf[0];
        D.m_rep = (!pxg_mask && !b->use_ror) ? out_m : mbuf[0];
        if (b->use_pxg) {
            D.x_pxg = b->use_ror ? xbuf[1] : out_x;
            D.m_pxg = pxg_mask ? (b->use_ror ? mbuf[1] : out_m) : nullptr;
            D.pxg_w00 = w00; D.pxg_w01 = w01; D.pxg_w11 = w11;
        }
        if (b->use_ror) {
            D.x_ror_in = b->use_pxg ? D.x_pxg : D.x_rep;
            D.m_ror_in = pxg_mask ? D.m_pxg : D.m_rep;
            D.x_ror = out_x;
            D.m_ror = out_m;
            D.ror_r2 = rcfg->radius_search * rcfg->radius_search;
            D.ror_min_nb = rcfg->radius_min_neighbors;
            D.ror_hw = rcfg->radius_window_size / 2;
        }
    }
    if ((size_t)(cur - (char*)b->d_mem) > b->items_off)
        return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "batch memory plan overflow");
    b->items_off = (size_t)(cur - (char*)b->d_mem);
    ZIM_CUDA_TRY(ctx, cudaMemcpy(b->d_pairs, b->host_pairs.data(), sizeof(PairDev) * n_pairs, cudaMemcpyHostToDevice));
    b->tma.assign(n_pairs, 0);
    for (int i = 0; i < n_pairs; i++) {
        const PairDev& D = b->host_pairs[i];
        b->tma[i] = zim_decode_tma_applies(D.frames[0], D.sample_type, D.dp) &&
                    zim_decode_tma_applies(D.frames[1], D.sample_type, D.dp);
    }
    b->n_lanes = 0;
    if (n_filtered) {
        zim_status s = setup_lanes(b, std::min(n_filtered, (int)zim_batch::MAX_LANES), lane_scratch);
        if (s) return s;
    }
    return requeue(b);
}

extern "C" ZIM_API zim_status zim_batch_run(zim_batch* b, void* stream) {
    if (!b) return ZIM_ERR_INVALID_ARG;
    if (!b->exec) return zim_fail(b->ctx, ZIM_ERR_INVALID_ARG, "nothing submitted");
    ZIM_CUDA_TRY(b->ctx, cudaGraphLaunch(b->exec, zim_stream(stream)));
    for (int q = 0; q < NQ; q++) b->ctx->launches += b->q.n[q] > 0 ? 1 : 0;  // kernels in the graph
    b->ctx->launches += b->lane_launches;
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_batch_get_tuning(const zim_batch* b, zim_batch_tuning* out) {
    if (!b || !out) return ZIM_ERR_INVALID_ARG;
    *out = b->tuning;
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_batch_autotune(zim_batch* b, void* stream, zim_batch_tuning* best, double* best_ms) {
    if (!b) return ZIM_ERR_INVALID_ARG;
    zim_ctx* ctx = b->ctx;
    if (!b->exec) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "nothing submitted");
    cudaStream_t st = zim_stream(stream);
    cudaEvent_t e0, e1;
    ZIM_CUDA_TRY(ctx, cudaEventCreate(&e0));
    ZIM_CUDA_TRY(ctx, cudaEventCreate(&e1));
    auto time_it = [&](double& ms) -> zim_status {
        zim_status s = requeue(b);
        if (s) return s;
        ZIM_CUDA_TRY(ctx, cudaGraphLaunch(b->exec, st));  // warm-up
        ZIM_CUDA_TRY(ctx, cudaEventRecord(e0, st));
        const int reps = 3;
        for (int r = 0; r < reps; r++) ZIM_CUDA_TRY(ctx, cudaGraphLaunch(b->exec, st));
        ZIM_CUDA_TRY(ctx, cudaEventRecord(e1, st));
        ZIM_CUDA_TRY(ctx, cudaEventSynchronize(e1));
        float f = 0.f;
        ZIM_CUDA_TRY(ctx, cudaEventElapsedTime(&f, e0, e1));
        ms = f / reps;
        return ZIM_OK;
    };
    // coordinate descent over the four tunables from the current tuning
    zim_batch_tuning cur = b->tuning;
    double cur_ms = 0;
    b->tuning = cur;
    zim_status s = time_it(cur_ms);
    const int cand[4][5] = {{1, 2, 4, 8, 16}, {1, 2, 4, 8, 16}, {1, 2, 4, 8, 16}, {1, 2, 4, 8, 16}};
    for (int pass = 0; pass < 2 && !s; pass++)
        for (int k = 0; k < 4 && !s; k++)
            for (int c = 0; c < 5 && !s; c++) {
                zim_batch_tuning t = cur;
                int* f = k == 0 ? &t.decode_rows : k == 1 ? &t.match_rows : k == 2 ? &t.filter_rows : &t.ctas_per_sm;
                if (*f == cand[k][c]) continue;
                *f = cand[k][c];
                b->tuning = t;
                double ms = 0;
                s = time_it(ms);
                if (!s && ms < cur_ms) {
                    cur = t;
                    cur_ms = ms;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->tuning = cur;
    zim_status s2 = requeue(b);
    if (s) return s;
    if (s2) return s2;
    b->tuned = true;
    if (best) *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return ZIM_OK;
}
