// decode.cu -- per-pixel N-step phase-shift decode: fused 3x3 pre-blur,
// wrapped phase (atan2) + normalised modulation with the validity threshold,
// then heterodyne (reference), hierarchical or Gray-code unwrapping.
//
// Reference: PhaseShiftGrayCode3D/src/JSLAB_PhaseShiftDecoder_V2.cpp:18-28
// (pre-blur), :54-182 (decode body); GPU port JSLAB_PhaseShiftDecoder_V2_GPU.cu:44-146.
//
// Arithmetic is FP32.  The pre-blur is linear, so the blurred sums
// S = -sum sin_k I_k, C = sum cos_k I_k, sum I_k are the 3x3 blur of the raw
// per-pixel sums: a CTA computes the raw sums over its tile + 1-pixel halo into
// shared memory once per frequency and blurs 3 channels instead of N frames.
// Unwrapping keeps integer cycle counts exact and only small fractional parts
// in FP32, so an order differs from the FP64 restatement only when a decision
// argument sits within ~1e-6 of its threshold.
#include <cmath>
#include <mutex>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "zim_tiles.cuh"

namespace {

using zt::DecodeParams;

template <typename T>
__global__ void __launch_bounds__(zt::DX* zt::DY) decode_kernel(const T* __restrict__ frames, DecodeParams p,
                                                                 int32_t* __restrict__ order,
                                                                 float* __restrict__ residual,
                                                                 float* __restrict__ mod_out,
                                                                 uint8_t* __restrict__ valid_out) {
    __shared__ zt::DecodeSmem sm;
    zt::decode_tile<T>(frames, p, blockIdx.x, blockIdx.y, threadIdx.y * zt::DX + threadIdx.x, sm, order, residual,
                       mod_out, valid_out);
}

// ------------------------------------------------------------ TMA staging --
// A decode tile's phase-shift samples (tile + 1-pixel halo, every frame) come
// in one bulk tensor copy (cp.async.bulk.tensor) completing on an mbarrier: a
// 3-D tensor map over (x, y, frame) of the frame stack, box BW x DHY x nfr with
// x starting XP pixels left of the tile (a copy's x must be 16-byte aligned)
// and y one row above.  Samples outside the image read as 0 and are never
// used: the sums clamp to the image, as decode_stage_sums does, and add in the
// same order, so the output is the same bit for bit.
template <typename T>
__host__ __device__ constexpr int tma_xpad() { return 16 / (int)sizeof(T); }
template <typename T>
__host__ __device__ constexpr int tma_bw() { return zt::DX + 2 * tma_xpad<T>(); }
constexpr int TMA_MAX_FRAMES = 24;            // box depth (phase-shift frames) the path takes
constexpr unsigned TMA_POLLS = 1u << 22;      // mbarrier polls before giving up (well over a second)
constexpr uint32_t ERR_DECODE_COPY = 0x20u;   // device error word: a tile copy did not land

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Phase 0 of the barrier completed; false after `polls` polls.
__device__ __forceinline__ bool mbar_wait0(unsigned bar, unsigned polls) {
    for (unsigned it = 0; it < polls; it++) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar)
            : "memory");
        if (done) return true;
    }
    return false;
}

// NPS / NS: frequency count and frames per frequency fixed at compile time
// (0: from p), so the sample loops unroll with constant table offsets.
template <typename T, int NPS, int NS>
__global__ void __launch_bounds__(zt::DX* zt::DY) decode_tma_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                     const T* __restrict__ frames, DecodeParams p,
                                                                     int nfr, int32_t* __restrict__ order,
                                                                     float* __restrict__ residual,
                                                                     float* __restrict__ mod_out,
                                                                     uint8_t* __restrict__ valid_out,
                                                                     uint32_t* __restrict__ err) {
    constexpr int XP = tma_xpad<T>(), BW = tma_bw<T>();
    __shared__ zt::DecodeSmem sm;
    __shared__ __align__(8) unsigned long long bar;
    extern __shared__ __align__(128) unsigned char box_raw[];  // [nfr][DHY][BW] samples
    const T* box = reinterpret_cast<const T*>(box_raw);
    const int tid = threadIdx.y * zt::DX + threadIdx.x;
    const int bx = blockIdx.x, by = blockIdx.y;
    const unsigned b = smem_addr(&bar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        const unsigned bytes = (unsigned)(BW * zt::DHY * nfr * (int)sizeof(T));
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];" ::"r"(smem_addr(box_raw)),
            "l"(reinterpret_cast<unsigned long long>(&tmap)), "r"(bx * zt::DX - XP), "r"(by * zt::DY - 1), "r"(0),
            "r"(b)
            : "memory");
    }
    // bounded: a copy that never lands flags the error word; the tile waits
    // once more (bounded) for it before leaving
    if (!__syncthreads_and(mbar_wait0(b, TMA_POLLS))) {
        if (tid == 0) atomicOr(err, ERR_DECODE_COPY);
        mbar_wait0(b, TMA_POLLS);
        return;
    }
    const int gx0 = bx * zt::DX - 1, gy0 = by * zt::DY - 1;
    const int ox = bx * zt::DX - XP, oy = by * zt::DY - 1;  // box origin
    const int plane = BW * zt::DHY;
    for (int h = tid; h < zt::DHX * zt::DHY; h += zt::DX * zt::DY) {
        const int hy = h / zt::DHX, hx = h - hy * zt::DHX;
        const int gy = min(max(gy0 + hy, 0), p.rows - 1), gx = min(max(gx0 + hx, 0), p.cols - 1);
        const T* bp = box + (gy - oy) * BW + (gx - ox);
        const int n_ps = NPS ? NPS : p.n_ps;
#pragma unroll
        for (int i = 0; i < (NPS ? NPS : zt::DEC_MAX_PS); i++) {
            if (i >= n_ps) break;
            const int f0 = NS ? i * NS : p.fbase[i];  // frequencies' frames are consecutive
            const int N = NS ? NS : p.shift[i];
            float2 sc = make_float2(0.f, 0.f);
            float mv = 0.f;
#pragma unroll
            for (int k = 0; k < (NS ? NS : 32); k++) {  // 3..32 steps
                if (k >= N) break;
                const float v = (float)bp[(f0 + k) * plane];
                sc = zt::sc_add(sc, p.sinv[f0 + k], p.cosv[f0 + k], v);
                mv += v;
            }
            sm.SC[i][hy][hx] = sc;
            sm.M[i][hy][hx] = mv;
        }
    }
    __syncthreads();
    zt::decode_finish<T, NPS, NS>(frames, p, bx, by, tid, sm, order, residual, mod_out, valid_out);
}

// cuTensorMapEncodeTiled from the driver, looked up once (no link to libcuda)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

// The frame stack's tensor map for decode_tma_kernel, or false when the path
// does not apply (HDR, row pitch or base not 16-byte aligned, too many
// frames, an image narrower than the box, no driver entry point).
template <typename T>
bool decode_tensor_map(const void* frames, const DecodeParams& p, CUtensorMap* m, int* nfr_out) {
    if (p.hdr) return false;
    int nfr = 0;
    for (int i = 0; i < p.n_ps; i++) nfr += p.shift[i];
    const size_t es = sizeof(T);
    if (nfr < 1 || nfr > TMA_MAX_FRAMES || ((size_t)p.cols * es) % 16 != 0 || ((uintptr_t)frames & 15) != 0 ||
        p.cols < tma_bw<T>() || p.rows < zt::DHY)
        return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)p.cols, (cuuint64_t)p.rows, (cuuint64_t)nfr};
    const cuuint64_t strides[2] = {(cuuint64_t)p.cols * es, (cuuint64_t)p.rows * p.cols * es};
    const cuuint32_t boxd[3] = {(cuuint32_t)tma_bw<T>(), (cuuint32_t)zt::DHY, (cuuint32_t)nfr};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(m, es == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 3,
                           const_cast<void*>(frames), dims, strides, boxd, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    *nfr_out = nfr;
    return true;
}

template <typename T>
bool launch_decode_tma(zim_ctx* ctx, const void* frames, const DecodeParams& p, dim3 grd, dim3 blk, int32_t* order,
                       float* residual, float* mod, uint8_t* valid, cudaStream_t st) {
    CUtensorMap m;
    int nfr = 0;
    if (!decode_tensor_map<T>(frames, p, &m, &nfr)) return false;
    const size_t dsm = (size_t)tma_bw<T>() * zt::DHY * nfr * sizeof(T);
    bool four = true;  // every frequency 4-step (the common configurations)
    for (int i = 0; i < p.n_ps; i++) four = four && p.shift[i] == 4;
    if (four && p.n_ps == 3)
        decode_tma_kernel<T, 3, 4><<<grd, blk, dsm, st>>>(m, (const T*)frames, p, nfr, order, residual, mod, valid,
                                                          ctx->d_error);
    else if (four && p.n_ps == 1)
        decode_tma_kernel<T, 1, 4><<<grd, blk, dsm, st>>>(m, (const T*)frames, p, nfr, order, residual, mod, valid,
                                                          ctx->d_error);
    else
        decode_tma_kernel<T, 0, 0><<<grd, blk, dsm, st>>>(m, (const T*)frames, p, nfr, order, residual, mod, valid,
                                                          ctx->d_error);
    return true;
}

// Absolute phase as f64 (startCalculate's CV_64F map; 0 where invalid), with
// the optional 3x3 post-smooth (fixed [1/4 1/2 1/4] kernel, BORDER_REPLICATE):
// post_smooth 1 blurs the phase map as is; 2 is the HDR form, the blur divided
// by the blurred validity, 0 at invalid pixels (JSLAB_PhaseShiftDecoder_V2.cpp:280-291);
// 3 is an HDR decode without smoothing.  An HDR decode marks invalid pixels
// with order -1 (a plain decode zeroes them, and Gray code can give a valid -1).
__global__ void phase_f64_kernel(const int32_t* __restrict__ order, const float* __restrict__ res, int rows, int cols,
                                 int post_smooth, double* __restrict__ out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= cols || y >= rows) return;
    const size_t oc = (size_t)y * cols + x;
    const bool hdr = post_smooth >= 2;
    if (post_smooth == 0 || post_smooth == 3) {
        out[oc] = hdr && order[oc] < 0 ? 0.0 : 6.283185307179586 * order[oc] + (double)res[oc];
        return;
    }
    if (hdr && order[oc] < 0) {
        out[oc] = 0.0;
        return;
    }
    double P = 0, W = 0;
    for (int a = -1; a <= 1; a++) {
        int yy = min(max(y + a, 0), rows - 1);
        for (int b = -1; b <= 1; b++) {
            int xx = min(max(x + b, 0), cols - 1);
            int w = (a == 0 ? 2 : 1) * (b == 0 ? 2 : 1);
            size_t o = (size_t)yy * cols + xx;
            if (hdr && order[o] < 0) continue;
            P += w * (6.283185307179586 * order[o] + (double)res[o]);
            W += w;
        }
    }
    out[oc] = hdr ? P / W : P / 16.0;
}

}  // namespace

bool zim_decode_tma_applies(const void* frames, int sample_type, const zt::DecodeParams& p) {
    CUtensorMap m;
    int nfr = 0;
    return sample_type == ZIM_SAMPLE_U8 ? decode_tensor_map<uint8_t>(frames, p, &m, &nfr)
                                        : decode_tensor_map<uint16_t>(frames, p, &m, &nfr);
}

bool zim_decode_tma_launch(zim_ctx* ctx, const void* frames, int sample_type, const zt::DecodeParams& p,
                           int32_t* order, float* residual, cudaStream_t st) {
    dim3 blk(zt::DX, zt::DY), grd((p.cols + zt::DX - 1) / zt::DX, (p.rows + zt::DY - 1) / zt::DY);
    const bool ok = sample_type == ZIM_SAMPLE_U8
                        ? launch_decode_tma<uint8_t>(ctx, frames, p, grd, blk, order, residual, nullptr, nullptr, st)
                        : launch_decode_tma<uint16_t>(ctx, frames, p, grd, blk, order, residual, nullptr, nullptr, st);
    if (ok) ctx->launches += 1;
    return ok;
}

zim_status zim_decode_launch(zim_ctx* ctx, const zim_decode_config* cfg, const void* frames, int sample_type, int rows,
                             int cols, int32_t* order, float* residual, float* mod, uint8_t* valid, cudaStream_t st) {
    DecodeParams p;
    zt::decode_params(cfg, rows, cols, p);
    dim3 blk(zt::DX, zt::DY), grd((cols + zt::DX - 1) / zt::DX, (rows + zt::DY - 1) / zt::DY);
    // the bulk tensor copy path where it applies, else per-thread loads
    const bool u8 = sample_type == ZIM_SAMPLE_U8;
    const bool tma = u8 ? launch_decode_tma<uint8_t>(ctx, frames, p, grd, blk, order, residual, mod, valid, st)
                        : launch_decode_tma<uint16_t>(ctx, frames, p, grd, blk, order, residual, mod, valid, st);
    if (tma) {
    } else if (u8)
        decode_kernel<uint8_t><<<grd, blk, 0, st>>>((const uint8_t*)frames, p, order, residual, mod, valid);
    else
        decode_kernel<uint16_t><<<grd, blk, 0, st>>>((const uint16_t*)frames, p, order, residual, mod, valid);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_decode(zim_ctx* ctx, const zim_decode_config* cfg, const void* frames,
                                         int sample_type, int rows, int cols, int32_t* order, float* residual,
                                         float* mod, uint8_t* valid, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    zim_status s = zim_decode_validate(cfg);
    if (s != ZIM_OK) return zim_fail(ctx, s, "invalid decode config");
    if (!frames || !order || !residual) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    if (rows <= 0 || cols <= 0 || (size_t)rows * cols > ((size_t)1 << 31))
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad image size %dx%d", cols, rows);
    if (sample_type != ZIM_SAMPLE_U8 && sample_type != ZIM_SAMPLE_U16)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad sample type");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return zim_decode_launch(ctx, cfg, frames, sample_type, rows, cols, order, residual, mod, valid, zim_stream(stream));
}

extern "C" ZIM_API zim_status zim_decode_phase_f64(zim_ctx* ctx, const int32_t* order, const float* residual, int rows,
                                                   int cols, int post_smooth, double* phase, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!order || !residual || !phase || rows <= 0 || cols <= 0)
        return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    dim3 blk(256), grd((cols + 255) / 256, rows);
    phase_f64_kernel<<<grd, blk, 0, zim_stream(stream)>>>(order, residual, rows, cols, post_smooth, phase);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    return ZIM_OK;
}
