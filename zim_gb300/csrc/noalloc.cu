// noalloc.cu -- point compaction that allocates no device memory.
//
// zim_compact_points needs a small per-call scratch (one count per 1024
// pixels) that it takes from the context's cudaMalloc'ed arena.  Some callers
// cannot call cudaMalloc: a host application that owns all device memory
// through its own pool and forbids libraries from allocating (frame-grabber
// SDKs, capture services that reserve memory once at start-up), or a capture
// loop that cannot afford the implicit device-wide synchronisation cudaMalloc
// and cudaFree may perform.  zim_compact_points_noalloc serves them: its
// scratch is the file-scope array below, so a call allocates nothing and needs
// no context.
//
// The array holds ZIM_NOALLOC_COMPACT_MAX_BLOCKS counts (256 KiB), enough for
// 64 Mi pixels (e.g. 8192 x 8192).  Every GPU that loads the library keeps it
// until the process exits.  All calls on a device share it and it keeps the
// last call's contents; every word a call reads is written earlier in that same
// call, so nothing needs clearing between calls.  Calls that overlap on the GPU
// (two streams, or two host threads) race on the array: serialise them.
//
// The first call on a device runs a one-time set-up (cudaGetSymbolAddress with
// that device current); make that first call before any stream capture.  The
// address found there is kept for the life of the process: a cudaDeviceReset
// of that device (which unloads this library's device code and may reload it
// elsewhere) leaves it stale, so do not call this entry point on a device
// after resetting it.
//
// Each of the three launches is checked through its own return code
// (cudaLaunchKernel), so an error left pending by other work on the calling
// thread is neither reported as this call's nor cleared by it.
#include <mutex>

#include "zim_internal.cuh"

#define ZIM_NOALLOC_COMPACT_BLOCK 1024
#define ZIM_NOALLOC_COMPACT_MAX_BLOCKS 65536
#define ZIM_NOALLOC_MAX_DEVICES 64

namespace {

// Per-block counts of valid pixels, then their exclusive prefix sums.
static __device__ __align__(256) uint32_t g_compact_blocks[ZIM_NOALLOC_COMPACT_MAX_BLOCKS];

std::mutex g_setup_mu;
uint32_t* g_blocks_addr[ZIM_NOALLOC_MAX_DEVICES] = {};

__global__ void na_count_kernel(const uint8_t* __restrict__ mask, size_t n, uint32_t* __restrict__ blocks) {
    __shared__ uint32_t warp_cnt[ZIM_NOALLOC_COMPACT_BLOCK / 32];
    const size_t i = (size_t)blockIdx.x * ZIM_NOALLOC_COMPACT_BLOCK + threadIdx.x;
    const unsigned b = __ballot_sync(0xffffffffu, i < n && mask[i] != 0);
    if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t s = warp_cnt[threadIdx.x];
        for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (threadIdx.x == 0) blocks[blockIdx.x] = s;
    }
}

// One CTA: exclusive prefix sum of the nb block counts in place; the total
// goes to *count_dev.
__global__ void na_scan_kernel(uint32_t* __restrict__ blocks, int nb, uint64_t* __restrict__ count_dev) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int base = 0; base < nb; base += ZIM_NOALLOC_COMPACT_BLOCK) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < nb ? blocks[i] : 0u;
        uint32_t x = v;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += t;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            uint32_t y = warp_tot[lane];
            for (int off = 1; off < 32; off <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, y, off);
                if (lane >= off) y += t;
            }
            warp_tot[lane] = y;
        }
        __syncthreads();
        const uint32_t incl = x + (w ? warp_tot[w - 1] : 0u);
        const uint32_t c = carry;
        if (i < nb) blocks[i] = c + incl - v;
        __syncthreads();
        if (threadIdx.x == ZIM_NOALLOC_COMPACT_BLOCK - 1) carry = c + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *count_dev = carry;
}

__global__ void na_write_kernel(const float* __restrict__ xyz, const uint8_t* __restrict__ mask, size_t n,
                                const uint32_t* __restrict__ offsets, zim_point_xyz* __restrict__ pts) {
    __shared__ uint32_t warp_off[ZIM_NOALLOC_COMPACT_BLOCK / 32];
    const size_t i = (size_t)blockIdx.x * ZIM_NOALLOC_COMPACT_BLOCK + threadIdx.x;
    const bool v = i < n && mask[i] != 0;
    const unsigned b = __ballot_sync(0xffffffffu, v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warp_off[w] = __popc(b);
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t s = warp_off[threadIdx.x], x = s;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += t;
        }
        warp_off[threadIdx.x] = x - s;
    }
    __syncthreads();
    if (v) {
        const uint32_t pos = offsets[blockIdx.x] + warp_off[w] + __popc(b & ((1u << lane) - 1u));
        pts[pos] = zim_point_xyz{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 1.0f};
    }
}

// Device address of g_compact_blocks for the current device (set-up on the
// first call per device, with that device current).
cudaError_t blocks_address(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= ZIM_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_blocks_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_compact_blocks);
        if (e != cudaSuccess) return e;
        g_blocks_addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_blocks_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" ZIM_API zim_status zim_compact_points_noalloc(const float* xyz, const uint8_t* mask, int rows, int cols,
                                                         zim_point_xyz* points, uint64_t* count_dev, void* stream) {
    if (!xyz || !mask || !points || !count_dev || rows <= 0 || cols <= 0) return ZIM_ERR_INVALID_ARG;
    const size_t n = (size_t)rows * cols;
    const size_t nb = (n + ZIM_NOALLOC_COMPACT_BLOCK - 1) / ZIM_NOALLOC_COMPACT_BLOCK;
    if (nb > ZIM_NOALLOC_COMPACT_MAX_BLOCKS) return ZIM_ERR_INVALID_ARG;  // more than 64 Mi pixels
    uint32_t* blocks = nullptr;
    if (blocks_address(&blocks) != cudaSuccess) {
        cudaGetLastError();
        return ZIM_ERR_CUDA;
    }
    cudaStream_t st = zim_stream(stream);
    int nbi = (int)nb;
    void* count_args[] = {(void*)&mask, (void*)&n, (void*)&blocks};
    void* scan_args[] = {(void*)&blocks, (void*)&nbi, (void*)&count_dev};
    void* write_args[] = {(void*)&xyz, (void*)&mask, (void*)&n, (void*)&blocks, (void*)&points};
    const dim3 grid((unsigned)nb), one(1), blk(ZIM_NOALLOC_COMPACT_BLOCK);
    cudaError_t e = cudaLaunchKernel((const void*)na_count_kernel, grid, blk, count_args, 0, st);
    if (e == cudaSuccess) e = cudaLaunchKernel((const void*)na_scan_kernel, one, blk, scan_args, 0, st);
    if (e == cudaSuccess) e = cudaLaunchKernel((const void*)na_write_kernel, grid, blk, write_args, 0, st);
    if (e != cudaSuccess) {
        cudaGetLastError();  // the failed launch recorded its own error: clear that one
        return ZIM_ERR_CUDA;
    }
    return ZIM_OK;
}
