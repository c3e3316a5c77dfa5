// mls.cu -- organised-window moving-least-squares smoothing.
//
// Reference: PhaseShiftGrayCode3D/src/JSLAB_MLS_Filter.cpp:11-441 (CPU) and
// JSLAB_MLS_Filter.cu:14-466 (GPU).  Per valid pixel, over the (2hw+1)^2
// window of valid neighbours within the 3-D cut-off: weights
// w = exp(-d^2 / 2 sigma^2), weighted centroid, weighted covariance, closed-form
// symmetric 3x3 eigen-decomposition (normal = smallest eigenvector), then an
// order-0/1/2 polynomial fit f(u, v) in the tangent frame by Cholesky with the
// 2 -> 1 -> 0 fallback, and projection of the point onto the fitted surface.
// Order selection follows the CPU reference: order drops to 0 when fewer than
// {3, 5, 8}[order] neighbours.  Coordinates are accumulated relative to the
// query point, which keeps FP32 sums at millimetre scale.
#include <cmath>

#include "zim_internal.cuh"

namespace {

constexpr int MX = 16, MY = 8;

__device__ void sym_eigen3(const float C[3][3], float ev[3], float E[3][3]) {
    const float p1 = C[0][1] * C[0][1] + C[0][2] * C[0][2] + C[1][2] * C[1][2];
    if (p1 < 1e-20f) {
        ev[0] = C[0][0]; ev[1] = C[1][1]; ev[2] = C[2][2];
        int id[3] = {0, 1, 2};
        for (int i = 0; i < 2; i++)
            for (int j = i + 1; j < 3; j++)
                if (ev[i] > ev[j]) {
                    float t = ev[i]; ev[i] = ev[j]; ev[j] = t;
                    int ti = id[i]; id[i] = id[j]; id[j] = ti;
                }
        for (int i = 0; i < 3; i++)
            for (int c = 0; c < 3; c++) E[i][c] = (c == id[i]) ? 1.f : 0.f;
        return;
    }
    const float tr = C[0][0] + C[1][1] + C[2][2];
    const float q = tr / 3.0f;
    float B[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B[i][j] = C[i][j] - (i == j ? q : 0.f);
    float p2 = B[0][0] * B[0][0] + B[1][1] * B[1][1] + B[2][2] * B[2][2] + 2.0f * p1;
    float p = sqrtf(p2 / 6.0f);
    float ip = p > 1e-15f ? 1.0f / p : 0.f;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B[i][j] *= ip;
    float det = B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) - B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
                B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
    float r = fminf(1.f, fmaxf(-1.f, det * 0.5f));
    float phi = acosf(r) / 3.0f;
    ev[0] = q + 2.0f * p * cosf(phi + 2.0f * ZIM_PI_F / 3.0f);
    ev[2] = q + 2.0f * p * cosf(phi);
    ev[1] = tr - ev[0] - ev[2];
    for (int idx = 0; idx < 3; idx++) {
        float A[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) A[i][j] = C[i][j] - (i == j ? ev[idx] : 0.f);
        float c01[3] = {A[0][1] * A[1][2] - A[0][2] * A[1][1], A[0][2] * A[1][0] - A[0][0] * A[1][2],
                        A[0][0] * A[1][1] - A[0][1] * A[1][0]};
        float c02[3] = {A[0][1] * A[2][2] - A[0][2] * A[2][1], A[0][2] * A[2][0] - A[0][0] * A[2][2],
                        A[0][0] * A[2][1] - A[0][1] * A[2][0]};
        float c12[3] = {A[1][1] * A[2][2] - A[1][2] * A[2][1], A[1][2] * A[2][0] - A[1][0] * A[2][2],
                        A[1][0] * A[2][1] - A[1][1] * A[2][0]};
        float l01 = c01[0] * c01[0] + c01[1] * c01[1] + c01[2] * c01[2];
        float l02 = c02[0] * c02[0] + c02[1] * c02[1] + c02[2] * c02[2];
        float l12 = c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2];
        float b0 = c12[0], b1 = c12[1], b2 = c12[2], bl = l12;
        if (l01 > bl) { b0 = c01[0]; b1 = c01[1]; b2 = c01[2]; bl = l01; }
        if (l02 > bl) { b0 = c02[0]; b1 = c02[1]; b2 = c02[2]; bl = l02; }
        float il = bl > 1e-20f ? rsqrtf(bl) : 0.f;
        E[idx][0] = b0 * il; E[idx][1] = b1 * il; E[idx][2] = b2 * il;
    }
}

// Cholesky solve; thr[i] is the singular-pivot threshold of row i (the
// reference's 1e-12 expressed in the scaled basis).
__device__ bool cholesky_solve(float A[6][6], const float b[6], float x[6], int nc, const float thr[6]) {
    float L[6][6];
    for (int i = 0; i < nc; i++)
        for (int j = 0; j <= i; j++) {
            float s = A[i][j];
            for (int k = 0; k < j; k++) s -= L[i][k] * L[j][k];
            if (i == j) {
                if (s <= thr[i]) return false;
                L[i][j] = sqrtf(s);
            } else {
                L[i][j] = s / L[j][j];
            }
        }
    float y[6];
    for (int i = 0; i < nc; i++) {
        float s = b[i];
        for (int k = 0; k < i; k++) s -= L[i][k] * y[k];
        y[i] = s / L[i][i];
    }
    for (int i = nc - 1; i >= 0; i--) {
        float s = y[i];
        for (int k = i + 1; k < nc; k++) s -= L[k][i] * x[k];
        x[i] = s / L[i][i];
    }
    return true;
}

// MLS of one valid point at pixel (x, y).  nb(i, j, dx, dy, dz) yields the
// offset of the neighbour at pixel (i, j) from the query point and whether it
// is a valid point; the window runs row-major over the pixels of the image.
template <typename Nb>
__device__ __forceinline__ void mls_point(int x, int y, int rows, int cols, int hw, float inv_2s2, int order,
                                          float r2c, Nb nb, float& ox, float& oy, float& oz, bool& moved) {
    moved = false;
    const int r0 = max(0, y - hw), r1 = min(rows, y + hw + 1), c0 = max(0, x - hw), c1 = min(cols, x + hw + 1);
    // 1. weighted centroid (relative to p)
    float cx = 0.f, cy = 0.f, cz = 0.f, ws = 0.f;
    int nv = 0;
    for (int i = r0; i < r1; i++)
        for (int j = c0; j < c1; j++) {
            float dx, dy, dz;
            if (!nb(i, j, dx, dy, dz)) continue;
            float d2 = dx * dx + dy * dy + dz * dz;
            if (!(d2 <= r2c)) continue;
            float w = __expf(-d2 * inv_2s2);
            cx = fmaf(w, dx, cx); cy = fmaf(w, dy, cy); cz = fmaf(w, dz, cz);
            ws += w;
            nv++;
        }
    if (nv < 3 || ws < 1e-12f) return;
    const float iw = 1.0f / ws;
    cx *= iw; cy *= iw; cz *= iw;
    // 2. weighted covariance
    float C[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    for (int i = r0; i < r1; i++)
        for (int j = c0; j < c1; j++) {
            float dx, dy, dz;
            if (!nb(i, j, dx, dy, dz)) continue;
            float d2 = dx * dx + dy * dy + dz * dz;
            if (!(d2 <= r2c)) continue;
            float w = __expf(-d2 * inv_2s2);
            float ex = dx - cx, ey = dy - cy, ez = dz - cz;
            C[0][0] = fmaf(w * ex, ex, C[0][0]); C[0][1] = fmaf(w * ex, ey, C[0][1]); C[0][2] = fmaf(w * ex, ez, C[0][2]);
            C[1][1] = fmaf(w * ey, ey, C[1][1]); C[1][2] = fmaf(w * ey, ez, C[1][2]); C[2][2] = fmaf(w * ez, ez, C[2][2]);
        }
    C[1][0] = C[0][1]; C[2][0] = C[0][2]; C[2][1] = C[1][2];
    float ev[3], E[3][3];
    sym_eigen3(C, ev, E);
    // Orthonormal tangent frame: t1 is re-orthogonalised against the normal and
    // t2 = n x t1.  Exact eigenvectors already satisfy this (up to sign, which
    // the projection is invariant to); in FP32 it keeps the polynomial basis
    // from degenerating when the two in-plane eigenvalues nearly coincide.
    float nx = E[0][0], ny = E[0][1], nz = E[0][2];
    float t1x = E[1][0], t1y = E[1][1], t1z = E[1][2];
    float t2x = E[2][0], t2y = E[2][1], t2z = E[2][2];
    {
        float nn = nx * nx + ny * ny + nz * nz;
        if (nn > 1e-30f) {
            float in = rsqrtf(nn);
            nx *= in; ny *= in; nz *= in;
            float d = t1x * nx + t1y * ny + t1z * nz;
            float ax = t1x - d * nx, ay = t1y - d * ny, az = t1z - d * nz;
            float aa = ax * ax + ay * ay + az * az;
            if (aa > 1e-30f) {
                float ia = rsqrtf(aa);
                t1x = ax * ia; t1y = ay * ia; t1z = az * ia;
                t2x = ny * t1z - nz * t1y;
                t2y = nz * t1x - nx * t1z;
                t2z = nx * t1y - ny * t1x;
            }
        }
    }
    const int min_nb = order == 2 ? 8 : (order == 1 ? 5 : 3);
    int cur = nv >= min_nb ? order : 0;
    // query point relative to the centroid: e0 = p - c = -c_rel
    const float ex0 = -cx, ey0 = -cy, ez0 = -cz;
    bool solved = false;
    float co[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    // Polynomial basis in tangent coordinates scaled by 1/h (h = cut-off
    // radius): the fitted surface is the same, the normal equations are O(1).
    const float is = rsqrtf(r2c);
    float thr[6];
    {
        const float s2 = is * is, s4 = s2 * s2;  // pivot of degree-d row scales by h^(-2d)
        thr[0] = 1e-12f; thr[1] = thr[2] = 1e-12f * s2; thr[3] = thr[4] = thr[5] = 1e-12f * s4;
    }
    if (cur > 0) {
        const int nc = cur == 1 ? 3 : 6;
        float A[6][6], bv[6];
#pragma unroll
        for (int a = 0; a < 6; a++) {
            bv[a] = 0.f;
#pragma unroll
            for (int b = 0; b < 6; b++) A[a][b] = 0.f;
        }
        for (int i = r0; i < r1; i++)
            for (int j = c0; j < c1; j++) {
                float dx, dy, dz;
                if (!nb(i, j, dx, dy, dz)) continue;
                float d2 = dx * dx + dy * dy + dz * dz;
                if (!(d2 <= r2c)) continue;
                float w = __expf(-d2 * inv_2s2);
                float ex = dx - cx, ey = dy - cy, ez = dz - cz;
                float u = (ex * t1x + ey * t1y + ez * t1z) * is;
                float v = (ex * t2x + ey * t2y + ez * t2z) * is;
                float f = ex * nx + ey * ny + ez * nz;
                float bs[6] = {1.f, u, v, u * u, u * v, v * v};
#pragma unroll
                for (int a = 0; a < 6; a++) {
                    if (a < nc) {
                        float wa = w * bs[a];
                        bv[a] = fmaf(wa, f, bv[a]);
#pragma unroll
                        for (int b = 0; b < 6; b++)
                            if (b >= a && b < nc) A[a][b] = fmaf(wa, bs[b], A[a][b]);
                    }
                }
            }
        for (int a = 0; a < nc; a++)
            for (int b = 0; b < a; b++) A[a][b] = A[b][a];
        solved = cholesky_solve(A, bv, co, nc, thr);
        if (!solved && cur == 2) {
            float A1[6][6], b1[6];
            for (int a = 0; a < 3; a++) {
                b1[a] = bv[a];
                for (int b = 0; b < 3; b++) A1[a][b] = A[a][b];
            }
            solved = cholesky_solve(A1, b1, co, 3, thr);
            if (solved) cur = 1;
        }
    }
    if (!solved) {
        float dot = ex0 * nx + ey0 * ny + ez0 * nz;
        ox = -dot * nx; oy = -dot * ny; oz = -dot * nz;
    } else {
        float u0 = ex0 * t1x + ey0 * t1y + ez0 * t1z;
        float v0 = ex0 * t2x + ey0 * t2y + ez0 * t2z;
        float us = u0 * is, vs = v0 * is;
        float ff = co[0] + co[1] * us + co[2] * vs;
        if (cur == 2) ff += co[3] * us * us + co[4] * us * vs + co[5] * vs * vs;
        // out = c + u0 t1 + v0 t2 + f n = p + (c_rel + u0 t1 + v0 t2 + f n)
        ox = cx + u0 * t1x + v0 * t2x + ff * nx;
        oy = cy + u0 * t1y + v0 * t2y + ff * ny;
        oz = cz + u0 * t1z + v0 * t2z + ff * nz;
    }
    moved = true;
}

// Neighbours straight from global memory (windows too wide for shared memory).
__global__ void __launch_bounds__(MX* MY) mls_kernel(const float* __restrict__ src, const uint8_t* __restrict__ mask,
                                                     int rows, int cols, int hw, float inv_2s2, int order, float r2c,
                                                     float* __restrict__ dst) {
    const int x = blockIdx.x * MX + threadIdx.x, y = blockIdx.y * MY + threadIdx.y;
    if (x >= cols || y >= rows) return;
    const size_t o = (size_t)y * cols + x;
    const float px = src[3 * o], py = src[3 * o + 1], pz = src[3 * o + 2];
    float ox = 0.f, oy = 0.f, oz = 0.f;
    bool moved = false;
    if (mask[o]) {
        auto nb = [&](int i, int j, float& dx, float& dy, float& dz) {
            const size_t q = (size_t)i * cols + j;
            if (!__ldg(mask + q)) return false;
            dx = __ldg(src + 3 * q) - px; dy = __ldg(src + 3 * q + 1) - py; dz = __ldg(src + 3 * q + 2) - pz;
            return true;
        };
        mls_point(x, y, rows, cols, hw, inv_2s2, order, r2c, nb, ox, oy, oz, moved);
    }
    dst[3 * o] = moved ? px + ox : px;
    dst[3 * o + 1] = moved ? py + oy : py;
    dst[3 * o + 2] = moved ? pz + oz : pz;
}

// The tile and its hw halo staged in shared memory as float4, NaN for invalid
// and off-image pixels (their distance test fails).
inline size_t mls_smem_bytes(int hw) { return (size_t)(MX + 2 * hw) * (MY + 2 * hw) * sizeof(float4); }

__global__ void __launch_bounds__(MX* MY) mls_smem_kernel(const float* __restrict__ src,
                                                          const uint8_t* __restrict__ mask, int rows, int cols, int hw,
                                                          float inv_2s2, int order, float r2c,
                                                          float* __restrict__ dst) {
    extern __shared__ float4 mls_sp[];
    const int TW = MX + 2 * hw, TH = MY + 2 * hw;
    const int gx0 = blockIdx.x * MX - hw, gy0 = blockIdx.y * MY - hw;
    const int tid = threadIdx.y * MX + threadIdx.x;
    for (int t = tid; t < TW * TH; t += MX * MY) {
        const int ty = t / TW, tx = t - ty * TW;
        const int gx = gx0 + tx, gy = gy0 + ty;
        float4 v = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
        if (gx >= 0 && gy >= 0 && gx < cols && gy < rows) {
            const size_t q = (size_t)gy * cols + gx;
            if (__ldg(mask + q)) v = make_float4(__ldg(src + 3 * q), __ldg(src + 3 * q + 1), __ldg(src + 3 * q + 2), 1.f);
        }
        mls_sp[t] = v;
    }
    __syncthreads();
    const int x = blockIdx.x * MX + threadIdx.x, y = blockIdx.y * MY + threadIdx.y;
    if (x >= cols || y >= rows) return;
    const size_t o = (size_t)y * cols + x;
    const float4 c = mls_sp[(threadIdx.y + hw) * TW + threadIdx.x + hw];
    const float px = src[3 * o], py = src[3 * o + 1], pz = src[3 * o + 2];
    float ox = 0.f, oy = 0.f, oz = 0.f;
    bool moved = false;
    if (c.w != 0.f) {
        auto nb = [&](int i, int j, float& dx, float& dy, float& dz) {
            const float4 q = mls_sp[(i - gy0) * TW + (j - gx0)];
            dx = q.x - px; dy = q.y - py; dz = q.z - pz;
            return true;  // invalid neighbours are NaN and fail the distance test
        };
        mls_point(x, y, rows, cols, hw, inv_2s2, order, r2c, nb, ox, oy, oz, moved);
    }
    dst[3 * o] = moved ? px + ox : px;
    dst[3 * o + 1] = moved ? py + oy : py;
    dst[3 * o + 2] = moved ? pz + oz : pz;
}

}  // namespace

size_t zim_mls_scratch_bytes(size_t n_points) { return zim_align256(n_points * 12); }

zim_status zim_mls_launch(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols, int window,
                          float sigma, int order, float max_radius, int iterations, float* out, float* tmp,
                          cudaStream_t st) {
    const float r2c = max_radius > 0.f ? max_radius * max_radius : 9.0f * sigma * sigma;
    const float inv_2s2 = 1.0f / (2.0f * sigma * sigma);
    const int ord = order < 0 ? 0 : (order > 2 ? 2 : order);
    const int n_iter = iterations < 1 ? 1 : iterations;
    dim3 blk(MX, MY), grd((cols + MX - 1) / MX, (rows + MY - 1) / MY);
    const size_t smem = mls_smem_bytes(window);
    const bool use_smem = smem <= 96 * 1024;
    if (use_smem)
        ZIM_CUDA_TRY(ctx, cudaFuncSetAttribute(mls_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // ping-pong so that the last pass lands in `out`
    const float* in = xyz;
    for (int it = 0; it < n_iter; it++) {
        float* dst = ((n_iter - 1 - it) % 2 == 0) ? out : tmp;
        if (dst == in) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "MLS in-place not supported");
        if (use_smem)
            mls_smem_kernel<<<grd, blk, smem, st>>>(in, mask, rows, cols, window, inv_2s2, ord, r2c, dst);
        else
            mls_kernel<<<grd, blk, 0, st>>>(in, mask, rows, cols, window, inv_2s2, ord, r2c, dst);
        ctx->launches += 1;
        ZIM_LAUNCH_CHECK(ctx);
        in = dst;
    }
    return ZIM_OK;
}

extern "C" ZIM_API zim_status zim_filter_mls(zim_ctx* ctx, const float* xyz, const uint8_t* mask, int rows, int cols,
                                             int window, float sigma, int order, float max_radius, int iterations,
                                             float* out, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!xyz || !mask || !out || rows <= 0 || cols <= 0) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad argument");
    if (window < 0 || window > 64 || !(sigma > 0)) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad MLS parameter");
    if (out == xyz) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "MLS in-place not supported");
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    float* tmp = nullptr;
    if (iterations > 1) {
        zim_status s = zim_scratch_reserve(ctx, zim_mls_scratch_bytes((size_t)rows * cols));
        if (s) return s;
        zim_scratch_reset(ctx);
        tmp = (float*)zim_scratch_take(ctx, (size_t)rows * cols * 12);
    }
    return zim_mls_launch(ctx, xyz, mask, rows, cols, window, sigma, order, max_radius, iterations, out, tmp,
                          zim_stream(stream));
}
