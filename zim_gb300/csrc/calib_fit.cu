// calib_fit.cu -- per-pixel cubic depth calibration from reference planes:
// JSLAB_StereoCalib_V2::computePixelwiseDepthCalibration
// (PhaseShiftGrayCode3D/src/JSLAB_StereoCalib_V2.cpp:113-240).
//
// 1. Each reference plane: the valid pixels (mask != 0, d > 0) are reprojected
//    through Q in the rectified frame; the plane through them is the PCA plane
//    (normal = eigenvector of the smallest eigenvalue of the scatter matrix,
//    D = -n . mean).  The scatter is reduced on the device in FP64 in a fixed
//    order (mean first, then centred products); the 3x3 eigenproblem is solved
//    on the host (cyclic Jacobi).
// 2. Each pixel: every plane where it is valid gives a sample (d, p - n (n.p + D)),
//    the reprojected point moved along the normal onto the plane; with at least
//    4 samples, X, Y and Z are fitted as cubics in d by least squares.  The
//    reference solves the raw Vandermonde system [1 d d^2 d^3] by SVD; here the
//    fit runs in FP64 on the scaled variable t = (d - m) / s in [-1, 1]
//    (condition number ~10^3 instead of ~10^14 for the normal equations in d),
//    by Cholesky of the 4x4 normal equations, with a Jacobi pseudo-inverse for
//    rank-deficient pixels; the cubic is then expanded back to powers of d.
//    For full-rank pixels this is the same least-squares polynomial.
#include <cmath>
#include <vector>

#include "zim_internal.cuh"

namespace {

constexpr int FIT_B = 256;
constexpr int MOM_BLOCKS = 608;  // fixed grid: the reduction order does not depend on the device
constexpr int MAX_PLANES = 64;

struct QParams {
    double q03, q13, q23, q32, q33;
};

__device__ __forceinline__ void q_point(const QParams& q, int c, int r, double d, double& x, double& y, double& z) {
    const double w = q.q32 * d + q.q33;
    x = ((double)c + q.q03) / w;
    y = ((double)r + q.q13) / w;
    z = q.q23 / w;
}

template <int NM>
__device__ __forceinline__ void block_sum(double* v, double* part) {
    __shared__ double ws[FIT_B / 32][NM];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int m = 0; m < NM; m++)
        for (int off = 16; off; off >>= 1) v[m] += __shfl_down_sync(0xffffffffu, v[m], off);
    if (lane == 0)
#pragma unroll
        for (int m = 0; m < NM; m++) ws[w][m] = v[m];
    __syncthreads();
    if (threadIdx.x < NM) {
        double s = 0.0;
        for (int k = 0; k < FIT_B / 32; k++) s += ws[k][threadIdx.x];
        part[(size_t)blockIdx.x * NM + threadIdx.x] = s;
    }
}

// pass 0: count, sum x, y, z; pass 1: centred xx, xy, xz, yy, yz, zz.
template <int PASS>
__global__ void __launch_bounds__(FIT_B) plane_moments_kernel(const float* __restrict__ disp,
                                                              const uint8_t* __restrict__ mask, int rows, int cols,
                                                              QParams q, double mx, double my, double mz,
                                                              double* __restrict__ part) {
    constexpr int NM = PASS == 0 ? 4 : 6;
    double v[NM];
#pragma unroll
    for (int m = 0; m < NM; m++) v[m] = 0.0;
    const size_t n = (size_t)rows * cols;
    for (size_t i = (size_t)blockIdx.x * FIT_B + threadIdx.x; i < n; i += (size_t)MOM_BLOCKS * FIT_B) {
        const float d = disp[i];
        if (!mask[i] || !(d > 0.f)) continue;
        double x, y, z;
        q_point(q, (int)(i % cols), (int)(i / cols), (double)d, x, y, z);
        if constexpr (PASS == 0) {
            v[0] += 1.0; v[1] += x; v[2] += y; v[3] += z;
        } else {
            x -= mx; y -= my; z -= mz;
            v[0] += x * x; v[1] += x * y; v[2] += x * z;
            v[3] += y * y; v[4] += y * z; v[5] += z * z;
        }
    }
    block_sum<NM>(v, part);
}

struct FitPlanes {
    const float* disp[MAX_PLANES];
    const uint8_t* mask[MAX_PLANES];
    double eq[MAX_PLANES][4];  // A, B, C, D with A^2 + B^2 + C^2 = 1
    int n;
};

// Symmetric 4x4 solve G a = b (3 right-hand sides): Cholesky, or for a
// rank-deficient G the pseudo-inverse from a cyclic Jacobi eigendecomposition
// (eigenvalues below 1e-12 of the largest are dropped).
__device__ void solve4(double G[4][4], double b[4][3], double a[4][3]) {
    double L[4][4] = {};
    bool ok = true;
    double dmax = 0.0;
    for (int i = 0; i < 4; i++) dmax = fmax(dmax, G[i][i]);
    for (int j = 0; j < 4 && ok; j++) {
        double s = G[j][j];
        for (int k = 0; k < j; k++) s -= L[j][k] * L[j][k];
        if (!(s > 1e-12 * dmax)) { ok = false; break; }
        L[j][j] = sqrt(s);
        for (int i = j + 1; i < 4; i++) {
            double t = G[i][j];
            for (int k = 0; k < j; k++) t -= L[i][k] * L[j][k];
            L[i][j] = t / L[j][j];
        }
    }
    if (ok) {
        for (int c = 0; c < 3; c++) {
            double y[4];
            for (int i = 0; i < 4; i++) {
                double t = b[i][c];
                for (int k = 0; k < i; k++) t -= L[i][k] * y[k];
                y[i] = t / L[i][i];
            }
            for (int i = 3; i >= 0; i--) {
                double t = y[i];
                for (int k = i + 1; k < 4; k++) t -= L[k][i] * a[k][c];
                a[i][c] = t / L[i][i];
            }
        }
        return;
    }
    double A[4][4], V[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            A[i][j] = G[i][j];
            V[i][j] = i == j ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 30; sweep++) {
        double off = 0.0;
        for (int p = 0; p < 4; p++)
            for (int r = p + 1; r < 4; r++) off += A[p][r] * A[p][r];
        if (off <= 1e-30 * (dmax * dmax + 1e-300)) break;
        for (int p = 0; p < 4; p++)
            for (int r = p + 1; r < 4; r++) {
                if (A[p][r] == 0.0) continue;
                const double th = (A[r][r] - A[p][p]) / (2.0 * A[p][r]);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 4; k++) {
                    const double akp = A[k][p], akr = A[k][r];
                    A[k][p] = c * akp - s * akr;
                    A[k][r] = s * akp + c * akr;
                }
                for (int k = 0; k < 4; k++) {
                    const double apk = A[p][k], ark = A[r][k];
                    A[p][k] = c * apk - s * ark;
                    A[r][k] = s * apk + c * ark;
                }
                for (int k = 0; k < 4; k++) {
                    const double vkp = V[k][p], vkr = V[k][r];
                    V[k][p] = c * vkp - s * vkr;
                    V[k][r] = s * vkp + c * vkr;
                }
            }
    }
    double lmax = 0.0;
    for (int i = 0; i < 4; i++) lmax = fmax(lmax, A[i][i]);
    for (int c = 0; c < 3; c++) {
        for (int i = 0; i < 4; i++) a[i][c] = 0.0;
        for (int e = 0; e < 4; e++) {
            if (!(A[e][e] > 1e-12 * lmax)) continue;
            double proj = 0.0;
            for (int k = 0; k < 4; k++) proj += V[k][e] * b[k][c];
            proj /= A[e][e];
            for (int i = 0; i < 4; i++) a[i][c] += V[i][e] * proj;
        }
    }
}

__global__ void __launch_bounds__(FIT_B) pixel_fit_kernel(const FitPlanes* __restrict__ P, int rows, int cols,
                                                          QParams q, float4* __restrict__ cx, float4* __restrict__ cy,
                                                          float4* __restrict__ cz) {
    const size_t n = (size_t)rows * cols;
    const size_t i = (size_t)blockIdx.x * FIT_B + threadIdx.x;
    if (i >= n) return;
    const int c = (int)(i % cols), r = (int)(i / cols);
    const int np = P->n;
    int cnt = 0;
    double dmin = INFINITY, dmax = -INFINITY;
    for (int k = 0; k < np; k++) {
        const float d = P->disp[k][i];
        if (!P->mask[k][i] || !(d > 0.f)) continue;
        cnt++;
        dmin = fmin(dmin, (double)d);
        dmax = fmax(dmax, (double)d);
    }
    float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    if (cnt < 4) {
        cx[i] = zero; cy[i] = zero; cz[i] = zero;
        return;
    }
    const double m = 0.5 * (dmin + dmax);
    const double s = dmax > dmin ? 0.5 * (dmax - dmin) : 1.0;
    double G[4][4] = {}, b[4][3] = {};
    for (int k = 0; k < np; k++) {
        const float df = P->disp[k][i];
        if (!P->mask[k][i] || !(df > 0.f)) continue;
        const double d = df;
        double x, y, z;
        q_point(q, c, r, d, x, y, z);
        const double A = P->eq[k][0], B = P->eq[k][1], C = P->eq[k][2], D = P->eq[k][3];
        const double dist = A * x + B * y + C * z + D;
        const double tgt[3] = {x - A * dist, y - B * dist, z - C * dist};
        const double t = (d - m) / s;
        const double v[4] = {1.0, t, t * t, t * t * t};
        for (int a = 0; a < 4; a++) {
            for (int e = 0; e <= a; e++) G[a][e] += v[a] * v[e];
            for (int h = 0; h < 3; h++) b[a][h] += v[a] * tgt[h];
        }
    }
    for (int a = 0; a < 4; a++)
        for (int e = a + 1; e < 4; e++) G[a][e] = G[e][a];
    double sol[4][3];
    solve4(G, b, sol);
    // p(d) = sum_k sol_k ((d - m) / s)^k  ->  sum_j c_j d^j
    const double binom[4][4] = {{1, 0, 0, 0}, {1, 1, 0, 0}, {1, 2, 1, 0}, {1, 3, 3, 1}};
    float out[3][4];
    for (int h = 0; h < 3; h++)
        for (int j = 0; j < 4; j++) {
            double acc = 0.0;
            for (int kk = j; kk < 4; kk++) {
                const double sk = sol[kk][h] / pow(s, (double)kk);
                acc += sk * binom[kk][j] * pow(-m, (double)(kk - j));
            }
            out[h][j] = (float)acc;
        }
    cx[i] = make_float4(out[0][0], out[0][1], out[0][2], out[0][3]);
    cy[i] = make_float4(out[1][0], out[1][1], out[1][2], out[1][3]);
    cz[i] = make_float4(out[2][0], out[2][1], out[2][2], out[2][3]);
}

// Cyclic Jacobi on a symmetric 3x3 matrix; returns the unit eigenvector of the
// smallest eigenvalue.
void smallest_eigvec3(double S[3][3], double n[3]) {
    double A[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) A[i][j] = S[i][j];
    for (int sweep = 0; sweep < 50; sweep++) {
        const double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        const double diag = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
        if (off <= 1e-32 * diag) break;
        for (int p = 0; p < 3; p++)
            for (int r = p + 1; r < 3; r++) {
                if (A[p][r] == 0.0) continue;
                const double th = (A[r][r] - A[p][p]) / (2.0 * A[p][r]);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; k++) {
                    const double akp = A[k][p], akr = A[k][r];
                    A[k][p] = c * akp - s * akr;
                    A[k][r] = s * akp + c * akr;
                }
                for (int k = 0; k < 3; k++) {
                    const double apk = A[p][k], ark = A[r][k];
                    A[p][k] = c * apk - s * ark;
                    A[r][k] = s * apk + c * ark;
                }
                for (int k = 0; k < 3; k++) {
                    const double vkp = V[k][p], vkr = V[k][r];
                    V[k][p] = c * vkp - s * vkr;
                    V[k][r] = s * vkp + c * vkr;
                }
            }
    }
    int e = 0;
    for (int i = 1; i < 3; i++)
        if (A[i][i] < A[e][e]) e = i;
    const double len = std::sqrt(V[0][e] * V[0][e] + V[1][e] * V[1][e] + V[2][e] * V[2][e]);
    for (int k = 0; k < 3; k++) n[k] = V[k][e] / len;
}

}  // namespace

extern "C" ZIM_API zim_status zim_fit_poly_calib(zim_ctx* ctx, const double Q[16], const float* const* disps,
                                                 const uint8_t* const* masks, int n_planes, int rows, int cols,
                                                 float* cx, float* cy, float* cz, double* plane_eqs, void* stream) {
    if (!ctx) return ZIM_ERR_INVALID_ARG;
    if (!Q || !disps || !masks || !cx || !cy || !cz) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null argument");
    if (n_planes < 1 || n_planes > MAX_PLANES) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "1..%d planes", MAX_PLANES);
    if (rows <= 0 || cols <= 0) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "bad size");
    for (int k = 0; k < n_planes; k++)
        if (!disps[k] || !masks[k]) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "null plane %d", k);
    ZIM_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = zim_stream(stream);
    const QParams q{Q[3], Q[7], Q[11], Q[14], Q[15]};
    zim_status s = zim_scratch_reserve(ctx, zim_align256(sizeof(FitPlanes)) + zim_align256(MOM_BLOCKS * 6 * 8) + 512);
    if (s) return s;
    zim_scratch_reset(ctx);
    FitPlanes* dP = (FitPlanes*)zim_scratch_take(ctx, sizeof(FitPlanes));
    double* part = (double*)zim_scratch_take(ctx, (size_t)MOM_BLOCKS * 6 * 8);
    if (!dP || !part) return zim_fail(ctx, ZIM_ERR_OUT_OF_MEMORY, "fit scratch");
    FitPlanes hP{};
    hP.n = n_planes;
    std::vector<double> hpart((size_t)MOM_BLOCKS * 6);
    for (int k = 0; k < n_planes; k++) {
        hP.disp[k] = disps[k];
        hP.mask[k] = masks[k];
        double sum[6] = {0, 0, 0, 0, 0, 0};
        plane_moments_kernel<0><<<MOM_BLOCKS, FIT_B, 0, st>>>(disps[k], masks[k], rows, cols, q, 0, 0, 0, part);
        ctx->launches += 1;
        ZIM_LAUNCH_CHECK(ctx);
        ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(hpart.data(), part, (size_t)MOM_BLOCKS * 4 * 8, cudaMemcpyDeviceToHost, st));
        ZIM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        for (int b = 0; b < MOM_BLOCKS; b++)
            for (int m = 0; m < 4; m++) sum[m] += hpart[(size_t)b * 4 + m];
        if (sum[0] < 3) return zim_fail(ctx, ZIM_ERR_INVALID_ARG, "plane %d has %g valid pixels (PCA needs 3)", k, sum[0]);
        const double mx = sum[1] / sum[0], my = sum[2] / sum[0], mz = sum[3] / sum[0];
        plane_moments_kernel<1><<<MOM_BLOCKS, FIT_B, 0, st>>>(disps[k], masks[k], rows, cols, q, mx, my, mz, part);
        ctx->launches += 1;
        ZIM_LAUNCH_CHECK(ctx);
        ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(hpart.data(), part, (size_t)MOM_BLOCKS * 6 * 8, cudaMemcpyDeviceToHost, st));
        ZIM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        double c6[6] = {0, 0, 0, 0, 0, 0};
        for (int b = 0; b < MOM_BLOCKS; b++)
            for (int m = 0; m < 6; m++) c6[m] += hpart[(size_t)b * 6 + m];
        double S[3][3] = {{c6[0], c6[1], c6[2]}, {c6[1], c6[3], c6[4]}, {c6[2], c6[4], c6[5]}};
        double nrm[3];
        smallest_eigvec3(S, nrm);
        hP.eq[k][0] = nrm[0];
        hP.eq[k][1] = nrm[1];
        hP.eq[k][2] = nrm[2];
        hP.eq[k][3] = -(nrm[0] * mx + nrm[1] * my + nrm[2] * mz);
        if (plane_eqs)
            for (int j = 0; j < 4; j++) plane_eqs[4 * k + j] = hP.eq[k][j];
    }
    ZIM_CUDA_TRY(ctx, cudaMemcpyAsync(dP, &hP, sizeof hP, cudaMemcpyHostToDevice, st));
    const size_t n = (size_t)rows * cols;
    pixel_fit_kernel<<<(unsigned)((n + FIT_B - 1) / FIT_B), FIT_B, 0, st>>>(dP, rows, cols, q, (float4*)cx,
                                                                            (float4*)cy, (float4*)cz);
    ctx->launches += 1;
    ZIM_LAUNCH_CHECK(ctx);
    // hP lives on this stack frame: the copy must finish before returning
    ZIM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return ZIM_OK;
}
