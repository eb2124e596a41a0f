// Spot-check correction of the learned scatter estimate (not in the reference): a smooth
// multiplicative correction fitted by least squares on the even spot-check SSS samples, judged on
// the odd ones, and applied to the whole sinogram. The fit is one block: per-sample products in
// FP32, summed by warp trees and then across warps in FP64, and the k x k normal equations
// solved by Cholesky in FP64 (FP64 on the GPU only for these normalisation sums and the solve);
// the apply is one grid-stride pass. The estimate then reads k + 2 numbers back, with no host
// arithmetic between its kernels.
#include "common.cuh"

namespace srf {

constexpr int kMaxBasis = 12;
constexpr int kFitThreads = 512;
constexpr int kFitWarps = kFitThreads / 32;

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int K>
__global__ void __launch_bounds__(kFitThreads)
k_spot_fit(const float *__restrict__ pred, int64_t nbins, const int64_t *__restrict__ bins,
           const float *__restrict__ ref, int n, const float *__restrict__ phi, double ridge,
           float *__restrict__ out) {
    constexpr int NG = K * (K + 1) / 2;  // packed upper triangle of the normal matrix
    constexpr int NS = NG + K;           // and the right-hand side
    __shared__ float part[kFitWarps][NS];
    __shared__ float part3[kFitWarps][3];
    __shared__ double ata[K][K], atb[K], beta[K];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // normal equations over the even samples: a_j = pred * phi_j. A sample whose bin lies
    // outside [0, nbins) is left out (the odd pass below does the same).
    float g[NS];
#pragma unroll
    for (int e = 0; e < NS; ++e) g[e] = 0.0f;
    for (int s = 2 * threadIdx.x; s < n; s += 2 * kFitThreads) {
        const int64_t b = bins[s];
        if ((uint64_t)b >= (uint64_t)nbins) continue;
        const float p = pred[b], y = ref[s];
        float a[K];
#pragma unroll
        for (int j = 0; j < K; ++j) a[j] = p * phi[j * nbins + b];
        int e = 0;
#pragma unroll
        for (int j = 0; j < K; ++j) {
#pragma unroll
            for (int l = j; l < K; ++l) {
                g[e] = fmaf(a[j], a[l], g[e]);
                ++e;
            }
        }
#pragma unroll
        for (int j = 0; j < K; ++j) g[NG + j] = fmaf(a[j], y, g[NG + j]);
    }
#pragma unroll
    for (int e = 0; e < NS; ++e) {
        const float v = warp_sum_f(g[e]);
        if (lane == 0) part[w][e] = v;
    }
    __syncthreads();
    if (threadIdx.x < NS) {  // entry e = threadIdx.x: (j, l) of the packed triangle, or rhs j
        double v = 0.0;
        for (int i = 0; i < kFitWarps; ++i) v += (double)part[i][threadIdx.x];
        int e = threadIdx.x;
        if (e >= NG) {
            atb[e - NG] = v;
        } else {
            int j = 0;
            while (e >= K - j) {
                e -= K - j;
                ++j;
            }
            ata[j][j + e] = ata[j + e][j] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tr = 0.0;
        for (int j = 0; j < K; ++j) tr += ata[j][j];
        int okay = tr > 0.0 && isfinite(tr);
        if (okay) {
            const double add = ridge * tr / K;
            for (int j = 0; j < K; ++j) ata[j][j] += add;
            // Cholesky ata = L L^T in place (lower triangle), then two triangular solves
            for (int j = 0; j < K && okay; ++j) {
                double d = ata[j][j];
                for (int m = 0; m < j; ++m) d -= ata[j][m] * ata[j][m];
                if (!(d > 0.0)) { okay = 0; break; }
                d = sqrt(d);
                ata[j][j] = d;
                for (int i = j + 1; i < K; ++i) {
                    double v = ata[i][j];
                    for (int m = 0; m < j; ++m) v -= ata[i][m] * ata[j][m];
                    ata[i][j] = v / d;
                }
            }
        }
        if (okay) {
            for (int i = 0; i < K; ++i) {  // L z = atb, z kept in atb
                double v = atb[i];
                for (int m = 0; m < i; ++m) v -= ata[i][m] * atb[m];
                atb[i] = v / ata[i][i];
            }
            for (int i = K - 1; i >= 0; --i) {  // L^T beta = z
                double v = atb[i];
                for (int m = i + 1; m < K; ++m) v -= ata[m][i] * beta[m];
                beta[i] = v / ata[i][i];
            }
        } else {
            for (int i = 0; i < K; ++i) beta[i] = (i == 0) ? 1.0 : 0.0;
        }
    }
    __syncthreads();
    // judged on the odd samples, which the fit has not seen
    float bf[K];
#pragma unroll
    for (int j = 0; j < K; ++j) bf[j] = (float)beta[j];
    float e2 = 0.0f, u2 = 0.0f, y2 = 0.0f;
    for (int s = 2 * threadIdx.x + 1; s < n; s += 2 * kFitThreads) {
        const int64_t b = bins[s];
        if ((uint64_t)b >= (uint64_t)nbins) continue;
        const float p = pred[b], y = ref[s];
        float c = 0.0f;
#pragma unroll
        for (int j = 0; j < K; ++j) c = fmaf(bf[j], phi[j * nbins + b], c);
        const float d = fmaf(p, c, -y), u = p - y;
        e2 = fmaf(d, d, e2);
        u2 = fmaf(u, u, u2);
        y2 = fmaf(y, y, y2);
    }
    e2 = warp_sum_f(e2);
    u2 = warp_sum_f(u2);
    y2 = warp_sum_f(y2);
    if (lane == 0) {
        part3[w][0] = e2;
        part3[w][1] = u2;
        part3[w][2] = y2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double se = 0.0, su = 0.0, sy = 0.0;
        for (int i = 0; i < kFitWarps; ++i) {
            se += (double)part3[i][0];
            su += (double)part3[i][1];
            sy += (double)part3[i][2];
        }
        const double den = sqrt(fmax(sy, 1e-60));
        for (int j = 0; j < K; ++j) out[j] = (float)beta[j];
        out[K] = (float)(sqrt(se) / den);
        out[K + 1] = (float)(sqrt(su) / den);
    }
}

template <int K>
static void launch_fit(const float *pred, int64_t nbins, const int64_t *bins, const float *ref, int n,
                       const float *phi, double ridge, float *out, cudaStream_t s) {
    k_spot_fit<K><<<1, kFitThreads, 0, s>>>(pred, nbins, bins, ref, n, phi, ridge, out);
}

__global__ void k_scale_by_basis(float *__restrict__ x, int64_t n, const float *__restrict__ phi, int k,
                                 const float *__restrict__ beta) {
    float b[kMaxBasis];
#pragma unroll
    for (int j = 0; j < kMaxBasis; ++j) b[j] = j < k ? beta[j] : 0.0f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float c = 0.0f;
#pragma unroll
        for (int j = 0; j < kMaxBasis; ++j)
            if (j < k) c = fmaf(b[j], __ldg(phi + j * n + i), c);
        x[i] *= c;
    }
}

}  // namespace srf

using namespace srf;

extern "C" {

int srf_spot_fit(const float *pred, int64_t nbins, const int64_t *bins, const float *ref, int32_t n,
                 const float *phi, int32_t k, double ridge, float *out, void *stream) {
    if (!pred || !bins || !ref || !phi || !out) return fail(SRF_EINVAL, "NULL pointer");
    if (nbins <= 0 || n < 2 || k < 1 || k > kMaxBasis) return fail(SRF_EINVAL, "bad sizes (nbins %lld, n %d, k %d)", (long long)nbins, n, k);
    if (!(ridge >= 0.0) || !std::isfinite(ridge)) return fail(SRF_EINVAL, "ridge must be finite and >= 0");
    const cudaStream_t s = (cudaStream_t)stream;
    switch (k) {
        case 1: launch_fit<1>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 2: launch_fit<2>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 3: launch_fit<3>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 4: launch_fit<4>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 5: launch_fit<5>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 6: launch_fit<6>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 7: launch_fit<7>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 8: launch_fit<8>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 9: launch_fit<9>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 10: launch_fit<10>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        case 11: launch_fit<11>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
        default: launch_fit<12>(pred, nbins, bins, ref, n, phi, ridge, out, s); break;
    }
    return check_cuda("spot fit launch");
}

int srf_scale_by_basis(float *x, int64_t n, const float *phi, int32_t k, const float *beta, void *stream) {
    if (!x || !phi || !beta) return fail(SRF_EINVAL, "NULL pointer");
    if (n < 0 || k < 1 || k > kMaxBasis) return fail(SRF_EINVAL, "bad sizes (n %lld, k %d)", (long long)n, k);
    if (n == 0) return ok();
    k_scale_by_basis<<<grid_for(k_scale_by_basis, n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(x, n, phi, k, beta);
    return check_cuda("scale launch");
}

}  // extern "C"
