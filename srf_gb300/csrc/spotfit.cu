// Spot-check correction of the learned scatter estimate (not in the reference): a smooth
// multiplicative correction fitted by least squares on the even spot-check SSS samples, judged on
// the odd ones, and applied to the whole sinogram. The fit is one block (a k x k normal-equation
// system in FP64, solved by Cholesky); the apply is one grid-stride pass. The estimate then reads
// k + 2 numbers back, with no host arithmetic between its kernels.
#include "common.cuh"

namespace srf {

constexpr int kMaxBasis = 12;
constexpr int kFitThreads = 256;
constexpr int kFitWarps = kFitThreads / 32;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sums v over the block into every thread's return value; `scratch` holds kFitWarps doubles and
// is free again when the function returns.
__device__ __forceinline__ double block_sum_d(double v, double *scratch) {
    v = warp_sum_d(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) scratch[w] = v;
    __syncthreads();
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < kFitWarps; ++i) t += scratch[i];
    __syncthreads();
    return t;
}

template <int K>
__global__ void __launch_bounds__(kFitThreads)
k_spot_fit(const float *__restrict__ pred, int64_t nbins, const int64_t *__restrict__ bins,
           const float *__restrict__ ref, int n, const float *__restrict__ phi, double ridge,
           float *__restrict__ out) {
    constexpr int NG = K * (K + 1) / 2;  // packed upper triangle of the normal matrix
    constexpr int NS = NG + K;           // and the right-hand side
    __shared__ double scratch[kFitWarps];
    __shared__ double part[kFitWarps][NS];
    __shared__ double ata[K][K], atb[K], beta[K];
    // normal equations over the even samples: a_j = pred * phi_j. A sample whose bin lies
    // outside [0, nbins) is left out (the odd pass below does the same).
    double g[NS];
#pragma unroll
    for (int e = 0; e < NS; ++e) g[e] = 0.0;
    for (int s = 2 * threadIdx.x; s < n; s += 2 * kFitThreads) {
        const int64_t b = bins[s];
        if ((uint64_t)b >= (uint64_t)nbins) continue;
        const double p = (double)pred[b], y = (double)ref[s];
        double a[K];
#pragma unroll
        for (int j = 0; j < K; ++j) a[j] = p * (double)phi[j * nbins + b];
        int e = 0;
#pragma unroll
        for (int j = 0; j < K; ++j) {
#pragma unroll
            for (int l = j; l < K; ++l) {
                g[e] = fma(a[j], a[l], g[e]);
                ++e;
            }
        }
#pragma unroll
        for (int j = 0; j < K; ++j) g[NG + j] = fma(a[j], y, g[NG + j]);
    }
    {
        const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
        for (int e = 0; e < NS; ++e) {
            const double v = warp_sum_d(g[e]);
            if (l == 0) part[w][e] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int e = 0;
        for (int j = 0; j < K; ++j)
            for (int l = j; l < K; ++l, ++e) {
                double v = 0.0;
                for (int w = 0; w < kFitWarps; ++w) v += part[w][e];
                ata[j][l] = ata[l][j] = v;
            }
        for (int j = 0; j < K; ++j) {
            double v = 0.0;
            for (int w = 0; w < kFitWarps; ++w) v += part[w][NG + j];
            atb[j] = v;
        }
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
            double z[K];
            for (int i = 0; i < K; ++i) {
                double v = atb[i];
                for (int m = 0; m < i; ++m) v -= ata[i][m] * z[m];
                z[i] = v / ata[i][i];
            }
            for (int i = K - 1; i >= 0; --i) {
                double v = z[i];
                for (int m = i + 1; m < K; ++m) v -= ata[m][i] * beta[m];
                beta[i] = v / ata[i][i];
            }
        } else {
            for (int i = 0; i < K; ++i) beta[i] = (i == 0) ? 1.0 : 0.0;
        }
    }
    __syncthreads();
    // judged on the odd samples, which the fit has not seen
    double e2 = 0.0, u2 = 0.0, y2 = 0.0;
    for (int s = 2 * threadIdx.x + 1; s < n; s += 2 * kFitThreads) {
        const int64_t b = bins[s];
        if ((uint64_t)b >= (uint64_t)nbins) continue;
        const double p = (double)pred[b], y = (double)ref[s];
        double c = 0.0;
#pragma unroll
        for (int j = 0; j < K; ++j) c = fma(beta[j], (double)phi[j * nbins + b], c);
        const double d = p * c - y, u = p - y;
        e2 = fma(d, d, e2);
        u2 = fma(u, u, u2);
        y2 = fma(y, y, y2);
    }
    e2 = block_sum_d(e2, scratch);
    u2 = block_sum_d(u2, scratch);
    y2 = block_sum_d(y2, scratch);
    if (threadIdx.x == 0) {
        const double den = sqrt(fmax(y2, 1e-60));
        for (int j = 0; j < K; ++j) out[j] = (float)beta[j];
        out[K] = (float)(sqrt(e2) / den);
        out[K + 1] = (float)(sqrt(u2) / den);
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
