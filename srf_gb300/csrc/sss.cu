// Single-scatter simulation core on the GPU.
//
// Follows srfnef/corrections/scattering/scatter_fraction/scatter_fraction.py:40-136 and
// kn_formula.py:6-46 (numba.cuda kernels loop_all_lors/loop_all_s in the reference):
//   for LOR pair (A, B) and scatter point S:
//     theta  = whole degrees of acos(-(|AS|^2 + |SB|^2 - |AB|^2) / (2 |AS| |SB|)), in radians
//     E'     = 511 / (2 - cos theta)
//     Ia     = atten_SA * atten_SB^(511/E') * em_SA ;  Ib = atten_SA^(511/E') * atten_SB * em_SB
//     term   = area(S->A) * eff(E') * area(S->B) * fkn(theta) * mu(S) * (Ia + Ib) / |SA|^2 / |SB|^2
//   scatter = sum_S term ;  scale = (|AB| / area(A->B))^2
// with area(P->Q) = ((Q - P) . n_Q) / |PQ|, n_Q the normal of Q's block (get_block_theta),
// eff(E) = sum_{e = low, low+5, .. < high} exp(-(e - E)^2 / (2 res^2)), res = sqrt(511)*resolution,
// and fkn's Klein-Nishina factor evaluated at the angle (the reference passes theta where the
// formula expects cos theta; kn_formula.py:11).
//
// GB300 design: because theta is quantised to whole degrees, cos theta, 511/E', eff(E') and the
// Klein-Nishina factor take at most 181 values; the host builds those tables once per call (double
// precision, then rounded) and each block copies them into shared memory, so the inner loop is
// table lookups plus two power functions; mu at each scatter point's nearest voxel is looked up once per block into shared
// memory. One warp per LOR pair, lanes over scatter points, so the crystal-major emission and
// attenuation rows are read coalesced. The angle is evaluated in FP32 with a bound on its
// rounding error (from the law-of-cosines operands and acosf's accuracy) and re-evaluated in
// FP64 only when a whole degree lies within four times that bound, so its quantisation agrees
// with a double-precision evaluation while the slow path stays rare.
#include "common.cuh"

namespace srf {

constexpr int kAngles = 181;
constexpr int kMaxScatterPoints = 12288;  // their mu values fill at most 48 KB of shared memory

// Block index of a crystal position (scatter_fraction.py:123-131, get_block_theta; its angle is
// acos(x / |p|) with the 3-D norm, a quirk kept as is), in double.
__device__ __forceinline__ int block_id_d(int ncpr, int nbpr, int gb1, double px, double py, double pz) {
    const double norm = sqrt(px * px + py * py + pz * pz);
    double th = acos(px / norm) / M_PI * 180.0;
    if (py < 0) th = 360.0 - th;
    double fixed = fmod(th + 180.0 / ncpr * gb1, 360.0);
    if (fixed < 0) fixed += 360.0;
    return (int)floor(fixed / 360.0 * nbpr);
}

// The same in FP32, re-evaluated in FP64 only when the block coordinate lies within 2e-3 of a
// block boundary or |x / |p|| is within 1e-5 of 1 (where acos is ill-conditioned): crystals sit
// inside their blocks, so the FP64 path stays cold. Every lane of a warp evaluates the same pair,
// and FP64 issues at a small fraction of the FP32 rate on this part: in FP64 throughout this
// step alone kept the FP64 pipe 84 % busy.
__device__ __forceinline__ int block_id(int ncpr, int nbpr, int gb1, float px, float py, float pz) {
    const float norm = sqrtf(px * px + py * py + pz * pz);
    const float c = px / norm;
    float th = acosf(c) * (float)(180.0 / M_PI);
    if (py < 0) th = 360.0f - th;
    float fixed = fmodf(th + 180.0f / ncpr * gb1, 360.0f);
    if (fixed < 0) fixed += 360.0f;
    const float q = fixed / 360.0f * nbpr;
    const float fr = q - floorf(q);
    if (fr < 2e-3f || fr > 1.0f - 2e-3f || fabsf(c) > 0.99999f) return block_id_d(ncpr, nbpr, gb1, px, py, pz);
    return (int)floorf(q);
}

// Per whole-degree angle: 511 / E' (the attenuation exponent), eff(E') and the Klein-Nishina factor
// as the reference evaluates it (fkn receives the angle). Built on the host in double and rounded
// to float, once per call, and passed by value (2.2 KB of kernel parameters).
struct SssTables {
    float g[kAngles], eff[kAngles], fk[kAngles];
    double cosd[kAngles];  // cos(t degrees): whole degrees of acos(x) = max{t : x <= cos(t deg)}
};

static SssTables sss_tables(int low, int high, double res) {
    SssTables T;
    for (int t = 0; t < kAngles; ++t) {
        const double ang = (double)t / 180.0 * M_PI;
        const double c = std::cos(ang);
        const double e_sc = 511.0 / (2.0 - c);
        double eff = 0.0;
        for (int e = low; e < high; e += 5) eff += std::exp(-((double)e - e_sc) * ((double)e - e_sc) / 2.0 / (res * res));
        const double a = ang;  // the reference's fkn receives the angle
        const double diff = 1.0 / ((2.0 - a) * (2.0 - a)) * ((1.0 + a * a) / 2.0 + (1.0 - a) * (1.0 - a) / 2.0 / (2.0 - a));
        const double sigma = M_PI * (40.0 / 9.0 - 3.0 * std::log(3.0));
        T.g[t] = (float)(511.0 / e_sc);
        T.eff[t] = (float)eff;
        T.fk[t] = (float)(diff / sigma);
        T.cosd[t] = c;
    }
    T.cosd[kAngles - 1] = -1.0;
    return T;
}

__global__ void __launch_bounds__(kBlock)
k_sss(const int32_t *__restrict__ pairs, int64_t n_pairs, int n_crystals, const float *__restrict__ cpos,
      const float *__restrict__ spos, int n_s, const float *__restrict__ em,
      const float *__restrict__ at, const float *__restrict__ umap, int u0, int u1, int u2,
      float us0, float us1, float us2, int ncpr, int nbpr, int gb1, const __grid_constant__ SssTables tab,
      float *__restrict__ scatter, float *__restrict__ scale) {
    __shared__ float t_g[kAngles], t_eff[kAngles], t_fk[kAngles];
    __shared__ double t_cos[kAngles];
    extern __shared__ float s_mu[];  // n_s entries: mu at the nearest voxel of each scatter point
    for (int t = threadIdx.x; t < n_s; t += blockDim.x) {
        // kn_formula.py:12-14; outside the map counts as 0
        const float sx = __ldg(spos + 3 * t), sy = __ldg(spos + 3 * t + 1), sz = __ldg(spos + 3 * t + 2);
        const int g0 = (int)((sx / us0 + 0.5f) * u0);
        const int g1 = (int)((sy / us1 + 0.5f) * u1);
        const int g2 = (int)((sz / us2 + 0.5f) * u2);
        float mu = 0.0f;
        if (g0 >= 0 && g0 < u0 && g1 >= 0 && g1 < u1 && g2 >= 0 && g2 < u2)
            mu = __ldg(umap + ((int64_t)g0 * u1 + g1) * u2 + g2);
        s_mu[t] = mu;
    }
    for (int t = threadIdx.x; t < kAngles; t += blockDim.x) {
        t_g[t] = tab.g[t];
        t_eff[t] = tab.eff[t];
        t_fk[t] = tab.fk[t];
        t_cos[t] = tab.cosd[t];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = warp; k < n_pairs; k += nwarps) {
        const int a = __ldg(pairs + 2 * k), b = __ldg(pairs + 2 * k + 1);
        if (a < 0 || a >= n_crystals || b < 0 || b >= n_crystals) {  // invalid id: no contribution
            if (lane == 0) { scatter[k] = 0.0f; scale[k] = 0.0f; }
            continue;
        }
        const float ax = __ldg(cpos + 3 * a), ay = __ldg(cpos + 3 * a + 1), az = __ldg(cpos + 3 * a + 2);
        const float bx = __ldg(cpos + 3 * b), by = __ldg(cpos + 3 * b + 1), bz = __ldg(cpos + 3 * b + 2);
        // block normals at id / nbpr * 2 pi
        float nax, nay, nbx, nby;
        sincospif(2.0f * (float)block_id(ncpr, nbpr, gb1, ax, ay, az) / (float)nbpr, &nay, &nax);
        sincospif(2.0f * (float)block_id(ncpr, nbpr, gb1, bx, by, bz) / (float)nbpr, &nby, &nbx);
        const float dabx = bx - ax, daby = by - ay, dabz = bz - az;
        const float ab2 = dabx * dabx + daby * daby + dabz * dabz;
        // |AB| in double, squared again as the reference does (kn_formula.py:36-41)
        const double Dab = sqrt((double)dabx * dabx + (double)daby * daby + (double)dabz * dabz);
        const float ab = sqrtf(ab2);
        const float *ema = em + (int64_t)a * n_s, *emb = em + (int64_t)b * n_s;
        const float *ata = at + (int64_t)a * n_s, *atb = at + (int64_t)b * n_s;
        float acc = 0.0f;
        for (int s = lane; s < n_s; s += 32) {
            const float sx = __ldg(spos + 3 * s), sy = __ldg(spos + 3 * s + 1), sz = __ldg(spos + 3 * s + 2);
            const float dax = ax - sx, day = ay - sy, daz = az - sz;
            const float dbx = bx - sx, dby = by - sy, dbz = bz - sz;
            const float as2 = dax * dax + day * day + daz * daz;
            const float sb2 = dbx * dbx + dby * dby + dbz * dbz;
            const float as = sqrtf(as2), sb = sqrtf(sb2);
            const float den = 2.0f * as * sb;
            float arg = -(as2 + sb2 - ab2) / den;
            arg = fminf(1.0f, fmaxf(-1.0f, arg));
            // |error of arg| <= 7u (as2 + sb2 + ab2) / den + 9u (u = 2^-24); acosf is within 5e-7
            // rad and the degree conversion within 2.2e-5 degree
            const float E = 5.0e-7f * (as2 + sb2 + ab2) / den + 6.0e-7f;
            const float m = fabsf(arg) + E;
            bool slow = m >= 0.9999f;
            float deg = 0.0f;
            if (!slow) {
                deg = acosf(arg) * (float)(180.0 / M_PI);
                const float tol = 4.0f * (57.2957795f * (E * rsqrtf(1.0f - m * m) + 5.0e-7f) + 2.2e-5f);
                const float fr = deg - floorf(deg);
                slow = fr < tol || fr > 1.0f - tol;
            }
            int ti;
            if (slow) {
                // the cosine in double (as the reference) from the same float coordinates, then
                // its whole degrees by comparison with cos(t deg): acos(x) >= t deg <=> x <= cos(t deg),
                // starting from the FP32 estimate (no FP64 acos: FP64 issues at a small fraction
                // of the FP32 rate here)
                const double Dax = (double)ax - sx, Day = (double)ay - sy, Daz = (double)az - sz;
                const double Dbx = (double)bx - sx, Dby = (double)by - sy, Dbz = (double)bz - sz;
                const double Das = sqrt(Dax * Dax + Day * Day + Daz * Daz);
                const double Dsb = sqrt(Dbx * Dbx + Dby * Dby + Dbz * Dbz);
                double dargs = -(Das * Das + Dsb * Dsb - Dab * Dab) / (2 * Das * Dsb);
                dargs = fmin(1.0, fmax(-1.0, dargs));
                int t = min(max((int)(acosf((float)dargs) * (float)(180.0 / M_PI)), 0), kAngles - 1);
                while (t < kAngles - 1 && dargs <= t_cos[t + 1]) ++t;
                while (t > 0 && dargs > t_cos[t]) --t;
                ti = t;
            } else {
                ti = (int)deg;
            }
            ti = min(max(ti, 0), kAngles - 1);
            const float mu = s_mu[s];
            const float gexp = t_g[ti];
            const float a_a = __ldg(ata + s), a_b = __ldg(atb + s);
            const float Ia = a_a * exp2f(__log2f(a_b) * gexp) * __ldg(ema + s);
            const float Ib = exp2f(__log2f(a_a) * gexp) * a_b * __ldg(emb + s);
            // area(S->A) uses A's block normal, area(S->B) B's; the divisions by |SA|, |SB| and
            // their squares as multiplications by correctly rounded reciprocals
            const float ias = __frcp_rn(as), isb = __frcp_rn(sb);
            const float pa = (dax * nax + day * nay) * ias;
            const float pb = (dbx * nbx + dby * nby) * isb;
            acc += pa * t_eff[ti] * pb * (t_fk[ti] * mu) * (Ia + Ib) * (ias * ias) * (isb * isb);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            scatter[k] = acc;
            const float area = (dabx * nbx + daby * nby) / ab;
            const float q = ab / area;
            scale[k] = q * q;
        }
    }
}

}  // namespace srf

using namespace srf;

extern "C" int srf_sss(const int32_t *pairs, int64_t n_pairs, const float *crystal_pos,
                       int32_t n_crystals, const float *scatter_pos, int32_t n_scatter,
                       const float *sumup_emission, const float *atten, const float *umap,
                       const int32_t umap_shape[3], const float umap_size[3],
                       int32_t nb_crystals_per_ring, int32_t nb_blocks_per_ring,
                       const int32_t grid_block[3], int32_t low_energy, int32_t high_energy,
                       float resolution, float *scatter, float *scale, void *stream) {
    if (n_pairs < 0 || n_crystals <= 0 || n_scatter < 0) return fail(SRF_EINVAL, "bad counts");
    if (n_pairs == 0) return ok();
    if (!pairs || !crystal_pos || !scatter || !scale || !umap_shape || !umap_size || !grid_block)
        return fail(SRF_EINVAL, "NULL argument");
    if (n_scatter > 0 && (!scatter_pos || !sumup_emission || !atten || !umap))
        return fail(SRF_EINVAL, "NULL scatter-point argument");
    if (nb_crystals_per_ring <= 0 || nb_blocks_per_ring <= 0)
        return fail(SRF_EINVAL, "ring counts must be positive");
    for (int k = 0; k < 3; ++k) {
        if (umap_shape[k] <= 0) return fail(SRF_EGRID, "umap_shape[%d] must be positive", k);
        if (!std::isfinite(umap_size[k]) || !(umap_size[k] > 0)) return fail(SRF_EGRID, "umap_size[%d] must be > 0", k);
    }
    if (!std::isfinite(resolution) || !(resolution > 0)) return fail(SRF_ENONFINITE, "resolution must be > 0");
    if (high_energy - low_energy > 5 * 100000) return fail(SRF_ERANGE, "energy window too wide");
    if (n_scatter > kMaxScatterPoints) return fail(SRF_ERANGE, "at most %d scatter points", kMaxScatterPoints);
    const double res = sqrt(511.0) * (double)resolution;
    const int smem = n_scatter * (int)sizeof(float);
    unsigned blocks = grid_for(k_sss, n_pairs, kBlock / 32, smem);
    k_sss<<<blocks, kBlock, smem, (cudaStream_t)stream>>>(
        pairs, n_pairs, n_crystals, crystal_pos, scatter_pos, n_scatter, sumup_emission, atten, umap,
        umap_shape[0], umap_shape[1], umap_shape[2], umap_size[0], umap_size[1], umap_size[2],
        nb_crystals_per_ring, nb_blocks_per_ring, grid_block[1], sss_tables(low_energy, high_energy, res),
        scatter, scale);
    return check_cuda("sss kernel launch");
}
