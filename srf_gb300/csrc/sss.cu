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
// with a double-precision evaluation while the slow path stays rare; those re-evaluations are
// queued per warp and run 32 at a time.
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
// to float, once per call, and passed by value (7.7 KB of kernel parameters). Whole degrees of
// acos(x) are max{t : x <= cos(t deg)}; `start` gives, for each of kBuckets equal slices of
// [-1, 1] in x, that t at the slice's upper end, from which a search over the cos table begins.
constexpr int kBuckets = 4096;
struct SssTables {
    float2 ge[kAngles];        // (511 / E', eff(E') * fkn), the factors of a term at t degrees
    float cosf_[kAngles + 2];  // cos(t deg) rounded to float; [kAngles..] = -2, below every cosine
    double cosd[kAngles];      // cos(t deg) in double
    unsigned char start[kBuckets];
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
        T.ge[t] = make_float2((float)(511.0 / e_sc), (float)(eff * (diff / sigma)));
        T.cosd[t] = c;
    }
    T.cosd[kAngles - 1] = -1.0;
    for (int t = 0; t < kAngles; ++t) T.cosf_[t] = (float)T.cosd[t];
    T.cosf_[kAngles] = T.cosf_[kAngles + 1] = -2.0f;
    for (int b = 0; b < kBuckets; ++b) {
        // a little above the slice (the float bucket index may round down)
        const double hi = std::min(1.0, -1.0 + 2.0 * (b + 1) / kBuckets + 1e-6);
        int t = (int)std::floor(std::acos(hi) * 180.0 / M_PI);
        T.start[b] = (unsigned char)std::min(std::max(t, 0), kAngles - 1);
    }
    return T;
}

// One crystal pair's geometry as every lane of its warp (or a lane of a deferred-angle flush) sees it.
struct PairGeo {
    float ax, ay, az, bx, by, bz;
    float nax, nay, nbx, nby;  // block normals of A and B
    float ab2;                 // |AB|^2 in FP32
    int ra, rb;                // offsets of A's and B's rows of the per-point tables (< 2^31)
};

__device__ __forceinline__ PairGeo pair_geo(int a, int b, const float *__restrict__ cpos, int n_s, int ncpr, int nbpr, int gb1) {
    PairGeo P;
    P.ax = __ldg(cpos + 3 * a); P.ay = __ldg(cpos + 3 * a + 1); P.az = __ldg(cpos + 3 * a + 2);
    P.bx = __ldg(cpos + 3 * b); P.by = __ldg(cpos + 3 * b + 1); P.bz = __ldg(cpos + 3 * b + 2);
    // block normals at id / nbpr * 2 pi
    sincospif(2.0f * (float)block_id(ncpr, nbpr, gb1, P.ax, P.ay, P.az) / (float)nbpr, &P.nay, &P.nax);
    sincospif(2.0f * (float)block_id(ncpr, nbpr, gb1, P.bx, P.by, P.bz) / (float)nbpr, &P.nby, &P.nbx);
    const float dabx = P.bx - P.ax, daby = P.by - P.ay, dabz = P.bz - P.az;
    P.ab2 = dabx * dabx + daby * daby + dabz * dabz;
    P.ra = a * n_s; P.rb = b * n_s;
    return P;
}

// Scatter point s of pair P: the law-of-cosines operands in FP32.
struct PointGeo {
    float dax, day, dbx, dby;  // in-plane components of A - S and B - S (the area terms)
    float as2, sb2, ias, isb;  // |SA|^2, |SB|^2 and their reciprocal square roots
    float sx, sy, sz;
};

__device__ __forceinline__ PointGeo point_geo(const PairGeo &P, const float *__restrict__ spos, int s) {
    PointGeo Q;
    Q.sx = __ldg(spos + 3 * s); Q.sy = __ldg(spos + 3 * s + 1); Q.sz = __ldg(spos + 3 * s + 2);
    Q.dax = P.ax - Q.sx; Q.day = P.ay - Q.sy;
    const float daz = P.az - Q.sz;
    Q.dbx = P.bx - Q.sx; Q.dby = P.by - Q.sy;
    const float dbz = P.bz - Q.sz;
    Q.as2 = Q.dax * Q.dax + Q.day * Q.day + daz * daz;
    Q.sb2 = Q.dbx * Q.dbx + Q.dby * Q.dby + dbz * dbz;
    Q.ias = rsqrtf(Q.as2); Q.isb = rsqrtf(Q.sb2);
    return Q;
}

// Whole degrees of the scattering angle from the FP32 cosine, or -1 when the FP32 value cannot
// decide them. With u = 2^-24: |SA|^2, |SB|^2 and |AB|^2 carry at most 5u relative error each
// (the float differences and three roundings), the numerator N = |SA|^2 + |SB|^2 - |AB|^2 at most
// 7u S (S = |SA|^2 + |SB|^2 + |AB|^2); rsqrtf is within 2 ulp, so 1 / den = rsqrt(|SA|^2) *
// rsqrt(|SB|^2) / 2 is within 14u, and arg = -N / den is within 15u |arg| + 7u S / den <=
// 22u S / den (S / den >= 1) of the cosine the double path computes. The angle is decided when
// arg lies more than four times that bound (plus the 3e-8 rounding of the float cosine table)
// from both cosines bracketing it; otherwise, and at |arg| = 1, the point goes to the double path.
__device__ __forceinline__ int fast_angle(const PairGeo &P, const PointGeo &Q, const float *t_cf,
                                          const unsigned char *t_start) {
    const float S = Q.as2 + Q.sb2 + P.ab2;
    const float iden = 0.5f * Q.ias * Q.isb;
    float arg = -(Q.as2 + Q.sb2 - P.ab2) * iden;
    arg = fminf(1.0f, fmaxf(-1.0f, arg));
    const float Em = 4.0f * 1.32e-6f * S * iden + 4.0e-8f;
    const int b = min(max((int)((arg + 1.0f) * (0.5f * kBuckets)), 0), kBuckets - 1);
    // t from the slice's start: at most two whole degrees lie in one slice (three steps cover
    // its widened upper end); a start above arg's angle, or more steps, goes to the double path
    int t = t_start[b];
    float hi = t_cf[t], lo = t_cf[t + 1];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const bool up = arg <= lo;
        t += up ? 1 : 0;
        hi = up ? lo : hi;
        lo = t_cf[t + 1];
    }
    if (arg > hi || arg <= lo) return -1;
    if (hi - arg <= Em || arg - lo <= Em) return -1;
    return t;
}

// The cosine in double (as the reference) from the same float coordinates, then its whole
// degrees by comparison with cos(t deg): acos(x) >= t deg <=> x <= cos(t deg), starting from the
// FP32 estimate (no FP64 acos: FP64 issues at a small fraction of the FP32 rate here).
__device__ __forceinline__ int slow_angle(const PairGeo &P, const PointGeo &Q, const double *t_cos) {
    // |AB| in double from the float difference, squared again as kn_formula.py:36-41 does
    const float dabx = P.bx - P.ax, daby = P.by - P.ay, dabz = P.bz - P.az;
    const double Dab = sqrt((double)dabx * dabx + (double)daby * daby + (double)dabz * dabz);
    const double Dax = (double)P.ax - Q.sx, Day = (double)P.ay - Q.sy, Daz = (double)P.az - Q.sz;
    const double Dbx = (double)P.bx - Q.sx, Dby = (double)P.by - Q.sy, Dbz = (double)P.bz - Q.sz;
    const double Das = sqrt(Dax * Dax + Day * Day + Daz * Daz);
    const double Dsb = sqrt(Dbx * Dbx + Dby * Dby + Dbz * Dbz);
    double dargs = -(Das * Das + Dsb * Dsb - Dab * Dab) / (2 * Das * Dsb);
    dargs = fmin(1.0, fmax(-1.0, dargs));
    int t = min(max((int)(acosf((float)dargs) * (float)(180.0 / M_PI)), 0), kAngles - 1);
    while (t < kAngles - 1 && dargs <= t_cos[t + 1]) ++t;
    while (t > 0 && dargs > t_cos[t]) --t;
    return t;
}

// The term of scatter point s at whole-degree angle ti (FP32).
__device__ __forceinline__ float ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float point_term(const PairGeo &P, const PointGeo &Q, int s, int ti,
                                            const float *__restrict__ em, const float *__restrict__ at,
                                            const float *s_mu, const float2 *t_ge) {
    const float2 ge = t_ge[ti];
    const float a_a = __ldg(at + P.ra + s), a_b = __ldg(at + P.rb + s);
    // atten^(511/E') as 2^(log2(atten) * 511/E'), both approximate (relative error ~1e-6)
    const float Ia = a_a * ex2(__log2f(a_b) * ge.x) * __ldg(em + P.ra + s);
    const float Ib = ex2(__log2f(a_a) * ge.x) * a_b * __ldg(em + P.rb + s);
    // area(S->A) uses A's block normal, area(S->B) B's; the divisions by |SA|, |SB| and their
    // squares as multiplications by the reciprocal square roots of |SA|^2, |SB|^2
    const float ias = Q.ias, isb = Q.isb;
    const float pa = (Q.dax * P.nax + Q.day * P.nay) * ias;
    const float pb = (Q.dbx * P.nbx + Q.dby * P.nby) * isb;
    return pa * ge.y * pb * s_mu[s] * (Ia + Ib) * (ias * ias) * (isb * isb);
}

// Deferred double-precision angles: a warp queues the (pair, point) items whose FP32 angle is
// undecided (about 2e-3 of them) and evaluates them 32 at a time, one per lane, instead of
// running the FP64 path for one or two lanes of a warp at a time. Entries pack pair << 14 | point.
constexpr int kQueue = 64;
constexpr int kPointBits = 14;
static_assert(kMaxScatterPoints <= (1 << kPointBits), "point index field too narrow");

// Evaluates the first `cnt` (<= 32) queued items of this warp, sums them per pair in queue order
// (a run of one pair is summed by the run's first lane) and drops them from the queue. Sums of
// pairs already written are added to their scatter values; the sum of pair `kcur`, the pair the
// warp is still accumulating, is returned (to every lane). Every pair in the queue belongs to
// this warp.
__device__ __forceinline__ float flush_deferred(unsigned long long *q, float *qv, int &qn, int cnt, int64_t kcur, int lane,
                                               const int32_t *__restrict__ pairs, const float *__restrict__ cpos,
                                               const float *__restrict__ spos, int n_s,
                                               const float *__restrict__ em, const float *__restrict__ at,
                                               int ncpr, int nbpr, int gb1, const float *s_mu,
                                               const float2 *t_ge,
                                               const double *t_cos, float *__restrict__ scatter) {
    __syncwarp();
    const unsigned long long e = lane < cnt ? q[lane] : 0ull;
    const int64_t kk = (int64_t)(e >> kPointBits);
    float c = 0.0f;
    if (lane < cnt) {
        const int s = (int)(e & ((1u << kPointBits) - 1));
        const PairGeo P = pair_geo(__ldg(pairs + 2 * kk), __ldg(pairs + 2 * kk + 1), cpos, n_s, ncpr, nbpr, gb1);
        const PointGeo Q = point_geo(P, spos, s);
        c = point_term(P, Q, s, slow_angle(P, Q, t_cos), em, at, s_mu, t_ge);
    }
    qv[lane] = c;
    __syncwarp();
    float cur = 0.0f;
    if (lane < cnt && (lane == 0 || (int64_t)(q[lane - 1] >> kPointBits) != kk)) {
        float sum = 0.0f;
        for (int j = lane; j < cnt && (int64_t)(q[j] >> kPointBits) == kk; ++j) sum += qv[j];
        if (kk == kcur) cur = sum;
        else scatter[kk] += sum;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cur += __shfl_xor_sync(0xffffffffu, cur, o);  // one lane holds it
    __syncwarp();
    const int rest = qn - cnt;  // < 32 entries stay
    const unsigned long long keep = lane < rest ? q[cnt + lane] : 0ull;
    __syncwarp();
    if (lane < rest) q[lane] = keep;
    __syncwarp();
    qn = rest;
    return cur;
}

// 128-thread blocks, 7 per SM: 72 registers without spills (256-thread blocks at 4 per SM forced
// 64 with spills in the point loop, at 3 per SM 24 warps; both measured slower; 8 per SM spills,
// 6 per SM (78 registers) measured 1.28 against 1.145 ms on 2e5 pairs x 576 points)
constexpr int kSssBlock = 128;

__global__ void __launch_bounds__(kSssBlock, 7)
k_sss(const int32_t *__restrict__ pairs, int64_t n_pairs, int n_crystals, const float *__restrict__ cpos,
      const float *__restrict__ spos, int n_s, const float *__restrict__ em,
      const float *__restrict__ at, const float *__restrict__ umap, int u0, int u1, int u2,
      float us0, float us1, float us2, int ncpr, int nbpr, int gb1, const __grid_constant__ SssTables tab,
      float *__restrict__ scatter, float *__restrict__ scale) {
    __shared__ float2 t_ge[kAngles];
    __shared__ float t_cf[kAngles + 2];
    __shared__ double t_cos[kAngles];
    __shared__ unsigned char t_start[kBuckets];
    __shared__ unsigned long long s_q[kSssBlock / 32][kQueue];
    __shared__ float s_qv[kSssBlock / 32][32];
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
        t_ge[t] = tab.ge[t];
        t_cos[t] = tab.cosd[t];
    }
    for (int t = threadIdx.x; t < kAngles + 2; t += blockDim.x) t_cf[t] = tab.cosf_[t];
    for (int t = threadIdx.x; t < kBuckets; t += blockDim.x) t_start[t] = tab.start[t];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    unsigned long long *q = s_q[threadIdx.x >> 5];
    float *qv = s_qv[threadIdx.x >> 5];
    int qn = 0;  // queued items of this warp (warp-uniform)
    const unsigned lt = (1u << lane) - 1u;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = warp; k < n_pairs; k += nwarps) {
        const int a = __ldg(pairs + 2 * k), b = __ldg(pairs + 2 * k + 1);
        if (a < 0 || a >= n_crystals || b < 0 || b >= n_crystals) {  // invalid id: no contribution
            if (lane == 0) { scatter[k] = 0.0f; scale[k] = 0.0f; }
            continue;
        }
        PairGeo P = pair_geo(a, b, cpos, n_s, ncpr, nbpr, gb1);
        float acc = 0.0f;
        for (int s0 = 0; s0 < n_s; s0 += 32) {
            const int s = s0 + lane;
            const bool act = s < n_s;
            PointGeo Q;
            int ti = 0;
            if (act) {
                Q = point_geo(P, spos, s);
                ti = fast_angle(P, Q, t_cf, t_start);
            }
            // undecided points are queued (qn < 32 here, so at most 63 entries)
            const unsigned slow = __ballot_sync(0xffffffffu, act && ti < 0);
            if (act && ti < 0) q[qn + __popc(slow & lt)] = ((unsigned long long)k << kPointBits) | (unsigned)s;
            qn += __popc(slow);
            if (act && ti >= 0) acc += point_term(P, Q, s, ti, em, at, s_mu, t_ge);
            if (qn >= 32) {
                const float cur = flush_deferred(q, qv, qn, 32, k, lane, pairs, cpos, spos, n_s, em, at, ncpr,
                                                 nbpr, gb1, s_mu, t_ge, t_cos, scatter);
                if (lane == 0) acc += cur;
                // rebuilt rather than kept live across the flush (registers); flushes are rare
                P = pair_geo(a, b, cpos, n_s, ncpr, nbpr, gb1);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            scatter[k] = acc;
            const float dabx = P.bx - P.ax, daby = P.by - P.ay;
            const float ab = sqrtf(P.ab2);
            const float area = (dabx * P.nbx + daby * P.nby) / ab;
            const float qq = ab / area;
            scale[k] = qq * qq;
        }
    }
    if (qn > 0)
        flush_deferred(q, qv, qn, qn, -1, lane, pairs, cpos, spos, n_s, em, at, ncpr, nbpr, gb1, s_mu, t_ge,
                       t_cos, scatter);
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
    if ((int64_t)n_crystals * n_scatter >= (int64_t(1) << 31))
        return fail(SRF_ERANGE, "n_crystals * n_scatter must be below 2^31");
    const double res = sqrt(511.0) * (double)resolution;
    const int smem = n_scatter * (int)sizeof(float);
    unsigned blocks = grid_for(k_sss, n_pairs, kSssBlock / 32, smem, kSssBlock);
    k_sss<<<blocks, kSssBlock, smem, (cudaStream_t)stream>>>(
        pairs, n_pairs, n_crystals, crystal_pos, scatter_pos, n_scatter, sumup_emission, atten, umap,
        umap_shape[0], umap_shape[1], umap_shape[2], umap_size[0], umap_size[1], umap_size[2],
        nb_crystals_per_ring, nb_blocks_per_ring, grid_block[1], sss_tables(low_energy, high_energy, res),
        scatter, scale);
    return check_cuda("sss kernel launch");
}
