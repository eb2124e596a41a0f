// Fused list-mode MLEM/OSEM subset step and the multiplicative image update.
//
// The reference runs each iteration as four separate device passes plus host round trips
// (srfnef/functions/mlem_full_tof.py:62-67: ProjectTof op, div_no_nan, BackProjectTof op, x*bp/emap,
// each op doing three blocking parameter copies and a transpose of LORs and image). Here one
// kernel does projection -> ratio -> backprojection per LOR while the LOR is in registers; the
// projections and ratios never touch memory. The update kernel then folds the y-fastest
// accumulator, applies x*bp/emap, refreshes the y-fastest copy of x and zeroes both
// accumulators in one pass over the image.
#include "common.cuh"
#include "fused.cuh"
#include "lean.cuh"

namespace srf {

// Generic path for a LOR whose projector and backprojector traverse along different axes
// (non-TOF with |xd| == |yd|): two setups, as in the standalone kernels.
template <int G, bool TOF>
__device__ __forceinline__ float tie_project(const float *l, float tv, int lane, const Grid &g, const TofParams &tp,
                                             const View &x, const View &xt) {
    float acc = 0.0f;
    LorSetup S;
    if (setup_lor<TOF, RULES_PROJ>(l[0], l[1], l[2], l[3], l[4], l[5], tv, g, tp, x.st, xt.st, xt.ptr != nullptr, S)) {
        const float *im = (!S.xdom && xt.ptr) ? xt.ptr : x.ptr;
        for (int ip = S.lo + lane; ip <= S.hi; ip += G)
            slab<TOF, RULES_PROJ>(S, ip, [&](int32_t off, float w) { acc += __ldg(im + off) * w; });
    }
    return group_sum<G>(acc);
}

template <int G, bool TOF>
__device__ __forceinline__ void tie_backproject(const float *l, float tv, float r, int lane, const Grid &g,
                                                const TofParams &tp, const View &bp, const View &bpt) {
    LorSetup S;
    if (r != 0.0f && setup_lor<TOF, RULES_BACK>(l[0], l[1], l[2], l[3], l[4], l[5], tv, g, tp, bp.st, bpt.st, bpt.ptr != nullptr, S)) {
        float *im = (!S.xdom && bpt.ptr) ? bpt.ptr : bp.ptr;
        for (int ip = S.lo + lane; ip <= S.hi; ip += G)
            slab<TOF, RULES_BACK>(S, ip, [&](int32_t off, float w) { atomicAdd(im + off, r * w); });
    }
}

template <int G, bool TOF>
__device__ __forceinline__ void tie_path(const float *l, float tv, float yv, float ad, int lane, const Grid &g,
                                         const TofParams &tp, const View &x, const View &xt,
                                         const View &bp, const View &bpt, int rule, float eps,
                                         double &ll, bool want_ll) {
    const float p = tie_project<G, TOF>(l, tv, lane, g, tp, x, xt);
    const float den = __fadd_rn(__fadd_rn(p, ad), eps);
    const float r = (rule == SRF_RATIO_DIV_NO_NAN) ? ((den == 0.0f) ? 0.0f : __fdiv_rn(yv, den)) : __fdiv_rn(yv, den);
    if (want_ll && lane == 0 && den > 0.0f) ll += (double)yv * log((double)den);  // FP64 term and sum
    tie_backproject<G, TOF>(l, tv, r, lane, g, tp, bp, bpt);
}

// What a traversal of osem_warp_batch does per LOR: the fused OSEM step, or one of its two halves
// on its own (the projector into out[i], or the backprojector of the values passed as y).
enum TraceMode : int { MODE_FUSED = 0, MODE_PROJ = 1, MODE_BACK = 2, MODE_ADJ = 3 };

// LORs [base, base + 32) of one study: lane-parallel setup of the 32 records into wrecs, then
// the warp's 32/G groups walk them (projection, ratio, backprojection per LOR) on the lean slab
// loop (lean.cuh). x/x_t and bp/bp_t have equal strides (offsets are computed once for the
// gather and the scatter). The projection walks the slabs the projector's endpoint rule keeps;
// when that is the whole slab range and it fits one chunk of G*U slabs (the usual case with a
// truncated TOF kernel), the backprojection reuses the chunk's offsets and weights.
template <int G, bool TOF, int U, int MODE = MODE_FUSED, bool QDIV = false>
__device__ __forceinline__ void osem_warp_batch(LeanRec *wrecs, const float *__restrict__ lors,
                                                int64_t n, int stride, const float *__restrict__ tof,
                                                int tof_stride, const Grid &g, const GridK &k,
                                                const TofParams &tp, const float *__restrict__ y,
                                                const float *__restrict__ add, int rule, float eps,
                                                const View &x, const View &xt,
                                                const View &bp, const View &bpt, int64_t base,
                                                bool want_ll, double &ll, float *__restrict__ out = nullptr) {
    constexpr int GPW = 32 / G;
    const int lane32 = threadIdx.x & 31;
    const int lane = threadIdx.x & (G - 1);
    const int gi = lane32 / G;
    const bool have_t = xt.ptr != nullptr;
    {  // lane-parallel setup of the warp's next 32 LORs
        const int64_t i = base + lane32;
        LeanRec E = {};
        E.lo = 1;
        if (i < n) {
            const float *l = lors + i * stride;
            float lv[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) lv[c] = __ldg(l + c);
            const float tv = TOF ? __ldg(tof + i * tof_stride) : 0.0f;
            const float yv = y ? __ldg(y + i) : 1.0f;
            LorRec R = setup_rec<TOF>(lv, tv, yv, g, k);
            R.ad = add ? __ldg(add + i) : 0.0f;
            E = make_lean<TOF>(R, g, k, x.st, xt.st, have_t);
        }
        store_lean(&wrecs[lane32], E);
    }
    __syncwarp();
    for (int j0 = 0; j0 < 32; j0 += GPW) {
        const int j = j0 + gi;
        const LeanRec E = load_lean(&wrecs[j]);
        const int64_t i = base + j;
        if (!TOF && (E.flags & F_TIE)) {  // ties exist only under the non-TOF projector rule
            float lv[6];
            const float *l = lors + i * stride;
#pragma unroll
            for (int c = 0; c < 6; ++c) lv[c] = __ldg(l + c);
            const float tv = TOF ? __ldg(tof + i * tof_stride) : 0.0f;
            if (MODE == MODE_FUSED) {
                tie_path<G, TOF>(lv, tv, E.yv, E.ad, lane, g, tp, x, xt, bp, bpt, rule, eps, ll, want_ll);
            } else if (MODE == MODE_PROJ) {
                const float p = tie_project<G, TOF>(lv, tv, lane, g, tp, x, xt);
                if (lane == 0) out[i] = p;
            } else {
                tie_backproject<G, TOF>(lv, tv, E.yv, lane, g, tp, bp, bpt);
            }
            continue;
        }
        const bool valid = E.flags & F_VALID;
        const bool xdom = E.flags & F_XDOM;
        const LeanAxes ax = lean_axes(E, g, x.st, xt.st, have_t);
        const float *xim = (!xdom && have_t) ? xt.ptr : x.ptr;
        float *bim = (!xdom && have_t) ? bpt.ptr : bp.ptr;
        // the projector's slabs: [plo, phi] (empty when the projector skips the LOR)
        const int plo = (E.flags & F_PROJ) ? max(E.lo, E.pmlo) : 1;
        const int phi = (E.flags & F_PROJ) ? min(E.hi, E.pmhi) : 0;
        const bool shared = (plo == E.lo) && (phi == E.hi) && (E.hi - E.lo + 1 <= G * U);
        int32_t o[U][3];
        float w[U][3];
        float acc = 0.0f;
        if (MODE != MODE_BACK && valid) {
            const float ppmax = (float)(phi - E.ic);
            for (int c0 = plo; c0 <= phi; c0 += G * U) {
                lean_chunk<TOF, U, G, QDIV>(E, ax, c0, phi, ppmax, lane, o, w);
                float xv[U][3];
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int c = 0; c < 3; ++c) xv[u][c] = (w[u][c] != 0.0f) ? __ldg(xim + o[u][c]) : 0.0f;
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int c = 0; c < 3; ++c) acc = fmaf(xv[u][c], w[u][c], acc);
            }
        }
        float r;
        if (MODE == MODE_BACK) {
            if (!valid) continue;
            r = E.yv;
        } else {
            const float p = group_sum<G>(acc) * E.invL2;
            if (MODE == MODE_PROJ) {
                if (lane == 0 && i < n) out[i] = p;  // 0 for a skipped LOR, as the reference's memset
                continue;
            }
            if (!valid) continue;
            const float den = __fadd_rn(__fadd_rn(p, E.ad), eps);
            if (rule == SRF_RATIO_DIV_NO_NAN)
                r = (den == 0.0f) ? 0.0f : __fdiv_rn(E.yv, den);
            else
                r = __fdiv_rn(E.yv, den);
            if (want_ll && lane == 0 && den > 0.0f) ll += (double)E.yv * log((double)den);  // FP64 term and sum
        }
        if (r == 0.0f) continue;
        if (MODE == MODE_FUSED && shared) {
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    if (w[u][c] != 0.0f) atomicAdd(bim + o[u][c], r * w[u][c]);
        } else {
            const float ppmax = (float)(E.hi - E.ic);
            for (int c0 = E.lo; c0 <= E.hi; c0 += G * U) {
                lean_chunk<TOF, U, G, QDIV>(E, ax, c0, E.hi, ppmax, lane, o, w);
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        if (w[u][c] != 0.0f) atomicAdd(bim + o[u][c], r * w[u][c]);
            }
        }
    }
    __syncwarp();
}

// One warp handles 32 consecutive LORs per round: lane j sets up LOR j into shared memory, then
// the warp's 32/G groups walk the records. x/x_t and bp/bp_t have equal strides (offsets are
// computed once for the gather and the scatter).
// Single-study blocks are 128 threads: with the 4-slab variant's register budget (<= 102 per
// thread at 5 blocks per SM) that is 20 resident warps per SM instead of 16 with 256-thread blocks.
constexpr int kOsemBlock = 128;

template <int G, bool TOF, int U, int MINB, bool QDIV>
__global__ void __launch_bounds__(kOsemBlock, MINB)
k_osem_subset(const float *__restrict__ lors, int64_t n, int stride, const float *__restrict__ tof,
              int tof_stride, Grid g, TofParams tp, const float *__restrict__ y,
              const float *__restrict__ add, int rule, float eps, View x, View xt, View bp, View bpt,
              double *__restrict__ loglik) {
    __shared__ LeanRec recs[kOsemBlock / 32][32];
    const int wib = threadIdx.x >> 5;
    const int lane32 = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const GridK k = make_gridk<TOF>(g, tp);
    const bool want_ll = loglik != nullptr;
    double ll = 0.0;
    for (int64_t base = warp * 32; base < n; base += nwarps * 32) {
        osem_warp_batch<G, TOF, U, MODE_FUSED, QDIV>(recs[wib], lors, n, stride, tof, tof_stride, g, k, tp, y, add, rule, eps, x, xt, bp, bpt, base, want_ll, ll);
    }
    if (want_ll) {
#pragma unroll
        for (int o2 = 16; o2 > 0; o2 >>= 1) ll += __shfl_xor_sync(0xffffffffu, ll, o2);
        if (lane32 == 0 && ll != 0.0) atomicAdd(loglik, ll);
    }
}

// The standalone projector (MODE_PROJ: out[i] for every LOR of x / x_t) and backprojector
// (MODE_BACK: values[i] into the accumulators bp / bp_t) on the fused kernel's traversal, for
// srf_projection(_tof) and srf_backprojection(_tof).
template <int G, bool TOF, int U, int MINB, int MODE, bool QDIV>
__global__ void __launch_bounds__(kOsemBlock, MINB)
k_trace_fused(const float *__restrict__ lors, int64_t n, int stride, const float *__restrict__ tof,
              int tof_stride, Grid g, TofParams tp, const float *__restrict__ values, float *__restrict__ out,
              View v, View vt) {
    __shared__ LeanRec recs[kOsemBlock / 32][32];
    const int wib = threadIdx.x >> 5;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const GridK k = make_gridk<TOF>(g, tp);
    double ll = 0.0;
    for (int64_t base = warp * 32; base < n; base += nwarps * 32)
        osem_warp_batch<G, TOF, U, MODE, QDIV>(recs[wib], lors, n, stride, tof, tof_stride, g, k, tp, values, nullptr,
                                         SRF_RATIO_PLAIN, 0.0f, v, vt, v, vt, base, false, ll, out);
}

// The x-dominant in-plane coordinate is divided by dy = (sy / ny) / (sx / nx) in the reference;
// dy == 1 (square transaxial voxels) makes that division an identity the kernels compile out.
inline bool grid_qdiv(const Grid &g) {
    const float dx_ = g.sx / (float)g.nx;
    return (g.sy / (float)g.ny) / dx_ != 1.0f;
}

template <int G, bool TOF, int MODE>
static int launch_trace_fused_g(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                                const Grid &g, const TofParams &tp, const float *values, float *out,
                                const View &v, const View &vt, cudaStream_t s) {
    auto kern = grid_qdiv(g) ? k_trace_fused<G, TOF, 4, 5, MODE, true> : k_trace_fused<G, TOF, 4, 5, MODE, false>;
    unsigned blocks = grid_for(kern, n, kOsemBlock, 0, kOsemBlock);
    kern<<<blocks, kOsemBlock, 0, s>>>(lors, n, stride, tof, tof_stride, g, tp, values, out, v, vt);
    return check_cuda("fused trace kernel launch");
}

template <bool TOF, int MODE>
static int launch_trace_fused(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                              const Grid &g, const TofParams &tp, const float *values, float *out,
                              const View &v, const View &vt, cudaStream_t s) {
    if (n == 0) return ok();
    switch (group_lanes()) {
    case 8: return launch_trace_fused_g<8, TOF, MODE>(lors, n, stride, tof, tof_stride, g, tp, values, out, v, vt, s);
    case 16: return launch_trace_fused_g<16, TOF, MODE>(lors, n, stride, tof, tof_stride, g, tp, values, out, v, vt, s);
    default: return launch_trace_fused_g<32, TOF, MODE>(lors, n, stride, tof, tof_stride, g, tp, values, out, v, vt, s);
    }
}

int fused_projection(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                     const Grid &g, const TofParams &tp, const View &v, const View &vt, float *out,
                     cudaStream_t s) {
    return tof ? launch_trace_fused<true, MODE_PROJ>(lors, n, stride, tof, tof_stride, g, tp, nullptr, out, v, vt, s)
               : launch_trace_fused<false, MODE_PROJ>(lors, n, stride, nullptr, 1, g, tp, nullptr, out, v, vt, s);
}

int fused_backprojection(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                         const Grid &g, const TofParams &tp, const float *values, const View &v,
                         const View &vt, cudaStream_t s) {
    return tof ? launch_trace_fused<true, MODE_BACK>(lors, n, stride, tof, tof_stride, g, tp, values, nullptr, v, vt, s)
               : launch_trace_fused<false, MODE_BACK>(lors, n, stride, nullptr, 1, g, tp, values, nullptr, v, vt, s);
}

// ---------------------------------------------------------------- sensitivity image
// Backprojection of 1 along every ordered crystal pair of the block-full sensitivity image, on the
// fused traversal: LOR k = ((i*nb + j)*m + a)*m + b runs from table row i*m + a to row j*m + b
// (the table holds the reference's float32 crystal positions), generated on the fly.
__device__ __forceinline__ void emap_endpoints(const float *__restrict__ table, int nb, int m, int64_t k,
                                               float (&lv)[6]) {
    const int64_t mm = (int64_t)m * m;
    const int64_t blk = k / mm, rem = k - blk * mm;
    const int i = (int)(blk / nb), j = (int)(blk - (blk / nb) * nb);
    const int a = (int)(rem / m), b = (int)(rem - (rem / m) * m);
    const float *e1 = table + 3 * ((int64_t)i * m + a);
    const float *e2 = table + 3 * ((int64_t)j * m + b);
    lv[0] = __ldg(e1); lv[1] = __ldg(e1 + 1); lv[2] = __ldg(e1 + 2);
    lv[3] = __ldg(e2); lv[4] = __ldg(e2 + 1); lv[5] = __ldg(e2 + 2);
}

template <int G, int U, bool QDIV>
__device__ __forceinline__ void emap_warp(LeanRec *wrecs, const float *__restrict__ table, int nb, int m, int64_t n,
                                          const Grid &g, const GridK &k, const TofParams &tp, const View &v,
                                          const View &vt, int64_t base) {
    constexpr int GPW = 32 / G;
    const int lane32 = threadIdx.x & 31;
    const int lane = threadIdx.x & (G - 1);
    const int gi = lane32 / G;
    const bool have_t = vt.ptr != nullptr;
    {
        const int64_t i = base + lane32;
        LeanRec E = {};
        E.lo = 1;
        if (i < n) {
            float lv[6];
            emap_endpoints(table, nb, m, i, lv);
            E = make_lean<false>(setup_rec<false>(lv, 0.0f, 1.0f, g, k), g, k, v.st, vt.st, have_t);
        }
        store_lean(&wrecs[lane32], E);
    }
    __syncwarp();
    for (int j0 = 0; j0 < 32; j0 += GPW) {
        const int j = j0 + gi;
        const LeanRec E = load_lean(&wrecs[j]);
        const int64_t i = base + j;
        if (E.flags & F_TIE) {  // the backprojector's own axis differs from the projector's: generic path
            float lv[6];
            emap_endpoints(table, nb, m, i, lv);
            tie_backproject<G, false>(lv, 0.0f, 1.0f, lane, g, tp, v, vt);
            continue;
        }
        if (!(E.flags & F_VALID)) continue;
        const LeanAxes ax = lean_axes(E, g, v.st, vt.st, have_t);
        float *im = (!(E.flags & F_XDOM) && have_t) ? vt.ptr : v.ptr;
        int32_t o[U][3];
        float w[U][3];
        const float ppmax = (float)(E.hi - E.ic);
        for (int c0 = E.lo; c0 <= E.hi; c0 += G * U) {
            lean_chunk<false, U, G, QDIV>(E, ax, c0, E.hi, ppmax, lane, o, w);
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    if (w[u][c] != 0.0f) atomicAdd(im + o[u][c], w[u][c]);
        }
    }
    __syncwarp();
}

template <int G, int U, int MINB, bool QDIV>
__global__ void __launch_bounds__(kOsemBlock, MINB)
k_emap_fused(const float *__restrict__ table, int nb, int m, Grid g, View v, View vt) {
    __shared__ LeanRec recs[kOsemBlock / 32][32];
    const int wib = threadIdx.x >> 5;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const TofParams tp{0, 0, 0};
    const GridK k = make_gridk<false>(g, tp);
    const int64_t n = (int64_t)nb * nb * (int64_t)m * m;
    for (int64_t base = warp * 32; base < n; base += nwarps * 32)
        emap_warp<G, U, QDIV>(recs[wib], table, nb, m, n, g, k, tp, v, vt, base);
}

int fused_emap(const float *table, int nb, int m, const Grid &g, const View &v, const View &vt, cudaStream_t s) {
    const int64_t n = (int64_t)nb * nb * (int64_t)m * m;
    if (n == 0) return ok();
    auto kern = grid_qdiv(g) ? k_emap_fused<32, 4, 5, true> : k_emap_fused<32, 4, 5, false>;
    unsigned blocks = grid_for(kern, n, kOsemBlock, 0, kOsemBlock);
    kern<<<blocks, kOsemBlock, 0, s>>>(table, nb, m, g, v, vt);
    return check_cuda("emap kernel launch");
}

// ---------------------------------------------------------------- batched projector / adjoint
// The projector (MODE_PROJ) and its exact adjoint (MODE_ADJ: projector rules, projector weights
// with 1/L^2, scattered) for nb <= kMaxBatch images that share the grid and the LORs: image b at
// element offset b * bstride in both layouts; values / out are nb rows of n at row stride ostride.
// Each LOR is set up once and its slab candidates are computed once for all images.
constexpr int kMaxBatch = 8;

template <int G, bool TOF, int MODE>
__device__ __forceinline__ void tie_batch(const float *l, float tv, int lane, const Grid &g, const TofParams &tp,
                                          const View &v, const View &vt, int nb, int64_t bstride,
                                          const float (&val)[kMaxBatch], float (&acc)[kMaxBatch]) {
    LorSetup S;
    if (!setup_lor<TOF, RULES_PROJ>(l[0], l[1], l[2], l[3], l[4], l[5], tv, g, tp, v.st, vt.st, vt.ptr != nullptr, S)) return;
    float *im = (!S.xdom && vt.ptr) ? vt.ptr : v.ptr;
    for (int ip = S.lo + lane; ip <= S.hi; ip += G)
        slab<TOF, RULES_PROJ>(S, ip, [&](int32_t off, float w) {
#pragma unroll
            for (int b = 0; b < kMaxBatch; ++b) {
                if (b >= nb) continue;
                if (MODE == MODE_PROJ) acc[b] = fmaf(__ldg(im + b * bstride + off), w, acc[b]);
                else if (val[b] != 0.0f) atomicAdd(im + b * bstride + off, val[b] * w);
            }
        });
}

template <int G, bool TOF, int U, int MODE, bool QDIV>
__device__ __forceinline__ void batch_warp(LeanRec *wrecs, const float *__restrict__ lors, int64_t n, int stride,
                                           const float *__restrict__ tof, int tof_stride, const Grid &g,
                                           const GridK &k, const TofParams &tp, int nb, int64_t bstride,
                                           const float *__restrict__ values, float *__restrict__ out,
                                           int64_t ostride, const View &v, const View &vt, int64_t base) {
    constexpr int GPW = 32 / G;
    const int lane32 = threadIdx.x & 31;
    const int lane = threadIdx.x & (G - 1);
    const int gi = lane32 / G;
    const bool have_t = vt.ptr != nullptr;
    {
        const int64_t i = base + lane32;
        LeanRec E = {};
        E.lo = 1;
        if (i < n) {
            const float *l = lors + i * stride;
            float lv[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) lv[c] = __ldg(l + c);
            const float tv = TOF ? __ldg(tof + i * tof_stride) : 0.0f;
            E = make_lean<TOF>(setup_rec<TOF>(lv, tv, 1.0f, g, k), g, k, v.st, vt.st, have_t);
        }
        store_lean(&wrecs[lane32], E);
    }
    __syncwarp();
    for (int j0 = 0; j0 < 32; j0 += GPW) {
        const int j = j0 + gi;
        const LeanRec E = load_lean(&wrecs[j]);
        const int64_t i = base + j;
        float acc[kMaxBatch], val[kMaxBatch];
        bool any = false;
#pragma unroll
        for (int b = 0; b < kMaxBatch; ++b) {
            acc[b] = 0.0f;
            val[b] = (MODE == MODE_ADJ && b < nb && i < n) ? __ldg(values + b * ostride + i) : 0.0f;
            any = any || val[b] != 0.0f;
        }
        if (!TOF && (E.flags & F_TIE)) {  // ties exist only under the non-TOF projector rule
            float lv[6];
            const float *l = lors + i * stride;
#pragma unroll
            for (int c = 0; c < 6; ++c) lv[c] = __ldg(l + c);
            if (MODE == MODE_PROJ || any) tie_batch<G, TOF, MODE>(lv, 0.0f, lane, g, tp, v, vt, nb, bstride, val, acc);
        } else if ((E.flags & F_VALID) && (E.flags & F_PROJ) && (MODE == MODE_PROJ || any)) {
            const LeanAxes ax = lean_axes(E, g, v.st, vt.st, have_t);
            float *im = (!(E.flags & F_XDOM) && have_t) ? vt.ptr : v.ptr;
            if (MODE == MODE_ADJ)
#pragma unroll
                for (int b = 0; b < kMaxBatch; ++b) val[b] *= E.invL2;
            // the projector's slabs: its endpoint rule keeps [pmlo, pmhi]
            const int plo = max(E.lo, E.pmlo), phi = min(E.hi, E.pmhi);
            const float ppmax = (float)(phi - E.ic);
            int32_t o[U][3];
            float w[U][3];
            for (int c0 = plo; c0 <= phi; c0 += G * U) {
                lean_chunk<TOF, U, G, QDIV>(E, ax, c0, phi, ppmax, lane, o, w);
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        if (w[u][c] == 0.0f) continue;
#pragma unroll
                        for (int b = 0; b < kMaxBatch; ++b) {
                            if (b >= nb) continue;
                            if (MODE == MODE_PROJ) acc[b] = fmaf(__ldg(im + b * bstride + o[u][c]), w[u][c], acc[b]);
                            else if (val[b] != 0.0f) atomicAdd(im + b * bstride + o[u][c], val[b] * w[u][c]);
                        }
                    }
            }
#pragma unroll
            for (int b = 0; b < kMaxBatch; ++b) acc[b] *= E.invL2;
        }
        if (MODE == MODE_PROJ) {
#pragma unroll
            for (int b = 0; b < kMaxBatch; ++b) {
                const float p = group_sum<G>(acc[b]);
                if (lane == 0 && i < n && b < nb) out[b * ostride + i] = p;
            }
        }
    }
    __syncwarp();
}

template <int G, bool TOF, int U, int MINB, int MODE, bool QDIV>
__global__ void __launch_bounds__(kOsemBlock, MINB)
k_trace_fused_batch(const float *__restrict__ lors, int64_t n, int stride, const float *__restrict__ tof,
                    int tof_stride, Grid g, TofParams tp, int nb, int64_t bstride,
                    const float *__restrict__ values, float *__restrict__ out, int64_t ostride, View v, View vt) {
    __shared__ LeanRec recs[kOsemBlock / 32][32];
    const int wib = threadIdx.x >> 5;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const GridK k = make_gridk<TOF>(g, tp);
    for (int64_t base = warp * 32; base < n; base += nwarps * 32)
        batch_warp<G, TOF, U, MODE, QDIV>(recs[wib], lors, n, stride, tof, tof_stride, g, k, tp, nb, bstride, values,
                                          out, ostride, v, vt, base);
}

template <bool TOF, int MODE>
static int launch_fused_batch(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                              const Grid &g, const TofParams &tp, int nb, int64_t bstride, const float *values,
                              float *out, int64_t ostride, const View &v, const View &vt, cudaStream_t s) {
    if (n == 0) return ok();
    auto kern = grid_qdiv(g) ? k_trace_fused_batch<32, TOF, 4, 4, MODE, true> : k_trace_fused_batch<32, TOF, 4, 4, MODE, false>;
    unsigned blocks = grid_for(kern, n, kOsemBlock, 0, kOsemBlock);
    kern<<<blocks, kOsemBlock, 0, s>>>(lors, n, stride, tof, tof_stride, g, tp, nb, bstride, values, out, ostride, v, vt);
    return check_cuda("batched projector kernel launch");
}

int fused_projection_batch(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                           const Grid &g, const TofParams &tp, int nb, int64_t bstride, const View &v,
                           const View &vt, float *out, int64_t ostride, cudaStream_t s) {
    return tof ? launch_fused_batch<true, MODE_PROJ>(lors, n, stride, tof, tof_stride, g, tp, nb, bstride, nullptr, out, ostride, v, vt, s)
               : launch_fused_batch<false, MODE_PROJ>(lors, n, stride, nullptr, 1, g, tp, nb, bstride, nullptr, out, ostride, v, vt, s);
}

int fused_adjoint_batch(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                        const Grid &g, const TofParams &tp, int nb, int64_t bstride, const float *values,
                        int64_t vstride, const View &v, const View &vt, cudaStream_t s) {
    return tof ? launch_fused_batch<true, MODE_ADJ>(lors, n, stride, tof, tof_stride, g, tp, nb, bstride, values, nullptr, vstride, v, vt, s)
               : launch_fused_batch<false, MODE_ADJ>(lors, n, stride, nullptr, 1, g, tp, nb, bstride, values, nullptr, vstride, v, vt, s);
}

template <int G, bool TOF, int U, int MINB>
static int launch_osem_g(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                         const Grid &g, const TofParams &tp, const float *y, const float *add, int rule, float eps,
                         const View &x, const View &xt, const View &bp, const View &bpt,
                         double *loglik, cudaStream_t s) {
    auto kern = grid_qdiv(g) ? k_osem_subset<G, TOF, U, MINB, true> : k_osem_subset<G, TOF, U, MINB, false>;
    unsigned blocks = grid_for(kern, n, kOsemBlock, 0, kOsemBlock);
    kern<<<blocks, kOsemBlock, 0, s>>>(lors, n, stride, tof, tof_stride, g, tp, y, add, rule, eps, x, xt, bp, bpt, loglik);
    return check_cuda("osem subset kernel launch");
}

template <int G, bool TOF>
static int launch_osem_u(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                         const Grid &g, const TofParams &tp, const float *y, const float *add, int rule, float eps,
                         const View &x, const View &xt, const View &bp, const View &bpt,
                         double *loglik, cudaStream_t s) {
    if (slabs_per_lane() == 2)
        return launch_osem_g<G, TOF, 2, 6>(lors, n, stride, tof, tof_stride, g, tp, y, add, rule, eps, x, xt, bp, bpt, loglik, s);
    return launch_osem_g<G, TOF, 4, 5>(lors, n, stride, tof, tof_stride, g, tp, y, add, rule, eps, x, xt, bp, bpt, loglik, s);
}

template <bool TOF>
static int launch_osem(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                       const Grid &g, const TofParams &tp, const float *y, const float *add, int rule, float eps,
                       const View &x, const View &xt, const View &bp, const View &bpt,
                       double *loglik, cudaStream_t s) {
    switch (group_lanes()) {
    case 8: return launch_osem_u<8, TOF>(lors, n, stride, tof, tof_stride, g, tp, y, add, rule, eps, x, xt, bp, bpt, loglik, s);
    case 16: return launch_osem_u<16, TOF>(lors, n, stride, tof, tof_stride, g, tp, y, add, rule, eps, x, xt, bp, bpt, loglik, s);
    default: return launch_osem_u<32, TOF>(lors, n, stride, tof, tof_stride, g, tp, y, add, rule, eps, x, xt, bp, bpt, loglik, s);
    }
}

// 32 x 32 (x, y) tiles of one z slice; 32 x 8 threads.
constexpr int kTile = 32;

// One 32 x 32 (x, y) tile of z slice bz; 32 x 8 threads.
__device__ __forceinline__ void update_tile(float *__restrict__ x, float *__restrict__ xt,
                                            float *__restrict__ bp, float *__restrict__ bpt,
                                            const float *__restrict__ emap, int guard, int nx,
                                            int ny, int tbx, int tby, int bz,
                                            float (&tin)[kTile][kTile + 1],
                                            float (&tout)[kTile][kTile + 1]) {
    constexpr int R = kTile / 8;  // rows per thread
    const int bx = tbx * kTile, by = tby * kTile;
    const int64_t zoff = (int64_t)bz * nx * ny;
    const int tx = threadIdx.x, ty = threadIdx.y;
    // issue every load of this thread before any store, so a thread has 4R loads in flight
    float vb[R], vx[R], ve[R], vt[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int iy = by + ty + 8 * r, ix = bx + tx;
        const bool in = ix < nx && iy < ny;
        const int64_t o = zoff + (int64_t)iy * nx + ix;
        vb[r] = in ? bp[o] : 0.0f;
        vx[r] = in ? x[o] : 0.0f;
        ve[r] = in ? emap[o] : 1.0f;
        if (bpt) {  // bpt is y-fastest: element (ix, iy) at ix*ny + iy
            const int jx = bx + ty + 8 * r, jy = by + tx;
            vt[r] = (jx < nx && jy < ny) ? bpt[zoff + (int64_t)jx * ny + jy] : 0.0f;
        }
    }
    if (bpt) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int jx = bx + ty + 8 * r, jy = by + tx;
            tin[ty + 8 * r][tx] = vt[r];  // [x_local][y_local]
            if (jx < nx && jy < ny) bpt[zoff + (int64_t)jx * ny + jy] = 0.0f;
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = ty + 8 * r;
        const int iy = by + j, ix = bx + tx;
        if (ix < nx && iy < ny) {
            const int64_t o = zoff + (int64_t)iy * nx + ix;
            float b = vb[r];
            if (bpt) b = __fadd_rn(b, tin[tx][j]);
            float e = ve[r];
            if (guard && e == 0.0f) e = 1e8f;
            const float xn = __fdiv_rn(__fmul_rn(vx[r], b), e);
            x[o] = xn;
            bp[o] = 0.0f;
            tout[j][tx] = xn;  // [y_local][x_local]
        }
    }
    if (xt) {
        __syncthreads();
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int j = ty + 8 * r;
            const int ix = bx + j, iy = by + tx;
            if (ix < nx && iy < ny) xt[zoff + (int64_t)ix * ny + iy] = tout[tx][j];
        }
    }
}


// The same update with 16-byte accesses: thread t of 256 covers four consecutive elements of row
// t / 8 of the tile (x-fastest arrays) and of column t / 8 (the y-fastest copies), so each thread
// moves 64 bytes per array pass with four loads in flight. Needs nx and ny multiples of 4 and
// 16-byte aligned arrays. Same arithmetic as update_tile.
__global__ void __launch_bounds__(kTile * 8)
k_osem_update4(float *__restrict__ x, float *__restrict__ xt, float *__restrict__ bp,
               float *__restrict__ bpt, const float *__restrict__ emap, int guard, int nx, int ny) {
    __shared__ float tin[kTile][kTile + 1];   // bpt tile: [x_local][y_local]
    __shared__ float tout[kTile][kTile + 1];  // new x:    [y_local][x_local]
    const int t = threadIdx.x;
    const int r = t >> 3, c = (t & 7) * 4;    // row of the tile, first of four columns
    const int bx = blockIdx.x * kTile, by = blockIdx.y * kTile;
    const int64_t zoff = (int64_t)blockIdx.z * nx * ny;
    const bool in = (bx + c < nx) && (by + r < ny);       // x-fastest element (bx + c .. + 3, by + r)
    const bool in_t = (bx + r < nx) && (by + c < ny);     // y-fastest element (bx + r, by + c .. + 3)
    const int64_t o = zoff + (int64_t)(by + r) * nx + bx + c;
    const int64_t ot = zoff + (int64_t)(bx + r) * ny + by + c;
    const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 vb = zero, vx = zero, ve = make_float4(1.0f, 1.0f, 1.0f, 1.0f), vt = zero;
    if (in) {
        vb = *reinterpret_cast<const float4 *>(bp + o);
        vx = *reinterpret_cast<const float4 *>(x + o);
        ve = __ldg(reinterpret_cast<const float4 *>(emap + o));
    }
    if (bpt) {
        if (in_t) vt = *reinterpret_cast<const float4 *>(bpt + ot);
        tin[r][c] = vt.x; tin[r][c + 1] = vt.y; tin[r][c + 2] = vt.z; tin[r][c + 3] = vt.w;
        __syncthreads();
        if (in_t) *reinterpret_cast<float4 *>(bpt + ot) = zero;
    }
    const float b_[4] = {vb.x, vb.y, vb.z, vb.w};
    const float x_[4] = {vx.x, vx.y, vx.z, vx.w};
    const float e_[4] = {ve.x, ve.y, ve.z, ve.w};
    float xn[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float b = b_[j];
        if (bpt) b = __fadd_rn(b, tin[c + j][r]);
        float e = e_[j];
        if (guard && e == 0.0f) e = 1e8f;
        xn[j] = __fdiv_rn(__fmul_rn(x_[j], b), e);
    }
    if (in) {
        *reinterpret_cast<float4 *>(x + o) = make_float4(xn[0], xn[1], xn[2], xn[3]);
        *reinterpret_cast<float4 *>(bp + o) = zero;
    }
    if (xt) {
#pragma unroll
        for (int j = 0; j < 4; ++j) tout[r][c + j] = xn[j];
        __syncthreads();
        if (in_t)
            *reinterpret_cast<float4 *>(xt + ot) =
                make_float4(tout[c][r], tout[c + 1][r], tout[c + 2][r], tout[c + 3][r]);
    }
}

__global__ void __launch_bounds__(kTile * 8)
k_osem_update(float *__restrict__ x, float *__restrict__ xt, float *__restrict__ bp,
              float *__restrict__ bpt, const float *__restrict__ emap, int guard, int nx, int ny) {
    __shared__ float tin[kTile][kTile + 1];
    __shared__ float tout[kTile][kTile + 1];
    update_tile(x, xt, bp, bpt, emap, guard, nx, ny, blockIdx.x, blockIdx.y, blockIdx.z, tin, tout);
}

// ---------------------------------------------------------------- many studies per launch

// Index of the segment holding `v` in an ascending offsets array off[0..n] (off[0] = 0).
__device__ __forceinline__ int find_segment(const int64_t *__restrict__ off, int n, int64_t v) {
    int lo = 0, hi = n;  // invariant: off[lo] <= v < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= v) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool study_ok(const srf_study &st) {
    return st.n >= 0 && st.lor_stride >= 6 && st.grid[0] > 0 && st.grid[1] > 0 && st.grid[2] > 0 &&
           st.grid[0] <= 65536 && st.grid[1] <= 65536 && st.grid[2] <= 65536 &&
           (int64_t)st.grid[0] * st.grid[1] * st.grid[2] < (int64_t(1) << 31) && st.lors &&
           st.x && st.bp && st.size[0] > 0.0f && st.size[1] > 0.0f && st.size[2] > 0.0f &&
           ((st.x_t == nullptr) == (st.bp_t == nullptr));
}

constexpr int kMaxStudiesSmem = 1024;

// One warp's current study, decoded once when the warp enters it and read through shared memory:
// in registers the grid constants and the four image views would push the traversal past its
// register budget (the single-study kernel gets them from the parameter bank instead).
struct WarpStudy {
    const float *lors, *tof, *y;
    int64_t n;
    int stride, tof_stride, ok;
    Grid g;
    GridK k;
    View x, xt, bp, bpt;
};

template <bool TOF>
__device__ __forceinline__ void decode_study(const srf_study &st, const TofParams &tp, WarpStudy &w) {
    w.ok = study_ok(st) && !(TOF && (st.tof == nullptr || st.tof_stride < 1));
    if (!w.ok) return;
    w.lors = st.lors; w.tof = st.tof; w.y = st.y;
    w.n = st.n; w.stride = st.lor_stride; w.tof_stride = st.tof_stride;
    w.g = Grid{st.grid[0], st.grid[1], st.grid[2], st.center[0], st.center[1], st.center[2],
               st.size[0], st.size[1], st.size[2]};
    w.k = make_gridk<TOF>(w.g, tp);
    const int64_t nxy = (int64_t)w.g.nx * w.g.ny;
    w.x = View{st.x, {1, w.g.nx, nxy}};
    w.bp = View{st.bp, {1, w.g.nx, nxy}};
    w.xt = View{st.x_t, {w.g.ny, 1, nxy}};
    w.bpt = View{st.bp_t, {w.g.ny, 1, nxy}};
}

// Persistent kernel over all studies' LOR batches: warp-batch b belongs to the study s with
// boff[s] <= b < boff[s + 1] (32 LORs per batch, each study padded to whole batches). Warps take
// batches in order from a ticket counter (work[0]) rather than by a fixed stride, so all warps
// stay within about one batch per warp of a common frontier: only the one or two studies under
// the frontier have their images in L2 (with fixed strides the warps drift apart and several
// studies' images compete for it). The last block to finish returns both counters to zero for
// the next launch in stream order. The batch offsets are staged in shared memory (when they
// fit), and a warp decodes a study descriptor only when it moves to another study.
template <int G, bool TOF, int U, int MINB>
__global__ void __launch_bounds__(kOsemBlock, MINB)
k_osem_batch(const srf_study *__restrict__ studies, int n_studies, const int64_t *__restrict__ boff,
             int64_t total_batches, TofParams tp, int rule, float eps, double *__restrict__ loglik) {
    __shared__ LeanRec recs[kOsemBlock / 32][32];
    __shared__ int64_t soff[kMaxStudiesSmem + 1];
    __shared__ WarpStudy wst[kOsemBlock / 32];
    const bool staged = n_studies <= kMaxStudiesSmem;
    if (staged)
        for (int t = threadIdx.x; t <= n_studies; t += blockDim.x) soff[t] = __ldg(boff + t);
    __syncthreads();
    const int64_t *off = staged ? soff : boff;
    unsigned long long *work = reinterpret_cast<unsigned long long *>(const_cast<int64_t *>(boff + n_studies + 1));
    const int wib = threadIdx.x >> 5;
    const int lane32 = threadIdx.x & 31;
    const bool want_ll = loglik != nullptr;
    WarpStudy &w = wst[wib];
    double ll = 0.0;
    int s = -1;
    for (;;) {
        unsigned long long ticket = 0;
        if (lane32 == 0) ticket = atomicAdd(work, 1ULL);
        const int64_t b = (int64_t)__shfl_sync(0xffffffffu, ticket, 0);
        if (b >= total_batches) break;
        if (s < 0 || b < off[s] || b >= off[s + 1]) {  // uniform over the warp
            int lo = 0, hi = n_studies;  // off[lo] <= b < off[hi]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (off[mid] <= b) lo = mid; else hi = mid;
            }
            s = lo;
            __syncwarp();
            if (lane32 == 0) decode_study<TOF>(studies[s], tp, w);
            __syncwarp();
        }
        if (!w.ok) continue;
        // one traversal for every study: the in-plane division (QDIV) is an identity for studies
        // with square transaxial voxels (a second inlined copy for them would spill)
        osem_warp_batch<G, TOF, U, MODE_FUSED, true>(recs[wib], w.lors, w.n, w.stride, w.tof, w.tof_stride,
                                                     w.g, w.k, tp, w.y, nullptr, rule, eps, w.x, w.xt,
                                                     w.bp, w.bpt, (b - off[s]) * 32, want_ll, ll);
    }
    if (want_ll) {
#pragma unroll
        for (int o2 = 16; o2 > 0; o2 >>= 1) ll += __shfl_xor_sync(0xffffffffu, ll, o2);
        if (lane32 == 0 && ll != 0.0) atomicAdd(loglik, ll);
    }
    __syncthreads();  // every warp of the block has taken its last ticket
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(work + 1, 1ULL) == gridDim.x - 1) {  // last block: reset for the next launch
            atomicExch(work, 0ULL);
            atomicExch(work + 1, 0ULL);
            __threadfence();
        }
    }
}

// Update of all studies: block t belongs to study s with toff[s] <= t < toff[s + 1].
__global__ void __launch_bounds__(kTile * 8)
k_osem_update_batch(const srf_study *__restrict__ studies, int n_studies,
                    const int64_t *__restrict__ toff, int guard) {
    __shared__ float tin[kTile][kTile + 1];
    __shared__ float tout[kTile][kTile + 1];
    const int64_t t = blockIdx.x;
    const int s = find_segment(toff, n_studies, t);
    const srf_study st = studies[s];
    if (!study_ok(st) || st.emap == nullptr) return;  // uniform over the block
    const int tx = (st.grid[0] + kTile - 1) / kTile, ty = (st.grid[1] + kTile - 1) / kTile;
    const int64_t local = t - __ldg(toff + s);
    if (local >= (int64_t)tx * ty * st.grid[2]) return;
    const int bz = (int)(local / ((int64_t)tx * ty));
    const int rem = (int)(local - (int64_t)bz * tx * ty);
    update_tile(st.x, st.x_t, st.bp, st.bp_t, st.emap, guard, st.grid[0], st.grid[1], rem % tx,
                rem / tx, bz, tin, tout);
}

template <int G, bool TOF, int U, int MINB>
static int launch_batch_g(const srf_study *studies, int n_studies, const int64_t *boff,
                          int64_t total, const TofParams &tp, int rule, float eps, double *ll,
                          cudaStream_t s) {
    auto kern = k_osem_batch<G, TOF, U, MINB>;
    unsigned blocks = grid_for(kern, total * 32, kOsemBlock, 0, kOsemBlock);
    kern<<<blocks, kOsemBlock, 0, s>>>(studies, n_studies, boff, total, tp, rule, eps, ll);
    return check_cuda("osem batch kernel launch");
}

template <bool TOF>
static int launch_batch(const srf_study *studies, int n_studies, const int64_t *boff, int64_t total,
                        const TofParams &tp, int rule, float eps, double *ll, cudaStream_t s) {
    const int u = slabs_per_lane();
    switch (group_lanes()) {
    case 8: return u == 2 ? launch_batch_g<8, TOF, 2, 6>(studies, n_studies, boff, total, tp, rule, eps, ll, s)
                          : launch_batch_g<8, TOF, 4, 5>(studies, n_studies, boff, total, tp, rule, eps, ll, s);
    case 16: return u == 2 ? launch_batch_g<16, TOF, 2, 6>(studies, n_studies, boff, total, tp, rule, eps, ll, s)
                           : launch_batch_g<16, TOF, 4, 5>(studies, n_studies, boff, total, tp, rule, eps, ll, s);
    default: return u == 2 ? launch_batch_g<32, TOF, 2, 6>(studies, n_studies, boff, total, tp, rule, eps, ll, s)
                           : launch_batch_g<32, TOF, 4, 5>(studies, n_studies, boff, total, tp, rule, eps, ll, s);
    }
}

}  // namespace srf

using namespace srf;

extern "C" {

int srf_osem_subset_batch(const srf_study *studies, int32_t n_studies,
                          const int64_t *batch_offsets, int64_t total_batches, int32_t use_tof,
                          float tof_bin, float tof_sigma2, float tof_nsigma, int32_t ratio_rule,
                          float eps, double *loglik, void *stream) {
    if (n_studies < 0 || total_batches < 0) return fail(SRF_EINVAL, "negative counts");
    if (n_studies == 0 || total_batches == 0) return ok();
    if (!studies || !batch_offsets) return fail(SRF_EINVAL, "studies and batch_offsets must not be NULL");
    if (ratio_rule != SRF_RATIO_DIV_NO_NAN && ratio_rule != SRF_RATIO_PLAIN)
        return fail(SRF_EINVAL, "unknown ratio rule %d", ratio_rule);
    if (!std::isfinite(eps)) return fail(SRF_ENONFINITE, "eps is not finite");
    cudaStream_t s = (cudaStream_t)stream;
    if (use_tof) {
        TofParams tp;
        int rc;
        if ((rc = check_tof_params(tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
        return launch_batch<true>(studies, n_studies, batch_offsets, total_batches, tp, ratio_rule, eps, loglik, s);
    }
    TofParams tp{0, 0, 0};
    return launch_batch<false>(studies, n_studies, batch_offsets, total_batches, tp, ratio_rule, eps, loglik, s);
}

int srf_osem_update_batch(const srf_study *studies, int32_t n_studies, const int64_t *tile_offsets,
                          int64_t total_tiles, int32_t guard_zero, void *stream) {
    if (n_studies < 0 || total_tiles < 0) return fail(SRF_EINVAL, "negative counts");
    if (n_studies == 0 || total_tiles == 0) return ok();
    if (!studies || !tile_offsets) return fail(SRF_EINVAL, "studies and tile_offsets must not be NULL");
    if (total_tiles > 0x7fffffffLL) return fail(SRF_ERANGE, "too many tiles");
    k_osem_update_batch<<<(unsigned)total_tiles, dim3(kTile, 8), 0, (cudaStream_t)stream>>>(
        studies, n_studies, tile_offsets, guard_zero);
    return check_cuda("osem update batch kernel launch");
}


int srf_osem_subset(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                    int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                    const float *y, const float *add, int32_t ratio_rule, float eps, const float *x,
                    const float *x_t, float *bp, float *bp_t, const int32_t grid[3],
                    const float center[3], const float size[3], double *loglik, void *stream) {
    Grid g; int rc;
    if ((rc = check_lors(lors, n, lor_stride))) return rc;
    if ((rc = check_geometry(grid, center, size, g))) return rc;
    if (ratio_rule != SRF_RATIO_DIV_NO_NAN && ratio_rule != SRF_RATIO_PLAIN)
        return fail(SRF_EINVAL, "unknown ratio rule %d", ratio_rule);
    if (!std::isfinite(eps)) return fail(SRF_ENONFINITE, "eps is not finite");
    const int64_t xs[3] = {1, g.nx, (int64_t)g.nx * g.ny};
    const int64_t ys[3] = {g.ny, 1, (int64_t)g.nx * g.ny};
    View vx, vxt, vbp, vbpt;
    if ((rc = check_view(x, xs, g, "x", vx, true))) return rc;
    if ((rc = check_view(x_t, ys, g, "x_t", vxt, false))) return rc;
    if ((rc = check_view(bp, xs, g, "bp", vbp, true))) return rc;
    if ((rc = check_view(bp_t, ys, g, "bp_t", vbpt, false))) return rc;
    if ((x_t == nullptr) != (bp_t == nullptr)) return fail(SRF_EINVAL, "x_t and bp_t must both be given or both be NULL");
    if (n == 0) return ok();
    cudaStream_t s = (cudaStream_t)stream;
    if (tof) {
        TofParams tp;
        if ((rc = check_tof(tof, n, tof_stride, tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
        return launch_osem<true>(lors, n, lor_stride, tof, tof_stride, g, tp, y, add, ratio_rule, eps, vx, vxt, vbp, vbpt, loglik, s);
    }
    TofParams tp{0, 0, 0};
    return launch_osem<false>(lors, n, lor_stride, nullptr, 1, g, tp, y, add, ratio_rule, eps, vx, vxt, vbp, vbpt, loglik, s);
}

int srf_osem_update(float *x, float *x_t, float *bp, float *bp_t, const float *emap,
                    int32_t guard_zero, const int32_t grid[3], void *stream) {
    if (!x || !bp || !emap) return fail(SRF_EINVAL, "x, bp and emap must not be NULL");
    if (!grid) return fail(SRF_EINVAL, "grid must not be NULL");
    Grid g; int rc;
    const float c[3] = {0, 0, 0}, sz[3] = {1, 1, 1};
    if ((rc = check_geometry(grid, c, sz, g))) return rc;
    dim3 blocks((g.nx + kTile - 1) / kTile, (g.ny + kTile - 1) / kTile, g.nz);
    auto a16 = [](const void *p) { return ((uintptr_t)p & 15) == 0; };
    if (g.nx % 4 == 0 && g.ny % 4 == 0 && a16(x) && a16(x_t) && a16(bp) && a16(bp_t) && a16(emap))
        k_osem_update4<<<blocks, kTile * 8, 0, (cudaStream_t)stream>>>(x, x_t, bp, bp_t, emap, guard_zero, g.nx, g.ny);
    else
        k_osem_update<<<blocks, dim3(kTile, 8), 0, (cudaStream_t)stream>>>(x, x_t, bp, bp_t, emap, guard_zero, g.nx, g.ny);
    return check_cuda("osem update kernel launch");
}

}  // extern "C"
