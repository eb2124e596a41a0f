// Per-LOR setup of the fused traversal (the list-mode MLEM/OSEM subset step and the standalone
// projector / backprojector built on it), organised for the GB300 memory system:
//
//  * LOR setup is lane-parallel: each lane of a warp prepares one of the warp's next 32 LORs
//    (endpoint scaling, skip rules, dominant axis, slab range clipped to the image box and TOF
//    window, the projector's endpoint slab range) into a record in shared memory, instead of
//    every lane of a group repeating the same setup. The group then walks the records one LOR
//    at a time (lean.cuh: the slab loop).
//  * one setup serves both passes: the projector and backprojector share the traversal (same
//    dominant axis except at |xd| == |yd| for non-TOF, which takes the generic path), and differ
//    only in the projector's endpoint slab rule, its LOR-level steep rule (non-TOF) and its 1/L^2.
//  * every value that decides a skip rule, the dominant axis or the projector's slab range is
//    computed with round-to-nearest intrinsics in the reference's operand order, in FP32 (FP64
//    issues at a small fraction of the FP32 rate on this part).
#pragma once
#include "siddon.cuh"

namespace srf {

// Per-LOR setup (setup_rec, one lane per LOR): endpoints in voxel units, skip rules, dominant
// axis, slab range, the projector's endpoint slab range and the linear forms of the boundary
// coordinates; make_lean (lean.cuh) derives the slab loop's record from it.
struct LorRec {
    float p1, p2, q1, z1;
    float kq, kz, wc, invL2;     // wc includes the TOF amplitude
    float ratio1, L, yv, pd;
    float Aq, Bq, Az, Bz;        // boundary(pp) ~= B pp + A, pp = ip - np/2
    float invq, invz, ad;        // invq, invz: 1 / (boundary step per slab) of q and z; ad: additive term
    int lo, hi, flags, pmlo;     // [pmlo, pmhi]: slabs the projector's endpoint rule keeps
    int pmhi;
};
constexpr int F_VALID = 1, F_PROJ = 2, F_XDOM = 4, F_TIE = 8;

// grid-wide constants, rounded exactly as in setup_lor
struct GridK {
    float dx_, dy, dz, nx2, ny2, nz2;
    float tof_bin_, expand, inv_expand, tof_amp, nsig2, nsw;  // nsw = nsigma * sqrt(expand)
    float k2;  // TOF exponent in log2 units: d^2 k2 = -t2 log2(e) / 2
    bool dy_one;
};

constexpr float kHalfLog2e = 0.72134752044448170f;  // log2(e) / 2: exp(-t2 / 2) = exp2(-t2 * this)

template <bool TOF>
__device__ __forceinline__ GridK make_gridk(const Grid &g, const TofParams &tp) {
    GridK k;
    k.dx_ = __fdiv_rn(g.sx, (float)g.nx);
    k.dy = __fdiv_rn(__fdiv_rn(g.sy, (float)g.ny), k.dx_);
    k.dz = __fdiv_rn(__fdiv_rn(g.sz, (float)g.nz), k.dx_);
    k.nx2 = __fdiv_rn((float)g.nx, 2.0f);
    k.ny2 = __fdiv_rn((float)g.ny, 2.0f);
    k.nz2 = __fdiv_rn((float)g.nz, 2.0f);
    k.dy_one = (k.dy == 1.0f);
    k.tof_bin_ = k.expand = k.inv_expand = k.tof_amp = k.nsig2 = k.nsw = 0.0f;
    k.k2 = 0.0f;
    if (TOF) {
        k.tof_bin_ = __fdiv_rn(tp.tof_bin, k.dx_);
        const float s2 = __fdiv_rn(__fdiv_rn(tp.tof_sigma2, k.dx_), k.dx_);
        k.expand = __fadd_rn(s2, __fdiv_rn(__fmul_rn(k.tof_bin_, k.tof_bin_), 12.0f));
        k.inv_expand = 1.0f / k.expand;
        k.tof_amp = k.tof_bin_ * rsqrtf(2.0f * 3.1415926f * k.expand);
        k.nsig2 = tp.nsigma * tp.nsigma;
        k.nsw = tp.nsigma * sqrtf(k.expand);
        k.k2 = -kHalfLog2e * k.inv_expand;
    }
    return k;
}

// The projector's endpoint slab rule at slab ip (pp1 = ip - np/2, pp2 = pp1 + 1, both exact):
// non-TOF keeps slabs up to endpoint 2 (siddon.cu.cc:56-57), TOF keeps slabs from endpoint 1 on
// (siddon_tof.cu.cc:68-75 for x, :228-235 for y, with their different strictness).
__device__ __forceinline__ bool proj_rule_at(float p1, float p2, bool xdom, bool tof, int ip, float np2) {
    const float pp1 = __fsub_rn((float)ip, np2);
    const float pp2 = __fadd_rn(pp1, 1.0f);
    if (!tof) return !((p1 < p2 && pp2 > p2) || (p1 >= p2 && pp1 < p2));
    if (xdom) return !((p2 > p1 && pp1 <= p1) || (p2 < p1 && pp2 >= p1));
    return !((p2 > p1 && pp1 < p1) || (p2 < p1 && pp2 > p1));
}

// The rule keeps a contiguous slab range [pmlo, pmhi] (one side open): the bound is estimated
// (within a slab) and then settled with the float predicate itself, so the range is exactly the
// rule's. Single precision throughout: FP64 issues at a small fraction of the FP32 rate here.
__device__ __forceinline__ void proj_slab_range(float p1, float p2, bool xdom, bool tof, float np2, int np,
                                                int &pmlo, int &pmhi) {
    pmlo = -2;
    pmhi = np + 1;
    const float a1 = p1 + np2, a2 = p2 + np2;
    int upper = 0;  // +1: rule keeps ip <= bound; -1: keeps ip >= bound; 0: keeps every slab
    float est = 0.0f;
    if (!tof) {
        if (p1 < p2) { upper = 1; est = floorf(a2 - 1.0f); } else { upper = -1; est = ceilf(a2); }
    } else if (p2 > p1) {
        upper = -1; est = xdom ? floorf(a1) + 1.0f : ceilf(a1);
    } else if (p2 < p1) {
        upper = 1; est = xdom ? ceilf(a1 - 1.0f) - 1.0f : floorf(a1 - 1.0f);
    }
    if (upper == 0) return;
    int b = (int)fminf(fmaxf(est, -2.0f), (float)np + 1.0f);
    if (upper > 0) {
        for (int t = 0; t < 4 && b < np + 1 && proj_rule_at(p1, p2, xdom, tof, b + 1, np2); ++t) ++b;
        for (int t = 0; t < 4 && b > -2 && !proj_rule_at(p1, p2, xdom, tof, b, np2); ++t) --b;
        pmhi = b;
    } else {
        for (int t = 0; t < 4 && b > -2 && proj_rule_at(p1, p2, xdom, tof, b - 1, np2); ++t) --b;
        for (int t = 0; t < 4 && b < np + 1 && !proj_rule_at(p1, p2, xdom, tof, b, np2); ++t) ++b;
        pmlo = b;
    }
}

// Lane-parallel setup of one LOR (both rule sets). Rounding of every value that feeds a floor or
// a skip predicate follows setup_lor.
template <bool TOF>
__device__ __forceinline__ LorRec setup_rec(const float *l, float tv, float yv, const Grid &g,
                                            const GridK &k) {
    LorRec R = {};
    R.flags = 0;
    R.lo = 1;
    R.hi = 0;
    R.yv = yv;
    const float x1 = __fdiv_rn(__fsub_rn(l[0], g.cx), k.dx_);
    const float y1 = __fdiv_rn(__fsub_rn(l[1], g.cy), k.dx_);
    const float z1 = __fdiv_rn(__fsub_rn(l[2], g.cz), k.dx_);
    const float x2 = __fdiv_rn(__fsub_rn(l[3], g.cx), k.dx_);
    const float y2 = __fdiv_rn(__fsub_rn(l[4], g.cy), k.dx_);
    const float z2 = __fdiv_rn(__fsub_rn(l[5], g.cz), k.dx_);
    const float xd = __fsub_rn(x2, x1), yd = __fsub_rn(y2, y1), zd = __fsub_rn(z2, z1);
    const float t2d = __fadd_rn(__fmul_rn(xd, xd), __fmul_rn(yd, yd));
    if (!(isfinite(t2d) && isfinite(zd)) || (TOF && !isfinite(tv))) return R;
    const float rt = __fsqrt_rn(t2d);
    if (rt < 10.0f) return R;
    const bool proj_ok = TOF || !(rt < absr(zd));
    const bool xdom = absr(xd) > absr(yd);          // backprojector (and TOF projector) rule
    const bool xdom_p = TOF ? xdom : (absr(xd) >= absr(yd));
    const float L = __fsqrt_rn(__fadd_rn(t2d, __fmul_rn(zd, zd)));
    R.p1 = xdom ? x1 : y1;
    R.p2 = xdom ? x2 : y2;
    R.q1 = xdom ? y1 : x1;
    R.z1 = z1;
    const float pd = xdom ? xd : yd;
    R.kq = __fdiv_rn(xdom ? yd : xd, pd);
    R.kz = __fdiv_rn(zd, pd);
    R.wc = sqrtf(1.0f + R.kq * R.kq + R.kz * R.kz) * k.dx_;
    R.invL2 = 1.0f / (L * L);
    R.L = L;
    R.ratio1 = 0.0f;
    R.flags = F_VALID | (proj_ok ? F_PROJ : 0) | (xdom ? F_XDOM : 0) | (xdom != xdom_p ? F_TIE : 0);
    const int np = xdom ? g.nx : g.ny, nq = xdom ? g.ny : g.nx;
    const float np2 = xdom ? k.nx2 : k.ny2, nq2 = xdom ? k.ny2 : k.nx2;
    const float dq = xdom ? k.dy : 1.0f;
    int lo = 0, hi = np - 1;
    clip_linear(__fadd_rn(__fdiv_rn(__fsub_rn(R.q1, __fmul_rn(R.kq, R.p1)), dq), nq2), R.kq / dq,
                -1.0f, (float)nq + 1.0f, np2, lo, hi);
    clip_linear(__fadd_rn(__fdiv_rn(__fsub_rn(z1, __fmul_rn(R.kz, R.p1)), k.dz), k.nz2),
                R.kz / k.dz, -1.0f, (float)g.nz + 1.0f, np2, lo, hi);
    if (TOF) {
        const float tl = __fdiv_rn(__fdiv_rn(tv, k.dx_), L);
        // the reference's (1.0 - tl) / 2 in double: 1 - tl is exact there and halving is exact,
        // so its one rounding to float is RN(1 - tl) / 2, which FP32 computes bit for bit
        R.ratio1 = __fmul_rn(__fsub_rn(1.0f, tl), 0.5f);
        if (k.nsig2 > 0.0f) {
            const float dpc = xdom ? 1.0f : k.dy;
            const float w = k.nsw / L;
            const float pa = R.p1 + (R.ratio1 - w) * pd;
            const float pb = R.p1 + (R.ratio1 + w) * pd;
            const float ia = pa / dpc + (float)(np / 2) - 0.5f;
            const float ib = pb / dpc + (float)(np / 2) - 0.5f;
            const float fl = floorf(fminf(ia, ib)) - 2.0f, fh = ceilf(fmaxf(ia, ib)) + 2.0f;
            if (fl > (float)lo) lo = (int)fminf(fl, (float)np);
            if (fh < (float)hi) hi = (int)fmaxf(fh, -1.0f);
        }
    }
    R.lo = max(lo, 0);
    R.hi = min(hi, np - 1);
    if (R.lo > R.hi && !(R.flags & F_TIE)) R.flags = 0;
    // linear forms of the boundary coordinates
    R.pd = pd;
    R.Bq = R.kq / dq;
    R.Aq = (R.q1 - R.kq * R.p1) / dq + nq2;
    R.Bz = R.kz / k.dz;
    R.Az = (z1 - R.kz * R.p1) / k.dz + k.nz2;
    R.invq = 1.0f / fabsf(R.Bq);  // inf when q never steps (then unused)
    R.invz = 1.0f / fabsf(R.Bz);
    if (TOF) R.wc *= k.tof_amp;
    proj_slab_range(R.p1, R.p2, xdom, TOF, np2, np, R.pmlo, R.pmhi);
    return R;
}

// The standalone projector / backprojector on the fused kernel's traversal (osem.cu). tof == NULL
// selects the non-TOF rules. Views with equal strides for the two layouts (v x-fastest, vt the
// optional y-fastest copy).
int fused_projection(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                     const Grid &g, const TofParams &tp, const View &v, const View &vt, float *out,
                     cudaStream_t s);
int fused_backprojection(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                         const Grid &g, const TofParams &tp, const float *values, const View &v,
                         const View &vt, cudaStream_t s);
// Block-full sensitivity image: backprojection of 1 along every ordered pair of table rows.
int fused_emap(const float *table, int nb, int m, const Grid &g, const View &v, const View &vt, cudaStream_t s);
// The projector and its exact adjoint for nb <= 8 images at element offsets b * bstride.
int fused_projection_batch(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                           const Grid &g, const TofParams &tp, int nb, int64_t bstride, const View &v,
                           const View &vt, float *out, int64_t ostride, cudaStream_t s);
int fused_adjoint_batch(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                        const Grid &g, const TofParams &tp, int nb, int64_t bstride, const float *values,
                        int64_t vstride, const View &v, const View &vt, cudaStream_t s);

}  // namespace srf
