// Siddon-style slab traversal for sm_103a: one LOR per group of G lanes, slabs spread over lanes.
//
// Semantics follow srfnef's four device functions (srfnef/cc/siddon/siddon.cu.cc:12-656 and
// srfnef/cc/siddon_tof/siddon_tof.cu.cc:14-707): for every slab of the dominant transaxial axis
// the entry/exit coordinates of the other two axes are floored to voxel indices and the slab's
// weight is split among at most three voxels by the crossing fractions. The rule sets differ as
//
//   rule                       proj non-TOF          proj TOF                back (both)
//   LOR skip transaxial < 10   siddon.cu.cc:34       siddon_tof.cu.cc:37     siddon.cu.cc:364, siddon_tof.cu.cc:395
//   LOR skip steep (> 45 deg)  siddon.cu.cc:38       -                       -
//   x dominant when            |xd| >= |yd| (:46)    |xd| > |yd| (:48)       |xd| > |yd| (:372, :405)
//   slab skip                  past endpoint 2       before endpoint 1       none
//                              (:56-57, :203-204)    (:67-74, :228-235)
//   weight                     frac*sqrt(1+k^2+kz^2)*dx_/L/L (:94)           frac*sqrt(..)*dx_ (:418)
//   TOF factor                 -                     Gaussian (:43-59)       Gaussian (:402-416)
//
// GB300 design (not the reference's thread-per-LOR loop over every slab):
//  * G lanes share a LOR; lane l takes slabs lo+l, lo+l+G, ... so consecutive lanes touch
//    consecutive voxels of the primary axis. With an image whose primary axis is the fastest one
//    (x-fastest for x-dominant LORs, an optional y-fastest copy for y-dominant LORs) a group's
//    gathers and reductions land in one or two 128-byte lines instead of G lines.
//  * the slab range is clipped per LOR to the slabs that can touch the image box, to the
//    projector's endpoint rule and (when enabled) to the TOF window; the exact per-slab
//    predicates are still evaluated, so the clip only removes slabs that contribute nothing.
//  * coordinates that feed floor() and the skip predicates are computed with round-to-nearest
//    intrinsics in the reference's operand order (no FMA contraction, IEEE division), so voxel
//    choices equal the reference's; weights and the TOF exponential use fast FP32 forms.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace srf {

enum Rules : int { RULES_PROJ = 0, RULES_BACK = 1 };

struct Grid {
    int nx, ny, nz;
    float cx, cy, cz;
    float sx, sy, sz;
};

// An image view: base pointer and element strides of the x, y and z axes.
struct View {
    float *ptr;
    int64_t st[3];
};

struct TofParams {
    float tof_bin;     // mm
    float tof_sigma2;  // mm^2
    float nsigma;      // 0 = reference-exact (no truncation)
};

// Everything one LOR needs for its slab loop.
struct LorSetup {
    int lo, hi;        // inclusive slab range (empty when lo > hi)
    int np, nq, nz;    // extents along primary, in-plane secondary, axial
    float p1, p2, q1, z1;
    float kq, kz;
    float dq, dz;      // divisors of the secondary/axial coordinates (dq = 1 for the y branch)
    float np2, nq2, nz2;
    float wc;          // sqrt(1+kq^2+kz^2)*dx_ (/L/L for the projector)
    // TOF
    float L, ratio1, dpc, pd, tof_amp, expand, nsig2;
    int np_half;
    // memory
    int32_t sp, sq, szs;
    int xdom;
};

__device__ __forceinline__ float absr(float v) { return v < 0 ? -v : v; }

// (a + k*(pp - p1)) / d + n2 in the reference's rounding order
__device__ __forceinline__ float bcoord(float a, float k, float pp, float p1, float d, float n2, bool d_is_one) {
    float t = __fadd_rn(a, __fmul_rn(k, __fsub_rn(pp, p1)));
    if (!d_is_one) t = __fdiv_rn(t, d);
    return __fadd_rn(t, n2);
}

// floor(x) as int, saturating like the hardware conversion
__device__ __forceinline__ int ifloor(float x) { return __float2int_rd(x); }

__device__ __forceinline__ void clip_linear(float A, float B, float lo_v, float hi_v, float np2,
                                            int &lo, int &hi) {
    // keep slabs ip whose coordinate A + B*pp (pp in [ip-np2, ip-np2+1]) can lie in [lo_v, hi_v]
    if (fabsf(B) < 1e-6f) {
        if (!(A >= lo_v - 1.0f && A <= hi_v + 1.0f)) { lo = 1; hi = 0; }
        return;
    }
    float a = (lo_v - A) / B, b = (hi_v - A) / B;
    float ppl = fminf(a, b), pph = fmaxf(a, b);
    // ppl, pph are finite here unless A is non-finite; NaN compares false and keeps the range
    float fl = floorf(ppl + np2) - 2.0f, fh = ceilf(pph + np2) + 1.0f;
    if (fl > (float)lo) lo = (fl > 2.0e9f) ? 0x7fffffff : (int)fl;
    if (fh < (float)hi) hi = (fh < -2.0e9f) ? -0x7fffffff : (int)fh;
}

// Per-LOR setup. Returns false when the LOR is skipped entirely (or non-finite).
template <bool TOF, int RULES>
__device__ __forceinline__ bool setup_lor(float x1_, float y1_, float z1_, float x2_, float y2_,
                                          float z2_, float tof_value, const Grid &g,
                                          const TofParams &tp, const int64_t stx[3],
                                          const int64_t sty[3], bool have_t, LorSetup &S) {
    const bool proj = (RULES == RULES_PROJ);
    const float dx_ = __fdiv_rn(g.sx, (float)g.nx);
    const float dy = __fdiv_rn(__fdiv_rn(g.sy, (float)g.ny), dx_);
    const float dz = __fdiv_rn(__fdiv_rn(g.sz, (float)g.nz), dx_);
    const float x1 = __fdiv_rn(__fsub_rn(x1_, g.cx), dx_);
    const float x2 = __fdiv_rn(__fsub_rn(x2_, g.cx), dx_);
    const float y1 = __fdiv_rn(__fsub_rn(y1_, g.cy), dx_);
    const float y2 = __fdiv_rn(__fsub_rn(y2_, g.cy), dx_);
    const float z1 = __fdiv_rn(__fsub_rn(z1_, g.cz), dx_);
    const float z2 = __fdiv_rn(__fsub_rn(z2_, g.cz), dx_);
    const float xd = __fsub_rn(x2, x1), yd = __fsub_rn(y2, y1), zd = __fsub_rn(z2, z1);
    const float t2d = __fadd_rn(__fmul_rn(xd, xd), __fmul_rn(yd, yd));
    if (!(isfinite(t2d) && isfinite(zd))) return false;
    if (TOF && !isfinite(tof_value)) return false;
    const float rt = __fsqrt_rn(t2d);
    if (rt < 10.0f) return false;
    if (proj && !TOF && rt < absr(zd)) return false;
    const float L = __fsqrt_rn(__fadd_rn(t2d, __fmul_rn(zd, zd)));

    const bool xdom = (proj && !TOF) ? (absr(xd) >= absr(yd)) : (absr(xd) > absr(yd));
    S.xdom = xdom;
    S.np = xdom ? g.nx : g.ny;
    S.nq = xdom ? g.ny : g.nx;
    S.nz = g.nz;
    S.p1 = xdom ? x1 : y1;
    S.p2 = xdom ? x2 : y2;
    S.q1 = xdom ? y1 : x1;
    S.z1 = z1;
    const float pd = xdom ? xd : yd;
    S.kq = __fdiv_rn(xdom ? yd : xd, pd);
    S.kz = __fdiv_rn(zd, pd);
    S.dq = xdom ? dy : 1.0f;
    S.dz = dz;
    S.np2 = __fdiv_rn((float)S.np, 2.0f);
    S.nq2 = __fdiv_rn((float)S.nq, 2.0f);
    S.nz2 = __fdiv_rn((float)g.nz, 2.0f);
    float wc = sqrtf(1.0f + S.kq * S.kq + S.kz * S.kz) * dx_;
    if (proj) wc = wc / L / L;
    S.wc = wc;
    S.L = L;

    // memory strides of the view this LOR reads or writes
    const int64_t *st = (!xdom && have_t) ? sty : stx;
    S.sp = (int32_t)(xdom ? st[0] : st[1]);
    S.sq = (int32_t)(xdom ? st[1] : st[0]);
    S.szs = (int32_t)st[2];

    int lo = 0, hi = S.np - 1;
    // image box in the secondary and axial directions
    clip_linear(__fadd_rn(__fdiv_rn(__fsub_rn(S.q1, __fmul_rn(S.kq, S.p1)), S.dq), S.nq2),
                S.kq / S.dq, -1.0f, (float)S.nq + 1.0f, S.np2, lo, hi);
    clip_linear(__fadd_rn(__fdiv_rn(__fsub_rn(S.z1, __fmul_rn(S.kz, S.p1)), S.dz), S.nz2),
                S.kz / S.dz, -1.0f, (float)S.nz + 1.0f, S.np2, lo, hi);
    // projector endpoint rules: keep a prefix or a suffix of the slabs (pp = ip - np2)
    if (proj) {
        if (!TOF) {
            if (S.p1 < S.p2) { float f = floorf(S.p2 + S.np2) + 1.0f; if (f < (float)hi) hi = (int)fmaxf(f, -1.0f); }
            else             { float f = floorf(S.p2 + S.np2) - 1.0f; if (f > (float)lo) lo = (int)fminf(f, (float)S.np); }
        } else {
            if (S.p2 > S.p1)      { float f = floorf(S.p1 + S.np2) - 1.0f; if (f > (float)lo) lo = (int)fminf(f, (float)S.np); }
            else if (S.p2 < S.p1) { float f = floorf(S.p1 + S.np2) + 1.0f; if (f < (float)hi) hi = (int)fmaxf(f, -1.0f); }
        }
    }
    if (TOF) {
        const float tof_bin_ = __fdiv_rn(tp.tof_bin, dx_);
        const float tof_sigma2_ = __fdiv_rn(__fdiv_rn(tp.tof_sigma2, dx_), dx_);
        const float expand = __fadd_rn(tof_sigma2_, __fdiv_rn(__fmul_rn(tof_bin_, tof_bin_), 12.0f));
        // ratio1 = (1.0 - tof/dx_/L) / 2 evaluated in double as in the reference, then rounded
        const float tl = __fdiv_rn(__fdiv_rn(tof_value, dx_), L);
        S.ratio1 = (float)((1.0 - (double)tl) * 0.5);
        S.dpc = xdom ? 1.0f : dy;
        S.np_half = S.np / 2;
        S.pd = __fsub_rn(S.p2, S.p1);
        S.tof_amp = tof_bin_ * rsqrtf(2.0f * 3.1415926f * expand);
        S.expand = expand;
        S.nsig2 = tp.nsigma * tp.nsigma;
        if (tp.nsigma > 0.0f) {
            // |((pc - p1)/(p2-p1) - ratio1) * L| <= nsigma*sqrt(expand), pc = (ip - np/2 + 0.5)*dpc
            const float w = tp.nsigma * sqrtf(expand) / L;
            const float pa = S.p1 + (S.ratio1 - w) * S.pd;
            const float pb = S.p1 + (S.ratio1 + w) * S.pd;
            const float ia = pa / S.dpc + (float)S.np_half - 0.5f;
            const float ib = pb / S.dpc + (float)S.np_half - 0.5f;
            const float fl = floorf(fminf(ia, ib)) - 2.0f, fh = ceilf(fmaxf(ia, ib)) + 2.0f;
            if (fl > (float)lo) lo = (int)fminf(fl, (float)S.np);
            if (fh < (float)hi) hi = (int)fmaxf(fh, -1.0f);
        }
    }
    S.lo = max(lo, 0);
    S.hi = min(hi, S.np - 1);
    return S.lo <= S.hi;
}

// One slab: computes up to three (offset, weight) visits and applies `visit(off, w)`.
template <bool TOF, int RULES, typename F>
__device__ __forceinline__ void slab(const LorSetup &S, int ip, F &&visit) {
    const bool proj = (RULES == RULES_PROJ);
    float w_tof = 1.0f;
    if (TOF) {
        const float pc = __fmul_rn(__fadd_rn((float)(ip - S.np_half), 0.5f), S.dpc);
        const float d2 = __fmul_rn(__fsub_rn(__fdiv_rn(__fsub_rn(pc, S.p1), S.pd), S.ratio1), S.L);
        const float t2 = __fdiv_rn(__fmul_rn(d2, d2), S.expand);
        if (S.nsig2 > 0.0f && t2 > S.nsig2) return;
        w_tof = S.tof_amp * __expf(-0.5f * t2);
    }
    const float pp1 = __fsub_rn((float)ip, S.np2);
    const float pp2 = __fadd_rn(pp1, 1.0f);
    if (proj) {
        if (!TOF) {
            if (S.p1 < S.p2 && pp2 > S.p2) return;
            if (S.p1 >= S.p2 && pp1 < S.p2) return;
        } else if (S.xdom) {
            if (S.p2 > S.p1 && pp1 <= S.p1) return;
            if (S.p2 < S.p1 && pp2 >= S.p1) return;
        } else {
            if (S.p2 > S.p1 && pp1 < S.p1) return;
            if (S.p2 < S.p1 && pp2 > S.p1) return;
        }
    }
    const bool q_one = (S.dq == 1.0f);
    const float qa = bcoord(S.q1, S.kq, pp1, S.p1, S.dq, S.nq2, q_one);
    const float qb = bcoord(S.q1, S.kq, pp2, S.p1, S.dq, S.nq2, q_one);
    const float za = bcoord(S.z1, S.kz, pp1, S.p1, S.dz, S.nz2, false);
    const float zb = bcoord(S.z1, S.kz, pp2, S.p1, S.dz, S.nz2, false);
    const float qq1 = (S.kq >= 0.0f) ? qa : qb, qq2 = (S.kq >= 0.0f) ? qb : qa;
    const float zz1 = (S.kz >= 0.0f) ? za : zb, zz2 = (S.kz >= 0.0f) ? zb : za;
    const int cq1 = ifloor(qq1), cq2 = ifloor(qq2);
    const int cz1 = ifloor(zz1), cz2 = ifloor(zz2);
    const int nq = S.nq, nz = S.nz;
    const int32_t base = ip * S.sp;
    const float wt = S.wc * w_tof;
#define SRF_V(cq, cz, frac) visit(base + (cq) * S.sq + (cz) * S.szs, (frac) * wt)
    if (cq1 == cq2) {
        if (0 <= cq1 && cq1 < nq) {
            if (cz1 == cz2) {
                if (0 <= cz1 && cz1 < nz) SRF_V(cq1, cz1, 1.0f);
            } else if (-1 <= cz1 && cz1 < nz) {
                const float rz = ((float)cz2 - zz1) / (zz2 - zz1);
                if (cz1 >= 0) SRF_V(cq1, cz1, rz);
                if (cz2 < nz) SRF_V(cq1, cz2, 1.0f - rz);
            }
        }
    } else if (-1 <= cq1 && cq1 < nq) {
        if (cz1 == cz2) {
            if (0 <= cz1 && cz1 < nz) {
                const float rq = ((float)cq2 - qq1) / (qq2 - qq1);
                if (cq1 >= 0) SRF_V(cq1, cz1, rq);
                if (cq2 < nq) SRF_V(cq2, cz1, 1.0f - rq);
            }
        } else if (-1 <= cz1 && cz1 < nz) {
            const float rq = ((float)cq2 - qq1) / (qq2 - qq1);
            const float rz = ((float)cz2 - zz1) / (zz2 - zz1);
            if (rq > rz) {
                if (cq1 >= 0 && cz1 >= 0) SRF_V(cq1, cz1, rz);
                if (cq1 >= 0 && cz2 < nz) SRF_V(cq1, cz2, rq - rz);
                if (cq2 < nq && cz2 < nz) SRF_V(cq2, cz2, 1.0f - rq);
            } else {
                if (cq1 >= 0 && cz1 >= 0) SRF_V(cq1, cz1, rq);
                if (cq2 < nq && cz1 >= 0) SRF_V(cq2, cz1, rz - rq);
                if (cq2 < nq && cz2 < nz) SRF_V(cq2, cz2, 1.0f - rz);
            }
        }
    }
#undef SRF_V
}

// Lanes of this thread's group of G (G a power of two <= 32, groups aligned within the warp).
template <int G>
__device__ __forceinline__ unsigned group_mask() {
    if constexpr (G == 32) return 0xffffffffu;
    else return ((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1));
}

// Sum over a group of G lanes. Only the group's own lanes take part, so groups of one warp may
// call it from different places.
template <int G>
__device__ __forceinline__ float group_sum(float v) {
    const unsigned m = group_mask<G>();
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o, G);
    return v;
}

}  // namespace srf
