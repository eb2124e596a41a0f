// Fused projection -> ratio -> backprojection for a batch of LORs (the list-mode MLEM/OSEM subset
// step), organised for the GB300 memory system:
//
//  * LOR setup is lane-parallel: each lane of a warp prepares one of the warp's next 32 LORs
//    (endpoint scaling, skip rules, dominant axis, slab range clipped to the image box and TOF
//    window) into a shared-memory record, instead of every lane of a group repeating the same
//    setup. The group then walks the records one LOR at a time.
//  * one setup serves both passes: the projector and backprojector share the traversal (same
//    dominant axis except at |xd| == |yd| for non-TOF, which takes the generic path), and differ
//    only in the projector's endpoint slab rule, its LOR-level steep rule (non-TOF) and its 1/L^2.
//  * a slab's voxel candidates are computed branch-free (three offsets and weights, weight 0 when
//    a voxel is not visited), U slabs per lane at a time, so a lane issues up to 3U independent
//    gathers before it consumes any of them.
//  * when a LOR's slab range fits in one chunk of G*U slabs (the usual case with a truncated TOF
//    kernel) the candidates stay in registers and the backprojection reuses them directly.
#pragma once
#include "siddon.cuh"

namespace srf {

// Per-LOR record in shared memory: everything the slab loop needs, computed once per LOR by one
// lane (setup_rec) and read by the LOR's group as seven 16-byte broadcasts.
struct __align__(16) LorRec {
    float p1, p2, q1, z1;
    float kq, kz, wc, invL2;     // wc includes the TOF amplitude
    float ratio1, L, yv, pd;
    float tA, Aq, Bq, Az;        // fast forms: boundary(pp) ~= fmaf(B, pp, A); TOF d(ip) ~= fmaf(tA, ip, tB)
    float Bz, mq, mz, ad;        // mq, mz: floor margins of the fast forms; ad: additive term
    int lo, hi, flags, pmlo;     // [pmlo, pmhi]: slabs the projector's endpoint rule keeps
    int pmhi;
    float tB, invq, invz;        // invq, invz: 1 / (boundary step per slab) of q and z
};
constexpr int F_VALID = 1, F_PROJ = 2, F_XDOM = 4, F_TIE = 8;
constexpr int kRecVec = sizeof(LorRec) / 16;
static_assert(sizeof(LorRec) == 112, "LorRec is seven 16-byte vectors");

__device__ __forceinline__ LorRec load_rec(const LorRec *src) {
    LorRec R;
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    float4 *d4 = reinterpret_cast<float4 *>(&R);
#pragma unroll
    for (int c = 0; c < kRecVec; ++c) d4[c] = s4[c];
    return R;
}

__device__ __forceinline__ void store_rec(LorRec *dst, const LorRec &R) {
    const float4 *s4 = reinterpret_cast<const float4 *>(&R);
    float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll
    for (int c = 0; c < kRecVec; ++c) d4[c] = s4[c];
}

// Relative margin on the TOF truncation test t2 <= nsigma^2 (fast t2 is within ~1e-5 relative).
constexpr float kTruncMargin = 2e-4f;

// grid-wide constants, rounded exactly as in setup_lor
struct GridK {
    float dx_, dy, dz, nx2, ny2, nz2;
    float tof_bin_, expand, inv_expand, tof_amp, nsig2, nsw;  // nsw = nsigma * sqrt(expand)
    float k2, e2cut, e2tol;  // fast TOF: e2 = d^2 k2 = -t2 log2(e) / 2; kept when e2 >= e2cut
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
    k.k2 = k.e2cut = k.e2tol = 0.0f;
    if (TOF) {
        k.tof_bin_ = __fdiv_rn(tp.tof_bin, k.dx_);
        const float s2 = __fdiv_rn(__fdiv_rn(tp.tof_sigma2, k.dx_), k.dx_);
        k.expand = __fadd_rn(s2, __fdiv_rn(__fmul_rn(k.tof_bin_, k.tof_bin_), 12.0f));
        k.inv_expand = 1.0f / k.expand;
        k.tof_amp = k.tof_bin_ * rsqrtf(2.0f * 3.1415926f * k.expand);
        k.nsig2 = tp.nsigma * tp.nsigma;
        k.nsw = tp.nsigma * sqrtf(k.expand);
        k.k2 = -kHalfLog2e * k.inv_expand;
        k.e2cut = -kHalfLog2e * k.nsig2;
        k.e2tol = kTruncMargin * kHalfLog2e * k.nsig2;
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
    // fast forms of the boundary coordinates and their floor margins: both the fast form and the
    // reference's operand sequence are within a few units of 2^-24 * S of the exact value,
    // S = (|k| (|p1| + np) + |a|) / d + |n2| + 2 over the LOR's slabs; 2^-20 * S bounds their
    // difference with room to spare.
    R.pd = pd;
    R.Bq = R.kq / dq;
    R.Aq = (R.q1 - R.kq * R.p1) / dq + nq2;
    R.Bz = R.kz / k.dz;
    R.Az = (z1 - R.kz * R.p1) / k.dz + k.nz2;
    R.invq = 1.0f / fabsf(R.Bq);  // inf when q never steps (then unused)
    R.invz = 1.0f / fabsf(R.Bz);
    const float e = 9.5367431640625e-7f;  // 2^-20
    R.mq = e * ((fabsf(R.kq) * (fabsf(R.p1) + (float)np) + fabsf(R.q1)) / dq + nq2 + 2.0f);
    R.mz = e * ((fabsf(R.kz) * (fabsf(R.p1) + (float)np) + fabsf(z1)) / k.dz + k.nz2 + 2.0f);
    R.tA = R.tB = 0.0f;
    if (TOF) {
        // d(ip) = ((pc(ip) - p1) / pd - ratio1) L with pc = (ip - np/2 + 0.5) dpc, linear in ip
        const float dpc = xdom ? 1.0f : k.dy;
        const float ipd = 1.0f / pd;
        R.tA = dpc * ipd * L;
        R.tB = (((0.5f - (float)(np / 2)) * dpc - R.p1) * ipd - R.ratio1) * L;
        R.wc *= k.tof_amp;
    }
    proj_slab_range(R.p1, R.p2, xdom, TOF, np2, np, R.pmlo, R.pmhi);
    return R;
}

// Per-LOR constants of the slab loop: the record plus the axis-dependent grid values.
struct LorRun {
    float p1, p2, q1, z1, kq, kz, wc, pd, ratio1, L;
    float np2, nq2, dq, dpc;
    float Aq, Bq, Az, Bz, mq, mz, tA, tB, invq, invz;
    int np, nq, nz, np_half, lo, hi, pmlo, pmhi;
    int32_t sp, sq, szs;
    bool xdom, dq_one;
};

__device__ __forceinline__ LorRun make_run(const LorRec &R, const Grid &g, const GridK &k,
                                           const int64_t stx[3], const int64_t sty[3],
                                           bool have_t) {
    LorRun r;
    r.xdom = R.flags & F_XDOM;
    r.p1 = R.p1; r.p2 = R.p2; r.q1 = R.q1; r.z1 = R.z1; r.kq = R.kq; r.kz = R.kz; r.wc = R.wc;
    r.pd = R.pd;
    r.ratio1 = R.ratio1;
    r.L = R.L;
    r.Aq = R.Aq; r.Bq = R.Bq; r.Az = R.Az; r.Bz = R.Bz; r.mq = R.mq; r.mz = R.mz;
    r.tA = R.tA; r.tB = R.tB; r.invq = R.invq; r.invz = R.invz; r.pmlo = R.pmlo; r.pmhi = R.pmhi;
    r.np = r.xdom ? g.nx : g.ny;
    r.nq = r.xdom ? g.ny : g.nx;
    r.nz = g.nz;
    r.np2 = r.xdom ? k.nx2 : k.ny2;
    r.nq2 = r.xdom ? k.ny2 : k.nx2;
    r.dq = r.xdom ? k.dy : 1.0f;
    r.dq_one = r.xdom ? k.dy_one : true;
    r.dpc = r.xdom ? 1.0f : k.dy;
    r.np_half = r.np / 2;
    r.lo = R.lo;
    r.hi = R.hi;
    const int64_t *st = (!r.xdom && have_t) ? sty : stx;
    r.sp = (int32_t)(r.xdom ? st[0] : st[1]);
    r.sq = (int32_t)(r.xdom ? st[1] : st[0]);
    r.szs = (int32_t)st[2];
    return r;
}

// Distance of t from the nearest integer is below m (a floor() of t could differ from the floor
// of a value within m of t).
__device__ __forceinline__ bool near_int(float t, float m) {
    return fabsf(t - rintf(t)) < m;
}


// Voxels of one slab from the boundary coordinates: the branch-free form of the reference's case
// analysis (siddon.cu.cc:86-189). With fq, fz the fractions of the slab before the q and z
// crossings (1 when no crossing), the near corner (cq1, cz1) takes min(fq, fz), the far corner
// (cq2, cz2) takes 1 - max of the crossings' fractions, and when both coordinates step the middle
// voxel takes |fq - fz| ((cq1, cz2) if z steps first, else (cq2, cz1)). w[c] == 0 marks a voxel
// that is not visited; the validity tests are the reference's range tests.
__device__ __forceinline__ void slab_voxels(const LorRun &r, int ip, bool keep, float qq1, float qq2,
                                            float zz1, float zz2, float wt, int32_t o[3], float w[3]) {
    const int cq1 = ifloor(qq1), cq2 = ifloor(qq2);
    const int cz1 = ifloor(zz1), cz2 = ifloor(zz2);
    const bool dq = cq1 != cq2, dz = cz1 != cz2;
    const float fq = ((float)cq2 - qq1) * r.invq;  // used only when dq
    const float fz = ((float)cz2 - zz1) * r.invz;  // used only when dz
    const float f0 = fminf(dq ? fq : 1.0f, dz ? fz : 1.0f);
    const float f2 = 1.0f - fmaxf(dq ? fq : 0.0f, dz ? fz : 0.0f);
    const int32_t base = ip * r.sp;
    const int32_t q1o = cq1 * r.sq, q2o = cq2 * r.sq, z1o = cz1 * r.szs, z2o = cz2 * r.szs;
    // the reference's range tests, with cq1 <= cq2 and cz1 <= cz2: c in [0, n) as one unsigned compare
    const bool a = (unsigned)cq1 < (unsigned)r.nq, b = (unsigned)cz1 < (unsigned)r.nz;
    const bool c = (unsigned)cq2 < (unsigned)r.nq, d = (unsigned)cz2 < (unsigned)r.nz;
    const bool q1m = cq1 >= -1, z1m = cz1 >= -1;
    const bool v0 = keep && a && b;
    const bool v2 = keep && (dq || dz) && c && d && q1m && z1m;
    const bool qfirst = fq > fz;
    const bool v1 = keep && dq && dz && (qfirst ? (a && d && z1m) : (c && b && q1m));
    o[0] = v0 ? base + q1o + z1o : 0;
    w[0] = v0 ? f0 * wt : 0.0f;
    o[2] = v2 ? base + q2o + z2o : 0;
    w[2] = v2 ? f2 * wt : 0.0f;
    o[1] = v1 ? base + (qfirst ? q1o + z2o : q2o + z1o) : 0;
    w[1] = v1 ? fabsf(fq - fz) * wt : 0.0f;
}


// Fast, branch-free candidates of slab ip. `bad` is set when a floor or the truncation test is
// within its rounding margin; the caller then recomputes the slab with candidates_exact.
template <bool TOF>
__device__ __forceinline__ void candidates_fast(const LorRun &r, const GridK &k, int ip, bool active,
                                                int32_t o[3], float w[3], bool &pm, bool &bad) {
    bool keep = active;
    bad = false;
    float w_tof = 1.0f;
    if (TOF) {
        const float d2 = fmaf(r.tA, (float)ip, r.tB);
        const float e2 = d2 * d2 * k.k2;  // -t2 log2(e) / 2
        if (k.nsig2 > 0.0f) {
            bad = fabsf(e2 - k.e2cut) <= k.e2tol;
            keep = keep && (e2 >= k.e2cut);
        }
        asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(w_tof) : "f"(e2));  // exp(-t2 / 2), amplitude in wc
    }
    const float pp1 = __fsub_rn((float)ip, r.np2);
    const float pp2 = __fadd_rn(pp1, 1.0f);
    pm = (ip >= r.pmlo) & (ip <= r.pmhi);
    float qa, qb;
    if (r.dq_one) {  // exact and cheap without a division
        qa = __fadd_rn(__fadd_rn(r.q1, __fmul_rn(r.kq, __fsub_rn(pp1, r.p1))), r.nq2);
        qb = __fadd_rn(__fadd_rn(r.q1, __fmul_rn(r.kq, __fsub_rn(pp2, r.p1))), r.nq2);
    } else {
        qa = fmaf(r.Bq, pp1, r.Aq);
        qb = fmaf(r.Bq, pp2, r.Aq);
        bad = bad || near_int(qa, r.mq) || near_int(qb, r.mq);
    }
    const float za = fmaf(r.Bz, pp1, r.Az);
    const float zb = fmaf(r.Bz, pp2, r.Az);
    bad = active && (bad || near_int(za, r.mz) || near_int(zb, r.mz));
    const float qq1 = (r.kq >= 0.0f) ? qa : qb, qq2 = (r.kq >= 0.0f) ? qb : qa;
    const float zz1 = (r.kz >= 0.0f) ? za : zb, zz2 = (r.kz >= 0.0f) ? zb : za;
    slab_voxels(r, ip, keep, qq1, qq2, zz1, zz2, r.wc * w_tof, o, w);
}

// The same slab with the reference's operand sequence for every value that decides a floor or
// the truncation test (IEEE division, no contraction).
template <bool TOF>
__device__ __forceinline__ void candidates_exact(const LorRun &r, const GridK &k, int ip, int32_t o[3],
                                              float w[3], bool &pm) {
    bool keep = true;
    float w_tof = 1.0f;
    if (TOF) {
        const float pc = __fmul_rn(__fadd_rn((float)(ip - r.np_half), 0.5f), r.dpc);
        const float d2 = __fmul_rn(__fsub_rn(__fdiv_rn(__fsub_rn(pc, r.p1), r.pd), r.ratio1), r.L);
        const float t2 = __fdiv_rn(__fmul_rn(d2, d2), k.expand);
        if (k.nsig2 > 0.0f) keep = t2 <= k.nsig2;
        w_tof = exp2f(t2 * -kHalfLog2e);  // the amplitude is in wc
    }
    const float pp1 = __fsub_rn((float)ip, r.np2);
    const float pp2 = __fadd_rn(pp1, 1.0f);
    pm = (ip >= r.pmlo) & (ip <= r.pmhi);
    const float qa = bcoord(r.q1, r.kq, pp1, r.p1, r.dq, r.nq2, r.dq_one);
    const float qb = bcoord(r.q1, r.kq, pp2, r.p1, r.dq, r.nq2, r.dq_one);
    const float za = bcoord(r.z1, r.kz, pp1, r.p1, k.dz, k.nz2, false);
    const float zb = bcoord(r.z1, r.kz, pp2, r.p1, k.dz, k.nz2, false);
    const float qq1 = (r.kq >= 0.0f) ? qa : qb, qq2 = (r.kq >= 0.0f) ? qb : qa;
    const float zz1 = (r.kz >= 0.0f) ? za : zb, zz2 = (r.kz >= 0.0f) ? zb : za;
    slab_voxels(r, ip, keep, qq1, qq2, zz1, zz2, r.wc * w_tof, o, w);
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
