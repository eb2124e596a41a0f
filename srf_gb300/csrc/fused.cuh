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

// per-LOR record in shared memory
struct LorRec {
    float p1, p2, q1, z1, kq, kz, wc, invL2, ratio1, L, yv;
    int lo, hi, flags;
};
constexpr int F_VALID = 1, F_PROJ = 2, F_XDOM = 4, F_TIE = 8;

// grid-wide constants, rounded exactly as in setup_lor
struct GridK {
    float dx_, dy, dz, nx2, ny2, nz2;
    float tof_bin_, expand, inv_expand, tof_amp, nsig2, nsw;  // nsw = nsigma * sqrt(expand)
    bool dy_one;
};

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
    if (TOF) {
        k.tof_bin_ = __fdiv_rn(tp.tof_bin, k.dx_);
        const float s2 = __fdiv_rn(__fdiv_rn(tp.tof_sigma2, k.dx_), k.dx_);
        k.expand = __fadd_rn(s2, __fdiv_rn(__fmul_rn(k.tof_bin_, k.tof_bin_), 12.0f));
        k.inv_expand = 1.0f / k.expand;
        k.tof_amp = k.tof_bin_ * rsqrtf(2.0f * 3.1415926f * k.expand);
        k.nsig2 = tp.nsigma * tp.nsigma;
        k.nsw = tp.nsigma * sqrtf(k.expand);
    }
    return k;
}

// Lane-parallel setup of one LOR (both rule sets). Rounding of every value that feeds a floor or
// a skip predicate follows setup_lor.
template <bool TOF>
__device__ __forceinline__ LorRec setup_rec(const float *l, float tv, float yv, const Grid &g,
                                            const GridK &k) {
    LorRec R;
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
        R.ratio1 = (float)((1.0 - (double)tl) * 0.5);
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
    return R;
}

// Per-LOR constants of the slab loop, derived from a record.
struct LorRun {
    float p1, p2, q1, z1, kq, kz, wc, pd, ratio1, L;
    float np2, nq2, dq, dpc;
    // fast forms: boundary(pp) ~= fmaf(B, pp, A); TOF d2 ~= ((pc - p1) * inv_pd - ratio1) * L
    float Aq, Bq, Az, Bz, inv_pd;
    float mq, mz;  // floor margins of the fast forms (bounds on |fast - reference rounding|)
    int np, nq, nz, np_half, lo, hi;
    int32_t sp, sq, szs;
    bool xdom, dq_one;
};

__device__ __forceinline__ LorRun make_run(const LorRec &R, const Grid &g, const GridK &k,
                                           const int64_t stx[3], const int64_t sty[3],
                                           bool have_t) {
    LorRun r;
    r.xdom = R.flags & F_XDOM;
    r.p1 = R.p1; r.p2 = R.p2; r.q1 = R.q1; r.z1 = R.z1; r.kq = R.kq; r.kz = R.kz; r.wc = R.wc;
    r.pd = __fsub_rn(R.p2, R.p1);
    r.ratio1 = R.ratio1;
    r.L = R.L;
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
    r.Bq = r.kq / r.dq;
    r.Aq = (r.q1 - r.kq * r.p1) / r.dq + r.nq2;
    r.Bz = r.kz / k.dz;
    r.Az = (r.z1 - r.kz * r.p1) / k.dz + k.nz2;
    r.inv_pd = 1.0f / r.pd;
    // Both the fast form and the reference's operand sequence are within a few units of
    // 2^-24 * S of the exact value, S = (|k| (|p1| + |pp|) + |a|) / d + |n2| + 2 with |pp| <= np;
    // 2^-20 * S (16 units) bounds their difference with room to spare.
    const float e = 9.5367431640625e-7f;  // 2^-20
    r.mq = e * ((fabsf(r.kq) * (fabsf(r.p1) + (float)r.np) + fabsf(r.q1)) / r.dq + r.nq2 + 2.0f);
    r.mz = e * ((fabsf(r.kz) * (fabsf(r.p1) + (float)r.np) + fabsf(r.z1)) / k.dz + k.nz2 + 2.0f);
    const int64_t *st = (!r.xdom && have_t) ? sty : stx;
    r.sp = (int32_t)(r.xdom ? st[0] : st[1]);
    r.sq = (int32_t)(r.xdom ? st[1] : st[0]);
    r.szs = (int32_t)st[2];
    return r;
}

// Distance of t from the nearest integer is below m (a floor() of t could differ from the floor
// of a value within m of t).
__device__ __forceinline__ bool near_int(float t, float m) {
    const float f = t - floorf(t);
    return f < m || f > 1.0f - m;
}

// Relative margin on the TOF truncation test t2 <= nsigma^2 (fast t2 is within ~1e-6 relative).
constexpr float kTruncMargin = 2e-4f;

// Voxel candidates of slab ip (branch-free form of the reference's case analysis,
// siddon.cu.cc:86-189). w[k] == 0 marks a voxel that is not visited. Also returns the
// projector's slab predicate in pm.
template <bool TOF>
__device__ __forceinline__ void candidates(const LorRun &r, const GridK &k, int ip, int32_t o[3],
                                           float w[3], bool &pm) {
    w[0] = w[1] = w[2] = 0.0f;
    o[0] = o[1] = o[2] = 0;
    pm = false;
    float w_tof = 1.0f;
    if (TOF) {
        const float pc = __fmul_rn(__fadd_rn((float)(ip - r.np_half), 0.5f), r.dpc);
        const float d2 = ((pc - r.p1) * r.inv_pd - r.ratio1) * r.L;
        float t2 = d2 * d2 * k.inv_expand;
        if (k.nsig2 > 0.0f) {
            if (fabsf(t2 - k.nsig2) <= kTruncMargin * k.nsig2) {
                const float d2e = __fmul_rn(__fsub_rn(__fdiv_rn(__fsub_rn(pc, r.p1), r.pd), r.ratio1), r.L);
                t2 = __fdiv_rn(__fmul_rn(d2e, d2e), k.expand);
            }
            if (t2 > k.nsig2) return;
        }
        w_tof = k.tof_amp * exp2f(t2 * -0.72134752044448170f);  // exp(-t2/2)
    }
    const float pp1 = __fsub_rn((float)ip, r.np2);
    const float pp2 = __fadd_rn(pp1, 1.0f);
    if (!TOF) {
        pm = !((r.p1 < r.p2 && pp2 > r.p2) || (r.p1 >= r.p2 && pp1 < r.p2));
    } else if (r.xdom) {
        pm = !((r.p2 > r.p1 && pp1 <= r.p1) || (r.p2 < r.p1 && pp2 >= r.p1));
    } else {
        pm = !((r.p2 > r.p1 && pp1 < r.p1) || (r.p2 < r.p1 && pp2 > r.p1));
    }
    float qa, qb;
    if (r.dq_one) {  // exact and cheap without a division
        qa = bcoord(r.q1, r.kq, pp1, r.p1, 1.0f, r.nq2, true);
        qb = bcoord(r.q1, r.kq, pp2, r.p1, 1.0f, r.nq2, true);
    } else {
        qa = fmaf(r.Bq, pp1, r.Aq);
        qb = fmaf(r.Bq, pp2, r.Aq);
        if (near_int(qa, r.mq)) qa = bcoord(r.q1, r.kq, pp1, r.p1, r.dq, r.nq2, false);
        if (near_int(qb, r.mq)) qb = bcoord(r.q1, r.kq, pp2, r.p1, r.dq, r.nq2, false);
    }
    float za = fmaf(r.Bz, pp1, r.Az);
    float zb = fmaf(r.Bz, pp2, r.Az);
    if (near_int(za, r.mz)) za = bcoord(r.z1, r.kz, pp1, r.p1, k.dz, k.nz2, false);
    if (near_int(zb, r.mz)) zb = bcoord(r.z1, r.kz, pp2, r.p1, k.dz, k.nz2, false);
    const float qq1 = (r.kq >= 0.0f) ? qa : qb, qq2 = (r.kq >= 0.0f) ? qb : qa;
    const float zz1 = (r.kz >= 0.0f) ? za : zb, zz2 = (r.kz >= 0.0f) ? zb : za;
    const int cq1 = ifloor(qq1), cq2 = ifloor(qq2);
    const int cz1 = ifloor(zz1), cz2 = ifloor(zz2);
    const bool dq = cq1 != cq2, dz = cz1 != cz2;
    // the case's range condition
    const bool R = (dq ? (cq1 >= -1) : (cq1 >= 0)) && cq1 < r.nq &&
                   (dz ? (cz1 >= -1) : (cz1 >= 0)) && cz1 < r.nz;
    if (!R) return;
    const float rq = dq ? __fdividef((float)cq2 - qq1, qq2 - qq1) : 0.0f;
    const float rz = dz ? __fdividef((float)cz2 - zz1, zz2 - zz1) : 0.0f;
    const float wt = r.wc * w_tof;
    const int32_t base = ip * r.sp;
    // near corner (cq1, cz1)
    const float f0 = dq ? (dz ? fminf(rq, rz) : rq) : (dz ? rz : 1.0f);
    if (cq1 >= 0 && cz1 >= 0) {
        o[0] = base + cq1 * r.sq + cz1 * r.szs;
        w[0] = f0 * wt;
    }
    // far corner (cq2, cz2)
    if ((dq || dz) && cq2 < r.nq && cz2 < r.nz) {
        const float f2 = 1.0f - (dq ? (dz ? fmaxf(rq, rz) : rq) : rz);
        o[2] = base + cq2 * r.sq + cz2 * r.szs;
        w[2] = f2 * wt;
    }
    // middle voxel when both coordinates step
    if (dq && dz) {
        const bool qfirst = rq > rz;  // z steps first: (cq1, cz2); else (cq2, cz1)
        const int mq = qfirst ? cq1 : cq2, mz = qfirst ? cz2 : cz1;
        if (mq >= 0 && mq < r.nq && mz >= 0 && mz < r.nz) {
            o[1] = base + mq * r.sq + mz * r.szs;
            w[1] = (qfirst ? (rq - rz) : (rz - rq)) * wt;
        }
    }
}

}  // namespace srf
