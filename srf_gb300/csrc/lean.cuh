// Lean slab loop of the fused traversal: per-LOR constants folded so that a slab costs a few
// dozen instructions, and the image-box range tests run only for slabs near the box's faces.
//
// A LOR's slab ip is evaluated from its relative index pp = ip - ic (ic: the middle of the LOR's
// slab range). The in-plane coordinate q at the slab's two faces follows the reference's operand
// order (srfnef/cc/siddon/siddon.cu.cc:59-73; siddon_tof.cu.cc:77-90), so its floors and crossing
// fractions are the reference's. The axial coordinate z uses the linear form
//   z at the near / far face (ordered, zz1 <= zz2) = fma(Bz, pp, Z1) / fma(Bz, pp, Z2)
// with the reference's per-slab division folded into the constants (siddon.cu.cc:74-84), one FMA
// per face instead of an IEEE division. Floors come from
// one round-down add of 1.5 * 2^23: the sum's bit pattern is 0x4B400000 + floor(v) for
// |v| < 2^22, which feeds the offset multiply-adds directly (the bias is folded into the LOR's
// base offset) and compares for the crossing tests.
//
// The slab's (up to) three voxels, with fq, fz the fractions of the slab before the q and z
// crossings (1 when that coordinate does not cross):
//   slot 0  (cq1, cz1)                                   weight min(fq, fz)
//   slot 1  (cq1, cz2) if fq > fz else (cq2, cz1)          weight |fq - fz|
//   slot 2  (cq2, cz2)                                   weight 1 - max(fq, fz)
// Slot 1 is the far voxel when one coordinate crosses and the middle voxel when both do; slot 2
// is non-zero only when both cross. This is the reference's case analysis (siddon.cu.cc:86-189)
// without branches: its weights are ry/rz, (ry - rz) or (rz - ry), 1 - ry or 1 - rz.
//
// Exactness. The linear z form differs from the reference's value by a few units in the last
// place. A z floor can therefore differ when a face coordinate lies within ~1e-5 of an integer;
// the weight that moves between the two neighbouring voxels is then of the same order (the slab
// weight is continuous in the face coordinates), far below the 1e-5 relative L2 parity bound.
// (With the linear form for q as well, the fractions of LORs nearly parallel to the dominant axis
// carried that rounding divided by the small slope: the clinical backprojection drifted to
// 1.2e-5 relative L2 from the oracle.) Everything discontinuous
// is decided exactly, per LOR, in the reference's arithmetic: the skip rules, the dominant axis,
// the projector's endpoint slab range and the truncated TOF window (t2 <= nsigma^2).
//
// Range tests. Per LOR, [ilo, ihi] is the slab range whose face coordinates all lie at least
// kInteriorMargin inside the image box, so every candidate voxel is inside. A group of 32 slabs
// entirely within it skips the reference's range tests (siddon.cu.cc:88-189); other groups run
// them. A chunk whose active groups all lie within it runs them without a branch between them, so
// that the groups' independent instruction chains interleave. Gathers and reductions are
// predicated on a non-zero weight (a zero-weight slot still has a valid address, so neither needs
// a range test).
#pragma once
#include "fused.cuh"

namespace srf {

constexpr float kFloorMagic = 12582912.0f;   // 1.5 * 2^23
constexpr int kFloorBits = 0x4B400000;       // bit pattern of kFloorMagic
constexpr float kInteriorMargin = 0.01f;     // voxel units

struct __align__(16) LeanRec {
    float invq, invz, Bz, Z1;     // 1/|q step|, 1/|z step| per slab; z faces: fma(Bz, pp, Z1 or Z2)
    float Z2, tS, tT, wc;         // TOF: exponent -(fma(tS, pp, tT))^2 in log2 units; wc with amplitude
    float invL2, yv, ad, ppmax;   // ppmax = hi - ic
    float p1, q1, kq, dq;         // the q face coordinate in the reference's operand order
    float rdq, icnp, nq2, pad0;   // rdq = RN(1 / dq); icnp = ic - np/2 (exact)
    int lo, hi, ic, flags;        // flags: F_VALID | F_PROJ | F_XDOM | F_TIE
    int ilo, ihi, pmlo, pmhi;     // interior slabs; projector endpoint rule
    int base, pad1, pad2, pad3;   // element offset of slab ic at the floor-bit origin (mod 2^32)
};
constexpr int kLeanVec = sizeof(LeanRec) / 16;
static_assert(sizeof(LeanRec) == 128, "LeanRec is eight 16-byte vectors");

__device__ __forceinline__ LeanRec load_lean(const LeanRec *src) {
    LeanRec R;
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    float4 *d4 = reinterpret_cast<float4 *>(&R);
#pragma unroll
    for (int c = 0; c < kLeanVec; ++c) d4[c] = s4[c];
    return R;
}

__device__ __forceinline__ void store_lean(LeanRec *dst, const LeanRec &R) {
    const float4 *s4 = reinterpret_cast<const float4 *>(&R);
    float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll
    for (int c = 0; c < kLeanVec; ++c) d4[c] = s4[c];
}

// The truncated TOF kernel keeps slab ip when t2 <= nsigma^2, t2 in the reference's arithmetic
// (siddon_tof.cu.cc:55-58: xc, d2_tof, t2), as the oracle applies it.
__device__ __forceinline__ bool tof_keep(const LorRec &R, const GridK &k, int ip, int np_half, float dpc) {
    const float pc = __fmul_rn(__fadd_rn((float)(ip - np_half), 0.5f), dpc);
    const float d2 = __fmul_rn(__fsub_rn(__fdiv_rn(__fsub_rn(pc, R.p1), R.pd), R.ratio1), R.L);
    const float t2 = __fdiv_rn(__fmul_rn(d2, d2), k.expand);
    return t2 <= k.nsig2;
}

// [a, b] of real face positions f where A + B f stays within [m, n - m] (its FP32 rounding is far
// inside the margin m).
__device__ __forceinline__ void face_interval(float A, float B, float n, float m, float &a, float &b) {
    if (B == 0.0f) {
        if (A >= m && A <= n - m) { a = -1e30f; b = 1e30f; } else { a = 1e30f; b = -1e30f; }
        return;
    }
    const float t1 = (m - A) / B, t2 = (n - m - A) / B;
    a = fminf(t1, t2);
    b = fmaxf(t1, t2);
}

// Lean record of a LOR from its setup record (lane-parallel, once per LOR).
template <bool TOF>
__device__ __forceinline__ LeanRec make_lean(const LorRec &R, const Grid &g, const GridK &k,
                                             const int64_t stx[3], const int64_t sty[3], bool have_t) {
    LeanRec E = {};
    E.flags = R.flags;
    E.yv = R.yv;
    E.ad = R.ad;
    E.invL2 = R.invL2;
    E.lo = R.lo;
    E.hi = R.hi;
    E.pmlo = R.pmlo;
    E.pmhi = R.pmhi;
    if (!(R.flags & F_VALID) || (R.flags & F_TIE)) return E;
    const bool xdom = R.flags & F_XDOM;
    const int np = xdom ? g.nx : g.ny, nq = xdom ? g.ny : g.nx;
    const float np2 = xdom ? k.nx2 : k.ny2;
    const int np_half = np / 2;
    const float dpc = xdom ? 1.0f : k.dy;
    // d(ip) = ((pc(ip) - p1) / pd - ratio1) L with pc(ip) = (ip - np/2 + 0.5) dpc is linear in ip
    const float tA = dpc / R.pd * R.L;
    int lo = R.lo, hi = R.hi;
    if (TOF && k.nsig2 > 0.0f && lo <= hi) {
        // exact truncated window: t2 <= nsigma^2 keeps an interval of slabs; estimate it (to a
        // slab) and settle both ends with the predicate itself
        const float tB = (((0.5f - (float)np_half) * dpc - R.p1) / R.pd - R.ratio1) * R.L;
        const float half = sqrtf(k.nsig2 * k.expand) / fabsf(tA);
        const float c = -tB / tA;
        int a = (int)fmaxf(fminf(ceilf(c - half), (float)hi + 1.0f), (float)lo - 1.0f);
        int b = (int)fmaxf(fminf(floorf(c + half), (float)hi + 1.0f), (float)lo - 1.0f);
        for (int t = 0; t < 6 && a > lo && tof_keep(R, k, a - 1, np_half, dpc); ++t) --a;
        for (int t = 0; t < 6 && a <= b && !tof_keep(R, k, a, np_half, dpc); ++t) ++a;
        for (int t = 0; t < 6 && b < hi && tof_keep(R, k, b + 1, np_half, dpc); ++t) ++b;
        for (int t = 0; t < 6 && b >= a && !tof_keep(R, k, b, np_half, dpc); ++t) --b;
        lo = max(lo, a);
        hi = min(hi, b);
    }
    if (lo > hi) {
        E.flags = 0;
        return E;
    }
    E.lo = lo;
    E.hi = hi;
    const int ic = (lo + hi) >> 1;
    E.ic = ic;
    E.ppmax = (float)(hi - ic);
    // z at face f (slab ip has faces ip and ip + 1): Az + Bz (f - np/2); at pp = ip - ic the
    // lower face is f = ip + (Bz < 0), the upper one f = ip + (Bz >= 0)
    const float icnp = __fsub_rn((float)ic, np2);  // exact
    const float s_lo = R.Bz < 0.0f ? 1.0f : 0.0f;
    E.Bz = R.Bz;
    E.Z1 = fmaf(R.Bz, icnp + s_lo, R.Az);
    E.Z2 = fmaf(R.Bz, icnp + (1.0f - s_lo), R.Az);
    E.invq = R.invq;
    E.invz = R.invz;
    E.wc = R.wc;
    E.p1 = R.p1;
    E.q1 = R.q1;
    E.kq = R.kq;
    E.dq = xdom ? k.dy : 1.0f;
    E.rdq = __frcp_rn(E.dq);
    E.icnp = icnp;
    E.nq2 = xdom ? k.ny2 : k.nx2;
    if (TOF) {
        // exponent of the Gaussian in log2 units: d(ip)^2 k2 = -(s d(ip))^2, s = sqrt(-k2), with
        // d = tA pp + d(ic), d(ic) in the reference's operand order
        const float s = sqrtf(-k.k2);
        const float pc = __fmul_rn(__fadd_rn((float)(ic - np_half), 0.5f), dpc);
        const float dic = __fmul_rn(__fsub_rn(__fdiv_rn(__fsub_rn(pc, R.p1), R.pd), R.ratio1), R.L);
        E.tS = tA * s;
        E.tT = dic * s;
    }
    // interior slabs: both faces of every slab within the box by the margin, in q and in z
    float qa, qb, za, zb;
    face_interval(R.Aq - R.Bq * np2, R.Bq, (float)nq, kInteriorMargin, qa, qb);
    face_interval(R.Az - R.Bz * np2, R.Bz, (float)g.nz, kInteriorMargin, za, zb);
    const float fa = fmaxf(qa, za), fb = fminf(qb, zb);   // faces f in [fa, fb]
    const float il = fmaxf(ceilf(fa), (float)lo), ih = fminf(floorf(fb) - 1.0f, (float)hi);
    E.ilo = il <= ih ? (int)il : 1;
    E.ihi = il <= ih ? (int)ih : 0;
    // element offset of (slab ic, floor bits 0x4B400000 + cq, 0x4B400000 + cz), modulo 2^32
    const int64_t *st = (!xdom && have_t) ? sty : stx;
    const uint32_t sp = (uint32_t)(xdom ? st[0] : st[1]);
    const uint32_t sq = (uint32_t)(xdom ? st[1] : st[0]);
    const uint32_t sz = (uint32_t)st[2];
    E.base = (int)((uint32_t)ic * sp - (uint32_t)kFloorBits * (sq + sz));
    return E;
}

// Per-lane strides of the LOR's view and grid extents (no per-slab selects).
struct LeanAxes {
    int32_t sp, sq, sz, nq, nz;
};

__device__ __forceinline__ LeanAxes lean_axes(const LeanRec &E, const Grid &g, const int64_t stx[3],
                                              const int64_t sty[3], bool have_t) {
    const bool xdom = E.flags & F_XDOM;
    const int64_t *st = (!xdom && have_t) ? sty : stx;
    LeanAxes a;
    a.sp = (int32_t)(xdom ? st[0] : st[1]);
    a.sq = (int32_t)(xdom ? st[1] : st[0]);
    a.sz = (int32_t)st[2];
    a.nq = xdom ? g.ny : g.nx;
    a.nz = g.nz;
    return a;
}

// a / b correctly rounded from rb = RN(1 / b): one Newton step on the residual, which the FMA
// computes exactly (Markstein's division; a / 1 returns a unchanged)
__device__ __forceinline__ float div_refined(float a, float b, float rb) {
    const float q0 = __fmul_rn(a, rb);
    const float r = __fmaf_rn(-q0, b, a);
    return __fmaf_rn(r, rb, q0);
}

// The slab's q face coordinates (qq1 <= qq2) in the reference's operand order
// (siddon.cu.cc:59-73: (q1 + kq (pp - p1)) / dq + nq2 at pp = ip - np/2 and ip - np/2 + 1), so
// that the q floors and crossing fractions are the reference's. QDIV: dq != 1 (non-square
// transaxial voxels, x-dominant LORs).
template <bool QDIV>
__device__ __forceinline__ void q_faces(const LeanRec &E, float pp, float &qq1, float &qq2) {
    const float ppf = __fadd_rn(pp, E.icnp);  // ip - np/2, exact
    float ta = __fadd_rn(E.q1, __fmul_rn(E.kq, __fsub_rn(ppf, E.p1)));
    float tb = __fadd_rn(E.q1, __fmul_rn(E.kq, __fsub_rn(__fadd_rn(ppf, 1.0f), E.p1)));
    if (QDIV) {
        ta = div_refined(ta, E.dq, E.rdq);
        tb = div_refined(tb, E.dq, E.rdq);
    }
    ta = __fadd_rn(ta, E.nq2);
    tb = __fadd_rn(tb, E.nq2);
    const bool up = E.kq >= 0.0f;
    qq1 = up ? ta : tb;
    qq2 = up ? tb : ta;
}

// One slab of a LOR: the three slots' element offsets and weights (zero for a voxel the slab
// does not visit). ipc = min(ip, hi); act = ip <= hi (an inactive lane contributes zero weight
// at a valid address). EDGE runs the reference's range tests; without it the caller guarantees
// that ipc lies in [ilo, ihi].
template <bool TOF, bool EDGE, bool QDIV>
__device__ __forceinline__ void lean_slab(const LeanRec &E, const LeanAxes &ax, int ipc, float pp, bool act,
                                          int32_t o[3], float w[3]) {
    float wt = E.wc;
    if (TOF) {
        const float d = fmaf(E.tS, pp, E.tT);
        float ex;
        asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(ex) : "f"(-d * d));
        wt *= ex;
    }
    wt = act ? wt : 0.0f;
    float qq1, qq2;
    q_faces<QDIV>(E, pp, qq1, qq2);
    const float zz1 = fmaf(E.Bz, pp, E.Z1), zz2 = fmaf(E.Bz, pp, E.Z2);
    const float fq1 = __fadd_rd(qq1, kFloorMagic), fq2 = __fadd_rd(qq2, kFloorMagic);
    const float fz1 = __fadd_rd(zz1, kFloorMagic), fz2 = __fadd_rd(zz2, kFloorMagic);
    const int bq1 = __float_as_int(fq1), bq2 = __float_as_int(fq2);
    const int bz1 = __float_as_int(fz1), bz2 = __float_as_int(fz2);
    const bool dq = bq1 != bq2, dz = bz1 != bz2;
    const float fq = dq ? ((fq2 - kFloorMagic) - qq1) * E.invq : 1.0f;
    const float fz = dz ? ((fz2 - kFloorMagic) - zz1) * E.invz : 1.0f;
    const bool qfirst = fq > fz;
    const float mn = fminf(fq, fz), mx = fmaxf(fq, fz);
    float w0 = mn * wt, w1 = fabsf(fq - fz) * wt, w2 = fmaf(-mx, wt, wt);
    const uint32_t base = (uint32_t)E.base + (uint32_t)(ipc - E.ic) * (uint32_t)ax.sp;
    const uint32_t t1 = (uint32_t)bz1 * (uint32_t)ax.sz + base;
    const uint32_t t2 = (uint32_t)bz2 * (uint32_t)ax.sz + base;
    int32_t o0 = (int32_t)((uint32_t)bq1 * (uint32_t)ax.sq + t1);
    const int32_t oa = (int32_t)((uint32_t)bq2 * (uint32_t)ax.sq + t1);   // (cq2, cz1)
    const int32_t ob = (int32_t)((uint32_t)bq1 * (uint32_t)ax.sq + t2);   // (cq1, cz2)
    int32_t o2 = (int32_t)((uint32_t)bq2 * (uint32_t)ax.sq + t2);
    int32_t o1 = qfirst ? ob : oa;
    if (EDGE) {
        // the reference's range tests (cq1 <= cq2, cz1 <= cz2): c in [0, n) as one unsigned compare
        const bool A = (unsigned)(bq1 - kFloorBits) < (unsigned)ax.nq;
        const bool B = (unsigned)(bz1 - kFloorBits) < (unsigned)ax.nz;
        const bool C = (unsigned)(bq2 - kFloorBits) < (unsigned)ax.nq;
        const bool D = (unsigned)(bz2 - kFloorBits) < (unsigned)ax.nz;
        const bool qm = bq1 >= kFloorBits - 1, zm = bz1 >= kFloorBits - 1;
        const bool v0 = A && B;
        const bool v1 = qfirst ? (A && D && zm) : (C && B && qm);
        const bool v2 = C && D && qm && zm;
        w0 = v0 ? w0 : 0.0f;
        w1 = v1 ? w1 : 0.0f;
        w2 = v2 ? w2 : 0.0f;
        o0 = v0 ? o0 : 0;
        o1 = v1 ? o1 : 0;
        o2 = v2 ? o2 : 0;
    }
    o[0] = o0; o[1] = o1; o[2] = o2;
    w[0] = w0; w[1] = w1; w[2] = w2;
}

// The first N groups of a chunk, all inside [ilo, ihi], as straight-line code (no branch
// between the groups, so their instruction streams interleave); groups N..U-1 are zero.
template <bool TOF, int U, int G, bool QDIV, int N>
__device__ __forceinline__ void lean_interior_groups(const LeanRec &E, const LeanAxes &ax, int c0, int whi,
                                                     float ppmax, float pp0, int lane, int32_t (&o)[U][3],
                                                     float (&w)[U][3]) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (u < N) {
            const int ip = c0 + G * u + lane;
            const bool act = ip <= whi;
            lean_slab<TOF, false, QDIV>(E, ax, act ? ip : whi, fminf(pp0 + (float)(G * u), ppmax), act, o[u], w[u]);
        } else {
            o[u][0] = o[u][1] = o[u][2] = 0;
            w[u][0] = w[u][1] = w[u][2] = 0.0f;
        }
    }
}

// U slabs of one chunk of a walk over slabs [c0, whi] with G lanes per LOR (slab
// c0 + lane + G u): offsets and weights. Groups of G slabs past whi are skipped; groups inside
// [ilo, ihi] skip the range tests. When every group with an active slab is inside, one switch on
// their number runs them as straight-line code.
template <bool TOF, int U, int G, bool QDIV>
__device__ __forceinline__ void lean_chunk(const LeanRec &E, const LeanAxes &ax, int c0, int whi, float ppmax,
                                           int lane, int32_t (&o)[U][3], float (&w)[U][3]) {
    const float pp0 = (float)(c0 + lane - E.ic);
    const int ng = min(U, (whi - c0) / G + 1);  // groups with an active slab (c0 <= whi)
    if (c0 >= E.ilo && min(c0 + G * ng - 1, whi) <= E.ihi) {
        static_assert(U >= 1 && U <= 4, "1 to 4 groups per chunk");
        switch (ng) {
        case 1: lean_interior_groups<TOF, U, G, QDIV, 1>(E, ax, c0, whi, ppmax, pp0, lane, o, w); return;
        case 2: lean_interior_groups<TOF, U, G, QDIV, (U >= 2 ? 2 : 1)>(E, ax, c0, whi, ppmax, pp0, lane, o, w); return;
        case 3: lean_interior_groups<TOF, U, G, QDIV, (U >= 3 ? 3 : 1)>(E, ax, c0, whi, ppmax, pp0, lane, o, w); return;
        default: lean_interior_groups<TOF, U, G, QDIV, U>(E, ax, c0, whi, ppmax, pp0, lane, o, w); return;
        }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int g0 = c0 + G * u;  // first slab of the group (uniform over the group)
        if (g0 > whi) {
            o[u][0] = o[u][1] = o[u][2] = 0;
            w[u][0] = w[u][1] = w[u][2] = 0.0f;
            continue;
        }
        const int ip = g0 + lane;
        const bool act = ip <= whi;
        const int ipc = act ? ip : whi;
        const float pp = fminf(pp0 + (float)(G * u), ppmax);
        if (g0 >= E.ilo && min(g0 + G - 1, whi) <= E.ihi)
            lean_slab<TOF, false, QDIV>(E, ax, ipc, pp, act, o[u], w[u]);
        else
            lean_slab<TOF, true, QDIV>(E, ax, ipc, pp, act, o[u], w[u]);
    }
}

}  // namespace srf
