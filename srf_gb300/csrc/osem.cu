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

namespace srf {

template <int G, bool TOF>
__global__ void __launch_bounds__(kBlock)
k_osem_subset(const float *__restrict__ lors, int64_t n, int stride, const float *__restrict__ tof,
              int tof_stride, Grid g, TofParams tp, const float *__restrict__ y, int rule, float eps,
              View x, View xt, View bp, View bpt, double *__restrict__ loglik) {
    constexpr int GPW = 32 / G;
    const int lane = threadIdx.x & (G - 1);
    const int gi = (threadIdx.x & 31) / G;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool have_xt = xt.ptr != nullptr, have_bpt = bpt.ptr != nullptr;
    double ll = 0.0;
    for (int64_t base = warp * GPW; base < n; base += nwarps * GPW) {
        const int64_t i = base + gi;
        const bool valid = i < n;
        float x1 = 0, y1 = 0, z1 = 0, x2 = 0, y2 = 0, z2 = 0, tv = 0;
        float acc = 0.0f;
        if (valid) {
            const float *l = lors + i * stride;
            x1 = __ldg(l); y1 = __ldg(l + 1); z1 = __ldg(l + 2);
            x2 = __ldg(l + 3); y2 = __ldg(l + 4); z2 = __ldg(l + 5);
            if (TOF) tv = __ldg(tof + i * tof_stride);
            LorSetup S;
            if (setup_lor<TOF, RULES_PROJ>(x1, y1, z1, x2, y2, z2, tv, g, tp, x.st, xt.st, have_xt, S)) {
                const float *im = (!S.xdom && have_xt) ? xt.ptr : x.ptr;
                for (int ip = S.lo + lane; ip <= S.hi; ip += G)
                    slab<TOF, RULES_PROJ>(S, ip, [&](int32_t off, float w) { acc += __ldg(im + off) * w; });
            }
        }
        const float p = group_sum<G>(acc);
        if (valid) {
            const float yv = y ? __ldg(y + i) : 1.0f;
            const float den = __fadd_rn(p, eps);
            float r;
            if (rule == SRF_RATIO_DIV_NO_NAN)
                r = (den == 0.0f) ? 0.0f : __fdiv_rn(yv, den);
            else
                r = __fdiv_rn(yv, den);
            if (loglik && lane == 0 && den > 0.0f) ll += (double)yv * (double)__logf(den);
            if (r != 0.0f) {
                LorSetup S;
                if (setup_lor<TOF, RULES_BACK>(x1, y1, z1, x2, y2, z2, tv, g, tp, bp.st, bpt.st, have_bpt, S)) {
                    float *im = (!S.xdom && have_bpt) ? bpt.ptr : bp.ptr;
                    for (int ip = S.lo + lane; ip <= S.hi; ip += G)
                        slab<TOF, RULES_BACK>(S, ip, [&](int32_t off, float w) { atomicAdd(im + off, r * w); });
                }
            }
        }
    }
    if (loglik) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ll += __shfl_xor_sync(0xffffffffu, ll, o);
        if ((threadIdx.x & 31) == 0 && ll != 0.0) atomicAdd(loglik, ll);
    }
}

template <int G, bool TOF>
static int launch_osem_g(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                         const Grid &g, const TofParams &tp, const float *y, int rule, float eps,
                         const View &x, const View &xt, const View &bp, const View &bpt,
                         double *loglik, cudaStream_t s) {
    auto kern = k_osem_subset<G, TOF>;
    unsigned blocks = grid_for(kern, n, kBlock / G);
    kern<<<blocks, kBlock, 0, s>>>(lors, n, stride, tof, tof_stride, g, tp, y, rule, eps, x, xt, bp, bpt, loglik);
    return check_cuda("osem subset kernel launch");
}

template <bool TOF>
static int launch_osem(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                       const Grid &g, const TofParams &tp, const float *y, int rule, float eps,
                       const View &x, const View &xt, const View &bp, const View &bpt,
                       double *loglik, cudaStream_t s) {
    switch (group_lanes()) {
    case 8: return launch_osem_g<8, TOF>(lors, n, stride, tof, tof_stride, g, tp, y, rule, eps, x, xt, bp, bpt, loglik, s);
    case 16: return launch_osem_g<16, TOF>(lors, n, stride, tof, tof_stride, g, tp, y, rule, eps, x, xt, bp, bpt, loglik, s);
    default: return launch_osem_g<32, TOF>(lors, n, stride, tof, tof_stride, g, tp, y, rule, eps, x, xt, bp, bpt, loglik, s);
    }
}

// 32 x 32 (x, y) tiles of one z slice; 32 x 8 threads.
constexpr int kTile = 32;

__global__ void __launch_bounds__(kTile * 8)
k_osem_update(float *__restrict__ x, float *__restrict__ xt, float *__restrict__ bp,
              float *__restrict__ bpt, const float *__restrict__ emap, int guard, int nx, int ny) {
    __shared__ float tin[kTile][kTile + 1];
    __shared__ float tout[kTile][kTile + 1];
    const int bx = blockIdx.x * kTile, by = blockIdx.y * kTile;
    const int64_t zoff = (int64_t)blockIdx.z * nx * ny;
    const int tx = threadIdx.x, ty = threadIdx.y;
    if (bpt) {
        // bpt is y-fastest: element (ix, iy) at ix*ny + iy
        for (int j = ty; j < kTile; j += 8) {
            const int ix = bx + j, iy = by + tx;
            float v = 0.0f;
            if (ix < nx && iy < ny) {
                const int64_t o = zoff + (int64_t)ix * ny + iy;
                v = bpt[o];
                bpt[o] = 0.0f;
            }
            tin[j][tx] = v;  // [x_local][y_local]
        }
        __syncthreads();
    }
    for (int j = ty; j < kTile; j += 8) {
        const int iy = by + j, ix = bx + tx;
        if (ix < nx && iy < ny) {
            const int64_t o = zoff + (int64_t)iy * nx + ix;
            float b = bp[o];
            if (bpt) b = __fadd_rn(b, tin[tx][j]);
            float e = emap[o];
            if (guard && e == 0.0f) e = 1e8f;
            const float xn = __fdiv_rn(__fmul_rn(x[o], b), e);
            x[o] = xn;
            bp[o] = 0.0f;
            tout[j][tx] = xn;  // [y_local][x_local]
        }
    }
    if (xt) {
        __syncthreads();
        for (int j = ty; j < kTile; j += 8) {
            const int ix = bx + j, iy = by + tx;
            if (ix < nx && iy < ny) xt[zoff + (int64_t)ix * ny + iy] = tout[tx][j];
        }
    }
}

}  // namespace srf

using namespace srf;

extern "C" {

int srf_osem_subset(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                    int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                    const float *y, int32_t ratio_rule, float eps, const float *x,
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
    if (n == 0) return ok();
    cudaStream_t s = (cudaStream_t)stream;
    if (tof) {
        TofParams tp;
        if ((rc = check_tof(tof, n, tof_stride, tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
        return launch_osem<true>(lors, n, lor_stride, tof, tof_stride, g, tp, y, ratio_rule, eps, vx, vxt, vbp, vbpt, loglik, s);
    }
    TofParams tp{0, 0, 0};
    return launch_osem<false>(lors, n, lor_stride, nullptr, 1, g, tp, y, ratio_rule, eps, vx, vxt, vbp, vbpt, loglik, s);
}

int srf_osem_update(float *x, float *x_t, float *bp, float *bp_t, const float *emap,
                    int32_t guard_zero, const int32_t grid[3], void *stream) {
    if (!x || !bp || !emap) return fail(SRF_EINVAL, "x, bp and emap must not be NULL");
    if (!grid) return fail(SRF_EINVAL, "grid must not be NULL");
    Grid g; int rc;
    const float c[3] = {0, 0, 0}, sz[3] = {1, 1, 1};
    if ((rc = check_geometry(grid, c, sz, g))) return rc;
    dim3 blocks((g.nx + kTile - 1) / kTile, (g.ny + kTile - 1) / kTile, g.nz);
    k_osem_update<<<blocks, dim3(kTile, 8), 0, (cudaStream_t)stream>>>(x, x_t, bp, bp_t, emap, guard_zero, g.nx, g.ny);
    return check_cuda("osem update kernel launch");
}

}  // extern "C"
