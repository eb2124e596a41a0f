// Projector family entry points: forward projection and backprojection (non-TOF and TOF; these run
// on the fused kernel's traversal in osem.cu), the exact adjoint (batched: the fused traversal;
// single image: k_trace, which measured faster there than the batched kernel with one image),
// visit counts, attenuation, and the view fold/copy helpers. k_trace here is grid-stride over LORs
// with G lanes per LOR and the per-slab setup of siddon.cuh; it also serves the visit counts and
// the allocation-free TOF backprojection.
#include "common.cuh"
#include "fused.cuh"

namespace srf {

enum Action : int { SCATTER = 1, COUNT = 2 };

// Warp-uniform loop over LORs: each warp takes 32/G consecutive LORs per round, so the group
// shuffles in group_sum always see all 32 lanes.
template <int G, bool TOF, int RULES, int ACTION>
__global__ void __launch_bounds__(kBlock)
k_trace(const float *__restrict__ lors, int64_t n, int stride, const float *__restrict__ tof,
        int tof_stride, Grid g, TofParams tp, View v, View vt, const float *__restrict__ values,
        float *__restrict__ out) {
    constexpr int GPW = 32 / G;
    const int lane = threadIdx.x & (G - 1);
    const int gi = (threadIdx.x & 31) / G;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool have_t = vt.ptr != nullptr;
    for (int64_t base = warp * GPW; base < n; base += nwarps * GPW) {
        const int64_t i = base + gi;
        const bool valid = i < n;
        float acc = 0.0f;
        if (valid) {
            const float *l = lors + i * stride;
            const float tv = TOF ? __ldg(tof + i * tof_stride) : 0.0f;
            LorSetup S;
            if (setup_lor<TOF, RULES>(__ldg(l), __ldg(l + 1), __ldg(l + 2), __ldg(l + 3),
                                      __ldg(l + 4), __ldg(l + 5), tv, g, tp, v.st, vt.st, have_t,
                                      S)) {
                float *im = (!S.xdom && have_t) ? vt.ptr : v.ptr;
                if (ACTION == COUNT) {
                    for (int ip = S.lo + lane; ip <= S.hi; ip += G)
                        slab<TOF, RULES>(S, ip, [&](int32_t, float) { acc += 1.0f; });
                } else {
                    const float val = __ldg(values + i);
                    if (val != 0.0f)
                        for (int ip = S.lo + lane; ip <= S.hi; ip += G)
                            slab<TOF, RULES>(S, ip, [&](int32_t off, float w) { atomicAdd(im + off, val * w); });
                }
            }
        }
        if (ACTION == COUNT) {
            acc = group_sum<G>(acc);  // < 2^24 visits per LOR, exact in FP32
            if (valid && lane == 0 && acc > 0.0f)
                atomicAdd((unsigned long long *)out, (unsigned long long)acc);
        }
    }
}

template <int G, bool TOF, int RULES, int ACTION>
static int launch_trace_g(const float *lors, int64_t n, int stride, const float *tof,
                          int tof_stride, const Grid &g, const TofParams &tp, const View &v,
                          const View &vt, const float *values, float *out, cudaStream_t s) {
    auto kern = k_trace<G, TOF, RULES, ACTION>;
    unsigned blocks = grid_for(kern, n, kBlock / G);
    kern<<<blocks, kBlock, 0, s>>>(lors, n, stride, tof, tof_stride, g, tp, v, vt, values, out);
    return check_cuda("trace kernel launch");
}

template <bool TOF, int RULES, int ACTION>
static int launch_trace(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                        const Grid &g, const TofParams &tp, const View &v, const View &vt,
                        const float *values, float *out, cudaStream_t s) {
    if (n == 0) return ok();
    switch (group_lanes()) {
    case 8: return launch_trace_g<8, TOF, RULES, ACTION>(lors, n, stride, tof, tof_stride, g, tp, v, vt, values, out, s);
    case 16: return launch_trace_g<16, TOF, RULES, ACTION>(lors, n, stride, tof, tof_stride, g, tp, v, vt, values, out, s);
    default: return launch_trace_g<32, TOF, RULES, ACTION>(lors, n, stride, tof, tof_stride, g, tp, v, vt, values, out, s);
    }
}

constexpr int kMaxBatch = 8;  // images per batched projector call (as the kernel in osem.cu)

// UmapProject's epilogue over projections already in out (attenuation_correct.py:34-40):
// a = exp(-(p * L * L / unit)) with L from the raw endpoints in FP32; out = values / a when values
// are given (AttenuationCorrect), else a.
__global__ void k_atten_epilogue(const float *__restrict__ lors, int64_t n, int stride, Grid g,
                                 const float *__restrict__ values, float *__restrict__ out) {
    const float unit = __fdiv_rn(g.sx, (float)g.nx);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float *l = lors + i * stride;
        const float dx = __fsub_rn(__ldg(l), __ldg(l + 3)), dy = __fsub_rn(__ldg(l + 1), __ldg(l + 4));
        const float dz = __fsub_rn(__ldg(l + 2), __ldg(l + 5));
        const float L = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
        const float v = __fdiv_rn(__fmul_rn(__fmul_rn(out[i], L), L), unit);
        const float a = expf(-v);
        out[i] = values ? __fdiv_rn(__ldg(values + i), a) : a;
    }
}

// Elementwise kernels over a grid with arbitrary views.
__global__ void k_fold(float *dst, View d, const float *src, View sv, int nx, int ny, int nz) {
    const int64_t total = (int64_t)nx * ny * nz;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ix = k % nx, iy = (k / nx) % ny, iz = k / ((int64_t)nx * ny);
        dst[ix * d.st[0] + iy * d.st[1] + iz * d.st[2]] += src[ix * sv.st[0] + iy * sv.st[1] + iz * sv.st[2]];
    }
}

__global__ void k_copy(float *dst, View d, const float *src, View sv, int nx, int ny, int nz) {
    const int64_t total = (int64_t)nx * ny * nz;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ix = k % nx, iy = (k / nx) % ny, iz = k / ((int64_t)nx * ny);
        dst[ix * d.st[0] + iy * d.st[1] + iz * d.st[2]] = src[ix * sv.st[0] + iy * sv.st[1] + iz * sv.st[2]];
    }
}

}  // namespace srf

using namespace srf;

extern "C" {

const char *srf_last_error(void) { return g_err; }

int srf_version(void) { return 100; }

int srf_set_group_lanes(int lanes) {
    if (lanes != 8 && lanes != 16 && lanes != 32) return fail(SRF_EINVAL, "lanes must be 8, 16 or 32");
    group_lanes() = lanes;
    return ok();
}

int srf_set_tuning(int lanes, int slabs_per_lane_) {
    if (lanes != 8 && lanes != 16 && lanes != 32) return fail(SRF_EINVAL, "lanes must be 8, 16 or 32");
    if (slabs_per_lane_ != 2 && slabs_per_lane_ != 4) return fail(SRF_EINVAL, "slabs_per_lane must be 2 or 4");
    group_lanes() = lanes;
    slabs_per_lane() = slabs_per_lane_;
    return ok();
}

static int common_args(const float *lors, int64_t n, int32_t lor_stride, const void *image,
                       const int64_t *st, const void *image_t, const int64_t *st_t,
                       const int32_t grid[3], const float center[3], const float size[3], Grid &g,
                       View &v, View &vt) {
    int rc;
    if ((rc = check_lors(lors, n, lor_stride))) return rc;
    if ((rc = check_geometry(grid, center, size, g))) return rc;
    if ((rc = check_view(image, st, g, "image", v, true))) return rc;
    if ((rc = check_view(image_t, st_t, g, "image_t", vt, false))) return rc;
    return SRF_OK;
}

int srf_projection(const float *lors, int64_t n, int32_t lor_stride, const float *image,
                   const int64_t image_strides[3], const float *image_t,
                   const int64_t image_t_strides[3], const int32_t grid[3], const float center[3],
                   const float size[3], float *out, void *stream) {
    Grid g; View v, vt; int rc;
    if ((rc = common_args(lors, n, lor_stride, image, image_strides, image_t, image_t_strides, grid, center, size, g, v, vt))) return rc;
    if (n > 0 && !out) return fail(SRF_EINVAL, "out must not be NULL");
    TofParams tp{0, 0, 0};
    return fused_projection(lors, n, lor_stride, nullptr, 1, g, tp, v, vt, out, (cudaStream_t)stream);
}

int srf_backprojection(const float *lors, int64_t n, int32_t lor_stride, const float *values,
                       float *image, const int64_t image_strides[3], float *image_t,
                       const int64_t image_t_strides[3], const int32_t grid[3],
                       const float center[3], const float size[3], void *stream) {
    Grid g; View v, vt; int rc;
    if ((rc = common_args(lors, n, lor_stride, image, image_strides, image_t, image_t_strides, grid, center, size, g, v, vt))) return rc;
    if (n > 0 && !values) return fail(SRF_EINVAL, "values must not be NULL");
    TofParams tp{0, 0, 0};
    return fused_backprojection(lors, n, lor_stride, nullptr, 1, g, tp, values, v, vt, (cudaStream_t)stream);
}

int srf_projection_tof(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                       int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                       const float *image, const int64_t image_strides[3], const float *image_t,
                       const int64_t image_t_strides[3], const int32_t grid[3],
                       const float center[3], const float size[3], float *out, void *stream) {
    Grid g; View v, vt; TofParams tp; int rc;
    if ((rc = common_args(lors, n, lor_stride, image, image_strides, image_t, image_t_strides, grid, center, size, g, v, vt))) return rc;
    if ((rc = check_tof(tof, n, tof_stride, tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
    if (n > 0 && !out) return fail(SRF_EINVAL, "out must not be NULL");
    return fused_projection(lors, n, lor_stride, tof, tof_stride, g, tp, v, vt, out, (cudaStream_t)stream);
}

int srf_backprojection_tof(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                           int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                           const float *values, float *image, const int64_t image_strides[3],
                           float *image_t, const int64_t image_t_strides[3],
                           const int32_t grid[3], const float center[3], const float size[3],
                           void *stream) {
    Grid g; View v, vt; TofParams tp; int rc;
    if ((rc = common_args(lors, n, lor_stride, image, image_strides, image_t, image_t_strides, grid, center, size, g, v, vt))) return rc;
    if ((rc = check_tof(tof, n, tof_stride, tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
    if (n > 0 && !values) return fail(SRF_EINVAL, "values must not be NULL");
    return fused_backprojection(lors, n, lor_stride, tof, tof_stride, g, tp, values, v, vt, (cudaStream_t)stream);
}

int srf_projection_adjoint(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                           int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                           const float *values, float *image, const int64_t image_strides[3],
                           float *image_t, const int64_t image_t_strides[3],
                           const int32_t grid[3], const float center[3], const float size[3],
                           void *stream) {
    Grid g; View v, vt; int rc;
    if ((rc = common_args(lors, n, lor_stride, image, image_strides, image_t, image_t_strides, grid, center, size, g, v, vt))) return rc;
    if (n > 0 && !values) return fail(SRF_EINVAL, "values must not be NULL");
    // the batched adjoint traversal with one image (bstride 0)
    if (tof) {
        TofParams tp;
        if ((rc = check_tof(tof, n, tof_stride, tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
        return fused_adjoint_batch(lors, n, lor_stride, tof, tof_stride, g, tp, 1, 0, values, n, v, vt, (cudaStream_t)stream);
    }
    TofParams tp{0, 0, 0};
    return fused_adjoint_batch(lors, n, lor_stride, nullptr, 1, g, tp, 1, 0, values, n, v, vt, (cudaStream_t)stream);
}

static int batch_args(int32_t n_images, int64_t batch_stride, int64_t row_stride, int64_t n,
                      const View &v, const View &vt, const Grid &g) {
    if (n_images < 1 || n_images > kMaxBatch) return fail(SRF_EINVAL, "n_images must be 1..%d", kMaxBatch);
    if (row_stride < n) return fail(SRF_EINVAL, "row stride of the LOR values is below n");
    int64_t span_v = 0, span_t = 0;  // largest element offset within one image, per layout
    for (int k = 0; k < 3; ++k) {
        const int64_t nk = k == 0 ? g.nx : (k == 1 ? g.ny : g.nz);
        span_v += (nk - 1) * v.st[k];
        span_t += (nk - 1) * vt.st[k];
    }
    const int64_t span = span_v > span_t ? span_v : span_t;
    if (n_images > 1 && batch_stride <= span) return fail(SRF_EGRID, "images of the batch overlap");
    return SRF_OK;
}

int srf_projection_batch(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                         int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                         int32_t n_images, int64_t batch_stride, const float *images,
                         const int64_t image_strides[3], const float *images_t,
                         const int64_t image_t_strides[3], const int32_t grid[3],
                         const float center[3], const float size[3], float *out, int64_t out_stride,
                         void *stream) {
    Grid g; View v, vt; int rc;
    if ((rc = common_args(lors, n, lor_stride, images, image_strides, images_t, image_t_strides, grid, center, size, g, v, vt))) return rc;
    if ((rc = batch_args(n_images, batch_stride, out_stride, n, v, vt, g))) return rc;
    if (n > 0 && !out) return fail(SRF_EINVAL, "out must not be NULL");
    cudaStream_t s = (cudaStream_t)stream;
    if (tof) {
        TofParams tp;
        if ((rc = check_tof(tof, n, tof_stride, tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
        return fused_projection_batch(lors, n, lor_stride, tof, tof_stride, g, tp, n_images, batch_stride, v, vt, out, out_stride, s);
    }
    TofParams tp{0, 0, 0};
    return fused_projection_batch(lors, n, lor_stride, nullptr, 1, g, tp, n_images, batch_stride, v, vt, out, out_stride, s);
}

int srf_projection_adjoint_batch(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                                 int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                                 int32_t n_images, const float *values, int64_t values_stride,
                                 float *images, int64_t batch_stride, const int64_t image_strides[3],
                                 float *images_t, const int64_t image_t_strides[3], const int32_t grid[3],
                                 const float center[3], const float size[3], void *stream) {
    Grid g; View v, vt; int rc;
    if ((rc = common_args(lors, n, lor_stride, images, image_strides, images_t, image_t_strides, grid, center, size, g, v, vt))) return rc;
    if ((rc = batch_args(n_images, batch_stride, values_stride, n, v, vt, g))) return rc;
    if (n > 0 && !values) return fail(SRF_EINVAL, "values must not be NULL");
    cudaStream_t s = (cudaStream_t)stream;
    if (tof) {
        TofParams tp;
        if ((rc = check_tof(tof, n, tof_stride, tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
        return fused_adjoint_batch(lors, n, lor_stride, tof, tof_stride, g, tp, n_images, batch_stride, values, values_stride, v, vt, s);
    }
    TofParams tp{0, 0, 0};
    return fused_adjoint_batch(lors, n, lor_stride, nullptr, 1, g, tp, n_images, batch_stride, values, values_stride, v, vt, s);
}

int srf_count_pairs(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                    int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                    int32_t rules, const int32_t grid[3], const float center[3],
                    const float size[3], unsigned long long *count, void *stream) {
    Grid g; int rc;
    if ((rc = check_lors(lors, n, lor_stride))) return rc;
    if ((rc = check_geometry(grid, center, size, g))) return rc;
    if (!count) return fail(SRF_EINVAL, "count must not be NULL");
    if (rules != RULES_PROJ && rules != RULES_BACK) return fail(SRF_EINVAL, "unknown rules %d", rules);
    const int64_t st[3] = {1, g.nx, (int64_t)g.nx * g.ny};
    View v{nullptr, {st[0], st[1], st[2]}}, vt{nullptr, {0, 0, 0}};
    float *out = (float *)count;
    cudaStream_t s = (cudaStream_t)stream;
    if (tof) {
        TofParams tp;
        if ((rc = check_tof(tof, n, tof_stride, tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
        return rules == RULES_PROJ
                   ? launch_trace<true, RULES_PROJ, COUNT>(lors, n, lor_stride, tof, tof_stride, g, tp, v, vt, nullptr, out, s)
                   : launch_trace<true, RULES_BACK, COUNT>(lors, n, lor_stride, tof, tof_stride, g, tp, v, vt, nullptr, out, s);
    }
    TofParams tp{0, 0, 0};
    return rules == RULES_PROJ
               ? launch_trace<false, RULES_PROJ, COUNT>(lors, n, lor_stride, nullptr, 1, g, tp, v, vt, nullptr, out, s)
               : launch_trace<false, RULES_BACK, COUNT>(lors, n, lor_stride, nullptr, 1, g, tp, v, vt, nullptr, out, s);
}

int srf_attenuation(const float *lors, int64_t n, int32_t lor_stride, const float *umap,
                    const int64_t umap_strides[3], const int32_t grid[3], const float center[3],
                    const float size[3], const float *values, float *out, void *stream) {
    Grid g; View v, vt; int rc;
    if ((rc = common_args(lors, n, lor_stride, umap, umap_strides, nullptr, nullptr, grid, center, size, g, v, vt))) return rc;
    if (n > 0 && !out) return fail(SRF_EINVAL, "out must not be NULL");
    TofParams tp{0, 0, 0};
    cudaStream_t s = (cudaStream_t)stream;
    int rc2 = fused_projection(lors, n, lor_stride, nullptr, 1, g, tp, v, vt, out, s);
    if (rc2 || n == 0) return rc2;
    k_atten_epilogue<<<grid_for(k_atten_epilogue, n, 256), 256, 0, s>>>(lors, n, lor_stride, g, values, out);
    return check_cuda("attenuation epilogue launch");
}

static int elementwise_args(const void *dst, const int64_t *ds, const void *src, const int64_t *ss,
                            const int32_t grid[3], Grid &g, View &d, View &sv) {
    if (!grid) return fail(SRF_EINVAL, "grid must not be NULL");
    const float c[3] = {0, 0, 0}, sz[3] = {1, 1, 1};
    int rc;
    if ((rc = check_geometry(grid, c, sz, g))) return rc;
    if ((rc = check_view(dst, ds, g, "dst", d, true))) return rc;
    if ((rc = check_view(src, ss, g, "src", sv, true))) return rc;
    return SRF_OK;
}

int srf_fold_views(float *dst, const int64_t dst_strides[3], const float *src,
                   const int64_t src_strides[3], const int32_t grid[3], void *stream) {
    Grid g; View d, sv; int rc;
    if ((rc = elementwise_args(dst, dst_strides, src, src_strides, grid, g, d, sv))) return rc;
    const int64_t total = (int64_t)g.nx * g.ny * g.nz;
    unsigned blocks = grid_for(k_fold, total, kBlock);
    k_fold<<<blocks, kBlock, 0, (cudaStream_t)stream>>>(dst, d, src, sv, g.nx, g.ny, g.nz);
    return check_cuda("fold kernel launch");
}

int srf_copy_view(float *dst, const int64_t dst_strides[3], const float *src,
                  const int64_t src_strides[3], const int32_t grid[3], void *stream) {
    Grid g; View d, sv; int rc;
    if ((rc = elementwise_args(dst, dst_strides, src, src_strides, grid, g, d, sv))) return rc;
    const int64_t total = (int64_t)g.nx * g.ny * g.nz;
    unsigned blocks = grid_for(k_copy, total, kBlock);
    k_copy<<<blocks, kBlock, 0, (cudaStream_t)stream>>>(dst, d, src, sv, g.nx, g.ny, g.nz);
    return check_cuda("copy kernel launch");
}

}  // extern "C"

namespace srf {

// TOF backprojection into caller-provided views (used by the no-allocation entry point in
// noalloc.cu, which supplies its own y-fastest accumulator). Arguments are checked by the caller.
// dst (x-fastest) += src (y-fastest) over a grid (used by noalloc.cu).
int fold_views(float *dst, const View &d, const float *src, const View &sv, const Grid &g,
               cudaStream_t s) {
    const int64_t total = (int64_t)g.nx * g.ny * g.nz;
    unsigned blocks = grid_for(k_fold, total, kBlock);
    k_fold<<<blocks, kBlock, 0, s>>>(dst, d, src, sv, g.nx, g.ny, g.nz);
    return check_cuda("fold kernel launch");
}

}  // namespace srf
