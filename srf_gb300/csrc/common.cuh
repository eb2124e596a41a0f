// Shared host-side plumbing of the C ABI: status codes, per-thread error text, argument checks,
// launch sizing.
#pragma once
#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cmath>
#include <cuda_runtime.h>

#include "srf_gb300.h"
#include "siddon.cuh"

namespace srf {

inline thread_local char g_err[512] = {0};

inline int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

inline int ok() {
    g_err[0] = 0;
    return SRF_OK;
}

inline int check_cuda(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SRF_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    return ok();
}

inline int num_sms() {
    int dev = 0;
    cudaGetDevice(&dev);
    static thread_local int cached_dev = -1, cached = 0;
    if (dev != cached_dev) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cached = v > 0 ? v : 1;
        cached_dev = dev;
    }
    return cached;
}

// Process-wide tuning knobs (srf_set_tuning): atomic, so a setter on one host thread does not race
// with launches reading them on others. Lanes per LOR of the traversal kernels (8, 16 or 32).
inline std::atomic<int> &group_lanes() {
    static std::atomic<int> lanes{32};
    return lanes;
}

// Slabs each lane of a LOR group handles per chunk in the fused OSEM kernel (2 or 4; default 4).
inline std::atomic<int> &slabs_per_lane() {
    static std::atomic<int> u{4};
    return u;
}

constexpr int kBlock = 256;

// Blocks for a grid-stride kernel over `units` work items of `per_block` items each: enough to
// fill every SM to its occupancy limit, never more than the work needs.
template <typename K>
inline unsigned grid_for(K kernel, int64_t units, int per_block, int smem = 0, int block = kBlock) {
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, block, smem);
    if (occ < 1) occ = 1;
    int64_t need = (units + per_block - 1) / per_block;
    int64_t cap = (int64_t)num_sms() * occ;
    int64_t g = need < cap ? need : cap;
    return (unsigned)(g < 1 ? 1 : g);
}

inline int check_geometry(const int32_t grid[3], const float center[3], const float size[3], Grid &g) {
    if (!grid || !center || !size) return fail(SRF_EINVAL, "grid/center/size must not be NULL");
    for (int k = 0; k < 3; ++k) {
        if (grid[k] <= 0 || grid[k] > 65536) return fail(SRF_EGRID, "grid[%d]=%d out of range (1..65536)", k, grid[k]);
        if (!std::isfinite(center[k])) return fail(SRF_ENONFINITE, "center[%d] is not finite", k);
        if (!std::isfinite(size[k]) || !(size[k] > 0)) return fail(SRF_EGRID, "size[%d] must be finite and > 0", k);
    }
    if ((int64_t)grid[0] * grid[1] * grid[2] >= (int64_t(1) << 31))
        return fail(SRF_EGRID, "image has 2^31 or more voxels");
    g.nx = grid[0]; g.ny = grid[1]; g.nz = grid[2];
    g.cx = center[0]; g.cy = center[1]; g.cz = center[2];
    g.sx = size[0]; g.sy = size[1]; g.sz = size[2];
    return SRF_OK;
}

// A view is valid when every voxel offset is in [0, 2^31).
inline int check_view(const void *ptr, const int64_t st[3], const Grid &g, const char *name, View &v,
                      bool required) {
    v.ptr = (float *)ptr;
    if (!ptr) {
        if (required) return fail(SRF_EINVAL, "%s must not be NULL", name);
        v.st[0] = v.st[1] = v.st[2] = 0;
        return SRF_OK;
    }
    if (!st) return fail(SRF_EINVAL, "%s strides must not be NULL", name);
    const int n[3] = {g.nx, g.ny, g.nz};
    int64_t maxoff = 0;
    for (int k = 0; k < 3; ++k) {
        if (st[k] < 0) return fail(SRF_EGRID, "%s stride[%d] is negative", name, k);
        maxoff += st[k] * (int64_t)(n[k] - 1);
        v.st[k] = st[k];
    }
    if (maxoff >= (int64_t(1) << 31)) return fail(SRF_EGRID, "%s spans 2^31 or more elements", name);
    return SRF_OK;
}

inline int check_lors(const float *lors, int64_t n, int32_t stride) {
    if (n < 0) return fail(SRF_EINVAL, "negative LOR count");
    if (n > 0 && !lors) return fail(SRF_EINVAL, "lors must not be NULL");
    if (stride < 6) return fail(SRF_EINVAL, "lor_stride %d < 6", stride);
    return SRF_OK;
}

inline int check_tof_params(float tof_bin, float tof_sigma2, float tof_nsigma, TofParams &tp) {
    if (!std::isfinite(tof_bin) || !std::isfinite(tof_sigma2) || !std::isfinite(tof_nsigma))
        return fail(SRF_ENONFINITE, "non-finite TOF parameter");
    if (tof_nsigma < 0) return fail(SRF_EINVAL, "tof_nsigma must be >= 0");
    tp.tof_bin = tof_bin;
    tp.tof_sigma2 = tof_sigma2;
    tp.nsigma = tof_nsigma;
    return SRF_OK;
}

inline int check_tof(const float *tof, int64_t n, int32_t tof_stride, float tof_bin, float tof_sigma2,
                     float tof_nsigma, TofParams &tp) {
    if (n > 0 && !tof) return fail(SRF_EINVAL, "tof must not be NULL");
    if (tof_stride < 1) return fail(SRF_EINVAL, "tof_stride %d < 1", tof_stride);
    if (!std::isfinite(tof_bin) || !std::isfinite(tof_sigma2) || !std::isfinite(tof_nsigma))
        return fail(SRF_ENONFINITE, "non-finite TOF parameter");
    if (tof_nsigma < 0) return fail(SRF_EINVAL, "tof_nsigma must be >= 0");
    tp.tof_bin = tof_bin;
    tp.tof_sigma2 = tof_sigma2;
    tp.nsigma = tof_nsigma;
    return SRF_OK;
}

}  // namespace srf
