// TOF backprojection that allocates no device memory.
//
// Some callers of this library cannot call cudaMalloc: a reconstruction plugin running inside a
// framework that owns all device memory through its own allocator (a TensorFlow op kernel may
// only take memory from its op context), or an acquisition-side service that reserves its device
// memory up front and may not allocate, nor take cudaMalloc's implicit device synchronisation,
// while the scanner is streaming. srf_backprojection_tof needs a second, y-fastest accumulator
// for the y-dominant LORs; this variant keeps that accumulator in a fixed static device array
// instead, so the caller passes only inputs and the output image.
//
// The array holds SRF_NOALLOC_MAX_VOXELS floats (18 MiB); every GPU that loads the library holds
// it until the process exits. All calls share it: calls that overlap on the GPU (different
// streams, or other threads) race on it and must be serialised by the caller.
//
// The traversal is srf_backprojection_tof's own (fused_backprojection), with the static array as
// its y-fastest accumulator, so the two entry points compute the same thing the same way.
//
// The array's device address is looked up once per device ordinal and cached for the life of
// the process. That assumes the CUDA runtime's primary context of each device: after
// cudaDeviceReset, or from a second context that the driver API made current on the same device,
// the cached address would no longer be this context's copy of the array.
#include <mutex>

#include "common.cuh"
#include "fused.cuh"

namespace srf {
int fold_views(float *dst, const View &d, const float *src, const View &sv, const Grid &g,
               cudaStream_t s);
}  // namespace srf

using namespace srf;

static __device__ __align__(256) float g_noalloc_scratch[SRF_NOALLOC_MAX_VOXELS];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
float *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device. In host code the array's name is
// only a host-side stand-in, so the address is looked up once per device (with that device
// current) and cached.
int scratch_for_current_device(float **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SRF_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(SRF_ERANGE, "device ordinal %d beyond %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(SRF_ECUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        g_scratch_ptr[dev] = (float *)p;
    }
    *out = g_scratch_ptr[dev];
    return SRF_OK;
}
}  // namespace

extern "C" int srf_backprojection_tof_noalloc(const float *lors, int64_t n, int32_t lor_stride,
                                              const float *tof, int32_t tof_stride, float tof_bin,
                                              float tof_sigma2, float tof_nsigma,
                                              const float *values, float *image,
                                              const int32_t grid[3], const float center[3],
                                              const float size[3], void *stream) {
    Grid g;
    TofParams tp;
    int rc;
    if ((rc = check_lors(lors, n, lor_stride))) return rc;
    if ((rc = check_geometry(grid, center, size, g))) return rc;
    if ((rc = check_tof(tof, n, tof_stride, tof_bin, tof_sigma2, tof_nsigma, tp))) return rc;
    if (n > 0 && !values) return fail(SRF_EINVAL, "values must not be NULL");
    if (!image) return fail(SRF_EINVAL, "image must not be NULL");
    const int64_t nvox = (int64_t)g.nx * g.ny * g.nz;
    if (nvox > SRF_NOALLOC_MAX_VOXELS)
        return fail(SRF_ERANGE, "image has %lld voxels; srf_backprojection_tof_noalloc handles at most %d",
                    (long long)nvox, SRF_NOALLOC_MAX_VOXELS);
    float *scratch = nullptr;
    if ((rc = scratch_for_current_device(&scratch))) return rc;
    if (n == 0) return ok();
    cudaStream_t s = (cudaStream_t)stream;
    // the scratch keeps the previous call's contents: clear the part this grid uses
    cudaError_t e = cudaMemsetAsync(scratch, 0, (size_t)nvox * sizeof(float), s);
    if (e != cudaSuccess) return fail(SRF_ECUDA, "clearing scratch: %s", cudaGetErrorString(e));
    View v{image, {1, g.nx, (int64_t)g.nx * g.ny}};
    View vt{scratch, {g.ny, 1, (int64_t)g.nx * g.ny}};
    if ((rc = fused_backprojection(lors, n, lor_stride, tof, tof_stride, g, tp, values, v, vt, s))) return rc;
    return fold_views(image, v, scratch, vt, g, s);
}
