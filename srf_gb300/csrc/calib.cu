// L2 calibration kernels: the denominators of the L2 gather and L2 atomic rooflines of the
// traversal kernels (not in the reference). Both touch a buffer small enough to stay in L2
// after the first pass, with the best-case pattern (a warp covers 32 consecutive words), so a
// traversal kernel's achieved gather bytes / red operations per second can be read as a
// fraction of what the L2 sustains for 4-byte words at all.
#include "common.cuh"

namespace srf {

// sink[tid] = sum of `reps` grid-stride passes of 4-byte loads over buf[0, n)
__global__ void k_l2_read(const float *__restrict__ buf, int64_t n, int reps, float *__restrict__ sink) {
    float acc = 0.0f;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; ++r)
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
            acc += __ldcg(buf + i);  // L2, not L1
    sink[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = acc;
}

// buf[i] += 1 for every i of `reps` grid-stride passes over [0, n), as reductions (no return value)
__global__ void k_l2_red(float *__restrict__ buf, int64_t n, int reps) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; ++r)
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
            atomicAdd(buf + i, 1.0f);
}

}  // namespace srf

using namespace srf;

extern "C" {

int srf_calib_l2(float *buf, int64_t n, int32_t reps, int32_t mode, float *sink, void *stream) {
    if (!buf || n <= 0 || reps <= 0) return fail(SRF_EINVAL, "bad arguments");
    if (mode != 0 && mode != 1) return fail(SRF_EINVAL, "mode must be 0 (read) or 1 (red)");
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned blocks = (unsigned)num_sms() * 8;
    if (mode == 0) {
        if (!sink) return fail(SRF_EINVAL, "sink must hold gridDim * 256 floats");
        k_l2_read<<<blocks, 256, 0, s>>>(buf, n, reps, sink);
    } else {
        k_l2_red<<<blocks, 256, 0, s>>>(buf, n, reps);
    }
    return check_cuda("calibration launch");
}

int srf_calib_sink_size(void) { return num_sms() * 8 * 256; }

}  // extern "C"
