/* Host driver around the reference's own Siddon device functions (test infrastructure only).
 *
 * oracle/Makefile extracts the part of srfnef/cc/siddon/siddon.cu.cc (lines 1-656) and
 * srfnef/cc/siddon_tof/siddon_tof.cu.cc (lines 1-707) that precedes the first __global__ into
 * oracle/_ref/*.inc and compiles them here, through shim/ref_shim.h, into oracle/_ref/libsrf_ref.so.
 * Nothing of the reference is copied into the repository; the recipe reads it in place.
 *
 * Each ref_* entry point is the body of the reference's grid-stride kernels
 * (siddon.cu.cc:658-704, siddon_tof.cu.cc:709-759) run sequentially over the LORs, with the
 * output memset of the TF ops (siddon.cc:82, siddon_tof.cc:89) done by the caller for the
 * backprojections and here for the projections. Images are flat with x fastest
 * (index ix + iy*nx + iz*nx*ny), which is what the TF wrappers pass after tf.transpose.
 */
#include "ref_shim.h"

int64_t ref_atomic_count = 0;

namespace ref_nontof {
#include "siddon_dev.inc"
}
#undef abs

namespace ref_tof {
#include "siddon_tof_dev.inc"
}
#undef abs

extern "C" {

int64_t ref_take_atomic_count(void) {
    int64_t c = ref_atomic_count;
    ref_atomic_count = 0;
    return c;
}

void ref_projection(const float *lors, int64_t n, int stride, const int *grid, const float *center,
                    const float *size, const float *image, float *out) {
    for (int64_t i = 0; i < n; ++i) {
        const float *l = lors + i * stride;
        out[i] = 0.0f;
        ref_nontof::project_device(l[0], l[1], l[2], l[3], l[4], l[5], grid[0], grid[1], grid[2],
                                   center[0], center[1], center[2], size[0], size[1], size[2], image,
                                   out + i);
    }
}

void ref_backprojection(const float *lors, int64_t n, int stride, const float *values,
                        const int *grid, const float *center, const float *size, float *image) {
    for (int64_t i = 0; i < n; ++i) {
        const float *l = lors + i * stride;
        ref_nontof::backproject_device(l[0], l[1], l[2], l[3], l[4], l[5], grid[0], grid[1],
                                       grid[2], center[0], center[1], center[2], size[0], size[1],
                                       size[2], values[i], image);
    }
}

void ref_projection_tof(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                        float tof_bin, float tof_sigma2, const int *grid, const float *center,
                        const float *size, const float *image, float *out) {
    for (int64_t i = 0; i < n; ++i) {
        const float *l = lors + i * stride;
        out[i] = 0.0f;
        ref_tof::project_device(l[0], l[1], l[2], l[3], l[4], l[5], grid[0], grid[1], grid[2],
                                center[0], center[1], center[2], size[0], size[1], size[2],
                                tof[i * tof_stride], tof_bin, tof_sigma2, image, out + i);
    }
}

void ref_backprojection_tof(const float *lors, int64_t n, int stride, const float *tof,
                            int tof_stride, float tof_bin, float tof_sigma2, const float *values,
                            const int *grid, const float *center, const float *size,
                            float *image) {
    for (int64_t i = 0; i < n; ++i) {
        const float *l = lors + i * stride;
        ref_tof::backproject_device(l[0], l[1], l[2], l[3], l[4], l[5], grid[0], grid[1], grid[2],
                                    center[0], center[1], center[2], size[0], size[1], size[2],
                                    tof[i * tof_stride], tof_bin, tof_sigma2, values[i], image);
    }
}

}  // extern "C"
