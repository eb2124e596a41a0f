// Image warping: displacement-field deformation, rigid shifts and in-plane rotation
// (srfnef/cc/deform/deform.cu.cc:13-233 and deform_tex.cu.cc:15-420, the TF ops Deform, Shift,
// ShiftZ, Rotate and DeformInvert used by motion correction and multi-bed merging).
//
// Images are x-fastest (index ix + iy nx + iz nx ny), as the reference's ops receive them.
// Every output voxel is one thread of a grid-stride loop: the kernels read the displacement
// fields (or nothing) coalesced, gather 4 or 8 neighbours through L1/L2 and write one float, so
// they are bound by HBM bandwidth (20 B per voxel for a deformation, 8 B for a shift).
//
// Two interpolation rules, as the reference has two op libraries:
//  * plain (deform.cu.cc): trilinear from the floor corner; a voxel whose 2x2x2 neighbourhood
//    leaves the image stays 0 (the op zero-fills its output). Deform and Rotate reject a corner
//    index of 0 (`xi <= 0`), Shift accepts it (`xi < 0`); ShiftZ interpolates along z only and
//    keeps the half-weight edge cases (deform.cu.cc:103-138). Sample positions: Deform
//    ix + mx, Shift ix + mx, Rotate about the grid centre with integer nx / 2.
//  * texture (deform_tex.cu.cc, what srfnef's DeformMixin calls): a linearly filtered, clamped
//    3-D texture read at (position + 0.5) in texel units. Deform samples ix + mx, Shift and
//    ShiftZ sample ix - mx (the opposite sign of the plain op), Rotate the rotated centre, and
//    DeformInvert iterates x <- -m(x + i) 30 times per component. The texture unit weights with
//    8-bit fractions; these kernels weight with FP32 fractions, which differ from a texture
//    fetch by at most 1/512 of a neighbour difference.
#include "common.cuh"

namespace srf {

struct Vol {
    int nx, ny, nz;
    int64_t nxy;
};

__device__ __forceinline__ int64_t vidx(const Vol &v, int x, int y, int z) {
    return (int64_t)x + (int64_t)y * v.nx + (int64_t)z * v.nxy;
}

// Trilinear interpolation from corner (xi, yi, zi) with weights of the upper neighbour (a, b, c),
// in the reference's expression order (deform.cu.cc:40-57).
__device__ __forceinline__ float trilinear(const float *__restrict__ img, const Vol &v, int xi, int yi,
                                           int zi, float wx2, float wy2, float wz2) {
    const float wx = 1.0f - wx2, wy = 1.0f - wy2, wz = 1.0f - wz2;
    const int xi2 = xi + 1, yi2 = yi + 1, zi2 = zi + 1;
    return __ldg(img + vidx(v, xi, yi, zi)) * wx * wy * wz +
           __ldg(img + vidx(v, xi, yi, zi2)) * wx * wy * wz2 +
           __ldg(img + vidx(v, xi, yi2, zi)) * wx * wy2 * wz +
           __ldg(img + vidx(v, xi, yi2, zi2)) * wx * wy2 * wz2 +
           __ldg(img + vidx(v, xi2, yi, zi)) * wx2 * wy * wz +
           __ldg(img + vidx(v, xi2, yi, zi2)) * wx2 * wy * wz2 +
           __ldg(img + vidx(v, xi2, yi2, zi)) * wx2 * wy2 * wz +
           __ldg(img + vidx(v, xi2, yi2, zi2)) * wx2 * wy2 * wz2;
}

// A clamped, linearly filtered texture read at (u, v, w) in unnormalised texel coordinates.
__device__ __forceinline__ float tex_sample(const float *__restrict__ img, const Vol &v, float u, float s,
                                            float t) {
    const float xb = u - 0.5f, yb = s - 0.5f, zb = t - 0.5f;
    const float fx = floorf(xb), fy = floorf(yb), fz = floorf(zb);
    const float a = xb - fx, b = yb - fy, c = zb - fz;
    const int x0 = (int)fminf(fmaxf(fx, 0.0f), (float)(v.nx - 1));
    const int x1 = (int)fminf(fmaxf(fx + 1.0f, 0.0f), (float)(v.nx - 1));
    const int y0 = (int)fminf(fmaxf(fy, 0.0f), (float)(v.ny - 1));
    const int y1 = (int)fminf(fmaxf(fy + 1.0f, 0.0f), (float)(v.ny - 1));
    const int z0 = (int)fminf(fmaxf(fz, 0.0f), (float)(v.nz - 1));
    const int z1 = (int)fminf(fmaxf(fz + 1.0f, 0.0f), (float)(v.nz - 1));
    const float c00 = __ldg(img + vidx(v, x0, y0, z0)) * (1.0f - a) + __ldg(img + vidx(v, x1, y0, z0)) * a;
    const float c10 = __ldg(img + vidx(v, x0, y1, z0)) * (1.0f - a) + __ldg(img + vidx(v, x1, y1, z0)) * a;
    const float c01 = __ldg(img + vidx(v, x0, y0, z1)) * (1.0f - a) + __ldg(img + vidx(v, x1, y0, z1)) * a;
    const float c11 = __ldg(img + vidx(v, x0, y1, z1)) * (1.0f - a) + __ldg(img + vidx(v, x1, y1, z1)) * a;
    const float c0 = c00 * (1.0f - b) + c10 * b;
    const float c1 = c01 * (1.0f - b) + c11 * b;
    return c0 * (1.0f - c) + c1 * c;
}

enum WarpOp : int { W_DEFORM = 0, W_SHIFT = 1, W_SHIFT_Z = 2, W_ROTATE = 3 };

// The rotated sample position of voxel (ix, iy) about the grid centre, integer nx / 2 and ny / 2
// as in the reference (deform.cu.cc:153-154), each operation rounded on its own.
__device__ __forceinline__ void rotated(const Vol &v, int ix, int iy, float c, float s, float &px, float &py) {
    const float cx = (float)(v.nx / 2), cy = (float)(v.ny / 2);
    const float u = __fsub_rn(__fadd_rn((float)ix, 0.5f), cx);
    const float w = __fsub_rn(__fadd_rn((float)iy, 0.5f), cy);
    px = __fadd_rn(__fsub_rn(__fmul_rn(u, c), __fmul_rn(w, s)), cx);
    py = __fadd_rn(__fadd_rn(__fmul_rn(u, s), __fmul_rn(w, c)), cy);
}

// One output voxel of a warp. Plain rule: the voxel is left untouched (the caller zero-fills)
// when the neighbourhood leaves the image.
template <int OP, bool TEX>
__global__ void k_warp(const float *__restrict__ img, const float *__restrict__ mxf,
                       const float *__restrict__ myf, const float *__restrict__ mzf, float p0, float p1,
                       float p2, Vol v, float *__restrict__ out) {
    const int64_t total = v.nxy * v.nz;
    for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
         id += (int64_t)gridDim.x * blockDim.x) {
        const int iz = (int)(id / v.nxy);
        const int64_t r = id - (int64_t)iz * v.nxy;
        const int iy = (int)(r / v.nx), ix = (int)(r - (int64_t)iy * v.nx);
        if (TEX) {
            float u, s, t;
            if (OP == W_DEFORM) {
                u = __fadd_rn(__fadd_rn((float)ix, __ldg(mxf + id)), 0.5f);
                s = __fadd_rn(__fadd_rn((float)iy, __ldg(myf + id)), 0.5f);
                t = __fadd_rn(__fadd_rn((float)iz, __ldg(mzf + id)), 0.5f);
            } else if (OP == W_SHIFT) {
                u = __fadd_rn(__fsub_rn((float)ix, p0), 0.5f);
                s = __fadd_rn(__fsub_rn((float)iy, p1), 0.5f);
                t = __fadd_rn(__fsub_rn((float)iz, p2), 0.5f);
            } else if (OP == W_SHIFT_Z) {
                u = ix + 0.5f; s = iy + 0.5f; t = __fadd_rn(__fsub_rn((float)iz, p2), 0.5f);
            } else {
                rotated(v, ix, iy, p0, p1, u, s);
                t = iz + 0.5f;
            }
            out[id] = tex_sample(img, v, u, s, t);
            continue;
        }
        if (OP == W_SHIFT_Z) {  // deform.cu.cc:103-138
            const int zi = (int)floorf(iz + p2);
            const int zi2 = zi + 1;
            const float wz2 = iz + p2 - zi;
            const float wz = 1.0f - wz2;
            float val = 0.0f;
            if (zi2 == 0) val = __ldg(img + vidx(v, ix, iy, zi2)) * wz2;
            else if (zi == v.nz - 1) val = __ldg(img + vidx(v, ix, iy, zi)) * wz;
            else if (0 <= zi && zi2 < v.nz)
                val = __ldg(img + vidx(v, ix, iy, zi)) * wz + __ldg(img + vidx(v, ix, iy, zi2)) * wz2;
            out[id] = val;
            continue;
        }
        float px, py, pz;
        if (OP == W_DEFORM) {
            px = __fadd_rn((float)ix, __ldg(mxf + id));
            py = __fadd_rn((float)iy, __ldg(myf + id));
            pz = __fadd_rn((float)iz, __ldg(mzf + id));
        } else if (OP == W_SHIFT) {
            px = __fadd_rn((float)ix, p0); py = __fadd_rn((float)iy, p1); pz = __fadd_rn((float)iz, p2);
        } else {
            rotated(v, ix, iy, p0, p1, px, py);
            pz = (float)iz;
        }
        const int xi = (int)floorf(px), yi = (int)floorf(py), zi = (int)floorf(pz);
        // Deform and Rotate exclude a corner at index 0 (deform.cu.cc:31-42, 159-166), Shift
        // does not (:76-87); Rotate interpolates within the slice
        const int lo = (OP == W_SHIFT) ? 0 : 1;
        if (xi < lo || xi + 1 >= v.nx || yi < lo || yi + 1 >= v.ny) continue;
        if (OP == W_ROTATE) {
            const float wx2 = px - xi, wx = 1.0f - wx2, wy2 = py - yi, wy = 1.0f - wy2;
            out[id] = __ldg(img + vidx(v, xi, yi, iz)) * wx * wy + __ldg(img + vidx(v, xi, yi + 1, iz)) * wx * wy2 +
                      __ldg(img + vidx(v, xi + 1, yi, iz)) * wx2 * wy + __ldg(img + vidx(v, xi + 1, yi + 1, iz)) * wx2 * wy2;
            continue;
        }
        if (zi < lo || zi + 1 >= v.nz) continue;
        out[id] = trilinear(img, v, xi, yi, zi, px - xi, py - yi, pz - zi);
    }
}

// DeformInvert (deform_tex.cu.cc:78-100): the inverse displacement by the fixed-point iteration
// x <- -m_x(x + i), y <- -m_y(.), z <- -m_z(.) from 0, each read a clamped linear texture fetch.
__global__ void k_deform_invert(const float *__restrict__ mx, const float *__restrict__ my,
                                const float *__restrict__ mz, Vol v, int iters, float *__restrict__ ox,
                                float *__restrict__ oy, float *__restrict__ oz) {
    const int64_t total = v.nxy * v.nz;
    for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
         id += (int64_t)gridDim.x * blockDim.x) {
        const int iz = (int)(id / v.nxy);
        const int64_t r = id - (int64_t)iz * v.nxy;
        const int iy = (int)(r / v.nx), ix = (int)(r - (int64_t)iy * v.nx);
        float x = 0.0f, y = 0.0f, z = 0.0f;
        for (int it = 0; it < iters; ++it) {
            x = -tex_sample(mx, v, x + ix + 0.5f, y + iy + 0.5f, z + iz + 0.5f);
            y = -tex_sample(my, v, x + ix + 0.5f, y + iy + 0.5f, z + iz + 0.5f);
            z = -tex_sample(mz, v, x + ix + 0.5f, y + iy + 0.5f, z + iz + 0.5f);
        }
        ox[id] = x;
        oy[id] = y;
        oz[id] = z;
    }
}

static int check_vol(const int32_t grid[3], Vol &v) {
    if (!grid) return fail(SRF_EINVAL, "grid must not be NULL");
    for (int k = 0; k < 3; ++k)
        if (grid[k] <= 0 || grid[k] > 65536) return fail(SRF_EGRID, "grid[%d]=%d out of range (1..65536)", k, grid[k]);
    v.nx = grid[0]; v.ny = grid[1]; v.nz = grid[2];
    v.nxy = (int64_t)v.nx * v.ny;
    if (v.nxy * v.nz >= (int64_t(1) << 40)) return fail(SRF_EGRID, "image too large");
    return SRF_OK;
}

template <int OP, bool TEX>
static int launch_warp(const float *img, const float *mx, const float *my, const float *mz, float p0, float p1,
                       float p2, const Vol &v, float *out, cudaStream_t s) {
    const int64_t total = v.nxy * v.nz;
    if (!TEX && OP != W_SHIFT_Z) {  // untouched voxels are 0, as the op's memset
        cudaError_t e = cudaMemsetAsync(out, 0, (size_t)total * sizeof(float), s);
        if (e != cudaSuccess) return fail(SRF_ECUDA, "clearing the output: %s", cudaGetErrorString(e));
    }
    auto kern = k_warp<OP, TEX>;
    unsigned blocks = grid_for(kern, total, kBlock);
    kern<<<blocks, kBlock, 0, s>>>(img, mx, my, mz, p0, p1, p2, v, out);
    return check_cuda("warp kernel launch");
}

}  // namespace srf

using namespace srf;

extern "C" {

int srf_deform(const float *image, const float *mx, const float *my, const float *mz,
               const int32_t grid[3], int32_t texture_rule, float *out, void *stream) {
    Vol v; int rc;
    if ((rc = check_vol(grid, v))) return rc;
    if (!image || !mx || !my || !mz || !out) return fail(SRF_EINVAL, "NULL image, field or output");
    cudaStream_t s = (cudaStream_t)stream;
    return texture_rule ? launch_warp<W_DEFORM, true>(image, mx, my, mz, 0, 0, 0, v, out, s)
                        : launch_warp<W_DEFORM, false>(image, mx, my, mz, 0, 0, 0, v, out, s);
}

int srf_shift(const float *image, float mx, float my, float mz, const int32_t grid[3],
              int32_t texture_rule, float *out, void *stream) {
    Vol v; int rc;
    if ((rc = check_vol(grid, v))) return rc;
    if (!image || !out) return fail(SRF_EINVAL, "NULL image or output");
    if (!std::isfinite(mx) || !std::isfinite(my) || !std::isfinite(mz)) return fail(SRF_ENONFINITE, "non-finite shift");
    cudaStream_t s = (cudaStream_t)stream;
    return texture_rule ? launch_warp<W_SHIFT, true>(image, nullptr, nullptr, nullptr, mx, my, mz, v, out, s)
                        : launch_warp<W_SHIFT, false>(image, nullptr, nullptr, nullptr, mx, my, mz, v, out, s);
}

int srf_shift_z(const float *image, float mz, const int32_t grid[3], int32_t texture_rule, float *out,
                void *stream) {
    Vol v; int rc;
    if ((rc = check_vol(grid, v))) return rc;
    if (!image || !out) return fail(SRF_EINVAL, "NULL image or output");
    if (!std::isfinite(mz)) return fail(SRF_ENONFINITE, "non-finite shift");
    cudaStream_t s = (cudaStream_t)stream;
    return texture_rule ? launch_warp<W_SHIFT_Z, true>(image, nullptr, nullptr, nullptr, 0, 0, mz, v, out, s)
                        : launch_warp<W_SHIFT_Z, false>(image, nullptr, nullptr, nullptr, 0, 0, mz, v, out, s);
}

int srf_rotate(const float *image, float cos_phi, float sin_phi, const int32_t grid[3], int32_t texture_rule,
               float *out, void *stream) {
    Vol v; int rc;
    if ((rc = check_vol(grid, v))) return rc;
    if (!image || !out) return fail(SRF_EINVAL, "NULL image or output");
    if (!std::isfinite(cos_phi) || !std::isfinite(sin_phi)) return fail(SRF_ENONFINITE, "non-finite angle");
    cudaStream_t s = (cudaStream_t)stream;
    return texture_rule ? launch_warp<W_ROTATE, true>(image, nullptr, nullptr, nullptr, cos_phi, sin_phi, 0, v, out, s)
                        : launch_warp<W_ROTATE, false>(image, nullptr, nullptr, nullptr, cos_phi, sin_phi, 0, v, out, s);
}

int srf_deform_invert(const float *mx, const float *my, const float *mz, const int32_t grid[3], int32_t iterations,
                      float *out_mx, float *out_my, float *out_mz, void *stream) {
    Vol v; int rc;
    if ((rc = check_vol(grid, v))) return rc;
    if (!mx || !my || !mz || !out_mx || !out_my || !out_mz) return fail(SRF_EINVAL, "NULL field");
    if (iterations < 0 || iterations > 1000) return fail(SRF_EINVAL, "iterations %d out of range (0..1000)", iterations);
    const int64_t total = v.nxy * v.nz;
    unsigned blocks = grid_for(k_deform_invert, total, kBlock);
    k_deform_invert<<<blocks, kBlock, 0, (cudaStream_t)stream>>>(mx, my, mz, v, iterations, out_mx, out_my, out_mz);
    return check_cuda("deform invert kernel launch");
}

}  // extern "C"
