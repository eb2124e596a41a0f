// List-mode ingestion on the GPU: crystal index <-> position, endpoint snapping, and
// histogramming into the triangular crystal-pair sinogram.
//
// * crystal index of a position: srfnef/functions/geometry/pet_ecat_scanner.py:15-60
//   (EcatCrystalPosToIndex): iblock = round(atan2(y, x) / angle_per_block) mod nb,
//   iring = floor((z + axial/2) / (gap + block_z)), iy = round(y_corr / unit_y - 0.5),
//   iz = round(z_corr / unit_z - 0.5); index = iy + iz*s1 + iblock*per_block + iring*per_ring.
//   With float32 positions numpy evaluates atan2, the block division and the ring floor in
//   float32 (Python scalars do not promote), the in-block offsets in float64 (int64 index times
//   a Python float), and rounds half to even; this code follows the same promotions.
// * position of an index: pet_ecat_scanner.py:63-89 (EcatIndexToCrystalPos), float64 then
//   rounded to float32, with numpy's floor-division/modulo semantics for the digit split.
// * snapping: srfnef/functions/data_transform/pet_ecat.py:43-60 (PetEcatListmodeTrans), TOF
//   column kept.
// * sinogram: srfnef/corrections/scattering/listmode2sinogram.py:17-23, 76-85 (change_id +
//   cal_sinogram): bin (hi - 1) * hi / 2 + lo of the ordered pair, float64 weights.
#include "common.cuh"

namespace srf {

struct EcatK {
    double avg_radius, angle_per_block, axial_length, gap, block_y, block_z, unit_y, unit_z;
    int64_t s1, s2, nb, per_block, per_ring, nb_crystals;
};

__device__ __forceinline__ int64_t floordiv(int64_t a, int64_t b) {
    int64_t q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
    return q;
}

__device__ __forceinline__ int64_t pymod(int64_t a, int64_t b) { return a - floordiv(a, b) * b; }

__device__ __forceinline__ int64_t crystal_index(const EcatK &s, float x, float y, float z) {
    const float bq = __fdiv_rn(atan2f(y, x), (float)s.angle_per_block);
    const int64_t iblock = pymod((int64_t)rintf(bq), s.nb);
    const float zr = __fdiv_rn(__fadd_rn(z, (float)(s.axial_length / 2)), (float)(s.gap + s.block_z));
    const int64_t iring = (int64_t)floorf(zr);
    const double ang = (double)iblock * s.angle_per_block;
    const double y_corr = -(double)x * sin(ang) + (double)y * cos(ang) + s.block_y / 2;
    const int64_t iy = (int64_t)rint(y_corr / s.unit_y - 0.5);
    const double z_corr = (double)__fadd_rn(z, (float)(s.axial_length / 2)) - (double)iring * (s.block_z + s.gap);
    const int64_t iz = (int64_t)rint(z_corr / s.unit_z - 0.5);
    return iy + iz * s.s1 + iblock * s.per_block + iring * s.per_ring;
}

__device__ __forceinline__ void crystal_position(const EcatK &s, int64_t ind, float out[3]) {
    const int64_t iy = pymod(ind, s.s1);
    const int64_t iz = pymod(floordiv(ind, s.s1), s.s2);
    const int64_t iblock = pymod(floordiv(floordiv(ind, s.s1), s.s2), s.nb);
    const int64_t iring = floordiv(floordiv(floordiv(ind, s.s1), s.s2), s.nb);
    const double x0 = s.avg_radius;
    const double y0 = ((double)iy + 0.5) * s.unit_y - s.block_y / 2;
    const double th = s.angle_per_block * (double)iblock;
    out[0] = (float)(x0 * cos(th) - y0 * sin(th));
    out[1] = (float)(x0 * sin(th) + y0 * cos(th));
    out[2] = (float)(((double)iz + 0.5) * s.unit_z + (double)iring * (s.gap + s.block_z) - s.axial_length / 2);
}

__global__ void k_snap(const float *__restrict__ lors, int64_t n, int stride, EcatK s,
                       float *__restrict__ out, int out_stride, int64_t *__restrict__ ids) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float *l = lors + i * stride;
        const int64_t a = crystal_index(s, l[0], l[1], l[2]);
        const int64_t b = crystal_index(s, l[3], l[4], l[5]);
        if (ids) {
            ids[2 * i] = a;
            ids[2 * i + 1] = b;
        }
        if (out) {
            float pa[3], pb[3];
            crystal_position(s, a, pa);
            crystal_position(s, b, pb);
            float *o = out + i * out_stride;
            o[0] = pa[0]; o[1] = pa[1]; o[2] = pa[2];
            o[3] = pb[0]; o[4] = pb[1]; o[5] = pb[2];
            for (int c = 6; c < out_stride && c < stride; ++c) o[c] = l[c];
        }
    }
}

__global__ void k_lm2sino(const float *__restrict__ lors, int64_t n, int stride,
                          const float *__restrict__ values, EcatK s, double *__restrict__ sino,
                          int64_t n_bins, unsigned long long *__restrict__ dropped) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float *l = lors + i * stride;
        const int64_t a = crystal_index(s, l[0], l[1], l[2]);
        const int64_t b = crystal_index(s, l[3], l[4], l[5]);
        const int64_t hi = a > b ? a : b, lo = a > b ? b : a;
        const int64_t bin = (hi - 1) * hi / 2 + lo;
        if (lo >= 0 && hi < s.nb_crystals && bin >= 0 && bin < n_bins)
            atomicAdd(sino + bin, (double)(values ? values[i] : 1.0f));
        else if (dropped)
            atomicAdd(dropped, 1ULL);
    }
}

inline int make_ecat(const double p[8], const int64_t shape[3], EcatK &s) {
    for (int k = 0; k < 8; ++k)
        if (!std::isfinite(p[k])) return fail(SRF_ENONFINITE, "scanner parameter %d is not finite", k);
    if (shape[0] <= 0 || shape[1] <= 0 || shape[2] <= 0) return fail(SRF_EGRID, "bad scanner shape");
    s.avg_radius = p[0]; s.angle_per_block = p[1]; s.axial_length = p[2]; s.gap = p[3];
    s.block_y = p[4]; s.block_z = p[5]; s.unit_y = p[6]; s.unit_z = p[7];
    if (!(s.angle_per_block > 0) || !(s.unit_y > 0) || !(s.unit_z > 0) || !(s.gap + s.block_z > 0))
        return fail(SRF_EGRID, "scanner sizes must be positive");
    s.s1 = shape[0]; s.s2 = shape[1]; s.nb = shape[2];
    s.per_block = s.s1 * s.s2;
    s.per_ring = s.per_block * s.nb;
    return SRF_OK;
}

}  // namespace srf

using namespace srf;

extern "C" {

int srf_listmode_snap(const float *lors, int64_t n, int32_t lor_stride, const double scanner[8],
                      const int64_t scanner_shape[4], float *out, int32_t out_stride,
                      int64_t *crystal_ids, void *stream) {
    int rc;
    if ((rc = check_lors(lors, n, lor_stride))) return rc;
    if (!scanner || !scanner_shape) return fail(SRF_EINVAL, "scanner must not be NULL");
    if (out && out_stride < 6) return fail(SRF_EINVAL, "out_stride %d < 6", out_stride);
    EcatK s;
    if ((rc = make_ecat(scanner, scanner_shape, s))) return rc;
    s.nb_crystals = s.per_ring * scanner_shape[3];
    if (n == 0) return ok();
    unsigned blocks = grid_for(k_snap, n, kBlock);
    k_snap<<<blocks, kBlock, 0, (cudaStream_t)stream>>>(lors, n, lor_stride, s, out, out_stride, crystal_ids);
    return check_cuda("snap kernel launch");
}

int srf_lm2sino(const float *lors, int64_t n, int32_t lor_stride, const float *values,
                const double scanner[8], const int64_t scanner_shape[4], double *sino,
                int64_t n_bins, unsigned long long *dropped, void *stream) {
    int rc;
    if ((rc = check_lors(lors, n, lor_stride))) return rc;
    if (!scanner || !scanner_shape || !sino) return fail(SRF_EINVAL, "NULL argument");
    EcatK s;
    if ((rc = make_ecat(scanner, scanner_shape, s))) return rc;
    s.nb_crystals = s.per_ring * scanner_shape[3];
    if (n_bins < 0) return fail(SRF_EINVAL, "negative bin count");
    if (n == 0) return ok();
    unsigned blocks = grid_for(k_lm2sino, n, kBlock);
    k_lm2sino<<<blocks, kBlock, 0, (cudaStream_t)stream>>>(lors, n, lor_stride, values, s, sino, n_bins, dropped);
    return check_cuda("lm2sino kernel launch");
}

}  // extern "C"
