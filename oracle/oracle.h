/* CPU oracle for the list-mode reconstruction hot path. TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of srfnef's Siddon projector / backprojector (non-TOF and TOF) and of its
 * single-scatter simulation, used by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg, as the reference the GPU results are compared with. The product (srf_gb300/)
 * never links, loads or calls it.
 *
 * Parity pin: siddon_oracle.c is checked bit-for-bit against the reference's own device functions
 * compiled on the host (oracle/_ref, see Makefile) and against the committed golden vectors
 * under tests/golden/. sss_oracle.c is checked against the reference's Python SSS run under
 * stub numba/tensorflow modules on small cases (tests/golden/make_golden.py).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* rule sets: which of the reference's four device functions the traversal follows */
#define OR_RULES_PROJ 0 /* project_device   (siddon.cu.cc:12-338 / siddon_tof.cu.cc:14-367) */
#define OR_RULES_BACK 1 /* backproject_device (siddon.cu.cc:342-656 / siddon_tof.cu.cc:371-707) */
/* actions */
#define OR_GATHER 0  /* out[i] = sum image * weight           */
#define OR_SCATTER 1 /* image += value[i] * weight             */

/* Generic traversal over n LORs. lors: row-major with `stride` floats per LOR (x1 y1 z1 x2 y2 z2 ...).
 * tof == NULL selects the non-TOF functions; otherwise tof[i*tof_stride] is the TOF value (mm).
 * tof_nsigma > 0 restricts the TOF kernel to slabs with t2 <= tof_nsigma^2 (0 = reference-exact).
 * image: flat, x fastest. Gather writes out[i] (the projections' memset is included). Scatter adds
 * into image (caller zeroes it). Returns the number of (LOR, voxel) pairs visited. */
int64_t or_trace(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                 float tof_bin, float tof_sigma2, float tof_nsigma, const int *grid,
                 const float *center, const float *size, int rules, int action,
                 const float *values, float *image_or_null, const float *image_in, float *out);

/* or_trace over `nthreads` OpenMP threads (CPU baseline timing) */
int64_t or_trace_mt(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                    float tof_bin, float tof_sigma2, float tof_nsigma, const int *grid,
                    const float *center, const float *size, int rules, int action,
                    const float *values, float *image_or_null, const float *image_in, float *out,
                    int nthreads);

/* convenience wrappers with the reference op semantics */
int64_t or_projection(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                      float tof_bin, float tof_sigma2, float tof_nsigma, const int *grid,
                      const float *center, const float *size, const float *image, float *out);
int64_t or_backprojection(const float *lors, int64_t n, int stride, const float *tof,
                          int tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                          const int *grid, const float *center, const float *size,
                          const float *values, float *image);
/* exact adjoint of or_projection: projector rules, scatter action */
int64_t or_projection_adjoint(const float *lors, int64_t n, int stride, const float *tof,
                              int tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                              const int *grid, const float *center, const float *size,
                              const float *values, float *image);

/* Single-scatter simulation core (scatter_fraction.py:40-136, kn_formula.py:6-46).
 * Per LOR pair k (crystal ids a=pairs[2k], b=pairs[2k+1]) writes the raw loop_all_s sum to
 * scatter[k] and get_scale to scale[k], before the host post-scaling of scatter_fraction.py:27-36. */
void or_sss(const int32_t *pairs, int64_t n_pairs, const float *crystal_pos, int n_crystals,
            const float *scatter_pos, int n_scatter, const float *sumup_emission,
            const float *atten, const float *umap, const int *umap_shape,
            const float *umap_size, int nb_crystals_per_ring, int nb_blocks_per_ring,
            const int *grid_block, int low_energy, int high_energy, double resolution_sqrt511,
            double *scatter, double *scale);

#ifdef __cplusplus
}
#endif
