/* srf_gb300 -- C ABI of the GB300 (sm_103a) list-mode PET reconstruction hot path.
 *
 * Drop-in for the CUDA side of srfnef's Siddon TF ops and their callers. Every entry point takes
 * plain device pointers, host-side sizes/parameters and a cudaStream_t (as void*, NULL = legacy
 * default stream), launches asynchronously on that stream and returns an int status:
 *   SRF_OK (0), or one of the SRF_E* codes below; srf_last_error() gives a message for the
 *   calling thread. No entry point allocates device memory, copies parameters device->host or
 *   synchronises, unless its comment says so.
 *
 * Conventions shared by the projector family:
 *   lors        N LORs, row-major, `lor_stride` floats per LOR (>= 6): x1 y1 z1 x2 y2 z2 [...] in mm.
 *   tof         TOF values in mm (d2 - d1), tof[i * tof_stride]; srfnef passes column 6 of its
 *               (N, 7) Lors array (srfnef/data/lors.py:20-22), i.e. tof = lors + 6, stride 7.
 *   grid        {nx, ny, nz}; center {cx, cy, cz} and size {sx, sy, sz} in mm (the image's
 *               ``shape``, ``center`` and ``size``; srfnef passes them as three small tensors).
 *   image       float32 voxels addressed ix*st[0] + iy*st[1] + iz*st[2] (element strides).
 *               srfnef's ops take the x-fastest array st = {1, nx, nx*ny}.
 *   image_t     optional second view of the same voxels used for y-dominant LORs; a y-fastest
 *               copy (st = {ny, 1, nx*ny}) makes those LORs' memory accesses coalesced. NULL: the
 *               first view serves all LORs. For backprojections image_t is a second accumulator
 *               that receives the y-dominant LORs; the result is image + image_t (see
 *               srf_fold_views), which the caller zeroes beforehand like image.
 *   tof_nsigma  0 reproduces the reference's untruncated Gaussian; > 0 drops slabs whose TOF
 *               argument exceeds tof_nsigma standard deviations (not in the reference).
 */
#ifndef SRF_GB300_H
#define SRF_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SRF_OK 0
#define SRF_EINVAL 1      /* null pointer, negative count, bad stride          */
#define SRF_EGRID 2       /* non-positive or oversized grid, bad size/strides  */
#define SRF_ENONFINITE 3  /* non-finite center/size/TOF parameter              */
#define SRF_ECUDA 4       /* CUDA launch or runtime error                      */
#define SRF_ERANGE 5      /* a size beyond a documented limit                  */

/* Message for the last non-zero status returned on this thread ("" if none). */
const char *srf_last_error(void);

/* ABI version (major*100 + minor). */
int srf_version(void);

/* Lanes per LOR used by the traversal kernels (8, 16 or 32; default 32). Process-wide. */
int srf_set_group_lanes(int lanes);

/* Lanes per LOR and slabs per lane per chunk of the fused OSEM kernel (2 or 4; default 4).
 * Process-wide; chosen by srf_gb300.autotune. */
int srf_set_tuning(int lanes, int slabs_per_lane);

/* ------------------------------------------------------------------ projector family */

/* p[i] = sum_v A_iv image_v, non-TOF.
 * Replaces the TF op "Projection" (srfnef/cc/siddon/siddon.cc:11-21, Compute :48-102) and its
 * launcher projection() (srfnef/cc/siddon/siddon.cu.cc:706-728). out[N] is fully written (the
 * op's memset is included). */
int srf_projection(const float *lors, int64_t n, int32_t lor_stride,
                   const float *image, const int64_t image_strides[3],
                   const float *image_t, const int64_t image_t_strides[3],
                   const int32_t grid[3], const float center[3], const float size[3],
                   float *out, void *stream);

/* image += A^T values, non-TOF (backprojector rules: no endpoint/steep skip, no 1/L^2).
 * Replaces "Backprojection" (siddon.cc:23-35, Compute :104-161) and backprojection()
 * (siddon.cu.cc:731-753). Accumulates; the op's memset is the caller's zero fill. */
int srf_backprojection(const float *lors, int64_t n, int32_t lor_stride, const float *values,
                       float *image, const int64_t image_strides[3],
                       float *image_t, const int64_t image_t_strides[3],
                       const int32_t grid[3], const float center[3], const float size[3],
                       void *stream);

/* TOF projection. Replaces "ProjectionTof" (srfnef/cc/siddon_tof/siddon_tof.cc:11-24,
 * Compute :56-119) and projection() (srfnef/cc/siddon_tof/siddon_tof.cu.cc:761-785). */
int srf_projection_tof(const float *lors, int64_t n, int32_t lor_stride,
                       const float *tof, int32_t tof_stride,
                       float tof_bin, float tof_sigma2, float tof_nsigma,
                       const float *image, const int64_t image_strides[3],
                       const float *image_t, const int64_t image_t_strides[3],
                       const int32_t grid[3], const float center[3], const float size[3],
                       float *out, void *stream);

/* TOF backprojection. Replaces "BackprojectionTof" (siddon_tof.cc:26-41, Compute :121-188) and
 * backprojection() (siddon_tof.cu.cc:787-812). Accumulates. */
int srf_backprojection_tof(const float *lors, int64_t n, int32_t lor_stride,
                           const float *tof, int32_t tof_stride,
                           float tof_bin, float tof_sigma2, float tof_nsigma,
                           const float *values,
                           float *image, const int64_t image_strides[3],
                           float *image_t, const int64_t image_t_strides[3],
                           const int32_t grid[3], const float center[3], const float size[3],
                           void *stream);

/* srf_backprojection_tof without any device allocation. No counterpart in the reference.
 * For callers that cannot call cudaMalloc (a plugin inside a framework that owns the device memory,
 * or an acquisition service with a fixed device-memory reservation): the y-dominant LORs are
 * accumulated in a static device array of SRF_NOALLOC_MAX_VOXELS floats (18 MiB, held by every GPU
 * that loads the library) and folded into `image` (x-fastest, strides {1, nx, nx*ny}), which is
 * accumulated into like srf_backprojection_tof. Grids with more voxels return SRF_ERANGE. The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress); make that first call
 * before any stream capture. The address is cached per device ordinal for the process, which
 * assumes the runtime's primary context: no cudaDeviceReset and no second driver-API context on the
 * device afterwards. All calls share the array: calls that overlap on the GPU race. */
#define SRF_NOALLOC_MAX_VOXELS 4718592
int srf_backprojection_tof_noalloc(const float *lors, int64_t n, int32_t lor_stride,
                                   const float *tof, int32_t tof_stride,
                                   float tof_bin, float tof_sigma2, float tof_nsigma,
                                   const float *values, float *image,
                                   const int32_t grid[3], const float center[3], const float size[3],
                                   void *stream);

/* image += P^T values for the projector P of srf_projection (tof == NULL) or
 * srf_projection_tof: the exact adjoint (projector rules, 1/L^2 weights), used as the backward
 * of the differentiable projector. The reference's backprojector is not this adjoint. */
int srf_projection_adjoint(const float *lors, int64_t n, int32_t lor_stride,
                           const float *tof, int32_t tof_stride,
                           float tof_bin, float tof_sigma2, float tof_nsigma,
                           const float *values,
                           float *image, const int64_t image_strides[3],
                           float *image_t, const int64_t image_t_strides[3],
                           const int32_t grid[3], const float center[3], const float size[3],
                           void *stream);

/* srf_projection / srf_projection_tof and srf_projection_adjoint for n_images (1..8) images that
 * share one grid and one set of LORs (no counterpart in the reference: the batched forward and
 * gradient of the differentiable projector). Image b starts batch_stride elements after image b-1
 * in each layout given (images and the optional images_t); LOR values / outputs are n_images rows
 * of n at row stride out_stride / values_stride. tof == NULL selects the non-TOF projector. Each
 * LOR is set up and traversed once for all images. */
int srf_projection_batch(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                         int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                         int32_t n_images, int64_t batch_stride, const float *images,
                         const int64_t image_strides[3], const float *images_t,
                         const int64_t image_t_strides[3], const int32_t grid[3],
                         const float center[3], const float size[3], float *out, int64_t out_stride,
                         void *stream);
int srf_projection_adjoint_batch(const float *lors, int64_t n, int32_t lor_stride, const float *tof,
                                 int32_t tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                                 int32_t n_images, const float *values, int64_t values_stride,
                                 float *images, int64_t batch_stride, const int64_t image_strides[3],
                                 float *images_t, const int64_t image_t_strides[3], const int32_t grid[3],
                                 const float center[3], const float size[3], void *stream);

/* *count += number of (LOR, voxel) weight visits the projector (rules 0) or backprojector
 * (rules 1) rule set makes for these LORs (tof == NULL: non-TOF rules). `count` is a device
 * unsigned 64-bit counter. These are the "LOR-voxel updates" of the throughput metric; the CPU
 * oracle counts the same visits. No counterpart in the reference. */
int srf_count_pairs(const float *lors, int64_t n, int32_t lor_stride,
                    const float *tof, int32_t tof_stride,
                    float tof_bin, float tof_sigma2, float tof_nsigma, int32_t rules,
                    const int32_t grid[3], const float center[3], const float size[3],
                    unsigned long long *count, void *stream);

/* dst[v] += src_t[v] for two views of one grid (folds a y-fastest accumulator into dst). */
int srf_fold_views(float *dst, const int64_t dst_strides[3], const float *src,
                   const int64_t src_strides[3], const int32_t grid[3], void *stream);

/* dst = src re-laid out (any strides to any strides), e.g. x-fastest -> y-fastest copy. */
int srf_copy_view(float *dst, const int64_t dst_strides[3], const float *src,
                  const int64_t src_strides[3], const int32_t grid[3], void *stream);

/* ------------------------------------------------------------------ MLEM / OSEM */

/* Ratio rules of the reference's update loops:
 *  SRF_RATIO_DIV_NO_NAN : r = tf.div_no_nan(y, p + eps)  (MlemFull eps=0, mlem_full.py:68;
 *                                                          MlemFullTof eps=1e-5, mlem_full_tof.py:64)
 *  SRF_RATIO_PLAIN      : r = y / (p + eps)               (Mlem eps=mean(y)*1e-8, mlem.py:41-42;
 *                                                          OsemFull eps=1e-8, osem_full.py:75-76) */
#define SRF_RATIO_DIV_NO_NAN 0
#define SRF_RATIO_PLAIN 1

/* One fused subset step of list-mode MLEM/OSEM for the LORs given:
 *   p_i = (A x)_i ; r_i = rule(y_i, p_i + add_i) ; bp += A_bp^T r
 * in a single pass over the LORs (each LOR's projection, ratio and backprojection are computed
 * back to back; p and r never reach memory). tof == NULL: non-TOF projector/backprojector pair of
 * srf_projection/srf_backprojection; otherwise the TOF pair. y == NULL means y_i = 1 (list mode).
 * x/x_t are read (x_t optional, y-fastest), bp/bp_t accumulate (bp_t optional, folded by
 * srf_osem_update). add (optional) is an additive expected count per LOR, e.g. a scatter estimate
 * (not in the reference; NULL = 0). loglik (optional, device double) += sum_i y_i log(p_i + add_i + eps).
 * Replaces the per-iteration bodies of mlem_full.py:66-70, mlem_full_tof.py:62-67,
 * mlem.py:39-43 and osem_full.py:74-77 up to the image update. */
int srf_osem_subset(const float *lors, int64_t n, int32_t lor_stride,
                    const float *tof, int32_t tof_stride,
                    float tof_bin, float tof_sigma2, float tof_nsigma,
                    const float *y, const float *add, int32_t ratio_rule, float eps,
                    const float *x, const float *x_t, float *bp, float *bp_t,
                    const int32_t grid[3], const float center[3], const float size[3],
                    double *loglik, void *stream);

/* Multiplicative update on x-fastest images (x_t/bp_t y-fastest, both optional):
 *   x <- (x * (bp + bp_t)) / e,  e = emap (guard_zero: emap == 0 -> 1e8, mlem_full_tof.py:56-58)
 * then x_t <- x (y-fastest copy) and bp, bp_t <- 0, ready for the next subset. */
int srf_osem_update(float *x, float *x_t, float *bp, float *bp_t, const float *emap,
                    int32_t guard_zero, const int32_t grid[3], void *stream);

/* Many independent studies per launch (not in the reference). One descriptor per study, in
 * DEVICE memory; images x/bp x-fastest ({1, nx, nx*ny}), x_t/bp_t y-fastest ({ny, 1, nx*ny}) or
 * both NULL; emap (x-fastest) is read by srf_osem_update_batch. Descriptors cannot be checked on
 * the host (no device-to-host copies); the kernels skip a study whose descriptor fails the
 * host-side checks of srf_osem_subset (grid range, NULL pointers, stride). */
typedef struct srf_study {
    const float *lors;    /* this subset's LORs of the study */
    int64_t n;
    int32_t lor_stride;
    int32_t tof_stride;   /* TOF values tof[i * tof_stride] (used when use_tof) */
    const float *tof;
    const float *y;       /* NULL: y_i = 1 */
    float *x, *x_t, *bp, *bp_t;
    const float *emap;
    int32_t grid[3];
    float center[3];
    float size[3];
} srf_study;

/* srf_osem_subset for every study at once: a persistent kernel walks all studies' 32-LOR batches.
 * batch_offsets (device, n_studies + 3 int64): study s owns batches [off[s], off[s + 1]),
 * off[s + 1] - off[s] = ceil(n_s / 32); total_batches = off[n_studies]. The two entries after
 * off[n_studies] are the kernel's work counters: zero them once when the array is made; every
 * launch leaves them at zero again. Launches sharing one array must be ordered (one stream). */
int srf_osem_subset_batch(const srf_study *studies, int32_t n_studies,
                          const int64_t *batch_offsets, int64_t total_batches, int32_t use_tof,
                          float tof_bin, float tof_sigma2, float tof_nsigma, int32_t ratio_rule,
                          float eps, double *loglik, void *stream);

/* srf_osem_update for every study at once. tile_offsets (device, n_studies + 1): study s owns
 * tiles [off[s], off[s + 1]), ceil(nx/32) * ceil(ny/32) * nz of them. */
int srf_osem_update_batch(const srf_study *studies, int32_t n_studies, const int64_t *tile_offsets,
                          int64_t total_tiles, int32_t guard_zero, void *stream);

/* ------------------------------------------------------------------ list-mode ingestion */

/* Scanner description for the list-mode kernels (PetEcatScanner, srfnef/geometry/pet_ecat_scanner.py):
 *   scanner[8]       = {average_radius, angle_per_block, axial_length, gap, block_size_y,
 *                       block_size_z, unit_size_y, unit_size_z}
 *   scanner_shape[4] = {block_shape_y, block_shape_z, nb_blocks_per_ring, nb_rings} */

/* Crystal ids of both endpoints (crystal_ids[2i], [2i+1], optional) and/or the LORs with both
 * endpoints snapped to crystal centres (out, out_stride floats per row; columns past 6 copied,
 * e.g. the TOF value). EcatCrystalPosToIndex + EcatIndexToCrystalPos + PetEcatListmodeTrans
 * (srfnef/functions/geometry/pet_ecat_scanner.py:15-89, functions/data_transform/pet_ecat.py:43-60). */
int srf_listmode_snap(const float *lors, int64_t n, int32_t lor_stride, const double scanner[8],
                      const int64_t scanner_shape[4], float *out, int32_t out_stride,
                      int64_t *crystal_ids, void *stream);

/* sino[bin] += values[i] (1 when NULL) with bin = (hi - 1) * hi / 2 + lo of the ordered crystal
 * pair: lm2sino / cal_sinogram (srfnef/corrections/scattering/listmode2sinogram.py:17-23, 76-85).
 * sino: float64, n_bins = n_crystals (n_crystals - 1) / 2. Events whose bin falls outside are
 * counted in *dropped (device, optional). */
int srf_lm2sino(const float *lors, int64_t n, int32_t lor_stride, const float *values,
                const double scanner[8], const int64_t scanner_shape[4], double *sino,
                int64_t n_bins, unsigned long long *dropped, void *stream);

/* out[i] = exp(-(P mu)_i * L_i^2 / (size[0] / grid[0])) (UmapProject, attenuation_correct.py:31-40),
 * or, with values != NULL, out[i] = values[i] / exp(-(...)) (AttenuationCorrect, :16-28): the
 * non-TOF projection of the mu map and its epilogue in one pass. */
int srf_attenuation(const float *lors, int64_t n, int32_t lor_stride, const float *umap,
                    const int64_t umap_strides[3], const int32_t grid[3], const float center[3],
                    const float size[3], const float *values, float *out, void *stream);

/* ------------------------------------------------------------------ image warping */
/* Replace the TF ops Deform, Shift, ShiftZ, Rotate (srfnef/cc/deform/deform.cc:12-51, kernels
 * deform.cu.cc:13-174) and their texture-library twins with DeformInvert (deform_tex.cc,
 * deform_tex.cu.cc:15-420), called by srfnef/ops/deform_mixins.py:18-89. Images and
 * displacement fields (in voxels) are x-fastest (index ix + iy*nx + iz*nx*ny), out is written
 * in full. texture_rule != 0: the texture library's rules (clamped linear reads at position + 0.5,
 * Shift/ShiftZ sampling at i - m), with FP32 interpolation weights; 0: the plain library's
 * (voxels whose neighbourhood leaves the image are 0). Grid and parameters are passed by value;
 * the reference copies the grid from the device on every call. */
int srf_deform(const float *image, const float *mx, const float *my, const float *mz,
               const int32_t grid[3], int32_t texture_rule, float *out, void *stream);
int srf_shift(const float *image, float mx, float my, float mz, const int32_t grid[3],
              int32_t texture_rule, float *out, void *stream);
int srf_shift_z(const float *image, float mz, const int32_t grid[3], int32_t texture_rule,
                float *out, void *stream);
int srf_rotate(const float *image, float cos_phi, float sin_phi, const int32_t grid[3],
               int32_t texture_rule, float *out, void *stream);
/* The inverse displacement field (deform_tex.cu.cc:78-100): per voxel, `iterations` (0..1000;
 * the reference uses 30) fixed-point steps x <- -mx(x + i), y <- -my(.), z <- -mz(.) from 0. */
int srf_deform_invert(const float *mx, const float *my, const float *mz, const int32_t grid[3],
                      int32_t iterations, float *out_mx, float *out_my, float *out_mz, void *stream);

/* ------------------------------------------------------------------ sensitivity image */

/* emap += sum over all ordered crystal pairs of the non-TOF backprojection of 1, generated on
 * the device from a crystal table in srfnef's 'block-full' order (n_blocks * m rows, m crystals
 * per block column; pairs (i*m+a, j*m+b) for all i, j, a, b, self pairs included), i.e.
 * EcatEmapGenerator('block-full') (srfnef/functions/emap_generator.py:77-111) without the
 * 2304 host-built LOR arrays. emap/emap_t as the backprojection views. */
int srf_emap_block_full(const float *crystal_table, int32_t n_blocks, int32_t m,
                        float *emap, const int64_t emap_strides[3],
                        float *emap_t, const int64_t emap_t_strides[3],
                        const int32_t grid[3], const float center[3], const float size[3],
                        void *stream);

/* ------------------------------------------------------------------ single-scatter simulation */

/* Raw single-scatter sums for crystal pairs (loop_all_lors / loop_all_s / get_scale of
 * srfnef/corrections/scattering/scatter_fraction/scatter_fraction.py:40-136 and fkn of
 * kn_formula.py:6-20, including the reference's whole-degree angle quantisation and its use of
 * the angle inside fkn):
 *   pairs          int32 (a, b) crystal ids, n_pairs rows
 *   crystal_pos    float32 (n_crystals, 3); scatter_pos float32 (n_scatter, 3), n_scatter <= 12288
 *   sumup_emission, atten  float32 (n_crystals, n_scatter), crystal-major, n_crystals * n_scatter < 2^31
 *   umap           float32 (shape0, shape1, shape2) C order, umap_size mm
 * Outputs scatter[k] and scale[k] before the host scaling of scatter_fraction.py:27-36. */
int srf_sss(const int32_t *pairs, int64_t n_pairs, const float *crystal_pos, int32_t n_crystals,
            const float *scatter_pos, int32_t n_scatter, const float *sumup_emission,
            const float *atten, const float *umap, const int32_t umap_shape[3],
            const float umap_size[3], int32_t nb_crystals_per_ring, int32_t nb_blocks_per_ring,
            const int32_t grid_block[3], int32_t low_energy, int32_t high_energy,
            float resolution, float *scatter, float *scale, void *stream);

/* ------------------------------------------------------------------ L2 calibration */
/* No counterpart in the reference: best-case L2 throughput for 4-byte words, the denominators of
 * the gather and atomic rooflines. mode 0: reps passes of loads over buf[0, n) (sink receives
 * srf_calib_sink_size() floats); mode 1: reps passes of buf[i] += 1 as reductions. Keep n * 4 B
 * well below the L2 size and time the call on `stream`. */
int srf_calib_l2(float *buf, int64_t n, int32_t reps, int32_t mode, float *sink, void *stream);
int srf_calib_sink_size(void);

/* ------------------------------------------------------------------ scatter surrogate network */
/* BF16 3-D U-Net building blocks with FP32 accumulation (not in the reference). Activations are
 * NDHWC bfloat16 described by int32[6] = {n, d, h, w, channel_stride, channel_offset} so a layer
 * reads or writes a channel slice of a wider buffer. Weights are [Cout][27][Cin] bfloat16. */

/* y = act(b + conv3x3x3(x, w)), pad 1; relu != 0 applies max(., 0). Cin, Cout multiples of 16.
 * yf (optional) receives the FP32 values. Runs on the tensor cores (mma.sync BF16). */
int srf_conv3d_fwd(const void *x, const int32_t xs[6], int32_t cin, const void *w, const float *bias,
                   int32_t cout, int32_t relu, void *y, const int32_t ys[6], float *yf, void *stream);
/* Kernels of srf_conv3d_fwd, process-wide, read at launch. mode 1 (the default): its
 * 128-voxel x 32-channel tiles run on tcgen05.mma with the accumulator in tensor memory; 2: in
 * addition, batch-1 layers with W >= 96 and Cout = 32 on the halo-tile tcgen05 kernel, halos
 * loaded by the threads (cp.async); 3: the same with the halos loaded by TMA; 0: mma.sync only. */
int srf_set_conv_tc(int32_t mode);
/* *status = 1 if a tcgen05 convolution gave up waiting for its tensor-core work (bounded waits),
 * else 0. Synchronises with the device. */
int srf_conv_tc_status(int32_t *status);
/* *path = the kernel of the last srf_conv3d_fwd launch: 0 mma.sync 64 x 64, 1 mma.sync 128 x 32,
 * 2 tcgen05 128 x 32 (gathered K steps), 3 tcgen05 on TMA halo tiles, 4 mma.sync split-K,
 * 5 tcgen05 on cp.async halo tiles; -1 before the first. */
int srf_conv_last_path(int32_t *path);
/* dw[co][tap][ci] += sum_v dy[v, co] x[v + tap - 1, ci] (FP32 accumulation). */
int srf_conv3d_wgrad(const void *x, const int32_t xs[6], int32_t cin, const void *dy, const int32_t ds[6],
                     int32_t cout, float *dw, void *stream);
/* wf[ci][26 - tap][co] = w[co][tap][ci]: weights of the data-gradient convolution. */
int srf_conv3d_flip_weights(const void *w, int32_t cout, int32_t cin, void *wf, void *stream);
/* g = 0 where y <= 0 (ReLU backward from the layer output). */
int srf_cnn_relu_bwd(void *g, const int32_t gs[6], const void *y, const int32_t ys[6], int32_t c, void *stream);
/* db[c] += sum_v g[v, c]. */
int srf_cnn_bias_grad(const void *g, const int32_t gs[6], int32_t c, float *db, void *stream);
/* 2x2x2 average pooling fine -> coarse (adjoint: coarse gradient -> fine gradient). */
int srf_cnn_pool2(const void *fine, const int32_t fs[6], void *coarse, const int32_t cs[6], int32_t c,
                  int32_t adjoint, void *stream);
/* nearest 2x upsampling coarse -> fine (adjoint: fine gradient summed into coarse). */
int srf_cnn_upsample2(const void *coarse, const int32_t cs[6], void *fine, const int32_t fs[6], int32_t c,
                      int32_t adjoint, void *stream);
/* Sub-voxel 1x1x1 head: 8 FP32 outputs per coarse voxel (z, y, x), output q = 4i + 2j + k written
   to fine voxel (2z + i, 2y + j, 2x + k) of out (n, fine[0], fine[1], fine[2]), fine <= 2 x coarse:
   out = b[q] + sum_c x[v, c] w[q * c + c']. With gout != NULL: gx (optional) = data gradient,
   gw[8][c] and gb[8] accumulate the parameter gradients. */
int srf_cnn_head8(const void *x, const int32_t xs[6], int32_t c, const float *w, const float *b, float *out,
                  const int32_t fine[3], const float *gout, void *gx, const int32_t gs[6], float *gw,
                  float *gb, void *stream);
/* dst slice += src slice. */
int srf_cnn_add(void *dst, const int32_t ds[6], const void *src, const int32_t ss[6], int32_t c, void *stream);
/* *loss += (1/n_samples) sum_s sum_i m (p - t)^2 inv_den[s] (FP64); grad = its gradient,
   2 m (p - t) inv_den[s] / n_samples. */
int srf_cnn_rel_mse(const float *pred, const float *target, const float *mask, const float *inv_den,
                    int64_t per_sample, int32_t n_samples, float *grad, double *loss, void *stream);
/* Adam step on FP32 parameters, refreshing an optional BF16 copy. */
int srf_cnn_adam(float *w, float *m, float *v, const float *g, void *bf16_copy, int64_t n, float lr,
                 float b1, float b2, float eps, int32_t step, void *stream);

/* ------------------------------------------------------------------ surrogate spot check */
/* No counterpart in the reference: the spot-check correction of the network's scatter sinogram.
 * pred: the estimate over nbins bins; bins[0..n), ref[0..n): the spot-check samples (bin, SSS
 * value); phi: k <= 12 basis rows of nbins values each (row j at phi + j * nbins).
 * beta minimises, over the even samples s, sum (ref[s] - pred[b] * sum_j beta_j phi_j[b])^2 with
 * b = bins[s], plus ridge * (trace / k) * |beta|^2 of the normal matrix (FP64 normal equations,
 * Cholesky); beta = e0 when that matrix is zero or not positive definite. Samples whose bin lies
 * outside [0, nbins) are left out. out (k + 2 floats): beta, then the relative L2 difference of
 * the corrected prediction from ref over the odd samples, then the same for the uncorrected one. */
int srf_spot_fit(const float *pred, int64_t nbins, const int64_t *bins, const float *ref, int32_t n,
                 const float *phi, int32_t k, double ridge, float *out, void *stream);
/* x[i] *= sum_j beta[j] * phi[j * n + i], beta (k <= 12 values) and phi on the device. */
int srf_scale_by_basis(float *x, int64_t n, const float *phi, int32_t k, const float *beta, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SRF_GB300_H */
