/* CPU restatement of srfnef's single-scatter simulation core. TEST INFRASTRUCTURE ONLY.
 *
 * Follows corrections/scattering/scatter_fraction/scatter_fraction.py and kn_formula.py:
 *   loop_all_lors  scatter_fraction.py:40-61   one LOR pair (a, b) per work item
 *   loop_all_s     scatter_fraction.py:70-91   sum over scatter points S
 *   get_scale      scatter_fraction.py:64-67   (|AB| / project_area(A, B))^2
 *   eff_with_scatter scatter_fraction.py:103-109 integer energy window, step 5 keV
 *   project_area   scatter_fraction.py:112-119
 *   get_block_theta scatter_fraction.py:122-131
 *   fkn            kn_formula.py:6-20   (receives the angle where the formula expects a cosine)
 *   get_scatter_cos_theta kn_formula.py:36-41 (angle quantised down to whole degrees)
 * The reference runs these as numba.cuda kernels whose scalar arithmetic promotes to float64;
 * this restatement evaluates everything in double from the float32 inputs.
 * One deliberate difference: the acos argument of the scatter angle is clamped to [-1, 1]
 * (the reference yields NaN there, which its int() conversion turns into an undefined value).
 */
#include <math.h>
#include <stdint.h>

#include "oracle.h"

static double dist3(double x1, double y1, double z1, double x2, double y2, double z2) {
    return sqrt((x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2) + (z1 - z2) * (z1 - z2));
}

static double block_theta(int ncpr, int nbpr, const int *grid_block, const float *p) {
    const double norm = dist3(p[0], p[1], p[2], 0, 0, 0);
    double th = acos(p[0] / norm) / M_PI * 180.0;
    if (p[1] < 0) th = 360.0 - th;
    double fixed = fmod(th + 180.0 / ncpr * grid_block[1], 360.0);
    if (fixed < 0) fixed += 360.0;
    const double id_block = floor(fixed / 360.0 * nbpr);
    return id_block / nbpr * 2.0 * M_PI;
}

/* cos-weighted area of the LOR pa->pb seen by the block of pb */
static double project_area(int ncpr, int nbpr, const int *grid_block, const float *pa,
                           const float *pb) {
    const double tn = block_theta(ncpr, nbpr, grid_block, pb);
    return ((pb[0] - pa[0]) * cos(tn) + (pb[1] - pa[1]) * sin(tn)) /
           dist3(pa[0], pa[1], pa[2], pb[0], pb[1], pb[2]);
}

/* whole-degree scatter angle in radians */
static double scatter_angle(const float *A, const float *S, const float *B) {
    const double ab = dist3(A[0], A[1], A[2], B[0], B[1], B[2]);
    const double as = dist3(A[0], A[1], A[2], S[0], S[1], S[2]);
    const double sb = dist3(S[0], S[1], S[2], B[0], B[1], B[2]);
    double arg = -(as * as + sb * sb - ab * ab) / (2 * as * sb);
    if (arg > 1.0) arg = 1.0;
    if (arg < -1.0) arg = -1.0;
    return (double)(int)(acos(arg) / M_PI * 180.0) / 180.0 * M_PI;
}

static double eff_with_scatter(int low, int high, double energy, double res) {
    double eff = 0.0;
    for (int e = low; e < high; e += 5) eff += exp(-((double)e - energy) * ((double)e - energy) / 2.0 / (res * res));
    return eff;
}

static double fkn(double angle, const float *S, const float *umap, const int *shape,
                  const float *size) {
    const int g0 = (int)((S[0] / (double)size[0] + 0.5) * shape[0]);
    const int g1 = (int)((S[1] / (double)size[1] + 0.5) * shape[1]);
    const int g2 = (int)((S[2] / (double)size[2] + 0.5) * shape[2]);
    const double c = angle;
    const double diff = 1.0 / ((2.0 - c) * (2.0 - c)) *
                        ((1.0 + c * c) / 2.0 + (1.0 - c) * (1.0 - c) / 2.0 / (2.0 - c));
    const double sigma = M_PI * (40.0 / 9.0 - 3.0 * log(3.0));
    return diff / sigma * umap[((int64_t)g0 * shape[1] + g1) * shape[2] + g2];
}

void or_sss(const int32_t *pairs, int64_t n_pairs, const float *crystal_pos, int n_crystals,
            const float *scatter_pos, int n_scatter, const float *sumup_emission,
            const float *atten, const float *umap, const int *umap_shape,
            const float *umap_size, int nb_crystals_per_ring, int nb_blocks_per_ring,
            const int *grid_block, int low_energy, int high_energy, double res,
            double *scatter, double *scale) {
    (void)n_crystals;
    for (int64_t k = 0; k < n_pairs; ++k) {
        const int a = pairs[2 * k], b = pairs[2 * k + 1];
        const float *A = crystal_pos + 3 * (int64_t)a;
        const float *B = crystal_pos + 3 * (int64_t)b;
        const float *ema = sumup_emission + (int64_t)a * n_scatter;
        const float *emb = sumup_emission + (int64_t)b * n_scatter;
        const float *ata = atten + (int64_t)a * n_scatter;
        const float *atb = atten + (int64_t)b * n_scatter;
        double acc = 0.0;
        for (int i = 0; i < n_scatter; ++i) {
            const float *S = scatter_pos + 3 * (int64_t)i;
            const double angle = scatter_angle(A, S, B);
            const double cos_theta = cos(angle);
            const double e_sc = 511.0 / (2.0 - cos_theta);
            const double Ia = ata[i] * exp(log((double)atb[i]) / e_sc * 511.0) * ema[i];
            const double Ib = exp(log((double)ata[i]) / e_sc * 511.0) * atb[i] * emb[i];
            const double dsa = dist3(S[0], S[1], S[2], A[0], A[1], A[2]);
            const double dsb = dist3(S[0], S[1], S[2], B[0], B[1], B[2]);
            acc += project_area(nb_crystals_per_ring, nb_blocks_per_ring, grid_block, S, A) *
                   eff_with_scatter(low_energy, high_energy, e_sc, res) *
                   project_area(nb_crystals_per_ring, nb_blocks_per_ring, grid_block, S, B) *
                   fkn(angle, S, umap, umap_shape, umap_size) * (Ia + Ib) / (dsa * dsa) /
                   (dsb * dsb);
        }
        scatter[k] = acc;
        const double area = project_area(nb_crystals_per_ring, nb_blocks_per_ring, grid_block, A, B);
        const double dab = dist3(A[0], A[1], A[2], B[0], B[1], B[2]);
        scale[k] = (dab / area) * (dab / area);
    }
}
