/* CPU restatement of srfnef's Siddon-style projector and backprojector. TEST INFRASTRUCTURE ONLY.
 *
 * One traversal covers the reference's four device functions; the differences between them are
 * the rule set (projector vs backprojector) and whether a TOF value is given:
 *
 *   rule                         proj non-TOF            proj TOF                 back (both)
 *   LOR skip: transaxial < 10    siddon.cu.cc:34         siddon_tof.cu.cc:37      siddon.cu.cc:364 / siddon_tof.cu.cc:395
 *   LOR skip: steeper than 45 deg siddon.cu.cc:38         -                        -
 *   x dominant when              |xd| >= |yd| (:46)      |xd| > |yd| (:48)        |xd| > |yd| (:372 / :405)
 *   slab skip                    past endpoint 2 (:56-57, :203-204)
 *                                                        before endpoint 1 (:67-74, :228-235)   none
 *   weight                       frac*sqrt(1+k^2+kz^2)*dx_/L/L (:94)              frac*sqrt(..)*dx_ (:418)
 *   TOF factor                   -                       w_tof (:43-59, :215-219) w_tof (:402-416)
 *
 * Expression trees follow the reference operand by operand (including its double-precision
 * promotions in the TOF weight) so that, compiled with -ffp-contract=off, results are bitwise equal
 * to the reference device functions compiled on the host (oracle/_ref).
 *
 * Two additions that are not in the reference, both off by default:
 *  - tof_nsigma > 0 drops slabs whose TOF argument t2 exceeds tof_nsigma^2 (truncated kernel);
 *  - OR_RULES_PROJ with OR_SCATTER is the exact adjoint of the projector.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "oracle.h"

#define REF_PI 3.1415926f /* siddon_tof.cu.cc:10, a float constant */

static inline float fabs_ref(float v) { return v < 0 ? -v : v; } /* siddon.cu.cc:6 */

typedef struct {
    int nx, ny, nz;
    float dx_, dy, dz;
} grid_t;

/* accumulate one (voxel, fraction) visit */
static inline void visit(int action, int64_t idx, float frac, float s, float dx_, float L, int proj,
                         int tof, float w_tof, const float *img_in, float *acc, float val,
                         float *img_out, int64_t *pairs) {
    float weight = frac * s * dx_;
    if (proj) weight = weight / L / L;
    if (action == OR_GATHER) {
        if (tof)
            *acc = *acc + img_in[idx] * weight * w_tof;
        else
            *acc = *acc + img_in[idx] * weight;
    } else {
        if (tof)
            img_out[idx] = img_out[idx] + val * weight * w_tof;
        else
            img_out[idx] = img_out[idx] + val * weight;
    }
    ++*pairs;
}

/* the first-voxel-only weight (cases with a single voxel) is sqrt(..)*dx_ without a fraction
 * multiply; 1.0f*s == s exactly, so visit(frac=1) reproduces it bit for bit. */

static void trace_one(const float *l, int has_tof, float tof_value, float tof_bin, float tof_sigma2,
                      float tof_nsigma, const int *grid, const float *center, const float *size,
                      int rules, int action, float val, const float *img_in, float *img_out,
                      float *acc, int64_t *pairs) {
    const int nx = grid[0], ny = grid[1], nz = grid[2];
    const float dx_ = size[0] / nx;
    const float dy = size[1] / ny / dx_;
    const float dz = size[2] / nz / dx_;
    const float x1 = (l[0] - center[0]) / dx_;
    const float x2 = (l[3] - center[0]) / dx_;
    const float y1 = (l[1] - center[1]) / dx_;
    const float y2 = (l[4] - center[1]) / dx_;
    const float z1 = (l[2] - center[2]) / dx_;
    const float z2 = (l[5] - center[2]) / dx_;
    const float xd = x2 - x1, yd = y2 - y1, zd = z2 - z1;
    const int proj = (rules == OR_RULES_PROJ);

    if (sqrtf(xd * xd + yd * yd) < 10.0f) return;
    if (proj && !has_tof && sqrtf(xd * xd + yd * yd) < fabs_ref(zd)) return;

    const float nx2 = nx / 2.0f, ny2 = ny / 2.0f, nz2 = nz / 2.0f;
    const float L = sqrtf(xd * xd + yd * yd + zd * zd);

    float ratio1 = 0.f, tof_bin_ = 0.f, expand = 0.f;
    if (has_tof) {
        ratio1 = (float)((1.0 - (double)(tof_value / dx_ / L)) / 2);
        tof_bin_ = tof_bin / dx_;
        const float tof_sigma2_ = tof_sigma2 / dx_ / dx_;
        expand = tof_sigma2_ + (tof_bin_ * tof_bin_) / 12;
    }
    const float nsig2 = tof_nsigma * tof_nsigma;

    const int xdom = (proj && !has_tof) ? (fabs_ref(xd) >= fabs_ref(yd)) : (fabs_ref(xd) > fabs_ref(yd));
    /* primary axis p (slab index), in-plane secondary q, axial z */
    const float p1 = xdom ? x1 : y1, p2 = xdom ? x2 : y2;
    const float q1 = xdom ? y1 : x1;
    const float pd = xdom ? xd : yd;
    const float kq = (xdom ? yd : xd) / pd;
    const float kz = zd / pd;
    const int np = xdom ? nx : ny, nq = xdom ? ny : nx;
    const float np2 = xdom ? nx2 : ny2, nq2 = xdom ? ny2 : nx2;
    const float dq = xdom ? dy : 1.0f;  /* the y branch adds nx2 without a division: a/1.0f == a */
    const float dpc = xdom ? 1.0f : dy; /* xc uses dx (=1), yc uses dy */
    const int64_t sp = xdom ? 1 : nx, sq = xdom ? nx : 1, sz = (int64_t)nx * ny;
    const float s = sqrtf(1 + kq * kq + kz * kz);

    for (int ip = 0; ip < np; ++ip) {
        float w_tof = 0.f;
        if (has_tof) {
            const float pc = (float)(((double)(ip - np / 2) + 0.5) * (double)dpc);
            const float d2_tof = ((pc - p1) / (p2 - p1) - ratio1) * L;
            const float t2 = d2_tof * d2_tof / expand;
            w_tof = (float)((double)tof_bin_ * exp(-0.5 * (double)t2) /
                            sqrt(2.0 * (double)REF_PI * (double)expand));
            if (nsig2 > 0.f && t2 > nsig2) continue;
        }
        const float pp1 = ip - np2;
        const float pp2 = pp1 + 1.0f;
        if (proj) {
            if (!has_tof) {
                if (p1 < p2 && pp2 > p2) continue;
                if (p1 >= p2 && pp1 < p2) continue;
            } else if (xdom) {
                if (p2 > p1 && pp1 <= p1) continue;
                if (p2 < p1 && pp2 >= p1) continue;
            } else {
                if (p2 > p1 && pp1 < p1) continue;
                if (p2 < p1 && pp2 > p1) continue;
            }
        }
        float qq1, qq2, zz1, zz2;
        if (kq >= 0.0f) {
            qq1 = (q1 + kq * (pp1 - p1)) / dq + nq2;
            qq2 = (q1 + kq * (pp2 - p1)) / dq + nq2;
        } else {
            qq1 = (q1 + kq * (pp2 - p1)) / dq + nq2;
            qq2 = (q1 + kq * (pp1 - p1)) / dq + nq2;
        }
        const int cq1 = (int)floorf(qq1), cq2 = (int)floorf(qq2);
        if (kz >= 0.0f) {
            zz1 = (z1 + kz * (pp1 - p1)) / dz + nz2;
            zz2 = (z1 + kz * (pp2 - p1)) / dz + nz2;
        } else {
            zz1 = (z1 + kz * (pp2 - p1)) / dz + nz2;
            zz2 = (z1 + kz * (pp1 - p1)) / dz + nz2;
        }
        const int cz1 = (int)floorf(zz1), cz2 = (int)floorf(zz2);
        const int64_t base = (int64_t)ip * sp;
#define V(cq, cz, frac)                                                                            \
    visit(action, base + (int64_t)(cq)*sq + (int64_t)(cz)*sz, (frac), s, dx_, L, proj, has_tof,   \
          w_tof, img_in, acc, val, img_out, pairs)
        if (cq1 == cq2) {
            if (0 <= cq1 && cq1 < nq) {
                if (cz1 == cz2) {
                    if (0 <= cz1 && cz1 < nz) V(cq1, cz1, 1.0f);
                } else if (-1 <= cz1 && cz1 < nz) {
                    const float rz = (cz2 - zz1) / (zz2 - zz1);
                    if (cz1 >= 0) V(cq1, cz1, rz);
                    if (cz2 < nz) V(cq1, cz2, 1 - rz);
                }
            }
        } else if (-1 <= cq1 && cq1 < nq) {
            if (cz1 == cz2) {
                if (0 <= cz1 && cz1 < nz) {
                    const float rq = (cq2 - qq1) / (qq2 - qq1);
                    if (cq1 >= 0) V(cq1, cz1, rq);
                    if (cq2 < nq) V(cq2, cz1, 1 - rq);
                }
            } else if (-1 <= cz1 && cz1 < nz) {
                const float rq = (cq2 - qq1) / (qq2 - qq1);
                const float rz = (cz2 - zz1) / (zz2 - zz1);
                if (rq > rz) {
                    if (cq1 >= 0 && cz1 >= 0) V(cq1, cz1, rz);
                    if (cq1 >= 0 && cz2 < nz) V(cq1, cz2, rq - rz);
                    if (cq2 < nq && cz2 < nz) V(cq2, cz2, 1 - rq);
                } else {
                    if (cq1 >= 0 && cz1 >= 0) V(cq1, cz1, rq);
                    if (cq2 < nq && cz1 >= 0) V(cq2, cz1, rz - rq);
                    if (cq2 < nq && cz2 < nz) V(cq2, cz2, 1 - rz);
                }
            }
        }
#undef V
    }
}

int64_t or_trace(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                 float tof_bin, float tof_sigma2, float tof_nsigma, const int *grid,
                 const float *center, const float *size, int rules, int action,
                 const float *values, float *image_out, const float *image_in, float *out) {
    int64_t pairs = 0;
    for (int64_t i = 0; i < n; ++i) {
        float acc = 0.0f;
        const float tv = tof ? tof[i * tof_stride] : 0.0f;
        const float val = (action == OR_SCATTER) ? values[i] : 0.0f;
        trace_one(lors + i * stride, tof != NULL, tv, tof_bin, tof_sigma2, tof_nsigma, grid,
                  center, size, rules, action, val, image_in, image_out, &acc, &pairs);
        if (action == OR_GATHER) out[i] = acc;
    }
    return pairs;
}

int64_t or_projection(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                      float tof_bin, float tof_sigma2, float tof_nsigma, const int *grid,
                      const float *center, const float *size, const float *image, float *out) {
    return or_trace(lors, n, stride, tof, tof_stride, tof_bin, tof_sigma2, tof_nsigma, grid, center,
                    size, OR_RULES_PROJ, OR_GATHER, NULL, NULL, image, out);
}

int64_t or_backprojection(const float *lors, int64_t n, int stride, const float *tof,
                          int tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                          const int *grid, const float *center, const float *size,
                          const float *values, float *image) {
    return or_trace(lors, n, stride, tof, tof_stride, tof_bin, tof_sigma2, tof_nsigma, grid, center,
                    size, OR_RULES_BACK, OR_SCATTER, values, image, NULL, NULL);
}

int64_t or_projection_adjoint(const float *lors, int64_t n, int stride, const float *tof,
                              int tof_stride, float tof_bin, float tof_sigma2, float tof_nsigma,
                              const int *grid, const float *center, const float *size,
                              const float *values, float *image) {
    return or_trace(lors, n, stride, tof, tof_stride, tof_bin, tof_sigma2, tof_nsigma, grid, center,
                    size, OR_RULES_PROJ, OR_SCATTER, values, image, NULL, NULL);
}

/* Multi-threaded variant used for the CPU baseline timing (OpenMP over LORs; scatter goes to
 * per-thread private images that are summed at the end, so results equal or_trace up to the
 * summation order of the backprojection). */
#ifdef _OPENMP
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#endif

int64_t or_trace_mt(const float *lors, int64_t n, int stride, const float *tof, int tof_stride,
                    float tof_bin, float tof_sigma2, float tof_nsigma, const int *grid,
                    const float *center, const float *size, int rules, int action,
                    const float *values, float *image_out, const float *image_in, float *out,
                    int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 1)
#endif
        return or_trace(lors, n, stride, tof, tof_stride, tof_bin, tof_sigma2, tof_nsigma, grid,
                        center, size, rules, action, values, image_out, image_in, out);
#ifdef _OPENMP
    const int64_t nvox = (int64_t)grid[0] * grid[1] * grid[2];
    int64_t pairs = 0;
    if (action == OR_GATHER) {
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256) reduction(+ : pairs)
        for (int64_t i = 0; i < n; ++i) {
            float acc = 0.0f;
            int64_t p = 0;
            trace_one(lors + i * stride, tof != NULL, tof ? tof[i * tof_stride] : 0.0f, tof_bin,
                      tof_sigma2, tof_nsigma, grid, center, size, rules, action, 0.0f, image_in,
                      NULL, &acc, &p);
            out[i] = acc;
            pairs += p;
        }
        return pairs;
    }
    float *priv = (float *)calloc((size_t)nthreads * (size_t)nvox, sizeof(float));
    if (!priv) return -1;
#pragma omp parallel num_threads(nthreads) reduction(+ : pairs)
    {
        float *mine = priv + (size_t)omp_get_thread_num() * (size_t)nvox;
        float acc = 0.0f;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            int64_t p = 0;
            trace_one(lors + i * stride, tof != NULL, tof ? tof[i * tof_stride] : 0.0f, tof_bin,
                      tof_sigma2, tof_nsigma, grid, center, size, rules, action, values[i], NULL,
                      mine, &acc, &p);
            pairs += p;
        }
#pragma omp for schedule(static)
        for (int64_t v = 0; v < nvox; ++v) {
            float s = image_out[v];
            for (int t = 0; t < nthreads; ++t) s += priv[(size_t)t * (size_t)nvox + v];
            image_out[v] = s;
        }
    }
    free(priv);
    return pairs;
#endif
}
