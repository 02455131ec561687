/*
 * oracle/directions.c -- CPU restatement of the reference's direction kernels.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of csrc/directions.cu).
 *
 * Follows:
 *   src/clcode/detect_ridges.cl:34-102         detectRidges (in-plane local maximum
 *                                               with trilinear sampling, outside = -1)
 *   src/clcode/adjust_directions.cl:29-43       extractMainDirections
 *   src/clcode/adjust_directions.cl:68-100      completeTransformations
 *   src/clcode/adjust_directions.cl:182-246     adjustNonRidgeSigns (nearest ridge point,
 *                                               strict <, so the lowest index wins ties)
 * OpenCL vector arithmetic is written out per component in the same order.
 */
#include <stdint.h>
#include <stdlib.h>
#include <math.h>
#include <float.h>
#include "qmath.h"

/* detectRidges; threshold is the double -D THRESHOLD of the reference */
void oracle_detect_ridges(int64_t d0, int64_t d1, int64_t d2, double threshold, float *ridge, const float *resp,
                          const float *quat3)
{
#pragma omp parallel for schedule(static)
    for (int64_t i0 = 0; i0 < d0; ++i0)
        for (int64_t i1 = 0; i1 < d1; ++i1)
            for (int64_t i2 = 0; i2 < d2; ++i2) {
                const int64_t i = i2 + d2 * (i1 + d1 * i0);
                float q[4], c1[3], c2[3];
                o_qexpand(quat3 + 3 * i, q);
                o_quat2mat_cols(q, NULL, c1, c2);
                const float pos[3] = {(float)i0, (float)i1, (float)i2};
                float maxv = -INFINITY;
                for (int j = 0; j < 8; ++j) {
                    const int a = (-1) * (j < 3) + (j > 4);
                    const int b = (j % 3) - 1 + (j == 4);
                    float p[3];
                    int o[3];
                    for (int k = 0; k < 3; ++k) {
                        p[k] = pos[k] + (float)a * c1[k] + (float)b * c2[k];
                        o[k] = (int)p[k];   /* convert_int3: toward zero */
                        p[k] = p[k] - (float)o[k];
                    }
                    float v = 0;
                    for (int k = 0; k < 8; ++k) {
                        const int r0 = k >> 2, r1 = (k >> 1) & 1, r2 = k & 1;
                        const int a0 = o[0] + r0, a1 = o[1] + r1, a2 = o[2] + r2;
                        const float w0 = r0 == 1 ? p[0] : 1 - p[0];
                        const float w1 = r1 == 1 ? p[1] : 1 - p[1];
                        const float w2 = r2 == 1 ? p[2] : 1 - p[2];
                        const int out = a0 < 0 || a1 < 0 || a2 < 0 || a0 >= d0 || a1 >= d1 || a2 >= d2;
                        const float s = out ? -1.0f : resp[a2 + d2 * (a1 + d1 * (int64_t)a0)];
                        v += s * w0 * w1 * w2;
                    }
                    maxv = v > maxv ? v : maxv;
                }
                ridge[i] = ((double)resp[i] > threshold && resp[i] > maxv) ? 1.0f : 0.0f;
            }
}

/* extractMainDirections: column 0 of R(qexpand(q)); in and out may alias */
void oracle_extract_main_directions(int64_t n, float *out3, const float *in3)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float q[4], c0[3];
        o_qexpand(in3 + 3 * i, q);
        o_quat2mat_cols(q, c0, NULL, NULL);
        out3[3 * i] = c0[0]; out3[3 * i + 1] = c0[1]; out3[3 * i + 2] = c0[2];
    }
}

/* normalize(v) of OpenCL with the all-zero vector kept (the shim's convention) */
static void o_normalize3(const float v[3], float o[3])
{
    const float l2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (l2 == 0.0f) { o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; return; }
    const float l = sqrtf(l2);
    o[0] = v[0] / l; o[1] = v[1] / l; o[2] = v[2] / l;
}

/* completeTransformations: frame from v, mat2quat, qsqueeze; in and out may alias */
void oracle_complete_transformations(int64_t n, float *out3, const float *in3)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float e0[3], e1[3], e2[3], t[3];
        o_normalize3(in3 + 3 * i, e0);
        if (fabsf(e0[0]) > fabsf(e0[1])) { t[0] = -e0[2]; t[1] = 0.0f; t[2] = e0[0]; }
        else { t[0] = 0.0f; t[1] = e0[2]; t[2] = -e0[1]; }
        o_normalize3(t, e1);
        e2[0] = e0[1] * e1[2] - e0[2] * e1[1];
        e2[1] = e0[2] * e1[0] - e0[0] * e1[2];
        e2[2] = e0[0] * e1[1] - e0[1] * e1[0];
        const float m[3][3] = {{e0[0], e1[0], e2[0]}, {e0[1], e1[1], e2[1]}, {e0[2], e1[2], e2[2]}};
        float q[4], s[3];
        o_mat2quat(m, q);
        o_qsqueeze(q, s);
        out3[3 * i] = s[0]; out3[3 * i + 1] = s[1]; out3[3 * i + 2] = s[2];
    }
}

/* adjustNonRidgeSigns: coords R x 3 (uint16, axis order 0, 1, 2), rdirs R x 3 */
void oracle_adjust_nonridge_signs(int64_t d0, int64_t d1, int64_t d2, float *dirs3, const uint16_t *coords,
                                  const float *rdirs, int64_t R, const float *scaling)
{
#pragma omp parallel for schedule(static)
    for (int64_t i0 = 0; i0 < d0; ++i0)
        for (int64_t i1 = 0; i1 < d1; ++i1)
            for (int64_t i2 = 0; i2 < d2; ++i2) {
                float best = INFINITY;
                int64_t bj = 0;
                for (int64_t j = 0; j < R; ++j) {
                    const int64_t c0 = coords[3 * j], c1 = coords[3 * j + 1], c2 = coords[3 * j + 2];
                    const float f0 = (float)(uint32_t)(i0 > c0 ? i0 - c0 : c0 - i0) * scaling[0];
                    const float f1 = (float)(uint32_t)(i1 > c1 ? i1 - c1 : c1 - i1) * scaling[1];
                    const float f2 = (float)(uint32_t)(i2 > c2 ? i2 - c2 : c2 - i2) * scaling[2];
                    const float d = f0 * f0 + f1 * f1 + f2 * f2;
                    if (d < best) { best = d; bj = j; }
                }
                const int64_t i = i2 + d2 * (i1 + d1 * i0);
                float *v = dirs3 + 3 * i;
                const float *w = rdirs + 3 * bj;
                if (v[0] * w[0] + v[1] * w[1] + v[2] * w[2] < 0) {
                    v[0] = -v[0]; v[1] = -v[1]; v[2] = -v[2];
                }
            }
}

/* The minimum spanning tree of the scaled ridge points (pts: n x 3 float64)
 * that the reference takes from SciPy over squareform(pdist(...))
 * (adjust_directions.py:376-379), with equal distances in (i, j) order: Prim's
 * algorithm under the strict total order (distance, min(i, j), max(i, j)),
 * whose tree is unique and equal to the stable Kruskal's.  Distances are
 * pdist's: sqrt of the squared differences summed in axis order.  Writes the
 * n - 1 edges as (lo[k], hi[k]), lo < hi, in the order Prim adds them.  O(n^2)
 * time, O(n) memory. */
void oracle_prim_mst(const double *pts, int64_t n, int64_t *lo_out, int64_t *hi_out)
{
    if (n < 2) return;
    double *best_w = malloc(sizeof(double) * n);
    int64_t *best_lo = malloc(sizeof(int64_t) * n), *best_hi = malloc(sizeof(int64_t) * n);
    char *in_tree = calloc(n, 1);
    for (int64_t j = 0; j < n; ++j) { best_w[j] = INFINITY; best_lo[j] = n; best_hi[j] = n; }
    int64_t cur = 0;
    for (int64_t k = 0; k < n - 1; ++k) {
        in_tree[cur] = 1;
        const double c0 = pts[3 * cur], c1 = pts[3 * cur + 1], c2 = pts[3 * cur + 2];
        int64_t nxt = -1;
        for (int64_t j = 0; j < n; ++j) {
            if (in_tree[j]) continue;
            const double e0 = pts[3 * j] - c0, e1 = pts[3 * j + 1] - c1, e2 = pts[3 * j + 2] - c2;
            const double d = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
            const int64_t lo = j < cur ? j : cur, hi = j < cur ? cur : j;
            if (d < best_w[j] || (d == best_w[j] && (lo < best_lo[j] || (lo == best_lo[j] && hi < best_hi[j])))) {
                best_w[j] = d; best_lo[j] = lo; best_hi[j] = hi;
            }
            if (nxt < 0 || best_w[j] < best_w[nxt] ||
                (best_w[j] == best_w[nxt] &&
                 (best_lo[j] < best_lo[nxt] || (best_lo[j] == best_lo[nxt] && best_hi[j] < best_hi[nxt]))))
                nxt = j;
        }
        lo_out[k] = best_lo[nxt];
        hi_out[k] = best_hi[nxt];
        cur = nxt;
    }
    free(best_w); free(best_lo); free(best_hi); free(in_tree);
}
