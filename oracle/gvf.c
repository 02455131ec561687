/*
 * oracle/gvf.c -- CPU restatement of the reference's gradient vector flow.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of csrc/gvf.cu).
 *
 * Follows:
 *   src/clcode/gvf.cl:44-99     gvfDelta   (7-point Laplacian, mirror boundary)
 *   src/clcode/gvf.cl:162-173   gvfUpdate
 *   src/clcode/gvf.cl:193-202   magDelta
 *   src/clcode/gvf.cl:215-232   gvfNormalize
 *   src/clcode/gvf.cl:246-253   response (|v|^2)
 *   src/processing/gradient_vector_flow.py:58-65 (time step), 171-232 (loop)
 * MU, DT and RSS0-2 are double -D macros in the reference, so products with
 * them are double and round to float on store, spelled out below.
 *
 * Edge case: for an axis of length 1 the reference's mirror indexing reads
 * outside the buffer; here both neighbours are the voxel itself, i.e. the
 * axis contributes nothing to the Laplacian.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

double oracle_sum_abs(const float *x, int64_t n);

/* time_step_for, gradient_vector_flow.py:58-65 */
double oracle_gvf_time_step(const double *voxel_size, double mu, int ndim)
{
    double m = voxel_size[0];
    for (int k = 1; k < ndim; ++k) if (voxel_size[k] < m) m = voxel_size[k];
    const double v = pow(m, ndim) / (pow(2.01, ndim) * mu);
    return v < 0.99 ? v : 0.99;
}

/* gvfDelta, gvf.cl:44-99 */
static void o_gvf_delta(int64_t d0, int64_t d1, int64_t d2, double mu, const double rss[3],
                        float *o0, float *o1, float *o2, const float *g0, const float *g1, const float *g2,
                        const float *v0, const float *v1, const float *v2, const float *r)
{
    const int64_t s0 = d1 * d2, s1 = d2;
#pragma omp parallel for schedule(static)
    for (int64_t i0 = 0; i0 < d0; ++i0)
        for (int64_t i1 = 0; i1 < d1; ++i1)
            for (int64_t i2 = 0; i2 < d2; ++i2) {
                const int64_t i = i2 + d2 * (i1 + d1 * i0);
                const float c0 = g0[i], c1 = g1[i], c2 = g2[i];
                float l0, l1, l2;
                int64_t b, a;
                b = d0 > 1 ? i + (i0 > 0 ? -s0 : s0) : i;
                a = d0 > 1 ? i + (i0 < d0 - 1 ? s0 : -s0) : i;
                l0 = (float)((double)(g0[b] + g0[a] - 2 * c0) * rss[0]);
                l1 = (float)((double)(g1[b] + g1[a] - 2 * c1) * rss[0]);
                l2 = (float)((double)(g2[b] + g2[a] - 2 * c2) * rss[0]);
                b = d1 > 1 ? i + (i1 > 0 ? -s1 : s1) : i;
                a = d1 > 1 ? i + (i1 < d1 - 1 ? s1 : -s1) : i;
                l0 = (float)((double)l0 + (double)(g0[b] + g0[a] - 2 * c0) * rss[1]);
                l1 = (float)((double)l1 + (double)(g1[b] + g1[a] - 2 * c1) * rss[1]);
                l2 = (float)((double)l2 + (double)(g2[b] + g2[a] - 2 * c2) * rss[1]);
                b = d2 > 1 ? i + (i2 > 0 ? -1 : 1) : i;
                a = d2 > 1 ? i + (i2 < d2 - 1 ? 1 : -1) : i;
                l0 = (float)((double)l0 + (double)(g0[b] + g0[a] - 2 * c0) * rss[2]);
                l1 = (float)((double)l1 + (double)(g1[b] + g1[a] - 2 * c1) * rss[2]);
                l2 = (float)((double)l2 + (double)(g2[b] + g2[a] - 2 * c2) * rss[2]);
                o0[i] = (float)((double)(r[i] * (c0 - v0[i])) - mu * (double)l0);
                o1[i] = (float)((double)(r[i] * (c1 - v1[i])) - mu * (double)l1);
                o2[i] = (float)((double)(r[i] * (c2 - v2[i])) - mu * (double)l2);
            }
}

/* Single gvfDelta, for kernel-level tests. */
void oracle_gvf_delta(int64_t d0, int64_t d1, int64_t d2, double mu, const double *voxel_size,
                      float *o0, float *o1, float *o2, const float *g0, const float *g1, const float *g2,
                      const float *v0, const float *v1, const float *v2, const float *r)
{
    const double rss[3] = {1.0 / (voxel_size[0] * voxel_size[0]), 1.0 / (voxel_size[1] * voxel_size[1]),
                           1.0 / (voxel_size[2] * voxel_size[2])};
    o_gvf_delta(d0, d1, d2, mu, rss, o0, o1, o2, g0, g1, g2, v0, v1, v2, r);
}

/*
 * GvfGpu(vfield, params, voxel_size, response).execute()
 * (gradient_vector_flow.py:72-108, 171-232).
 *   v3        N x 3 interleaved vector field (z, y, x, 3)
 *   response  N weights, or NULL for |v|^2
 *   g3        output N x 3 interleaved
 *   mags      optional log of the mean |delta| of every check
 * Returns the number of iterations run.
 */
int oracle_gvf_run(const float *v3, const float *response, int64_t d0, int64_t d1, int64_t d2,
                   const double *voxel_size, double mu, int maxiter, int update, double tol, int normalize,
                   float *g3, double *mags, int *n_mags)
{
    const int64_t n = d0 * d1 * d2;
    const double vs1[3] = {1.0, 1.0, 1.0};
    const double *vs = voxel_size ? voxel_size : vs1;
    const double dt = oracle_gvf_time_step(vs, mu, 3);
    /* rss = 1 / voxel_size ** 2 (numpy: 1. / (vs ** 2)) */
    const double rss[3] = {1.0 / (vs[0] * vs[0]), 1.0 / (vs[1] * vs[1]), 1.0 / (vs[2] * vs[2])};
    float *buf = (float *)calloc((size_t)n * 11, sizeof(float));
    float *v0 = buf, *v1 = buf + n, *v2 = buf + 2 * n, *r = buf + 3 * n;
    float *g0 = buf + 4 * n, *g1 = buf + 5 * n, *g2 = buf + 6 * n;
    float *e0 = buf + 7 * n, *e1 = buf + 8 * n, *e2 = buf + 9 * n, *m = buf + 10 * n;
    for (int64_t i = 0; i < n; ++i) {
        v0[i] = v3[3 * i]; v1[i] = v3[3 * i + 1]; v2[i] = v3[3 * i + 2];
        r[i] = response ? response[i] : v0[i] * v0[i] + v1[i] * v1[i] + v2[i] * v2[i];
    }
    int it, checks = 0;
    for (it = 0; it < maxiter; ++it) {
        o_gvf_delta(d0, d1, d2, mu, rss, e0, e1, e2, g0, g1, g2, v0, v1, v2, r);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {   /* gvfUpdate */
            g0[i] = (float)((double)g0[i] - dt * (double)e0[i]);
            g1[i] = (float)((double)g1[i] - dt * (double)e1[i]);
            g2[i] = (float)((double)g2[i] - dt * (double)e2[i]);
        }
        if (update > 0 && it % update == 0) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i)   /* magDelta (native_sqrt) */
                m[i] = sqrtf(e0[i] * e0[i] + e1[i] * e1[i] + e2[i] * e2[i]);
            const double mag = oracle_sum_abs(m, n) / (double)n;
            if (mags) mags[checks] = mag;
            ++checks;
            if (mag < tol) { ++it; break; }
        }
    }
    if (normalize) {
        for (int64_t i = 0; i < n; ++i) {   /* gvfNormalize */
            float nrm = sqrtf(g0[i] * g0[i] + g1[i] * g1[i] + g2[i] * g2[i]);
            if (nrm != 0) {
                nrm = 1 / nrm;
                g0[i] = nrm * g0[i]; g1[i] = nrm * g1[i]; g2[i] = nrm * g2[i];
            }
        }
    }
    for (int64_t i = 0; i < n; ++i) {
        g3[3 * i] = g0[i]; g3[3 * i + 1] = g1[i]; g3[3 * i + 2] = g2[i];
    }
    if (n_mags) *n_mags = checks;
    free(buf);
    return it;
}
