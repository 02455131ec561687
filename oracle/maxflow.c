/*
 * oracle/maxflow.c -- CPU restatement of the reference's continuous max-flow
 * with anisotropic total variation (ATV).
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and the CPU
 * baseline of bench.py call this as the checker; the product path never does.
 *
 * Follows, line by line:
 *   src/clcode-anisotropic/update_qp.cl:67-137   h_dot / h_t_dot / h_inv_dot
 *   src/clcode-anisotropic/update_qp.cl:150-232  update_p
 *   src/clcode-anisotropic/update_qp.cl:241-300  update_u (+ SUPERVISED)
 *   src/clcode-anisotropic/update_qp.cl:311-316  update_tmp
 *   src/clcode/sum_abs.cl:25-58 + src/helpers/cl_helpers.py:232-298  residual
 *   src/processing/continuous_cut_anisotropic_gpu.py:104-129, 198-344  solve loop
 * The -D macros RCC, RS0-2, SS0-2 and SQEVAL0-2 of the reference are double
 * constants, so
 * every product with them is a double product rounded to float on store;
 * that is spelled out below with explicit casts.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "qmath.h"

typedef struct {
    double rcc, rs[3], ss[3];
    int const_evals;     /* 1: sqevals[3] constant; 0: per-voxel sqeigs (N x 3) */
    double sqeval[3];
} o_mf_consts;

/* _reinit_clprograms, continuous_cut_anisotropic_gpu.py:104-129 */
static void o_mf_make_consts(o_mf_consts *k, const double scaling[3], double cc, double steps)
{
    double smin = scaling[0];
    if (scaling[1] < smin) smin = scaling[1];
    if (scaling[2] < smin) smin = scaling[2];
    for (int a = 0; a < 3; ++a) {
        k->rs[a] = 1.0 / scaling[a];
        k->ss[a] = steps / scaling[a] * (smin * smin);   /* np.divide(steps, s) * min_s ** 2 */
    }
    k->rcc = 1.0 / (cc * (smin * smin));
}

/* update_p, update_qp.cl:150-232.  quat3: squeezed quaternions (N x 3);
 * sqeigs: per-voxel square roots of the eigenvalues (N x 3) or NULL. */
static void o_update_p(const o_mf_consts *k, int64_t d0, int64_t d1, int64_t d2,
                       float *hp0, float *hp1, float *hp2, const float *tmp,
                       const float *quat3, const float *sqeigs, const float *alpha)
{
    const int64_t s0 = d1 * d2, s1 = d2;
#pragma omp parallel for schedule(static)
    for (int64_t i0 = 0; i0 < d0; ++i0)
        for (int64_t i1 = 0; i1 < d1; ++i1)
            for (int64_t i2 = 0; i2 < d2; ++i2) {
                const int64_t i = i2 + d2 * (i1 + d1 * i0);
                float g[3];
                g[0] = i0 < d0 - 1 ? (float)((double)(tmp[i + s0] - tmp[i]) * k->ss[0]) : 0.f;
                g[1] = i1 < d1 - 1 ? (float)((double)(tmp[i + s1] - tmp[i]) * k->ss[1]) : 0.f;
                g[2] = i2 < d2 - 1 ? (float)((double)(tmp[i + 1] - tmp[i]) * k->ss[2]) : 0.f;
                float q[4];
                o_qexpand(quat3 + 3 * i, q);
                const float *se = sqeigs ? sqeigs + 3 * i : NULL;
                /* h_t_dot: rotate by the transpose, then scale by sqrt(eig) */
                q[0] = -q[0];
                o_qrot(q, g, g);
                q[0] = -q[0];
                for (int a = 0; a < 3; ++a)
                    g[a] = se ? g[a] * se[a] : (float)((double)g[a] * k->sqeval[a]);
                /* h_inv_dot of hp */
                float p[3] = {hp0[i], hp1[i], hp2[i]};
                q[0] = -q[0];
                o_qrot(q, p, p);
                q[0] = -q[0];
                for (int a = 0; a < 3; ++a)
                    p[a] = se ? p[a] / se[a] : (float)((double)p[a] / k->sqeval[a]);
                p[0] += g[0]; p[1] += g[1]; p[2] += g[2];
                /* projection onto |p| <= alpha (native_sqrt) */
                const float norm = sqrtf(o_sq(p[0]) + o_sq(p[1]) + o_sq(p[2]));
                const float radius = alpha[i];
                const float scale = norm > radius ? radius / norm : 1.f;
                p[0] *= scale; p[1] *= scale; p[2] *= scale;
                /* h_dot: scale, then rotate */
                for (int a = 0; a < 3; ++a)
                    p[a] = se ? se[a] * p[a] : (float)(k->sqeval[a] * (double)p[a]);
                o_qrot(q, p, p);
                hp0[i] = p[0]; hp1[i] = p[1]; hp2[i] = p[2];
            }
}

/* update_u, update_qp.cl:241-300 (labels != NULL: the SUPERVISED variant). */
static void o_update_u(const o_mf_consts *k, int64_t d0, int64_t d1, int64_t d2,
                       const float *hp0, const float *hp1, const float *hp2, float *tmp,
                       const float *cs, const float *ct, float *pt, float *u,
                       const uint8_t *labels)
{
    const int64_t s0 = d1 * d2, s1 = d2;
#pragma omp parallel for schedule(static)
    for (int64_t i0 = 0; i0 < d0; ++i0)
        for (int64_t i1 = 0; i1 < d1; ++i1)
            for (int64_t i2 = 0; i2 < d2; ++i2) {
                const int64_t i = i2 + d2 * (i1 + d1 * i0);
                const float a0 = (i0 < d0 - 1 ? hp0[i] : 0.f) - (i0 > 0 ? hp0[i - s0] : 0.f);
                const float a1 = (i1 < d1 - 1 ? hp1[i] : 0.f) - (i1 > 0 ? hp1[i - s1] : 0.f);
                const float a2 = (i2 < d2 - 1 ? hp2[i] : 0.f) - (i2 > 0 ? hp2[i - 1] : 0.f);
                const float divhp = (float)((double)a0 * k->rs[0] + (double)a1 * k->rs[1] +
                                            (double)a2 * k->rs[2]);
                float u_i = u[i];
                float ps, pt_i;
                if (labels) {
                    const float uf = (float)(labels[i] & 1);
                    const float ub = (float)(!(labels[i] & 2));
                    ps = o_min((float)((double)(divhp + pt[i]) - k->rcc * (double)(u_i - ub)), cs[i]);
                    pt_i = o_min((float)((double)(-divhp + ps) + k->rcc * (double)(u_i - uf)), ct[i]);
                } else {
                    ps = o_min((float)((double)(divhp + pt[i]) - k->rcc * (double)(u_i - 1.0f)), cs[i]);
                    pt_i = o_min((float)((double)(-divhp + ps) + k->rcc * (double)u_i), ct[i]);
                }
                pt[i] = pt_i;
                const float err = divhp - ps + pt_i;
                u_i = (float)((double)u_i - (double)err / k->rcc);
                u[i] = u_i;
                tmp[i] = err;
            }
}

/* update_tmp, update_qp.cl:311-316 */
static void o_update_tmp(const o_mf_consts *k, int64_t n, float *tmp, const float *u)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        tmp[i] = (float)((double)tmp[i] - (double)u[i] * k->rcc);
}

/* The reference's Reducer with the sum_abs kernel (WGSIZE 1024): passes of
 * "|x[g]| + |x[g+G]|" followed by a shared-memory tree, until at most 1024
 * partials remain; the host then sums those (np.sum, float32).  The last
 * host step is done here in double; that only shifts the residual in its
 * last bits and decides nothing but the stopping iteration. */
double oracle_sum_abs(const float *x, int64_t n)
{
    const int64_t WG = 1024;
    if (n <= 0) return 0.0;
    float *a = (float *)malloc(sizeof(float) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) a[i] = fabsf(x[i]);
    int64_t m = n;
    float *b = NULL;
    while (m > WG) {
        const int64_t outn = (((m + 1) / 2) + WG - 1) / WG;
        const int64_t G = outn * WG;
        b = (float *)malloc(sizeof(float) * (size_t)outn);
        float scratch[1024];
        for (int64_t grp = 0; grp < outn; ++grp) {
            for (int64_t l = 0; l < WG; ++l) {
                const int64_t g = grp * WG + l;
                const float first = g < m ? a[g] : 0.f;  /* reads past m only beyond the data */
                scratch[l] = first + (g + G < m ? a[g + G] : 0.f);
            }
            for (int64_t s = WG >> 1; s > 0; s >>= 1)
                for (int64_t l = 0; l < s; ++l) scratch[l] += scratch[l + s];
            b[grp] = scratch[0];
        }
        free(a);
        a = b;
        m = outn;
    }
    double acc = 0.0;
    for (int64_t i = 0; i < m; ++i) acc += a[i];
    free(a);
    return acc;
}

/*
 * One full solve, CmfCutQAnisotropicGpu._execute (continuous_cut_anisotropic_gpu.py:198-344).
 *   img      N floats, the image used for u's initialisation u = img / (max(img) + tiny)
 *   quat3    N x 3 squeezed quaternions
 *   sqeval3  3 constant sqrt-eigenvalues (sqeigs == NULL) ...
 *   sqeigs   ... or N x 3 per-voxel sqrt-eigenvalues
 *   alpha, cs, ct  N floats;  labels  N bytes or NULL
 *   resid_log  optional, receives the residual of every check (max num_iter/update + 1)
 * Returns the number of update_p/update_u iterations executed.
 */
int oracle_maxflow_solve(const float *img, const float *quat3, const double *sqeval3,
                         const float *sqeigs, const float *alpha, const float *cs,
                         const float *ct, const uint8_t *labels,
                         int64_t d0, int64_t d1, int64_t d2, const double *scaling,
                         double cc, double steps, int num_iter, int update, double error_bound,
                         float *u, double *resid_log, int *n_checks)
{
    const int64_t n = d0 * d1 * d2;
    o_mf_consts k;
    memset(&k, 0, sizeof k);
    const double unit[3] = {1.0, 1.0, 1.0};
    o_mf_make_consts(&k, scaling ? scaling : unit, cc, steps);
    if (!sqeigs) for (int a = 0; a < 3; ++a) k.sqeval[a] = sqeval3[a];

    float *hp0 = (float *)calloc((size_t)n, sizeof(float));
    float *hp1 = (float *)calloc((size_t)n, sizeof(float));
    float *hp2 = (float *)calloc((size_t)n, sizeof(float));
    float *pt = (float *)malloc(sizeof(float) * (size_t)n);
    float *tmp = (float *)calloc((size_t)n, sizeof(float));

    /* pt = el_min(cs, ct) (helpers.cl:127-133: fmin) */
    for (int64_t i = 0; i < n; ++i) pt[i] = fminf(cs[i], ct[i]);
    /* u = img / (max(img) + tiny), float32 arithmetic (numpy) */
    float mx = img[0];
    for (int64_t i = 0; i < n; ++i) {
        if (img[i] != img[i]) { mx = img[i]; break; }   /* np.max propagates NaN */
        if (img[i] > mx) mx = img[i];
    }
    const float denom = mx + FLT_MIN;
    for (int64_t i = 0; i < n; ++i) u[i] = img[i] / denom;
    /* tmp = 0 - u * RCC */
    o_update_tmp(&k, n, tmp, u);

    int it, checks = 0;
    for (it = 0; it < num_iter; ++it) {
        o_update_p(&k, d0, d1, d2, hp0, hp1, hp2, tmp, quat3, sqeigs, alpha);
        o_update_u(&k, d0, d1, d2, hp0, hp1, hp2, tmp, cs, ct, pt, u, labels);
        if (update > 0 && it % update == 0) {
            const double err = oracle_sum_abs(tmp, n) / ((double)n * k.rcc);
            if (resid_log) resid_log[checks] = err;
            ++checks;
            if (isnan(err) || err < error_bound) { ++it; break; }
        }
        o_update_tmp(&k, n, tmp, u);
    }
    if (n_checks) *n_checks = checks;
    free(hp0); free(hp1); free(hp2); free(pt); free(tmp);
    return it;
}

/* Single-kernel entry points, used by the kernel-level parity tests. */
void oracle_mf_update_p(int64_t d0, int64_t d1, int64_t d2, const double *scaling,
                        double cc, double steps, const double *sqeval3,
                        float *hp0, float *hp1, float *hp2, const float *tmp,
                        const float *quat3, const float *sqeigs, const float *alpha)
{
    o_mf_consts k;
    memset(&k, 0, sizeof k);
    o_mf_make_consts(&k, scaling, cc, steps);
    if (!sqeigs) for (int a = 0; a < 3; ++a) k.sqeval[a] = sqeval3[a];
    o_update_p(&k, d0, d1, d2, hp0, hp1, hp2, tmp, quat3, sqeigs, alpha);
}

void oracle_mf_update_u(int64_t d0, int64_t d1, int64_t d2, const double *scaling,
                        double cc, double steps, const float *hp0, const float *hp1,
                        const float *hp2, float *tmp, const float *cs, const float *ct,
                        float *pt, float *u, const uint8_t *labels)
{
    o_mf_consts k;
    memset(&k, 0, sizeof k);
    o_mf_make_consts(&k, scaling, cc, steps);
    o_update_u(&k, d0, d1, d2, hp0, hp1, hp2, tmp, cs, ct, pt, u, labels);
}

void oracle_mf_update_tmp(int64_t n, const double *scaling, double cc, float *tmp, const float *u)
{
    o_mf_consts k;
    memset(&k, 0, sizeof k);
    const double steps = 0.0;
    o_mf_make_consts(&k, scaling, cc, steps);
    o_update_tmp(&k, n, tmp, u);
}
