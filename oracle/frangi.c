/*
 * oracle/frangi.c -- CPU restatement of the reference's Frangi vesselness.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of csrc/frangi.cu).
 *
 * Follows:
 *   src/clcode/convolve_naive.cl:25-166   axis0/axis1/axis2: reversed taps,
 *                                          mirror boundary with period 2(n-1)
 *   src/processing/qfrangi_gpu.py:208-271  Hessian: entry order 00,11,22,01,02,12,
 *                                          each filtered along axis 0, then 1, then 2
 *   src/clcode/qeigs.cl:35-92, 146-256     cyclic Jacobi with approximate Givens
 *                                          rotations, quaternion accumulation,
 *                                          sort by |lambda|, squeeze
 *   src/clcode/frangi.cl:46-115            updateVesselness, calculateNorm
 *   src/clcode/max.cl:25-58                NaN-neutral maximum
 * Gaussian taps are computed by the caller (oracle.py, in numpy exactly as
 * qfrangi_gpu.py:158-185 does) and passed in as float32.
 *
 * Edge case: for an axis of length 1 the reference's period 2(n-1) is zero
 * (a division by zero); here every tap then reads the single voxel.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#include "qmath.h"

/* one 1-D convolution pass along `axis` of a (d0, d1, d2) volume */
void oracle_convolve(int axis, int64_t d0, int64_t d1, int64_t d2, float *out, const float *in,
                     const float *taps, int radius)
{
    const int64_t dims[3] = {d0, d1, d2};
    const int64_t n = dims[axis];
    const int64_t period = 2 * (n - 1);
    const int K = 2 * radius + 1;
    const int64_t stride = axis == 0 ? d1 * d2 : (axis == 1 ? d2 : 1);
#pragma omp parallel for schedule(static)
    for (int64_t i0 = 0; i0 < d0; ++i0)
        for (int64_t i1 = 0; i1 < d1; ++i1)
            for (int64_t i2 = 0; i2 < d2; ++i2) {
                const int64_t pos = axis == 0 ? i0 : (axis == 1 ? i1 : i2);
                const int64_t base = (i2 + d2 * (i1 + d1 * i0)) - pos * stride;
                float acc = 0.0f;
                int64_t t = 0;
                if (period > 0) {
                    t = (pos - radius - 1) % period;
                    if (t < 0) t += period;
                }
                for (int j = 0; j < K; ++j) {
                    int64_t m = 0;
                    if (period > 0) {
                        ++t;
                        if (t == period) t = 0;
                        m = t < n ? t : period - t;
                    }
                    acc += taps[K - j - 1] * in[base + m * stride];
                }
                out[i2 + d2 * (i1 + d1 * i0)] = acc;
            }
}

/*
 * Hessian of one scale (qfrangi_gpu.py:208-271) into h6 (N x 6, entries
 * 00, 11, 22, 01, 02, 12).  taps[axis][order] point at 2*radius[axis]+1
 * float taps already multiplied by sigma**order.
 */
void oracle_hessian(int64_t d0, int64_t d1, int64_t d2, const float *img, const float *const *taps,
                    const int *radius, float *h6)
{
    const int64_t n = d0 * d1 * d2;
    float *a = (float *)malloc(sizeof(float) * (size_t)n);
    float *b = (float *)malloc(sizeof(float) * (size_t)n);
    static const int ij[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 0}, {2, 0}, {2, 1}};
    for (int e = 0; e < 6; ++e) {
        int order[3] = {0, 0, 0};
        order[ij[e][0]] = 1;
        order[ij[e][1]] += 1;
        /* copy, then axis 0 -> axis 1 -> axis 2, ping-ponging two buffers */
        memcpy(a, img, sizeof(float) * (size_t)n);
        oracle_convolve(0, d0, d1, d2, b, a, taps[0 * 4 + order[0]], radius[0]);
        oracle_convolve(1, d0, d1, d2, a, b, taps[1 * 4 + order[1]], radius[1]);
        oracle_convolve(2, d0, d1, d2, b, a, taps[2 * 4 + order[2]], radius[2]);
        for (int64_t i = 0; i < n; ++i) h6[6 * i + e] = b[i];
    }
    free(a);
    free(b);
}

/* eigcmp of qfrangi_gpu.py:300: ascending absolute value */
static inline int o_eigcmp(float a, float b) { return fabsf(a) < fabsf(b); }

/* SORTER_QUAT, qeigs.cl:43-48 (scalar part last), float-rounded */
static const double O_SQ2 = 0.7071067811865475244;
static void o_sorter_quat(int k, float q[4])
{
    static const double t[6][4] = {{0., 0., 0., 1.}, {0., -1., 1., 0.}, {-1., 1., 0., 0.},
                                   {-0.5, -0.5, -0.5, 0.5}, {0.5, 0.5, 0.5, 0.5}, {-1., 0., 1., 0.}};
    for (int c = 0; c < 4; ++c) {
        double v = t[k][c];
        if (k == 1 || k == 2 || k == 5) v = v * O_SQ2;   /* the +-SQ2 entries */
        q[c] = (float)v;
    }
}

/* cqmult, qeigs.cl:35-41 */
static void o_cqmult(const float l[4], const float r[4], float o[4])
{
    o[3] = l[3] * r[3] - (l[0] * r[0] + l[1] * r[1] + l[2] * r[2]);
    o[0] = l[3] * r[0] + l[0] * r[3] + l[1] * r[2] - l[2] * r[1];
    o[1] = l[3] * r[1] - l[0] * r[2] + l[1] * r[3] + l[2] * r[0];
    o[2] = l[3] * r[2] + l[0] * r[1] - l[1] * r[0] + l[2] * r[3];
}

/* sortEigs, qeigs.cl:60-92 */
static void o_sort_eigs(float q[4], float v[3])
{
    int order[3], otmp;
    const float inq[4] = {q[0], q[1], q[2], q[3]};
    float vt;
    int c;
    c = o_eigcmp(v[0], v[1]);
    vt = v[0];
    v[0] = c ? v[0] : v[1]; order[0] = c ? 0 : 1;
    v[1] = c ? v[1] : vt;   order[1] = c ? 1 : 0;
    c = o_eigcmp(v[1], v[2]);
    vt = v[1]; otmp = order[1];
    v[1] = c ? v[1] : v[2]; order[1] = c ? order[1] : 2;
    v[2] = c ? v[2] : vt;   order[2] = c ? 2 : otmp;
    c = o_eigcmp(v[0], v[1]);
    vt = v[0]; otmp = order[0];
    v[0] = c ? v[0] : v[1]; order[0] = c ? order[0] : order[1];
    v[1] = c ? v[1] : vt;   order[1] = c ? order[1] : otmp;
    float s[4];
    o_sorter_quat((order[0] << 1) | (order[1] > order[2]), s);
    o_cqmult(s, inq, q);
}

/* eigs, qeigs.cl:146-256, one matrix: in6 -> out6 (may alias) */
static void o_eig3(const float *in6, float *out6)
{
    const double GAMMA = 5.8284271247461900976, C_STAR = 0.9238795325112867561,
                 S_STAR = 0.3826834323650897717;
    float on[3] = {in6[0], in6[1], in6[2]};
    float off[3] = {in6[5], in6[4], in6[3]};
    float oq[4] = {0.f, 0.f, 0.f, 1.f};
    float t1 = fabsf(on[0]), t2;
    t2 = fabsf(on[1]);  t1 = t1 < t2 ? t2 : t1;
    t2 = fabsf(on[2]);  t1 = t1 < t2 ? t2 : t1;
    t2 = fabsf(off[0]); t1 = t1 < t2 ? t2 : t1;
    t2 = fabsf(off[1]); t1 = t1 < t2 ? t2 : t1;
    t2 = fabsf(off[2]); t1 = t1 < t2 ? t2 : t1;
    const float TOL = t1 * FLT_EPSILON;
    for (int it = 0; it < 50; ++it) {
        if ((fabsf(off[0]) + fabsf(off[1]) + fabsf(off[2])) <= TOL) {
            o_sort_eigs(oq, on);
            oq[3] = -oq[3];
            float sq[3];
            o_qsqueeze_last(oq, sq);
            out6[0] = on[0]; out6[1] = on[1]; out6[2] = on[2];
            out6[3] = sq[0]; out6[4] = sq[1]; out6[5] = sq[2];
            return;
        }
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                const int r = 3 ^ (p | q);
                float c = (float)(2. * (double)(on[q] - on[p]));
                float s = off[r];
                t1 = s * s;
                t2 = c * c;
                int cond = (GAMMA * (double)t1 < (double)t2);
                t1 = o_rsqrtf(t1 + t2);
                c = cond ? (float)(double)(t1 * c) : (float)C_STAR;
                s = cond ? (float)(double)(t1 * s) : (float)S_STAR;
                t1 = c * oq[p] - s * oq[q];
                t2 = c * oq[q] + s * oq[p];
                oq[p] = t1; oq[q] = t2;
                cond = (r == 1);
                t1 = c * oq[3] + (cond ? s : -s) * oq[r];
                t2 = c * oq[r] + (cond ? -s : s) * oq[3];
                oq[3] = t1; oq[r] = t2;
                t1 = 1 - 2 * o_sq(s);
                s = 2 * c * s;
                c = t1;
                t1 = off[r] * c + on[p] * s;
                t2 = on[q] * c + off[r] * s;
                on[p] = c * (on[p] * c - off[r] * s) - s * (off[r] * c - on[q] * s);
                on[q] = c * t2 + s * t1;
                off[r] = c * t1 - s * t2;
                t2 = off[q];
                off[q] = c * t2 - s * off[p];
                off[p] = c * off[p] + s * t2;
            }
    }
    for (int k = 0; k < 6; ++k) out6[k] = NAN;
}

void oracle_eigs(int64_t n, const float *in6, float *out6)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) o_eig3(in6 + 6 * i, out6 + 6 * i);
}

/* calculateNorm + redMax (NaN-neutral maximum), frangi.cl:107-115, max.cl */
float oracle_max_norm(int64_t n, const float *eig6)
{
    float m = NAN;
    for (int64_t i = 0; i < n; ++i) {
        const float *e = eig6 + 6 * i;
        const float v = sqrtf(o_sq(e[0]) + o_sq(e[1]) + o_sq(e[2]));
        m = fmaxf(m, v);
    }
    return m;
}

/* updateVesselness, frangi.cl:46-92 */
void oracle_update_vesselness(int64_t n, float *val, float *quat3, const float *eig6, float alpha, float beta,
                              float c, int bright)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const float *e = eig6 + 6 * i;
        const float l1 = fabsf(e[0]);
        float l2 = e[1], l3 = e[2];
        l2 = bright ? l2 : -l2;
        l3 = bright ? l3 : -l3;
        const int valid = l2 < 0 && l3 < 0;
        l2 = fabsf(l2);
        l3 = fabsf(l3);
        const float rb = l1 / (sqrtf(l2 * l3) + FLT_MIN);
        const float ra = l2 / (l3 + FLT_MIN);
        const float ss = o_sq(l1) + o_sq(l2) + o_sq(l3);
        const float v = (float)valid * ((1.0f - expf(-0.5f * o_sq(ra / alpha))) * expf(-0.5f * o_sq(rb / beta)) *
                                        (1.0f - expf(-0.5f * ss / o_sq(c))));
        if (v > val[i]) {
            val[i] = v;
            quat3[3 * i] = e[3]; quat3[3 * i + 1] = e[4]; quat3[3 * i + 2] = e[5];
        }
    }
}

/*
 * VesselnessCalculation.execute (qfrangi_gpu.py:511-580) for M scales:
 * taps[m][axis][order] as in oracle_hessian.  c < 0 derives c per scale as
 * half the maximum Hessian norm.  val starts at -inf; quat3 at 0.
 */
void oracle_frangi(int64_t d0, int64_t d1, int64_t d2, const float *img, int nscales, const float *const *taps,
                   const int *radius, float alpha, float beta, float c, int bright, float *val, float *quat3,
                   float *c_used)
{
    const int64_t n = d0 * d1 * d2;
    float *h6 = (float *)malloc(sizeof(float) * 6 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        val[i] = -INFINITY;
        quat3[3 * i] = quat3[3 * i + 1] = quat3[3 * i + 2] = 0.f;
    }
    for (int m = 0; m < nscales; ++m) {
        oracle_hessian(d0, d1, d2, img, taps + 12 * m, radius + 3 * m, h6);
        oracle_eigs(n, h6, h6);
        float cm = c;
        if (c < 0) cm = 0.5f * oracle_max_norm(n, h6);
        if (c_used) c_used[m] = cm;
        oracle_update_vesselness(n, val, quat3, h6, alpha, beta, cm, bright);
    }
    free(h6);
}
