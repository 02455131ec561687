/*
 * oracle/qmath.h -- CPU restatement of the reference's quaternion helpers.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path includes this file;
 * it is the checker the CUDA kernels are compared against.
 *
 * The reference writes these helpers in OpenCL C (src/clcode/quaternion_math.h)
 * where an unsuffixed literal such as 0.5 is a double, so mixed expressions
 * are evaluated in double and rounded to float on assignment.  The restatement
 * below spells out every such promotion with explicit casts so that it gives
 * the same bits as the reference source compiled as C/C++ (the build uses
 * -ffp-contract=off so no multiply-add is fused behind our back).
 */
#ifndef ORACLE_QMATH_H
#define ORACLE_QMATH_H

#include <math.h>
#include <float.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static inline float o_sq(float x) { return x * x; }

/* OpenCL min(float, float): "returns y if y < x, otherwise x". */
static inline float o_min(float x, float y) { return y < x ? y : x; }

/* Float cosine and sine evaluated as the double function rounded to float:
 * the correctly rounded value on every platform.  The reference's OpenCL
 * cos(float) has implementation-defined accuracy and libm's cosf/sinf are not
 * correctly rounded on every platform, so this is the portable reading. */
static inline float o_cosf(float x) { return (float)cos((double)x); }
static inline float o_sinf(float x) { return (float)sin((double)x); }

/* qexpand, quaternion_math.h:79-90.  The half angles are (float sum) * 0.5
 * in double, stored to float; cos/sin of theta take a double argument. */
static inline void o_qexpand(const float v[3], float q[4])
{
    const float pp = (float)((double)(v[0] + v[2]) * 0.5);
    const float pm = (float)((double)(v[0] - v[2]) * 0.5);
    const float ct = (float)cos((double)v[1] * 0.5);
    const float st = (float)sin((double)v[1] * 0.5);
    q[0] = o_cosf(pp) * ct;
    q[1] = o_cosf(pm) * st;
    q[2] = o_sinf(pm) * st;
    q[3] = o_sinf(pp) * ct;
}

/* qrot, quaternion_math.h:114-147: out = q v q^-1 via two Hamilton
 * products (qmult_vector, then the product with the inverse). */
static inline void o_qrot(const float q[4], const float v[3], float out[3])
{
    const float t0 = -(q[1] * v[0] + q[2] * v[1] + q[3] * v[2]);
    const float t1 = q[0] * v[0] + q[2] * v[2] - q[3] * v[1];
    const float t2 = q[0] * v[1] - q[1] * v[2] + q[3] * v[0];
    const float t3 = q[0] * v[2] + q[1] * v[1] - q[2] * v[0];
    out[0] = -t0 * q[1] + t1 * q[0] - t2 * q[3] + t3 * q[2];
    out[1] = -t0 * q[2] + t1 * q[3] + t2 * q[0] - t3 * q[1];
    out[2] = -t0 * q[3] - t1 * q[2] + t2 * q[1] + t3 * q[0];
}

/* safeatan2 macro, quaternion_math.h:6 (both arguments cast to float). */
static inline float o_safeatan2(double x, double y)
{
    return (x == 0.0 && y == 0.0) ? 0.0f : atan2f((float)x, (float)y);
}

static inline float o_clampf(float x, float lo, float hi)
{
    return x < lo ? lo : (x > hi ? hi : x);
}

/* qsqueeze, quaternion_math.h:20-39 (scalar part first). */
static inline void o_qsqueeze(const float q[4], float v[3])
{
    const float q1spq2s = o_sq(q[1]) + o_sq(q[2]);
    const int c1 = q1spq2s < FLT_EPSILON;
    const int c2 = c1 || (1 - q1spq2s) < FLT_EPSILON;
    const float q1q3 = q[1] * q[3];
    const float q2q0 = q[2] * q[0];
    const float q1q0 = q[1] * q[0];
    const float q2q3 = q[2] * q[3];
    v[0] = o_safeatan2((double)(q1q3 + q2q0), (double)(q1q0 - q2q3));
    v[1] = (float)((c1 ? 0.0 : M_PI) * c2 +
                   (double)(acosf(o_clampf(1 - 2 * q1spq2s, -1.0f, 1.0f)) * (float)(!c2)));
    float at2 = (q[1] * q[2] - q[0] * q[3]) * (float)c2 + (q1q3 - q2q0) * (float)(!c2);
    at2 = o_safeatan2((double)at2,
                      (0.5 - (double)(o_sq(q[2]) + o_sq(q[3]))) * c2 + (double)((q1q0 + q2q3) * (float)(!c2)));
    v[2] = (-at2 + v[0] * (float)(c1 ? -1 : 1)) * (float)c2 + at2 * (float)(!c2);
}

/* qsqueezeLast, quaternion_math.h:45-69 (scalar part last). */
static inline void o_qsqueeze_last(const float qin[4], float v[3])
{
    const float q[4] = {qin[3], qin[0], qin[1], qin[2]};
    o_qsqueeze(q, v);
}

/* Column 0/1/2 of quat2matFloat3, quaternion_math.h:257-289. */
static inline void o_quat2mat_cols(const float q[4], float c0[3], float c1[3], float c2[3])
{
    const float qx2 = o_sq(q[1]), qy2 = o_sq(q[2]), qz2 = o_sq(q[3]);
    const float qwqx = q[0] * q[1], qwqy = q[0] * q[2], qwqz = q[0] * q[3];
    const float qxqy = q[1] * q[2], qxqz = q[1] * q[3], qyqz = q[2] * q[3];
    if (c0) { c0[0] = 1 - 2 * (qy2 + qz2); c0[1] = 2 * (qxqy + qwqz); c0[2] = 2 * (qxqz - qwqy); }
    if (c1) { c1[0] = 2 * (qxqy - qwqz); c1[1] = 1 - 2 * (qx2 + qz2); c1[2] = 2 * (qyqz + qwqx); }
    if (c2) { c2[0] = 2 * (qxqz + qwqy); c2[1] = 2 * (qyqz - qwqx); c2[2] = 1 - 2 * (qx2 + qy2); }
}

/* OpenCL native_rsqrt on float (the argument of a double expression is
 * converted to float first, as the built-in has float overloads only). */
static inline float o_rsqrtf(float x) { return 1.0f / sqrtf(x); }

/* mat2quat, quaternion_math.h:301-340; m[row][col]. */
static inline void o_mat2quat(const float m[3][3], float q[4])
{
    float s = m[0][0] + m[1][1] + m[2][2];
    if (s > 0) {
        s = (float)((double)o_rsqrtf((float)((double)s + 1.0)) * 0.5);
        q[0] = (float)(0.25 / (double)s);
        q[1] = (m[2][1] - m[1][2]) * s;
        q[2] = (m[0][2] - m[2][0]) * s;
        q[3] = (m[1][0] - m[0][1]) * s;
    } else if (m[0][0] > m[1][1] && m[0][0] > m[2][2]) {
        s = (float)((double)o_rsqrtf((float)(1.0 + (double)m[0][0] - (double)m[1][1] - (double)m[2][2])) * 0.5);
        q[0] = (m[2][1] - m[1][2]) * s;
        q[1] = (float)(0.25 / (double)s);
        q[2] = (m[0][1] + m[1][0]) * s;
        q[3] = (m[0][2] + m[2][0]) * s;
    } else if (m[1][1] > m[2][2]) {
        s = (float)((double)o_rsqrtf((float)(1.0 + (double)m[1][1] - (double)m[0][0] - (double)m[2][2])) * 0.5);
        q[0] = (m[0][2] - m[2][0]) * s;
        q[1] = (m[0][1] + m[1][0]) * s;
        q[2] = (float)(0.25 / (double)s);
        q[3] = (m[1][2] + m[2][1]) * s;
    } else {
        s = (float)((double)o_rsqrtf((float)(1.0 + (double)m[2][2] - (double)m[0][0] - (double)m[1][1])) * 0.5);
        q[0] = (m[1][0] - m[0][1]) * s;
        q[1] = (m[0][2] + m[2][0]) * s;
        q[2] = (m[1][2] + m[2][1]) * s;
        q[3] = (float)(0.25 / (double)s);
    }
}

#endif /* ORACLE_QMATH_H */
