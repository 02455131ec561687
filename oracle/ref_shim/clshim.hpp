/*
 * oracle/ref_shim/clshim.hpp -- a small OpenCL-C-on-C++ compatibility layer.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py prepends this header to the
 * reference's own OpenCL C kernels (read in place from the reference checkout,
 * never copied) and compiles them with g++ into oracle/_ref/libref.so, so the
 * oracle restatement can be checked against the reference source itself.
 *
 * Work-items are emulated by plain loops; get_global_id()/get_global_size()
 * read thread-local variables that the launchers in oracle/ref_shim/launch.inc
 * set before every work-item.  Only what the reference's non-barrier kernels
 * use is provided.
 */
#ifndef ORACLE_CLSHIM_HPP
#define ORACLE_CLSHIM_HPP

#include <math.h>
#include <float.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>

/* cos/sin of a float as the double function rounded to float (correctly
 * rounded on every platform; OpenCL leaves the accuracy of the float
 * built-ins implementation-defined).  Double arguments keep the double
 * functions. */
static inline float shim_cos(float x) { return (float)cos((double)x); }
static inline double shim_cos(double x) { return cos(x); }
static inline float shim_sin(float x) { return (float)sin((double)x); }
static inline double shim_sin(double x) { return sin(x); }
#define cos(x) shim_cos(x)
#define sin(x) shim_sin(x)

#define __kernel
#define __global
#define __local
#define __constant const
#define __read_only
#define __write_only

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;

static __thread size_t shim_gid[3];
static __thread size_t shim_gsz[3];

static inline size_t get_global_id(int d) { return shim_gid[d]; }
static inline size_t get_global_size(int d) { return shim_gsz[d]; }

/* OpenCL built-ins with the float overloads the kernels rely on. */
static inline float native_sqrt(float x) { return sqrtf(x); }
static inline float native_rsqrt(float x) { return 1.0f / sqrtf(x); }
static inline float rsqrt(float x) { return 1.0f / sqrtf(x); }
static inline float clamp(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }
static inline float min(float x, float y) { return y < x ? y : x; }
static inline float max(float x, float y) { return x < y ? y : x; }

/* ---- vector types (only the members and operators the kernels use) ---- */
struct float3 { float s0, s1, s2, s3; };
struct float4 { float s0, s1, s2, s3; };
struct int3 { int s0, s1, s2, s3; };
struct uint3 { uint s0, s1, s2, s3; };
struct uint4 { uint s0, s1, s2, s3; };
struct int2 { int s0, s1; };

static inline float3 make_float3(float a, float b, float c) { float3 r = {a, b, c, 0.f}; return r; }
static inline int3 make_int3(int a, int b, int c) { int3 r = {a, b, c, 0}; return r; }
static inline uint3 make_uint3(uint a, uint b, uint c) { uint3 r = {a, b, c, 0u}; return r; }
static inline float4 make_float4(float a, float b, float c, float d) { float4 r = {a, b, c, d}; return r; }
static inline int2 make_int2(int a, int b) { int2 r = {a, b}; return r; }

static inline float3 operator+(float3 a, float3 b) { return make_float3(a.s0 + b.s0, a.s1 + b.s1, a.s2 + b.s2); }
static inline float3 operator-(float3 a, float3 b) { return make_float3(a.s0 - b.s0, a.s1 - b.s1, a.s2 - b.s2); }
static inline float3 operator*(float3 a, float3 b) { return make_float3(a.s0 * b.s0, a.s1 * b.s1, a.s2 * b.s2); }
static inline float3 operator-(float3 a) { return make_float3(-a.s0, -a.s1, -a.s2); }
/* scalar-vector arithmetic: the scalar is converted to float first */
static inline float3 operator*(float s, float3 a) { return make_float3(s * a.s0, s * a.s1, s * a.s2); }
static inline float3 operator*(float3 a, float s) { return make_float3(a.s0 * s, a.s1 * s, a.s2 * s); }
static inline float3 operator*(int s, float3 a) { return (float)s * a; }
static inline float3 operator-(float s, float3 a) { return make_float3(s - a.s0, s - a.s1, s - a.s2); }
static inline float3 operator-(int s, float3 a) { return (float)s - a; }

static inline int3 operator+(int3 a, int3 b) { return make_int3(a.s0 + b.s0, a.s1 + b.s1, a.s2 + b.s2); }
static inline int3 &operator+=(int3 &a, int3 b) { a = a + b; return a; }
/* relational operators on vectors give -1 (true) / 0 (false) per component */
static inline int3 operator==(int3 a, int b) { return make_int3(-(a.s0 == b), -(a.s1 == b), -(a.s2 == b)); }
static inline int3 operator<(int3 a, int b) { return make_int3(-(a.s0 < b), -(a.s1 < b), -(a.s2 < b)); }
static inline int3 operator>=(int3 a, int3 b) { return make_int3(-(a.s0 >= b.s0), -(a.s1 >= b.s1), -(a.s2 >= b.s2)); }
static inline int any(int3 m) { return (m.s0 < 0) || (m.s1 < 0) || (m.s2 < 0); }
/* vector "m ? a : b" (selects a where the mask's sign bit is set) */
static inline float3 shim_vselect(int3 m, float3 a, float3 b)
{
    return make_float3(m.s0 < 0 ? a.s0 : b.s0, m.s1 < 0 ? a.s1 : b.s1, m.s2 < 0 ? a.s2 : b.s2);
}

/* convert_int3 of float: round toward zero (the OpenCL default for float->int) */
static inline int3 convert_int3(float3 a) { return make_int3((int)a.s0, (int)a.s1, (int)a.s2); }
static inline float3 convert_float3(int3 a) { return make_float3((float)a.s0, (float)a.s1, (float)a.s2); }
static inline float3 convert_float3(uint3 a) { return make_float3((float)a.s0, (float)a.s1, (float)a.s2); }
static inline uint abs_diff1(uint a, uint b) { return a > b ? a - b : b - a; }
static inline uint3 abs_diff(uint3 a, uint3 b)
{
    return make_uint3(abs_diff1(a.s0, b.s0), abs_diff1(a.s1, b.s1), abs_diff1(a.s2, b.s2));
}
static inline uint3 as_uint3(uint4 a) { return make_uint3(a.s0, a.s1, a.s2); }
static inline int3 as_int3(uint4 a) { return make_int3((int)a.s0, (int)a.s1, (int)a.s2); }
static inline float3 as_float3(float4 a) { return make_float3(a.s0, a.s1, a.s2); }

static inline float dot(float3 a, float3 b) { return a.s0 * b.s0 + a.s1 * b.s1 + a.s2 * b.s2; }
static inline float length(float3 a) { return sqrtf(dot(a, a)); }
static inline float3 cross(float3 a, float3 b)
{
    return make_float3(a.s1 * b.s2 - a.s2 * b.s1, a.s2 * b.s0 - a.s0 * b.s2, a.s0 * b.s1 - a.s1 * b.s0);
}
/* normalize(v): v / |v|; the all-zero vector is returned unchanged */
static inline float3 normalize(float3 a)
{
    const float l2 = dot(a, a);
    if (l2 == 0.0f) return a;
    const float l = sqrtf(l2);
    return make_float3(a.s0 / l, a.s1 / l, a.s2 / l);
}
static inline float3 vload3(size_t i, const float *p) { return make_float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
static inline void vstore3(float3 v, size_t i, float *p) { p[3 * i] = v.s0; p[3 * i + 1] = v.s1; p[3 * i + 2] = v.s2; }

/* ---- 2D images ----
 * The reference packs an N x 3 list into an RGBA image 8192 entries wide
 * (src/helpers/cl_helpers.py:46-81) and reads entry `index` at the
 * coordinate (index >> 13, index & 8191).  The stand-in stores the list
 * flat as [row][8192][4], so coordinate (s0, s1) is entry s0 * 8192 + s1. */
typedef int sampler_t;
#define CLK_NORMALIZED_COORDS_FALSE 0
#define CLK_ADDRESS_NONE 0
#define CLK_FILTER_NEAREST 0
struct shim_image2d { const void *data; int width; };
typedef const shim_image2d *image2d_t;
static inline uint4 read_imageui(image2d_t im, sampler_t, int2 c)
{
    const uint16_t *p = (const uint16_t *)im->data + 4 * ((size_t)c.s0 * im->width + c.s1);
    uint4 r = {p[0], p[1], p[2], p[3]};
    return r;
}
static inline float4 read_imagef(image2d_t im, sampler_t, int2 c)
{
    const float *p = (const float *)im->data + 4 * ((size_t)c.s0 * im->width + c.s1);
    return make_float4(p[0], p[1], p[2], p[3]);
}

/* ---- work-item launchers ---- */
template <class F>
static void shim_launch3(size_t g0, size_t g1, size_t g2, F f)
{
#pragma omp parallel for schedule(static)
    for (long z = 0; z < (long)g2; ++z) {
        shim_gsz[0] = g0; shim_gsz[1] = g1; shim_gsz[2] = g2;
        for (size_t y = 0; y < g1; ++y)
            for (size_t x = 0; x < g0; ++x) {
                shim_gid[0] = x; shim_gid[1] = y; shim_gid[2] = (size_t)z;
                f();
            }
    }
}
template <class F>
static void shim_launch1(size_t n, F f)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; ++i) {
        shim_gsz[0] = n; shim_gsz[1] = 1; shim_gsz[2] = 1;
        shim_gid[0] = (size_t)i; shim_gid[1] = 0; shim_gid[2] = 0;
        f();
    }
}

#endif /* ORACLE_CLSHIM_HPP */
