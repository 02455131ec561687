// common.cuh -- shared device helpers for the sm_103a kernels.
//
// Volumes are C-ordered (z, y, x) float32 arrays, x fastest.  Device code
// works in fp32; the quaternion helpers below restate the reference's
// (src/clcode/quaternion_math.h) for CUDA.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/miccai2016_gb300.h"

#define M16_CUDA_TRY(expr)                                \
    do {                                                  \
        cudaError_t e__ = (expr);                         \
        if (e__ != cudaSuccess) return M16_ERR_CUDA;      \
    } while (0)

namespace m16 {

constexpr int kSMs = 152;  // GB300

__host__ __device__ inline int64_t div_up(int64_t a, int64_t b) { return (a + b - 1) / b; }
__host__ __device__ inline size_t align_up(size_t a, size_t b) { return (a + b - 1) / b * b; }

// qexpand (quaternion_math.h:79-90): squeezed z-x-z Euler angles -> unit
// quaternion, scalar part first.
__device__ __forceinline__ float4 qexpand(float phi, float theta, float psi)
{
    const float pp = (phi + psi) * 0.5f;
    const float pm = (phi - psi) * 0.5f;
    float st, ct, spp, cpp, spm, cpm;
    sincosf(theta * 0.5f, &st, &ct);
    sincosf(pp, &spp, &cpp);
    sincosf(pm, &spm, &cpm);
    return make_float4(cpp * ct, cpm * st, spm * st, spp * ct);
}

// Columns of the rotation matrix of unit quaternion q (quat2matFloat3,
// quaternion_math.h:257-289).
struct Rot {
    float c0x, c0y, c0z, c1x, c1y, c1z, c2x, c2y, c2z;
};

__device__ __forceinline__ Rot quat2rot(float4 q)
{
    const float qx2 = q.y * q.y, qy2 = q.z * q.z, qz2 = q.w * q.w;
    const float qwqx = q.x * q.y, qwqy = q.x * q.z, qwqz = q.x * q.w;
    const float qxqy = q.y * q.z, qxqz = q.y * q.w, qyqz = q.z * q.w;
    Rot r;
    r.c0x = 1.f - 2.f * (qy2 + qz2); r.c0y = 2.f * (qxqy + qwqz); r.c0z = 2.f * (qxqz - qwqy);
    r.c1x = 2.f * (qxqy - qwqz); r.c1y = 1.f - 2.f * (qx2 + qz2); r.c1z = 2.f * (qyqz + qwqx);
    r.c2x = 2.f * (qxqz + qwqy); r.c2y = 2.f * (qyqz - qwqx); r.c2z = 1.f - 2.f * (qx2 + qy2);
    return r;
}

// R^T v
__device__ __forceinline__ float3 rot_t(const Rot &r, float3 v)
{
    return make_float3(r.c0x * v.x + r.c0y * v.y + r.c0z * v.z,
                       r.c1x * v.x + r.c1y * v.y + r.c1z * v.z,
                       r.c2x * v.x + r.c2y * v.y + r.c2z * v.z);
}

// R v
__device__ __forceinline__ float3 rot(const Rot &r, float3 v)
{
    return make_float3(r.c0x * v.x + r.c1x * v.y + r.c2x * v.z,
                       r.c0y * v.x + r.c1y * v.y + r.c2y * v.z,
                       r.c0z * v.x + r.c1z * v.y + r.c2z * v.z);
}

// Block-wide sum of one float per thread (blockDim.x * blockDim.y threads,
// a multiple of 32); the result is valid in thread 0.  Fixed reduction order.
__device__ __forceinline__ float block_sum(float v, float *smem32)
{
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) smem32[tid >> 5] = v;
    __syncthreads();
    float r = 0.f;
    if (tid < 32) {
        r = tid < (nthreads >> 5) ? smem32[tid] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;
}


// ---- programmatic dependent launch --------------------------------------------
// The iteration sweeps are launched with programmatic stream serialization: a
// sweep's grid may be scheduled while the previous one's last blocks still
// run, and each block waits (griddepcontrol.wait: until the previous grid has
// completed and its memory is visible) before it reads anything.  Every block
// lets the next grid launch as soon as it starts; the next grid is then
// launched once every block of this one has started, so it never takes an SM
// slot that one of this grid's blocks still needs.  Without the launch
// attribute both instructions return at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_next() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// a launch with programmatic stream serialization when pdl is set (the kernel
// waits for its predecessor itself), a plain stream-ordered launch otherwise
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, bool pdl,
                              Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace m16
