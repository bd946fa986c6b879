// Host definitions of the CUDA keywords and intrinsics that the device ZFP
// decoder (webgpu-bcmc_gb300/csrc/zfp_device.cuh) and the marching-cubes
// vertex code (mc_vertex.cuh) use, so that the same headers compile as host
// C++ for their CPU tests (test infrastructure only; the product builds the
// headers with nvcc).  Build with -ffp-contract=off: each float operation
// below then rounds on its own, as the device intrinsics do.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>
#include <algorithm>

#define __device__
#define __host__
#define __forceinline__ inline
#define __global__
#define __restrict__

using std::max;
using std::min;

struct uint2 { uint32_t x, y; };
struct uint4 { uint32_t x, y, z, w; };
struct float4 { float x, y, z, w; };
static inline uint2 make_uint2(uint32_t a, uint32_t b) { return {a, b}; }
static inline float4 make_float4(float a, float b, float c, float d) { return {a, b, c, d}; }
struct bcmc_dim3 { uint32_t x, y, z; };
static bcmc_dim3 threadIdx = {0, 0, 0};
static bcmc_dim3 blockDim = {1, 1, 1};

// funnel shifts (wrap mode: the count is taken mod 32)
static inline uint32_t __funnelshift_r(uint32_t lo, uint32_t hi, uint32_t sh)
{
    return (uint32_t)((((uint64_t)hi << 32) | lo) >> (sh & 31u));
}
static inline uint32_t __funnelshift_l(uint32_t lo, uint32_t hi, uint32_t sh)
{
    return (uint32_t)(((((uint64_t)hi << 32) | lo) << (sh & 31u)) >> 32);
}
static inline int __ffs(uint32_t x) { return x ? __builtin_ctz(x) + 1 : 0; }
// selector nibble i picks byte (sel & 7) of {x, y} for result byte i (no sign mode used)
static inline uint32_t __byte_perm(uint32_t x, uint32_t y, uint32_t s)
{
    const uint64_t xy = ((uint64_t)y << 32) | x;
    uint32_t r = 0;
    for (int i = 0; i < 4; ++i) r |= (uint32_t)((xy >> (8 * ((s >> (4 * i)) & 7u))) & 255u) << (8 * i);
    return r;
}
static inline float __int_as_float(int32_t i)
{
    float f;
    memcpy(&f, &i, 4);
    return f;
}
static inline float __int2float_rn(int32_t i) { return (float)i; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fdiv_rn(float a, float b) { return a / b; }
// round toward zero, saturating (NaN -> 0)
static inline uint32_t __float2uint_rz(float f)
{
    return !(f > 0.0f) ? 0u : (f >= 4294967296.0f ? 0xffffffffu : (uint32_t)f);
}
template <class T>
static inline T __ldg(const T* p) { return *p; }
static inline void __syncwarp(unsigned = 0xffffffffu) {}
// the encoder's word writer (not exercised by the decode test)
static inline unsigned long long atomicOr(unsigned long long* p, unsigned long long v)
{
    const unsigned long long o = *p;
    *p = o | v;
    return o;
}
