// visg_math.cuh — float3 arithmetic with one IEEE-754 rounding per operation.
//
// Every operation is written with the round-to-nearest intrinsics so that the
// compiler never contracts a multiply and an add into an FMA, whatever the build
// flags.  This reproduces the reference's GLM 0.9.9.8 expressions operation by
// operation (dot = (x*x' + y*y') + z*z', normalize(v) = v * (1/sqrt(dot(v,v))),
// vector / scalar divides each component), which is what makes the Morton codes,
// boxes and positions bit-identical to the reference's own kernels compiled
// without contraction.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace visg {

struct f3 {
    float x, y, z;
};

__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 add(f3 a, f3 b) {
    return f3{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 sub(f3 a, f3 b) {
    return f3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 mul(f3 a, float s) {
    return f3{__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)};
}
__device__ __forceinline__ f3 mul(float s, f3 a) {
    return f3{__fmul_rn(s, a.x), __fmul_rn(s, a.y), __fmul_rn(s, a.z)};
}
__device__ __forceinline__ f3 divs(f3 a, float s) {
    return f3{__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)};
}
__device__ __forceinline__ f3 divv(f3 a, f3 b) {
    return f3{__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y), __fdiv_rn(a.z, b.z)};
}
__device__ __forceinline__ float dot(f3 a, f3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return f3{__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(b.y, a.z)),
              __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(b.z, a.x)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(b.x, a.y))};
}
__device__ __forceinline__ float length(f3 v) { return __fsqrt_rn(dot(v, v)); }
// 1/sqrt(x) correctly rounded twice, as GLM's inversesqrt = 1 / sqrt(x)
__device__ __forceinline__ f3 normalize(f3 v) { return mul(v, __frcp_rn(__fsqrt_rn(dot(v, v)))); }

__device__ __forceinline__ f3 xyz(float4 v) { return f3{v.x, v.y, v.z}; }

// Order-preserving map float -> uint32 (for atomicMin/atomicMax on floats).
__device__ __forceinline__ uint32_t f2ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float ord2f(uint32_t u) {
    uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(v);
#else
    float f;
    __builtin_memcpy(&f, &v, 4);
    return f;
#endif
}

}  // namespace visg
