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

// ---- packed pairs (sm_100+ f32x2 instructions) -----------------------------------------
// Two floats in one 64-bit register pair; every packed operation rounds each lane
// to nearest on its own, so a lane gets exactly the bits the scalar intrinsic
// (__fadd_rn, __fmul_rn, __fmaf_rn) gives, in half the instructions.
typedef unsigned long long fp2;
__device__ __forceinline__ fp2 pk2(float lo, float hi) {
    fp2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float lo2(fp2 v) {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return a;
}
__device__ __forceinline__ float hi2(fp2 v) {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return b;
}
__device__ __forceinline__ fp2 add2(fp2 a, fp2 b) {
    fp2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ fp2 sub2(fp2 a, fp2 b) {
    fp2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ fp2 mul2(fp2 a, fp2 b) {
    fp2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ fp2 fma2(fp2 a, fp2 b, fp2 c) {  // a * b + c, one rounding per lane
    fp2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ fp2 splat2(float v) { return pk2(v, v); }

// ---- correctly rounded square root and reciprocal, two lanes at once -------------------
// For s in [2^-100, 2^100):  q = RN(sqrt(s))  and  r = RN(1 / q), bit for bit what
// __fsqrt_rn(s) and __frcp_rn(__fsqrt_rn(s)) return (checked against them on every
// float of that range by visg_selftest_exact_math).  Method: Markstein's correction
// of a hardware approximation by one Newton step whose residual an FMA forms with a
// single rounding (P. W. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Develop. 34(1), 1990; the square-root form is
// the one of M. Cornea, J. Harrison, P. T. P. Tang, "Scientific Computing on
// Itanium-based Systems", Intel Press, 2002, ch. 8):
//   y ~ 1/sqrt(s) (rsqrt.approx), g = s y, h = y/2;  d = s - g^2 (one FMA);  q = g + d h.
//   z ~ 1/q (rcp.approx);  e = 1 - q z (one FMA);  r = z + z e.
// Lanes outside the range take the intrinsics.  (Below 2^-100 the remainder s - g^2
// can fall among the subnormals and lose the bits the last correction needs.)
constexpr uint32_t kExactLo = 27u << 23;                     // 2^-100
constexpr uint32_t kExactSpan = (227u << 23) - (27u << 23);  // up to 2^100
__device__ __forceinline__ bool exact_fast_domain(float s) { return __float_as_uint(s) - kExactLo < kExactSpan; }

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void sqrt_rcp_pair(fp2 s, fp2& q, fp2& r) {
    const float sa = lo2(s), sb = hi2(s);
    if (exact_fast_domain(sa) && exact_fast_domain(sb)) {
        const fp2 y = pk2(rsqrt_approx(sa), rsqrt_approx(sb));
        const fp2 nh = mul2(y, splat2(-0.5f));  // -h
        const fp2 g = mul2(s, y);
        const fp2 dn = fma2(g, g, mul2(s, splat2(-1.0f)));  // g^2 - s
        q = fma2(dn, nh, g);                                // g + (s - g^2) h
        const fp2 nq = mul2(q, splat2(-1.0f));
        fp2 z = pk2(rcp_approx(lo2(q)), rcp_approx(hi2(q)));
        const fp2 e = fma2(nq, z, splat2(1.0f));
        r = fma2(z, e, z);
    } else {
        const float qa = __fsqrt_rn(sa), qb = __fsqrt_rn(sb);
        q = pk2(qa, qb);
        r = pk2(__frcp_rn(qa), __frcp_rn(qb));
    }
}

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
