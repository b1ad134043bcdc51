// f32x2.cuh - packed FP32 pairs for Blackwell's two-wide FP32 pipe
// (PTX add/sub/fma .rn.f32x2, sm_100 family).
//
// Each lane of a packed operation rounds exactly as the scalar operation
// (IEEE round-to-nearest), so a pair of independent FP32 chains can be
// computed two at a time without changing a bit of either - provided no
// product is contracted into a neighbouring sum.  ptxas contracts a packed
// mul.rn.f32x2 into a following add or sub (even under -fmad=false, and even
// when the sum is written as an FMA with a unit factor), which rounds once
// where the scalar code rounds twice.  So this header has no plain packed
// product: mul2 is an FMA whose addend is -0.0 held in a register whose value
// the compiler cannot see (a kernel argument).  a * b + (-0) equals RN(a * b)
// for every a and b, signed zeros included, and an FMA result is not
// contracted any further.
#pragma once
#include <stdint.h>

namespace taa_dev {

struct f2 {
    uint64_t v;
};

// the (-0.0, -0.0) pair the host passes to kernels that use mul2
constexpr uint64_t kNegZeroPair = 0x8000000080000000ull;

__device__ __forceinline__ f2 pk(float lo, float hi) {
    return f2{(static_cast<uint64_t>(__float_as_uint(hi)) << 32) | __float_as_uint(lo)};
}
__device__ __forceinline__ f2 dup(float a) { return pk(a, a); }
__device__ __forceinline__ float f2lo(f2 a) { return __uint_as_float(static_cast<uint32_t>(a.v)); }
__device__ __forceinline__ float f2hi(f2 a) { return __uint_as_float(static_cast<uint32_t>(a.v >> 32)); }

__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
// a * b + c with one rounding per lane
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return d;
}
// RN(a * b) per lane; z is the (-0.0, -0.0) pair from a kernel argument
__device__ __forceinline__ f2 mul2(f2 a, f2 b, f2 z) { return fma2(a, b, z); }
// sign flip of both lanes (exact)
__device__ __forceinline__ f2 neg2(f2 a) { return f2{a.v ^ 0x8000000080000000ull}; }

// A 16-byte aligned float4 as two pairs, (x, y) and (z, w).
__device__ __forceinline__ void load_pairs(const float4* p, f2& xy, f2& zw) {
    const ulonglong2 t = *reinterpret_cast<const ulonglong2*>(p);
    xy.v = t.x;
    zw.v = t.y;
}

// Correctly rounded x / d for a constant divisor, both lanes (div_const_rn).
__device__ __forceinline__ f2 div_const_rn2(f2 x, f2 neg_d, f2 rd, f2 z) {
    f2 q = mul2(x, rd, z);
    f2 r = fma2(neg_d, q, x);
    return fma2(r, rd, q);
}

}  // namespace taa_dev
