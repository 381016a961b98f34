#pragma once
// rt_ff.cuh -- float-float (unevaluated sum of two FP32 numbers, about 48
// significant bits) arithmetic and the exact integer slicing of FP64 and
// float-float values into pre-scaled 7-bit BF16 digits.
//
// Slicing: every value x of a row (or column) with |x| < 2^S is written as
//   x ~= 2^S * sum_{t=1..s} d_t 2^(-7t),  d_1 in [-128,128], d_t in [-64,64],
// computed with integer arithmetic on the bit patterns (round to nearest of
// x * 2^(7s-S), then balanced base-128 digits).  Digit t is stored as the
// BF16 number d_t * 2^(-7(t-2)) (exact: at most 8 significant bits), so
// that the product of digits t and u carries the weight 2^(-7(t+u-4)) of the
// products it is summed with.
//
// Exactness of the FP32 sums of the three leading product diagonals (1, 2
// and 3 digit products per k) over a GEMM depth K: with d_1 in [-128,128] a
// diagonal reaches 16384, 16384 and 20480 units per k, below 2^24 units for
// K <= 819 ("narrow" slicing).  Deeper operands are sliced "wide": S one
// larger (|x| < 2^(S-1)), so every digit lies in [-64,64], at most 4096
// units per product, exact for K <= 1365, at the cost of one bit.
constexpr int KMAX_NARROW = 819;
constexpr int KMAX_EXACT = 1365;
__host__ __device__ __forceinline__ int slicing_wide(long long K) { return K > KMAX_NARROW ? 1 : 0; }

#include <cuda_bf16.h>
#include <stdint.h>

namespace rt {

struct ff {
    float hi, lo;
};

__host__ __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__host__ __device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    e = b - (s - a);
}

// a + sg * b, sg = +-1
__host__ __device__ __forceinline__ float2 ff_add(float2 a, float2 b, float sg) {
    float s, e;
    two_sum(a.x, sg * b.x, s, e);
    float t = a.y + sg * b.y + e;
    float h, l;
    fast_two_sum(s, t, h, l);
    return make_float2(h, l);
}

__host__ __device__ __forceinline__ double ff_to_double(float2 a) {
    return (double)a.x + (double)a.y;
}

// slicing exponent S of a double: |x| < 2^(S-wide) (S = -2000 for zero/denormal)
__host__ __device__ __forceinline__ int scale_exp_f64(double x, int wide) {
    union { double d; uint64_t u; } v;
    v.d = x;
    int e = (int)((v.u >> 52) & 0x7FF);
    return e == 0 ? -2000 : e - 1022 + wide;
}

__host__ __device__ __forceinline__ int scale_exp_f32(float x, int wide) {
    union { float f; uint32_t u; } v;
    v.f = x;
    int e = (int)((v.u >> 23) & 0xFF);
    return e == 0 ? -2000 : e - 126 + wide;
}

// round(|m| * 2^shift) for a non-negative integer mantissa m (< 2^53)
__host__ __device__ __forceinline__ int64_t shift_round(uint64_t m, int shift) {
    if (shift >= 0) return (int64_t)(m << (shift > 10 ? 10 : shift));  // callers keep shift <= 10
    int r = -shift;
    if (r >= 63) return 0;
    return (int64_t)((m + (1ull << (r - 1))) >> r);
}

// fixed-point integer round(x * 2^(7s - S)) of a double
__host__ __device__ __forceinline__ int64_t fixed_f64(double x, int S, int s) {
    union { double d; uint64_t u; } v;
    v.d = x;
    int e = (int)((v.u >> 52) & 0x7FF);
    if (e == 0) return 0;
    uint64_t m = (v.u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    int64_t X = shift_round(m, e - 1075 + 7 * s - S);
    return (v.u >> 63) ? -X : X;
}

__host__ __device__ __forceinline__ int64_t fixed_f32(float x, int S, int s) {
    union { float f; uint32_t u; } v;
    v.f = x;
    int e = (int)((v.u >> 23) & 0xFF);
    if (e == 0) return 0;
    uint64_t m = (uint64_t)((v.u & 0x7FFFFFu) | (1u << 23));
    int shift = e - 150 + 7 * s - S;
    int64_t X;
    if (shift >= 0) X = (int64_t)(m << (shift > 39 ? 39 : shift));
    else X = shift_round(m, shift);
    return (v.u >> 31) ? -X : X;
}

// balanced base-128 digits of X (|X| <= 2^(7s)+1): d[0] = d_1 ... d[s-1] = d_s
__host__ __device__ __forceinline__ void digits7(int64_t X, int s, int* d) {
    for (int t = s - 1; t >= 1; --t) {
        int64_t q = (X + 64) >> 7;  // arithmetic shift: floor division
        d[t] = (int)(X - q * 128);
        X = q;
    }
    d[0] = (int)X;
}

// BF16 value of digit t (0-based) pre-scaled by 2^(-7(t-1))
__device__ __forceinline__ __nv_bfloat16 digit_bf16(int d, int t) {
    return __float2bfloat16_rn(ldexpf((float)d, -7 * (t - 1)));
}

// 2^k as a float for -126 <= k <= 127 (0 below)
__host__ __device__ __forceinline__ float pow2f_safe(int k) {
    if (k < -126) return 0.0f;
    if (k > 127) k = 127;
    union { uint32_t u; float f; } v;
    v.u = (uint32_t)(k + 127) << 23;
    return v.f;
}

// Float-float split of a double by bit operations (no FP64 arithmetic):
// hi = the leading 24 mantissa bits (truncated), lo = the remaining 29 bits
// rounded to 24.  hi + lo = x to 2^-48 relative.  |x| must lie in the
// normal float range (values beyond it give hi = lo = 0 or saturate).
__device__ __forceinline__ float2 ff_from_double(double x) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const int e = (int)((u >> 52) & 0x7FF);
    const int fe = e - 1023 + 127;
    if (e == 0 || fe <= 0) return make_float2(0.f, 0.f);
    const uint32_t sign = (uint32_t)(u >> 63) << 31;
    const uint64_t m = u & 0xFFFFFFFFFFFFFull;
    const float hi = __uint_as_float(sign | ((uint32_t)min(fe, 254) << 23) | (uint32_t)(m >> 29));
    const float rest = (float)(uint32_t)(m & 0x1FFFFFFFu);  // units of 2^(e-1075)
    float lo = rest * pow2f_safe(e - 1075 + 0) ;
    if (e - 1075 < -126) lo = rest * pow2f_safe(e - 1075 + 64) * 5.421010862427522e-20f;  // 2^-64
    return make_float2(hi, sign ? -lo : lo);
}

// Digits of a float-float value y = yh + yl with |y| < 1 (already scaled by
// 2^-S): d_1 = rint(128 yh) in [-128,128] ([-64,64] when |y| < 1/2, wide
// slicing), then d_t in [-64,64]; each step is exact (products by 128, rint,
// Sterbenz subtraction, TwoSum).
// Writes the pre-scaled BF16 digits d_t * 2^(-7(t-2)) to out[t].
template <int S>
__device__ __forceinline__ void ff_digits(float yh, float yl, __nv_bfloat16* out) {
#pragma unroll
    for (int t = 0; t < S; ++t) {
        const float a = yh * 128.0f, b = yl * 128.0f;
        const float d = rintf(a);
        const float r = a - d;
        float h, l;
        two_sum(r, b, h, l);
        yh = h;
        yl = l;
        out[t] = __float2bfloat16_rn(d * pow2f_safe(7 - 7 * t));
    }
}

}  // namespace rt
