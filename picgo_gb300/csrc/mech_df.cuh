// Double-float arithmetic for the mixed engine's ill-conditioned excluded-
// volume pairs: a value is the unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi) / 2, about 48 significant bits, computed on the FP32 pipe.
//
// Why: on this GPU a warp's FP64 instruction holds its SM sub-partition's FP64
// pipe for ~78 cycles whatever the number of active lanes, so the pair formula
// (~1,000 FP64 operations) takes ~37 us for even one pair; the same formula in
// double-float runs ~10 FP32 operations per operation at the FP32 rate.
//
// Algorithms (published): Knuth's TwoSum and Dekker's FastTwoSum; TwoProd by
// FMA; the accurate double-word addition (two TwoSums) and the division with
// one correction step of Hida, Li and Bailey's double-double library (2001),
// restated for floats; square root by one Newton correction of the float
// root.  The arctangent reduces |t| <= 1 to |u| <= 1/128 around the nearest
// k/64 with atan t = atan(k/64) + atan((t - k/64) / (1 + t k/64)), the table
// evaluated at compile time from Euler's series
//   atan x = sum_n 2^(2n) (n!)^2 / (2n+1)! * x^(2n+1) / (1 + x^2)^(n+1),
// and sums u - u^3/3 + u^5/5 - u^7/7 + u^9/9.
//
// Only what the pair formulas use is defined; comparisons order by (hi, lo).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace mech {

// the overloads below would hide the C library's functions from unqualified
// calls inside this namespace; keep both visible
using ::atan2;
using ::fabs;
using ::fmax;
using ::sqrt;

__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void df_fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

struct df {
    float hi, lo;
    df() = default;
    __device__ __forceinline__ constexpr df(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ constexpr df(int v) : hi((float)v), lo(0.f) {}   // small integers: exact
    __device__ __forceinline__ constexpr df(float v) : hi(v), lo(0.f) {}
    // constants only: the split is folded at compile time
    __device__ __forceinline__ explicit constexpr df(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
    __device__ __forceinline__ float to_float() const { return __fadd_rn(hi, lo); }
};

__device__ __forceinline__ df operator-(const df& a) { return df(-a.hi, -a.lo); }

__device__ __forceinline__ df operator+(const df& a, const df& b) {
    float s, e, t, f;
    df_two_sum(a.hi, b.hi, s, e);
    df_two_sum(a.lo, b.lo, t, f);
    e = __fadd_rn(e, t);
    df_fast_two_sum(s, e, s, e);
    e = __fadd_rn(e, f);
    df_fast_two_sum(s, e, s, e);
    return df(s, e);
}
__device__ __forceinline__ df operator-(const df& a, const df& b) { return a + (-b); }

__device__ __forceinline__ df operator*(const df& a, const df& b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);                  // a.hi * b.hi = p + e exactly
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    float s, l;
    df_fast_two_sum(p, e, s, l);
    return df(s, l);
}

__device__ __forceinline__ df operator/(const df& a, const df& b) {
    const float rb = __frcp_rn(b.hi);
    const float q1 = __fmul_rn(a.hi, rb);
    const df r = a - b * df(q1);                      // remainder, nearly exact
    const float q2 = __fmul_rn(__fadd_rn(r.hi, r.lo), rb);
    float s, e;
    df_fast_two_sum(q1, q2, s, e);
    return df(s, e);
}

__device__ __forceinline__ bool operator<(const df& a, const df& b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(const df& a, const df& b) { return b < a; }

__device__ __forceinline__ df fabs(const df& a) { return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f) ? -a : a; }
__device__ __forceinline__ df fmax(const df& a, const df& b) { return a < b ? b : a; }

// not finite (the pair formulas' usability test)
__device__ __forceinline__ bool bad_value(const df& x) { return !(fabsf(x.hi) < INFINITY) || !(fabsf(x.lo) < INFINITY); }

__device__ __forceinline__ df sqrt(const df& a) {
    if (!(a.hi > 0.f)) return df(a.hi == 0.f ? 0.f : __int_as_float(0x7fffffff), 0.f);   // 0 -> 0; < 0, NaN -> NaN
    const float s = sqrtf(a.hi);
    const float p = __fmul_rn(s, s);
    const float pe = fmaf(s, s, -p);                  // s * s = p + pe exactly
    // a - s^2 (a.hi - p is exact: s is the rounded root)
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);
    const float c = __fmul_rn(r, __fmul_rn(0.5f, __frcp_rn(s)));
    float h, l;
    df_fast_two_sum(s, c, h, l);
    return df(h, l);
}

// ---- arctangent ---------------------------------------------------------
struct DfAtanTable {
    float hi[65], lo[65];
};
constexpr double euler_atan(double x) {
    const double q = 1.0 + x * x, y = x * x / q;
    double term = x / q, sum = term;
    for (int n = 1; n < 90 && term > sum * 1e-20; ++n) {   // stop before the terms underflow
        term *= y * (2.0 * n) / (2.0 * n + 1.0);
        sum += term;
    }
    return sum;
}
constexpr DfAtanTable make_df_atan_table() {
    DfAtanTable t{};
    for (int k = 0; k <= 64; ++k) {
        const double v = euler_atan(k / 64.0);
        t.hi[k] = (float)v;
        t.lo[k] = (float)(v - (double)t.hi[k]);
    }
    return t;
}
constexpr DfAtanTable kDfAtanTable = make_df_atan_table();
__device__ const DfAtanTable g_df_atan = kDfAtanTable;

constexpr double kDfPi = 3.14159265358979323846, kDfPi2 = 1.57079632679489661923;

// atan t for 0 <= t <= 1
__device__ __forceinline__ df df_atan_unit(const df& t) {
    const int k = min(max(__float2int_rn(__fmul_rn(t.hi, 64.f)), 0), 64);
    const float t0 = __fmul_rn((float)k, 1.f / 64.f);   // exact
    const df u = (t - df(t0)) / (df(1) + t * df(t0));   // |u| <= 1/128 (a little more from rounding)
    const df u2 = u * u;
    const df u3 = u2 * u;
    // u^5/5 - u^7/7 + u^9/9 is below 2^-28 |u|: single precision suffices
    const float z = u2.hi;
    const float tail = __fmul_rn(__fmul_rn(u3.hi, z), fmaf(z, fmaf(z, 1.f / 9.f, -1.f / 7.f), 1.f / 5.f));
    const df third = u3 * df(1.0 / 3.0);
    const df base = df(__ldg(&g_df_atan.hi[k]), __ldg(&g_df_atan.lo[k]));
    return base + (u - third) + df(tail);
}

// atan2(y, x) in (-pi, pi]
__device__ __forceinline__ df atan2(const df& y, const df& x) {
    const df ay = fabs(y), ax = fabs(x);
    const bool swap = ax < ay;
    df r = df_atan_unit(swap ? ax / ay : ay / ax);
    if (swap) r = df(kDfPi2) - r;
    if (x.hi < 0.f) r = df(kDfPi) - r;
    return y.hi < 0.f ? -r : r;
}
__device__ __forceinline__ df atan_of(const df& x) { return atan2(x, df(1)); }

}  // namespace mech
