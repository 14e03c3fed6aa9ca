// Excluded-volume pair mathematics shared by the pair kernels (one object per
// engine precision) and the Hessian-vector-product kernels: the invariants of a
// segment pair, the analytic energy and forces of the double integral of 1/r^4
// (CylinderExclVolRepulsion.cpp:330-882, paths relative to medyan-5.4.0/src),
// and the reference's coplanarity test and move.  Everything here is a
// template over the arithmetic type or a static inline helper, so every
// translation unit compiles it with its own flags.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace mech {

template <typename T>
struct PairInv {
    T a, b, c, d, e, F, g, h, I, D2, E2;
    T AA, BB, CC, DD, EE, FF, GG, HH, JJ;
    T ATG1, ATG2, ATG3, ATG4;
};

// Arctangent from argument reduction and the alternating series, with + - * /
// only: compiled without contraction it rounds exactly like the oracle's
// restatement on the host, which keeps FP64 parity free of libm differences
// (nearly coplanar pairs amplify a one-ulp arctangent difference ~1e6 times).
// atan(x) = -atan(-x); = pi/2 - atan(1/x) for x > 1;
// = pi/6 + atan((sqrt(3) x - 1)/(x + sqrt(3))) for x > tan(pi/12);
// then sum_k (-1)^k x^(2k+1)/(2k+1), k <= 18.
static __device__ __forceinline__ double series_atan(double x) {
    constexpr double kPi2 = 1.5707963267948966, kPi6 = 0.52359877559829882, kSqrt3 = 1.7320508075688772,
                     kTan15 = 0.26794919243112270;
    constexpr double kInvOdd[19] = {1.0 / 1,  1.0 / 3,  1.0 / 5,  1.0 / 7,  1.0 / 9,  1.0 / 11, 1.0 / 13,
                                    1.0 / 15, 1.0 / 17, 1.0 / 19, 1.0 / 21, 1.0 / 23, 1.0 / 25, 1.0 / 27,
                                    1.0 / 29, 1.0 / 31, 1.0 / 33, 1.0 / 35, 1.0 / 37};
    const bool neg = x < 0;
    double a = neg ? -x : x;
    const bool inv = a > 1.0;
    if (inv) a = 1.0 / a;
    const bool red = a > kTan15;
    if (red) a = (a * kSqrt3 - 1.0) / (a + kSqrt3);
    const double z = a * a;
    double p = kInvOdd[18];
#pragma unroll
    for (int k = 17; k >= 0; --k) p = kInvOdd[k] - z * p;
    double r = a * p;
    if (red) r = kPi6 + r;
    if (inv) r = kPi2 - r;
    return neg ? -r : r;
}
static __device__ __forceinline__ double atan_of(double x) { return series_atan(x); }
static __device__ __forceinline__ float atan_of(float x) { return atanf(x); }

template <typename T>
__device__ __forceinline__ T dot3(const T* u, const T* v) {
    return u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
}

// Scalar products and the AA..JJ terms (:355-420) from the difference
// vectors v12 = c2 - c1, v34 = c4 - c3, v31 = c1 - c3, v14 = c4 - c1,
// v32 = c2 - c3.  `cross` selects the forms used in single precision: by
// Lagrange's identity AA = |v12 x v31|, BB = |v34 x v31|, EE = |v12 x v14|,
// FF = |v34 x v32|, and CC, DD, GG are dot products of cross products, which
// avoids the cancellation of the reference's sqrt((ac + e)(ac - e)) forms.
template <typename T>
__device__ __forceinline__ void pair_inv(const T* v12, const T* v34, const T* v31, const T* v14, const T* v32,
                                         const T* v24, PairInv<T>& p, bool cross) {
    p.a = dot3(v12, v12);
    p.b = dot3(v34, v34);
    p.c = dot3(v31, v31);
    p.d = dot3(v12, v34);
    p.e = dot3(v12, v31);
    p.F = dot3(v34, v31);
    p.g = dot3(v12, v14);
    p.h = dot3(v34, v32);
    p.I = dot3(v34, v14);
    p.D2 = dot3(v14, v14);
    p.E2 = dot3(v32, v32);
    // (c1 - c2) x (c3 - c4) . (c3 - c1) = (v12 x v34) . v31 up to sign; squared
    const T x21[3] = {v34[1] * v12[2] - v34[2] * v12[1], v34[2] * v12[0] - v34[0] * v12[2],
                      v34[0] * v12[1] - v34[1] * v12[0]};
    const T trip = -(x21[0] * v31[0] + x21[1] * v31[1] + x21[2] * v31[2]);
    p.JJ = -trip * trip;
    if (cross) {
        const T x13[3] = {v12[1] * v31[2] - v12[2] * v31[1], v12[2] * v31[0] - v12[0] * v31[2],
                          v12[0] * v31[1] - v12[1] * v31[0]};
        const T x23[3] = {v34[1] * v31[2] - v34[2] * v31[1], v34[2] * v31[0] - v34[0] * v31[2],
                          v34[0] * v31[1] - v34[1] * v31[0]};
        const T x14[3] = {v12[1] * v14[2] - v12[2] * v14[1], v12[2] * v14[0] - v12[0] * v14[2],
                          v12[0] * v14[1] - v12[1] * v14[0]};
        const T x32[3] = {v34[1] * v32[2] - v34[2] * v32[1], v34[2] * v32[0] - v34[0] * v32[2],
                          v34[0] * v32[1] - v34[1] * v32[0]};
        p.AA = sqrt(dot3(x13, x13));
        p.BB = sqrt(dot3(x23, x23));
        p.EE = sqrt(dot3(x14, x14));
        p.FF = sqrt(dot3(x32, x32));
        p.CC = dot3(x13, x21);
        p.DD = dot3(x21, x23);
        p.GG = dot3(x14, x21);
    } else {
        const T ac = sqrt(p.a * p.c), bc = sqrt(p.b * p.c), aD = sqrt(p.a * p.D2), bE = sqrt(p.b * p.E2);
        p.AA = sqrt(fmax((T)0, (ac + p.e) * (ac - p.e)));
        p.BB = sqrt(fmax((T)0, (bc + p.F) * (bc - p.F)));
        p.CC = p.d * p.e - p.a * p.F;
        p.DD = p.b * p.e - p.d * p.F;
        p.EE = sqrt(fmax((T)0, (aD + p.g) * (aD - p.g)));
        p.FF = sqrt(fmax((T)0, (bE + p.h) * (bE - p.h)));
        p.GG = p.d * p.g - p.a * p.I;
    }
    p.HH = p.CC + p.GG - p.DD;
    if (cross) {
        // each arctangent difference as one atan2 (exact identities, e.g.
        // atan((a+e)/AA) - atan(e/AA) = atan2(AA, c + e) with c + e = v31 . v32),
        // free of the cancellation between two angles near +-pi/2
        p.ATG1 = atan2(p.AA, dot3(v31, v32));
        p.ATG2 = atan2(p.EE, dot3(v14, v24));
        p.ATG3 = atan2(p.BB, -dot3(v31, v14));
        p.ATG4 = atan2(p.FF, -dot3(v32, v24));
    } else {
        p.ATG1 = atan_of((p.a + p.e) / p.AA) - atan_of(p.e / p.AA);
        p.ATG2 = atan_of((p.a + p.e - p.d) / p.EE) - atan_of((p.e - p.d) / p.EE);
        p.ATG3 = atan_of((p.F) / p.BB) - atan_of((p.F - p.b) / p.BB);
        p.ATG4 = atan_of((p.d + p.F) / p.FF) - atan_of((p.d + p.F - p.b) / p.FF);
    }
}

template <typename T>
__device__ __forceinline__ void diffs_of(const double* c1, const double* c2, const double* c3, const double* c4, T* v12,
                                         T* v34, T* v31, T* v14, T* v32, T* v24) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        v12[k] = (T)(c2[k] - c1[k]);
        v34[k] = (T)(c4[k] - c3[k]);
        v31[k] = (T)(c1[k] - c3[k]);
        v14[k] = (T)(c4[k] - c1[k]);
        v32[k] = (T)(c2[k] - c3[k]);
        v24[k] = (T)(c4[k] - c2[k]);
    }
}

template <typename T>
__device__ __forceinline__ bool bad_value(T x) { return !(fabs(x) < (T)(1.0 / 0.0)); }

// Analytic pair energy (:427-436) in the arithmetic type; NaN when unusable
// (inf, NaN or < -1).
template <typename T>
__device__ __forceinline__ T energy_value(const PairInv<T>& p, T kRepScaled) {
    const T U = (T)0.5 * kRepScaled / p.JJ *
                (p.CC / p.AA * p.ATG1 + p.GG / p.EE * p.ATG2 + p.DD / p.BB * p.ATG3 + p.HH / p.FF * p.ATG4);
    if (bad_value(U) || U < (T)-1) return (T)(0.0 / 0.0);
    return U;
}
template <typename T>
__device__ __forceinline__ double energy_from(const PairInv<T>& p, T kRepScaled) {
    return (double)energy_value(p, kRepScaled);
}

// |n_hat . v3_hat| of areInPlane (MathFunctions.h:1101-1134), n = (c2-c1) x (c3-c1), v3 = c4 - c1.
template <typename T>
__device__ __forceinline__ T coplanarity(const double* c1, const double* c2, const double* c3, const double* c4) {
    T v1[3], v2[3], v3[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        v1[k] = (T)(c2[k] - c1[k]);
        v2[k] = (T)(c3[k] - c1[k]);
        v3[k] = (T)(c4[k] - c1[k]);
    }
    T n[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
    const T nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] = n[0] / nn; n[1] = n[1] / nn; n[2] = n[2] / nn;
    const T vv = sqrt(v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2]);
    v3[0] = v3[0] / vv; v3[1] = v3[1] / vv; v3[2] = v3[2] / vv;
    return fabs(n[0] * v3[0] + n[1] * v3[1] + n[2] * v3[2] - (T)0);
}

// c2 moved 0.01 nm along the unit normal of (c1, c2, c3) (MathFunctions.h:1221-1273)
static __device__ __forceinline__ void push_c2(const double* c1, const double* c2, const double* c3, double* out) {
    double v1[3], v2[3];
    for (int k = 0; k < 3; ++k) { v1[k] = c2[k] - c1[k]; v2[k] = c3[k] - c1[k]; }
    double n[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
    const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) out[k] = (c2[k] + (n[k] / nn) * 0.01);
}
static __device__ __forceinline__ void push_c1(const double* c1, const double* c2, const double* c3, double* out) {
    double v1[3], v2[3];
    for (int k = 0; k < 3; ++k) { v1[k] = c2[k] - c1[k]; v2[k] = c3[k] - c1[k]; }
    double n[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
    const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) out[k] = (c1[k] + (n[k] / nn) * 0.01);
}

// Analytic forces (:597-860) from the invariants and v1 = c2 - c1,
// v2 = c4 - c3, v3 = c1 - c3; returns false when a component is not finite.
// Fast = false divides exactly as the reference writes it (the FP64 engine's
// parity); Fast = true multiplies by the four reciprocals 1/AA, 1/EE, 1/BB,
// 1/FF instead (13 divisions per pair instead of 51; within an ulp or two of
// each quotient, for the mixed engine).
template <bool Fast, typename T>
__device__ bool forces_from(const PairInv<T>& p, const T* v1, const T* v2, const T* v3, T kRepScaled, T out[4][3]) {
    const T a = p.a, b = p.b, c = p.c, d = p.d, e = p.e, F = p.F;
    const T AA = p.AA, BB = p.BB, CC = p.CC, DD = p.DD, EE = p.EE, FF = p.FF, GG = p.GG, HH = p.HH;
    T rA = 0, rE = 0, rB = 0, rF = 0;
    if constexpr (Fast) {
        rA = (T)1 / AA;
        rE = (T)1 / EE;
        rB = (T)1 / BB;
        rF = (T)1 / FF;
    }
    // x / Y, x / Y^2, x / Y^3 for Y in {AA, EE, BB, FF}
    auto q1 = [](T x, T Y, T rY) -> T {
        if constexpr (Fast) return x * rY;
        else return x / Y;
    };
    auto q2 = [](T x, T Y, T rY) -> T {
        if constexpr (Fast) return x * (rY * rY);
        else return x / (Y * Y);
    };
    auto q3 = [](T x, T Y, T rY) -> T {
        if constexpr (Fast) return x * (rY * rY * rY);
        else return x / (Y * Y * Y);
    };
    const T invJJ = (T)1 / p.JJ;
    const T S = q1(CC, AA, rA) * p.ATG1 + q1(GG, EE, rE) * p.ATG2 + q1(DD, BB, rB) * p.ATG3 + q1(HH, FF, rF) * p.ATG4;
    const T pref = kRepScaled * invJJ / (T)2;
    const T A1 = AA * AA / (AA * AA + (a + e) * (a + e));
    const T A2 = AA * AA / (AA * AA + e * e);
    const T E1 = EE * EE / (EE * EE + (a + e - d) * (a + e - d));
    const T E2 = EE * EE / (EE * EE + (e - d) * (e - d));
    const T B1 = BB * BB / (BB * BB + F * F);
    const T B2 = BB * BB / (BB * BB + (F - b) * (F - b));
    const T F1 = FF * FF / (FF * FF + (d + F) * (d + F));
    const T F2 = FF * FF / (FF * FF + (d + F - b) * (d + F - b));
    // partials of the four terms of S in their own arguments
    const T tA_C = q1(p.ATG1, AA, rA);
    const T tA_X = q2(-(p.ATG1 * CC), AA, rA) + q3((-A1 * (a + e) + A2 * e) * CC, AA, rA);
    const T tA_e = q2((A1 - A2) * CC, AA, rA);
    const T tA_a = q2(A1 * CC, AA, rA);
    const T tE_G = q1(p.ATG2, EE, rE);
    const T tE_X = q2(-(p.ATG2 * GG), EE, rE) + q3((-E1 * (a + e - d) + E2 * (e - d)) * GG, EE, rE);
    const T tE_em = q2((E1 - E2) * GG, EE, rE);
    const T tE_a = q2(E1 * GG, EE, rE);
    const T tB_D = q1(p.ATG3, BB, rB);
    const T tB_X = q2(-(p.ATG3 * DD), BB, rB) + q3((-B1 * F + B2 * (F - b)) * DD, BB, rB);
    const T tB_fm = q2((B1 - B2) * DD, BB, rB);
    const T tB_b = q2(B1 * DD, BB, rB);
    const T tF_H = q1(p.ATG4, FF, rF);
    const T tF_X = q2(-(p.ATG4 * HH), FF, rF) + q3((-F1 * (d + F) + F2 * (d + F - b)) * HH, FF, rF);
    const T tF_dfm = q2((F1 - F2) * HH, FF, rF);
    const T tF_b = q2(F1 * HH, FF, rF);
    T G[3][3];
    G[0][0] = tA_C * (-2 * F) + tA_X * q1(c, AA, rA) + tA_a * 2 + tE_G * (2 * (F - b)) + tE_X * q1(b + c - 2 * F, EE, rE) +
              tE_a * 2 + tF_H * (-2 * b) + tF_X * q1(b, FF, rF);
    G[0][1] = tA_C * e + tE_G * (2 * d - e) + tE_X * q1(e - d, EE, rE) + tE_em * (-1) + tB_D * (-F) + tF_H * (2 * d + F) +
              tF_X * q1(-(d + F), FF, rF) + tF_dfm;
    G[0][2] = tA_C * d + tA_X * q1(-e, AA, rA) + tA_e + tE_G * (-d) + tE_X * q1(-(e - d), EE, rE) + tE_em + tB_D * b +
              tF_H * (-b) + tF_X * q1(b, FF, rF);
    G[1][0] = G[0][1];
    G[1][1] = tE_G * (-2 * a) + tE_X * q1(a, EE, rE) + tB_D * (2 * e) + tB_X * q1(c, BB, rB) + tB_fm * (-2) + tB_b * 2 +
              tF_H * (-2 * (a + e)) + tF_X * q1(a + c + 2 * e, FF, rF) + tF_dfm * (-2) + tF_b * 2;
    G[1][2] = tA_C * (-a) + tE_G * a + tE_X * q1(-a, EE, rE) + tB_D * (-d) + tB_X * q1(-F, BB, rB) + tB_fm + tF_H * d +
              tF_X * q1(-(d + F), FF, rF) + tF_dfm;
    G[2][0] = G[0][2];
    G[2][1] = G[1][2];
    G[2][2] = tA_X * q1(a, AA, rA) + tE_X * q1(a, EE, rE) + tB_X * q1(b, BB, rB) + tF_X * q1(b, FF, rF);
    T J[3][3];
    J[0][0] = 2 * (-b * c + F * F);
    J[0][1] = 2 * (c * d - e * F);
    J[0][2] = 2 * (b * e - d * F);
    J[1][0] = J[0][1];
    J[1][1] = 2 * (-a * c + e * e);
    J[1][2] = 2 * (-d * e + a * F);
    J[2][0] = J[0][2];
    J[2][1] = J[1][2];
    J[2][2] = 2 * (d * d - a * b);
    bool ok = true;
    T dv[4][3];
#pragma unroll
    for (int y = 0; y < 3; ++y) {
        dv[0][y] = pref * (-invJJ * S * (J[2][y] - J[0][y]) + (G[2][y] - G[0][y]));
        dv[1][y] = pref * (-invJJ * S * (J[0][y]) + (G[0][y]));
        dv[2][y] = pref * (-invJJ * S * (-J[2][y] - J[1][y]) + (-G[2][y] - G[1][y]));
        dv[3][y] = pref * (-invJJ * S * (J[1][y]) + (G[1][y]));
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            out[q][k] = -(dv[q][0] * v1[k] + dv[q][1] * v2[k] + dv[q][2] * v3[k]);
            if (bad_value(out[q][k])) ok = false;
        }
    return ok;
}
}  // namespace mech
