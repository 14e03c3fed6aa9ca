// Cylinder-cylinder excluded volume: the analytic double integral of 1/r^4
// over two segments (CylinderExclVolRepulsion.cpp:330-882, paths relative to
// medyan-5.4.0/src), with the reference's composite-Simpson fallbacks
// (:884-1254) for pairs whose analytic value is not usable.
//
// This file is compiled once per precision (MECH_EXVOL_REAL = double or
// float).  The FP64 object is built without FMA contraction: the formula is
// ill-conditioned for nearly coplanar pairs, and rounding each operation as
// written keeps the GPU within a few ulps of the CPU restatement there.  In
// mixed precision the pair geometry is single precision, with cancellation-free
// cross-product forms of the invariants; the 1/JJ * (sum) form still loses
// accuracy as the normalized triple product q = |(v12 x v34) . v31| /
// (|v12| |v34| |v31|) goes to zero (nearly coplanar or nearly touching
// segments), so pairs with q under a threshold are evaluated in FP64 by a
// second pass over a compacted list.  The reference's coplanarity move (forces
// only) is decided and applied in single precision, except for pairs whose
// test lies within rounding of its threshold, which go to the FP64 pass.
#include <cuda_runtime.h>

#include "mech_device.cuh"

#ifndef MECH_EXVOL_REAL
#define MECH_EXVOL_REAL double
#endif

namespace mech {

constexpr int kFbNodesEnergy = 400;       // Simpson intervals, energy (:929-930)
constexpr int kFbNodesForce = 10000;      // Simpson intervals, forces (:1041-1042)

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
__device__ __forceinline__ double series_atan(double x) {
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
__device__ __forceinline__ double atan_of(double x) { return series_atan(x); }
__device__ __forceinline__ float atan_of(float x) { return atanf(x); }

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

// Analytic pair energy (:427-436); NaN when unusable (inf, NaN or < -1).
template <typename T>
__device__ __forceinline__ double energy_from(const PairInv<T>& p, T kRepScaled) {
    const T U = (T)0.5 * kRepScaled / p.JJ *
                (p.CC / p.AA * p.ATG1 + p.GG / p.EE * p.ATG2 + p.DD / p.BB * p.ATG3 + p.HH / p.FF * p.ATG4);
    if (bad_value(U) || U < (T)-1) return __longlong_as_double(0x7ff8000000000000ULL);
    return (double)U;
}
// `ref` selects the reference's forms (the FP64 engine, for parity);
// otherwise the cancellation-free forms (the mixed engine's FP64 pass).
static __device__ double pair_energy_d(const double* c1, const double* c2, const double* c3, const double* c4, double kRep,
                                       bool ref = true) {
    double v12[3], v34[3], v31[3], v14[3], v32[3], v24[3];
    diffs_of(c1, c2, c3, c4, v12, v34, v31, v14, v32, v24);
    PairInv<double> p;
    pair_inv(v12, v34, v31, v14, v32, v24, p, !ref);
    return energy_from(p, kRep);
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
__device__ __forceinline__ void push_c2(const double* c1, const double* c2, const double* c3, double* out) {
    double v1[3], v2[3];
    for (int k = 0; k < 3; ++k) { v1[k] = c2[k] - c1[k]; v2[k] = c3[k] - c1[k]; }
    double n[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
    const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) out[k] = (c2[k] + (n[k] / nn) * 0.01);
}
__device__ __forceinline__ void push_c1(const double* c1, const double* c2, const double* c3, double* out) {
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

// FP64 forces of a pair at double positions, with the reference's coplanar
// move of c2 (:610-626, force path only).
static __device__ bool pair_forces_d(const double* c1, const double* c2in, const double* c3, const double* c4, double kRep,
                                     double out[4][3], bool ref = true) {
    double moved2[3];
    const double* c2 = c2in;
    if (coplanarity<double>(c1, c2in, c3, c4) < 0.1) {
        push_c2(c1, c2in, c3, moved2);
        c2 = moved2;
    }
    double v12[3], v34[3], v31[3], v14[3], v32[3], v24[3];
    diffs_of(c1, c2, c3, c4, v12, v34, v31, v14, v32, v24);
    PairInv<double> p;
    pair_inv(v12, v34, v31, v14, v32, v24, p, !ref);
    return ref ? forces_from<false>(p, v12, v34, v31, kRep, out) : forces_from<true>(p, v12, v34, v31, kRep, out);
}

// ---------------------------------------------------------------------------
// composite-Simpson fallbacks (FP64, whatever the engine precision)
// ---------------------------------------------------------------------------
struct Quad {
    double a, b, c, d, e, F;
};
__device__ __forceinline__ Quad quad_of(const double* c1, const double* c2, const double* c3, const double* c4) {
    Quad q;
    double v12[3], v34[3], v31[3];
    for (int k = 0; k < 3; ++k) { v12[k] = c2[k] - c1[k]; v34[k] = c4[k] - c3[k]; v31[k] = c1[k] - c3[k]; }
    q.a = dot3(v12, v12); q.b = dot3(v34, v34); q.c = dot3(v31, v31);
    q.d = dot3(v12, v34); q.e = dot3(v12, v31); q.F = dot3(v34, v31);
    return q;
}
__device__ __forceinline__ double r2_at(const Quad& q, double s, double t) {
    return q.c + 2 * s * q.e + s * s * q.a - 2 * t * q.F - 2 * s * t * q.d + t * t * q.b;
}
// Node i of N: endpoints 0 and 1; interior nodes at (i+1)/N, the positions
// the reference's loop visits (its node counter is advanced before use).
__device__ __forceinline__ double node(int i, int N) { return i == 0 ? 0.0 : (i == N ? 1.0 : (double)(i + 1) / N); }
__device__ __forceinline__ double weight(int i, int N) { return (i == 0 || i == N) ? 1.0 : ((i & 1) ? 4.0 : 2.0); }

template <typename Real>
__global__ void __launch_bounds__(kBlock) k_exvol_fb_energy(DevNet<Real> n) {
    __shared__ double sh[32];
    const int cnt = min(*n.ev_fb_count, kExvolFallbackCap);
    for (int k = blockIdx.x; k < cnt; k += gridDim.x) {
        const int pr = n.ev_fb_list[2 * k + 1];
        const int4 bs = n.ev_bead[pr];
        const CGState& S = n.st[n.ev_fb_list[2 * k]];
        // positions of this evaluation: the entry records the trial lambda (0: plain evaluation)
        const double lam = __longlong_as_double(((const long long*)n.ev_fb_energy)[kExvolFallbackCap + k]);
        const bool tr = lam != 0.0;
        double c1[3], c2[3], c3[3], c4[3];
        to_double(bead_at(n.x[S.xbuf], n.d, bs.x, tr, lam), c1);
        to_double(bead_at(n.x[S.xbuf], n.d, bs.y, tr, lam), c2);
        to_double(bead_at(n.x[S.xbuf], n.d, bs.z, tr, lam), c3);
        to_double(bead_at(n.x[S.xbuf], n.d, bs.w, tr, lam), c4);
        const Quad q = quad_of(c1, c2, c3, c4);
        const int N = kFbNodesEnergy;
        double acc = 0.0;
        for (int w = threadIdx.x; w < (N + 1) * (N + 1); w += blockDim.x) {
            const int i = w / (N + 1), j = w % (N + 1);
            const double r2 = r2_at(q, node(i, N), node(j, N));
            acc += weight(i, N) * weight(j, N) * (1.0 / (r2 * r2));
        }
        acc = block_sum(acc, sh);
        if (threadIdx.x == 0) {
            const double kRepScaled = (double)n.ev_k[pr] * (double)n.ev_la[pr] * (double)n.ev_lb[pr];
            const double ds = 1.0 / N;
            const double U = kRepScaled * (ds * ds / 9.0) * acc;
            n.ev_fb_energy[k] = (bad_value(U) || U < -1.0) ? -1.0 : U;
        }
        __syncthreads();
    }
}

// numeric forces: partial moments of (entry, chunk), combined by the last chunk
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_exvol_fb_force(DevNet<Real> n, double* moments, int* tickets) {
    __shared__ double sh[32];
    __shared__ int s_last;
    const int cnt = min(*n.ev_fb_count, kExvolFallbackCap);
    const int N = kFbNodesForce;
    for (int wi = blockIdx.x; wi < cnt * kFbChunks; wi += gridDim.x) {
        const int k = wi / kFbChunks, ch = wi % kFbChunks;
        const int pr = n.ev_fb_list[2 * k + 1];
        const int4 bs = n.ev_bead[pr];
        const CGState& S = n.st[n.ev_fb_list[2 * k]];
        const Real* X = n.x[S.xbuf];
        double c1[3], c2[3], c3[3], c4[3];
        to_double(load_pos(X, bs.x), c1);
        to_double(load_pos(X, bs.y), c2);
        to_double(load_pos(X, bs.z), c3);
        to_double(load_pos(X, bs.w), c4);
        const Quad q = quad_of(c1, c2, c3, c4);
        const int i0 = (int)((long long)(N + 1) * ch / kFbChunks), i1 = (int)((long long)(N + 1) * (ch + 1) / kFbChunks);
        double m[6] = {0, 0, 0, 0, 0, 0};
        for (int i = i0; i < i1; ++i) {
            const double s = node(i, N), ws = weight(i, N);
            for (int j = threadIdx.x; j <= N; j += blockDim.x) {
                const double t = node(j, N), w = ws * weight(j, N);
                const double r2 = r2_at(q, s, t);
                const double x = w * (1.0 / (r2 * r2 * r2));
                m[0] += x; m[1] += s * x; m[2] += s * s * x; m[3] += s * t * x; m[4] += t * x; m[5] += t * t * x;
            }
        }
        for (int qd = 0; qd < 6; ++qd) {
            const double v = block_sum(m[qd], sh);
            if (threadIdx.x == 0) moments[((size_t)k * kFbChunks + ch) * 6 + qd] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            const int tk = atomicAdd(tickets + k, 1);
            s_last = (tk == kFbChunks - 1);
            if (s_last) tickets[k] = 0;
        }
        __syncthreads();
        if (s_last && threadIdx.x == 0) {
            __threadfence();
            double I[6] = {0, 0, 0, 0, 0, 0};
            for (int cc = 0; cc < kFbChunks; ++cc)
                for (int qd = 0; qd < 6; ++qd) I[qd] += __ldcg(moments + ((size_t)k * kFbChunks + cc) * 6 + qd);
            const double ds = 1.0 / N;
            for (int qd = 0; qd < 6; ++qd) I[qd] *= (ds * ds / 9.0);
            const double kRepScaled = (double)n.ev_k[pr] * (double)n.ev_la[pr] * (double)n.ev_lb[pr];
            double vA[3], vB[3], vC[3], out[4][3];
            for (int kk = 0; kk < 3; ++kk) { vA[kk] = c1[kk] - c2[kk]; vB[kk] = c3[kk] - c4[kk]; vC[kk] = c3[kk] - c1[kk]; }
            bool ok = true;
            for (int kk = 0; kk < 3; ++kk) {
                out[0][kk] = 4.0 * kRepScaled * (-I[0] * vC[kk] + I[1] * (vC[kk] - vA[kk]) + I[2] * vA[kk] + I[4] * vB[kk] - I[3] * vB[kk]);
                out[1][kk] = 4.0 * kRepScaled * (-I[1] * vC[kk] - I[2] * vA[kk] + I[3] * vB[kk]);
                out[2][kk] = 4.0 * kRepScaled * (I[0] * vC[kk] + I[1] * vA[kk] - I[4] * (vB[kk] + vC[kk]) - I[3] * vA[kk] + I[5] * vB[kk]);
                out[3][kk] = 4.0 * kRepScaled * (I[4] * vC[kk] + I[3] * vA[kk] - I[5] * vB[kk]);
            }
            for (int a = 0; a < 4; ++a)
                for (int kk = 0; kk < 3; ++kk) ok = ok && !bad_value(out[a][kk]);
            if (!ok) {
                // Nothing finite is left to use: the reference exits the process
                // here (CylinderExclVolRepulsion.cpp:1195-1254).
                atomicOr(n.err, 1u);
                for (int a = 0; a < 4; ++a)
                    for (int kk = 0; kk < 3; ++kk) out[a][kk] = __longlong_as_double(0x7ff8000000000000ULL);
            }
            for (int a = 0; a < 4; ++a) {
                Real* cdst = slot_ptr(n, n.slot_base[K_EXVOL] + 4 * pr + a);
                for (int kk = 0; kk < 3; ++kk) cdst[kk] = (Real)out[a][kk];
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// main pair kernel (energy partials or force contributions)
// ---------------------------------------------------------------------------
template <typename Real>
__device__ __forceinline__ void flag_fallback(const DevNet<Real>& n, int r, int pr, double lam) {
    const int k = atomicAdd(n.ev_fb_count, 1);
    if (k < kExvolFallbackCap) {
        n.ev_fb_list[2 * k] = r;
        n.ev_fb_list[2 * k + 1] = pr;
        ((long long*)n.ev_fb_energy)[kExvolFallbackCap + k] = __double_as_longlong(lam);
    } else {
        atomicOr(n.err, 2u);
    }
}

constexpr float kMixedTauEnergy = 0.005f;  // FP64 below this normalized triple product (energy)
constexpr float kMixedTauForce = 0.02f;    // (forces, whose formula loses more to cancellation)

// Warp-aggregated append of (replica, pair) to the FP64 pair list.
template <typename Real>
__device__ __forceinline__ void append_fp64(const DevNet<Real>& n, bool need, int r, int pr) {
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(n.ev_list_count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need) {
        const int k = base + __popc(m & ((1u << lane) - 1u));
        if (k < n.n_ev) {
            n.ev_list[2 * k] = r;
            n.ev_list[2 * k + 1] = pr;
        } else {
            atomicOr(n.err, 4u);
        }
    }
}

template <typename Real>
__global__ void __launch_bounds__(kBlock) k_exvol(DevNet<Real> n, int want, int trial, int force, int tile_off) {
    __shared__ double sh[32];
    __shared__ int s_go, s_xb;
    __shared__ double s_lam;
    const int ti = tile_off + blockIdx.x;
    const Tile t = n.stile[ti];
    const int r = t.replica;
    if (threadIdx.x == 0) {
        const CGState& S = n.st[r];
        s_go = want < 0 ? (S.active != 0) : (S.phase == want);
        s_xb = S.xbuf;
        s_lam = S.lambda;
    }
    __syncthreads();
    if (!s_go) return;
    const Real* X = n.x[s_xb];
    const bool tr = trial != 0;
    const int i = t.begin + threadIdx.x;
    const bool valid = i < t.end;
    double e = 0.0;
    bool need64 = false;
    if (valid) {
        const int4 bs = n.ev_bead[i];
        const Pos<Real> p1 = bead_at(X, n.d, bs.x, tr, s_lam), p2 = bead_at(X, n.d, bs.y, tr, s_lam);
        const Pos<Real> p3 = bead_at(X, n.d, bs.z, tr, s_lam), p4 = bead_at(X, n.d, bs.w, tr, s_lam);
        const double kRepD = (double)n.ev_k[i] * (double)n.ev_la[i] * (double)n.ev_lb[i];
        if constexpr (sizeof(Real) == 8) {
            // FP64 engine: the reference's formulas, every pair
            double c1[3], c2[3], c3[3], c4[3];
            to_double(p1, c1);
            to_double(p2, c2);
            to_double(p3, c3);
            to_double(p4, c4);
            if (!force) {
                const double u = pair_energy_d(c1, c2, c3, c4, kRepD);
                if (u != u) flag_fallback(n, r, i, tr ? s_lam : 0.0);
                else e = u;
            } else {
                double out[4][3];
                const bool ok = pair_forces_d(c1, c2, c3, c4, kRepD, out);
                for (int a = 0; a < 4; ++a) {
                    Real* cdst = slot_ptr(n, n.slot_base[K_EXVOL] + 4 * i + a);
                    for (int k = 0; k < 3; ++k) cdst[k] = (Real)out[a][k];
                }
                if (!ok) flag_fallback(n, r, i, 0.0);
            }
        } else {
            // mixed engine: single precision unless the pair is ill-conditioned
            float v12[3], v34[3], v31[3], v14[3], v32[3], v24[3];
            pdiff(p2, p1, v12);
            pdiff(p4, p3, v34);
            pdiff(p1, p3, v31);
            pdiff(p4, p1, v14);
            pdiff(p2, p3, v32);
            pdiff(p4, p2, v24);
            const float cx = v12[1] * v34[2] - v12[2] * v34[1], cy = v12[2] * v34[0] - v12[0] * v34[2],
                        cz = v12[0] * v34[1] - v12[1] * v34[0];
            const float trip = fabsf(cx * v31[0] + cy * v31[1] + cz * v31[2]);
            const float q = trip / (sqrtf(dot3(v12, v12)) * sqrtf(dot3(v34, v34)) * sqrtf(dot3(v31, v31)));
            need64 = !(q >= (force ? kMixedTauForce : kMixedTauEnergy));
            if (force && !need64) {
                // the reference moves c2 0.01 nm along the unit normal of (c1, c2, c3)
                // when it judges the pair coplanar (|n . v3| < 0.1 with
                // n = (c2-c1) x (c3-c1), v3 = c4 - c1; :610-626).  Pairs whose test
                // single precision cannot decide go to FP64; the others are moved
                // here (with q >= kMixedTauForce the move leaves them well conditioned).
                const float nx = v12[1] * v31[2] - v12[2] * v31[1], ny = v12[2] * v31[0] - v12[0] * v31[2],
                            nz = v12[0] * v31[1] - v12[1] * v31[0];   // = -n
                const float nn = sqrtf(nx * nx + ny * ny + nz * nz);
                const float cop = fabsf(nx * v14[0] + ny * v14[1] + nz * v14[2]) / (nn * sqrtf(dot3(v14, v14)));
                if (!(fabsf(cop - 0.1f) >= 2e-3f)) {
                    need64 = true;
                } else if (cop < 0.1f) {
                    const float s = -0.01f / nn;
                    const float dx = s * nx, dy = s * ny, dz = s * nz;   // c2 moves by +0.01 n / |n|
                    v12[0] += dx; v12[1] += dy; v12[2] += dz;
                    v32[0] += dx; v32[1] += dy; v32[2] += dz;
                    v24[0] -= dx; v24[1] -= dy; v24[2] -= dz;
                }
            }
            if (!need64) {
                PairInv<float> pi;
                pair_inv(v12, v34, v31, v14, v32, v24, pi, true);
                if (!force) {
                    const double u = energy_from(pi, (float)kRepD);
                    if (u != u) need64 = true;
                    else e = u;
                } else {
                    float out[4][3];
                    if (forces_from<true>(pi, v12, v34, v31, (float)kRepD, out)) {
                        for (int a = 0; a < 4; ++a) {
                            Real* cdst = slot_ptr(n, n.slot_base[K_EXVOL] + 4 * i + a);
                            for (int k = 0; k < 3; ++k) cdst[k] = (Real)out[a][k];
                        }
                    } else {
                        need64 = true;
                    }
                }
            }
            if (!force) n.ev_energy[i] = need64 ? 0.0 : e;
        }
    }
    if constexpr (sizeof(Real) == 4) append_fp64(n, need64, r, i);
    if (!force && sizeof(Real) == 8) {
        e = block_sum(e, sh);
        if (threadIdx.x == 0) n.part_sp[ti] = e;
    }
}

// Mixed engine: the listed pairs in FP64 with the reference's formulas.
template <typename Real>
__global__ void __launch_bounds__(128) k_exvol_fp64(DevNet<Real> n, int trial, int force) {
    const int cnt = min(*n.ev_list_count, n.n_ev);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
        const int r = n.ev_list[2 * k], i = n.ev_list[2 * k + 1];
        const CGState& S = n.st[r];
        const Real* X = n.x[S.xbuf];
        const bool tr = trial != 0;
        const double lam = S.lambda;
        const int4 bs = n.ev_bead[i];
        double c1[3], c2[3], c3[3], c4[3];
        to_double(bead_at(X, n.d, bs.x, tr, lam), c1);
        to_double(bead_at(X, n.d, bs.y, tr, lam), c2);
        to_double(bead_at(X, n.d, bs.z, tr, lam), c3);
        to_double(bead_at(X, n.d, bs.w, tr, lam), c4);
        const double kRepD = (double)n.ev_k[i] * (double)n.ev_la[i] * (double)n.ev_lb[i];
        if (!force) {
            const double u = pair_energy_d(c1, c2, c3, c4, kRepD, false);
            if (u != u) {
                flag_fallback(n, r, i, tr ? lam : 0.0);
                n.ev_energy[i] = 0.0;
            } else {
                n.ev_energy[i] = u;
            }
        } else {
            double out[4][3];
            const bool ok = pair_forces_d(c1, c2, c3, c4, kRepD, out, false);
            for (int a = 0; a < 4; ++a) {
                Real* cdst = slot_ptr(n, n.slot_base[K_EXVOL] + 4 * i + a);
                for (int q = 0; q < 3; ++q) cdst[q] = (Real)out[a][q];
            }
            if (!ok) flag_fallback(n, r, i, 0.0);
        }
    }
}

// Mixed engine: deterministic per-tile sums of the per-pair energies.
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_exvol_tilesum(DevNet<Real> n, int want, int tile_off) {
    __shared__ double sh[32];
    const int ti = tile_off + blockIdx.x;
    const Tile t = n.stile[ti];
    const CGState& S = n.st[t.replica];
    const bool go = want < 0 ? (S.active != 0) : (S.phase == want);
    if (!go) return;
    const int i = t.begin + threadIdx.x;
    double e = i < t.end ? n.ev_energy[i] : 0.0;
    e = block_sum(e, sh);
    if (threadIdx.x == 0) n.part_sp[ti] = e;
}

template <typename Real>
static inline int ev_tiles_of(const DevNet<Real>& n, int* off) {
    *off = n.sp_tiles[K_LINKER] + n.sp_tiles[K_MOTOR];
    return n.sp_tiles[K_EXVOL];
}

template <typename Real>
int launch_exvol_energy(const DevNet<Real>& n, int want, int trial, cudaStream_t s) {
    int off = 0;
    const int nt = ev_tiles_of(n, &off);
    if (nt == 0) return 0;
    cudaMemsetAsync(n.ev_list_count, 0, sizeof(int), s);
    cudaMemsetAsync(n.ev_fb_count, 0, sizeof(int), s);
    k_exvol<Real><<<nt, kBlock, 0, s>>>(n, want, trial, 0, off);
    int k = 1;
    if (sizeof(Real) == 4) {
        k_exvol_fp64<Real><<<2 * 152, 128, 0, s>>>(n, trial, 0);
        ++k;
    }
    k_exvol_fb_energy<Real><<<64, kBlock, 0, s>>>(n);
    ++k;
    if (sizeof(Real) == 4) {
        k_exvol_tilesum<Real><<<nt, kBlock, 0, s>>>(n, want, off);
        ++k;
    }
    return k;
}

template <typename Real>
int launch_exvol_forces(const DevNet<Real>& n, int want, cudaStream_t s) {
    int off = 0;
    const int nt = ev_tiles_of(n, &off);
    if (nt == 0) return 0;
    cudaMemsetAsync(n.ev_list_count, 0, sizeof(int), s);
    cudaMemsetAsync(n.ev_fb_count, 0, sizeof(int), s);
    k_exvol<Real><<<nt, kBlock, 0, s>>>(n, want, 0, 1, off);
    int k = 1;
    if (sizeof(Real) == 4) {
        k_exvol_fp64<Real><<<2 * 152, 128, 0, s>>>(n, 0, 1);
        ++k;
    }
    k_exvol_fb_force<Real><<<4 * 152, kBlock, 0, s>>>(n, n.fb_moments, n.fb_tickets);
    return k + 1;
}

template int launch_exvol_energy<MECH_EXVOL_REAL>(const DevNet<MECH_EXVOL_REAL>&, int, int, cudaStream_t);
template int launch_exvol_forces<MECH_EXVOL_REAL>(const DevNet<MECH_EXVOL_REAL>&, int, cudaStream_t);

}  // namespace mech
