// CPU FP64 restatement of MEDYAN 5.4.0's mechanical-equilibration path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the checker the parity
// tests, the smoke test and the CPU baseline of the benchmark run against.  It
// is never linked into, loaded by or called from the product library
// (picgo_gb300/csrc), and the product path never falls back to it.
//
// It restates, loop for loop and in the reference's operation order, the
// mathematics of these reference files (paths relative to medyan-5.4.0/src):
//   Mechanics/Minimizer/CGMethod.hpp:238-373        backtracking line search
//   Mechanics/Minimizer/CGMethod.hpp:826-1743       CGMethod::minimize
//   Mechanics/Minimizer/CGMethod.cpp:43-46,317-360  CG vector helpers
//   Mechanics/ForceField/ForceFieldManager.cpp:96-290  energy / forces manager
//   Mechanics/ForceField/Filament/FilamentStretchingHarmonic.cpp:185-275
//   Mechanics/ForceField/Filament/FilamentBendingCosine.cpp:199-398
//   Mechanics/ForceField/Linker/LinkerStretchingHarmonic.cpp:191-336
//   Mechanics/ForceField/MotorGhost/MotorGhostStretchingHarmonic.cpp:234-340
//   Mechanics/ForceField/Volume/CylinderExclVolRepulsion.cpp:330-1254
//   Mechanics/ForceField/Boundary/BoundaryCylinderRepulsionExp.cpp:27-110
//   Structure/BoundaryElementImpl.h:30-106          plane distance / normal
//   Structure/HybridNeighborListImpl.cpp:332-471    half-list pair predicate
//   Structure/NeighborListImpl.cpp:738-751          boundary-cylinder list
//   Controller/MController.h:273-339                recovery move
//   MathFunctions.h:294-298,469-477,963-969,1101-1134,1221-1273; utility.h:75-83
//
// Parity status: pinned for the excluded-volume and boundary kernels and the
// CG convergence criterion by the reference's own Catch2 cases (restated in
// tests/); the other kernels have no reference test and are pinned by
// analytic known answers, energy/force consistency and finite differences.
//
// Built without -ffast-math and with -ffp-contract=off so each expression
// rounds as written.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace {

using std::sqrt;

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// (v2 - v1) . (v4 - v3), summed x, y, z (MathFunctions.h:469-477)
inline double sprod(const double* v1, const double* v2, const double* v3, const double* v4) {
    return ((v2[0] - v1[0]) * (v4[0] - v3[0]) +
            (v2[1] - v1[1]) * (v4[1] - v3[1]) +
            (v2[2] - v1[2]) * (v4[2] - v3[2]));
}

inline double dist2pt(const double* v1, const double* v2) {
    return sqrt((v2[0] - v1[0]) * (v2[0] - v1[0]) + (v2[1] - v1[1]) * (v2[1] - v1[1]) +
                (v2[2] - v1[2]) * (v2[2] - v1[2]));
}

// v = v1 * (1 - alpha) + alpha * v2  (MathFunctions.h:963-969)
inline void lerp(double* v, const double* v1, const double* v2, double alpha) {
    const double beta = 1 - alpha;
    v[0] = (v1[0] * beta + alpha * v2[0]);
    v[1] = (v1[1] * beta + alpha * v2[1]);
    v[2] = (v1[2] * beta + alpha * v2[2]);
}

inline void cross3(double* cp, const double* a, const double* b) {
    cp[0] = a[1] * b[2] - a[2] * b[1];
    cp[1] = a[2] * b[0] - a[0] * b[2];
    cp[2] = a[0] * b[1] - a[1] * b[0];
}

inline void unit3(double* v) {
    const double x2 = v[0] * v[0], y2 = v[1] * v[1], z2 = v[2] * v[2];
    const double n = sqrt(x2 + y2 + z2);
    v[0] = v[0] / n; v[1] = v[1] / n; v[2] = v[2] / n;
}

// |n_hat . v3_hat| < 0.1 with n = (p2-p1) x (p3-p1), v3 = p4 - p1
// (MathFunctions.h:1101-1134 with areEqualLT, utility.h:80-83)
bool coplanar(const double* p1, const double* p2, const double* p3, const double* p4) {
    double v1[3], v2[3], v3[3], cp[3];
    for (int k = 0; k < 3; ++k) { v1[k] = p2[k] - p1[k]; v2[k] = p3[k] - p1[k]; v3[k] = p4[k] - p1[k]; }
    cross3(cp, v1, v2);
    unit3(cp);
    unit3(v3);
    return std::fabs(dot3(v3, cp) - 0.0) < 0.1;
}

// point `which` (1..4) moved by `d` along the unit normal of plane (p1, p2, p3)
// (MathFunctions.h:1221-1273)
void push_off_plane(const double* p1, const double* p2, const double* p3, const double* p4,
                    double* out, int which, double d) {
    double v1[3], v2[3], nrm[3];
    for (int k = 0; k < 3; ++k) { v1[k] = p2[k] - p1[k]; v2[k] = p3[k] - p1[k]; }
    cross3(nrm, v1, v2);
    unit3(nrm);
    const double* src = which == 1 ? p1 : which == 2 ? p2 : which == 3 ? p3 : p4;
    for (int k = 0; k < 3; ++k) out[k] = (src[k] + nrm[k] * d);
}

inline bool bad(double x) { return std::fabs(x) == std::numeric_limits<double>::infinity() || x != x; }

// When set, force routines accumulate |contribution| instead of the
// contribution: the per-component scale that parity tolerances refer to.
bool g_abs = false;
inline void acc(double& dst, double v) { dst += g_abs ? std::fabs(v) : v; }

// Arctangent from argument reduction and the alternating series, written with
// + - * / only so that it rounds identically on every IEEE machine compiled
// without contraction.  atan(x) = -atan(-x); atan(x) = pi/2 - atan(1/x) for
// x > 1; atan(x) = pi/6 + atan((sqrt(3) x - 1) / (x + sqrt(3))) for
// x > tan(pi/12); then sum_k (-1)^k x^(2k+1) / (2k+1) to k = 18.
double series_atan(double x) {
    const double kPi2 = 1.5707963267948966, kPi6 = 0.52359877559829882, kSqrt3 = 1.7320508075688772,
                 kTan15 = 0.26794919243112270;
    const bool neg = x < 0;
    double a = neg ? -x : x;
    const bool inv = a > 1.0;
    if (inv) a = 1.0 / a;
    const bool red = a > kTan15;
    if (red) a = (a * kSqrt3 - 1.0) / (a + kSqrt3);
    const double z = a * a;
    double p = 1.0 / 37.0;
    for (int k = 17; k >= 0; --k) p = 1.0 / (2 * k + 1) - z * p;
    double r = a * p;
    if (red) r = kPi6 + r;
    if (inv) r = kPi2 - r;
    return neg ? -r : r;
}
bool g_series_atan = false;
inline double atan_(double x) { return g_series_atan ? series_atan(x) : std::atan(x); }

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Filament stretching, harmonic (FilamentStretchingHarmonic.cpp:185-275)
// U = 1/2 k (|b2 - b1| - l0)^2 ; F_b2 += -f0 (b2 - b1), F_b1 -= same, f0 = k (L - l0)/L
// ---------------------------------------------------------------------------
double orc_stretch_energy(const double* coord, int n, const int* bs, const double* k, const double* l0) {
    double U = 0.0;
    for (int i = 0; i < n; ++i) {
        const double* c1 = coord + bs[2 * i];
        const double* c2 = coord + bs[2 * i + 1];
        const double dist = dist2pt(c1, c2) - l0[i];
        U += 0.5 * k[i] * dist * dist;
    }
    return U;
}

void orc_stretch_forces(const double* coord, double* f, int n, const int* bs, const double* k, const double* l0) {
    for (int i = 0; i < n; ++i) {
        const double* c1 = coord + bs[2 * i];
        const double* c2 = coord + bs[2 * i + 1];
        const double L = dist2pt(c1, c2);
        const double invL = 1 / L;
        const double f0 = k[i] * (L - l0[i]) * invL;
        double* f1 = f + bs[2 * i];
        double* f2 = f + bs[2 * i + 1];
        const double F[3] = {-f0 * (c2[0] - c1[0]), -f0 * (c2[1] - c1[1]), -f0 * (c2[2] - c1[2])};
        for (int d = 0; d < 3; ++d) acc(f2[d], F[d]);
        for (int d = 0; d < 3; ++d) acc(f1[d], -F[d]);
    }
}

// ---------------------------------------------------------------------------
// Filament bending, cosine (FilamentBendingCosine.cpp:199-345)
// x = (b2-b1).(b3-b2)/(L1 L2) clamped; U = k (1 - x) if theta0 ~ 0 else k (1 - cos(theta - theta0))
// ---------------------------------------------------------------------------
static inline bool near_zero(double t) { return std::fabs(t - 0.0) < 1e-6; }  // areEqual, utility.h:75-78

double orc_bend_energy(const double* coord, int n, const int* bs, const double* k, const double* t0) {
    double U = 0.0;
    for (int i = 0; i < n; ++i) {
        const double* c1 = coord + bs[3 * i];
        const double* c2 = coord + bs[3 * i + 1];
        const double* c3 = coord + bs[3 * i + 2];
        const double L1 = sqrt(sprod(c1, c2, c1, c2));
        const double L2 = sqrt(sprod(c2, c3, c2, c3));
        const double L1L2 = L1 * L2;
        const double l1l2 = sprod(c1, c2, c2, c3);
        double x = l1l2 / L1L2;
        if (x < -1.0) x = -1.0;
        else if (x > 1.0) x = 1.0;
        double Ui;
        if (near_zero(t0[i])) {
            Ui = k[i] * (1 - x);
        } else {
            const double cosA = x;
            const double sinA = std::max(sqrt(1 - cosA * cosA), 0.0);
            const double cosAmB = cosA * std::cos(t0[i]) + sinA * std::sin(t0[i]);
            Ui = k[i] * (1 - cosAmB);
        }
        U += Ui;
    }
    return U;
}

void orc_bend_forces(const double* coord, double* f, int n, const int* bs, const double* k, const double* t0) {
    for (int i = 0; i < n; ++i) {
        const double* c1 = coord + bs[3 * i];
        const double* c2 = coord + bs[3 * i + 1];
        const double* c3 = coord + bs[3 * i + 2];
        const double L1sq = sprod(c1, c2, c1, c2);
        const double L2sq = sprod(c2, c3, c2, c3);
        const double l1l2 = sprod(c1, c2, c2, c3);
        const double A = 1 / sqrt(L1sq * L2sq);
        double x = l1l2 * A;
        const double B = x / L1sq;
        const double C = x / L2sq;
        double kk;
        if (near_zero(t0[i])) {
            kk = k[i];
        } else {
            if (std::fabs(std::fabs(x) - 1.0) < 0.001) x = 0.999 * x;
            if (x < -1.0) x = -1.0;
            else if (x > 1.0) x = 1.0;
            const double cosp = x;
            const double sinp = sqrt(std::max((1 - cosp * cosp), 0.0));
            const double sinpmq = sinp * std::cos(t0[i]) - cosp * std::sin(t0[i]);
            kk = k[i] * sinpmq / sinp;
        }
        double r1[3], r2[3], F1[3], F2[3];
        for (int d = 0; d < 3; ++d) { r1[d] = c2[d] - c1[d]; r2[d] = c3[d] - c2[d]; }
        for (int d = 0; d < 3; ++d) {
            F1[d] = kk * (r2[d] * A - r1[d] * B);
            F2[d] = kk * (r1[d] * A - r2[d] * C);
        }
        double* f1 = f + bs[3 * i];
        double* f2 = f + bs[3 * i + 1];
        double* f3 = f + bs[3 * i + 2];
        for (int d = 0; d < 3; ++d) acc(f1[d], -F1[d]);
        for (int d = 0; d < 3; ++d) acc(f2[d], F1[d] - F2[d]);
        for (int d = 0; d < 3; ++d) acc(f3[d], F2[d]);
    }
}

// ---------------------------------------------------------------------------
// Linker / motor harmonic stretching between interpolated points
// (LinkerStretchingHarmonic.cpp:191-293, MotorGhostStretchingHarmonic.cpp:234-340)
// ---------------------------------------------------------------------------
double orc_bond_energy(const double* coord, int n, const int* bs, const double* k, const double* l0,
                       const double* s1, const double* s2) {
    double U = 0.0;
    for (int i = 0; i < n; ++i) {
        double v1[3], v2[3];
        lerp(v1, coord + bs[4 * i], coord + bs[4 * i + 1], s1[i]);
        lerp(v2, coord + bs[4 * i + 2], coord + bs[4 * i + 3], s2[i]);
        const double dist = dist2pt(v1, v2) - l0[i];
        U += 0.5 * k[i] * dist * dist;
    }
    return U;
}

void orc_bond_forces(const double* coord, double* f, int n, const int* bs, const double* k, const double* l0,
                     const double* s1, const double* s2, double* stretchforce) {
    for (int i = 0; i < n; ++i) {
        double v1[3], v2[3];
        lerp(v1, coord + bs[4 * i], coord + bs[4 * i + 1], s1[i]);
        lerp(v2, coord + bs[4 * i + 2], coord + bs[4 * i + 3], s2[i]);
        const double dist = dist2pt(v1, v2);
        const double invL = 1 / dist;
        const double f0 = k[i] * (dist - l0[i]) * invL;
        double Fl[3];
        for (int d = 0; d < 3; ++d) Fl[d] = -f0 * (v2[d] - v1[d]);
        double* f1 = f + bs[4 * i];
        double* f2 = f + bs[4 * i + 1];
        double* f3 = f + bs[4 * i + 2];
        double* f4 = f + bs[4 * i + 3];
        for (int d = 0; d < 3; ++d) acc(f1[d], -Fl[d] * (1 - s1[i]));
        for (int d = 0; d < 3; ++d) acc(f2[d], -Fl[d] * (s1[i]));
        for (int d = 0; d < 3; ++d) acc(f3[d], Fl[d] * (1 - s2[i]));
        for (int d = 0; d < 3; ++d) acc(f4[d], Fl[d] * (s2[i]));
        if (stretchforce) stretchforce[i] = f0 / invL;
    }
}

// ---------------------------------------------------------------------------
// Cylinder-cylinder excluded volume (CylinderExclVolRepulsion.cpp)
// ---------------------------------------------------------------------------

// Invariants of a segment pair.  v1 = c2 - c1, v2 = c4 - c3, v3 = c1 - c3.
struct PairInv {
    double a, b, c, d, e, F, g, h, I, D2, E2;
    double AA, BB, CC, DD, EE, FF, GG, HH, JJ;
    double ATG1, ATG2, ATG3, ATG4;
};

// Shared front half of the analytic energy and force (:355-420, :637-700):
// scalar products, the loss-of-significance-safe AA..FF forms, the triple
// product JJ = -((c1-c2) x (c3-c4) . (c3-c1))^2, and the four arctangent
// differences.
static void pair_invariants(const double* c1, const double* c2, const double* c3, const double* c4, PairInv& p) {
    p.a = sprod(c1, c2, c1, c2);
    p.b = sprod(c3, c4, c3, c4);
    p.c = sprod(c3, c1, c3, c1);
    p.d = sprod(c1, c2, c3, c4);
    p.e = sprod(c1, c2, c3, c1);
    p.F = sprod(c3, c4, c3, c1);
    p.g = sprod(c1, c2, c1, c4);
    p.h = sprod(c3, c4, c3, c2);
    p.I = sprod(c3, c4, c1, c4);
    {   // |c1 - c4|^2 and |c3 - c2|^2 as (c1 - c2)^2 summed (MathFunctions.h:203-210)
        double x = c1[0] - c4[0], y = c1[1] - c4[1], z = c1[2] - c4[2];
        p.D2 = (x * x + y * y + z * z);
        x = c3[0] - c2[0]; y = c3[1] - c2[1]; z = c3[2] - c2[2];
        p.E2 = (x * x + y * y + z * z);
    }
    double A[3], Bv[3], Cv[3], cp[3];
    for (int k = 0; k < 3; ++k) { A[k] = c1[k] - c2[k]; Bv[k] = c3[k] - c4[k]; Cv[k] = c3[k] - c1[k]; }
    const double ac = sqrt(p.a * p.c);
    const double bc = sqrt(p.b * p.c);
    const double aD = sqrt(p.a * p.D2);
    const double bE = sqrt(p.b * p.E2);
    p.AA = sqrt(std::max(0.0, (ac + p.e) * (ac - p.e)));
    p.BB = sqrt(std::max(0.0, (bc + p.F) * (bc - p.F)));
    p.CC = p.d * p.e - p.a * p.F;
    p.DD = p.b * p.e - p.d * p.F;
    p.EE = sqrt(std::max(0.0, (aD + p.g) * (aD - p.g)));
    p.FF = sqrt(std::max(0.0, (bE + p.h) * (bE - p.h)));
    p.GG = p.d * p.g - p.a * p.I;
    p.HH = p.CC + p.GG - p.DD;
    cross3(cp, A, Bv);
    const double trip = cp[0] * Cv[0] + cp[1] * Cv[1] + cp[2] * Cv[2];
    p.JJ = -trip * trip;
    p.ATG1 = atan_((p.a + p.e) / p.AA) - atan_(p.e / p.AA);
    p.ATG2 = atan_((p.a + p.e - p.d) / p.EE) - atan_((p.e - p.d) / p.EE);
    p.ATG3 = atan_((p.F) / p.BB) - atan_((p.F - p.b) / p.BB);
    p.ATG4 = atan_((p.d + p.F) / p.FF) - atan_((p.d + p.F - p.b) / p.FF);
}

// 1 / r(s,t)^4 and its r^-6 moments on the two segments (CylinderExclVolRepulsion.h:53-72)
static inline double r2_of(double a, double b, double c, double d, double e, double F, double s, double t) {
    return c + 2 * s * e + s * s * a - 2 * t * F - 2 * s * t * d + t * t * b;
}

// 2-D composite Simpson fallback for the energy (:884-982).  The interior
// nodes are (i+1)/N, as in the reference's loop, whose node counter is
// advanced before first use.
static double exvol_energy_numeric(const double* c1, const double* c2, const double* c3, const double* c4,
                                   double kRepScaled, int N) {
    const double a = sprod(c1, c2, c1, c2), b = sprod(c3, c4, c3, c4), c = sprod(c3, c1, c3, c1);
    const double d = sprod(c1, c2, c3, c4), e = sprod(c1, c2, c3, c1), F = sprod(c3, c4, c3, c1);
    auto integrand = [&](double s, double t) {
        const double r2 = r2_of(a, b, c, d, e, F, s, t);
        return (1.0 / (r2 * r2));
    };
    const double ds = 1.0 / double(N), dt = 1.0 / double(N);
    const double T1 = integrand(0.0, 0.0) + integrand(0.0, 1.0) + integrand(1.0, 0.0) + integrand(1.0, 1.0);
    double T2 = 0, T3 = 0, T4 = 0, s = 0.0;
    for (int i = 0; i <= N; ++i) {
        double t = 0.0;
        s += ds;
        const double ws = (i % 2 == 0) ? 2.0 : 4.0;
        if (i > 0 && i < N) T2 += ws * (integrand(s, 0.0) + integrand(s, 1.0));
        for (int j = 0; j <= N; ++j) {
            t += dt;
            const double wt = (j % 2 == 0) ? 2.0 : 4.0;
            if (j > 0 && j < N) {
                if (i == 0) T3 += wt * (integrand(0.0, t) + integrand(1.0, t));
                else if (i < N) T4 += ws * wt * integrand(s, t);
            }
        }
    }
    return kRepScaled * (ds * dt / 9.0) * (T1 + T2 + T3 + T4);
}

static int g_exvol_force_N = 10000;   // Simpson nodes of the force fallback (:1041)
void orc_set_exvol_force_nodes(int n) { g_exvol_force_N = n; }

// Composite Simpson fallback for the forces (:1001-1254); returns false when
// the result is not finite.
static bool exvol_forces_numeric(const double* c1, const double* c2, const double* c3, const double* c4,
                                 double kRepScaled, double out[4][3]) {
    const double a = sprod(c1, c2, c1, c2), b = sprod(c3, c4, c3, c4), c = sprod(c3, c1, c3, c1);
    const double d = sprod(c1, c2, c3, c4), e = sprod(c1, c2, c3, c1), F = sprod(c3, c4, c3, c1);
    double vA[3], vB[3], vC[3];
    for (int k = 0; k < 3; ++k) { vA[k] = c1[k] - c2[k]; vB[k] = c3[k] - c4[k]; vC[k] = c3[k] - c1[k]; }
    const int N = g_exvol_force_N;
    auto moments = [&](double s, double t, double* m) {
        const double r2 = r2_of(a, b, c, d, e, F, s, t);
        const double x = (1.0 / (r2 * r2 * r2));
        m[0] = x; m[1] = s * x; m[2] = s * s * x; m[3] = s * t * x; m[4] = t * x; m[5] = t * t * x;
    };
    const double ds = 1.0 / double(N), dt = 1.0 / double(N);
    double T1[6] = {0}, T2[6] = {0}, T3[6] = {0}, T4[6] = {0}, m[6];
    const double lim[2] = {0.0, 1.0};
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            moments(lim[i], lim[j], m);
            for (int q = 0; q < 6; ++q) T1[q] += m[q];
        }
    double s = 0.0;
    for (int i = 0; i <= N; ++i) {
        double t = 0.0;
        s += ds;
        const double ws = (i % 2 == 0) ? 2.0 : 4.0;
        if (i > 0 && i < N)
            for (int l = 0; l < 2; ++l) {
                moments(s, lim[l], m);
                for (int q = 0; q < 6; ++q) T2[q] += ws * m[q];
            }
        for (int j = 0; j <= N; ++j) {
            t += dt;
            const double wt = (j % 2 == 0) ? 2.0 : 4.0;
            if (j > 0 && j < N) {
                if (i == 0) {
                    for (int l = 0; l < 2; ++l) {
                        moments(lim[l], t, m);
                        for (int q = 0; q < 6; ++q) T3[q] += wt * m[q];
                    }
                } else if (i < N) {
                    moments(s, t, m);
                    for (int q = 0; q < 6; ++q) T4[q] += ws * wt * m[q];
                }
            }
        }
    }
    double I[6];
    for (int q = 0; q < 6; ++q) I[q] = (ds * dt / 9.0) * (T1[q] + T2[q] + T3[q] + T4[q]);
    bool ok = true;
    for (int k = 0; k < 3; ++k) {
        out[0][k] = 4.0 * kRepScaled * (-I[0] * vC[k] + I[1] * (vC[k] - vA[k]) + I[2] * vA[k] + I[4] * vB[k] - I[3] * vB[k]);
        out[1][k] = 4.0 * kRepScaled * (-I[1] * vC[k] - I[2] * vA[k] + I[3] * vB[k]);
        out[2][k] = 4.0 * kRepScaled * (I[0] * vC[k] + I[1] * vA[k] - I[4] * (vB[k] + vC[k]) - I[3] * vA[k] + I[5] * vB[k]);
        out[3][k] = 4.0 * kRepScaled * (I[4] * vC[k] + I[3] * vA[k] - I[5] * vB[k]);
    }
    for (int q = 0; q < 4; ++q)
        for (int k = 0; k < 3; ++k)
            if (bad(out[q][k])) ok = false;
    return ok;
}

// Energy of one pair, analytic with the numeric fallback; returns the
// reference's -1 sentinel when both fail (:356-481).
double orc_exvol_pair_energy(const double* c1, const double* c2, const double* c3, const double* c4,
                             double krep, double l0a, double l0b) {
    const double kRepScaled = krep * l0a * l0b;
    PairInv p;
    pair_invariants(c1, c2, c3, c4, p);
    double Ui = 0.5 * kRepScaled / p.JJ *
                (p.CC / p.AA * p.ATG1 + p.GG / p.EE * p.ATG2 + p.DD / p.BB * p.ATG3 + p.HH / p.FF * p.ATG4);
    if (bad(Ui) || Ui < -1.0) {
        // The numeric fallback's retry with moved beads discards its own
        // result in the reference (:976-982), so only the first attempt counts.
        Ui = exvol_energy_numeric(c1, c2, c3, c4, kRepScaled, 400);
        if (bad(Ui) || Ui < -1.0) return -1.0;
    }
    return Ui;
}

double orc_exvol_energy(const double* coord, int n, const int* bs, const double* krep, const double* eqlen) {
    double U = 0.0;
    for (int i = 0; i < n; ++i) {
        const double Ui = orc_exvol_pair_energy(coord + bs[4 * i], coord + bs[4 * i + 1], coord + bs[4 * i + 2],
                                                coord + bs[4 * i + 3], krep[i], eqlen[2 * i], eqlen[2 * i + 1]);
        if (Ui == -1.0) return -1.0;
        U += Ui;
    }
    return U;
}

// Analytic forces of one pair (:597-860).  Before the analytic formula, a
// pair judged coplanar has c2 moved 0.01 nm along the plane normal; the energy
// path has no such move.  Returns 1 if the numeric fallback was used.
int orc_exvol_pair_forces(const double* c1, const double* c2in, const double* c3, const double* c4,
                          double krep, double l0a, double l0b, double out[4][3]) {
    const double kRepScaled = krep * l0a * l0b;
    double moved[3];
    const double* c2 = c2in;
    if (coplanar(c1, c2in, c3, c4)) {
        push_off_plane(c1, c2in, c3, c4, moved, 2, 0.01);
        c2 = moved;
    }
    PairInv p;
    pair_invariants(c1, c2, c3, c4, p);
    const double a = p.a, b = p.b, c = p.c, d = p.d, e = p.e, F = p.F;
    const double AA = p.AA, BB = p.BB, CC = p.CC, DD = p.DD, EE = p.EE, FF = p.FF, GG = p.GG, HH = p.HH;
    const double invJJ = 1 / p.JJ;
    const double S = CC / AA * p.ATG1 + GG / EE * p.ATG2 + DD / BB * p.ATG3 + HH / FF * p.ATG4;
    const double pref = kRepScaled * invJJ / 2;

    // d(atan(u/X))/d(u) * X reduced to X^2 / (X^2 + u^2) for each arctangent.
    const double A1 = AA * AA / (AA * AA + (a + e) * (a + e));
    const double A2 = AA * AA / (AA * AA + e * e);
    const double E1 = EE * EE / (EE * EE + (a + e - d) * (a + e - d));
    const double E2 = EE * EE / (EE * EE + (e - d) * (e - d));
    const double B1 = BB * BB / (BB * BB + F * F);
    const double B2 = BB * BB / (BB * BB + (F - b) * (F - b));
    const double F1 = FF * FF / (FF * FF + (d + F) * (d + F));
    const double F2 = FF * FF / (FF * FF + (d + F - b) * (d + F - b));

    // Partials of the four terms of S with respect to their own arguments,
    // treating (AA, CC, a, e), (EE, GG, a, e-d), (BB, DD, b, F-b) and
    // (FF, HH, b, d+F-b) as independent.
    const double tA_C = p.ATG1 / AA;
    const double tA_X = -(p.ATG1 * CC) / (AA * AA) + (-A1 * (a + e) + A2 * e) * CC / (AA * AA * AA);
    const double tA_e = ((A1 - A2) * CC) / (AA * AA);
    const double tA_a = (A1 * CC) / (AA * AA);
    const double tE_G = p.ATG2 / EE;
    const double tE_X = -(p.ATG2 * GG) / (EE * EE) + (-E1 * (a + e - d) + E2 * (e - d)) * GG / (EE * EE * EE);
    const double tE_em = ((E1 - E2) * GG) / (EE * EE);
    const double tE_a = (E1 * GG) / (EE * EE);
    const double tB_D = p.ATG3 / BB;
    const double tB_X = -(p.ATG3 * DD) / (BB * BB) + (-B1 * F + B2 * (F - b)) * DD / (BB * BB * BB);
    const double tB_fm = ((B1 - B2) * DD) / (BB * BB);
    const double tB_b = (B1 * DD) / (BB * BB);
    const double tF_H = p.ATG4 / FF;
    const double tF_X = -(p.ATG4 * HH) / (FF * FF) + (-F1 * (d + F) + F2 * (d + F - b)) * HH / (FF * FF * FF);
    const double tF_dfm = ((F1 - F2) * HH) / (FF * FF);
    const double tF_b = (F1 * HH) / (FF * FF);

    // G[x][y]: component along v_y of dS/dv_x, from the chain rule through
    // a..F (dA/dv etc. expressed in v1, v2, v3).
    double G[3][3];
    G[0][0] = tA_C * (-2 * F) + tA_X * (c / AA) + tA_a * 2 + tE_G * (2 * (F - b)) + tE_X * ((b + c - 2 * F) / EE) +
              tE_a * 2 + tF_H * (-2 * b) + tF_X * (b / FF);
    G[0][1] = tA_C * e + tE_G * (2 * d - e) + tE_X * ((e - d) / EE) + tE_em * (-1) + tB_D * (-F) + tF_H * (2 * d + F) +
              tF_X * (-(d + F) / FF) + tF_dfm;
    G[0][2] = tA_C * d + tA_X * (-e / AA) + tA_e + tE_G * (-d) + tE_X * (-(e - d) / EE) + tE_em + tB_D * b +
              tF_H * (-b) + tF_X * (b / FF);
    G[1][0] = G[0][1];
    G[1][1] = tE_G * (-2 * a) + tE_X * (a / EE) + tB_D * (2 * e) + tB_X * (c / BB) + tB_fm * (-2) + tB_b * 2 +
              tF_H * (-2 * (a + e)) + tF_X * ((a + c + 2 * e) / FF) + tF_dfm * (-2) + tF_b * 2;
    G[1][2] = tA_C * (-a) + tE_G * a + tE_X * (-a / EE) + tB_D * (-d) + tB_X * (-F / BB) + tB_fm + tF_H * d +
              tF_X * (-(d + F) / FF) + tF_dfm;
    G[2][0] = G[0][2];
    G[2][1] = G[1][2];
    G[2][2] = tA_X * (a / AA) + tE_X * (a / EE) + tB_X * (b / BB) + tF_X * (b / FF);

    // dJJ/dv_x along v_y
    double J[3][3];
    J[0][0] = 2 * (-b * c + F * F);
    J[0][1] = 2 * (c * d - e * F);
    J[0][2] = 2 * (b * e - d * F);
    J[1][0] = J[0][1];
    J[1][1] = 2 * (-a * c + e * e);
    J[1][2] = 2 * (-d * e + a * F);
    J[2][0] = J[0][2];
    J[2][1] = J[1][2];
    J[2][2] = 2 * (d * d - a * b);

    // gradient of U on c1..c4 along (v1, v2, v3): c1 = v3 - v1, c2 = v1, c3 = -v3 - v2, c4 = v2
    double deriv[4][3];
    for (int y = 0; y < 3; ++y) {
        deriv[0][y] = pref * (-invJJ * S * (J[2][y] - J[0][y]) + (G[2][y] - G[0][y]));
        deriv[1][y] = pref * (-invJJ * S * (J[0][y]) + (G[0][y]));
        deriv[2][y] = pref * (-invJJ * S * (-J[2][y] - J[1][y]) + (-G[2][y] - G[1][y]));
        deriv[3][y] = pref * (-invJJ * S * (J[1][y]) + (G[1][y]));
    }
    bool finite = true;
    for (int q = 0; q < 4; ++q)
        for (int k = 0; k < 3; ++k) {
            out[q][k] = -(deriv[q][0] * (c2[k] - c1[k]) + deriv[q][1] * (c4[k] - c3[k]) + deriv[q][2] * (c1[k] - c3[k]));
            if (bad(out[q][k])) finite = false;
        }
    if (finite) return 0;
    // Numeric fallback on the unmoved beads; a second failure retries with c1
    // and c2 both moved off the plane (:1001-1254).
    if (exvol_forces_numeric(c1, c2in, c3, c4, kRepScaled, out)) return 1;
    if (coplanar(c1, c2in, c3, c4)) {
        double m1[3], m2[3];
        push_off_plane(c1, c2in, c3, c4, m2, 2, 0.01);
        push_off_plane(c1, c2in, c3, c4, m1, 1, 0.01);
        if (exvol_forces_numeric(m1, m2, c3, c4, kRepScaled, out)) return 1;
    }
    return -1;
}

int orc_exvol_forces(const double* coord, double* f, int n, const int* bs, const double* krep, const double* eqlen) {
    int nfallback = 0;
    for (int i = 0; i < n; ++i) {
        double out[4][3];
        const int r = orc_exvol_pair_forces(coord + bs[4 * i], coord + bs[4 * i + 1], coord + bs[4 * i + 2],
                                            coord + bs[4 * i + 3], krep[i], eqlen[2 * i], eqlen[2 * i + 1], out);
        if (r < 0) return -1;     // the reference exits the process here
        nfallback += r;
        for (int q = 0; q < 4; ++q)
            for (int k = 0; k < 3; ++k) acc(f[bs[4 * i + q] + k], out[q][k]);
    }
    return nfallback;
}

// ---------------------------------------------------------------------------
// Boundary exponential repulsion on planes (BoundaryCylinderRepulsionExp.cpp:27-110)
// r = (a x + b y + c z + d) / |n| ; U = K exp(-r / lambda) ; F += K exp(-r/lambda)/lambda * n
// ---------------------------------------------------------------------------
static inline double plane_distance(const double* pl, const double* x) {
    return (pl[0] * x[0] + pl[1] * x[1] + pl[2] * x[2] + pl[3]) / sqrt(std::pow(pl[0], 2) + std::pow(pl[1], 2) + std::pow(pl[2], 2));
}

double orc_plane_distance(const double* plane, const double* x) { return plane_distance(plane, x); }

double orc_boundary_energy(const double* coord, int nplanes, const double* planes, const int* nn, const int* bs,
                           const double* krep, const double* slen) {
    double U = 0.0;
    int off = 0;
    for (int p = 0; p < nplanes; ++p) {
        for (int j = 0; j < nn[p]; ++j) {
            const double r = plane_distance(planes + 4 * p, coord + bs[off + j]);
            const double R = -r / slen[off + j];
            U += krep[off + j] * std::exp(R);
        }
        off += nn[p];
    }
    return U;
}

void orc_boundary_forces(const double* coord, double* f, int nplanes, const double* planes, const int* nn,
                         const int* bs, const double* krep, const double* slen) {
    int off = 0;
    for (int p = 0; p < nplanes; ++p) {
        const double* pl = planes + 4 * p;
        for (int j = 0; j < nn[p]; ++j) {
            const double r = plane_distance(pl, coord + bs[off + j]);
            const double R = -r / slen[off + j];
            const double f0 = krep[off + j] * std::exp(R) / slen[off + j];
            double* fb = f + bs[off + j];
            acc(fb[0], f0 * pl[0]);
            acc(fb[1], f0 * pl[1]);
            acc(fb[2], f0 * pl[2]);
        }
        off += nn[p];
    }
}

// ---------------------------------------------------------------------------
// Neighbor lists
// ---------------------------------------------------------------------------

// Half cylinder-cylinder list by brute force over all pairs, with the
// predicate of HybridCylinderCylinderNL::updateNeighborsbin (:413-443)
// (one search is registered per filament-type pair, CylinderExclVolume.h:94-109,
// so every type combination is listed):
// keep (c, n) when id_c > id_n, not (same filament and |pos_c - pos_n| <= 2),
// and rMin^2 <= d^2 <= rMax^2, d^2 summed from 0 as (m_n - m_c)^2 over x, y, z
// (Util/Math/Vec.hpp:378-385) and the bounds held as float (HybridNeighborList.h:37).
// The bin-and-stencil traversal of the reference prunes only bins that cannot
// hold a neighbor, so the pair set equals this brute-force set.  Pairs are
// written as (c, n) cylinder indices ordered by c, then by n.
int64_t orc_cyl_pairs(int ncyl, const double* mid, const int64_t* id, const int* fil, const int* pos, const int* type,
                      double rmax, double rmin, int32_t* out, int64_t cap) {
    const float rmaxsq = float(rmax * rmax), rminsq = float(rmin * rmin);
    int64_t np = 0;
    for (int ci = 0; ci < ncyl; ++ci) {
        for (int ni = 0; ni < ncyl; ++ni) {
            if (id[ci] <= id[ni]) continue;
            if (fil[ci] == fil[ni] && std::abs(pos[ci] - pos[ni]) <= 2) continue;
            (void)type;
            double d2 = 0;
            for (int k = 0; k < 3; ++k) d2 += (mid[3 * ni + k] - mid[3 * ci + k]) * (mid[3 * ni + k] - mid[3 * ci + k]);
            if (d2 < rminsq || d2 > rmaxsq) continue;
            if (np < cap) { out[2 * np] = ci; out[2 * np + 1] = ni; }
            ++np;
        }
    }
    return np;
}

// The same set from a uniform cell grid with cells no smaller than rMax and a
// 27-cell stencil, as the reference's bin grid (HybridNeighborListImpl.cpp:176-240),
// used to check that binning does not change the set.
int64_t orc_cyl_pairs_binned(int ncyl, const double* mid, const int64_t* id, const int* fil, const int* pos,
                             const int* type, double rmax, double rmin, double box, double cell, int32_t* out, int64_t cap) {
    const float rmaxsq = float(rmax * rmax), rminsq = float(rmin * rmin);
    if (cell < rmax) cell = rmax;
    const int G = std::max(1, int(std::ceil(box / cell)));
    std::vector<std::vector<int>> bins(size_t(G) * G * G);
    auto cidx = [&](double x) { int i = int(std::floor(x / cell)); return std::min(std::max(i, 0), G - 1); };
    for (int c = 0; c < ncyl; ++c)
        bins[(size_t(cidx(mid[3 * c])) * G + cidx(mid[3 * c + 1])) * G + cidx(mid[3 * c + 2])].push_back(c);
    std::vector<int32_t> tmp;
    int64_t np = 0;
    for (int ci = 0; ci < ncyl; ++ci) {
        tmp.clear();
        const int ix = cidx(mid[3 * ci]), iy = cidx(mid[3 * ci + 1]), iz = cidx(mid[3 * ci + 2]);
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    const int jx = ix + dx, jy = iy + dy, jz = iz + dz;
                    if (jx < 0 || jy < 0 || jz < 0 || jx >= G || jy >= G || jz >= G) continue;
                    for (int ni : bins[(size_t(jx) * G + jy) * G + jz]) {
                        if (id[ci] <= id[ni]) continue;
                        if (fil[ci] == fil[ni] && std::abs(pos[ci] - pos[ni]) <= 2) continue;
                        double d2 = 0;
                        for (int k = 0; k < 3; ++k)
                            d2 += (mid[3 * ni + k] - mid[3 * ci + k]) * (mid[3 * ni + k] - mid[3 * ci + k]);
                        if (d2 < rminsq || d2 > rmaxsq) continue;
                        tmp.push_back(ni);
                    }
                }
        std::sort(tmp.begin(), tmp.end());
        for (int ni : tmp) {
            if (np < cap) { out[2 * np] = ci; out[2 * np + 1] = ni; }
            ++np;
        }
    }
    return np;
}

// Boundary-cylinder list (NeighborListImpl.cpp:738-751): for each plane in
// order, every cylinder (in order) whose midpoint (b1 * 0.5 + 0.5 * b2) has
// signed plane distance < cutoff.  Writes cylinder indices; counts per plane in nn.
int64_t orc_boundary_list(int ncyl, const double* coord, const int* b1, const int* b2, int nplanes, const double* planes,
                          double cutoff, int* nn, int32_t* out, int64_t cap) {
    int64_t m = 0;
    for (int p = 0; p < nplanes; ++p) {
        int cnt = 0;
        for (int c = 0; c < ncyl; ++c) {
            double mp[3];
            lerp(mp, coord + 3 * b1[c], coord + 3 * b2[c], 0.5);
            if (plane_distance(planes + 4 * p, mp) < cutoff) {
                if (m < cap) out[m] = c;
                ++m;
                ++cnt;
            }
        }
        nn[p] = cnt;
    }
    return m;
}

// ---------------------------------------------------------------------------
// Boundary load forces on filament ends after a minimization
// (ForceFieldManager::computeLoadForces, ForceFieldManager.cpp:292-311;
// BoundaryCylinderRepulsion<Exp>::computeLoadForces and its helper,
// BoundaryCylinderRepulsion.cpp:122-192; the Exp load force,
// BoundaryCylinderRepulsionExp.cpp:113-118).  Every filament end bead starts
// at zero; then for each plane in order and each cylinder of its boundary
// list in order: a plus-end cylinder loads its second bead (polymerizing away
// from its first), a minus-end cylinder its first bead (away from its second).
// For monomer i of the end, at x_i = bd + (i * monSize) * dir with
// dir = (bd - bo) / |bd - bo|:
//   load[i] += max(-(n . dir), 0) * K exp(-dist(x_i) / lambda) / lambda
// with n = (a, b, c) of the plane as stored (PlaneBoundaryElement::normal,
// BoundaryElementImpl.h:99-105) and dist its signed distance.  Output per
// filament f: plus[f * stride + i], minus[f * stride + i], i < n_mon of the
// filament's type (entries beyond stay zero).
// ---------------------------------------------------------------------------
static void load_force_end(const double* bo, const double* bd, const double* pl, double K, double lam, double mon,
                           int nmon, double* load) {
    double dir[3] = {bd[0] - bo[0], bd[1] - bo[1], bd[2] - bo[2]};
    double m2 = 0.0;
    for (int k = 0; k < 3; ++k) m2 += dir[k] * dir[k];
    const double norm = std::sqrt(m2);
    for (int k = 0; k < 3; ++k) dir[k] /= norm;
    double dn = 0.0;
    for (int k = 0; k < 3; ++k) dn += pl[k] * dir[k];
    const double proj = std::max(-dn, 0.0);
    for (int i = 0; i < nmon; ++i) {
        const double step = i * mon;
        const double x[3] = {bd[0] + step * dir[0], bd[1] + step * dir[1], bd[2] + step * dir[2]};
        const double R = -plane_distance(pl, x) / lam;
        const double f = K * std::exp(R) / lam;
        load[i] += proj * f;
    }
}

int orc_boundary_load_forces(int nfil, const int* fil_cyl_start, const int* b1, const int* b2, const int* cyl_type,
                             const double* coord, int nplanes, const double* planes, const double* plane_k,
                             const double* plane_slen, const int* nn, const int32_t* list, const double* mon_size,
                             const int* n_mon, int stride, double* plus, double* minus) {
    const int ncyl = fil_cyl_start[nfil];
    std::vector<int> fil(ncyl);
    for (int f = 0; f < nfil; ++f)
        for (int c = fil_cyl_start[f]; c < fil_cyl_start[f + 1]; ++c) fil[c] = f;
    std::fill(plus, plus + (size_t)nfil * stride, 0.0);
    std::fill(minus, minus + (size_t)nfil * stride, 0.0);
    int off = 0;
    for (int p = 0; p < nplanes; ++p) {
        for (int j = 0; j < nn[p]; ++j) {
            const int c = list[off + j];
            const int f = fil[c];
            const int t = cyl_type[c];
            const int nm = std::min(n_mon[t], stride);
            if (c == fil_cyl_start[f + 1] - 1)
                load_force_end(coord + 3 * b1[c], coord + 3 * b2[c], planes + 4 * p, plane_k[p], plane_slen[p],
                               mon_size[t], nm, plus + (size_t)f * stride);
            if (c == fil_cyl_start[f])
                load_force_end(coord + 3 * b2[c], coord + 3 * b1[c], planes + 4 * p, plane_k[p], plane_slen[p],
                               mon_size[t], nm, minus + (size_t)f * stride);
        }
        off += nn[p];
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Force-field manager (ForceFieldManager.cpp:96-290) over the six configured
// force fields in MController's order (MController.cpp:65-196).
// ---------------------------------------------------------------------------
struct OrcSystem {
    int n_stretch; const int* st_bs; const double* st_k; const double* st_l0;
    int n_bend; const int* bd_bs; const double* bd_k; const double* bd_t0;
    int n_linker; const int* lk_bs; const double* lk_k; const double* lk_l0; const double* lk_s1; const double* lk_s2;
    int n_motor; const int* mt_bs; const double* mt_k; const double* mt_l0; const double* mt_s1; const double* mt_s2;
    int n_exvol; const int* ev_bs; const double* ev_k; const double* ev_len;
    int n_planes; const double* planes; const int* bd_nn; const int* bb_bs; const double* bb_k; const double* bb_slen;
};

enum { FF_STRETCH, FF_BEND, FF_LINKER, FF_MOTOR, FF_EXVOL, FF_BOUNDARY, FF_COUNT };

// Host threads for the CPU baseline (orc_set_threads).  1, the default, keeps
// every loop serial in the order the reference runs it, which is what the
// parity tests compare against; more threads split each force field's
// interactions into contiguous chunks (per-thread force buffers, chunk sums
// added in chunk order) and the CG vector loops, so sums round differently.
static int g_threads = 1;

}  // extern "C"

template <class Fn>
static double chunked_energy(int n, Fn fn) {
    const int T = g_threads;
    if (T <= 1 || n < 2048) return fn(0, n);
    std::vector<double> part(T, 0.0);
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t) {
        const int b = (int)((long long)n * t / T), e = (int)((long long)n * (t + 1) / T);
        part[t] = fn(b, e - b);
    }
    double U = 0.0;
    for (int t = 0; t < T; ++t) {
        if (part[t] == -1.0) return -1.0;
        U += part[t];
    }
    return U;
}

// fn(begin, count, force buffer) accumulates one chunk into a per-thread
// buffer that covers only the DOF range its interactions touch (bs: `stride`
// DOF offsets per interaction); the buffers are then added into f in thread
// order.  Returns the chunks' summed status (-1 if any failed).
template <class Fn>
static int chunked_forces(int n, int stride, const int* bs, double* f, int nvar, Fn fn) {
    const int T = g_threads;
    if (T <= 1 || n < 2048) return fn(0, n, f);
    static std::vector<std::vector<double>> bufs;   // one per worker, reused across calls
    if ((int)bufs.size() < T) bufs.resize(T);
    std::vector<int> st(T, 0), lo(T, 0), hi(T, 0);
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t) {
        const int b = (int)((long long)n * t / T), e = (int)((long long)n * (t + 1) / T);
        int l = nvar, h = 0;
        for (long long k = (long long)stride * b; k < (long long)stride * e; ++k) {
            l = std::min(l, bs[k]);
            h = std::max(h, bs[k] + 3);
        }
        if (l >= h) { lo[t] = hi[t] = 0; continue; }
        lo[t] = l;
        hi[t] = h;
        auto& B = bufs[t];
        if ((int)B.size() < nvar) B.resize(nvar);
        std::fill(B.begin() + l, B.begin() + h, 0.0);
        st[t] = fn(b, e - b, B.data());
    }
#pragma omp parallel for num_threads(T) schedule(static)
    for (int i = 0; i < nvar; ++i) {
        double v = f[i];
        for (int t = 0; t < T; ++t)
            if (i >= lo[t] && i < hi[t]) v += bufs[t][i];
        f[i] = v;
    }
    int r = 0;
    for (int t = 0; t < T; ++t) {
        if (st[t] < 0) return -1;
        r += st[t];
    }
    return r;
}

extern "C" {

static double ff_energy(const OrcSystem* s, int which, const double* x) {
    switch (which) {
        case FF_STRETCH:
            return chunked_energy(s->n_stretch, [&](int b, int c) {
                return orc_stretch_energy(x, c, s->st_bs + 2 * b, s->st_k + b, s->st_l0 + b);
            });
        case FF_BEND:
            return chunked_energy(s->n_bend, [&](int b, int c) {
                return orc_bend_energy(x, c, s->bd_bs + 3 * b, s->bd_k + b, s->bd_t0 + b);
            });
        case FF_LINKER:
            return chunked_energy(s->n_linker, [&](int b, int c) {
                return orc_bond_energy(x, c, s->lk_bs + 4 * b, s->lk_k + b, s->lk_l0 + b, s->lk_s1 + b, s->lk_s2 + b);
            });
        case FF_MOTOR:
            return chunked_energy(s->n_motor, [&](int b, int c) {
                return orc_bond_energy(x, c, s->mt_bs + 4 * b, s->mt_k + b, s->mt_l0 + b, s->mt_s1 + b, s->mt_s2 + b);
            });
        case FF_EXVOL:
            return chunked_energy(s->n_exvol, [&](int b, int c) {
                return orc_exvol_energy(x, c, s->ev_bs + 4 * b, s->ev_k + b, s->ev_len + 2 * b);
            });
        case FF_BOUNDARY: return orc_boundary_energy(x, s->n_planes, s->planes, s->bd_nn, s->bb_bs, s->bb_k, s->bb_slen);
    }
    return 0.0;
}

// computeEnergy: sum in FF order; an FF reporting <= -1 makes the total +inf.
double orc_system_energy(const OrcSystem* s, const double* x) {
    double U = 0.0;
    for (int ff = 0; ff < FF_COUNT; ++ff) {
        const double e = ff_energy(s, ff, x);
        if (e <= -1) return std::numeric_limits<double>::infinity();
        U += e;
    }
    return U;
}

// computeIndividualEnergies: per-FF energies and their plain sum.
double orc_system_energies(const OrcSystem* s, const double* x, double* per_ff) {
    double U = 0.0;
    for (int ff = 0; ff < FF_COUNT; ++ff) {
        const double e = ff_energy(s, ff, x);
        if (per_ff) per_ff[ff] = e;
        U += e;
    }
    return U;
}

// computeForces: zero-fill then every FF accumulates, in order.
int orc_system_forces(const OrcSystem* s, const double* x, double* f, int nvar, double* lk_sf, double* mt_sf) {
    std::fill(f, f + nvar, 0.0);
    if (g_threads <= 1) {
        orc_stretch_forces(x, f, s->n_stretch, s->st_bs, s->st_k, s->st_l0);
        orc_bend_forces(x, f, s->n_bend, s->bd_bs, s->bd_k, s->bd_t0);
        orc_bond_forces(x, f, s->n_linker, s->lk_bs, s->lk_k, s->lk_l0, s->lk_s1, s->lk_s2, lk_sf);
        orc_bond_forces(x, f, s->n_motor, s->mt_bs, s->mt_k, s->mt_l0, s->mt_s1, s->mt_s2, mt_sf);
        const int r = orc_exvol_forces(x, f, s->n_exvol, s->ev_bs, s->ev_k, s->ev_len);
        orc_boundary_forces(x, f, s->n_planes, s->planes, s->bd_nn, s->bb_bs, s->bb_k, s->bb_slen);
        return r;
    }
    chunked_forces(s->n_stretch, 2, s->st_bs, f, nvar, [&](int b, int c, double* F) {
        orc_stretch_forces(x, F, c, s->st_bs + 2 * b, s->st_k + b, s->st_l0 + b);
        return 0;
    });
    chunked_forces(s->n_bend, 3, s->bd_bs, f, nvar, [&](int b, int c, double* F) {
        orc_bend_forces(x, F, c, s->bd_bs + 3 * b, s->bd_k + b, s->bd_t0 + b);
        return 0;
    });
    // linkers and motors touch beads all over the network: serial (a few ms)
    orc_bond_forces(x, f, s->n_linker, s->lk_bs, s->lk_k, s->lk_l0, s->lk_s1, s->lk_s2, lk_sf);
    orc_bond_forces(x, f, s->n_motor, s->mt_bs, s->mt_k, s->mt_l0, s->mt_s1, s->mt_s2, mt_sf);
    // excluded volume: pair contributions in parallel, accumulated in pair order
    int r = 0;
    {
        const int n = s->n_exvol;
        static std::vector<double> contrib;
        static std::vector<int> status;
        contrib.resize(12 * (size_t)n);
        status.resize(n);
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            const int* q = s->ev_bs + 4 * i;
            double out[4][3];
            status[i] = orc_exvol_pair_forces(x + q[0], x + q[1], x + q[2], x + q[3], s->ev_k[i], s->ev_len[2 * i],
                                              s->ev_len[2 * i + 1], out);
            std::memcpy(&contrib[12 * (size_t)i], out, sizeof(out));
        }
        for (int i = 0; i < n && r >= 0; ++i) {
            if (status[i] < 0) { r = -1; break; }
            r += status[i];
            const int* q = s->ev_bs + 4 * i;
            for (int a = 0; a < 4; ++a)
                for (int k = 0; k < 3; ++k) acc(f[q[a] + k], contrib[12 * (size_t)i + 3 * a + k]);
        }
    }
    orc_boundary_forces(x, f, s->n_planes, s->planes, s->bd_nn, s->bb_bs, s->bb_k, s->bb_slen);
    return r;
}

// ---------------------------------------------------------------------------
// Conjugate-gradient minimizer (CGMethod.hpp:826-1743) with the backtracking
// line search (:238-373) and MController's recovery move (MController.h:273-339).
// ---------------------------------------------------------------------------
struct OrcCGParams {
    int method;            // 0 steepest, 1 Fletcher-Reeves, 2 Polak-Ribiere
    double maxDist;
    double lambdaMax;
    double gradTol;
    double energyRelTol;
    int energyCallLimit;   // 0: none
    int forceCallLimit;    // 0: none
    int reportOnCallLimit;
    int tryToRecover;
};

struct OrcCGResult {
    uint32_t errorFlags;   // bit 0: line search error
    int numEnergyCall, energyCallLimit, numForceCall, forceCallLimit;
    int numIter, numSafeMode, numRecover, numLineSearchTrials;
    double gradInfNorm, gradTol, energyRelChange, energyRelTol;
    double energiesBefore[FF_COUNT + 1];   // per FF, then total
    double energiesAfter[FF_COUNT + 1];
    int usedBackup;
    int status;            // 0 ok; 1 maxF not finite (reference throws); 2 recovery step infinite
};

static double vdot(const std::vector<double>& a, const std::vector<double>& b, int n) {
    double r = 0.0;
    if (g_threads <= 1) {
        for (int i = 0; i < n; ++i) r += a[i] * b[i];
        return r;
    }
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(+ : r)
    for (int i = 0; i < n; ++i) r += a[i] * b[i];
    return r;
}

// y[i] = x[i] + s * d[i] (serial with one thread)
static void vaxpy(double* y, const double* x, double s, const double* d, int n) {
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
    for (int i = 0; i < n; ++i) y[i] = x[i] + s * d[i];
}

int orc_minimize(const OrcSystem* s, const OrcCGParams* prm, double* coord_io, int ndof, int nbeads,
                 double* force_out, OrcCGResult* res) {
    const double LAMBDAREDUCE = 0.5, LAMBDATOL = 1e-8, BACKTRACKSLOPE = 0.4;
    std::memset(res, 0, sizeof(*res));
    res->energyCallLimit = prm->energyCallLimit;
    res->gradTol = prm->gradTol;
    res->energyRelTol = prm->energyRelTol;
    res->forceCallLimit = std::max(prm->forceCallLimit, 3 * nbeads);
    res->gradInfNorm = std::numeric_limits<double>::infinity();
    res->energyRelChange = std::numeric_limits<double>::infinity();

    const int n = ndof;
    std::vector<double> x(coord_io, coord_io + n), f(n, 0.0), fprev(n, 0.0), d(n, 0.0), xt(n, 0.0), xbest;
    double minimumE = std::numeric_limits<double>::infinity(), totalEnergy = 0.0;

    auto maxF = [&](double& out) {
        double m = 0;
        if (g_threads <= 1) {
            for (int i = 0; i < n; ++i) m = std::max(m, std::fabs(f[i]));
        } else {
            bool nonfinite = false;
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(max : m) reduction(|| : nonfinite)
            for (int i = 0; i < n; ++i) {
                const double a = std::fabs(f[i]);
                if (!(a <= std::numeric_limits<double>::max())) nonfinite = true;
                else m = std::max(m, a);
            }
            if (nonfinite) m = std::numeric_limits<double>::infinity();
        }
        out = m;
        return std::isfinite(m);
    };
    auto callLimit = [&] {
        return (res->energyCallLimit != 0 && res->numEnergyCall > res->energyCallLimit) ||
               (res->forceCallLimit != 0 && res->numForceCall > res->forceCallLimit);
    };
    auto converged = [&] { return res->gradInfNorm < res->gradTol || res->energyRelChange < res->energyRelTol; };

    res->energiesBefore[FF_COUNT] = orc_system_energies(s, x.data(), res->energiesBefore);
    ++res->numEnergyCall;
    orc_system_forces(s, x.data(), f.data(), n, nullptr, nullptr);
    ++res->numForceCall;
    if (!maxF(res->gradInfNorm)) { res->status = 1; return 1; }
    double prevEnergy = res->energiesBefore[FF_COUNT];

    bool safeMode = false;
    double lastFdotF = 0;
    auto resetCG = [&] {
        for (int i = 0; i < n; ++i) d[i] = f[i] + 0.0 * d[i];
        if (prm->method >= 1) lastFdotF = vdot(f, f, n);
        if (prm->method == 2) fprev = f;
    };
    resetCG();

    while (!callLimit() && !converged()) {
        ++res->numIter;
        // ---- backtracking line search ----
        double lambda = 0.0, newEnergy = 0.0;
        {
            const double armijo = safeMode ? 0.0 : BACKTRACKSLOPE;
            if (res->gradInfNorm == 0.0) {
                lambda = 0.0; newEnergy = 0.0;
            } else {
                lambda = std::min(prm->lambdaMax, prm->maxDist / res->gradInfNorm);
                const double E0 = orc_system_energy(s, x.data());
                ++res->numEnergyCall;
                const double reducedSlope = armijo * vdot(d, f, n);
                bool done = false;
                double Elam = 0.0;
                while (!done) {
                    vaxpy(xt.data(), x.data(), lambda, d.data(), n);
                    Elam = orc_system_energy(s, xt.data());
                    ++res->numEnergyCall;
                    ++res->numLineSearchTrials;
                    const double ideal = -reducedSlope * lambda;
                    if (lambda < 0 || ideal > 0) { done = true; lambda = 0.0; }
                    const double change = Elam - E0;
                    if (change <= ideal) done = true;
                    else lambda *= LAMBDAREDUCE;
                    if (lambda <= 0.0 || lambda <= LAMBDATOL) { done = true; lambda = 0.0; Elam = E0; }
                }
                totalEnergy = Elam;
                newEnergy = Elam;
            }
        }
        if (lambda == 0) {
            if (prm->tryToRecover) {
                if (safeMode) {
                    // move along d by the largest step keeping every component within maxDist
                    double step = std::numeric_limits<double>::infinity();
                    for (int i = 0; i < 3 * nbeads && i < n; ++i) step = std::min(step, prm->maxDist / std::fabs(d[i]));
                    if (step == std::numeric_limits<double>::infinity()) { res->status = 2; break; }
                    for (int i = 0; i < n; ++i) x[i] += step * d[i];
                    ++res->numRecover;
                    orc_system_forces(s, x.data(), f.data(), n, nullptr, nullptr);
                    ++res->numForceCall;
                    if (!maxF(res->gradInfNorm)) { res->status = 1; break; }
                    resetCG();
                    safeMode = false;
                } else {
                    resetCG();
                    safeMode = true;
                    ++res->numSafeMode;
                }
            } else {
                res->errorFlags |= 1u;
                break;
            }
            continue;
        }
        vaxpy(x.data(), x.data(), lambda, d.data(), n);
        orc_system_forces(s, x.data(), f.data(), n, nullptr, nullptr);
        ++res->numForceCall;
        if (!maxF(res->gradInfNorm)) { res->status = 1; break; }
        res->energyRelChange = std::fabs(newEnergy - prevEnergy) / std::fabs(prevEnergy);
        prevEnergy = newEnergy;

        double newGrad = 0, prevGrad = 0, beta = 0;
        if (prm->method == 1) newGrad = vdot(f, f, n);
        else if (prm->method == 2) { newGrad = vdot(f, f, n); prevGrad = vdot(f, fprev, n); }
        if (prm->method == 1) beta = newGrad / lastFdotF;
        else if (prm->method == 2) beta = std::max(0.0, (newGrad - prevGrad) / lastFdotF);
        vaxpy(d.data(), f.data(), beta, d.data(), n);
        if (vdot(d, f, n) <= 0) resetCG();
        if (prm->method == 2) fprev = f;

        bool relaxed = true;
        for (int i = 0; i < n; ++i)
            if (std::fabs(f[i]) > 10 * prm->gradTol) { relaxed = false; break; }
        if (relaxed && res->numIter > res->forceCallLimit / 2) {
            if (totalEnergy <= minimumE) { minimumE = totalEnergy; xbest = x; }
        }
        if (prm->method >= 1) lastFdotF = newGrad;
    }

    if (prm->reportOnCallLimit && callLimit() && !xbest.empty()) {
        x = xbest;
        res->usedBackup = 1;
    }
    res->energiesAfter[FF_COUNT] = orc_system_energies(s, x.data(), res->energiesAfter);
    ++res->numEnergyCall;
    std::copy(x.begin(), x.end(), coord_io);
    if (force_out) std::copy(f.begin(), f.end(), force_out);
    return res->status;
}

// Plain CG on a caller-supplied separable quadratic, to run the reference's
// minimizer unit case (TESTS/Mechanics/Minimizer/TestCGMethod.cpp:9-93)
// through the same state machine: U = sum_i 1/2 w_i (x_i - o_i)^2.
struct QuadSys { int n; const double* w; const double* o; };

int orc_minimize_quadratic(int n, const double* w, const double* o, const OrcCGParams* prm, double* x_io,
                           double* f_out, OrcCGResult* res) {
    // A network with one "stretch" term per coordinate cannot express a
    // weighted bowl, so this routine repeats the minimizer loop on closures.
    const double LAMBDAREDUCE = 0.5, LAMBDATOL = 1e-8, BACKTRACKSLOPE = 0.4;
    std::memset(res, 0, sizeof(*res));
    res->gradTol = prm->gradTol;
    res->energyRelTol = prm->energyRelTol;
    res->energyCallLimit = prm->energyCallLimit;
    res->forceCallLimit = std::max(prm->forceCallLimit, 0);
    res->gradInfNorm = std::numeric_limits<double>::infinity();
    res->energyRelChange = std::numeric_limits<double>::infinity();
    auto E = [&](const std::vector<double>& x) {
        double e = 0;
        for (int i = 0; i < n; ++i) e += 0.5 * w[i] * (x[i] - o[i]) * (x[i] - o[i]);
        return e;
    };
    auto Fn = [&](const std::vector<double>& x, std::vector<double>& f) {
        for (int i = 0; i < n; ++i) f[i] = -w[i] * (x[i] - o[i]);
    };
    std::vector<double> x(x_io, x_io + n), f(n), fprev(n, 0.0), d(n, 0.0), xt(n);
    auto callLimit = [&] {
        return (res->energyCallLimit != 0 && res->numEnergyCall > res->energyCallLimit) ||
               (res->forceCallLimit != 0 && res->numForceCall > res->forceCallLimit);
    };
    auto maxF = [&] { double m = 0; for (int i = 0; i < n; ++i) m = std::max(m, std::fabs(f[i])); return m; };
    res->energiesBefore[FF_COUNT] = E(x);
    ++res->numEnergyCall;
    Fn(x, f);
    ++res->numForceCall;
    res->gradInfNorm = maxF();
    double prevEnergy = res->energiesBefore[FF_COUNT], lastFdotF = 0;
    bool safeMode = false;
    auto resetCG = [&] {
        for (int i = 0; i < n; ++i) d[i] = f[i] + 0.0 * d[i];
        if (prm->method >= 1) lastFdotF = vdot(f, f, n);
        if (prm->method == 2) fprev = f;
    };
    resetCG();
    while (!callLimit() && !(res->gradInfNorm < res->gradTol || res->energyRelChange < res->energyRelTol)) {
        ++res->numIter;
        double lambda = 0, newEnergy = 0;
        if (res->gradInfNorm != 0.0) {
            const double armijo = safeMode ? 0.0 : BACKTRACKSLOPE;
            lambda = std::min(prm->lambdaMax, prm->maxDist / res->gradInfNorm);
            const double E0 = E(x);
            ++res->numEnergyCall;
            const double rs = armijo * vdot(d, f, n);
            bool done = false;
            double El = 0;
            while (!done) {
                for (int i = 0; i < n; ++i) xt[i] = x[i] + lambda * d[i];
                El = E(xt);
                ++res->numEnergyCall;
                const double ideal = -rs * lambda;
                if (lambda < 0 || ideal > 0) { done = true; lambda = 0.0; }
                if (El - E0 <= ideal) done = true;
                else lambda *= LAMBDAREDUCE;
                if (lambda <= 0.0 || lambda <= LAMBDATOL) { done = true; lambda = 0.0; El = E0; }
            }
            newEnergy = El;
        }
        if (lambda == 0) {
            if (prm->tryToRecover) {
                if (safeMode) { resetCG(); safeMode = false; }
                else { resetCG(); safeMode = true; }
            } else { res->errorFlags |= 1u; break; }
            continue;
        }
        for (int i = 0; i < n; ++i) x[i] += lambda * d[i];
        Fn(x, f);
        ++res->numForceCall;
        res->gradInfNorm = maxF();
        res->energyRelChange = std::fabs(newEnergy - prevEnergy) / std::fabs(prevEnergy);
        prevEnergy = newEnergy;
        double newGrad = 0, prevGrad = 0, beta = 0;
        if (prm->method == 1) newGrad = vdot(f, f, n);
        else if (prm->method == 2) { newGrad = vdot(f, f, n); prevGrad = vdot(f, fprev, n); }
        if (prm->method == 1) beta = newGrad / lastFdotF;
        else if (prm->method == 2) beta = std::max(0.0, (newGrad - prevGrad) / lastFdotF);
        for (int i = 0; i < n; ++i) d[i] = f[i] + beta * d[i];
        if (vdot(d, f, n) <= 0) resetCG();
        if (prm->method == 2) fprev = f;
        if (prm->method >= 1) lastFdotF = newGrad;
    }
    res->energiesAfter[FF_COUNT] = E(x);
    ++res->numEnergyCall;
    std::copy(x.begin(), x.end(), x_io);
    std::copy(f.begin(), f.end(), f_out);
    return 0;
}

int orc_version(void) { return 1; }
void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_get_threads(void) { return g_threads; }

// Arctangent used by the excluded-volume formula: 0 = the C library's atan
// (the reference's), 1 = series_atan above (rounds identically on the GPU).
void orc_set_series_atan(int on) { g_series_atan = on != 0; }
double orc_series_atan(double x) { return series_atan(x); }

// Per-component sum of |contribution| over every interaction.
void orc_system_force_scale(const OrcSystem* s, const double* x, double* scale, int nvar) {
    g_abs = true;
    orc_system_forces(s, x, scale, nvar, nullptr, nullptr);
    g_abs = false;
}

}  // extern "C"
