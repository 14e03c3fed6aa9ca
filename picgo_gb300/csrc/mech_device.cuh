// Device helpers shared by the kernel translation units: deterministic block
// reductions, the per-replica finalizers of the CG state machine, and the
// per-interaction force-field math of the filament, linker/motor and boundary
// potentials.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "mech_internal.cuh"

namespace mech {

constexpr int kBlock = 256;
constexpr double kLambdaTol = 1e-8;      // CGMethod::LAMBDATOL (CGMethod.hpp:98)
constexpr double kLambdaReduce = 0.5;    // CGMethod::LAMBDAREDUCE
constexpr double kBacktrackSlope = 0.4;  // CGMethod::BACKTRACKSLOPE

// ---------------------------------------------------------------------------
// Block reductions with a fixed combination tree (results do not depend on
// scheduling).  All threads of a kBlock block must call them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Sum over the block; valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* sh /* >= 32 */) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (l < (blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_sum(r);
    }
    return r;
}
__device__ __forceinline__ double block_max(double v, double* sh) {
    v = warp_max(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (l < (blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_max(r);
    }
    return r;
}

// Combine per-warp results (valid in lane 0 of each warp) over the block in a
// fixed order; results valid in thread 0.  op[k]: 0 sum, 1 max.
// `sh` holds at least 32 * N doubles.
template <int N>
__device__ __forceinline__ void block_combine(double (&w)[N], const int (&op)[N], double* sh) {
    const int wi = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) sh[k * 32 + wi] = w[k];
    }
    __syncthreads();
    if (wi == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double r = l < nw ? sh[k * 32 + l] : (op[k] ? -1.0 / 0.0 : 0.0);
            r = op[k] ? warp_max(r) : warp_sum(r);
            w[k] = r;
        }
    }
}

// Deterministic sum of part[i * stride + off] for i in [b, e), whole block; result in thread 0.
__device__ __forceinline__ double sum_slots(const double* part, int stride, int off, int b, int e, double* sh) {
    double acc = 0.0;
    for (int i = b + threadIdx.x; i < e; i += blockDim.x) acc += __ldcg(part + (size_t)i * stride + off);
    return block_sum(acc, sh);
}
__device__ __forceinline__ double max_slots(const double* part, int stride, int off, int b, int e, double* sh) {
    double acc = 0.0;
    for (int i = b + threadIdx.x; i < e; i += blockDim.x) acc = fmax(acc, __ldcg(part + (size_t)i * stride + off));
    return block_max(acc, sh);
}

// Ticket: returns true in every thread of the block that finished replica r's
// last tile of this kernel.  Must be called by all threads after the block's
// partials are written.
__device__ __forceinline__ bool last_tile(int* ticket, int r, int ntiles, int* sh_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const int t = atomicAdd(ticket + r, 1);
        *sh_flag = (t == ntiles - 1);
        if (*sh_flag) ticket[r] = 0;
    }
    __syncthreads();
    const bool last = *sh_flag != 0;
    if (last) __threadfence();
    return last;
}

// ---------------------------------------------------------------------------
// CG state machine pieces (CGMethod.hpp:826-1743), run by one thread.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool call_limit(const CGState& S) {
    return (S.energyCallLimit != 0 && S.numEnergyCall > S.energyCallLimit) ||
           (S.forceCallLimit != 0 && S.numForceCall > S.forceCallLimit);
}
__device__ __forceinline__ bool converged(const CGState& S) {
    return S.maxF < S.gradTol || S.energyRelChange < S.energyRelTol;
}

// lambda = 0 after a line search (CGMethod.hpp:1337-1367): stop with
// errorLineSearch, enter safe mode, or (already in safe mode) hand MController's
// recovery move to the host.  Applied where the line search fails, so no launch
// of its own has to look for failed replicas.
__device__ __forceinline__ void dispatch_failed(CGState& S) {
    if (!S.tryToRecover) {
        S.errorFlags |= 1u;
        S.status = MECH_ERR_LINESEARCH;
        S.phase = PH_DONE;
    } else if (!S.safeMode) {
        S.safeMode = 1;
        S.numSafeMode++;
        S.phase = PH_RESET;
    } else {
        S.safeMode = 0;
        S.numRecover++;
        S.phase = PH_RECOVER;
    }
}

// Loop head and the start of backtrackingLineSearch (CGMethod.hpp:238-296, :1279-1320).
// The energy at the current coordinates is the cached E0: it is the accepted
// trial's energy, bit for bit, because the trial coordinates x + lambda d are
// the coordinates the move produces.
__device__ __forceinline__ void begin_iteration(CGState& S) {
    if (call_limit(S) || converged(S)) {
        S.phase = PH_DONE;
        return;
    }
    S.numIter++;
    if (S.maxF == 0.0) {     // "return zero if no forces": lambda 0, no energy call
        S.lambda = 0.0;
        S.phase = PH_FAILED;
        dispatch_failed(S);
        return;
    }
    S.lambda = fmin(S.lambdaMax, S.maxDist / S.maxF);
    S.numEnergyCall++;       // the reference evaluates E0 here
    const double armijo = S.safeMode ? 0.0 : kBacktrackSlope;
    S.reducedSlope = armijo * S.slope;
    S.phase = PH_LS_TRIAL;
}

// One backtracking step after the trial energy E (CGMethod.hpp:296-361);
// `trial_buf` is the position buffer holding that trial's coordinates.
__device__ __forceinline__ void line_search_step(CGState& S, double E, int trial_buf) {
    S.numEnergyCall++;
    S.numTrials++;
    double lambda = S.lambda;
    double Elam = E;
    const double ideal = -S.reducedSlope * lambda;
    bool done = false;
    if (lambda < 0 || ideal > 0) {
        done = true;
        lambda = 0.0;
    }
    const double change = Elam - S.E0;
    if (change <= ideal) done = true;
    else lambda *= kLambdaReduce;
    if (lambda <= 0.0 || lambda <= kLambdaTol) {
        done = true;
        lambda = 0.0;
        Elam = S.E0;
    }
    S.lambda = lambda;
    if (!done) return;                 // next trial at the halved lambda
    S.totalEnergy = Elam;
    if (lambda == 0.0) {
        S.phase = PH_FAILED;
        dispatch_failed(S);
        return;
    }
    S.newEnergy = Elam;
    S.E0 = Elam;                       // energy at the moved coordinates
    S.xbuf = trial_buf;                // the trial buffer becomes current
    S.phase = PH_FORCE;
}

// ---------------------------------------------------------------------------
// Bead positions.  FP64 engine: three doubles per bead.  Mixed engine: each
// component is an unevaluated sum hi + lo of two floats (about 48 significant
// bits), so positions, trial moves and difference vectors need no FP64
// arithmetic, which runs at 1/57 of the FP32 rate on this GPU.  Both formats
// take 24 bytes per bead.
// ---------------------------------------------------------------------------
template <typename Real> struct Pos;
template <> struct Pos<double> { double x[3]; };
template <> struct Pos<float> { float h[3], l[3]; };

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    e = b - (s - a);
}

__device__ __forceinline__ Pos<double> load_pos(const double* X, int b) {
    Pos<double> p;
    const double* q = X + 3 * (size_t)b;
    p.x[0] = q[0]; p.x[1] = q[1]; p.x[2] = q[2];
    return p;
}
__device__ __forceinline__ Pos<float> load_pos(const float* X, int b) {
    Pos<float> p;
    const float2* q = reinterpret_cast<const float2*>(X + 6 * (size_t)b);
    const float2 a = q[0], c = q[1], e = q[2];
    p.h[0] = a.x; p.h[1] = a.y; p.h[2] = c.x; p.l[0] = c.y; p.l[1] = e.x; p.l[2] = e.y;
    return p;
}
__device__ __forceinline__ void store_pos(double* X, int b, const Pos<double>& p) {
    double* q = X + 3 * (size_t)b;
    q[0] = p.x[0]; q[1] = p.x[1]; q[2] = p.x[2];
}
__device__ __forceinline__ void store_pos(float* X, int b, const Pos<float>& p) {
    float2* q = reinterpret_cast<float2*>(X + 6 * (size_t)b);
    q[0] = make_float2(p.h[0], p.h[1]);
    q[1] = make_float2(p.h[2], p.l[0]);
    q[2] = make_float2(p.l[1], p.l[2]);
}

// x + lambda d (CGMethod.cpp:43-46).  Every kernel that needs the trial
// position uses these, so the materialized trial coordinates and the ones
// formed on the fly are identical.
__device__ __forceinline__ Pos<double> moved(const Pos<double>& p, const double* D, int b, double lam) {
    Pos<double> o;
    const double* d = D + 3 * (size_t)b;
#pragma unroll
    for (int k = 0; k < 3; ++k) o.x[k] = fma(lam, d[k], p.x[k]);
    return o;
}
__device__ __forceinline__ Pos<float> moved(const Pos<float>& p, const float* D, int b, double lam) {
    Pos<float> o;
    const float* d = D + 3 * (size_t)b;
    const float lf = (float)lam;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float s, e, lo;
        two_sum(p.h[k], __fmul_rn(lf, d[k]), s, e);
        lo = __fadd_rn(p.l[k], e);
        fast_two_sum(s, lo, o.h[k], o.l[k]);
    }
    return o;
}

template <typename Real>
__device__ __forceinline__ Pos<Real> bead_at(const Real* X, const Real* D, int b, bool trial, double lam) {
    const Pos<Real> p = load_pos(X, b);
    return trial ? moved(p, D, b, lam) : p;
}
// single-precision step already rounded by the caller (same result as the double-lambda form)
__device__ __forceinline__ Pos<float> moved_f(const Pos<float>& p, const float* D, int b, float lf) {
    Pos<float> o;
    const float* d = D + 3 * (size_t)b;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float s, e, lo;
        two_sum(p.h[k], __fmul_rn(lf, d[k]), s, e);
        lo = __fadd_rn(p.l[k], e);
        fast_two_sum(s, lo, o.h[k], o.l[k]);
    }
    return o;
}

// compensated single-precision accumulator
struct FF {
    float h = 0.f, l = 0.f;
    __device__ __forceinline__ void add(float v) {
        float s, e;
        two_sum(h, v, s, e);
        const float lo = __fadd_rn(l, e);
        fast_two_sum(s, lo, h, l);
    }
};
// warp sum of (h, l) pairs in place, result in lane 0
__device__ __forceinline__ void warp_reduce_pair(float& s, float& e) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_down_sync(0xffffffffu, s, o), e2 = __shfl_down_sync(0xffffffffu, e, o);
        float t, te;
        two_sum(s, s2, t, te);
        te = __fadd_rn(te, __fadd_rn(e, e2));
        fast_two_sum(t, te, s, e);
    }
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
// Block reduction with no double arithmetic: N compensated pairs and M maxima
// of non-negative floats (`m` may be null when M is 0), in a fixed order;
// results valid in thread 0.  A warp's FP64 instruction holds its sub-
// partition's FP64 pipe for ~78 cycles on this part, so a per-tile double tree
// costs more than the tile's loads.  `sh` holds 32 * (2N + M) floats.
template <int N, int M>
__device__ __forceinline__ void block_reduce_ff(FF (&a)[N], float* m, float* sh) {
    const int wi = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) warp_reduce_pair(a[k].h, a[k].l);
#pragma unroll
    for (int k = 0; k < M; ++k) m[k] = warp_max_f(m[k]);
    __syncthreads();
    if (l == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            sh[(2 * k) * 32 + wi] = a[k].h;
            sh[(2 * k + 1) * 32 + wi] = a[k].l;
        }
#pragma unroll
        for (int k = 0; k < M; ++k) sh[(2 * N + k) * 32 + wi] = m[k];
    }
    __syncthreads();
    if (wi == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            a[k].h = l < nw ? sh[(2 * k) * 32 + l] : 0.f;
            a[k].l = l < nw ? sh[(2 * k + 1) * 32 + l] : 0.f;
            warp_reduce_pair(a[k].h, a[k].l);
        }
#pragma unroll
        for (int k = 0; k < M; ++k) m[k] = warp_max_f(l < nw ? sh[(2 * N + k) * 32 + l] : 0.f);
    }
}
template <int N, int M>
__device__ __forceinline__ void block_reduce_pairs(FF (&a)[N], float (&m)[M], float* sh) {
    block_reduce_ff<N, M>(a, m, sh);
}

// Mixed-engine partial slots: a compensated (hi, lo) float pair stored in the
// 8 bytes of a double slot, so partial sums never pass through FP64.
__device__ __forceinline__ void store_pair(double* slot, float h, float l) {
    *reinterpret_cast<float2*>(slot) = make_float2(h, l);
}
__device__ __forceinline__ float2 load_pair(const double* slot) { return __ldcg(reinterpret_cast<const float2*>(slot)); }
__device__ __forceinline__ void add_pair(FF& acc, float2 v) {
    acc.add(v.x);
    acc.add(v.y);
}

// a - b as Real
__device__ __forceinline__ void pdiff(const Pos<double>& a, const Pos<double>& b, double r[3]) {
    r[0] = a.x[0] - b.x[0]; r[1] = a.x[1] - b.x[1]; r[2] = a.x[2] - b.x[2];
}
__device__ __forceinline__ void pdiff(const Pos<float>& a, const Pos<float>& b, float r[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = __fadd_rn(__fsub_rn(a.h[k], b.h[k]), __fsub_rn(a.l[k], b.l[k]));
}
__device__ __forceinline__ void to_double(const Pos<double>& p, double o[3]) { o[0] = p.x[0]; o[1] = p.x[1]; o[2] = p.x[2]; }
__device__ __forceinline__ void to_double(const Pos<float>& p, double o[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = (double)p.h[k] + (double)p.l[k];   // exact
}
__device__ __forceinline__ Pos<float> split(const double x[3]) {
    Pos<float> p;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        p.h[k] = (float)x[k];
        p.l[k] = (float)(x[k] - (double)p.h[k]);
    }
    return p;
}

// ---------------------------------------------------------------------------
// Reductions of per-thread values of the engine's precision.  FP64: plain
// double tree.  Mixed: float pairs (hi, lo) summed with error-free
// transformations within each warp, then double across warps and tiles.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum_ff(float v) {
    float s = v, e = 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_down_sync(0xffffffffu, s, o), e2 = __shfl_down_sync(0xffffffffu, e, o);
        float t, te;
        two_sum(s, s2, t, te);
        te = __fadd_rn(te, __fadd_rn(e, e2));
        fast_two_sum(t, te, s, e);
    }
    double r = 0.0;
    if ((threadIdx.x & 31) == 0) r = (double)s + (double)e;
    return r;
}
__device__ __forceinline__ double warp_sum_r(double v) { return warp_sum(v); }
__device__ __forceinline__ double warp_sum_r(float v) { return warp_sum_ff(v); }
__device__ __forceinline__ double warp_max_r(double v) { return warp_max(v); }
__device__ __forceinline__ double warp_max_r(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    double r = 0.0;
    if ((threadIdx.x & 31) == 0) r = (double)v;
    return r;
}
__device__ __forceinline__ double block_sum_r(double v, double* sh) { return block_sum(v, sh); }
__device__ __forceinline__ double block_sum_r(float v, double* sh) {
    const double w = warp_sum_ff(v);
    const int wi = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[wi] = w;
    __syncthreads();
    double r = 0.0;
    if (wi == 0) {
        r = (l < (blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_sum(r);
    }
    return r;
}
__device__ __forceinline__ double block_max_r(double v, double* sh) { return block_max(v, sh); }
__device__ __forceinline__ double block_max_r(float v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    const int wi = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[wi] = (double)v;
    __syncthreads();
    double r = 0.0;
    if (wi == 0) {
        r = (l < (blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_max(r);
    }
    return r;
}

// areEqual(theta0, 0) (utility.h:75-78), in the engine's precision
__device__ __forceinline__ bool near_zero_theta(double t) { return fabs(t - 0.0) < 1e-6; }
__device__ __forceinline__ bool near_zero_theta(float t) { return fabsf(t) < 1e-6f; }

// the four filament constants of a bead slot in one vector load
__device__ __forceinline__ void load_par(const float* P, int j, float& ks, float& l0, float& kb, float& t0) {
    const float4 v = reinterpret_cast<const float4*>(P)[j];
    ks = v.x; l0 = v.y; kb = v.z; t0 = v.w;
}
__device__ __forceinline__ void load_par(const double* P, int j, double& ks, double& l0, double& kb, double& t0) {
    const double2 a = reinterpret_cast<const double2*>(P)[2 * (size_t)j];
    const double2 b = reinterpret_cast<const double2*>(P)[2 * (size_t)j + 1];
    ks = a.x; l0 = a.y; kb = b.x; t0 = b.y;
}

// ---------------------------------------------------------------------------
// Filament stretching (FilamentStretchingHarmonic.cpp:185-275) and cosine
// bending (FilamentBendingCosine.cpp:199-345) on difference vectors.
// ---------------------------------------------------------------------------
template <typename Real>
__device__ __forceinline__ Real stretch_energy(Real rx, Real ry, Real rz, Real k, Real l0) {
    const Real L = sqrt(rx * rx + ry * ry + rz * rz);
    const Real dl = L - l0;
    return (Real)0.5 * k * dl * dl;
}

// Force on the second bead (the first gets the negation).
template <typename Real>
__device__ __forceinline__ void stretch_force(Real rx, Real ry, Real rz, Real k, Real l0, Real F[3]) {
    const Real L = sqrt(rx * rx + ry * ry + rz * rz);
    const Real invL = (Real)1 / L;
    const Real f0 = k * (L - l0) * invL;
    F[0] = -f0 * rx;
    F[1] = -f0 * ry;
    F[2] = -f0 * rz;
}

template <typename Real>
__device__ __forceinline__ Real bend_energy(const Real r1[3], const Real r2[3], Real k, Real t0) {
    const Real L1sq = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
    const Real L2sq = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
    const Real l1l2 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
    const Real L1L2 = sqrt(L1sq) * sqrt(L2sq);
    Real x = l1l2 / L1L2;
    if (x < (Real)-1) x = (Real)-1;
    else if (x > (Real)1) x = (Real)1;
    if (near_zero_theta(t0)) {
        if (sizeof(Real) == 4 && l1l2 > (Real)0) {
            // 1 - cos = |r1 x r2|^2 / (L1 L2 (L1 L2 + r1.r2)): no cancellation in single precision
            const Real cx = r1[1] * r2[2] - r1[2] * r2[1];
            const Real cy = r1[2] * r2[0] - r1[0] * r2[2];
            const Real cz = r1[0] * r2[1] - r1[1] * r2[0];
            const Real om = (cx * cx + cy * cy + cz * cz) / (L1L2 * (L1L2 + l1l2));
            return k * om;
        }
        return k * ((Real)1 - x);
    }
    const Real cosA = x;
    const Real sinA = fmax(sqrt((Real)1 - cosA * cosA), (Real)0);
    const Real cAmB = cosA * cos(t0) + sinA * sin(t0);
    return k * ((Real)1 - cAmB);
}

// Fr1, Fr2 of the reference: forces are b1: -Fr1, b2: Fr1 - Fr2, b3: Fr2.
template <typename Real>
__device__ __forceinline__ void bend_force(const Real r1[3], const Real r2[3], Real k, Real t0, Real Fr1[3], Real Fr2[3]) {
    const Real L1sq = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
    const Real L2sq = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
    const Real l1l2 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
    const Real A = (Real)1 / sqrt(L1sq * L2sq);
    Real x = l1l2 * A;
    const Real B = x / L1sq;
    const Real C = x / L2sq;
    Real kk;
    if (near_zero_theta(t0)) {
        kk = k;
    } else {
        if (fabs(fabs(x) - (Real)1) < (Real)0.001) x = (Real)0.999 * x;
        if (x < (Real)-1) x = (Real)-1;
        else if (x > (Real)1) x = (Real)1;
        const Real sinp = sqrt(fmax((Real)1 - x * x, (Real)0));
        const Real sinpmq = sinp * cos(t0) - x * sin(t0);
        kk = k * sinpmq / sinp;
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        Fr1[q] = kk * (r2[q] * A - r1[q] * B);
        Fr2[q] = kk * (r1[q] * A - r2[q] * C);
    }
}

// ---------------------------------------------------------------------------
// Linker / motor stretching between interpolated points
// (LinkerStretchingHarmonic.cpp:191-293).  p = b1 (1 - s) + s b2.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void lerp3(const double a[3], const double b[3], double s, double out[3]) {
    const double t = 1 - s;
    out[0] = (a[0] * t + s * b[0]);
    out[1] = (a[1] * t + s * b[1]);
    out[2] = (a[2] * t + s * b[2]);
}

// ---------------------------------------------------------------------------
// Plane distance (BoundaryElementImpl.h:49-53): (a x + b y + c z + d) / |n|.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double plane_dist(const double* pl, const double p[3]) {
    return (pl[0] * p[0] + pl[1] * p[1] + pl[2] * p[2] + pl[3]) / sqrt(pl[0] * pl[0] + pl[1] * pl[1] + pl[2] * pl[2]);
}

}  // namespace mech
