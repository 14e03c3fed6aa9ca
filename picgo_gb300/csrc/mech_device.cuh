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
        return;
    }
    S.lambda = fmin(S.lambdaMax, S.maxDist / S.maxF);
    S.numEnergyCall++;       // the reference evaluates E0 here
    const double armijo = S.safeMode ? 0.0 : kBacktrackSlope;
    S.reducedSlope = armijo * S.slope;
    S.phase = PH_LS_TRIAL;
}

// One backtracking step after the trial energy E (CGMethod.hpp:296-361).
__device__ __forceinline__ void line_search_step(CGState& S, double E) {
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
        return;
    }
    S.newEnergy = Elam;
    S.E0 = Elam;                       // energy at the moved coordinates
    S.xbuf ^= 1;                       // the trial buffer becomes current
    S.phase = PH_FORCE;
}

// ---------------------------------------------------------------------------
// Bead loads.
// ---------------------------------------------------------------------------
template <typename Real>
__device__ __forceinline__ void bead_pos(const double* X, const Real* D, int b, bool trial, double lam, double p[3]) {
    const double* xb = X + 3 * (size_t)b;
    if (trial) {
        const Real* db = D + 3 * (size_t)b;
        p[0] = fma(lam, (double)db[0], xb[0]);
        p[1] = fma(lam, (double)db[1], xb[1]);
        p[2] = fma(lam, (double)db[2], xb[2]);
    } else {
        p[0] = xb[0];
        p[1] = xb[1];
        p[2] = xb[2];
    }
}

__device__ __forceinline__ bool near_zero_theta(double t) { return fabs(t - 0.0) < 1e-6; }  // areEqual (utility.h:75-78)

// ---------------------------------------------------------------------------
// Filament stretching (FilamentStretchingHarmonic.cpp:185-275) and cosine
// bending (FilamentBendingCosine.cpp:199-345) on difference vectors.
// ---------------------------------------------------------------------------
template <typename Real>
__device__ __forceinline__ double stretch_energy(Real rx, Real ry, Real rz, Real k, Real l0) {
    const Real L = sqrt(rx * rx + ry * ry + rz * rz);
    const Real dl = L - l0;
    return (double)((Real)0.5 * k * dl * dl);
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
__device__ __forceinline__ double bend_energy(const Real r1[3], const Real r2[3], Real k, Real t0) {
    const Real L1sq = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
    const Real L2sq = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
    const Real l1l2 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
    const Real L1L2 = sqrt(L1sq) * sqrt(L2sq);
    Real x = l1l2 / L1L2;
    if (x < (Real)-1) x = (Real)-1;
    else if (x > (Real)1) x = (Real)1;
    if (near_zero_theta((double)t0)) {
        if (sizeof(Real) == 4 && l1l2 > (Real)0) {
            // 1 - cos = |r1 x r2|^2 / (L1 L2 (L1 L2 + r1.r2)): no cancellation in single precision
            const Real cx = r1[1] * r2[2] - r1[2] * r2[1];
            const Real cy = r1[2] * r2[0] - r1[0] * r2[2];
            const Real cz = r1[0] * r2[1] - r1[1] * r2[0];
            const Real om = (cx * cx + cy * cy + cz * cz) / (L1L2 * (L1L2 + l1l2));
            return (double)(k * om);
        }
        return (double)(k * ((Real)1 - x));
    }
    const Real cosA = x;
    const Real sinA = fmax(sqrt((Real)1 - cosA * cosA), (Real)0);
    const Real cAmB = cosA * cos(t0) + sinA * sin(t0);
    return (double)(k * ((Real)1 - cAmB));
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
    if (near_zero_theta((double)t0)) {
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
