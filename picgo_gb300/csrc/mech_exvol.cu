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
// segments), so pairs with q under a threshold are evaluated again in FP64 by
// an extended pass over a compacted list (k_exvol_ext, shaped around this
// GPU's FP64 pipe).  The reference's coplanarity move (forces only) is decided
// and applied in single precision, except for pairs whose test lies within
// rounding of its threshold, which go to the extended pass.
#include <cuda_runtime.h>

#include "mech_device.cuh"
#include "mech_exvol_math.cuh"

#ifndef MECH_EXVOL_REAL
#define MECH_EXVOL_REAL double
#endif

namespace mech {

constexpr int kFbNodesEnergy = 400;       // Simpson intervals, energy (:929-930)
constexpr int kFbNodesForce = 10000;      // Simpson intervals, forces (:1041-1042)

// FP64 engine: the reference's forms, for parity.
static __device__ double pair_energy_d(const double* c1, const double* c2, const double* c3, const double* c4,
                                       double kRep) {
    double v12[3], v34[3], v31[3], v14[3], v32[3], v24[3];
    diffs_of(c1, c2, c3, c4, v12, v34, v31, v14, v32, v24);
    PairInv<double> p;
    pair_inv(v12, v34, v31, v14, v32, v24, p, false);
    return energy_from(p, kRep);
}


// FP64 forces of a pair at double positions, with the reference's coplanar
// move of c2 (:610-626, force path only).
static __device__ bool pair_forces_d(const double* c1, const double* c2in, const double* c3, const double* c4, double kRep,
                                     double out[4][3]) {
    double moved2[3];
    const double* c2 = c2in;
    if (coplanarity<double>(c1, c2in, c3, c4) < 0.1) {
        push_c2(c1, c2in, c3, moved2);
        c2 = moved2;
    }
    double v12[3], v34[3], v31[3], v14[3], v32[3], v24[3];
    diffs_of(c1, c2, c3, c4, v12, v34, v31, v14, v32, v24);
    PairInv<double> p;
    pair_inv(v12, v34, v31, v14, v32, v24, p, false);
    return forces_from<false>(p, v12, v34, v31, kRep, out);
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

// Simpson energies of the flagged pairs: block `blk` of `nblk` takes entries
// blk, blk + nblk, ...
template <typename Real>
__device__ void fb_energy_blocks(const DevNet<Real>& n, int blk, int nblk, double* sh) {
    const int cnt = min(*n.ev_fb_count, kExvolFallbackCap);
    for (int k = blk; k < cnt; k += nblk) {
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
    MECH_TRACE_KERNEL(n, TK_EXVOL_FB_FORCE);
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

constexpr float kMixedTauEnergy = 0.005f;  // extended pass below this normalized triple product (energy)
constexpr float kMixedTauForce = 0.02f;    // (forces, whose formula loses more to cancellation)

// Warp-aggregated append of (replica, pair) to the extended-pass pair list.
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
        if (k < 2 * n.n_ev) {   // room for both trials of a two-trial pass
            n.ev_list[2 * k] = r;
            n.ev_list[2 * k + 1] = pr;
        } else {
            atomicOr(n.err, 4u);
        }
    }
}

// Mixed engine: the energy of one pair in single precision, or need64 when the
// pair is ill-conditioned (normalized triple product under kMixedTauEnergy) or
// the formula gives no number; such pairs go to the extended pass.
__device__ __forceinline__ float mixed_pair_energy(const Pos<float>& p1, const Pos<float>& p2, const Pos<float>& p3,
                                                   const Pos<float>& p4, float kRep, bool& need64) {
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
    need64 = !(q >= kMixedTauEnergy);
    if (need64) return 0.f;
    PairInv<float> pi;
    pair_inv(v12, v34, v31, v14, v32, v24, pi, true);
    const float u = energy_value(pi, kRep);
    if (u != u) {
        need64 = true;
        return 0.f;
    }
    return u;
}

template <typename Real>
__global__ void __launch_bounds__(kBlock) k_exvol(DevNet<Real> n, int want, int trial, int force, int tile_off) {
    MECH_TRACE_KERNEL(n, TK_EXVOL);
    __shared__ double sh[32];
    __shared__ int s_go, s_xb;
    __shared__ double s_lam;
    __shared__ float s_lf;   // the step rounded once (mixed engine)
    const int ti = tile_off + blockIdx.x;
    const Tile t = n.stile[ti];
    const int r = t.replica;
    if (threadIdx.x == 0) {
        const CGState& S = n.st[r];
        s_go = want < 0 ? (S.active != 0) : (S.phase == want);
        s_xb = S.xbuf;
        s_lam = S.lambda;
        s_lf = (float)S.lambda;
    }
    __syncthreads();
    if (!s_go) return;
    const Real* X = n.x[s_xb];
    const bool tr = trial != 0;
    const int i = t.begin + threadIdx.x;
    const bool valid = i < t.end;
    double e = 0.0;   // FP64 engine
    float ef = 0.f;   // mixed engine
    bool need64 = false, need64b = false;
    // a two-trial pass also evaluates the energy at lambda / 2 (mixed engine)
    const bool dual = sizeof(Real) == 4 && trial == kTrialDual && !force;
    if (valid) {
        const int4 bs = n.ev_bead[i];
        auto pos = [&](int b) -> Pos<Real> {
            if constexpr (sizeof(Real) == 4) {
                const Pos<float> p = load_pos(X, b);
                return tr ? moved_f(p, n.d, b, s_lf) : p;
            } else {
                return bead_at(X, n.d, b, tr, s_lam);
            }
        };
        const Pos<Real> p1 = pos(bs.x), p2 = pos(bs.y), p3 = pos(bs.z), p4 = pos(bs.w);
        if constexpr (sizeof(Real) == 8) {
            const double kRepD = (double)n.ev_k[i] * (double)n.ev_la[i] * (double)n.ev_lb[i];
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
        } else if (!force) {
            // mixed engine: single precision unless the pair is ill-conditioned
            const float kRep = n.ev_k[i] * n.ev_la[i] * n.ev_lb[i];
            ef = mixed_pair_energy(p1, p2, p3, p4, kRep, need64);
            store_pair(n.ev_energy + i, ef, 0.f);
            if (dual) {
                const float lh = 0.5f * s_lf;
                const float ef2 = mixed_pair_energy(moved_f(load_pos(X, bs.x), n.d, bs.x, lh),
                                                    moved_f(load_pos(X, bs.y), n.d, bs.y, lh),
                                                    moved_f(load_pos(X, bs.z), n.d, bs.z, lh),
                                                    moved_f(load_pos(X, bs.w), n.d, bs.w, lh), kRep, need64b);
                store_pair(n.ev_energy2 + i, ef2, 0.f);
            }
        } else {
            // mixed engine, forces: single precision unless the pair is ill-conditioned
            const float kRep = n.ev_k[i] * n.ev_la[i] * n.ev_lb[i];
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
                // single precision cannot decide go to the extended pass; the others are moved
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
                float out[4][3];
                if (forces_from<true>(pi, v12, v34, v31, kRep, out)) {
                    for (int a = 0; a < 4; ++a) {
                        Real* cdst = slot_ptr(n, n.slot_base[K_EXVOL] + 4 * i + a);
                        for (int k = 0; k < 3; ++k) cdst[k] = (Real)out[a][k];
                    }
                } else {
                    need64 = true;
                }
            }
        }
    }
    if constexpr (sizeof(Real) == 4) {
        append_fp64(n, need64, r, i);
        if (dual) append_fp64(n, need64b, r, i | kExtSecond);   // block-uniform
    }
    if (!force && sizeof(Real) == 8) {
        e = block_sum(e, sh);
        if (threadIdx.x == 0) n.part_sp[ti] = e;
    }
}

// Mixed engine's extended pass: the listed (ill-conditioned) pairs in FP64,
// split over the four warps of a block.  On this GPU a warp's FP64
// instruction holds its SM sub-partition's FP64 pipe for ~78 cycles whatever
// the number of active lanes, so the time of the pass is the FP64 instruction
// count of one warp's path, not the pair count: one pair's ~1,000 FP64
// operations in one warp took ~35 us.  Here lane l of every warp takes pair
// 32 g + l of the block's group g, and warp w evaluates the w-th of the four
// arctangent terms of the integral (A, E, B, F below: cross product, norm,
// numerator, arctangent and, for forces, its partial derivatives); the shared
// invariants are formed by every warp, the six entries of the G matrix are
// split over the warps, and warp w forms the force on bead w.  Partial results
// pass through shared memory.  The cancellation-free forms of pair_inv
// (cross = true) and forces_from<true> are followed term by term, with the
// reference's coplanar move of c2 (:610-626, forces only, decided without
// divisions: (n . v3)^2 < 0.01 |n|^2 |v3|^2).
constexpr int kExtBlocks = 152;   // one 4-warp block per SM: one warp per sub-partition

// per-term operands: cross product u x v, arctangent argument p . q (negated for B, F),
// and the two arctangent abscissae alpha, beta (A: a+e, e; E: a+e-d, e-d; B: F, F-b; F: d+F, d+F-b)
struct ExtTerm {
    double N, rY, ATG, tN, tXr, tlo, thi, S;
};

template <typename Real>
__global__ void __launch_bounds__(128) k_exvol_ext(DevNet<Real> n, int trial, int force) {
    MECH_TRACE_KERNEL(n, TK_EXVOL_EXT);
    __shared__ double s_c[4][32][3];       // bead positions
    __shared__ double s_N[3][32];          // CC, GG, DD for the F term's HH
    __shared__ ExtTerm s_t[4][32];
    __shared__ double s_G[6][32];
    __shared__ int s_bad[32];
    const int cnt = min(*n.ev_list_count, 2 * n.n_ev);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int ngroups = (cnt + 31) >> 5;
    for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
        const int k = 32 * g + l;
        const bool valid = k < cnt;
        int r = 0, i = 0;
        bool second = false;   // the lambda / 2 trial of a two-trial pass
        double lam = 0.0;
        if (valid) {
            r = n.ev_list[2 * k];
            i = n.ev_list[2 * k + 1];
            second = (i & kExtSecond) != 0;
            i &= ~kExtSecond;
            lam = n.st[r].lambda;
            if (second) lam *= 0.5;
        }
        // ---- positions: warp w converts bead w of every pair
        if (valid) {
            const CGState& S = n.st[r];
            const int4 bs = n.ev_bead[i];
            const int bead = w == 0 ? bs.x : w == 1 ? bs.y : w == 2 ? bs.z : bs.w;
            double c[3];
            to_double(bead_at(n.x[S.xbuf], n.d, bead, trial != 0, lam), c);
            s_c[w][l][0] = c[0];
            s_c[w][l][1] = c[1];
            s_c[w][l][2] = c[2];
        }
        if (w == 0) s_bad[l] = 0;
        __syncthreads();
        double v12[3], v34[3], v31[3], v14[3], v32[3], v24[3];
        double a = 0, b = 0, c = 0, d = 0, e = 0, F = 0, JJ = 1, kRep = 0;
        double x21[3] = {0, 0, 0};
        if (valid) {
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const double c1 = s_c[0][l][q], c2 = s_c[1][l][q], c3 = s_c[2][l][q], c4 = s_c[3][l][q];
                v12[q] = c2 - c1;
                v34[q] = c4 - c3;
                v31[q] = c1 - c3;
                v14[q] = c4 - c1;
                v32[q] = c2 - c3;
                v24[q] = c4 - c2;
            }
            if (force) {
                // n = (c2 - c1) x (c3 - c1) = -(v12 x v31), v3 = c4 - c1 = v14
                const double nx = v12[2] * v31[1] - v12[1] * v31[2], ny = v12[0] * v31[2] - v12[2] * v31[0],
                             nz = v12[1] * v31[0] - v12[0] * v31[1];
                const double nn = nx * nx + ny * ny + nz * nz, nv = nx * v14[0] + ny * v14[1] + nz * v14[2];
                if (nv * nv < 0.01 * nn * dot3(v14, v14)) {
                    const double sc = 0.01 / sqrt(nn);
                    const double dn[3] = {sc * nx, sc * ny, sc * nz};
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        v12[q] += dn[q];
                        v32[q] += dn[q];
                        v24[q] -= dn[q];
                    }
                }
            }
            a = dot3(v12, v12);
            b = dot3(v34, v34);
            c = dot3(v31, v31);
            d = dot3(v12, v34);
            e = dot3(v12, v31);
            F = dot3(v34, v31);
            x21[0] = v34[1] * v12[2] - v34[2] * v12[1];
            x21[1] = v34[2] * v12[0] - v34[0] * v12[2];
            x21[2] = v34[0] * v12[1] - v34[1] * v12[0];
            const double trip = -(x21[0] * v31[0] + x21[1] * v31[1] + x21[2] * v31[2]);
            JJ = -trip * trip;
            kRep = (double)n.ev_k[i] * (double)n.ev_la[i] * (double)n.ev_lb[i];
        }
        // ---- term w: cross product, norm, numerator
        double xu[3] = {0, 0, 0}, Y = 1, N = 0;
        if (valid) {
            double u[3], v[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {   // selects, not pointers: the vectors stay in registers
                u[q] = w < 2 ? v12[q] : v34[q];
                v[q] = w == 0 ? v31[q] : w == 1 ? v14[q] : w == 2 ? v31[q] : v32[q];
            }
            xu[0] = u[1] * v[2] - u[2] * v[1];
            xu[1] = u[2] * v[0] - u[0] * v[2];
            xu[2] = u[0] * v[1] - u[1] * v[0];
            Y = sqrt(dot3(xu, xu));
            if (w < 3) {
                N = dot3(xu, x21);   // CC = x13 . x21, GG = x14 . x21, DD = x21 . x23
                s_N[w][l] = N;
            }
        }
        __syncthreads();
        if (valid) {
            if (w == 3) N = s_N[0][l] + s_N[1][l] - s_N[2][l];   // HH = CC + GG - DD
            double p[3], q[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                p[j] = w == 0 ? v31[j] : w == 1 ? v14[j] : w == 2 ? v31[j] : v32[j];
                q[j] = w == 0 ? v32[j] : w == 1 ? v24[j] : w == 2 ? v14[j] : v24[j];
            }
            const double arg = w < 2 ? dot3(p, q) : -dot3(p, q);
            ExtTerm t;
            t.N = N;
            t.ATG = atan2(Y, arg);
            t.rY = 1.0 / Y;
            t.S = N * t.rY * t.ATG;
            if (force) {
                const double al = w == 0 ? a + e : w == 1 ? a + e - d : w == 2 ? F : d + F;
                const double be = al - (w < 2 ? a : b);
                const double Y2 = Y * Y;
                const double T1 = Y2 / (Y2 + al * al), T2 = Y2 / (Y2 + be * be);
                const double r2 = t.rY * t.rY;
                t.tN = t.ATG * t.rY;
                const double tX = -(t.ATG * N) * r2 + ((-T1 * al + T2 * be) * N) * (r2 * t.rY);
                t.tXr = tX * t.rY;
                t.tlo = ((T1 - T2) * N) * r2;
                t.thi = (T1 * N) * r2;
            }
            s_t[w][l] = t;
        }
        __syncthreads();
        if (!force) {
            if (w == 0 && valid) {
                const double Ssum = s_t[0][l].S + s_t[1][l].S + s_t[2][l].S + s_t[3][l].S;
                const double U = 0.5 * kRep / JJ * Ssum;
                double* dst = (second ? n.ev_energy2 : n.ev_energy) + i;
                if (!(fabs(U) < 1.0 / 0.0) || U < -1.0) {
                    flag_fallback(n, r, i, trial != 0 ? lam : 0.0);
                    store_pair(dst, 0.f, 0.f);
                } else {
                    const float h = (float)U;
                    store_pair(dst, h, (float)(U - (double)h));
                }
            }
            __syncthreads();   // shared arrays are reused by the next group
            continue;
        }
        // ---- G entries, split over the warps (0: G00, G12; 1: G01, G22; 2: G02; 3: G11)
        if (valid) {
            const ExtTerm A = s_t[0][l], E = s_t[1][l], B = s_t[2][l], FT = s_t[3][l];
            if (w == 0) {
                s_G[0][l] = A.tN * (-2 * F) + A.tXr * c + A.thi * 2 + E.tN * (2 * (F - b)) + E.tXr * (b + c - 2 * F) +
                            E.thi * 2 + FT.tN * (-2 * b) + FT.tXr * b;
                s_G[4][l] = A.tN * (-a) + E.tN * a + E.tXr * (-a) + B.tN * (-d) + B.tXr * (-F) + B.tlo + FT.tN * d +
                            FT.tXr * (-(d + F)) + FT.tlo;
            } else if (w == 1) {
                s_G[1][l] = A.tN * e + E.tN * (2 * d - e) + E.tXr * (e - d) - E.tlo + B.tN * (-F) + FT.tN * (2 * d + F) +
                            FT.tXr * (-(d + F)) + FT.tlo;
                s_G[5][l] = A.tXr * a + E.tXr * a + B.tXr * b + FT.tXr * b;
            } else if (w == 2) {
                s_G[2][l] = A.tN * d + A.tXr * (-e) + A.tlo + E.tN * (-d) + E.tXr * (-(e - d)) + E.tlo + B.tN * b +
                            FT.tN * (-b) + FT.tXr * b;
            } else {
                s_G[3][l] = E.tN * (-2 * a) + E.tXr * a + B.tN * (2 * e) + B.tXr * c + B.tlo * (-2) + B.thi * 2 +
                            FT.tN * (-2 * (a + e)) + FT.tXr * (a + c + 2 * e) + FT.tlo * (-2) + FT.thi * 2;
            }
        }
        __syncthreads();
        // ---- warp w: the force on bead w
        if (valid) {
            const double G[3][3] = {{s_G[0][l], s_G[1][l], s_G[2][l]},
                                    {s_G[1][l], s_G[3][l], s_G[4][l]},
                                    {s_G[2][l], s_G[4][l], s_G[5][l]}};
            const double J[3][3] = {{2 * (-b * c + F * F), 2 * (c * d - e * F), 2 * (b * e - d * F)},
                                    {2 * (c * d - e * F), 2 * (-a * c + e * e), 2 * (-d * e + a * F)},
                                    {2 * (b * e - d * F), 2 * (-d * e + a * F), 2 * (d * d - a * b)}};
            const double invJJ = 1.0 / JJ;
            const double Ssum = s_t[0][l].S + s_t[1][l].S + s_t[2][l].S + s_t[3][l].S;
            const double pref = kRep * invJJ / 2.0, m = -invJJ * Ssum;
            double dv[3];
#pragma unroll
            for (int y = 0; y < 3; ++y) {
                const double Jw = w == 0 ? J[2][y] - J[0][y] : w == 1 ? J[0][y] : w == 2 ? -J[2][y] - J[1][y] : J[1][y];
                const double Gw = w == 0 ? G[2][y] - G[0][y] : w == 1 ? G[0][y] : w == 2 ? -G[2][y] - G[1][y] : G[1][y];
                dv[y] = pref * (m * Jw + Gw);
            }
            Real* cdst = slot_ptr(n, n.slot_base[K_EXVOL] + 4 * i + w);
            bool bad = false;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const double o = -(dv[0] * v12[q] + dv[1] * v34[q] + dv[2] * v31[q]);
                if (!(fabs(o) < 1.0 / 0.0)) bad = true;
                cdst[q] = (Real)o;
            }
            if (bad) atomicOr(&s_bad[l], 1);
        }
        __syncthreads();
        if (w == 0 && valid && s_bad[l]) flag_fallback(n, r, i, 0.0);
        __syncthreads();   // shared arrays are reused by the next group
    }
}

// The end of an energy evaluation's excluded-volume chain, one launch:
// blocks [0, kFbEnergyBlocks) compute the Simpson energies of flagged pairs;
// in the mixed engine the following blocks form the deterministic per-tile
// sums of the per-pair energies (one block per exvol tile).
constexpr int kFbEnergyBlocks = 64;
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_exvol_energy_tail(DevNet<Real> n, int want, int trial, int tile_off) {
    MECH_TRACE_KERNEL(n, TK_EXVOL_TAIL);
    __shared__ double sh[64];   // block_reduce_ff<2>: 32 * 4 floats
    if ((int)blockIdx.x < kFbEnergyBlocks) {
        fb_energy_blocks(n, blockIdx.x, kFbEnergyBlocks, sh);
    } else {
        const int ti = tile_off + (int)blockIdx.x - kFbEnergyBlocks;
        const Tile t = n.stile[ti];
        const CGState& S = n.st[t.replica];
        const bool go = want < 0 ? (S.active != 0) : (S.phase == want);
        if constexpr (sizeof(Real) == 4) {
            if (go) {   // block-uniform
                // per-pair energies as (hi, lo) pairs, summed compensated in single precision
                const int i = t.begin + threadIdx.x;
                if (trial == kTrialDual) {   // both trials of a two-trial pass
                    FF a[2];
                    if (i < t.end) {
                        add_pair(a[0], load_pair(n.ev_energy + i));
                        add_pair(a[1], load_pair(n.ev_energy2 + i));
                    }
                    block_reduce_ff<2, 0>(a, nullptr, reinterpret_cast<float*>(sh));
                    if (threadIdx.x == 0) {
                        store_pair(n.part_sp + ti, a[0].h, a[0].l);
                        store_pair(n.part_sp2 + ti, a[1].h, a[1].l);
                    }
                } else {
                    FF a[1];
                    if (i < t.end) add_pair(a[0], load_pair(n.ev_energy + i));
                    block_reduce_ff<1, 0>(a, nullptr, reinterpret_cast<float*>(sh));
                    if (threadIdx.x == 0) store_pair(n.part_sp + ti, a[0].h, a[0].l);
                }
            }
        }
    }
}

// zero the extended-pass and fallback work-list counts (one memset when they are
// neighbours in one buffer)
template <typename Real>
static inline void reset_counts(const DevNet<Real>& n, cudaStream_t s) {
    if (n.ev_fb_count == n.ev_list_count + 2) {
        cudaMemsetAsync(n.ev_list_count, 0, 4 * sizeof(int), s);
    } else {
        cudaMemsetAsync(n.ev_list_count, 0, sizeof(int), s);
        cudaMemsetAsync(n.ev_fb_count, 0, sizeof(int), s);
    }
}

template <typename Real>
static inline int ev_tiles_of(const DevNet<Real>& n, int* off) {
    *off = n.sp_tiles[K_LINKER] + n.sp_tiles[K_MOTOR];
    return n.sp_tiles[K_EXVOL];
}

// Inside an evaluation (standalone = false) the work-list counts are zero on
// entry: the evaluation's reduction kernel zeroes them for the next one, which
// keeps a memset off the head of the excluded-volume lane.  A standalone
// launch zeroes them first and leaves them as they end.
template <typename Real>
int launch_exvol_energy(const DevNet<Real>& n, int want, int trial, cudaStream_t s, bool standalone) {
    int off = 0;
    const int nt = ev_tiles_of(n, &off);
    if (nt == 0) return 0;
    if (standalone) reset_counts(n, s);
    k_exvol<Real><<<nt, kBlock, 0, s>>>(n, want, trial, 0, off);
    int k = 1;
    if constexpr (sizeof(Real) == 4) {
        k_exvol_ext<Real><<<kExtBlocks, 128, 0, s>>>(n, trial, 0);
        ++k;
    }
    k_exvol_energy_tail<Real><<<kFbEnergyBlocks + (sizeof(Real) == 4 ? nt : 0), kBlock, 0, s>>>(n, want, trial, off);
    return k + 1;
}

template <typename Real>
int launch_exvol_forces(const DevNet<Real>& n, int want, cudaStream_t s, bool standalone) {
    int off = 0;
    const int nt = ev_tiles_of(n, &off);
    if (nt == 0) return 0;
    if (standalone) reset_counts(n, s);
    k_exvol<Real><<<nt, kBlock, 0, s>>>(n, want, 0, 1, off);
    int k = 1;
    if constexpr (sizeof(Real) == 4) {
        k_exvol_ext<Real><<<kExtBlocks, 128, 0, s>>>(n, 0, 1);
        ++k;
    }
    k_exvol_fb_force<Real><<<4 * 152, kBlock, 0, s>>>(n, n.fb_moments, n.fb_tickets);
    return k + 1;
}

template int launch_exvol_energy<MECH_EXVOL_REAL>(const DevNet<MECH_EXVOL_REAL>&, int, int, cudaStream_t, bool);
template int launch_exvol_forces<MECH_EXVOL_REAL>(const DevNet<MECH_EXVOL_REAL>&, int, cudaStream_t, bool);

}  // namespace mech
