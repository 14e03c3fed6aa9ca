// The per-replica reductions and CG step logic of the device-resident
// minimizer (CGMethod.hpp:238-373 and :826-1743, ForceFieldManager.cpp:96-290;
// paths relative to medyan-5.4.0/src), shared by the translation units whose
// kernels end an evaluation: the separate finalizer kernels (one block per
// replica) and, for a single replica, the last block of the kernel that
// writes an evaluation's final partial sums.
#pragma once

#include "mech_device.cuh"

namespace mech {

__device__ __forceinline__ bool replica_selected(const CGState& S, int want) {
    return want < 0 ? (S.active != 0) : (S.phase == want);
}

// ---------------------------------------------------------------------------
// finalizers (run by the whole last block of a replica)
// ---------------------------------------------------------------------------
// Partial-sum slots of a replica's tile range [b, e): the FP64 kernels write
// one per tile (stride 1); the persistent mixed kernels write one per run of
// tiles, at b and at every multiple of their tiles-per-block inside (b, e).
__device__ __forceinline__ int run_slots(int b, int e, int stride) {
    const int m0 = (b / stride + 1) * stride;
    return 1 + (m0 < e ? (e - 1 - m0) / stride + 1 : 0);
}
__device__ __forceinline__ int run_slot(int b, int stride, int k) {
    return k == 0 ? b : (b / stride + 1) * stride + (k - 1) * stride;
}

// The CG step logic of the finalizers runs in thread 0 on a register copy of
// its replica's state, loaded at the start so that the loads overlap the
// block's reduction, and stored back once: done field by field on global
// memory, the branchy logic waits on one dependent load after another.
// Per force field energies of one evaluation from the reduced partial sums
// `e`, with the numeric fallback energies of the replica's flagged pairs
// added in pair order (only entries recorded at step `lam` when `match_lam`).
// A failed pair makes the force field report -1 (CylinderExclVolRepulsion.cpp:442-481).
template <typename Real>
__device__ void add_fallback_energies(const DevNet<Real>& n, int r, int fb_count, bool match_lam, double lam,
                                      double* e) {
    const int cnt = min(fb_count, kExvolFallbackCap);
    int last = -1;
    bool ev_failed = false;
    for (;;) {
        int best = -1, bestPair = 0x7fffffff;
        for (int k = 0; k < cnt; ++k) {
            const int rep = __ldcg(n.ev_fb_list + 2 * k), pr = __ldcg(n.ev_fb_list + 2 * k + 1);
            if (rep != r || pr <= last || pr >= bestPair) continue;
            if (match_lam &&
                __longlong_as_double(__ldcg((const long long*)n.ev_fb_energy + kExvolFallbackCap + k)) != lam)
                continue;
            best = k;
            bestPair = pr;
        }
        if (best < 0) break;
        const double u = __ldcg(n.ev_fb_energy + best);
        if (u == -1.0) ev_failed = true;
        else e[MECH_FF_EXVOL] += u;
        last = bestPair;
    }
    if (ev_failed) e[MECH_FF_EXVOL] = -1.0;
}

// The evaluation's per force field energies into S.eval; returns the
// computeEnergy value (+inf when a force field failed).
__device__ __forceinline__ double record_energies(CGState& S, const double* e) {
    double tot = 0.0;
    bool failed = false;
    for (int k = 0; k < MECH_NUM_FF; ++k) {
        S.eval[k] = e[k];
        tot += e[k];
        if (e[k] <= -1) failed = true;
    }
    S.eval[MECH_NUM_FF] = tot;
    S.evalFailed = failed;
    S.numEnergyEval++;
    return failed ? (1.0 / 0.0) : tot;
}

// The finalizers take the replica's tile ranges and (thread 0) a register copy
// of its state, both loaded by the kernel at its start together with the
// phase it selects on: on this GPU every dependent round trip to L2 (partial
// slots written by the other die's SMs) costs about a microsecond, and a
// finalizer is a chain of them on the minimizer's critical path.
template <typename Real>
__device__ void finalize_energy(const DevNet<Real>& n, int r, int trial, const RepTiles& rt, CGState& S, double* sh) {
    const int stride = sizeof(Real) == 4 ? n.ptiles[0] : 1;
    const int nslot = run_slots(rt.fil_begin, rt.fil_end, stride);
    const int ffk[K_NUM_SPARSE] = {MECH_FF_LINKER, MECH_FF_MOTOR, MECH_FF_EXVOL, MECH_FF_BOUNDARY};
    double e[MECH_NUM_FF], e2[MECH_NUM_FF];
    const bool dual = sizeof(Real) == 4 && trial == kTrialDual;
    // the fallback list's length, loaded now so that thread 0's step logic does
    // not wait on it at the end
    const int fb_count = threadIdx.x == 0 ? __ldcg(n.ev_fb_count) : 0;
    MECH_TRACE_STAMP(ts_load);
    if constexpr (sizeof(Real) == 4) {
        // mixed: (hi, lo) pair slots summed compensated in single precision;
        // the doubles are formed in thread 0 only.  acc[0, 6): the (first)
        // trial, acc[6, 12): the second trial of a two-trial pass.
        FF acc[2 * MECH_NUM_FF];
        // each sparse kind's first slot of this thread, loaded with the first filament slots
        float2 sp0[K_NUM_SPARSE], sp1[K_NUM_SPARSE];
#pragma unroll
        for (int k = 0; k < K_NUM_SPARSE; ++k) {
            const int i = rt.sp_begin[k] + threadIdx.x;
            sp0[k] = sp1[k] = make_float2(0.f, 0.f);
            if (i < rt.sp_end[k]) {
                sp0[k] = load_pair(n.part_sp + i);
                if (dual) sp1[k] = load_pair(n.part_sp2 + i);
            }
        }
#pragma unroll 8
        for (int k = threadIdx.x; k < nslot; k += blockDim.x) {
            const double* slot = n.part_fil + 4 * (size_t)run_slot(rt.fil_begin, stride, k);
            add_pair(acc[MECH_FF_STRETCHING], load_pair(slot));
            add_pair(acc[MECH_FF_BENDING], load_pair(slot + 1));
            if (dual) {
                add_pair(acc[MECH_NUM_FF + MECH_FF_STRETCHING], load_pair(slot + 2));
                add_pair(acc[MECH_NUM_FF + MECH_FF_BENDING], load_pair(slot + 3));
            }
        }
#pragma unroll
        for (int k = 0; k < K_NUM_SPARSE; ++k) {
            const int i0 = rt.sp_begin[k] + threadIdx.x;
            if (i0 < rt.sp_end[k]) {
                add_pair(acc[ffk[k]], sp0[k]);
                if (dual) add_pair(acc[MECH_NUM_FF + ffk[k]], sp1[k]);
            }
#pragma unroll 4
            for (int i = i0 + blockDim.x; i < rt.sp_end[k]; i += blockDim.x) {
                add_pair(acc[ffk[k]], load_pair(n.part_sp + i));
                if (dual) add_pair(acc[MECH_NUM_FF + ffk[k]], load_pair(n.part_sp2 + i));
            }
        }
        MECH_TRACE_SECTION(n, TK_SEC_FE_LOAD, ts_load);
        MECH_TRACE_STAMP(ts_red);
        if (dual) {
            block_reduce_ff<2 * MECH_NUM_FF, 0>(acc, nullptr, reinterpret_cast<float*>(sh));
        } else {
            FF (&a6)[MECH_NUM_FF] = *reinterpret_cast<FF(*)[MECH_NUM_FF]>(acc);
            block_reduce_ff<MECH_NUM_FF, 0>(a6, nullptr, reinterpret_cast<float*>(sh));
        }
        MECH_TRACE_SECTION(n, TK_SEC_FE_REDUCE, ts_red);
        if (threadIdx.x >= 32) return;
        // hi + lo in double, one pair per lane of warp 0: an FP64 warp
        // instruction costs the same with 1 or 12 active lanes, so the
        // conversions take 3 warp instructions instead of 36 in thread 0
        const int lane = threadIdx.x;
        float ph = 0.f, pl = 0.f;
#pragma unroll
        for (int k = 0; k < 2 * MECH_NUM_FF; ++k) {
            const float h = __shfl_sync(0xffffffffu, acc[k].h, 0), l = __shfl_sync(0xffffffffu, acc[k].l, 0);
            if (lane == k) {
                ph = h;
                pl = l;
            }
        }
        const double v = (double)ph + (double)pl;
#pragma unroll
        for (int k = 0; k < MECH_NUM_FF; ++k) {
            e[k] = __shfl_sync(0xffffffffu, v, k);
            e2[k] = __shfl_sync(0xffffffffu, v, MECH_NUM_FF + k);
        }
        if (threadIdx.x != 0) return;
    } else {
        // every thread issues its loads back to back, then sums in a fixed order
        double acc[MECH_NUM_FF] = {0, 0, 0, 0, 0, 0};
#pragma unroll 8
        for (int k = threadIdx.x; k < nslot; k += blockDim.x) {
            const int i = run_slot(rt.fil_begin, stride, k);
            const double2 v = __ldcg(reinterpret_cast<const double2*>(n.part_fil + 4 * (size_t)i));
            acc[MECH_FF_STRETCHING] += v.x;
            acc[MECH_FF_BENDING] += v.y;
        }
#pragma unroll
        for (int k = 0; k < K_NUM_SPARSE; ++k) {
#pragma unroll 8
            for (int i = rt.sp_begin[k] + threadIdx.x; i < rt.sp_end[k]; i += blockDim.x)
                acc[ffk[k]] += __ldcg(n.part_sp + i);
        }
#pragma unroll
        for (int k = 0; k < MECH_NUM_FF; ++k) e[k] = warp_sum(acc[k]);
        const int ops[MECH_NUM_FF] = {0, 0, 0, 0, 0, 0};
        block_combine<MECH_NUM_FF>(e, ops, sh);
        if (threadIdx.x != 0) return;
    }
    MECH_TRACE_STAMP(ts_tail);
    const double lam = S.lambda;   // the (first) trial's step, before the line search moves it
    const int xb = S.xbuf;
    add_fallback_energies(n, r, fb_count, dual, lam, e);
    const double E = record_energies(S, e);
    if (trial && S.phase == PH_LS_TRIAL) {
        S.Etrial = E;
        // the trial positions: the other buffer (FP64), or the next of three (mixed)
        line_search_step(S, E, sizeof(Real) == 4 ? (xb + 1) % 3 : xb ^ 1);
        if (dual && S.phase == PH_LS_TRIAL) {
            // rejected at lambda and halved: the reference's next trial, at
            // lambda / 2, was evaluated by the same pass (positions in the third buffer)
            add_fallback_energies(n, r, fb_count, true, S.lambda, e2);
            const double E2 = record_energies(S, e2);
            S.Etrial = E2;
            line_search_step(S, E2, (xb + 2) % 3);
        } else if (dual) {
            S.numEnergyEval++;   // the second trial was evaluated but not needed
        }
    } else if (S.phase == PH_RECOVER_ENERGY) {
        S.E0 = E;
        S.phase = PH_RESET;
    } else {
        S.E0 = E;
    }
    n.st[r] = S;
    MECH_TRACE_SECTION(n, TK_SEC_FE_TAIL, ts_tail);
}

// CG bookkeeping after the forces (CGMethod.hpp:1540-1580): max |F|, beta.
__device__ __forceinline__ void force_step(CGState& S, double mx, double ff, double ffp) {
    const int ph = S.phase;
    if (ph == PH_FORCE || ph == PH_RECOVER_FORCE) S.numForceCall++;
    S.maxF = mx;
    S.FdotF = ff;
    S.fbuf ^= 1;
    if (!isfinite(mx)) {   // CGMethod::maxF throws (CGMethod.hpp:207-210)
        S.status = MECH_ERR_NONFINITE;
        S.phase = PH_ERROR;
        return;
    }
    if (ph == PH_FORCE) {
        S.energyRelChange = fabs(S.newEnergy - S.prevEnergy) / fabs(S.prevEnergy);
        S.prevEnergy = S.newEnergy;
        double beta = 0.0;
        if (S.method == 1) {
            S.newGrad = ff;
            beta = S.newGrad / S.lastFdotF;
        } else if (S.method == 2) {
            S.newGrad = ff;
            S.prevGrad = ffp;
            beta = fmax(0.0, (S.newGrad - S.prevGrad) / S.lastFdotF);
        }
        S.beta = beta;
        // minimum-energy backup once past half the call limit (CGMethod.hpp:1564-1566)
        if (mx <= 10 * S.gradTol && S.numIter > S.forceCallLimit / 2 && S.totalEnergy <= S.minimumE) {
            S.minimumE = S.totalEnergy;
            S.backupPending = 1;
        }
        S.phase = PH_DIR;
    } else if (ph == PH_RECOVER_FORCE) {
        S.phase = PH_RECOVER_ENERGY;
    }
}

// `store`: write the state back (k_tail_coop runs this in every block on the
// block's own copy and stores it from one block).
template <typename Real>
__device__ void finalize_force(const DevNet<Real>& n, int r, const RepTiles& rt, CGState& S, double* sh,
                               bool store = true) {
    // k_force_gather writes one slot per tile, k_force_gather_mx one per run of
    // a replica's tiles in a block
    const int stride = sizeof(Real) == 4 ? kGatherTiles : 1;
    const int nslot = run_slots(rt.fil_begin, rt.fil_end, stride);
    double mx, ff, ffp;
    MECH_TRACE_STAMP(ts_load);
    if constexpr (sizeof(Real) == 4) {
        // mixed slots hold float maxima and (hi, lo) pairs; sum them compensated
        // in single precision and form the doubles in thread 0 only
        FF a[2];
        float m[1] = {0.f};
#pragma unroll 4
        for (int k = threadIdx.x; k < nslot; k += blockDim.x) {
            const float* p = reinterpret_cast<const float*>(n.part_fil + 4 * (size_t)run_slot(rt.fil_begin, stride, k));
            const float4 v = __ldcg(reinterpret_cast<const float4*>(p));
            const float w = __ldcg(p + 4);
            m[0] = fmaxf(m[0], v.x);
            a[0].add(v.y);
            a[0].add(v.z);
            a[1].add(v.w);
            a[1].add(w);
        }
        MECH_TRACE_SECTION(n, TK_SEC_FF_LOAD, ts_load);
        MECH_TRACE_STAMP(ts_red);
        block_reduce_pairs<2, 1>(a, m, reinterpret_cast<float*>(sh));
        MECH_TRACE_SECTION(n, TK_SEC_FF_REDUCE, ts_red);
        if (threadIdx.x != 0) return;
        mx = (double)m[0];
        ff = (double)a[0].h + (double)a[0].l;
        ffp = (double)a[1].h + (double)a[1].l;
    } else {
        double a_mx = 0.0, a_ff = 0.0, a_ffp = 0.0;
#pragma unroll 8
        for (int k = threadIdx.x; k < nslot; k += blockDim.x) {
            const int i = run_slot(rt.fil_begin, stride, k);
            const double2 v = __ldcg(reinterpret_cast<const double2*>(n.part_fil + 4 * (size_t)i));
            const double w = __ldcg(n.part_fil + 4 * (size_t)i + 2);
            a_mx = fmax(a_mx, v.x);
            a_ff += v.y;
            a_ffp += w;
        }
        double red[3] = {warp_max(a_mx), warp_sum(a_ff), warp_sum(a_ffp)};
        const int ops[3] = {1, 0, 0};
        block_combine<3>(red, ops, sh);
        mx = red[0];
        ff = red[1];
        ffp = red[2];
        if (threadIdx.x != 0) return;
    }
    MECH_TRACE_STAMP(ts_tail);
    force_step(S, mx, ff, ffp);
    if (store) n.st[r] = S;
    MECH_TRACE_SECTION(n, TK_SEC_FF_TAIL, ts_tail);
}

// One block per replica after the direction update: the slope d.F, the
// conjugacy test and the next iteration's start (CGMethod.hpp:1553-1560).
template <typename Real>
__device__ void finalize_direction(const DevNet<Real>& n, int r, const RepTiles& rt, CGState& S, double* sh,
                                   bool store = true) {
    double slope;
    if constexpr (sizeof(Real) == 8) {
        slope = sum_slots(n.part_fil, 4, 3, rt.fil_begin, rt.fil_end, sh);
    } else {
        FF a[1];
        const int nslot = run_slots(rt.fil_begin, rt.fil_end, n.ptiles[2]);
#pragma unroll 8
        for (int k = threadIdx.x; k < nslot; k += blockDim.x)
            add_pair(a[0], load_pair(n.part_fil + 4 * (size_t)run_slot(rt.fil_begin, n.ptiles[2], k) + 3));
        block_reduce_ff<1, 0>(a, nullptr, reinterpret_cast<float*>(sh));
        slope = threadIdx.x == 0 ? (double)a[0].h + (double)a[0].l : 0.0;
    }
    if (threadIdx.x == 0) {
        if (S.backupPending) {
            S.backupValid = 1;
            S.backupPending = 0;
        }
        if (slope <= 0) {          // conjugacy lost: reset to steepest descent
            S.phase = PH_RESET;
        } else {
            S.slope = slope;
            if (S.method >= 1) S.lastFdotF = S.newGrad;
            begin_iteration(S);
        }
        if (store) n.st[r] = S;
    }
}

}  // namespace mech
