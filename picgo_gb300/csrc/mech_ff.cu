// Filament, linker/motor and boundary force-field kernels, the CG vector
// kernels and the per-replica finalizers of the device-resident minimizer.
//
// Reference behaviour restated here (paths relative to medyan-5.4.0/src):
//   FilamentStretchingHarmonic.cpp:185-275, FilamentBendingCosine.cpp:199-345,
//   LinkerStretchingHarmonic.cpp:191-293, MotorGhostStretchingHarmonic.cpp:234-340,
//   BoundaryCylinderRepulsionExp.cpp:27-110, ForceFieldManager.cpp:96-290,
//   CGMethod.hpp:238-373 and :826-1743, CGMethod.cpp:317-360,
//   MController.h:273-339 (recovery move).
//
// Filament forces are computed owner-side: a block loads its 256 beads plus a
// two-bead halo into shared memory, evaluates every cylinder and bending
// triple touching its beads once, and each bead sums its own terms in the
// reference's order (stretching, then bending, then the sparse force fields
// through the CSR gather), so no floating-point atomics are used and FP64
// forces follow the reference's per-bead summation order.
#include <cuda_runtime.h>

#include <algorithm>

#include "mech_bulk.cuh"
#include "mech_cg.cuh"
#include "mech_device.cuh"

namespace mech {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
// the three products of one bead, in the engine's precision; the sum over
// beads is carried by block_sum_r (compensated within a warp, then double)
__device__ __forceinline__ double bead_dot(double a0, double a1, double a2, double b0, double b1, double b2) {
    return a0 * b0 + a1 * b1 + a2 * b2;
}
__device__ __forceinline__ float bead_dot(float a0, float a1, float a2, float b0, float b1, float b2) {
    return fmaf(a2, b2, fmaf(a1, b1, a0 * b0));
}

// plane distance of a position (BoundaryElementImpl.h:49-53)
__device__ __forceinline__ double plane_dist_p(const double* pl, const Pos<double>& p) { return plane_dist(pl, p.x); }
__device__ __forceinline__ float plane_dist_p(const double* pl, const Pos<float>& p) {
    const float a = (float)pl[0], b = (float)pl[1], c = (float)pl[2], d = (float)pl[3];
    const float hi = a * p.h[0] + b * p.h[1] + c * p.h[2] + d;
    const float lo = a * p.l[0] + b * p.l[1] + c * p.l[2];
    return (hi + lo) / sqrtf(a * a + b * b + c * c);
}

// vector from the point at s1 on (c1, c2) to the point at s2 on (c3, c4)
// (LinkerStretchingHarmonic.cpp:200-216).  FP64: the interpolated points
// themselves, as the reference; mixed: the same vector from differences only,
// (c3 - c1) + s2 (c4 - c3) - s1 (c2 - c1).
__device__ __forceinline__ void bond_vector(const Pos<double>& c1, const Pos<double>& c2, const Pos<double>& c3,
                                            const Pos<double>& c4, double s1, double s2, double v[3]) {
    double p1[3], p2[3];
    lerp3(c1.x, c2.x, s1, p1);
    lerp3(c3.x, c4.x, s2, p2);
    v[0] = p2[0] - p1[0];
    v[1] = p2[1] - p1[1];
    v[2] = p2[2] - p1[2];
}
__device__ __forceinline__ void bond_vector(const Pos<float>& c1, const Pos<float>& c2, const Pos<float>& c3,
                                            const Pos<float>& c4, float s1, float s2, float v[3]) {
    float d31[3], d43[3], d21[3];
    pdiff(c3, c1, d31);
    pdiff(c4, c3, d43);
    pdiff(c2, c1, d21);
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] = fmaf(s2, d43[k], fmaf(-s1, d21[k], d31[k]));
}

// ---------------------------------------------------------------------------
// Conditions of the minimizer's conditional graph (GraphConds).
// ---------------------------------------------------------------------------
constexpr int kCondTrial = 2, kCondForce = 3, kCondDir = 4, kCondMisc = 5;   // counter slots

// Which phases the replicas are in, read past L1 (other blocks wrote the
// states); every thread of one block calls it, thread 0 sets the handles.
// `head`: the kernel at the head of a loop body, which also counts bodies and
// decides whether the loop runs another one after this body.
template <typename Real>
__device__ void set_conditions(const DevNet<Real>& n, bool head, int phase_slot) {
    int tr = 0, fo = 0, di = 0, mi = 0, host = 0;
    for (int r = threadIdx.x; r < n.R; r += blockDim.x) {
        const int ph = __ldcg(&n.st[r].phase);
        tr |= ph == PH_LS_TRIAL;
        fo |= ph == PH_FORCE;
        di |= ph == PH_DIR;
        mi |= ph == PH_RESET || ph == PH_FAILED;
        host |= ph >= PH_RECOVER;   // the recovery move is sequenced by the host
    }
    tr = __syncthreads_or(tr);
    fo = __syncthreads_or(fo);
    di = __syncthreads_or(di);
    mi = __syncthreads_or(mi);
    host = __syncthreads_or(host);
    if (threadIdx.x != 0) return;
    cudaGraphSetConditional(n.cond.trial, tr ? 1u : 0u);
    cudaGraphSetConditional(n.cond.force, fo ? 1u : 0u);
    cudaGraphSetConditional(n.cond.dir, di ? 1u : 0u);
    cudaGraphSetConditional(n.cond.misc, mi ? 1u : 0u);
    if (phase_slot >= 0) n.cond.counter[phase_slot]++;
    if (head) {
        // the loop ends after this body when nothing is left to do on the
        // device, an error is latched or the body budget of the launch is spent
        const int bodies = ++n.cond.counter[0];
        const bool more = (tr | fo | di | mi) && !host && __ldcg(n.err) == 0 && bodies < n.cond.cap;
        cudaGraphSetConditional(n.cond.loop, more ? 1u : 0u);
    }
}

// After a phase's per-replica reduction (one block per replica): the last
// block to finish sets the conditions of the phases that follow in the body.
template <typename Real>
__device__ void after_phase(const DevNet<Real>& n, int phase_slot, int* s_flag) {
    if (!n.cond.on) return;
    if (last_tile(n.cond.counter + 1, 0, gridDim.x, s_flag)) set_conditions(n, false, phase_slot);
}

// After an evaluation's per-replica reduction: the last block zeroes the
// excluded-volume work-list counts for the next evaluation (every block has
// read them by then), then sets the graph conditions when there are any.
template <typename Real>
__device__ void after_evaluation(const DevNet<Real>& n, int phase_slot, int* s_flag) {
    if (gridDim.x == 1) __syncthreads();   // one replica: this block is the last, no ticket needed
    else if (!last_tile(n.gticket, 0, gridDim.x, s_flag)) return;
    if (threadIdx.x == 0) {
        if (n.ev_list_count) *n.ev_list_count = 0;
        if (n.ev_fb_count) *n.ev_fb_count = 0;
    }
    if (n.cond.on) set_conditions(n, false, phase_slot);
}

// The kernel at the head of every body of the minimizer's while loop.
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_body_head(DevNet<Real> n) {
    MECH_TRACE_KERNEL(n, TK_BODY_HEAD);
    set_conditions(n, true, -1);
}

// ---------------------------------------------------------------------------
// filament energy: stretching + bending of the tile's own cylinders/triples
// ---------------------------------------------------------------------------
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_fil_energy(DevNet<Real> n, int want, int trial) {
    pdl_wait();      // the previous kernel of the main lane has finished
    MECH_TRACE_KERNEL(n, TK_FIL_ENERGY);
    __shared__ Pos<Real> xs[kFilTile + 4];
    __shared__ double sh[32 * MECH_NUM_FF];
    __shared__ int s_go, s_xb;
    __shared__ double s_lam;
    const Tile t = n.ftile[blockIdx.x];
    const int r = t.replica;
    if (threadIdx.x == 0) {
        const CGState& S = n.st[r];
        s_go = replica_selected(S, want);
        s_xb = S.xbuf;
        s_lam = S.lambda;
    }
    __syncthreads();
    if (s_go) {
        const int T = t.end - t.begin;
        const Real* X = n.x[s_xb];
        const bool tr = trial != 0;
        for (int i = threadIdx.x; i < T + 4; i += blockDim.x) {
            const int b = t.begin - 2 + i;
            if (b >= 0 && b < n.nb) xs[i] = bead_at(X, n.d, b, tr, s_lam);
        }
        __syncthreads();
        Real es = 0, eb = 0;
        const int i = threadIdx.x;
        if (i < T) {
            const int j = t.begin + i;
            const int fl = n.bflag[j];
            if (tr) store_pos(n.x[s_xb ^ 1], j, xs[i + 2]);   // materialize the owned trial position
            if (fl & 1) {
                Real ks, l0, kb, t0;
                load_par(n.bpar, j, ks, l0, kb, t0);
                Real r2[3];
                pdiff(xs[i + 3], xs[i + 2], r2);
                es = stretch_energy<Real>(r2[0], r2[1], r2[2], ks, l0);
                if (fl & 2) {
                    Real r1[3];
                    pdiff(xs[i + 2], xs[i + 1], r1);
                    eb = bend_energy<Real>(r1, r2, kb, t0);
                }
                if (n.terms) {
                    n.terms[j] = es;
                    n.terms[(size_t)n.nb + j] = eb;
                }
            }
        }
        double red[2] = {warp_sum_r(es), warp_sum_r(eb)};
        const int ops[2] = {0, 0};
        block_combine<2>(red, ops, sh);
        if (threadIdx.x == 0) {
            n.part_fil[4 * (size_t)blockIdx.x + 0] = red[0];
            n.part_fil[4 * (size_t)blockIdx.x + 1] = red[1];
        }
    }
}

// ---------------------------------------------------------------------------
// filament forces of the tile's own beads (the sparse force fields' shares are
// added by k_force_gather once they are written)
// ---------------------------------------------------------------------------
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_fil_force(DevNet<Real> n, int want) {
    pdl_wait();      // the previous kernel of the main lane has finished
    MECH_TRACE_KERNEL(n, TK_FIL_FORCE);
    __shared__ Pos<Real> xs[kFilTile + 4];
    __shared__ Real fs[(kFilTile + 2) * 3];    // stretch force on the second bead
    __shared__ Real f1[(kFilTile + 2) * 3];    // bending Fr1
    __shared__ Real f2[(kFilTile + 2) * 3];    // bending Fr2
    __shared__ int s_go, s_xb, s_fb;
    const Tile t = n.ftile[blockIdx.x];
    const int r = t.replica;
    if (threadIdx.x == 0) {
        const CGState& S = n.st[r];
        s_go = replica_selected(S, want);
        s_xb = S.xbuf;
        s_fb = S.fbuf;
    }
    __syncthreads();
    if (!s_go) return;
    const int T = t.end - t.begin;
    const Real* X = n.x[s_xb];
    for (int i = threadIdx.x; i < T + 4; i += blockDim.x) {
        const int b = t.begin - 2 + i;
        if (b >= 0 && b < n.nb) xs[i] = load_pos(X, b);
    }
    __syncthreads();
    // interaction slots s in [0, T + 2): bead j = begin - 1 + s, shared index s + 1
    for (int s = threadIdx.x; s < T + 2; s += blockDim.x) {
        const int j = t.begin - 1 + s;
        Real a[3] = {0, 0, 0}, b1[3] = {0, 0, 0}, b2[3] = {0, 0, 0};
        if (j >= 0 && j < n.nb) {
            const int fl = n.bflag[j];
            if (fl & 1) {
                Real ks, l0, kb, t0;
                load_par(n.bpar, j, ks, l0, kb, t0);
                Real r2[3];
                pdiff(xs[s + 2], xs[s + 1], r2);
                stretch_force<Real>(r2[0], r2[1], r2[2], ks, l0, a);
                if (fl & 2) {
                    Real r1[3];
                    pdiff(xs[s + 1], xs[s], r1);
                    bend_force<Real>(r1, r2, kb, t0, b1, b2);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            fs[3 * s + q] = a[q];
            f1[3 * s + q] = b1[q];
            f2[3 * s + q] = b2[q];
        }
    }
    __syncthreads();
    const int i = threadIdx.x;
    if (i < T) {
        const int b = t.begin + i;
        Real* Fo = n.f[s_fb ^ 1] + 3 * (size_t)b;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            // stretching: cylinder (b-1, b) then (b, b+1); bending: triples
            // centred on b-1, b, b+1 (the reference's interaction order)
            Real v = fs[3 * i + q];
            v += -fs[3 * (i + 1) + q];
            v += f2[3 * i + q];
            v += f1[3 * (i + 1) + q] - f2[3 * (i + 1) + q];
            v += -f1[3 * (i + 2) + q];
            Fo[q] = v;
        }
    }
}

// ---------------------------------------------------------------------------
// Every bead adds its sparse contributions (contiguous, in the CSR order) to
// its filament force, then the CG partials: max |F|, F.F, F.Fprev per tile,
// reduced by k_finalize_force (a per-tile completion ticket on one address
// per replica would serialize thousands of atomics).  FP64 engine: each block
// takes kGatherTiles consecutive tiles and issues the loads of all of them
// before the per-tile reductions, so a thread keeps several beads' loads in
// flight; the mixed engine's version is k_force_gather_mx below.
// ---------------------------------------------------------------------------

template <typename Real>
__device__ __forceinline__ void gather_bead(const DevNet<Real>& n, int b, int fb, Real& mx, Real& ff, Real& ffp) {
    Real* Fo = n.f[fb ^ 1] + 3 * (size_t)b;
    const Real* Fp = n.f[fb] + 3 * (size_t)b;
    Real F[3] = {Fo[0], Fo[1], Fo[2]};
    const int c0 = n.csr_off[b], c1 = n.csr_off[b + 1];
    for (int c = c0; c < c1; ++c) {
        F[0] += n.contrib[3 * (size_t)c];
        F[1] += n.contrib[3 * (size_t)c + 1];
        F[2] += n.contrib[3 * (size_t)c + 2];
    }
    Fo[0] = F[0];
    Fo[1] = F[1];
    Fo[2] = F[2];
    // a non-finite component makes the bead's max infinite (fmax would drop a NaN)
    const bool fin = F[0] - F[0] == 0 && F[1] - F[1] == 0 && F[2] - F[2] == 0;
    mx = fin ? fmax(fmax(fabs(F[0]), fabs(F[1])), fabs(F[2])) : Real(1.0 / 0.0);
    ff = bead_dot(F[0], F[1], F[2], F[0], F[1], F[2]);
    ffp = bead_dot(F[0], F[1], F[2], Fp[0], Fp[1], Fp[2]);
}

template <typename Real>
__global__ void __launch_bounds__(kBlock) k_force_gather(DevNet<Real> n, int want) {
    pdl_trigger();   // the next kernel of the main lane may be scheduled now
    MECH_TRACE_KERNEL(n, TK_GATHER);
    __shared__ double sh[32 * 3];
    __shared__ int s_go[kGatherTiles], s_fb[kGatherTiles];
    const int t0 = blockIdx.x * kGatherTiles;
    if (threadIdx.x < kGatherTiles) {
        const int ti = t0 + threadIdx.x;
        int go = 0, fb = 0;
        if (ti < n.n_ftiles) {
            const CGState& S = n.st[n.ftile[ti].replica];
            go = replica_selected(S, want);
            fb = S.fbuf;
        }
        s_go[threadIdx.x] = go;
        s_fb[threadIdx.x] = fb;
    }
    __syncthreads();
    Real mx[kGatherTiles], ff[kGatherTiles], ffp[kGatherTiles];
#pragma unroll
    for (int j = 0; j < kGatherTiles; ++j) {
        mx[j] = 0;
        ff[j] = 0;
        ffp[j] = 0;
        if (!s_go[j]) continue;
        const Tile t = n.ftile[t0 + j];
        const int b = t.begin + threadIdx.x;
        if (b < t.end) gather_bead(n, b, s_fb[j], mx[j], ff[j], ffp[j]);
    }
#pragma unroll
    for (int j = 0; j < kGatherTiles; ++j) {
        if (!s_go[j]) continue;   // block-uniform
        const size_t slot = 4 * (size_t)(t0 + j);
        double red[3] = {warp_max_r(mx[j]), warp_sum_r(ff[j]), warp_sum_r(ffp[j])};
        const int ops[3] = {1, 0, 0};
        block_combine<3>(red, ops, sh);
        if (threadIdx.x == 0) {
            n.part_fil[slot + 0] = red[0];
            n.part_fil[slot + 1] = red[1];
            n.part_fil[slot + 2] = red[2];
        }
    }
}

// Mixed engine gather: 64 threads per tile, each taking 4 consecutive beads
// whose force records (4 x 12 B) move as three 16-byte vectors, when the tile
// starts on a multiple of 4 beads (always, unless a replica before it has a
// bead count that is not; a partial group at the tile's end goes bead by
// bead); otherwise 4 beads strided by 64.  The block's partials combine, in
// warp order, the warps of each run of its tiles that belong to one replica,
// into the slot of the run's first tile (run_slot with stride kGatherTiles),
// so the force finalizer reads a quarter of the slots one per tile would take.
struct GatherMxShared {
    float sh[8][5];   // per warp: F.F (hi, lo), F.Fprev (hi, lo), max
    int go[kGatherTiles], fb[kGatherTiles], rep[kGatherTiles];
};

// One gather unit (kGatherTiles consecutive tiles): the body of a
// k_force_gather_mx block, also run unit after unit by k_tail_coop.
__device__ void gather_mx_unit(const DevNet<float>& n, int want, int unit, GatherMxShared& g) {
    static_assert(kFilTile == 256 && kBlock == 64 * kGatherTiles, "64 threads x 4 beads per tile");
    float (&sh)[8][5] = g.sh;
    int* s_go = g.go;
    int* s_fb = g.fb;
    int* s_rep = g.rep;
    const int t0 = unit * kGatherTiles;
    if (threadIdx.x < kGatherTiles) {
        const int ti = t0 + threadIdx.x;
        int go = 0, fb = 0, rep = -1;
        if (ti < n.n_ftiles) {
            rep = n.ftile[ti].replica;
            const CGState& S = n.st[rep];
            go = replica_selected(S, want);
            fb = S.fbuf;
        }
        s_go[threadIdx.x] = go;
        s_fb[threadIdx.x] = fb;
        s_rep[threadIdx.x] = rep;
    }
    __syncthreads();
    const int j = threadIdx.x >> 6, tt = threadIdx.x & 63;
    FF aff, affp;
    float mx = 0.f;
    if (s_go[j]) {   // uniform over the tile's two warps
        const Tile t = n.ftile[t0 + j];
        const int fb = s_fb[j];
        const int b0 = t.begin + 4 * tt;
        const bool vec_tile = (t.begin & 3) == 0;   // uniform over the tile
        if (vec_tile && b0 + 4 <= t.end) {
            float* Fo = n.f[fb ^ 1] + 3 * (size_t)b0;
            const float* Fp = n.f[fb] + 3 * (size_t)b0;
            const float4 u0 = reinterpret_cast<const float4*>(Fo)[0], u1 = reinterpret_cast<const float4*>(Fo)[1],
                         u2 = reinterpret_cast<const float4*>(Fo)[2];
            const float4 p0 = reinterpret_cast<const float4*>(Fp)[0], p1 = reinterpret_cast<const float4*>(Fp)[1],
                         p2 = reinterpret_cast<const float4*>(Fp)[2];
            float F[12] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w, u2.x, u2.y, u2.z, u2.w};
            const float P[12] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w, p2.x, p2.y, p2.z, p2.w};
            int off[5];
#pragma unroll
            for (int q = 0; q < 5; ++q) off[q] = n.csr_off[b0 + q];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                for (int c = off[k]; c < off[k + 1]; ++c) {
                    F[3 * k] += n.contrib[3 * (size_t)c];
                    F[3 * k + 1] += n.contrib[3 * (size_t)c + 1];
                    F[3 * k + 2] += n.contrib[3 * (size_t)c + 2];
                }
            reinterpret_cast<float4*>(Fo)[0] = make_float4(F[0], F[1], F[2], F[3]);
            reinterpret_cast<float4*>(Fo)[1] = make_float4(F[4], F[5], F[6], F[7]);
            reinterpret_cast<float4*>(Fo)[2] = make_float4(F[8], F[9], F[10], F[11]);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float* f = F + 3 * k;
                const bool fin = f[0] - f[0] == 0 && f[1] - f[1] == 0 && f[2] - f[2] == 0;
                mx = fmaxf(mx, fin ? fmaxf(fmaxf(fabsf(f[0]), fabsf(f[1])), fabsf(f[2])) : INFINITY);
                aff.add(bead_dot(f[0], f[1], f[2], f[0], f[1], f[2]));
                affp.add(bead_dot(f[0], f[1], f[2], P[3 * k], P[3 * k + 1], P[3 * k + 2]));
            }
        } else {
            // the partial group at the end of a vector tile, or a tile that
            // starts off the 4-bead grid: 4 beads strided by 64
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int b = vec_tile ? b0 + q : t.begin + tt + 64 * q;
                if (b < t.end) {
                    float m1, f1, f2;
                    gather_bead(n, b, fb, m1, f1, f2);
                    mx = fmaxf(mx, m1);
                    aff.add(f1);
                    affp.add(f2);
                }
            }
        }
    }
    warp_reduce_pair(aff.h, aff.l);
    warp_reduce_pair(affp.h, affp.l);
    mx = warp_max_f(mx);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        sh[w][0] = aff.h;
        sh[w][1] = aff.l;
        sh[w][2] = affp.h;
        sh[w][3] = affp.l;
        sh[w][4] = mx;
    }
    __syncthreads();
    const int j0 = threadIdx.x;
    if (j0 < kGatherTiles && s_go[j0] && (j0 == 0 || s_rep[j0 - 1] != s_rep[j0])) {
        // thread j0 starts a run: its tile and the following tiles of the same
        // replica, their warps' pairs added in order to compensated sums
        FF f1, f2;
        float m = 0.f;
        for (int j = j0; j < kGatherTiles && s_rep[j] == s_rep[j0]; ++j)
            for (int w = 2 * j; w < 2 * j + 2; ++w) {
                f1.add(sh[w][0]);
                f1.add(sh[w][1]);
                f2.add(sh[w][2]);
                f2.add(sh[w][3]);
                m = fmaxf(m, sh[w][4]);
            }
        float* p = reinterpret_cast<float*>(n.part_fil + 4 * (size_t)(t0 + j0));
        *reinterpret_cast<float4*>(p) = make_float4(m, f1.h, f1.l, f2.h);
        p[4] = f2.l;
    }
}

__global__ void __launch_bounds__(kBlock) k_force_gather_mx(DevNet<float> n, int want) {
    pdl_trigger();   // the next kernel of the main lane may be scheduled now
    MECH_TRACE_KERNEL(n, TK_GATHER_MX);
    __shared__ GatherMxShared g;
    gather_mx_unit(n, want, blockIdx.x, g);
}

// One block per replica: max |F|, the dots and the CG step logic after the gather.
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_finalize_force(DevNet<Real> n, int want) {
    pdl_wait();      // the previous kernel of the main lane has finished
    pdl_trigger();   // the next kernel of the main lane may be scheduled now
    MECH_TRACE_KERNEL(n, TK_FIN_FORCE);
    __shared__ double sh[32 * 3];
    __shared__ int s_flag;
    const int r = blockIdx.x;
    CGState S;
    if (threadIdx.x == 0) S = n.st[r];   // issued together with the loads below
    const RepTiles rt = n.rt[r];
    if (replica_selected(n.st[r], want)) finalize_force(n, r, rt, S, sh);
    after_evaluation(n, kCondForce, &s_flag);
}

// One block per replica: the energy reduction and the line-search step, after
// every kernel of the evaluation has written its partial sums.
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_finalize_energy(DevNet<Real> n, int want, int trial) {
    pdl_trigger();   // the next kernel of the main lane may be scheduled now
    MECH_TRACE_KERNEL(n, TK_FIN_ENERGY);
    __shared__ double sh[32 * 2 * MECH_NUM_FF];   // block_reduce_ff<12> of a two-trial pass: 32 * 24 floats
    __shared__ int s_flag;
    const int r = blockIdx.x;
    CGState S;
    if (threadIdx.x == 0) S = n.st[r];   // issued together with the loads below
    const RepTiles rt = n.rt[r];
    if (replica_selected(n.st[r], want)) finalize_energy(n, r, trial, rt, S, sh);
    after_evaluation(n, kCondTrial, &s_flag);
}

// ---------------------------------------------------------------------------
// Mixed engine: persistent, barrier-free filament kernels.  Each block walks
// `ptiles` consecutive tiles; every thread owns one bead per tile and
// recomputes in single precision the few neighbouring stretching and bending
// terms it needs (cheaper than staging through shared memory at the FP32
// rate), keeps compensated sums in registers across tiles, and the block
// reduces once per run of tiles of the same replica.
// ---------------------------------------------------------------------------


// Store a run's compensated partial sums as (hi, lo) pairs in the slot of its
// first tile; the reduction kernel that follows the evaluation reads them.
template <int N>
__device__ __forceinline__ void write_run(const DevNet<float>& n, int first, FF (&a)[N], double* sh) {
    block_reduce_ff<N, 0>(a, nullptr, reinterpret_cast<float*>(sh));
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) store_pair(n.part_fil + 4 * (size_t)first + k, a[k].h, a[k].l);
    }
}

__device__ __forceinline__ Pos<float> pos_at(const DevNet<float>& n, const float* X, int b, bool tr, float lf) {
    const Pos<float> p = load_pos(X, b);
    return tr ? moved_f(p, n.d, b, lf) : p;
}


// ---------------------------------------------------------------------------
// Mixed engine, bulk-staged filament energy: a persistent walk over runs of
// tiles with run-start partial slots (see write_run), where each selected
// tile's positions (with a one-bead halo),
// constants, flags and (for a trial) search direction arrive in shared memory
// by cp.async.bulk on a three-stage mbarrier ring, so a block keeps several
// ~14 KB transfers in flight instead of per-thread dependent loads.  Ranges
// are rounded outward to the 16-byte copy granularity; the bead arrays are
// allocated with the padding that rounding needs.
// ---------------------------------------------------------------------------
constexpr int kBulkStages = 3;
constexpr int kBulkXBeads = kFilTile + 4;    // tile + 1-bead halo, even-aligned ends
constexpr int kBulkDBeads = kFilTile + 8;    // tile + halo, 4-bead aligned ends
constexpr int kBulkFlags = kFilTile + 32;    // tile + halo, 16-byte aligned ends
constexpr int kBulkWaitLimit = 1 << 22;      // mbarrier polls before a stage counts as lost

struct __align__(16) EnergyStage {
    float x[6 * kBulkXBeads];      // float-float positions, beads [xs, xe)
    float4 par[kFilTile];          // k_str, l0, k_bend, theta0, beads [tb, te)
    float d[3 * kBulkDBeads];      // search direction, beads [ds, de)
    uint8_t flag[kBulkFlags];      // bead flags, beads [fs, fe)
};

struct StageRange {
    int xs, xe, ds, de, fs, fe;
};
// Staged ranges of tile [tb, te) with `halo` beads each side, clamped to the
// network and rounded outward: positions to even beads (24 B each), the
// direction to multiples of 4 beads (12 B), flags to 16 beads (1 B).
__device__ __forceinline__ StageRange stage_range(int tb, int te, int nb, int halo) {
    StageRange r;
    const int lo = max(tb - halo, 0), hi = min(te + halo, nb);
    r.xs = lo & ~1;
    r.xe = (hi + 1) & ~1;
    r.ds = lo & ~3;
    r.de = (hi + 3) & ~3;
    r.fs = lo & ~15;
    r.fe = (hi + 15) & ~15;
    return r;
}

// A block's tile descriptors, read once at kernel start (one thread per tile)
// so the producing thread issues copies without chasing global pointers:
// (begin, end, replica, bits) with bit 0 = selected by this launch, bits 1-2 =
// xbuf, bit 3 = fbuf of the tile's replica, plus that replica's lambda.  A
// replica's state cannot change while this block still holds unprocessed
// tiles of it (its finalizer waits for every tile), so the copies stay valid.
constexpr int kBulkMaxTiles = kFilBulkMaxTiles;

__device__ __forceinline__ void load_descriptors(const DevNet<float>& n, int t0, int nt, int want, int4* desc,
                                                 float* lf) {
    for (int k = threadIdx.x; k < nt; k += blockDim.x) {
        const Tile t = n.ftile[t0 + k];
        const CGState& S = n.st[t.replica];
        desc[k] = make_int4(t.begin, t.end, t.replica,
                            (replica_selected(S, want) ? 1 : 0) | (S.xbuf << 1) | (S.fbuf << 3));
        lf[k] = (float)S.lambda;
    }
}

// Issue the copies of a tile into stage `st` (thread 0).  A range that fails
// the alignment check is not copied: the barrier is completed without it and
// the error word records it.
__device__ void issue_energy_stage(const DevNet<float>& n, int4 t, bool tr, EnergyStage* st, uint64_t* bar) {
    const float* X = n.x[(t.w >> 1) & 3];
    const StageRange rg = stage_range(t.x, t.y, n.nb, 1);
    const void* src[4] = {X + 6 * (size_t)rg.xs, n.bpar + 4 * (size_t)t.x, n.d + 3 * (size_t)rg.ds, n.bflag + rg.fs};
    void* dst[4] = {st->x, st->par, st->d, st->flag};
    const unsigned bytes[4] = {24u * (unsigned)(rg.xe - rg.xs), 16u * (unsigned)(t.y - t.x),
                               tr ? 12u * (unsigned)(rg.de - rg.ds) : 0u, (unsigned)(rg.fe - rg.fs)};
    unsigned total = 0;
    bool ok = true;
    for (int k = 0; k < 4; ++k) {
        if (!bytes[k]) continue;
        if (!aligned16(src[k], bytes[k]) || !aligned16(dst[k], bytes[k])) ok = false;
        total += bytes[k];
    }
    fence_proxy_async_smem();
    if (!ok) {
        atomicOr(n.err, 16u);
        mbar_arrive_expect_tx(bar, 0);
        return;
    }
    mbar_arrive_expect_tx(bar, total);
    for (int k = 0; k < 4; ++k)
        if (bytes[k]) bulk_copy_g2s(dst[k], src[k], bytes[k], bar);
}

// True in every thread when a launch selects no replica of the block's tile
// range [t0, t1): tiles are ordered by replica, so a range whose first and
// last tiles share a replica belongs to it alone.  The block then exits before
// any barrier or descriptor setup.
__device__ __forceinline__ bool idle_range(const DevNet<float>& n, int t0, int t1, int want, int* s_flag) {
    if (threadIdx.x == 0) {
        int idle = t1 <= t0;
        if (!idle) {
            const int ra = n.ftile[t0].replica, rb = n.ftile[t1 - 1].replica;
            idle = ra == rb && !replica_selected(n.st[ra], want);
        }
        *s_flag = idle;
    }
    __syncthreads();
    return *s_flag != 0;
}

__global__ void __launch_bounds__(kBlock, 4) k_fil_energy_bulk(DevNet<float> n, int want, int trial) {
    pdl_wait();      // the previous kernel of the main lane has finished
    MECH_TRACE_KERNEL(n, TK_FIL_ENERGY_BULK);
    __shared__ EnergyStage stage[kBulkStages];
    __shared__ __align__(8) uint64_t bar[kBulkStages];
    __shared__ int4 s_desc[kBulkMaxTiles];
    __shared__ float s_lf[kBulkMaxTiles];
    __shared__ double sh[32 * 4];   // write_run<4>: 32 * 8 floats
    __shared__ __align__(16) float s_mv[6 * kBulkXBeads];   // the staged beads moved to a trial
    __shared__ int s_abort;
    const int t0 = blockIdx.x * n.ptiles[0], t1 = min(t0 + n.ptiles[0], n.n_ftiles);
    const int nt = t1 - t0;
    const bool tr = trial != 0;
    if (idle_range(n, t0, t1, want, &s_abort)) return;
    if (threadIdx.x == 0) {
        for (int k = 0; k < kBulkStages; ++k) mbar_init(&bar[k], 1);
        mbar_init_fence();
        s_abort = 0;
    }
    if (nt > kBulkMaxTiles) {   // the launch geometry caps tiles per block; refuse rather than overrun
        if (threadIdx.x == 0) atomicOr(n.err, 16u);
        return;
    }
    load_descriptors(n, t0, nt, want, s_desc, s_lf);
    __syncthreads();
    // producer state (thread 0): next tile to consider, copies issued
    int pi = 0, issued = 0;
    if (threadIdx.x == 0) {
        for (; pi < nt && issued < kBulkStages; ++pi)
            if (s_desc[pi].w & 1) {
                issue_energy_stage(n, s_desc[pi], tr, &stage[issued % kBulkStages], &bar[issued % kBulkStages]);
                ++issued;
            }
    }
    // a two-trial pass (trial == kTrialDual): energies at lambda into slots 0, 1
    // of the run and at lambda / 2 into slots 2, 3; trial positions into the
    // two buffers after the current one
    const bool dual = trial == kTrialDual;
    int cur = -1, first = 0, cnt = 0, xb = 0, j = 0;
    bool go = false;
    float lf = 0.f;
    FF es, eb, es2, eb2;
    auto flush = [&]() {
        if (dual) {
            FF a[4] = {es, eb, es2, eb2};
            write_run<4>(n, first, a, sh);
        } else {
            FF a[2] = {es, eb};
            write_run<2>(n, first, a, sh);
        }
    };
    for (int k = 0; k < nt; ++k) {
        const int4 t = s_desc[k];
        if (t.z != cur) {
            if (cnt) flush();
            cur = t.z;
            first = t0 + k;
            cnt = 0;
            es = FF();
            eb = FF();
            es2 = FF();
            eb2 = FF();
            go = t.w & 1;
            xb = (t.w >> 1) & 3;
            lf = s_lf[k];
        }
        if (!go) continue;
        ++cnt;
        const int sidx = j % kBulkStages;
        if (!mbar_wait_bounded(&bar[sidx], (unsigned)((j / kBulkStages) & 1), kBulkWaitLimit)) {
            atomicOr(n.err, 32u);
            s_abort = 1;
        }
        const EnergyStage& S = stage[sidx];
        const int b = t.x + threadIdx.x;
        const StageRange rg = stage_range(t.x, t.y, n.nb, 1);
        const bool own = b < t.y;
        int fl = 0;
        float4 pr = make_float4(0.f, 0.f, 0.f, 0.f);
        if (own) {
            fl = S.flag[b - rg.fs];
            pr = S.par[b - t.x];
        }
        // one trial per pass of this loop (two in a two-trial pass: lambda,
        // then lambda / 2, exact in float).  For a trial the block first moves
        // every staged bead once (tile and halo) into shared memory, so each
        // bead's neighbours are read, not moved again by every thread that
        // needs them; a plain evaluation reads the staged positions directly.
#pragma unroll 1
        for (int ch = 0; ch < (dual ? 2 : 1); ++ch) {
            const float* P = S.x;
            if (tr) {
                const float lch = ch ? 0.5f * lf : lf;
                for (int q = threadIdx.x; q < rg.xe - rg.xs; q += blockDim.x)
                    store_pos(s_mv, q, moved_f(load_pos(S.x, q), S.d, q + rg.xs - rg.ds, lch));
                __syncthreads();
                P = s_mv;
            }
            if (own) {
                const Pos<float> p0 = load_pos(P, b - rg.xs);
                if (tr) store_pos(n.x[(xb + 1 + ch) % 3], b, p0);   // materialize the owned trial position
                if (fl & 1) {
                    const Pos<float> pp = load_pos(P, b + 1 - rg.xs);
                    float r2[3];
                    pdiff(pp, p0, r2);
                    const float ts = stretch_energy<float>(r2[0], r2[1], r2[2], pr.x, pr.y);
                    if (ch) es2.add(ts);
                    else es.add(ts);
                    float tb = 0.f;
                    if (fl & 2) {
                        const Pos<float> pm = load_pos(P, b - 1 - rg.xs);
                        float r1[3];
                        pdiff(p0, pm, r1);
                        tb = bend_energy<float>(r1, r2, pr.z, pr.w);
                        if (ch) eb2.add(tb);
                        else eb.add(tb);
                    }
                    if (n.terms && !ch) {
                        n.terms[b] = ts;
                        n.terms[(size_t)n.nb + b] = tb;
                    }
                }
            }
            if (tr) __syncthreads();   // s_mv is refilled by the next trial or tile
        }
        ++j;
        __syncthreads();   // stage sidx fully read
        if (s_abort) break;
        if (threadIdx.x == 0) {
            for (; pi < nt; ++pi)
                if (s_desc[pi].w & 1) {
                    issue_energy_stage(n, s_desc[pi], tr, &stage[issued % kBulkStages], &bar[issued % kBulkStages]);
                    ++issued;
                    ++pi;
                    break;
                }
        }
    }
    if (s_abort) {
        // drain: copies still in flight must land before the block's shared memory is released
        if (threadIdx.x == 0)
            for (int q = max(j - 1, 0); q < issued; ++q)
                mbar_wait_bounded(&bar[q % kBulkStages], (unsigned)((q / kBulkStages) & 1), kBulkWaitLimit);
        return;
    }
    if (cnt) flush();
}


// ---------------------------------------------------------------------------
// Mixed engine, bulk-staged filament forces: the same walk, with each
// selected tile's positions (two-bead halo), constants and flags of
// the neighbouring beads, previous forces and CSR offsets staged by
// cp.async.bulk like k_fil_energy_bulk; the bead's gathered contributions are
// contiguous in memory and read directly.
// ---------------------------------------------------------------------------
constexpr int kBulkFXBeads = kFilTile + 8;    // tile + 2-bead halo, even-aligned ends
constexpr int kBulkFPar = kFilTile + 4;       // constants of beads tb - 1 .. te

struct __align__(16) ForceStage {
    float x[6 * kBulkFXBeads];
    float4 par[kBulkFPar];
    uint8_t flag[kBulkFlags];
};

struct ForceRange {
    int xs, xe, ps, pe, fs, fe;
};
__device__ __forceinline__ ForceRange force_range(int tb, int te, int nb) {
    ForceRange r;
    const int lo2 = max(tb - 2, 0), hi2 = min(te + 2, nb);
    r.xs = lo2 & ~1;
    r.xe = (hi2 + 1) & ~1;
    r.ps = max(tb - 1, 0);
    r.pe = min(te + 1, nb);
    r.fs = lo2 & ~15;
    r.fe = (hi2 + 15) & ~15;
    return r;
}

__device__ void issue_force_stage(const DevNet<float>& n, int4 t, ForceStage* st, uint64_t* bar) {
    const float* X = n.x[(t.w >> 1) & 3];
    const ForceRange rg = force_range(t.x, t.y, n.nb);
    const void* src[3] = {X + 6 * (size_t)rg.xs, n.bpar + 4 * (size_t)rg.ps, n.bflag + rg.fs};
    void* dst[3] = {st->x, st->par, st->flag};
    const unsigned bytes[3] = {24u * (unsigned)(rg.xe - rg.xs), 16u * (unsigned)(rg.pe - rg.ps),
                               (unsigned)(rg.fe - rg.fs)};
    unsigned total = 0;
    bool ok = true;
    for (int k = 0; k < 3; ++k) {
        if (!bytes[k]) continue;
        if (!aligned16(src[k], bytes[k]) || !aligned16(dst[k], bytes[k])) ok = false;
        total += bytes[k];
    }
    fence_proxy_async_smem();
    if (!ok) {
        atomicOr(n.err, 16u);
        mbar_arrive_expect_tx(bar, 0);
        return;
    }
    mbar_arrive_expect_tx(bar, total);
    for (int k = 0; k < 3; ++k)
        if (bytes[k]) bulk_copy_g2s(dst[k], src[k], bytes[k], bar);
}

// Mixed engine, bulk-staged filament forces: each selected tile's positions
// (two-bead halo), the constants and flags of its beads and their neighbours
// arrive by cp.async.bulk like k_fil_energy_bulk; every bead's filament force
// is written to the force buffer, where k_force_gather adds the bead's sparse
// contributions and forms the CG partials.
__global__ void __launch_bounds__(kBlock) k_fil_force_bulk(DevNet<float> n, int want) {
    pdl_wait();      // the previous kernel of the main lane has finished
    MECH_TRACE_KERNEL(n, TK_FIL_FORCE_BULK);
    __shared__ ForceStage stage[kBulkStages];
    __shared__ __align__(8) uint64_t bar[kBulkStages];
    __shared__ int4 s_desc[kBulkMaxTiles];
    __shared__ float s_lf[kBulkMaxTiles];
    __shared__ int s_abort;
    // per tile: stretching force of each cylinder (q, q + 1) and the two bending
    // terms of each triple centred on q, for q = tile begin - 1 .. tile end
    __shared__ float s_st[kFilTile + 2][3], s_a1[kFilTile + 2][3], s_a2[kFilTile + 2][3];
    const int t0 = blockIdx.x * n.ptiles[1], t1 = min(t0 + n.ptiles[1], n.n_ftiles);
    const int nt = t1 - t0;
    if (idle_range(n, t0, t1, want, &s_abort)) return;
    if (threadIdx.x == 0) {
        for (int k = 0; k < kBulkStages; ++k) mbar_init(&bar[k], 1);
        mbar_init_fence();
        s_abort = 0;
    }
    if (nt > kBulkMaxTiles) {   // the launch geometry caps tiles per block; refuse rather than overrun
        if (threadIdx.x == 0) atomicOr(n.err, 16u);
        return;
    }
    load_descriptors(n, t0, nt, want, s_desc, s_lf);
    __syncthreads();
    int pi = 0, issued = 0;
    if (threadIdx.x == 0) {
        for (; pi < nt && issued < kBulkStages; ++pi)
            if (s_desc[pi].w & 1) {
                issue_force_stage(n, s_desc[pi], &stage[issued % kBulkStages], &bar[issued % kBulkStages]);
                ++issued;
            }
    }
    int j = 0;
    for (int k = 0; k < nt; ++k) {
        const int4 t = s_desc[k];
        if (!(t.w & 1)) continue;
        const int fb = (t.w >> 3) & 1;
        const int sidx = j % kBulkStages;
        if (!mbar_wait_bounded(&bar[sidx], (unsigned)((j / kBulkStages) & 1), kBulkWaitLimit)) {
            atomicOr(n.err, 32u);
            s_abort = 1;
        }
        const ForceStage& S = stage[sidx];
        const ForceRange rg = force_range(t.x, t.y, n.nb);
        // every stretching and bending term touching the tile, once: term slot i
        // belongs to bead q = t.x - 1 + i (the cylinder (q, q + 1) and the triple
        // centred on q), for the tile and one halo bead on each side
        for (int i = threadIdx.x; i < t.y - t.x + 2; i += blockDim.x) {
            const int q = t.x - 1 + i;
            if (q < 0 || q >= n.nb) continue;
            const int fq = S.flag[q - rg.fs];
            if (!(fq & 1)) continue;
            const Pos<float> c0 = load_pos(S.x, q - rg.xs), c1 = load_pos(S.x, q + 1 - rg.xs);
            const float4 pq = S.par[q - rg.ps];
            float rp[3], st[3];
            pdiff(c1, c0, rp);
            stretch_force<float>(rp[0], rp[1], rp[2], pq.x, pq.y, st);
            s_st[i][0] = st[0]; s_st[i][1] = st[1]; s_st[i][2] = st[2];
            if (fq & 2) {
                const Pos<float> cm = load_pos(S.x, q - 1 - rg.xs);
                float rm[3], a1[3], a2[3];
                pdiff(c0, cm, rm);
                bend_force<float>(rm, rp, pq.z, pq.w, a1, a2);
                s_a1[i][0] = a1[0]; s_a1[i][1] = a1[1]; s_a1[i][2] = a1[2];
                s_a2[i][0] = a2[0]; s_a2[i][1] = a2[1]; s_a2[i][2] = a2[2];
            }
        }
        __syncthreads();
        const int b = t.x + threadIdx.x;
        if (b < t.y) {
            const int f0 = S.flag[b - rg.fs];
            const int fm = (f0 & 2) ? S.flag[b - 1 - rg.fs] : 0;
            const int fp = (f0 & 1) ? S.flag[b + 1 - rg.fs] : 0;
            const int i = threadIdx.x + 1;   // this bead's term slot
            // stretching: cylinder (b-1, b) then (b, b+1); bending: triples centred on b-1, b, b+1
            float F[3] = {0.f, 0.f, 0.f};
            if (f0 & 2) { F[0] += s_st[i - 1][0]; F[1] += s_st[i - 1][1]; F[2] += s_st[i - 1][2]; }
            if (f0 & 1) { F[0] += -s_st[i][0]; F[1] += -s_st[i][1]; F[2] += -s_st[i][2]; }
            if ((f0 & 2) && (fm & 2)) { F[0] += s_a2[i - 1][0]; F[1] += s_a2[i - 1][1]; F[2] += s_a2[i - 1][2]; }
            if ((f0 & 3) == 3) {
                F[0] += s_a1[i][0] - s_a2[i][0];
                F[1] += s_a1[i][1] - s_a2[i][1];
                F[2] += s_a1[i][2] - s_a2[i][2];
            }
            if ((f0 & 1) && (fp & 1)) { F[0] += -s_a1[i + 1][0]; F[1] += -s_a1[i + 1][1]; F[2] += -s_a1[i + 1][2]; }
            float* Fo = n.f[fb ^ 1] + 3 * (size_t)b;
            Fo[0] = F[0];
            Fo[1] = F[1];
            Fo[2] = F[2];
        }
        ++j;
        __syncthreads();   // stage sidx fully read
        if (s_abort) break;
        if (threadIdx.x == 0) {
            for (; pi < nt; ++pi)
                if (s_desc[pi].w & 1) {
                    issue_force_stage(n, s_desc[pi], &stage[issued % kBulkStages], &bar[issued % kBulkStages]);
                    ++issued;
                    ++pi;
                    break;
                }
        }
    }
    if (s_abort && threadIdx.x == 0)   // drain copies still in flight before shared memory is released
        for (int q = max(j - 1, 0); q < issued; ++q)
            mbar_wait_bounded(&bar[q % kBulkStages], (unsigned)((q / kBulkStages) & 1), kBulkWaitLimit);
}

// What the direction update needs of a replica's state.
struct DirState {
    int go, fb, xb, bk;
    float beta;
};

// One direction unit (n.ptiles[2] consecutive tiles): the body of a
// k_direction_mx block, also run unit after unit by k_tail_coop, which passes
// the state its blocks hold instead of the one in memory.
template <typename StateOf>
__device__ void direction_mx_unit(const DevNet<float>& n, int unit, double* sh, StateOf state_of) {
    const int t0 = unit * n.ptiles[2], t1 = min(t0 + n.ptiles[2], n.n_ftiles);
    int cur = -1, first = 0, cnt = 0, fb = 0, xb = 0, bk = 0;
    bool go = false;
    float beta = 0.f;
    FF dF;
    // the run's partial goes to slot 3 of its first tile, as a (hi, lo) pair
    auto finish = [&](int) {
        FF a[1] = {dF};
        block_reduce_ff<1, 0>(a, nullptr, reinterpret_cast<float*>(sh));
        if (threadIdx.x == 0) store_pair(n.part_fil + 4 * (size_t)first + 3, a[0].h, a[0].l);
    };
    for (int ti = t0; ti < t1; ++ti) {
        const Tile t = n.ftile[ti];
        if (t.replica != cur) {
            if (cnt) finish(cur);
            cur = t.replica;
            first = ti;
            cnt = 0;
            dF = FF();
            const DirState ds = state_of(cur);
            go = ds.go;
            fb = ds.fb;
            xb = ds.xb;
            bk = ds.bk;
            beta = ds.beta;
        }
        if (!go) continue;
        ++cnt;
        const int b = t.begin + threadIdx.x;
        if (b < t.end) {
            const float* F = n.f[fb] + 3 * (size_t)b;
            float* D = n.d + 3 * (size_t)b;
            const float d0 = F[0] + beta * D[0], d1 = F[1] + beta * D[1], d2 = F[2] + beta * D[2];
            D[0] = d0;
            D[1] = d1;
            D[2] = d2;
            dF.add(bead_dot(d0, d1, d2, F[0], F[1], F[2]));
            if (bk) store_pos(n.xbest, b, load_pos(n.x[xb], b));
        }
    }
    if (cnt) finish(cur);
}

// Mixed engine: persistent direction update d = F + beta d with the d.F partials.
__global__ void __launch_bounds__(kBlock) k_direction_mx(DevNet<float> n) {
    pdl_wait();      // the previous kernel of the main lane has finished
    pdl_trigger();   // the next kernel of the main lane may be scheduled now
    MECH_TRACE_KERNEL(n, TK_DIRECTION_MX);
    __shared__ double sh[32];
    direction_mx_unit(n, blockIdx.x, sh, [&](int r) {
        const CGState& S = n.st[r];
        return DirState{S.phase == PH_DIR, S.fbuf, S.xbuf, S.backupPending, (float)S.beta};
    });
}

// ---------------------------------------------------------------------------
// Mixed engine, one replica: the tail of an iteration after the force lanes
// as one cooperatively launched grid (every block resident at once): the
// force gather, the force finalizer, the direction update, the direction
// finalizer and the reset, with grid barriers where the separate launches
// had a launch boundary.  The finalizers' reductions run in every block over
// the same partial slots in the same order, so every block holds the same new
// state, and block 0 stores it.  Work units, partial slots and reduction
// order are those of k_force_gather_mx, k_finalize_force, k_direction_mx,
// k_finalize_direction and k_reset, so the minimization is bitwise the one
// the separate launches give.
// ---------------------------------------------------------------------------
constexpr unsigned kGridWaitLimit = 1u << 22;   // polls before a grid barrier counts as lost

// Barrier over the blocks of a co-resident grid: gbar[0] counts arrivals,
// gbar[1] is the generation that the last arrival advances.  A wait gives up
// after kGridWaitLimit polls, sets error bit 64 and returns false in every
// thread of its block.
__device__ bool grid_sync(unsigned* gbar, unsigned* err) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = gbar + 1;
        const unsigned g0 = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(gbar, 1u);
        int ok = 1;
        if (arrived == gridDim.x - 1) {
            atomicExch(gbar, 0u);
            __threadfence();
            atomicAdd(gbar + 1, 1u);
        } else {
            unsigned polls = 0;
            while (*gen == g0) {
                if (++polls > kGridWaitLimit) {
                    atomicOr(err, 64u);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__global__ void __launch_bounds__(kBlock) k_tail_coop(DevNet<float> n) {
    MECH_TRACE_KERNEL(n, TK_TAIL_COOP);
    __shared__ GatherMxShared g;
    __shared__ double sh[32 * 3];
    __shared__ int s_phase, s_fb, s_xb, s_bk;
    __shared__ float s_beta;
    __shared__ CGState S;   // the block's copy of the replica's state (thread 0 works on it)
    if (threadIdx.x == 0) {
        S = n.st[0];
        s_phase = S.phase;
        s_fb = S.fbuf;
        if (blockIdx.x == 0) {   // as after every force evaluation: the exvol work lists restart empty
            if (n.ev_list_count) *n.ev_list_count = 0;
            if (n.ev_fb_count) *n.ev_fb_count = 0;
        }
    }
    __syncthreads();
    const int start = s_phase;
    if (start != PH_FORCE && start != PH_RESET) return;   // the same decision in every block
    const RepTiles rt = n.rt[0];
    int phase = start;
    if (phase == PH_FORCE) {
        const int units = (n.n_ftiles + kGatherTiles - 1) / kGatherTiles;
        for (int u = blockIdx.x; u < units; u += gridDim.x) {
            gather_mx_unit(n, PH_FORCE, u, g);
            __syncthreads();
        }
        if (!grid_sync(n.gbar, n.err)) return;
        finalize_force(n, 0, rt, S, sh, false);
        if (threadIdx.x == 0) {
            s_phase = S.phase;
            s_fb = S.fbuf;
            s_xb = S.xbuf;
            s_bk = S.backupPending;
            s_beta = (float)S.beta;
        }
        __syncthreads();
        phase = s_phase;
        if (phase == PH_DIR) {
            const DirState ds{1, s_fb, s_xb, s_bk, s_beta};
            for (int u = blockIdx.x; u < n.pgrid[2]; u += gridDim.x) {
                direction_mx_unit(n, u, sh, [&](int) { return ds; });
                __syncthreads();
            }
            if (!grid_sync(n.gbar, n.err)) return;
            finalize_direction(n, 0, rt, S, sh, false);
            if (threadIdx.x == 0) {
                s_phase = S.phase;
                s_fb = S.fbuf;
            }
            __syncthreads();
            phase = s_phase;
        }
    }
    if (phase == PH_RESET) {   // d = F, then the new slope and the next iteration's start
        const float* F = n.f[s_fb];
        const size_t nv = 3 * (size_t)n.nb;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x)
            n.d[i] = F[i];
        if (threadIdx.x == 0) {
            S.slope = S.FdotF;
            S.lastFdotF = S.FdotF;
            begin_iteration(S);
        }
        // every block has read the state before block 0 replaces it (on the
        // force path the barriers above already ensure that)
        if (start == PH_RESET && !grid_sync(n.gbar, n.err)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) n.st[0] = S;
}

int coop_tail_grid(int device) {
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tail_coop, kBlock, 0) != cudaSuccess) return 0;
    return sms * per_sm;
}

static void launch_tail_coop(const DevNet<float>& n, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_tail_coop, n);
}

// ---------------------------------------------------------------------------
// linker, motor and boundary interactions (energy or force contributions)
// ---------------------------------------------------------------------------
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_bond_bnd(DevNet<Real> n, int want, int trial, int force, int n_lm_tiles,
                                                     int ev_tiles) {
    MECH_TRACE_KERNEL(n, TK_BOND);
    __shared__ double sh[64];   // block_reduce_ff<2>: 32 * 4 floats
    __shared__ int s_go, s_xb;
    __shared__ double s_lam;
    __shared__ float s_lf;   // the step rounded once (mixed engine)
    const int ti = blockIdx.x < n_lm_tiles ? blockIdx.x : blockIdx.x + ev_tiles;
    const Tile t = n.stile[ti];
    const int kind = n.stile_kind[ti];
    const int r = t.replica;
    if (threadIdx.x == 0) {
        const CGState& S = n.st[r];
        s_go = replica_selected(S, want);
        s_xb = S.xbuf;
        s_lam = S.lambda;
        s_lf = (float)S.lambda;
    }
    __syncthreads();
    if (!s_go) return;
    const Real* X = n.x[s_xb];
    const bool tr = trial != 0;
    // a two-trial pass also evaluates the energy at lambda / 2 (mixed engine)
    const bool dual = sizeof(Real) == 4 && trial == kTrialDual && !force;
    auto pos_at = [&](int b, float lfs) -> Pos<Real> {
        if constexpr (sizeof(Real) == 4) {
            const Pos<float> p = load_pos(X, b);
            return tr ? moved_f(p, n.d, b, lfs) : p;
        } else {
            return bead_at(X, n.d, b, tr, s_lam);
        }
    };
    auto pos = [&](int b) -> Pos<Real> { return pos_at(b, s_lf); };
    const int i = t.begin + threadIdx.x;
    Real e = 0, e2 = 0;
    if (i < t.end) {
        if (kind == K_BOUNDARY) {
            const int b = n.bb_bead[i];
            const double* pl = n.planes + 4 * n.bb_plane[i];
            const Pos<Real> p = pos(b);
            const Real rr = plane_dist_p(pl, p);
            const Real K = n.bb_k[i], sl = n.bb_slen[i];
            const Real R = -rr / sl;
            const Real ex = exp(R);
            if (!force) {
                e = K * ex;
                if (dual) {
                    const Real rr2 = plane_dist_p(pl, pos_at(b, 0.5f * s_lf));
                    e2 = K * exp(-rr2 / sl);
                }
            } else {
                const Real f0 = K * ex / sl;
                Real* c = slot_ptr(n, n.slot_base[K_BOUNDARY] + i);
                c[0] = f0 * (Real)pl[0];
                c[1] = f0 * (Real)pl[1];
                c[2] = f0 * (Real)pl[2];
            }
        } else {
            const bool lk = kind == K_LINKER;
            const int4 bs = lk ? n.lk_bead[i] : n.mt_bead[i];
            const Real k = lk ? n.lk_k[i] : n.mt_k[i];
            const Real l0 = lk ? n.lk_l0[i] : n.mt_l0[i];
            const Real s1 = lk ? n.lk_s1[i] : n.mt_s1[i];
            const Real s2 = lk ? n.lk_s2[i] : n.mt_s2[i];
            const Pos<Real> c1 = pos(bs.x), c2 = pos(bs.y), c3 = pos(bs.z), c4 = pos(bs.w);
            Real v[3];
            bond_vector(c1, c2, c3, c4, s1, s2, v);
            const Real lx = v[0], ly = v[1], lz = v[2];
            const Real dist = sqrt(lx * lx + ly * ly + lz * lz);
            if (!force) {
                const Real dd = dist - l0;
                e = (Real)0.5 * k * dd * dd;
                if (dual) {
                    const float lh = 0.5f * s_lf;
                    Real w[3];
                    bond_vector(pos_at(bs.x, lh), pos_at(bs.y, lh), pos_at(bs.z, lh), pos_at(bs.w, lh), s1, s2, w);
                    const Real d2 = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]) - l0;
                    e2 = (Real)0.5 * k * d2 * d2;
                }
            } else {
                const Real invL = (Real)1 / dist;
                const Real f0 = k * (dist - l0) * invL;
                const Real Fl[3] = {-f0 * lx, -f0 * ly, -f0 * lz};
                const int sb = n.slot_base[kind] + 4 * i;
                Real* ca = slot_ptr(n, sb);
                Real* cb = slot_ptr(n, sb + 1);
                Real* cc = slot_ptr(n, sb + 2);
                Real* cd = slot_ptr(n, sb + 3);
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    ca[q] = -Fl[q] * ((Real)1 - s1);
                    cb[q] = -Fl[q] * (s1);
                    cc[q] = Fl[q] * ((Real)1 - s2);
                    cd[q] = Fl[q] * (s2);
                }
                (lk ? n.lk_sf : n.mt_sf)[i] = (double)(f0 / invL);
            }
        }
    }
    if (!force) {
        if constexpr (sizeof(Real) == 4) {
            if (dual) {
                FF a[2];
                a[0].h = e;
                a[1].h = e2;
                block_reduce_ff<2, 0>(a, nullptr, reinterpret_cast<float*>(sh));
                if (threadIdx.x == 0) {
                    store_pair(n.part_sp + ti, a[0].h, a[0].l);
                    store_pair(n.part_sp2 + ti, a[1].h, a[1].l);
                }
            } else {
                FF a[1];
                a[0].h = e;
                block_reduce_ff<1, 0>(a, nullptr, reinterpret_cast<float*>(sh));
                if (threadIdx.x == 0) store_pair(n.part_sp + ti, a[0].h, a[0].l);
            }
        } else {
            const double se = block_sum_r(e, sh);
            if (threadIdx.x == 0) n.part_sp[ti] = se;
        }
    }
}

// ---------------------------------------------------------------------------
// direction update d = F + beta d, conjugacy check, backup copy
// ---------------------------------------------------------------------------
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_direction(DevNet<Real> n) {
    pdl_wait();      // the previous kernel of the main lane has finished
    pdl_trigger();   // the next kernel of the main lane may be scheduled now
    MECH_TRACE_KERNEL(n, TK_DIRECTION);
    __shared__ double sh[32];
    __shared__ int s_go, s_fb, s_xb, s_bk;
    __shared__ double s_beta;
    const Tile t = n.ftile[blockIdx.x];
    const int r = t.replica;
    if (threadIdx.x == 0) {
        const CGState& S = n.st[r];
        s_go = S.phase == PH_DIR;
        s_fb = S.fbuf;
        s_xb = S.xbuf;
        s_bk = S.backupPending;
        s_beta = S.beta;
    }
    __syncthreads();
    if (!s_go) return;
    const int b = t.begin + threadIdx.x;
    Real dF = 0;
    if (b < t.end) {
        const Real* F = n.f[s_fb] + 3 * (size_t)b;
        Real* D = n.d + 3 * (size_t)b;
        const Real beta = (Real)s_beta;
        const Real d0 = F[0] + beta * D[0], d1 = F[1] + beta * D[1], d2 = F[2] + beta * D[2];
        D[0] = d0;
        D[1] = d1;
        D[2] = d2;
        dF = bead_dot(d0, d1, d2, F[0], F[1], F[2]);
        if (s_bk) store_pos(n.xbest, b, load_pos(n.x[s_xb], b));
    }
    const double sdF = block_sum_r(dF, sh);
    if (threadIdx.x == 0) n.part_fil[4 * (size_t)blockIdx.x + 3] = sdF;
}

template <typename Real>
__global__ void __launch_bounds__(kBlock) k_finalize_direction(DevNet<Real> n) {
    pdl_wait();      // the previous kernel of the main lane has finished
    pdl_trigger();   // the next kernel of the main lane may be scheduled now
    MECH_TRACE_KERNEL(n, TK_FIN_DIRECTION);
    __shared__ double sh[32];
    __shared__ int s_flag;
    const int r = blockIdx.x;
    CGState S;
    if (threadIdx.x == 0) S = n.st[r];   // issued together with the loads below
    const RepTiles rt = n.rt[r];
    if (n.st[r].phase == PH_DIR) finalize_direction(n, r, rt, S, sh);
    after_phase(n, kCondDir, &s_flag);
}

// d = F (resetCGParams, CGMethod.hpp:963-972); the new slope d.F is F.F.
// kGatherTiles tiles per block, so that the launch costs little when no
// replica is resetting (it is in every iteration of the graph).
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_reset(DevNet<Real> n) {
    pdl_wait();      // the previous kernel of the main lane has finished
    pdl_trigger();   // the next kernel of the main lane may be scheduled now
    MECH_TRACE_KERNEL(n, TK_RESET);
    // the misc body of the conditional graph (failure dispatch is applied where a
    // line search fails) counts its launches here
    if (n.cond.on && blockIdx.x == 0 && threadIdx.x == 0) ++n.cond.counter[kCondMisc];
    __shared__ int s_go[kGatherTiles], s_fb[kGatherTiles], s_flag;
    const int t0 = blockIdx.x * kGatherTiles;
    if (threadIdx.x < kGatherTiles) {
        const int ti = t0 + threadIdx.x;
        int go = 0, fb = 0;
        if (ti < n.n_ftiles) {
            const CGState& S = n.st[n.ftile[ti].replica];
            go = S.phase == PH_RESET;
            fb = S.fbuf;
        }
        s_go[threadIdx.x] = go;
        s_fb[threadIdx.x] = fb;
    }
    __syncthreads();
    for (int j = 0; j < kGatherTiles; ++j) {
        if (!s_go[j]) continue;   // block-uniform
        const Tile t = n.ftile[t0 + j];
        const int r = t.replica;
        const int b = t.begin + threadIdx.x;
        if (b < t.end) {
            const Real* F = n.f[s_fb[j]] + 3 * (size_t)b;
            Real* D = n.d + 3 * (size_t)b;
            D[0] = F[0];
            D[1] = F[1];
            D[2] = F[2];
        }
        const RepTiles rt = n.rt[r];
        if (last_tile(n.ticket, r, rt.fil_end - rt.fil_begin, &s_flag)) {
            if (threadIdx.x == 0) {
                CGState& S = n.st[r];
                S.slope = S.FdotF;
                S.lastFdotF = S.FdotF;
                begin_iteration(S);
            }
        }
    }
}


// Recovery move: step = maxDist / max_i |d_i|, x += step d (MController.h:273-339).
template <typename Real>
__global__ void __launch_bounds__(kBlock) k_recover_maxabs(DevNet<Real> n) {
    MECH_TRACE_KERNEL(n, TK_RECOVER_MAXABS);
    __shared__ double sh[32];
    __shared__ int s_go, s_flag;
    const Tile t = n.ftile[blockIdx.x];
    const int r = t.replica;
    if (threadIdx.x == 0) s_go = n.st[r].phase == PH_RECOVER;
    __syncthreads();
    if (!s_go) return;
    const int b = t.begin + threadIdx.x;
    Real m = 0;
    if (b < t.end) {
        const Real* D = n.d + 3 * (size_t)b;
        m = fmax(fmax(fabs(D[0]), fabs(D[1])), fabs(D[2]));
    }
    const double sm = block_max_r(m, sh);
    if (threadIdx.x == 0) n.part_fil[4 * (size_t)blockIdx.x + 3] = sm;
    const RepTiles rt = n.rt[r];
    if (last_tile(n.ticket, r, rt.fil_end - rt.fil_begin, &s_flag)) {
        const double mx = max_slots(n.part_fil, 4, 3, rt.fil_begin, rt.fil_end, sh);
        if (threadIdx.x == 0) {
            CGState& S = n.st[r];
            const double step = S.maxDist / mx;
            if (!(step < (1.0 / 0.0))) {   // "step size is infinity" (MController.h:311-316)
                S.status = MECH_ERR_NONFINITE;
                S.phase = PH_ERROR;
            } else {
                S.lambda = step;
                S.phase = PH_RECOVER_MOVE;
            }
        }
    }
}

template <typename Real>
__global__ void __launch_bounds__(kBlock) k_recover_move(DevNet<Real> n) {
    MECH_TRACE_KERNEL(n, TK_RECOVER_MOVE);
    __shared__ int s_go, s_xb, s_flag;
    __shared__ double s_step;
    const Tile t = n.ftile[blockIdx.x];
    const int r = t.replica;
    if (threadIdx.x == 0) {
        const CGState& S = n.st[r];
        s_go = S.phase == PH_RECOVER_MOVE;
        s_xb = S.xbuf;
        s_step = S.lambda;
    }
    __syncthreads();
    if (!s_go) return;
    const int b = t.begin + threadIdx.x;
    if (b < t.end) {   // coord += step * d (MController.h:321-323)
        Real* X = n.x[s_xb];
        store_pos(X, b, moved(load_pos(X, b), n.d, b, s_step));
    }
    const RepTiles rt = n.rt[r];
    if (last_tile(n.ticket, r, rt.fil_end - rt.fil_begin, &s_flag)) {
        if (threadIdx.x == 0) n.st[r].phase = PH_RECOVER_FORCE;
    }
}

template <typename Real>
__global__ void __launch_bounds__(kBlock) k_backup_restore(DevNet<Real> n) {
    MECH_TRACE_KERNEL(n, TK_BACKUP);
    const Tile t = n.ftile[blockIdx.x];
    const CGState& S = n.st[t.replica];
    if (!S.restore) return;
    const int b = t.begin + threadIdx.x;
    if (b < t.end) store_pos(n.x[S.xbuf], b, load_pos(n.xbest, b));
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename Real>
static int n_lm_tiles(const DevNet<Real>& n, int* ev_tiles, int* bb_tiles) {
    *ev_tiles = n.sp_tiles[K_EXVOL];
    *bb_tiles = n.sp_tiles[K_BOUNDARY];
    return n.sp_tiles[K_LINKER] + n.sp_tiles[K_MOTOR];
}

// The excluded-volume chain and the linker/motor/boundary kernel on side
// lanes, the filament kernel on the main lane, then (after the joins) the
// reduction on the main lane.
// The filament kernel of an evaluation is launched before the side lanes when
// its residency is capped (n.fil_first[k]): its blocks then start streaming at
// once and the excluded-volume and linker kernels fill the room the cap leaves;
// uncapped, it fills every SM and is launched after them.
template <typename Real>
int launch_energy(const DevNet<Real>& n, int want, int trial, const Lanes& L) {
    int ev_t = 0, bb_t = 0;
    const int lm = n_lm_tiles(n, &ev_t, &bb_t);
    int launched = 0;
    cudaEventRecord(L.fork, L.main);
    cudaStreamWaitEvent(L.side, L.fork, 0);
    cudaStreamWaitEvent(L.side2, L.fork, 0);
    auto fil = [&] {
        if constexpr (sizeof(Real) == 4) launch_k(n.pdl, k_fil_energy_bulk, n.pgrid[0], kBlock, L.main, n, want, trial);
        else launch_k(n.pdl, k_fil_energy<Real>, n.n_ftiles, kBlock, L.main, n, want, trial);
    };
    if (n.fil_first[0]) fil();
    launched += launch_exvol_energy<Real>(n, want, trial, L.side, false);
    cudaEventRecord(L.join, L.side);
    if (lm + bb_t > 0) {
        k_bond_bnd<Real><<<lm + bb_t, kBlock, 0, L.side2>>>(n, want, trial, 0, lm, ev_t);
        ++launched;
    }
    cudaEventRecord(L.join2, L.side2);
    if (!n.fil_first[0]) fil();
    cudaStreamWaitEvent(L.main, L.join, 0);
    cudaStreamWaitEvent(L.main, L.join2, 0);
    k_finalize_energy<Real><<<n.R, kBlock, 0, L.main>>>(n, want, trial);
    return launched + 2;
}

template <typename Real>
int launch_forces(const DevNet<Real>& n, int want, const Lanes& L, int coop_grid) {
    int ev_t = 0, bb_t = 0;
    const int lm = n_lm_tiles(n, &ev_t, &bb_t);
    int launched = 0;
    cudaEventRecord(L.fork, L.main);
    cudaStreamWaitEvent(L.side, L.fork, 0);
    cudaStreamWaitEvent(L.side2, L.fork, 0);
    auto fil = [&] {
        if constexpr (sizeof(Real) == 4) launch_k(n.pdl, k_fil_force_bulk, n.pgrid[1], kBlock, L.main, n, want);
        else launch_k(n.pdl, k_fil_force<Real>, n.n_ftiles, kBlock, L.main, n, want);
    };
    if (n.fil_first[1]) fil();
    launched += launch_exvol_forces<Real>(n, want, L.side, false);
    cudaEventRecord(L.join, L.side);
    if (lm + bb_t > 0) {
        k_bond_bnd<Real><<<lm + bb_t, kBlock, 0, L.side2>>>(n, want, 0, 1, lm, ev_t);
        ++launched;
    }
    cudaEventRecord(L.join2, L.side2);
    if (!n.fil_first[1]) fil();
    cudaStreamWaitEvent(L.main, L.join, 0);
    cudaStreamWaitEvent(L.main, L.join2, 0);
    if constexpr (sizeof(Real) == 4) {
        if (coop_grid > 0) {
            launch_tail_coop(n, coop_grid, L.main);
            return launched + 2;
        }
    }
    if constexpr (sizeof(Real) == 4) k_force_gather_mx<<<(n.n_ftiles + kGatherTiles - 1) / kGatherTiles, kBlock, 0, L.main>>>(n, want);
    else k_force_gather<Real><<<(n.n_ftiles + kGatherTiles - 1) / kGatherTiles, kBlock, 0, L.main>>>(n, want);
    launch_k(n.pdl, k_finalize_force<Real>, n.R, kBlock, L.main, n, want);
    return launched + 3;
}

template <typename Real>
int launch_direction(const DevNet<Real>& n, cudaStream_t s) {
    if constexpr (sizeof(Real) == 4) launch_k(n.pdl, k_direction_mx, n.pgrid[2], kBlock, s, n);
    else launch_k(n.pdl, k_direction<Real>, n.n_ftiles, kBlock, s, n);
    launch_k(n.pdl, k_finalize_direction<Real>, n.R, kBlock, s, n);
    return 2;
}

template <typename Real>
int launch_reset(const DevNet<Real>& n, cudaStream_t s) {
    launch_k(n.pdl, k_reset<Real>, (n.n_ftiles + kGatherTiles - 1) / kGatherTiles, kBlock, s, n);
    return 1;
}

template <typename Real>
int launch_body_head(const DevNet<Real>& n, cudaStream_t s) {
    k_body_head<Real><<<1, kBlock, 0, s>>>(n);
    return 1;
}


template <typename Real>
int launch_recover(const DevNet<Real>& n, const Lanes& L) {
    int k = 0;
    k_recover_maxabs<Real><<<n.n_ftiles, kBlock, 0, L.main>>>(n);
    k_recover_move<Real><<<n.n_ftiles, kBlock, 0, L.main>>>(n);
    k += 2;
    k += launch_forces<Real>(n, PH_RECOVER_FORCE, L);
    k += launch_energy<Real>(n, PH_RECOVER_ENERGY, 0, L);
    k += launch_reset<Real>(n, L.main);
    return k;
}

template <typename Real>
int launch_backup_restore(const DevNet<Real>& n, cudaStream_t s) {
    k_backup_restore<Real><<<n.n_ftiles, kBlock, 0, s>>>(n);
    return 1;
}

template <typename Real>
int launch_part(const DevNet<Real>& n, int which, cudaStream_t s) {
    int ev_t = 0, bb_t = 0;
    const int lm = n_lm_tiles(n, &ev_t, &bb_t);
    switch (which) {
        case 0:
            if constexpr (sizeof(Real) == 4) k_fil_energy_bulk<<<n.pgrid[0], kBlock, 0, s>>>(n, -1, 0);
            else k_fil_energy<Real><<<n.n_ftiles, kBlock, 0, s>>>(n, -1, 0);
            return 1;
        case 1:
            if constexpr (sizeof(Real) == 4) k_fil_force_bulk<<<n.pgrid[1], kBlock, 0, s>>>(n, -1);
            else k_fil_force<Real><<<n.n_ftiles, kBlock, 0, s>>>(n, -1);
            if constexpr (sizeof(Real) == 4) k_force_gather_mx<<<(n.n_ftiles + kGatherTiles - 1) / kGatherTiles, kBlock, 0, s>>>(n, -1);
            else k_force_gather<Real><<<(n.n_ftiles + kGatherTiles - 1) / kGatherTiles, kBlock, 0, s>>>(n, -1);
            k_finalize_force<Real><<<n.R, kBlock, 0, s>>>(n, -1);
            return 3;
        case 2: if (lm + bb_t > 0) { k_bond_bnd<Real><<<lm + bb_t, kBlock, 0, s>>>(n, -1, 0, 0, lm, ev_t); return 1; } return 0;
        case 3: if (lm + bb_t > 0) { k_bond_bnd<Real><<<lm + bb_t, kBlock, 0, s>>>(n, -1, 0, 1, lm, ev_t); return 1; } return 0;
        case 4:   // filament energy of a line-search pass (positions x + lambda d formed and written;
                  // mixed: the two-trial pass, lambda and lambda / 2)
            if constexpr (sizeof(Real) == 4) k_fil_energy_bulk<<<n.pgrid[0], kBlock, 0, s>>>(n, -1, kTrialDual);
            else k_fil_energy<Real><<<n.n_ftiles, kBlock, 0, s>>>(n, -1, 1);
            return 1;
        case 5:   // filament forces alone
            if constexpr (sizeof(Real) == 4) k_fil_force_bulk<<<n.pgrid[1], kBlock, 0, s>>>(n, -1);
            else k_fil_force<Real><<<n.n_ftiles, kBlock, 0, s>>>(n, -1);
            return 1;
        case 6:   // the sparse gather with the CG partials alone
            if constexpr (sizeof(Real) == 4) k_force_gather_mx<<<(n.n_ftiles + kGatherTiles - 1) / kGatherTiles, kBlock, 0, s>>>(n, -1);
            else k_force_gather<Real><<<(n.n_ftiles + kGatherTiles - 1) / kGatherTiles, kBlock, 0, s>>>(n, -1);
            return 1;
    }
    return 0;
}

// Grid of the mixed engine's persistent filament kernels: every SM holding as
// many blocks as fit, or at most `per_sm` of them (leaving room on each SM for
// the kernels of the other lanes).
int persistent_blocks(int device, int which, int per_sm) {
    static int cached_dev = -1, sms = 0, occ[3] = {0, 0, 0};
    if (cached_dev != device) {
        int b[3] = {0, 0, 0};
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[0], k_fil_energy_bulk, kBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[1], k_fil_force_bulk, kBlock, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[2], k_direction_mx, kBlock, 0);
        for (int k = 0; k < 3; ++k) occ[k] = std::max(1, b[k]);
        sms = std::max(1, sms);
        cached_dev = device;
    }
    const int per = per_sm > 0 ? std::min(per_sm, occ[which]) : occ[which];
    return sms * per;
}

#define MECH_INSTANTIATE(R)                                                             \
    template int launch_part<R>(const DevNet<R>&, int, cudaStream_t);                   \
    template int launch_energy<R>(const DevNet<R>&, int, int, const Lanes&);            \
    template int launch_forces<R>(const DevNet<R>&, int, const Lanes&, int);            \
    template int launch_direction<R>(const DevNet<R>&, cudaStream_t);                   \
    template int launch_reset<R>(const DevNet<R>&, cudaStream_t);                       \
    template int launch_body_head<R>(const DevNet<R>&, cudaStream_t);                   \
    template int launch_recover<R>(const DevNet<R>&, const Lanes&);                     \
    template int launch_backup_restore<R>(const DevNet<R>&, cudaStream_t);
MECH_INSTANTIATE(double)
MECH_INSTANTIATE(float)
#undef MECH_INSTANTIATE

}  // namespace mech
