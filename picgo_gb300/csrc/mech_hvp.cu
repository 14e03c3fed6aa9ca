// Hessian-vector products of the full energy and the solves built on them
// (FP64 engine): the conjugate-gradient solve of (H + shift I) y = b used by
// the implicit adjoint and by Newton refinement of an equilibrium, and the
// per-linker parameter gradient of the adjoint.
//
// H v is the forward-mode derivative of the force routines along v: every
// force field is evaluated once on dual numbers (value, derivative) at x + eps v,
// and -dF/deps is written where the force kernels write F, so the sparse force
// fields scatter to the same bead-ordered contribution slots and each bead
// gathers its own (no float atomics; the order is fixed).  The excluded-volume
// pair uses the cancellation-free invariants and atan2 forms (identical
// functions to the reference's, better conditioned).  The reference's force
// routine moves nearly coplanar pairs off their plane before evaluating them
// (CylinderExclVolRepulsion.cpp:610-626, paths relative to medyan-5.4.0/src),
// so its forces are not exactly the energy's gradient there: the solves use
// the exact (symmetric) Hessian of the energy, and the force Jacobian with the
// move differentiated is available separately.  Positions are read from x[0]:
// callers bring every replica's current coordinates there first.
#include <cuda_runtime.h>

#include "mech_device.cuh"
#include "mech_dual.cuh"
#include "mech_exvol_math.cuh"

namespace mech {

namespace {

constexpr int kHvpBlock = 256;

__device__ __forceinline__ void dual_bead(const double* X, const double* V, int b, Dual p[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) p[k] = Dual(X[3 * (size_t)b + k], V[3 * (size_t)b + k]);
}

// write -dF/deps (= the H v part) of one bead's contribution
__device__ __forceinline__ void put_hv(const DevNet<double>& n, int slot, const Dual F[3]) {
    double* c = slot_ptr(n, slot);
    c[0] = -F[0].d;
    c[1] = -F[1].d;
    c[2] = -F[2].d;
}

// Excluded-volume pair forces on dual positions; `jac` applies the
// reference's coplanarity move as its force routine does (the force Jacobian,
// not symmetric), otherwise the energy's own gradient (the exact Hessian).
__device__ bool pair_forces_dual(const Dual* c1, const Dual* c2in, const Dual* c3, const Dual* c4, double kRep,
                                 bool jac, Dual out[4][3]) {
    double w1[3], w2[3], w3[3], w4[3];
    for (int k = 0; k < 3; ++k) {
        w1[k] = c1[k].v;
        w2[k] = c2in[k].v;
        w3[k] = c3[k].v;
        w4[k] = c4[k].v;
    }
    Dual c2[3] = {c2in[0], c2in[1], c2in[2]};
    if (jac && coplanarity<double>(w1, w2, w3, w4) < 0.1) {
        Dual a[3], b[3];
        for (int k = 0; k < 3; ++k) {
            a[k] = c2in[k] - c1[k];
            b[k] = c3[k] - c1[k];
        }
        const Dual nx = a[1] * b[2] - a[2] * b[1], ny = a[2] * b[0] - a[0] * b[2], nz = a[0] * b[1] - a[1] * b[0];
        const Dual nn = sqrt(nx * nx + ny * ny + nz * nz);
        c2[0] = c2in[0] + (nx / nn) * 0.01;
        c2[1] = c2in[1] + (ny / nn) * 0.01;
        c2[2] = c2in[2] + (nz / nn) * 0.01;
    }
    Dual v12[3], v34[3], v31[3], v14[3], v32[3], v24[3];
    for (int k = 0; k < 3; ++k) {
        v12[k] = c2[k] - c1[k];
        v34[k] = c4[k] - c3[k];
        v31[k] = c1[k] - c3[k];
        v14[k] = c4[k] - c1[k];
        v32[k] = c2[k] - c3[k];
        v24[k] = c4[k] - c2[k];
    }
    PairInv<Dual> p;
    pair_inv(v12, v34, v31, v14, v32, v24, p, true);
    return forces_from<true>(p, v12, v34, v31, Dual(kRep), out);
}

__global__ void __launch_bounds__(kHvpBlock) k_hvp_sparse(DevNet<double> n, const double* __restrict__ V, int jac) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double* X = n.x[0];
    const int nlm = n.n_lk + n.n_mt;
    if (i < nlm) {
        const bool lk = i < n.n_lk;
        const int j = lk ? i : i - n.n_lk;
        const int4 bs = lk ? n.lk_bead[j] : n.mt_bead[j];
        const double k = lk ? n.lk_k[j] : n.mt_k[j], l0 = lk ? n.lk_l0[j] : n.mt_l0[j];
        const double s1 = lk ? n.lk_s1[j] : n.mt_s1[j], s2 = lk ? n.lk_s2[j] : n.mt_s2[j];
        Dual c1[3], c2[3], c3[3], c4[3];
        dual_bead(X, V, bs.x, c1);
        dual_bead(X, V, bs.y, c2);
        dual_bead(X, V, bs.z, c3);
        dual_bead(X, V, bs.w, c4);
        Dual l[3];
        for (int q = 0; q < 3; ++q) l[q] = (c3[q] + (c4[q] - c3[q]) * s2) - (c1[q] + (c2[q] - c1[q]) * s1);
        const Dual dist = sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
        const Dual f0 = k * (dist - l0) / dist;
        Dual Fa[3], Fb[3], Fc[3], Fd[3];
        for (int q = 0; q < 3; ++q) {
            const Dual Fl = -f0 * l[q];
            Fa[q] = -Fl * (1.0 - s1);
            Fb[q] = -Fl * s1;
            Fc[q] = Fl * (1.0 - s2);
            Fd[q] = Fl * s2;
        }
        const int sb = n.slot_base[lk ? K_LINKER : K_MOTOR] + 4 * j;
        put_hv(n, sb, Fa);
        put_hv(n, sb + 1, Fb);
        put_hv(n, sb + 2, Fc);
        put_hv(n, sb + 3, Fd);
        return;
    }
    const int e = i - nlm;
    if (e < n.n_ev) {
        const int4 bs = n.ev_bead[e];
        Dual c1[3], c2[3], c3[3], c4[3];
        dual_bead(X, V, bs.x, c1);
        dual_bead(X, V, bs.y, c2);
        dual_bead(X, V, bs.z, c3);
        dual_bead(X, V, bs.w, c4);
        Dual out[4][3];
        if (!pair_forces_dual(c1, c2, c3, c4, n.ev_k[e] * n.ev_la[e] * n.ev_lb[e], jac != 0, out)) atomicOr(n.err, 8u);
        for (int a = 0; a < 4; ++a) put_hv(n, n.slot_base[K_EXVOL] + 4 * e + a, out[a]);
        return;
    }
    const int m = e - n.n_ev;
    if (m < n.n_bb) {
        const int b = n.bb_bead[m];
        const double* pl = n.planes + 4 * n.bb_plane[m];
        Dual p[3];
        dual_bead(X, V, b, p);
        const double nrm = sqrt(pl[0] * pl[0] + pl[1] * pl[1] + pl[2] * pl[2]);
        const Dual r = (p[0] * pl[0] + p[1] * pl[1] + p[2] * pl[2] + pl[3]) / nrm;
        const double K = n.bb_k[m], sl = n.bb_slen[m];
        const Dual f0 = K * exp(-r / sl) / sl;
        const Dual F[3] = {f0 * pl[0], f0 * pl[1], f0 * pl[2]};
        put_hv(n, n.slot_base[K_BOUNDARY] + m, F);
    }
}

// Owner side: the filament terms touching bead b on duals, plus the bead's
// gathered sparse contributions; hv = -dF + shift v.
__global__ void __launch_bounds__(kHvpBlock) k_hvp_fil(DevNet<double> n, const double* __restrict__ V, double shift,
                                                      double* __restrict__ HV) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n.nb) return;
    const double* X = n.x[0];
    const int f0 = n.bflag[b];
    const int fm = (f0 & 2) ? n.bflag[b - 1] : 0;
    const int fp = (f0 & 1) ? n.bflag[b + 1] : 0;
    Dual p0[3], pm1[3], pp1[3], pm2[3], pp2[3];
    dual_bead(X, V, b, p0);
    if (f0 & 2) dual_bead(X, V, b - 1, pm1);
    if (f0 & 1) dual_bead(X, V, b + 1, pp1);
    if (fm & 2) dual_bead(X, V, b - 2, pm2);
    if (fp & 1) dual_bead(X, V, b + 2, pp2);
    Dual F[3];
    Dual rm[3], rp[3];
    for (int q = 0; q < 3; ++q) {
        rm[q] = p0[q] - pm1[q];
        rp[q] = pp1[q] - p0[q];
    }
    double ksm = 0, l0m = 0, kbm = 0, thm = 0, ks = 0, l0 = 0, kb = 0, th = 0;
    if (f0 & 2) load_par(n.bpar, b - 1, ksm, l0m, kbm, thm);
    if (f0 & 1) load_par(n.bpar, b, ks, l0, kb, th);
    if (f0 & 2) {
        Dual S1[3];
        stretch_force<Dual>(rm[0], rm[1], rm[2], Dual(ksm), Dual(l0m), S1);
        for (int q = 0; q < 3; ++q) F[q] += S1[q];
    }
    if (f0 & 1) {
        Dual S2[3];
        stretch_force<Dual>(rp[0], rp[1], rp[2], Dual(ks), Dual(l0), S2);
        for (int q = 0; q < 3; ++q) F[q] -= S2[q];
    }
    if ((f0 & 2) && (fm & 2)) {
        Dual r1[3], a1[3], a2[3];
        for (int q = 0; q < 3; ++q) r1[q] = pm1[q] - pm2[q];
        bend_force<Dual>(r1, rm, Dual(kbm), Dual(thm), a1, a2);
        for (int q = 0; q < 3; ++q) F[q] += a2[q];
    }
    if ((f0 & 3) == 3) {
        Dual a1[3], a2[3];
        bend_force<Dual>(rm, rp, Dual(kb), Dual(th), a1, a2);
        for (int q = 0; q < 3; ++q) F[q] += a1[q] - a2[q];
    }
    if ((f0 & 1) && (fp & 1)) {
        double ksp, l0p, kbp, thp;
        load_par(n.bpar, b + 1, ksp, l0p, kbp, thp);
        Dual r2[3], a1[3], a2[3];
        for (int q = 0; q < 3; ++q) r2[q] = pp2[q] - pp1[q];
        bend_force<Dual>(rp, r2, Dual(kbp), Dual(thp), a1, a2);
        for (int q = 0; q < 3; ++q) F[q] -= a1[q];
    }
    double h[3] = {-F[0].d, -F[1].d, -F[2].d};
    const int c0 = n.csr_off[b], c1 = n.csr_off[b + 1];
    for (int c = c0; c < c1; ++c) {
        h[0] += n.contrib[3 * (size_t)c];
        h[1] += n.contrib[3 * (size_t)c + 1];
        h[2] += n.contrib[3 * (size_t)c + 2];
    }
    for (int q = 0; q < 3; ++q) HV[3 * (size_t)b + q] = h[q] + shift * V[3 * (size_t)b + q];
}

// ---- CG vector kernels: deterministic dots (fixed grid, per-block slots, the
// last block sums the slots in order) and fused updates -----------------------
constexpr int kCgBlocks = 304;

// scal: [0] rr, [1] pAp, [2] rr_new, [3] bb
__device__ __forceinline__ void finish_dot(double v, double* part, unsigned* ticket, double* out, double* sh) {
    v = block_sum(v, sh);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = v;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double a = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) a += __ldcg(part + k);
    a = block_sum(a, sh);
    if (threadIdx.x == 0) {
        *out = a;
        *ticket = 0u;
    }
}

__global__ void __launch_bounds__(kHvpBlock) k_dot(const double* __restrict__ a, const double* __restrict__ b, long long n,
                                                   double* part, unsigned* ticket, double* out) {
    __shared__ double sh[32];
    double v = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v += a[i] * b[i];
    finish_dot(v, part, ticket, out, sh);
}

// x += alpha p, r -= alpha Ap, alpha = rr / pAp; rr_new = r . r
__global__ void __launch_bounds__(kHvpBlock) k_cg_step(double* __restrict__ x, double* __restrict__ r,
                                                       const double* __restrict__ p, const double* __restrict__ Ap,
                                                       long long n, double* scal, double* part, unsigned* ticket) {
    __shared__ double sh[32];
    // scal[4] latches non-positive curvature p.Ap <= 0: the iterate is frozen
    // there (the truncated solution is what the caller gets)
    const bool stop = scal[4] != 0.0 || !(scal[1] > 0.0);
    if (stop && blockIdx.x == 0 && threadIdx.x == 0) scal[4] = 1.0;
    const double alpha = stop ? 0.0 : scal[0] / scal[1];
    double v = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * Ap[i];
        r[i] = ri;
        v += ri * ri;
    }
    finish_dot(v, part, ticket, scal + 2, sh);
}

// p = r + (rr_new / rr) p; rr = rr_new
__global__ void __launch_bounds__(kHvpBlock) k_cg_dir(double* __restrict__ p, const double* __restrict__ r, long long n,
                                                      double* scal) {
    const double beta = scal[2] / scal[0];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = r[i] + beta * p[i];
}

__global__ void k_cg_roll(double* scal) {
    if (threadIdx.x == 0 && blockIdx.x == 0) scal[0] = scal[2];
}

// Linker parameter gradient of the implicit adjoint, per linker j:
// dL/dk = wE (d - l0)^2 / 2 - (d - l0) g,  dL/dl0 = -wE k (d - l0) + k g,
// with g = lambda . grad_x d (the linker's length gradient at its beads).
__global__ void __launch_bounds__(kHvpBlock) k_linker_grad(DevNet<double> n, int lk0, int nlk,
                                                           const double* __restrict__ L, double wE,
                                                           double* __restrict__ dk, double* __restrict__ dl0) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nlk) return;
    const int j = lk0 + t;
    const int4 bs = n.lk_bead[j];
    const double* X = n.x[0];
    const double s1 = n.lk_s1[j], s2 = n.lk_s2[j], k = n.lk_k[j], l0 = n.lk_l0[j];
    double l[3], lam[3];
    for (int q = 0; q < 3; ++q) {
        const double p1 = X[3 * (size_t)bs.x + q] + (X[3 * (size_t)bs.y + q] - X[3 * (size_t)bs.x + q]) * s1;
        const double p2 = X[3 * (size_t)bs.z + q] + (X[3 * (size_t)bs.w + q] - X[3 * (size_t)bs.z + q]) * s2;
        l[q] = p2 - p1;
        lam[q] = ((1.0 - s2) * L[3 * (size_t)bs.z + q] + s2 * L[3 * (size_t)bs.w + q]) -
                 ((1.0 - s1) * L[3 * (size_t)bs.x + q] + s1 * L[3 * (size_t)bs.y + q]);
    }
    const double d = sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
    const double g = (l[0] * lam[0] + l[1] * lam[1] + l[2] * lam[2]) / d;
    const double dd = d - l0;
    dk[t] = wE * 0.5 * dd * dd - dd * g;
    dl0[t] = -wE * k * dd + k * g;
}

}  // namespace

int launch_hvp(const DevNet<double>& n, const double* v, double* hv, double shift, bool jacobian, cudaStream_t s) {
    const int ns = n.n_lk + n.n_mt + n.n_ev + n.n_bb;
    int k = 0;
    if (ns > 0) {
        k_hvp_sparse<<<(ns + kHvpBlock - 1) / kHvpBlock, kHvpBlock, 0, s>>>(n, v, jacobian ? 1 : 0);
        ++k;
    }
    k_hvp_fil<<<(n.nb + kHvpBlock - 1) / kHvpBlock, kHvpBlock, 0, s>>>(n, v, shift, hv);
    return k + 1;
}

cudaError_t hvp_cg_solve(const DevNet<double>& n, const double* b, double* x, const HvpCgWork& w, double rel_tol,
                         int max_iter, double shift, cudaStream_t s, HvpCgResult* res) {
    const long long N = 3LL * n.nb;
    const int G = kCgBlocks, B = kHvpBlock;
    cudaError_t e;
    res->iterations = 0;
    res->launches = 0;
    res->rel_residual = 0.0;
    res->converged = 0;
    res->negative_curvature = 0;
    // x = 0, r = b, p = b; rr = bb = b . b; no curvature flag
    if ((e = cudaMemsetAsync(x, 0, sizeof(double) * N, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(w.scal, 0, sizeof(double) * 8, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(w.r, b, sizeof(double) * N, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(w.p, b, sizeof(double) * N, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(w.ticket, 0, sizeof(unsigned), s)) != cudaSuccess) return e;
    k_dot<<<G, B, 0, s>>>(b, b, N, w.part, w.ticket, w.scal + 0);
    k_dot<<<G, B, 0, s>>>(b, b, N, w.part, w.ticket, w.scal + 3);
    double h[5];
    if ((e = cudaMemcpyAsync(h, w.scal, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    const double bb = h[3];
    if (!(bb > 0.0)) {
        res->converged = 1;
        return cudaSuccess;
    }
    const double tol2 = rel_tol * rel_tol * bb;
    // kCheck iterations per CUDA graph launch; the host reads the residual between launches
    constexpr int kCheck = 16;
    int per_iter = 0;
    auto iteration = [&]() {
        per_iter = launch_hvp(n, w.p, w.Ap, shift, false, s);
        k_dot<<<G, B, 0, s>>>(w.p, w.Ap, N, w.part, w.ticket, w.scal + 1);
        k_cg_step<<<G, B, 0, s>>>(x, w.r, w.p, w.Ap, N, w.scal, w.part, w.ticket);
        k_cg_dir<<<G, B, 0, s>>>(w.p, w.r, N, w.scal);
        k_cg_roll<<<1, 32, 0, s>>>(w.scal);
        per_iter += 4;
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    for (int j = 0; j < kCheck; ++j) iteration();
    e = cudaStreamEndCapture(s, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) return e;
    for (int it = 0; it < max_iter;) {
        if (max_iter - it >= kCheck) {
            e = cudaGraphLaunch(exec, s);
            it += kCheck;
            res->launches += (long long)kCheck * per_iter;
        } else {
            for (; it < max_iter; ++it) {
                iteration();
                res->launches += per_iter;
            }
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(h, w.scal, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        res->iterations = it;
        res->rel_residual = sqrt(h[0] / bb);
        if (h[4] != 0.0) {   // non-positive curvature met: the iterate stopped there
            res->negative_curvature = 1;
            break;
        }
        if (h[0] <= tol2) {
            res->converged = 1;
            break;
        }
    }
    cudaGraphExecDestroy(exec);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

void launch_linker_grad(const DevNet<double>& n, int lk0, int nlk, const double* lambda, double wE, double* dk,
                        double* dl0, cudaStream_t s) {
    if (nlk <= 0) return;
    k_linker_grad<<<(nlk + kHvpBlock - 1) / kHvpBlock, kHvpBlock, 0, s>>>(n, lk0, nlk, lambda, wE, dk, dl0);
}

}  // namespace mech
