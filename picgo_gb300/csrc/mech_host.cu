// Host side of the engine: the context, network upload (serializeDof +
// vectorizeAllForceFields), neighbor-list rebuild orchestration, the CUDA-graph
// driven minimizer loop, and the C ABI of include/medyan_mech.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "mech_device.cuh"
#include "mech_internal.cuh"
#include "mech_nl.cuh"

namespace mech {

static thread_local std::string g_last_error;

static int set_err(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int set_error_text(int code, const std::string& msg) { return set_err(code, msg); }

#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess)                                                                     \
            return set_err(MECH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));     \
    } while (0)

struct ReplicaHost {
    int nb = 0, bead_begin = 0;
    int ncyl = 0, cyl_begin = 0;
    int nfil = 0;
    int nlk = 0, lk_begin = 0, nmt = 0, mt_begin = 0;
    int nplanes = 0, plane_begin = 0;
    std::vector<int> perm;     // caller bead -> internal local index
    std::vector<int> inv;      // internal local index -> caller bead
    double box[3] = {0, 0, 0};
    double rmax = 0, bcut = 0;
    // set by the last rebuild
    long long nev = 0, ev_begin = 0, nbb = 0, bb_begin = 0, nbcyl = 0;
    long long bq_begin = 0;    // first boundary-list entry (plane, cylinder) of this replica
    std::vector<int> fil_end_cyl;   // per filament: first and last cylinder (replica-local)
    std::vector<int> fil_type;      // per filament: type of its cylinders
    double cell = 0;
    int gx = 1, gy = 1, gz = 1;
    long long cell_off = 0;
};

}  // namespace mech

using namespace mech;

struct MechContext {
    int device = 0;
    int precision = MECH_PREC_FP64;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr, side2 = nullptr;      // lanes of the sparse force fields
    cudaEvent_t fork = nullptr, join = nullptr, join2 = nullptr;
    Lanes lanes() const { return Lanes{stream, side, side2, fork, join, join2}; }
    int R = 0;
    int nb = 0, ncyl = 0, nlk = 0, nmt = 0, nplanes = 0;
    long long nev = 0, nbb = 0, nbcyl = 0;
    std::vector<ReplicaHost> reps;
    bool have_net = false, have_lists = false;
    // beads
    DeviceBuffer x[3], f[2], d, xbest, xinit, bflag, bpar;   // x[2]: mixed engine's second trial buffer
    // cylinders
    DeviceBuffer cyl_b1, cyl_id, cyl_fil, cyl_pos, cyl_rep, cyl_minus, cyl_kex, cyl_type, cyl_l0;
    // linkers / motors
    DeviceBuffer lk_bead, lk_k, lk_l0, lk_s1, lk_s2, lk_sf, mt_bead, mt_k, mt_l0, mt_s1, mt_s2, mt_sf;
    // boundary
    DeviceBuffer planes, plane_k, plane_slen, bb_k, bb_slen;
    // excluded volume
    DeviceBuffer ev_bead, ev_k, ev_la, ev_lb, ev_list, ev_list_count, ev_energy, ev_energy2;
    // tiles, partials, state
    DeviceBuffer ftile, stile, stile_kind, rt, part_fil, part_sp, part_sp2, st, ticket, gticket, err, cond_counter;
    int graph_mode = MECH_GRAPH_UNROLLED;
    DeviceBuffer contrib, ev_fb_count, ev_fb_list, ev_fb_energy, fb_moments, fb_tickets;
    // rebuild scratch
    PairBuild pb;
    BndBuild bbuild;
    CsrBuild cb;
    DeviceBuffer rep_cell, rep_dims, rep_rmax2, rep_rmin2, rep_margin, rep_q, rep_ncyl, rep_plane, rep_cyl, rep_bcut,
        gather_idx, gather_out;
    DeviceBuffer perm_all, stage;   // caller -> internal bead map of all replicas; coordinate staging
    // Hessian-vector products, adjoint and Newton solves (FP64 engine)
    DeviceBuffer hv_a, hv_b, cg_x, cg_r, cg_p, cg_Ap, cg_scal, cg_part, cg_ticket;
    DeviceBuffer gbar;   // grid barrier of the cooperative iteration tail (2 unsigned)
    int n_ftiles = 0, n_stiles = 0;
    int sp_tiles[K_NUM_SPARSE] = {0, 0, 0, 0};
    // host copies of the full tile lists, and the compacted view that a
    // batched minimization switches to once most replicas have finished
    std::vector<Tile> h_ftiles, h_stiles;
    std::vector<int> h_skind;
    DeviceBuffer ftile_c, stile_c, stile_kind_c, rt_c;
    bool compact = false;
    int n_ftiles_c = 0, n_stiles_c = 0;
    // tuning (mech_autotune): tiles per block of the mixed filament energy and
    // force kernels, and a multiplier on the default neighbor-list bin edge
    int tile_cap[2] = {kFilBulkMaxTiles, kFilBulkMaxTiles};
    // resident blocks per SM of the persistent filament energy / force kernels
    // (0: as many as fit); fewer leave room for the lanes running beside them,
    // and a capped kernel is launched before those lanes.  The force kernel
    // defaults to 2: its blocks stream from the start of the evaluation while
    // the excluded-volume chain (FP32 pass, extended-precision pass, fallbacks)
    // and the linker kernel keep room on every SM.  Force evaluation on the
    // 1M-cylinder network, graph replays at fixed states: 77 us at 2 blocks,
    // 95 at 3, 125 uncapped (the kernel alone: 28.7, 22.6, 20.5 us).  A cap on
    // the energy kernel only delays the excluded-volume chain (trial pass 78 us
    // uncapped, 90 at 2, 107 at 3).
    int blocks_per_sm[2] = {0, 2};
    double cell_scale = 1.0;
    int sp_tiles_c[K_NUM_SPARSE] = {0, 0, 0, 0};
    int slot_base[K_NUM_SPARSE + 1] = {0, 0, 0, 0, 0};
    std::vector<RepTiles> h_rt;
    CGState* h_st = nullptr;   // pinned mirror of the states
    unsigned* h_err = nullptr;
    // pinned snapshots taken after each minimizer graph launch: states, error
    // word and the conditional graph's body counters, double-buffered
    struct Snapshot {
        CGState* st = nullptr;
        unsigned* err = nullptr;   // [0] error word, [1..8] body counters
        cudaEvent_t done = nullptr;
    } snap[2];
    MechTiming timing{};
#ifdef MECH_TRACE
    DeviceBuffer trace;   // kernel timeline of the diagnostic build (MECH_TRACE_FILE names the dump)
#endif
    std::vector<int32_t> cyl_local_first;   // replica-local cylinder -> internal global first bead

    ~MechContext() {
        if (h_st) cudaFreeHost(h_st);
        if (h_err) cudaFreeHost(h_err);
        for (auto& k : snap) {
            if (k.st) cudaFreeHost(k.st);
            if (k.err) cudaFreeHost(k.err);
            if (k.done) cudaEventDestroy(k.done);
        }
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (join2) cudaEventDestroy(join2);
        if (side) cudaStreamDestroy(side);
        if (side2) cudaStreamDestroy(side2);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

template <typename T>
int upload(DeviceBuffer& b, const std::vector<T>& v, cudaStream_t s) {
    CU(b.ensure(sizeof(T) * std::max<size_t>(v.size(), 1)));
    if (!v.empty()) CU(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
    return MECH_OK;
}

template <typename Real>
DevNet<Real> make_devnet(MechContext* c) {
    DevNet<Real> n{};
    n.nb = c->nb;
    n.R = c->R;
    n.x[0] = c->x[0].as<Real>();
    n.x[1] = c->x[1].as<Real>();
    n.x[2] = c->x[2].as<Real>();
    n.f[0] = c->f[0].as<Real>();
    n.f[1] = c->f[1].as<Real>();
    n.d = c->d.as<Real>();
    n.xbest = c->xbest.as<Real>();
    n.ev_list = c->ev_list.as<int>();
    n.ev_list_count = c->ev_list_count.as<int>();
    n.ev_energy = c->ev_energy.as<double>();
    n.ev_energy2 = c->ev_energy2.as<double>();
    n.bflag = c->bflag.as<uint8_t>();
    n.bpar = c->bpar.as<Real>();
    n.n_ftiles = c->compact ? c->n_ftiles_c : c->n_ftiles;
    n.ftile = (c->compact ? c->ftile_c : c->ftile).as<Tile>();
    for (int k = 0; k < 3; ++k) {
        const int per_sm = k < 2 ? c->blocks_per_sm[k] : 0;
        if (k < 2) n.fil_first[k] = (c->precision == MECH_PREC_MIXED && per_sm > 0) ? 1 : 0;
        const int resident = persistent_blocks(c->device, k, per_sm);
        n.pgrid[k] = std::max(1, std::min(n.n_ftiles, resident));
        n.ptiles[k] = (n.n_ftiles + n.pgrid[k] - 1) / n.pgrid[k];
        if (k < 2) {
            // the bulk-staged energy/force kernels keep a block's tile descriptors in
            // shared memory (at most kFilBulkMaxTiles); a tuned smaller run length adds
            // waves, unless a residency cap is set, which the grid then keeps to
            n.ptiles[k] = std::max(1, std::min(n.ptiles[k], c->tile_cap[k]));
            if (per_sm > 0) n.ptiles[k] = std::max(n.ptiles[k], (n.n_ftiles + resident - 1) / resident);
            n.ptiles[k] = std::min(n.ptiles[k], kFilBulkMaxTiles);
        }
        n.pgrid[k] = (n.n_ftiles + n.ptiles[k] - 1) / n.ptiles[k];
    }
    n.n_lk = c->nlk;
    n.n_mt = c->nmt;
    n.n_ev = (int)c->nev;
    n.n_bb = (int)c->nbb;
    n.lk_bead = c->lk_bead.as<int4>();
    n.lk_k = c->lk_k.as<Real>();
    n.lk_l0 = c->lk_l0.as<Real>();
    n.lk_s1 = c->lk_s1.as<Real>();
    n.lk_s2 = c->lk_s2.as<Real>();
    n.mt_bead = c->mt_bead.as<int4>();
    n.mt_k = c->mt_k.as<Real>();
    n.mt_l0 = c->mt_l0.as<Real>();
    n.mt_s1 = c->mt_s1.as<Real>();
    n.mt_s2 = c->mt_s2.as<Real>();
    n.ev_bead = c->ev_bead.as<int4>();
    n.ev_k = c->ev_k.as<Real>();
    n.ev_la = c->ev_la.as<Real>();
    n.ev_lb = c->ev_lb.as<Real>();
    n.bb_bead = c->bbuild.bead.as<int>();
    n.bb_plane = c->bbuild.plane.as<int>();
    n.planes = c->planes.as<double>();
    n.bb_k = c->bb_k.as<Real>();
    n.bb_slen = c->bb_slen.as<Real>();
    n.n_stiles = c->compact ? c->n_stiles_c : c->n_stiles;
    n.stile = (c->compact ? c->stile_c : c->stile).as<Tile>();
    n.stile_kind = (c->compact ? c->stile_kind_c : c->stile_kind).as<int>();
    for (int k = 0; k < K_NUM_SPARSE; ++k) n.sp_tiles[k] = c->compact ? c->sp_tiles_c[k] : c->sp_tiles[k];
    n.contrib = c->contrib.as<Real>();
    for (int k = 0; k <= K_NUM_SPARSE; ++k) n.slot_base[k] = c->slot_base[k];
    n.csr_off = c->cb.off.as<int>();
    n.slot_pos = c->cb.pos.as<int>();
    n.lk_sf = c->lk_sf.as<double>();
    n.mt_sf = c->mt_sf.as<double>();
    // the fallback count sits beside the FP64-pass count once the lists exist (one reset for both)
    n.ev_fb_count = c->ev_list_count.p ? c->ev_list_count.as<int>() + 2 : c->ev_fb_count.as<int>();
    n.ev_fb_list = c->ev_fb_list.as<int>();
    n.ev_fb_energy = c->ev_fb_energy.as<double>();
    n.fb_moments = c->fb_moments.as<double>();
    n.fb_tickets = c->fb_tickets.as<int>();
    n.part_fil = c->part_fil.as<double>();
    n.part_sp = c->part_sp.as<double>();
    n.part_sp2 = c->part_sp2.as<double>();
    n.st = c->st.as<CGState>();
    n.rt = (c->compact ? c->rt_c : c->rt).as<RepTiles>();
    n.ticket = c->ticket.as<int>();
    n.gticket = c->gticket.as<int>();
    n.err = c->err.as<unsigned>();
#ifdef MECH_TRACE
    n.trace = c->trace.as<unsigned long long>();
#endif
    return n;
}

// Precision-typed upload of a double vector.
int upload_real(MechContext* c, DeviceBuffer& b, const std::vector<double>& v) {
    if (c->precision == MECH_PREC_FP64) return upload(b, v, c->stream);
    std::vector<float> w(v.begin(), v.end());
    return upload(b, w, c->stream);
}

size_t real_size(const MechContext* c) { return c->precision == MECH_PREC_FP64 ? 8 : 4; }

// Fill the per-interaction boundary constants and the exvol interaction
// arrays after a rebuild.
template <typename Real>
__global__ void k_ev_build(const int2* pairs, long long P, const int* cyl_b1, const double* kex, const int* type,
                           const double* l0, int4* ev_bead, Real* ev_k, Real* ev_la, Real* ev_lb) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int2 pr = pairs[i];
    const int bc = cyl_b1[pr.x], bn = cyl_b1[pr.y];
    ev_bead[i] = make_int4(bc, bc + 1, bn, bn + 1);
    // VolumeK of the cylinder, the larger of the two for mixed types (CylinderExclVolume.cpp:113-121)
    const double k = type[pr.x] == type[pr.y] ? kex[pr.x] : fmax(kex[pr.x], kex[pr.y]);
    ev_k[i] = (Real)k;
    ev_la[i] = (Real)l0[pr.x];
    ev_lb[i] = (Real)l0[pr.y];
}

template <typename Real>
__global__ void k_bb_build(const int* bb_plane, long long n, const double* pk, const double* ps, Real* bk, Real* bs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bk[i] = (Real)pk[bb_plane[i]];
    bs[i] = (Real)ps[bb_plane[i]];
}

__global__ void k_gather_i32(const int* src, const long long* idx, int n, long long* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = src[idx[i]];
}

// caller order <-> internal order of one replica's coordinates / forces
__device__ __forceinline__ void put_pos(double* X, int j, const double v[3]) {
    Pos<double> p;
    p.x[0] = v[0]; p.x[1] = v[1]; p.x[2] = v[2];
    store_pos(X, j, p);
}
__device__ __forceinline__ void put_pos(float* X, int j, const double v[3]) { store_pos(X, j, split(v)); }

template <typename Real>
__global__ void k_scatter_coords(const double* in, const int* perm, int nb, int base, Real* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const double v[3] = {in[3 * (size_t)i], in[3 * (size_t)i + 1], in[3 * (size_t)i + 2]};
    put_pos(out, base + perm[i], v);
}

template <typename Real>
__global__ void k_gather_pos(const Real* X, const int* perm, int nb, int base, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    double v[3];
    to_double(load_pos(X, base + perm[i]), v);
    out[3 * (size_t)i] = v[0];
    out[3 * (size_t)i + 1] = v[1];
    out[3 * (size_t)i + 2] = v[2];
}

// Boundary load forces of one replica's filament ends (one thread per filament,
// end and monomer), planes in order as ForceFieldManager::computeLoadForces
// visits them (ForceFieldManager.cpp:292-311, BoundaryCylinderRepulsion.cpp:122-192,
// BoundaryCylinderRepulsionExp.cpp:113-118).  ends[2 f] / ends[2 f + 1]: the
// filament's first (minus-end) and last (plus-end) cylinder, replica-local.
struct LoadForceArgs {
    const int* ends;           // [2 * nfil]
    const int* fil_type;       // [nfil]
    const double* mon_size;    // per filament type
    const int* n_mon;          // per filament type
    int ntypes, nfil, stride;
    const int* cyl_b1;         // internal first bead of each (global) cylinder
    int cyl_begin, ncyl;
    const int* bcnt;           // boundary list entry counts of the last rebuild, replica's first entry
    int nplanes;
    const double* planes;      // replica's planes (a, b, c, d)
    const double* plane_k;
    const double* plane_slen;
    double* out;               // [nfil][2][stride]: minus end, then plus end
};
template <typename Real>
__global__ void k_load_forces(const Real* X, LoadForceArgs a) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2LL * a.nfil * a.stride) return;
    const int i = (int)(t % a.stride);
    const int e = (int)((t / a.stride) % 2);      // 0 minus end, 1 plus end
    const int f = (int)(t / (2LL * a.stride));
    const int c = a.ends[2 * f + e];
    const int ty = a.fil_type[f];
    double load = 0.0;
    if (ty >= 0 && ty < a.ntypes && i < a.n_mon[ty] && c >= 0 && c < a.ncyl) {
        const int b1 = a.cyl_b1[a.cyl_begin + c];
        double p1[3], p2[3];
        to_double(load_pos(X, b1), p1);
        to_double(load_pos(X, b1 + 1), p2);
        const double* bo = e ? p1 : p2;
        const double* bd = e ? p2 : p1;
        double dir[3] = {bd[0] - bo[0], bd[1] - bo[1], bd[2] - bo[2]};
        double m2 = 0.0;
        for (int k = 0; k < 3; ++k) m2 = __dadd_rn(m2, __dmul_rn(dir[k], dir[k]));
        const double nrm = __dsqrt_rn(m2);
        for (int k = 0; k < 3; ++k) dir[k] = __ddiv_rn(dir[k], nrm);
        const double step = __dmul_rn((double)i, a.mon_size[ty]);
        double x[3];
        for (int k = 0; k < 3; ++k) x[k] = __dadd_rn(bd[k], __dmul_rn(step, dir[k]));
        for (int p = 0; p < a.nplanes; ++p) {
            if (!a.bcnt[(long long)p * a.ncyl + c]) continue;
            const double* pl = a.planes + 4 * p;
            double dn = 0.0;
            for (int k = 0; k < 3; ++k) dn = __dadd_rn(dn, __dmul_rn(pl[k], dir[k]));
            const double proj = fmax(-dn, 0.0);
            double num = __dmul_rn(pl[0], x[0]);
            num = __dadd_rn(num, __dmul_rn(pl[1], x[1]));
            num = __dadd_rn(num, __dmul_rn(pl[2], x[2]));
            num = __dadd_rn(num, pl[3]);
            const double den = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(pl[0], pl[0]), __dmul_rn(pl[1], pl[1])),
                                                   __dmul_rn(pl[2], pl[2])));
            const double R = __ddiv_rn(-__ddiv_rn(num, den), a.plane_slen[p]);
            const double lf = __ddiv_rn(__dmul_rn(a.plane_k[p], exp(R)), a.plane_slen[p]);
            load = __dadd_rn(load, __dmul_rn(proj, lf));
        }
    }
    a.out[t] = load;
}

// Per-cylinder view of the per-bead filament energy terms the energy kernels
// stored (stretching of cylinder c, bending of the triple centred on its first
// bead; zero for a filament's first cylinder).
template <typename Real>
__global__ void k_terms_by_cylinder(const Real* terms, int nb, const int* cyl_b1, int cyl_begin, int ncyl,
                                    double* stretch, double* bend) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncyl) return;
    const int b = cyl_b1[cyl_begin + c];
    stretch[c] = terms[b];
    bend[c] = terms[(size_t)nb + b];
}

template <typename Real>
__global__ void k_gather_coords(const Real* in, const int* perm, int nb, int base, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const int j = base + perm[i];
    out[3 * (size_t)i] = (double)in[3 * (size_t)j];
    out[3 * (size_t)i + 1] = (double)in[3 * (size_t)j + 1];
    out[3 * (size_t)i + 2] = (double)in[3 * (size_t)j + 2];
}

__global__ void k_cg_init(CGState* st, int R) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    CGState& S = st[r];
    if (!S.active) return;
    S.numEnergyCall = 1;
    S.numForceCall = 1;
    S.prevEnergy = S.eval[MECH_NUM_FF];   // energiesBefore.total
    if (!isfinite(S.maxF)) {
        S.status = MECH_ERR_NONFINITE;
        S.phase = PH_ERROR;
        return;
    }
    S.phase = PH_RESET;                   // resetCGParams, then the loop head
}

// the replica's slice of the caller -> internal map (replica-local indices)
const int* perm_of(MechContext* c, int r) { return c->perm_all.as<int>() + c->reps[r].bead_begin; }

}  // namespace

// ===========================================================================
// network upload
// ===========================================================================
// bytes past the last bead of the position and direction buffers: bulk copies
// round bead ranges outward to 16-byte multiples and may read into it
static constexpr size_t kBulkPad = 256;

static int set_networks(MechContext* c, int R, const MechNetwork* nets) {
    if (R <= 0 || !nets) return set_err(MECH_ERR_ARG, "no networks");
    c->reps.assign(R, ReplicaHost());
    c->R = R;
    int nb = 0, ncyl = 0, nlk = 0, nmt = 0, npl = 0;
    std::vector<double> x, kstr, l0b, kbend, t0, cyl_kex, cyl_l0, lkk, lkl, lks1, lks2, mtk, mtl, mts1, mts2, planes,
        pk, ps;
    std::vector<uint8_t> flags, minus;
    std::vector<int> cyl_b1, cyl_fil, cyl_pos, cyl_rep, cyl_type;
    std::vector<int64_t> cyl_id;
    std::vector<int4> lkb, mtb;
    c->cyl_local_first.clear();
    for (int r = 0; r < R; ++r) {
        const MechNetwork& N = nets[r];
        ReplicaHost& h = c->reps[r];
        if (N.n_beads <= 0 || !N.coord || N.n_filaments <= 0 || !N.fil_cyl_start || N.n_cylinders <= 0 || !N.cyl_bead)
            return set_err(MECH_ERR_ARG, "replica " + std::to_string(r) + ": empty network");
        if (N.fil_cyl_start[0] != 0 || N.fil_cyl_start[N.n_filaments] != N.n_cylinders)
            return set_err(MECH_ERR_ARG, "fil_cyl_start does not cover the cylinders");
        h.nb = N.n_beads;
        h.bead_begin = nb;
        h.ncyl = N.n_cylinders;
        h.cyl_begin = ncyl;
        h.nfil = N.n_filaments;
        h.fil_end_cyl.resize(2 * (size_t)N.n_filaments);
        h.fil_type.resize(N.n_filaments);
        for (int f = 0; f < N.n_filaments; ++f) {
            h.fil_end_cyl[2 * (size_t)f] = N.fil_cyl_start[f];
            h.fil_end_cyl[2 * (size_t)f + 1] = N.fil_cyl_start[f + 1] - 1;
            h.fil_type[f] = N.cyl_type && N.fil_cyl_start[f + 1] > N.fil_cyl_start[f] ? N.cyl_type[N.fil_cyl_start[f]] : 0;
        }
        h.perm.assign(N.n_beads, -1);
        h.inv.assign(N.n_beads, -1);
        for (int k = 0; k < 3; ++k) h.box[k] = N.box[k];
        h.rmax = N.exvol_cutoff;
        h.bcut = N.boundary_cutoff;
        // internal bead order: filament by filament, minus end first
        int li = 0;
        std::vector<int> first_local(N.n_cylinders, -1);
        for (int f = 0; f < N.n_filaments; ++f) {
            const int cs = N.fil_cyl_start[f], ce = N.fil_cyl_start[f + 1];
            if (ce <= cs) return set_err(MECH_ERR_TOPOLOGY, "filament without cylinders");
            for (int cc = cs; cc < ce; ++cc) {
                const int b1 = N.cyl_bead[2 * cc], b2 = N.cyl_bead[2 * cc + 1];
                if (b1 < 0 || b2 < 0 || b1 >= N.n_beads || b2 >= N.n_beads)
                    return set_err(MECH_ERR_ARG, "cylinder bead out of range");
                if (cc == cs) {
                    if (h.perm[b1] != -1) return set_err(MECH_ERR_TOPOLOGY, "bead shared between filaments");
                    h.perm[b1] = li;
                    h.inv[li] = b1;
                    ++li;
                } else if (N.cyl_bead[2 * (cc - 1) + 1] != b1) {
                    return set_err(MECH_ERR_TOPOLOGY, "cylinders of a filament do not chain");
                }
                first_local[cc] = li - 1;
                if (h.perm[b2] != -1) return set_err(MECH_ERR_TOPOLOGY, "bead used twice");
                h.perm[b2] = li;
                h.inv[li] = b2;
                ++li;
            }
        }
        if (li != N.n_beads) return set_err(MECH_ERR_TOPOLOGY, "beads outside filaments");
        // bead arrays in internal order
        const size_t xoff = x.size();
        x.resize(xoff + 3 * (size_t)N.n_beads);
        flags.resize(nb + N.n_beads, 0);
        kstr.resize(nb + N.n_beads, 0.0);
        l0b.resize(nb + N.n_beads, 0.0);
        kbend.resize(nb + N.n_beads, 0.0);
        t0.resize(nb + N.n_beads, 0.0);
        for (int b = 0; b < N.n_beads; ++b)
            for (int k = 0; k < 3; ++k) x[xoff + 3 * (size_t)h.perm[b] + k] = N.coord[3 * (size_t)b + k];
        for (int f = 0; f < N.n_filaments; ++f) {
            const int cs = N.fil_cyl_start[f], ce = N.fil_cyl_start[f + 1];
            for (int cc = cs; cc < ce; ++cc) {
                const int j = nb + first_local[cc];   // slot of the cylinder's first bead
                flags[j] |= 1;
                flags[j + 1] |= 2;
                kstr[j] = N.cyl_k_stretch[cc];
                l0b[j] = N.cyl_eq_length[cc];
                // the bending triple centred on j uses the constants of cylinder (j, j+1)
                kbend[j] = N.cyl_k_bend[cc];
                t0[j] = N.cyl_eq_theta ? N.cyl_eq_theta[cc] : 0.0;
            }
        }
        for (int cc = 0; cc < N.n_cylinders; ++cc) {
            cyl_b1.push_back(nb + first_local[cc]);
            cyl_id.push_back(N.cyl_id[cc]);
            cyl_fil.push_back(N.cyl_filament_id[cc]);
            cyl_pos.push_back(N.cyl_position[cc]);
            cyl_rep.push_back(r);
            cyl_type.push_back(N.cyl_type ? N.cyl_type[cc] : 0);
            cyl_kex.push_back(N.cyl_k_exvol[cc]);
            cyl_l0.push_back(N.cyl_eq_length[cc]);
            c->cyl_local_first.push_back(nb + first_local[cc]);
        }
        minus.resize(ncyl + N.n_cylinders, 0);
        for (int f = 0; f < N.n_filaments; ++f) minus[ncyl + N.fil_cyl_start[f]] = 1;
        // linkers / motors
        auto bonds = [&](int n, const int32_t* cyl, const double* pos, const double* k, const double* eql,
                         std::vector<int4>& bead, std::vector<double>& kk, std::vector<double>& ll,
                         std::vector<double>& s1, std::vector<double>& s2) -> int {
            for (int i = 0; i < n; ++i) {
                const int c1 = cyl[2 * i], c2 = cyl[2 * i + 1];
                if (c1 < 0 || c2 < 0 || c1 >= N.n_cylinders || c2 >= N.n_cylinders) return MECH_ERR_ARG;
                const int a = nb + first_local[c1], b = nb + first_local[c2];
                bead.push_back(make_int4(a, a + 1, b, b + 1));
                kk.push_back(k[i]);
                ll.push_back(eql[i]);
                s1.push_back(pos[2 * i]);
                s2.push_back(pos[2 * i + 1]);
            }
            return MECH_OK;
        };
        h.lk_begin = nlk;
        h.nlk = N.n_linkers;
        if (N.n_linkers > 0 && bonds(N.n_linkers, N.lk_cyl, N.lk_pos, N.lk_k, N.lk_eq_length, lkb, lkk, lkl, lks1, lks2))
            return set_err(MECH_ERR_ARG, "linker cylinder out of range");
        h.mt_begin = nmt;
        h.nmt = N.n_motors;
        if (N.n_motors > 0 && bonds(N.n_motors, N.mt_cyl, N.mt_pos, N.mt_k, N.mt_eq_length, mtb, mtk, mtl, mts1, mts2))
            return set_err(MECH_ERR_ARG, "motor cylinder out of range");
        h.plane_begin = npl;
        h.nplanes = N.n_planes;
        for (int p = 0; p < N.n_planes; ++p) {
            for (int k = 0; k < 4; ++k) planes.push_back(N.planes[4 * p + k]);
            pk.push_back(N.plane_k[p]);
            ps.push_back(N.plane_screen[p]);
        }
        nb += N.n_beads;
        ncyl += N.n_cylinders;
        nlk += N.n_linkers;
        nmt += N.n_motors;
        npl += N.n_planes;
    }
    {
        std::vector<int> pa;
        pa.reserve(nb);
        for (int r = 0; r < R; ++r) pa.insert(pa.end(), c->reps[r].perm.begin(), c->reps[r].perm.end());
        int rc0 = upload(c->perm_all, pa, c->stream);
        if (rc0) return rc0;
        CU(c->stage.ensure(sizeof(double) * 3 * (size_t)std::max(nb, 1)));
    }
    c->nb = nb;
    c->ncyl = ncyl;
    c->nlk = nlk;
    c->nmt = nmt;
    c->nplanes = npl;
    cudaStream_t s = c->stream;
    const size_t rs = real_size(c);
    int rc;
    // positions in the engine's format (24 bytes per bead either way)
    {
        DeviceBuffer xd, ident;
        if ((rc = upload(xd, x, s))) return rc;
        std::vector<int> id(nb);
        for (int i = 0; i < nb; ++i) id[i] = i;
        if ((rc = upload(ident, id, s))) return rc;
        CU(c->x[0].ensure(sizeof(double) * x.size() + kBulkPad));
        if (c->precision == MECH_PREC_FP64)
            k_scatter_coords<double><<<(nb + 255) / 256, 256, 0, s>>>(xd.as<double>(), ident.as<int>(), nb, 0, c->x[0].as<double>());
        else
            k_scatter_coords<float><<<(nb + 255) / 256, 256, 0, s>>>(xd.as<double>(), ident.as<int>(), nb, 0, c->x[0].as<float>());
        CU(cudaGetLastError());
        CU(cudaStreamSynchronize(s));
    }
    CU(c->x[1].ensure(sizeof(double) * x.size() + kBulkPad));
    CU(cudaMemcpyAsync(c->x[1].p, c->x[0].p, sizeof(double) * x.size(), cudaMemcpyDeviceToDevice, s));
    if (c->precision == MECH_PREC_MIXED) {   // the second trial buffer of the two-trial line-search passes
        CU(c->x[2].ensure(sizeof(double) * x.size() + kBulkPad));
        CU(cudaMemcpyAsync(c->x[2].p, c->x[0].p, sizeof(double) * x.size(), cudaMemcpyDeviceToDevice, s));
    }
    CU(c->xbest.ensure(sizeof(double) * x.size()));
    CU(c->xinit.ensure(sizeof(double) * x.size()));
    CU(cudaMemcpyAsync(c->xinit.p, c->x[0].p, sizeof(double) * x.size(), cudaMemcpyDeviceToDevice, s));
    CU(c->f[0].ensure(rs * x.size() + kBulkPad));
    CU(c->f[1].ensure(rs * x.size() + kBulkPad));
    CU(c->d.ensure(rs * x.size() + kBulkPad));
    CU(cudaMemsetAsync(c->f[0].p, 0, rs * x.size(), s));
    CU(cudaMemsetAsync(c->f[1].p, 0, rs * x.size(), s));
    CU(cudaMemsetAsync(c->d.p, 0, rs * x.size(), s));
    flags.resize((size_t)nb + 32, 0);   // tail padding read by 16-byte-rounded bulk copies
    if ((rc = upload(c->bflag, flags, s))) return rc;
    {
        std::vector<double> par(4 * (size_t)nb);
        for (int i = 0; i < nb; ++i) {
            par[4 * (size_t)i] = kstr[i];
            par[4 * (size_t)i + 1] = l0b[i];
            par[4 * (size_t)i + 2] = kbend[i];
            par[4 * (size_t)i + 3] = t0[i];
        }
        if ((rc = upload_real(c, c->bpar, par))) return rc;
    }
    if ((rc = upload(c->cyl_b1, cyl_b1, s)) || (rc = upload(c->cyl_id, cyl_id, s)) || (rc = upload(c->cyl_fil, cyl_fil, s)) ||
        (rc = upload(c->cyl_pos, cyl_pos, s)) || (rc = upload(c->cyl_rep, cyl_rep, s)) || (rc = upload(c->cyl_type, cyl_type, s)) ||
        (rc = upload(c->cyl_kex, cyl_kex, s)) || (rc = upload(c->cyl_l0, cyl_l0, s)) || (rc = upload(c->cyl_minus, minus, s)))
        return rc;
    if ((rc = upload(c->lk_bead, lkb, s)) || (rc = upload_real(c, c->lk_k, lkk)) || (rc = upload_real(c, c->lk_l0, lkl)) ||
        (rc = upload_real(c, c->lk_s1, lks1)) || (rc = upload_real(c, c->lk_s2, lks2)))
        return rc;
    if ((rc = upload(c->mt_bead, mtb, s)) || (rc = upload_real(c, c->mt_k, mtk)) || (rc = upload_real(c, c->mt_l0, mtl)) ||
        (rc = upload_real(c, c->mt_s1, mts1)) || (rc = upload_real(c, c->mt_s2, mts2)))
        return rc;
    CU(c->lk_sf.ensure(sizeof(double) * std::max(nlk, 1)));
    CU(c->mt_sf.ensure(sizeof(double) * std::max(nmt, 1)));
    if ((rc = upload(c->planes, planes, s)) || (rc = upload(c->plane_k, pk, s)) || (rc = upload(c->plane_slen, ps, s)))
        return rc;
    // filament tiles (static)
    std::vector<Tile> ft;
    c->h_rt.assign(R, RepTiles{});
    for (int r = 0; r < R; ++r) {
        const ReplicaHost& h = c->reps[r];
        c->h_rt[r].fil_begin = (int)ft.size();
        for (int b = 0; b < h.nb; b += kFilTile)
            ft.push_back(Tile{r, h.bead_begin + b, h.bead_begin + std::min(h.nb, b + kFilTile), 0});
        c->h_rt[r].fil_end = (int)ft.size();
    }
    c->n_ftiles = (int)ft.size();
    c->h_ftiles = ft;
    c->compact = false;
    if ((rc = upload(c->ftile, ft, s))) return rc;
    CU(c->part_fil.ensure(sizeof(double) * 4 * ft.size()));
    // states
    CU(c->st.ensure(sizeof(CGState) * R));
    CU(cudaMemsetAsync(c->st.p, 0, sizeof(CGState) * R, s));
    CU(c->ticket.ensure(sizeof(int) * R));
    CU(cudaMemsetAsync(c->ticket.p, 0, sizeof(int) * R, s));
    CU(c->gticket.ensure(sizeof(int) * 4));
    CU(cudaMemsetAsync(c->gticket.p, 0, sizeof(int) * 4, s));
    CU(c->cond_counter.ensure(sizeof(int) * 8));
    CU(cudaMemsetAsync(c->cond_counter.p, 0, sizeof(int) * 8, s));
    CU(c->err.ensure(sizeof(unsigned) * 4));
    CU(cudaMemsetAsync(c->err.p, 0, sizeof(unsigned) * 4, s));
    CU(c->ev_fb_count.ensure(sizeof(int) * 4));
    CU(cudaMemsetAsync(c->ev_fb_count.p, 0, sizeof(int) * 4, s));
    CU(c->ev_fb_list.ensure(sizeof(int) * 2 * kExvolFallbackCap));
    CU(c->ev_fb_energy.ensure(sizeof(double) * 2 * kExvolFallbackCap));
    CU(c->fb_moments.ensure(sizeof(double) * 6 * kFbChunks * (size_t)kExvolFallbackCap));
    CU(c->fb_tickets.ensure(sizeof(int) * kExvolFallbackCap));
    CU(cudaMemsetAsync(c->fb_tickets.p, 0, sizeof(int) * kExvolFallbackCap, s));
    if (c->h_st) cudaFreeHost(c->h_st);
    CU(cudaMallocHost(&c->h_st, sizeof(CGState) * R));
    if (!c->h_err) CU(cudaMallocHost(&c->h_err, sizeof(unsigned) * 4));
    for (auto& k : c->snap) {
        if (k.st) cudaFreeHost(k.st);
        k.st = nullptr;
        CU(cudaMallocHost(&k.st, sizeof(CGState) * R));
        if (!k.err) CU(cudaMallocHost(&k.err, sizeof(unsigned) * 9));
        if (!k.done) CU(cudaEventCreateWithFlags(&k.done, cudaEventDisableTiming));
    }
    CU(cudaStreamSynchronize(s));
    c->have_net = true;
    c->have_lists = false;
    return MECH_OK;
}

// ===========================================================================
// neighbor lists
// ===========================================================================
// Bring every replica's current coordinates to x[0] (a replica whose last
// accepted step left them in a trial buffer is copied back) and reset its xbuf.
static int canonicalize_x(MechContext* c) {
    cudaStream_t s = c->stream;
    CU(cudaMemcpyAsync(c->h_st, c->st.p, sizeof(CGState) * c->R, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    bool moved = false;
    for (int r = 0; r < c->R; ++r) {
        if (c->h_st[r].xbuf) {
            const ReplicaHost& h = c->reps[r];
            CU(cudaMemcpyAsync(c->x[0].as<char>() + 24 * (size_t)h.bead_begin,
                               c->x[c->h_st[r].xbuf].as<char>() + 24 * (size_t)h.bead_begin,
                               24 * (size_t)h.nb, cudaMemcpyDeviceToDevice, s));
            c->h_st[r].xbuf = 0;
            moved = true;
        }
    }
    if (moved) CU(cudaMemcpyAsync(c->st.p, c->h_st, sizeof(CGState) * c->R, cudaMemcpyHostToDevice, s));
    return MECH_OK;
}

static int rebuild(MechContext* c, double cell_req, MechListInfo* info) {
    if (!c->have_net) return set_err(MECH_ERR_STATE, "no network");
    cudaStream_t s = c->stream;
    const int R = c->R;
    // per replica grid
    std::vector<double> rcell(R), rmax2(R), rmin2(R), bcut(R);
    std::vector<int4> dims(R);
    std::vector<float> margin(R);
    long long ncells = 0;
    for (int r = 0; r < R; ++r) {
        ReplicaHost& h = c->reps[r];
        double cell = cell_req;
        const double vol = std::max(1.0, h.box[0] * h.box[1] * h.box[2]);
        if (cell <= 0) {
            // about half a cylinder per cell; never below the reference's 1.125 rMax
            cell = std::max(1.125 * h.rmax, std::cbrt(vol / std::max(1, h.ncyl)) * 0.7937) * c->cell_scale;
        }
        cell = std::max(cell, h.rmax);
        auto g = [&](double L) { return std::max(1, (int)std::ceil(std::max(L, cell) / cell)); };
        h.gx = g(h.box[0]);
        h.gy = g(h.box[1]);
        h.gz = g(h.box[2]);
        // keep the cell array bounded: grow the edge until cells <= 8 * cylinders + 4096
        while ((long long)h.gx * h.gy * h.gz > 8LL * h.ncyl + 4096) {
            cell *= 1.25;
            h.gx = g(h.box[0]);
            h.gy = g(h.box[1]);
            h.gz = g(h.box[2]);
        }
        h.cell = cell;
        h.cell_off = ncells;
        ncells += (long long)h.gx * h.gy * h.gz;
        rcell[r] = cell;
        dims[r] = make_int4(h.gx, h.gy, h.gz, (int)h.cell_off);
        rmax2[r] = (double)(float)(h.rmax * h.rmax);
        rmin2[r] = 0.0;
        bcut[r] = h.bcut;
        // float-midpoint prefilter slack (coordinates up to a few boxes from the origin)
        const double M = 4.0 * std::max(h.box[0], std::max(h.box[1], h.box[2])) + 1e4;
        const double delta = (2.0 * M + h.rmax) * 6.0e-8;
        margin[r] = (float)(2.0 * h.rmax * std::sqrt(3.0) * delta + 3.0 * delta * delta + 4e-7 * h.rmax * h.rmax + 1e-2);
    }
    if (ncells > 2000000000LL) return set_err(MECH_ERR_CAPACITY, "bin grid too large");
    int rc;
    if ((rc = upload(c->rep_cell, rcell, s)) || (rc = upload(c->rep_dims, dims, s)) || (rc = upload(c->rep_rmax2, rmax2, s)) ||
        (rc = upload(c->rep_rmin2, rmin2, s)) || (rc = upload(c->rep_margin, margin, s)) || (rc = upload(c->rep_bcut, bcut, s)))
        return rc;
    NLInput in{};
    in.ncyl = c->ncyl;
    in.cyl_b1 = c->cyl_b1.as<int>();
    in.cyl_id = c->cyl_id.as<int64_t>();
    in.cyl_fil = c->cyl_fil.as<int>();
    in.cyl_pos = c->cyl_pos.as<int>();
    in.cyl_rep = c->cyl_rep.as<int>();
    // current coordinates: replica buffers may differ; gather them into x[0] first
    in.x = nullptr;
    in.rep_cell = c->rep_cell.as<double>();
    in.rep_dims = c->rep_dims.as<int4>();
    in.rep_rmax2 = c->rep_rmax2.as<double>();
    in.rep_rmin2 = c->rep_rmin2.as<double>();
    in.R = R;
    in.ncells = ncells;
    // Current coordinates live in x[xbuf] per replica; canonicalize them to
    // x[0] (and reset xbuf) so the lists read one array.
    if ((rc = canonicalize_x(c))) return rc;
    in.x = c->x[0].p;
    in.mixed = c->precision == MECH_PREC_MIXED;
    long long P = 0;
    CU(build_pairs(in, c->pb, c->rep_margin.as<float>(), &P, s));
    c->nev = P;
    // per replica pair ranges: pair offsets at the replicas' first cylinders
    {
        std::vector<long long> idx(R + 1);
        for (int r = 0; r < R; ++r) idx[r] = c->reps[r].cyl_begin;
        idx[R] = c->ncyl;
        if ((rc = upload(c->gather_idx, idx, s))) return rc;
        CU(c->gather_out.ensure(sizeof(long long) * (R + 1)));
        k_gather_i32<<<(R + 1 + 127) / 128, 128, 0, s>>>(c->pb.off.as<int>(), c->gather_idx.as<long long>(), R + 1,
                                                      c->gather_out.as<long long>());
        std::vector<long long> o(R + 1);
        CU(cudaMemcpyAsync(o.data(), c->gather_out.p, sizeof(long long) * (R + 1), cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        for (int r = 0; r < R; ++r) {
            c->reps[r].ev_begin = o[r];
            c->reps[r].nev = o[r + 1] - o[r];
        }
    }
    const size_t rs = real_size(c);
    CU(c->ev_bead.ensure(sizeof(int4) * std::max<long long>(P, 1)));
    CU(c->ev_k.ensure(rs * std::max<long long>(P, 1)));
    CU(c->ev_la.ensure(rs * std::max<long long>(P, 1)));
    CU(c->ev_lb.ensure(rs * std::max<long long>(P, 1)));
    // the extended-pass list holds up to two entries per pair (both trials of a two-trial pass)
    CU(c->ev_list.ensure(sizeof(int) * 4 * std::max<long long>(P, 1)));
    CU(c->ev_energy.ensure(sizeof(double) * std::max<long long>(P, 1)));
    CU(c->ev_energy2.ensure(sizeof(double) * std::max<long long>(P, 1)));
    CU(c->ev_list_count.ensure(sizeof(int) * 4));
    CU(cudaMemsetAsync(c->ev_list_count.p, 0, sizeof(int) * 4, s));
    if (P > 0) {
        const unsigned nbk = (unsigned)((P + 255) / 256);
        if (c->precision == MECH_PREC_FP64)
            k_ev_build<double><<<nbk, 256, 0, s>>>(c->pb.pairs.as<int2>(), P, c->cyl_b1.as<int>(), c->cyl_kex.as<double>(),
                                                   c->cyl_type.as<int>(), c->cyl_l0.as<double>(), c->ev_bead.as<int4>(),
                                                   c->ev_k.as<double>(), c->ev_la.as<double>(), c->ev_lb.as<double>());
        else
            k_ev_build<float><<<nbk, 256, 0, s>>>(c->pb.pairs.as<int2>(), P, c->cyl_b1.as<int>(), c->cyl_kex.as<double>(),
                                                  c->cyl_type.as<int>(), c->cyl_l0.as<double>(), c->ev_bead.as<int4>(),
                                                  c->ev_k.as<float>(), c->ev_la.as<float>(), c->ev_lb.as<float>());
    }
    // boundary lists
    {
        std::vector<long long> rq(R);
        std::vector<int> rnc(R), rpl(R), rcy(R);
        long long nq = 0;
        for (int r = 0; r < R; ++r) {
            rq[r] = nq;
            rnc[r] = c->reps[r].ncyl;
            rpl[r] = c->reps[r].plane_begin;
            rcy[r] = c->reps[r].cyl_begin;
            nq += (long long)c->reps[r].nplanes * c->reps[r].ncyl;
        }
        if ((rc = upload(c->rep_q, rq, s)) || (rc = upload(c->rep_ncyl, rnc, s)) || (rc = upload(c->rep_plane, rpl, s)) ||
            (rc = upload(c->rep_cyl, rcy, s)))
            return rc;
        BndInput bi{};
        bi.nq = nq;
        bi.R = R;
        bi.rep_q = c->rep_q.as<long long>();
        bi.rep_ncyl = c->rep_ncyl.as<int>();
        bi.rep_plane = c->rep_plane.as<int>();
        bi.rep_cyl = c->rep_cyl.as<int>();
        bi.cutoff = c->rep_bcut.as<double>();
        bi.planes = c->planes.as<double>();
        bi.cyl_b1 = c->cyl_b1.as<int>();
        bi.cyl_minus = c->cyl_minus.as<uint8_t>();
        long long nbb = 0, nbcyl = 0;
        CU(build_boundary(bi, c->pb.mid.as<double>(), c->bbuild, &nbb, &nbcyl, s));
        c->nbb = nbb;
        c->nbcyl = nbcyl;
        for (int r = 0; r < R; ++r) c->reps[r].bq_begin = rq[r];
        std::vector<long long> idx(R + 1);
        for (int r = 0; r < R; ++r) idx[r] = rq[r];
        idx[R] = nq;
        if ((rc = upload(c->gather_idx, idx, s))) return rc;
        k_gather_i32<<<(R + 1 + 127) / 128, 128, 0, s>>>(c->bbuild.off.as<int>(), c->gather_idx.as<long long>(), R + 1,
                                                      c->gather_out.as<long long>());
        std::vector<long long> o(R + 1);
        CU(cudaMemcpyAsync(o.data(), c->gather_out.p, sizeof(long long) * (R + 1), cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        for (int r = 0; r < R; ++r) {
            c->reps[r].bb_begin = o[r];
            c->reps[r].nbb = o[r + 1] - o[r];
        }
        CU(c->bb_k.ensure(rs * std::max<long long>(nbb, 1)));
        CU(c->bb_slen.ensure(rs * std::max<long long>(nbb, 1)));
        if (nbb > 0) {
            const unsigned nbk = (unsigned)((nbb + 255) / 256);
            if (c->precision == MECH_PREC_FP64)
                k_bb_build<double><<<nbk, 256, 0, s>>>(c->bbuild.plane.as<int>(), nbb, c->plane_k.as<double>(),
                                                       c->plane_slen.as<double>(), c->bb_k.as<double>(), c->bb_slen.as<double>());
            else
                k_bb_build<float><<<nbk, 256, 0, s>>>(c->bbuild.plane.as<int>(), nbb, c->plane_k.as<double>(),
                                                      c->plane_slen.as<double>(), c->bb_k.as<float>(), c->bb_slen.as<float>());
        }
    }
    // sparse tiles: linker, motor, exvol, boundary; each replica's interactions tiled separately
    {
        std::vector<Tile> st;
        std::vector<int> kind;
        for (int k = 0; k < K_NUM_SPARSE; ++k) {
            const int t0 = (int)st.size();
            for (int r = 0; r < R; ++r) {
                const ReplicaHost& h = c->reps[r];
                long long b = 0, n = 0;
                if (k == K_LINKER) { b = h.lk_begin; n = h.nlk; }
                if (k == K_MOTOR) { b = h.mt_begin; n = h.nmt; }
                if (k == K_EXVOL) { b = h.ev_begin; n = h.nev; }
                if (k == K_BOUNDARY) { b = h.bb_begin; n = h.nbb; }
                c->h_rt[r].sp_begin[k] = (int)st.size();
                for (long long i = 0; i < n; i += kSparseTile) {
                    st.push_back(Tile{r, (int)(b + i), (int)(b + std::min<long long>(n, i + kSparseTile)), 0});
                    kind.push_back(k);
                }
                c->h_rt[r].sp_end[k] = (int)st.size();
            }
            c->sp_tiles[k] = (int)st.size() - t0;
        }
        c->n_stiles = (int)st.size();
        c->h_stiles = st;
        c->h_skind = kind;
        c->compact = false;
        if ((rc = upload(c->stile, st, s)) || (rc = upload(c->stile_kind, kind, s)) || (rc = upload(c->rt, c->h_rt, s)))
            return rc;
        CU(c->part_sp.ensure(sizeof(double) * std::max<size_t>(st.size(), 1)));
        CU(c->part_sp2.ensure(sizeof(double) * std::max<size_t>(st.size(), 1)));
    }
    // contribution slots and the gather index
    c->slot_base[K_LINKER] = 0;
    c->slot_base[K_MOTOR] = 4 * c->nlk;
    c->slot_base[K_EXVOL] = 4 * c->nlk + 4 * c->nmt;
    c->slot_base[K_BOUNDARY] = (int)(c->slot_base[K_EXVOL] + 4 * P);
    c->slot_base[K_NUM_SPARSE] = (int)(c->slot_base[K_BOUNDARY] + c->nbb);
    CU(c->contrib.ensure(rs * 3 * std::max(1, c->slot_base[K_NUM_SPARSE])));
    CU(cudaMemsetAsync(c->contrib.p, 0, rs * 3 * std::max(1, c->slot_base[K_NUM_SPARSE]), s));
    {
        CsrInput ci{};
        ci.nb = c->nb;
        for (int k = 0; k <= K_NUM_SPARSE; ++k) ci.base[k] = c->slot_base[k];
        ci.lk = c->lk_bead.as<int4>();
        ci.mt = c->mt_bead.as<int4>();
        ci.ev = c->ev_bead.as<int4>();
        ci.bb = c->bbuild.bead.as<int>();
        CU(build_csr(ci, c->cb, s));
    }
    CU(cudaStreamSynchronize(s));
    CU(cudaGetLastError());
    c->have_lists = true;
    if (info) {
        info->n_exvol_pairs = P;
        info->n_boundary_beads = c->nbb;
        info->n_boundary_cyl = c->nbcyl;
        info->cell_size = c->reps[0].cell;
        info->n_cells = ncells;
    }
    return MECH_OK;
}

// ===========================================================================
// evaluation and minimization
// ===========================================================================
static int pull_states(MechContext* c) {
    CU(cudaMemcpyAsync(c->h_st, c->st.p, sizeof(CGState) * c->R, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(c->h_err, c->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return MECH_OK;
}
// Status of the device error word's bits (kernels set them with atomicOr).
static int err_status(unsigned bits) {
    if (bits & 64u) return set_err(MECH_ERR_ITER_LIMIT, "a grid barrier of the cooperative iteration tail timed out");
    if (bits & 32u) return set_err(MECH_ERR_ITER_LIMIT, "a bulk shared-memory copy did not complete in time");
    if (bits & 16u) return set_err(MECH_ERR_CUDA, "a bulk shared-memory copy range was misaligned");
    if (bits & 1u) return set_err(MECH_ERR_NONFINITE, "excluded-volume numeric fallback failed");
    if (bits & 8u) return set_err(MECH_ERR_NONFINITE, "non-finite excluded-volume Hessian term");
    return set_err(MECH_ERR_CAPACITY, "excluded-volume work list overflow");
}

static int push_states(MechContext* c) {
    CU(cudaMemcpyAsync(c->st.p, c->h_st, sizeof(CGState) * c->R, cudaMemcpyHostToDevice, c->stream));
    return MECH_OK;
}

template <typename Real>
static int eval_energy(MechContext* c, int replica) {
    int rc;
    if ((rc = pull_states(c))) return rc;
    for (int r = 0; r < c->R; ++r) c->h_st[r].active = (replica < 0 || r == replica);
    if ((rc = push_states(c))) return rc;
    CU(cudaMemsetAsync(c->err.p, 0, sizeof(unsigned), c->stream));
    const DevNet<Real> n = make_devnet<Real>(c);
    c->timing.launches += launch_energy<Real>(n, -1, 0, c->lanes());
    CU(cudaGetLastError());
    return pull_states(c);
}

template <typename Real>
static int eval_forces(MechContext* c, int replica) {
    int rc;
    if ((rc = pull_states(c))) return rc;
    for (int r = 0; r < c->R; ++r) c->h_st[r].active = (replica < 0 || r == replica);
    if ((rc = push_states(c))) return rc;
    CU(cudaMemsetAsync(c->err.p, 0, sizeof(unsigned), c->stream));
    const DevNet<Real> n = make_devnet<Real>(c);
    c->timing.launches += launch_forces<Real>(n, -1, c->lanes());
    CU(cudaGetLastError());
    return pull_states(c);
}

static constexpr int kBlocksPerGraph = 8;
// Line-search launches per iteration block: FP64, two single-trial passes;
// mixed, one two-trial pass (lambda and lambda / 2).
template <typename Real>
static int trial_launches(const DevNet<Real>& n, const Lanes& L) {
    if constexpr (sizeof(Real) == 4) return launch_energy<Real>(n, PH_LS_TRIAL, kTrialDual, L);
    return launch_energy<Real>(n, PH_LS_TRIAL, 1, L) + launch_energy<Real>(n, PH_LS_TRIAL, 1, L);
}

template <typename Real>
static int capture_iteration_graph(MechContext* c, cudaGraphExec_t* exec, int* nlaunch) {
    DevNet<Real> n = make_devnet<Real>(c);
    n.pdl = c->graph_mode == MECH_GRAPH_UNROLLED_PDL ? 1 : 0;
    // the cooperative tail: mixed engine, one replica (its blocks reduce for replica 0)
    int coop_grid = 0;
    if (c->graph_mode == MECH_GRAPH_UNROLLED_COOP && sizeof(Real) == 4 && c->R == 1) {
        coop_grid = coop_tail_grid(c->device);
        if (coop_grid <= 0) return set_err(MECH_ERR_CUDA, "cooperative tail: no resident blocks");
        CU(c->gbar.ensure(2 * sizeof(unsigned)));
        CU(cudaMemsetAsync(c->gbar.p, 0, 2 * sizeof(unsigned), c->stream));
        n.gbar = c->gbar.as<unsigned>();
    }
    cudaGraph_t g = nullptr;
    CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int k = 0;
    for (int b = 0; b < kBlocksPerGraph; ++b) {
        k += trial_launches<Real>(n, c->lanes());
        if (coop_grid > 0) {
            k += launch_forces<Real>(n, PH_FORCE, c->lanes(), coop_grid);
            continue;
        }
        k += launch_forces<Real>(n, PH_FORCE, c->lanes());
        k += launch_direction<Real>(n, c->stream);
        k += launch_reset<Real>(n, c->stream);
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return set_err(MECH_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(exec, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_err(MECH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    *nlaunch = k;
    return MECH_OK;
}

// Kernels per body part of the conditional graph (for the launch count).
struct CondGraphCounts {
    int head, trial, force, dir, misc;
};
static constexpr int kBodiesPerLaunch = 512;

// The minimizer as one conditional graph: a while loop whose body is
//   head -> if (trial) energy at x + lambda d -> if (force) forces
//        -> if (direction) d = F + beta d -> if (misc) reset (d = F).
// The head sets the four conditions from the replicas' phases and whether the
// loop runs another body; each phase's reduction sets them again for the
// phases after it in the same body.  Only phases some replica is in run, and
// control returns to the host when no replica has device work left, a
// recovery move or an error needs the host, or kBodiesPerLaunch bodies ran.
// The active kernels and their order are those of the unrolled graph.
template <typename Real>
static int capture_conditional_graph(MechContext* c, cudaGraphExec_t* exec, CondGraphCounts* counts) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    auto fail = [&](cudaError_t err, const char* what) {
        if (g) cudaGraphDestroy(g);
        return set_err(MECH_ERR_CUDA, std::string("conditional graph, ") + what + ": " + cudaGetErrorString(err));
    };
    if (e != cudaSuccess) return fail(e, "create");
    cudaMemsetParams mp{};
    mp.dst = c->cond_counter.p;
    mp.value = 0;
    mp.elementSize = 4;
    mp.width = 8;
    mp.height = 1;
    cudaGraphNode_t reset_node = nullptr;
    if ((e = cudaGraphAddMemsetNode(&reset_node, g, nullptr, 0, &mp)) != cudaSuccess) return fail(e, "counter reset");
    cudaGraphConditionalHandle h_loop = 0;
    if ((e = cudaGraphConditionalHandleCreate(&h_loop, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess)
        return fail(e, "loop handle");
    cudaGraphNodeParams wp{};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = h_loop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t loop_node = nullptr;
    if ((e = cudaGraphAddNode(&loop_node, g, &reset_node, nullptr, 1, &wp)) != cudaSuccess) return fail(e, "loop node");
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    cudaGraphConditionalHandle h[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; ++k)
        if ((e = cudaGraphConditionalHandleCreate(&h[k], body, 0, 0)) != cudaSuccess) return fail(e, "phase handle");
    DevNet<Real> n = make_devnet<Real>(c);
    n.cond = GraphConds{h[0], h[1], h[2], h[3], h_loop, c->cond_counter.as<int>(), kBodiesPerLaunch, 1};
    // capture `fn` into `graph` after `dep` (none when null)
    auto capture_into = [&](cudaGraph_t graph, const cudaGraphNode_t* dep, auto&& fn) -> cudaError_t {
        cudaError_t err = cudaStreamBeginCaptureToGraph(c->stream, graph, dep, nullptr, dep ? 1 : 0,
                                                        cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) return err;
        fn();
        cudaGraph_t out = nullptr;
        return cudaStreamEndCapture(c->stream, &out);
    };
    if ((e = capture_into(body, nullptr, [&] { counts->head = launch_body_head<Real>(n, c->stream); })) != cudaSuccess)
        return fail(e, "head capture");
    cudaGraphNode_t prev = nullptr;
    size_t nn = 1;
    if ((e = cudaGraphGetNodes(body, &prev, &nn)) != cudaSuccess || nn != 1) return fail(e, "head node");
    auto add_if = [&](cudaGraphConditionalHandle hc, auto&& fn) -> cudaError_t {
        cudaGraphNodeParams ip{};
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = hc;
        ip.conditional.type = cudaGraphCondTypeIf;
        ip.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        cudaError_t err = cudaGraphAddNode(&node, body, &prev, nullptr, 1, &ip);
        if (err != cudaSuccess) return err;
        prev = node;
        return capture_into(ip.conditional.phGraph_out[0], nullptr, fn);
    };
    if ((e = add_if(h[0], [&] {
             counts->trial = launch_energy<Real>(n, PH_LS_TRIAL, sizeof(Real) == 4 ? kTrialDual : 1, c->lanes());
         })) != cudaSuccess)
        return fail(e, "trial body");
    if ((e = add_if(h[1], [&] { counts->force = launch_forces<Real>(n, PH_FORCE, c->lanes()); })) != cudaSuccess)
        return fail(e, "force body");
    if ((e = add_if(h[2], [&] { counts->dir = launch_direction<Real>(n, c->stream); })) != cudaSuccess)
        return fail(e, "direction body");
    if ((e = add_if(h[3], [&] {
             counts->misc = launch_reset<Real>(n, c->stream);
         })) != cudaSuccess)
        return fail(e, "reset body");
    e = cudaGraphInstantiate(exec, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    g = nullptr;
    if (e != cudaSuccess) return set_err(MECH_ERR_CUDA, std::string("conditional graph, instantiate: ") + cudaGetErrorString(e));
    return MECH_OK;
}

// Tile lists of the replicas still minimizing (in the same order, with the
// same per-replica tile counts, so tickets and partial slots work unchanged);
// finished replicas get empty ranges.  The kernels' grids then cover only the
// remaining work.
static int compact_tiles(MechContext* c, const std::vector<char>& active) {
    std::vector<Tile> ft, st;
    std::vector<int> kind;
    std::vector<RepTiles> rt(c->R, RepTiles{});
    for (int r = 0; r < c->R; ++r) {
        if (!active[r]) continue;
        const RepTiles& full = c->h_rt[r];
        rt[r].fil_begin = (int)ft.size();
        ft.insert(ft.end(), c->h_ftiles.begin() + full.fil_begin, c->h_ftiles.begin() + full.fil_end);
        rt[r].fil_end = (int)ft.size();
    }
    for (int k = 0; k < K_NUM_SPARSE; ++k) {
        const int t0 = (int)st.size();
        for (int r = 0; r < c->R; ++r) {
            if (!active[r]) continue;
            const RepTiles& full = c->h_rt[r];
            rt[r].sp_begin[k] = (int)st.size();
            st.insert(st.end(), c->h_stiles.begin() + full.sp_begin[k], c->h_stiles.begin() + full.sp_end[k]);
            kind.insert(kind.end(), (size_t)(full.sp_end[k] - full.sp_begin[k]), k);
            rt[r].sp_end[k] = (int)st.size();
        }
        c->sp_tiles_c[k] = (int)st.size() - t0;
    }
    int rc;
    if ((rc = upload(c->ftile_c, ft, c->stream)) || (rc = upload(c->stile_c, st, c->stream)) ||
        (rc = upload(c->stile_kind_c, kind, c->stream)) || (rc = upload(c->rt_c, rt, c->stream)))
        return rc;
    c->n_ftiles_c = (int)ft.size();
    c->n_stiles_c = (int)st.size();
    c->compact = true;
    return MECH_OK;
}

template <typename Real>
static int minimize_impl(MechContext* c, const MechCGParams* p, MechResult* res) {
    struct FullTilesOnExit {
        MechContext* c;
        ~FullTilesOnExit() { c->compact = false; }
    } full_tiles_on_exit{c};
    if (!c->have_lists) {
        int rc = rebuild(c, 0.0, nullptr);
        if (rc) return rc;
    }
    auto t_start = std::chrono::steady_clock::now();
    cudaStream_t s = c->stream;
    int rc;
    if ((rc = pull_states(c))) return rc;
    for (int r = 0; r < c->R; ++r) {
        CGState& S = c->h_st[r];
        const int xb = S.xbuf, fb = S.fbuf;
        std::memset(&S, 0, sizeof(S));
        S.xbuf = xb;
        S.fbuf = fb;
        S.method = p->method;
        S.maxDist = p->max_dist;
        S.lambdaMax = p->lambda_max;
        S.gradTol = p->grad_tol;
        S.energyRelTol = p->energy_rel_tol;
        S.energyCallLimit = p->energy_call_limit;
        S.forceCallLimit = std::max(p->force_call_limit, 3 * c->reps[r].nb);
        S.tryToRecover = p->try_to_recover;
        S.minimumE = std::numeric_limits<double>::infinity();
        S.maxF = std::numeric_limits<double>::infinity();
        S.energyRelChange = std::numeric_limits<double>::infinity();
        S.active = 1;
        S.phase = PH_IDLE;
    }
    if ((rc = push_states(c))) return rc;
    CU(cudaMemsetAsync(c->err.p, 0, sizeof(unsigned), s));
    c->compact = false;
    DevNet<Real> n = make_devnet<Real>(c);
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    CU(cudaEventRecord(e0, s));
    // energiesBefore, initial forces, resetCGParams, loop head
    long long launches = 0;
    launches += launch_energy<Real>(n, -1, 0, c->lanes());
    launches += launch_forces<Real>(n, -1, c->lanes());
    k_cg_init<<<(c->R + 127) / 128, 128, 0, s>>>(n.st, c->R);
    launches += 1 + launch_reset<Real>(n, s);
    CU(cudaGetLastError());
    if ((rc = pull_states(c))) return rc;
    std::vector<std::vector<double>> before(c->R);
    for (int r = 0; r < c->R; ++r) before[r].assign(c->h_st[r].eval, c->h_st[r].eval + MECH_NUM_FF + 1);
    cudaGraphExec_t exec = nullptr;
    int per_graph = 0;
    CondGraphCounts cc{};
    const bool conditional = c->graph_mode == MECH_GRAPH_CONDITIONAL;
    auto build_graph = [&]() {
        return conditional ? capture_conditional_graph<Real>(c, &exec, &cc)
                           : capture_iteration_graph<Real>(c, &exec, &per_graph);
    };
    if ((rc = build_graph())) return rc;
    long long graphs = 0;
    long long max_graphs = 0;
    for (int r = 0; r < c->R; ++r)
        max_graphs = std::max<long long>(max_graphs, 4LL * c->h_st[r].forceCallLimit / kBlocksPerGraph + 1000);
    int status = MECH_OK;
    // The next graph is launched before the host reads the snapshot of the
    // previous one, so the device does not idle while the host checks the
    // states.  A launch after every replica has finished, or while one waits
    // for the host, only runs kernels that find nothing to do; before acting
    // on a finished, failed or compactable state the host drains the launch
    // in flight and acts on the newest snapshot.
    auto launch = [&](int k) -> int {
        CU(cudaGraphLaunch(exec, s));
        ++graphs;
        auto& sn = c->snap[k];
        CU(cudaMemcpyAsync(sn.st, c->st.p, sizeof(CGState) * c->R, cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(sn.err, c->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        if (conditional)   // bodies and phases this launch ran
            CU(cudaMemcpyAsync(sn.err + 1, c->cond_counter.p, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
        CU(cudaEventRecord(sn.done, s));
        return MECH_OK;
    };
    // launches of snapshot k's graph (the conditional graph counts what its bodies ran)
    auto account = [&](int k) {
        const int* bc = reinterpret_cast<const int*>(c->snap[k].err + 1);
        launches += conditional ? (long long)bc[0] * cc.head + (long long)bc[2] * cc.trial +
                                      (long long)bc[3] * cc.force + (long long)bc[4] * cc.dir + (long long)bc[5] * cc.misc
                                : per_graph;
    };
    auto wants_host = [&](const CGState* st, unsigned err, bool* all_done) {
        bool done = true, host = false;
        long long live = 0;
        for (int r = 0; r < c->R; ++r) {
            const int ph = st[r].phase;
            const bool act = ph != PH_DONE && ph != PH_ERROR;
            if (act) {
                done = false;
                live += c->h_rt[r].fil_end - c->h_rt[r].fil_begin;
            }
            if (ph == PH_RECOVER) host = true;
        }
        *all_done = done;
        // batched runs: relaunch over the live replicas once they hold at most half of the tiles
        const bool compactable = c->R > 1 && !done && 2 * live <= (long long)n.n_ftiles;
        return err != 0 || done || host || compactable || graphs > max_graphs;
    };
    int cur = 0;
    if ((rc = launch(cur))) { cudaGraphExecDestroy(exec); return rc; }
    for (;;) {
        const int nxt = cur ^ 1;
        if ((rc = launch(nxt))) { cudaGraphExecDestroy(exec); return rc; }
        CU(cudaEventSynchronize(c->snap[cur].done));
        account(cur);
        bool all_done = false;
        if (!wants_host(c->snap[cur].st, *c->snap[cur].err, &all_done)) {
            cur = nxt;
            continue;
        }
        // drain the launch in flight and act on its (newest) snapshot
        CU(cudaEventSynchronize(c->snap[nxt].done));
        account(nxt);
        std::memcpy(c->h_st, c->snap[nxt].st, sizeof(CGState) * c->R);
        *c->h_err = *c->snap[nxt].err;
        if (*c->h_err) {
            status = err_status(*c->h_err);
            break;
        }
        bool recover = false;
        std::vector<char> act(c->R, 0);
        long long live = 0;
        all_done = true;
        for (int r = 0; r < c->R; ++r) {
            const int ph = c->h_st[r].phase;
            act[r] = ph != PH_DONE && ph != PH_ERROR;
            if (act[r]) {
                all_done = false;
                live += c->h_rt[r].fil_end - c->h_rt[r].fil_begin;
            }
            if (ph == PH_RECOVER) recover = true;
        }
        if (all_done) break;
        if (graphs > max_graphs) {
            status = set_err(MECH_ERR_ITER_LIMIT, "minimizer loop exceeded its iteration cap");
            break;
        }
        if (recover) {
            launches += launch_recover<Real>(n, c->lanes());
            CU(cudaGetLastError());
        }
        if (c->R > 1 && 2 * live <= (long long)n.n_ftiles) {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
            if ((rc = compact_tiles(c, act))) { c->compact = false; return rc; }
            n = make_devnet<Real>(c);
            if ((rc = build_graph())) { c->compact = false; return rc; }
        }
        cur = nxt ^ 1;
        if ((rc = launch(cur))) { cudaGraphExecDestroy(exec); return rc; }
    }
    CU(cudaStreamSynchronize(s));
    if (exec) cudaGraphExecDestroy(exec);
    c->compact = false;   // the full lists again for energiesAfter and later calls
    n = make_devnet<Real>(c);
    // call-limit exit restores the minimum-energy backup (CGMethod.hpp:1589-1610)
    bool restore = false;
    for (int r = 0; r < c->R; ++r) {
        CGState& S = c->h_st[r];
        const bool limit = (S.energyCallLimit != 0 && S.numEnergyCall > S.energyCallLimit) ||
                           (S.forceCallLimit != 0 && S.numForceCall > S.forceCallLimit);
        S.restore = (p->report_on_call_limit && limit && S.backupValid) ? 1 : 0;
        restore = restore || S.restore;
        S.active = 1;
    }
    if ((rc = push_states(c))) return rc;
    if (restore) launches += launch_backup_restore<Real>(n, s);
    launches += launch_energy<Real>(n, -1, 0, c->lanes());   // energiesAfter
    CU(cudaEventRecord(e1, s));
    if ((rc = pull_states(c))) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    c->timing.ms_total = ms;
    c->timing.launches = launches;
    c->timing.graph_launches = graphs;
    for (int r = 0; r < c->R; ++r) {
        const CGState& S = c->h_st[r];
        MechResult& o = res[r];
        std::memset(&o, 0, sizeof(o));
        o.error_flags = (uint32_t)S.errorFlags;
        o.status = status != MECH_OK ? status : (S.phase == PH_ERROR ? S.status : (S.errorFlags ? MECH_ERR_LINESEARCH : MECH_OK));
        o.num_energy_call = S.numEnergyCall + 1;
        o.energy_call_limit = S.energyCallLimit;
        o.num_force_call = S.numForceCall;
        o.force_call_limit = S.forceCallLimit;
        o.num_iter = S.numIter;
        o.num_safe_mode = S.numSafeMode;
        o.num_recover = S.numRecover;
        o.num_line_search_trials = S.numTrials;
        o.num_energy_eval = S.numEnergyEval;
        o.used_backup = S.restore;
        o.grad_inf_norm = S.maxF;
        o.grad_tol = S.gradTol;
        o.energy_rel_change = S.energyRelChange;
        o.energy_rel_tol = S.energyRelTol;
        for (int k = 0; k <= MECH_NUM_FF; ++k) {
            o.energies_before[k] = before[r][k];
            o.energies_after[k] = S.eval[k];
        }
        o.seconds = secs;
    }
    return status;
}

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int32_t mech_abi_version(void) { return MECH_ABI_VERSION; }
const char* mech_last_error(void) { return g_last_error.c_str(); }

int32_t mech_ctx_create(int32_t precision, int32_t device, MechContext** out) {
    if (!out) return set_err(MECH_ERR_ARG, "out is null");
    if (precision != MECH_PREC_FP64 && precision != MECH_PREC_MIXED) return set_err(MECH_ERR_ARG, "bad precision");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_err(MECH_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev) return set_err(MECH_ERR_ARG, "bad device");
    CU(cudaSetDevice(device));
    MechContext* c = new MechContext();
    c->device = device;
    c->precision = precision;
    // The sparse lanes get the device's highest stream priority (kept by the
    // kernel nodes captured from them): the excluded-volume chain is the
    // longest lane, and the persistent filament kernel on the main lane would
    // otherwise fill the register files before its blocks are placed.
    int prio_least = 0, prio_greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->side2, cudaStreamNonBlocking, prio_greatest);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join2, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete c;
        return set_err(MECH_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = c;
    return MECH_OK;
}

int32_t mech_ctx_destroy(MechContext* ctx) {
    if (!ctx) return MECH_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->side);
    cudaStreamSynchronize(ctx->side2);
    cudaStreamSynchronize(ctx->stream);
    delete ctx;
    return MECH_OK;
}

int32_t mech_set_networks(MechContext* ctx, int32_t n_replicas, const MechNetwork* nets) {
    if (!ctx) return set_err(MECH_ERR_ARG, "null context");
    CU(cudaSetDevice(ctx->device));
    const int rc = set_networks(ctx, n_replicas, nets);
    if (rc) return rc;
    return rebuild(ctx, 0.0, nullptr);
}

static int check_replica(MechContext* ctx, int32_t r) {
    if (!ctx) return set_err(MECH_ERR_ARG, "null context");
    if (!ctx->have_net) return set_err(MECH_ERR_STATE, "no network");
    if (r < 0 || r >= ctx->R) return set_err(MECH_ERR_ARG, "bad replica");
    return MECH_OK;
}

int32_t mech_set_coords(MechContext* ctx, int32_t r, const double* coord) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (!coord) return set_err(MECH_ERR_ARG, "null coord");
    CU(cudaSetDevice(ctx->device));
    if ((rc = pull_states(ctx))) return rc;
    const ReplicaHost& h = ctx->reps[r];
    CU(cudaMemcpyAsync(ctx->stage.p, coord, sizeof(double) * 3 * h.nb, cudaMemcpyHostToDevice, ctx->stream));
    void* X = ctx->x[ctx->h_st[r].xbuf].p;
    if (ctx->precision == MECH_PREC_FP64)
        k_scatter_coords<double><<<(h.nb + 255) / 256, 256, 0, ctx->stream>>>(ctx->stage.as<double>(), perm_of(ctx, r),
                                                                              h.nb, h.bead_begin, (double*)X);
    else
        k_scatter_coords<float><<<(h.nb + 255) / 256, 256, 0, ctx->stream>>>(ctx->stage.as<double>(), perm_of(ctx, r),
                                                                             h.nb, h.bead_begin, (float*)X);
    CU(cudaGetLastError());
    CU(cudaStreamSynchronize(ctx->stream));
    return MECH_OK;
}

int32_t mech_get_coords(MechContext* ctx, int32_t r, double* coord) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (!coord) return set_err(MECH_ERR_ARG, "null coord");
    CU(cudaSetDevice(ctx->device));
    if ((rc = pull_states(ctx))) return rc;
    const ReplicaHost& h = ctx->reps[r];
    const void* X = ctx->x[ctx->h_st[r].xbuf].p;
    if (ctx->precision == MECH_PREC_FP64)
        k_gather_pos<double><<<(h.nb + 255) / 256, 256, 0, ctx->stream>>>((const double*)X, perm_of(ctx, r), h.nb,
                                                                          h.bead_begin, ctx->stage.as<double>());
    else
        k_gather_pos<float><<<(h.nb + 255) / 256, 256, 0, ctx->stream>>>((const float*)X, perm_of(ctx, r), h.nb,
                                                                         h.bead_begin, ctx->stage.as<double>());
    CU(cudaMemcpyAsync(coord, ctx->stage.p, sizeof(double) * 3 * h.nb, cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return MECH_OK;
}

int32_t mech_get_forces(MechContext* ctx, int32_t r, double* f_out) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (!f_out) return set_err(MECH_ERR_ARG, "null output");
    CU(cudaSetDevice(ctx->device));
    if ((rc = pull_states(ctx))) return rc;
    const ReplicaHost& h = ctx->reps[r];
    const int fb = ctx->h_st[r].fbuf;
    if (ctx->precision == MECH_PREC_FP64)
        k_gather_coords<double><<<(h.nb + 255) / 256, 256, 0, ctx->stream>>>(ctx->f[fb].as<double>(), perm_of(ctx, r), h.nb,
                                                                           h.bead_begin, ctx->stage.as<double>());
    else
        k_gather_coords<float><<<(h.nb + 255) / 256, 256, 0, ctx->stream>>>(ctx->f[fb].as<float>(), perm_of(ctx, r), h.nb,
                                                                          h.bead_begin, ctx->stage.as<double>());
    CU(cudaMemcpyAsync(f_out, ctx->stage.p, sizeof(double) * 3 * h.nb, cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return MECH_OK;
}

int32_t mech_rebuild_neighbors(MechContext* ctx, double cell_size, MechListInfo* info) {
    if (!ctx) return set_err(MECH_ERR_ARG, "null context");
    CU(cudaSetDevice(ctx->device));
    return rebuild(ctx, cell_size, info);
}

int32_t mech_get_pairs(MechContext* ctx, int32_t r, int32_t* pairs, int64_t cap, int64_t* count) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (!ctx->have_lists) return set_err(MECH_ERR_STATE, "no lists");
    const ReplicaHost& h = ctx->reps[r];
    if (count) *count = h.nev;
    const long long n = std::min<long long>(cap, h.nev);
    if (n > 0 && pairs) {
        CU(cudaMemcpy(pairs, ctx->pb.pairs.as<int2>() + h.ev_begin, sizeof(int2) * n, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < 2 * n; ++i) pairs[i] -= h.cyl_begin;
    }
    return MECH_OK;
}

int32_t mech_get_boundary_list(MechContext* ctx, int32_t r, int32_t* entries, int64_t cap, int64_t* count) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (!ctx->have_lists) return set_err(MECH_ERR_STATE, "no lists");
    const ReplicaHost& h = ctx->reps[r];
    const long long nq = (long long)h.nplanes * h.ncyl;
    std::vector<int> cnt((size_t)std::max(nq, 1LL));
    if (nq > 0)
        CU(cudaMemcpy(cnt.data(), ctx->bbuild.cnt.as<int>() + h.bq_begin, sizeof(int) * nq, cudaMemcpyDeviceToHost));
    long long k = 0;
    for (long long q = 0; q < nq; ++q) {
        if (!cnt[q]) continue;
        if (entries && k < cap) {
            entries[2 * k] = (int32_t)(q / h.ncyl);
            entries[2 * k + 1] = (int32_t)(q % h.ncyl);
        }
        ++k;
    }
    if (count) *count = k;
    return MECH_OK;
}

int32_t mech_load_forces(MechContext* ctx, int32_t r, int32_t n_types, const double* mon_size, const int32_t* n_mon,
                         int32_t stride, double* plus, double* minus) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (n_types < 1 || !mon_size || !n_mon || stride < 1 || !plus || !minus)
        return set_err(MECH_ERR_ARG, "mech_load_forces: bad argument");
    if (!ctx->have_lists) return set_err(MECH_ERR_STATE, "no lists");
    CU(cudaSetDevice(ctx->device));
    if ((rc = pull_states(ctx))) return rc;
    const ReplicaHost& h = ctx->reps[r];
    const size_t nout = 2 * (size_t)h.nfil * (size_t)stride;
    DeviceBuffer ends, types, ms, nm, out;
    cudaStream_t s = ctx->stream;
    if ((rc = upload(ends, h.fil_end_cyl, s)) || (rc = upload(types, h.fil_type, s))) return rc;
    if ((rc = upload(ms, std::vector<double>(mon_size, mon_size + n_types), s)) ||
        (rc = upload(nm, std::vector<int>(n_mon, n_mon + n_types), s)))
        return rc;
    CU(out.ensure(sizeof(double) * nout));
    LoadForceArgs a{};
    a.ends = ends.as<int>();
    a.fil_type = types.as<int>();
    a.mon_size = ms.as<double>();
    a.n_mon = nm.as<int>();
    a.ntypes = n_types;
    a.nfil = h.nfil;
    a.stride = stride;
    a.cyl_b1 = ctx->cyl_b1.as<int>();
    a.cyl_begin = h.cyl_begin;
    a.ncyl = h.ncyl;
    a.bcnt = ctx->bbuild.cnt.as<int>() + h.bq_begin;
    a.nplanes = h.nplanes;
    a.planes = ctx->planes.as<double>() + 4 * (size_t)h.plane_begin;
    a.plane_k = ctx->plane_k.as<double>() + h.plane_begin;
    a.plane_slen = ctx->plane_slen.as<double>() + h.plane_begin;
    a.out = out.as<double>();
    const void* X = ctx->x[ctx->h_st[r].xbuf].p;
    const unsigned nblk = (unsigned)((nout + 255) / 256);
    if (ctx->precision == MECH_PREC_FP64) k_load_forces<double><<<nblk, 256, 0, s>>>((const double*)X, a);
    else k_load_forces<float><<<nblk, 256, 0, s>>>((const float*)X, a);
    CU(cudaGetLastError());
    std::vector<double> hout(nout);
    CU(cudaMemcpyAsync(hout.data(), out.p, sizeof(double) * nout, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    for (int f = 0; f < h.nfil; ++f)
        for (int i = 0; i < stride; ++i) {
            minus[(size_t)f * stride + i] = hout[(2 * (size_t)f) * stride + i];
            plus[(size_t)f * stride + i] = hout[(2 * (size_t)f + 1) * stride + i];
        }
    return MECH_OK;
}

int32_t mech_energy_terms(MechContext* ctx, int32_t r, double* stretch, double* bend) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (!stretch || !bend) return set_err(MECH_ERR_ARG, "null output");
    if (!ctx->have_lists && (rc = rebuild(ctx, 0.0, nullptr))) return rc;
    CU(cudaSetDevice(ctx->device));
    if ((rc = pull_states(ctx))) return rc;
    for (int q = 0; q < ctx->R; ++q) ctx->h_st[q].active = (q == r);
    if ((rc = push_states(ctx))) return rc;
    const ReplicaHost& h = ctx->reps[r];
    DeviceBuffer terms, out;
    const size_t rs = real_size(ctx);
    CU(terms.ensure(rs * 2 * (size_t)ctx->nb));
    CU(out.ensure(sizeof(double) * 2 * (size_t)h.ncyl));
    cudaStream_t s = ctx->stream;
    CU(cudaMemsetAsync(terms.p, 0, rs * 2 * (size_t)ctx->nb, s));
    // the filament energy kernel of a plain evaluation, storing its terms
    const unsigned nblk = (unsigned)((h.ncyl + 255) / 256);
    double* o = out.as<double>();
    if (ctx->precision == MECH_PREC_FP64) {
        DevNet<double> n = make_devnet<double>(ctx);
        n.terms = terms.as<double>();
        launch_part<double>(n, 0, s);
        k_terms_by_cylinder<<<nblk, 256, 0, s>>>(terms.as<double>(), ctx->nb, ctx->cyl_b1.as<int>(), h.cyl_begin,
                                                h.ncyl, o, o + h.ncyl);
    } else {
        DevNet<float> n = make_devnet<float>(ctx);
        n.terms = terms.as<float>();
        launch_part<float>(n, 0, s);
        k_terms_by_cylinder<<<nblk, 256, 0, s>>>(terms.as<float>(), ctx->nb, ctx->cyl_b1.as<int>(), h.cyl_begin,
                                                h.ncyl, o, o + h.ncyl);
    }
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(stretch, o, sizeof(double) * h.ncyl, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(bend, o + h.ncyl, sizeof(double) * h.ncyl, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    return MECH_OK;
}

int32_t mech_energy(MechContext* ctx, int32_t r, const double* coord, double* per_ff, double* total, double* energy) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (coord && (rc = mech_set_coords(ctx, r, coord))) return rc;
    if (!ctx->have_lists && (rc = rebuild(ctx, 0.0, nullptr))) return rc;
    rc = ctx->precision == MECH_PREC_FP64 ? eval_energy<double>(ctx, r) : eval_energy<float>(ctx, r);
    if (rc) return rc;
    if (*ctx->h_err & (2u | 4u | 16u | 32u)) return err_status(*ctx->h_err);
    const CGState& S = ctx->h_st[r];
    if (per_ff)
        for (int k = 0; k < MECH_NUM_FF; ++k) per_ff[k] = S.eval[k];
    if (total) *total = S.eval[MECH_NUM_FF];
    if (energy) *energy = S.E0;
    return MECH_OK;
}

int32_t mech_forces(MechContext* ctx, int32_t r, const double* coord, double* f_out) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (coord && (rc = mech_set_coords(ctx, r, coord))) return rc;
    if (!ctx->have_lists && (rc = rebuild(ctx, 0.0, nullptr))) return rc;
    rc = ctx->precision == MECH_PREC_FP64 ? eval_forces<double>(ctx, r) : eval_forces<float>(ctx, r);
    if (rc) return rc;
    if (*ctx->h_err) return err_status(*ctx->h_err);
    return f_out ? mech_get_forces(ctx, r, f_out) : MECH_OK;
}

int32_t mech_minimize(MechContext* ctx, const MechCGParams* params, MechResult* results) {
    if (!ctx || !params || !results) return set_err(MECH_ERR_ARG, "null argument");
    if (!ctx->have_net) return set_err(MECH_ERR_STATE, "no network");
    if (params->method < 0 || params->method > 2) return set_err(MECH_ERR_ARG, "bad method");
    CU(cudaSetDevice(ctx->device));
#ifdef MECH_TRACE
    // diagnostic build: every block of every kernel of this minimization appends
    // (start, end, kernel, block) records; written to $MECH_TRACE_FILE at the end
    const char* tf = std::getenv("MECH_TRACE_FILE");
    if (tf) {
        const unsigned long long cap = 16ull << 20;
        CU(ctx->trace.ensure(sizeof(unsigned long long) * (2 + 3 * cap)));
        const unsigned long long hdr[2] = {0ull, cap};
        CU(cudaMemcpy(ctx->trace.p, hdr, sizeof(hdr), cudaMemcpyHostToDevice));
    }
    const int trc = ctx->precision == MECH_PREC_FP64 ? minimize_impl<double>(ctx, params, results)
                                            : minimize_impl<float>(ctx, params, results);
    if (tf) {
        cudaDeviceSynchronize();
        unsigned long long hdr[2] = {0, 0};
        cudaMemcpy(hdr, ctx->trace.p, sizeof(hdr), cudaMemcpyDeviceToHost);
        const unsigned long long nrec = std::min(hdr[0], hdr[1]);
        std::vector<unsigned long long> rec(3 * nrec);
        if (nrec) cudaMemcpy(rec.data(), ctx->trace.as<unsigned long long>() + 2, sizeof(unsigned long long) * 3 * nrec,
                             cudaMemcpyDeviceToHost);
        if (FILE* fh = std::fopen(tf, "wb")) {
            std::fwrite(rec.data(), sizeof(unsigned long long), rec.size(), fh);
            std::fclose(fh);
        }
        ctx->trace.release();
    }
    return trc;
#else
    return ctx->precision == MECH_PREC_FP64 ? minimize_impl<double>(ctx, params, results)
                                            : minimize_impl<float>(ctx, params, results);
#endif
}

int32_t mech_get_stretch_forces(MechContext* ctx, int32_t r, double* linker_f, double* motor_f) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    const ReplicaHost& h = ctx->reps[r];
    if (linker_f && h.nlk > 0)
        CU(cudaMemcpy(linker_f, ctx->lk_sf.as<double>() + h.lk_begin, sizeof(double) * h.nlk, cudaMemcpyDeviceToHost));
    if (motor_f && h.nmt > 0)
        CU(cudaMemcpy(motor_f, ctx->mt_sf.as<double>() + h.mt_begin, sizeof(double) * h.nmt, cudaMemcpyDeviceToHost));
    return MECH_OK;
}

int32_t mech_set_graph_mode(MechContext* ctx, int32_t mode) {
    if (!ctx) return set_err(MECH_ERR_ARG, "null context");
    if (mode != MECH_GRAPH_CONDITIONAL && mode != MECH_GRAPH_UNROLLED && mode != MECH_GRAPH_UNROLLED_PDL &&
        mode != MECH_GRAPH_UNROLLED_COOP)
        return set_err(MECH_ERR_ARG, "bad graph mode");
    ctx->graph_mode = mode;
    return MECH_OK;
}

int32_t mech_reset_coords(MechContext* ctx) {
    if (!ctx) return set_err(MECH_ERR_ARG, "null context");
    if (!ctx->have_net) return set_err(MECH_ERR_STATE, "no network");
    CU(cudaSetDevice(ctx->device));
    int rc;
    if ((rc = pull_states(ctx))) return rc;
    for (int r = 0; r < ctx->R; ++r) ctx->h_st[r].xbuf = 0;
    if ((rc = push_states(ctx))) return rc;
    CU(cudaMemcpyAsync(ctx->x[0].p, ctx->xinit.p, 24 * (size_t)ctx->nb, cudaMemcpyDeviceToDevice, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return MECH_OK;
}

}  // extern "C"

template <typename Real>
static int profile_impl(MechContext* c, int iters, MechProfile* o) {
    int rc;
    if (!c->have_lists && (rc = rebuild(c, 0.0, nullptr))) return rc;
    if ((rc = pull_states(c))) return rc;
    for (int r = 0; r < c->R; ++r) c->h_st[r].active = 1;
    if ((rc = push_states(c))) return rc;
    const DevNet<Real> n = make_devnet<Real>(c);
    cudaStream_t s = c->stream;
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    // Each evaluation is captured once as a CUDA graph and replayed, the way
    // the minimizer runs it: direct launches of a three-lane evaluation are
    // bound by the host's launch rate, not by the device.
    cudaError_t gerr = cudaSuccess;
    auto timeit = [&](auto&& fn) -> double {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            fn();
            e = cudaStreamEndCapture(s, &g);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, cudaGraphInstantiateFlagUseNodePriority);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaGraphLaunch(ge, s);   // warm
        if (e == cudaSuccess) {
            cudaEventRecord(e0, s);
            for (int i = 0; i < iters && e == cudaSuccess; ++i) e = cudaGraphLaunch(ge, s);
            cudaEventRecord(e1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
        }
        if (ge) cudaGraphExecDestroy(ge);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess && gerr == cudaSuccess) gerr = e;
        return ms / iters;
    };
    o->ms_energy_eval = timeit([&] { launch_energy<Real>(n, -1, 0, c->lanes()); });
    o->ms_force_eval = timeit([&] { launch_forces<Real>(n, -1, c->lanes()); });
    o->ms_fil_energy = timeit([&] { launch_part<Real>(n, 0, s); });
    o->ms_fil_force = timeit([&] { launch_part<Real>(n, 1, s); });
    o->ms_bond_energy = timeit([&] { launch_part<Real>(n, 2, s); });
    o->ms_bond_force = timeit([&] { launch_part<Real>(n, 3, s); });
    o->ms_fil_energy_trial = timeit([&] { launch_part<Real>(n, 4, s); });
    o->ms_fil_force_kernel = timeit([&] { launch_part<Real>(n, 5, s); });
    o->ms_force_gather = timeit([&] { launch_part<Real>(n, 6, s); });
    // the last evaluation's extended-pass and Simpson-fallback list lengths
    auto counts = [&](int64_t* ext, int64_t* fb) {
        int v[2] = {0, 0};
        if (c->ev_list_count.p) cudaMemcpy(&v[0], c->ev_list_count.p, sizeof(int), cudaMemcpyDeviceToHost);
        cudaMemcpy(&v[1], n.ev_fb_count, sizeof(int), cudaMemcpyDeviceToHost);
        *ext = c->precision == MECH_PREC_MIXED ? v[0] : c->nev;
        *fb = v[1];
    };
    o->ms_exvol_energy = timeit([&] { launch_exvol_energy<Real>(n, -1, 0, s, true); });
    counts(&o->n_exvol_ext_energy, &o->n_exvol_fallback_energy);
    o->ms_exvol_force = timeit([&] { launch_exvol_forces<Real>(n, -1, s, true); });
    counts(&o->n_exvol_ext_force, &o->n_exvol_fallback_force);
    // evaluations expect zero counts on entry
    if (c->ev_list_count.p) CU(cudaMemsetAsync(c->ev_list_count.p, 0, 4 * sizeof(int), s));
    CU(cudaMemsetAsync(n.ev_fb_count, 0, sizeof(int), s));
    // a line-search trial: positions x + lambda d formed and materialized on the fly
    o->ms_trial_energy_eval = timeit([&] { launch_energy<Real>(n, -1, sizeof(Real) == 4 ? kTrialDual : 1, c->lanes()); });
    // every replica finished: each launch of an iteration block reads its phase and exits
    const std::vector<CGState> saved(c->h_st, c->h_st + c->R);
    for (int r = 0; r < c->R; ++r) c->h_st[r].phase = PH_DONE;
    if ((rc = push_states(c))) return rc;
    o->ms_iteration_idle = timeit([&] {
        trial_launches<Real>(n, c->lanes());
        launch_forces<Real>(n, PH_FORCE, c->lanes());
        launch_direction<Real>(n, s);
        launch_reset<Real>(n, s);
    });
    std::copy(saved.begin(), saved.end(), c->h_st);
    if ((rc = push_states(c))) return rc;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CU(gerr);
    CU(cudaGetLastError());
    o->n_beads = c->nb;
    o->n_exvol_pairs = c->nev;
    o->n_boundary = c->nbb;
    o->n_linkers = c->nlk;
    o->n_motors = c->nmt;
    o->n_slots = c->slot_base[K_NUM_SPARSE];
    return pull_states(c);
}

// ===========================================================================
// autotuner: tiles per block of the mixed filament kernels, bin-edge scale
// ===========================================================================
namespace {

struct TuneKey {
    int precision, nb, nftiles, R;
    long long nev;
    bool operator<(const TuneKey& o) const {
        if (precision != o.precision) return precision < o.precision;
        if (nb != o.nb) return nb < o.nb;
        if (nftiles != o.nftiles) return nftiles < o.nftiles;
        if (R != o.R) return R < o.R;
        return nev < o.nev;
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, MechTuning> g_tune_cache;

}  // namespace

template <typename Real>
static int autotune_impl(MechContext* c, int flags, MechTuning* out) {
    int rc;
    if (!c->have_lists && (rc = rebuild(c, 0.0, nullptr))) return rc;
    const TuneKey key{c->precision, c->nb, c->n_ftiles, c->R, c->nev};
    if (!(flags & MECH_TUNE_FORCE)) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            *out = it->second;
            c->tile_cap[0] = out->energy_tiles_per_block;
            c->tile_cap[1] = out->force_tiles_per_block;
            c->blocks_per_sm[0] = out->energy_blocks_per_sm;
            c->blocks_per_sm[1] = out->force_blocks_per_sm;
            c->cell_scale = out->cell_scale;
            return MECH_OK;
        }
    }
    MechTuning t{};
    t.energy_tiles_per_block = c->tile_cap[0];
    t.force_tiles_per_block = c->tile_cap[1];
    t.energy_blocks_per_sm = c->blocks_per_sm[0];
    t.force_blocks_per_sm = c->blocks_per_sm[1];
    t.cell_scale = c->cell_scale;
    cudaStream_t s = c->stream;
    if ((rc = pull_states(c))) return rc;
    for (int r = 0; r < c->R; ++r) c->h_st[r].active = 1;
    if ((rc = push_states(c))) return rc;
    if ((flags & MECH_TUNE_KERNELS) && c->precision == MECH_PREC_MIXED) {
        cudaEvent_t e0, e1;
        CU(cudaEventCreate(&e0));
        CU(cudaEventCreate(&e1));
        const int cands[] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64};
        for (int which = 0; which < 2; ++which) {
            double best = 1e300;
            int best_cap = c->tile_cap[which];
            for (int cap : cands) {
                if (cap > kFilBulkMaxTiles) continue;
                c->tile_cap[which] = cap;
                const DevNet<Real> n = make_devnet<Real>(c);
                // the energy kernel as the minimizer runs it: a line-search pass
                const int part = which == 0 ? 4 : 1;
                launch_part<Real>(n, part, s);   // warm
                cudaEventRecord(e0, s);
                for (int i = 0; i < 10; ++i) launch_part<Real>(n, part, s);
                cudaEventRecord(e1, s);
                CU(cudaEventSynchronize(e1));
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms / 10 < best) {
                    best = ms / 10;
                    best_cap = cap;
                }
            }
            c->tile_cap[which] = best_cap;
            if (which == 0) { t.energy_tiles_per_block = best_cap; t.ms_energy = best; }
            else { t.force_tiles_per_block = best_cap; t.ms_force = best; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        CU(cudaGetLastError());
    }
    if (flags & MECH_TUNE_CELL) {
        const double cands[] = {0.6, 0.8, 1.0, 1.3, 1.7, 2.2, 3.0};
        double best = 1e300, best_scale = c->cell_scale;
        for (double sc : cands) {
            c->cell_scale = sc;
            double tmin = 1e300;
            for (int rep = 0; rep < 3; ++rep) {
                const auto a = std::chrono::steady_clock::now();
                if ((rc = rebuild(c, 0.0, nullptr))) return rc;
                tmin = std::min(tmin, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count());
            }
            if (tmin < best) {
                best = tmin;
                best_scale = sc;
            }
        }
        c->cell_scale = best_scale;
        t.cell_scale = best_scale;
        t.ms_rebuild = best;
        if ((rc = rebuild(c, 0.0, nullptr))) return rc;   // leave the lists of the chosen edge
    }
    if ((rc = pull_states(c))) return rc;
    *out = t;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = t;
    return MECH_OK;
}

// ===========================================================================
// Hessian-vector products, implicit adjoint, Newton refinement (FP64 engine)
// ===========================================================================
namespace {

// caller-order vector of replica r -> internal slots of a full-length vector
__global__ void k_scatter_vec(const double* in, const int* perm, int nb, int base, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const size_t j = 3 * (size_t)(base + perm[i]);
    out[j] = in[3 * (size_t)i];
    out[j + 1] = in[3 * (size_t)i + 1];
    out[j + 2] = in[3 * (size_t)i + 2];
}

// x = x0 + alpha dx
__global__ void k_axpy_from(double* x, const double* x0, double alpha, const double* dx, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = x0[i] + alpha * dx[i];
}

}  // namespace

// the solver's work vectors (3 * nb doubles each) and scalars
static int hvp_buffers(MechContext* c, HvpCgWork* w) {
    const size_t v = sizeof(double) * 3 * (size_t)std::max(c->nb, 1);
    CU(c->hv_a.ensure(v));
    CU(c->hv_b.ensure(std::max(v, sizeof(double) * 2 * (size_t)std::max(c->nlk, 1))));
    CU(c->cg_x.ensure(v));
    CU(c->cg_r.ensure(v));
    CU(c->cg_p.ensure(v));
    CU(c->cg_Ap.ensure(v));
    CU(c->cg_scal.ensure(sizeof(double) * 8));
    CU(c->cg_part.ensure(sizeof(double) * 512));
    CU(c->cg_ticket.ensure(sizeof(unsigned) * 4));
    w->r = c->cg_r.as<double>();
    w->p = c->cg_p.as<double>();
    w->Ap = c->cg_Ap.as<double>();
    w->scal = c->cg_scal.as<double>();
    w->part = c->cg_part.as<double>();
    w->ticket = c->cg_ticket.as<unsigned>();
    return MECH_OK;
}

static int hvp_ready(MechContext* c) {
    if (c->precision != MECH_PREC_FP64)
        return set_err(MECH_ERR_STATE, "Hessian-vector products, adjoint and Newton solves need an FP64 context");
    int rc;
    if (!c->have_lists && (rc = rebuild(c, 0.0, nullptr))) return rc;
    return canonicalize_x(c);
}

// caller-order host vector of replica r -> full internal-order device vector (zero elsewhere)
static int put_replica_vec(MechContext* c, int r, const double* host, DeviceBuffer& dst) {
    const ReplicaHost& h = c->reps[r];
    cudaStream_t s = c->stream;
    CU(cudaMemsetAsync(dst.p, 0, sizeof(double) * 3 * (size_t)c->nb, s));
    CU(cudaMemcpyAsync(c->stage.p, host, sizeof(double) * 3 * h.nb, cudaMemcpyHostToDevice, s));
    k_scatter_vec<<<(h.nb + 255) / 256, 256, 0, s>>>(c->stage.as<double>(), perm_of(c, r), h.nb, h.bead_begin,
                                                      dst.as<double>());
    CU(cudaGetLastError());
    return MECH_OK;
}

static int get_replica_vec(MechContext* c, int r, const DeviceBuffer& src, double* host) {
    const ReplicaHost& h = c->reps[r];
    cudaStream_t s = c->stream;
    k_gather_coords<double><<<(h.nb + 255) / 256, 256, 0, s>>>(src.as<double>(), perm_of(c, r), h.nb, h.bead_begin,
                                                               c->stage.as<double>());
    CU(cudaMemcpyAsync(host, c->stage.p, sizeof(double) * 3 * h.nb, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    return MECH_OK;
}

static void fill_info(MechSolveInfo* info, const HvpCgResult& cr) {
    if (!info) return;
    info->iterations = cr.iterations;
    info->converged = cr.converged;
    info->rel_residual = cr.rel_residual;
    info->launches = cr.launches;
    info->negative_curvature = cr.negative_curvature;
}

extern "C" {

int32_t mech_hvp(MechContext* ctx, int32_t r, int32_t mode, const double* v, double* hv) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (!v || !hv) return set_err(MECH_ERR_ARG, "null vector");
    if (mode != MECH_HVP_ENERGY && mode != MECH_HVP_FORCE_JACOBIAN) return set_err(MECH_ERR_ARG, "bad mode");
    CU(cudaSetDevice(ctx->device));
    if ((rc = hvp_ready(ctx))) return rc;
    HvpCgWork w{};
    if ((rc = hvp_buffers(ctx, &w))) return rc;
    if ((rc = put_replica_vec(ctx, r, v, ctx->hv_a))) return rc;
    CU(cudaMemsetAsync(ctx->err.p, 0, sizeof(unsigned), ctx->stream));
    const DevNet<double> n = make_devnet<double>(ctx);
    ctx->timing.launches += launch_hvp(n, ctx->hv_a.as<double>(), ctx->hv_b.as<double>(), 0.0,
                                       mode == MECH_HVP_FORCE_JACOBIAN, ctx->stream);
    CU(cudaGetLastError());
    if ((rc = get_replica_vec(ctx, r, ctx->hv_b, hv))) return rc;
    if ((rc = pull_states(ctx))) return rc;
    if (*ctx->h_err & 8u) return set_err(MECH_ERR_NONFINITE, "non-finite excluded-volume Hessian term");
    return MECH_OK;
}

int32_t mech_set_linker_params(MechContext* ctx, int32_t r, const double* k, const double* eq_length) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    CU(cudaSetDevice(ctx->device));
    const ReplicaHost& h = ctx->reps[r];
    if (h.nlk == 0) return MECH_OK;
    const size_t rs = real_size(ctx);
    auto put = [&](DeviceBuffer& dst, const double* src) -> int {
        if (!src) return MECH_OK;
        if (ctx->precision == MECH_PREC_FP64) {
            CU(cudaMemcpyAsync(dst.as<double>() + h.lk_begin, src, sizeof(double) * h.nlk, cudaMemcpyHostToDevice,
                               ctx->stream));
        } else {
            std::vector<float> f(src, src + h.nlk);
            CU(cudaMemcpyAsync(dst.as<float>() + h.lk_begin, f.data(), rs * h.nlk, cudaMemcpyHostToDevice, ctx->stream));
            CU(cudaStreamSynchronize(ctx->stream));
        }
        return MECH_OK;
    };
    if ((rc = put(ctx->lk_k, k)) || (rc = put(ctx->lk_l0, eq_length))) return rc;
    CU(cudaStreamSynchronize(ctx->stream));
    return MECH_OK;
}

int32_t mech_adjoint(MechContext* ctx, int32_t r, const double* dL_dx, double dL_dE, const MechSolveParams* sp,
                     double* dL_dk, double* dL_dl0, MechSolveInfo* info) {
    int rc = check_replica(ctx, r);
    if (rc) return rc;
    if (!dL_dx || !sp || !dL_dk || !dL_dl0) return set_err(MECH_ERR_ARG, "null argument");
    if (!(sp->rel_tol > 0) || sp->max_iter <= 0) return set_err(MECH_ERR_ARG, "bad solve parameters");
    CU(cudaSetDevice(ctx->device));
    if ((rc = hvp_ready(ctx))) return rc;
    HvpCgWork w{};
    if ((rc = hvp_buffers(ctx, &w))) return rc;
    if ((rc = put_replica_vec(ctx, r, dL_dx, ctx->hv_a))) return rc;
    CU(cudaMemsetAsync(ctx->err.p, 0, sizeof(unsigned), ctx->stream));
    const DevNet<double> n = make_devnet<double>(ctx);
    HvpCgResult cr{};
    CU(hvp_cg_solve(n, ctx->hv_a.as<double>(), ctx->cg_x.as<double>(), w, sp->rel_tol, sp->max_iter, sp->shift,
                    ctx->stream, &cr));
    ctx->timing.launches += cr.launches;
    fill_info(info, cr);
    const ReplicaHost& h = ctx->reps[r];
    if (h.nlk > 0) {
        double* dk = ctx->hv_b.as<double>();
        launch_linker_grad(n, h.lk_begin, h.nlk, ctx->cg_x.as<double>(), dL_dE, dk, dk + h.nlk, ctx->stream);
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(dL_dk, dk, sizeof(double) * h.nlk, cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaMemcpyAsync(dL_dl0, dk + h.nlk, sizeof(double) * h.nlk, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if ((rc = pull_states(ctx))) return rc;
    if (*ctx->h_err & 8u) return set_err(MECH_ERR_NONFINITE, "non-finite excluded-volume Hessian term");
    if (!cr.converged) return set_err(MECH_ERR_ITER_LIMIT, "adjoint CG did not reach its tolerance");
    return MECH_OK;
}

int32_t mech_newton_refine(MechContext* ctx, int32_t max_steps, double force_tol, const MechSolveParams* sp,
                           MechSolveInfo* info) {
    if (!ctx || !sp) return set_err(MECH_ERR_ARG, "null argument");
    if (!ctx->have_net) return set_err(MECH_ERR_STATE, "no network");
    if (!(sp->rel_tol > 0) || sp->max_iter <= 0 || max_steps < 0 || !(sp->shift >= 0))
        return set_err(MECH_ERR_ARG, "bad solve parameters");
    CU(cudaSetDevice(ctx->device));
    int rc;
    if ((rc = hvp_ready(ctx))) return rc;
    HvpCgWork w{};
    if ((rc = hvp_buffers(ctx, &w))) return rc;
    cudaStream_t s = ctx->stream;
    const long long N = 3LL * ctx->nb;
    HvpCgResult total{};
    int steps = 0;
    // max |F| and total energy over the replicas at x[0]
    auto evaluate = [&](double* m, double* e) -> int {
        int r2;
        if ((r2 = eval_energy<double>(ctx, -1))) return r2;
        double E = 0.0;
        for (int r = 0; r < ctx->R; ++r) E += ctx->h_st[r].eval[MECH_NUM_FF];
        if ((r2 = eval_forces<double>(ctx, -1))) return r2;
        if (*ctx->h_err) return err_status(*ctx->h_err);
        double v = 0.0;
        for (int r = 0; r < ctx->R; ++r) v = std::max(v, ctx->h_st[r].maxF);
        *m = v;
        *e = E;
        return MECH_OK;
    };
    double maxF = 0.0, E = 0.0;
    if ((rc = evaluate(&maxF, &E))) return rc;
    // Levenberg-Marquardt damped Newton: dx = (H + mu I)^-1 F; mu grows tenfold
    // when a solve meets non-positive curvature or no step length helps, and
    // shrinks tenfold after an accepted step.  A step x + alpha dx (alpha
    // halved from 1) is accepted when the energy drops or max |F| halves.
    double mu = sp->shift;
    constexpr double kMuFloor = 1e-6;   // pN/nm, first damping when mu starts at 0
    while (maxF >= force_tol && steps < max_steps) {
        for (int r = 0; r < ctx->R; ++r) {
            const ReplicaHost& h = ctx->reps[r];
            CU(cudaMemcpyAsync(ctx->hv_a.as<double>() + 3 * (size_t)h.bead_begin,
                               ctx->f[ctx->h_st[r].fbuf].as<double>() + 3 * (size_t)h.bead_begin,
                               sizeof(double) * 3 * h.nb, cudaMemcpyDeviceToDevice, s));
        }
        CU(cudaMemcpyAsync(ctx->hv_b.p, ctx->x[0].p, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
        bool accepted = false;
        double trialF = 0.0, trialE = 0.0;
        for (int attempt = 0; attempt < 16 && !accepted; ++attempt) {
            const DevNet<double> n = make_devnet<double>(ctx);
            HvpCgResult cr{};
            CU(hvp_cg_solve(n, ctx->hv_a.as<double>(), ctx->cg_x.as<double>(), w, sp->rel_tol, sp->max_iter, mu, s,
                            &cr));
            total.iterations += cr.iterations;
            total.launches += cr.launches;
            total.rel_residual = cr.rel_residual;
            total.converged = cr.converged;
            total.negative_curvature |= cr.negative_curvature;
            if (!cr.negative_curvature) {
                double alpha = 1.0;
                for (int t = 0; t < 30; ++t, alpha *= 0.5) {
                    k_axpy_from<<<304, 256, 0, s>>>(ctx->x[0].as<double>(), ctx->hv_b.as<double>(), alpha,
                                                    ctx->cg_x.as<double>(), N);
                    CU(cudaGetLastError());
                    rc = evaluate(&trialF, &trialE);
                    if (rc && rc != MECH_ERR_NONFINITE) return rc;
                    if (rc == MECH_OK && (trialE < E || trialF < 0.5 * maxF)) {
                        accepted = true;
                        break;
                    }
                }
            }
            if (!accepted) mu = std::max(10.0 * mu, kMuFloor);
        }
        ++steps;
        if (!accepted) {   // no progress even with strong damping: restore and stop
            CU(cudaMemcpyAsync(ctx->x[0].p, ctx->hv_b.p, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
            if ((rc = evaluate(&maxF, &E))) return rc;
            break;
        }
        maxF = trialF;
        E = trialE;
        mu = mu < 10.0 * kMuFloor ? 0.0 : 0.1 * mu;
    }
    ctx->timing.launches += total.launches;
    fill_info(info, total);
    if (info) {
        info->newton_steps = steps;
        info->max_force = maxF;
    }
    return MECH_OK;
}

}  // extern "C"

extern "C" {

int32_t mech_profile(MechContext* ctx, int32_t iters, MechProfile* out) {
    if (!ctx || !out || iters <= 0) return set_err(MECH_ERR_ARG, "bad argument");
    if (!ctx->have_net) return set_err(MECH_ERR_STATE, "no network");
    CU(cudaSetDevice(ctx->device));
    return ctx->precision == MECH_PREC_FP64 ? profile_impl<double>(ctx, iters, out) : profile_impl<float>(ctx, iters, out);
}

int32_t mech_autotune(MechContext* ctx, int32_t flags, MechTuning* out) {
    if (!ctx || !out) return set_err(MECH_ERR_ARG, "null argument");
    if (!ctx->have_net) return set_err(MECH_ERR_STATE, "no network");
    CU(cudaSetDevice(ctx->device));
    return ctx->precision == MECH_PREC_FP64 ? autotune_impl<double>(ctx, flags, out) : autotune_impl<float>(ctx, flags, out);
}

int32_t mech_set_tuning(MechContext* ctx, const MechTuning* t) {
    if (!ctx || !t) return set_err(MECH_ERR_ARG, "null argument");
    if (t->energy_tiles_per_block < 1 || t->energy_tiles_per_block > kFilBulkMaxTiles || t->force_tiles_per_block < 1 ||
        t->force_tiles_per_block > kFilBulkMaxTiles || !(t->cell_scale > 0))
        return set_err(MECH_ERR_ARG, "tuning out of range");
    ctx->tile_cap[0] = t->energy_tiles_per_block;
    ctx->tile_cap[1] = t->force_tiles_per_block;
    ctx->blocks_per_sm[0] = std::max(0, t->energy_blocks_per_sm);
    ctx->blocks_per_sm[1] = std::max(0, t->force_blocks_per_sm);
    ctx->cell_scale = t->cell_scale;
    return MECH_OK;
}

int32_t mech_get_timing(MechContext* ctx, MechTiming* t) {
    if (!ctx || !t) return set_err(MECH_ERR_ARG, "null argument");
    *t = ctx->timing;
    return MECH_OK;
}

}  // extern "C"
