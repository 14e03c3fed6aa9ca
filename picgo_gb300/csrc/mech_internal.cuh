// Internal declarations shared by the engine's translation units.
//
// Layout in HBM (one context, R replica networks concatenated):
//   beads     internal order = filament by filament, minus end first, replica
//             after replica; coordinates x[2][3*nb] double (AoS, current and
//             trial buffer), forces f[2][3*nb] Real (current and previous),
//             search direction d[3*nb] Real.
//   per bead  flag byte (bit0: cylinder to the next bead, bit1: cylinder from
//             the previous bead); the cylinder (i, i+1) keeps its k_str, l0 at
//             slot i; the bending triple centred on i keeps the constants of
//             the cylinder (i, i+1) at slot i.
//   sparse    linkers, motors, excluded-volume pairs and boundary beads as
//             interaction lists of internal bead indices; their force
//             contributions go to a slot buffer and every bead gathers its own
//             slots through a CSR index, in a fixed order (no float atomics).
//   tiles     every kernel works on tiles that never straddle replicas; each
//             tile (or run of tiles) writes its partial sums to a fixed slot
//             and a reduction kernel (one block per replica) reduces the slots
//             in order, so every sum is deterministic.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/medyan_mech.h"

namespace mech {

constexpr int kFilTile = 256;     // beads per filament tile (one block)
constexpr int kGatherTiles = 4;   // filament tiles per block of the force gather kernels
constexpr int kSparseTile = 256;  // interactions per sparse tile (one block)
constexpr int kFilBulkMaxTiles = 64;   // filament tiles per block of the bulk-staged mixed kernels
constexpr int kExvolFallbackCap = 4096;
constexpr int kFbChunks = 64;       // work split of one numeric force fallback
// `trial` argument of the evaluation kernels: 0 plain evaluation at x, 1 one
// line-search trial at x + lambda d, 2 (mixed engine) two trials in one pass,
// at x + lambda d and at x + (lambda / 2) d, the next step of the backtracking
// search, with the second trial's energies in their own partial slots
constexpr int kTrialDual = 2;
// the ext-pass list marks entries of the second trial with this bit of the pair index
constexpr int kExtSecond = 1 << 30;

enum Kind : int { K_LINKER = 0, K_MOTOR = 1, K_EXVOL = 2, K_BOUNDARY = 3, K_NUM_SPARSE = 4 };

enum Phase : int {
    PH_IDLE = 0,
    PH_LS_TRIAL = 1,   // a line-search trial energy is pending
    PH_FORCE = 2,      // trial accepted: forces at the new coordinates pending
    PH_DIR = 3,        // forces, beta ready: direction update pending
    PH_RESET = 4,      // conjugacy lost: d = F pending
    PH_FAILED = 5,     // line search returned lambda = 0: host decides
    PH_DONE = 6,       // converged or call limit
    PH_ERROR = 7,      // non-finite max force or other fatal condition
    PH_RECOVER = 8,         // safe-mode failure: recovery move pending (MController.h:273-339)
    PH_RECOVER_MOVE = 9,
    PH_RECOVER_FORCE = 10,
    PH_RECOVER_ENERGY = 11,
};

// Per-replica minimizer state, resident in device memory.
struct CGState {
    // line search
    double lambda;
    double E0;             // energy at the current coordinates (computeEnergy value)
    double Etrial;
    double reducedSlope;
    double slope;          // d . F
    // convergence bookkeeping
    double maxF;           // gradInfNorm
    double FdotF;          // F . F of the current forces
    double lastFdotF;
    double newGrad, prevGrad, beta;
    double prevEnergy;
    double energyRelChange;
    double newEnergy;
    double minimumE;
    double totalEnergy;
    // parameters
    double maxDist, lambdaMax, gradTol, energyRelTol;
    int method, energyCallLimit, forceCallLimit, tryToRecover;
    // energies of the last evaluation: per FF, then the plain total
    double eval[MECH_NUM_FF + 1];
    int evalFailed;        // an FF reported failure in the last evaluation
    int phase;
    int safeMode;
    int xbuf, fbuf;
    int numIter, numEnergyCall, numForceCall, numEnergyEval, numTrials, numSafeMode, numRecover;
    int backupValid, backupPending;
    int errorFlags, status;
    int active;            // replica participates in the current minimization
    int restore;           // copy the backup coordinates back (host request)
};

// Tile of consecutive items of one replica.
struct Tile {
    int replica;
    int begin;
    int end;
    int pad;
};

// Per-replica tile ranges, by tile family.
struct RepTiles {
    int fil_begin, fil_end;          // filament (bead) tiles
    int sp_begin[K_NUM_SPARSE], sp_end[K_NUM_SPARSE];
};

// Conditions of the minimizer's conditional graph: a while loop whose body
// runs one guarded phase after another (line-search trial, forces, direction,
// failure dispatch + reset).  The kernel at the head of a body and the last
// block of each phase's reduction set them from the replicas' phases; outside
// that graph `on` is 0 and no kernel touches them.
struct GraphConds {
    unsigned long long trial, force, dir, misc, loop;   // cudaGraphConditionalHandle values
    int* counter;   // [0] bodies run in this graph launch, [1] reduction ticket,
                    // [2..5] trial, force, direction, failure-dispatch bodies run (for the launch count)
    int cap;        // bodies per graph launch before control returns to the host
    int on;
};

// Everything the kernels read, passed by value.
template <typename Real>
struct DevNet {
    int nb;                 // beads, all replicas
    int R;
    // positions: double[3] per bead (FP64) or float hi[3], lo[3] per bead
    // (mixed); x[xbuf] is current, the others receive line-search trial
    // positions (FP64: one trial buffer; mixed: two, for lambda and lambda / 2)
    Real* x[3];
    Real* f[2];
    Real* d;
    Real* xbest;
    const uint8_t* bflag;
    const Real* bpar;       // per bead slot: k_str, l0 of cylinder (i, i+1); k_bend, theta0 of the triple on i
    // filament tiles; the mixed engine's persistent filament kernels give each
    // block `ptiles` consecutive tiles on a grid of `pgrid` blocks
    int n_ftiles;
    const Tile* ftile;
    int pgrid[3], ptiles[3];   // [0] energy, [1] force, [2] direction kernels
    int fil_first[2];          // energy / force: filament kernel launched before the side lanes (capped residency)
    // sparse interactions (internal bead indices)
    int n_lk, n_mt, n_ev, n_bb;
    const int4* lk_bead; const Real* lk_k; const Real* lk_l0; const Real* lk_s1; const Real* lk_s2;
    const int4* mt_bead; const Real* mt_k; const Real* mt_l0; const Real* mt_s1; const Real* mt_s2;
    const int4* ev_bead; const Real* ev_k; const Real* ev_la; const Real* ev_lb;
    const int* bb_bead; const int* bb_plane;     // plane index into planes
    const double* planes;                         // [4 * n_planes_total] a, b, c, d
    const Real* bb_k; const Real* bb_slen;
    // sparse tiles
    int n_stiles;
    const Tile* stile;      // concatenated: linker, motor, exvol, boundary tiles
    const int* stile_kind;
    int sp_tiles[K_NUM_SPARSE];   // tiles per kind
    // contributions and gather index
    Real* contrib;          // [3 * n_slots] in bead order: bead b's are [csr_off[b], csr_off[b+1])
    int slot_base[K_NUM_SPARSE + 1];
    const int* csr_off;     // [nb + 1]
    const int* slot_pos;    // slot (interaction-major) -> its position in contrib
    // stretch forces of linkers / motors (assignforcemags)
    double* lk_sf; double* mt_sf;
    // exvol numeric fallback list: count, (replica, pair) entries, energies
    // [cap] followed by the lambda of each entry [cap]; force-fallback scratch
    int* ev_fb_count; int* ev_fb_list; double* ev_fb_energy;
    double* fb_moments;     // [cap * kFbChunks * 6]
    int* fb_tickets;        // [cap]
    // mixed precision: pairs evaluated in FP64 (compacted list) and per-pair energies
    int* ev_list; int* ev_list_count; double* ev_energy;
    // mixed-precision line-search passes at lambda and lambda / 2: the second
    // trial's per-pair excluded-volume energies and sparse tile partials
    double* ev_energy2; double* part_sp2;
    // partial sums
    double* part_fil;       // [n_ftiles * 4]
    double* part_sp;        // [n_stiles]
    // per replica
    CGState* st;
    const RepTiles* rt;
    int* ticket;            // [R] last-tile tickets
    int* gticket;           // whole-grid ticket
    unsigned* err;          // device error word
    GraphConds cond;
    // programmatic dependent launch on the main lane (MECH_GRAPH_UNROLLED_PDL):
    // the kernels that follow a reduction, and the reductions themselves, are
    // scheduled while their predecessor runs and wait for it (griddepcontrol)
    int pdl;
    // diagnostic (mech_energy_terms; null otherwise): the filament energy
    // kernels also store each bead's stretching [b] and bending [nb + b] term,
    // in the engine's precision (a conversion to double in the mixed kernels
    // would be scheduled whether or not the store happens)
    Real* terms;
    // grid barrier of the cooperative iteration tail: [0] arrivals, [1] generation
    unsigned* gbar;
    // kernel timeline (builds with MECH_TRACE only; null otherwise):
    // [0] records written, [1] capacity, then (start ns, end ns, kernel << 32 | block) per block
    unsigned long long* trace;
};

// Kernel ids of the timeline records.
enum TraceKernel : unsigned {
    TK_FIL_ENERGY = 1, TK_FIL_FORCE, TK_GATHER, TK_FIN_FORCE, TK_FIN_ENERGY, TK_FIL_ENERGY_BULK, TK_FIL_FORCE_BULK,
    TK_DIRECTION_MX, TK_BOND, TK_DIRECTION, TK_FIN_DIRECTION, TK_RESET, TK_RECOVER_MAXABS, TK_RECOVER_MOVE,
    TK_BACKUP, TK_EXVOL_FB_FORCE, TK_EXVOL, TK_EXVOL_EXT, TK_EXVOL_TAIL, TK_BODY_HEAD, TK_GATHER_MX,
    // sections of the energy / force finalizers (thread 0's view): partial
    // loads, block reduction, the CG step logic and the state store
    TK_SEC_FE_LOAD, TK_SEC_FE_REDUCE, TK_SEC_FE_TAIL, TK_SEC_FF_LOAD, TK_SEC_FF_REDUCE, TK_SEC_FF_TAIL,
    TK_TAIL_COOP,
};

#if defined(__CUDACC__) && defined(MECH_TRACE)
// Thread 0 of every block appends (start, end, kernel, block) to the timeline
// when it leaves the kernel's scope.
struct TraceGuard {
    unsigned long long* buf;
    unsigned kid;
    unsigned long long t0;
    __device__ static unsigned long long now() {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        return t;
    }
    __device__ TraceGuard(unsigned long long* b, unsigned k) : buf(b), kid(k), t0(0) {
        if (buf && threadIdx.x == 0) t0 = now();
    }
    __device__ static void record(unsigned long long* b, unsigned k, unsigned long long a, unsigned long long e) {
        const unsigned long long i = atomicAdd(b, 1ull);
        if (i < b[1]) {
            b[2 + 3 * i] = a;
            b[3 + 3 * i] = e;
            b[4 + 3 * i] = ((unsigned long long)k << 32) | blockIdx.x;
        }
    }
    __device__ ~TraceGuard() {
        if (buf && threadIdx.x == 0) record(buf, kid, t0, now());
    }
};
#define MECH_TRACE_KERNEL(n, kid) TraceGuard mech_trace_guard_((n).trace, (kid))
// a section of a single-block kernel, as seen by thread 0: from stamp `t` to now
#define MECH_TRACE_STAMP(t) const unsigned long long t = threadIdx.x == 0 ? TraceGuard::now() : 0ull
#define MECH_TRACE_SECTION(n, kid, t)                                                  \
    do {                                                                               \
        if ((n).trace && threadIdx.x == 0) TraceGuard::record((n).trace, (kid), (t), TraceGuard::now()); \
    } while (0)
#else
#define MECH_TRACE_KERNEL(n, kid) ((void)0)
#define MECH_TRACE_STAMP(t) ((void)0)
#define MECH_TRACE_SECTION(n, kid, t) ((void)0)
#endif

#ifdef __CUDACC__
// Where the contribution of slot `slot` (= slot_base[kind] + interaction * beads + bead) is written.
template <typename Real>
__device__ __forceinline__ Real* slot_ptr(const DevNet<Real>& n, int slot) {
    return n.contrib + 3 * (size_t)__ldg(n.slot_pos + slot);
}
#endif

// Launch of `kernel` on stream `s`, with programmatic stream serialization when
// `pdl` is set: the kernel may then start while the previous kernel of the
// stream is still running (once that kernel's blocks have called pdl_trigger()),
// and calls pdl_wait() before it reads anything the previous kernel wrote.
template <typename... KArgs, typename... Args>
inline void launch_k(bool pdl, void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s,
                     Args... args) {
    if (!pdl) {
        kernel<<<grid, block, 0, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
#ifdef __CUDACC__
// no-ops for a kernel launched without programmatic serialization
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" :::); }
#endif

// ---- kernels (mech_ff.cu) -------------------------------------------------
// mode: 0 = line-search trial at x + lambda d (replicas in PH_LS_TRIAL),
//       1 = plain evaluation at x (replicas with active != 0)
// `want` selects the replicas a launch works on: replicas whose phase equals
// `want`, or every replica with active != 0 when want < 0.  `trial` evaluates
// at x + lambda d instead of x.  Each returns the number of kernels launched.
// An evaluation runs the excluded-volume chain on `side` and the linker,
// motor and boundary kernel on `side2` while the filament kernel runs on
// `main`; `fork` starts them, `join` / `join2` end them, then the reduction
// runs on `main`.
struct Lanes {
    cudaStream_t main, side, side2;
    cudaEvent_t fork, join, join2;
};
template <typename Real> int launch_energy(const DevNet<Real>& n, int want, int trial, const Lanes& L);
// coop_grid > 0 (mixed engine, one replica): the gather, both finalizers, the
// direction update and the reset run as one cooperative launch of that many
// blocks (k_tail_coop) instead of launch_forces' gather and finalizer plus
// launch_direction and launch_reset
template <typename Real> int launch_forces(const DevNet<Real>& n, int want, const Lanes& L, int coop_grid = 0);
// blocks of the cooperative iteration tail on `device` (all resident at once)
int coop_tail_grid(int device);
template <typename Real> int launch_direction(const DevNet<Real>& n, cudaStream_t s);
template <typename Real> int launch_reset(const DevNet<Real>& n, cudaStream_t s);
// head of a body of the minimizer's conditional graph: sets the phase
// conditions, counts the body and decides whether the loop continues
template <typename Real> int launch_body_head(const DevNet<Real>& n, cudaStream_t s);
template <typename Real> int launch_recover(const DevNet<Real>& n, const Lanes& L);
template <typename Real> int launch_backup_restore(const DevNet<Real>& n, cudaStream_t s);
// single kernel families in plain-evaluation mode, for profiling:
// 0 filament energy, 1 filament force, 2 bond/boundary energy, 3 bond/boundary force
template <typename Real> int launch_part(const DevNet<Real>& n, int which, cudaStream_t s);
// blocks of the mixed engine's persistent filament kernels on `device`
// (which: 0 energy, 1 force, 2 direction), at most per_sm per SM (0: no cap)
int persistent_blocks(int device, int which, int per_sm);

// Records the text mech_last_error returns on this thread; returns `code`.
int set_error_text(int code, const std::string& msg);
// excluded-volume kernels (mech_exvol.cu, one object per precision)
// (standalone: zero the work-list counts first; inside an evaluation they are
// zero on entry, reset by the evaluation's reduction kernel)
template <typename Real> int launch_exvol_energy(const DevNet<Real>& n, int want, int trial, cudaStream_t s,
                                                 bool standalone);
template <typename Real> int launch_exvol_forces(const DevNet<Real>& n, int want, cudaStream_t s, bool standalone);

// ---- Hessian-vector products and solves (mech_hvp.cu, FP64 engine) --------
// hv = (H + shift I) v at the positions in x[0], v and hv in internal bead
// order; H is the energy's Hessian, or with `jacobian` minus the Jacobian of
// the force routine (which moves nearly coplanar excluded-volume pairs)
int launch_hvp(const DevNet<double>& n, const double* v, double* hv, double shift, bool jacobian, cudaStream_t s);
struct HvpCgWork {
    double* r; double* p; double* Ap;   // [3 * nb] each
    double* scal;                        // [8]: r.r, p.Ap, new r.r, b.b, curvature flag
    double* part;                        // [304] per-block partial sums
    unsigned* ticket;
};
struct HvpCgResult {
    int iterations, converged, negative_curvature;
    double rel_residual;
    long long launches;
};
// (H + shift I) x = b by conjugate gradients from x = 0, to |r| <= rel_tol |b|
cudaError_t hvp_cg_solve(const DevNet<double>& n, const double* b, double* x, const HvpCgWork& w, double rel_tol,
                         int max_iter, double shift, cudaStream_t s, HvpCgResult* res);
// adjoint gradient of linkers [lk0, lk0 + nlk) from the adjoint solution lambda
void launch_linker_grad(const DevNet<double>& n, int lk0, int nlk, const double* lambda, double wE, double* dk,
                        double* dl0, cudaStream_t s);

struct DeviceBuffer {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t nbytes);
    void release();
    ~DeviceBuffer() { release(); }
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

// exclusive scan of n int32 values into out (n + 1 entries, out[n] = total)
cudaError_t exclusive_scan_i32(const int* in, int* out, long long n, DeviceBuffer& tmp, cudaStream_t s);

}  // namespace mech
