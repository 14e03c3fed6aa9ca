/*
 * medyan_mech.h — C ABI of the GB300 mechanical-equilibration engine.
 *
 * Drop-in for the path MEDYAN's MController drives before handing control
 * back to the chemistry: the ForceFieldManager / ForceField plugin set, the
 * CGMethod Polak-Ribiere minimizer with backtracking line search, and the
 * neighbor lists those force fields read.  Paths below are relative to
 * medyan-5.4.0/src of the reference.
 *
 * Conventions
 *   - every function returns MECH_OK (0) or a MECH_ERR_* code; nothing throws
 *     across the ABI;
 *   - host arrays are copied in; the library keeps no caller pointer;
 *   - coordinates and forces use the reference's DOF layout: one double per
 *     component, bead after bead (x0 y0 z0 x1 ...), in the caller's bead
 *     order (Structure/DofSerializer.hpp:64-187);
 *   - one context binds one CUDA device and one stream; calls on a context
 *     are not thread-safe, contexts are independent.
 */
#ifndef MEDYAN_MECH_H
#define MEDYAN_MECH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MECH_ABI_VERSION 1

/* Status codes. */
#define MECH_OK                  0
#define MECH_ERR_ARG            -1   /* bad argument or size */
#define MECH_ERR_TOPOLOGY       -2   /* filament cylinders do not chain bead to bead */
#define MECH_ERR_CUDA           -3   /* a CUDA call failed; see mech_last_error */
#define MECH_ERR_NONFINITE      -4   /* max |F| not finite (CGMethod.hpp:202-212 throws here) */
#define MECH_ERR_LINESEARCH     -5   /* line search failed with recovery disabled (MinimizationResult::errorLineSearch) */
#define MECH_ERR_ITER_LIMIT     -6   /* device loop gave up after its own iteration cap */
#define MECH_ERR_CAPACITY       -7   /* a device list outgrew its capacity */
#define MECH_ERR_NO_DEVICE      -8   /* no CUDA device visible */
#define MECH_ERR_STATE          -9   /* call made in the wrong order (e.g. no network) */

/* Precision of the force/geometry arithmetic. */
#define MECH_PREC_FP64   0   /* everything in FP64 */
#define MECH_PREC_MIXED  1   /* FP32 forces and pair geometry; FP64 energy sums, dots, beta, Armijo */

/* Force fields, in MController's order (Controller/MController.cpp:65-196). */
#define MECH_FF_STRETCHING  0   /* FilamentStretching<Harmonic>   */
#define MECH_FF_BENDING     1   /* FilamentBending<Cosine>        */
#define MECH_FF_LINKER      2   /* LinkerStretching<Harmonic>     */
#define MECH_FF_MOTOR       3   /* MotorGhostStretching<Harmonic> */
#define MECH_FF_EXVOL       4   /* CylinderExclVolume<CylinderExclVolRepulsion> */
#define MECH_FF_BOUNDARY    5   /* BoundaryCylinderRepulsion<Exp> */
#define MECH_NUM_FF         6

/*
 * One network: what serializeDof + the force fields' vectorize() consume.
 * Cylinders are listed filament by filament, minus end first; cylinder i of a
 * filament shares its second bead with cylinder i+1's first bead.
 */
typedef struct MechNetwork {
    int32_t n_beads;
    const double* coord;            /* [3*n_beads] */

    int32_t n_filaments;
    const int32_t* fil_cyl_start;   /* [n_filaments+1] cylinder ranges */

    int32_t n_cylinders;
    const int32_t* cyl_bead;        /* [2*n_cylinders] first, second bead */
    const int64_t* cyl_id;          /* unique cylinder IDs: half list keeps id_c > id_n */
    const int32_t* cyl_filament_id; /* filament ID (same-filament exclusion) */
    const int32_t* cyl_position;    /* position on filament */
    const int32_t* cyl_type;        /* filament type */
    const double* cyl_eq_length;    /* l0 (MCylinder::getEqLength) */
    const double* cyl_k_stretch;    /* MCylinder::getStretchingConst */
    const double* cyl_k_bend;       /* MCylinder::getBendingConst */
    const double* cyl_eq_theta;     /* MCylinder::getEqTheta */
    const double* cyl_k_exvol;      /* MCylinder::getExVolConst */

    int32_t n_linkers;
    const int32_t* lk_cyl;          /* [2*n] first, second cylinder */
    const double* lk_pos;           /* [2*n] relative positions on each cylinder */
    const double* lk_k;
    const double* lk_eq_length;

    int32_t n_motors;
    const int32_t* mt_cyl;
    const double* mt_pos;
    const double* mt_k;
    const double* mt_eq_length;

    int32_t n_planes;               /* plane boundary elements */
    const double* planes;           /* [4*n_planes] a, b, c, d of a x + b y + c z + d = 0 */
    const double* plane_k;          /* repulsion constant */
    const double* plane_screen;     /* screening length */

    double box[3];                  /* extent of the bin grid (SysParams NX*compartmentSizeX, ...) */
    double exvol_cutoff;            /* VolumeCutoff (rMax of the cylinder pair list; rMin = 0) */
    double boundary_cutoff;         /* BoundaryCutoff */
} MechNetwork;

/* Mirrors ConjugateGradientParams (Mechanics/Minimizer/CGMethod.hpp:44-63). */
typedef struct MechCGParams {
    int32_t method;                 /* 0 steepest, 1 Fletcher-Reeves, 2 Polak-Ribiere */
    double max_dist;
    double lambda_max;
    double grad_tol;
    double energy_rel_tol;
    int32_t energy_call_limit;      /* 0: none */
    int32_t force_call_limit;       /* effective limit is max(this, 3 * beads) */
    int32_t report_on_call_limit;
    int32_t try_to_recover;
} MechCGParams;

/* Mirrors MinimizationResult (Mechanics/Minimizer/MinimizationTypes.hpp:10-66)
 * and the two EnergyReports, plus device-side counters. */
typedef struct MechResult {
    uint32_t error_flags;           /* bit 0: line search error */
    int32_t status;                 /* MECH_OK or MECH_ERR_* */
    int32_t num_energy_call;        /* counted as the reference counts them */
    int32_t energy_call_limit;
    int32_t num_force_call;
    int32_t force_call_limit;
    int32_t num_iter;
    int32_t num_safe_mode;
    int32_t num_recover;
    int32_t num_line_search_trials;
    int32_t num_energy_eval;        /* energy evaluations actually run */
    int32_t used_backup;
    double grad_inf_norm;
    double grad_tol;
    double energy_rel_change;
    double energy_rel_tol;
    double energies_before[MECH_NUM_FF + 1];   /* per force field, then total */
    double energies_after[MECH_NUM_FF + 1];
    double seconds;                 /* wall time of the minimization on the host clock */
} MechResult;

/* Counts of the lists built by the last neighbor-list rebuild. */
typedef struct MechListInfo {
    int64_t n_exvol_pairs;          /* cylinder-cylinder half list */
    int64_t n_boundary_beads;       /* boundary interactions (beads) */
    int64_t n_boundary_cyl;         /* boundary-cylinder neighbor entries */
    double cell_size;               /* bin edge used by the rebuild */
    int64_t n_cells;
} MechListInfo;

typedef struct MechContext MechContext;

/* Version and error text. */
int32_t mech_abi_version(void);
const char* mech_last_error(void);

/*
 * Context with `n_replicas` independent networks, minimized together.
 * Replaces ForceFieldManager construction + MController::initialize
 * (Controller/MController.h:97-104); one replica is the plain MEDYAN case.
 */
int32_t mech_ctx_create(int32_t precision, int32_t device, MechContext** out);
int32_t mech_ctx_destroy(MechContext* ctx);

/*
 * Load networks: serializeDof + ForceFieldManager::vectorizeAllForceFields
 * (Structure/DofSerializer.hpp:64-187, Mechanics/ForceField/ForceFieldManager.cpp:35-93).
 * Rebuilds the neighbor lists at the given coordinates.
 */
int32_t mech_set_networks(MechContext* ctx, int32_t n_replicas, const MechNetwork* nets);

/* Replace the coordinates of replica r (caller bead order); lists are kept. */
int32_t mech_set_coords(MechContext* ctx, int32_t replica, const double* coord);
int32_t mech_get_coords(MechContext* ctx, int32_t replica, double* coord);

/*
 * SubSystem::resetNeighborLists for the hot path (Structure/SubSystem.cpp:193-206):
 * HybridCylinderCylinderNL (HybridNeighborListImpl.cpp:527-556) and
 * BoundaryCylinderNL (NeighborListImpl.cpp:801-809), at the current coordinates.
 * cell_size <= 0 lets the library choose the bin edge (any edge >= rMax gives
 * the same list).
 */
int32_t mech_rebuild_neighbors(MechContext* ctx, double cell_size, MechListInfo* info);

/*
 * The sorted cylinder pair list of replica r as (c, n) cylinder indices,
 * id_c > id_n, ordered by c then n.  Writes min(cap, count) pairs; *count
 * receives the total.
 */
int32_t mech_get_pairs(MechContext* ctx, int32_t replica, int32_t* pairs, int64_t cap, int64_t* count);

/*
 * The BoundaryCylinderNL of replica r built by the last rebuild
 * (Structure/NeighborListImpl.cpp:801-809): for each plane in order, the
 * cylinders whose midpoint lies closer than BoundaryCutoff, ascending, as
 * (plane, cylinder) pairs.  Writes min(cap, count) pairs; *count receives the
 * total.
 */
int32_t mech_get_boundary_list(MechContext* ctx, int32_t replica, int32_t* entries, int64_t cap, int64_t* count);

/*
 * Boundary load forces on the filament ends of replica r at its current
 * coordinates, with the boundary list of the last rebuild: what
 * ForceFieldManager::computeLoadForces (ForceFieldManager.cpp:292-311) leaves
 * in Bead::loadForcesP / loadForcesM after a minimization
 * (MController::afterMinimization_, Controller/MController.h:240-268) for the
 * chemistry's polymerization rate changers.  For each plane in order and each
 * listed cylinder, a plus-end cylinder loads its second bead and a minus-end
 * cylinder its first (BoundaryCylinderRepulsion.cpp:122-192): monomer i at
 * bd + i * mon_size * dir, dir the unit vector from the other bead, gets
 * max(-n . dir, 0) * K exp(-dist / lambda) / lambda
 * (BoundaryCylinderRepulsionExp.cpp:113-118).  mon_size[t] and n_mon[t]
 * (SysParams::Geometry().monomerSize, cylinderNumMon) are given per filament
 * type t < n_types.  plus / minus: [n_filaments * stride] doubles, filament f's
 * monomers at f * stride; entries with i >= n_mon of the filament's type are 0.
 */
int32_t mech_load_forces(MechContext* ctx, int32_t replica, int32_t n_types, const double* mon_size,
                         const int32_t* n_mon, int32_t stride, double* plus, double* minus);

/*
 * Diagnostic: the filament energy terms of replica r at its current
 * coordinates as the engine computes them before summing (FP32 terms in a
 * mixed context, FP64 in an FP64 one), per cylinder in the caller's order:
 * stretch[c] its stretching energy, bend[c] the bending energy of the triple
 * ending in it (0 for a filament's first cylinder).  Summing these exactly
 * and comparing with mech_energy separates the engine's accumulation error
 * from the error of its terms.  No reference counterpart.
 */
int32_t mech_energy_terms(MechContext* ctx, int32_t replica, double* stretch, double* bend);

/*
 * ForceFieldManager::computeIndividualEnergies and ::computeEnergy
 * (ForceFieldManager.cpp:96-227) at `coord` (NULL: current coordinates).
 * per_ff receives MECH_NUM_FF energies; *total the plain sum and *energy the
 * computeEnergy value (+inf when a force field reports failure).
 */
int32_t mech_energy(MechContext* ctx, int32_t replica, const double* coord, double* per_ff, double* total,
                    double* energy);

/* ForceFieldManager::computeForces (ForceFieldManager.cpp:242-290): f_out is
 * overwritten with the total force at `coord` (NULL: current coordinates). */
int32_t mech_forces(MechContext* ctx, int32_t replica, const double* coord, double* f_out);

/*
 * CGMethod::minimize (CGMethod.hpp:826-1743) with MController's recovery move
 * (MController.h:273-339), on every replica at once, starting from the current
 * coordinates.  results[r] is filled per replica; the final coordinates stay in
 * the context (mech_get_coords) and the final forces can be read with
 * mech_get_forces.
 */
int32_t mech_minimize(MechContext* ctx, const MechCGParams* params, MechResult* results);
int32_t mech_get_forces(MechContext* ctx, int32_t replica, double* f_out);

/*
 * How mech_minimize drives the device.  MECH_GRAPH_UNROLLED (default): a graph
 * of 8 unrolled iteration blocks (line search: 2 single-trial passes, FP64,
 * or one two-trial pass, mixed; forces, direction,
 * reset) relaunched by the host, every kernel reading its replica's phase and
 * exiting when it has nothing to do.  MECH_GRAPH_CONDITIONAL: one CUDA graph
 * whose device while loop runs, per body, only the phases some replica is in
 * (line-search pass, forces, direction, reset to steepest descent); the host is
 * involved only for recovery moves, errors and every 512 bodies.  Both run the
 * same active kernels in the same order and give bitwise the same results; on
 * GB300 with driver 580 the conditional bodies cost more than the idle
 * launches they replace (1M-cylinder minimization: 242 vs 199 us per
 * iteration).  No reference counterpart (the reference minimizer is a host
 * loop).
 */
#define MECH_GRAPH_CONDITIONAL 0
#define MECH_GRAPH_UNROLLED 1
/* the unrolled graph with programmatic dependent launch on its main lane: the
 * kernels around each single-block reduction are scheduled while their
 * predecessor runs and wait for it on the device (same results) */
#define MECH_GRAPH_UNROLLED_PDL 2
/* the unrolled graph with each iteration's tail after the force lanes (force
 * gather, force reduction, direction update, its reduction, reset) run as one
 * cooperative launch whose blocks meet at grid barriers instead of five
 * launches (mixed contexts with one replica; other contexts use
 * MECH_GRAPH_UNROLLED).  Same work units, partial slots and reduction order:
 * bitwise the same results.  A grid barrier that waits too long ends the
 * minimization with MECH_ERR_ITER_LIMIT. */
#define MECH_GRAPH_UNROLLED_COOP 3
int32_t mech_set_graph_mode(MechContext* ctx, int32_t mode);

/*
 * Per-linker stretch forces of the last force evaluation
 * (LinkerStretching::assignforcemags, LinkerStretching.cpp:117-123; motors alike).
 */
int32_t mech_get_stretch_forces(MechContext* ctx, int32_t replica, double* linker_f, double* motor_f);

/* Device time of the kernels of the last mech_minimize, by kernel family
 * (milliseconds, CUDA events), and the number of kernel launches. */
typedef struct MechTiming {
    double ms_total;
    double ms_line_search;
    double ms_force;
    double ms_direction;
    double ms_rebuild;
    int64_t launches;
    int64_t graph_launches;
} MechTiming;
int32_t mech_get_timing(MechContext* ctx, MechTiming* t);

/* Restore every replica's coordinates to those given at mech_set_networks
 * (device-to-device; no host transfer). */
int32_t mech_reset_coords(MechContext* ctx);

/*
 * Average device time per launch (milliseconds, CUDA events on the context's
 * stream) of the evaluation kernels at the current coordinates, each captured
 * once as a CUDA graph and replayed `iters` times in plain-evaluation mode: a
 * full energy evaluation, a full force evaluation, their parts, and an idle
 * iteration block.
 */
typedef struct MechProfile {
    double ms_energy_eval;         /* all kernels of one energy evaluation */
    double ms_force_eval;          /* all kernels of one force evaluation */
    double ms_fil_energy;          /* filament stretching + bending energy */
    double ms_fil_force;           /* filament forces + sparse gather + CG partials */
    double ms_bond_energy;         /* linkers, motors, boundary: energy */
    double ms_bond_force;          /* linkers, motors, boundary: contributions */
    double ms_exvol_energy;        /* excluded volume (with its fallback check) */
    double ms_exvol_force;
    int64_t n_beads, n_exvol_pairs, n_boundary, n_linkers, n_motors, n_slots;
    int64_t n_exvol_ext_energy;    /* mixed engine: pairs its last energy pass sent to the extended-precision pass */
    int64_t n_exvol_ext_force;     /* and its last force pass */
    double ms_iteration_idle;      /* one minimizer iteration block (two line-search trials, forces,
                                      direction, reset) with no replica selected:
                                      the cost of the launches that find nothing to do */
    double ms_trial_energy_eval;   /* one line-search trial: energy at x + lambda d, trial positions written */
    int64_t n_exvol_fallback_energy;   /* pairs the last energy pass sent to the Simpson fallback */
    int64_t n_exvol_fallback_force;    /* and the last force pass */
    double ms_fil_energy_trial;    /* filament energy of a trial (x + lambda d formed and written) */
    double ms_fil_force_kernel;    /* filament forces alone (without the gather and reduction) */
    double ms_force_gather;        /* sparse gather with the CG partials alone */
} MechProfile;
int32_t mech_profile(MechContext* ctx, int32_t iters, MechProfile* out);

/*
 * Autotuner: times the candidate launch geometries of this context's kernels
 * on its own networks and keeps the fastest (CUDA events; the neighbor-list
 * bin edge by wall time of a rebuild, since any edge >= rMax gives the same
 * pair list).  Results are cached per network shape for the process; a later
 * context of the same shape reuses them unless MECH_TUNE_FORCE is given.  No
 * reference counterpart (MEDYAN fixes its bin size in the input file).
 */
#define MECH_TUNE_KERNELS  1   /* tiles per block of the mixed filament kernels */
#define MECH_TUNE_CELL     2   /* neighbor-list bin edge (scale of the default) */
#define MECH_TUNE_FORCE    4   /* ignore the cache */
typedef struct MechTuning {
    int32_t energy_tiles_per_block;
    int32_t force_tiles_per_block;
    double cell_scale;              /* multiplier on the default bin edge */
    double ms_energy, ms_force;     /* best filament-kernel times found (ms) */
    double ms_rebuild;              /* best rebuild wall time found (ms) */
    int32_t energy_blocks_per_sm;   /* resident blocks per SM of the persistent filament energy kernel */
    int32_t force_blocks_per_sm;    /* and of the filament force kernel (0: as many as fit); fewer leave SM
                                       room for the excluded-volume and linker lanes running beside them.
                                       A new context uses 0 (energy) and 2 (force); with a cap the grid
                                       holds one resident wave, its runs lengthened as needed, and the
                                       kernel is launched before the side lanes */
} MechTuning;
int32_t mech_autotune(MechContext* ctx, int32_t flags, MechTuning* out);
int32_t mech_set_tuning(MechContext* ctx, const MechTuning* t);

/*
 * Second-order calls (FP64 contexts; a mixed context returns MECH_ERR_STATE).
 * They replace ForceFieldManager::computeHessian's finite-difference Hessian
 * (Mechanics/ForceField/ForceFieldManager.cpp:354-489) with exact
 * Hessian-vector products: every force field differentiated in forward mode
 * along v, at the context's current coordinates and neighbor lists.
 */
typedef struct MechSolveParams {
    double rel_tol;                 /* CG stops at |r| <= rel_tol |b| */
    int32_t max_iter;               /* CG iterations per solve */
    double shift;                   /* solves (H + shift I) y = b; 0 for the plain Hessian */
} MechSolveParams;

typedef struct MechSolveInfo {
    int32_t iterations;             /* CG iterations (summed over Newton steps) */
    int32_t converged;              /* last solve reached rel_tol */
    double rel_residual;            /* |r| / |b| of the last solve */
    int64_t launches;               /* kernel launches */
    int32_t newton_steps;           /* mech_newton_refine only */
    double max_force;               /* mech_newton_refine: max |F| at exit */
    int32_t negative_curvature;     /* a solve met p . H p <= 0 and stopped there */
} MechSolveInfo;

/*
 * hv = H v for replica r (caller bead order, 3 doubles per bead).
 * MECH_HVP_ENERGY: the exact Hessian of the total energy (symmetric).
 * MECH_HVP_FORCE_JACOBIAN: minus the Jacobian of computeForces as the
 * reference evaluates it, including its move of nearly coplanar
 * excluded-volume pairs off their plane (CylinderExclVolRepulsion.cpp:610-626),
 * which makes it slightly non-symmetric; this is what the reference's
 * finite-difference computeHessian approximates before symmetrizing.
 */
#define MECH_HVP_ENERGY          0
#define MECH_HVP_FORCE_JACOBIAN  1
int32_t mech_hvp(MechContext* ctx, int32_t replica, int32_t mode, const double* v, double* hv);

/* Replace the stiffness and/or rest length of replica r's linkers (NULL keeps
 * one); the parameters the adjoint differentiates. */
int32_t mech_set_linker_params(MechContext* ctx, int32_t replica, const double* k, const double* eq_length);

/*
 * Implicit adjoint at an equilibrium x* of replica r: for a loss
 * L(x*, theta) = dL_dE * E(x*, theta) + R(x*) with dL_dx = dR/dx at x*,
 * solves H lambda = dL_dx by CG and returns, per linker,
 *   dL/dk  = dL_dE * dE/dk  - lambda . d(grad_x E)/dk
 *   dL/dl0 = dL_dE * dE/dl0 - lambda . d(grad_x E)/dl0
 * (the E term contributes no implicit part since grad_x E = 0 at x*).
 * Returns MECH_ERR_ITER_LIMIT (gradients still written) if CG stopped early.
 */
int32_t mech_adjoint(MechContext* ctx, int32_t replica, const double* dL_dx, double dL_dE, const MechSolveParams* sp,
                     double* dL_dk, double* dL_dl0, MechSolveInfo* info);

/* Newton refinement of every replica's equilibrium (run after mech_minimize):
 * dx = (H + shift I)^-1 F by CG (truncated at non-positive curvature), then
 * x += alpha dx, alpha halved from 1 until the energy drops or max |F|
 * halves (shift grows tenfold when no alpha does); repeated until
 * max |F| < force_tol, max_steps steps, or no progress. */
int32_t mech_newton_refine(MechContext* ctx, int32_t max_steps, double force_tol, const MechSolveParams* sp,
                           MechSolveInfo* info);

/*
 * Filament stretching and bending energies (FP64) of one network held in
 * caller-owned DEVICE memory, without allocating: no reference counterpart
 * (MEDYAN evaluates these inside ForceFieldManager::computeIndividualEnergies;
 * this is a stand-alone variant for callers that cannot allocate).
 *
 * For callers that must not allocate device memory at this point: cudaMalloc
 * and cudaFree can synchronize the whole device, and some hosts hand every
 * byte of HBM to their own pool up front.  The call needs no context; its
 * scratch is a fixed 131,328-byte device array inside the library.
 *
 * Inputs (device pointers, current device): fil_cyl_start[n_filaments+1]
 * strictly ascending cylinder ranges from 0 to n_cylinders: every filament
 * holds at least one cylinder, as every MEDYAN filament does (not checked:
 * the arrays are on the device; an empty filament shifts the beads of every
 * later filament and gives wrong energies); coord[3 * (n_cylinders + n_filaments)] with the
 * beads filament by filament, minus end first (cylinder c of filament f joins
 * beads c + f and c + f + 1); per-cylinder k_stretch, eq_length, k_bend,
 * eq_theta (the bending triple ending in cylinder c uses c's constants).
 * Output: energies[2] = {stretching, bending}, written on `stream` (a
 * cudaStream_t; NULL = legacy default stream); synchronize before reading.
 *
 * Limits: n_cylinders <= 2,097,152, else MECH_ERR_CAPACITY and nothing runs.
 * The first call in each CUDA context of a device looks up the scratch
 * address (again after a cudaDeviceReset or any other re-creation of the
 * context, since the array can move): make that call before any stream
 * capture on that device.  The scratch's completion ticket must be
 * zero at launch: the call clears it on `stream` and the kernel leaves it
 * zero.  Calls that overlap in time on one device share the scratch and
 * race: issue them on one stream or order them.
 */
int32_t mech_filament_energy_device(int32_t n_filaments, int32_t n_cylinders, const int32_t* fil_cyl_start,
                                    const double* coord, const double* k_stretch, const double* eq_length,
                                    const double* k_bend, const double* eq_theta, double* energies, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MEDYAN_MECH_H */
