// medyan_mech.hpp — header-only C++ front end of the C ABI in medyan_mech.h.
//
// Shaped like the two interfaces MEDYAN's MController binds (paths relative
// to medyan-5.4.0/src of the reference):
//   * ForceFieldSet mirrors ForceFieldManager's evaluation calls
//     (Mechanics/ForceField/ForceFieldManager.h:64-123): computeEnergy,
//     computeIndividualEnergies, computeForces, assignallforcemags;
//   * ForceFieldSet::minimize mirrors CGMethod::minimize
//     (Mechanics/Minimizer/CGMethod.hpp:826-836) returning a result record.
// Errors surface as exceptions on this side, as the reference's minimizer
// throws std::runtime_error (CGMethod.hpp:202-212); the C ABI underneath
// never throws.  Only the C ABI crosses the library boundary.
#pragma once

#include <cmath>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "medyan_mech.h"

namespace medyan_mech {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int32_t rc, const char* where) {
    if (rc != MECH_OK) {
        const char* msg = mech_last_error();
        throw Error(rc, std::string(where) + ": " + (msg ? msg : "") + " (status " + std::to_string(rc) + ")");
    }
}

enum class Precision : int32_t { FP64 = MECH_PREC_FP64, Mixed = MECH_PREC_MIXED };

// CG parameters with MController's defaults and the example input's LAMBDAMAX
// (Controller/MController.cpp:34-63).
inline MechCGParams default_cg_params() {
    MechCGParams p{};
    p.method = 2;
    p.max_dist = 1.0;
    p.lambda_max = 0.01;
    p.grad_tol = 1.0;
    p.energy_rel_tol = 1e-9;
    p.energy_call_limit = 0;
    p.force_call_limit = 10000;
    p.report_on_call_limit = 1;
    p.try_to_recover = 1;
    return p;
}

// One device context holding one network (replica 0) or an ensemble.
class ForceFieldSet {
public:
    explicit ForceFieldSet(Precision prec = Precision::FP64, int device = 0) {
        check(mech_ctx_create(static_cast<int32_t>(prec), device, &ctx_), "mech_ctx_create");
    }
    ~ForceFieldSet() {
        if (ctx_) mech_ctx_destroy(ctx_);
    }
    ForceFieldSet(const ForceFieldSet&) = delete;
    ForceFieldSet& operator=(const ForceFieldSet&) = delete;
    ForceFieldSet(ForceFieldSet&& o) noexcept : ctx_(std::exchange(o.ctx_, nullptr)), nbeads_(std::move(o.nbeads_)) {}

    // vectorizeAllForceFields + serializeDof: copies the network in and
    // builds the neighbor lists at its coordinates.
    void vectorize(const std::vector<MechNetwork>& nets) {
        check(mech_set_networks(ctx_, static_cast<int32_t>(nets.size()), nets.data()), "mech_set_networks");
        nbeads_.clear();
        for (const auto& n : nets) nbeads_.push_back(n.n_beads);
    }
    void vectorize(const MechNetwork& net) { vectorize(std::vector<MechNetwork>{net}); }

    // SubSystem::resetNeighborLists for the hot path.
    MechListInfo resetNeighborLists(double cell_size = 0.0) {
        MechListInfo info{};
        check(mech_rebuild_neighbors(ctx_, cell_size, &info), "mech_rebuild_neighbors");
        return info;
    }

    // computeEnergy: +inf when a force field reports failure.
    double computeEnergy(const double* coord, int replica = 0) {
        double per[MECH_NUM_FF], total = 0, energy = 0;
        check(mech_energy(ctx_, replica, coord, per, &total, &energy), "mech_energy");
        return energy;
    }
    // computeIndividualEnergies: one entry per force field, MController's order.
    std::vector<double> computeIndividualEnergies(const double* coord, int replica = 0) {
        std::vector<double> per(MECH_NUM_FF);
        double total = 0, energy = 0;
        check(mech_energy(ctx_, replica, coord, per.data(), &total, &energy), "mech_energy");
        return per;
    }
    // computeForces: f is overwritten (zero-fill + every force field).
    void computeForces(const double* coord, double* f, int replica = 0) {
        check(mech_forces(ctx_, replica, coord, f), "mech_forces");
    }

    // CGMethod::minimize on every replica from the current coordinates; the
    // minimized coordinates are copied into coord_out (if given) and the final
    // forces into force_out (if given), as minimize() hands back its force vector.
    std::vector<MechResult> minimize(const MechCGParams& params, double* coord_out = nullptr,
                                     double* force_out = nullptr, int replica = 0) {
        std::vector<MechResult> res(nbeads_.size());
        const int32_t rc = mech_minimize(ctx_, &params, res.data());
        if (rc != MECH_OK && rc != MECH_ERR_LINESEARCH) check(rc, "mech_minimize");
        if (coord_out) check(mech_get_coords(ctx_, replica, coord_out), "mech_get_coords");
        if (force_out) check(mech_get_forces(ctx_, replica, force_out), "mech_get_forces");
        return res;
    }

    void setCoordinates(const double* coord, int replica = 0) {
        check(mech_set_coords(ctx_, replica, coord), "mech_set_coords");
    }
    // assignallforcemags for linkers and motors: stretch force of each.
    void linkerMotorForces(double* linker_f, double* motor_f, int replica = 0) {
        check(mech_get_stretch_forces(ctx_, replica, linker_f, motor_f), "mech_get_stretch_forces");
    }

    MechContext* handle() const { return ctx_; }

private:
    MechContext* ctx_ = nullptr;
    std::vector<int32_t> nbeads_;
};

}  // namespace medyan_mech
