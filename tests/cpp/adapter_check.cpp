// C++ host check of include/medyan_mech.hpp: loads a network written by
// tests/test_cpp_adapter.py (raw little-endian arrays in a directory), then
// evaluates energies and forces, minimizes, and writes the results back as
// raw arrays for the test to compare.
//
//   adapter_check <dir> <precision 0|1>
// Exit status: 0 ok, 3 no CUDA device (MECH_ERR_NO_DEVICE), 1 any other error.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "medyan_mech.hpp"

namespace {

template <typename T>
std::vector<T> load(const std::string& dir, const std::string& name) {
    std::ifstream f(dir + "/" + name + ".bin", std::ios::binary | std::ios::ate);
    if (!f) throw std::runtime_error("missing " + name);
    const std::streamsize n = f.tellg();
    f.seekg(0);
    std::vector<T> v(static_cast<size_t>(n) / sizeof(T));
    f.read(reinterpret_cast<char*>(v.data()), n);
    return v;
}

template <typename T>
void save(const std::string& dir, const std::string& name, const std::vector<T>& v) {
    std::ofstream f(dir + "/" + name + ".bin", std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <dir> <precision>\n", argv[0]);
        return 1;
    }
    const std::string dir = argv[1];
    const int prec = std::atoi(argv[2]);
    try {
        const auto coord = load<double>(dir, "coord");
        const auto fcs = load<int32_t>(dir, "fil_cyl_start");
        const auto cyl_bead = load<int32_t>(dir, "cyl_bead");
        const auto cyl_id = load<int64_t>(dir, "cyl_id");
        const auto cyl_fil = load<int32_t>(dir, "cyl_filament_id");
        const auto cyl_pos = load<int32_t>(dir, "cyl_position");
        const auto cyl_type = load<int32_t>(dir, "cyl_type");
        const auto l0 = load<double>(dir, "cyl_eq_length");
        const auto ks = load<double>(dir, "cyl_k_stretch");
        const auto kb = load<double>(dir, "cyl_k_bend");
        const auto t0 = load<double>(dir, "cyl_eq_theta");
        const auto kex = load<double>(dir, "cyl_k_exvol");
        const auto lk_cyl = load<int32_t>(dir, "lk_cyl");
        const auto lk_pos = load<double>(dir, "lk_pos");
        const auto lk_k = load<double>(dir, "lk_k");
        const auto lk_l0 = load<double>(dir, "lk_eq_length");
        const auto planes = load<double>(dir, "planes");
        const auto plane_k = load<double>(dir, "plane_k");
        const auto plane_s = load<double>(dir, "plane_screen");
        const auto misc = load<double>(dir, "misc");   // box, exvol cutoff, boundary cutoff

        MechNetwork net{};
        net.n_beads = static_cast<int32_t>(coord.size() / 3);
        net.coord = coord.data();
        net.n_filaments = static_cast<int32_t>(fcs.size() - 1);
        net.fil_cyl_start = fcs.data();
        net.n_cylinders = static_cast<int32_t>(l0.size());
        net.cyl_bead = cyl_bead.data();
        net.cyl_id = cyl_id.data();
        net.cyl_filament_id = cyl_fil.data();
        net.cyl_position = cyl_pos.data();
        net.cyl_type = cyl_type.data();
        net.cyl_eq_length = l0.data();
        net.cyl_k_stretch = ks.data();
        net.cyl_k_bend = kb.data();
        net.cyl_eq_theta = t0.data();
        net.cyl_k_exvol = kex.data();
        net.n_linkers = static_cast<int32_t>(lk_k.size());
        net.lk_cyl = lk_cyl.data();
        net.lk_pos = lk_pos.data();
        net.lk_k = lk_k.data();
        net.lk_eq_length = lk_l0.data();
        net.n_motors = 0;
        net.n_planes = static_cast<int32_t>(plane_k.size());
        net.planes = planes.data();
        net.plane_k = plane_k.data();
        net.plane_screen = plane_s.data();
        for (int k = 0; k < 3; ++k) net.box[k] = misc[0];
        net.exvol_cutoff = misc[1];
        net.boundary_cutoff = misc[2];

        medyan_mech::ForceFieldSet ffs(prec ? medyan_mech::Precision::Mixed : medyan_mech::Precision::FP64);
        ffs.vectorize(net);
        std::vector<double> per = ffs.computeIndividualEnergies(coord.data());
        per.push_back(ffs.computeEnergy(coord.data()));
        std::vector<double> f(coord.size());
        ffs.computeForces(coord.data(), f.data());
        MechCGParams p = medyan_mech::default_cg_params();
        std::vector<double> xmin(coord.size()), fmin(coord.size());
        const auto res = ffs.minimize(p, xmin.data(), fmin.data());
        save(dir, "out_energies", per);
        save(dir, "out_forces", f);
        save(dir, "out_coord", xmin);
        save(dir, "out_min_forces", fmin);
        save(dir, "out_result", std::vector<double>{static_cast<double>(res[0].status), res[0].grad_inf_norm,
                                                    static_cast<double>(res[0].num_iter),
                                                    res[0].energies_after[MECH_NUM_FF]});
        std::printf("ok: E=%.10g maxF=%.4g after %d iterations\n", per.back(), res[0].grad_inf_norm, res[0].num_iter);
        return 0;
    } catch (const medyan_mech::Error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return e.code() == MECH_ERR_NO_DEVICE ? 3 : 1;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
