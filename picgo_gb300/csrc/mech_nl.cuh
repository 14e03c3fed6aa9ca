// Inputs and scratch of the neighbor-list and CSR builds (mech_nl.cu).
#pragma once

#include "mech_internal.cuh"

namespace mech {

struct NLInput {
    int ncyl;                  // all replicas
    const int* cyl_b1;         // internal index of the first bead (the second is +1)
    const int64_t* cyl_id;
    const int* cyl_fil;
    const int* cyl_pos;
    const int* cyl_rep;
    const void* x;             // current coordinates (engine format)
    int mixed;                 // 1: float hi/lo pairs, 0: doubles
    const double* rep_cell;    // [R] cell edge
    const int4* rep_dims;      // [R] gx, gy, gz, first cell index
    const double* rep_rmax2;   // [R] rMax^2 rounded to float, held as double
    const double* rep_rmin2;
    int R;
    long long ncells;
};

struct PairBuild {
    DeviceBuffer cell_count, cell_start, cell_cursor, sorted, mid, midf, cell_of, cnt, off, pairs, scan_tmp;
};

// Half pair list into pb.pairs (int2 (c, n)); *npairs receives the count.
// rep_margin[r] is the single-precision prefilter slack of replica r.
cudaError_t build_pairs(const NLInput& in, PairBuild& pb, const float* rep_margin, long long* npairs, cudaStream_t s);

struct BndInput {
    long long nq;              // sum over replicas of planes * cylinders
    int R;
    const long long* rep_q;    // [R] first entry of replica r
    const int* rep_ncyl;       // [R]
    const int* rep_plane;      // [R] first global plane
    const int* rep_cyl;        // [R] first global cylinder
    const double* cutoff;      // [R]
    const double* planes;      // [4 * planes]
    const int* cyl_b1;
    const uint8_t* cyl_minus;  // filament minus-end cylinder
};

struct BndBuild {
    DeviceBuffer cnt, off, bead, plane, scan_tmp, ncyl;
};

// cnt[q] (kept until the next rebuild) is 0 for an entry q = (plane, cylinder)
// outside the list, else the beads it contributes (2 for a minus-end cylinder);
// *ncyl receives the number of listed (plane, cylinder) entries.
cudaError_t build_boundary(const BndInput& in, const double* mid, BndBuild& bb, long long* nbeads, long long* ncyl,
                           cudaStream_t s);

struct CsrInput {
    int nb;
    int base[5];               // slot ranges: linker, motor, exvol, boundary, end
    const int4* lk;
    const int4* mt;
    const int4* ev;
    const int* bb;
};

struct CsrBuild {
    DeviceBuffer cnt, cursor, off, slots, pos, scan_tmp;   // pos: slot -> its CSR position
};

cudaError_t build_csr(const CsrInput& in, CsrBuild& cb, cudaStream_t s);

}  // namespace mech
