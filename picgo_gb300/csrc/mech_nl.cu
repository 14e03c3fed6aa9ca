// Neighbor-list rebuild on the device, the exclusive scan it uses, and the
// bead-to-contribution CSR index of the sparse force fields.
//
// Cylinder-cylinder half list (HybridCylinderCylinderNL, paths relative to
// medyan-5.4.0/src: Structure/HybridNeighborListImpl.cpp:176-471 and
// Structure/BinGrid.h:134-199): midpoints binned on a uniform grid whose cell
// edge is at least rMax, a 27-cell stencil, and the reference's predicate --
// keep (c, n) when id_c > id_n, the two are not within two positions of the
// same filament, and rMin^2 <= |m_n - m_c|^2 <= rMax^2 with the square summed
// in double from zero and the bounds rounded to float as the reference stores
// them.  The stencil covers every cell that can hold a neighbor, so the set is
// the same for every cell edge >= rMax; a single-precision distance prefilter
// with a conservative margin only skips candidates that cannot pass.  Each
// cylinder's neighbors are written in ascending cylinder order.
//
// Boundary-cylinder list (Structure/NeighborListImpl.cpp:738-751): per plane,
// every cylinder whose midpoint lies closer than BoundaryCutoff (signed
// distance), plane by plane in cylinder order; a filament's minus-end cylinder
// contributes its first bead as well as its second
// (Mechanics/ForceField/Boundary/BoundaryCylinderRepulsion.cpp:33-88).
#include <cuda_runtime.h>

#include "mech_device.cuh"
#include "mech_nl.cuh"

namespace mech {

cudaError_t DeviceBuffer::ensure(size_t nbytes) {
    if (nbytes <= bytes && p) return cudaSuccess;
    release();
    size_t want = nbytes < 256 ? 256 : nbytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        p = nullptr;
        bytes = 0;
        return e;
    }
    bytes = want;
    return cudaSuccess;
}

void DeviceBuffer::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

// ---------------------------------------------------------------------------
// exclusive scan (three passes; recursive over block sums)
// ---------------------------------------------------------------------------
constexpr int kScanItems = 4;
constexpr int kScanBlock = 256;
constexpr int kScanTile = kScanItems * kScanBlock;

__global__ void k_scan_tile(const int* in, int* out, int* sums, long long n) {
    __shared__ int sh[kScanBlock];
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int run = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        run += v[k];
    }
    sh[threadIdx.x] = run;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {
        const int add = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += add;
        __syncthreads();
    }
    int pre = sh[threadIdx.x] - run;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = pre;
        pre += v[k];
    }
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = sh[threadIdx.x];
}

__global__ void k_scan_add(int* out, const int* offs, long long n) {
    const long long base = (long long)blockIdx.x * kScanTile;
    const int add = offs[blockIdx.x];
    for (int k = threadIdx.x; k < kScanTile; k += blockDim.x)
        if (base + k < n) out[base + k] += add;
}

__global__ void k_scan_total(const int* in, int* out, long long n) {
    // out[n] = out[n-1] + in[n-1]
    if (n > 0) out[n] = out[n - 1] + in[n - 1];
    else out[0] = 0;
}

static cudaError_t scan_rec(const int* in, int* out, long long n, int* tmp, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const long long nb = (n + kScanTile - 1) / kScanTile;
    int* sums = tmp;
    int* sums_scan = tmp + nb;
    k_scan_tile<<<(unsigned)nb, kScanBlock, 0, s>>>(in, out, sums, n);
    if (nb > 1) {
        cudaError_t e = scan_rec(sums, sums_scan, nb, tmp + 2 * nb, s);
        if (e != cudaSuccess) return e;
        k_scan_add<<<(unsigned)nb, kScanBlock, 0, s>>>(out, sums_scan, n);
    }
    return cudaGetLastError();
}

cudaError_t exclusive_scan_i32(const int* in, int* out, long long n, DeviceBuffer& tmp, cudaStream_t s) {
    // scratch for all recursion levels: < 2 * (n / kScanTile) * (1 + 1/kScanTile + ...) + slack
    long long need = 64;
    for (long long m = n; m > 1; m = (m + kScanTile - 1) / kScanTile) need += 2 * ((m + kScanTile - 1) / kScanTile) + 2;
    cudaError_t e = tmp.ensure(sizeof(int) * (size_t)need);
    if (e != cudaSuccess) return e;
    e = scan_rec(in, out, n, tmp.as<int>(), s);
    if (e != cudaSuccess) return e;
    k_scan_total<<<1, 1, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// cylinder pair list
// ---------------------------------------------------------------------------
__device__ __forceinline__ int cell_axis(double m, double cell, int g) {
    int i = (int)floor(m / cell);
    return i < 0 ? 0 : (i >= g ? g - 1 : i);
}

__global__ void k_nl_mid(NLInput in, double* mid, float4* midf, int* cell_of, int* cell_count) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= in.ncyl) return;
    const int b = in.cyl_b1[c];
    double x1[3], x2[3];
    if (in.mixed) {
        to_double(load_pos(static_cast<const float*>(in.x), b), x1);
        to_double(load_pos(static_cast<const float*>(in.x), b + 1), x2);
    } else {
        to_double(load_pos(static_cast<const double*>(in.x), b), x1);
        to_double(load_pos(static_cast<const double*>(in.x), b + 1), x2);
    }
    // 0.5 * (b1 + b2) (Structure/Cylinder.cpp:45-46); equal to the boundary
    // list's b1 * 0.5 + 0.5 * b2 bit for bit
    const double m0 = 0.5 * (x1[0] + x2[0]), m1 = 0.5 * (x1[1] + x2[1]), m2 = 0.5 * (x1[2] + x2[2]);
    mid[3 * (size_t)c] = m0;
    mid[3 * (size_t)c + 1] = m1;
    mid[3 * (size_t)c + 2] = m2;
    midf[c] = make_float4((float)m0, (float)m1, (float)m2, 0.f);
    const int r = in.cyl_rep[c];
    const double cell = in.rep_cell[r];
    const int4 g = in.rep_dims[r];
    const int id = g.w + (cell_axis(m0, cell, g.x) * g.y + cell_axis(m1, cell, g.y)) * g.z + cell_axis(m2, cell, g.z);
    cell_of[c] = id;
    atomicAdd(cell_count + id, 1);
}

__global__ void k_nl_scatter(int n, const int* cell_of, const int* cell_start, int* cursor, int* sorted) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int id = cell_of[c];
    sorted[cell_start[id] + atomicAdd(cursor + id, 1)] = c;
}

// visit every candidate of cylinder c; F(n) is called for accepted neighbors
template <typename F>
__device__ __forceinline__ void nl_visit(const NLInput& in, const double* mid, const float4* midf, const int* cell_start,
                                         const int* sorted, const float* rep_margin, int c, F&& accept) {
    const int r = in.cyl_rep[c];
    const double cell = in.rep_cell[r];
    const int4 g = in.rep_dims[r];
    const double mc0 = mid[3 * (size_t)c], mc1 = mid[3 * (size_t)c + 1], mc2 = mid[3 * (size_t)c + 2];
    const float4 fc = midf[c];
    const double rmax2 = in.rep_rmax2[r], rmin2 = in.rep_rmin2[r];
    const float pre = (float)rmax2 + rep_margin[r];
    const int ix = cell_axis(mc0, cell, g.x), iy = cell_axis(mc1, cell, g.y), iz = cell_axis(mc2, cell, g.z);
    const long long idc = in.cyl_id[c];
    const int filc = in.cyl_fil[c], posc = in.cyl_pos[c];
    for (int dx = -1; dx <= 1; ++dx) {
        const int jx = ix + dx;
        if (jx < 0 || jx >= g.x) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int jy = iy + dy;
            if (jy < 0 || jy >= g.y) continue;
            for (int dz = -1; dz <= 1; ++dz) {
                const int jz = iz + dz;
                if (jz < 0 || jz >= g.z) continue;
                const int id = g.w + (jx * g.y + jy) * g.z + jz;
                const int s0 = cell_start[id], s1 = cell_start[id + 1];
                for (int s = s0; s < s1; ++s) {
                    const int n = sorted[s];
                    const float4 fn = midf[n];
                    const float ex = fn.x - fc.x, ey = fn.y - fc.y, ez = fn.z - fc.z;
                    if (ex * ex + ey * ey + ez * ez > pre) continue;
                    if (idc <= in.cyl_id[n]) continue;
                    if (filc == in.cyl_fil[n] && abs(posc - in.cyl_pos[n]) <= 2) continue;
                    double d2 = 0.0;
                    const double dx0 = mid[3 * (size_t)n] - mc0, dx1 = mid[3 * (size_t)n + 1] - mc1,
                                 dx2 = mid[3 * (size_t)n + 2] - mc2;
                    d2 = __dadd_rn(d2, __dmul_rn(dx0, dx0));
                    d2 = __dadd_rn(d2, __dmul_rn(dx1, dx1));
                    d2 = __dadd_rn(d2, __dmul_rn(dx2, dx2));
                    if (d2 < rmin2 || d2 > rmax2) continue;
                    accept(n);
                }
            }
        }
    }
}

__global__ void k_nl_count(NLInput in, const double* mid, const float4* midf, const int* cell_start, const int* sorted,
                           const float* rep_margin, int* cnt) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= in.ncyl) return;
    int k = 0;
    nl_visit(in, mid, midf, cell_start, sorted, rep_margin, c, [&](int) { ++k; });
    cnt[c] = k;
}

__global__ void k_nl_write(NLInput in, const double* mid, const float4* midf, const int* cell_start, const int* sorted,
                           const float* rep_margin, const int* off, int2* pairs) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= in.ncyl) return;
    const int o = off[c];
    int k = 0;
    nl_visit(in, mid, midf, cell_start, sorted, rep_margin, c, [&](int n) { pairs[o + (k++)] = make_int2(c, n); });
    // ascending neighbor order (insertion sort of this cylinder's short segment)
    for (int i = 1; i < k; ++i) {
        const int2 v = pairs[o + i];
        int j = i - 1;
        while (j >= 0 && pairs[o + j].y > v.y) {
            pairs[o + j + 1] = pairs[o + j];
            --j;
        }
        pairs[o + j + 1] = v;
    }
}

cudaError_t build_pairs(const NLInput& in, PairBuild& pb, const float* rep_margin, long long* npairs, cudaStream_t s) {
    cudaError_t e;
    const int n = in.ncyl;
    if ((e = pb.cell_count.ensure(sizeof(int) * (size_t)(in.ncells + 1))) != cudaSuccess) return e;
    if ((e = pb.cell_start.ensure(sizeof(int) * (size_t)(in.ncells + 1))) != cudaSuccess) return e;
    if ((e = pb.cell_cursor.ensure(sizeof(int) * (size_t)(in.ncells + 1))) != cudaSuccess) return e;
    if ((e = pb.sorted.ensure(sizeof(int) * (size_t)n)) != cudaSuccess) return e;
    if ((e = pb.mid.ensure(sizeof(double) * 3 * (size_t)n)) != cudaSuccess) return e;
    if ((e = pb.midf.ensure(sizeof(float4) * (size_t)n)) != cudaSuccess) return e;
    if ((e = pb.cell_of.ensure(sizeof(int) * (size_t)n)) != cudaSuccess) return e;
    if ((e = pb.cnt.ensure(sizeof(int) * (size_t)(n + 1))) != cudaSuccess) return e;
    if ((e = pb.off.ensure(sizeof(int) * (size_t)(n + 1))) != cudaSuccess) return e;
    cudaMemsetAsync(pb.cell_count.p, 0, sizeof(int) * (size_t)(in.ncells + 1), s);
    cudaMemsetAsync(pb.cell_cursor.p, 0, sizeof(int) * (size_t)(in.ncells + 1), s);
    const int tb = 256, nblk = (n + tb - 1) / tb;
    if (n > 0) {
        k_nl_mid<<<nblk, tb, 0, s>>>(in, pb.mid.as<double>(), pb.midf.as<float4>(), pb.cell_of.as<int>(),
                                     pb.cell_count.as<int>());
    }
    if ((e = exclusive_scan_i32(pb.cell_count.as<int>(), pb.cell_start.as<int>(), in.ncells, pb.scan_tmp, s)) !=
        cudaSuccess)
        return e;
    if (n > 0) {
        k_nl_scatter<<<nblk, tb, 0, s>>>(n, pb.cell_of.as<int>(), pb.cell_start.as<int>(), pb.cell_cursor.as<int>(),
                                         pb.sorted.as<int>());
        k_nl_count<<<nblk, tb, 0, s>>>(in, pb.mid.as<double>(), pb.midf.as<float4>(), pb.cell_start.as<int>(),
                                       pb.sorted.as<int>(), rep_margin, pb.cnt.as<int>());
    }
    if ((e = exclusive_scan_i32(pb.cnt.as<int>(), pb.off.as<int>(), n, pb.scan_tmp, s)) != cudaSuccess) return e;
    int total = 0;
    if ((e = cudaMemcpyAsync(&total, pb.off.as<int>() + n, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    if ((e = pb.pairs.ensure(sizeof(int2) * (size_t)(total > 0 ? total : 1))) != cudaSuccess) return e;
    if (n > 0 && total > 0) {
        k_nl_write<<<nblk, tb, 0, s>>>(in, pb.mid.as<double>(), pb.midf.as<float4>(), pb.cell_start.as<int>(),
                                       pb.sorted.as<int>(), rep_margin, pb.off.as<int>(), pb.pairs.as<int2>());
    }
    *npairs = total;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// boundary list
// ---------------------------------------------------------------------------
// entry q of replica r: plane p = q / nc_r, cylinder c = q % nc_r (replica-local)
__device__ __forceinline__ int rep_of(const BndInput& in, long long q) {
    int lo = 0, hi = in.R - 1;   // last r with rep_q[r] <= q
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (in.rep_q[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
__global__ void k_bnd_count(BndInput in, const double* mid, int* cnt, int* ncyl) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= in.nq) return;
    const int r = rep_of(in, q);
    const long long lq = q - in.rep_q[r];
    const int nc = in.rep_ncyl[r];
    const int p = in.rep_plane[r] + (int)(lq / nc);
    const int c = in.rep_cyl[r] + (int)(lq % nc);
    const double* pl = in.planes + 4 * p;
    // (a x + b y + c z + d) / |n| rounded operation by operation, as the reference's list test
    double num = __dmul_rn(pl[0], mid[3 * (size_t)c]);
    num = __dadd_rn(num, __dmul_rn(pl[1], mid[3 * (size_t)c + 1]));
    num = __dadd_rn(num, __dmul_rn(pl[2], mid[3 * (size_t)c + 2]));
    num = __dadd_rn(num, pl[3]);
    const double nrm = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(pl[0], pl[0]), __dmul_rn(pl[1], pl[1])), __dmul_rn(pl[2], pl[2])));
    const double d = __ddiv_rn(num, nrm);
    const bool listed = d < in.cutoff[r];
    cnt[q] = listed ? (in.cyl_minus[c] ? 2 : 1) : 0;
    const unsigned m = __ballot_sync(__activemask(), listed);
    if (m && (threadIdx.x & 31) == __ffs(__activemask()) - 1) atomicAdd(ncyl, __popc(m));
}

__global__ void k_bnd_write(BndInput in, const int* cnt, const int* off, int* bb_bead, int* bb_plane) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= in.nq) return;
    const int k = cnt[q];
    if (!k) return;
    const int r = rep_of(in, q);
    const long long lq = q - in.rep_q[r];
    const int nc = in.rep_ncyl[r];
    const int p = in.rep_plane[r] + (int)(lq / nc);
    const int c = in.rep_cyl[r] + (int)(lq % nc);
    const int o = off[q];
    const int b1 = in.cyl_b1[c];
    if (k == 2) {
        bb_bead[o] = b1;
        bb_plane[o] = p;
        bb_bead[o + 1] = b1 + 1;
        bb_plane[o + 1] = p;
    } else {
        bb_bead[o] = b1 + 1;
        bb_plane[o] = p;
    }
}

cudaError_t build_boundary(const BndInput& in, const double* mid, BndBuild& bb, long long* nbeads, long long* ncyl,
                           cudaStream_t s) {
    cudaError_t e;
    if ((e = bb.cnt.ensure(sizeof(int) * (size_t)(in.nq + 1))) != cudaSuccess) return e;
    if ((e = bb.off.ensure(sizeof(int) * (size_t)(in.nq + 1))) != cudaSuccess) return e;
    if ((e = bb.ncyl.ensure(sizeof(int))) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(bb.ncyl.p, 0, sizeof(int), s)) != cudaSuccess) return e;
    const int tb = 256;
    const unsigned nblk = (unsigned)((in.nq + tb - 1) / tb);
    if (in.nq > 0) k_bnd_count<<<nblk, tb, 0, s>>>(in, mid, bb.cnt.as<int>(), bb.ncyl.as<int>());
    if ((e = exclusive_scan_i32(bb.cnt.as<int>(), bb.off.as<int>(), in.nq, bb.scan_tmp, s)) != cudaSuccess) return e;
    int total = 0, listed = 0;
    if ((e = cudaMemcpyAsync(&total, bb.off.as<int>() + in.nq, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(&listed, bb.ncyl.p, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    if ((e = bb.bead.ensure(sizeof(int) * (size_t)(total > 0 ? total : 1))) != cudaSuccess) return e;
    if ((e = bb.plane.ensure(sizeof(int) * (size_t)(total > 0 ? total : 1))) != cudaSuccess) return e;
    if (in.nq > 0 && total > 0)
        k_bnd_write<<<nblk, tb, 0, s>>>(in, bb.cnt.as<int>(), bb.off.as<int>(), bb.bead.as<int>(), bb.plane.as<int>());
    *nbeads = total;
    *ncyl = listed;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// CSR of sparse contribution slots per bead
// ---------------------------------------------------------------------------
__device__ __forceinline__ int slot_bead(const CsrInput& in, int s) {
    if (s < in.base[1]) { const int4 b = in.lk[(s - in.base[0]) >> 2]; const int q = (s - in.base[0]) & 3; return q == 0 ? b.x : q == 1 ? b.y : q == 2 ? b.z : b.w; }
    if (s < in.base[2]) { const int4 b = in.mt[(s - in.base[1]) >> 2]; const int q = (s - in.base[1]) & 3; return q == 0 ? b.x : q == 1 ? b.y : q == 2 ? b.z : b.w; }
    if (s < in.base[3]) { const int4 b = in.ev[(s - in.base[2]) >> 2]; const int q = (s - in.base[2]) & 3; return q == 0 ? b.x : q == 1 ? b.y : q == 2 ? b.z : b.w; }
    return in.bb[s - in.base[3]];
}

__global__ void k_csr_count(CsrInput in, int* cnt) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= in.base[4]) return;
    atomicAdd(cnt + slot_bead(in, s), 1);
}
__global__ void k_csr_fill(CsrInput in, const int* off, int* cursor, int* slots) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= in.base[4]) return;
    const int b = slot_bead(in, s);
    slots[off[b] + atomicAdd(cursor + b, 1)] = s;
}
__global__ void k_csr_sort(int nb, const int* off, int* slots) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int o = off[b], k = off[b + 1] - o;
    for (int i = 1; i < k; ++i) {
        const int v = slots[o + i];
        int j = i - 1;
        while (j >= 0 && slots[o + j] > v) {
            slots[o + j + 1] = slots[o + j];
            --j;
        }
        slots[o + j + 1] = v;
    }
}

// Position of every slot in the bead-ordered CSR sequence: the sparse force
// kernels write each contribution there, so a bead's contributions are
// contiguous, in the CSR order, for the filament force kernels to read.
__global__ void k_csr_inverse(int ns, const int* slots, int* pos) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ns) return;
    pos[slots[c]] = c;
}

cudaError_t build_csr(const CsrInput& in, CsrBuild& cb, cudaStream_t s) {
    cudaError_t e;
    const int ns = in.base[4];
    if ((e = cb.cnt.ensure(sizeof(int) * (size_t)(in.nb + 1))) != cudaSuccess) return e;
    if ((e = cb.cursor.ensure(sizeof(int) * (size_t)(in.nb + 1))) != cudaSuccess) return e;
    // offsets padded for bulk copies that round their ranges up to 16 bytes
    if ((e = cb.off.ensure(sizeof(int) * (size_t)(in.nb + 1) + 64)) != cudaSuccess) return e;
    if ((e = cb.slots.ensure(sizeof(int) * (size_t)(ns > 0 ? ns : 1))) != cudaSuccess) return e;
    if ((e = cb.pos.ensure(sizeof(int) * (size_t)(ns > 0 ? ns : 1))) != cudaSuccess) return e;
    cudaMemsetAsync(cb.cnt.p, 0, sizeof(int) * (size_t)(in.nb + 1), s);
    cudaMemsetAsync(cb.cursor.p, 0, sizeof(int) * (size_t)(in.nb + 1), s);
    const int tb = 256;
    if (ns > 0) k_csr_count<<<(ns + tb - 1) / tb, tb, 0, s>>>(in, cb.cnt.as<int>());
    if ((e = exclusive_scan_i32(cb.cnt.as<int>(), cb.off.as<int>(), in.nb, cb.scan_tmp, s)) != cudaSuccess) return e;
    if (ns > 0) {
        k_csr_fill<<<(ns + tb - 1) / tb, tb, 0, s>>>(in, cb.off.as<int>(), cb.cursor.as<int>(), cb.slots.as<int>());
        k_csr_sort<<<(in.nb + tb - 1) / tb, tb, 0, s>>>(in.nb, cb.off.as<int>(), cb.slots.as<int>());
        k_csr_inverse<<<(ns + tb - 1) / tb, tb, 0, s>>>(ns, cb.slots.as<int>(), cb.pos.as<int>());
    }
    return cudaGetLastError();
}

}  // namespace mech
