// Filament stretching + bending energies of one network that already sits in
// caller-owned device memory, computed without allocating anything.
//
// This is the FP64 filament-energy kernel (FilamentStretchingHarmonic.cpp:185-275
// and FilamentBendingCosine.cpp:199-345, paths relative to medyan-5.4.0/src)
// in a stateless form: the per-block partial sums and the completion ticket
// live in a fixed file-scope device array instead of context buffers, so the
// call makes no cudaMalloc/cudaFree (which can synchronize the whole device)
// and needs no context.
//
// Scratch layout (kScratchBytes):
//   [0, 256)                      completion ticket (one unsigned int); must be
//                                 zero when the kernel starts: the entry point
//                                 clears it on the caller's stream before each
//                                 launch and the last block leaves it at zero
//   [256, 256 + 16 * kMaxBlocks)  per-block (stretching, bending) partial sums
// Calls that overlap in time (different streams or host threads, same
// device) share this scratch and race; the caller orders them.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "mech_device.cuh"
#include "mech_internal.cuh"

namespace mech {

constexpr int kStaticBlock = 256;        // cylinders per block
constexpr int kStaticMaxBlocks = 8192;   // partial-sum slots: up to 2,097,152 cylinders
constexpr size_t kStaticScratchBytes = 256 + 16 * (size_t)kStaticMaxBlocks;   // 131,328 bytes
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Filament of cylinder c: the largest f with fcs[f] <= c (fcs ascending).
__device__ __forceinline__ int filament_of(const int32_t* __restrict__ fcs, int nfil, int c) {
    int lo = 0, hi = nfil - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(fcs + mid) <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One thread per cylinder: its stretching term and, unless it is the first
// cylinder of its filament, the bending term of the triple it closes
// (constants of the second cylinder).  Beads are filament-contiguous, so
// cylinder c of filament f joins beads c + f and c + f + 1.
__global__ void __launch_bounds__(kStaticBlock)
k_fil_energy_static(const double* __restrict__ x, const int32_t* __restrict__ fcs, int nfil, int ncyl,
                    const double* __restrict__ ks, const double* __restrict__ l0, const double* __restrict__ kb,
                    const double* __restrict__ t0, unsigned char* scratch, double* out) {
    __shared__ double sh[64];
    __shared__ int s_last;
    unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch);
    double2* part = reinterpret_cast<double2*>(scratch + 256);
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double es = 0.0, eb = 0.0;
    if (c < ncyl) {
        const int f = filament_of(fcs, nfil, c);
        const size_t b = (size_t)c + (size_t)f;
        const double* p0 = x + 3 * b;
        const double* p1 = p0 + 3;
        es = stretch_energy<double>(p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], ks[c], l0[c]);
        if (c > __ldg(fcs + f)) {
            const double* pm = p0 - 3;
            const double r1[3] = {p0[0] - pm[0], p0[1] - pm[1], p0[2] - pm[2]};
            const double r2[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
            eb = bend_energy<double>(r1, r2, kb[c], t0[c]);
        }
    }
    double w[2] = {warp_sum(es), warp_sum(eb)};
    const int ops[2] = {0, 0};
    block_combine<2>(w, ops, sh);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = make_double2(w[0], w[1]);
        __threadfence();
        s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    // last block: slots in a fixed order (thread t takes t, t + 256, ...), then the block tree
    __threadfence();
    double a = 0.0, bsum = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
        const double2 v = __ldcg(part + k);
        a += v.x;
        bsum += v.y;
    }
    double t[2] = {warp_sum(a), warp_sum(bsum)};
    block_combine<2>(t, ops, sh);
    if (threadIdx.x == 0) {
        out[0] = t[0];
        out[1] = t[1];
        *ticket = 0u;
    }
}

// The scratch address belongs to the module loaded into one CUDA context: a
// context that is destroyed and re-created (cudaDeviceReset, a primary
// context released by every user) reloads the module and the array can move.
// So the address is cached per (device, current context) and looked up again
// whenever the current context of that device changes.  The context handle
// comes from the driver's cuCtxGetCurrent, reached through the runtime's
// entry-point query so that the library needs no link against libcuda.
using CtxGetCurrentFn = int (*)(void**);   // CUresult cuCtxGetCurrent(CUcontext*)

static std::mutex g_static_mu;
static void* g_static_ptr[kStaticMaxDevices];
static void* g_static_ctx[kStaticMaxDevices];
static CtxGetCurrentFn g_ctx_get_current = nullptr;
static bool g_ctx_query_done = false;

static void* current_context() {
    if (!g_ctx_query_done) {
        g_ctx_query_done = true;
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
        else
            cudaGetLastError();
    }
    void* ctx = nullptr;
    if (!g_ctx_get_current || g_ctx_get_current(&ctx) != 0) return nullptr;
    return ctx;
}

// Device address of the scratch array in the current context of device
// `dev` (which must be current), looked up at the first call in that context.
static int static_scratch(int dev, unsigned char** out) {
    if (dev < 0 || dev >= kStaticMaxDevices) return set_error_text(MECH_ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_static_mu);
    void* ctx = current_context();
    if (!g_static_ptr[dev] || !ctx || ctx != g_static_ctx[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return set_error_text(MECH_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_static_ptr[dev] = p;
        g_static_ctx[dev] = current_context();   // the lookup itself makes the primary context current
    }
    *out = static_cast<unsigned char*>(g_static_ptr[dev]);
    return MECH_OK;
}

}  // namespace mech

extern "C" int32_t mech_filament_energy_device(int32_t n_filaments, int32_t n_cylinders, const int32_t* fil_cyl_start,
                                               const double* coord, const double* k_stretch, const double* eq_length,
                                               const double* k_bend, const double* eq_theta, double* energies,
                                               void* stream) {
    using namespace mech;
    if (n_filaments < 1 || n_cylinders < 0 || !fil_cyl_start || !coord || !k_stretch || !eq_length || !k_bend ||
        !eq_theta || !energies)
        return set_error_text(MECH_ERR_ARG, "mech_filament_energy_device: null pointer or bad count");
    const long long blocks = ((long long)n_cylinders + kStaticBlock - 1) / kStaticBlock;
    if (blocks > kStaticMaxBlocks)
        return set_error_text(MECH_ERR_CAPACITY,
                              "mech_filament_energy_device: n_cylinders " + std::to_string(n_cylinders) +
                                  " exceeds the fixed scratch limit of " +
                                  std::to_string((long long)kStaticMaxBlocks * kStaticBlock) + " cylinders");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error_text(MECH_ERR_NO_DEVICE, "no CUDA device visible");
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error_text(MECH_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    unsigned char* scratch = nullptr;
    int rc = static_scratch(dev, &scratch);
    if (rc != MECH_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n_cylinders == 0) {
        e = cudaMemsetAsync(energies, 0, 2 * sizeof(double), s);
        if (e != cudaSuccess) return set_error_text(MECH_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
        return MECH_OK;
    }
    e = cudaMemsetAsync(scratch, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return set_error_text(MECH_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    k_fil_energy_static<<<(unsigned)blocks, kStaticBlock, 0, s>>>(coord, fil_cyl_start, n_filaments, n_cylinders,
                                                                  k_stretch, eq_length, k_bend, eq_theta, scratch,
                                                                  energies);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error_text(MECH_ERR_CUDA, std::string("k_fil_energy_static: ") + cudaGetErrorString(e));
    return MECH_OK;
}
