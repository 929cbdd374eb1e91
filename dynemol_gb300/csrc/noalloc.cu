// Allocation-free variant of the one-particle Taylor propagation.
//
// Some callers cannot call cudaMalloc: a host that hands all device memory to
// its own pool allocator at start-up, code that runs while another component
// is capturing the device's work into a CUDA graph (cudaMalloc is not allowed
// there), and integrations that must not add the implicit device-wide
// synchronisation cudaMalloc / cudaFree can cause.  For them this entry point
// runs the same persistent Taylor kernel as propagation_gpucaller_ with all of
// its scratch -- the expansion-vector slots, the per-CTA partial sums, the
// grid-barrier counters, the error flag and the per-particle results -- in one
// file-scope device array of fixed size, so the call allocates nothing.  The
// caller passes device pointers for H' and Psi and a stream.
//
// The array belongs to this file's device module (about 0.9 MB).  With CUDA's
// lazy module loading (the default since CUDA 12.2) the driver places it in
// device memory when the module is first loaded on a device: by gpu_init_ /
// the library's context set-up (which call fixed_scratch_prepare), or
// else by the first call of this entry point on that device.  From then on the
// device holds it until the process exits.  A caller whose pool allocator
// takes the device memory should therefore call gpu_init_ (or this entry point
// once) first, and before any stream capture.  All calls on a device share the
// array and it keeps the contents of the last call; the barrier counters and
// the error flag are cleared at the start of every call.  Calls whose work
// overlaps on the GPU (for example on two streams) race on the array.
#include <mutex>

#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kFixedMaxN = 4096;    // largest basis the fixed scratch holds
constexpr int kFixedMaxGrid = 256;  // largest grid (one CTA per SM)
constexpr int kMaxDevices = 64;

struct FixedScratch {
    double2 slots[kSlots * 2 * kFixedMaxN];  // one particle: 6 slots x (bra, ket)
    double partials[2 * 2 * kFixedMaxGrid * 16];
    TaylorParticle part[2];
    alignas(8) unsigned bar[2];  // the grid barrier's 64-bit count
    int err;
};

static __device__ __align__(256) FixedScratch g_fixed_scratch;

std::mutex g_fixed_mu;
FixedScratch *g_fixed_addr[kMaxDevices] = {};

// Device address of the scratch for the current device (the host-side symbol
// is only a stand-in, never a device address).  Looked up once per device.
int fixed_scratch(FixedScratch **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ELHL_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(g_fixed_mu);
    if (!g_fixed_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_fixed_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "elhlprop: cudaGetSymbolAddress(fixed scratch) failed: %s\n", cudaGetErrorString(e));
            return ELHL_ERR_CUDA;
        }
        g_fixed_addr[dev] = (FixedScratch *)p;
    }
    *out = g_fixed_addr[dev];
    return ELHL_OK;
}

#define FX_TRY(expr)                                                                       \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            fprintf(stderr, "elhlprop: %s failed: %s\n", #expr, cudaGetErrorString(e_));  \
            return ELHL_ERR_CUDA;                                                          \
        }                                                                                  \
    } while (0)

}  // namespace
}  // namespace elhl

using namespace elhl;

extern "C" int elhl_propagate_fixed_scratch(int n, const double *d_H, int ld, elhl_zcomplex *d_psi_bra,
                                            elhl_zcomplex *d_psi_ket, double t_init, double t_max, double tau,
                                            double *save_tau, void *stream) {
    if (n < 1 || n > kFixedMaxN || ld < n || !d_H || !d_psi_bra || !d_psi_ket) {
        if (n > kFixedMaxN)
            fprintf(stderr, "elhlprop: elhl_propagate_fixed_scratch: n = %d exceeds the fixed scratch limit %d\n", n,
                    kFixedMaxN);
        return ELHL_ERR_BAD_ARG;
    }
    int grid = 0;
    if (taylor_grid_size(kTaylorBlock, &grid)) return ELHL_ERR_CUDA;
    if (grid > kFixedMaxGrid) grid = kFixedMaxGrid;
    FixedScratch *fs = nullptr;
    if (int rc = fixed_scratch(&fs)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t vb = (size_t)n * sizeof(double2);
    double2 *bra0 = fs->slots, *ket0 = fs->slots + kFixedMaxN;  // slot 0 of the particle
    TaylorParticle hp{};
    hp.tau_in = tau;
    FX_TRY(cudaMemsetAsync(fs->bar, 0, sizeof(fs->bar), st));
    FX_TRY(cudaMemsetAsync(&fs->err, 0, sizeof(int), st));
    FX_TRY(cudaMemcpyAsync(fs->part, &hp, sizeof(TaylorParticle), cudaMemcpyHostToDevice, st));
    FX_TRY(cudaMemcpyAsync(bra0, d_psi_bra, vb, cudaMemcpyDeviceToDevice, st));
    FX_TRY(cudaMemcpyAsync(ket0, d_psi_ket, vb, cudaMemcpyDeviceToDevice, st));
    TaylorLaunch L{};
    L.H = d_H;
    L.N = n;
    L.ld = ld;
    L.nparticles = 1;
    L.slots = fs->slots;
    L.ldv = kFixedMaxN;
    L.part = fs->part;
    L.t_init = t_init;
    L.t_max = t_max;
    L.tol = 1.0e-8;       // Taylor_gpu.cpp:118-119
    L.norm_tol = 1.0e-8;
    L.max_conv_calls = 10000;
    L.nsteps = 1;
    L.it0 = 2;
    L.dt_frame = t_max - t_init;
    L.tau_max = tau;
    L.pops = nullptr;
    L.ao_frag = nullptr;
    L.nfrag = 0;
    L.t_final = nullptr;
    L.partials = fs->partials;
    L.bar_count = fs->bar;
    L.error = &fs->err;
    FX_TRY(launch_taylor(L, grid, kTaylorBlock, st));
    // Status first: the caller's Psi is overwritten only by a converged step,
    // so a call that fails (timeout, no convergence) can be retried.
    TaylorParticle res{};
    int err = 0;
    FX_TRY(cudaMemcpyAsync(&res, fs->part, sizeof(TaylorParticle), cudaMemcpyDeviceToHost, st));
    FX_TRY(cudaMemcpyAsync(&err, &fs->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FX_TRY(cudaStreamSynchronize(st));
    if (err) return err;
    if (res.status) return res.status;
    FX_TRY(cudaMemcpyAsync(d_psi_bra, bra0, vb, cudaMemcpyDeviceToDevice, st));
    FX_TRY(cudaMemcpyAsync(d_psi_ket, ket0, vb, cudaMemcpyDeviceToDevice, st));
    FX_TRY(cudaStreamSynchronize(st));
    if (save_tau) *save_tau = res.save_tau;
    return ELHL_OK;
}

// Loads this module on the current device and resolves the array's address,
// so that the array is resident before a caller's pool allocator or stream
// capture starts.  Called from the library's context set-up (gpu_init_).
namespace elhl {
int fixed_scratch_prepare() {
    FixedScratch *fs = nullptr;
    return fixed_scratch(&fs);
}
}  // namespace elhl
