// hc_noalloc.cu -- diagnostics sums with no device allocation.
//
// Some callers of this library cannot allocate device memory at the moment
// they need the energy / virial / angular-momentum sums: a runtime that hands
// the library only pre-registered buffers from its own memory pool (and
// accounts for every byte of device memory itself), or a real-time loop that
// must not pay cudaMalloc's implicit device synchronisation between its
// steps.  hc_diagnostics_noalloc serves them: the caller passes device
// pointers to the body arrays and to a 36-double result, and the per-block
// partial sums live in the file-scope array below instead of in memory the
// library would allocate.  The potential energy is 0.5 sum m phi with phi as
// passed: a caller with an external field passes phi + phi_ext, as
// hc_diagnostics counts it.
//
// Limits and sharing:
//   * the array holds HC_NOALLOC_MAX_BLOCKS partials of 36 doubles (576 KiB);
//     each block sums HC_NOALLOC_BODIES_PER_BLOCK bodies, so at most
//     HC_NOALLOC_MAX_BODIES = 2048 * 4096 = 8,388,608 bodies per call; larger
//     n is rejected with HC_ERR_ARG;
//   * every GPU that loads the library holds the array until the process
//     exits; all calls on a device share it, so calls whose kernels overlap on
//     the GPU (different streams, no ordering between them) race and must be
//     serialised by the caller;
//   * the array keeps the last call's contents, and nothing has to start at
//     zero: each call reads only the partial slots its own first kernel wrote.
#include <atomic>
#include "hc_internal.cuh"

#define HC_NOALLOC_MAX_BLOCKS 2048
#define HC_NOALLOC_BODIES_PER_BLOCK 4096
#define HC_NOALLOC_MAX_BODIES ((int64_t)HC_NOALLOC_MAX_BLOCKS * HC_NOALLOC_BODIES_PER_BLOCK)

namespace {

constexpr int NSUM = 36;   // KE, PE, keten[9], peten[9], m x_i v_j [9], sum m x[3], sum m v[3], mtot
constexpr int THREADS = 256;

static __device__ __align__(256) double g_partials[HC_NOALLOC_MAX_BLOCKS * NSUM];

// Host side: the device address of g_partials, looked up once per device.
// (In host code the name g_partials is only a stand-in, not a device address.)
// Threads whose first calls on a device race all store the same address, so
// the slots are atomics and no lock is needed.  A failed lookup or launch
// drops the slot, and the next call looks the address up again.  The address
// belongs to the device's primary context: after cudaDeviceReset of a device
// the cached slot is stale, so a process that resets a device must not call
// this entry point on that device afterwards.
constexpr int MAX_DEVICES = 64;
std::atomic<double *> g_partials_addr[MAX_DEVICES];

__device__ __forceinline__ double wsum(double v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One block per HC_NOALLOC_BODIES_PER_BLOCK bodies; block b writes slot b.
__global__ void __launch_bounds__(THREADS) k_diag_static_part(int64_t n, const double *mass, const double *px,
                                                              const double *py, const double *pz, const double *vx,
                                                              const double *vy, const double *vz, const double *ax,
                                                              const double *ay, const double *az, const double *phi,
                                                              double *part)
{
    double acc[NSUM];
#pragma unroll
    for (int q = 0; q < NSUM; q++) acc[q] = 0.0;
    const int64_t beg = (int64_t)blockIdx.x * HC_NOALLOC_BODIES_PER_BLOCK;
    const int64_t end = beg + HC_NOALLOC_BODIES_PER_BLOCK < n ? beg + HC_NOALLOC_BODIES_PER_BLOCK : n;
    for (int64_t i = beg + threadIdx.x; i < end; i += THREADS) {
        const double x[3] = {px[i], py[i], pz[i]}, v[3] = {vx[i], vy[i], vz[i]}, a[3] = {ax[i], ay[i], az[i]};
        hc_diag_body(acc, mass[i], x, v, a, phi[i]);     // PE from phi as passed
    }
    __shared__ double sh[THREADS / 32][NSUM];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NSUM; q++) {
        const double s = wsum(acc[q]);
        if (lane == 0) sh[wid][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < NSUM) {
        double s = 0.0;
        for (int w = 0; w < THREADS / 32; w++) s += sh[w][threadIdx.x];
        part[(int64_t)blockIdx.x * NSUM + threadIdx.x] = s;
    }
}

__global__ void k_diag_static_final(const double *part, int nparts, double *out)
{
    const int q = threadIdx.x;
    if (q < NSUM) {
        double s = 0.0;
        for (int b = 0; b < nparts; b++) s += part[(int64_t)b * NSUM + q];
        out[q] = s;
    }
}

}  // namespace

extern "C" int hc_diagnostics_noalloc(int64_t n, const double *mass, const double *x, const double *y,
                                      const double *z, const double *vx, const double *vy, const double *vz,
                                      const double *ax, const double *ay, const double *az, const double *phi,
                                      double *out36, void *stream)
{
    if (n < 1 || n > HC_NOALLOC_MAX_BODIES) return HC_ERR_ARG;   // beyond the static scratch
    if (!mass || !x || !y || !z || !vx || !vy || !vz || !ax || !ay || !az || !phi || !out36) return HC_ERR_ARG;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return HC_ERR_CUDA;
    double *part = g_partials_addr[dev].load(std::memory_order_acquire);
    if (!part) {
        // first call on this device: resolve the array's device address with
        // the device current (do this before any stream capture)
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_partials) != cudaSuccess || !p) return HC_ERR_CUDA;
        part = (double *)p;
        g_partials_addr[dev].store(part, std::memory_order_release);
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int nblocks = (int)((n + HC_NOALLOC_BODIES_PER_BLOCK - 1) / HC_NOALLOC_BODIES_PER_BLOCK);
    k_diag_static_part<<<nblocks, THREADS, 0, s>>>(n, mass, x, y, z, vx, vy, vz, ax, ay, az, phi, part);
    k_diag_static_final<<<1, 64, 0, s>>>(part, nblocks, out36);
    if (cudaPeekAtLastError() != cudaSuccess) {
        g_partials_addr[dev].store(nullptr, std::memory_order_release);
        return HC_ERR_CUDA;
    }
    return HC_OK;
}
