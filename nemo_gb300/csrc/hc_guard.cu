// hc_guard.cu -- per-evaluation guard of the approximate opening criteria.
//
// The group, error-bound and learned criteria trade exactness of the
// reference's per-body rule (grav.c:122-131) for fewer interactions.  The
// guard keeps their error bounded: after each of their walks the
// accelerations of a fixed sample of bodies are compared with a direct sum
// over all bodies; when the RMS relative error over the sample exceeds the
// budget, a flag is raised on the device and the walk that follows in the
// same launch sequence (the per-body rule at the context's tol) recomputes
// every force.  That walk's closing half-kick, v += (a_new - a_stored) dt/2,
// starts from the accelerations the approximate walk stored, so the velocity
// ends as if only the fallback walk had run.  No host round trip: the whole
// sequence is captured in the evaluation's CUDA graph.
//
// Direct sum: FP32, partial sums per source slice, reduced in FP64 in slice
// order (deterministic).  With softening the positions are rounded to FP32:
// on a Plummer sphere of 2^20 bodies that changes the sampled forces by 3e-8
// (eps 0.01), 3e-7 (eps 1e-3) and 2e-6 (eps 1e-4) RMS relative, far below any
// error budget, and a separation is one subtraction.  Without softening close
// pairs are not bounded by eps: positions are split into float hi + lo parts
// and separations formed as (hi - hi) + (lo - lo).
#include "hc_internal.cuh"

namespace {

constexpr int GT = 256;


// One thread per sampled body, a block per slice of the sources.  The slice
// is staged in shared memory in pairs (both bodies' values of one quantity
// adjacent: the operands of one packed FP32x2 instruction) and summed two
// sources per step.  Softened (eps2 > 0): FP32 positions, 12 packed
// operations and two rsqrt per pair of sources; the sample's own term is
// exactly zero (a zero separation).
__global__ void __launch_bounds__(GT) k_guard_direct_soft(int64_t n, const double *mass, const double *px,
                                                          const double *py, const double *pz, const int64_t *idx,
                                                          int ns, float eps2, int64_t slice, float4 *part)
{
    __shared__ float4 sp[GT / 2][2];      // (x x' y y') (z z' m m') for two sources
    const int s = blockIdx.y * GT + threadIdx.x;
    const bool valid = s < ns;
    const int64_t me = valid ? idx[s] : -1;
    const float2 nx = splat2(valid ? -hc_d2f_rn(px[me]) : 0.f), ny = splat2(valid ? -hc_d2f_rn(py[me]) : 0.f),
                 nz = splat2(valid ? -hc_d2f_rn(pz[me]) : 0.f), e2 = splat2(eps2);
    const int64_t j0 = (int64_t)blockIdx.x * slice;
    const int64_t j1 = j0 + slice < n ? j0 + slice : n;
    float2 ax = splat2(0.f), ay = ax, az = ax;
    float *f = reinterpret_cast<float *>(sp[threadIdx.x >> 1]) + (threadIdx.x & 1);
    for (int64_t base = j0; base < j1; base += GT) {
        const int64_t j = base + threadIdx.x;
        if (j < j1) {
            f[0] = hc_d2f_rn(px[j]);
            f[2] = hc_d2f_rn(py[j]);
            f[4] = hc_d2f_rn(pz[j]);
            f[6] = hc_d2f_rn(mass[j]);
        } else {                                 // pad: massless, far away
            f[0] = f[2] = f[4] = 1.0e4f;
            f[6] = 0.f;
        }
        __syncthreads();
        const int cnt = j1 - base < GT ? (int)(j1 - base) : GT;
        for (int p = 0; p < (cnt + 1) >> 1; p++) {
            const float4 P = sp[p][0], Q = sp[p][1];
            const float2 dx = __fadd2_rn(lo2(P), nx), dy = __fadd2_rn(hi2(P), ny), dz = __fadd2_rn(lo2(Q), nz);
            const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
            const float2 w = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
            const float2 mr3 = __fmul2_rn(hi2(Q), __fmul2_rn(w, __fmul2_rn(w, w)));
            ax = __ffma2_rn(mr3, dx, ax);
            ay = __ffma2_rn(mr3, dy, ay);
            az = __ffma2_rn(mr3, dz, az);
        }
        __syncthreads();
    }
    if (valid) part[(int64_t)blockIdx.x * ns + s] = make_float4(ax.x + ax.y, ay.x + ay.y, az.x + az.y, 0.f);
}

// Without softening: positions as hi + lo floats, the sample skips itself
// explicitly.
__global__ void __launch_bounds__(GT) k_guard_direct_exact(int64_t n, const double *mass, const double *px,
                                                     const double *py, const double *pz, const int64_t *idx, int ns,
                                                     float eps2, int64_t slice, float4 *part)
{
    __shared__ float4 sp[GT / 2][4];      // (hx hy) (hz m) (lx ly) (lz -), each for two sources
    const int s = blockIdx.y * GT + threadIdx.x;
    const bool valid = s < ns;
    const int64_t me = valid ? idx[s] : -1;
    const double xd = valid ? px[me] : 0.0, yd = valid ? py[me] : 0.0, zd = valid ? pz[me] : 0.0;
    float xh, yh, zh, xl, yl, zl;
    hc_split_hilo(xd, &xh, &xl);
    hc_split_hilo(yd, &yh, &yl);
    hc_split_hilo(zd, &zh, &zl);
    const int64_t j0 = (int64_t)blockIdx.x * slice;
    const int64_t j1 = j0 + slice < n ? j0 + slice : n;
    const float2 nxh = splat2(-xh), nyh = splat2(-yh), nzh = splat2(-zh);
    const float2 nxl = splat2(-xl), nyl = splat2(-yl), nzl = splat2(-zl), e2 = splat2(eps2);
    float2 ax = splat2(0.f), ay = ax, az = ax;
    float *f = reinterpret_cast<float *>(sp[threadIdx.x >> 1]) + (threadIdx.x & 1);
    for (int64_t base = j0; base < j1; base += GT) {
        const int64_t j = base + threadIdx.x;
        if (j < j1) {
            // hi + lo parts on the doubles' bits (no FP64-pipe conversions)
            hc_split_hilo(px[j], &f[0], &f[8]);
            hc_split_hilo(py[j], &f[2], &f[10]);
            hc_split_hilo(pz[j], &f[4], &f[12]);
            f[6] = hc_d2f_rn(mass[j]);
        } else {                                 // pad: massless, far away
            f[0] = f[2] = f[4] = 1.0e4f;
            f[6] = f[8] = f[10] = f[12] = 0.f;
        }
        __syncthreads();
        const int cnt = j1 - base < GT ? (int)(j1 - base) : GT;
        const int self = (int)(me - base);               // the sample's slot in this tile, if any
        for (int p = 0; p < (cnt + 1) >> 1; p++) {
            const float4 H0 = sp[p][0], H1 = sp[p][1], L0 = sp[p][2], L1 = sp[p][3];
            const float2 dx = __fadd2_rn(__fadd2_rn(lo2(H0), nxh), __fadd2_rn(lo2(L0), nxl));
            const float2 dy = __fadd2_rn(__fadd2_rn(hi2(H0), nyh), __fadd2_rn(hi2(L0), nyl));
            const float2 dz = __fadd2_rn(__fadd2_rn(lo2(H1), nzh), __fadd2_rn(lo2(L1), nzl));
            const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
            float2 w = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
            w = make_float2(2 * p == self ? 0.f : w.x, 2 * p + 1 == self ? 0.f : w.y);
            const float2 mr3 = __fmul2_rn(hi2(H1), __fmul2_rn(w, __fmul2_rn(w, w)));
            ax = __ffma2_rn(mr3, dx, ax);
            ay = __ffma2_rn(mr3, dy, ay);
            az = __ffma2_rn(mr3, dz, az);
        }
        __syncthreads();
    }
    if (valid) part[(int64_t)blockIdx.x * ns + s] = make_float4(ax.x + ax.y, ay.x + ay.y, az.x + az.y, 0.f);
}

// Per sampled body: its direct-sum acceleration (partials summed in slice
// order, FP64) and its squared relative error.
__global__ void __launch_bounds__(128) k_guard_rel(const float4 *part, int slices, int ns, const int64_t *idx,
                                                   const double *ax, const double *ay, const double *az,
                                                   double *rel2)
{
    __shared__ double r[3][128];
    const int s = blockIdx.x;
    double dx = 0.0, dy = 0.0, dz = 0.0;
    for (int b = threadIdx.x; b < slices; b += 128) {
        const float4 p = part[(int64_t)b * ns + s];
        dx += (double)p.x;
        dy += (double)p.y;
        dz += (double)p.z;
    }
    r[0][threadIdx.x] = dx;
    r[1][threadIdx.x] = dy;
    r[2][threadIdx.x] = dz;
    __syncthreads();
    for (int o = 64; o; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 3; q++) r[q][threadIdx.x] += r[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int64_t i = idx[s];
        const double ex = ax[i] - r[0][0], ey = ay[i] - r[1][0], ez = az[i] - r[2][0];
        const double a2 = r[0][0] * r[0][0] + r[1][0] * r[1][0] + r[2][0] * r[2][0];
        rel2[s] = a2 > 0.0 ? (ex * ex + ey * ey + ez * ez) / a2 : 0.0;
    }
}

__global__ void __launch_bounds__(GT) k_guard_check(const double *rel2, int ns, double rms_max, hc_guard_state *gs,
                                                    hc_status *st)
{
    __shared__ double red[GT];
    double acc = 0.0;
    for (int s = threadIdx.x; s < ns; s += GT) acc += rel2[s];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = GT / 2; o; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double rms = sqrt(red[0] / (double)ns);
        const bool trip = !(rms <= rms_max);   // NaN trips
        gs->last_rms = rms;
        gs->checks++;
        gs->flag = trip ? 1 : 0;
        if (trip) {
            gs->trips++;
            st->n2b = 0;                        // the fallback walk's counts replace these
            st->nbc = 0;
        }
    }
}

}  // namespace

int hc_guard_slices(hc_ctx *c)
{
    int dev = 0, nsm = 0;
    HC_CUDA(cudaGetDevice(&dev));
    HC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    return 8 * nsm;
}

// Beside the build the direct sum would take every SM's thread slots and
// registers for its whole run, and the build's kernels would wait for them.
// Each guard block therefore reserves shared memory it does not use, so that
// at most four share an SM; the rest of each SM stays free for the build,
// whose stream has the higher priority.  Four per SM measured best at
// N = 2^20 (the build beside the guard: 0.86 ms, against 0.885 ms with eight
// per SM, 0.87 with three or five, 0.885 with two, 0.78 ms with no guard).
int hc_guard_setup(hc_ctx *c)
{
    int dev = 0, smem_sm = 0;
    HC_CUDA(cudaGetDevice(&dev));
    HC_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    cudaFuncAttributes fa;
    HC_CUDA(cudaFuncGetAttributes(&fa, k_guard_direct_exact));   // the larger static footprint of the two
    const int per_block = smem_sm / 4 - (int)fa.sharedSizeBytes - 1024;   // 1 KB per block is the system's
    c->guard_smem = per_block > 0 ? per_block : 0;
    HC_CUDA(cudaFuncSetAttribute(k_guard_direct_soft, cudaFuncAttributeMaxDynamicSharedMemorySize, c->guard_smem));
    HC_CUDA(cudaFuncSetAttribute(k_guard_direct_exact, cudaFuncAttributeMaxDynamicSharedMemorySize, c->guard_smem));
    return HC_OK;
}

// No CUDA queries here: this runs inside stream capture.
static int guard_slices_used(const hc_ctx *c, int64_t *slice)
{
    const int64_t want = c->guard_slices;
    *slice = (c->n + want - 1) / want;
    if (*slice < 1) *slice = 1;
    return (int)((c->n + *slice - 1) / *slice);
}

// The direct sum needs only positions and masses: it runs on a side stream
// while the tree is built, in the gaps the latency-bound build kernels leave.
void hc_guard_direct_launch(hc_ctx *c, cudaStream_t s)
{
    const int ns = (int)c->guard_n;
    int64_t slice;
    const int slices = guard_slices_used(c, &slice);
    const dim3 grid((unsigned)slices, (unsigned)((ns + GT - 1) / GT));
    const float eps2 = (float)(c->prm.eps * c->prm.eps);
    if (eps2 > 0.f)
        k_guard_direct_soft<<<grid, GT, c->guard_smem, s>>>(c->n, c->mass, c->px, c->py, c->pz, c->guard_idx, ns,
                                                         eps2, slice, c->guard_part);
    else
        k_guard_direct_exact<<<grid, GT, c->guard_smem, s>>>(c->n, c->mass, c->px, c->py, c->pz, c->guard_idx, ns,
                                                          eps2, slice, c->guard_part);
    c->launches++;
}

void hc_guard_check_launch(hc_ctx *c)
{
    const int ns = (int)c->guard_n;
    int64_t slice;
    const int slices = guard_slices_used(c, &slice);
    double *rel2 = reinterpret_cast<double *>(c->guard_part + (int64_t)c->guard_slices * ns);
    k_guard_rel<<<ns, 128, 0, c->stream>>>(c->guard_part, slices, ns, c->guard_idx, c->ax, c->ay, c->az, rel2);
    k_guard_check<<<1, GT, 0, c->stream>>>(rel2, ns, c->guard_rms_max, c->guard, c->st);
    c->launches += 2;
}

void hc_guard_launch(hc_ctx *c)
{
    hc_guard_direct_launch(c, c->stream);
    hc_guard_check_launch(c);
}
