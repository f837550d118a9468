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
// Direct sum: FP32 with positions split into float hi + lo parts (separations
// formed as (hi - hi) + (lo - lo)), partial sums per source slice, reduced in
// FP64 in slice order (deterministic).
#include "hc_internal.cuh"

namespace {

constexpr int GT = 256;


// One thread per sampled body, a block per slice of the sources.  The slice
// is staged in shared memory in pairs (both bodies' values of one quantity
// adjacent: the operands of one packed FP32x2 instruction) and summed two
// sources per step.  With softening the sample's own term is exactly zero (a
// zero separation); without it (SELF) the sample skips itself explicitly.
template <bool SELF>
__global__ void __launch_bounds__(GT) k_guard_direct(int64_t n, const double *mass, const double *px,
                                                     const double *py, const double *pz, const int64_t *idx, int ns,
                                                     float eps2, int64_t slice, float4 *part)
{
    __shared__ float4 sp[GT / 2][4];      // (hx hy) (hz m) (lx ly) (lz -), each for two sources
    const int s = blockIdx.y * GT + threadIdx.x;
    const bool valid = s < ns;
    const int64_t me = valid ? idx[s] : -1;
    const double xd = valid ? px[me] : 0.0, yd = valid ? py[me] : 0.0, zd = valid ? pz[me] : 0.0;
    const float xh = __double2float_rn(xd), yh = __double2float_rn(yd), zh = __double2float_rn(zd);
    const float xl = __double2float_rn(xd - (double)xh), yl = __double2float_rn(yd - (double)yh),
                zl = __double2float_rn(zd - (double)zh);
    const int64_t j0 = (int64_t)blockIdx.x * slice;
    const int64_t j1 = j0 + slice < n ? j0 + slice : n;
    const float2 nxh = splat2(-xh), nyh = splat2(-yh), nzh = splat2(-zh);
    const float2 nxl = splat2(-xl), nyl = splat2(-yl), nzl = splat2(-zl), e2 = splat2(eps2);
    float2 ax = splat2(0.f), ay = ax, az = ax;
    float *f = reinterpret_cast<float *>(sp[threadIdx.x >> 1]) + (threadIdx.x & 1);
    for (int64_t base = j0; base < j1; base += GT) {
        const int64_t j = base + threadIdx.x;
        if (j < j1) {
            const double x = px[j], y = py[j], z = pz[j];
            const float h0 = __double2float_rn(x), h1 = __double2float_rn(y), h2 = __double2float_rn(z);
            f[0] = h0;
            f[2] = h1;
            f[4] = h2;
            f[6] = __double2float_rn(mass[j]);
            f[8] = __double2float_rn(x - (double)h0);
            f[10] = __double2float_rn(y - (double)h1);
            f[12] = __double2float_rn(z - (double)h2);
        } else {                                 // pad: massless, far away
            f[0] = f[2] = f[4] = 1.0e4f;
            f[6] = f[8] = f[10] = f[12] = 0.f;
        }
        __syncthreads();
        const int cnt = j1 - base < GT ? (int)(j1 - base) : GT;
        const int self = SELF ? (int)(me - base) : -1;   // the sample's slot in this tile, if any
        for (int p = 0; p < (cnt + 1) >> 1; p++) {
            const float4 H0 = sp[p][0], H1 = sp[p][1], L0 = sp[p][2], L1 = sp[p][3];
            const float2 dx = __fadd2_rn(__fadd2_rn(lo2(H0), nxh), __fadd2_rn(lo2(L0), nxl));
            const float2 dy = __fadd2_rn(__fadd2_rn(hi2(H0), nyh), __fadd2_rn(hi2(L0), nyl));
            const float2 dz = __fadd2_rn(__fadd2_rn(lo2(H1), nzh), __fadd2_rn(lo2(L1), nzl));
            const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
            float2 w = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
            if (SELF) w = make_float2(2 * p == self ? 0.f : w.x, 2 * p + 1 == self ? 0.f : w.y);
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

// No CUDA queries here: this runs inside stream capture.
static int guard_slices_used(const hc_ctx *c, int64_t *slice)
{
    const int64_t want = c->guard_narrow ? (c->guard_slices + 15) / 16 : c->guard_slices;
    *slice = (c->n + want - 1) / want;
    if (*slice < 1) *slice = 1;
    return (int)((c->n + *slice - 1) / *slice);
}

// The direct sum needs only positions and masses: it can run while the tree
// is built.  Beside the build it runs on a sixteenth of the slices (one block
// per two SMs), leaving the latency-bound build kernels room.
void hc_guard_direct_launch(hc_ctx *c, cudaStream_t s)
{
    const int ns = (int)c->guard_n;
    int64_t slice;
    const int slices = guard_slices_used(c, &slice);
    const dim3 grid((unsigned)slices, (unsigned)((ns + GT - 1) / GT));
    const float eps2 = (float)(c->prm.eps * c->prm.eps);
    if (eps2 > 0.f)
        k_guard_direct<false><<<grid, GT, 0, s>>>(c->n, c->mass, c->px, c->py, c->pz, c->guard_idx, ns, eps2, slice,
                                                   c->guard_part);
    else
        k_guard_direct<true><<<grid, GT, 0, s>>>(c->n, c->mass, c->px, c->py, c->pz, c->guard_idx, ns, eps2, slice,
                                                  c->guard_part);
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
