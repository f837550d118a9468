#include <algorithm>
// hc_step.cu -- FP64 leapfrog update, diagnostics reductions and the FP64
// direct-sum sample on the GPU.
//
// References: stepsystem (src/nbody/evolve/hackcode/hackcode1/code.c:159-191),
// diagnostics (code_io.c:160-197).  All arithmetic is FP64 with explicit
// round-to-nearest intrinsics so that no multiply-add is fused and the
// kick/drift sequence matches the reference operation for operation.
#include "hc_internal.cuh"

namespace {

constexpr int DIAG_BLOCKS = 304;
constexpr int DIAG_THREADS = 256;
constexpr int NDIAG = 36;   // KE, PE, keten[9], peten[9], amten_raw[9], m x[3], m v[3], mtot

// v1/2 = v + a dt/2; x += v1/2 dt; v = v1/2 + a dt/2   (code.c:182-188)
__global__ void k_kick_drift(int64_t n, double dt, double *px, double *py, double *pz, double *vx, double *vy,
                             double *vz, const double *ax, const double *ay, const double *az)
{
    const double dthf = 0.5 * dt;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double *p[3] = {px, py, pz}, *v[3] = {vx, vy, vz};
        const double *a[3] = {ax, ay, az};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            double dvel = __dmul_rn(a[k][i], dthf);
            double vel1 = __dadd_rn(v[k][i], dvel);
            double dpos = __dmul_rn(vel1, dt);
            p[k][i] = __dadd_rn(p[k][i], dpos);
            v[k][i] = __dadd_rn(vel1, dvel);
        }
    }
}

// External potentials of NEMO's potential plug-ins (pattern speed 0),
// restated: plummer (M, a) -M/sqrt(r^2 + a^2); hernquist (M, a) -M/(r + a);
// miyamoto (M, a, b) -M/sqrt(R^2 + (a + sqrt(y^2 + b^2))^2), R^2 = x^2 + z^2; log (m_c, r_c,
// q, r) (m_c/r_c) ln(r_c^2 + x^2 + y^2/q^2 + z^2/r^2).
__device__ __forceinline__ void ext_field(int kind, const double *p, double x, double y, double z, double *ax,
                                          double *ay, double *az, double *pot)
{
    if (kind == HC_EXTPOT_PLUMMER) {
        const double t = 1.0 / (p[1] * p[1] + x * x + y * y + z * z), s = -sqrt(t);
        *pot = p[0] * s;
        const double f = t * s * p[0];
        *ax = f * x;
        *ay = f * y;
        *az = f * z;
    } else if (kind == HC_EXTPOT_HERNQUIST) {
        const double r = sqrt(x * x + y * y + z * z), f = 1.0 / (r + p[1]);
        *pot = -p[0] * f;
        const double g = r > 0.0 ? -p[0] * f * f / r : 0.0;
        *ax = g * x;
        *ay = g * y;
        *az = g * z;
    } else if (kind == HC_EXTPOT_MIYAMOTO) {
        // NEMO builds miyamoto.c without -DY/-DZ, which selects its re-oriented
        // "XZY" setup (miyamoto.c:45-56): the disk's symmetry axis is y
        const double R = sqrt(x * x + z * z);
        const double q = sqrt(y * y + p[2] * p[2]), s = sqrt(R * R + (p[1] + q) * (p[1] + q));
        *pot = -p[0] / s;
        const double t = *pot / (s * s);
        *ax = t * x;
        *ay = t * y * (p[1] > 0.0 ? (p[1] + q) / q : 1.0);
        *az = t * z;
    } else {                                     // HC_EXTPOT_LOG
        const double mor = p[1] > 0.0 ? p[0] / p[1] : p[0];
        const double iq = 1.0 / (p[2] * p[2]), ir = 1.0 / (p[3] * p[3]);
        const double rad = p[1] * p[1] + x * x + y * y * iq + z * z * ir;
        *pot = mor * log(rad);
        const double f = -2.0 * mor / rad;
        *ax = f * x;
        *ay = f * y * iq;
        *az = f * z * ir;
    }
}

// External field added to every body after the walk (hackcode3/grav.c:34-38),
// and the rest of the closing half-kick: the walk kicked with the tree part
// against the previous total acceleration.
__global__ void k_extpot(int64_t n, int kind, double p0, double p1, double p2, double p3, const double *px,
                         const double *py, const double *pz, double *ax, double *ay, double *az, double *phi,
                         double *phi_ext, double *vx, double *vy, double *vz, double kick_dthf, int64_t nstep)
{
    const double p[4] = {p0, p1, p2, p3};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double fx, fy, fz, pot;
        ext_field(kind, p, px[i], py[i], pz[i], &fx, &fy, &fz, &pot);
        if (kick_dthf != 0.0 && nstep > 0) {
            vx[i] = __dadd_rn(vx[i], __dmul_rn(fx, kick_dthf));
            vy[i] = __dadd_rn(vy[i], __dmul_rn(fy, kick_dthf));
            vz[i] = __dadd_rn(vz[i], __dmul_rn(fz, kick_dthf));
        }
        ax[i] = __dadd_rn(ax[i], fx);
        ay[i] = __dadd_rn(ay[i], fy);
        az[i] = __dadd_rn(az[i], fz);
        phi[i] = __dadd_rn(phi[i], pot);
        phi_ext[i] = pot;
    }
}

__device__ __forceinline__ double wsum(double v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-block partial sums in a fixed order (deterministic for a given launch shape).
__global__ void __launch_bounds__(DIAG_THREADS) k_diag_part(int64_t n, const double *mass, const double *px,
                                                            const double *py, const double *pz, const double *vx,
                                                            const double *vy, const double *vz, const double *ax,
                                                            const double *ay, const double *az, const double *phi,
                                                            const double *phi_ext, double *part)
{
    double acc[NDIAG];
#pragma unroll
    for (int q = 0; q < NDIAG; q++) acc[q] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x[3] = {px[i], py[i], pz[i]}, v[3] = {vx[i], vy[i], vz[i]}, a[3] = {ax[i], ay[i], az[i]};
        // with an external field phi holds tree + external; its energy
        // counts the external part once more (hackcode3/code_io.c:180-186)
        hc_diag_body(acc, mass[i], x, v, a, phi_ext ? __dadd_rn(phi[i], phi_ext[i]) : phi[i]);
    }
    __shared__ double sh[DIAG_THREADS / 32][NDIAG];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NDIAG; q++) {
        double s = wsum(acc[q]);
        if (lane == 0) sh[wid][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < NDIAG) {
        double s = 0.0;
        for (int w = 0; w < DIAG_THREADS / 32; w++) s += sh[w][threadIdx.x];
        part[(int64_t)blockIdx.x * NDIAG + threadIdx.x] = s;
    }
}

__global__ void k_diag_final(const double *part, int nparts, double *out)
{
    int q = threadIdx.x;
    if (q < NDIAG) {
        double s = 0.0;
        for (int b = 0; b < nparts; b++) s += part[(int64_t)b * NDIAG + q];
        out[q] = s;
    }
}

// FP64 direct sum at sampled bodies (self skipped), sources staged through
// shared memory in tiles.  Exact limit of the walk (tol = 0).
constexpr int DTILE = 256;
__global__ void __launch_bounds__(DTILE) k_direct(int64_t n, const double *mass, const double *px, const double *py,
                                                  const double *pz, const int64_t *idx, int64_t ns, double eps2,
                                                  double *oacc, double *ophi)
{
    __shared__ double sm[DTILE], sx[DTILE], sy[DTILE], sz[DTILE];
    const int64_t t = blockIdx.x * (int64_t)DTILE + threadIdx.x;
    const bool valid = t < ns;
    const int64_t me = valid ? idx[t] : -1;
    const double x = valid ? px[me] : 0.0, y = valid ? py[me] : 0.0, z = valid ? pz[me] : 0.0;
    double ax = 0.0, ay = 0.0, az = 0.0, ph = 0.0;
    for (int64_t base = 0; base < n; base += DTILE) {
        const int64_t j = base + threadIdx.x;
        sm[threadIdx.x] = j < n ? mass[j] : 0.0;
        sx[threadIdx.x] = j < n ? px[j] : 0.0;
        sy[threadIdx.x] = j < n ? py[j] : 0.0;
        sz[threadIdx.x] = j < n ? pz[j] : 0.0;
        __syncthreads();
        const int cnt = (n - base) < DTILE ? (int)(n - base) : DTILE;
        for (int k = 0; k < cnt; k++) {
            if (base + k == me) continue;
            const double m = sm[k];
            const double dx = sx[k] - x, dy = sy[k] - y, dz = sz[k] - z;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double rinv = 1.0 / sqrt(r2);
            const double mr = m * rinv, mr3 = mr * rinv * rinv;
            ph -= mr;
            ax += mr3 * dx;
            ay += mr3 * dy;
            az += mr3 * dz;
        }
        __syncthreads();
    }
    if (valid) {
        oacc[3 * t] = ax;
        oacc[3 * t + 1] = ay;
        oacc[3 * t + 2] = az;
        ophi[t] = ph;
    }
}

// FP32 FMA throughput probe: 8 independent FMA chains per thread.
constexpr int PEAK_ITERS = 4096;
__global__ void __launch_bounds__(256) k_fma_peak(float seed, float *sink)
{
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f, a4 = a0 + 4.f, a5 = a0 + 5.f,
          a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.999999f, k = 1e-7f;
#pragma unroll 16
    for (int i = 0; i < PEAK_ITERS; i++) {
        a0 = fmaf(a0, m, k);
        a1 = fmaf(a1, m, k);
        a2 = fmaf(a2, m, k);
        a3 = fmaf(a3, m, k);
        a4 = fmaf(a4, m, k);
        a5 = fmaf(a5, m, k);
        a6 = fmaf(a6, m, k);
        a7 = fmaf(a7, m, k);
    }
    float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 1234.5f) sink[threadIdx.x] = r;   // keeps the chains live
}

}  // namespace

int hc_fma_peak_impl(hc_ctx *c, double *tflops)
{
    int dev = 0, nsm = 0;
    HC_CUDA(cudaGetDevice(&dev));
    HC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = nsm * 16;
    float *sink = (float *)c->diag_part;
    k_fma_peak<<<blocks, 256, 0, c->stream>>>(1.0f, sink);     // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 5; rep++) {
        HC_CUDA(cudaEventRecord(c->ev[0], c->stream));
        k_fma_peak<<<blocks, 256, 0, c->stream>>>(1.0f + rep, sink);
        HC_CUDA(cudaEventRecord(c->ev[1], c->stream));
        HC_CUDA(cudaEventSynchronize(c->ev[1]));
        float ms;
        HC_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        if (ms < best) best = ms;
    }
    const double flops = 2.0 * 8.0 * PEAK_ITERS * (double)blocks * 256.0;
    *tflops = flops / (best * 1e-3) / 1e12;
    return HC_OK;
}

void hc_kick_drift(hc_ctx *c, double dt)
{
    k_kick_drift<<<hc_grid(c->n, 256), 256, 0, c->stream>>>(c->n, dt, c->px, c->py, c->pz, c->vx, c->vy, c->vz,
                                                            c->ax, c->ay, c->az);
    c->launches++;
}

void hc_extpot_launch(hc_ctx *c, double kick_dthf, int64_t nstep)
{
    const double *q = c->extpot_par;
    k_extpot<<<hc_grid(c->n, 256), 256, 0, c->stream>>>(c->n, c->extpot, q[0], q[1], q[2], q[3], c->px, c->py, c->pz,
                                                        c->ax, c->ay, c->az, c->phi, c->phi_ext, c->vx, c->vy, c->vz,
                                                        kick_dthf, nstep);
    c->launches++;
}

// out36 (device): KE, PE, keten, peten, amten(raw), sum m x, sum m v, mtot
void hc_diag_launch(hc_ctx *c, double *out36)
{
    int nb = (int)std::min<int64_t>(DIAG_BLOCKS, (c->n + DIAG_THREADS - 1) / DIAG_THREADS);
    if (nb < 1) nb = 1;
    k_diag_part<<<nb, DIAG_THREADS, 0, c->stream>>>(c->n, c->mass, c->px, c->py, c->pz, c->vx, c->vy, c->vz, c->ax,
                                                    c->ay, c->az, c->phi, c->extpot ? c->phi_ext : nullptr,
                                                    c->diag_part);
    k_diag_final<<<1, 64, 0, c->stream>>>(c->diag_part, nb, out36);
    c->launches += 2;
}

void hc_direct_launch(hc_ctx *c, const int64_t *idx_dev, int64_t ns, double *oacc, double *ophi)
{
    int nb = (int)((ns + DTILE - 1) / DTILE);
    k_direct<<<nb, DTILE, 0, c->stream>>>(c->n, c->mass, c->px, c->py, c->pz, idx_dev, ns,
                                          c->prm.eps * c->prm.eps, oacc, ophi);
    c->launches++;
}
