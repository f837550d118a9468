// hc_ensemble.cu -- ensembles of independent systems of uneven size, stepped
// together (no counterpart in hackcode1, which evolves one system per run).
//
// Layout (internal order: tree systems first, then direct-sum systems; the
// host API converts from and to the caller's order):
//   FP64 SoA over all bodies: mass, x/y/z (each system in its own
//   coordinates), v, a, phi.  The tree systems' mass / v / a / phi arrays
//   are the first n_tree entries of these and are shared with one forest
//   context (hc_ctx) whose positions are forest coordinates.
//
// One step, all of it captured in one CUDA graph:
//   1. per tree system, hackcode1's expandbox replay (load.c:68-95) on its
//      own persistent root box, which starts at (-2,-2,-2), 4 (code.c:119-120)
//      and only grows -- one warp per system, bodies in order;
//   2. slot layout: every system box is placed in its own slot of one forest
//      box (slots of the largest system's size on a G^3 grid, G a power of
//      two), so that the system box is exactly a forest cell; positions are
//      translated into the slot;
//   3. the single-system build (keys, sort, cells, upward pass, groups) on
//      the forest -- cells never straddle systems, and every walk group lies
//      in one system;
//   4. the walk of each group starts at its system's root cell (found from
//      the pre-order cells), so no system sees another;
//   5. systems of at most direct_max bodies: FP32 direct sum, one block per
//      system, positions split hi + lo relative to the system's first body;
//   6. closing half-kick inside 3-5 (code.c:175-179), per-system energies,
//      then kick-drift of every body (code.c:182-188).
//
// Differences from running hackcode1 once per system: a system's keys keep
// 30 - depth(system root in the forest) bits per axis (bodies closer than
// that are reported as coincident), and the one-body cells that hackcode1
// grafts when its second body expands the box twice or more are not formed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "hc_internal.cuh"

#define HC_TRY(x)                   \
    do {                            \
        int r_ = (x);               \
        if (r_ != HC_OK) return r_; \
    } while (0)

namespace {

constexpr int DTHREADS = 256;       // energy kernel; the direct sum's block size is tuned (128..512)

struct SysBox {
    double rmin[3];
    double rsize;
};

__device__ __forceinline__ bool inbox_d(double x, double y, double z, const double *rmin, double rsize)
{
    // intcoord (load.c:135-156): 0 <= (x - rmin) / rsize < 1 on every axis
    const double p[3] = {x, y, z};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double s = __ddiv_rn(__dsub_rn(p[k], rmin[k]), rsize);
        if (!(0.0 <= s && s < 1.0)) return false;
    }
    return true;
}

// 1. expandbox replay, one warp per tree system.  The box only grows, so a
// body found inside stays inside: each pass finds the first body of the
// remaining range outside the current box and expands for it.
__global__ void k_ens_replay(int nsys_tree, const int64_t *off, const double *mass, const double *px,
                             const double *py, const double *pz, SysBox *box, hc_status *st)
{
    const int lane = threadIdx.x & 31;
    const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= nsys_tree) return;
    double rmin[3] = {box[s].rmin[0], box[s].rmin[1], box[s].rmin[2]};
    double rsize = box[s].rsize;
    const int64_t b0 = off[s], b1 = off[s + 1];
    for (int64_t base = b0; base < b1; base += 32) {
        const int64_t i = base + lane;
        bool out = false;
        if (i < b1 && mass[i] != 0.0) out = !inbox_d(px[i], py[i], pz[i], rmin, rsize);
        unsigned m = __ballot_sync(0xffffffffu, out);
        while (m) {
            const int f = __ffs(m) - 1;
            const int64_t j = base + f;
            const double x[3] = {px[j], py[j], pz[j]};
            int k = 0;
            while (!inbox_d(x[0], x[1], x[2], rmin, rsize)) {     // load.c:74-93 (same on every lane)
                if (++k > 1100) {                                  // non-finite position
                    if (lane == 0) {
                        atomicCAS(&st->error, 0, HC_ERR_ARG);
                        st->info = (int)j;
                    }
                    return;
                }
                double rmid[3];
                for (int d = 0; d < 3; d++) rmid[d] = __dadd_rn(rmin[d], __dmul_rn(0.5, rsize));
                for (int d = 0; d < 3; d++)
                    if (x[d] < rmid[d]) rmin[d] = __dsub_rn(rmin[d], rsize);
                rsize = __dmul_rn(2.0, rsize);
            }
            // bodies after f in this chunk: test again against the grown box
            out = false;
            if (lane > f && i < b1 && mass[i] != 0.0) out = !inbox_d(px[i], py[i], pz[i], rmin, rsize);
            m = __ballot_sync(0xffffffffu, out);
        }
    }
    if (lane == 0) box[s] = SysBox{{rmin[0], rmin[1], rmin[2]}, rsize};
}

// 2a. slot layout (one block): slot size = largest system box, G^3 slots;
// forest box (0,0,0), G * slot; depth of each system root in the forest.
__global__ void k_ens_layout(int nsys_tree, int gbits, const SysBox *box, double *origin, int32_t *depth,
                             int32_t *root, hc_box *fbox, hc_status *st)
{
    __shared__ double smax;
    if (threadIdx.x == 0) smax = 0.0;
    __syncthreads();
    double lmax = 0.0;
    for (int s = threadIdx.x; s < nsys_tree; s += blockDim.x) lmax = fmax(lmax, box[s].rsize);
    // block max via shared atomics on the bit pattern (positive doubles order like integers)
    atomicMax(reinterpret_cast<unsigned long long *>(&smax), (unsigned long long)__double_as_longlong(lmax));
    __syncthreads();
    const double S = smax;
    const int G = 1 << gbits;
    for (int s = threadIdx.x; s < nsys_tree; s += blockDim.x) {
        const int gx = s & (G - 1), gy = (s >> gbits) & (G - 1), gz = s >> (2 * gbits);
        origin[3 * s + 0] = __dmul_rn((double)gx, S);
        origin[3 * s + 1] = __dmul_rn((double)gy, S);
        origin[3 * s + 2] = __dmul_rn((double)gz, S);
        // rsize values are 4 * 2^k: S / rsize is an exact power of two
        int e = 0;
        double r = box[s].rsize;
        while (r < S && e < 64) {
            r = __dmul_rn(2.0, r);
            e++;
        }
        depth[s] = gbits + e;
        root[s] = -1;
        if (gbits + e > 29) {                 // no key bits left inside the system
            atomicCAS(&st->error, 0, HC_ERR_ARG);
            st->info = s;
        }
    }
    if (threadIdx.x == 0) {
        fbox->rmin[0] = fbox->rmin[1] = fbox->rmin[2] = 0.0;
        fbox->rsize = __dmul_rn((double)G, S);
        fbox->first_massive = -1;
        fbox->chain_lmax = fbox->chain_lmin = -1;
    }
}

// 2b. forest coordinates: x_f = (x - rmin_s) + origin_s; a massive body stays
// inside its system's cell (massless ones are only targets and may lie outside)
__global__ void k_ens_translate(int64_t n_tree, const int32_t *body_sys, const SysBox *box, const double *origin,
                                const double *mass, const double *px, const double *py, const double *pz,
                                double *fx, double *fy, double *fz)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_tree;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int s = body_sys[i];
        const SysBox b = box[s];
        const bool massive = mass[i] != 0.0;
        const double p[3] = {px[i], py[i], pz[i]};
        double q[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const double o = origin[3 * s + k];
            double v = __dadd_rn(__dsub_rn(p[k], b.rmin[k]), o);
            const double hi = __dadd_rn(o, b.rsize);
            if (massive && v >= hi) v = nextafter(hi, o);      // rounding must not leave the cell
            if (massive && v < o) v = o;
            q[k] = v;
        }
        fx[i] = q[0];
        fy[i] = q[1];
        fz[i] = q[2];
    }
}

// 4. root cell of each tree system: the cell at the system's depth that
// holds its first body in key order
__global__ void k_ens_roots(const hc_box *fbox, const int32_t *pre_depth, const int32_t *pre_a, const uint32_t *midx,
                            const uint32_t *pre2bfs, const int32_t *body_sys, const int32_t *depth, int32_t *root)
{
    const int nn = fbox->nnode;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nn; p += gridDim.x * blockDim.x) {
        const int a = pre_a[p];
        if (a < 0) continue;                          // a body
        const int s = body_sys[midx[a]];
        if (pre_depth[p] == depth[s]) root[s] = (int32_t)pre2bfs[p];
    }
}

__device__ __forceinline__ void kahan(float &sum, float &comp, float x)
{
    const float y = __fsub_rn(x, comp);
    const float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

// 5. direct sum of one small system per block (FP32, hi + lo positions
// relative to the system's first body; Kahan over 64-body partials); any
// block size up to 512 threads
__global__ void __launch_bounds__(512) k_ens_direct(const int32_t *dsys, const int64_t *off, const double *mass,
                                                         const double *px, const double *py, const double *pz,
                                                         float eps2, double kick_dthf, int64_t nstep, double *vx,
                                                         double *vy, double *vz, double *ax, double *ay, double *az,
                                                         double *phi)
{
    extern __shared__ float4 sm[];
    const int s = dsys[blockIdx.x];
    const int64_t b0 = off[s];
    const int n = (int)(off[s + 1] - b0);
    float4 *H = sm, *L = sm + n;
    const double cx = px[b0], cy = py[b0], cz = pz[b0];
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double dx = px[b0 + j] - cx, dy = py[b0 + j] - cy, dz = pz[b0 + j] - cz;
        float4 h, l;
        hc_split_hilo(dx, &h.x, &l.x);          // on the doubles' bits (no FP64-pipe conversions)
        hc_split_hilo(dy, &h.y, &l.y);
        hc_split_hilo(dz, &h.z, &l.z);
        h.w = hc_d2f_rn(mass[b0 + j]);
        l.w = 0.f;
        H[j] = h;
        L[j] = l;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float4 Hi = H[i], Li = L[i];
        float sx = 0.f, sy = 0.f, sz = 0.f, sp = 0.f, cxs = 0.f, cys = 0.f, czs = 0.f, cps = 0.f;
        for (int j0 = 0; j0 < n; j0 += 64) {
            const int j1 = j0 + 64 < n ? j0 + 64 : n;
            float qx = 0.f, qy = 0.f, qz = 0.f, qp = 0.f;
            for (int j = j0; j < j1; j++) {
                const float4 Hj = H[j], Lj = L[j];
                const float dx = (Hj.x - Hi.x) + (Lj.x - Li.x), dy = (Hj.y - Hi.y) + (Lj.y - Li.y),
                            dz = (Hj.z - Hi.z) + (Lj.z - Li.z);
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                const float rinv = rsqrtf(r2);
                const float mr = j == i ? 0.f : Hj.w * rinv;
                const float mr3 = mr * rinv * rinv;
                qp -= mr;
                qx = fmaf(mr3, dx, qx);
                qy = fmaf(mr3, dy, qy);
                qz = fmaf(mr3, dz, qz);
            }
            kahan(sx, cxs, qx);
            kahan(sy, cys, qy);
            kahan(sz, czs, qz);
            kahan(sp, cps, qp);
        }
        const int64_t o = b0 + i;
        const double rx = (double)sx - (double)cxs, ry = (double)sy - (double)cys, rz = (double)sz - (double)czs;
        if (kick_dthf != 0.0 && nstep > 0) {          // closing half kick (code.c:175-179)
            vx[o] = __dadd_rn(vx[o], __dmul_rn(__dsub_rn(rx, ax[o]), kick_dthf));
            vy[o] = __dadd_rn(vy[o], __dmul_rn(__dsub_rn(ry, ay[o]), kick_dthf));
            vz[o] = __dadd_rn(vz[o], __dmul_rn(__dsub_rn(rz, az[o]), kick_dthf));
        }
        ax[o] = rx;
        ay[o] = ry;
        az[o] = rz;
        phi[o] = (double)sp - (double)cps;
    }
}

// 6a. kinetic and potential energy of each system (code_io.c:160-197)
__global__ void __launch_bounds__(DTHREADS) k_ens_energy(const int64_t *off, const int32_t *user_of, const double *mass,
                                                         const double *vx, const double *vy, const double *vz,
                                                         const double *phi, double *out)
{
    const int s = blockIdx.x;
    double ke = 0.0, pe = 0.0;
    for (int64_t i = off[s] + threadIdx.x; i < off[s + 1]; i += DTHREADS) {
        const double hm = __dmul_rn(0.5, mass[i]);
        double v2 = __dmul_rn(vx[i], vx[i]);
        v2 = __dadd_rn(v2, __dmul_rn(vy[i], vy[i]));
        v2 = __dadd_rn(v2, __dmul_rn(vz[i], vz[i]));
        ke += __dmul_rn(hm, v2);
        pe += __dmul_rn(hm, phi[i]);
    }
    __shared__ double rk[DTHREADS], rp[DTHREADS];
    rk[threadIdx.x] = ke;
    rp[threadIdx.x] = pe;
    __syncthreads();
    for (int o = DTHREADS / 2; o; o >>= 1) {
        if (threadIdx.x < o) {
            rk[threadIdx.x] += rk[threadIdx.x + o];
            rp[threadIdx.x] += rp[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int u = user_of[s];
        out[3 * u + 0] = rk[0];
        out[3 * u + 1] = rp[0];
        out[3 * u + 2] = rk[0] + rp[0];
    }
}

// 6b. v += a dt/2; x += v dt; v += a dt/2  (code.c:182-188)
__global__ void k_ens_kick_drift(int64_t n, double dt, double *px, double *py, double *pz, double *vx, double *vy,
                                 double *vz, const double *ax, const double *ay, const double *az)
{
    const double dthf = 0.5 * dt;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double *p[3] = {px, py, pz}, *v[3] = {vx, vy, vz};
        const double *a[3] = {ax, ay, az};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const double dvel = __dmul_rn(a[k][i], dthf);
            const double vel1 = __dadd_rn(v[k][i], dvel);
            p[k][i] = __dadd_rn(p[k][i], __dmul_rn(vel1, dt));
            v[k][i] = __dadd_rn(vel1, dvel);
        }
    }
}

__global__ void k_unpack_sys(const double *phase, int64_t n, double *px, double *py, double *pz, double *vx,
                             double *vy, double *vz)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double *q = phase + 6 * i;
        px[i] = q[0];
        py[i] = q[1];
        pz[i] = q[2];
        vx[i] = q[3];
        vy[i] = q[4];
        vz[i] = q[5];
    }
}

__global__ void k_init_boxes(int n, SysBox *box)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        box[s] = SysBox{{-2.0, -2.0, -2.0}, 4.0};    // code.c:119-120
}

template <typename T>
int ens_alloc(std::string &err, T **p, int64_t count)
{
    const size_t bytes = sizeof(T) * (size_t)std::max<int64_t>(count, 1);
    if (cudaMalloc((void **)p, bytes) != cudaSuccess) {
        err = "cudaMalloc(" + std::to_string(bytes) + ") failed";
        *p = nullptr;
        return HC_ERR_NOMEM;
    }
    return HC_OK;
}

}  // namespace

struct hc_ens {
    std::string err;
    hc_ens_params prm{};
    int nsys = 0, nsys_tree = 0, nsys_direct = 0, gbits = 0;
    int64_t ntot = 0, n_tree = 0;
    std::vector<int64_t> user_count, user_off;   // caller's order
    std::vector<int> order;                      // internal slot -> caller's system
    std::vector<int64_t> int_off;                // internal offsets [nsys + 1]
    hc_ctx *forest = nullptr;                    // tree systems (n_tree bodies), or null
    cudaStream_t stream = nullptr;               // forest's stream or own
    bool own_stream = false;
    cudaEvent_t ev[4] = {};
    // device, internal order
    double *mass = nullptr, *px = nullptr, *py = nullptr, *pz = nullptr, *vx = nullptr, *vy = nullptr,
           *vz = nullptr, *ax = nullptr, *ay = nullptr, *az = nullptr, *phi = nullptr;
    int64_t *d_off = nullptr;
    int32_t *d_body_sys = nullptr, *d_user_of = nullptr, *d_dsys = nullptr;
    int32_t *d_root = nullptr, *d_depth = nullptr;
    SysBox *d_box = nullptr;
    double *d_origin = nullptr, *d_energy = nullptr, *h_energy = nullptr, *d_stage = nullptr;
    int max_direct_n = 0;
    int direct_threads = 256;                    // block size of the direct sum (tuned)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    double graph_dt[2] = {0.0, 0.0};
    int64_t launches = 0, graph_launches[2] = {0, 0};
    float tree_ms = 0.f, direct_ms = 0.f;
};

#define EC(call)                                                                 \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) {                                                 \
            e->err = std::string(#call) + ": " + cudaGetErrorString(e_);         \
            return HC_ERR_CUDA;                                                  \
        }                                                                        \
    } while (0)

namespace {

// Everything of one step after the positions are final, on e->stream,
// without host synchronisation (graph-capturable).
int ens_enqueue(hc_ens *e, double kick_dthf, int64_t nstep, double dt, bool capturing, bool advance = true)
{
    cudaStream_t s = e->stream;
    const unsigned rflags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    e->launches = 0;
    EC(cudaEventRecordWithFlags(e->ev[0], s, rflags));
    if (e->forest) {
        hc_ctx *c = e->forest;
        EC(cudaMemsetAsync(c->st, 0, sizeof(hc_status), s));
        k_ens_replay<<<(e->nsys_tree + 3) / 4, 128, 0, s>>>(e->nsys_tree, e->d_off, e->mass, e->px, e->py, e->pz,
                                                          e->d_box, c->st);
        k_ens_layout<<<1, 256, 0, s>>>(e->nsys_tree, e->gbits, e->d_box, e->d_origin, e->d_depth, e->d_root, c->box,
                                       c->st);
        k_ens_translate<<<hc_grid(e->n_tree, 256), 256, 0, s>>>(e->n_tree, e->d_body_sys, e->d_box, e->d_origin,
                                                                e->mass, e->px, e->py, e->pz, c->px, c->py, c->pz);
        e->launches += 3;
        c->launches = 0;
        int r = hc_tree_build(c);
        if (r != HC_OK) {
            e->err = c->err;
            return r;
        }
        k_ens_roots<<<hc_grid(c->maxnode, 256), 256, 0, s>>>(c->box, c->pre_info, c->pre_a, c->midx, c->pre2bfs,
                                                             e->d_body_sys, e->d_depth, e->d_root);
        r = hc_walk_launch(c, true, c->n, c->tord, c->px, c->py, c->pz, c->ax, c->ay, c->az, c->phi, kick_dthf,
                           nstep);
        if (r != HC_OK) {
            e->err = c->err;
            return r;
        }
        e->launches += c->launches + 1;
    }
    EC(cudaEventRecordWithFlags(e->ev[1], s, rflags));
    if (e->nsys_direct > 0) {
        const size_t smem = sizeof(float4) * 2 * (size_t)e->max_direct_n;
        k_ens_direct<<<e->nsys_direct, e->direct_threads, smem, s>>>(e->d_dsys, e->d_off, e->mass, e->px, e->py, e->pz,
                                                             (float)(e->prm.eps * e->prm.eps), kick_dthf, nstep,
                                                             e->vx, e->vy, e->vz, e->ax, e->ay, e->az, e->phi);
        e->launches++;
    }
    EC(cudaEventRecordWithFlags(e->ev[2], s, rflags));
    if (!advance) return HC_OK;          // forces only (the autotuner's evaluations)
    k_ens_energy<<<e->nsys, DTHREADS, 0, s>>>(e->d_off, e->d_user_of, e->mass, e->vx, e->vy, e->vz, e->phi,
                                              e->d_energy);
    k_ens_kick_drift<<<hc_grid(e->ntot, 256), 256, 0, s>>>(e->ntot, dt, e->px, e->py, e->pz, e->vx, e->vy, e->vz,
                                                           e->ax, e->ay, e->az);
    e->launches += 2;
    EC(cudaMemcpyAsync(e->h_energy, e->d_energy, sizeof(double) * 3 * e->nsys, cudaMemcpyDeviceToHost, s));
    if (e->forest) EC(cudaMemcpyAsync(e->forest->h_st, e->forest->st, sizeof(hc_status), cudaMemcpyDeviceToHost, s));
    return HC_OK;
}

const char *status_text(int code)
{
    switch (code) {
    case HC_ERR_COINCIDENT: return "two bodies of one system share a key at the forest's resolution";
    case HC_ERR_CELLS: return "cell pool exhausted";
    case HC_ERR_STACK: return "walk stack overflow";
    case HC_ERR_ARG: return "non-finite position, or a system box too large for the forest";
    case HC_ERR_STATE: return "a tree system has no root cell";
    default: return "device error";
    }
}

}  // namespace

extern "C" {

int hc_ens_create(hc_ens **out, int nsys, const int64_t *counts, const hc_ens_params *params)
{
    if (!out || nsys < 1 || !counts || !params) return HC_ERR_ARG;
    if (params->direct_max < 0 || params->direct_max > HC_ENS_DIRECT_LIMIT || !(params->eps >= 0.0) ||
        !(params->tol >= 0.0) || !std::isfinite(params->eps) || !std::isfinite(params->tol))
        return HC_ERR_ARG;
    hc_ens *e = new hc_ens();
    *out = e;
    e->prm = *params;
    e->nsys = nsys;
    e->user_count.assign(counts, counts + nsys);
    e->user_off.assign(nsys + 1, 0);
    for (int s = 0; s < nsys; s++) {
        if (counts[s] < 1) {
            e->err = "every system needs at least one body";
            return HC_ERR_ARG;
        }
        if (counts[s] > (1LL << 28) || e->user_off[s] + counts[s] > (1LL << 28)) {
            e->err = "at most 2^28 bodies in all";
            return HC_ERR_ARG;
        }
        e->user_off[s + 1] = e->user_off[s] + counts[s];
    }
    e->ntot = e->user_off[nsys];
    if (e->ntot > (1LL << 28)) {
        e->err = "at most 2^28 bodies in all";
        return HC_ERR_ARG;
    }
    // internal order: tree systems (more than direct_max bodies) first
    for (int s = 0; s < nsys; s++)
        if (counts[s] > params->direct_max) e->order.push_back(s);
    e->nsys_tree = (int)e->order.size();
    for (int s = 0; s < nsys; s++)
        if (counts[s] <= params->direct_max) {
            e->order.push_back(s);
            e->max_direct_n = std::max<int>(e->max_direct_n, (int)counts[s]);
        }
    e->nsys_direct = nsys - e->nsys_tree;
    e->int_off.assign(nsys + 1, 0);
    for (int k = 0; k < nsys; k++) e->int_off[k + 1] = e->int_off[k] + counts[e->order[k]];
    e->n_tree = e->int_off[e->nsys_tree];
    while ((1LL << (3 * e->gbits)) < e->nsys_tree) e->gbits++;

    const int64_t n = e->ntot;
    double **arrs[] = {&e->mass, &e->px, &e->py, &e->pz, &e->vx, &e->vy, &e->vz, &e->ax, &e->ay, &e->az, &e->phi};
    for (double **p : arrs) HC_TRY(ens_alloc(e->err, p, n));
    HC_TRY(ens_alloc(e->err, &e->d_off, nsys + 1));
    HC_TRY(ens_alloc(e->err, &e->d_body_sys, n));
    HC_TRY(ens_alloc(e->err, &e->d_user_of, nsys));
    HC_TRY(ens_alloc(e->err, &e->d_dsys, std::max(1, e->nsys_direct)));
    HC_TRY(ens_alloc(e->err, &e->d_root, std::max(1, e->nsys_tree)));
    HC_TRY(ens_alloc(e->err, &e->d_depth, std::max(1, e->nsys_tree)));
    HC_TRY(ens_alloc(e->err, &e->d_box, std::max(1, e->nsys_tree)));
    HC_TRY(ens_alloc(e->err, &e->d_origin, 3 * std::max(1, e->nsys_tree)));
    HC_TRY(ens_alloc(e->err, &e->d_energy, 3 * nsys));
    EC(cudaMallocHost((void **)&e->h_energy, sizeof(double) * 3 * nsys));
    {
        std::vector<int32_t> body_sys(n), user_of(nsys), dsys(std::max(1, e->nsys_direct));
        for (int k = 0; k < nsys; k++) {
            user_of[k] = e->order[k];
            for (int64_t i = e->int_off[k]; i < e->int_off[k + 1]; i++) body_sys[i] = k;
            if (k >= e->nsys_tree) dsys[k - e->nsys_tree] = k;
        }
        EC(cudaMemcpy(e->d_off, e->int_off.data(), sizeof(int64_t) * (nsys + 1), cudaMemcpyHostToDevice));
        EC(cudaMemcpy(e->d_body_sys, body_sys.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        EC(cudaMemcpy(e->d_user_of, user_of.data(), sizeof(int32_t) * nsys, cudaMemcpyHostToDevice));
        EC(cudaMemcpy(e->d_dsys, dsys.data(), sizeof(int32_t) * dsys.size(), cudaMemcpyHostToDevice));
    }
    if (e->nsys_tree > 0) {
        hc_params p = {params->tol, params->eps, params->fcells > 0 ? params->fcells : 1.0, params->usequad, 0};
        int r = hc_create(&e->forest, e->n_tree, &p);
        if (r != HC_OK) {
            e->err = e->forest ? std::string("forest: ") + e->forest->err : "forest context";
            return r;
        }
        hc_ctx *c = e->forest;
        // the forest shares the tree systems' mass, velocity, acceleration, potential
        double **mine[] = {&c->mass, &c->vx, &c->vy, &c->vz, &c->ax, &c->ay, &c->az, &c->phi};
        double *ens[] = {e->mass, e->vx, e->vy, e->vz, e->ax, e->ay, e->az, e->phi};
        for (int k = 0; k < 8; k++) {
            cudaFree(*mine[k]);
            *mine[k] = ens[k];
        }
        c->group_kind = HC_GROUPS_TREE;      // groups must not straddle systems
        c->walk_sys_root = e->d_root;
        c->walk_body_sys = e->d_body_sys;
        e->stream = c->stream;
        k_init_boxes<<<hc_grid(e->nsys_tree, 256), 256, 0, e->stream>>>(e->nsys_tree, e->d_box);
    } else {
        EC(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        e->own_stream = true;
    }
    for (auto &ev : e->ev) EC(cudaEventCreate(&ev));
    if (e->max_direct_n > 0) {
        const size_t smem = sizeof(float4) * 2 * (size_t)e->max_direct_n;
        EC(cudaFuncSetAttribute(k_ens_direct, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    EC(cudaStreamSynchronize(e->stream));
    return HC_OK;
}

void hc_ens_destroy(hc_ens *e)
{
    if (!e) return;
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (auto &g : e->graph)
        if (g) cudaGraphExecDestroy(g);
    if (e->forest) {
        hc_ctx *c = e->forest;
        c->mass = c->vx = c->vy = c->vz = c->ax = c->ay = c->az = c->phi = nullptr;   // owned here
        hc_destroy(c);
    } else if (e->own_stream && e->stream) {
        cudaStreamDestroy(e->stream);
    }
    void *ptrs[] = {e->mass, e->px, e->py, e->pz, e->vx, e->vy, e->vz, e->ax, e->ay, e->az, e->phi, e->d_off,
                    e->d_body_sys, e->d_user_of, e->d_dsys, e->d_root, e->d_depth, e->d_box, e->d_origin,
                    e->d_energy, e->d_stage};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (e->h_energy) cudaFreeHost(e->h_energy);
    for (auto &ev : e->ev)
        if (ev) cudaEventDestroy(ev);
    delete e;
}

const char *hc_ens_last_error(const hc_ens *e) { return e ? e->err.c_str() : "null ensemble"; }

int hc_ens_upload(hc_ens *e, const double *mass, const double *phase)
{
    if (!e || !mass || !phase) return HC_ERR_ARG;
    const int64_t n = e->ntot;
    std::vector<double> m(n), ph(6 * n);
    for (int k = 0; k < e->nsys; k++) {
        const int u = e->order[k];
        const int64_t cnt = e->user_count[u];
        std::memcpy(&m[e->int_off[k]], mass + e->user_off[u], sizeof(double) * cnt);
        std::memcpy(&ph[6 * e->int_off[k]], phase + 6 * e->user_off[u], sizeof(double) * 6 * cnt);
    }
    for (int64_t i = 0; i < n; i++)
        if (!std::isfinite(m[i]) || !(m[i] > 0.0)) {
            // a massless body is walked in a run of 32 with its neighbours in
            // key order, which may belong to another system
            e->err = "ensemble bodies need positive, finite masses";
            return HC_ERR_ARG;
        }
    if (!e->d_stage) HC_TRY(ens_alloc(e->err, &e->d_stage, 6 * n));
    EC(cudaMemcpyAsync(e->mass, m.data(), sizeof(double) * n, cudaMemcpyHostToDevice, e->stream));
    EC(cudaMemcpyAsync(e->d_stage, ph.data(), sizeof(double) * 6 * n, cudaMemcpyHostToDevice, e->stream));
    k_unpack_sys<<<hc_grid(n, 256), 256, 0, e->stream>>>(e->d_stage, n, e->px, e->py, e->pz, e->vx, e->vy, e->vz);
    double *z[] = {e->ax, e->ay, e->az, e->phi};
    for (double *p : z) EC(cudaMemsetAsync(p, 0, sizeof(double) * n, e->stream));
    if (e->nsys_tree > 0)
        k_init_boxes<<<hc_grid(e->nsys_tree, 256), 256, 0, e->stream>>>(e->nsys_tree, e->d_box);
    EC(cudaStreamSynchronize(e->stream));
    EC(cudaGetLastError());
    return HC_OK;
}

int hc_ens_step(hc_ens *e, double dt, int64_t nstep, double *energy)
{
    if (!e || !(dt > 0) || nstep < 0) return HC_ERR_ARG;
    const double kick = nstep > 0 ? 0.5 * dt : 0.0;
    const int slot = nstep > 0 ? 1 : 0;
    if (!e->graph[slot] || e->graph_dt[slot] != dt) {
        if (e->graph[slot]) cudaGraphExecDestroy(e->graph[slot]);
        e->graph[slot] = nullptr;
        cudaGraph_t g = nullptr;
        EC(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        int r = ens_enqueue(e, kick, nstep > 0 ? 1 : 0, dt, true);
        cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        if (r != HC_OK) {
            if (g) cudaGraphDestroy(g);
            return r;
        }
        if (ce != cudaSuccess) {
            e->err = std::string("stream capture: ") + cudaGetErrorString(ce);
            return HC_ERR_CUDA;
        }
        ce = cudaGraphInstantiate(&e->graph[slot], g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            e->graph[slot] = nullptr;
            e->err = std::string("graph instantiate: ") + cudaGetErrorString(ce);
            return HC_ERR_CUDA;
        }
        e->graph_dt[slot] = dt;
        e->graph_launches[slot] = e->launches;
    }
    EC(cudaGraphLaunch(e->graph[slot], e->stream));
    e->launches = e->graph_launches[slot];
    EC(cudaStreamSynchronize(e->stream));
    EC(cudaGetLastError());
    if (e->forest) {
        const hc_status &st = *e->forest->h_st;
        if (st.error) {
            e->err = std::string("ensemble step: ") + status_text(st.error) + " (info " + std::to_string(st.info) + ")";
            return st.error;
        }
    }
    EC(cudaEventElapsedTime(&e->tree_ms, e->ev[0], e->ev[1]));
    EC(cudaEventElapsedTime(&e->direct_ms, e->ev[1], e->ev[2]));
    if (energy) std::memcpy(energy, e->h_energy, sizeof(double) * 3 * e->nsys);
    return HC_OK;
}

int hc_ens_set_tuning(hc_ens *e, const hc_ens_tuning *t)
{
    if (!e || !t) return HC_ERR_ARG;
    if (t->direct_threads != 128 && t->direct_threads != 256 && t->direct_threads != 512) {
        e->err = "hc_ens_set_tuning: direct_threads 128, 256 or 512";
        return HC_ERR_ARG;
    }
    if (e->forest) {
        hc_tuning w{t->group_max, t->list_depth, HC_GROUPS_TREE, 0.0};   // forest groups never straddle systems
        int r = hc_set_tuning(e->forest, &w);
        if (r != HC_OK) {
            e->err = std::string("forest: ") + e->forest->err;
            return r;
        }
    }
    e->direct_threads = t->direct_threads;
    for (int k = 0; k < 2; k++)
        if (e->graph[k]) {
            cudaGraphExecDestroy(e->graph[k]);
            e->graph[k] = nullptr;
        }
    return HC_OK;
}

int hc_ens_get_tuning(hc_ens *e, hc_ens_tuning *t)
{
    if (!e || !t) return HC_ERR_ARG;
    hc_tuning w{HC_GROUP2, 64, HC_GROUPS_TREE, 0.0};
    if (e->forest) hc_get_tuning(e->forest, &w);
    t->group_max = w.group_max;
    t->list_depth = w.list_depth;
    t->direct_threads = e->direct_threads;
    t->tree_ms = t->direct_ms = 0.0;
    return HC_OK;
}

// Times the force phases (tree systems, direct systems) of the current bodies
// for each candidate and keeps the fastest.  Positions and velocities do not
// move; the accelerations and potentials the step in progress needs are
// restored afterwards.
int hc_ens_autotune(hc_ens *e, hc_ens_tuning *best)
{
    if (!e) return HC_ERR_ARG;
    if (!e->d_stage) {
        e->err = "hc_ens_autotune: upload the bodies first";
        return HC_ERR_STATE;
    }
    const int64_t n = e->ntot;
    const size_t b = sizeof(double) * (size_t)n;
    double *const keep[4] = {e->ax, e->ay, e->az, e->phi};
    for (int k = 0; k < 4; k++) EC(cudaMemcpyAsync(e->d_stage + k * n, keep[k], b, cudaMemcpyDeviceToDevice, e->stream));
    hc_ens_tuning cur;
    hc_ens_get_tuning(e, &cur);
    auto timed = [&](const hc_ens_tuning &t, double *tree, double *direct) -> int {
        HC_TRY(hc_ens_set_tuning(e, &t));
        *tree = *direct = 1e300;
        for (int rep = 0; rep < 3; rep++) {
            HC_TRY(ens_enqueue(e, 0.0, 0, 0.0, false, false));
            EC(cudaStreamSynchronize(e->stream));
            if (e->forest) {
                EC(cudaMemcpy(e->forest->h_st, e->forest->st, sizeof(hc_status), cudaMemcpyDeviceToHost));
                if (e->forest->h_st->error) {
                    e->err = std::string("ensemble autotune: ") + status_text(e->forest->h_st->error);
                    return e->forest->h_st->error;
                }
            }
            float t0 = 0.f, t1 = 0.f;
            EC(cudaEventElapsedTime(&t0, e->ev[0], e->ev[1]));
            EC(cudaEventElapsedTime(&t1, e->ev[1], e->ev[2]));
            *tree = std::min(*tree, (double)t0);
            *direct = std::min(*direct, (double)t1);
        }
        return HC_OK;
    };
    hc_ens_tuning win = cur;
    win.tree_ms = win.direct_ms = 1e300;
    int r = HC_OK;
    // the two phases are independent: tree tuning first, then the direct block size
    const int gms[] = {HC_GROUP2 / 2, 3 * HC_GROUP2 / 4, HC_GROUP2}, lds[] = {32, 48, 64}, dts[] = {128, 256, 512};
    for (int gm : gms) {
        if (!e->forest && gm != cur.group_max) continue;
        for (int ld : lds) {
            if (!e->forest && ld != cur.list_depth) continue;
            hc_ens_tuning t{gm, ld, cur.direct_threads, 0.0, 0.0};
            double tr, di;
            if ((r = timed(t, &tr, &di)) != HC_OK) break;
            if (tr < win.tree_ms) {
                win.group_max = gm;
                win.list_depth = ld;
                win.tree_ms = tr;
            }
        }
        if (r != HC_OK) break;
    }
    for (int dt : dts) {
        if (r != HC_OK || e->nsys_direct == 0) break;
        hc_ens_tuning t{win.group_max, win.list_depth, dt, 0.0, 0.0};
        double tr, di;
        if ((r = timed(t, &tr, &di)) != HC_OK) break;
        if (di < win.direct_ms) {
            win.direct_threads = dt;
            win.direct_ms = di;
        }
    }
    for (int k = 0; k < 4; k++) EC(cudaMemcpyAsync(keep[k], e->d_stage + k * n, b, cudaMemcpyDeviceToDevice, e->stream));
    EC(cudaStreamSynchronize(e->stream));
    if (r != HC_OK) {                        // keep the caller's tuning and the error message
        const std::string err = e->err;
        hc_ens_set_tuning(e, &cur);
        e->err = err;
        return r;
    }
    HC_TRY(hc_ens_set_tuning(e, &win));
    if (e->nsys_direct == 0) win.direct_ms = 0.0;
    if (!e->forest) win.tree_ms = 0.0;
    if (best) *best = win;
    return HC_OK;
}

int hc_ens_download(hc_ens *e, double *phase, double *acc, double *phi)
{
    if (!e) return HC_ERR_ARG;
    const int64_t n = e->ntot;
    EC(cudaStreamSynchronize(e->stream));
    auto fetch = [&](const double *d, std::vector<double> &h) -> int {
        h.resize(n);
        EC(cudaMemcpy(h.data(), d, sizeof(double) * n, cudaMemcpyDeviceToHost));
        return HC_OK;
    };
    std::vector<double> a, b, c2;
    if (phase) {
        const double *src[6] = {e->px, e->py, e->pz, e->vx, e->vy, e->vz};
        for (int q = 0; q < 6; q++) {
            HC_TRY(fetch(src[q], a));
            for (int k = 0; k < e->nsys; k++) {
                const int u = e->order[k];
                for (int64_t i = 0; i < e->user_count[u]; i++) phase[6 * (e->user_off[u] + i) + q] = a[e->int_off[k] + i];
            }
        }
    }
    if (acc) {
        const double *src[3] = {e->ax, e->ay, e->az};
        for (int q = 0; q < 3; q++) {
            HC_TRY(fetch(src[q], a));
            for (int k = 0; k < e->nsys; k++) {
                const int u = e->order[k];
                for (int64_t i = 0; i < e->user_count[u]; i++) acc[3 * (e->user_off[u] + i) + q] = a[e->int_off[k] + i];
            }
        }
    }
    if (phi) {
        HC_TRY(fetch(e->phi, b));
        for (int k = 0; k < e->nsys; k++) {
            const int u = e->order[k];
            std::memcpy(phi + e->user_off[u], &b[e->int_off[k]], sizeof(double) * e->user_count[u]);
        }
    }
    (void)c2;
    return HC_OK;
}

int hc_ens_info(hc_ens *e, hc_ens_stats *out)
{
    if (!e || !out) return HC_ERR_ARG;
    std::memset(out, 0, sizeof *out);
    out->nsys_tree = e->nsys_tree;
    out->nsys_direct = e->nsys_direct;
    out->bodies_tree = e->n_tree;
    out->bodies_direct = e->ntot - e->n_tree;
    int64_t pairs = 0;
    for (int k = e->nsys_tree; k < e->nsys; k++) {
        const int64_t c = e->int_off[k + 1] - e->int_off[k];
        pairs += c * (c - 1);
    }
    out->interactions_direct = pairs;
    if (e->forest) {
        out->interactions_tree = (int64_t)(e->forest->h_st->n2b + e->forest->h_st->nbc);
    }
    out->tree_ms = e->tree_ms;
    out->direct_ms = e->direct_ms;
    out->launches = e->launches;
    return HC_OK;
}

}  // extern "C"
