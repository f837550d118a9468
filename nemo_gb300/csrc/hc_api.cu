// hc_api.cu -- the C ABI declared in include/hackcode_gpu.h.
//
// Every entry point validates its arguments, launches on the context's own
// stream, checks the device status word when it synchronises, and returns an
// HC_* code with the message kept in the context (hc_last_error).  Nothing
// here exits the process; nothing here falls back to a CPU path.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <unordered_set>
#include <vector>
#include "hc_internal.cuh"
#include "hc_mlp.cuh"

namespace {

template <typename T>
int dalloc(hc_ctx *c, T **p, int64_t count)
{
    size_t bytes = sizeof(T) * (size_t)std::max<int64_t>(count, 1);
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e != cudaSuccess) {
        c->err = std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e);
        *p = nullptr;
        return HC_ERR_NOMEM;
    }
    return HC_OK;
}

#define HC_TRY(x)                  \
    do {                           \
        int r_ = (x);              \
        if (r_ != HC_OK) return r_; \
    } while (0)

int check_status(hc_ctx *c)
{
    HC_CUDA(cudaMemcpyAsync(c->h_st, c->st, sizeof(hc_status), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    const hc_status &s = *c->h_st;
    if (s.error == 0) return HC_OK;
    char buf[256];
    switch (s.error) {
    case HC_ERR_CELLS:
        snprintf(buf, sizeof buf, "makecell: need more than %d cells; increase fcells", s.info);
        break;
    case HC_ERR_COINCIDENT:
        snprintf(buf, sizeof buf, "loadtree: body %d shares its integer coordinates with another body", s.info);
        break;
    case HC_ERR_STACK:
        snprintf(buf, sizeof buf, "walk: traversal stack of %d entries exhausted", s.info);
        break;
    default:
        snprintf(buf, sizeof buf, "device error %d (info %d)", s.error, s.info);
    }
    c->err = buf;
    return s.error;
}

void free_all(hc_ctx *c)
{
    void *ptrs[] = {c->mass, c->px, c->py, c->pz, c->vx, c->vy, c->vz, c->ax, c->ay, c->az, c->phi, c->cnt_b,
                    c->cnt_c, c->khi[0], c->khi[1], c->klo[0], c->klo[1], c->kval[0], c->kval[1], c->s_rank,
                    c->leaf_of_sorted, c->tord, c->gstart, c->gcount, c->gcnt, c->goff, c->mhi, c->mlo, c->midx, c->mpos, c->dlcp, c->ccount, c->pre_info, c->pre_a, c->bfs_a,
                    c->dkey[0], c->dkey[1], c->dval[0], c->dval[1], c->pre2bfs, c->parent, c->lastc, c->cperm, c->cbins,
                    c->nodeA, c->nodeB, c->nodeQ, c->nodeC, c->nm, c->ncx, c->ncy, c->ncz, c->flags,
                    c->scan_tmp, c->hist, c->cand, c->ncand, c->diag_part, c->st, c->box, c->tx, c->ty, c->tz,
                    c->tax, c->tay, c->taz, c->tphi, c->tkhi[0], c->tkhi[1], c->tklo[0], c->tklo[1],
                    c->tkval[0], c->tkval[1], c->thist};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    void *mptrs[] = {c->mlp_p, c->mlp_m, c->mlp_v, c->mlp_grad, c->mlp_loss, c->mlp_gpart, c->mlp_lpart,
                     c->mlp_packed, c->sample_count, c->sample_x, c->sample_amin, c->sample_y, c->sample_rel,
                     c->sample_w, c->sample_group, c->sample_node, c->guard_idx, c->guard_part, c->guard,
                     c->rcrit2, c->phi_ext};
    for (void *p : mptrs)
        if (p) cudaFree(p);
    if (c->h_st) cudaFreeHost(c->h_st);
    if (c->h_box) cudaFreeHost(c->h_box);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
}

int alloc_all(hc_ctx *c)
{
    const int64_t n = c->n;
    double **bd[] = {&c->mass, &c->px, &c->py, &c->pz, &c->vx, &c->vy, &c->vz, &c->ax, &c->ay, &c->az, &c->phi};
    for (double **p : bd) HC_TRY(dalloc(c, p, n));
    HC_TRY(dalloc(c, &c->cnt_b, n));
    HC_TRY(dalloc(c, &c->cnt_c, n));
    for (int i = 0; i < 2; i++) {
        HC_TRY(dalloc(c, &c->khi[i], n));
        HC_TRY(dalloc(c, &c->klo[i], n));
        HC_TRY(dalloc(c, &c->kval[i], n));
    }
    HC_TRY(dalloc(c, &c->s_rank, n));
    HC_TRY(dalloc(c, &c->tord, n));
    HC_TRY(dalloc(c, &c->gstart, n));
    HC_TRY(dalloc(c, &c->gcount, n));
    HC_TRY(dalloc(c, &c->leaf_of_sorted, n));
    HC_TRY(dalloc(c, &c->mhi, n));
    HC_TRY(dalloc(c, &c->mlo, n));
    HC_TRY(dalloc(c, &c->midx, n));
    HC_TRY(dalloc(c, &c->mpos, n));
    HC_TRY(dalloc(c, &c->dlcp, n));
    HC_TRY(dalloc(c, &c->ccount, n + 1));
    const int64_t mn = c->maxnode;
    HC_TRY(dalloc(c, &c->pre_info, mn));
    HC_TRY(dalloc(c, &c->pre_a, mn));
    HC_TRY(dalloc(c, &c->bfs_a, mn));
    for (int i = 0; i < 2; i++) {
        HC_TRY(dalloc(c, &c->dkey[i], mn));
        HC_TRY(dalloc(c, &c->dval[i], mn));
    }
    HC_TRY(dalloc(c, &c->pre2bfs, mn));
    HC_TRY(dalloc(c, &c->parent, mn));
    HC_TRY(dalloc(c, &c->lastc, mn));
    HC_TRY(dalloc(c, &c->cperm, mn));
    HC_TRY(dalloc(c, &c->cbins, 520));
    HC_TRY(dalloc(c, &c->gcnt, mn + 1));
    HC_TRY(dalloc(c, &c->goff, mn + 1));
    HC_TRY(dalloc(c, &c->nodeA, mn));
    HC_TRY(dalloc(c, &c->nodeB, mn));
    HC_TRY(dalloc(c, &c->nodeQ, 2 * mn));
    HC_TRY(dalloc(c, &c->nodeC, mn));
    HC_TRY(dalloc(c, &c->nm, mn));
    HC_TRY(dalloc(c, &c->ncx, mn));
    HC_TRY(dalloc(c, &c->ncy, mn));
    HC_TRY(dalloc(c, &c->ncz, mn));
    HC_TRY(dalloc(c, &c->flags, 4 * n + 8));
    const int64_t big = std::max<int64_t>(n, mn);
    HC_TRY(dalloc(c, &c->scan_tmp, hc_scan_scratch_words(big + 1)));
    HC_TRY(dalloc(c, &c->hist, hc_sort_scratch_words(big)));
    HC_TRY(dalloc(c, &c->cand, n));
    HC_TRY(dalloc(c, &c->ncand, 4));
    HC_TRY(dalloc(c, &c->diag_part, 36 * 1024));
    HC_TRY(dalloc(c, &c->st, 2));
    HC_TRY(dalloc(c, &c->mlp_p, hc_mlp_nparams()));
    HC_TRY(dalloc(c, &c->mlp_m, hc_mlp_nparams()));
    HC_TRY(dalloc(c, &c->mlp_v, hc_mlp_nparams()));
    HC_TRY(dalloc(c, &c->mlp_grad, hc_mlp_nparams()));
    HC_TRY(dalloc(c, &c->mlp_loss, 1));
    c->mlp_gcap = 128;
    HC_TRY(dalloc(c, &c->mlp_gpart, (int64_t)c->mlp_gcap * hc_mlp_nparams()));
    HC_TRY(dalloc(c, &c->mlp_lpart, c->mlp_gcap));
    {
        char *pk = nullptr;
        HC_CUDA(cudaMalloc((void **)&pk, sizeof(MlpSmem)));
        c->mlp_packed = (MlpSmem *)pk;
        HC_CUDA(cudaMemset(pk, 0, sizeof(MlpSmem)));
    }
    HC_TRY(dalloc(c, &c->sample_count, 2));
    HC_TRY(dalloc(c, &c->box, 1));
    HC_CUDA(cudaMallocHost((void **)&c->h_st, sizeof(hc_status)));
    HC_CUDA(cudaMallocHost((void **)&c->h_box, sizeof(hc_box)));
    return HC_OK;
}

// Test-point buffers, grown on demand.  Their sort has its own scratch
// (thist): the tree's (hist) is baked into captured graphs and never moves.
// A failed allocation leaves the buffers null and the capacity 0.
int ensure_test_capacity(hc_ctx *c, int64_t nt)
{
    if (nt <= c->tcap) return HC_OK;
    c->tcap = 0;
    void **ptrs[] = {(void **)&c->tx, (void **)&c->ty, (void **)&c->tz, (void **)&c->tax, (void **)&c->tay,
                     (void **)&c->taz, (void **)&c->tphi, (void **)&c->tkhi[0], (void **)&c->tkhi[1],
                     (void **)&c->tklo[0], (void **)&c->tklo[1], (void **)&c->tkval[0], (void **)&c->tkval[1],
                     (void **)&c->thist};
    for (void **p : ptrs) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    double **dd[] = {&c->tx, &c->ty, &c->tz, &c->tax, &c->tay, &c->taz, &c->tphi};
    for (double **p : dd) HC_TRY(dalloc(c, p, nt));
    for (int i = 0; i < 2; i++) {
        HC_TRY(dalloc(c, &c->tkhi[i], nt));
        HC_TRY(dalloc(c, &c->tklo[i], nt));
        HC_TRY(dalloc(c, &c->tkval[i], nt));
    }
    HC_TRY(dalloc(c, &c->thist, hc_sort_scratch_words(nt)));
    c->tcap = nt;
    return HC_OK;
}

void reset_status(hc_ctx *c) { cudaMemsetAsync(c->st, 0, sizeof(hc_status), c->stream); }

// SoA <-> reference AoS layouts
__global__ void k_unpack_phase(const double *phase, int64_t n, double *px, double *py, double *pz, double *vx,
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

__global__ void k_pack3(const double *x, const double *y, const double *z, int64_t n, double *out, int stride,
                        int off)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        out[stride * i + off] = x[i];
        out[stride * i + off + 1] = y[i];
        out[stride * i + off + 2] = z[i];
    }
}

__global__ void k_unpack3(const double *in, int64_t n, double *x, double *y, double *z)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = in[3 * i];
        y[i] = in[3 * i + 1];
        z[i] = in[3 * i + 2];
    }
}

// staging buffer for host <-> device conversions (device side)
struct Staging {
    double *d = nullptr;
    int64_t cap = 0;
};

int staging(hc_ctx *c, Staging &s, int64_t count)
{
    if (count <= s.cap) return HC_OK;
    if (s.d) cudaFree(s.d);
    s.d = nullptr;
    s.cap = 0;
    HC_TRY(dalloc(c, &s.d, count));
    s.cap = count;
    return HC_OK;
}

}  // namespace

struct GraphSlot {
    cudaGraphExec_t exec = nullptr;
    double kick = 0.0;
    int64_t launches = 0;
};

struct hc_ctx_ext : hc_ctx {
    Staging stage;
    Staging stage_acc;            // hc_evaluate_host: previous accelerations
    // 0: build + walk, 1: build + walk with closing kick + diagnostics,
    // 2: build + walk that waits for ev_acc (hc_evaluate_host) before the walk
    GraphSlot graphs[3];
    cudaStream_t xfer = nullptr;  // hc_evaluate_host: the previous accelerations' copy, beside the build
    cudaEvent_t ev_acc = nullptr;
    bool use_graphs = true;
    double *h_diag = nullptr;     // pinned
    double *d_diag = nullptr;
    int64_t *d_idx = nullptr;
    int64_t idx_cap = 0;
    double *d_out = nullptr;
    int64_t out_cap = 0;
};

extern "C" {

int hc_create(hc_ctx **out, int64_t nbody, const hc_params *params)
{
    if (!out || nbody < 1 || !params) return HC_ERR_ARG;
    if (nbody > (1LL << 28)) return HC_ERR_ARG;
    if (!std::isfinite(params->tol) || !std::isfinite(params->eps) || !std::isfinite(params->fcells))
        return HC_ERR_ARG;
    // bodies + cells must stay below 2^30: the radix sort's look-back words
    // carry 30-bit counts
    if ((double)nbody * (1.0 + std::max(params->fcells, 0.0)) >= (double)(1LL << 30)) return HC_ERR_ARG;
    hc_ctx_ext *c = new hc_ctx_ext();   // value-initialised: all pointers null
    c->n = nbody;
    c->prm = *params;
    c->maxcell = (int64_t)(params->fcells * (double)nbody);   // load.c:50
    if (c->maxcell < 1) c->maxcell = 1;
    c->maxnode = nbody + c->maxcell;
    c->mlp_band = 1.0f;
    c->mlp_band_hi = 3.0f;
    c->group_max = HC_GROUP2;
    c->list_depth = 64;
    *out = c;
    // The evaluation's stream has the highest priority and the side stream
    // (the guard's direct sum beside the build) the lowest: when both have
    // blocks waiting for an SM, the build's go first.
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess) {
        c->err = "cudaStreamCreate failed";
        return HC_ERR_CUDA;
    }
    for (auto &e : c->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return HC_ERR_CUDA;
    if (cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        c->err = "cudaStreamCreate / cudaEventCreate failed";
        return HC_ERR_CUDA;
    }
    int r = alloc_all(c);
    if (r != HC_OK) return r;
    HC_CUDA(cudaMalloc((void **)&c->d_diag, 64 * sizeof(double)));
    hc_box b;
    std::memset(&b, 0, sizeof b);
    b.rmin[0] = b.rmin[1] = b.rmin[2] = -2.0;   // code.c:119-120
    b.rsize = 4.0;
    b.first_massive = -1;
    b.chain_lmax = b.chain_lmin = -1;
    HC_CUDA(cudaMemcpy(c->box, &b, sizeof b, cudaMemcpyHostToDevice));
    HC_CUDA(cudaMemset(c->st, 0, 2 * sizeof(hc_status)));
    HC_CUDA(cudaMallocHost((void **)&c->h_diag, 64 * sizeof(double)));
    HC_TRY(hc_guard_setup(c));
    int r2 = hc_tree_setup(c);
    return r2 != HC_OK ? r2 : hc_walk_setup(c);
}

void hc_destroy(hc_ctx *ctx)
{
    if (!ctx) return;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->stage.d) cudaFree(c->stage.d);
    if (c->stage_acc.d) cudaFree(c->stage_acc.d);
    if (c->xfer) {
        cudaStreamSynchronize(c->xfer);
        cudaStreamDestroy(c->xfer);
    }
    if (c->ev_acc) cudaEventDestroy(c->ev_acc);
    if (c->d_diag) cudaFree(c->d_diag);
    if (c->d_idx) cudaFree(c->d_idx);
    if (c->d_out) cudaFree(c->d_out);
    if (c->h_diag) cudaFreeHost(c->h_diag);
    for (auto &g : c->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    free_all(c);
    delete c;
}

const char *hc_last_error(const hc_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int hc_set_params(hc_ctx *c, const hc_params *p)
{
    if (!c || !p) return HC_ERR_ARG;
    if (!std::isfinite(p->tol) || !std::isfinite(p->eps)) {
        c->err = "tol and eps must be finite";
        return HC_ERR_ARG;
    }
    if ((int64_t)(p->fcells * (double)c->n) != c->maxcell) {
        c->err = "fcells is fixed when the context is created (load.c:49-53 allocates the cell pool once)";
        return HC_ERR_ARG;
    }
    c->prm = *p;
    for (auto &g : static_cast<hc_ctx_ext *>(c)->graphs)   // captured graphs bake tol / eps / usequad
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    return HC_OK;
}

int hc_upload(hc_ctx *ctx, const double *mass, const double *phase)
{
    if (!ctx || !mass || !phase) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    const int64_t n = c->n;
    HC_TRY(staging(c, c->stage, 6 * n));
    HC_CUDA(cudaMemcpyAsync(c->mass, mass, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    HC_CUDA(cudaMemcpyAsync(c->stage.d, phase, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, c->stream));
    k_unpack_phase<<<hc_grid(n, 256), 256, 0, c->stream>>>(c->stage.d, n, c->px, c->py, c->pz, c->vx, c->vy, c->vz);
    HC_CUDA(cudaMemsetAsync(c->ax, 0, sizeof(double) * n, c->stream));
    HC_CUDA(cudaMemsetAsync(c->ay, 0, sizeof(double) * n, c->stream));
    HC_CUDA(cudaMemsetAsync(c->az, 0, sizeof(double) * n, c->stream));
    HC_CUDA(cudaMemsetAsync(c->phi, 0, sizeof(double) * n, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    c->have_tree = c->have_forces = false;
    return HC_OK;
}

int hc_set_forces(hc_ctx *ctx, const double *acc, const double *phi)
{
    if (!ctx) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    const int64_t n = c->n;
    if (acc) {
        HC_TRY(staging(c, c->stage, 6 * n));
        HC_CUDA(cudaMemcpyAsync(c->stage.d, acc, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
        k_unpack3<<<hc_grid(n, 256), 256, 0, c->stream>>>(c->stage.d, n, c->ax, c->ay, c->az);
    }
    if (phi) HC_CUDA(cudaMemcpyAsync(c->phi, phi, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int hc_set_box(hc_ctx *c, const double rmin[3], double rsize)
{
    if (!c || !rmin || !(rsize > 0) || !std::isfinite(rsize)) return HC_ERR_ARG;
    for (int k = 0; k < 3; k++)
        if (!std::isfinite(rmin[k])) return HC_ERR_ARG;
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaMemcpy(c->h_box, c->box, sizeof(hc_box), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 3; k++) c->h_box->rmin[k] = rmin[k];
    c->h_box->rsize = rsize;
    HC_CUDA(cudaMemcpy(c->box, c->h_box, sizeof(hc_box), cudaMemcpyHostToDevice));
    c->have_tree = false;
    return HC_OK;
}

int hc_get_box(hc_ctx *c, double rmin[3], double *rsize)
{
    if (!c || !rmin || !rsize) return HC_ERR_ARG;
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaMemcpy(c->h_box, c->box, sizeof(hc_box), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 3; k++) rmin[k] = c->h_box->rmin[k];
    *rsize = c->h_box->rsize;
    return HC_OK;
}

int hc_build_tree(hc_ctx *c)
{
    if (!c) return HC_ERR_ARG;
    c->launches = 0;
    reset_status(c);
    HC_CUDA(cudaEventRecord(c->ev[0], c->stream));
    int r = hc_tree_build(c);
    if (r != HC_OK) {
        check_status(c);
        return r;
    }
    HC_CUDA(cudaEventRecord(c->ev[1], c->stream));
    r = check_status(c);
    if (r != HC_OK) return r;
    HC_CUDA(cudaEventElapsedTime(&c->build_ms, c->ev[0], c->ev[1]));
    c->have_tree = true;
    c->have_forces = false;
    return HC_OK;
}

int hc_tree_summary(hc_ctx *c, hc_tree_info *info)
{
    if (!c || !info) return HC_ERR_ARG;
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaMemcpy(c->h_box, c->box, sizeof(hc_box), cudaMemcpyDeviceToHost));
    info->nbody_massive = c->h_box->nmassive;
    info->ncell = c->h_box->ncell;
    info->max_level = c->h_box->max_depth;
    for (int k = 0; k < 3; k++) info->rmin[k] = c->h_box->rmin[k];
    info->rsize = c->h_box->rsize;
    return HC_OK;
}

int hc_dump_tree(hc_ctx *c, int32_t *level, int32_t *corner, int32_t *count, double *mass, double *cm,
                 double *quad, int32_t *body_parent_level)
{
    if (!c) return HC_ERR_ARG;
    if (!c->have_tree) {
        c->err = "hc_dump_tree: no tree (call hc_build_tree first)";
        return HC_ERR_STATE;
    }
    HC_CUDA(cudaStreamSynchronize(c->stream));
    int r = hc_tree_dump_impl(c, level, corner, count, mass, cm, quad, body_parent_level);
    return r < 0 ? r : HC_OK;
}

int hc_tree_rcrit(hc_ctx *c, int criterion, double theta, double *rcrit2)
{
    if (!c || !rcrit2 || criterion < HC_CRITERION_BH86 || criterion > HC_CRITERION_BARNES || !(theta >= 0.0))
        return HC_ERR_ARG;
    if (!c->have_tree) {
        c->err = "hc_tree_rcrit: no tree (call hc_build_tree first)";
        return HC_ERR_STATE;
    }
    if (!c->rcrit2) HC_TRY(dalloc(c, &c->rcrit2, c->maxnode));
    hc_rcrit_launch(c, criterion - HC_CRITERION_BH86 + 1, theta);
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaMemcpy(c->h_box, c->box, sizeof(hc_box), cudaMemcpyDeviceToHost));
    const int nn = c->h_box->nnode;
    if (nn <= 0) return HC_OK;
    std::vector<int2> C(nn);
    std::vector<float> r(nn);
    HC_CUDA(cudaMemcpy(C.data(), c->nodeC, sizeof(int2) * nn, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(r.data(), c->rcrit2, sizeof(float) * nn, cudaMemcpyDeviceToHost));
    int64_t ci = 0;
    for (int k = 0; k < nn; k++)             // cells in breadth-first order, as hc_dump_tree lists them
        if (C[k].x >= 0) rcrit2[ci++] = (double)r[k];
    return HC_OK;
}

static int forces_self(hc_ctx *c, double kick_dthf, int64_t nstep)
{
    if (!c->have_tree) {
        c->err = "forces requested before hc_build_tree";
        return HC_ERR_STATE;
    }
    reset_status(c);
    HC_CUDA(cudaEventRecord(c->ev[2], c->stream));
    HC_TRY(hc_walk_launch(c, true, c->n, c->tord, c->px, c->py, c->pz, c->ax, c->ay, c->az, c->phi, kick_dthf,
                          nstep));
    HC_CUDA(cudaEventRecord(c->ev[3], c->stream));
    HC_TRY(check_status(c));
    HC_CUDA(cudaEventElapsedTime(&c->walk_ms, c->ev[2], c->ev[3]));
    c->have_forces = true;
    return HC_OK;
}

int hc_forces(hc_ctx *c)
{
    if (!c) return HC_ERR_ARG;
    return forces_self(c, 0.0, 0);
}

int hc_forces_at(hc_ctx *ctx, const double *test_pos, int64_t ntest, double *acc, double *phi)
{
    if (!ctx || ntest < 0 || (ntest > 0 && (!test_pos || !acc || !phi))) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    if (!c->have_tree) {
        c->err = "hc_forces_at before hc_build_tree";
        return HC_ERR_STATE;
    }
    if (ntest == 0) return HC_OK;
    HC_TRY(ensure_test_capacity(c, ntest));
    HC_TRY(staging(c, c->stage, 3 * ntest));
    reset_status(c);
    HC_CUDA(cudaMemcpyAsync(c->stage.d, test_pos, sizeof(double) * 3 * ntest, cudaMemcpyHostToDevice, c->stream));
    k_unpack3<<<hc_grid(ntest, 256), 256, 0, c->stream>>>(c->stage.d, ntest, c->tx, c->ty, c->tz);
    hc_keys_for_points(c, c->tx, c->ty, c->tz, ntest, c->tkhi[0], c->tklo[0], c->tkval[0]);
    int sel = hc_radix_sort_keys(c, c->thist, c->tkhi, c->tklo, c->tkval, ntest, 0, 64, false);
    HC_CUDA(cudaEventRecord(c->ev[2], c->stream));
    HC_TRY(hc_walk_launch(c, false, ntest, c->tkval[sel], c->tx, c->ty, c->tz, c->tax, c->tay, c->taz, c->tphi,
                          0.0, 0));
    HC_CUDA(cudaEventRecord(c->ev[3], c->stream));
    k_pack3<<<hc_grid(ntest, 256), 256, 0, c->stream>>>(c->tax, c->tay, c->taz, ntest, c->stage.d, 3, 0);
    HC_CUDA(cudaMemcpyAsync(acc, c->stage.d, sizeof(double) * 3 * ntest, cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaMemcpyAsync(phi, c->tphi, sizeof(double) * ntest, cudaMemcpyDeviceToHost, c->stream));
    HC_TRY(check_status(c));
    HC_CUDA(cudaEventElapsedTime(&c->walk_ms, c->ev[2], c->ev[3]));
    return HC_OK;
}

int hc_download(hc_ctx *ctx, double *phase, double *acc, double *phi)
{
    if (!ctx) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    const int64_t n = c->n;
    HC_TRY(staging(c, c->stage, 6 * n));
    if (phase) {
        k_pack3<<<hc_grid(n, 256), 256, 0, c->stream>>>(c->px, c->py, c->pz, n, c->stage.d, 6, 0);
        k_pack3<<<hc_grid(n, 256), 256, 0, c->stream>>>(c->vx, c->vy, c->vz, n, c->stage.d, 6, 3);
        HC_CUDA(cudaMemcpyAsync(phase, c->stage.d, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, c->stream));
        HC_CUDA(cudaStreamSynchronize(c->stream));
    }
    if (acc) {
        k_pack3<<<hc_grid(n, 256), 256, 0, c->stream>>>(c->ax, c->ay, c->az, n, c->stage.d, 3, 0);
        HC_CUDA(cudaMemcpyAsync(acc, c->stage.d, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
        HC_CUDA(cudaStreamSynchronize(c->stream));
    }
    if (phi) HC_CUDA(cudaMemcpyAsync(phi, c->phi, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int hc_body_counts(hc_ctx *c, int32_t *n2b, int32_t *nbc)
{
    if (!c) return HC_ERR_ARG;
    if (!c->prm.count_per_body || !c->have_forces) {
        c->err = "hc_body_counts: needs count_per_body and a completed hc_forces";
        return HC_ERR_STATE;
    }
    if (n2b) HC_CUDA(cudaMemcpyAsync(n2b, c->cnt_b, sizeof(int32_t) * c->n, cudaMemcpyDeviceToHost, c->stream));
    if (nbc) HC_CUDA(cudaMemcpyAsync(nbc, c->cnt_c, sizeof(int32_t) * c->n, cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    return HC_OK;
}

static void unpack_diag(hc_ctx_ext *c, const double *h, hc_diag *d)
{
    std::memset(d, 0, sizeof *d);
    d->etot[1] = h[0];
    d->etot[2] = h[1];
    d->etot[0] = d->etot[1] + d->etot[2];
    for (int k = 0; k < 9; k++) {
        d->keten[k] = h[2 + k];
        d->peten[k] = h[11 + k];
    }
    for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++) d->amten[3 * j + k] = h[20 + 3 * j + k] - h[20 + 3 * k + j];
    d->mtot = h[35];
    for (int k = 0; k < 3; k++) {
        d->cmphase[k] = h[29 + k] / d->mtot;
        d->cmphase[3 + k] = h[32 + k] / d->mtot;
    }
    d->n2b = (int64_t)c->h_st->n2b;
    d->nbc = (int64_t)c->h_st->nbc;
    d->nfcalc = c->n;
}

static int fill_diag(hc_ctx_ext *c, hc_diag *d)
{
    hc_diag_launch(c, c->d_diag);
    HC_CUDA(cudaMemcpyAsync(c->h_diag, c->d_diag, 36 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    unpack_diag(c, c->h_diag, d);
    return HC_OK;
}

// One force evaluation (build + walk of every body, optional closing kick
// and diagnostics) enqueued without host synchronisation: the body of both
// the captured graphs and the direct path.
static int enqueue_evaluation(hc_ctx_ext *c, double kick_dthf, int64_t nstep, bool with_diag, bool capturing,
                              cudaEvent_t before_walk = nullptr)
{
    // inside stream capture an event record must be an explicit graph node
    const unsigned rflags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    HC_CUDA(cudaMemsetAsync(c->st, 0, sizeof(hc_status), c->stream));
    HC_CUDA(cudaEventRecordWithFlags(c->ev[0], c->stream, rflags));
    const bool guard = c->guard_n > 0 && c->criterion != HC_CRITERION_BODY;
    if (guard) {
        // the guard's direct sum on the side stream, alongside the first build
        // steps (they leave most SMs idle); joined before the upward pass
        HC_CUDA(cudaEventRecord(c->ev_fork, c->stream));
        HC_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
        hc_guard_direct_launch(c, c->side);
        HC_CUDA(cudaEventRecord(c->ev_join, c->side));
        c->join_pending = true;
    }
    const int rb = hc_tree_build(c);
    if (c->join_pending) {                    // the build left before the upward pass
        c->join_pending = false;
        HC_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    }
    if (rb != HC_OK) return rb;
    if (c->criterion >= HC_CRITERION_BH86) hc_rcrit_launch(c, c->criterion - HC_CRITERION_BH86 + 1, c->group_theta);
    // inputs the walk alone reads (previous accelerations) may arrive beside the build
    if (before_walk)
        HC_CUDA(cudaStreamWaitEvent(c->stream, before_walk, capturing ? cudaEventWaitExternal : 0));
    HC_CUDA(cudaEventRecordWithFlags(c->ev[1], c->stream, rflags));
    HC_CUDA(cudaEventRecordWithFlags(c->ev[2], c->stream, rflags));
    HC_TRY(hc_walk_launch(c, true, c->n, c->tord, c->px, c->py, c->pz, c->ax, c->ay, c->az, c->phi, kick_dthf,
                          nstep));
    if (guard) {
        // compare with the walk's forces; on failure the per-body rule redoes the walk
        hc_guard_check_launch(c);
        HC_TRY(hc_walk_launch(c, true, c->n, c->tord, c->px, c->py, c->pz, c->ax, c->ay, c->az, c->phi, kick_dthf,
                              nstep, &c->guard->flag, true));
    }
    if (c->extpot) hc_extpot_launch(c, kick_dthf, nstep);
    HC_CUDA(cudaEventRecordWithFlags(c->ev[3], c->stream, rflags));
    if (with_diag) {
        hc_diag_launch(c, c->d_diag);
        HC_CUDA(cudaMemcpyAsync(c->h_diag, c->d_diag, 36 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    HC_CUDA(cudaMemcpyAsync(c->h_st, c->st, sizeof(hc_status), cudaMemcpyDeviceToHost, c->stream));
    return HC_OK;
}

static int finish_evaluation(hc_ctx_ext *c)
{
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    int r = check_status(c);
    if (r != HC_OK) return r;
    HC_CUDA(cudaEventElapsedTime(&c->build_ms, c->ev[0], c->ev[1]));
    HC_CUDA(cudaEventElapsedTime(&c->walk_ms, c->ev[2], c->ev[3]));
    c->have_tree = c->have_forces = true;
    return HC_OK;
}

// Run an evaluation through a captured CUDA graph (captured on first use,
// replayed afterwards), or directly when graphs are off.
static int launch_evaluation(hc_ctx_ext *c, int slot, double kick_dthf, int64_t nstep, bool with_diag)
{
    cudaEvent_t before_walk = slot == 2 ? c->ev_acc : nullptr;
    if (!c->use_graphs) {
        c->launches = 0;
        return enqueue_evaluation(c, kick_dthf, nstep, with_diag, false, before_walk);
    }
    GraphSlot &g = c->graphs[slot];
    if (!g.exec || g.kick != kick_dthf) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        cudaGraph_t graph = nullptr;
        HC_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        c->launches = 0;
        int r = enqueue_evaluation(c, kick_dthf, nstep, with_diag, true, before_walk);
        cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        if (r != HC_OK) {
            if (graph) cudaGraphDestroy(graph);
            return r;
        }
        if (e != cudaSuccess) {
            c->err = std::string("stream capture: ") + cudaGetErrorString(e);
            return HC_ERR_CUDA;
        }
        // kernel nodes keep the priorities of the streams they were captured on
        e = cudaGraphInstantiate(&g.exec, graph, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            g.exec = nullptr;
            c->err = std::string("graph instantiate: ") + cudaGetErrorString(e);
            return HC_ERR_CUDA;
        }
        g.kick = kick_dthf;
        g.launches = c->launches;
    }
    HC_CUDA(cudaGraphLaunch(g.exec, c->stream));
    c->launches = g.launches;
    return HC_OK;
}

static int run_evaluation(hc_ctx_ext *c, int slot, double kick_dthf, int64_t nstep, bool with_diag)
{
    HC_TRY(launch_evaluation(c, slot, kick_dthf, nstep, with_diag));
    return finish_evaluation(c);
}

int hc_diagnostics(hc_ctx *ctx, hc_diag *diag)
{
    if (!ctx || !diag) return HC_ERR_ARG;
    return fill_diag(static_cast<hc_ctx_ext *>(ctx), diag);
}

int hc_evaluate(hc_ctx *ctx)
{
    if (!ctx) return HC_ERR_ARG;
    return run_evaluation(static_cast<hc_ctx_ext *>(ctx), 0, 0.0, 0, false);
}

int hc_evaluate_host(hc_ctx *ctx, const double *pos, const double *prev_acc, double *acc, double *phi)
{
    if (!ctx || !pos) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    const int64_t n = c->n;
    if (!c->xfer) {
        if (cudaStreamCreateWithFlags(&c->xfer, cudaStreamNonBlocking) != cudaSuccess) {
            c->xfer = nullptr;
            c->err = "cudaStreamCreate failed";
            return HC_ERR_CUDA;
        }
        HC_CUDA(cudaEventCreateWithFlags(&c->ev_acc, cudaEventDisableTiming));
    }
    HC_TRY(staging(c, c->stage, 3 * n));
    if (prev_acc) HC_TRY(staging(c, c->stage_acc, 3 * n));
    // positions: the build needs them first
    HC_CUDA(cudaMemcpyAsync(c->stage.d, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    k_unpack3<<<hc_grid(n, 256), 256, 0, c->stream>>>(c->stage.d, n, c->px, c->py, c->pz);
    // previous accelerations (read by the error and learned criteria in the
    // walk only): copied on their own stream while the tree is built; the walk
    // waits for ev_acc.  The previous call ended synchronised, so nothing
    // still reads the acceleration arrays.
    if (prev_acc) {
        HC_CUDA(cudaMemcpyAsync(c->stage_acc.d, prev_acc, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->xfer));
        k_unpack3<<<hc_grid(n, 256), 256, 0, c->xfer>>>(c->stage_acc.d, n, c->ax, c->ay, c->az);
        HC_CUDA(cudaEventRecord(c->ev_acc, c->xfer));
    }
    c->have_tree = c->have_forces = false;
    HC_TRY(launch_evaluation(c, 2, 0.0, 0, false));
    // results out behind the evaluation, one synchronisation for all
    if (acc) {
        k_pack3<<<hc_grid(n, 256), 256, 0, c->stream>>>(c->ax, c->ay, c->az, n, c->stage.d, 3, 0);
        HC_CUDA(cudaMemcpyAsync(acc, c->stage.d, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    }
    if (phi) HC_CUDA(cudaMemcpyAsync(phi, c->phi, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    return finish_evaluation(c);       // synchronises, then checks the device status
}

int hc_set_graphs(hc_ctx *ctx, int on)
{
    if (!ctx) return HC_ERR_ARG;
    static_cast<hc_ctx_ext *>(ctx)->use_graphs = on != 0;
    return HC_OK;
}

int hc_step(hc_ctx *ctx, double dt, int64_t nstep, hc_diag *diag, double *snap_phase, double *snap_acc,
            double *snap_phi)
{
    if (!ctx || !(dt > 0)) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    if (nstep > 0) {
        HC_TRY(run_evaluation(c, 1, 0.5 * dt, 1, true));   // graph: kick active
    } else {
        c->launches = 0;                                   // first step: no kick, not captured
        HC_TRY(enqueue_evaluation(c, 0.0, 0, true, false));
        HC_TRY(finish_evaluation(c));
    }
    if (diag) unpack_diag(c, c->h_diag, diag);
    if (snap_phase || snap_acc || snap_phi) HC_TRY(hc_download(c, snap_phase, snap_acc, snap_phi));
    hc_kick_drift(c, dt);
    c->launches++;
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    c->have_tree = false;
    return HC_OK;
}

int hc_direct_sample(hc_ctx *ctx, const int64_t *index, int64_t ns, double *acc, double *phi)
{
    if (!ctx || ns < 0 || (ns > 0 && (!index || !acc || !phi))) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    for (int64_t i = 0; i < ns; i++)
        if (index[i] < 0 || index[i] >= c->n) {
            c->err = "hc_direct_sample: index out of range";
            return HC_ERR_ARG;
        }
    if (ns == 0) return HC_OK;
    if (ns > c->idx_cap) {
        if (c->d_idx) cudaFree(c->d_idx);
        if (c->d_out) cudaFree(c->d_out);
        c->d_idx = nullptr;
        c->d_out = nullptr;
        c->idx_cap = 0;
        HC_TRY(dalloc(c, &c->d_idx, ns));
        HC_TRY(dalloc(c, &c->d_out, 4 * ns));
        c->idx_cap = ns;
    }
    HC_CUDA(cudaMemcpyAsync(c->d_idx, index, sizeof(int64_t) * ns, cudaMemcpyHostToDevice, c->stream));
    hc_direct_launch(c, c->d_idx, ns, c->d_out, c->d_out + 3 * ns);
    HC_CUDA(cudaMemcpyAsync(acc, c->d_out, sizeof(double) * 3 * ns, cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaMemcpyAsync(phi, c->d_out + 3 * ns, sizeof(double) * ns, cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int hc_set_criterion(hc_ctx *ctx, int criterion, double theta)
{
    if (!ctx || criterion < HC_CRITERION_BODY || criterion > HC_CRITERION_BARNES) return HC_ERR_ARG;
    if (criterion != HC_CRITERION_BODY && !(theta >= 0.0)) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    if (criterion >= HC_CRITERION_BH86 && !c->rcrit2) HC_TRY(dalloc(c, &c->rcrit2, c->maxnode));
    c->criterion = criterion;
    c->group_theta = theta;
    for (auto &g : c->graphs)        // captured graphs bake the walk variant
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    return HC_OK;
}

int hc_set_guard(hc_ctx *ctx, int64_t nsample, double rms_max, uint64_t seed)
{
    if (!ctx || nsample < 0 || nsample > HC_GUARD_MAX_SAMPLE) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    if (nsample > c->n || (nsample > 0 && !(rms_max > 0.0))) {
        c->err = "hc_set_guard: need 0 <= nsample <= nbody and rms_max > 0";
        return HC_ERR_ARG;
    }
    HC_CUDA(cudaStreamSynchronize(c->stream));
    if (c->guard_idx) cudaFree(c->guard_idx);
    if (c->guard_part) cudaFree(c->guard_part);
    c->guard_idx = nullptr;
    c->guard_part = nullptr;
    c->guard_n = 0;
    for (auto &g : c->graphs)        // captured graphs bake the guard nodes
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    if (nsample == 0) return HC_OK;
    // seeded uniform sample without replacement (Floyd's algorithm), ascending
    std::vector<int64_t> pick;
    {
        std::unordered_set<int64_t> seen;
        uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;
        auto next = [&st]() {
            st += 0x9E3779B97F4A7C15ULL;            // splitmix64
            uint64_t z = st;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
            return z ^ (z >> 31);
        };
        for (int64_t j = c->n - nsample; j < c->n; j++) {
            const int64_t t = (int64_t)(next() % (uint64_t)(j + 1));
            if (seen.insert(t).second) pick.push_back(t);
            else {
                seen.insert(j);
                pick.push_back(j);
            }
        }
        std::sort(pick.begin(), pick.end());
    }
    if (!c->guard) {
        HC_TRY(dalloc(c, &c->guard, 1));
        HC_CUDA(cudaMemset(c->guard, 0, sizeof(hc_guard_state)));
    }
    const int slices = hc_guard_slices(c);
    if (slices <= 0) return HC_ERR_CUDA;
    HC_TRY(dalloc(c, &c->guard_idx, nsample));
    HC_TRY(dalloc(c, &c->guard_part, (int64_t)slices * nsample + (nsample + 1) / 2));   // + rel2[nsample] (FP64)
    HC_CUDA(cudaMemcpy(c->guard_idx, pick.data(), sizeof(int64_t) * nsample, cudaMemcpyHostToDevice));
    c->guard_slices = slices;
    c->guard_rms_max = rms_max;
    c->guard_n = nsample;
    return HC_OK;
}

int hc_guard_stats(hc_ctx *ctx, int64_t *checks, int64_t *trips, double *last_rms)
{
    if (!ctx) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    hc_guard_state g = {};
    if (c->guard) {
        HC_CUDA(cudaStreamSynchronize(c->stream));
        HC_CUDA(cudaMemcpy(&g, c->guard, sizeof g, cudaMemcpyDeviceToHost));
    }
    if (checks) *checks = (int64_t)g.checks;
    if (trips) *trips = (int64_t)g.trips;
    if (last_rms) *last_rms = g.last_rms;
    return HC_OK;
}

static void drop_graphs(hc_ctx_ext *c)
{
    for (auto &g : c->graphs)
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
}

int hc_set_extpot(hc_ctx *ctx, const char *name, const double *par, int npar)
{
    if (!ctx || npar < 0 || (npar > 0 && !par)) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    const std::string nm = name ? name : "";
    int kind = 0;
    double p[4] = {1.0, 1.0, 1.0, 1.0};          // defaults of the plug-ins
    if (nm.empty() || nm == "null") kind = 0;
    else if (nm == "plummer") kind = HC_EXTPOT_PLUMMER;
    else if (nm == "hernquist") kind = HC_EXTPOT_HERNQUIST;
    else if (nm == "miyamoto") {
        kind = HC_EXTPOT_MIYAMOTO;
        p[1] = 0.0;                              // miyamoto.c: a = 0, b = 1
    } else if (nm == "log") {
        kind = HC_EXTPOT_LOG;
    } else {
        c->err = "hc_set_extpot: unknown potential '" + nm + "' (plummer, hernquist, miyamoto, log)";
        return HC_ERR_ARG;
    }
    if (npar > 0 && par[0] != 0.0) {
        c->err = "hc_set_extpot: a rotating frame (pattern speed != 0) is not supported";
        return HC_ERR_ARG;
    }
    const int nmax = kind == HC_EXTPOT_LOG ? 5 : (kind == HC_EXTPOT_MIYAMOTO ? 4 : 3);
    if (kind && npar > nmax) {
        c->err = "hc_set_extpot: too many parameters for " + nm;
        return HC_ERR_ARG;
    }
    for (int k = 1; k < npar; k++) p[k - 1] = par[k];
    if (kind == HC_EXTPOT_LOG && npar <= 4) p[3] = p[2];      // log.c: r defaults to q
    if (kind && !c->phi_ext) HC_TRY(dalloc(c, &c->phi_ext, c->n));
    c->extpot = kind;
    for (int k = 0; k < 4; k++) c->extpot_par[k] = p[k];
    drop_graphs(c);
    return HC_OK;
}

int hc_set_tuning(hc_ctx *ctx, const hc_tuning *t)
{
    if (!ctx || !t) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    if (t->group_max < 1 || t->group_max > HC_GROUP2 || t->list_depth < 32 || t->list_depth > 64 ||
        (t->grouping != HC_GROUPS_CONSECUTIVE && t->grouping != HC_GROUPS_TREE)) {
        c->err = "hc_set_tuning: group_max 1..64, list_depth 32..64, grouping HC_GROUPS_*";
        return HC_ERR_ARG;
    }
    c->group_max = t->group_max;
    c->list_depth = t->list_depth;
    c->group_kind = t->grouping;
    drop_graphs(c);
    return HC_OK;
}

int hc_get_tuning(hc_ctx *ctx, hc_tuning *t)
{
    if (!ctx || !t) return HC_ERR_ARG;
    t->group_max = ctx->group_max;
    t->list_depth = ctx->list_depth;
    t->grouping = ctx->group_kind;
    t->ms = 0.0;
    return HC_OK;
}

int hc_autotune(hc_ctx *ctx, hc_tuning *best)
{
    if (!ctx) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    hc_tuning keep;
    hc_get_tuning(ctx, &keep);
    std::vector<hc_tuning> cand;
    // the per-body rule walks groups of up to 32 bodies, the group criteria up to 64
    const bool body = c->criterion == HC_CRITERION_BODY;
    const int gms_body[] = {16, 24, 32}, gms_group[] = {HC_GROUP2 / 2, 3 * HC_GROUP2 / 4, HC_GROUP2}, lds[] = {32, 48, 64};
    for (int gm : body ? gms_body : gms_group)
        for (int ld : lds) cand.push_back(hc_tuning{gm, ld, HC_GROUPS_TREE, 0.0});
    if (c->criterion == HC_CRITERION_BODY)      // the other criteria always walk tree groups
        for (int ld : lds) cand.push_back(hc_tuning{HC_GROUP, ld, HC_GROUPS_CONSECUTIVE, 0.0});
    hc_tuning win = keep;
    win.ms = 1e300;
    for (hc_tuning &t : cand) {
        double ms = 1e300;
        int r = hc_set_tuning(ctx, &t);
        for (int rep = 0; rep < 3 && r == HC_OK; rep++) {
            r = run_evaluation(c, 0, 0.0, 0, false);
            ms = std::min(ms, (double)c->build_ms + (double)c->walk_ms);
        }
        if (r != HC_OK) {                  // keep the caller's tuning and the error message
            const std::string err = c->err;
            hc_set_tuning(ctx, &keep);
            c->err = err;
            return r;
        }
        t.ms = ms;
        if (ms < win.ms) win = t;
    }
    HC_TRY(hc_set_tuning(ctx, &win));
    if (best) *best = win;
    return HC_OK;
}

int hc_set_grouping(hc_ctx *ctx, int kind)
{
    if (!ctx || (kind != HC_GROUPS_CONSECUTIVE && kind != HC_GROUPS_TREE)) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    c->group_kind = kind;
    for (auto &g : c->graphs)
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    return HC_OK;
}


// ---------------------------------------------------------------- learned criterion

static int ensure_samples(hc_ctx *c, int64_t cap)
{
    if (cap <= c->sample_capacity) return HC_OK;
    c->sample_capacity = 0;          // a failed allocation leaves the buffers null
    void **ptrs[] = {(void **)&c->sample_x, (void **)&c->sample_amin, (void **)&c->sample_y,
                     (void **)&c->sample_rel, (void **)&c->sample_w, (void **)&c->sample_group,
                     (void **)&c->sample_node};
    for (void **p : ptrs) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    HC_TRY(dalloc(c, &c->sample_x, 12 * cap));
    HC_TRY(dalloc(c, &c->sample_amin, cap));
    HC_TRY(dalloc(c, &c->sample_y, cap));
    HC_TRY(dalloc(c, &c->sample_rel, cap));
    HC_TRY(dalloc(c, &c->sample_w, cap));
    HC_TRY(dalloc(c, &c->sample_group, cap));
    HC_TRY(dalloc(c, &c->sample_node, cap));
    c->sample_capacity = (int)cap;
    return HC_OK;
}

int hc_learn_nparams(void) { return hc_mlp_nparams(); }

int hc_learn_set_params(hc_ctx *c, const float *p, int count)
{
    if (!c || !p || count != hc_mlp_nparams()) return HC_ERR_ARG;
    HC_CUDA(cudaMemcpyAsync(c->mlp_p, p, sizeof(float) * count, cudaMemcpyHostToDevice, c->stream));
    HC_CUDA(cudaMemsetAsync(c->mlp_m, 0, sizeof(float) * count, c->stream));
    HC_CUDA(cudaMemsetAsync(c->mlp_v, 0, sizeof(float) * count, c->stream));
    c->mlp_step = 0;
    HC_TRY(hc_mlp_pack(c));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int hc_learn_get_params(hc_ctx *c, float *p, int count)
{
    if (!c || !p || count != hc_mlp_nparams()) return HC_ERR_ARG;
    HC_CUDA(cudaMemcpyAsync(p, c->mlp_p, sizeof(float) * count, cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    return HC_OK;
}

int hc_learn_init(hc_ctx *c, uint64_t seed)
{
    if (!c) return HC_ERR_ARG;
    const int np = hc_mlp_nparams();
    std::vector<float> p(np, 0.f);
    uint64_t st = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto uni = [&]() {               // uniform in (-1, 1) from a 64-bit LCG
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        return ((double)(st >> 11) / (double)(1ULL << 53)) * 2.0 - 1.0;
    };
    const int H = 64, I = 12;
    const double a1 = std::sqrt(6.0 / (I + H)), a2 = std::sqrt(6.0 / (H + H)), a3 = std::sqrt(6.0 / (H + 1));
    int o = 0;
    for (int i = 0; i < H * I; i++) p[o++] = (float)(a1 * uni());
    o += H;
    for (int i = 0; i < H * H; i++) p[o++] = (float)(a2 * uni());
    o += H;
    for (int i = 0; i < H; i++) p[o++] = (float)(a3 * uni());
    return hc_learn_set_params(c, p.data(), np);
}

int hc_learn_infer(hc_ctx *ctx, const float *x, int64_t n, float *logits)
{
    if (!ctx || n < 0 || (n > 0 && (!x || !logits))) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    if (n == 0) return HC_OK;
    HC_TRY(staging(c, c->stage, (13 * n + 1) / 2 + 1));
    float *dx = (float *)c->stage.d, *dl = dx + 12 * n;
    HC_CUDA(cudaMemcpyAsync(dx, x, sizeof(float) * 12 * n, cudaMemcpyHostToDevice, c->stream));
    HC_TRY(hc_mlp_infer_impl(c, dx, n, dl));
    HC_CUDA(cudaMemcpyAsync(logits, dl, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int hc_learn_gradient(hc_ctx *ctx, const float *x, const float *y, const float *w, int64_t n, float *grad,
                      float *loss)
{
    if (!ctx || n <= 0 || !x || !y || !grad) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    if (n > (int64_t)c->mlp_gcap * 64) return HC_ERR_ARG;
    HC_TRY(staging(c, c->stage, (14 * n + 1) / 2 + 1));
    float *dx = (float *)c->stage.d, *dy = dx + 12 * n, *dw = dy + n;
    HC_CUDA(cudaMemcpyAsync(dx, x, sizeof(float) * 12 * n, cudaMemcpyHostToDevice, c->stream));
    HC_CUDA(cudaMemcpyAsync(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
    double wsum = (double)n;
    if (w) {
        HC_CUDA(cudaMemcpyAsync(dw, w, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
        wsum = 0;
        for (int64_t i = 0; i < n; i++) wsum += w[i];
    }
    HC_TRY(hc_mlp_grad_impl(c, dx, dy, w ? dw : nullptr, n, (float)(1.0 / wsum), c->mlp_grad, c->mlp_loss));
    HC_CUDA(cudaMemcpyAsync(grad, c->mlp_grad, sizeof(float) * hc_mlp_nparams(), cudaMemcpyDeviceToHost,
                            c->stream));
    if (loss) HC_CUDA(cudaMemcpyAsync(loss, c->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int hc_learn_relabel(hc_ctx *c, double thr)
{
    if (!c) return HC_ERR_ARG;
    HC_TRY(hc_relabel_impl(c, (float)thr));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    return HC_OK;
}

int hc_learn_set_band(hc_ctx *ctx, double lo, double hi)
{
    if (!ctx || !(lo >= 0) || !(hi >= 0)) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    c->mlp_band = (float)lo;
    c->mlp_band_hi = (float)hi;
    for (auto &g : c->graphs)
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    return HC_OK;
}

int hc_learn_set_threshold(hc_ctx *ctx, double t)
{
    if (!ctx) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    c->mlp_threshold = (float)t;
    for (auto &g : c->graphs)
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    return HC_OK;
}

int hc_learn_collect(hc_ctx *ctx, double theta, int64_t target, int64_t *nsamples)
{
    if (!ctx || !(theta > 0) || target <= 0) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    HC_TRY(ensure_samples(c, target + target / 4 + 1024));
    HC_TRY(ensure_test_capacity(c, c->n));      // label walk results go to scratch, not to the state
    const int crit = c->criterion;
    const double th = c->group_theta;
    c->criterion = HC_CRITERION_LEARNED;
    c->group_theta = theta;
    c->collect = 1;
    // tree of the current positions
    HC_CUDA(cudaMemsetAsync(c->st, 0, sizeof(hc_status), c->stream));
    int r = hc_tree_build(c);
    if (r == HC_OK) r = check_status(c);
    int64_t counts[2] = {0, 0};
    for (int pass = 0; pass < 2 && r == HC_OK; pass++) {
        // pass 0 counts the band candidates, pass 1 keeps ~target of them
        c->collect_cap = pass == 0 ? 0 : c->sample_capacity;
        double frac = pass == 0 ? 1.0 : std::min(1.0, (double)target / std::max<int64_t>(1, counts[0]));
        c->keep24 = (unsigned)std::min(16777216.0, frac * 16777216.0);
        HC_CUDA(cudaMemsetAsync(c->sample_count, 0, sizeof(int), c->stream));
        HC_CUDA(cudaMemsetAsync(c->st, 0, sizeof(hc_status), c->stream));
        r = hc_walk_launch(c, true, c->n, c->tord, c->px, c->py, c->pz, c->tax, c->tay, c->taz, c->tphi, 0.0, 0);
        int cnt = 0;
        if (r == HC_OK) HC_CUDA(cudaMemcpyAsync(&cnt, c->sample_count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        if (r == HC_OK) r = check_status(c);
        counts[pass] = cnt;
    }
    c->collect = 0;
    c->criterion = crit;
    c->group_theta = th;
    if (r != HC_OK) return r;
    const int ns = (int)std::min<int64_t>(counts[1], c->sample_capacity);
    HC_TRY(hc_label_launch(c, ns, (float)theta));
    std::vector<float> ones(ns > 0 ? ns : 1, 1.0f);
    if (ns > 0) HC_CUDA(cudaMemcpyAsync(c->sample_w, ones.data(), sizeof(float) * ns, cudaMemcpyHostToDevice, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    c->nsample = ns;
    c->band_total = counts[0];
    if (nsamples) *nsamples = ns;
    return HC_OK;
}

int hc_learn_samples(hc_ctx *ctx, float *x, float *y, float *rel, int64_t cap, int64_t *n)
{
    if (!ctx || !n) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    const int64_t k = std::min<int64_t>(cap, c->nsample);
    if (k > 0) {
        if (x) HC_CUDA(cudaMemcpyAsync(x, c->sample_x, sizeof(float) * 12 * k, cudaMemcpyDeviceToHost, c->stream));
        if (y) HC_CUDA(cudaMemcpyAsync(y, c->sample_y, sizeof(float) * k, cudaMemcpyDeviceToHost, c->stream));
        if (rel) HC_CUDA(cudaMemcpyAsync(rel, c->sample_rel, sizeof(float) * k, cudaMemcpyDeviceToHost, c->stream));
        HC_CUDA(cudaStreamSynchronize(c->stream));
    }
    *n = c->nsample;
    return HC_OK;
}

int hc_learn_load_samples(hc_ctx *ctx, const float *x, const float *y, const float *w, int64_t n)
{
    if (!ctx || n <= 0 || !x || !y) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    HC_TRY(ensure_samples(c, n));
    HC_CUDA(cudaMemcpyAsync(c->sample_x, x, sizeof(float) * 12 * n, cudaMemcpyHostToDevice, c->stream));
    HC_CUDA(cudaMemcpyAsync(c->sample_y, y, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
    std::vector<float> ones;
    if (!w) {
        ones.assign(n, 1.0f);
        w = ones.data();
    }
    HC_CUDA(cudaMemcpyAsync(c->sample_w, w, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    c->nsample = (int)n;
    return HC_OK;
}

__global__ void k_gather_samples(const int *perm, int n, const float *x, const float *y, const float *w, float *ox,
                                 float *oy, float *ow)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int j = perm[i];
        for (int k = 0; k < 12; k++) ox[(int64_t)i * 12 + k] = x[(int64_t)j * 12 + k];
        oy[i] = y[j];
        ow[i] = w[j];
    }
}

int hc_learn_train(hc_ctx *ctx, int epochs, int batch, double lr, uint64_t seed, double *loss)
{
    if (!ctx || epochs < 1 || batch < 64 || !(lr > 0)) return HC_ERR_ARG;
    hc_ctx_ext *c = static_cast<hc_ctx_ext *>(ctx);
    const int n = c->nsample;
    if (n < 64) {
        c->err = "hc_learn_train: fewer than 64 samples";
        return HC_ERR_STATE;
    }
    batch = std::min(batch, c->mlp_gcap * 64);
    // shuffle once into the staging area (the samples are reused every epoch in this order)
    HC_TRY(staging(c, c->stage, (int64_t)n * 8 + 8));
    float *sx = (float *)c->stage.d, *sy = sx + 12 * (int64_t)n, *sw = sy + n;
    int *dperm = (int *)(sw + n);
    std::vector<int> perm(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    uint64_t st = seed * 2862933555777941757ULL + 3037000493ULL;
    for (int i = n - 1; i > 0; i--) {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        const int j = (int)((st >> 33) % (uint64_t)(i + 1));
        std::swap(perm[i], perm[j]);
    }
    HC_CUDA(cudaMemcpyAsync(dperm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
    k_gather_samples<<<hc_grid(n, 256), 256, 0, c->stream>>>(dperm, n, c->sample_x, c->sample_y, c->sample_w, sx, sy, sw);
    double last = 0;
    std::vector<float> wv(n);
    HC_CUDA(cudaMemcpyAsync(wv.data(), sw, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    for (int e = 0; e < epochs; e++) {
        double esum = 0, wtot = 0;
        for (int b0 = 0; b0 + 64 <= n; b0 += batch) {
            const int nb = std::min(batch, n - b0);
            double ws = 0;
            for (int i = 0; i < nb; i++) ws += wv[b0 + i];
            HC_TRY(hc_mlp_grad_impl(c, sx + 12 * (int64_t)b0, sy + b0, sw + b0, nb, (float)(1.0 / ws), c->mlp_grad,
                                    c->mlp_loss));
            c->mlp_step++;
            HC_TRY(hc_mlp_adam_impl(c, c->mlp_grad, (float)lr, c->mlp_step));
            float l = 0;
            if (b0 + batch >= n - 63 || (b0 / batch) % 16 == 0) {
                HC_CUDA(cudaMemcpyAsync(&l, c->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
                HC_CUDA(cudaStreamSynchronize(c->stream));
                esum += l;
                wtot += ws;
            }
        }
        last = wtot > 0 ? esum / wtot : 0;
    }
    HC_TRY(hc_mlp_pack(c));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    for (auto &g : c->graphs)
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    if (loss) *loss = last;
    return HC_OK;
}

int hc_walk_statistics(hc_ctx *c, hc_walk_stats *o)
{
    if (!c || !o) return HC_ERR_ARG;
    HC_CUDA(cudaMemcpyAsync(c->h_st, c->st, sizeof(hc_status), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    o->candidates = (int64_t)c->h_st->ncand;
    o->mixed = (int64_t)c->h_st->nmixed;
    o->entries_body = (int64_t)c->h_st->nentry_b;
    o->entries_cell = (int64_t)c->h_st->nentry_c;
    o->borderline = c->h_st->nborder;
    o->max_stack = c->h_st->max_stack;
    o->network = (int64_t)c->h_st->nmlp;
    o->network_rounds = (int64_t)c->h_st->nmlp_rounds;
    for (int i = 0; i < 33; i++) o->mask_hist[i] = (int64_t)c->h_st->mask_hist[i];
    return HC_OK;
}

int hc_timer_start(hc_ctx *c)
{
    if (!c) return HC_ERR_ARG;
    HC_CUDA(cudaEventRecord(c->ev[4], c->stream));
    return HC_OK;
}

int hc_timer_stop(hc_ctx *c, double *ms)
{
    if (!c || !ms) return HC_ERR_ARG;
    HC_CUDA(cudaEventRecord(c->ev[5], c->stream));
    HC_CUDA(cudaEventSynchronize(c->ev[5]));
    float f = 0.f;
    HC_CUDA(cudaEventElapsedTime(&f, c->ev[4], c->ev[5]));
    *ms = f;
    return HC_OK;
}

int hc_fp32_peak(hc_ctx *c, double *tflops)
{
    if (!c || !tflops) return HC_ERR_ARG;
    return hc_fma_peak_impl(c, tflops);
}

int hc_last_timing(hc_ctx *c, double *build_ms, double *walk_ms, int64_t *launches)
{
    if (!c) return HC_ERR_ARG;
    if (build_ms) *build_ms = c->build_ms;
    if (walk_ms) *walk_ms = c->walk_ms;
    if (launches) *launches = c->launches;
    return HC_OK;
}

}  // extern "C"
