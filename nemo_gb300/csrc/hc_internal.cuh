// hc_internal.cuh -- shared definitions of the GB300 hackcode1 library.
//
// Data layout in HBM (one context = one system of nbody bodies):
//   bodies, original order, FP64 SoA: mass, pos[3], vel[3], acc[3], phi
//   keys, sorted order: 63-bit high key (top 21 bits per axis, Morton
//     interleaved, x most significant) + 27-bit low key + original index
//   tree nodes (bodies and cells) in breadth-first order, children of a
//     cell contiguous and in subindex order 0..7 (load.c:162-177):
//       nodeA float4 (cm_hi.xyz, mass)   nodeB float4 (cm_lo.xyz, size^2)
//       nodeC int2   (first child | -1-body slot, nchild | depth<<8)
//       nodeQ 2 x float4 (Qxx Qxy Qxz Qyy | Qyz Qzz 0 0)
//       FP64 mass / cm / quad per node for the upward pass and for exact
//       re-evaluation of borderline opening decisions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "../../include/hackcode_gpu.h"
#include "hc_f32split.h"

#define HC_IMAX (1 << 30)     // defs.h:124-128
#define HC_MAXLEVEL 31        // levels 0..30
#define HC_GROUP 32           // bodies per walk group of the per-body rule (one warp, one body per lane)
#define HC_BPL 2              // bodies per lane of the group criteria's walk (3 was measured: 6% slower
                              // with 64-body groups, and groups of more than 64 bodies ran 50 times
                              // longer for a reason not yet found; not used)
#define HC_GROUP2 (32 * HC_BPL)  // bodies per walk group of the group criteria

// Device status word (written by kernels, read by the host after a sync).
// Guard record, kept across evaluations.
struct hc_guard_state {
    double last_rms;              // RMS relative force error of the last check
    unsigned long long checks, trips;
    int flag;                     // 1: the last check failed and the fallback walk runs
    int pad;
};

struct hc_status {
    int error;                // 0 or HC_ERR_*
    int info;
    unsigned long long n2b;   // interaction totals of the last walk
    unsigned long long nbc;
    int max_stack;            // deepest walk stack seen
    int nborder;              // borderline opening decisions re-done in FP64
    unsigned long long ncand;     // candidate nodes classified by the walk
    unsigned long long nmixed;    // ... that needed the per-body test
    unsigned long long nentry_b;  // body-list entries evaluated (32 lanes each)
    unsigned long long nentry_c;  // cell-list entries evaluated
    unsigned long long mask_hist[33];  // entries by accept-mask popcount (counting walk only)
    unsigned long long nmlp;      // learned walk: candidates decided by the network
    unsigned long long nmlp_rounds;   // learned walk: network evaluations
};

// Root box state, kept on the device so the whole step can run without a
// host round trip (expandbox replay happens on the GPU).
struct hc_box {
    double rmin[3];
    double rsize;
    int chain_body;           // original index of the first massive body or -1
    int chain_lmax;           // deepest one-body expansion cell level (or -1)
    int chain_lmin;
    int nmassive;             // massive bodies
    int first_massive;        // original index of the first massive body
    int ncell;                // cells of the last build
    int max_depth;            // deepest node depth of the last build
    int nnode;                // nmassive + ncell
    int ngroups;              // tree-aligned walk groups of the massive bodies
    int level_start[HC_MAXLEVEL + 2];  // BFS offset of each depth
    double dsq[HC_MAXLEVEL + 1];       // rsize^2 / 4^level (grav.c:86,105)
};

struct hc_ctx {
    int64_t n;                // bodies
    int64_t maxcell;          // (int)(fcells * n), load.c:50
    hc_params prm;
    cudaStream_t stream;
    cudaStream_t side;        // the guard's direct sum, forked from stream, joined before the upward pass
    cudaEvent_t ev_fork, ev_join;
    bool join_pending;        // the build waits on ev_join before the upward pass
    cudaEvent_t ev[6];        // 0-1 build, 2-3 walk, 4-5 user timer
    std::string err;
    bool have_tree, have_forces;
    int64_t launches;
    float build_ms, walk_ms;

    // bodies (original order)
    double *mass, *px, *py, *pz, *vx, *vy, *vz, *ax, *ay, *az, *phi;
    int32_t *cnt_b, *cnt_c;   // per-body counts (optional)

    // keys and sort (n entries, double-buffered)
    unsigned long long *khi[2];
    uint32_t *klo[2];
    uint32_t *kval[2];
    int sort_sel;             // which buffer holds the sorted result
    uint32_t *sidx;           // sorted position -> original index (all bodies)
    int32_t *s_rank;          // sorted position -> massive rank or -1
    int32_t *leaf_of_sorted;  // sorted position -> BFS node of its leaf or -1
    uint32_t *tord;           // walk target order: massive in key order, then massless
    int32_t *gcnt, *goff;     // groups per node, their offsets (maxnode + 1)
    int32_t *gstart, *gcount; // tree-aligned groups: first massive rank, count
    int group_kind;           // 0: 32 consecutive bodies, 1: tree-aligned groups

    // massive bodies in key order
    unsigned long long *mhi;
    uint32_t *mlo;
    uint32_t *midx;           // massive rank -> original index
    uint32_t *mpos;           // massive rank -> sorted position
    int32_t *dlcp;            // lcp in octal digits of adjacent massive keys
    int32_t *ccount;          // cells starting at each massive rank (scan -> offsets)

    // nodes
    int64_t maxnode;
    int32_t *pre_info;        // pre-order: level (cell) or -1 (body); bit 31 unused
    int32_t *pre_a;           // pre-order: massive rank of first body
    uint32_t *bfs_a;          // breadth-first order: pre_a of each node (the depth sort's payload)
    unsigned long long *dkey[2]; // depth sort keys
    uint32_t *dval[2];
    uint32_t *bfs2pre, *pre2bfs;
    int32_t *parent, *lastc;
    int4 *cperm;              // upward pass: cells (index, first child, nodeC.y) grouped by depth, then child count
    uint32_t *cbins;          // their group offsets [257] and placement cursors [256]
    float4 *nodeA, *nodeB, *nodeQ;
    int2 *nodeC;
    double *nm, *ncx, *ncy, *ncz;         // FP64 mass and centre of mass per node
    int cofm_grid;                        // co-resident blocks of the upward-pass kernel
    int walk_blocks[20];                  // resident blocks of each walk variant
    // learned opening criterion: network, training state, samples
    struct MlpSmem *mlp_packed;           // BF16 image used by the walk
    float *mlp_p, *mlp_m, *mlp_v;         // FP32 master weights, Adam moments
    float *mlp_gpart, *mlp_lpart, *mlp_grad, *mlp_loss;
    int mlp_gcap;                         // blocks of one training mini-batch
    int mlp_step;                         // Adam step count
    float mlp_threshold;
    float mlp_band, mlp_band_hi;          // learned walk: network band [-band, band_hi] in log2(proxy/budget)
    int collect;                          // 1 while the label walk runs
    unsigned keep24;
    int collect_cap;                      // 0: count band candidates only
    int sample_capacity;
    int *sample_count;
    float *sample_x, *sample_amin, *sample_y, *sample_rel, *sample_w;
    int *sample_group, *sample_node;
    int nsample;                          // samples held on the device
    int64_t band_total;                   // band candidates seen by the last collection walk
    int criterion;                        // HC_CRITERION_* of include/hackcode_gpu.h
    float *rcrit2;                        // treecode1 criteria: critical radius^2 per node (lazy)
    int extpot;                           // external potential (HC_EXTPOT_*), 0: none
    double extpot_par[4];                 // its parameters after the pattern speed
    double *phi_ext;                      // external potential per body (lazy)
    int group_max;                        // bodies per tree-aligned walk group (<= HC_GROUP)
    int list_depth;                       // interaction-list entries evaluated per flush (32..64)
    // forest of independent systems (hc_ensemble.cu): the walk of a group
    // starts at its system's root cell instead of node 0
    const int32_t *walk_sys_root;         // [system] BFS index of the root cell (-1: none)
    const int32_t *walk_body_sys;         // [body] system of each body
    // per-evaluation guard of the approximate criteria (hc_guard.cu)
    int64_t guard_n;                      // sampled bodies (0: off)
    double guard_rms_max;
    int guard_slices;                     // source slices of the direct sum
    int guard_smem;                       // dynamic shared memory reserved per guard block (residency)
    int64_t *guard_idx;                   // sampled body indices (ascending)
    float4 *guard_part;                   // [slices][guard_n] partial accelerations
    struct hc_guard_state *guard;
    double group_theta;                   // opening angle of the group criterion

    // scratch
    int32_t *flags;           // n
    uint32_t *scan_tmp;       // single-pass scan: tile counter and look-back words
    uint32_t *hist;           // radix histograms
    int32_t *cand;            // expandbox candidates (original indices)
    int32_t *ncand;
    double *diag_part;        // per-block diagnostics partials
    hc_status *st;            // device status
    hc_box *box;              // device box
    hc_status *h_st;          // pinned host mirrors
    hc_box *h_box;

    // test points for hc_forces_at
    int64_t tcap;
    double *tx, *ty, *tz, *tax, *tay, *taz, *tphi;
    unsigned long long *tkhi[2];
    uint32_t *tklo[2], *tkval[2];
    uint32_t *thist;          // their radix sort's scratch (hist is baked into captured graphs)
};

// ---- host-side launchers implemented in the .cu files ----
// scan / sort (hc_sort.cu)
void hc_scan_exclusive_i32(hc_ctx *c, const int32_t *in, int32_t *out, int64_t n, int32_t *total_dev);
int64_t hc_scan_scratch_words(int64_t n);
// 32-bit words of sort scratch for sorting n keys (n < 2^30)
int64_t hc_sort_scratch_words(int64_t n);
int hc_sort_setup(hc_ctx *c);
// scratch: hc_sort_scratch_words(n) words (c->hist for the tree, c->thist for test points)
int hc_radix_sort_keys(hc_ctx *c, uint32_t *scratch, unsigned long long *khi[2], uint32_t *klo[2],
                       uint32_t *kval[2], int64_t n, int begin_bit, int end_bit, bool tie_fix,
                       const int *n_dev = nullptr);
// tree (hc_tree.cu)
int hc_tree_build(hc_ctx *c);
int hc_tree_setup(hc_ctx *c);
int hc_tree_dump_impl(hc_ctx *c, int32_t *level, int32_t *corner, int32_t *count, double *mass,
                      double *cm, double *quad, int32_t *bparent);
void hc_keys_for_points(hc_ctx *c, const double *x, const double *y, const double *z, int64_t n,
                        unsigned long long *khi, uint32_t *klo, uint32_t *kval);
// walk (hc_walk.cu)
int hc_walk_launch(hc_ctx *c, bool self, int64_t ntarget, const uint32_t *tsorted,
                   const double *tx, const double *ty, const double *tz, double *oax, double *oay,
                   double *oaz, double *ophi, double kick_dthf, int64_t nstep,
                   const int *run_flag = nullptr, bool body_rule = false);
int hc_walk_setup(hc_ctx *c);
struct MlpSmem;
int hc_label_launch(hc_ctx *c, int nsample, float eps_label);
// learned criterion network (hc_learn.cu)
int hc_mlp_nparams();
int hc_mlp_pack(hc_ctx *c);
int hc_mlp_infer_impl(hc_ctx *c, const float *x_dev, int64_t n, float *logits_dev);
int hc_mlp_grad_impl(hc_ctx *c, const float *x, const float *y, const float *w, int64_t n, float inv_norm,
                     float *grad_dev, float *loss_dev);
int hc_mlp_adam_impl(hc_ctx *c, const float *grad_dev, float lr, int t);
int hc_relabel_impl(hc_ctx *c, float thr);
// step (hc_step.cu)
void hc_kick_drift(hc_ctx *c, double dt);
void hc_diag_launch(hc_ctx *c, double *out36);
void hc_extpot_launch(hc_ctx *c, double kick_dthf, int64_t nstep);
void hc_direct_launch(hc_ctx *c, const int64_t *idx_dev, int64_t ns, double *oacc, double *ophi);
void hc_rcrit_launch(hc_ctx *c, int kind, double theta);
// guard (hc_guard.cu)
int hc_guard_slices(hc_ctx *c);
void hc_guard_launch(hc_ctx *c);
// the guard in two parts: the sampled direct sum (on any stream), then the
// comparison with the walk's forces and the check (on c->stream)
void hc_guard_direct_launch(hc_ctx *c, cudaStream_t s);
int hc_guard_setup(hc_ctx *c);
void hc_guard_check_launch(hc_ctx *c);
int hc_fma_peak_impl(hc_ctx *c, double *tflops);

#define HC_CUDA(call)                                                               \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            c->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
            return HC_ERR_CUDA;                                                     \
        }                                                                           \
    } while (0)

#ifdef __CUDACC__
// Diagnostics sums of one body (code_io.c:160-197) added into acc[36] in the
// order every diagnostics kernel uses: KE, PE (0.5 m pe_phi), KE tensor[9],
// m x_i a_j [9], m x_i v_j [9], m x [3], m v [3], m.  Products are rounded
// separately, as the reference computes them.
__device__ __forceinline__ void hc_diag_body(double *acc, double m, const double x[3], const double v[3],
                                             const double a[3], double pe_phi)
{
    double velsq = __dmul_rn(v[0], v[0]);
    velsq = __dadd_rn(velsq, __dmul_rn(v[1], v[1]));
    velsq = __dadd_rn(velsq, __dmul_rn(v[2], v[2]));
    const double hm = __dmul_rn(0.5, m);
    acc[0] += __dmul_rn(hm, velsq);
    acc[1] += __dmul_rn(hm, pe_phi);
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const double tv = __dmul_rn(v[j], hm), tx = __dmul_rn(x[j], m);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            acc[2 + 3 * j + k] += __dmul_rn(tv, v[k]);
            acc[11 + 3 * j + k] += __dmul_rn(tx, a[k]);
            acc[20 + 3 * j + k] += __dmul_rn(tx, v[k]);
        }
        acc[29 + j] += tx;
        acc[32 + j] += __dmul_rn(v[j], m);
    }
    acc[35] += m;
}

// Operands of the packed FP32x2 instructions (__ffma2_rn and relatives): a
// float2 is one register pair.  Lists stored in pairs keep both entries'
// values of one quantity adjacent, so lo2 / hi2 of a float4 row give them.
__device__ __forceinline__ float2 lo2(const float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 splat2(float v) { return make_float2(v, v); }
#endif

// Largest tree-aligned walk group of the build: up to 64 bodies when a
// group criterion walks the tree, 32 for the per-body rule.
static inline int hc_table_gmax(const hc_ctx *c)
{
    const int cap = c->criterion == 0 ? HC_GROUP : HC_GROUP2;
    return c->group_max >= 1 && c->group_max <= cap ? c->group_max : cap;
}

// m != 0.0 on the double's bits (a compare is an FP64-pipe instruction):
// true for NaN, false for +0 and -0
__device__ __forceinline__ bool hc_nonzero(double m) { return (hc_dbits(m) << 1) != 0; }

static inline int hc_grid(int64_t n, int block, int cap = 152 * 16)
{
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}
