/*
 * hackcode_gpu.h -- C ABI of the GB300 hackcode1 treecode library
 * (nemo_gb300/libhackcode_gpu.so).
 *
 * NEMO has no plugin interface for force solvers: the reference's "operator
 * API" for this path is the hackcode1 / hackforce programs themselves
 * (src/nbody/evolve/hackcode/hackcode1/code.c:21-51 keywords,
 * hackforce.c:38-50).  This header is the thin C layer those programs (and the
 * ctypes mirror in nemo_gb300/hackcode.py) call.  Each entry point names the
 * reference routine it replaces.
 *
 * Conventions: plain C types only; every function returns HC_OK (0) or a
 * negative HC_ERR_* code and never exits; hc_last_error() gives the message.
 * Host arrays are FP64 in the reference's layouts (Mass[n],
 * PhaseSpace[n][2][3], Acceleration[n][3], Potential[n]).  One context owns
 * one CUDA stream and all device memory for one system; one host thread
 * drives a context at a time.
 */
#ifndef HACKCODE_GPU_H
#define HACKCODE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    HC_OK = 0,
    HC_ERR_ARG = -1,        /* bad argument */
    HC_ERR_CUDA = -2,       /* CUDA runtime error */
    HC_ERR_CELLS = -3,      /* more than fcells*nbody cells needed (load.c:237-239) */
    HC_ERR_COINCIDENT = -4, /* two massive bodies share integer coords (load.c:113) */
    HC_ERR_STACK = -5,      /* walk traversal stack exhausted */
    HC_ERR_STATE = -6,      /* call out of order (e.g. forces before tree) */
    HC_ERR_NOMEM = -7       /* device allocation failed */
};

typedef struct hc_ctx hc_ctx;

/* Run parameters (hackcode1 keywords tol= eps= fcells= and usequad=, the
 * switch between the hackcode1 and hackcode1_qp builds,
 * hackcode1/Makefile:99-115). */
typedef struct {
    double tol;      /* cell-opening tolerance, grav.c:122-131 (tol=0: direct sum) */
    double eps;      /* Plummer softening, grav.c:42-73 */
    double fcells;   /* cell pool = fcells * nbody (load.c:49-53) */
    int usequad;     /* 1: quadrupole moments (QUADPOLE build) */
    int count_per_body; /* 1: keep per-body interaction counts */
} hc_params;

/* Diagnostics of code_io.c:160-197 plus interaction totals of the last force
 * evaluation (64-bit: the reference's int counters wrap at N=1M). */
typedef struct {
    double etot[3];      /* T+U, T, U (U = 1/2 sum m phi) */
    double keten[9];     /* kinetic energy tensor */
    double peten[9];     /* potential energy tensor sum m x_i a_j */
    double amten[9];     /* antisymmetric angular momentum tensor */
    double cmphase[6];   /* centre of mass position, velocity */
    double mtot;
    int64_t n2b;         /* body-body interactions */
    int64_t nbc;         /* body-cell interactions */
    int64_t nfcalc;      /* force evaluations (bodies walked) */
} hc_diag;

/* Tree summary (for the structural parity check against maketree). */
typedef struct {
    int64_t nbody_massive;
    int64_t ncell;
    int32_t max_level;
    double rmin[3];
    double rsize;
} hc_tree_info;

/* Create a context for nbody bodies.  Allocates all device memory once
 * (the reference allocates its cell pool once too, load.c:49-53).
 * nbody <= 2^28, nbody * (1 + fcells) < 2^30 and finite tol, eps and fcells,
 * else HC_ERR_ARG.
 * Replaces: startrun's allocation and box set-up, code.c:70-122. */
int hc_create(hc_ctx **out, int64_t nbody, const hc_params *params);
void hc_destroy(hc_ctx *ctx);
const char *hc_last_error(const hc_ctx *ctx);
int hc_set_params(hc_ctx *ctx, const hc_params *params);

/* Upload Mass[n] and PhaseSpace[n][2][3] from host memory.
 * Replaces: inputdata / get_snap body fill, code_io.c:35-56. */
int hc_upload(hc_ctx *ctx, const double *mass, const double *phase);

/* Restore Acceleration[n][3] and Potential[n] of a saved state (restart=,
 * code_io.c:254-284): the next hc_step's closing half-kick uses them as the
 * old accelerations.  Either pointer may be NULL. */
int hc_set_forces(hc_ctx *ctx, const double *acc, const double *phi);

/* Root box (rmin, rsize); starts at (-2,-2,-2), 4 (code.c:119-120) and only
 * grows (expandbox, load.c:68-95). */
int hc_set_box(hc_ctx *ctx, const double rmin[3], double rsize);
int hc_get_box(hc_ctx *ctx, double rmin[3], double *rsize);

/* Build the octree of the massive bodies: expandbox replay, 90-bit keys,
 * radix sort, cell linking, monopole/quadrupole upward pass.
 * Replaces: maketree + hackcofm, load.c:32-248. */
int hc_build_tree(hc_ctx *ctx);
int hc_tree_summary(hc_ctx *ctx, hc_tree_info *info);

/* Cell dump for the structural check (a): per cell its level, integer lower
 * corner on the 2^30 grid, body count, mass, centre of mass and quadrupole
 * (xx,xy,xz,yy,yz,zz); per body (original order) its parent cell level or
 * -1.  Arrays sized by hc_tree_summary().ncell / nbody. */
int hc_dump_tree(hc_ctx *ctx, int32_t *level, int32_t *corner, int32_t *count, double *mass,
                 double *cm, double *quad, int32_t *body_parent_level);

/* Forces at every body, its own body skipped (hackgrav for each body,
 * grav.c:22-32 as looped in code.c:169-180).  Results stay on the device
 * (hc_download).  Requires hc_build_tree. */
int hc_forces(hc_ctx *ctx);

/* One full force evaluation -- hc_build_tree then hc_forces -- replayed
 * from a CUDA graph captured on the first call (no host round trip inside). */
int hc_evaluate(hc_ctx *ctx);

/* One force evaluation of host-resident positions, hackforce's per-call
 * contract (hackforce.c:177-215) with one host round trip: pos [n][3] in
 * (masses and velocities stay as last uploaded), optionally the previous
 * evaluation's accelerations prev_acc [n][3] that the error and learned
 * criteria read (NULL keeps the context's), and acc [n][3] / phi [n] out
 * (either may be NULL).  The previous accelerations are copied on a stream of
 * their own while the tree is built; the walk waits for them.  Host buffers
 * should be page-locked for the copies to run asynchronously. */
int hc_evaluate_host(hc_ctx *ctx, const double *pos, const double *prev_acc, double *acc, double *phi);

/* CUDA-graph replay of hc_step / hc_evaluate on (1, default) or off (0);
 * results are identical either way. */
int hc_set_graphs(hc_ctx *ctx, int on);

/* Forces at ntest separate test points that are not part of the tree
 * (hackforce test=, hackforce.c:206-213).  test_pos is host [ntest][3];
 * acc [ntest][3] / phi [ntest] receive the results (host). */
int hc_forces_at(hc_ctx *ctx, const double *test_pos, int64_t ntest, double *acc, double *phi);

/* Download PhaseSpace / Acceleration / Potential (any may be NULL).
 * Replaces: the put_snap body gather, code_io.c:147-151. */
int hc_download(hc_ctx *ctx, double *phase, double *acc, double *phi);

/* Per-body interaction counts of the last hc_forces (original order);
 * requires params.count_per_body. */
int hc_body_counts(hc_ctx *ctx, int32_t *n2b, int32_t *nbc);

/* One hackcode1 leapfrog step (stepsystem, code.c:159-191): maketree,
 * forces with the closing half-kick v += (a_new - a_old) dt/2 when
 * nstep > 0, diagnostics into *diag (may be NULL), then the kick-drift
 * v1/2 = v + a dt/2, x += v1/2 dt, v = v1/2 + a dt/2.  The state after the
 * force evaluation (what output() writes) is captured in *diag and, when
 * snap_phase/snap_acc/snap_phi are non-NULL, copied to those host arrays
 * before the drift. */
int hc_step(hc_ctx *ctx, double dt, int64_t nstep, hc_diag *diag, double *snap_phase,
            double *snap_acc, double *snap_phi);

/* Diagnostics of the current device state (code_io.c:160-197). */
int hc_diagnostics(hc_ctx *ctx, hc_diag *diag);

/* FP64 direct-sum accelerations/potentials at nsample bodies (indices into
 * the original order, self skipped): the exact (tol=0) limit of the walk,
 * used to state force errors.  Results to host acc [nsample][3], phi. */
int hc_direct_sample(hc_ctx *ctx, const int64_t *index, int64_t nsample, double *acc, double *phi);

/* Timing of the last hc_build_tree / hc_forces (milliseconds, CUDA events on
 * the context stream) and kernel launch count of the last call. */
int hc_last_timing(hc_ctx *ctx, double *build_ms, double *walk_ms, int64_t *launches);

/* Opening criterion of the walk.
 * HC_CRITERION_BODY  (default): the reference's rule, per body -- open iff
 *     tol^2 |cm - x|^2 < size^2 (subdivp, grav.c:122-131); interaction sets
 *     identical to hackcode1's.
 * HC_CRITERION_GROUP: one decision per group (a tree cell of up to 64 bodies,
 *     see hc_tuning) -- open iff
 *     theta^2 dmin^2 < size^2, dmin the distance from the group's bounding box
 *     to the cell's centre of mass (a group walk in the manner of treecode1's
 *     walktree, treegrav.c:380-419).  No counterpart in hackcode1. */
/* HC_CRITERION_ERROR: one decision per group -- accept iff the expansion's
 *     leading truncation error m b^p / (dmin - b)^(p+2) is at most theta
 *     times the group's smallest |a| from the previous force evaluation
 *     (b: radius around the cell's centre of mass holding all its bodies;
 *     p = 3 with quadrupoles, 2 without); the group rule at theta = 1 when
 *     no previous accelerations exist.  No counterpart in hackcode1. */
/* HC_CRITERION_LEARNED: the error rule decides clear cases; candidates whose
 *     error proxy lies in the band of hc_learn_set_band around the budget
 *     theta * |a| are decided by the trained network (hc_learn_*), accepted
 *     when its logit exceeds the threshold of hc_learn_set_threshold.  No
 *     counterpart in hackcode1. */
/* HC_CRITERION_BH86, _SW94, _BARNES: treecode1's critical radii (setrcrit,
 *     treecode1/treeload.c:232-252: (size/theta)^2; (largest distance from
 *     the centre of mass to a cell corner / theta)^2; the default
 *     (size/theta + |cm - cell centre|)^2) in a group walk: a cell is
 *     accepted for the group iff the squared distance from the group's
 *     bounding box to its centre of mass exceeds the critical radius
 *     (treecode1/treegrav.c:137-157 tests the box of the target cell, and
 *     adds an adjacency test a bounding box does not need). */
enum { HC_CRITERION_BODY = 0, HC_CRITERION_GROUP = 1, HC_CRITERION_ERROR = 2, HC_CRITERION_LEARNED = 3,
       HC_CRITERION_BH86 = 4, HC_CRITERION_SW94 = 5, HC_CRITERION_BARNES = 6 };
/* The critical radius^2 of every cell of the current tree under one of
 * treecode1's criteria (HC_CRITERION_BH86/_SW94/_BARNES) at opening angle
 * theta, as the walk uses them -- setrcrit, treecode1/treeload.c:232-252,
 * with the cell's geometric centre and size and its centre of mass -- into
 * rcrit2[ncell], in hc_dump_tree's cell order (FP32 values widened). */
int hc_tree_rcrit(hc_ctx *ctx, int criterion, double theta, double *rcrit2);
int hc_set_criterion(hc_ctx *ctx, int criterion, double theta);

/* Guard of the group, error and learned criteria (no counterpart in
 * hackcode1): after each of their force evaluations the accelerations of
 * `nsample` bodies (a uniform sample drawn once from `seed`) are compared on
 * the device with an FP32 direct sum over all bodies; when the RMS relative
 * error exceeds rms_max the evaluation's forces are recomputed with the
 * per-body rule at the context's tol (closing half-kick included), inside the
 * same CUDA graph.  nsample = 0 turns it off.  hc_guard_stats: checks made,
 * checks failed, RMS of the last check. */
#define HC_GUARD_MAX_SAMPLE 65536
int hc_set_guard(hc_ctx *ctx, int64_t nsample, double rms_max, uint64_t seed);
int hc_guard_stats(hc_ctx *ctx, int64_t *checks, int64_t *trips, double *last_rms);

/* ---- learned opening criterion (no counterpart in hackcode1) ----
 * The network: 12 features of a (group, cell) pair -> 64 -> 64 (SiLU) -> 1
 * logit; BF16 weights, FP32 accumulation; FP32 master weights in the flat
 * order W1[64][12], b1[64], W2[64][64], b2[64], W3[64], b3. */
int hc_learn_nparams(void);
int hc_learn_init(hc_ctx *ctx, uint64_t seed);
int hc_learn_set_params(hc_ctx *ctx, const float *params, int count);
int hc_learn_get_params(hc_ctx *ctx, float *params, int count);
/* logits of n feature rows [n][12] (host arrays) through the walk's kernel */
int hc_learn_infer(hc_ctx *ctx, const float *x, int64_t n, float *logits);
/* gradient of the mean weighted binary cross-entropy over n <= 8192 rows
 * (host arrays; w may be NULL) and the summed loss */
int hc_learn_gradient(hc_ctx *ctx, const float *x, const float *y, const float *w, int64_t n, float *grad,
                      float *loss);
/* Labels from the method itself: with the tree built and accelerations of a
 * previous evaluation on the device, walk with the error rule at budget
 * theta, sample about `target` band candidates, and label each by comparing
 * the cell's multipole with a refined walk of its subtree (label 1 when the
 * group's largest relative error is at most theta).  *nsamples receives the
 * count kept on the device. */
int hc_learn_collect(hc_ctx *ctx, double theta, int64_t target, int64_t *nsamples);
int hc_learn_samples(hc_ctx *ctx, float *x, float *y, float *rel, int64_t cap, int64_t *n);
int hc_learn_load_samples(hc_ctx *ctx, const float *x, const float *y, const float *w, int64_t n);
/* Adam on the device samples; *loss receives the last epoch's mean loss */
int hc_learn_train(hc_ctx *ctx, int epochs, int batch, double lr, uint64_t seed, double *loss);
int hc_learn_set_threshold(hc_ctx *ctx, double logit_threshold);
/* label the device samples again: 1 when their measured relative error is at
 * most rel_threshold */
int hc_learn_relabel(hc_ctx *ctx, double rel_threshold);
/* the band the network decides, in log2 of (error proxy / budget):
 * [-lo, hi] (defaults 1 and 3); below it the cell is accepted, above opened */
int hc_learn_set_band(hc_ctx *ctx, double lo, double hi);

/* How the per-body rule groups the bodies of a warp: HC_GROUPS_CONSECUTIVE
 * (32 bodies consecutive in key order) or HC_GROUPS_TREE (the bodies of one
 * cell holding at most 32, siblings packed).  Its interaction sets do not
 * depend on it (the rounding of the FP32 sums does).  The other criteria
 * always walk tree groups of up to 64 bodies (two per lane). */
enum { HC_GROUPS_CONSECUTIVE = 0, HC_GROUPS_TREE = 1 };
int hc_set_grouping(hc_ctx *ctx, int kind);

/* External potential added to every body's acceleration and potential after
 * the walk, as hackcode3 does with potname= / potpars= (hackcode3/grav.c:34-38,
 * code.c:136-139): NEMO's plug-ins plummer (par: omega, M, a), hernquist
 * (omega, M, a), miyamoto (omega, M, a, b; symmetry axis y, as NEMO builds
 * miyamoto.c) and log (omega, m_c, r_c, q, r), restated on the device with the
 * plug-ins' defaults for missing parameters;
 * the pattern speed omega must be 0.  The energy in hc_diag counts the
 * external potential as hackcode3's diagnostics do (code_io.c:180-186).
 * name NULL, "" or "null" turns it off. */
enum { HC_EXTPOT_PLUMMER = 1, HC_EXTPOT_HERNQUIST = 2, HC_EXTPOT_MIYAMOTO = 3, HC_EXTPOT_LOG = 4 };
int hc_set_extpot(hc_ctx *ctx, const char *name, const double *par, int npar);

/* Walk tuning (no counterpart in hackcode1): the largest walk group of tree
 * grouping (1..64 bodies per warp; the per-body rule, one body per lane, uses
 * at most 32, the group criteria two bodies per lane), the interaction-list
 * depth evaluated per flush (32..64 entries) and the grouping kind (the group
 * criteria always walk tree groups).  hc_autotune times one evaluation of the
 * bodies and criterion currently set for each candidate (group_max 16/24/32
 * for the per-body rule, 32/48/64 for the group criteria, x list_depth
 * 32/48/64 on tree groups, plus consecutive groups for the per-body rule),
 * keeps the fastest and returns it with its time in ms.  With the per-body rule the interaction sets do not depend on
 * the tuning; with the approximate criteria the group size changes which
 * cells are accepted. */
typedef struct {
    int group_max, list_depth, grouping;
    double ms;
} hc_tuning;
int hc_set_tuning(hc_ctx *ctx, const hc_tuning *t);
int hc_get_tuning(hc_ctx *ctx, hc_tuning *t);
int hc_autotune(hc_ctx *ctx, hc_tuning *best);

/* Walk statistics of the last force evaluation: candidates classified,
 * candidates needing the per-body test, interaction-list entries evaluated
 * (bodies, cells; 32 lanes each), borderline decisions re-done in FP64 and the
 * deepest traversal stack. */
typedef struct {
    int64_t candidates, mixed, entries_body, entries_cell, borderline, max_stack;
    int64_t network;           /* candidates decided by the learned criterion's network */
    int64_t network_rounds;    /* network evaluations (each decides up to 32 candidates) */
    int64_t mask_hist[33];   /* entries by accept-mask popcount (only with count_per_body) */
} hc_walk_stats;
int hc_walk_statistics(hc_ctx *ctx, hc_walk_stats *out);

/* Device timers on the context stream (CUDA events): start, then stop
 * returns the elapsed milliseconds; both bracket whatever was launched on the
 * context between them. */
int hc_timer_start(hc_ctx *ctx);
int hc_timer_stop(hc_ctx *ctx, double *ms);

/* Measured FP32 FMA throughput of this GPU (TFLOP/s, FMA = 2 flops): the
 * denominator of the walk's roofline fraction. */
int hc_fp32_peak(hc_ctx *ctx, double *tflops);

/* Initial conditions (host, FP64), drawn with NEMO's xrandom/ran3:
 * mkplummer with its default keywords (src/nbody/init/mkplummer.c:257-422)
 * and hackcode1's nbody= test data (hackcode1/code.c:129-153). */
void hc_mkplummer(int n, int seed, double *mass, double *phase);
void hc_make_testdata(int n, int seed, int cencon, double *mass, double *phase);
/* Isotropic Hernquist sphere, G = M = a = 1, truncated at rtrunc (no
 * counterpart in hackcode1; NEMO's mkhernquist / mkhalo differ): radii from
 * the truncated mass profile, velocities from the Eddington-inverted
 * distribution function (Hernquist 1990, eq. 17), equal masses M(rtrunc)/n,
 * centre of mass at rest at the origin; ran3 seeded with seed. */
void hc_mkhernquist(int n, int seed, double rtrunc, double *mass, double *phase);
/* Composite disk galaxy, G = 1 (no counterpart in hackcode1; NEMO's mkexpdisk,
 * mkhalo and magalie differ): exponential sech^2 disk (M 0.1, R_d 1, z0 0.1,
 * Toomre Q 1.5 epicyclic velocities), Hernquist bulge (M 0.033, a 0.2) and
 * NFW halo (M_vir 1, c 10, r_vir 30, truncated at r_vir) with isotropic
 * velocities from Eddington's inversion in the total potential; bodies in
 * the order disk, bulge, halo; ran3 seeded with seed. */
void hc_mkgalaxy(int64_t n_disk, int64_t n_bulge, int64_t n_halo, int seed, double *mass, double *phase);

/* Initial conditions drawn on the device straight into the context's bodies
 * (replaces hc_upload; forces and potentials are zeroed).  model "plummer":
 * mkplummer's model and sampling steps (src/nbody/init/mkplummer.c:257-422),
 * par[0] = mfrac (default 0.999, capped at the mass inside rfrac); model
 * "hernquist": hc_mkhernquist's model, par[0] = rtrunc (default 100); model
 * "galaxy": hc_mkgalaxy's model with its tables and per-body steps, par[0] =
 * n_disk (default n/4), par[1] = n_bulge (default n/16), the rest halo.  Every
 * body draws from its own counter-based stream of seed, so the sample is
 * another draw of the same model than the host generators give, equal for
 * equal (n, seed) on every device.  Centre of mass and its velocity are
 * removed.  HC_ERR_ARG for an unknown model or bad parameters; HC_ERR_STATE
 * if a velocity rejection loop hit its iteration limit. */
int hc_generate(hc_ctx *ctx, const char *model, uint64_t seed, const double *par, int npar);

/* Host services of the drop-in programs, exported for tests: copy every
 * snapshot of a filestruct file through the reader and writer (returns the
 * snapshot count or -1), and evaluate a keyword expression as getdparam does
 * (src/kernel/io/getparam.c). */
int hc_snapcopy(const char *in, const char *out);
double hc_nemo_eval(const char *expr, int *ok);

/* Diagnostics sums of device-resident bodies without any device allocation
 * (no counterpart in the reference: an addition for callers that cannot
 * allocate device memory -- a runtime that only lends pre-registered buffers
 * from its own pool, or a real-time loop that must not pay cudaMalloc's
 * implicit synchronisation).  All pointers are device pointers of n FP64
 * values; out36 receives the 36 raw sums {KE, PE, KE tensor[9],
 * sum m x_i a_j [9], sum m x_i v_j [9], sum m x[3], sum m v[3], total mass}
 * on `stream` (a cudaStream_t, NULL = default).  PE is 0.5 sum m phi with phi
 * as passed: with an external field pass phi + phi_ext (hc_diagnostics adds
 * the external part itself).  The per-block partials use a static device
 * array sized for at most 8,388,608 bodies; larger n returns HC_ERR_ARG.  The
 * first call on a device looks the array up (cudaGetSymbolAddress) and should
 * come before any stream capture; with lazy module loading the CUDA driver may
 * also load the entry point's kernels at that call, which takes device memory
 * for their code (later calls take none); after cudaDeviceReset of a device the
 * looked-up address is stale and the entry point must not be called on it
 * again.  All calls on a device share the array: calls that overlap on the
 * GPU race and must be serialised by the caller. */
int hc_diagnostics_noalloc(int64_t n, const double *mass, const double *x, const double *y, const double *z,
                           const double *vx, const double *vy, const double *vz, const double *ax,
                           const double *ay, const double *az, const double *phi, double *out36, void *stream);

/* ---- ensembles of independent systems (no counterpart in hackcode1, which
 * evolves one system per run) ----
 * nsys systems of counts[s] bodies, stepped together with hackcode1's
 * leapfrog: systems of more than direct_max bodies share one octree build
 * (each in its own slot of a forest box, with its own persistent expandbox
 * root box starting at (-2,-2,-2), 4) and are walked with the per-body rule
 * at tol; the others use an FP32 direct sum, one thread block per system.
 * Arrays are the systems' bodies concatenated in the given order; every
 * body needs a positive mass (hc_ens_upload returns HC_ERR_ARG otherwise). */
#define HC_ENS_DIRECT_LIMIT 4096
typedef struct hc_ens hc_ens;
typedef struct {
    double tol, eps;
    int usequad;
    int direct_max;     /* 0..HC_ENS_DIRECT_LIMIT */
    double fcells;      /* cell pool of the forest per tree body (0: 1.0) */
} hc_ens_params;
typedef struct {
    int nsys_tree, nsys_direct;
    int64_t bodies_tree, bodies_direct;
    int64_t interactions_tree, interactions_direct;   /* of the last step */
    double tree_ms, direct_ms;                         /* device time of the last step */
    int64_t launches;                                  /* kernels of one step */
} hc_ens_stats;
int hc_ens_create(hc_ens **out, int nsys, const int64_t *counts, const hc_ens_params *params);
void hc_ens_destroy(hc_ens *e);
const char *hc_ens_last_error(const hc_ens *e);
int hc_ens_upload(hc_ens *e, const double *mass, const double *phase);
/* one step (stepsystem, code.c:159-191): forces with the closing half-kick
 * when nstep > 0, per-system energies (energy[nsys][3] = KE, PE, total;
 * may be NULL), then kick-drift.  One CUDA graph per step. */
int hc_ens_step(hc_ens *e, double dt, int64_t nstep, double *energy);
int hc_ens_download(hc_ens *e, double *phase, double *acc, double *phi);
int hc_ens_info(hc_ens *e, hc_ens_stats *out);
/* Tuning of an ensemble's step (no counterpart in the reference): the tree
 * systems' walk groups (group_max 1..64 bodies, list_depth 32..64; always
 * tree-aligned) and the direct sum's block size (128, 256 or 512 threads).
 * hc_ens_autotune times the two force phases for every candidate on the
 * current bodies (after hc_ens_upload; positions, velocities, accelerations
 * and potentials are left as they were) and keeps the fastest; tree_ms /
 * direct_ms are the winners' phase times. */
typedef struct {
    int group_max, list_depth, direct_threads;
    double tree_ms, direct_ms;
} hc_ens_tuning;
int hc_ens_set_tuning(hc_ens *e, const hc_ens_tuning *t);
int hc_ens_get_tuning(hc_ens *e, hc_ens_tuning *t);
int hc_ens_autotune(hc_ens *e, hc_ens_tuning *best);

#ifdef __cplusplus
}
#endif
#endif
