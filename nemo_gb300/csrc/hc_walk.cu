// hc_walk.cu -- the Barnes-Hut force walk on sm_103a.
//
// Reference: hackgrav / hackwalk / walksub / subdivp / gravsub,
// src/nbody/evolve/hackcode/hackcode1/grav.c:22-131.
//
// The reference walks the tree once per body, recursively: a cell is opened
// iff tol^2 * |cm - x|^2 < size^2 (subdivp, grav.c:122-131, no test whether
// the cell contains the body), an accepted node other than the body itself is
// added by gravsub (Plummer-softened monopole, plus the quadrupole term in the
// QUADPOLE build).
//
// Here one warp walks for a group of bodies: under the reference's per-body
// rule up to 32 (one per lane) that are consecutive in Morton order (a compact
// patch of space) or make up a small cell; under the group criteria a cell of
// up to 64 (two per lane).  Under the per-body rule every traversal entry
// carries a 32-bit lane mask: the bodies whose own walk reaches that node (all
// ancestors opened for them).  Candidates are processed 32 at a time, one per
// lane:
//   * against the group's bounding box: accepted by all bodies in the mask,
//     opened by all, or "mixed";
//   * mixed candidates are re-tested per body (broadcast by shuffle); a test
//     inside a thin band around tol^2 d^2 = size^2 is redone in FP64 exactly
//     as subdivp does, so every body's accept/open decision -- and therefore
//     its interaction set and counts -- is the reference's.
// Opened cells push their contiguous child range with the opening mask on a
// per-warp shared-memory stack; accepted bodies and cells are appended to two
// shared-memory interaction lists with their accept masks, and each list is
// evaluated by all 32 lanes when it fills (broadcast shared-memory reads,
// packed FP32x2 arithmetic over two entries at a time, rsqrt), lanes outside
// an entry's mask contributing zero.
//
// Precision: positions are taken relative to the group centre (FP64 centre,
// node centres stored as FP32 hi/lo pairs), the interaction arithmetic is
// FP32, and each list evaluation's partial sums are added into the running
// per-body totals with Kahan compensation; results are stored in FP64.
//
// Flop count per interaction (FMA = 2, rsqrt = 1): monopole 20, quadrupole
// cell 59.  These are the per-interaction figures used for the roofline.
#include <cstring>
#include "hc_internal.cuh"
#include "hc_mlp.cuh"

namespace {

constexpr int WARPS = 4;        // warps per block
constexpr int STACK = 256;      // traversal stack entries per warp (deepest seen at N=1M: 136)
constexpr int BCAP = 64;        // body interaction list entries per warp
constexpr int CCAP = 64;        // cell interaction list entries per warp
constexpr unsigned FULL = 0xffffffffu;
constexpr int QCAP = 64;        // learned walk: queued band candidates per warp

// Learned walk, per warp: band candidates waiting for the network (the
// scalars their features need) and the feature tile of one network round.
struct QueueSmem {
    __nv_bfloat16 x[32 * MLP_XS];     // features of the round's rows
    int node[QCAP];
    unsigned mask[QCAP];
    float dmin2[QCAP], dmax2[QCAP], err[QCAP];   // err: the error rule's proxy
    float z[32];                      // the round's logits
};

// Interaction lists in pairs: entry e sits in half e & 1 of pair e >> 1, so
// that both entries' values of one quantity are adjacent floats, the operands
// of one packed FP32x2 instruction.
struct WarpSmem {
    uint2 stack[STACK];         // x = first node << 3 | (count - 1), y = lane mask
    float4 bp[BCAP / 2][4];     // body pairs, each quantity for both entries: (hx hy) (hz m) (lx ly) (lz mask)
                                // (hi and lo parts of the position relative to the group, mass, accept mask)
    float4 cp[CCAP / 2][5];     // cell pairs, likewise: (x y) (z m) (-Qxx -Qxy) (-Qxz -Qyy) (-Qyz -Qzz)
    uint2 cmask[CCAP / 2];      // cell pairs: accept masks (per-body rule, counting walk)
    unsigned long long stat[8]; // warp totals (lane 0 writes): see the ST_* indices
    float gu[16];               // the group's uniform values (see GU_* below), read where used
};
enum { ST_N2B, ST_NBC, ST_CAND, ST_MIXED, ST_EB, ST_EC, ST_MLP, ST_ROUNDS };

struct WalkArgs {
    const float4 *nodeA, *nodeB, *nodeQ;
    const int2 *nodeC;
    const double *ncx, *ncy, *ncz;
    const hc_box *box;
    int64_t ntarget;
    const uint32_t *tsorted;              // sorted slot -> target index
    const double *tx, *ty, *tz;           // target positions (target order)
    int self_mode;                        // targets are the tree's own bodies
    float tol2f, eps2f;
    double tol2d;
    double *oax, *oay, *oaz, *ophi;       // results (target order)
    int32_t *cnt_b, *cnt_c;               // optional per-target counts
    double kick_dthf;                     // closing half kick (code.c:175-179)
    int64_t nstep;
    double *vx, *vy, *vz;
    hc_status *st;
    unsigned *group_counter;
    const int32_t *gstart, *gcount;       // tree-aligned groups of the massive targets
    int use_table;                        // 1: table groups, then massless targets in 32s
    float eps_acc;                        // MODE 2/3 error budget relative to |a|
    const double *pax, *pay, *paz;        // MODE 2/3: accelerations of the previous evaluation
    const int *run_flag;                  // when set: the walk runs only if *run_flag != 0
    int flush_at;                         // lists are evaluated once they hold more entries (<= 32;
                                          // one iteration appends at most 32)
    const float *rcrit2;                  // MODE 1, treecode1 criteria: accept iff dmin^2 > rcrit2[node]
    const int32_t *sys_root, *body_sys;   // forest: root cell of each group's system
    const MlpSmem *mlp;                   // MODE 3: packed network
    float mlp_threshold;                  // MODE 3: accept iff logit > threshold
    float band_lo_f, band_hi_f;           // MODE 3: network band [budget band_lo_f, budget band_hi_f] of the proxy
    int collect;                          // MODE 3: decide analytically, record sampled band candidates
    unsigned keep24;                      // sampling threshold on a 24-bit hash
    int sample_cap;
    int *sample_count;
    float *sample_x;                      // [cap][12]
    int *sample_group, *sample_node;
    float *sample_amin;
};

// Features of a (group, cell) pair for the opening network; logarithms are
// base 2 and scaled to O(1).  p is log2(error proxy / (eps amin)).
__device__ __forceinline__ void cell_features_inl(float *f, float dmin2, float dmax2, float dsq, float m, float b, float gap,
                                              float4 Q0, float4 Q1, float amin, float rg2, float eps2, int depth,
                                              int ngroup, float p_raw)
{
    const float L_dmin = 0.5f * __log2f(fmaxf(dmin2, 1e-30f));
    const float qf = sqrtf(Q0.x * Q0.x + Q0.w * Q0.w + Q1.y * Q1.y +
                           2.f * (Q0.y * Q0.y + Q0.z * Q0.z + Q1.x * Q1.x));
    f[0] = 0.5f * __log2f(fmaxf(dsq, 1e-30f)) - L_dmin;                 // size / dmin
    f[1] = __log2f(fmaxf(b, 1e-30f)) - L_dmin;                           // bmax / dmin
    f[2] = __log2f(fmaxf(m, 1e-30f)) - 2.f * L_dmin - __log2f(fmaxf(amin, 1e-30f));
    f[3] = p_raw;                                                        // truncation-error proxy
    f[4] = __log2f(fmaxf(qf, 1e-30f)) - __log2f(fmaxf(m * b * b, 1e-30f));
    f[5] = 0.5f * __log2f(fmaxf(rg2, 1e-30f)) - L_dmin;                  // group extent / dmin
    f[6] = L_dmin - 0.5f * __log2f(fmaxf(dmax2, 1e-30f));                // dmin / dmax
    f[7] = __log2f(fmaxf(Q1.z, 1.f));                                    // bodies in the cell
    f[8] = 0.5f * __log2f(fmaxf(eps2, 1e-30f)) - L_dmin;                 // softening / dmin
    f[9] = (float)depth;
    f[10] = (float)ngroup;
    f[11] = __log2f(fmaxf(gap, 1e-30f)) - L_dmin;
    const float scale[12] = {0.5f, 0.25f, 0.125f, 0.25f, 0.25f, 0.25f, 0.5f, 0.125f, 0.125f, 0.0625f, 0.03125f, 0.5f};
#pragma unroll
    for (int i = 0; i < 12; i++) f[i] = fminf(8.f, fmaxf(-8.f, f[i] * scale[i]));
}


// Out-of-line copy for the sampling path (label collection), which is rare.
__device__ __noinline__ void cell_features(float *f, float dmin2, float dmax2, float dsq, float m, float b, float gap,
                                           float4 Q0, float4 Q1, float amin, float rg2, float eps2, int depth,
                                           int ngroup, float p_raw)
{
    cell_features_inl(f, dmin2, dmax2, dsq, m, b, gap, Q0, Q1, amin, rg2, eps2, depth, ngroup, p_raw);
}

__device__ __forceinline__ unsigned hash2(unsigned a, unsigned b)
{
    unsigned h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u + (a << 6) + (a >> 2));
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ float wmin(float v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ float wmax(float v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ double wmind(double v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmin(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ double wmaxd(double v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float x)
{
    float y = __fsub_rn(x, comp);
    float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

// a - b = s + e exactly (Knuth's TwoSum on a + (-b))
__device__ __forceinline__ void two_diff(float a, float b, float &s, float &e)
{
    s = __fsub_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(-b, bb));
}

// subdivp in FP64 (grav.c:122-131): open iff tol^2 * |cm - x|^2 < dsq.
// quantity k (0-based) of list entry e in a pair array with float4 rows
__device__ __forceinline__ float *pair_slot(float4 *row, int e) { return reinterpret_cast<float *>(row) + (e & 1); }

__device__ __forceinline__ bool open_exact(double cx, double cy, double cz, double x, double y, double z,
                                           double tol2, double dsq)
{
    double dx = __dsub_rn(cx, x), dy = __dsub_rn(cy, y), dz = __dsub_rn(cz, z);
    double d2 = __dmul_rn(dx, dx);
    d2 = __dadd_rn(d2, __dmul_rn(dy, dy));
    d2 = __dadd_rn(d2, __dmul_rn(dz, dz));
    return __dmul_rn(tol2, d2) < dsq;
}

// gravsub (grav.c:42-73) for one cell in group-relative FP32; `on` = this
// lane's body takes the interaction.  Accumulates into the chunk partials.
template <bool QUAD>
__device__ __forceinline__ void cell_term(const float4 P, const float4 Q0, const float qyz, const float qzz, bool on,
                                          float bx, float by, float bz, float eps2, float &pphi, float &pax,
                                          float &pay, float &paz)
{
    const float dx = P.x - bx, dy = P.y - by, dz = P.z - bz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    const float rinv = rsqrtf(r2);
    const float rinv2 = rinv * rinv;
    const float mr = on ? P.w * rinv : 0.f;
    const float mr3 = mr * rinv2;
    if (!QUAD) {
        pphi -= mr;
        pax = fmaf(mr3, dx, pax);
        pay = fmaf(mr3, dy, pay);
        paz = fmaf(mr3, dz, paz);
        return;
    }
    const float qx = fmaf(Q0.x, dx, fmaf(Q0.y, dy, Q0.z * dz));
    const float qy = fmaf(Q0.y, dx, fmaf(Q0.w, dy, qyz * dz));
    const float qz = fmaf(Q0.z, dx, fmaf(qyz, dy, qzz * dz));
    const float dqd = fmaf(qx, dx, fmaf(qy, dy, qz * dz));
    const float r5 = (on ? rinv2 : 0.f) * (rinv2 * rinv);
    const float t = dqd * r5;                 // dr.Q.dr / r^5
    pphi -= fmaf(0.5f, t, mr);                // phi: -m/r - t/2
    // a = dr (m/r^3 + 5/2 t/r^2) - Q.dr / r^5: one coefficient on dr
    const float c = fmaf(2.5f * rinv2, t, mr3);
    pax = fmaf(c, dx, fmaf(-r5, qx, pax));
    pay = fmaf(c, dy, fmaf(-r5, qy, pay));
    paz = fmaf(c, dz, fmaf(-r5, qz, paz));
}

// MODE 0: the reference's per-body opening rule (exact interaction sets).
// MODE 1: group rule -- a cell is accepted for the whole group when
//         tol^2 * dmin^2 >= size^2 with dmin the distance from the group's
//         bounding box to the cell's centre of mass, else opened for all.
// MODE 2: group error rule -- accepted when the leading truncation error of
//         its expansion, m b^p / (dmin - b)^(p+2) (b: radius holding the
//         cell's bodies; p = 3 with quadrupoles, 2 without), is at most
//         eps_acc times the group's smallest |a| of the previous evaluation.
// COLLECT (learned walk only): the label walk -- analytic decisions, sampled
// band candidates recorded -- compiled as its own variant, so that the
// network's walk carries none of its code.
// Register budget: 96 (5 blocks of 4 warps per SM) for the per-body rule,
// 128 (4 blocks) for the group, error and learned rules.
template <bool QUAD, bool COUNT, int MODE, bool COLLECT = false>
__global__ void __launch_bounds__(WARPS * 32, MODE == 0 ? 5 : 4) k_walk(WalkArgs g)
{
    if (g.run_flag && *g.run_flag == 0) return;   // guard passed: no fallback walk
    // group criteria accept a cell for the whole group (a cell holding the
    // group's own bodies is always opened): cell entries need no lane mask
    constexpr bool MASKED = MODE == 0;
    extern __shared__ float4 smem_raw[];
    WarpSmem &S = reinterpret_cast<WarpSmem *>(smem_raw)[threadIdx.x >> 5];
    // MODE 3: per-warp queues after the warp areas, then the network's
    // weights, copied once per block (14 KB, read by every warp's rounds)
    QueueSmem *Qs = reinterpret_cast<QueueSmem *>(reinterpret_cast<WarpSmem *>(smem_raw) + WARPS) + (threadIdx.x >> 5);
    MlpSmem *Ms = reinterpret_cast<MlpSmem *>(reinterpret_cast<QueueSmem *>(reinterpret_cast<WarpSmem *>(smem_raw) + WARPS) + WARPS);
    if (MODE == 3 && g.mlp) {
        mlp_load(*Ms, g.mlp);
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    // Bodies per lane: the group criteria walk groups of up to 64 bodies
    // (bodies lane and lane + 32 on each lane: every list entry is loaded
    // once for both); the per-body rule, whose list entries carry one accept
    // bit per body, walks groups of up to 32.
    constexpr int BPL = MODE == 0 ? 1 : HC_BPL;
    constexpr int GW = 32 * BPL;
    const int64_t nmassive = g.use_table ? g.box->nmassive : 0;
    const int64_t ng_table = g.use_table ? g.box->ngroups : 0;
    const int64_t ngroups = ng_table + (g.ntarget - nmassive + GW - 1) / GW;
    const int nnode = g.box->nnode;
    const float tol2 = g.tol2f, eps2 = g.eps2f;
    // warp-uniform totals live in shared memory, not in registers
    if (lane < 8) S.stat[lane] = 0ull;
    __syncwarp();
    int max_sp = 0, nborder = 0;

    while (true) {
        int64_t grp;
        {
            unsigned v = 0;
            if (lane == 0) v = atomicAdd(g.group_counter, 1u);
            grp = (int64_t)__shfl_sync(FULL, v, 0);
        }
        if (grp >= ngroups) break;
        int64_t s0, cnt;
        if (grp < ng_table) {
            s0 = g.gstart[grp];
            cnt = g.gcount[grp];
        } else {
            s0 = nmassive + (grp - ng_table) * GW;
            cnt = g.ntarget - s0 < GW ? g.ntarget - s0 : GW;
        }
        // the group's bodies; an absent body repeats the lane's first (or the
        // group's first) so that it changes no group extent
        bool valid[BPL];
        uint32_t o[BPL];
        double xd[BPL], yd[BPL], zd[BPL];
#pragma unroll
        for (int k = 0; k < BPL; k++) {
            valid[k] = lane + 32 * k < cnt;
            o[k] = valid[k] ? g.tsorted[s0 + lane + 32 * k] : (k == 0 ? g.tsorted[s0] : o[0]);
            xd[k] = g.tx[o[k]];
            yd[k] = g.ty[o[k]];
            zd[k] = g.tz[o[k]];
        }
        const unsigned vmask = __ballot_sync(FULL, valid[0]);

        // group centre (FP64) and body positions relative to it (FP32)
        double gx, gy, gz;
        {
            double lox = xd[0], hix = xd[0], loy = yd[0], hiy = yd[0], loz = zd[0], hiz = zd[0];
#pragma unroll
            for (int k = 1; k < BPL; k++) {
                lox = fmin(lox, xd[k]);
                hix = fmax(hix, xd[k]);
                loy = fmin(loy, yd[k]);
                hiy = fmax(hiy, yd[k]);
                loz = fmin(loz, zd[k]);
                hiz = fmax(hiz, zd[k]);
            }
            gx = 0.5 * (wmind(lox) + wmaxd(hix));
            gy = 0.5 * (wmind(loy) + wmaxd(hiy));
            gz = 0.5 * (wmind(loz) + wmaxd(hiz));
        }
        const float ghx = __double2float_rn(gx), ghy = __double2float_rn(gy), ghz = __double2float_rn(gz);
        const float glx = __double2float_rn(gx - (double)ghx), gly = __double2float_rn(gy - (double)ghy),
                    glz = __double2float_rn(gz - (double)ghz);
        // low parts: body-body separations are formed as (hi - hi) + (lo - lo)
        float bx[BPL], by[BPL], bz[BPL], blx[BPL], bly[BPL], blz[BPL];
        float mnx = 3.0e38f, mxx = -3.0e38f, mny = 3.0e38f, mxy = -3.0e38f, mnz = 3.0e38f, mxz = -3.0e38f, r2m = 0.f;
#pragma unroll
        for (int k = 0; k < BPL; k++) {
            bx[k] = __double2float_rn(xd[k] - gx);
            by[k] = __double2float_rn(yd[k] - gy);
            bz[k] = __double2float_rn(zd[k] - gz);
            blx[k] = __double2float_rn((xd[k] - gx) - (double)bx[k]);
            bly[k] = __double2float_rn((yd[k] - gy) - (double)by[k]);
            blz[k] = __double2float_rn((zd[k] - gz) - (double)bz[k]);
            mnx = fminf(mnx, bx[k]);
            mxx = fmaxf(mxx, bx[k]);
            mny = fminf(mny, by[k]);
            mxy = fmaxf(mxy, by[k]);
            mnz = fminf(mnz, bz[k]);
            mxz = fmaxf(mxz, bz[k]);
            r2m = fmaxf(r2m, bx[k] * bx[k] + by[k] * by[k] + bz[k] * bz[k]);
        }
        const float gminx = wmin(mnx), gmaxx = wmax(mxx), gminy = wmin(mny), gmaxy = wmax(mxy), gminz = wmin(mnz),
                    gmaxz = wmax(mxz);
        const float rg2 = wmax(r2m);
        float amin = 0.f;                        // MODE 2: group's smallest |a| (previous evaluation)
        if (MODE >= 2) {
            float am = 3.0e38f;
#pragma unroll
            for (int k = 0; k < BPL; k++) {
                const float ax1 = (float)g.pax[o[k]], ay1 = (float)g.pay[o[k]], az1 = (float)g.paz[o[k]];
                if (valid[k]) am = fminf(am, sqrtf(fmaf(ax1, ax1, fmaf(ay1, ay1, az1 * az1))));
            }
            amin = wmin(am);
        }
        const float cR = 2e-6f * tol2 * rg2;     // absolute band term of the FP32 decision
        // Under the group criteria the traversal loop reads these warp-uniform
        // values from shared memory (volatile: not kept in registers), which
        // leaves its registers to the per-lane state; the per-body rule, which
        // reads them per lane in every mixed test, keeps them in registers.
        volatile float *gu = S.gu;
#define GUV(i, reg) (MODE == 0 ? (reg) : gu[i])
        __syncwarp();
        if (lane == 0) {
            const float v[15] = {ghx, ghy, ghz, glx, gly, glz, gminx, gmaxx, gminy, gmaxy, gminz, gmaxz, rg2, amin, cR};
#pragma unroll
            for (int k = 0; k < 15; k++) gu[k] = v[k];
        }
        __syncwarp();

        float sphi[BPL], sax[BPL], say[BPL], saz[BPL];    // Kahan sums per body
        float cphi[BPL], cax[BPL], cay[BPL], caz[BPL];
        int myb[BPL], myc[BPL];                            // per-body counts
#pragma unroll
        for (int k = 0; k < BPL; k++) {
            sphi[k] = sax[k] = say[k] = saz[k] = cphi[k] = cax[k] = cay[k] = caz[k] = 0.f;
            myb[k] = myc[k] = 0;
        }
        unsigned gb = 0, gc = 0;                           // this lane's accepted-node interactions

        // The list loops take two entries per step in packed FP32x2
        // arithmetic (each half rounds as the scalar instruction would); an odd
        // list is padded with a massless entry far from the group.  Both halves
        // are summed at the end of the flush, then added with Kahan's rule.
        // Body entries carry the accept mask (per-body rule) or the group slot
        // of the body that is the entry itself (group criteria; -1: none).
        const unsigned lanebit = 1u << lane;
        // bodies k of the lanes exist only for k < ceil(cnt / 32): the flushes
        // skip the others (warp-uniform)
        const int nact = (int)((cnt + 31) / 32);
        auto pad_entry = [&](float4 *row, int e, int nq) {
            float *f = pair_slot(row, e);
            f[0] = 1.0e4f;
            f[2] = 1.0e4f;
            f[4] = 1.0e4f;
            for (int k = 3; k < nq; k++) f[2 * k] = 0.f;
        };
        auto flush_bodies = [&](int nb) {
            if (lane == 0) {
                S.stat[ST_EB] += nb;
                if (nb & 1) {
                    pad_entry(S.bp[nb >> 1], nb, 8);
                    if (MODE != 0) pair_slot(S.bp[nb >> 1], nb)[14] = __int_as_float(-1);
                }
            }
            __syncwarp();
            float2 nphi[BPL], ax[BPL], ay[BPL], az[BPL];
#pragma unroll
            for (int k = 0; k < BPL; k++) nphi[k] = ax[k] = ay[k] = az[k] = splat2(0.f);
            const float2 e2 = splat2(eps2);
            for (int p = 0; p < (nb + 1) >> 1; p++) {
                const float4 H0 = S.bp[p][0], H1 = S.bp[p][1], L0 = S.bp[p][2], L1 = S.bp[p][3];
#pragma unroll
                for (int k = 0; k < BPL; k++) {
                    if (k > 0 && k >= nact) continue;
                    const float2 dx = __fadd2_rn(__fadd2_rn(lo2(H0), splat2(-bx[k])), __fadd2_rn(lo2(L0), splat2(-blx[k])));
                    const float2 dy = __fadd2_rn(__fadd2_rn(hi2(H0), splat2(-by[k])), __fadd2_rn(hi2(L0), splat2(-bly[k])));
                    const float2 dz = __fadd2_rn(__fadd2_rn(lo2(H1), splat2(-bz[k])), __fadd2_rn(lo2(L1), splat2(-blz[k])));
                    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
                    bool b0, b1;
                    if (MODE == 0) {
                        b0 = __float_as_uint(L1.z) & lanebit;
                        b1 = __float_as_uint(L1.w) & lanebit;
                    } else {
                        b0 = __float_as_int(L1.z) != lane + 32 * k;
                        b1 = __float_as_int(L1.w) != lane + 32 * k;
                    }
                    const float2 w = make_float2(b0 ? rsqrtf(r2.x) : 0.f, b1 ? rsqrtf(r2.y) : 0.f);
                    const float2 mr = __fmul2_rn(hi2(H1), w);
                    const float2 mr3 = __fmul2_rn(mr, __fmul2_rn(w, w));
                    nphi[k] = __fadd2_rn(nphi[k], mr);
                    ax[k] = __ffma2_rn(mr3, dx, ax[k]);
                    ay[k] = __ffma2_rn(mr3, dy, ay[k]);
                    az[k] = __ffma2_rn(mr3, dz, az[k]);
                    if (COUNT) myb[k] += (int)b0 + (int)b1;
                }
            }
#pragma unroll
            for (int k = 0; k < BPL; k++) {
                if (COUNT && MODE != 0 && (nb & 1)) myb[k] -= 1;      // the pad counted as a body
                kahan_add(sphi[k], cphi[k], -(nphi[k].x + nphi[k].y));
                kahan_add(sax[k], cax[k], ax[k].x + ax[k].y);
                kahan_add(say[k], cay[k], ay[k].x + ay[k].y);
                kahan_add(saz[k], caz[k], az[k].x + az[k].y);
            }
        };
        auto flush_cells = [&](int nc) {
            if (lane == 0) {
                S.stat[ST_EC] += nc;
                if (nc & 1) {
                    pad_entry(S.cp[nc >> 1], nc, QUAD ? 10 : 4);
                    if (MASKED) S.cmask[nc >> 1].y = 0u;
                }
            }
            __syncwarp();
            float2 nphi[BPL], ax[BPL], ay[BPL], az[BPL];
#pragma unroll
            for (int k = 0; k < BPL; k++) nphi[k] = ax[k] = ay[k] = az[k] = splat2(0.f);
            const float2 e2 = splat2(eps2);
#pragma unroll 2
            for (int p = 0; p < (nc + 1) >> 1; p++) {
                const float4 P0 = S.cp[p][0], P1 = S.cp[p][1];
                bool m0 = true, m1 = true;
                if (MASKED) {
                    const uint2 mk = S.cmask[p];
                    m0 = mk.x & lanebit;
                    m1 = mk.y & lanebit;
                    if (COUNT) myc[0] += (int)m0 + (int)m1;
                }
                float4 Q0, Q1, Q2;
                if (QUAD) {
                    Q0 = S.cp[p][2];
                    Q1 = S.cp[p][3];
                    Q2 = S.cp[p][4];
                }
#pragma unroll
                for (int k = 0; k < BPL; k++) {
                    if (k > 0 && k >= nact) continue;
                    const float2 dx = __fadd2_rn(lo2(P0), splat2(-bx[k])), dy = __fadd2_rn(hi2(P0), splat2(-by[k])),
                                 dz = __fadd2_rn(lo2(P1), splat2(-bz[k]));
                    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
                    float2 w = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                    const float2 rinv2 = __fmul2_rn(w, w);
                    if (MASKED) w = make_float2(m0 ? w.x : 0.f, m1 ? w.y : 0.f);
                    const float2 mr = __fmul2_rn(hi2(P1), w);            // m / r (0 for a masked lane)
                    const float2 mr3 = __fmul2_rn(mr, rinv2);
                    if (!QUAD) {
                        nphi[k] = __fadd2_rn(nphi[k], mr);
                        ax[k] = __ffma2_rn(mr3, dx, ax[k]);
                        ay[k] = __ffma2_rn(mr3, dy, ay[k]);
                        az[k] = __ffma2_rn(mr3, dz, az[k]);
                        continue;
                    }
                    // gravsub's quadrupole term (grav.c:62-72) with the list's -Q:
                    // q = -Q.dr, t = -dr.Q.dr / r^5
                    const float2 qx = __ffma2_rn(lo2(Q0), dx, __ffma2_rn(hi2(Q0), dy, __fmul2_rn(lo2(Q1), dz)));
                    const float2 qy = __ffma2_rn(hi2(Q0), dx, __ffma2_rn(hi2(Q1), dy, __fmul2_rn(lo2(Q2), dz)));
                    const float2 qz = __ffma2_rn(lo2(Q1), dx, __ffma2_rn(lo2(Q2), dy, __fmul2_rn(hi2(Q2), dz)));
                    const float2 dqd = __ffma2_rn(qx, dx, __ffma2_rn(qy, dy, __fmul2_rn(qz, dz)));
                    const float2 r5 = __fmul2_rn(__fmul2_rn(w, rinv2), rinv2);
                    const float2 t = __fmul2_rn(dqd, r5);
                    // -phi += m/r + dr.Q.dr / (2 r^5);  a += dr (m/r^3 + 5/2 dr.Q.dr/r^7) - Q.dr / r^5
                    nphi[k] = __ffma2_rn(splat2(-0.5f), t, __fadd2_rn(nphi[k], mr));
                    const float2 c = __ffma2_rn(__fmul2_rn(splat2(-2.5f), rinv2), t, mr3);
                    ax[k] = __ffma2_rn(c, dx, __ffma2_rn(r5, qx, ax[k]));
                    ay[k] = __ffma2_rn(c, dy, __ffma2_rn(r5, qy, ay[k]));
                    az[k] = __ffma2_rn(c, dz, __ffma2_rn(r5, qz, az[k]));
                }
            }
#pragma unroll
            for (int k = 0; k < BPL; k++) {
                if (COUNT && !MASKED) myc[k] += nc;
                kahan_add(sphi[k], cphi[k], -(nphi[k].x + nphi[k].y));
                kahan_add(sax[k], cax[k], ax[k].x + ax[k].y);
                kahan_add(say[k], cay[k], ay[k].x + ay[k].y);
                kahan_add(saz[k], caz[k], az[k].x + az[k].y);
            }
        };

        int sp = 0, nb = 0, nc = 0;
        bool overflow = false;
        int root = 0;
        if (g.sys_root) {                     // forest: this group's system root
            root = g.sys_root[g.body_sys[__shfl_sync(FULL, o[0], 0)]];
            if (root < 0 || root >= nnode) {
                if (lane == 0) atomicCAS(&g.st->error, 0, HC_ERR_STATE);
                continue;
            }
        }
        if (nnode > 0) {
            if (lane == 0) S.stack[0] = make_uint2((unsigned)root << 3, vmask);   // root, one node
            sp = 1;
        }
        __syncwarp();
        int qn = 0;                                          // MODE 3: queued band candidates
        while (sp > 0 || qn > 0) {
            int ncand = 0, my_node = 0;
            unsigned my_mask = 0;
            // MODE 3: a network round decides the first (up to) 32 queued candidates
            const bool mlp_round = MODE == 3 && (qn >= 32 || sp == 0);
            float logit = 0.f, q_dmin2 = 0.f, q_dmax2 = 0.f, q_err = 1.f;
            if (mlp_round) {
                ncand = qn < 32 ? qn : 32;
                if (lane < ncand) {
                    my_node = Qs->node[lane];
                    my_mask = Qs->mask[lane];
                    q_dmin2 = Qs->dmin2[lane];
                    q_dmax2 = Qs->dmax2[lane];
                    q_err = Qs->err[lane];
                }
                __syncwarp();
                // shift the rest of the queue down
                const int rest = qn - ncand;
                if (lane < rest) {
                    Qs->node[lane] = Qs->node[32 + lane];
                    Qs->mask[lane] = Qs->mask[32 + lane];
                    Qs->dmin2[lane] = Qs->dmin2[32 + lane];
                    Qs->dmax2[lane] = Qs->dmax2[32 + lane];
                    Qs->err[lane] = Qs->err[32 + lane];
                }
                qn = rest;
                if (lane == 0) {
                    S.stat[ST_MLP] += ncand;
                    S.stat[ST_ROUNDS]++;
                }
            }
            // ---- gather up to 32 candidates from the top of the stack ----
            // Each candidate taken adds at most one entry (its child range), so
            // taking at most half the free entries keeps the stack within
            // capacity; near it the walk takes fewer candidates per iteration,
            // down to one, instead of dropping to one at a fixed threshold.
            const int gfree = (STACK - sp) / 2;
            const int gmax = gfree >= 32 ? 32 : (gfree >= 1 ? gfree : 1);
            while (!mlp_round && ncand < gmax && sp > 0) {
                const uint2 e = S.stack[sp - 1];
                const int start = (int)(e.x >> 3), ecnt = (int)(e.x & 7u) + 1;
                const int take = min(ecnt, gmax - ncand);
                const int rel = lane - ncand;
                if (rel >= 0 && rel < take) {
                    my_node = start + ecnt - take + rel;
                    my_mask = e.y;
                }
                ncand += take;
                if (take == ecnt) sp--;
                else if (lane == 0) S.stack[sp - 1].x = ((unsigned)start << 3) | (unsigned)(ecnt - take - 1);
            }
            __syncwarp();
            const bool have = lane < ncand && my_node < nnode;
            if (lane < ncand && my_node >= nnode) atomicCAS(&g.st->error, 0, HC_ERR_STATE);

            // ---- classify each candidate against the group ----
            float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A;
            int2 C = make_int2(0, 0);
            if (have) {
                A = g.nodeA[my_node];
                B = g.nodeB[my_node];
                C = g.nodeC[my_node];
            }
            if (MODE == 3 && mlp_round) {
                // lane r builds the feature row of the round's candidate r (rows
                // beyond the round are zero); then the warp evaluates the network
                uint32_t *row = reinterpret_cast<uint32_t *>(Qs->x) + lane * (MLP_XS / 2);
                uint32_t w[6] = {0u, 0u, 0u, 0u, 0u, 0u};
                if (have) {
                    const float4 Q0 = g.nodeQ[2 * (int64_t)my_node], Q1 = g.nodeQ[2 * (int64_t)my_node + 1];
                    float f[12];
                    cell_features_inl(f, q_dmin2, q_dmax2, B.w, A.w, Q1.w, q_dmin2 * rsqrtf(q_dmin2) - Q1.w, Q0, Q1, GUV(13, amin), GUV(12, rg2),
                                      eps2, C.y >> 8, (int)cnt,
                                      __log2f(fmaxf(q_err, 1e-38f)) - __log2f(g.eps_acc * GUV(13, amin)));
#pragma unroll
                    for (int k = 0; k < 6; k++) w[k] = pack_bf16(f[2 * k], f[2 * k + 1]);
                }
#pragma unroll
                for (int k = 0; k < 6; k++) row[k] = w[k];
#pragma unroll
                for (int k = 6; k < MLP_XS / 2; k++) row[k] = 0u;
                __syncwarp();
                logit = mlp_warp_lean(*Ms, Qs->x, Qs->z, ncand);
            }
            const float cx = (A.x - GUV(0, ghx)) + (B.x - GUV(3, glx)), cy = (A.y - GUV(1, ghy)) + (B.y - GUV(4, gly)), cz = (A.z - GUV(2, ghz)) + (B.z - GUV(5, glz));
            const bool isbody = C.x < 0;
            unsigned openm = 0, accm = 0;
            int selfslot = -1;                 // group criteria: group slot of a body leaf in the group
            bool mixed = false;
            bool band = false;                 // MODE 3: queued for the network
            float bd_dmin2 = 0.f, bd_dmax2 = 0.f, bd_err = 0.f;
            if (have) {
                if (isbody) {
                    const int64_t slot = (int64_t)(-1 - C.x) - s0;     // leaf holds its massive rank
                    if (MODE == 0) {
                        const unsigned self = (g.self_mode && slot >= 0 && slot < 32) ? (1u << slot) : 0u;
                        accm = my_mask & ~self;
                    } else {
                        selfslot = (g.self_mode && slot >= 0 && slot < cnt) ? (int)slot : -1;
                        accm = cnt > (selfslot >= 0 ? 1 : 0) ? my_mask : 0u;
                    }
                } else {
                    const float dsq = B.w;
                    const float ex = fmaxf(0.f, fmaxf(GUV(6, gminx) - cx, cx - GUV(7, gmaxx)));
                    const float ey = fmaxf(0.f, fmaxf(GUV(8, gminy) - cy, cy - GUV(9, gmaxy)));
                    const float ez = fmaxf(0.f, fmaxf(GUV(10, gminz) - cz, cz - GUV(11, gmaxz)));
                    const float fx = fmaxf(fabsf(cx - GUV(6, gminx)), fabsf(cx - GUV(7, gmaxx)));
                    const float fy = fmaxf(fabsf(cy - GUV(8, gminy)), fabsf(cy - GUV(9, gmaxy)));
                    const float fz = fmaxf(fabsf(cz - GUV(10, gminz)), fabsf(cz - GUV(11, gmaxz)));
                    const float dmin2 = ex * ex + ey * ey + ez * ez;
                    const float dmax2 = fx * fx + fy * fy + fz * fz;
                    const float tmin = tol2 * dmin2, tmax = tol2 * dmax2;
                    if (MODE == 3 && mlp_round) {
                        if (logit > g.mlp_threshold) accm = my_mask;
                        else openm = my_mask;
                    } else if (MODE == 1 || (MODE >= 2 && !(GUV(13, amin) > 0.f))) {
                        const bool acc = (MODE == 1 && g.rcrit2) ? dmin2 > g.rcrit2[my_node] : tmin >= dsq;
                        if (acc) accm = my_mask;
                        else openm = my_mask;
                    } else if (MODE == 3) {
                        const float4 Q1 = g.nodeQ[2 * (int64_t)my_node + 1];
                        const float b = Q1.w;
                        // approximate square root and reciprocal: the proxy decides
                        // nothing exactly (dmin2 = 0 gives a NaN gap: opened)
                        const float gap = dmin2 * rsqrtf(dmin2) - b;
                        float err = 3.0e38f;           // no expansion (gap <= 0 or size/dmin > 4): open
                        if (gap > 0.f && tmin >= dsq * 0.0625f) {
                            const float gi = __fdividef(1.f, gap), bg = b * gi;
                            err = A.w * gi * gi * bg * bg * (QUAD ? bg : 1.f);
                        }
                        const float budget = g.eps_acc * GUV(13, amin);
                        if (err < budget * g.band_lo_f) accm = my_mask;          // below the band
                        else if (err > budget * g.band_hi_f) openm = my_mask;    // above it
                        else if (COLLECT) {
                            // label walk: analytic decision, sampled record of the band candidate
                            const float p_raw = __log2f(fmaxf(err, 1e-38f)) - __log2f(budget);
                            if (err <= budget) accm = my_mask;
                            else openm = my_mask;
                            if ((hash2((unsigned)grp, (unsigned)my_node) >> 8) < g.keep24) {
                                const int slot = atomicAdd(g.sample_count, 1);
                                if (slot < g.sample_cap) {
                                    float f[12];
                                    cell_features(f, dmin2, dmax2, dsq, A.w, b, gap, g.nodeQ[2 * (int64_t)my_node], Q1,
                                                  GUV(13, amin), GUV(12, rg2), eps2, C.y >> 8, (int)cnt, p_raw);
                                    for (int k = 0; k < 12; k++) g.sample_x[(int64_t)slot * 12 + k] = f[k];
                                    g.sample_group[slot] = (int)grp;
                                    g.sample_node[slot] = my_node;
                                    g.sample_amin[slot] = GUV(13, amin);
                                }
                            }
                        } else {
                            // queue for the network: decision in a later round
                            band = true;
                            bd_dmin2 = dmin2;
                            bd_dmax2 = dmax2;
                            bd_err = err;
                        }
                    } else if (MODE == 2) {
                        const float b = g.nodeQ[2 * (int64_t)my_node + 1].w;
                        const float gap = dmin2 * rsqrtf(dmin2) - b;          // as in MODE 3
                        bool acc_ok = gap > 0.f && tmin >= dsq * 0.0625f;     // never beyond size/dmin = 4
                        if (acc_ok) {
                            const float gi = __fdividef(1.f, gap), bg = b * gi;
                            const float err = A.w * gi * gi * bg * bg * (QUAD ? bg : 1.f);
                            acc_ok = err <= g.eps_acc * GUV(13, amin);
                        }
                        if (acc_ok) accm = my_mask;
                        else openm = my_mask;
                    } else if (tmin - dsq > 8e-6f * tmin + GUV(14, cR)) accm = my_mask;  // every body accepts
                    else if (dsq - tmax > 8e-6f * tmax + GUV(14, cR)) openm = my_mask;    // every body opens
                    else mixed = true;
                }
            }
            if (MODE == 3) {                   // enqueue band candidates
                // (the warp syncs at the end of this iteration order these
                // writes before the round that reads them)
                const unsigned qb = __ballot_sync(FULL, band);
                if (qb) {
                    if (band) {
                        const int row = qn + __popc(qb & lt);
                        Qs->node[row] = my_node;
                        Qs->mask[row] = my_mask;
                        Qs->dmin2[row] = bd_dmin2;
                        Qs->dmax2[row] = bd_dmax2;
                        Qs->err[row] = bd_err;
                    }
                    qn += __popc(qb);
                }
            }
            unsigned mixedb = MODE == 0 ? __ballot_sync(FULL, mixed) : 0u;
            if (lane == 0) {
                S.stat[ST_CAND] += ncand;
                S.stat[ST_MIXED] += __popc(mixedb);
            }
            while (mixedb) {
                const int j = __ffs(mixedb) - 1;
                mixedb &= mixedb - 1;
                const float jx = __shfl_sync(FULL, cx, j), jy = __shfl_sync(FULL, cy, j),
                            jz = __shfl_sync(FULL, cz, j), jd = __shfl_sync(FULL, B.w, j);
                const unsigned jm = __shfl_sync(FULL, my_mask, j);
                const int jn = __shfl_sync(FULL, my_node, j);
                const int jdepth = __shfl_sync(FULL, C.y, j) >> 8;
                const bool in = (jm >> lane) & 1u;
                const float dx = jx - bx[0], dy = jy - by[0], dz = jz - bz[0];
                const float d2 = dx * dx + dy * dy + dz * dz;
                const float t = tol2 * d2 - jd;
                bool op = t < 0.f;
                if (in && fabsf(t) <= 8e-6f * tol2 * d2 + GUV(14, cR)) {
                    // borderline: decide exactly as subdivp does, in FP64
                    op = open_exact(g.ncx[jn], g.ncy[jn], g.ncz[jn], xd[0], yd[0], zd[0], g.tol2d, g.box->dsq[jdepth]);
                    nborder++;
                }
                const unsigned ob = __ballot_sync(FULL, in && op), ab = __ballot_sync(FULL, in && !op);
                if (lane == j) {
                    openm = ob;
                    accm = ab;
                }
            }

            // ---- push opened cells' child ranges ----
            // children always follow their parent and number 1..8
            const bool push = openm != 0u && C.x > my_node && (C.y & 255) >= 1 && (C.y & 255) <= 8;
            const unsigned pb = __ballot_sync(FULL, push);
            const int npush = __popc(pb);
            if (sp + npush > STACK) {
                overflow = true;
                break;
            }
            if (push)
                S.stack[sp + __popc(pb & lt)] = make_uint2(((unsigned)C.x << 3) | (unsigned)((C.y & 255) - 1), openm);
            sp += npush;
            if (sp > max_sp) max_sp = sp;

            // ---- append accepted nodes to the interaction lists ----
            const bool ab = accm != 0u && isbody, ac = accm != 0u && !isbody;
            // histogram of the bodies an accepted node serves, in lanes (HC_BPL bodies per lane for the group criteria)
            if (COUNT && accm != 0u) atomicAdd(&g.st->mask_hist[MODE == 0 ? __popc(accm) : (int)(cnt + BPL - 1) / BPL], 1ull);
            const unsigned bbal = __ballot_sync(FULL, ab), cbal = __ballot_sync(FULL, ac);
            if (ab) {
                // node - centre as an unevaluated float sum hi + lo (TwoSum of the hi parts)
                const int pos = nb + __popc(bbal & lt);
                float hx, hy, hz, ex, ey, ez;
                two_diff(A.x, GUV(0, ghx), hx, ex);
                two_diff(A.y, GUV(1, ghy), hy, ey);
                two_diff(A.z, GUV(2, ghz), hz, ez);
                float *f = pair_slot(S.bp[pos >> 1], pos);
                f[0] = hx;
                f[2] = hy;
                f[4] = hz;
                f[6] = A.w;
                f[8] = ex + (B.x - GUV(3, glx));
                f[10] = ey + (B.y - GUV(4, gly));
                f[12] = ez + (B.z - GUV(5, glz));
                f[14] = MODE == 0 ? __uint_as_float(accm) : __int_as_float(selfslot);
                gb += MODE == 0 ? __popc(accm) : (unsigned)cnt - (selfslot >= 0 ? 1u : 0u);
            }
            if (ac) {
                const int pos = nc + __popc(cbal & lt);
                float *f = pair_slot(S.cp[pos >> 1], pos);
                f[0] = cx;
                f[2] = cy;
                f[4] = cz;
                f[6] = A.w;
                if (QUAD) {
                    const float4 q0 = g.nodeQ[2 * (int64_t)my_node], q1 = g.nodeQ[2 * (int64_t)my_node + 1];
                    f[8] = -q0.x;
                    f[10] = -q0.y;
                    f[12] = -q0.z;
                    f[14] = -q0.w;
                    f[16] = -q1.x;
                    f[18] = -q1.y;
                }
                if (MASKED) (pos & 1 ? S.cmask[pos >> 1].y : S.cmask[pos >> 1].x) = accm;
                gc += MODE == 0 ? __popc(accm) : (unsigned)cnt;
            }
            nb += __popc(bbal);
            nc += __popc(cbal);
            __syncwarp();
            if (nb > g.flush_at) {
                flush_bodies(nb);
                nb = 0;
            }
            if (nc > g.flush_at) {
                flush_cells(nc);
                nc = 0;
            }
            __syncwarp();
        }
#undef GUV
        if (overflow) {
            if (lane == 0) {
                atomicCAS(&g.st->error, 0, HC_ERR_STACK);
                g.st->info = STACK;
            }
            continue;
        }
        if (nb) flush_bodies(nb);
        if (nc) flush_cells(nc);
        {
            unsigned long long sb = gb, sc = gc;           // group totals (up to 32 n: 64-bit)
#pragma unroll
            for (int off = 16; off; off >>= 1) {
                sb += __shfl_xor_sync(FULL, sb, off);
                sc += __shfl_xor_sync(FULL, sc, off);
            }
            if (lane == 0) {
                S.stat[ST_N2B] += sb;
                S.stat[ST_NBC] += sc;
            }
        }
        __syncwarp();

#pragma unroll
        for (int k = 0; k < BPL; k++) {
            if (!valid[k]) continue;
            const uint32_t ok = o[k];
            const double rphi = (double)sphi[k] - (double)cphi[k];
            const double rax = (double)sax[k] - (double)cax[k], ray = (double)say[k] - (double)cay[k],
                         raz = (double)saz[k] - (double)caz[k];
            if (g.kick_dthf != 0.0 && g.nstep > 0) {
                // closing half kick with the new acceleration (code.c:175-179)
                g.vx[ok] = __dadd_rn(g.vx[ok], __dmul_rn(__dsub_rn(rax, g.oax[ok]), g.kick_dthf));
                g.vy[ok] = __dadd_rn(g.vy[ok], __dmul_rn(__dsub_rn(ray, g.oay[ok]), g.kick_dthf));
                g.vz[ok] = __dadd_rn(g.vz[ok], __dmul_rn(__dsub_rn(raz, g.oaz[ok]), g.kick_dthf));
            }
            g.oax[ok] = rax;
            g.oay[ok] = ray;
            g.oaz[ok] = raz;
            g.ophi[ok] = rphi;
            if (COUNT) {
                g.cnt_b[ok] = myb[k];
                g.cnt_c[ok] = myc[k];
            }
        }
    }
    // interaction totals and stats
#pragma unroll
    for (int off = 16; off; off >>= 1) nborder += __shfl_xor_sync(FULL, nborder, off);
    __syncwarp();
    if (lane == 0) {
        atomicAdd(&g.st->n2b, S.stat[ST_N2B]);
        atomicAdd(&g.st->nbc, S.stat[ST_NBC]);
        atomicMax(&g.st->max_stack, max_sp);
        atomicAdd(&g.st->nborder, nborder);
        atomicAdd(&g.st->ncand, S.stat[ST_CAND]);
        atomicAdd(&g.st->nmixed, S.stat[ST_MIXED]);
        atomicAdd(&g.st->nentry_b, S.stat[ST_EB]);
        atomicAdd(&g.st->nentry_c, S.stat[ST_EC]);
        if (MODE == 3) {
            atomicAdd(&g.st->nmlp, S.stat[ST_MLP]);
            atomicAdd(&g.st->nmlp_rounds, S.stat[ST_ROUNDS]);
        }
    }
}

constexpr size_t walk_smem(int mode)
{
    return sizeof(WarpSmem) * WARPS + (mode == 3 ? sizeof(QueueSmem) * WARPS + sizeof(MlpSmem) : 0);
}

template <bool Q, bool C, int M, bool L = false>
int configure(hc_ctx *c, int variant)
{
    const size_t smem = walk_smem(M);
    HC_CUDA(cudaFuncSetAttribute(k_walk<Q, C, M, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, nsm = 0, per_sm = 0;
    HC_CUDA(cudaGetDevice(&dev));
    HC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    HC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<Q, C, M, L>, WARPS * 32, smem));
    c->walk_blocks[variant] = nsm * (per_sm < 1 ? 1 : per_sm);
    return HC_OK;
}

// No CUDA queries here: this runs inside stream capture.
template <bool Q, bool C, int M, bool L = false>
int launch(hc_ctx *c, WalkArgs &a, int variant)
{
    const size_t smem = walk_smem(M);
    int64_t blocks = c->walk_blocks[variant];               // persistent: groups are fetched dynamically
    int64_t need = ((a.ntarget + 31) / 32 + WARPS - 1) / WARPS;
    if (!a.use_table && blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    k_walk<Q, C, M, L><<<(unsigned)blocks, WARPS * 32, smem, c->stream>>>(a);
    c->launches++;
    return HC_OK;
}

}  // namespace

int hc_walk_launch(hc_ctx *c, bool self, int64_t ntarget, const uint32_t *tsorted, const double *tx,
                   const double *ty, const double *tz, double *oax, double *oay, double *oaz, double *ophi,
                   double kick_dthf, int64_t nstep, const int *run_flag, bool body_rule)
{
    if (ntarget <= 0) return HC_OK;
    WalkArgs a;
    a.run_flag = run_flag;
    a.rcrit2 = nullptr;
    {
        const int depth = c->list_depth >= 32 && c->list_depth <= BCAP ? c->list_depth : BCAP;
        a.flush_at = depth - 32;          // an iteration appends at most 32 entries
    }
    a.sys_root = self ? c->walk_sys_root : nullptr;
    a.body_sys = c->walk_body_sys;
    a.nodeA = c->nodeA;
    a.nodeB = c->nodeB;
    a.nodeQ = c->nodeQ;
    a.nodeC = c->nodeC;
    a.ncx = c->ncx;
    a.ncy = c->ncy;
    a.ncz = c->ncz;
    a.box = c->box;
    a.ntarget = ntarget;
    a.tsorted = tsorted;
    a.tx = tx;
    a.ty = ty;
    a.tz = tz;
    a.self_mode = self ? 1 : 0;
    a.tol2d = c->prm.tol * c->prm.tol;
    a.tol2f = (float)a.tol2d;
    a.eps2f = (float)(c->prm.eps * c->prm.eps);
    a.oax = oax;
    a.oay = oay;
    a.oaz = oaz;
    a.ophi = ophi;
    a.cnt_b = c->cnt_b;
    a.cnt_c = c->cnt_c;
    a.kick_dthf = kick_dthf;
    a.nstep = nstep;
    a.vx = c->vx;
    a.vy = c->vy;
    a.vz = c->vz;
    a.st = c->st;
    a.group_counter = (unsigned *)(c->st + 1);
    a.pax = c->ax;
    a.pay = c->ay;
    a.paz = c->az;
    a.gstart = c->gstart;
    a.gcount = c->gcount;
    // group criteria walk the tree groups (up to 64 bodies); the per-body
    // rule walks them when chosen and they hold at most 32 bodies (its own
    // criterion), else 32 consecutive bodies (also the guard's fallback walk)
    const bool per_body = body_rule || c->criterion == HC_CRITERION_BODY;
    a.use_table = (self && (!per_body || (c->criterion == HC_CRITERION_BODY && c->group_kind == 1))) ? 1 : 0;
    HC_CUDA(cudaMemsetAsync(a.group_counter, 0, sizeof(unsigned), c->stream));
    const bool count = c->prm.count_per_body && self && c->cnt_b;
    const int v = (c->prm.usequad ? 2 : 0) + (count ? 1 : 0);
    a.eps_acc = (float)c->group_theta;
    const bool rc = c->criterion == HC_CRITERION_BH86 || c->criterion == HC_CRITERION_SW94 ||
                    c->criterion == HC_CRITERION_BARNES;
    if (!body_rule && (c->criterion == HC_CRITERION_GROUP || rc)) {
        if (rc) a.rcrit2 = c->rcrit2;
        a.tol2d = c->group_theta * c->group_theta;
        a.tol2f = (float)a.tol2d;
        switch (v) {
        case 0: return launch<false, false, 1>(c, a, 4);
        case 1: return launch<false, true, 1>(c, a, 5);
        case 2: return launch<true, false, 1>(c, a, 6);
        default: return launch<true, true, 1>(c, a, 7);
        }
    }
    if (!body_rule && c->criterion == HC_CRITERION_LEARNED) {
        a.tol2d = 0.25;     // fallback geometric rule (no previous accelerations): theta = 0.5
        a.tol2f = 0.25f;
        a.mlp = c->mlp_packed;
        a.mlp_threshold = c->mlp_threshold;
        a.band_lo_f = exp2f(-c->mlp_band);
        a.band_hi_f = exp2f(c->mlp_band_hi);
        a.collect = c->collect;
        a.keep24 = c->keep24;
        a.sample_cap = c->collect_cap;
        a.sample_count = c->sample_count;
        a.sample_x = c->sample_x;
        a.sample_group = c->sample_group;
        a.sample_node = c->sample_node;
        a.sample_amin = c->sample_amin;
        if (a.collect) {
            switch (v) {
            case 0: return launch<false, false, 3, true>(c, a, 16);
            case 1: return launch<false, true, 3, true>(c, a, 17);
            case 2: return launch<true, false, 3, true>(c, a, 18);
            default: return launch<true, true, 3, true>(c, a, 19);
            }
        }
        switch (v) {
        case 0: return launch<false, false, 3>(c, a, 12);
        case 1: return launch<false, true, 3>(c, a, 13);
        case 2: return launch<true, false, 3>(c, a, 14);
        default: return launch<true, true, 3>(c, a, 15);
        }
    }
    if (!body_rule && c->criterion == HC_CRITERION_ERROR) {
        a.tol2d = 1.0;      // fallback geometric rule (no previous accelerations): theta = 1
        a.tol2f = 1.0f;
        switch (v) {
        case 0: return launch<false, false, 2>(c, a, 8);
        case 1: return launch<false, true, 2>(c, a, 9);
        case 2: return launch<true, false, 2>(c, a, 10);
        default: return launch<true, true, 2>(c, a, 11);
        }
    }
    switch (v) {
    case 0: return launch<false, false, 0>(c, a, 0);
    case 1: return launch<false, true, 0>(c, a, 1);
    case 2: return launch<true, false, 0>(c, a, 2);
    default: return launch<true, true, 0>(c, a, 3);
    }
}

int hc_walk_setup(hc_ctx *c)
{
    int r = configure<false, false, 0>(c, 0);
    if (r == HC_OK) r = configure<false, true, 0>(c, 1);
    if (r == HC_OK) r = configure<true, false, 0>(c, 2);
    if (r == HC_OK) r = configure<true, true, 0>(c, 3);
    if (r == HC_OK) r = configure<false, false, 1>(c, 4);
    if (r == HC_OK) r = configure<false, true, 1>(c, 5);
    if (r == HC_OK) r = configure<true, false, 1>(c, 6);
    if (r == HC_OK) r = configure<true, true, 1>(c, 7);
    if (r == HC_OK) r = configure<false, false, 2>(c, 8);
    if (r == HC_OK) r = configure<false, true, 2>(c, 9);
    if (r == HC_OK) r = configure<true, false, 2>(c, 10);
    if (r == HC_OK) r = configure<true, true, 2>(c, 11);
    if (r == HC_OK) r = configure<false, false, 3>(c, 12);
    if (r == HC_OK) r = configure<false, true, 3>(c, 13);
    if (r == HC_OK) r = configure<true, false, 3>(c, 14);
    if (r == HC_OK) r = configure<true, true, 3>(c, 15);
    if (r == HC_OK) r = configure<false, false, 3, true>(c, 16);
    if (r == HC_OK) r = configure<false, true, 3, true>(c, 17);
    if (r == HC_OK) r = configure<true, false, 3, true>(c, 18);
    if (r == HC_OK) r = configure<true, true, 3, true>(c, 19);
    return r;
}

// ---------------- labels for the learned criterion ----------------
// For each sampled (group, cell) pair: the cell's multipole acceleration at
// every body of the group against a refined reference -- the cell's subtree
// walked with one decision per group, a node accepted only when its mass
// radius b satisfies b / (dmin - b) < 0.1 (so the reference's own truncation
// error is ~1e-3 of the cell's).  label = 1 if the largest relative error
// |a_multipole - a_reference| / |a_body| of the group is at most eps.
namespace {
constexpr int LSTACK = 256;
template <bool QUAD>
__global__ void __launch_bounds__(128) k_label(WalkArgs g, const int *gstart, const int *gcount, const uint32_t *tord,
                                               const double *px, const double *py, const double *pz,
                                               const double *ax, const double *ay, const double *az,
                                               const int *sample_group, const int *sample_node, int nsample,
                                               float eps_label, float *y, float *rel_out)
{
    __shared__ int stk[4][LSTACK];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * 4 + w;
    if (i >= nsample) return;
    const int grp = sample_group[i], node = sample_node[i];
    const int s0 = gstart[grp], cnt = gcount[grp];
    // groups of up to 32 HC_BPL bodies: bodies lane + 32 k on each lane
    constexpr int BPL = HC_BPL;
    bool valid[BPL];
    uint32_t o[BPL];
    double xd[BPL], yd[BPL], zd[BPL];
#pragma unroll
    for (int k = 0; k < BPL; k++) {
        valid[k] = lane + 32 * k < cnt;
        o[k] = valid[k] ? tord[s0 + lane + 32 * k] : (k == 0 ? tord[s0] : o[0]);
        xd[k] = px[o[k]];
        yd[k] = py[o[k]];
        zd[k] = pz[o[k]];
    }
    double lox = xd[0], hix = xd[0], loy = yd[0], hiy = yd[0], loz = zd[0], hiz = zd[0];
#pragma unroll
    for (int k = 1; k < BPL; k++) {
        lox = fmin(lox, xd[k]);
        hix = fmax(hix, xd[k]);
        loy = fmin(loy, yd[k]);
        hiy = fmax(hiy, yd[k]);
        loz = fmin(loz, zd[k]);
        hiz = fmax(hiz, zd[k]);
    }
    const double gx = 0.5 * (wmind(lox) + wmaxd(hix)), gy = 0.5 * (wmind(loy) + wmaxd(hiy)),
                 gz = 0.5 * (wmind(loz) + wmaxd(hiz));
    const float ghx = __double2float_rn(gx), ghy = __double2float_rn(gy), ghz = __double2float_rn(gz);
    const float glx = __double2float_rn(gx - (double)ghx), gly = __double2float_rn(gy - (double)ghy),
                glz = __double2float_rn(gz - (double)ghz);
    float bx[BPL], by[BPL], bz[BPL], amag[BPL];
#pragma unroll
    for (int k = 0; k < BPL; k++) {
        bx[k] = __double2float_rn(xd[k] - gx);
        by[k] = __double2float_rn(yd[k] - gy);
        bz[k] = __double2float_rn(zd[k] - gz);
        const uint32_t q = o[k];
        amag[k] = (float)sqrt(ax[q] * ax[q] + ay[q] * ay[q] + az[q] * az[q]);
    }
    float mnx = bx[0], mxx = bx[0], mny = by[0], mxy = by[0], mnz = bz[0], mxz = bz[0];
#pragma unroll
    for (int k = 1; k < BPL; k++) {
        mnx = fminf(mnx, bx[k]);
        mxx = fmaxf(mxx, bx[k]);
        mny = fminf(mny, by[k]);
        mxy = fmaxf(mxy, by[k]);
        mnz = fminf(mnz, bz[k]);
        mxz = fmaxf(mxz, bz[k]);
    }
    const float gminx = wmin(mnx), gmaxx = wmax(mxx), gminy = wmin(mny), gmaxy = wmax(mxy), gminz = wmin(mnz),
                gmaxz = wmax(mxz);
    const float eps2 = g.eps2f;
    auto rel_pos = [&](int k, float &cx, float &cy, float &cz) {
        const float4 A = g.nodeA[k], B = g.nodeB[k];
        cx = (A.x - ghx) + (B.x - glx);
        cy = (A.y - ghy) + (B.y - gly);
        cz = (A.z - ghz) + (B.z - glz);
        return A.w;
    };
    // multipole of the sampled cell
    float mphi[BPL], max_[BPL], may[BPL], maz[BPL];
    {
        float cx, cy, cz;
        const float m = rel_pos(node, cx, cy, cz);
        const float4 Q0 = g.nodeQ[2 * (int64_t)node], Q1 = g.nodeQ[2 * (int64_t)node + 1];
#pragma unroll
        for (int k = 0; k < BPL; k++) {
            mphi[k] = max_[k] = may[k] = maz[k] = 0.f;
            cell_term<QUAD>(make_float4(cx, cy, cz, m), Q0, Q1.x, Q1.y, valid[k], bx[k], by[k], bz[k], eps2, mphi[k],
                            max_[k], may[k], maz[k]);
        }
    }
    // refined reference over the subtree
    float rphi[BPL], rax[BPL], ray[BPL], raz[BPL];
#pragma unroll
    for (int k = 0; k < BPL; k++) rphi[k] = rax[k] = ray[k] = raz[k] = 0.f;
    int sp = 0;
    {
        const int2 C = g.nodeC[node];
        const int nc = C.y & 255;
        if (lane < nc) stk[w][lane] = C.x + lane;
        sp = nc;
    }
    __syncwarp();
    int guard = 0;
    while (sp > 0 && guard < (1 << 22)) {
        guard++;
        const int k = stk[w][sp - 1];
        sp--;
        __syncwarp();
        const int2 C = g.nodeC[k];
        float cx, cy, cz;
        const float m = rel_pos(k, cx, cy, cz);
        if (C.x < 0) {
#pragma unroll
            for (int j = 0; j < BPL; j++)
                cell_term<false>(make_float4(cx, cy, cz, m), make_float4(0.f, 0.f, 0.f, 0.f), 0.f, 0.f, valid[j], bx[j],
                                 by[j], bz[j], eps2, rphi[j], rax[j], ray[j], raz[j]);
            continue;
        }
        const float ex = fmaxf(0.f, fmaxf(gminx - cx, cx - gmaxx)), ey = fmaxf(0.f, fmaxf(gminy - cy, cy - gmaxy)),
                    ez = fmaxf(0.f, fmaxf(gminz - cz, cz - gmaxz));
        const float dmin = sqrtf(ex * ex + ey * ey + ez * ez);
        const float4 Q1 = g.nodeQ[2 * (int64_t)k + 1];
        const float b = Q1.w;
        if (dmin - b > 10.f * b) {
            const float4 Q0 = g.nodeQ[2 * (int64_t)k];
#pragma unroll
            for (int j = 0; j < BPL; j++)
                cell_term<QUAD>(make_float4(cx, cy, cz, m), Q0, Q1.x, Q1.y, valid[j], bx[j], by[j], bz[j], eps2,
                                rphi[j], rax[j], ray[j], raz[j]);
        } else {
            const int nc = C.y & 255;
            if (sp + nc > LSTACK) {
                // cannot happen for depth <= 31; a truncated reference would give a
                // wrong label, so the label walk reports it instead of passing quietly
                if (lane == 0) {
                    atomicCAS(&g.st->error, 0, HC_ERR_STACK);
                    g.st->info = LSTACK;
                }
                break;
            }
            if (lane < nc) stk[w][sp + lane] = C.x + lane;
            sp += nc;
            __syncwarp();
        }
    }
    float rel = 0.f;
#pragma unroll
    for (int k = 0; k < BPL; k++) {
        const float dx = max_[k] - rax[k], dy = may[k] - ray[k], dz = maz[k] - raz[k];
        if (valid[k] && amag[k] > 0.f) rel = fmaxf(rel, sqrtf(dx * dx + dy * dy + dz * dz) / amag[k]);
    }
    const float rmax = wmax(rel);
    if (lane == 0) {
        y[i] = rmax <= eps_label ? 1.f : 0.f;
        rel_out[i] = rmax;
    }
}
}  // namespace

int hc_label_launch(hc_ctx *c, int nsample, float eps_label)
{
    if (nsample <= 0) return HC_OK;
    WalkArgs a;
    memset(&a, 0, sizeof a);
    a.nodeA = c->nodeA;
    a.nodeB = c->nodeB;
    a.nodeQ = c->nodeQ;
    a.nodeC = c->nodeC;
    a.eps2f = (float)(c->prm.eps * c->prm.eps);
    const int blocks = (nsample + 3) / 4;
    if (c->prm.usequad)
        k_label<true><<<blocks, 128, 0, c->stream>>>(a, c->gstart, c->gcount, c->tord, c->px, c->py, c->pz, c->ax,
                                                     c->ay, c->az, c->sample_group, c->sample_node, nsample, eps_label,
                                                     c->sample_y, c->sample_rel);
    else
        k_label<false><<<blocks, 128, 0, c->stream>>>(a, c->gstart, c->gcount, c->tord, c->px, c->py, c->pz, c->ax,
                                                      c->ay, c->az, c->sample_group, c->sample_node, nsample,
                                                      eps_label, c->sample_y, c->sample_rel);
    c->launches++;
    return HC_OK;
}
