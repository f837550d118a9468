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
// Here one warp walks for a group of 32 bodies that are consecutive in Morton
// order (a compact patch of space).  Every traversal entry carries a 32-bit
// lane mask: the bodies whose own walk reaches that node (all ancestors
// opened for them).  Candidates are processed 32 at a time, one per lane:
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
// FP32 FMA, rsqrt), lanes outside an entry's mask contributing zero.
//
// Precision: positions are taken relative to the group centre (FP64 centre,
// node centres stored as FP32 hi/lo pairs), the interaction arithmetic is
// FP32, and each list evaluation's partial sums are added into the running
// per-body totals with Kahan compensation; results are stored in FP64.
//
// Flop count per interaction (FMA = 2, rsqrt = 1): monopole 20, quadrupole
// cell 59.  These are the per-interaction figures used for the roofline.
#include "hc_internal.cuh"

namespace {

constexpr int WARPS = 4;        // warps per block
constexpr int STACK = 256;      // traversal stack entries per warp (deepest seen at N=1M: 136)
constexpr int BCAP = 64;        // body interaction list entries per warp
constexpr int CCAP = 64;        // cell interaction list entries per warp
constexpr unsigned FULL = 0xffffffffu;

struct WarpSmem {
    uint2 stack[STACK];         // x = first node << 3 | (count - 1), y = lane mask
    float4 bl[BCAP];            // body list: rel pos (hi), mass
    float4 bl2[BCAP];           // body list: rel pos (lo), accept mask (bits)
    float4 cl[CCAP];            // cell list: rel pos, mass
    float4 cq0[CCAP];           // Qxx Qxy Qxz Qyy
    float4 cq1[CCAP];           // Qyz Qzz mask(bits) 0
};

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
};

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
    pphi -= mr;
    pax = fmaf(mr3, dx, pax);
    pay = fmaf(mr3, dy, pay);
    paz = fmaf(mr3, dz, paz);
    if (QUAD) {
        const float qx = fmaf(Q0.x, dx, fmaf(Q0.y, dy, Q0.z * dz));
        const float qy = fmaf(Q0.y, dx, fmaf(Q0.w, dy, qyz * dz));
        const float qz = fmaf(Q0.z, dx, fmaf(qyz, dy, qzz * dz));
        const float dqd = fmaf(qx, dx, fmaf(qy, dy, qz * dz));
        const float r5 = on ? rinv2 * rinv2 * rinv : 0.f;
        const float t = dqd * r5;                 // dr.Q.dr / r^5
        pphi = fmaf(-0.5f, t, pphi);              // phiquad = -t/2
        const float sq = 2.5f * t * rinv2;        // -5 phiquad / r^2
        pax = fmaf(sq, dx, fmaf(-r5, qx, pax));
        pay = fmaf(sq, dy, fmaf(-r5, qy, pay));
        paz = fmaf(sq, dz, fmaf(-r5, qz, paz));
    }
}

template <bool QUAD, bool COUNT>
__global__ void __launch_bounds__(WARPS * 32) k_walk(WalkArgs g)
{
    extern __shared__ float4 smem_raw[];
    WarpSmem &S = reinterpret_cast<WarpSmem *>(smem_raw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t ngroups = (g.ntarget + 31) / 32;
    const int nnode = g.box->nnode;
    const float tol2 = g.tol2f, eps2 = g.eps2f;
    unsigned long long tot_b = 0, tot_c = 0, st_cand = 0, st_mixed = 0, st_eb = 0, st_ec = 0;
    int max_sp = 0, nborder = 0;

    while (true) {
        int64_t grp;
        {
            unsigned v = 0;
            if (lane == 0) v = atomicAdd(g.group_counter, 1u);
            grp = (int64_t)__shfl_sync(FULL, v, 0);
        }
        if (grp >= ngroups) break;
        const int64_t s0 = grp * 32;
        const int64_t s = s0 + lane;
        const bool valid = s < g.ntarget;
        const unsigned vmask = __ballot_sync(FULL, valid);
        const uint32_t o = g.tsorted[valid ? s : s0];
        const double xd = g.tx[o], yd = g.ty[o], zd = g.tz[o];

        // group centre (FP64) and body positions relative to it (FP32)
        double gx, gy, gz;
        {
            double lox = wmind(xd), hix = wmaxd(xd), loy = wmind(yd), hiy = wmaxd(yd), loz = wmind(zd),
                   hiz = wmaxd(zd);
            gx = 0.5 * (lox + hix);
            gy = 0.5 * (loy + hiy);
            gz = 0.5 * (loz + hiz);
        }
        const float ghx = __double2float_rn(gx), ghy = __double2float_rn(gy), ghz = __double2float_rn(gz);
        const float glx = __double2float_rn(gx - (double)ghx), gly = __double2float_rn(gy - (double)ghy),
                    glz = __double2float_rn(gz - (double)ghz);
        const float bx = __double2float_rn(xd - gx), by = __double2float_rn(yd - gy), bz = __double2float_rn(zd - gz);
        // low parts: body-body separations are formed as (hi - hi) + (lo - lo)
        const float blx = __double2float_rn((xd - gx) - (double)bx), bly = __double2float_rn((yd - gy) - (double)by),
                    blz = __double2float_rn((zd - gz) - (double)bz);
        const float gminx = wmin(bx), gmaxx = wmax(bx), gminy = wmin(by), gmaxy = wmax(by), gminz = wmin(bz),
                    gmaxz = wmax(bz);
        const float rg2 = wmax(bx * bx + by * by + bz * bz);
        const float cR = 2e-6f * tol2 * rg2;     // absolute band term of the FP32 decision

        float sphi = 0.f, sax = 0.f, say = 0.f, saz = 0.f;   // Kahan sums
        float cphi = 0.f, cax = 0.f, cay = 0.f, caz = 0.f;
        int myb = 0, myc = 0;                              // per-body counts

        auto flush_bodies = [&](int nb) {
            st_eb += nb;
            float pphi = 0.f, pax = 0.f, pay = 0.f, paz = 0.f;
            for (int e = 0; e < nb; e++) {
                const float4 P = S.bl[e];
                const float4 L = S.bl2[e];
                const unsigned m = __float_as_uint(L.w);
                const bool bit = (m >> lane) & 1u;
                const float dx = (P.x - bx) + (L.x - blx), dy = (P.y - by) + (L.y - bly), dz = (P.z - bz) + (L.z - blz);
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                const float rinv = rsqrtf(r2);
                const float mr = bit ? P.w * rinv : 0.f;
                const float mr3 = mr * (rinv * rinv);
                pphi -= mr;
                pax = fmaf(mr3, dx, pax);
                pay = fmaf(mr3, dy, pay);
                paz = fmaf(mr3, dz, paz);
                if (COUNT) myb += bit;
            }
            kahan_add(sphi, cphi, pphi);
            kahan_add(sax, cax, pax);
            kahan_add(say, cay, pay);
            kahan_add(saz, caz, paz);
        };
        auto flush_cells = [&](int nc) {
            st_ec += nc;
            float pphi = 0.f, pax = 0.f, pay = 0.f, paz = 0.f;
            for (int e = 0; e < nc; e++) {
                const float4 P = S.cl[e];
                const float4 Q1 = S.cq1[e];
                const bool bit = (__float_as_uint(Q1.z) >> lane) & 1u;
                const float4 Q0 = QUAD ? S.cq0[e] : make_float4(0.f, 0.f, 0.f, 0.f);
                cell_term<QUAD>(P, Q0, Q1.x, Q1.y, bit, bx, by, bz, eps2, pphi, pax, pay, paz);
                if (COUNT) myc += bit;
            }
            kahan_add(sphi, cphi, pphi);
            kahan_add(sax, cax, pax);
            kahan_add(say, cay, pay);
            kahan_add(saz, caz, paz);
        };

        int sp = 0, nb = 0, nc = 0;
        bool overflow = false;
        if (nnode > 0) {
            if (lane == 0) S.stack[0] = make_uint2(0u, vmask);   // root, one node
            sp = 1;
        }
        __syncwarp();
        while (sp > 0) {
            // ---- gather up to 32 candidates from the top of the stack ----
            int ncand = 0, my_node = 0;
            unsigned my_mask = 0;
            while (ncand < 32 && sp > 0) {
                const uint2 e = S.stack[sp - 1];
                const int start = (int)(e.x >> 3), cnt = (int)(e.x & 7u) + 1;
                const int take = min(cnt, 32 - ncand);
                const int rel = lane - ncand;
                if (rel >= 0 && rel < take) {
                    my_node = start + cnt - take + rel;
                    my_mask = e.y;
                }
                ncand += take;
                if (take == cnt) sp--;
                else if (lane == 0) S.stack[sp - 1].x = ((unsigned)start << 3) | (unsigned)(cnt - take - 1);
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
            const float cx = (A.x - ghx) + (B.x - glx), cy = (A.y - ghy) + (B.y - gly), cz = (A.z - ghz) + (B.z - glz);
            const bool isbody = C.x < 0;
            unsigned openm = 0, accm = 0;
            bool mixed = false;
            if (have) {
                if (isbody) {
                    const int64_t slot = (int64_t)(-1 - C.x) - s0;
                    const unsigned self = (g.self_mode && slot >= 0 && slot < 32) ? (1u << slot) : 0u;
                    accm = my_mask & ~self;
                } else {
                    const float dsq = B.w;
                    const float ex = fmaxf(0.f, fmaxf(gminx - cx, cx - gmaxx));
                    const float ey = fmaxf(0.f, fmaxf(gminy - cy, cy - gmaxy));
                    const float ez = fmaxf(0.f, fmaxf(gminz - cz, cz - gmaxz));
                    const float fx = fmaxf(fabsf(cx - gminx), fabsf(cx - gmaxx));
                    const float fy = fmaxf(fabsf(cy - gminy), fabsf(cy - gmaxy));
                    const float fz = fmaxf(fabsf(cz - gminz), fabsf(cz - gmaxz));
                    const float dmin2 = ex * ex + ey * ey + ez * ez;
                    const float dmax2 = fx * fx + fy * fy + fz * fz;
                    const float tmin = tol2 * dmin2, tmax = tol2 * dmax2;
                    if (tmin - dsq > 8e-6f * tmin + cR) accm = my_mask;          // every body accepts
                    else if (dsq - tmax > 8e-6f * tmax + cR) openm = my_mask;    // every body opens
                    else mixed = true;
                }
            }
            unsigned mixedb = __ballot_sync(FULL, mixed);
            st_cand += ncand;
            st_mixed += __popc(mixedb);
            while (mixedb) {
                const int j = __ffs(mixedb) - 1;
                mixedb &= mixedb - 1;
                const float jx = __shfl_sync(FULL, cx, j), jy = __shfl_sync(FULL, cy, j),
                            jz = __shfl_sync(FULL, cz, j), jd = __shfl_sync(FULL, B.w, j);
                const unsigned jm = __shfl_sync(FULL, my_mask, j);
                const int jn = __shfl_sync(FULL, my_node, j);
                const int jdepth = __shfl_sync(FULL, C.y, j) >> 8;
                const bool in = (jm >> lane) & 1u;
                const float dx = jx - bx, dy = jy - by, dz = jz - bz;
                const float d2 = dx * dx + dy * dy + dz * dz;
                const float t = tol2 * d2 - jd;
                bool op = t < 0.f;
                if (in && fabsf(t) <= 8e-6f * tol2 * d2 + cR) {
                    // borderline: decide exactly as subdivp does, in FP64
                    op = open_exact(g.ncx[jn], g.ncy[jn], g.ncz[jn], xd, yd, zd, g.tol2d, g.box->dsq[jdepth]);
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
            if (COUNT && accm != 0u) atomicAdd(&g.st->mask_hist[__popc(accm)], 1ull);
            const unsigned bbal = __ballot_sync(FULL, ab), cbal = __ballot_sync(FULL, ac);
            if (ab) {
                // node - centre as an unevaluated float sum hi + lo (TwoSum of the hi parts)
                const int pos = nb + __popc(bbal & lt);
                float hx, hy, hz, ex, ey, ez;
                two_diff(A.x, ghx, hx, ex);
                two_diff(A.y, ghy, hy, ey);
                two_diff(A.z, ghz, hz, ez);
                S.bl[pos] = make_float4(hx, hy, hz, A.w);
                S.bl2[pos] = make_float4(ex + (B.x - glx), ey + (B.y - gly), ez + (B.z - glz), __uint_as_float(accm));
                tot_b += __popc(accm);
            }
            if (ac) {
                const int pos = nc + __popc(cbal & lt);
                S.cl[pos] = make_float4(cx, cy, cz, A.w);
                if (QUAD) {
                    const float4 q0 = g.nodeQ[2 * (int64_t)my_node], q1 = g.nodeQ[2 * (int64_t)my_node + 1];
                    S.cq0[pos] = q0;
                    S.cq1[pos] = make_float4(q1.x, q1.y, __uint_as_float(accm), 0.f);
                } else {
                    S.cq1[pos] = make_float4(0.f, 0.f, __uint_as_float(accm), 0.f);
                }
                tot_c += __popc(accm);
            }
            nb += __popc(bbal);
            nc += __popc(cbal);
            __syncwarp();
            if (nb > BCAP - 32) {
                flush_bodies(nb);
                nb = 0;
            }
            if (nc > CCAP - 32) {
                flush_cells(nc);
                nc = 0;
            }
            __syncwarp();
        }
        if (overflow) {
            if (lane == 0) {
                atomicCAS(&g.st->error, 0, HC_ERR_STACK);
                g.st->info = STACK;
            }
            continue;
        }
        if (nb) flush_bodies(nb);
        if (nc) flush_cells(nc);
        __syncwarp();

        if (valid) {
            const double rphi = (double)sphi - (double)cphi;
            const double rax = (double)sax - (double)cax, ray = (double)say - (double)cay,
                         raz = (double)saz - (double)caz;
            if (g.kick_dthf != 0.0 && g.nstep > 0) {
                // closing half kick with the new acceleration (code.c:175-179)
                g.vx[o] = __dadd_rn(g.vx[o], __dmul_rn(__dsub_rn(rax, g.oax[o]), g.kick_dthf));
                g.vy[o] = __dadd_rn(g.vy[o], __dmul_rn(__dsub_rn(ray, g.oay[o]), g.kick_dthf));
                g.vz[o] = __dadd_rn(g.vz[o], __dmul_rn(__dsub_rn(raz, g.oaz[o]), g.kick_dthf));
            }
            g.oax[o] = rax;
            g.oay[o] = ray;
            g.oaz[o] = raz;
            g.ophi[o] = rphi;
            if (COUNT) {
                g.cnt_b[o] = myb;
                g.cnt_c[o] = myc;
            }
        }
    }
    // interaction totals and stats
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        tot_b += __shfl_xor_sync(FULL, tot_b, off);
        tot_c += __shfl_xor_sync(FULL, tot_c, off);
        nborder += __shfl_xor_sync(FULL, nborder, off);
    }
    if (lane == 0) {
        atomicAdd(&g.st->n2b, tot_b);
        atomicAdd(&g.st->nbc, tot_c);
        atomicMax(&g.st->max_stack, max_sp);
        atomicAdd(&g.st->nborder, nborder);
        atomicAdd(&g.st->ncand, st_cand);
        atomicAdd(&g.st->nmixed, st_mixed);
        atomicAdd(&g.st->nentry_b, st_eb);
        atomicAdd(&g.st->nentry_c, st_ec);
    }
}

template <bool Q, bool C>
int configure(hc_ctx *c, int variant)
{
    const size_t smem = sizeof(WarpSmem) * WARPS;
    HC_CUDA(cudaFuncSetAttribute(k_walk<Q, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, nsm = 0, per_sm = 0;
    HC_CUDA(cudaGetDevice(&dev));
    HC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    HC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<Q, C>, WARPS * 32, smem));
    c->walk_blocks[variant] = nsm * (per_sm < 1 ? 1 : per_sm);
    return HC_OK;
}

// No CUDA queries here: this runs inside stream capture.
template <bool Q, bool C>
int launch(hc_ctx *c, WalkArgs &a, int variant)
{
    const size_t smem = sizeof(WarpSmem) * WARPS;
    int64_t ngroups = (a.ntarget + 31) / 32;
    int64_t blocks = c->walk_blocks[variant];
    int64_t need = (ngroups + WARPS - 1) / WARPS;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    k_walk<Q, C><<<(unsigned)blocks, WARPS * 32, smem, c->stream>>>(a);
    c->launches++;
    return HC_OK;
}

}  // namespace

int hc_walk_launch(hc_ctx *c, bool self, int64_t ntarget, const uint32_t *tsorted, const double *tx,
                   const double *ty, const double *tz, double *oax, double *oay, double *oaz, double *ophi,
                   double kick_dthf, int64_t nstep)
{
    if (ntarget <= 0) return HC_OK;
    WalkArgs a;
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
    HC_CUDA(cudaMemsetAsync(a.group_counter, 0, sizeof(unsigned), c->stream));
    const bool count = c->prm.count_per_body && self && c->cnt_b;
    if (c->prm.usequad) return count ? launch<true, true>(c, a, 3) : launch<true, false>(c, a, 2);
    return count ? launch<false, true>(c, a, 1) : launch<false, false>(c, a, 0);
}

int hc_walk_setup(hc_ctx *c)
{
    int r = configure<false, false>(c, 0);
    if (r == HC_OK) r = configure<false, true>(c, 1);
    if (r == HC_OK) r = configure<true, false>(c, 2);
    if (r == HC_OK) r = configure<true, true>(c, 3);
    return r;
}
