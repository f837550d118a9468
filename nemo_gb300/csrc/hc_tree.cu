// hc_tree.cu -- octree construction and moments on the GPU.
//
// Reference: maketree/expandbox/loadtree/intcoord/subindex/hackcofm,
// src/nbody/evolve/hackcode/hackcode1/load.c:32-248.
//
// The reference inserts massive bodies one at a time.  Its final tree is a
// pure function of the root box and the multiset of integer coordinates: a
// cell exists for every octree node (integer prefix) holding two or more
// massive bodies, bodies are leaves, there is no leaf bucket and no path
// compression.  The one exception is expandbox (load.c:68-95): when the second
// massive body forces the box to double K >= 2 times, the K-1 intermediate
// root cells hold only the first body.  The build here reproduces that set:
//
//   1. expandbox replay on the device (one block, FP64, body order),
//   2. 90-bit keys: floor(2^30 (x - rmin) / rsize) per axis, Morton order,
//   3. radix sort, compaction of the massive bodies,
//   4. d[a] = common octal digits of adjacent keys; cells starting at sorted
//      body a have levels (d[a-1], d[a]], which lays cells and bodies out in
//      DFS pre-order directly,
//   5. stable sort of the pre-order by depth -> breadth-first layout with the
//      children of each cell contiguous and in subindex order 0..7,
//   6. level-synchronous upward pass (one cooperative kernel, a grid barrier
//      per level): mass and centre of mass in FP64, children summed in the
//      same order as hackcofm so they are bit-identical (they decide cell
//      openings); the quadrupole, which the walk consumes in FP32, is
//      accumulated in FP32 from FP64 offsets.
#include <cooperative_groups.h>
#include <memory>
#include "hc_internal.cuh"

namespace cg = cooperative_groups;

namespace {

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// (x - rmin) / rsize.  A power-of-two rsize (hackcode1's box is 4 * 2^k)
// divides exactly as a multiplication by its reciprocal: the same correctly
// rounded result, without an FP64 division.
__device__ __forceinline__ double scaled(double x, double rmin, double rsize)
{
    int e;
    const double f = frexp(rsize, &e);
    return f == 0.5 ? dmul(dsub(x, rmin), ldexp(1.0, 1 - e)) : ddiv(dsub(x, rmin), rsize);
}

// intcoord (load.c:135-156): xsc = (x - rmin)/rsize; inside iff 0 <= xsc < 1.
__device__ __forceinline__ bool intcoord1(double x, double rmin, double rsize, int *xi)
{
    double xsc = scaled(x, rmin, rsize);
    if (0.0 <= xsc && xsc < 1.0) {
        *xi = (int)floor(dmul((double)HC_IMAX, xsc));
        return true;
    }
    return false;
}

__device__ __forceinline__ bool inbox(double x, double y, double z, const double *rmin, double rsize)
{
    int t;
    bool a = intcoord1(x, rmin[0], rsize, &t);
    bool b = intcoord1(y, rmin[1], rsize, &t);
    bool c = intcoord1(z, rmin[2], rsize, &t);
    return a && b && c;
}

// ---------------- expandbox replay ----------------

// FP32 value of a double from its high word (sign, exponent, top 20 mantissa
// bits) with integer operations only: relative error below 2^-20; false for
// zeros, denormals, infinities, NaNs and magnitudes outside the FP32 range.
__device__ __forceinline__ bool approx_f32(double x, float *f)
{
    const int hi = __double2hiint(x);
    const int e = ((hi >> 20) & 0x7ff) - 1023 + 127;
    if (e < 1 || e > 254) return false;
    *f = __int_as_float((hi & (int)0x80000000) | (e << 23) | ((hi & 0xfffff) << 3));
    return true;
}

// the two smallest of two pairs of ascending body indices (INT_MAX: none)
__device__ __forceinline__ int2 min2(int2 a, int2 b)
{
    return make_int2(min(a.x, b.x), min(max(a.x, b.x), min(a.y, b.y)));
}

__device__ __forceinline__ int2 warp_min2(int2 v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const int2 w = make_int2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
        v = min2(v, w);
    }
    return v;
}

// Whether a massive body lies outside the box (intcoord's test,
// load.c:135-156), and each block's first two massive bodies in body order
// (the expansion replay needs the first two of all).  A body clearly inside
// by an FP32 estimate with a margin far above its error skips the exact FP64
// test (the FP64 pipe runs at a small fraction of the FP32 rate); the rest
// take it.
__global__ void __launch_bounds__(256) k_box_flags(const double *mass, const double *px, const double *py,
                                                   const double *pz, int64_t n, const hc_box *box, int32_t *outside,
                                                   int2 *first2)
{
    __shared__ int2 wf[8];
    double rmin[3] = {box->rmin[0], box->rmin[1], box->rmin[2]};
    double rsize = box->rsize;
    const float lo[3] = {hc_d2f_rn(rmin[0]), hc_d2f_rn(rmin[1]), hc_d2f_rn(rmin[2])}, sz = hc_d2f_rn(rsize);
    int2 f2 = make_int2(INT_MAX, INT_MAX);     // this thread's first two massive bodies (ascending i)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const bool m = hc_nonzero(mass[i]);
        if (m && f2.y == INT_MAX) {
            if (f2.x == INT_MAX) f2.x = (int)i;
            else f2.y = (int)i;
        }
        const double x[3] = {px[i], py[i], pz[i]};
        bool clear = true;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float f;
            if (!approx_f32(x[k], &f)) {
                clear = false;
                continue;
            }
            const float u = f - lo[k], margin = 0x1p-16f * sz + 0x1p-18f * fabsf(f);
            clear = clear && u >= margin && u <= sz - margin;
        }
        outside[i] = m && !(clear || inbox(x[0], x[1], x[2], rmin, rsize));
    }
    f2 = warp_min2(f2);
    if ((threadIdx.x & 31) == 0) wf[threadIdx.x >> 5] = f2;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) f2 = min2(f2, wf[w]);
        first2[blockIdx.x] = f2;
    }
}

__global__ void k_box_compact(const int32_t *outside, const int32_t *opos, int64_t n, int32_t *cand)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (outside[i]) cand[opos[i]] = (int32_t)i;
}

// One block replays expandbox over the bodies that were outside the box at
// the start, in body order.  The box only grows, so a body inside stays
// inside; each round finds the first remaining body outside, expands for
// it, and continues after it.
// The first two massive bodies come from k_box_flags' per-block pairs: the
// first one (original order) is where the expansion-chain cells hang, the
// second is the body whose insertion may graft them.
__global__ void __launch_bounds__(256) k_box_replay(const double *px, const double *py, const double *pz,
                                                    const int32_t *cand, const int32_t *ncand_p, const int2 *first2,
                                                    int nblk, hc_box *box, hc_status *st)
{
    __shared__ int first;
    __shared__ double rmin[3], rsize;
    __shared__ int doublings, chain_before, chain_k;
    __shared__ int2 wf[8];
    __shared__ int second_massive;
    const int ncand = *ncand_p;
    {
        int2 f2 = make_int2(INT_MAX, INT_MAX);
        for (int b = threadIdx.x; b < nblk; b += blockDim.x) f2 = min2(f2, first2[b]);
        f2 = warp_min2(f2);
        if ((threadIdx.x & 31) == 0) wf[threadIdx.x >> 5] = f2;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); w++) f2 = min2(f2, wf[w]);
            box->first_massive = f2.x == INT_MAX ? -1 : f2.x;
            second_massive = f2.y == INT_MAX ? -1 : f2.y;
        }
    }
    if (threadIdx.x == 0) {
        rmin[0] = box->rmin[0];
        rmin[1] = box->rmin[1];
        rmin[2] = box->rmin[2];
        rsize = box->rsize;
        doublings = 0;
        chain_before = -1;
        chain_k = 0;
    }
    __syncthreads();
    int pos = 0;
    while (pos < ncand) {
        if (threadIdx.x == 0) first = INT_MAX;
        __syncthreads();
        for (int base = pos; base < ncand; base += blockDim.x) {
            int i = base + threadIdx.x;
            if (i < ncand) {
                int b = cand[i];
                if (!inbox(px[b], py[b], pz[b], rmin, rsize)) atomicMin(&first, i);
            }
            __syncthreads();
            if (first != INT_MAX) break;
            __syncthreads();
        }
        int f = first;
        __syncthreads();
        if (f == INT_MAX) break;
        if (threadIdx.x == 0) {
            int b = cand[f];
            double x[3] = {px[b], py[b], pz[b]};
            int k = 0;
            while (!inbox(x[0], x[1], x[2], rmin, rsize)) {     // load.c:74-93
                if (k >= 1100) {          // non-finite position: the box can never hold it
                    doublings = -1000000;
                    break;
                }
                double rmid[3];
                for (int d = 0; d < 3; d++) rmid[d] = dadd(rmin[d], dmul(0.5, rsize));
                for (int d = 0; d < 3; d++)
                    if (x[d] < rmid[d]) rmin[d] = dsub(rmin[d], rsize);
                rsize = dmul(2.0, rsize);
                k++;
            }
            if (b == second_massive && k >= 2) {   // grafted over a lone first body
                chain_before = doublings;
                chain_k = k;
            }
            doublings += k;
        }
        __syncthreads();
        pos = f + 1;
    }
    if (threadIdx.x == 0 && doublings < 0) {      // non-finite position of a massive body
        atomicCAS(&st->error, 0, HC_ERR_ARG);
        st->info = -1;
        return;
    }
    if (threadIdx.x == 0) {
        box->rmin[0] = rmin[0];
        box->rmin[1] = rmin[1];
        box->rmin[2] = rmin[2];
        box->rsize = rsize;
        if (chain_before >= 0) {
            int e = doublings - chain_before;       // levels between that box and the final root
            box->chain_lmax = e - 1;
            box->chain_lmin = e - chain_k + 1;
        } else {
            box->chain_lmax = -1;
            box->chain_lmin = -1;
        }
        double d = dmul(rsize, rsize);
        for (int l = 0; l <= HC_MAXLEVEL; l++) {
            box->dsq[l] = d;
            d = ddiv(d, 4.0);
        }
    }
}

// ---------------- keys ----------------

__device__ __forceinline__ unsigned long long spread21(unsigned v)
{
    unsigned long long x = v & 0x1fffffull;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__device__ __forceinline__ uint32_t spread9(unsigned v)
{
    uint32_t x = v & 0x1ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__device__ __forceinline__ int intcoord_clamped(double x, double rmin, double rsize)
{
    int xi;
    if (intcoord1(x, rmin, rsize, &xi)) return xi;
    double xsc = scaled(x, rmin, rsize);
    return xsc < 0.0 ? 0 : HC_IMAX - 1;   // massless bodies / test points outside the box
}

// intcoord_clamped for a box of size 2^E, with one FP64 operation.  With a
// power-of-two size the reference's only rounding step is d = x - rmin (the
// scaling by 2^-E and by IMAX = 2^30 is exact), so
// floor(IMAX (x - rmin) / rsize) is d's significand shifted right by
// 22 + E - exponent(d), and 0 <= xsc < 1 reads off d's sign and exponent.
// Outside the box: 0 below it (negative d), IMAX - 1 above it and for NaN.
__device__ __forceinline__ int intcoord_pow2(double x, double rmin, int E)
{
    const long long b = __double_as_longlong(dsub(x, rmin));
    const int ef = (int)((b >> 52) & 0x7ff);
    const long long frac = b & 0xfffffffffffffll;
    if (ef == 0x7ff) return frac ? HC_IMAX - 1 : (b < 0 ? 0 : HC_IMAX - 1);   // NaN, -inf, +inf
    if (b < 0) return 0;                    // negative, or -0.0 (inside, cell 0)
    const int ex = ef ? ef - 1023 : -1022;  // d = sig * 2^(ex - 52)
    if (ex >= E) return HC_IMAX - 1;        // d >= 2^E: xsc >= 1
    const long long sig = ef ? (frac | (1ll << 52)) : frac;
    const int s = 22 + E - ex;              // > 22
    return s >= 64 ? 0 : (int)(sig >> s);
}

__global__ void k_keys(const double *x, const double *y, const double *z, int64_t n, const hc_box *box,
                       unsigned long long *khi, uint32_t *klo, uint32_t *kval)
{
    double r0 = box->rmin[0], r1 = box->rmin[1], r2 = box->rmin[2], rs = box->rsize;
    // rs = 2^E exactly when its significand bits are zero (a normal double)
    const uint64_t rb = hc_dbits(rs);
    const int ref = (int)((rb >> 52) & 0x7ff), E = ref - 1023;
    const bool pow2 = (rb & 0xfffffffffffffull) == 0 && ref > 0 && ref < 0x7ff && !(rb >> 63);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        unsigned ix, iy, iz;
        if (pow2) {
            ix = intcoord_pow2(x[i], r0, E);
            iy = intcoord_pow2(y[i], r1, E);
            iz = intcoord_pow2(z[i], r2, E);
        } else {
            ix = intcoord_clamped(x[i], r0, rs);
            iy = intcoord_clamped(y[i], r1, rs);
            iz = intcoord_clamped(z[i], r2, rs);
        }
        khi[i] = (spread21(ix >> 9) << 2) | (spread21(iy >> 9) << 1) | spread21(iz >> 9);
        klo[i] = (spread9(ix) << 2) | (spread9(iy) << 1) | spread9(iz);
        kval[i] = (uint32_t)i;
    }
}

// ---------------- massive compaction and cell enumeration ----------------

__global__ void k_sorted_massive(const uint32_t *sidx, const double *mass, int64_t n, int32_t *flag)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x)
        flag[s] = hc_nonzero(mass[sidx[s]]);
}

// Massive bodies in key order (tree input) and the walk's target order:
// massive bodies in key order, then massless ones in key order.
__global__ void k_mcompact(const int32_t *flag, const int32_t *rank, int64_t n, const unsigned long long *khi,
                           const uint32_t *klo, const uint32_t *sidx, const hc_box *box, unsigned long long *mhi,
                           uint32_t *mlo, uint32_t *midx, uint32_t *mpos, int32_t *s_rank, int32_t *leaf_of_sorted,
                           uint32_t *tord)
{
    const int M = box->nmassive;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        leaf_of_sorted[s] = -1;
        int r = rank[s];
        if (flag[s]) {
            mhi[r] = khi[s];
            mlo[r] = klo[s];
            midx[r] = sidx[s];
            mpos[r] = (uint32_t)s;
            s_rank[s] = r;
            tord[r] = sidx[s];
        } else {
            s_rank[s] = -1;
            tord[M + (s - r)] = sidx[s];
        }
    }
}

// common leading octal digits of two 90-bit keys (30 = identical)
__device__ __forceinline__ int lcp_digits(unsigned long long ha, uint32_t la, unsigned long long hb, uint32_t lb)
{
    unsigned long long x = ha ^ hb;
    if (x) return (__clzll(x) - 1) / 3;
    uint32_t y = la ^ lb;
    if (y) return 21 + (__clz(y) - 5) / 3;
    return 30;
}

__device__ __forceinline__ int dprime(const int32_t *d, const uint32_t *midx, int a, const hc_box *box)
{
    int v = d[a];
    if ((int)midx[a] == box->first_massive && box->chain_lmax > v) v = box->chain_lmax;
    return v;
}

__global__ void k_lcp(const unsigned long long *mhi, const uint32_t *mlo, const uint32_t *midx, hc_box *box,
                      int32_t *d, hc_status *st)
{
    const int M = box->nmassive;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < M; a += gridDim.x * blockDim.x) {
        int v = -1;
        if (a + 1 < M) {
            v = lcp_digits(mhi[a], mlo[a], mhi[a + 1], mlo[a + 1]);
            if (v >= 30) {                     // assert(l != 0), load.c:113
                atomicCAS(&st->error, 0, HC_ERR_COINCIDENT);
                st->info = (int)midx[a];
                v = 29;
            }
        }
        d[a] = v;
    }
}

__global__ void k_ccount(const int32_t *d, const uint32_t *midx, const hc_box *box, int32_t *ccount)
{
    const int M = box->nmassive;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < M; a += gridDim.x * blockDim.x) {
        int dp = a > 0 ? d[a - 1] : -1;
        int dm = dprime(d, midx, a, box);
        ccount[a] = dm > dp ? dm - dp : 0;
    }
}

__global__ void k_post_count(int32_t *cstart, hc_box *box, int64_t maxcell, hc_status *st)
{
    const int M = box->nmassive;
    int ncell = cstart[M];
    box->ncell = ncell;
    box->nnode = M + ncell;
    if (ncell > maxcell) {                      // makecell, load.c:237-239
        atomicCAS(&st->error, 0, HC_ERR_CELLS);
        st->info = (int)maxcell;
        box->nnode = 0;                         // later kernels see an empty tree
        box->ncell = 0;
    }
}

// Pre-order layout: for each sorted massive body a, the cells that start
// at a (levels dprev+1 .. d'[a], outermost first), then body a itself.
__global__ void k_emit_preorder(const int32_t *d, const uint32_t *midx, const int32_t *cstart, const hc_box *box,
                                int64_t maxnode, int32_t *pre_depth, int32_t *pre_a,
                                unsigned long long *dkey, uint32_t *dval)
{
    const int M = box->nmassive;
    if (box->nnode > maxnode || box->nnode == 0) return;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < M; a += gridDim.x * blockDim.x) {
        int dp = a > 0 ? d[a - 1] : -1;
        int dm = dprime(d, midx, a, box);
        int base = a + cstart[a];
        int p = base;
        for (int L = dp + 1; L <= dm; L++, p++) {
            pre_depth[p] = L;
            pre_a[p] = a;
            dkey[p] = (unsigned long long)L;
            dval[p] = (uint32_t)p;
        }
        int depth = (dp > dm ? dp : dm) + 1;    // parent is the deepest cell holding a
        p = a + cstart[a + 1];
        pre_depth[p] = depth;
        pre_a[p] = -1 - a;
        dkey[p] = (unsigned long long)depth;
        dval[p] = (uint32_t)p;
    }
}

__global__ void k_levels(const uint32_t *offs, hc_box *box)
{
    // offs: the depth sort's digit offsets (exclusive scan of its depth counts)
    int D = threadIdx.x;
    if (D <= HC_MAXLEVEL + 1) {
        int v = D <= HC_MAXLEVEL ? (int)offs[D] : box->nnode;
        if (v > box->nnode) v = box->nnode;
        box->level_start[D] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int md = 0;
        for (int l = 0; l <= HC_MAXLEVEL; l++)
            if (box->level_start[l + 1] > box->level_start[l]) md = l;
        box->max_depth = md;
    }
}

__global__ void k_pre2bfs(const uint32_t *bfs2pre, const hc_box *box, uint32_t *pre2bfs)
{
    const int nn = box->nnode;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x)
        pre2bfs[bfs2pre[k]] = (uint32_t)k;
}

// parent = the node one level up with the largest pre-order index below ours
// (bdep: each node's depth in breadth-first order, the depth sort's keys)
__global__ void k_parent(const uint32_t *bfs2pre, const unsigned long long *bdep, const hc_box *box, int32_t *parent)
{
    const int nn = box->nnode;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
        uint32_t p = bfs2pre[k];
        int D = (int)bdep[k];
        if (D == 0) {
            parent[k] = -1;
            continue;
        }
        int lo = box->level_start[D - 1], hi = box->level_start[D] - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (bfs2pre[mid] < p) lo = mid;
            else hi = mid - 1;
        }
        parent[k] = lo;
    }
}

__global__ void k_children(const int32_t *parent, const unsigned long long *bdep, const hc_box *box, int2 *nodeC,
                           int32_t *lastc)
{
    const int nn = box->nnode;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
        int p = parent[k];
        if (p < 0) continue;
        int D = (int)bdep[k];
        int ls = box->level_start[D], le = box->level_start[D + 1];
        if (k == ls || parent[k - 1] != p) nodeC[p].x = k;
        if (k + 1 == le || parent[k + 1] != p) lastc[p] = k;
    }
}

// hi = RN_f32(v), lo = RN_f32(v - hi), on the double's bits (no FP64 pipe)
__device__ __forceinline__ void split_hilo(double v, float *hi, float *lo) { hc_split_hilo(v, hi, lo); }

// Node fields that do not need the upward pass: body leaves (mass and
// position from the body arrays) and the child range of every cell.  bdep,
// ba: each node's depth and first massive body (-1 - rank for a body leaf)
// in breadth-first order, carried through the depth sort.
__global__ void k_node_init(const unsigned long long *bdep, const uint32_t *ba, const uint32_t *midx, const uint32_t *mpos, const double *mass, const double *px,
                            const double *py, const double *pz, const hc_box *box, int2 *nodeC,
                            const int32_t *lastc, float4 *nodeA, float4 *nodeB, float4 *nodeQ, double *nm,
                            double *ncx, double *ncy, double *ncz, int32_t *leaf_of_sorted,
                            hc_status *st)
{
    const int nn = box->nnode;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
        int D = (int)bdep[k], a = (int)ba[k];
        if (a < 0) {
            a = -1 - a;
            uint32_t o = midx[a], s = mpos[a];
            double m = mass[o], x = px[o], y = py[o], z = pz[o];
            nm[k] = m;
            ncx[k] = x;
            ncy[k] = y;
            ncz[k] = z;
            float4 A, B;
            split_hilo(x, &A.x, &B.x);
            split_hilo(y, &A.y, &B.y);
            split_hilo(z, &A.z, &B.z);
            A.w = hc_d2f_rn(m);
            B.w = -1.0f;
            nodeA[k] = A;
            nodeB[k] = B;
            nodeQ[2 * (int64_t)k] = make_float4(0.f, 0.f, 0.f, 0.f);
            nodeQ[2 * (int64_t)k + 1] = make_float4(0.f, 0.f, 1.f, 0.f);   // no quadrupole, one body, bmax 0
            nodeC[k] = make_int2(-1 - a, D << 8);      // body leaf: -1 - massive rank
            leaf_of_sorted[s] = k;
        } else {
            int fc = nodeC[k].x, nc = lastc[k] - fc + 1;
            if (fc <= k || nc < 1 || nc > 8 || fc + nc > nn) {   // children follow their parent
                atomicCAS(&st->error, 0, HC_ERR_STATE);
                st->info = k;
                fc = k + 1;
                nc = 0;
            }
            nodeC[k] = make_int2(fc, nc | (D << 8));
        }
    }
}

// hackcofm (load.c:183-226), all levels, deepest first, one grid barrier
// per level.  Children are summed in subindex order exactly as hackcofm does.
// The upward pass takes each level's cells only, grouped by child count: the
// cells of a warp then run the same number of FP64 child steps and no lane
// idles on a body leaf (the levels interleave cells and leaves in key order).
// Group of a cell: depth * 8 + (children - 1); order inside a group is free.
__device__ __forceinline__ int cell_group(int2 C) { return min((C.y >> 8), 31) * 8 + (C.y & 255) - 1; }

__global__ void k_cell_count(const int2 *nodeC, const hc_box *box, uint32_t *cnt)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int nn = box->nnode;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
        const int2 C = nodeC[k];
        if (C.x >= 0 && (C.y & 255) >= 1) atomicAdd(&h[cell_group(C)], 1u);
    }
    __syncthreads();
    if (h[threadIdx.x]) atomicAdd(&cnt[threadIdx.x], h[threadIdx.x]);
}

// group offsets off[0..256] (exclusive scan of the 256 counts) and placement
// cursors cur[0..255]; one block of 256 threads: warp scans, then the warp sums
__global__ void k_cell_offsets(uint32_t *off, uint32_t *cur)
{
    __shared__ uint32_t wsum[8];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint32_t v = off[t];
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int i = 0; i < w; i++) before += wsum[i];
    const uint32_t ex = before + x - v;
    off[t] = ex;
    cur[t] = ex;
    if (t == 255) off[256] = ex + v;
}

// places each block's cells: one reservation per group per block, then slots
// handed out inside the reservation
__global__ void k_cell_place(const int2 *nodeC, const hc_box *box, uint32_t *cur, int4 *perm)
{
    __shared__ uint32_t h[256], base[256];
    const int nn = box->nnode;
    for (int k0 = blockIdx.x * blockDim.x; k0 < nn; k0 += gridDim.x * blockDim.x) {
        const int k = k0 + threadIdx.x;
        h[threadIdx.x] = 0;
        __syncthreads();
        int grp = -1, slot = 0;
        int2 C = make_int2(-1, 0);
        if (k < nn) {
            C = nodeC[k];
            if (C.x >= 0 && (C.y & 255) >= 1) {
                grp = cell_group(C);
                slot = (int)atomicAdd(&h[grp], 1u);
            }
        }
        __syncthreads();
        if (h[threadIdx.x]) base[threadIdx.x] = atomicAdd(&cur[threadIdx.x], h[threadIdx.x]);
        __syncthreads();
        if (grp >= 0) perm[base[grp] + slot] = make_int4(k, C.x, C.y, 0);   // the cell and its child links
        __syncthreads();
    }
}

__device__ __forceinline__ void prefetch_l1(const void *p)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

__global__ void __launch_bounds__(256, 2) k_cofm_all(int usequad, const hc_box *box, const int2 *nodeC, double *nm,
                                                     double *ncx, double *ncy, double *ncz, float4 *nodeA,
                                                     float4 *nodeB, float4 *nodeQ, const int4 *cperm,
                                                     const uint32_t *coff)
{
    cg::grid_group grid = cg::this_grid();
    const int maxd = box->nnode > 0 ? box->max_depth : -1;
    // A warp takes 32 consecutive cells of a level (one child-count group,
    // so its FP64 child loop is uniform); consecutive 32-cell chunks go to
    // consecutive blocks, which sit on different SMs.  A level of a few
    // thousand cells then spreads over the whole GPU instead of crowding
    // the FP64 units of the first few SMs.
    const int nwarps = (int)(grid.size() >> 5);
    const int wrank = (int)(threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x;
    const int lane = (int)(threadIdx.x & 31);
    for (int D = maxd; D >= 0; D--) {
        // the level's cells only, grouped by child count (coff: group offsets)
        const int ls = (int)coff[D * 8], le = (int)coff[D * 8 + 8];
        const float dsqf = __double2float_rn(box->dsq[D]);
        for (int j = ls + wrank * 32 + lane; j < le; j += nwarps * 32) {
            // the cell with its child links in one load (one dependent round trip less)
            const int4 P = cperm[j];
            const int k = P.x, fc = P.y, nc = P.z & 255;
            // the children's FP32 node data are needed after the FP64 sums: start
            // bringing their lines into L1 now, beside the FP64 loads
            prefetch_l1(nodeA + fc);
            prefetch_l1(nodeA + fc + nc - 1);
            prefetch_l1(nodeB + fc);
            prefetch_l1(nodeB + fc + nc - 1);
            prefetch_l1(nodeQ + 2 * (int64_t)fc);
            prefetch_l1(nodeQ + 2 * (int64_t)(fc + nc) - 1);
            // The children's loads are issued together (predicated on the
            // child count), not one dependent round trip per child.  FP64 mass
            // and first moments in hackcofm's order (load.c:193-224; bit-exact).
            double m = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
#pragma unroll
            for (int h = 0; h < 8; h += 4) {
                double cm[4], px[4], py[4], pz[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    if (h + i < nc) {
                        cm[i] = nm[fc + h + i];
                        px[i] = ncx[fc + h + i];
                        py[i] = ncy[fc + h + i];
                        pz[i] = ncz[fc + h + i];
                    }
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    if (h + i < nc) {
                        m = dadd(m, cm[i]);
                        cx = dadd(cx, dmul(px[i], cm[i]));
                        cy = dadd(cy, dmul(py[i], cm[i]));
                        cz = dadd(cz, dmul(pz[i], cm[i]));
                    }
                }
            }
            cx = ddiv(cx, m);
            cy = ddiv(cy, m);
            cz = ddiv(cz, m);
            float4 A, B;
            split_hilo(cx, &A.x, &B.x);
            split_hilo(cy, &A.y, &B.y);
            split_hilo(cz, &A.z, &B.z);
            // children's offsets from the centre of mass in FP32, from the
            // hi + lo positions ((hi - hi) + (lo - lo)): no FP64 work per child.
            // bmax: children's extents shifted to the new centre; Q = sum_child
            // [ m (3 dr dr^T - |dr|^2 I) + Q_child ], dr = x_child - x_cm.
            // Four children at a time, their loads in flight together.
            float bmax = 0.f, nbody = 0.f;
            float Q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int h = 0; h < 8; h += 4) {
                float4 ca[4], cb[4], q0[4], q1[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int ch = fc + h + i;
                    if (h + i < nc) {
                        ca[i] = nodeA[ch];
                        cb[i] = nodeB[ch];
                        q1[i] = nodeQ[2 * (int64_t)ch + 1];
                        if (usequad) q0[i] = nodeQ[2 * (int64_t)ch];
                    }
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    if (h + i >= nc) continue;
                    const float dx = (ca[i].x - A.x) + (cb[i].x - B.x), dy = (ca[i].y - A.y) + (cb[i].y - B.y),
                                dz = (ca[i].z - A.z) + (cb[i].z - B.z);
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    bmax = fmaxf(bmax, sqrtf(r2) + q1[i].w);
                    nbody += q1[i].z;                // bodies in the cell (exact below 2^24)
                    if (usequad) {
                        const float mr = ca[i].w;
                        Q[0] += mr * (3.f * dx * dx - r2) + q0[i].x;
                        Q[1] += mr * (3.f * dx * dy) + q0[i].y;
                        Q[2] += mr * (3.f * dx * dz) + q0[i].z;
                        Q[3] += mr * (3.f * dy * dy - r2) + q0[i].w;
                        Q[4] += mr * (3.f * dy * dz) + q1[i].x;
                        Q[5] += mr * (3.f * dz * dz - r2) + q1[i].y;
                    }
                }
            }
            nm[k] = m;
            ncx[k] = cx;
            ncy[k] = cy;
            ncz[k] = cz;
            A.w = hc_d2f_rn(m);
            B.w = dsqf;
            nodeA[k] = A;
            nodeB[k] = B;
            nodeQ[2 * (int64_t)k] = make_float4(Q[0], Q[1], Q[2], Q[3]);
            nodeQ[2 * (int64_t)k + 1] = make_float4(Q[4], Q[5], nbody, bmax);
        }
        grid.sync();
    }
}

// clear the child links of the nodes of this build
__global__ void k_clear_links(const hc_box *box, int64_t maxnode, int2 *nodeC, int32_t *lastc)
{
    const int64_t nn = box->nnode < maxnode ? box->nnode : maxnode;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nn; k += (int64_t)gridDim.x * blockDim.x) {
        nodeC[k] = make_int2(-1, -1);
        lastc[k] = -1;
    }
}

__global__ void k_set_nmassive(const int32_t *total, hc_box *box) { box->nmassive = *total; }

// ---------------- walk groups aligned with the tree ----------------
// A group is a run of massive bodies (in key order) that lie in one cell of
// at most gmax (<= HC_GROUP) bodies: the cells (and lone bodies) with <= gmax bodies
// whose parent has more, consecutive siblings packed while they fit.

// A node's first massive body (key order) and its body count: the upward
// pass's count (FP32, exact below 2^24; above it only "more than gmax"
// matters here).
__device__ __forceinline__ int node_count(const uint32_t *ba, const float4 *nodeQ, int k, int *first)
{
    const int a = (int)ba[k];
    if (a < 0) {
        *first = -1 - a;
        return 1;
    }
    *first = a;
    return (int)fminf(nodeQ[2 * (int64_t)k + 1].z, 2.0e9f);
}

template <bool EMIT>
__global__ void k_groups(const uint32_t *ba, const float4 *nodeQ, const int32_t *parent,
                         const int2 *nodeC, const hc_box *box, int64_t maxnode, int gmax, int32_t *ng,
                         const int32_t *goff, int32_t *gstart, int32_t *gcount)
{
    const int nn = box->nnode;
    for (int64_t kk = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; kk < maxnode;
         kk += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)kk;
        if (k >= nn) {
            if (!EMIT) ng[k] = 0;
            continue;
        }
        int first;
        const int cnt = node_count(ba, nodeQ, k, &first);
        int out = EMIT ? goff[k] : 0, packs = 0;
        if (cnt <= gmax) {                         // only the root can be a small group on its own here
            if (parent[k] < 0) {
                if (EMIT) {
                    gstart[out] = first;
                    gcount[out] = cnt;
                }
                packs = 1;
            }
        } else {
            const int fc = nodeC[k].x, nc = nodeC[k].y & 255;
            int cur = 0, cur_first = 0;
            for (int i = 0; i < nc; i++) {
                int f;
                const int cc = node_count(ba, nodeQ, fc + i, &f);
                if (cc > gmax || cur + cc > gmax) {
                    if (cur > 0) {
                        if (EMIT) {
                            gstart[out + packs] = cur_first;
                            gcount[out + packs] = cur;
                        }
                        packs++;
                        cur = 0;
                    }
                    if (cc > gmax) continue;
                }
                if (cur == 0) cur_first = f;
                cur += cc;
            }
            if (cur > 0) {
                if (EMIT) {
                    gstart[out + packs] = cur_first;
                    gcount[out + packs] = cur;
                }
                packs++;
            }
        }
        if (!EMIT) ng[k] = packs;
    }
}

__global__ void k_set_ngroups(const int32_t *goff, int64_t maxnode, hc_box *box) { box->ngroups = goff[maxnode]; }

// ---------------- treecode1 critical radii ----------------
// setrcrit (treecode1/treeload.c:232-252) for every cell: the cell's centre
// and size follow from the integer coordinate of its first body at the
// cell's depth; cm is the FP64 centre of mass.
//   bh86: (size/theta)^2;  sw94: (max distance from cm to a corner)^2/theta^2;
//   "new" (treecode1's default): (size/theta + |cm - centre|)^2;
//   theta = 0: (2 rsize)^2 (always open).
__global__ void k_rcrit(int kind, double theta, const hc_box *box, const uint32_t *ba,
                        const uint32_t *midx, const double *px, const double *py, const double *pz, const int2 *nodeC,
                        const double *ncx, const double *ncy, const double *ncz, float *rcrit2)
{
    const int nn = box->nnode;
    const double rsize = box->rsize;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
        const int2 C = nodeC[k];
        if (C.x < 0) continue;                           // body leaf
        const int D = C.y >> 8;
        const uint32_t o = midx[ba[k]];
        const double p[3] = {px[o], py[o], pz[o]}, cm[3] = {ncx[k], ncy[k], ncz[k]};
        const double size = ldexp(rsize, -D), unit = ldexp(rsize, -30);
        const int shift = 30 - D;
        double off2 = 0.0, bmax2 = 0.0;
        for (int d = 0; d < 3; d++) {
            int xi = 0;
            intcoord1(p[d], box->rmin[d], rsize, &xi);
            const double corner = box->rmin[d] + (double)((xi >> shift) << shift) * unit;
            const double dk = cm[d] - (corner + 0.5 * size);       // offset of cm from the centre
            off2 += dk * dk;
            const double dc = dk + 0.5 * size;                      // distance from the low corner
            const double m = dc > size - dc ? dc : size - dc;
            bmax2 += m * m;
        }
        double r2;
        if (theta == 0.0) r2 = 4.0 * rsize * rsize;
        else if (kind == 1) r2 = (size / theta) * (size / theta);
        else if (kind == 2) r2 = bmax2 / (theta * theta);
        else {
            const double r = size / theta + sqrt(off2);
            r2 = r * r;
        }
        rcrit2[k] = (float)r2;
    }
}

}  // namespace

void hc_rcrit_launch(hc_ctx *c, int kind, double theta)
{
    k_rcrit<<<hc_grid(c->maxnode, 256), 256, 0, c->stream>>>(kind, theta, c->box, c->bfs_a, c->midx,
                                                              c->px, c->py, c->pz, c->nodeC, c->ncx, c->ncy, c->ncz,
                                                              c->rcrit2);
    c->launches++;
}

void hc_keys_for_points(hc_ctx *c, const double *x, const double *y, const double *z, int64_t n,
                        unsigned long long *khi, uint32_t *klo, uint32_t *kval)
{
    k_keys<<<hc_grid(n, 256), 256, 0, c->stream>>>(x, y, z, n, c->box, khi, klo, kval);
    c->launches++;
}

// Launch the whole build on the context stream without host synchronisation
// (graph-capturable); errors land in the device status word.
int hc_tree_build(hc_ctx *c)
{
    const int64_t n = c->n;
    cudaStream_t s = c->stream;
    const int B = 256;
    const int G = hc_grid(n, B);
    int32_t *outside = c->flags;
    int32_t *opos = c->flags + 2 * n;
    int2 *first2 = reinterpret_cast<int2 *>(c->flags + 3 * n + (n & 1));   // [G], 8-byte aligned

    // 1. expandbox replay
    k_box_flags<<<G, B, 0, s>>>(c->mass, c->px, c->py, c->pz, n, c->box, outside, first2);
    hc_scan_exclusive_i32(c, outside, opos, n, c->ncand);
    k_box_compact<<<G, B, 0, s>>>(outside, opos, n, c->cand);
    k_box_replay<<<1, 256, 0, s>>>(c->px, c->py, c->pz, c->cand, c->ncand, first2, G, c->box, c->st);
    c->launches += 3;

    // 2-3. keys, sort, massive compaction
    hc_keys_for_points(c, c->px, c->py, c->pz, n, c->khi[0], c->klo[0], c->kval[0]);
    int sel = hc_radix_sort_keys(c, c->hist, c->khi, c->klo, c->kval, n, 0, 64, true);
    c->sort_sel = sel;
    c->sidx = c->kval[sel];
    int32_t *sflag = c->flags;            // reuse (outside no longer needed)
    int32_t *srank = c->flags + n;
    k_sorted_massive<<<G, B, 0, s>>>(c->sidx, c->mass, n, sflag);
    hc_scan_exclusive_i32(c, sflag, srank, n, c->flags + 2 * n);
    k_set_nmassive<<<1, 1, 0, s>>>(c->flags + 2 * n, c->box);
    k_mcompact<<<G, B, 0, s>>>(sflag, srank, n, c->khi[sel], c->klo[sel], c->sidx, c->box, c->mhi, c->mlo,
                               c->midx, c->mpos, c->s_rank, c->leaf_of_sorted, c->tord);
    c->launches += 3;

    // 4. cells in pre-order
    k_lcp<<<G, B, 0, s>>>(c->mhi, c->mlo, c->midx, c->box, c->dlcp, c->st);
    int32_t *cstart = c->flags + n;       // [n+1]
    HC_CUDA(cudaMemsetAsync(c->ccount, 0, sizeof(int32_t) * (n + 1), s));
    k_ccount<<<G, B, 0, s>>>(c->dlcp, c->midx, c->box, c->ccount);
    hc_scan_exclusive_i32(c, c->ccount, cstart, n + 1, nullptr);
    k_post_count<<<1, 1, 0, s>>>(cstart, c->box, c->maxcell, c->st);
    const int Gn = hc_grid(c->maxnode, B);
    k_emit_preorder<<<G, B, 0, s>>>(c->dlcp, c->midx, cstart, c->box, c->maxnode, c->pre_info, c->pre_a,
                                    c->dkey[0], c->dval[0]);
    c->launches += 5;

    // 5. breadth-first layout: stable sort of the pre-order by depth (count on the device)
    // the pre-order's first bodies ride along as the sort's low words, so the
    // later kernels read depth and first body in breadth-first order
    uint32_t *alo[2] = {reinterpret_cast<uint32_t *>(c->pre_a), c->bfs_a};
    int dsel = hc_radix_sort_keys(c, c->hist, c->dkey, alo, c->dval, c->maxnode, 0, 8, false, &c->box->nnode);
    if (dsel != 1) {          // one 8-bit pass: the result is in the second buffers
        c->err = "depth sort: unexpected pass count";
        return HC_ERR_STATE;
    }
    c->bfs2pre = c->dval[dsel];
    const unsigned long long *bdep = c->dkey[dsel];
    k_levels<<<1, 64, 0, s>>>(c->hist, c->box);      // the sort leaves its digit offsets at hist[0..255]
    k_pre2bfs<<<Gn, B, 0, s>>>(c->bfs2pre, c->box, c->pre2bfs);
    k_parent<<<Gn, B, 0, s>>>(c->bfs2pre, bdep, c->box, c->parent);
    k_clear_links<<<Gn, B, 0, s>>>(c->box, c->maxnode, c->nodeC, c->lastc);
    k_children<<<Gn, B, 0, s>>>(c->parent, bdep, c->box, c->nodeC, c->lastc);
    k_node_init<<<Gn, B, 0, s>>>(bdep, c->bfs_a, c->midx, c->mpos, c->mass, c->px, c->py,
                                 c->pz, c->box, c->nodeC, c->lastc, c->nodeA, c->nodeB, c->nodeQ, c->nm, c->ncx,
                                 c->ncy, c->ncz, c->leaf_of_sorted, c->st);
    c->launches += 7;

    // 6. upward pass, deepest level first, one cooperative launch, over the
    // cells grouped by depth and child count.  Work forked onto the side
    // stream joins here: nothing else runs beside the cooperative launch.
    if (c->join_pending) {
        c->join_pending = false;
        HC_CUDA(cudaStreamWaitEvent(s, c->ev_join, 0));
    }
    HC_CUDA(cudaMemsetAsync(c->cbins, 0, sizeof(uint32_t) * 520, s));
    k_cell_count<<<Gn, B, 0, s>>>(c->nodeC, c->box, c->cbins);
    k_cell_offsets<<<1, 256, 0, s>>>(c->cbins, c->cbins + 260);
    k_cell_place<<<Gn, B, 0, s>>>(c->nodeC, c->box, c->cbins + 260, c->cperm);
    c->launches += 3;
    {
        int usequad = c->prm.usequad;
        void *args[] = {&usequad, &c->box, &c->nodeC, &c->nm, &c->ncx, &c->ncy, &c->ncz, &c->nodeA, &c->nodeB,
                        &c->nodeQ, &c->cperm, &c->cbins};
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(c->cofm_grid);
        cfg.blockDim = dim3(256);
        cfg.stream = s;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeCooperative;
        attr.val.cooperative = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        HC_CUDA(cudaLaunchKernelExC(&cfg, (const void *)k_cofm_all, args));
        c->launches++;
    }

    // 7. walk groups aligned with the tree
    const int gmax = hc_table_gmax(c);
    k_groups<false><<<Gn, B, 0, s>>>(c->bfs_a, c->nodeQ, c->parent, c->nodeC,
                                     c->box, c->maxnode, gmax, c->gcnt, nullptr, nullptr, nullptr);
    hc_scan_exclusive_i32(c, c->gcnt, c->goff, c->maxnode + 1, nullptr);
    k_set_ngroups<<<1, 1, 0, s>>>(c->goff, c->maxnode, c->box);
    k_groups<true><<<Gn, B, 0, s>>>(c->bfs_a, c->nodeQ, c->parent, c->nodeC, c->box, c->maxnode,
                                    gmax, nullptr, c->goff, c->gstart, c->gcount);
    c->launches += 3;
    return HC_OK;
}

int hc_tree_setup(hc_ctx *c)
{
    if (int r = hc_sort_setup(c)) return r;
    int dev = 0, nsm = 0, per = 0;
    HC_CUDA(cudaGetDevice(&dev));
    HC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    HC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cofm_all, 256, 0));
    if (per < 1) per = 1;
    c->cofm_grid = nsm * (per > 4 ? 4 : per);
    return HC_OK;
}

// ---------------- tree dump (host assembly from device arrays) ----------------

int hc_tree_dump_impl(hc_ctx *c, int32_t *level, int32_t *corner, int32_t *count, double *mass, double *cm,
                      double *quad, int32_t *bparent)
{
    HC_CUDA(cudaMemcpy(c->h_box, c->box, sizeof(hc_box), cudaMemcpyDeviceToHost));
    const int M = c->h_box->nmassive, nn = c->h_box->nnode;
    for (int64_t i = 0; i < c->n && bparent; i++) bparent[i] = -1;
    if (nn <= 0) return 0;
    auto H = [&](size_t bytes) { return std::unique_ptr<char[]>(new char[bytes > 0 ? bytes : 1]); };
    auto hb = H(sizeof(uint32_t) * nn), hd = H(sizeof(int32_t) * nn), ha = H(sizeof(int32_t) * nn),
         hbb = H(sizeof(int32_t) * nn), hmhi = H(sizeof(unsigned long long) * M), hmlo = H(sizeof(uint32_t) * M),
         hmidx = H(sizeof(uint32_t) * M), hnm = H(sizeof(double) * nn), hx = H(sizeof(double) * nn),
         hy = H(sizeof(double) * nn), hz = H(sizeof(double) * nn), hq = H(sizeof(float4) * 2 * nn);
    uint32_t *bfs2pre = (uint32_t *)hb.get();
    int32_t *pd = (int32_t *)hd.get(), *pa = (int32_t *)ha.get(), *pb = (int32_t *)hbb.get();
    unsigned long long *mhi = (unsigned long long *)hmhi.get();
    uint32_t *mlo = (uint32_t *)hmlo.get(), *midx = (uint32_t *)hmidx.get();
    double *nm = (double *)hnm.get(), *nx = (double *)hx.get(), *ny = (double *)hy.get(), *nz = (double *)hz.get();
    float *nq = (float *)hq.get();
    HC_CUDA(cudaMemcpy(bfs2pre, c->bfs2pre, sizeof(uint32_t) * nn, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(pd, c->pre_info, sizeof(int32_t) * nn, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(pa, c->pre_a, sizeof(int32_t) * nn, cudaMemcpyDeviceToHost));
    // bodies per node, summed up the children links (breadth-first: children
    // follow their parent, so one pass from the back)
    {
        std::unique_ptr<int2[]> C(new int2[nn]);
        HC_CUDA(cudaMemcpy(C.get(), c->nodeC, sizeof(int2) * nn, cudaMemcpyDeviceToHost));
        for (int k = nn - 1; k >= 0; k--) {
            int cnt = 1;
            if (C[k].x >= 0) {
                cnt = 0;
                for (int i = 0; i < (C[k].y & 255); i++) cnt += pb[C[k].x + i];
            }
            pb[k] = cnt;
        }
    }
    HC_CUDA(cudaMemcpy(mhi, c->mhi, sizeof(unsigned long long) * M, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(mlo, c->mlo, sizeof(uint32_t) * M, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(midx, c->midx, sizeof(uint32_t) * M, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(nm, c->nm, sizeof(double) * nn, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(nx, c->ncx, sizeof(double) * nn, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(ny, c->ncy, sizeof(double) * nn, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(nz, c->ncz, sizeof(double) * nn, cudaMemcpyDeviceToHost));
    HC_CUDA(cudaMemcpy(nq, c->nodeQ, sizeof(float4) * 2 * nn, cudaMemcpyDeviceToHost));
    auto unspread = [](unsigned long long hi, uint32_t lo, int axis) {
        // axis 0 = x (bit 2 of each digit), 1 = y, 2 = z
        unsigned v = 0;
        int sh = 2 - axis;
        for (int b = 0; b < 21; b++) v |= (unsigned)((hi >> (3 * b + sh)) & 1ull) << (b + 9);
        for (int b = 0; b < 9; b++) v |= ((lo >> (3 * b + sh)) & 1u) << b;
        return v;
    };
    int ci = 0;
    for (int k = 0; k < nn; k++) {
        uint32_t p = bfs2pre[k];
        int D = pd[p], a = pa[p];
        if (a < 0) {
            if (bparent) bparent[midx[-1 - a]] = D - 1;
            continue;
        }
        if (level) level[ci] = D;
        if (corner) {
            for (int ax = 0; ax < 3; ax++) {
                unsigned v = unspread(mhi[a], mlo[a], ax);
                unsigned mask = D >= 30 ? 0xffffffffu : ~((1u << (30 - D)) - 1u);
                corner[3 * ci + ax] = (int32_t)(v & mask);
            }
        }
        if (count) count[ci] = pb[k];
        if (mass) mass[ci] = nm[k];
        if (cm) {
            cm[3 * ci] = nx[k];
            cm[3 * ci + 1] = ny[k];
            cm[3 * ci + 2] = nz[k];
        }
        if (quad)
            for (int q = 0; q < 6; q++) quad[6 * ci + q] = nq[(int64_t)8 * k + q];
        ci++;
    }
    return ci;
}
