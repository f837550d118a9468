// hc_sort.cu -- device scan and LSD radix sort for the octree keys.
//
// The reference inserts bodies one by one (loadtree, load.c:101-128); the
// GB300 build instead sorts all bodies by their 90-bit integer-coordinate key
// (top 63 bits radix sorted, the low 27 bits resolved inside runs of equal
// high keys), so that every octree cell is a contiguous run of sorted bodies.
// Integer work with little arithmetic: coalesced tile loads, block-local
// histograms and ranks in shared memory, a stable scatter staged in digit
// order.  At N=1M each sort pass moves 32 MB (5 us at HBM rate) and is bound
// by latency instead (about 20 us per pass).
#include <algorithm>
#include "hc_internal.cuh"

namespace {

constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 16;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;

template <typename T>
__device__ T block_exclusive_scan(T v, T *sh, T *total)
{
    // Hillis-Steele over warps: warp scan with shuffles, then scan of warp sums.
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        T w = lane < nw ? sh[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) sh[lane] = w;
    }
    __syncthreads();
    T base = wid > 0 ? sh[wid - 1] : T(0);
    if (total) *total = sh[nw - 1];
    __syncthreads();
    return base + x - v;
}

// Single-pass exclusive scan with decoupled look-back (Merrill and Garland,
// 2016): tiles of 4096 values take their index from a counter in launch
// order, publish their sum, and one warp per tile sums the earlier tiles'
// published values 32 at a time, back to the first tile that already holds
// its inclusive prefix.  A tile waits only on tiles that hold their index,
// so every wait ends; each wait is bounded nonetheless and reports an error.
// Values and prefixes stay below 2^30 (bodies + cells < 2^30).  Loads and
// stores go through shared memory (one pad word per 32) so that the global
// accesses are coalesced and each thread scans 16 consecutive values.
// In place is allowed: a tile reads its inputs before writing its outputs.
constexpr int SCAN_THREADS = 256, SCAN_ITEMS = 16, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr uint32_t SC_AGG = 1u << 30, SC_PRE = 2u << 30, SC_VAL = (1u << 30) - 1u;
constexpr int SC_SPIN = 1 << 20;

__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u32(uint32_t *p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int scan_pad(int e) { return e + (e >> 5); }

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_onepass(const int32_t *in, int32_t *out, int64_t n,
                                                                uint32_t *status, uint32_t *ctr, int32_t *total,
                                                                int *err)
{
    __shared__ int32_t s[SCAN_TILE + SCAN_TILE / 32];
    __shared__ int32_t sh[32];
    __shared__ uint32_t s_tile;
    __shared__ int32_t s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(ctr, 1u);
    __syncthreads();
    const int64_t tile = s_tile, base = tile * SCAN_TILE;
    const int tn = (int)(n - base < SCAN_TILE ? n - base : SCAN_TILE);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        const int e = j * SCAN_THREADS + tid;
        s[scan_pad(e)] = e < tn ? in[base + e] : 0;
    }
    __syncthreads();
    int32_t v[SCAN_ITEMS], sum = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        v[j] = s[scan_pad(tid * SCAN_ITEMS + j)];
        sum += v[j];
    }
    int32_t agg;
    const int32_t excl = block_exclusive_scan<int32_t>(sum, sh, &agg);
    if (wid == 0) {
        uint32_t prefix = 0;
        if (tile == 0) {
            if (lane == 0) st_relaxed_u32(status, SC_PRE | (uint32_t)agg);
        } else {
            if (lane == 0) st_relaxed_u32(status + tile, SC_AGG | (uint32_t)agg);
            for (int64_t t0 = tile - 1;; t0 -= 32) {
                const int64_t t = t0 - lane;
                uint32_t w = SC_PRE;                      // before tile 0: an empty prefix
                if (t >= 0) {
                    w = ld_relaxed_u32(status + t);
                    for (int spin = 0; (w & ~SC_VAL) == 0 && spin < SC_SPIN; spin++) w = ld_relaxed_u32(status + t);
                    if ((w & ~SC_VAL) == 0) {             // a tile that never published: report, stop
                        atomicCAS(err, 0, HC_ERR_STATE);
                        w = SC_PRE;
                    }
                }
                const unsigned pre = __ballot_sync(0xffffffffu, (w & ~SC_VAL) == SC_PRE);
                const int stop = pre ? __ffs(pre) - 1 : 31;
                uint32_t x = lane <= stop ? (w & SC_VAL) : 0u;
#pragma unroll
                for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                prefix += x;
                if (pre) break;
            }
            if (lane == 0) st_relaxed_u32(status + tile, SC_PRE | (prefix + (uint32_t)agg));
        }
        if (lane == 0) s_prefix = (int32_t)prefix;
    }
    __syncthreads();
    int32_t run = s_prefix + excl;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        s[scan_pad(tid * SCAN_ITEMS + j)] = run;
        run += v[j];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        const int e = j * SCAN_THREADS + tid;
        if (e < tn) out[base + e] = s[scan_pad(e)];
    }
    if (total && tid == 0 && base + SCAN_TILE >= n) *total = s_prefix + agg;   // the last tile
}

// scratch: [0] tile counter, [32, 32 + ntiles) look-back words
template <typename T>
void scan_exclusive(cudaStream_t s, const T *in, T *out, int64_t n, uint32_t *scratch, T *total_dev, int *err,
                    int64_t *launches)
{
    if (n <= 0) {
        if (total_dev) cudaMemsetAsync(total_dev, 0, sizeof(T), s);
        return;
    }
    const int64_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * (32 + ntiles), s);
    k_scan_onepass<<<(unsigned)ntiles, SCAN_THREADS, 0, s>>>(in, out, n, scratch + 32, scratch, total_dev, err);
    *launches += 1;
}

// ---- radix sort passes over the 64-bit high key ----
//
// One-sweep LSD radix sort: one kernel counts the digits of every pass over
// all keys, one block turns the counts into each pass's digit offsets, then
// one kernel per 8-bit pass.  A pass's tiles (4096 keys) take their tile index
// from a counter in launch order, count their digits, publish the counts and
// find the counts of all earlier tiles by decoupled look-back (Merrill and
// Garland, "Single-pass parallel prefix scan with decoupled look-back", 2016):
// each tile's word per digit holds a flag (aggregate or inclusive prefix) and a
// count, so a tile sums aggregates backwards until it meets a prefix.  A tile
// only waits on tiles that already hold their index, so every wait ends; each
// has an iteration limit nonetheless, after which the status word reports an
// error.  Scatter is stable (keys of a tile ranked in index order).

constexpr uint32_t LB_AGG = 1u << 30, LB_PRE = 2u << 30, LB_VAL = (1u << 30) - 1u;
constexpr int LB_SPIN = 1 << 20;
constexpr int LB_WIN = 8;        // earlier tiles read per look-back step
constexpr int NPASS_MAX = 8;

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// digit counts of every pass: ghist[pass][256]
__global__ void __launch_bounds__(SORT_THREADS) k_sort_hist(const unsigned long long *khi, int64_t n, const int *n_dev,
                                                             int begin_bit, int npass, uint32_t *ghist)
{
    if (n_dev && *n_dev < n) n = *n_dev;
    __shared__ uint32_t h[NPASS_MAX][256];
    for (int p = 0; p < NPASS_MAX; p++) h[p][threadIdx.x] = 0;
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * SORT_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * SORT_THREADS) {
        const unsigned long long k = khi[i];
        for (int p = 0; p < npass; p++) atomicAdd(&h[p][(k >> (begin_bit + 8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int p = 0; p < npass; p++)
        if (h[p][threadIdx.x]) atomicAdd(&ghist[p * 256 + threadIdx.x], h[p][threadIdx.x]);
}

// exclusive scan of each pass's 256 digit counts (one block of 256 threads)
__global__ void k_sort_offsets(uint32_t *ghist, int npass)
{
    __shared__ uint32_t sh[32];
    for (int p = 0; p < npass; p++) {
        const uint32_t v = ghist[p * 256 + threadIdx.x];
        const uint32_t ex = block_exclusive_scan<uint32_t>(v, sh, nullptr);
        ghist[p * 256 + threadIdx.x] = ex;
    }
}

// dynamic shared memory of k_sort_pass: the tile's keys, low keys and values
// in digit order (staged so that each digit's run is written out contiguously)
constexpr size_t SORT_PASS_SMEM = (size_t)SORT_TILE * (sizeof(unsigned long long) + 2 * sizeof(uint32_t));
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int WARP_KEYS = SORT_TILE / SORT_WARPS;      // contiguous keys ranked by one warp

__global__ void __launch_bounds__(SORT_THREADS) k_sort_pass(
    const unsigned long long *__restrict__ ihi, const uint32_t *__restrict__ ilo, const uint32_t *__restrict__ ival,
    unsigned long long *__restrict__ ohi, uint32_t *__restrict__ olo, uint32_t *__restrict__ oval, int64_t n,
    const int *n_dev, int shift, const uint32_t *goff, uint32_t *look, uint32_t *tile_ctr, int *err)
{
    if (n_dev && *n_dev < n) n = *n_dev;
    extern __shared__ unsigned long long stage_k[];                    // [SORT_TILE]
    uint32_t *stage_lo = reinterpret_cast<uint32_t *>(stage_k + SORT_TILE);   // [SORT_TILE]
    uint32_t *stage_v = stage_lo + SORT_TILE;                          // [SORT_TILE]
    __shared__ uint32_t s_tile;
    __shared__ uint32_t gbase[256];        // global position of the tile's first key of each digit
    __shared__ uint32_t lbase[256];        // start of each digit's run in the stage
    __shared__ uint32_t wcnt[SORT_WARPS][256];   // per warp: digit counts, then the warp's offsets in a run
    __shared__ uint32_t scan_sh[32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
#pragma unroll
    for (int w = 0; w < SORT_WARPS; w++) wcnt[w][tid] = 0;
    __syncthreads();
    const int64_t tile = s_tile;
    const int64_t ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    if (tile >= ntiles) return;                       // the whole block
    const int64_t base = tile * SORT_TILE;
    const int tn = (int)(n - base < SORT_TILE ? n - base : SORT_TILE);
    // each warp loads and ranks its contiguous slice [wid * WARP_KEYS, +WARP_KEYS)
    // in index order with warp-private digit counters (no block barrier per round)
    unsigned long long k[SORT_ITEMS];
    uint32_t lo[SORT_ITEMS], va[SORT_ITEMS];
#pragma unroll
    for (int r = 0; r < SORT_ITEMS; r++) {
        const int e = wid * WARP_KEYS + r * 32 + lane;
        const bool valid = e < tn;
        k[r] = valid ? ihi[base + e] : 0ull;
        lo[r] = (valid && ilo) ? ilo[base + e] : 0u;
        va[r] = valid ? ival[base + e] : 0u;
    }
    uint32_t rk[SORT_ITEMS / 2];           // ranks in the warp, two 16-bit values per word
#pragma unroll
    for (int r = 0; r < SORT_ITEMS; r++) {
        const int e = wid * WARP_KEYS + r * 32 + lane;
        const int dr = e < tn ? (int)((k[r] >> shift) & 255u) : 256 + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, dr);
        const int leader = __ffs(peers) - 1;
        uint32_t before = 0;
        if (dr < 256 && lane == leader) {
            before = wcnt[wid][dr];
            wcnt[wid][dr] = before + __popc(peers);
        }
        before = __shfl_sync(0xffffffffu, before, leader);
        const uint32_t rank = before + __popc(peers & lt);
        if (r & 1) rk[r >> 1] |= rank << 16;
        else rk[r >> 1] = rank;
        __syncwarp();
    }
    __syncthreads();
    // thread = digit: the tile's count, each warp's offset inside the digit's run
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < SORT_WARPS; w++) {
        const uint32_t c = wcnt[w][tid];
        wcnt[w][tid] = cnt;
        cnt += c;
    }
    // publish, then look back over the earlier tiles
    uint32_t *mine = look + tile * 256 + tid;
    uint32_t prefix = 0;
    if (tile == 0) {
        st_relaxed(mine, LB_PRE | cnt);
    } else {
        st_relaxed(mine, LB_AGG | cnt);
        // walk back LB_WIN tiles per step: their words are loaded together
        bool done = false;
        for (int64_t t0 = tile - 1; t0 >= 0 && !done; t0 -= LB_WIN) {
            uint32_t v[LB_WIN];
#pragma unroll
            for (int j = 0; j < LB_WIN; j++) v[j] = t0 - j >= 0 ? ld_relaxed(look + (t0 - j) * 256 + tid) : LB_PRE;
#pragma unroll
            for (int j = 0; j < LB_WIN; j++) {
                if (done || t0 - j < 0) continue;
                const uint32_t *q = look + (t0 - j) * 256 + tid;
                for (int spin = 0; (v[j] & ~LB_VAL) == 0 && spin < LB_SPIN; spin++) v[j] = ld_relaxed(q);
                if ((v[j] & ~LB_VAL) == 0) {          // a tile that never published: report, stop
                    atomicCAS(err, 0, HC_ERR_STATE);
                    done = true;
                    continue;
                }
                prefix += v[j] & LB_VAL;
                if ((v[j] & ~LB_VAL) == LB_PRE) done = true;
            }
        }
        st_relaxed(mine, LB_PRE | (prefix + cnt));
    }
    gbase[tid] = goff[tid] + prefix;
    lbase[tid] = block_exclusive_scan<uint32_t>(cnt, scan_sh, nullptr);
    __syncthreads();
    // stage in digit order: run start + earlier warps' keys of the digit + rank in the warp
#pragma unroll
    for (int r = 0; r < SORT_ITEMS; r++) {
        const int e = wid * WARP_KEYS + r * 32 + lane;
        if (e >= tn) continue;
        const int dr = (int)((k[r] >> shift) & 255u);
        const uint32_t rank = (rk[r >> 1] >> ((r & 1) * 16)) & 0xffffu;
        const uint32_t off = lbase[dr] + wcnt[wid][dr] + rank;
        stage_k[off] = k[r];
        stage_lo[off] = lo[r];
        stage_v[off] = va[r];
    }
    __syncthreads();
    // write out in stage order: consecutive keys of one digit go to consecutive places
    for (int e = tid; e < tn; e += SORT_THREADS) {
        const unsigned long long key = stage_k[e];
        const int dd = (int)((key >> shift) & 255u);
        const uint32_t pos = gbase[dd] + (uint32_t)e - lbase[dd];
        ohi[pos] = key;
        if (olo) olo[pos] = stage_lo[e];
        oval[pos] = stage_v[e];
    }
}

// Runs of equal 63-bit high keys (two bodies closer than 2^-21 of the root
// box) are ordered by the low 27 key bits; runs are a few entries long.
__global__ void k_tie_fix(unsigned long long *hi, uint32_t *lo, uint32_t *val, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i + 1 >= n || hi[i + 1] != hi[i]) continue;
        if (i > 0 && hi[i - 1] == hi[i]) continue;
        int64_t e = i + 1;
        while (e + 1 < n && hi[e + 1] == hi[i]) e++;
        for (int64_t a = i + 1; a <= e; a++) {      // stable insertion sort by lo
            uint32_t kl = lo[a], kv = val[a];
            int64_t b = a - 1;
            while (b >= i && lo[b] > kl) {
                lo[b + 1] = lo[b];
                val[b + 1] = val[b];
                b--;
            }
            lo[b + 1] = kl;
            val[b + 1] = kv;
        }
    }
}

}  // namespace

void hc_scan_exclusive_i32(hc_ctx *c, const int32_t *in, int32_t *out, int64_t n, int32_t *total_dev)
{
    scan_exclusive<int32_t>(c->stream, in, out, n, c->scan_tmp, total_dev, &c->st->error, &c->launches);
}

int64_t hc_scan_scratch_words(int64_t n) { return 32 + (n + SCAN_TILE - 1) / SCAN_TILE; }

// Sort (khi, klo, kval)[sel] by the high key bits [begin_bit, end_bit) in
// 8-bit passes, then order equal-high-key runs by the low key when tie_fix.
// n bounds the launch; when n_dev is given the kernels sort min(n, *n_dev)
// entries (a count only the device knows).  Returns the result's buffer.
// once per context, before any capture: k_sort_pass stages 64 KB per block
int hc_sort_setup(hc_ctx *c)
{
    HC_CUDA(cudaFuncSetAttribute(k_sort_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SORT_PASS_SMEM));
    return HC_OK;
}

int64_t hc_sort_scratch_words(int64_t n)
{
    const int64_t ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    return 4096 + (int64_t)NPASS_MAX * 256 * (ntiles < 1 ? 1 : ntiles);
}

int hc_radix_sort_keys(hc_ctx *c, uint32_t *scratch, unsigned long long *khi[2], uint32_t *klo[2],
                       uint32_t *kval[2], int64_t n, int begin_bit, int end_bit, bool tie_fix, const int *n_dev)
{
    int sel = 0;
    if (n <= 0) return sel;
    const int npass = (end_bit - begin_bit + 7) / 8;
    const int64_t ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    // scratch: [0, 2048) digit counts -> offsets per pass (left there: the
    // depth sort's offsets are the tree's level starts), [2048, 2056) tile
    // counters, [4096, ...) look-back words, ntiles x 256 per pass
    uint32_t *ghist = scratch, *ctr = scratch + 2048, *look = scratch + 4096;
    cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * (4096 + (size_t)npass * 256 * ntiles), c->stream);
    const int hblocks = (int)std::min<int64_t>((n + SORT_TILE - 1) / SORT_TILE, 152 * 8);
    k_sort_hist<<<hblocks < 1 ? 1 : hblocks, SORT_THREADS, 0, c->stream>>>(khi[sel], n, n_dev, begin_bit, npass,
                                                                          ghist);
    k_sort_offsets<<<1, 256, 0, c->stream>>>(ghist, npass);
    c->launches += 2;
    for (int p = 0; p < npass; p++) {
        k_sort_pass<<<(unsigned)ntiles, SORT_THREADS, SORT_PASS_SMEM, c->stream>>>(
            khi[sel], klo[sel], kval[sel], khi[sel ^ 1], klo[sel ^ 1], kval[sel ^ 1], n, n_dev, begin_bit + 8 * p,
            ghist + 256 * p, look + (int64_t)p * 256 * ntiles, ctr + p, &c->st->error);
        c->launches++;
        sel ^= 1;
    }
    if (tie_fix) {
        k_tie_fix<<<hc_grid(n, 256), 256, 0, c->stream>>>(khi[sel], klo[sel], kval[sel], n);
        c->launches++;
    }
    return sel;
}
