// hc_sort.cu -- device scan and LSD radix sort for the octree keys.
//
// The reference inserts bodies one by one (loadtree, load.c:101-128); the
// GB300 build instead sorts all bodies by their 90-bit integer-coordinate key
// (top 63 bits radix sorted, the low 27 bits resolved inside runs of equal
// high keys), so that every octree cell is a contiguous run of sorted bodies.
// Both kernels here are HBM-bound integer work: coalesced tile loads, block-
// local histograms in shared memory, stable scatter.
#include "hc_internal.cuh"

namespace {

constexpr int SCAN_BLOCK = 512;
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

// Phase 1: per-block sums of contiguous chunks.
template <typename T>
__global__ void k_scan_reduce(const T *in, int64_t n, int64_t chunk, T *part)
{
    __shared__ T sh[32];
    int64_t beg = (int64_t)blockIdx.x * chunk, end = min(beg + chunk, n);
    T s = 0;
    for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) s += in[i];
    T tot;
    block_exclusive_scan<T>(s, sh, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// Phase 2: exclusive scan of the block sums (one block, <= SCAN_BLOCK parts).
template <typename T>
__global__ void k_scan_parts(T *part, int nparts, T *total)
{
    __shared__ T sh[32];
    T v = threadIdx.x < nparts ? part[threadIdx.x] : T(0);
    T tot;
    T ex = block_exclusive_scan<T>(v, sh, &tot);
    if (threadIdx.x < nparts) part[threadIdx.x] = ex;
    if (threadIdx.x == 0 && total) *total = tot;
}

// Phase 3: scan each chunk in tiles of blockDim, offset by its block prefix.
template <typename T>
__global__ void k_scan_down(const T *in, T *out, int64_t n, int64_t chunk, const T *part)
{
    __shared__ T sh[32];
    int64_t beg = (int64_t)blockIdx.x * chunk, end = min(beg + chunk, n);
    T carry = part[blockIdx.x];
    for (int64_t t = beg; t < end; t += blockDim.x) {
        int64_t i = t + threadIdx.x;
        T v = i < end ? in[i] : T(0);
        T tot;
        T ex = block_exclusive_scan<T>(v, sh, &tot);
        if (i < end) out[i] = carry + ex;
        carry += tot;
    }
}

template <typename T>
void scan_exclusive(cudaStream_t s, const T *in, T *out, int64_t n, T *part, T *total_dev, int64_t *launches)
{
    int64_t np = (n + 4095) / 4096;
    int nparts = (int)(np < 1 ? 1 : (np > SCAN_BLOCK ? SCAN_BLOCK : np));
    int64_t chunk = (n + nparts - 1) / nparts;
    if (chunk < 1) chunk = 1;
    k_scan_reduce<T><<<nparts, 256, 0, s>>>(in, n, chunk, part);
    k_scan_parts<T><<<1, SCAN_BLOCK, 0, s>>>(part, nparts, total_dev);
    k_scan_down<T><<<nparts, 256, 0, s>>>(in, out, n, chunk, part);
    *launches += 3;
}

// ---- radix sort passes over the 64-bit high key ----

__global__ void k_radix_hist(const unsigned long long *khi, int64_t n, const int *n_dev, int shift, uint32_t *hist,
                             int nblk)
{
    if (n_dev && *n_dev < n) n = *n_dev;
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * SORT_TILE;
#pragma unroll 4
    for (int r = 0; r < SORT_ITEMS; r++) {
        int64_t i = base + r * SORT_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(khi[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(SORT_THREADS) k_radix_scatter(
    const unsigned long long *ihi, const uint32_t *ilo, const uint32_t *ival,
    unsigned long long *ohi, uint32_t *olo, uint32_t *oval, int64_t n, const int *n_dev, int shift,
    const uint32_t *offs, int nblk)
{
    if (n_dev && *n_dev < n) n = *n_dev;
    __shared__ uint32_t running[256];
    __shared__ uint32_t wcnt[SORT_THREADS / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    running[tid] = offs[(int64_t)tid * nblk + blockIdx.x];
#pragma unroll
    for (int w = 0; w < SORT_THREADS / 32; w++) wcnt[w][tid] = 0;
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    int64_t base = (int64_t)blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_ITEMS; r++) {
        int64_t i = base + r * SORT_THREADS + tid;
        bool valid = i < n;
        unsigned long long k = valid ? ihi[i] : 0ull;
        uint32_t lo = (valid && ilo) ? ilo[i] : 0u, v = valid ? ival[i] : 0u;
        int d = valid ? (int)((k >> shift) & 255u) : (0x1000 | lane);
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int wrank = __popc(peers & lt);
        if (valid && (__ffs(peers) - 1) == lane) wcnt[wid][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t off = running[d] + wrank;
            for (int w = 0; w < wid; w++) off += wcnt[w][d];
            ohi[off] = k;
            if (olo) olo[off] = lo;
            oval[off] = v;
        }
        __syncthreads();
        uint32_t tot = 0;
#pragma unroll
        for (int w = 0; w < SORT_THREADS / 32; w++) {
            tot += wcnt[w][tid];
            wcnt[w][tid] = 0;
        }
        running[tid] += tot;
        __syncthreads();
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
    scan_exclusive<int32_t>(c->stream, in, out, n, c->scan_tmp, total_dev, &c->launches);
}

// Sort (khi, klo, kval)[sel] by the high key bits [begin_bit, end_bit) in
// 8-bit passes, then order equal-high-key runs by the low key when tie_fix.
// n bounds the launch; when n_dev is given the kernels sort min(n, *n_dev)
// entries (a count only the device knows).  Returns the result's buffer.
int hc_radix_sort_keys(hc_ctx *c, unsigned long long *khi[2], uint32_t *klo[2], uint32_t *kval[2],
                       int64_t n, int begin_bit, int end_bit, bool tie_fix, const int *n_dev)
{
    int sel = 0;
    if (n <= 0) return sel;
    int nblk = (int)((n + SORT_TILE - 1) / SORT_TILE);
    int64_t nh = (int64_t)256 * nblk;
    for (int shift = begin_bit; shift < end_bit; shift += 8) {
        k_radix_hist<<<nblk, SORT_THREADS, 0, c->stream>>>(khi[sel], n, n_dev, shift, c->hist, nblk);
        scan_exclusive<uint32_t>(c->stream, c->hist, c->hist, nh, (uint32_t *)c->scan_tmp, nullptr,
                                 &c->launches);
        k_radix_scatter<<<nblk, SORT_THREADS, 0, c->stream>>>(khi[sel], klo[sel], kval[sel], khi[sel ^ 1],
                                                              klo[sel ^ 1], kval[sel ^ 1], n, n_dev, shift,
                                                              c->hist, nblk);
        c->launches += 2;
        sel ^= 1;
    }
    if (tie_fix) {
        k_tie_fix<<<hc_grid(n, 256), 256, 0, c->stream>>>(khi[sel], klo[sel], kval[sel], n);
        c->launches++;
    }
    return sel;
}
