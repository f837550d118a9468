// hc_mlp.cuh -- the opening-criterion network: 12 inputs, two hidden layers
// of 64 SiLU units, one logit.  BF16 weights and activations, FP32
// accumulation, evaluated by one warp for 32 rows at a time with
// mma.sync.m16n8k16 (bf16 x bf16 -> f32).
//
// Shared-memory image (bf16 weights transposed, rows padded so that the
// B-fragment loads of the 8 row groups hit distinct banks):
//   w1t[64][MLP_S1]  (k = input feature, 12 used of 16)
//   w2t[64][MLP_S2]
//   w3t[8][MLP_S2]   (row 0 = output weights, rows 1..7 zero)
//   b1[64], b2[64], b3 (fp32)
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#define MLP_IN 12
#define MLP_H 64
#define MLP_K1 16            // padded input width
#define MLP_S1 24            // row stride (bf16) of w1t
#define MLP_S2 72            // row stride (bf16) of w2t / w3t
#define MLP_XS 24            // row stride (bf16) of a 32 x 16 input tile

struct MlpSmem {
    __nv_bfloat16 w1t[MLP_H * MLP_S1];
    __nv_bfloat16 w2t[MLP_H * MLP_S2];
    __nv_bfloat16 w3t[8 * MLP_S2];
    float b1[MLP_H], b2[MLP_H], b3;
};

// Packed parameters in global memory (same layout as MlpSmem).
struct MlpParams {
    MlpSmem s;
};

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

// tanh.approx.f32: one MUFU operation (PTX ISA, "tanh" instruction).
__device__ __forceinline__ float tanh_fast(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// logistic sigma(x) = (1 + tanh(x/2)) / 2 and silu(x) = x sigma(x) = h + h tanh(h)
// with h = x/2; training and inference use the same tanh so the trained
// network is the evaluated one.
__device__ __forceinline__ float sigm_fast(float x) { return fmaf(0.5f, tanh_fast(0.5f * x), 0.5f); }
__device__ __forceinline__ float silu(float x)
{
    const float h = 0.5f * x;
    return fmaf(h, tanh_fast(h), h);
}

// Copy packed parameters into shared memory (whole block cooperates).
__device__ __forceinline__ void mlp_load(MlpSmem &dst, const MlpSmem *src)
{
    const uint32_t *s = reinterpret_cast<const uint32_t *>(src);
    uint32_t *d = reinterpret_cast<uint32_t *>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(MlpSmem) / 4); i += blockDim.x) d[i] = s[i];
}

// Logits of MT * 16 rows (MT = 1 or 2).  x: this warp's 32 x MLP_XS bf16
// input tile (row r = lane r's candidate, columns 12..15 zero).  Returns the
// logit of row `lane` (rows >= MT * 16: undefined).  The two m-tiles share
// every weight-fragment load.  Callers keep it out of line (mlp_warp32, or a
// non-inlined caller of their own): its fragments would otherwise raise the
// register count of the code around it.
template <int MT>
__device__ __forceinline__ float mlp_warp(const MlpSmem &P, const __nv_bfloat16 *x)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t *xw = reinterpret_cast<const uint32_t *>(x);
    const uint32_t *w1 = reinterpret_cast<const uint32_t *>(P.w1t);
    const uint32_t *w2 = reinterpret_cast<const uint32_t *>(P.w2t);
    const uint32_t *w3 = reinterpret_cast<const uint32_t *>(P.w3t);
    // ---- layer 1: [16 x 16] x [16 x 64] per m-tile ----
    uint32_t a[MT][4];
#pragma unroll
    for (int mt = 0; mt < MT; mt++) {
        const int r0 = mt * 16;
        a[mt][0] = xw[((r0 + g) * MLP_XS + 2 * t) >> 1];
        a[mt][1] = xw[((r0 + g + 8) * MLP_XS + 2 * t) >> 1];
        a[mt][2] = xw[((r0 + g) * MLP_XS + 2 * t + 8) >> 1];
        a[mt][3] = xw[((r0 + g + 8) * MLP_XS + 2 * t + 8) >> 1];
    }
    uint32_t h1[MT][4][4];                   // layer-1 activations as layer-2 A fragments (k-tiles 0..3)
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int n = nt * 8 + g, col = nt * 8 + 2 * t;
        const uint32_t b0 = w1[(n * MLP_S1 + 2 * t) >> 1], b1 = w1[(n * MLP_S1 + 2 * t + 8) >> 1];
        const float bias0 = P.b1[col], bias1 = P.b1[col + 1];
#pragma unroll
        for (int mt = 0; mt < MT; mt++) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            mma_bf16_16816(c, a[mt], b0, b1);
            const int kt = nt >> 1, half = nt & 1;
            h1[mt][kt][half * 2 + 0] = pack_bf16(silu(c[0] + bias0), silu(c[1] + bias1));   // row g
            h1[mt][kt][half * 2 + 1] = pack_bf16(silu(c[2] + bias0), silu(c[3] + bias1));   // row g + 8
        }
    }
    // ---- layer 2: [16 x 64] x [64 x 64], then layer 3 on the fly ----
    float c3[MT][4], hold[MT][4];
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
        for (int q = 0; q < 4; q++) c3[mt][q] = hold[mt][q] = 0.f;
#pragma unroll 2
    for (int nt = 0; nt < 8; nt++) {
        const int n = nt * 8 + g, col = nt * 8 + 2 * t;
        uint32_t b[4][2];
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            b[kt][0] = w2[(n * MLP_S2 + kt * 16 + 2 * t) >> 1];
            b[kt][1] = w2[(n * MLP_S2 + kt * 16 + 2 * t + 8) >> 1];
        }
        const float bias0 = P.b2[col], bias1 = P.b2[col + 1];
        uint32_t w3b0 = 0u, w3b1 = 0u;
        if (nt & 1) {
            const int kt = nt >> 1;
            w3b0 = w3[(g * MLP_S2 + kt * 16 + 2 * t) >> 1];
            w3b1 = w3[(g * MLP_S2 + kt * 16 + 2 * t + 8) >> 1];
        }
#pragma unroll
        for (int mt = 0; mt < MT; mt++) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kt = 0; kt < 4; kt++) mma_bf16_16816(c, h1[mt][kt], b[kt][0], b[kt][1]);
            const float v0 = silu(c[0] + bias0), v1 = silu(c[1] + bias1);
            const float v2 = silu(c[2] + bias0), v3 = silu(c[3] + bias1);
            // layer 3 consumes k-tile nt/2 of the layer-2 output when both halves are ready
            if (nt & 1) {
                // A fragment: rows g / g+8 of n-tiles nt-1 (held) and nt
                const uint32_t af[4] = {pack_bf16(hold[mt][0], hold[mt][1]), pack_bf16(hold[mt][2], hold[mt][3]),
                                        pack_bf16(v0, v1), pack_bf16(v2, v3)};
                mma_bf16_16816(c3[mt], af, w3b0, w3b1);
            } else {
                hold[mt][0] = v0;
                hold[mt][1] = v1;
                hold[mt][2] = v2;
                hold[mt][3] = v3;
            }
        }
    }
    // column 0 of c3 (t == 0 lanes) holds rows g and g + 8 of each m-tile.
    // Lane r wants row r: rows (r&7) and (r&7)+8 of its m-tile sit in lane 4 (r&7).
    const int rr = lane & 15, src_lane = (rr & 7) * 4;
    const float a0 = __shfl_sync(0xffffffffu, c3[0][0], src_lane), a1 = __shfl_sync(0xffffffffu, c3[0][2], src_lane);
    float v = rr < 8 ? a0 : a1;
    if (MT == 2) {
        const float b0 = __shfl_sync(0xffffffffu, c3[MT - 1][0], src_lane);
        const float b1 = __shfl_sync(0xffffffffu, c3[MT - 1][2], src_lane);
        if (lane >= 16) v = rr < 8 ? b0 : b1;
    }
    return v + P.b3;
}

// Register-lean form of mlp_warp for use inline in a register-heavy kernel:
// one m-tile at a time, weight fragments loaded per use; the logits pass
// through z[32] (shared memory of the warp).  Rows >= nrows are skipped in
// 16-row steps.
__device__ __forceinline__ float mlp_warp_lean(const MlpSmem &P, const __nv_bfloat16 *x, float *z, int nrows)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t *xw = reinterpret_cast<const uint32_t *>(x);
    const uint32_t *w1 = reinterpret_cast<const uint32_t *>(P.w1t);
    const uint32_t *w2 = reinterpret_cast<const uint32_t *>(P.w2t);
    const uint32_t *w3 = reinterpret_cast<const uint32_t *>(P.w3t);
    const int nmt = nrows <= 16 ? 1 : 2;
#pragma unroll 1
    for (int mt = 0; mt < nmt; mt++) {
        const int r0 = mt * 16;
        uint32_t a[4];
        a[0] = xw[((r0 + g) * MLP_XS + 2 * t) >> 1];
        a[1] = xw[((r0 + g + 8) * MLP_XS + 2 * t) >> 1];
        a[2] = xw[((r0 + g) * MLP_XS + 2 * t + 8) >> 1];
        a[3] = xw[((r0 + g + 8) * MLP_XS + 2 * t + 8) >> 1];
        uint32_t h1[4][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int n = nt * 8 + g, col = nt * 8 + 2 * t;
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            mma_bf16_16816(c, a, w1[(n * MLP_S1 + 2 * t) >> 1], w1[(n * MLP_S1 + 2 * t + 8) >> 1]);
            const float bias0 = P.b1[col], bias1 = P.b1[col + 1];
            const int kt = nt >> 1, half = nt & 1;
            h1[kt][half * 2 + 0] = pack_bf16(silu(c[0] + bias0), silu(c[1] + bias1));
            h1[kt][half * 2 + 1] = pack_bf16(silu(c[2] + bias0), silu(c[3] + bias1));
        }
        float c3[4] = {0.f, 0.f, 0.f, 0.f};
        float hold[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
        for (int nt = 0; nt < 8; nt++) {
            const int n = nt * 8 + g, col = nt * 8 + 2 * t;
            // k-tiles 0,1 and 2,3 in two independent accumulators (shorter mma chain)
            float c[4] = {0.f, 0.f, 0.f, 0.f}, e[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kt = 0; kt < 2; kt++) {
                mma_bf16_16816(c, h1[kt], w2[(n * MLP_S2 + kt * 16 + 2 * t) >> 1],
                               w2[(n * MLP_S2 + kt * 16 + 2 * t + 8) >> 1]);
                mma_bf16_16816(e, h1[kt + 2], w2[(n * MLP_S2 + (kt + 2) * 16 + 2 * t) >> 1],
                               w2[(n * MLP_S2 + (kt + 2) * 16 + 2 * t + 8) >> 1]);
            }
#pragma unroll
            for (int q = 0; q < 4; q++) c[q] += e[q];
            const float bias0 = P.b2[col], bias1 = P.b2[col + 1];
            const float v0 = silu(c[0] + bias0), v1 = silu(c[1] + bias1);
            const float v2 = silu(c[2] + bias0), v3 = silu(c[3] + bias1);
            if (nt & 1) {
                const int kt = nt >> 1;
                const uint32_t af[4] = {pack_bf16(hold[0], hold[1]), pack_bf16(hold[2], hold[3]), pack_bf16(v0, v1),
                                        pack_bf16(v2, v3)};
                mma_bf16_16816(c3, af, w3[(g * MLP_S2 + kt * 16 + 2 * t) >> 1],
                               w3[(g * MLP_S2 + kt * 16 + 2 * t + 8) >> 1]);
            } else {
                hold[0] = v0;
                hold[1] = v1;
                hold[2] = v2;
                hold[3] = v3;
            }
        }
        if (t == 0) {                        // column 0: rows g and g + 8 of this m-tile
            z[r0 + g] = c3[0];
            z[r0 + g + 8] = c3[2];
        }
    }
    __syncwarp();
    const float v = z[lane] + P.b3;
    __syncwarp();
    return v;
}

// Logits of the 32 rows of x (see mlp_warp); rows < nrows are needed.
static __device__ __noinline__ float mlp_warp32(const MlpSmem &P, const __nv_bfloat16 *x, int nrows = 32)
{
    return nrows <= 16 ? mlp_warp<1>(P, x) : mlp_warp<2>(P, x);
}
