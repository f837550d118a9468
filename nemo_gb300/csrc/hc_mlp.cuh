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

struct __align__(16) MlpSmem {     // 16-byte aligned: ldmatrix row addresses
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

// Four 8x8 bf16 matrices from shared memory in one instruction (PTX
// ldmatrix): lane i gives the row address of row i % 8 of matrix i / 8 and
// receives r[m] = elements 2 (i % 4), +1 of row i / 4 of matrix m -- for a
// weight stored as W^T[n][k] that is the B fragment (n = g, k = 2t, 2t+1) of
// mma.m16n8k16.  Row addresses must be 16-byte aligned.
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const __nv_bfloat16 *row)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// silu of a pair of values: the products and sums in packed FP32x2 (each half
// rounded as the scalar instruction would), the tanh per value
__device__ __forceinline__ float2 silu2(float2 x)
{
    const float2 h = __fmul2_rn(x, make_float2(0.5f, 0.5f));
    return __ffma2_rn(h, make_float2(tanh_fast(h.x), tanh_fast(h.y)), h);
}

__device__ __forceinline__ uint32_t pack_bf16_2(float2 v) { return pack_bf16(v.x, v.y); }

// Logits of the rows of x, for use inline in a register-heavy kernel: one
// 16-row m-tile at a time (rows >= nrows are skipped in 16-row steps), weight
// fragments loaded per use with ldmatrix, biases as the accumulators' initial
// values, activations in packed FP32x2; the logits pass through z[32]
// (shared memory of the warp).  x: this warp's 32 x MLP_XS bf16 input tile
// (row r = lane r's candidate, columns 12..15 zero).  Returns the logit of row
// `lane`.
__device__ __forceinline__ float mlp_warp_lean(const MlpSmem &P, const __nv_bfloat16 *x, float *z, int nrows)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int lr = lane & 7, lm = lane >> 3;     // ldmatrix: row and matrix this lane addresses
    const uint32_t *xw = reinterpret_cast<const uint32_t *>(x);
    const int nmt = nrows <= 16 ? 1 : 2;
#pragma unroll 1
    for (int mt = 0; mt < nmt; mt++) {
        const int r0 = mt * 16;
        uint32_t a[4];
        a[0] = xw[((r0 + g) * MLP_XS + 2 * t) >> 1];
        a[1] = xw[((r0 + g + 8) * MLP_XS + 2 * t) >> 1];
        a[2] = xw[((r0 + g) * MLP_XS + 2 * t + 8) >> 1];
        a[3] = xw[((r0 + g + 8) * MLP_XS + 2 * t + 8) >> 1];
        // ---- layer 1: [16 x 16] x [16 x 64], two n-tiles per ldmatrix ----
        uint32_t h1[4][4];                   // activations as layer-2 A fragments (k-tiles 0..3)
#pragma unroll
        for (int np = 0; np < 4; np++) {
            uint32_t b[4];                   // n-tiles 2np, 2np+1: (k 0-7, k 8-15) each
            ldsm_x4(b, P.w1t + (16 * np + 8 * (lm >> 1) + lr) * MLP_S1 + 8 * (lm & 1));
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int col = (2 * np + hh) * 8 + 2 * t;
                const float2 bias = make_float2(P.b1[col], P.b1[col + 1]);
                float c[4] = {bias.x, bias.y, bias.x, bias.y};
                mma_bf16_16816(c, a, b[2 * hh], b[2 * hh + 1]);
                h1[np][hh * 2 + 0] = pack_bf16_2(silu2(make_float2(c[0], c[1])));   // row g
                h1[np][hh * 2 + 1] = pack_bf16_2(silu2(make_float2(c[2], c[3])));   // row g + 8
            }
        }
        // ---- layer 2: [16 x 64] x [64 x 64], then layer 3 on the fly ----
        float c3[4] = {0.f, 0.f, 0.f, 0.f};
        float2 hold0 = make_float2(0.f, 0.f), hold1 = hold0;
#pragma unroll 2
        for (int nt = 0; nt < 8; nt++) {
            const int col = nt * 8 + 2 * t;
            uint32_t b01[4], b23[4];         // k-tiles 0,1 and 2,3 of n-tile nt
            ldsm_x4(b01, P.w2t + (8 * nt + lr) * MLP_S2 + 8 * lm);
            ldsm_x4(b23, P.w2t + (8 * nt + lr) * MLP_S2 + 32 + 8 * lm);
            // k-tiles 0,1 and 2,3 in two independent accumulators (shorter mma chain)
            const float2 bias = make_float2(P.b2[col], P.b2[col + 1]);
            float c[4] = {bias.x, bias.y, bias.x, bias.y}, e[4] = {0.f, 0.f, 0.f, 0.f};
            mma_bf16_16816(c, h1[0], b01[0], b01[1]);
            mma_bf16_16816(e, h1[2], b23[0], b23[1]);
            mma_bf16_16816(c, h1[1], b01[2], b01[3]);
            mma_bf16_16816(e, h1[3], b23[2], b23[3]);
            const float2 v01 = silu2(__fadd2_rn(make_float2(c[0], c[1]), make_float2(e[0], e[1])));
            const float2 v23 = silu2(__fadd2_rn(make_float2(c[2], c[3]), make_float2(e[2], e[3])));
            if (nt & 1) {
                const int kt = nt >> 1;
                // A fragment: rows g / g+8 of n-tiles nt-1 (held) and nt
                const uint32_t af[4] = {pack_bf16_2(hold0), pack_bf16_2(hold1), pack_bf16_2(v01), pack_bf16_2(v23)};
                const uint32_t *w3 = reinterpret_cast<const uint32_t *>(P.w3t);
                mma_bf16_16816(c3, af, w3[(g * MLP_S2 + kt * 16 + 2 * t) >> 1],
                               w3[(g * MLP_S2 + kt * 16 + 2 * t + 8) >> 1]);
            } else {
                hold0 = v01;
                hold1 = v23;
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

