// hc_learn.cu -- training and test-inference kernels of the learned opening
// criterion's network (hc_mlp.cuh).
//
// Parameters are kept as FP32 master weights in a flat vector
//   W1[64][12], b1[64], W2[64][64], b2[64], W3[64], b3     (5057 floats)
// and packed into the BF16 shared-memory image used by the walk.  Training is
// mini-batch Adam on a binary cross-entropy loss; the forward pass rounds
// weights and activations to BF16 exactly where inference does (straight-
// through gradients), so the trained network is the one the walk evaluates.
#include <cmath>
#include "hc_internal.cuh"
#include "hc_mlp.cuh"

namespace {

constexpr int NP = MLP_H * MLP_IN + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1;   // 5057
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + MLP_H * MLP_IN, OFF_W2 = OFF_B1 + MLP_H,
              OFF_B2 = OFF_W2 + MLP_H * MLP_H, OFF_W3 = OFF_B2 + MLP_H, OFF_B3 = OFF_W3 + MLP_H;

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float sigm(float x) { return sigm_fast(x); }          // hidden units (as inference)
__device__ __forceinline__ float sig_out(float x) { return __frcp_rn(1.0f + __expf(-x)); }   // output probability

__global__ void k_mlp_pack(const float *p, MlpSmem *out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_H * MLP_S2; i += gridDim.x * blockDim.x) {
        const int n = i / MLP_S2, k = i % MLP_S2;
        out->w2t[i] = __float2bfloat16_rn(k < MLP_H ? p[OFF_W2 + n * MLP_H + k] : 0.f);
        if (n < 8) out->w3t[i] = __float2bfloat16_rn((n == 0 && k < MLP_H) ? p[OFF_W3 + k] : 0.f);
        if (k < MLP_S1) out->w1t[n * MLP_S1 + k] = __float2bfloat16_rn(k < MLP_IN ? p[OFF_W1 + n * MLP_IN + k] : 0.f);
    }
    if (blockIdx.x == 0) {
        for (int j = threadIdx.x; j < MLP_H; j += blockDim.x) {
            out->b1[j] = p[OFF_B1 + j];
            out->b2[j] = p[OFF_B2 + j];
        }
        if (threadIdx.x == 0) out->b3 = p[OFF_B3];
    }
}

// Test inference: 32 rows per warp through the walk's mma.sync network.
__global__ void k_mlp_infer(const MlpSmem *params, const float *x, int64_t n, float *logits)
{
    __shared__ MlpSmem P;
    __shared__ __nv_bfloat16 tile[4][32 * MLP_XS];
    __shared__ float zbuf[4][32];
    mlp_load(P, params);
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t row = ((int64_t)blockIdx.x * 4 + w) * 32 + lane;
    for (int k = 0; k < MLP_XS; k++)
        tile[w][lane * MLP_XS + k] = __float2bfloat16_rn((row < n && k < MLP_IN) ? x[row * MLP_IN + k] : 0.f);
    __syncwarp();
    const float z = mlp_warp_lean(P, tile[w], zbuf[w], 32);     // the walk's network round
    if (row < n) logits[row] = z;
}

// Gradient of the mean (weighted) binary cross-entropy over rows [0, n) of
// one mini-batch: each block takes TB rows and writes its partial gradient
// (NP floats) and loss.
constexpr int TB = 64;
constexpr int GT = 256;

__global__ void __launch_bounds__(GT) k_mlp_grad(const float *p, const float *x, const float *y, const float *wt,
                                                 int64_t n, float inv_norm, float *gpart, float *lpart)
{
    extern __shared__ float sm[];
    float *W2 = sm;                          // [64][64] (bf16-rounded)
    float *X = W2 + MLP_H * MLP_H;           // [TB][12]
    float *Z1 = X + TB * MLP_IN;             // [TB][64] pre-activations
    float *H1 = Z1 + TB * MLP_H;             // [TB][64]
    float *Z2 = H1 + TB * MLP_H;
    float *H2 = Z2 + TB * MLP_H;
    float *D = H2 + TB * MLP_H;              // [TB] dL/dz3
    float *W1 = D + TB;                      // [64][12]
    float *W3 = W1 + MLP_H * MLP_IN;         // [64]
    float *red = W3 + MLP_H;                 // [GT]
    const int tid = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * TB;
    for (int i = tid; i < MLP_H * MLP_H; i += GT) W2[i] = bf(p[OFF_W2 + i]);
    for (int i = tid; i < MLP_H * MLP_IN; i += GT) W1[i] = bf(p[OFF_W1 + i]);
    for (int i = tid; i < MLP_H; i += GT) W3[i] = bf(p[OFF_W3 + i]);
    for (int i = tid; i < TB * MLP_IN; i += GT) {
        const int64_t r = r0 + i / MLP_IN;
        X[i] = r < n ? bf(x[r * MLP_IN + i % MLP_IN]) : 0.f;
    }
    __syncthreads();
    // forward
    for (int i = tid; i < TB * MLP_H; i += GT) {
        const int s = i / MLP_H, j = i % MLP_H;
        float z = p[OFF_B1 + j];
        for (int k = 0; k < MLP_IN; k++) z = fmaf(W1[j * MLP_IN + k], X[s * MLP_IN + k], z);
        Z1[i] = z;
        H1[i] = bf(silu(z));
    }
    __syncthreads();
    for (int i = tid; i < TB * MLP_H; i += GT) {
        const int s = i / MLP_H, j = i % MLP_H;
        float z = p[OFF_B2 + j];
        for (int k = 0; k < MLP_H; k++) z = fmaf(W2[j * MLP_H + k], H1[s * MLP_H + k], z);
        Z2[i] = z;
        H2[i] = bf(silu(z));
    }
    __syncthreads();
    float lsum = 0.f;
    for (int s = tid; s < TB; s += GT) {
        const int64_t r = r0 + s;
        float z = p[OFF_B3];
        for (int k = 0; k < MLP_H; k++) z = fmaf(W3[k], H2[s * MLP_H + k], z);
        float d = 0.f;
        if (r < n) {
            const float yy = y[r], ww = wt ? wt[r] : 1.f;
            // BCE with logits: max(z,0) - z y + log(1 + exp(-|z|))
            lsum += ww * (fmaxf(z, 0.f) - z * yy + log1pf(__expf(-fabsf(z))));
            d = ww * (sig_out(z) - yy) * inv_norm;
        }
        D[s] = d;
    }
    red[tid] = lsum;
    __syncthreads();
    // backward: dz2 = d * w3 * silu'(z2)  (stored over Z2)
    for (int i = tid; i < TB * MLP_H; i += GT) {
        const int s = i / MLP_H, j = i % MLP_H;
        const float z = Z2[i], sg = sigm(z);
        Z2[i] = D[s] * W3[j] * sg * (1.f + z * (1.f - sg));
    }
    __syncthreads();
    // dh1 = W2^T dz2 ; dz1 = dh1 * silu'(z1)  (stored over Z1)
    for (int i = tid; i < TB * MLP_H; i += GT) {
        const int s = i / MLP_H, k = i % MLP_H;
        float dh = 0.f;
        for (int j = 0; j < MLP_H; j++) dh = fmaf(W2[j * MLP_H + k], Z2[s * MLP_H + j], dh);
        const float z = Z1[i], sg = sigm(z);
        Z1[i] = dh * sg * (1.f + z * (1.f - sg));
    }
    __syncthreads();
    // parameter gradients (sums over this block's rows)
    float *gp = gpart + (int64_t)blockIdx.x * NP;
    for (int i = tid; i < NP; i += GT) {
        float g = 0.f;
        if (i < OFF_B1) {
            const int j = i / MLP_IN, k = i % MLP_IN;
            for (int s = 0; s < TB; s++) g = fmaf(Z1[s * MLP_H + j], X[s * MLP_IN + k], g);
        } else if (i < OFF_W2) {
            const int j = i - OFF_B1;
            for (int s = 0; s < TB; s++) g += Z1[s * MLP_H + j];
        } else if (i < OFF_B2) {
            const int j = (i - OFF_W2) / MLP_H, k = (i - OFF_W2) % MLP_H;
            for (int s = 0; s < TB; s++) g = fmaf(Z2[s * MLP_H + j], H1[s * MLP_H + k], g);
        } else if (i < OFF_W3) {
            const int j = i - OFF_B2;
            for (int s = 0; s < TB; s++) g += Z2[s * MLP_H + j];
        } else if (i < OFF_B3) {
            const int k = i - OFF_W3;
            for (int s = 0; s < TB; s++) g = fmaf(D[s], H2[s * MLP_H + k], g);
        } else {
            for (int s = 0; s < TB; s++) g += D[s];
        }
        gp[i] = g;
    }
    for (int o = GT / 2; o > 0; o >>= 1) {
        if (tid < o) red[tid] += red[tid + o];
        __syncthreads();
    }
    if (tid == 0) lpart[blockIdx.x] = red[0];
}

__global__ void k_mlp_reduce(const float *gpart, int nblk, float *grad, const float *lpart, float *loss)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NP; i += gridDim.x * blockDim.x) {
        float g = 0.f;
        for (int b = 0; b < nblk; b++) g += gpart[(int64_t)b * NP + i];
        grad[i] = g;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && loss) {
        float l = 0.f;
        for (int b = 0; b < nblk; b++) l += lpart[b];
        *loss = l;
    }
}

__global__ void k_adam(float *p, const float *grad, float *m, float *v, float lr, float b1, float b2, float eps, int t)
{
    const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NP; i += gridDim.x * blockDim.x) {
        const float g = grad[i];
        m[i] = b1 * m[i] + (1.f - b1) * g;
        v[i] = b2 * v[i] + (1.f - b2) * g * g;
        p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
    }
}

constexpr size_t grad_smem()
{
    return sizeof(float) * (MLP_H * MLP_H + TB * MLP_IN + 4 * TB * MLP_H + TB + MLP_H * MLP_IN + MLP_H + GT);
}

}  // namespace

int hc_mlp_nparams() { return NP; }

int hc_mlp_pack(hc_ctx *c)
{
    k_mlp_pack<<<32, 256, 0, c->stream>>>(c->mlp_p, c->mlp_packed);
    c->launches++;
    return HC_OK;
}

int hc_mlp_infer_impl(hc_ctx *c, const float *x_dev, int64_t n, float *logits_dev)
{
    const int64_t blocks = (n + 127) / 128;
    k_mlp_infer<<<(unsigned)blocks, 128, 0, c->stream>>>(c->mlp_packed, x_dev, n, logits_dev);
    c->launches++;
    return HC_OK;
}

// mean-loss gradient over rows [0, n) (norm = 1/sum of weights), into grad_dev
int hc_mlp_grad_impl(hc_ctx *c, const float *x, const float *y, const float *w, int64_t n, float inv_norm,
                     float *grad_dev, float *loss_dev)
{
    // per call: the attribute belongs to the current device, and a process may
    // drive contexts on several
    HC_CUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)grad_smem()));
    const int nblk = (int)((n + TB - 1) / TB);
    if (nblk > c->mlp_gcap) return HC_ERR_ARG;
    k_mlp_grad<<<nblk, GT, grad_smem(), c->stream>>>(c->mlp_p, x, y, w, n, inv_norm, c->mlp_gpart, c->mlp_lpart);
    k_mlp_reduce<<<(NP + 255) / 256, 256, 0, c->stream>>>(c->mlp_gpart, nblk, grad_dev, c->mlp_lpart, loss_dev);
    c->launches += 2;
    return HC_OK;
}

int hc_mlp_adam_impl(hc_ctx *c, const float *grad_dev, float lr, int t)
{
    k_adam<<<(NP + 255) / 256, 256, 0, c->stream>>>(c->mlp_p, grad_dev, c->mlp_m, c->mlp_v, lr, 0.9f, 0.999f, 1e-8f, t);
    c->launches++;
    return HC_OK;
}

namespace {
__global__ void k_relabel(const float *rel, int n, float thr, float *y)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = rel[i] <= thr ? 1.f : 0.f;
}
}  // namespace

int hc_relabel_impl(hc_ctx *c, float thr)
{
    if (c->nsample <= 0) return HC_OK;
    k_relabel<<<hc_grid(c->nsample, 256), 256, 0, c->stream>>>(c->sample_rel, c->nsample, thr, c->sample_y);
    c->launches++;
    return HC_OK;
}
