/*
 * valuenet.cu -- kernels of the value network that orders the search.
 *
 * The network follows the reference's ValueNetwork (python/model.py:16-84)
 * with bit features per test case: a shared per-test encoder
 * 176 -> 256 -> 256 (ReLU), mean and max pooling over the task's tests,
 * concatenated with the live mask (8 bits) and the state's depth, a trunk
 * 528 -> 256 -> 128 (ReLU) and a 16-wide head whose column 0 is the
 * "can finish optimally" logit and columns 1..9 the remaining-steps logits.
 * ~281K parameters.
 *
 * Features per (state, test), 176 columns (164 used, zero padded): input 0
 * bits (16), input 1 bits (16), target bits (16), r1..r7 bits (7 x 16),
 * flag bits (4). Every state has 32 feature rows; rows of tests >= T are
 * zero and are left out of the pooling.
 *
 * The matrix products run on the fifth-generation tensor cores
 * (valuenet_tc.cu: the fused scoring encoder and the training GEMM); this
 * file holds the features, pooling, loss, Adam and sampling kernels.
 * Parameters are FP32 masters with BF16 copies (row-major [out][in] and
 * transposed [in][out]) refreshed by the Adam kernel. Launches go to the
 * stream the caller passes.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <stdint.h>

#include <cmath>

#include "../../include/pca_gb300.h"

namespace {

/* Features of states in the engine's level layout. Row (state i, test t)
 * of X[n*32][176] is eleven 16-bit words expanded to 0.0 / 1.0 bf16 values,
 * bit 0 first: input 0, input 1, target, r1..r7, the flags (4 bits, then
 * zeros); rows of tests >= T are zero. One thread per (row, word), writing
 * its 16 values as two 16-byte pieces. */
__device__ __forceinline__ uint4 bits8_to_bf16(uint32_t b)
{
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const uint32_t t = b >> (2 * j);
        w[j] = (t & 1u) * 0x3F80u + (t & 2u) * 0x1FC00000u;
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

__global__ void k_features(const uint16_t *regs, const uint8_t *flags, const uint16_t *task, int TP,
                           int n, const uint16_t *task_io, const int32_t *task_T,
                           __nv_bfloat16 *X)
{
    const size_t items = (size_t)n * 32 * 11;
    for (size_t it = (size_t)blockIdx.x * blockDim.x + threadIdx.x; it < items;
         it += (size_t)gridDim.x * blockDim.x) {
        const size_t row = it / 11;
        const int w = (int)(it - row * 11);
        const int i = (int)(row >> 5), t = (int)(row & 31);
        const int tid = task[i];
        uint32_t word = 0;
        if (t < task_T[tid]) {
            if (w < 3) word = task_io[((size_t)tid * 3 + w) * 32 + t];
            else if (w < 10) word = regs[((size_t)i * 8 + (w - 2)) * TP + t];
            else word = flags[(size_t)i * TP + t] & 0xFu;
        }
        uint4 *dst = reinterpret_cast<uint4 *>(X + row * 176 + w * 16);
        dst[0] = bits8_to_bf16(word & 0xFFu);
        dst[1] = bits8_to_bf16(word >> 8);
    }
}

/* Mean and max over each state's valid test rows of H[n*32][256], plus
 * live bits and depth: P[n][528]; argmax row per (state, unit). */
__global__ void k_pool(const __nv_bfloat16 *H, const uint8_t *live, const uint16_t *task,
                       const int32_t *task_T, const uint8_t *depth, int n, __nv_bfloat16 *P,
                       uint8_t *argmax)
{
    const int i = blockIdx.x;
    const int u = threadIdx.x;  /* 0..255 */
    if (i >= n) return;
    const int T = task_T[task[i]];
    float s = 0.f, mx = -1e30f;
    int am = 0;
    for (int t = 0; t < T; t++) {
        const float v = __bfloat162float(H[((size_t)i * 32 + t) * 256 + u]);
        s += v;
        if (v > mx) { mx = v; am = t; }
    }
    P[(size_t)i * 528 + u] = __float2bfloat16(s / (float)T);
    P[(size_t)i * 528 + 256 + u] = __float2bfloat16(mx);
    argmax[(size_t)i * 256 + u] = (uint8_t)am;
    if (u < 16) {
        float g = 0.f;
        if (u < 8) g = (float)((live[i] >> u) & 1u);
        else if (u == 8) g = (float)depth[i];
        P[(size_t)i * 528 + 512 + u] = __float2bfloat16(g);
    }
}

/* Backward of k_pool, then of the ReLU that produced H, into dH[n*32][256]:
   rows >= T and units whose H is not positive get zero. */
__global__ void k_pool_bwd(const __nv_bfloat16 *dP, const uint8_t *argmax, const uint16_t *task,
                           const int32_t *task_T, const __nv_bfloat16 *H, int n,
                           __nv_bfloat16 *dH)
{
    const int i = blockIdx.x, u = threadIdx.x;
    if (i >= n) return;
    const int T = task_T[task[i]];
    const float dm = __bfloat162float(dP[(size_t)i * 528 + u]) / (float)T;
    const float dx = __bfloat162float(dP[(size_t)i * 528 + 256 + u]);
    const int am = argmax[(size_t)i * 256 + u];
    for (int t = 0; t < 32; t++) {
        const size_t at = ((size_t)i * 32 + t) * 256 + u;
        float g = 0.f;
        if (t < T && __bfloat162float(H[at]) > 0.f) g = dm + (t == am ? dx : 0.f);
        dH[at] = __float2bfloat16(g);
    }
}

/* Loss of the reference's recipe (python/train.py:48-60): BCE with
 * pos_weight on column 0, plus 0.5 x cross entropy of columns 1..9 against
 * the remaining steps over the positives. Writes dLogits[n][16] (bf16) of the
 * mean loss, and accumulates [bce_sum, ce_sum, n_pos] into stats. */
__global__ void k_loss(const float *logits, const float *label, const int32_t *remaining, int n,
                       float pos_weight, const float *n_pos, __nv_bfloat16 *dlogits, float *stats)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float n_pos_total = *n_pos;   /* positives in the batch (on the device) */
    const float *z = logits + (size_t)i * 16;
    const float y = label[i];
    const float zr = z[0];
    /* softplus(x) = log(1 + e^x), stable */
    auto softplus = [](float x) { return x > 0 ? x + log1pf(expf(-x)) : log1pf(expf(x)); };
    const float bce = pos_weight * y * softplus(-zr) + (1.f - y) * softplus(zr);
    const float sg = 1.f / (1.f + expf(-zr));
    float d[16] = {};
    d[0] = (-pos_weight * y * (1.f - sg) + (1.f - y) * sg) / (float)n;
    float ce = 0.f;
    if (y > 0.5f && n_pos_total > 0) {
        float mx = -1e30f;
        for (int j = 1; j <= 9; j++) mx = fmaxf(mx, z[j]);
        float se = 0.f;
        for (int j = 1; j <= 9; j++) se += expf(z[j] - mx);
        int k = remaining[i];
        k = k < 0 ? 0 : (k > 8 ? 8 : k);
        ce = -(z[1 + k] - mx - logf(se));
        for (int j = 1; j <= 9; j++) {
            const float p = expf(z[j] - mx) / se;
            d[j] = 0.5f * (p - (j - 1 == k ? 1.f : 0.f)) / n_pos_total;
        }
        atomicAdd(&stats[2], 1.f);
    }
    for (int j = 0; j < 16; j++) dlogits[(size_t)i * 16 + j] = __float2bfloat16(d[j]);
    atomicAdd(&stats[0], bce);
    atomicAdd(&stats[1], ce);
}

/* Adam on fp32 masters, then the bf16 copies [out][in] and [in][out]. The
   step count lives on the device (so a captured training step replays with
   the right bias corrections). */
__global__ void k_adam(float *W, const float *G, float *m, float *v, int out, int in, float lr,
                       float b1, float b2, float eps, const int *step, __nv_bfloat16 *Wb,
                       __nv_bfloat16 *Wt)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= out * in) return;
    const float bc1 = 1.f - powf(b1, (float)*step), bc2 = 1.f - powf(b2, (float)*step);
    const float g = G[idx];
    const float mi = b1 * m[idx] + (1.f - b1) * g;
    const float vi = b2 * v[idx] + (1.f - b2) * g * g;
    m[idx] = mi;
    v[idx] = vi;
    const float w = W[idx] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    W[idx] = w;
    if (Wb) Wb[idx] = __float2bfloat16(w);
    if (Wt) {
        const int o = idx / in, i = idx % in;
        Wt[(size_t)i * out + o] = __float2bfloat16(w);
    }
}

__global__ void k_to_bf16(const float *src, __nv_bfloat16 *dst, size_t count)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (size_t)gridDim.x * blockDim.x)
        dst[i] = __float2bfloat16(src[i]);
}

/* Column sums of a bf16 [rows][cols] matrix (leading dimension ld, both
   multiples of 8), in two deterministic stages: k_colsum_part gives each
   block's partial sums (a thread per 8 columns and row slot, eight rows in
   flight per thread, 16-byte loads, the 8 row slots of a block reduced in
   shared memory) in part[block][cols]; k_colsum_final adds the blocks'
   partials of each column into out (32 columns per block, 32 slices of the
   partials, reduced in shared memory). No atomics: a column's sum does not
   depend on the order blocks finish in. */
constexpr int kColsumRows = 8;   /* rows a thread loads before adding */

__global__ void __launch_bounds__(256) k_colsum_part(const __nv_bfloat16 *Y, long long rows,
                                                    int cols, int ld, float *part)
{
    __shared__ float sp[8][32][8];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const long long stride = (long long)gridDim.x * 8;
    for (int g0 = 0; g0 < cols / 8; g0 += 32) {
        const int g = g0 + tx;
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (g < cols / 8) {
            long long r = (long long)blockIdx.x * 8 + ty;
            for (; r + (kColsumRows - 1) * stride < rows; r += kColsumRows * stride) {
                uint4 w[kColsumRows];
#pragma unroll
                for (int u = 0; u < kColsumRows; u++)
                    w[u] = *(const uint4 *)(Y + (r + u * stride) * ld + g * 8);
#pragma unroll
                for (int u = 0; u < kColsumRows; u++) {
                    const __nv_bfloat162 *h = (const __nv_bfloat162 *)&w[u];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const float2 f = __bfloat1622float2(h[j]);
                        acc[2 * j] += f.x;
                        acc[2 * j + 1] += f.y;
                    }
                }
            }
            for (; r < rows; r += stride) {
                const uint4 w = *(const uint4 *)(Y + r * ld + g * 8);
                const __nv_bfloat162 *h = (const __nv_bfloat162 *)&w;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const float2 f = __bfloat1622float2(h[j]);
                    acc[2 * j] += f.x;
                    acc[2 * j + 1] += f.y;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 8; j++) sp[ty][tx][j] = acc[j];
        __syncthreads();
        if (ty == 0 && g < cols / 8) {
#pragma unroll
            for (int j = 0; j < 8; j++) {
                float v = 0;
                for (int y = 0; y < 8; y++) v += sp[y][tx][j];
                part[(size_t)blockIdx.x * cols + g * 8 + j] = v;
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(1024) k_colsum_final(const float *part, int blocks, int cols,
                                                      float *out)
{
    __shared__ float sp[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int c = blockIdx.x * 32 + tx;
    float v = 0;
    if (c < cols)
        for (int b = ty; b < blocks; b += 32) v += part[(size_t)b * cols + c];
    sp[ty][tx] = v;
    __syncthreads();
    if (ty == 0 && c < cols) {
        float t = 0;
        for (int y = 0; y < 32; y++) t += sp[y][tx];
        out[c] += t;
    }
}

int launch_ok()
{
    return cudaGetLastError() == cudaSuccess ? PCAGB_OK : PCAGB_ECUDA;
}

}  // namespace

/* Where a sampled ranking reads its states: kept in device memory so that
 * a captured CUDA graph of the ranking replays on any level. Sample i is
 * state (a * i + b) mod n, with a coprime to n: the map is a bijection of
 * 0..n-1, so the sample and the rest of the order partition the level. */
struct SampleSrc {
    const uint16_t *regs;
    const uint8_t *flags;
    const uint8_t *live;
    const uint16_t *task;
    unsigned long long n, a, b;
    unsigned int depth, pad;
};

__device__ __forceinline__ unsigned long long sample_pos(const SampleSrc &S, unsigned long long i)
{
    return (S.a * i + S.b) % S.n;
}

/* Copy sample i's state (registers, flags, live, task) into row i. */
__global__ void k_gather_sample(const SampleSrc *src, uint16_t *regs, uint8_t *flags, uint8_t *live,
                                uint16_t *task, uint8_t *depth, int m, int TP)
{
    const SampleSrc S = *src;
    if (S.n == 0) return;   /* no level: nothing to read (and no modulus) */
    for (int i = blockIdx.x; i < m; i += gridDim.x) {
        const unsigned long long p = sample_pos(S, (unsigned long long)i);
        for (int k = threadIdx.x; k < 8 * TP; k += blockDim.x)
            regs[(size_t)i * 8 * TP + k] = S.regs[p * 8 * TP + k];
        for (int k = threadIdx.x; k < TP; k += blockDim.x)
            flags[(size_t)i * TP + k] = S.flags[p * TP + k];
        if (threadIdx.x == 0) {
            live[i] = S.live[p];
            task[i] = S.task[p];
            depth[i] = (uint8_t)S.depth;
        }
    }
}

/* The order: the sample by rank (ranked[i] = sample index), then every
   other state in sample-map order. */
__global__ void k_compose_order(const SampleSrc *src, const long long *ranked, int m,
                                uint32_t *order)
{
    const SampleSrc S = *src;
    if (S.n == 0) return;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < S.n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        order[i] = (uint32_t)sample_pos(S, i < (unsigned long long)m ? (unsigned long long)ranked[i] : i);
}

extern "C" {

/* out[c] += sum over rows of Y[r][c] (the bias gradient of a layer from
   its output gradient). cols and ld multiples of 8, Y 16-byte aligned;
   part: scratch for pcagb_vnet_colsum_blocks(rows, sms) x cols floats. */
int pcagb_vnet_colsum_blocks(long long rows, int sms)
{
    return (int)std::max<long long>(1, std::min<long long>((rows + 7) / 8,
                                                           (long long)std::max(sms, 1) * 2));
}

int pcagb_vnet_colsum(const void *Y, long long rows, int cols, int ld, float *out, float *part,
                      int sms, void *stream)
{
    if (rows <= 0 || cols <= 0) return PCAGB_OK;
    if (!Y || !out || !part || (cols & 7) || (ld & 7) || ld < cols || ((uintptr_t)Y & 15))
        return PCAGB_EINVAL;
    const int blocks = pcagb_vnet_colsum_blocks(rows, sms);
    k_colsum_part<<<blocks, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)Y, rows, cols,
                                                            ld, part);
    int rc = launch_ok();
    if (rc) return rc;
    k_colsum_final<<<(cols + 31) / 32, 1024, 0, (cudaStream_t)stream>>>(part, blocks, cols, out);
    return launch_ok();
}

int pcagb_vnet_gather_sample(const void *src, uint16_t *regs, uint8_t *flags, uint8_t *live,
                             uint16_t *task, uint8_t *depth, int m, int TP, void *stream)
{
    if (m <= 0) return PCAGB_OK;
    k_gather_sample<<<std::min(m, 4096), 128, 0, (cudaStream_t)stream>>>(
        (const SampleSrc *)src, regs, flags, live, task, depth, m, TP);
    return launch_ok();
}

int pcagb_vnet_compose_order(const void *src, const long long *ranked, int m, uint32_t *order,
                             unsigned long long n, void *stream)
{
    if (n == 0) return PCAGB_OK;
    const unsigned blocks = (unsigned)std::min<unsigned long long>((n + 255) / 256, 4096);
    k_compose_order<<<blocks, 256, 0, (cudaStream_t)stream>>>((const SampleSrc *)src, ranked, m,
                                                             order);
    return launch_ok();
}

int pcagb_vnet_features(const uint16_t *regs, const uint8_t *flags, const uint16_t *task, int TP,
                        int n, const uint16_t *task_io, const int32_t *task_T, void *X,
                        void *stream)
{
    if (n <= 0) return PCAGB_OK;
    if ((uintptr_t)X & 15) return PCAGB_EINVAL;
    const size_t items = (size_t)n * 32 * 11;
    const unsigned blocks = (unsigned)std::min<size_t>((items + 255) / 256, 65536);
    k_features<<<blocks, 256, 0, (cudaStream_t)stream>>>(regs, flags, task, TP, n, task_io, task_T,
                                                         (__nv_bfloat16 *)X);
    return launch_ok();
}

int pcagb_vnet_pool(const void *H, const uint8_t *live, const uint16_t *task,
                    const int32_t *task_T, const uint8_t *depth, int n, void *P, uint8_t *argmax,
                    void *stream)
{
    if (n <= 0) return PCAGB_OK;
    k_pool<<<n, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)H, live, task, task_T, depth,
                                                n, (__nv_bfloat16 *)P, argmax);
    return launch_ok();
}

int pcagb_vnet_pool_bwd(const void *dP, const uint8_t *argmax, const uint16_t *task,
                        const int32_t *task_T, const void *H, int n, void *dH, void *stream)
{
    if (n <= 0) return PCAGB_OK;
    k_pool_bwd<<<n, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)dP, argmax, task, task_T,
                                                    (const __nv_bfloat16 *)H, n,
                                                    (__nv_bfloat16 *)dH);
    return launch_ok();
}

int pcagb_vnet_loss(const float *logits, const float *label, const int32_t *remaining, int n,
                    float pos_weight, const float *n_pos, void *dlogits, float *stats,
                    void *stream)
{
    if (n <= 0) return PCAGB_OK;
    k_loss<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        logits, label, remaining, n, pos_weight, n_pos, (__nv_bfloat16 *)dlogits, stats);
    return launch_ok();
}

int pcagb_vnet_adam(float *W, const float *G, float *m, float *v, int out, int in, float lr,
                    float b1, float b2, float eps, const int *step, void *Wb, void *Wt,
                    void *stream)
{
    const int count = out * in;
    k_adam<<<(count + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        W, G, m, v, out, in, lr, b1, b2, eps, step, (__nv_bfloat16 *)Wb, (__nv_bfloat16 *)Wt);
    return launch_ok();
}

int pcagb_vnet_to_bf16(const float *src, void *dst, size_t count, void *stream)
{
    k_to_bf16<<<1024, 256, 0, (cudaStream_t)stream>>>(src, (__nv_bfloat16 *)dst, count);
    return launch_ok();
}

}  // extern "C"
