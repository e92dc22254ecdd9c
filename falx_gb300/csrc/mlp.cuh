// Entry-region predictor for the speculative index: a small MLP that reads
// the leading bytes of a tile and guesses the region automaton's state at
// the tile's first byte (csv_hash: NORMAL / QUOTE / COMMENT).
//
//   input   256 leading bytes, each one-hot over 8 byte classes (2048 BF16)
//   layer 1 2048 -> 256, ReLU        (one-hot input: a gather-sum of rows)
//   layer 2  256 -> 256, ReLU
//   layer 3  256 -> 3, softmax (FP32)
//
// Every product takes BF16 operands (weights rounded from the FP32 master
// copy, activations rounded after the ReLU) and accumulates in FP32. The
// network has no counterpart in the reference: it only replaces the
// reference's fixed guess for a chunk's entry state (csv_geo.rs:95-149
// assumes "outside quotes" and re-indexes odd-parity chunks), and the exact
// scan verifies every prediction, so the index never depends on it.
//
// Training is plain minibatch Adam on softmax cross-entropy, with the
// forward and backward passes below; labels come from the exact scan.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace falx {
namespace mlp {

constexpr int kPos = 256;               // leading bytes read
constexpr int kCls = 8;                 // byte classes
constexpr int kIn = kPos * kCls;        // 2048
constexpr int kHid = 256;
constexpr int kOut = 3;
// Offsets of the parameters in the flat FP32 vector (master, gradient,
// Adam moments all share it).
constexpr uint64_t kOffW1 = 0;                          // [kIn][kHid], row = pos * 8 + class
constexpr uint64_t kOffB1 = kOffW1 + (uint64_t)kIn * kHid;
constexpr uint64_t kOffW2 = kOffB1 + kHid;              // [kHid in][kHid out]
constexpr uint64_t kOffB2 = kOffW2 + (uint64_t)kHid * kHid;
constexpr uint64_t kOffW3 = kOffB2 + kHid;              // [kHid in][kOut]
constexpr uint64_t kOffB3 = kOffW3 + (uint64_t)kHid * kOut;
constexpr uint64_t kParams = kOffB3 + kOut;

// Byte classes: '"' '#' '\n' ',' '\r' digit letter other.
__host__ __device__ __forceinline__ uint8_t byte_class(uint8_t c) {
    if (c == '"') return 0;
    if (c == '#') return 1;
    if (c == '\n') return 2;
    if (c == ',') return 3;
    if (c == '\r') return 4;
    if (c >= '0' && c <= '9') return 5;
    if ((c | 0x20) >= 'a' && (c | 0x20) <= 'z') return 6;
    return 7;
}

struct Model {
    float *w = nullptr;            // FP32 master parameters [kParams]
    float *m = nullptr, *v = nullptr;  // Adam moments
    uint32_t step = 0;
    __nv_bfloat16 *w1 = nullptr;   // [kIn][kHid]
    __nv_bfloat16 *w1t = nullptr;  // [kHid][kIn]   (out, in)
    __nv_bfloat16 *w2 = nullptr;   // [kHid][kHid]  (in, out)
    __nv_bfloat16 *w2t = nullptr;  // [kHid][kHid]  (out, in)
    __nv_bfloat16 *w3 = nullptr;   // [kHid][kOut]
};

// Scratch activations for n samples.
struct Acts {
    float *a1, *a2;                // pre-activations [n][kHid]
    __nv_bfloat16 *h1, *h2;        // rounded ReLU outputs [n][kHid]
    float *z;                      // logits [n][kOut]
    float *dz;                     // [n][kOut]
    float *d2, *d1;                // gradients at the pre-activations [n][kHid]
    float *loss;                   // [1]
};

// Classes of kPos bytes from each start offset (bytes outside [0, len)
// are class 7, like the zero padding they stand for).
__global__ void classes_kernel(const uint8_t *data, uint64_t len, const int64_t *starts, int64_t stride,
                               int64_t first, uint32_t n, uint8_t *cls) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)n * kPos) return;
    const uint32_t s = (uint32_t)(i / kPos), k = (uint32_t)(i % kPos);
    const int64_t at = (starts ? starts[s] : first + (int64_t)s * stride) + k;
    cls[i] = (at >= 0 && (uint64_t)at < len) ? byte_class(data[at]) : 7;
}

// Layer 1: a1[s][j] = b1[j] + sum_p W1[p*8 + cls[s][p]][j]; h1 = bf16(relu(a1)).
// One thread per hidden unit, eight samples per block.
constexpr int kL1Samples = 8;
__global__ void __launch_bounds__(kHid) l1_forward(const uint8_t *cls, uint32_t n, const __nv_bfloat16 *w1,
                                                   const float *b1, float *a1, __nv_bfloat16 *h1) {
    __shared__ uint8_t sc[kL1Samples][kPos];
    const int j = threadIdx.x;
    const uint32_t s0 = blockIdx.x * kL1Samples;
    for (int i = j; i < kL1Samples * kPos; i += kHid) {
        const uint32_t s = s0 + i / kPos;
        sc[i / kPos][i % kPos] = s < n ? cls[(uint64_t)s * kPos + i % kPos] : 7;
    }
    __syncthreads();
    float acc[kL1Samples];
#pragma unroll
    for (int t = 0; t < kL1Samples; t++) acc[t] = 0.f;
    for (int p = 0; p < kPos; p++) {
        const __nv_bfloat16 *row = w1 + (uint64_t)p * kCls * kHid + j;
#pragma unroll
        for (int t = 0; t < kL1Samples; t++) acc[t] += __bfloat162float(row[(uint32_t)sc[t][p] * kHid]);
    }
    const float b = b1[j];
#pragma unroll
    for (int t = 0; t < kL1Samples; t++) {
        const uint32_t s = s0 + t;
        if (s >= n) break;
        const float a = acc[t] + b;
        if (a1) a1[(uint64_t)s * kHid + j] = a;
        h1[(uint64_t)s * kHid + j] = __float2bfloat16_rn(a > 0.f ? a : 0.f);
    }
}

// Layer 2: a2[s][j] = b2[j] + sum_i h1[s][i] * W2[i][j]; h2 = bf16(relu(a2)).
constexpr int kL2Samples = 16;
__global__ void __launch_bounds__(kHid) l2_forward(const __nv_bfloat16 *h1, uint32_t n, const __nv_bfloat16 *w2,
                                                   const float *b2, float *a2, __nv_bfloat16 *h2) {
    __shared__ float sh[kL2Samples][kHid];
    const int j = threadIdx.x;
    const uint32_t s0 = blockIdx.x * kL2Samples;
    for (int t = 0; t < kL2Samples; t++) {
        const uint32_t s = s0 + t;
        sh[t][j] = s < n ? __bfloat162float(h1[(uint64_t)s * kHid + j]) : 0.f;
    }
    __syncthreads();
    float acc[kL2Samples];
#pragma unroll
    for (int t = 0; t < kL2Samples; t++) acc[t] = 0.f;
    for (int i = 0; i < kHid; i++) {
        const float w = __bfloat162float(w2[i * kHid + j]);
#pragma unroll
        for (int t = 0; t < kL2Samples; t++) acc[t] = fmaf(sh[t][i], w, acc[t]);
    }
    const float b = b2[j];
#pragma unroll
    for (int t = 0; t < kL2Samples; t++) {
        const uint32_t s = s0 + t;
        if (s >= n) break;
        const float a = acc[t] + b;
        if (a2) a2[(uint64_t)s * kHid + j] = a;
        h2[(uint64_t)s * kHid + j] = __float2bfloat16_rn(a > 0.f ? a : 0.f);
    }
}

// Layer 3 (one warp per sample): logits, and optionally the arg-max as a
// predicted state (ties to the lower state).
// kNoGuess: a predicted state whose softmax probability is below
// `min_prob` is replaced by kNoGuess (the tile then counts every entry).
constexpr uint8_t kNoGuess = 0xFF;
__global__ void l3_forward(const __nv_bfloat16 *h2, uint32_t n, const __nv_bfloat16 *w3, const float *b3, float *z,
                          uint8_t *pred, float min_prob = 0.f) {
    const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= n) return;
    float acc[kOut] = {0.f, 0.f, 0.f};
    for (int i = lane; i < kHid; i += 32) {
        const float h = __bfloat162float(h2[(uint64_t)s * kHid + i]);
#pragma unroll
        for (int k = 0; k < kOut; k++) acc[k] = fmaf(h, __bfloat162float(w3[i * kOut + k]), acc[k]);
    }
#pragma unroll
    for (int k = 0; k < kOut; k++)
        for (int d = 16; d > 0; d >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], d);
    if (lane == 0) {
        float best = -3.0e38f, zz[kOut];
        int arg = 0;
        for (int k = 0; k < kOut; k++) {
            const float v = acc[k] + b3[k];
            zz[k] = v;
            if (z) z[(uint64_t)s * kOut + k] = v;
            if (v > best) { best = v; arg = k; }
        }
        if (pred) {
            float sum = 0.f;
            for (int k = 0; k < kOut; k++) sum += expf(zz[k] - best);
            pred[s] = (1.f / sum) < min_prob ? kNoGuess : (uint8_t)arg;
        }
    }
}

// Softmax cross-entropy: dz = (softmax(z) - onehot(label)) / n; loss summed.
__global__ void xent_kernel(const float *z, const uint8_t *label, uint32_t n, float *dz, float *loss) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (s < n) {
        float zz[kOut], mx = -3.0e38f;
        for (int k = 0; k < kOut; k++) { zz[k] = z[(uint64_t)s * kOut + k]; mx = fmaxf(mx, zz[k]); }
        float sum = 0.f;
        for (int k = 0; k < kOut; k++) { zz[k] = expf(zz[k] - mx); sum += zz[k]; }
        const uint32_t y = label[s] < kOut ? label[s] : 0;
        for (int k = 0; k < kOut; k++) dz[(uint64_t)s * kOut + k] = (zz[k] / sum - (k == (int)y ? 1.f : 0.f)) / (float)n;
        l = -logf(zz[y] / sum) / (float)n;
    }
    for (int d = 16; d > 0; d >>= 1) l += __shfl_xor_sync(0xffffffffu, l, d);
    if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

// dW3[i][k] = sum_s h2[s][i] dz[s][k]; db3[k] = sum_s dz[s][k];
// d2[s][i] = (sum_k dz[s][k] W3[i][k]) * [a2[s][i] > 0].
__global__ void __launch_bounds__(kHid) l3_backward(const __nv_bfloat16 *h2, const float *a2, const float *dz,
                                                    uint32_t n, const __nv_bfloat16 *w3, float *g, float *d2) {
    const int i = threadIdx.x;
    if (blockIdx.x == 0) {
        float acc[kOut] = {0.f, 0.f, 0.f}, bacc[kOut] = {0.f, 0.f, 0.f};
        for (uint32_t s = 0; s < n; s++) {
            const float h = __bfloat162float(h2[(uint64_t)s * kHid + i]);
#pragma unroll
            for (int k = 0; k < kOut; k++) {
                const float d = dz[(uint64_t)s * kOut + k];
                acc[k] = fmaf(h, d, acc[k]);
                bacc[k] += d;
            }
        }
#pragma unroll
        for (int k = 0; k < kOut; k++) g[kOffW3 + i * kOut + k] = acc[k];
        if (i < kOut) g[kOffB3 + i] = bacc[i];
    }
    float w[kOut];
#pragma unroll
    for (int k = 0; k < kOut; k++) w[k] = __bfloat162float(w3[i * kOut + k]);
    for (uint32_t s = blockIdx.x; s < n; s += gridDim.x) {
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < kOut; k++) acc = fmaf(dz[(uint64_t)s * kOut + k], w[k], acc);
        d2[(uint64_t)s * kHid + i] = a2[(uint64_t)s * kHid + i] > 0.f ? acc : 0.f;
    }
}

// dW2[i][j] = sum_s h1[s][i] d2[s][j] (block i, thread j); db2[j] = sum_s d2[s][j].
__global__ void __launch_bounds__(kHid) l2_wgrad(const __nv_bfloat16 *h1, const float *d2, uint32_t n, float *g) {
    const int i = blockIdx.x, j = threadIdx.x;
    float acc = 0.f, bacc = 0.f;
    for (uint32_t s = 0; s < n; s++) {
        const float d = d2[(uint64_t)s * kHid + j];
        acc = fmaf(__bfloat162float(h1[(uint64_t)s * kHid + i]), d, acc);
        bacc += d;
    }
    g[kOffW2 + (uint64_t)i * kHid + j] = acc;
    if (i == 0) g[kOffB2 + j] = bacc;
}

// d1[s][i] = (sum_j d2[s][j] W2[i][j]) * [a1[s][i] > 0], through the
// transposed copy so the reads of W2 coalesce.
__global__ void __launch_bounds__(kHid) l2_dgrad(const float *d2, const float *a1, uint32_t n,
                                                 const __nv_bfloat16 *w2t, float *d1) {
    __shared__ float sd[kL2Samples][kHid];
    const int i = threadIdx.x;
    const uint32_t s0 = blockIdx.x * kL2Samples;
    for (int t = 0; t < kL2Samples; t++) {
        const uint32_t s = s0 + t;
        sd[t][i] = s < n ? d2[(uint64_t)s * kHid + i] : 0.f;
    }
    __syncthreads();
    float acc[kL2Samples];
#pragma unroll
    for (int t = 0; t < kL2Samples; t++) acc[t] = 0.f;
    for (int j = 0; j < kHid; j++) {
        const float w = __bfloat162float(w2t[j * kHid + i]);
#pragma unroll
        for (int t = 0; t < kL2Samples; t++) acc[t] = fmaf(sd[t][j], w, acc[t]);
    }
#pragma unroll
    for (int t = 0; t < kL2Samples; t++) {
        const uint32_t s = s0 + t;
        if (s >= n) break;
        d1[(uint64_t)s * kHid + i] = a1[(uint64_t)s * kHid + i] > 0.f ? acc[t] : 0.f;
    }
}

// dW1[p*8 + c][j] = sum over samples whose byte p has class c of d1[s][j]
// (block p, thread j, one shared accumulator row per class);
// db1[j] = sum_s d1[s][j] (block 0).
__global__ void __launch_bounds__(kHid) l1_wgrad(const uint8_t *cls, const float *d1, uint32_t n, float *g) {
    __shared__ float acc[kCls][kHid];
    const int p = blockIdx.x, j = threadIdx.x;
#pragma unroll
    for (int c = 0; c < kCls; c++) acc[c][j] = 0.f;
    float bacc = 0.f;
    for (uint32_t s = 0; s < n; s++) {
        const float d = d1[(uint64_t)s * kHid + j];
        acc[cls[(uint64_t)s * kPos + p]][j] += d;
        bacc += d;
    }
#pragma unroll
    for (int c = 0; c < kCls; c++) g[kOffW1 + ((uint64_t)p * kCls + c) * kHid + j] = acc[c][j];
    if (p == 0) g[kOffB1 + j] = bacc;
}

// Adam on the master weights, then the BF16 copies.
__global__ void adam_kernel(float *w, float *m, float *v, const float *g, uint64_t count, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void refresh_bf16(const float *w, __nv_bfloat16 *w1, __nv_bfloat16 *w1t, __nv_bfloat16 *w2,
                             __nv_bfloat16 *w2t, __nv_bfloat16 *w3) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (uint64_t)kIn * kHid) {
        const __nv_bfloat16 b = __float2bfloat16_rn(w[kOffW1 + i]);
        w1[i] = b;
        w1t[(i % kHid) * kIn + i / kHid] = b;
    }
    if (i < (uint64_t)kHid * kHid) {
        const __nv_bfloat16 b = __float2bfloat16_rn(w[kOffW2 + i]);
        w2[i] = b;
        const uint64_t r = i / kHid, c = i % kHid;
        w2t[c * kHid + r] = b;
    }
    if (i < (uint64_t)kHid * kOut) w3[i] = __float2bfloat16_rn(w[kOffW3 + i]);
}

// ---------------------------------------------------------------------------
// Inference layers on the tensor cores: mma.sync m16n8k16, BF16 operands,
// FP32 accumulation. One CTA computes 128 samples x 256 outputs; warp w
// owns rows 16 (w & 7) .. +16 and columns 128 (w >> 3) .. +128 (one A
// fragment feeds 16 MMAs). K is staged
// 64 at a time (weights as [out][in] rows, padded to 72 elements so the
// ldmatrix row addresses of a phase fall in distinct banks), double
// buffered with cp.async. Layer 1 builds its one-hot A fragments in
// registers from the byte classes; layer 2 reads A with ldmatrix.
// ---------------------------------------------------------------------------
constexpr int kMmaRows = 128;
constexpr int kMmaThreads = 512;
constexpr int kKC = 64;
constexpr int kRowPad = kKC + 8;

struct MmaSmem {
    __nv_bfloat16 b[2][kHid][kRowPad];
    union {
        uint8_t cls[kMmaRows][kPos + 16];
        __nv_bfloat16 a[2][kMmaRows][kRowPad];
    };
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                 "{%8, %9}, {%0, %1, %2, %3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// The two BF16 one-hot entries (classes 2t, 2t+1) of a byte of class c.
__device__ __forceinline__ uint32_t onehot_pair(uint32_t c, uint32_t t) {
    return (c >> 1) == t ? ((c & 1) ? 0x3F800000u : 0x00003F80u) : 0u;
}

// ONEHOT: input = classes of 256 bytes per sample, from `data` at
// first + s * stride (bytes outside [0, len) are class 7) or from `cls`.
// Otherwise input = a[M][256] BF16. Output h = bf16(relu(x W + bias)).
template <bool ONEHOT>
__global__ void __launch_bounds__(kMmaThreads, 1)
    mma_layer(const uint8_t *data, uint64_t len, int64_t first, int64_t stride, const uint8_t *cls,
              const __nv_bfloat16 *a, uint32_t M, const __nv_bfloat16 *wt, const float *bias, __nv_bfloat16 *h) {
    constexpr int K = ONEHOT ? kIn : kHid;
    extern __shared__ __align__(128) uint8_t mma_smem_raw[];
    MmaSmem &S = *reinterpret_cast<MmaSmem *>(mma_smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp & 7, wn = warp >> 3;
    const int g = lane >> 2, t = lane & 3, q = lane >> 3, r8 = lane & 7;
    const uint32_t row0 = blockIdx.x * kMmaRows;

    auto load_b = [&](int kc, int buf) {
        for (int i = tid; i < kHid * (kKC / 8); i += kMmaThreads) {
            const int n = i / (kKC / 8), c = i % (kKC / 8);
            cp_async16(&S.b[buf][n][c * 8], wt + (uint64_t)n * K + kc * kKC + c * 8);
        }
    };
    auto load_a = [&](int kc, int buf) {
        for (int i = tid; i < kMmaRows * (kKC / 8); i += kMmaThreads) {
            const int m = i / (kKC / 8), c = i % (kKC / 8);
            if (row0 + m < M) cp_async16(&S.a[buf][m][c * 8], a + (uint64_t)(row0 + m) * K + kc * kKC + c * 8);
            else *reinterpret_cast<uint4 *>(&S.a[buf][m][c * 8]) = make_uint4(0, 0, 0, 0);
        }
    };
    if (ONEHOT) {
        // 16 bytes per load. With data, sample starts are 16-byte aligned
        // (tile starts); a 16-byte block that holds a byte of the input is
        // readable whole, and bytes outside the input are class 7.
        for (int i = tid; i < kMmaRows * (kPos / 16); i += kMmaThreads) {
            const int m = i / (kPos / 16), k = (i % (kPos / 16)) * 16;
            uint32_t wv[4] = {0x07070707u, 0x07070707u, 0x07070707u, 0x07070707u};
            if (row0 + m < M) {
                if (data) {
                    const int64_t at = first + (int64_t)(row0 + m) * stride + k;
                    if (at + 16 > 0 && at < (int64_t)len) {
                        const uint4 raw = *reinterpret_cast<const uint4 *>(data + at);
                        const uint32_t rw[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
                        for (int b = 0; b < 16; b++) {
                            const int64_t pos = at + b;
                            const uint32_t v = (pos >= 0 && pos < (int64_t)len)
                                                   ? byte_class((uint8_t)(rw[b >> 2] >> (8 * (b & 3)))) : 7u;
                            wv[b >> 2] = (wv[b >> 2] & ~(0xFFu << (8 * (b & 3)))) | (v << (8 * (b & 3)));
                        }
                    }
                } else {
                    const uint4 raw = *reinterpret_cast<const uint4 *>(cls + (uint64_t)(row0 + m) * kPos + k);
                    wv[0] = raw.x; wv[1] = raw.y; wv[2] = raw.z; wv[3] = raw.w;
                }
            }
            *reinterpret_cast<uint4 *>(&S.cls[m][k]) = make_uint4(wv[0], wv[1], wv[2], wv[3]);
        }
    }
    load_b(0, 0);
    if (!ONEHOT) load_a(0, 0);
    cp_async_commit();

    float acc[16][4];
#pragma unroll
    for (int nt = 0; nt < 16; nt++)
#pragma unroll
        for (int e = 0; e < 4; e++) acc[nt][e] = 0.f;

    constexpr int kChunks = K / kKC;
    for (int kc = 0; kc < kChunks; kc++) {
        const int buf = kc & 1;
        if (kc + 1 < kChunks) {
            load_b(kc + 1, buf ^ 1);
            if (!ONEHOT) load_a(kc + 1, buf ^ 1);
        }
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < kKC / 16; ks++) {
            uint32_t af[4];
            const int rb = wm * 16;
            if (ONEHOT) {
                // byte positions p0, p0 + 1 of rows g and g + 8
                const int p0 = (kc * kKC + ks * 16) / kCls;
                const uint32_t lo = *reinterpret_cast<const uint16_t *>(&S.cls[rb + g][p0]);
                const uint32_t hi = *reinterpret_cast<const uint16_t *>(&S.cls[rb + g + 8][p0]);
                af[0] = onehot_pair(lo & 0xFF, t);
                af[1] = onehot_pair(hi & 0xFF, t);
                af[2] = onehot_pair(lo >> 8, t);
                af[3] = onehot_pair(hi >> 8, t);
            } else {
                ldsm_x4(af, &S.a[buf][rb + (q & 1) * 8 + r8][ks * 16 + (q >> 1) * 8]);
            }
#pragma unroll
            for (int np = 0; np < 8; np++) {
                uint32_t bf[4];
                ldsm_x4(bf, &S.b[buf][wn * 128 + np * 16 + (q >> 1) * 8 + r8][ks * 16 + (q & 1) * 8]);
                mma_bf16(acc[2 * np], af, bf[0], bf[1]);
                mma_bf16(acc[2 * np + 1], af, bf[2], bf[3]);
            }
        }
        __syncthreads();
    }
    cp_async_wait<0>();
#pragma unroll
    for (int nt = 0; nt < 16; nt++) {
        const int col = wn * 128 + nt * 8 + 2 * t;
        const float b0 = bias[col], b1 = bias[col + 1];
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
            const uint32_t row = row0 + wm * 16 + g + hh * 8;
            if (row >= M) continue;
            const float v0 = fmaxf(acc[nt][2 * hh] + b0, 0.f), v1 = fmaxf(acc[nt][2 * hh + 1] + b1, 0.f);
            __nv_bfloat162 o;
            o.x = __float2bfloat16_rn(v0);
            o.y = __float2bfloat16_rn(v1);
            *reinterpret_cast<__nv_bfloat162 *>(h + (uint64_t)row * kHid + col) = o;
        }
    }
}

}  // namespace mlp
}  // namespace falx
