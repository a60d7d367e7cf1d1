// Learned time-of-impact proposal: a 20-128-128-2 MLP (SiLU), BF16 weights
// and activations, FP32 accumulation, trained on the GPU by the kernels here.
//
// No counterpart in the reference.  Inputs are 20 FP32 features of a CCD
// pair query (relative pose 3x3 + translation, relative linear and angular
// velocity, the two surrogate-root radii), standardised; outputs are the
// normalised time of impact and a hit logit.  The exact CCD always runs, so
// the network can only propose; it never changes a result.
//
// Layers run on the tensor cores with mma.sync m16n8k16 (BF16 in, FP32
// accumulate): a block takes 64 samples, each warp 16 rows, and every layer is
// one pass of 16x8 output tiles over K in steps of 16.  Weights are stored
// output-major ([N][K], K contiguous), which is the column layout mma wants
// for its B operand; activations row-major ([row][K]).  Backward: the output
// gradient is elementwise, dH1 = dZ2 * W2 runs on the tensor cores against the
// transposed copy W2T, and the weight gradients are FP32 sums over the
// block's rows, added to the global gradient with atomics.  Adam keeps FP32
// master weights and refreshes the BF16 copies.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "d2g_internal.hpp"

namespace d2g {
namespace {

constexpr int kIn = 20, kInPad = 32, kHid = 128, kOut = 2, kOutPad = 8;
constexpr int kRows = 64;  // samples per block
constexpr int kThreads = 128;
// parameter offsets in the FP32 master vector
constexpr int oW1 = 0, oB1 = oW1 + kHid * kIn, oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid, oW3 = oB2 + kHid,
              oB3 = oW3 + kOut * kHid, kParams = oB3 + kOut;

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// D = A(16x16, row) * B(16x8, col) + D, BF16 inputs, FP32 accumulators.
__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment of rows [r0, r0+16) and columns [k0, k0+16) of a row-major
// BF16 matrix with leading dimension ld.
__device__ __forceinline__ void load_a(uint32_t* a, const __nv_bfloat16* m, int ld, int r0, int k0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    a[0] = ld32(m + (size_t)(r0 + g) * ld + k0 + 2 * t);
    a[1] = ld32(m + (size_t)(r0 + g + 8) * ld + k0 + 2 * t);
    a[2] = ld32(m + (size_t)(r0 + g) * ld + k0 + 8 + 2 * t);
    a[3] = ld32(m + (size_t)(r0 + g + 8) * ld + k0 + 8 + 2 * t);
}
// B fragment of output columns [n0, n0+8) and K [k0, k0+16) of an
// output-major ([N][K]) BF16 matrix with leading dimension ld.
__device__ __forceinline__ void load_b(uint32_t* b, const __nv_bfloat16* w, int ld, int n0, int k0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    b[0] = ld32(w + (size_t)(n0 + g) * ld + k0 + 2 * t);
    b[1] = ld32(w + (size_t)(n0 + g) * ld + k0 + 8 + 2 * t);
}

// Forward pass of n samples: X [n][32] BF16 (features 20..31 zero).
// W1b [128][32], W2b [128][128], W3b [8][128] (rows 2..7 zero) BF16; biases
// FP32.  out [n][2] FP32.  With training buffers: Z1, Z2 [n][128] FP32
// pre-activations, H1, H2 [n][128] BF16 activations.
__global__ void __launch_bounds__(kThreads) k_mlp_forward(int n, const __nv_bfloat16* __restrict__ X,
                                                          const __nv_bfloat16* __restrict__ W1b,
                                                          const __nv_bfloat16* __restrict__ W2b,
                                                          const __nv_bfloat16* __restrict__ W3b,
                                                          const float* __restrict__ P, float* __restrict__ out,
                                                          float* __restrict__ Z1, float* __restrict__ Z2,
                                                          __nv_bfloat16* __restrict__ H1,
                                                          __nv_bfloat16* __restrict__ H2) {
    __shared__ __align__(16) __nv_bfloat16 s_h[kRows][kHid + 8];  // one layer's activations, padded rows
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int row0 = blockIdx.x * kRows + warp * 16;  // this warp's first sample
    const int lr0 = warp * 16;                        // in the block's tile
    // Rows past n read the zero padding of X (allocated to a multiple of 64
    // rows); their results are dropped.
    float acc[16][4];
    // ---- layer 1: K = 32
#pragma unroll
    for (int j = 0; j < 16; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[j][q] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < kInPad; k0 += 16) {
        uint32_t a[4];
        load_a(a, X, kInPad, row0, k0, lane);
#pragma unroll
        for (int j = 0; j < 16; j++) {
            uint32_t b[2];
            load_b(b, W1b, kInPad, 8 * j, k0, lane);
            mma_bf16(acc[j], a, b);
        }
    }
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const int c = 8 * j + 2 * t;
        const float b0 = P[oB1 + c], b1 = P[oB1 + c + 1];
        const float z00 = acc[j][0] + b0, z01 = acc[j][1] + b1, z10 = acc[j][2] + b0, z11 = acc[j][3] + b1;
        if (Z1) {
            const int r = row0 + g;
            if (r < n) *reinterpret_cast<float2*>(Z1 + (size_t)r * kHid + c) = make_float2(z00, z01);
            if (r + 8 < n) *reinterpret_cast<float2*>(Z1 + (size_t)(r + 8) * kHid + c) = make_float2(z10, z11);
        }
        *reinterpret_cast<uint32_t*>(&s_h[lr0 + g][c]) = pack_bf16(silu(z00), silu(z01));
        *reinterpret_cast<uint32_t*>(&s_h[lr0 + g + 8][c]) = pack_bf16(silu(z10), silu(z11));
    }
    __syncwarp();
    if (H1)
        for (int i = lane; i < 16 * (kHid / 2); i += 32) {
            const int r = i / (kHid / 2), c = 2 * (i % (kHid / 2));
            if (row0 + r < n)
                *reinterpret_cast<uint32_t*>(H1 + (size_t)(row0 + r) * kHid + c) =
                    *reinterpret_cast<const uint32_t*>(&s_h[lr0 + r][c]);
        }
    // ---- layer 2: K = 128
#pragma unroll
    for (int j = 0; j < 16; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[j][q] = 0.f;
#pragma unroll 2
    for (int k0 = 0; k0 < kHid; k0 += 16) {
        uint32_t a[4];
        load_a(a, &s_h[0][0], kHid + 8, lr0, k0, lane);
#pragma unroll
        for (int j = 0; j < 16; j++) {
            uint32_t b[2];
            load_b(b, W2b, kHid, 8 * j, k0, lane);
            mma_bf16(acc[j], a, b);
        }
    }
    __syncwarp();  // every lane has read its layer-1 rows before they are overwritten
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const int c = 8 * j + 2 * t;
        const float b0 = P[oB2 + c], b1 = P[oB2 + c + 1];
        const float z00 = acc[j][0] + b0, z01 = acc[j][1] + b1, z10 = acc[j][2] + b0, z11 = acc[j][3] + b1;
        if (Z2) {
            const int r = row0 + g;
            if (r < n) *reinterpret_cast<float2*>(Z2 + (size_t)r * kHid + c) = make_float2(z00, z01);
            if (r + 8 < n) *reinterpret_cast<float2*>(Z2 + (size_t)(r + 8) * kHid + c) = make_float2(z10, z11);
        }
        *reinterpret_cast<uint32_t*>(&s_h[lr0 + g][c]) = pack_bf16(silu(z00), silu(z01));
        *reinterpret_cast<uint32_t*>(&s_h[lr0 + g + 8][c]) = pack_bf16(silu(z10), silu(z11));
    }
    __syncwarp();
    if (H2)
        for (int i = lane; i < 16 * (kHid / 2); i += 32) {
            const int r = i / (kHid / 2), c = 2 * (i % (kHid / 2));
            if (row0 + r < n)
                *reinterpret_cast<uint32_t*>(H2 + (size_t)(row0 + r) * kHid + c) =
                    *reinterpret_cast<const uint32_t*>(&s_h[lr0 + r][c]);
        }
    // ---- layer 3: N = 8 (2 used), K = 128
    float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k0 = 0; k0 < kHid; k0 += 16) {
        uint32_t a[4], b[2];
        load_a(a, &s_h[0][0], kHid + 8, lr0, k0, lane);
        load_b(b, W3b, kHid, 0, k0, lane);
        mma_bf16(o, a, b);
    }
    if (t == 0) {  // columns 0 and 1 live in the lanes with t == 0
        const int r = row0 + g;
        if (r < n) *reinterpret_cast<float2*>(out + (size_t)r * 2) = make_float2(o[0] + P[oB3], o[1] + P[oB3 + 1]);
        if (r + 8 < n)
            *reinterpret_cast<float2*>(out + (size_t)(r + 8) * 2) = make_float2(o[2] + P[oB3], o[3] + P[oB3 + 1]);
    }
}

// Loss of one sample: squared error of the normalised time of impact plus
// the binary cross-entropy of the hit logit; d_out is its gradient.
__device__ __forceinline__ float sample_loss(float o0, float o1, float y0, float y1, float* d0, float* d1) {
    const float e = o0 - y0;
    const float p = 1.0f / (1.0f + expf(-o1));
    *d0 = 2.0f * e;
    *d1 = p - y1;
    // log(1 + exp(-|x|)) + max(x, 0) - x*y
    return e * e + (log1pf(expf(-fabsf(o1))) + fmaxf(o1, 0.0f) - o1 * y1);
}

// Backward pass of one block of 64 samples (after k_mlp_forward with the
// training buffers).  Accumulates the mean loss into *loss and the gradient
// of the mean loss into G (FP32, parameter layout of the master vector).
__global__ void __launch_bounds__(kThreads) k_mlp_backward(int n, float inv_n, const __nv_bfloat16* __restrict__ X,
                                                           const float* __restrict__ Y, const float* __restrict__ out,
                                                           const float* __restrict__ Z1, const float* __restrict__ Z2,
                                                           const __nv_bfloat16* __restrict__ H1,
                                                           const __nv_bfloat16* __restrict__ H2,
                                                           const __nv_bfloat16* __restrict__ W2T,
                                                           const __nv_bfloat16* __restrict__ W3b,
                                                           float* __restrict__ G, float* __restrict__ loss) {
    extern __shared__ __align__(16) unsigned char smem[];
    float* s_dz2 = reinterpret_cast<float*>(smem);                         // [64][128]
    float* s_dz1 = s_dz2 + kRows * kHid;                                  // [64][128]
    __nv_bfloat16* s_dz2b = reinterpret_cast<__nv_bfloat16*>(s_dz1 + kRows * kHid);  // [64][136]
    __shared__ float s_dout[kRows][2];
    __shared__ float s_loss[kThreads / 32];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int base = blockIdx.x * kRows;
    const int rows = min(kRows, n - base);
    // ---- output gradient and loss
    float l = 0.f;
    if (tid < kRows) {
        float d0 = 0.f, d1 = 0.f;
        if (tid < rows) {
            const int r = base + tid;
            l = sample_loss(out[2 * (size_t)r], out[2 * (size_t)r + 1], Y[2 * (size_t)r], Y[2 * (size_t)r + 1], &d0,
                            &d1);
            d0 *= inv_n;
            d1 *= inv_n;
        }
        s_dout[tid][0] = d0;
        s_dout[tid][1] = d1;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if (lane == 0) s_loss[warp] = l;
    __syncthreads();
    if (tid == 0) {
        float sum = 0.f;
        for (int w = 0; w < kThreads / 32; w++) sum += s_loss[w];
        atomicAdd(loss, sum * inv_n);
    }
    // ---- dZ2 = (dOut * W3) .* silu'(Z2)
    for (int i = tid; i < kRows * kHid; i += kThreads) {
        const int r = i / kHid, j = i % kHid;
        float v = 0.f;
        if (r < rows) {
            const float dh = s_dout[r][0] * __bfloat162float(W3b[j]) + s_dout[r][1] * __bfloat162float(W3b[kHid + j]);
            v = dh * silu_grad(Z2[(size_t)(base + r) * kHid + j]);
        }
        s_dz2[r * kHid + j] = v;
        s_dz2b[r * (kHid + 8) + j] = __float2bfloat16_rn(v);
    }
    __syncthreads();
    // ---- dH1 = dZ2 * W2 on the tensor cores (W2T is [k][n]), dZ1 = dH1 .* silu'(Z1)
    {
        const int g = lane >> 2, t = lane & 3, lr0 = warp * 16;
        float acc[16][4];
#pragma unroll
        for (int j = 0; j < 16; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[j][q] = 0.f;
#pragma unroll 2
        for (int k0 = 0; k0 < kHid; k0 += 16) {
            uint32_t a[4];
            load_a(a, s_dz2b, kHid + 8, lr0, k0, lane);
#pragma unroll
            for (int j = 0; j < 16; j++) {
                uint32_t b[2];
                load_b(b, W2T, kHid, 8 * j, k0, lane);
                mma_bf16(acc[j], a, b);
            }
        }
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int c = 8 * j + 2 * t;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int r = lr0 + g + 8 * h;
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    float v = 0.f;
                    if (r < rows) v = acc[j][2 * h + e] * silu_grad(Z1[(size_t)(base + r) * kHid + c + e]);
                    s_dz1[r * kHid + c + e] = v;
                }
            }
        }
    }
    __syncthreads();
    // ---- weight and bias gradients: FP32 sums over the block's rows
    {
        const int nn = tid;  // output neuron of layers 1 and 2
        float b1 = 0.f, b2 = 0.f;
        float w1[kIn];
#pragma unroll
        for (int k = 0; k < kIn; k++) w1[k] = 0.f;
        for (int r = 0; r < rows; r++) {
            const float d1 = s_dz1[r * kHid + nn];
            b1 += d1;
            b2 += s_dz2[r * kHid + nn];
#pragma unroll
            for (int k = 0; k < kIn; k++) w1[k] += d1 * __bfloat162float(X[(size_t)(base + r) * kInPad + k]);
        }
        atomicAdd(&G[oB1 + nn], b1);
        atomicAdd(&G[oB2 + nn], b2);
#pragma unroll
        for (int k = 0; k < kIn; k++) atomicAdd(&G[oW1 + nn * kIn + k], w1[k]);
        for (int k0 = 0; k0 < kHid; k0 += 32) {
            float w2[32];
#pragma unroll
            for (int k = 0; k < 32; k++) w2[k] = 0.f;
            for (int r = 0; r < rows; r++) {
                const float d2 = s_dz2[r * kHid + nn];
                const __nv_bfloat16* h = H1 + (size_t)(base + r) * kHid + k0;
#pragma unroll
                for (int k = 0; k < 32; k++) w2[k] += d2 * __bfloat162float(h[k]);
            }
#pragma unroll
            for (int k = 0; k < 32; k++) atomicAdd(&G[oW2 + nn * kHid + k0 + k], w2[k]);
        }
        // layer 3: thread j sums dOut[r][o] * H2[r][j]
        float w3a = 0.f, w3b = 0.f;
        for (int r = 0; r < rows; r++) {
            const float h = __bfloat162float(H2[(size_t)(base + r) * kHid + nn]);
            w3a += s_dout[r][0] * h;
            w3b += s_dout[r][1] * h;
        }
        atomicAdd(&G[oW3 + nn], w3a);
        atomicAdd(&G[oW3 + kHid + nn], w3b);
        if (tid < 2) {
            float b3 = 0.f;
            for (int r = 0; r < rows; r++) b3 += s_dout[r][tid];
            atomicAdd(&G[oB3 + tid], b3);
        }
    }
}

// Adam on the FP32 master parameters (step t >= 1).
__global__ void k_mlp_adam(int n, float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M,
                           float* __restrict__ V, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float m = b1 * M[i] + (1.0f - b1) * g;
    const float v = b2 * V[i] + (1.0f - b2) * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

// BF16 copies of the weights for the tensor-core layers (padding zero).
__global__ void k_mlp_refresh(const float* __restrict__ P, __nv_bfloat16* __restrict__ W1b,
                              __nv_bfloat16* __restrict__ W2b, __nv_bfloat16* __restrict__ W2T,
                              __nv_bfloat16* __restrict__ W3b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kHid * kInPad) {
        const int nn = i / kInPad, k = i % kInPad;
        W1b[i] = __float2bfloat16_rn(k < kIn ? P[oW1 + nn * kIn + k] : 0.0f);
    }
    if (i < kHid * kHid) {
        const int nn = i / kHid, k = i % kHid;
        const __nv_bfloat16 w = __float2bfloat16_rn(P[oW2 + i]);
        W2b[i] = w;
        W2T[k * kHid + nn] = w;
    }
    if (i < kOutPad * kHid) {
        const int o = i / kHid, k = i % kHid;
        W3b[i] = __float2bfloat16_rn(o < kOut ? P[oW3 + o * kHid + k] : 0.0f);
    }
}

// Standardised BF16 features ([n][32], zero padded to a multiple of 64 rows).
__global__ void k_mlp_features(int n, int n_pad, const float* __restrict__ F, const float* __restrict__ mean,
                               const float* __restrict__ inv_std, __nv_bfloat16* __restrict__ X) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad * kInPad) return;
    const int r = i / kInPad, k = i % kInPad;
    float v = 0.f;
    if (r < n && k < kIn) v = (F[(size_t)r * kIn + k] - mean[k]) * inv_std[k];
    X[i] = __float2bfloat16_rn(v);
}

// A shuffled batch: standardised BF16 features and targets of rows idx[0..n).
__global__ void k_mlp_gather(int n, int n_pad, const int32_t* __restrict__ idx, const float* __restrict__ F,
                             const float* __restrict__ Yall, const float* __restrict__ mean,
                             const float* __restrict__ inv_std, __nv_bfloat16* __restrict__ X,
                             float* __restrict__ Y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad * kInPad) return;
    const int r = i / kInPad, k = i % kInPad;
    float v = 0.f;
    if (r < n && k < kIn) v = (F[(size_t)idx[r] * kIn + k] - mean[k]) * inv_std[k];
    X[i] = __float2bfloat16_rn(v);
    if (r < n && k < 2) Y[2 * (size_t)r + k] = Yall[2 * (size_t)idx[r] + k];
}

}  // namespace

struct MlpState {
    d2g_ctx* ctx = nullptr;  // null once the context was destroyed
    int device = 0;
    DBuf<float> P, G, M, V, mean, inv_std, loss, F, Y, out, Z1, Z2, Fb, Yb;
    DBuf<__nv_bfloat16> W1b, W2b, W2T, W3b, X, H1, H2;
    DBuf<int32_t> perm;
    int64_t adam_t = 0;
};

}  // namespace d2g

struct d2g_mlp {
    d2g::MlpState s;
};

namespace d2g {
namespace {

#define MRC(x)                         \
    do {                               \
        if (int rc_ = (x)) return rc_; \
    } while (0)

inline int mblocks(long long n, int b = 256) { return (int)((n + b - 1) / b); }

int refresh(MlpState& S) {
    k_mlp_refresh<<<mblocks(kHid * kHid), 256, 0, S.ctx->stream>>>(S.P.p, S.W1b.p, S.W2b.p, S.W2T.p, S.W3b.p);
    S.ctx->eng.launches++;
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

// Features (host [n][20] FP32) to standardised BF16 rows in S.X.
int load_features(MlpState& S, const float* h_feat, int n, int* n_pad) {
    *n_pad = ((n + kRows - 1) / kRows) * kRows;
    MRC(S.F.ensure((size_t)n * kIn + 1));
    MRC(S.X.ensure((size_t)(*n_pad) * kInPad + 1));
    if (n) D2G_CUDA(cudaMemcpyAsync(S.F.p, h_feat, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, S.ctx->stream));
    k_mlp_features<<<mblocks((long long)(*n_pad) * kInPad), 256, 0, S.ctx->stream>>>(n, *n_pad, S.F.p, S.mean.p,
                                                                                     S.inv_std.p, S.X.p);
    S.ctx->eng.launches++;
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

int ensure_train(MlpState& S, int n_pad) {
    MRC(S.out.ensure(2 * (size_t)n_pad));
    MRC(S.Z1.ensure((size_t)n_pad * kHid));
    MRC(S.Z2.ensure((size_t)n_pad * kHid));
    MRC(S.H1.ensure((size_t)n_pad * kHid));
    MRC(S.H2.ensure((size_t)n_pad * kHid));
    return D2G_OK;
}

constexpr size_t kBackSmem = (size_t)2 * kRows * kHid * sizeof(float) + (size_t)kRows * (kHid + 8) * 2;

// Forward + backward over n samples already in S.X (and targets in d_y):
// G = gradient of the mean loss, *d_loss += mean loss.
int grad_pass(MlpState& S, int n, int n_pad, const float* d_y) {
    cudaStream_t s = S.ctx->stream;
    MRC(ensure_train(S, n_pad));
    D2G_CUDA(cudaMemsetAsync(S.G.p, 0, kParams * sizeof(float), s));
    const int blocks = n_pad / kRows;
    k_mlp_forward<<<blocks, kThreads, 0, s>>>(n, S.X.p, S.W1b.p, S.W2b.p, S.W3b.p, S.P.p, S.out.p, S.Z1.p, S.Z2.p,
                                              S.H1.p, S.H2.p);
    D2G_CUDA(cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBackSmem));
    k_mlp_backward<<<blocks, kThreads, kBackSmem, s>>>(n, 1.0f / (float)n, S.X.p, d_y, S.out.p, S.Z1.p, S.Z2.p,
                                                       S.H1.p, S.H2.p, S.W2T.p, S.W3b.p, S.G.p, S.loss.p);
    S.ctx->eng.launches += 2;
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

// Host PCG-free generator for the initial weights: SplitMix64.
uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
double unit(uint64_t& x) { return (double)(splitmix(x) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace
}  // namespace d2g

using d2g::MlpState;

namespace d2g {

// Forward pass over n feature rows already in device memory (d_feat [n][20]
// FP32, on the context's stream): *d_out points to n (TOI, hit logit) pairs
// in the network's own buffer, valid until its next call.
int mlp_forward_device(d2g_mlp* m, const float* d_feat, int n, const float** d_out) {
    MlpState& S = m->s;
    const int n_pad = ((n + kRows - 1) / kRows) * kRows;
    MRC(S.X.ensure((size_t)n_pad * kInPad + 1));
    MRC(S.out.ensure(2 * (size_t)n_pad + 2));
    if (n_pad) {
        k_mlp_features<<<mblocks((long long)n_pad * kInPad), 256, 0, S.ctx->stream>>>(n, n_pad, d_feat, S.mean.p,
                                                                                       S.inv_std.p, S.X.p);
        k_mlp_forward<<<n_pad / kRows, kThreads, 0, S.ctx->stream>>>(n, S.X.p, S.W1b.p, S.W2b.p, S.W3b.p, S.P.p,
                                                                     S.out.p, nullptr, nullptr, nullptr, nullptr);
        S.ctx->eng.launches += 2;
        D2G_CUDA(cudaGetLastError());
    }
    *d_out = S.out.p;
    return D2G_OK;
}

d2g_ctx* mlp_context(d2g_mlp* m) { return m->s.ctx; }

void mlp_orphan_all(d2g_ctx* ctx) {
    for (d2g_mlp* m : ctx->nets) m->s.ctx = nullptr;
    ctx->nets.clear();
}

}  // namespace d2g

namespace d2g {
namespace {
// A network whose context was destroyed keeps only its memory.
int mlp_live(d2g_mlp* m) {
    if (!m) {
        set_error("null network");
        return D2G_ERR_INVALID;
    }
    if (!m->s.ctx) {
        set_error("the network's context was destroyed");
        return D2G_ERR_STATE;
    }
    return D2G_OK;
}
}  // namespace
}  // namespace d2g

extern "C" {

int d2g_mlp_create(d2g_ctx* ctx, uint64_t seed, d2g_mlp** out) {
    using namespace d2g;
    if (!ctx || !out) {
        set_error("null argument");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaSetDevice(ctx->device));
    d2g_mlp* m = new d2g_mlp();
    MlpState& S = m->s;
    S.ctx = ctx;
    S.device = ctx->device;
    int rc = D2G_OK;
    for (DBuf<float>* b : {&S.P, &S.G, &S.M, &S.V})
        if (!rc) rc = b->ensure(kParams);
    if (!rc) rc = S.mean.ensure(kIn);
    if (!rc) rc = S.inv_std.ensure(kIn);
    if (!rc) rc = S.loss.ensure(1);
    if (!rc) rc = S.W1b.ensure(kHid * kInPad);
    if (!rc) rc = S.W2b.ensure(kHid * kHid);
    if (!rc) rc = S.W2T.ensure(kHid * kHid);
    if (!rc) rc = S.W3b.ensure(kOutPad * kHid);
    if (rc) {
        delete m;
        return rc;
    }
    // PyTorch-style Linear initialisation: U(-1/sqrt(fan_in), 1/sqrt(fan_in))
    std::vector<float> p(kParams);
    uint64_t st = seed;
    auto fill = [&](int off, int cnt, int fan_in) {
        const double bnd = 1.0 / std::sqrt((double)fan_in);
        for (int i = 0; i < cnt; i++) p[off + i] = (float)((2.0 * unit(st) - 1.0) * bnd);
    };
    fill(oW1, kHid * kIn, kIn);
    fill(oB1, kHid, kIn);
    fill(oW2, kHid * kHid, kHid);
    fill(oB2, kHid, kHid);
    fill(oW3, kOut * kHid, kHid);
    fill(oB3, kOut, kHid);
    std::vector<float> zero(kParams, 0.f), mean(kIn, 0.f), one(kIn, 1.f);
    cudaStream_t s = ctx->stream;
    D2G_CUDA(cudaMemcpyAsync(S.P.p, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice, s));
    D2G_CUDA(cudaMemcpyAsync(S.M.p, zero.data(), kParams * sizeof(float), cudaMemcpyHostToDevice, s));
    D2G_CUDA(cudaMemcpyAsync(S.V.p, zero.data(), kParams * sizeof(float), cudaMemcpyHostToDevice, s));
    D2G_CUDA(cudaMemcpyAsync(S.mean.p, mean.data(), kIn * sizeof(float), cudaMemcpyHostToDevice, s));
    D2G_CUDA(cudaMemcpyAsync(S.inv_std.p, one.data(), kIn * sizeof(float), cudaMemcpyHostToDevice, s));
    if ((rc = refresh(S))) {
        delete m;
        return rc;
    }
    D2G_CUDA(cudaStreamSynchronize(s));
    ctx->nets.push_back(m);
    *out = m;
    return D2G_OK;
}

void d2g_mlp_destroy(d2g_mlp* m) {
    if (!m) return;
    cudaSetDevice(m->s.device);
    if (d2g_ctx* c = m->s.ctx) {
        cudaStreamSynchronize(c->stream);
        if (c->eng.proposal == m) c->eng.proposal = nullptr;  // the CCD stops consulting it
        for (size_t i = 0; i < c->nets.size(); i++)
            if (c->nets[i] == m) {
                c->nets.erase(c->nets.begin() + (long)i);
                break;
            }
    }
    delete m;  // frees the device buffers (the device is current)
}

int d2g_mlp_params(d2g_mlp* m, float* params, int32_t n) {
    using namespace d2g;
    MRC(mlp_live(m));
    if (!m || !params || n != kParams) {
        set_error("parameter buffer must hold D2G_MLP_PARAMS floats");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaMemcpyAsync(params, m->s.P.p, kParams * sizeof(float), cudaMemcpyDeviceToHost, m->s.ctx->stream));
    D2G_CUDA(cudaStreamSynchronize(m->s.ctx->stream));
    return D2G_OK;
}

int d2g_mlp_set_params(d2g_mlp* m, const float* params, int32_t n) {
    using namespace d2g;
    MRC(mlp_live(m));
    if (!m || !params || n != kParams) {
        set_error("parameter buffer must hold D2G_MLP_PARAMS floats");
        return D2G_ERR_INVALID;
    }
    D2G_CUDA(cudaMemcpyAsync(m->s.P.p, params, kParams * sizeof(float), cudaMemcpyHostToDevice, m->s.ctx->stream));
    MRC(refresh(m->s));
    D2G_CUDA(cudaStreamSynchronize(m->s.ctx->stream));
    return D2G_OK;
}

int d2g_mlp_set_normalization(d2g_mlp* m, const float* mean, const float* std_dev) {
    using namespace d2g;
    MRC(mlp_live(m));
    if (!m || !mean || !std_dev) {
        set_error("null argument");
        return D2G_ERR_INVALID;
    }
    float inv[kIn];
    for (int k = 0; k < kIn; k++) inv[k] = std_dev[k] > 0.f ? 1.0f / std_dev[k] : 1.0f;
    D2G_CUDA(cudaMemcpyAsync(m->s.mean.p, mean, kIn * sizeof(float), cudaMemcpyHostToDevice, m->s.ctx->stream));
    D2G_CUDA(cudaMemcpyAsync(m->s.inv_std.p, inv, kIn * sizeof(float), cudaMemcpyHostToDevice, m->s.ctx->stream));
    D2G_CUDA(cudaStreamSynchronize(m->s.ctx->stream));
    return D2G_OK;
}

int d2g_mlp_predict(d2g_mlp* m, const float* features, int32_t n, float* out) {
    using namespace d2g;
    MRC(mlp_live(m));
    if (!m || n < 0 || (n > 0 && (!features || !out))) {
        set_error("invalid arguments");
        return D2G_ERR_INVALID;
    }
    MlpState& S = m->s;
    int n_pad = 0;
    MRC(load_features(S, features, n, &n_pad));
    MRC(S.out.ensure(2 * (size_t)n_pad + 2));
    if (n_pad) {
        k_mlp_forward<<<n_pad / kRows, kThreads, 0, S.ctx->stream>>>(n, S.X.p, S.W1b.p, S.W2b.p, S.W3b.p, S.P.p,
                                                                     S.out.p, nullptr, nullptr, nullptr, nullptr);
        S.ctx->eng.launches++;
        D2G_CUDA(cudaGetLastError());
        D2G_CUDA(cudaMemcpyAsync(out, S.out.p, 2 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, S.ctx->stream));
    }
    D2G_CUDA(cudaStreamSynchronize(S.ctx->stream));
    return D2G_OK;
}

int d2g_mlp_gradient(d2g_mlp* m, const float* features, const float* targets, int32_t n, float* grad, float* loss) {
    using namespace d2g;
    MRC(mlp_live(m));
    if (!m || n <= 0 || !features || !targets || !grad || !loss) {
        set_error("invalid arguments");
        return D2G_ERR_INVALID;
    }
    MlpState& S = m->s;
    int n_pad = 0;
    MRC(load_features(S, features, n, &n_pad));
    MRC(S.Y.ensure(2 * (size_t)n + 2));
    D2G_CUDA(cudaMemcpyAsync(S.Y.p, targets, 2 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice, S.ctx->stream));
    D2G_CUDA(cudaMemsetAsync(S.loss.p, 0, sizeof(float), S.ctx->stream));
    MRC(grad_pass(S, n, n_pad, S.Y.p));
    D2G_CUDA(cudaMemcpyAsync(grad, S.G.p, kParams * sizeof(float), cudaMemcpyDeviceToHost, S.ctx->stream));
    D2G_CUDA(cudaMemcpyAsync(loss, S.loss.p, sizeof(float), cudaMemcpyDeviceToHost, S.ctx->stream));
    D2G_CUDA(cudaStreamSynchronize(S.ctx->stream));
    return D2G_OK;
}

}  // extern "C"

extern "C" int d2g_mlp_train(d2g_mlp* m, const float* features, const float* targets, int32_t n, int32_t epochs,
                             int32_t batch, float lr, uint64_t seed, float* epoch_loss) {
    using namespace d2g;
    MRC(mlp_live(m));
    if (!m || n <= 0 || !features || !targets || epochs < 0 || batch <= 0) {
        set_error("invalid arguments");
        return D2G_ERR_INVALID;
    }
    MlpState& S = m->s;
    cudaStream_t s = S.ctx->stream;
    const int b_pad = ((batch + kRows - 1) / kRows) * kRows;
    MRC(S.F.ensure((size_t)n * kIn + 1));
    MRC(S.Y.ensure(2 * (size_t)n + 2));
    MRC(S.Yb.ensure(2 * (size_t)b_pad + 2));
    MRC(S.X.ensure((size_t)b_pad * kInPad + 1));
    MRC(S.perm.ensure((size_t)n + 1));
    D2G_CUDA(cudaMemcpyAsync(S.F.p, features, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, s));
    D2G_CUDA(cudaMemcpyAsync(S.Y.p, targets, 2 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s));
    std::vector<int32_t> perm(n);
    uint64_t st = seed;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int e = 0; e < epochs; e++) {
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = n - 1; i > 0; i--) {  // Fisher-Yates
            const int j = (int)(splitmix(st) % (uint64_t)(i + 1));
            const int t = perm[i];
            perm[i] = perm[j];
            perm[j] = t;
        }
        D2G_CUDA(cudaMemcpyAsync(S.perm.p, perm.data(), (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        D2G_CUDA(cudaMemsetAsync(S.loss.p, 0, sizeof(float), s));
        int steps = 0;
        for (int off = 0; off < n; off += batch) {
            const int nb = std::min(batch, n - off);
            const int np = ((nb + kRows - 1) / kRows) * kRows;
            k_mlp_gather<<<mblocks((long long)np * kInPad), 256, 0, s>>>(nb, np, S.perm.p + off, S.F.p, S.Y.p,
                                                                         S.mean.p, S.inv_std.p, S.X.p, S.Yb.p);
            S.ctx->eng.launches++;
            MRC(grad_pass(S, nb, np, S.Yb.p));
            S.adam_t++;
            const float c1 = 1.0f - std::pow(b1, (float)S.adam_t), c2 = 1.0f - std::pow(b2, (float)S.adam_t);
            k_mlp_adam<<<mblocks(kParams), 256, 0, s>>>(kParams, S.P.p, S.G.p, S.M.p, S.V.p, lr, b1, b2, eps, c1, c2);
            S.ctx->eng.launches++;
            MRC(refresh(S));
            steps++;
        }
        float l = 0.f;
        D2G_CUDA(cudaMemcpyAsync(&l, S.loss.p, sizeof(float), cudaMemcpyDeviceToHost, s));
        D2G_CUDA(cudaStreamSynchronize(s));
        if (epoch_loss) epoch_loss[e] = l / (float)std::max(steps, 1);
    }
    D2G_CUDA(cudaStreamSynchronize(s));
    return D2G_OK;
}
