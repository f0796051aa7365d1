/*
 * mlp.cuh -- the learned aerodynamic closure: a 12 -> 64 -> 64 -> 64 -> 2 perceptron with GELU
 * hidden activations, BF16 weights and activations, FP32 accumulation, evaluated by one warp per
 * tile of 16 samples on the tensor cores (mma.sync m16n8k16 BF16 -> FP32).
 *
 * Parameter vector (FP32 master copy, the layout every entry point shares):
 *   W1[64][16] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[8][64] b4[8]
 *   in_shift[16] in_scale[16] out_shift[2] out_scale[2]
 * (W rows are outputs; the 12 inputs are padded to 16 and the 2 outputs to 8 with zero rows.)
 * Inputs are normalised as (x - in_shift) * in_scale; outputs are y * out_scale + out_shift.
 *
 * The device copy holds, besides the FP32 master, BF16 weights in two layouts: W in the fragment
 * order of `layer` (the B operand of the forward pass) and W^T (input-major, the B operand of the
 * backward pass).
 *
 * Fragment layouts of mma.m16n8k16 (PTX ISA), g = lane / 4, t = lane % 4:
 *   A (16x16, row): reg0 = A[g][2t..2t+1], reg1 = A[g+8][2t..], reg2 = A[g][2t+8..], reg3 = A[g+8][2t+8..]
 *   B (16x8, col):  reg0 = B[2t..2t+1][g], reg1 = B[2t+8..][g]
 *   C (16x8):       c0,c1 = C[g][2t..2t+1], c2,c3 = C[g+8][2t..2t+1]
 * so the C fragments of one layer are the A fragments of the next after BF16 packing.
 */
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace fjsph {
namespace mlp {

constexpr int kIn = 12, kInP = 16, kHid = 64, kOut = 2, kOutP = 8;

/* offsets into the FP32 parameter vector */
constexpr int oW1 = 0;
constexpr int oB1 = oW1 + kHid * kInP;
constexpr int oW2 = oB1 + kHid;
constexpr int oB2 = oW2 + kHid * kHid;
constexpr int oW3 = oB2 + kHid;
constexpr int oB3 = oW3 + kHid * kHid;
constexpr int oW4 = oB3 + kHid;
constexpr int oB4 = oW4 + kOutP * kHid;
constexpr int kNumWeights = oB4 + kOutP; /* trainable */
constexpr int oInShift = kNumWeights;
constexpr int oInScale = oInShift + kInP;
constexpr int oOutShift = oInScale + kInP;
constexpr int oOutScale = oOutShift + kOut;
constexpr int kNumParams = oOutScale + kOut;

/* BF16 copies: element offsets (in bf16 units) of each matrix, forward (W) and transposed (WT) */
constexpr int bW1 = 0, bW2 = bW1 + kHid * kInP, bW3 = bW2 + kHid * kHid, bW4 = bW3 + kHid * kHid;
constexpr int kNumBf16 = bW4 + kOutP * kHid;

struct DevMlp {
    const float *params;          /* FP32 master (kNumParams)                  */
    const __nv_bfloat16 *w;       /* forward weights, fragment order, kNumBf16   */
    const __nv_bfloat16 *wt;      /* transposed layout, kNumBf16                */
};

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

/* GELU in its tanh form (Hendrycks & Gimpel 2016), x/2 (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))),
 * on the SFU's tanh.approx.f32 (relative error about 2^-11, below the BF16 rounding that follows). */
__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float kGeluS = 0.7978845608028654f; /* sqrt(2/pi) */
constexpr float kGeluC = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
    const float u = kGeluS * (x + kGeluC * x * x * x);
    return 0.5f * x * (1.f + tanh_fast(u));
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float u = kGeluS * (x + kGeluC * x * x * x);
    const float th = tanh_fast(u);
    return 0.5f * (1.f + th) + 0.5f * x * (1.f - th * th) * kGeluS * (1.f + 3.f * kGeluC * x * x);
}

/* One lane's B fragments of output fragment nt (K/8 words).  The loads are volatile asm, like
 * the MMAs, so they stay in program order: `layer` fetches one fragment ahead of the MMAs that use
 * it instead of hoisting every weight load of the layer into registers at once. */
template <int KS>
__device__ __forceinline__ void load_b(const uint32_t *src, uint32_t (&b)[2 * KS]) {
    if constexpr (KS == 1) {
        asm volatile("ld.global.nc.v2.u32 {%0,%1}, [%2];\n" : "=r"(b[0]), "=r"(b[1]) : "l"(src));
    } else {
#pragma unroll
        for (int q = 0; q < KS / 2; ++q)
            asm volatile("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];\n"
                         : "=r"(b[4 * q]), "=r"(b[4 * q + 1]), "=r"(b[4 * q + 2]), "=r"(b[4 * q + 3])
                         : "l"(src + 4 * q));
    }
}

template <int K, int N>
__device__ __forceinline__ void layer(const uint32_t (&A)[K / 16][4], const __nv_bfloat16 *Wf, const float *bias,
                                      float (&C)[N / 8][4]) {
    constexpr int KS = K / 16, NT = N / 8;
    const int lane = threadIdx.x & 31, t = lane & 3;
    const uint32_t *base = reinterpret_cast<const uint32_t *>(Wf) + lane * (2 * KS);
    uint32_t b[2][2 * KS];
    load_b<KS>(base, b[0]);
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        if (nt + 1 < NT) load_b<KS>(base + (nt + 1) * 32 * (2 * KS), b[(nt + 1) & 1]);
        float b0 = 0.f, b1 = 0.f;
        if (bias)
            asm volatile("ld.global.nc.v2.f32 {%0,%1}, [%2];\n"
                         : "=f"(b0), "=f"(b1)
                         : "l"(bias + nt * 8 + 2 * t));
        C[nt][0] = b0;
        C[nt][1] = b1;
        C[nt][2] = b0;
        C[nt][3] = b1;
#pragma unroll
        for (int ks = 0; ks < KS; ++ks) mma16816(C[nt], A[ks], b[nt & 1][2 * ks], b[nt & 1][2 * ks + 1]);
    }
}

/* position of W[n][k] (K inputs) in the fragment order of `layer` */
__host__ __device__ __forceinline__ int frag_index(int n, int k, int K) {
    const int nt = n / 8, g = n % 8, ks = k / 16, h = (k % 16) / 8, t = (k % 8) / 2, e = k % 2;
    const int lane = g * 4 + t;
    return ((((nt * 32 + lane) * (K / 16) + ks) * 2 + h) * 2) + e;
}

/* GELU on a C tile, then BF16 A fragments for the next layer (K_next = N). */
template <int N>
__device__ __forceinline__ void gelu_to_a(const float (&C)[N / 8][4], uint32_t (&A)[N / 16][4]) {
#pragma unroll
    for (int ks = 0; ks < N / 16; ++ks) {
        A[ks][0] = pack2(gelu(C[2 * ks][0]), gelu(C[2 * ks][1]));
        A[ks][1] = pack2(gelu(C[2 * ks][2]), gelu(C[2 * ks][3]));
        A[ks][2] = pack2(gelu(C[2 * ks + 1][0]), gelu(C[2 * ks + 1][1]));
        A[ks][3] = pack2(gelu(C[2 * ks + 1][2]), gelu(C[2 * ks + 1][3]));
    }
}

/* Input fragment of a 16-sample tile from a per-warp shared tile X[16][16] (BF16, normalised). */
__device__ __forceinline__ void load_a16(const __nv_bfloat16 *X, uint32_t (&A)[1][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t *X32 = reinterpret_cast<const uint32_t *>(X);
    A[0][0] = X32[g * 8 + t];
    A[0][1] = X32[(g + 8) * 8 + t];
    A[0][2] = X32[g * 8 + 4 + t];
    A[0][3] = X32[(g + 8) * 8 + 4 + t];
}

/* A hidden layer (K inputs -> N outputs) with GELU, straight into the next layer's A fragments:
 * the output fragments are computed two at a time (one 16-wide k-tile of the next layer), so 8
 * accumulators are live instead of N / 2 -- the same MMAs, bias, GELU and BF16 packing as
 * `layer` followed by `gelu_to_a`, in fewer registers (the network runs inside the force kernel
 * under its register budget).  Each fragment's weights are fetched right before its MMAs: a
 * fetch one fragment ahead measured slower here (its registers cost more spills than the
 * latency it hides). */
template <int K, int N>
__device__ __forceinline__ void layer_gelu(const uint32_t (&A)[K / 16][4], const __nv_bfloat16 *Wf, const float *bias,
                                           uint32_t (&Aout)[N / 16][4]) {
    constexpr int KS = K / 16;
    const int lane = threadIdx.x & 31, t = lane & 3;
    const uint32_t *base = reinterpret_cast<const uint32_t *>(Wf) + lane * (2 * KS);
#pragma unroll
    for (int ko = 0; ko < N / 16; ++ko) {
        float C[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int nt = 2 * ko + h;
            uint32_t b[2 * KS];
            load_b<KS>(base + nt * 32 * (2 * KS), b);
            float b0, b1;
            asm volatile("ld.global.nc.v2.f32 {%0,%1}, [%2];\n" : "=f"(b0), "=f"(b1) : "l"(bias + nt * 8 + 2 * t));
            C[h][0] = b0;
            C[h][1] = b1;
            C[h][2] = b0;
            C[h][3] = b1;
#pragma unroll
            for (int ks = 0; ks < KS; ++ks) mma16816(C[h], A[ks], b[2 * ks], b[2 * ks + 1]);
        }
        Aout[ko][0] = pack2(gelu(C[0][0]), gelu(C[0][1]));
        Aout[ko][1] = pack2(gelu(C[0][2]), gelu(C[0][3]));
        Aout[ko][2] = pack2(gelu(C[1][0]), gelu(C[1][1]));
        Aout[ko][3] = pack2(gelu(C[1][2]), gelu(C[1][3]));
    }
}

/* Forward pass of one 16-sample tile from its input A fragment (normalised, BF16); Y receives the
 * (un-normalised) 2 outputs of row g and g+8 for lanes with t == 0 (Y[0], Y[1] of row g; Y[2],
 * Y[3] of row g+8). */
__device__ __forceinline__ void forward_frag(const DevMlp &M, const uint32_t (&A0)[1][4], float (&Y)[4]) {
    uint32_t A1[kHid / 16][4];
    layer_gelu<kInP, kHid>(A0, M.w + bW1, M.params + oB1, A1);
    uint32_t A2[kHid / 16][4];
    layer_gelu<kHid, kHid>(A1, M.w + bW2, M.params + oB2, A2);
    uint32_t A3[kHid / 16][4];
    layer_gelu<kHid, kHid>(A2, M.w + bW3, M.params + oB3, A3);
    float C4[1][4];
    layer<kHid, kOutP>(A3, M.w + bW4, M.params + oB4, C4);
    const float s0 = __ldg(M.params + oOutScale), s1 = __ldg(M.params + oOutScale + 1);
    const float h0 = __ldg(M.params + oOutShift), h1 = __ldg(M.params + oOutShift + 1);
    Y[0] = C4[0][0] * s0 + h0;
    Y[1] = C4[0][1] * s1 + h1;
    Y[2] = C4[0][2] * s0 + h0;
    Y[3] = C4[0][3] * s1 + h1;
}

/* The same from a shared tile X[16][16]. */
__device__ __forceinline__ void forward_tile(const DevMlp &M, const __nv_bfloat16 *X, float (&Y)[4]) {
    uint32_t A0[1][4];
    load_a16(X, A0);
    forward_frag(M, A0, Y);
}

} // namespace mlp
} // namespace fjsph
