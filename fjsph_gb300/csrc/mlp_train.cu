/*
 * mlp_train.cu -- training and batch inference of the learned aerodynamic closure (mlp.cuh).
 *
 * One CTA = two warps; a warp takes tiles of 16 samples.  Per tile:
 *   forward:  H0 = x_norm, Z_l = H_{l-1} W_l^T + b_l, H_l = GELU(Z_l) (l = 1..3), Y = H3 W4^T + b4
 *   loss:     sum over samples and both outputs of (Y - t_norm)^2, scaled by 1 / batch
 *   backward: dZ4 = 2 (Y - t_norm) / batch; dH_{l-1} = dZ_l W_l; dZ_{l-1} = dH_{l-1} * GELU'(Z_{l-1});
 *             dW_l += dZ_l^T H_{l-1}; db_l += column sums of dZ_l
 * All matrix products are BF16 x BF16 -> FP32 tensor-core MMAs; Z_l and H_l of the tile are kept
 * in shared memory between the passes; weight gradients accumulate in shared memory and are added
 * to the global gradient once per CTA.  Adam updates the FP32 master and re-casts the BF16 copies.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/fjsph_gb300.h"
#include "mlp.cuh"

namespace fjsph {
namespace mlp {

/* transposed (input-major) BF16 layouts used by the backward pass */
constexpr int tW1 = 0;                      /* [16 in][64 out] */
constexpr int tW2 = tW1 + kInP * kHid;      /* [64][64]        */
constexpr int tW3 = tW2 + kHid * kHid;      /* [64][64]        */
constexpr int tW4 = tW3 + kHid * kHid;      /* [64 in][16 out], outputs 8..15 zero */
constexpr int kNumBf16T = tW4 + kHid * 16;

namespace {

constexpr int kWarps = 2;

struct WarpSmem {
    __nv_bfloat16 X[16][kInP];
    __nv_bfloat16 H[3][16][kHid];
    float Z[3][16][kHid];
    __nv_bfloat16 dZ[16][kHid];
};

struct CtaSmem {
    WarpSmem w[kWarps];
    float grad[kNumWeights];
};

/* normalised input tile of a warp: rows past n are zero */
__device__ void stage_inputs(const float *params, const float *X, int64_t n, int64_t row0, __nv_bfloat16 (*Xs)[kInP]) {
    const int lane = threadIdx.x & 31;
    for (int e = lane; e < 16 * kInP; e += 32) {
        const int r = e / kInP, c = e % kInP;
        float v = 0.f;
        if (row0 + r < n && c < kIn) v = (X[(row0 + r) * kIn + c] - params[oInShift + c]) * params[oInScale + c];
        Xs[r][c] = __float2bfloat16_rn(v);
    }
    __syncwarp();
}

/* C tile -> shared (fp32 Z and bf16 GELU(Z)) */
template <int N>
__device__ void store_zh(const float (&C)[N / 8][4], float (*Z)[kHid], __nv_bfloat16 (*H)[kHid]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = g + (q >> 1) * 8, c = nt * 8 + 2 * t + (q & 1);
            Z[r][c] = C[nt][q];
            H[r][c] = __float2bfloat16_rn(gelu(C[nt][q]));
        }
}

/* dH = dZ W for a layer with N outputs and K inputs: A = dZ (C fragments, N/8), B from W^T. */
template <int N, int K>
__device__ void backprop(const float (&dZ)[N / 8][4], const __nv_bfloat16 *WT, float (&dH)[K / 8][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    constexpr int KS = (N + 15) / 16;
    uint32_t A[KS][4];
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
        const int n0 = 2 * ks, n1 = 2 * ks + 1;
        A[ks][0] = pack2(dZ[n0][0], dZ[n0][1]);
        A[ks][1] = pack2(dZ[n0][2], dZ[n0][3]);
        A[ks][2] = n1 < N / 8 ? pack2(dZ[n1][0], dZ[n1][1]) : 0u;
        A[ks][3] = n1 < N / 8 ? pack2(dZ[n1][2], dZ[n1][3]) : 0u;
    }
    constexpr int LD = KS * 16; /* row length of W^T (outputs, padded) */
    const uint32_t *WT32 = reinterpret_cast<const uint32_t *>(WT);
#pragma unroll
    for (int nt = 0; nt < K / 8; ++nt) {
        dH[nt][0] = dH[nt][1] = dH[nt][2] = dH[nt][3] = 0.f;
        const uint32_t *row = WT32 + (nt * 8 + g) * (LD / 2);
#pragma unroll
        for (int ks = 0; ks < KS; ++ks) mma16816(dH[nt], A[ks], __ldg(row + ks * 8 + t), __ldg(row + ks * 8 + 4 + t));
    }
}

/* dW[out][in] += sum_s dZ[s][out] H[s][in]; dZs is dZ in shared (bf16 [16][N]); H is [16][ld]. */
template <int N, int K>
__device__ void weight_grad(const __nv_bfloat16 (*dZs)[kHid], const __nv_bfloat16 *Hs, int ldh, float *gW) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    constexpr int MT = (N + 15) / 16;
    auto dz = [&](int s, int o) -> __nv_bfloat16 { return o < N ? dZs[s][o] : __float2bfloat16_rn(0.f); };
    auto pk = [](__nv_bfloat16 a, __nv_bfloat16 b) -> uint32_t {
        __nv_bfloat162 v;
        v.x = a;
        v.y = b;
        return *reinterpret_cast<uint32_t *>(&v);
    };
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
        uint32_t A[4];
        const int o0 = mt * 16 + g, o1 = o0 + 8;
        A[0] = pk(dz(2 * t, o0), dz(2 * t + 1, o0));
        A[1] = pk(dz(2 * t, o1), dz(2 * t + 1, o1));
        A[2] = pk(dz(8 + 2 * t, o0), dz(9 + 2 * t, o0));
        A[3] = pk(dz(8 + 2 * t, o1), dz(9 + 2 * t, o1));
#pragma unroll
        for (int nt = 0; nt < K / 8; ++nt) {
            const int in = nt * 8 + g;
            const uint32_t b0 = pk(Hs[(2 * t) * ldh + in], Hs[(2 * t + 1) * ldh + in]);
            const uint32_t b1 = pk(Hs[(8 + 2 * t) * ldh + in], Hs[(9 + 2 * t) * ldh + in]);
            float C[4] = {0.f, 0.f, 0.f, 0.f};
            uint32_t Af[4] = {A[0], A[1], A[2], A[3]};
            mma16816(C, Af, b0, b1);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int o = mt * 16 + g + (q >> 1) * 8, c = nt * 8 + 2 * t + (q & 1);
                if (o < N) atomicAdd(&gW[o * K + c], C[q]);
            }
        }
    }
}

/* column sums of a C tile (bias gradient) */
template <int N>
__device__ void bias_grad(const float (&dZ)[N / 8][4], float *gb, int nvalid) {
    const int lane = threadIdx.x & 31, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
        float v0 = dZ[nt][0] + dZ[nt][2], v1 = dZ[nt][1] + dZ[nt][3];
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            v0 += __shfl_xor_sync(0xffffffffu, v0, o);
            v1 += __shfl_xor_sync(0xffffffffu, v1, o);
        }
        if (lane < 4) {
            const int c = nt * 8 + 2 * t;
            if (c < nvalid) atomicAdd(&gb[c], v0);
            if (c + 1 < nvalid) atomicAdd(&gb[c + 1], v1);
        }
    }
}

template <int N>
__device__ void to_shared_bf16(const float (&C)[N / 8][4], __nv_bfloat16 (*S)[kHid]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) S[g + (q >> 1) * 8][nt * 8 + 2 * t + (q & 1)] = __float2bfloat16_rn(C[nt][q]);
}

__global__ void __launch_bounds__(32 * kWarps) k_mlp_grad(DevMlp M, const __nv_bfloat16 *wt, const float *X,
                                                           const float *T, int64_t n, float inv_batch, float *grad,
                                                           double *loss) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CtaSmem &S = *reinterpret_cast<CtaSmem *>(smem_raw);
    for (int e = threadIdx.x; e < kNumWeights; e += blockDim.x) S.grad[e] = 0.f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    WarpSmem &W = S.w[warp];
    const int64_t ntiles = (n + 15) / 16;
    double lsum = 0.0;
    for (int64_t tile = (int64_t)blockIdx.x * kWarps + warp; tile < ntiles; tile += (int64_t)gridDim.x * kWarps) {
        const int64_t row0 = tile * 16;
        stage_inputs(M.params, X, n, row0, W.X);
        uint32_t A0[1][4];
        load_a16(&W.X[0][0], A0);
        float C1[8][4], C2[8][4], C3[8][4], C4[1][4];
        layer<kInP, kHid>(A0, M.w + bW1, M.params + oB1, C1);
        store_zh<kHid>(C1, W.Z[0], W.H[0]);
        uint32_t A1[4][4];
        gelu_to_a<kHid>(C1, A1);
        layer<kHid, kHid>(A1, M.w + bW2, M.params + oB2, C2);
        store_zh<kHid>(C2, W.Z[1], W.H[1]);
        uint32_t A2[4][4];
        gelu_to_a<kHid>(C2, A2);
        layer<kHid, kHid>(A2, M.w + bW3, M.params + oB3, C3);
        store_zh<kHid>(C3, W.Z[2], W.H[2]);
        uint32_t A3[4][4];
        gelu_to_a<kHid>(C3, A3);
        layer<kHid, kOutP>(A3, M.w + bW4, M.params + oB4, C4);
        __syncwarp();
        /* dY on the 2 real outputs (columns 0, 1: lanes with t == 0) */
        float dY[1][4] = {{0.f, 0.f, 0.f, 0.f}};
        if (t == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int r = g + (q >> 1) * 8, o = q & 1;
                if (row0 + r < n) {
                    const float tn = (T[(row0 + r) * kOut + o] - M.params[oOutShift + o]) / M.params[oOutScale + o];
                    const float e = C4[0][q] - tn;
                    lsum += (double)e * e;
                    dY[0][q] = 2.f * e * inv_batch;
                }
            }
        }
        /* layer 4 */
        to_shared_bf16<kOutP>(dY, W.dZ);
        __syncwarp();
        weight_grad<kOutP, kHid>(W.dZ, &W.H[2][0][0], kHid, S.grad + oW4);
        bias_grad<kOutP>(dY, S.grad + oB4, kOut);
        float dH[8][4];
        backprop<kOutP, kHid>(dY, wt + tW4, dH);
        /* layer 3 */
        float dZ[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                dZ[nt][q] = dH[nt][q] * gelu_grad(W.Z[2][g + (q >> 1) * 8][nt * 8 + 2 * t + (q & 1)]);
        __syncwarp();
        to_shared_bf16<kHid>(dZ, W.dZ);
        __syncwarp();
        weight_grad<kHid, kHid>(W.dZ, &W.H[1][0][0], kHid, S.grad + oW3);
        bias_grad<kHid>(dZ, S.grad + oB3, kHid);
        backprop<kHid, kHid>(dZ, wt + tW3, dH);
        /* layer 2 */
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                dZ[nt][q] = dH[nt][q] * gelu_grad(W.Z[1][g + (q >> 1) * 8][nt * 8 + 2 * t + (q & 1)]);
        __syncwarp();
        to_shared_bf16<kHid>(dZ, W.dZ);
        __syncwarp();
        weight_grad<kHid, kHid>(W.dZ, &W.H[0][0][0], kHid, S.grad + oW2);
        bias_grad<kHid>(dZ, S.grad + oB2, kHid);
        backprop<kHid, kHid>(dZ, wt + tW2, dH);
        /* layer 1 */
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                dZ[nt][q] = dH[nt][q] * gelu_grad(W.Z[0][g + (q >> 1) * 8][nt * 8 + 2 * t + (q & 1)]);
        __syncwarp();
        to_shared_bf16<kHid>(dZ, W.dZ);
        __syncwarp();
        weight_grad<kHid, kInP>(W.dZ, &W.X[0][0], kInP, S.grad + oW1);
        bias_grad<kHid>(dZ, S.grad + oB1, kHid);
        __syncwarp();
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kNumWeights; e += blockDim.x)
        if (S.grad[e] != 0.f) atomicAdd(&grad[e], S.grad[e]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0 && loss) atomicAdd(loss, lsum); /* sum of squared errors */
}

/* BF16 forward and transposed copies from the FP32 master */
__global__ void k_mlp_cast(const float *params, __nv_bfloat16 *w, __nv_bfloat16 *wt) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kNumBf16; e += gridDim.x * blockDim.x) {
        /* forward copy: each matrix (row = output) scattered into the fragment order of layer() */
        int src, dst;
        if (e < bW2) {
            const int n = (e - bW1) / kInP, k = (e - bW1) % kInP;
            src = oW1 + e - bW1;
            dst = bW1 + frag_index(n, k, kInP);
        } else if (e < bW3) {
            const int n = (e - bW2) / kHid, k = (e - bW2) % kHid;
            src = oW2 + e - bW2;
            dst = bW2 + frag_index(n, k, kHid);
        } else if (e < bW4) {
            const int n = (e - bW3) / kHid, k = (e - bW3) % kHid;
            src = oW3 + e - bW3;
            dst = bW3 + frag_index(n, k, kHid);
        } else {
            const int n = (e - bW4) / kHid, k = (e - bW4) % kHid;
            src = oW4 + e - bW4;
            dst = bW4 + frag_index(n, k, kHid);
        }
        w[dst] = __float2bfloat16_rn(params[src]);
    }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kNumBf16T; e += gridDim.x * blockDim.x) {
        float v = 0.f;
        if (e < tW2) { /* [in 16][out 64] <- W1[out][in] */
            const int in = (e - tW1) / kHid, out = (e - tW1) % kHid;
            v = params[oW1 + out * kInP + in];
        } else if (e < tW3) {
            const int in = (e - tW2) / kHid, out = (e - tW2) % kHid;
            v = params[oW2 + out * kHid + in];
        } else if (e < tW4) {
            const int in = (e - tW3) / kHid, out = (e - tW3) % kHid;
            v = params[oW3 + out * kHid + in];
        } else { /* [in 64][out 16] <- W4[out 8][in 64] */
            const int in = (e - tW4) / 16, out = (e - tW4) % 16;
            v = out < kOutP ? params[oW4 + out * kHid + in] : 0.f;
        }
        wt[e] = __float2bfloat16_rn(v);
    }
}

__global__ void k_adam(float *params, float *grad, float *m, float *v, int step, float lr, float b1, float b2,
                       float eps) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kNumWeights; e += gridDim.x * blockDim.x) {
        const float gr = grad[e];
        const float mm = b1 * m[e] + (1.f - b1) * gr;
        const float vv = b2 * v[e] + (1.f - b2) * gr * gr;
        m[e] = mm;
        v[e] = vv;
        params[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
        grad[e] = 0.f;
    }
}

__global__ void __launch_bounds__(32 * kWarps) k_mlp_infer(DevMlp M, const float *X, int64_t n, float *Y) {
    __shared__ __align__(16) __nv_bfloat16 Xs[kWarps][16][kInP];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int64_t ntiles = (n + 15) / 16;
    for (int64_t tile = (int64_t)blockIdx.x * kWarps + warp; tile < ntiles; tile += (int64_t)gridDim.x * kWarps) {
        const int64_t row0 = tile * 16;
        stage_inputs(M.params, X, n, row0, Xs[warp]);
        float Yv[4];
        forward_tile(M, &Xs[warp][0][0], Yv);
        if (t == 0) {
            if (row0 + g < n) {
                Y[(row0 + g) * kOut] = Yv[0];
                Y[(row0 + g) * kOut + 1] = Yv[1];
            }
            if (row0 + g + 8 < n) {
                Y[(row0 + g + 8) * kOut] = Yv[2];
                Y[(row0 + g + 8) * kOut + 1] = Yv[3];
            }
        }
        __syncwarp();
    }
}

__global__ void k_gather_samples(const float *X, const float *T, const int32_t *perm, int64_t n, float *Xp, float *Tp) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = perm[i];
#pragma unroll
        for (int c = 0; c < kIn; ++c) Xp[i * kIn + c] = X[s * kIn + c];
        Tp[i * kOut] = T[s * kOut];
        Tp[i * kOut + 1] = T[s * kOut + 1];
    }
}

/* CTAs for a gradient launch over `tiles` 16-sample tiles: at least four tiles per warp */
unsigned grad_grid(int64_t tiles) {
    const int64_t per_cta = 4 * kWarps;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((tiles + per_cta - 1) / per_cta, 2 * 152));
}

/* ---- device buffers of one network (host helper) --------------------------------------------- */
struct Net {
    float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *w = nullptr, *wt = nullptr;
    double *loss = nullptr;
    int alloc() {
        if (cudaMalloc(&params, sizeof(float) * kNumParams) != cudaSuccess) return FJSPH_E_CUDA;
        if (cudaMalloc(&grad, sizeof(float) * kNumWeights) != cudaSuccess) return FJSPH_E_CUDA;
        if (cudaMalloc(&m, sizeof(float) * kNumWeights) != cudaSuccess) return FJSPH_E_CUDA;
        if (cudaMalloc(&v, sizeof(float) * kNumWeights) != cudaSuccess) return FJSPH_E_CUDA;
        if (cudaMalloc(&w, sizeof(__nv_bfloat16) * kNumBf16) != cudaSuccess) return FJSPH_E_CUDA;
        if (cudaMalloc(&wt, sizeof(__nv_bfloat16) * kNumBf16T) != cudaSuccess) return FJSPH_E_CUDA;
        if (cudaMalloc(&loss, sizeof(double)) != cudaSuccess) return FJSPH_E_CUDA;
        cudaMemset(grad, 0, sizeof(float) * kNumWeights);
        cudaMemset(m, 0, sizeof(float) * kNumWeights);
        cudaMemset(v, 0, sizeof(float) * kNumWeights);
        return FJSPH_OK;
    }
    void release() {
        cudaFree(params);
        cudaFree(grad);
        cudaFree(m);
        cudaFree(v);
        cudaFree(w);
        cudaFree(wt);
        cudaFree(loss);
    }
    DevMlp dev() const { return DevMlp{params, w, wt}; }
};

int grad_smem_setup() {
    const int bytes = (int)sizeof(CtaSmem);
    if (cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
        return FJSPH_E_CUDA;
    return FJSPH_OK;
}

} // namespace

/* exported to the context code: upload params (host) and cast */
int mlp_upload(const float *host_params, float *dparams, __nv_bfloat16 *dw, __nv_bfloat16 *dwt, cudaStream_t s) {
    if (cudaMemcpyAsync(dparams, host_params, sizeof(float) * kNumParams, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return FJSPH_E_CUDA;
    k_mlp_cast<<<16, 256, 0, s>>>(dparams, dw, dwt);
    return cudaGetLastError() == cudaSuccess ? FJSPH_OK : FJSPH_E_CUDA;
}

int mlp_num_bf16_t() { return kNumBf16T; }

} // namespace mlp
} // namespace fjsph

using namespace fjsph::mlp;

extern "C" int fjsph_mlp_num_params(void) { return kNumParams; }

extern "C" int fjsph_mlp_forward(const float *params, const float *X, int64_t n, float *Y) {
    if (!params || (n > 0 && (!X || !Y)) || n < 0) return FJSPH_E_ARG;
    Net net;
    int r = net.alloc();
    float *dX = nullptr, *dY = nullptr;
    if (r == FJSPH_OK && n > 0) {
        if (cudaMalloc(&dX, sizeof(float) * kIn * n) != cudaSuccess || cudaMalloc(&dY, sizeof(float) * kOut * n) != cudaSuccess)
            r = FJSPH_E_CUDA;
    }
    if (r == FJSPH_OK) r = mlp_upload(params, net.params, net.w, net.wt, 0);
    if (r == FJSPH_OK && n > 0) {
        cudaMemcpy(dX, X, sizeof(float) * kIn * n, cudaMemcpyHostToDevice);
        const int64_t tiles = (n + 15) / 16;
        const unsigned grid = (unsigned)std::min<int64_t>((tiles + kWarps - 1) / kWarps, 4096);
        k_mlp_infer<<<grid, 32 * kWarps>>>(net.dev(), dX, n, dY);
        if (cudaMemcpy(Y, dY, sizeof(float) * kOut * n, cudaMemcpyDeviceToHost) != cudaSuccess) r = FJSPH_E_CUDA;
    }
    cudaFree(dX);
    cudaFree(dY);
    net.release();
    return r;
}

extern "C" int fjsph_mlp_gradient(const float *params, const float *X, const float *T, int64_t n, float *grad,
                                  double *loss) {
    if (!params || !X || !T || !grad || n <= 0) return FJSPH_E_ARG;
    Net net;
    int r = net.alloc();
    float *dX = nullptr, *dT = nullptr;
    if (r == FJSPH_OK && (cudaMalloc(&dX, sizeof(float) * kIn * n) != cudaSuccess ||
                          cudaMalloc(&dT, sizeof(float) * kOut * n) != cudaSuccess))
        r = FJSPH_E_CUDA;
    if (r == FJSPH_OK) r = mlp_upload(params, net.params, net.w, net.wt, 0);
    if (r == FJSPH_OK) r = grad_smem_setup();
    if (r == FJSPH_OK) {
        cudaMemcpy(dX, X, sizeof(float) * kIn * n, cudaMemcpyHostToDevice);
        cudaMemcpy(dT, T, sizeof(float) * kOut * n, cudaMemcpyHostToDevice);
        cudaMemset(net.loss, 0, sizeof(double));
        k_mlp_grad<<<grad_grid((n + 15) / 16), 32 * kWarps, sizeof(CtaSmem)>>>(net.dev(), net.wt, dX, dT, n,
                                                                              1.f / (float)n, net.grad, net.loss);
        if (cudaMemcpy(grad, net.grad, sizeof(float) * kNumWeights, cudaMemcpyDeviceToHost) != cudaSuccess)
            r = FJSPH_E_CUDA;
        double l = 0.0;
        if (r == FJSPH_OK && cudaMemcpy(&l, net.loss, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
            r = FJSPH_E_CUDA;
        if (loss) *loss = l / (double)n;
    }
    cudaFree(dX);
    cudaFree(dT);
    net.release();
    return r;
}

extern "C" int fjsph_mlp_train(float *params, const float *X, const float *T, int64_t n, int32_t epochs,
                               int32_t batch, float lr, uint64_t seed, double *final_loss) {
    if (!params || !X || !T || n <= 0 || n >= ((int64_t)1 << 31) || epochs < 0 || batch < 16 || !(lr > 0.f))
        return FJSPH_E_ARG;
    Net net;
    int r = net.alloc();
    float *dX = nullptr, *dT = nullptr, *dXp = nullptr, *dTp = nullptr;
    int32_t *dperm = nullptr;
    if (r == FJSPH_OK && (cudaMalloc(&dX, sizeof(float) * kIn * n) != cudaSuccess ||
                          cudaMalloc(&dT, sizeof(float) * kOut * n) != cudaSuccess ||
                          cudaMalloc(&dXp, sizeof(float) * kIn * n) != cudaSuccess ||
                          cudaMalloc(&dTp, sizeof(float) * kOut * n) != cudaSuccess ||
                          cudaMalloc(&dperm, sizeof(int32_t) * n) != cudaSuccess))
        r = FJSPH_E_CUDA;
    if (r == FJSPH_OK) r = mlp_upload(params, net.params, net.w, net.wt, 0);
    if (r == FJSPH_OK) r = grad_smem_setup();
    if (r == FJSPH_OK && (cudaMemcpy(dX, X, sizeof(float) * kIn * n, cudaMemcpyHostToDevice) != cudaSuccess ||
                          cudaMemcpy(dT, T, sizeof(float) * kOut * n, cudaMemcpyHostToDevice) != cudaSuccess))
        r = FJSPH_E_CUDA;
    double last = 0.0;
    if (r == FJSPH_OK) {
        /* sample order: a seeded shuffle per epoch, applied on the device */
        std::vector<int32_t> perm(n);
        for (int64_t i = 0; i < n; ++i) perm[i] = (int32_t)i;
        std::mt19937_64 rng(seed);
        int step = 0;
        const int64_t nbatches = (n + batch - 1) / batch;
        const int64_t total = (int64_t)epochs * nbatches;
        for (int ep = 0; ep < epochs && r == FJSPH_OK; ++ep) {
            std::shuffle(perm.begin(), perm.end(), rng);
            if (cudaMemcpy(dperm, perm.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
                r = FJSPH_E_CUDA;
                break;
            }
            k_gather_samples<<<4 * 152, 256>>>(dX, dT, dperm, n, dXp, dTp);
            cudaMemset(net.loss, 0, sizeof(double));
            for (int64_t b0 = 0; b0 < n; b0 += batch) {
                const int64_t nb = std::min<int64_t>(batch, n - b0);
                k_mlp_grad<<<grad_grid((nb + 15) / 16), 32 * kWarps, sizeof(CtaSmem)>>>(
                    net.dev(), net.wt, dXp + b0 * kIn, dTp + b0 * kOut, nb, 1.f / (float)nb, net.grad, net.loss);
                /* cosine decay from lr to lr / 20 over all steps */
                const float prog = total > 1 ? (float)step / (float)(total - 1) : 1.f;
                const float lr_t = lr * (0.05f + 0.95f * 0.5f * (1.f + cosf(3.14159265f * prog)));
                ++step;
                k_adam<<<40, 256>>>(net.params, net.grad, net.m, net.v, step, lr_t, 0.9f, 0.999f, 1e-8f);
                k_mlp_cast<<<16, 256>>>(net.params, net.w, net.wt);
            }
            double l = 0.0;
            if (cudaMemcpy(&l, net.loss, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) r = FJSPH_E_CUDA;
            last = l / (double)n; /* mean loss of the epoch (weights moving during it) */
        }
        if (r == FJSPH_OK && cudaGetLastError() != cudaSuccess) r = FJSPH_E_CUDA;
        if (r == FJSPH_OK &&
            cudaMemcpy(params, net.params, sizeof(float) * kNumWeights, cudaMemcpyDeviceToHost) != cudaSuccess)
            r = FJSPH_E_CUDA;
    }
    if (final_loss) *final_loss = last;
    cudaFree(dX);
    cudaFree(dT);
    cudaFree(dXp);
    cudaFree(dTp);
    cudaFree(dperm);
    net.release();
    return r;
}
