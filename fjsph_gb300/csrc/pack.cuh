/*
 * pack.cuh -- the FP32 split-precision inputs of one particle, packed from its FP64 state
 * (shared by the packing pass and the integrator's stage updates, which write them as they
 * produce the new state).
 */
#pragma once

#include <cuda_bf16.h>

#include "kernels.h"
#include "split.cuh"

namespace fjsph {

/* Two bf16 (round to nearest even) in one 32-bit word, the first in the low half. */
__device__ __forceinline__ float pack_bf16x2(float a, float b) {
    const uint32_t lo = __bfloat16_as_ushort(__float2bfloat16_rn(a));
    const uint32_t hi = __bfloat16_as_ushort(__float2bfloat16_rn(b));
    return __uint_as_float(lo | (hi << 16));
}
constexpr uint32_t kLoBound = 1u, kLoFluid = 2u;
/* the residual's compact inputs (Packed::Lo) */
__device__ __forceinline__ float4 pack_lo(const float *xl, const float *vl, float pr, int bits) {
    const int b = bits & 7;
    const uint32_t flags = (b == FJSPH_BOUND ? kLoBound : 0u) | (b > FJSPH_PISTON ? kLoFluid : 0u);
    return make_float4(pack_bf16x2(xl[0], xl[1]), pack_bf16x2(xl[2], vl[0]), pack_bf16x2(vl[1], vl[2]),
                       __uint_as_float((__float_as_uint(pr) & ~3u) | flags));
}

/* A = (fl32(x), vol), C = (fl32(v), rho - rho0), R = rho - rho0, F = (vPert, p),
 * Lo = (bf16 of x - fl32(x) and v - fl32(v), p / rho^2 with type flags), bits.  vol and
 * p / rho^2 are FP32 quotients of the FP32-rounded operands (an FP64 divide per particle costs
 * more than the pass's memory traffic on this GPU); rounded to nearest in every translation
 * unit.  The FP64 -> FP32
 * roundings run in integer arithmetic (split.cuh), bit-identical to the conversions. */
template <int D>
__device__ __forceinline__ void pack_particle(const Params &P, const DevState &W, const Packed &K, int64_t i) {
    float xh[3] = {0, 0, 0}, xl[3] = {0, 0, 0}, vh[3] = {0, 0, 0}, vl[3] = {0, 0, 0}, vp[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < D; ++k) {
        split_f32(W.x[k][i], xh[k], xl[k]);
        split_f32(W.v[k][i], vh[k], vl[k]);
        vp[k] = to_f32(W.vPert[k][i]);
    }
    const double rho = W.rho[i], p = W.p[i];
    const float rf = to_f32(rho), pf = to_f32(p);
    const float pr = __fdiv_rn(pf, rf * rf);
    const float dr = to_f32(rho - P.rho_rest);
    K.A[i] = make_float4(xh[0], xh[1], xh[2], __fdiv_rn(to_f32(W.m[i]), rf));
    K.C[i] = make_float4(vh[0], vh[1], vh[2], dr);
    K.R[i] = dr;
    const int bits = (W.b[i] & 7) | ((W.surf[i] & 1) << 3) | ((W.surfzone[i] & 1) << 4);
    K.F[i] = make_float4(vp[0], vp[1], vp[2], pf);
    K.Lo[i] = pack_lo(xl, vl, pr, bits);
    K.bits[i] = bits;
}

/* The same inputs from a freshly integrated state held in registers (x, v, rho, p); mass,
 * perturbation velocity and flags are unchanged by an integration stage and are taken from the
 * current packed arrays. */
template <int D>
__device__ __forceinline__ void pack_moved(const Params &P, const DevState &W, const Packed &K, int64_t i,
                                           const double *x, const double *v, double rho, double p) {
    float xh[3] = {0, 0, 0}, xl[3] = {0, 0, 0}, vh[3] = {0, 0, 0}, vl[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < D; ++k) {
        split_f32(x[k], xh[k], xl[k]);
        split_f32(v[k], vh[k], vl[k]);
    }
    const float rf = to_f32(rho), pf = to_f32(p);
    const float pr = __fdiv_rn(pf, rf * rf);
    const int bits = K.bits[i];
    const float dr = to_f32(rho - P.rho_rest);
    K.A[i] = make_float4(xh[0], xh[1], xh[2], __fdiv_rn(to_f32(W.m[i]), rf));
    K.C[i] = make_float4(vh[0], vh[1], vh[2], dr);
    K.R[i] = dr;
    reinterpret_cast<float *>(K.F + i)[3] = pf;
    K.Lo[i] = pack_lo(xl, vl, pr, bits);
}

/* pack_moved of slot i from its current x, v, rho and p in W */
template <int D>
__device__ __forceinline__ void pack_slot(const Params &P, const DevState &W, const Packed &K, int64_t i) {
    double x[3] = {0, 0, 0}, v[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < D; ++k) {
        x[k] = W.x[k][i];
        v[k] = W.v[k][i];
    }
    pack_moved<D>(P, W, K, i, x, v, W.rho[i], W.p[i]);
}

} // namespace fjsph
