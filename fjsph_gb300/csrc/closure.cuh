/*
 * closure.cuh -- the learned stand-in for the Gissler occlusion and drag-coefficient closure
 * (src/Aero.h:37-98, occlusion factor src/Geometry.cpp:233-255), evaluated inside the residual
 * kernel of the split-precision form.
 *
 * Per particle the network maps 12 inputs to 2 outputs:
 *   inputs  0  sum_j w_j max(c_j, 0)     c_j = -(x_j - x_i).V / (|V| r_ij): cosine between the
 *           1  sum_j w_j max(-c_j, 0)    neighbour direction and the upwind direction, V = v_inf - v_i
 *           2  sum_j w_j c_j^2           as in the occlusion test; w_j = vol_j W(r_ij)
 *           3  max(0, max_j c_j)         the plain closure's occlusion statistic before clamping
 *           4  neighbour count / n_full
 *           5  log10(1 + |U|)            U = cellV - v at the stage (relative air velocity)
 *           6  log10(1 + We)             We = rho_air |U|^2 L / sigma (0 without surface tension)
 *           7  log10(1 + Re)             Re = 2 rho_air |U| L / mu_air
 *           8  |n|                       surface normal
 *           9  n.U / |U|
 *          10  lambda_nb
 *          11  lambda
 *   outputs 0  log10(Cd_i A_i / A_sphere) drag coefficient x un-occluded area, sphere-referenced
 *           1  woccl                     occlusion factor (clamped to [0, 1] on use)
 * and the force is the plain closure's  a = |U| U / (2 sos^2) gamma p_air Cd_i A_i (1 - woccl) / m.
 * Inputs 0-3 come from the surface-curvature pass (which already walks the neighbours for the
 * occlusion test); the others are read at the stage.  Particles past the lambda_nb cutoff keep
 * woccl = 1 (zero force) without the network, as in the plain closure.
 */
#pragma once

#include "aero.cuh"
#include "common.cuh"
#include "mlp.cuh"

namespace fjsph {

enum ClosureMode : int32_t { kClosurePlain = 0, kClosureLearned = 1, kClosureJudge = 2, kClosureLog = 3 };

struct Closure {
    int32_t mode;
    mlp::DevMlp M;
    const float4 *occ;             /* inputs 0-3 per slot (surface-curvature pass)           */
    double *judge;                 /* [3]: sum |a_l - a_p|^2, sum |a_p|^2, particles judged    */
    float *logX, *logT;            /* sample log: 12 inputs, 2 targets per sample              */
    unsigned long long *log_count; /* samples offered (may exceed log_cap)                    */
    int64_t log_cap;
};

/* Lane of the r-th set bit (r counted from 0, r < popc(bal)): the largest s with fewer than r + 1
 * set bits below it, found by binary search on popc. */
__device__ __forceinline__ int nth_set_lane(unsigned bal, int r) {
    int s = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
        if (__popc(bal & ((1u << (s + step)) - 1u)) <= r) s += step;
    return s;
}

/* The 12 network inputs of particle i (FP32; U = cellV - v, nneigh the neighbour count). */
template <int D>
__device__ __forceinline__ void closure_inputs(const Params &P, float4 occ, float nneigh, const float *U,
                                               float cellRho, float4 nrm, float lam, float (&x)[mlp::kIn]) {
    const FConst &c = P.fc;
    float U2 = 0.f;
#pragma unroll
    for (int k = 0; k < D; ++k) U2 += U[k] * U[k];
    const float Un = sqrtf(U2);
    x[0] = occ.x;
    x[1] = occ.y;
    x[2] = occ.z;
    x[3] = occ.w;
    x[4] = nneigh * c.i_n_full;
    x[5] = log10f(1.f + Un);
    x[6] = c.we_coef > 0.f ? log10f(1.f + cellRho * U2 * c.we_coef) : 0.f;
    x[7] = log10f(1.f + c.re_coef * cellRho * Un);
    const float n[3] = {nrm.x, nrm.y, nrm.z};
    float nn = 0.f, nu = 0.f;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        nn += n[k] * n[k];
        nu += n[k] * U[k];
    }
    x[8] = sqrtf(nn);
    x[9] = Un > 0.f ? nu / Un : 0.f;
    x[10] = nrm.w;
    x[11] = lam;
}

/* Network outputs for the lanes with `want` set; every lane of the warp must call.  The covered
 * lanes form the rows of 16-row tiles in lane order (row r is the lane of the r-th set bit of the
 * ballot; rows past the count are zero).  A lane builds its tile's input A fragment from the
 * source rows' packed inputs and takes its outputs from the C fragment by shuffles, so the network
 * holds no shared memory and the kernel's L1 keeps its whole capacity for the neighbour gathers. */
__device__ __forceinline__ void mlp_warp(const mlp::DevMlp &M, bool want, const float (&x)[mlp::kIn], float &y0,
                                         float &y1) {
    const unsigned bal = __ballot_sync(0xffffffffu, want);
    if (bal == 0u) return;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int cnt = __popc(bal);
    const int rank = __popc(bal & ((1u << lane) - 1u));
    /* this lane's normalised inputs as BF16 pairs: word q holds columns 2q (low half) and 2q + 1;
     * words 6 and 7 (columns 12-15) are the zero padding */
    uint32_t p[mlp::kIn / 2];
#pragma unroll
    for (int q = 0; q < mlp::kIn / 2; ++q) {
        p[q] = 0u;
        if (want) {
            const int c = 2 * q;
            p[q] = mlp::pack2((x[c] - __ldg(M.params + mlp::oInShift + c)) * __ldg(M.params + mlp::oInScale + c),
                              (x[c + 1] - __ldg(M.params + mlp::oInShift + c + 1)) *
                                  __ldg(M.params + mlp::oInScale + c + 1));
        }
    }
    for (int tile = 0; tile * 16 < cnt; ++tile) {
        const int r0 = tile * 16 + g, r1 = r0 + 8;
        const int s0 = r0 < cnt ? nth_set_lane(bal, r0) : lane;
        const int s1 = r1 < cnt ? nth_set_lane(bal, r1) : lane;
        /* A fragment: reg0 = row r0 word t, reg1 = row r1 word t, reg2 = row r0 word t + 4,
         * reg3 = row r1 word t + 4 */
        uint32_t A[1][4] = {{0u, 0u, 0u, 0u}};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t a0 = __shfl_sync(0xffffffffu, p[q], s0);
            const uint32_t a1 = __shfl_sync(0xffffffffu, p[q], s1);
            if (q == t) {
                A[0][0] = a0;
                A[0][1] = a1;
            }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) { /* words 4 and 5; 6 and 7 stay zero */
            const uint32_t a2 = __shfl_sync(0xffffffffu, p[q + 4], s0);
            const uint32_t a3 = __shfl_sync(0xffffffffu, p[q + 4], s1);
            if (q == t) {
                A[0][2] = a2;
                A[0][3] = a3;
            }
        }
        if (r0 >= cnt) A[0][0] = A[0][2] = 0u;
        if (r1 >= cnt) A[0][1] = A[0][3] = 0u;
        float Y[4];
        mlp::forward_frag(M, A, Y);
        /* row rr of this tile: outputs in lane 4 (rr % 8), Y[0..1] for rr < 8, Y[2..3] above */
        const int rr = rank - tile * 16;
        const int src = 4 * (rr & 7);
        const float v0 = __shfl_sync(0xffffffffu, Y[0], src), v1 = __shfl_sync(0xffffffffu, Y[1], src);
        const float v2 = __shfl_sync(0xffffffffu, Y[2], src), v3 = __shfl_sync(0xffffffffu, Y[3], src);
        if (want && rr >= 0 && rr < 16) {
            y0 = rr < 8 ? v0 : v2;
            y1 = rr < 8 ? v1 : v3;
        }
    }
}

/* Aerodynamic acceleration of a live, aero-active particle from the closure outputs (FP32,
 * U = cellV - v). */
template <int D>
__device__ __forceinline__ void learned_acc(const Params &P, const DevState &W, int64_t i, const float *U, float y0,
                                            float y1, double *out) {
    float U2 = 0.f;
#pragma unroll
    for (int k = 0; k < D; ++k) U2 += U[k] * U[k];
    const float Un = sqrtf(U2);
    const float CdA = exp10f(y0) * P.fc.A_sphere;
    const float wo = fminf(fmaxf(y1, 0.f), 1.f);
    const float tail = P.fc.force_coef * to_f32(W.cellP[i]) * CdA * (1.f - wo) / to_f32(W.m[i]);
    const float cc = 0.5f * Un * tail;
#pragma unroll
    for (int k = 0; k < D; ++k) out[k] = to_f64(cc * U[k]);
}

/* The plain closure in the split-precision form: Gissler's in FP32 (gissler_acc_f32), the other
 * closures in FP64 (aero_acc).  A fully occluded particle (woccl exactly 1) gets no force, as in
 * aero_acc. */
template <int D>
__device__ __forceinline__ void plain_acc(const Params &P, const DevState &W, int64_t i, const float *U,
                                          double nneigh, double *out) {
    if (P.acase != FJSPH_GISSLER) {
        double Ud[D];
#pragma unroll
        for (int k = 0; k < D; ++k) Ud[k] = W.cellV[k][i] - W.v[k][i];
        aero_acc<D>(P, W, i, Ud, W.lam_nb[i], nneigh, out);
        return;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) out[k] = 0.0;
    bool finite = true;
#pragma unroll
    for (int k = 0; k < D; ++k) finite = finite && isfinite(U[k]);
    const double wo = W.woccl[i];
    if (__double_as_longlong(wo) == __double_as_longlong(1.0) && finite) return;
    float o[3];
    gissler_acc_f32<D>(P, U, to_f32(W.cellRho[i]), to_f32(W.cellP[i]), to_f32(1.0 - wo), to_f32(W.m[i]),
                       to_f32(W.lam_nb[i]), to_f32(nneigh), o);
#pragma unroll
    for (int k = 0; k < D; ++k) out[k] = to_f64(o[k]);
}

/* The aerodynamic term of the residual for particle i under the closure mode.  All lanes of the
 * warp call (the network runs on whole warps); lanes with live == false contribute nothing.
 * Not inlined: the residual's register allocation then does not absorb the network's. */
template <int D>
__device__ __noinline__ void closure_aero(const Params &P, const DevState &W, const Closure &C, const float4 *Kn,
                                             const float4 *Kg, int64_t i, bool live, double nneigh, bool &aero_on,
                                             double *aero) {
#pragma unroll
    for (int k = 0; k < D; ++k) aero[k] = 0.0;
    aero_on = live && W.cellID[i] != -1;
    /* relative air velocity in FP32, from the integer FP64 -> FP32 roundings */
    float U[3] = {0.f, 0.f, 0.f};
    if (aero_on) {
#pragma unroll
        for (int k = 0; k < D; ++k) U[k] = to_f32(W.cellV[k][i]) - to_f32(W.v[k][i]);
    }
    if (C.mode == kClosurePlain) {
        if (aero_on) plain_acc<D>(P, W, i, U, nneigh, aero);
        return;
    }
    /* the network covers the particles whose occlusion factor is not fixed at 1 by lambda_nb */
    const bool want = aero_on && to_f32(W.lam_nb[i]) < to_f32(P.lam_cutoff);
    float x[mlp::kIn];
    if (want) closure_inputs<D>(P, C.occ[i], to_f32(nneigh), U, to_f32(W.cellRho[i]), Kn[i], Kg[i].w, x);
    if (C.mode == kClosureLog) {
        if (aero_on) plain_acc<D>(P, W, i, U, nneigh, aero);
        const unsigned bal = __ballot_sync(0xffffffffu, want);
        if (bal == 0u) return;
        const int lane = threadIdx.x & 31;
        unsigned long long base = 0;
        if (lane == __ffs(bal) - 1) base = atomicAdd(C.log_count, (unsigned long long)__popc(bal));
        base = __shfl_sync(0xffffffffu, base, __ffs(bal) - 1);
        if (want) {
            const unsigned long long slot = base + (unsigned long long)__popc(bal & ((1u << lane) - 1u));
            if (slot < (unsigned long long)C.log_cap) {
                /* the targets: the plain closure's own coefficients (FP64) */
                double Ud[D], Cdi, Aun;
#pragma unroll
                for (int k = 0; k < D; ++k) Ud[k] = W.cellV[k][i] - W.v[k][i];
                const double Un = vnorm<D, double>(Ud);
                gissler_coeff<D>(P, W.cellRho[i], Un, dot<D, double>(Ud, Ud), W.lam_nb[i], nneigh, Cdi, Aun);
#pragma unroll
                for (int c = 0; c < mlp::kIn; ++c) C.logX[slot * mlp::kIn + c] = x[c];
                C.logT[slot * 2] = (float)log10(Cdi * Aun / P.A_sphere);
                C.logT[slot * 2 + 1] = (float)W.woccl[i];
            }
        }
        return;
    }
    float y0 = 0.f, y1 = 0.f;
    mlp_warp(C.M, want, x, y0, y1);
    if (want)
        learned_acc<D>(P, W, i, U, y0, y1, aero);
    else if (aero_on)
        plain_acc<D>(P, W, i, U, nneigh, aero);
    if (C.mode == kClosureJudge) {
        double d2 = 0.0, p2 = 0.0, cnt = 0.0;
        if (want) {
            /* the reference: the plain closure in FP64 */
            double ref[D], Ud[D];
#pragma unroll
            for (int k = 0; k < D; ++k) Ud[k] = W.cellV[k][i] - W.v[k][i];
            aero_acc<D>(P, W, i, Ud, W.lam_nb[i], nneigh, ref);
#pragma unroll
            for (int k = 0; k < D; ++k) {
                d2 += (aero[k] - ref[k]) * (aero[k] - ref[k]);
                p2 += ref[k] * ref[k];
            }
            cnt = 1.0;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            d2 += __shfl_xor_sync(0xffffffffu, d2, o);
            p2 += __shfl_xor_sync(0xffffffffu, p2, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if ((threadIdx.x & 31) == 0 && cnt > 0.0) {
            atomicAdd(&C.judge[0], d2);
            atomicAdd(&C.judge[1], p2);
            atomicAdd(&C.judge[2], cnt);
        }
    }
}

} // namespace fjsph
