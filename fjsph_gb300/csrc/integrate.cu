/*
 * integrate.cu -- pointwise stage updates of the Runge-Kutta and Newmark-Beta integrators, the
 * inlet buffer particles, and the FP64 reductions (error norms, CFL time-step bounds).
 *
 * The reference copies whole particle states per RK stage (src/Runge_Kutta.cpp:34,240,487-488).
 * Here a stage overwrites the working state in place and the RK4 weighted sums of velocity,
 * acceleration and density rate are carried in three running accumulators.  They add the stage
 * terms in the reference's order, ((a + 2b) + 2c) + d, and 2b is exact, so the sums round as the
 * reference's expressions do.
 */
#include "kernels.h"
#include "pack.cuh"

namespace fjsph {

namespace {

constexpr int kThreads = 256;
constexpr int kRedThreads = 256;

/* ---- boundary density / pressure updates --------------------------------------------------- */
/* mode 0: RK intermediate (src/Runge_Kutta.cpp:73-131); mode 1: RK final (:278-349);
 * mode 2: Newmark-Beta (src/Newmark_Beta.cpp:142-197).  In mode 0, sum_w (0, 2 or 1 for stages
 * 1, 2, 3) adds the stage's final boundary density rate to the RK4 sum. */
__global__ void k_bound_rho_update(Params P, DevState pn, DevState W, RKScratch S, int mode, double sum_w,
                                   const double *dt_dev, double dt_scale) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    const int solver = P.blocks[W.blk[i]].bound_solver;
    if (solver == FJSPH_PRESSURE_G) return;
    const double dt = dt_scale * dt_dev[grp_of(P, i)];
    double target;
    if (mode == 0) {
        target = pn.rho[i] + dt * W.Rrho[i];
    } else if (mode == 1) {
        target = pn.rho[i] + (dt / 6.0) * S.Sr[i];
    } else {
        target = pn.rho[i] + dt * (P.nb_gamma * W.Rrho[i] + (1 - P.nb_gamma) * pn.Rrho[i]);
    }
    if (solver == FJSPH_DBC || !S.near_inlet[i]) {
        const double rho = clamp_rho(P, P.rho_min, target);
        W.rho[i] = rho;
        W.p[i] = eos_pressure(P, rho);
        /* DBC final step: part_np1.Rrho = st_3.Rrho, which W already holds */
    } else { /* ghost wall next to the inlet: no negative pressure */
        const double rho = clamp_rho(P, P.rho_rest, target);
        W.rho[i] = rho;
        W.p[i] = eos_pressure(P, rho);
        W.Rrho[i] = fmax(0.0, W.Rrho[i]);
    }
    if (mode == 0 && sum_w != 0.0) S.Sr[i] = S.Sr[i] + sum_w * W.Rrho[i];
}

/* Sums at Runge_Kutta4 entry: st_1 = W, so
 *   Sv = pn.acc + 2 st1.acc,  Sr = pn.Rrho + 2 st1.Rrho,  Sx = (pn.v [+ pn.vPert]) + 2 (st1.v [+ vPert]).
 * Boundary slots carry Sr only (DBC / ghost final densities). */
template <int D>
__global__ void k_rk_init_sums(Params P, DevState pn, DevState W, RKScratch S) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    S.Sr[i] = pn.Rrho[i] + 2.0 * W.Rrho[i];
    if (i < P.nb) return;
    const bool ale = has(P, FJSPH_VAR_ALE);
#pragma unroll
    for (int k = 0; k < D; ++k) {
        S.Sv[k][i] = pn.acc[k][i] + 2.0 * W.acc[k][i];
        const double a = ale ? (pn.v[k][i] + pn.vPert[k][i]) : pn.v[k][i];
        const double b = ale ? (W.v[k][i] + W.vPert[k][i]) : W.v[k][i];
        S.Sx[k][i] = a + 2.0 * b;
    }
}

/* Fluid part of do_runge_kutta_intermediate_step (src/Runge_Kutta.cpp:142-172).  stage selects
 * how the RK4 sums advance:
 *   stage 1 (Get_First_RK): none; Runge_Kutta4 re-initialises them from st_1;
 *   stage 2: Sv += 2 f(st_1), Sr += 2 f(st_1), and after the update Sx += 2 (v_st2 [+ vPert]);
 *   stage 3: Sv += f(st_2), Sr += f(st_2); v_st3 enters Sx in the final step. */
template <int D>
__global__ void k_rk_stage_update(Params P, DevState pn, DevState W, RKScratch S, int stage, const double *dt_dev,
                                  double dt_scale, Packed K) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const bool ale = has(P, FJSPH_VAR_ALE);
    const double dt = dt_scale * dt_dev[grp_of(P, i)];
    const int b = W.b[i];
    if (stage >= 2) {
        const double w = (stage == 2) ? 2.0 : 1.0;
        S.Sr[i] = S.Sr[i] + w * W.Rrho[i];
#pragma unroll
        for (int k = 0; k < D; ++k) S.Sv[k][i] = S.Sv[k][i] + w * W.acc[k][i];
    }
    if (b > FJSPH_BUFFER) {
        double xn[D], vn[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double vv = ale ? (W.v[k][i] + W.vPert[k][i]) : W.v[k][i];
            xn[k] = pn.x[k][i] + dt * vv;
        }
#pragma unroll
        for (int k = 0; k < D; ++k) vn[k] = pn.v[k][i] + dt * W.acc[k][i];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            W.x[k][i] = xn[k];
            W.v[k][i] = vn[k];
        }
        const double rho = clamp_rho(P, P.rho_min, pn.rho[i] + dt * W.Rrho[i]);
        const double p = eos_pressure(P, rho);
        W.rho[i] = rho;
        W.p[i] = p;
        if (K.A) pack_moved<D>(P, W, K, i, xn, vn, rho, p); /* split-precision inputs of the new state */
    }
    if (stage == 2) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double v2 = ale ? (W.v[k][i] + W.vPert[k][i]) : W.v[k][i];
            S.Sx[k][i] = S.Sx[k][i] + 2.0 * v2;
        }
    }
}

/* Fluid part of do_runge_kutta_final_step (src/Runge_Kutta.cpp:357-394).  W holds st_3 with
 * acc = f(st_3); the sums already hold pn + 2 st_1 + 2 st_2 + st_3 for acc and Rrho. */
template <int D>
__global__ void k_rk_final_update(Params P, DevState pn, DevState W, RKScratch S, const double *dt_dev, Packed K) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const bool ale = has(P, FJSPH_VAR_ALE);
    const double dt = dt_dev[grp_of(P, i)];
    const int b = W.b[i];
    if (b > FJSPH_BUFFER && b != FJSPH_OUTLET) {
        double xn[D], vn[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double v3 = ale ? (W.v[k][i] + W.vPert[k][i]) : W.v[k][i];
            xn[k] = pn.x[k][i] + (dt / 6.0) * (S.Sx[k][i] + v3);
            vn[k] = pn.v[k][i] + (dt / 6.0) * S.Sv[k][i];
        }
#pragma unroll
        for (int k = 0; k < D; ++k) {
            W.x[k][i] = xn[k];
            W.v[k][i] = vn[k];
        }
        const double rho = clamp_rho(P, P.rho_min, pn.rho[i] + (dt / 6.0) * S.Sr[i]);
        const double p = eos_pressure(P, rho);
        W.rho[i] = rho;
        W.p[i] = p;
        if (K.A) pack_moved<D>(P, W, K, i, xn, vn, rho, p);
    } else if (b == FJSPH_OUTLET) {
#pragma unroll
        for (int k = 0; k < D; ++k) W.x[k][i] = pn.x[k][i] + dt * W.v[k][i];
        if (K.A) pack_particle<D>(P, W, K, i);
    }
}

/* Fluid part of Newmark_Beta::Do_NB_Iter (src/Newmark_Beta.cpp:199-240). */
template <int D>
__global__ void k_nb_update(Params P, DevState pn, DevState W, const double *dt_dev) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const bool ale = has(P, FJSPH_VAR_ALE);
    const double dt = dt_dev[grp_of(P, i)], dt2 = dt * dt;
    const double g1 = P.nb_gamma, g2 = 1 - g1, b1 = P.nb_beta, b2 = 0.5 * (1 - 2 * b1);
    const int b = W.b[i];
    if (b > FJSPH_BUFFER && b != FJSPH_OUTLET) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double an = pn.acc[k][i], a1 = W.acc[k][i];
            if (ale)
                W.x[k][i] = pn.x[k][i] + dt * (pn.v[k][i] + W.vPert[k][i]) + dt2 * (b1 * a1 + b2 * an);
            else
                W.x[k][i] = pn.x[k][i] + dt * pn.v[k][i] + dt2 * (b2 * an + b1 * a1);
            W.v[k][i] = pn.v[k][i] + dt * (g1 * a1 + g2 * an);
        }
        const double rho = clamp_rho(P, P.rho_min, pn.rho[i] + dt * (g1 * W.Rrho[i] + g2 * pn.Rrho[i]));
        W.rho[i] = rho;
        W.p[i] = eos_pressure(P, rho);
    } else if (b == FJSPH_OUTLET) {
#pragma unroll
        for (int k = 0; k < D; ++k) W.x[k][i] = pn.x[k][i] + dt * W.v[k][i];
    }
}

/* Inlet buffer particles (src/Runge_Kutta.cpp:175-228, :397-452; src/Newmark_Beta.cpp:243-297).
 * One thread per back particle walks its buffer column. */
template <int D>
__global__ void k_inlet_buffers(Params P, DevState pn, DevState W, RKScratch S, DevInlet I, int mode,
                                const double *dt_dev, double dt_scale, Packed K) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= I.n_back) return;
    const double dt = dt_scale * (*dt_dev);
    if (I.fixed_vel_or_dynamic == 1) {
        const int64_t back = I.back[c];
        for (int64_t jj = 0; jj < I.depth; ++jj) {
            const int64_t bid = I.buffer[c * I.depth + jj];
#pragma unroll
            for (int k = 0; k < D; ++k) {
                W.x[k][bid] = W.x[k][back] - P.dx * (jj + 1.0) * I.unorm[k];
                W.v[k][bid] = W.v[k][back];
            }
            W.rho[bid] = W.rho[back];
            W.p[bid] = W.p[back];
            if (K.A) pack_slot<D>(P, W, K, bid); /* the split-precision inputs of the moved particle */
        }
    } else {
        for (int64_t jj = 0; jj < I.depth; ++jj) {
            const int64_t bid = I.buffer[c * I.depth + jj];
            double target;
            if (mode == 0)
                target = pn.rho[bid] + dt * W.Rrho[bid];
            else if (mode == 1) /* S.Sr holds pn + 2 st_1 + 2 st_2 + st_3 */
                target = pn.rho[bid] + (dt / 6.0) * S.Sr[bid];
            else
                target = pn.rho[bid] + dt * (P.nb_gamma * W.Rrho[bid] + (1 - P.nb_gamma) * pn.Rrho[bid]);
            const double rho = clamp_rho(P, P.rho_min, target);
            W.rho[bid] = rho;
            W.p[bid] = eos_pressure(P, rho);
#pragma unroll
            for (int k = 0; k < D; ++k) W.x[k][bid] = pn.x[k][bid] + dt * pn.v[k][bid];
            if (K.A) pack_slot<D>(P, W, K, bid);
        }
    }
}

/* update_data's zero-density guard (src/Integration.cpp:116-124). */
template <int D>
__global__ void k_density_guard(Params P, DevState W, Packed K) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    if (W.rho[i] < 0.0001) {
        W.rho[i] = P.rho_rest;
        if (K.A) pack_slot<D>(P, W, K, i); /* the split-precision inputs of the reset particle */
    }
}

/* ---- reductions ------------------------------------------------------------------------------- */
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

/* Block-wide reduction of NV values; op[k] = 0 sum, 1 max, 2 min.  Thread 0 writes part[blk*NV+k]. */
template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], const int (&op)[NV], double *part) {
    __shared__ double sh[NV][kRedThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double t = op[k] == 0 ? warp_sum(v[k]) : (op[k] == 1 ? warp_max(v[k]) : warp_min(v[k]));
        if (lane == 0) sh[k][wid] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = sh[k][0];
            for (int w = 1; w < kRedThreads / 32; ++w)
                t = op[k] == 0 ? t + sh[k][w] : (op[k] == 1 ? fmax(t, sh[k][w]) : fmin(t, sh[k][w]));
            part[blockIdx.x * NV + k] = t;
        }
    }
}

template <int NV>
__global__ void k_finish(const double *part, int64_t nblk, double init0, int opsel, double *out) {
    /* single block: reduce nblk partial rows of NV values in a fixed order (strided per thread,
     * then across the warp, then across the warps) */
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; ++k) {
        const int op = (opsel >> (2 * k)) & 3;
        double t = op == 0 ? 0.0 : (op == 1 ? -INFINITY : INFINITY);
        for (int64_t b = threadIdx.x; b < nblk; b += blockDim.x) {
            const double x = part[b * NV + k];
            t = op == 0 ? t + x : (op == 1 ? fmax(t, x) : fmin(t, x));
        }
        t = op == 0 ? warp_sum(t) : (op == 1 ? warp_max(t) : warp_min(t));
        if (lane == 0) sh[k][wid] = t;
    }
    __syncthreads();
    if ((int)threadIdx.x < NV) {
        const int k = threadIdx.x;
        const int op = (opsel >> (2 * k)) & 3;
        double t = sh[k][0];
        for (int w = 1; w < nw; ++w) t = op == 0 ? t + sh[k][w] : (op == 1 ? fmax(t, sh[k][w]) : fmin(t, sh[k][w]));
        out[k] = t;
    }
    (void)init0;
}

__global__ void k_sum(const double *in, int64_t n, double *part) {
    double v[1] = {0.0};
    const int op[1] = {0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[0] += in[i];
    block_reduce<1>(v, op, part);
}

template <int D>
__global__ void k_sq_disp(Params P, DevState W, const double *r0, const double *r1, const double *r2, double *part) {
    const double *const ref[3] = {r0, r1, r2};
    double v[1] = {0.0};
    const int op[1] = {0};
    for (int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double d = W.x[k][i] - ref[k][i];
            s += d * d;
        }
        v[0] += s;
    }
    block_reduce<1>(v, op, part);
}

/* find_timestep reductions (src/Integration.cpp:384-402).  Norms and the surface-tension
 * bound enter as the squares / the square-root arguments they are taken of: the square root is
 * monotonic and correctly rounded, so the root of the extreme argument is the extreme root,
 * bit for bit, for one square root per search instead of five per particle
 * (timestep_maxima applies them). */
template <int D>
__global__ void k_timestep(Params P, DevState W, double *part) {
    const bool ale = has(P, FJSPH_VAR_ALE);
    double v[7] = {0.0, 0.0, kEps, kEps, INFINITY, 0.0, 0.0};
    const int op[7] = {1, 1, 1, 1, 2, 1, 1};
    for (int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double a[D], af[D], vv[D];
        load3<D>(W.acc, i, a);
        load3<D>(W.Af, i, af);
        load3<D>(W.v, i, vv);
        v[0] = fmax(v[0], dot<D, double>(a, a));
        v[1] = fmax(v[1], dot<D, double>(af, af));
        v[2] = fmax(v[2], fabs(W.Rrho[i]));
        const double rho = W.rho[i];
        v[3] = fmax(v[3], fabs(rho - P.rho_rest));
        v[4] = fmin(v[4], rho * P.dx * P.dx / (2.0 * kPi * P.sig * fabs(W.curve[i])));
        v[5] = fmax(v[5], dot<D, double>(vv, vv));
        if (ale) {
            double vp[D];
            load3<D>(W.vPert, i, vp);
            v[6] = fmax(v[6], dot<D, double>(vp, vp));
        }
    }
    block_reduce<7>(v, op, part);
}

inline unsigned red_grid(int64_t n, int64_t part_len, int nv) {
    int64_t g = (n + kRedThreads - 1) / kRedThreads;
    if (g > 1216) g = 1216; /* 8 blocks per SM on 152 SMs */
    if (g * nv > part_len) g = part_len / nv;
    if (g < 1) g = 1;
    return (unsigned)g;
}

} // namespace

#define FJSPH_DISPATCH2(D_, KERNEL, GRID, BLOCK, ...)                                   \
    do {                                                                                \
        if ((GRID) == 0) break;                                                         \
        if ((D_) == 2)                                                                  \
            KERNEL<2><<<(GRID), (BLOCK), 0, s>>>(__VA_ARGS__);                          \
        else                                                                            \
            KERNEL<3><<<(GRID), (BLOCK), 0, s>>>(__VA_ARGS__);                          \
    } while (0)

void launch_bound_rho_update(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S, int mode,
                             double sum_w, const double *dt_dev, double dt_scale, cudaStream_t s) {
    const unsigned g = grid_for(P.nb, kThreads);
    if (g) k_bound_rho_update<<<g, kThreads, 0, s>>>(P, pn, W, S, mode, sum_w, dt_dev, dt_scale);
}
void launch_rk_init_sums(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S, cudaStream_t s) {
    FJSPH_DISPATCH2(P.D, k_rk_init_sums, grid_for(P.n, kThreads), kThreads, P, pn, W, S);
}
void launch_rk_stage_update(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S, int stage,
                            const double *dt_dev, double dt_scale, const Packed *K, cudaStream_t s) {
    const Packed none{};
    FJSPH_DISPATCH2(P.D, k_rk_stage_update, grid_for(P.n - P.nb, kThreads), kThreads, P, pn, W, S, stage, dt_dev,
                    dt_scale, K ? *K : none);
}
void launch_rk_final_update(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S,
                            const double *dt_dev, const Packed *K, cudaStream_t s) {
    const Packed none{};
    FJSPH_DISPATCH2(P.D, k_rk_final_update, grid_for(P.n - P.nb, kThreads), kThreads, P, pn, W, S, dt_dev,
                    K ? *K : none);
}
void launch_nb_update(const Params &P, const DevState &pn, const DevState &W, const double *dt_dev, cudaStream_t s) {
    FJSPH_DISPATCH2(P.D, k_nb_update, grid_for(P.n - P.nb, kThreads), kThreads, P, pn, W, dt_dev);
}
void launch_inlet_buffers(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S,
                          const DevInlet &I, int mode, const double *dt_dev, double dt_scale, const Packed *K,
                          cudaStream_t s) {
    const Packed none{};
    FJSPH_DISPATCH2(P.D, k_inlet_buffers, grid_for(I.n_back, 64), 64, P, pn, W, S, I, mode, dt_dev, dt_scale,
                    K ? *K : none);
}
void launch_density_guard(const Params &P, const DevState &W, const Packed *K, cudaStream_t s) {
    const Packed none{};
    FJSPH_DISPATCH2(P.D, k_density_guard, grid_for(P.n - P.nb, kThreads), kThreads, P, W, K ? *K : none);
}
void launch_sum(const double *in, int64_t n, double *part, int64_t part_len, double *out, cudaStream_t s) {
    const unsigned g = red_grid(n, part_len, 1);
    k_sum<<<g, kRedThreads, 0, s>>>(in, n, part);
    k_finish<1><<<1, kRedThreads, 0, s>>>(part, g, 0.0, 0, out);
}
void launch_sq_disp_sum(const Params &P, const DevState &W, double *const ref[3], RKScratch &S, double *out,
                        cudaStream_t s) {
    const unsigned g = red_grid(P.n - P.nb, S.part_len, 1);
    FJSPH_DISPATCH2(P.D, k_sq_disp, g, kRedThreads, P, W, ref[0], ref[1], ref[2], S.part);
    k_finish<1><<<1, kRedThreads, 0, s>>>(S.part, g, 0.0, 0, out);
}
void timestep_maxima(const double *red, double *r) {
    r[0] = std::max(kEps, std::sqrt(red[0]));
    r[1] = std::max(kEps, std::sqrt(red[1]));
    r[2] = red[2];
    r[3] = red[3];
    r[4] = std::min(9999999.0, std::sqrt(red[4]));
    r[5] = std::max(kEps, std::sqrt(red[5]));
    r[6] = std::sqrt(red[6]);
}

void launch_timestep_reduce(const Params &P, const DevState &W, RKScratch &S, double *out, cudaStream_t s) {
    const unsigned g = red_grid(P.n - P.nb, S.part_len, 7);
    FJSPH_DISPATCH2(P.D, k_timestep, g, kRedThreads, P, W, S.part);
    /* ops: max,max,max,max,min,max,max -> 2 bits each */
    const int opsel = (1 << 0) | (1 << 2) | (1 << 4) | (1 << 6) | (2 << 8) | (1 << 10) | (1 << 12);
    k_finish<7><<<1, 128, 0, s>>>(S.part, g, 0.0, opsel, out);
}

} // namespace fjsph
