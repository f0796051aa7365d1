/*
 * groups.cu -- independent simulations in one context (the batched-droplet workload): the
 * per-simulation reductions and scalar updates that a single simulation does on the host.
 *
 * Every slot carries its group (simulation) id; per-group scalars live in device arrays, so a
 * whole step of all groups is enqueued without a host round trip and can be captured in one
 * CUDA graph.  What each group computes is exactly what a context holding that simulation alone
 * computes: its own npd (src/Shifting.cpp:116-119), its own CFL time step
 * (src/Integration.cpp:370-443), its own Runge-Kutta error norm (src/Runge_Kutta.cpp:17-23) and
 * its own adaptive CFL (src/Integration.cpp:270-300).  Group sums use atomics, so they differ
 * from a single simulation's two-pass sums by FP64 rounding only.
 */
#include "kernels.h"

namespace fjsph {

namespace {

constexpr int kT = 256;

/* warp-aggregated atomic add of v into out[g]: lanes holding the same group combine first */
__device__ __forceinline__ void group_add(double *out, int32_t g, double v, bool active) {
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!active) return;
    const unsigned peers = __match_any_sync(act, g);
    const int leader = __ffs(peers) - 1;
    const int lane = threadIdx.x & 31;
    /* sum over peers in lane order */
    double s = 0.0;
    for (unsigned m = peers; m; m &= m - 1) {
        const int l = __ffs(m) - 1;
        const double x = __shfl_sync(peers, v, l);
        s += x;
    }
    if (lane == leader) atomicAdd(&out[g], s);
}

/* max / min of non-negative doubles through their bit patterns (monotonic for v >= 0); NaN is
 * skipped, as fmax / fmin skip it in the single-simulation reduction */
__device__ __forceinline__ void atomic_max_nonneg(double *a, double v) {
    if (v >= 0.0) atomicMax(reinterpret_cast<unsigned long long *>(a), (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_min_nonneg(double *a, double v) {
    if (v >= 0.0) atomicMin(reinterpret_cast<unsigned long long *>(a), (unsigned long long)__double_as_longlong(v));
}

__global__ void k_group_fill(double *a, int64_t n, double v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

/* sum of vals[i] over slots [i0, i1) per group */
__global__ void k_group_sum(const int32_t *grp, const double *vals, int64_t i0, int64_t i1, double *out) {
    const int64_t i = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool on = i < i1;
    group_add(out, on ? grp[i] : 0, on ? vals[i] : 0.0, on);
}

/* sum over fluid slots of |W.x - ref|^2 per group */
template <int D>
__global__ void k_group_sq_disp(Params P, DevState W, const double *r0, const double *r1, const double *r2,
                                double *out) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool on = i < P.n;
    double e = 0.0;
    if (on) {
        const double *ref[3] = {r0, r1, r2};
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double d = W.x[k][i] - ref[k][i];
            e += d * d;
        }
    }
    group_add(out, on ? P.grp[i] : 0, e, on);
}

/* the seven maxima / minima of find_timestep per group; red[g * 8 + k] */
template <int D>
__global__ void k_group_timestep(Params P, DevState W, double *red) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const int32_t g = P.grp[i];
    double a[D], af[D], vv[D];
    load3<D>(W.acc, i, a);
    load3<D>(W.Af, i, af);
    load3<D>(W.v, i, vv);
    double *r = red + 8 * g;
    /* norms as their squares and the surface-tension bound as its square-root argument (the
     * roots are taken once per group in k_group_dt, as the single-simulation reduction does) */
    atomic_max_nonneg(&r[0], dot<D, double>(a, a));
    atomic_max_nonneg(&r[1], dot<D, double>(af, af));
    atomic_max_nonneg(&r[2], fabs(W.Rrho[i]));
    const double rho = W.rho[i];
    atomic_max_nonneg(&r[3], fabs(rho - P.rho_rest));
    atomic_min_nonneg(&r[4], rho * P.dx * P.dx / (2.0 * kPi * P.sig * fabs(W.curve[i])));
    atomic_max_nonneg(&r[5], dot<D, double>(vv, vv));
    if (has(P, FJSPH_VAR_ALE)) {
        double vp[D];
        load3<D>(W.vPert, i, vp);
        atomic_max_nonneg(&r[6], dot<D, double>(vp, vp));
    }
}

__global__ void k_group_red_init(double *red, int32_t G) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    double *r = red + 8 * g;
    r[0] = r[1] = r[5] = r[6] = r[7] = 0.0;
    r[2] = r[3] = kEps;
    r[4] = INFINITY;
}

/* dt per group from its maxima (the host tail of find_timestep) */
__global__ void k_group_dt(GroupDev G, const double *red, int32_t ng, GroupConst K) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const double *r = red + 8 * g;
    const double maxf = fmax(kEps, sqrt(r[0])), maxU = fmax(kEps, sqrt(r[5])), maxdrho = r[2], maxRhoi = r[3];
    const double minST = fmin(9999999.0, sqrt(r[4]));
    if (K.ale) G.maxShift[g] = fmax(G.maxShift[g], sqrt(r[6]));
    G.maxRho_pc[g] = 100 * maxRhoi / K.rho_rest;
    const double fac[6] = {0.25 * sqrt(K.H / maxf),         2 * K.H / maxU, 0.125 * K.H_sq * K.rho_rest / K.mu,
                           0.067 * minST, 0.5 * sqrt(K.H / maxdrho), 1.5 * K.H / K.speed_sound};
    double mn = fac[0];
    for (int k = 1; k < 6; ++k)
        if (fac[k] < mn) mn = fac[k];
    double dt = G.cfl[g] * (0.75 * mn);
    if (dt < K.dt_min)
        dt = K.dt_min;
    else if (dt > K.dt_max)
        dt = K.dt_max;
    if (dt > K.last_frame_time + K.frame_interval - G.time[g]) dt = K.last_frame_time + K.frame_interval - G.time[g] + K.dt_min;
    G.dt[g] = dt;
}

/* npd per group: kernel sums over the group's particles / its particle count */
__global__ void k_group_npd(double *npd, const double *sum, const int64_t *count, int32_t ng) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < ng) npd[g] = sum[g] / double(count[g]);
}

/* log10 RMS position change per group; mode 0: logbase, mode 1: error relative to logbase */
__global__ void k_group_err(GroupDev G, const double *sum, int32_t ng, int mode) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const double e = log10(sqrt(sum[g] / double(G.nfluid[g])));
    if (mode == 0)
        G.logbase[g] = e;
    else
        G.err[g] = e - G.logbase[g];
}

/* end of step: time and adaptive CFL (src/Integration.cpp:268-300; Runge-Kutta: iteration 0) */
__global__ void k_group_adapt(GroupDev G, int32_t ng, GroupConst K) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    G.time[g] += G.dt[g];
    double cfl = G.cfl[g];
    int nu = G.n_unstable[g], ns = G.n_stable[g];
    const double err = G.err[g];
    if (err > K.min_residual || G.maxRho_pc[g] > K.rho_max_iter) {
        if (err > 0.6 * K.min_residual) {
            cfl = fmax(K.cfl_min, cfl - K.cfl_step);
            nu = 0;
        } else if (nu > K.n_unstable_limit) {
            cfl = fmax(K.cfl_min, cfl - K.cfl_step);
            nu = 0;
        } else
            nu++;
    } else
        nu = 0;
    if (0 < K.subits_factor * K.max_subits && nu == 0) {
        if (ns > K.n_stable_limit) {
            cfl = fmin(K.cfl_max, cfl + K.cfl_step);
            ns = 0;
        } else
            ns++;
    } else
        ns = 0;
    G.cfl[g] = cfl;
    G.n_unstable[g] = nu;
    G.n_stable[g] = ns;
    G.steps[g] += 1;
}

} // namespace

void launch_group_fill(double *a, int64_t n, double v, cudaStream_t s) {
    if (n > 0) k_group_fill<<<grid_for(n, kT), kT, 0, s>>>(a, n, v);
}

void launch_group_sum(const int32_t *grp, const double *vals, int64_t i0, int64_t i1, double *out, cudaStream_t s) {
    if (i1 > i0) k_group_sum<<<grid_for(i1 - i0, kT), kT, 0, s>>>(grp, vals, i0, i1, out);
}

void launch_group_sq_disp(const Params &P, const DevState &W, double *const ref[3], double *out, cudaStream_t s) {
    const unsigned g = grid_for(P.n - P.nb, kT);
    if (g == 0) return;
    if (P.D == 2)
        k_group_sq_disp<2><<<g, kT, 0, s>>>(P, W, ref[0], ref[1], ref[2], out);
    else
        k_group_sq_disp<3><<<g, kT, 0, s>>>(P, W, ref[0], ref[1], ref[2], out);
}

void launch_group_timestep(const Params &P, const DevState &W, double *red, int32_t ng, cudaStream_t s) {
    k_group_red_init<<<grid_for(ng, 128), 128, 0, s>>>(red, ng);
    const unsigned g = grid_for(P.n - P.nb, kT);
    if (g == 0) return;
    if (P.D == 2)
        k_group_timestep<2><<<g, kT, 0, s>>>(P, W, red);
    else
        k_group_timestep<3><<<g, kT, 0, s>>>(P, W, red);
}

void launch_group_dt(const GroupDev &G, const double *red, int32_t ng, const GroupConst &K, cudaStream_t s) {
    k_group_dt<<<grid_for(ng, 128), 128, 0, s>>>(G, red, ng, K);
}

void launch_group_npd(double *npd, const double *sum, const int64_t *count, int32_t ng, cudaStream_t s) {
    k_group_npd<<<grid_for(ng, 128), 128, 0, s>>>(npd, sum, count, ng);
}

void launch_group_err(const GroupDev &G, const double *sum, int32_t ng, int mode, cudaStream_t s) {
    k_group_err<<<grid_for(ng, 128), 128, 0, s>>>(G, sum, ng, mode);
}

void launch_group_adapt(const GroupDev &G, int32_t ng, const GroupConst &K, cudaStream_t s) {
    k_group_adapt<<<grid_for(ng, 128), 128, 0, s>>>(G, ng, K);
}

} // namespace fjsph
