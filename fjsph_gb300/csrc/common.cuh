/*
 * common.cuh -- device-side layout and helpers shared by the GB300 WCSPH kernels.
 *
 * Particle state lives in HBM as structure-of-arrays: one array per scalar component, so that a
 * warp reading one field of 32 consecutive particles issues one 256-byte (FP64) transaction.
 * A context holds two full states, pn (time n) and W (the working state pnp1 of the reference),
 * plus the neighbour lists and the scratch arrays of the integrators.
 *
 * Particles are kept in "slot" order: boundary particles first (slots [0, nb)), then fluid
 * particles, each group sorted by grid cell at the last re-ordering.  Every slot carries its
 * reference ordinal (`key`), from which download restores the reference index order.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fjsph_gb300.h"

#define FJSPH_HD __host__ __device__ __forceinline__

namespace fjsph {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEps = 2.220446049250313080847e-16; /* numeric_limits<double>::epsilon() */
constexpr double kDefaultVal = 9999999.0;
constexpr int64_t kNoCell = -3;
/* cellID of a particle that left the mesh through its outer boundary (deleted with the step's
 * other deletions) */
constexpr int64_t kMeshLost = -4;
constexpr int kInletZone = 6;
constexpr int kMaxBlocks = 32;

/* One full particle state on the device (structure of arrays, capacity-sized). */
struct DevState {
    double *x[3], *v[3], *acc[3], *Af[3], *aVisc[3], *cellV[3], *gradRho[3], *norm[3], *vPert[3];
    double *L[9];
    double *Rrho, *rho, *p, *m, *curve, *norm_curve, *woccl, *pDist, *deltaD;
    double *cellP, *cellRho, *colourG, *colour, *lam, *lam_nb, *kernsum;
    int64_t *part_id, *cellID, *key;
    int32_t *b, *surf, *surfzone, *blk;
};

/* Block (LIMITS entry) data the kernels need. */
struct DevBlock {
    int32_t is_fluid, bound_solver, no_slip, block_type, fixed_vel_or_dynamic, n_times;
    double vel_rk[3], vel_nb[3]; /* boundary velocity at the current time, RK and NB rules */
    double aero_norm[3], aeroconst;
    double insert_unorm[3];
};

/* FP32 constants of the split-precision pair terms, converted once on the host. */
struct FConst {
    float H, H_sq, Wc, W_dx, rho0, Bgam, nu, alpha, dsph_cont, max_shift_vel;
    float grav[3];
    float pi3o4_H;   /* 3 pi / (4 H), pairwise surface tension  */
    float fac_bound; /* 1 + cos(7 pi / 18) / 2 (Kernel.h:88-113) */
    float pad;
    double st_coef;  /* sigma / (2 lambda) of the pairwise model: npdm2 = st_coef / npd^2 */
    /* the Gissler closure's constants for the split-precision form's FP32 evaluation */
    float re_coef;   /* 2 L / mu_air: Re = re_coef rho_air |U|        */
    float interp_fac, i_n_full, ycoef, L, CbL, A_sphere, A_plate;
    float force_coef; /* gamma_air / sos^2                              */
    float st_coef_f;  /* st_coef in FP32                                */
    float we_coef;    /* L / sigma (0 without surface tension): We = we_coef rho_air |U|^2 */
    float surf_h;     /* 1.33 dx, the surface test's offset (src/Geometry.cpp)       */
    float lam_cutoff; /* lambda_nb below which the occlusion factor is computed      */
};

/* Everything a kernel reads that is constant over one launch. */
struct Params {
    int32_t D;
    uint32_t variant;
    int32_t st_model, pressure_rel, acase, use_lam, use_TAB_def;
    double H, H_sq, sr, W_correc, W_dx, dx, particle_step;
    double rho_rest_inv; /* 1 / rho_rest: the equation of state multiplies (no FP64 divide) */
    double rho_rest, B, gam, speed_sound, press_back, rho_min, rho_max;
    double visc_alpha, mu, nu, sig, dsph_cont, max_shift_vel;
    double grav[3], v_inf[3];
    double L, A_sphere, A_plate, mu_g, sos, gamma_g, lam_cutoff, interp_fac, i_n_full, ycoef, Cb, rho_g;
    double nb_beta, nb_gamma;
    int64_t n, nb; /* total particles, boundary particles (slots [0, nb)) */
    int32_t nblocks;
    DevBlock blocks[kMaxBlocks];
    /* Independent simulations sharing the context (batched droplets): group of every slot and
     * each group's free-stream velocity; null for a single simulation.  Per-group dt and npd
     * are then arrays indexed by group. */
    const int32_t *grp;
    const double *g_vinf; /* 3 per group */
    /* air velocity per slot (3 per slot) when the air source is position dependent; null for
     * the uniform v_inf */
    const double *air_v;
    /* launch configuration of the split-precision pair sweeps (the autotuner's choices) */
    int32_t sweep_threads, resid_threads, list_ahead;
    /* SM-local work order of the residual (0 = grid order): warps claim 32-particle chunks from
     * per-SM regions through these counters (kMaxRegions, zeroed before each launch) */
    int32_t sm_order;
    int32_t *region_next;
    FConst fc;
    /* neighbour-search cell edges (support radius along x, radius / kCellDiv across) and their
     * reciprocals, so cell coordinates cost a multiply instead of an FP64 divide */
    double cell_edge[3], cell_inv[3];
};

/* Cells are the support radius long along x (the contiguous direction of a bucket row) and
 * radius / kCellDiv across it. */
#ifndef CELL_DIV_DEFAULT
#define CELL_DIV_DEFAULT 2
#endif
constexpr int kCellDiv = CELL_DIV_DEFAULT;

__device__ __forceinline__ int32_t grp_of(const Params &P, int64_t i) { return P.grp ? P.grp[i] : 0; }
__device__ __forceinline__ double vinf_of(const Params &P, int64_t i, int k) {
    if (P.air_v) return P.air_v[3 * i + k]; /* position-dependent source (vortex lattice) */
    return P.grp ? P.g_vinf[3 * P.grp[i] + k] : P.v_inf[k];
}

/* Neighbour lists plus the positions at search time (the reference keeps the squared distance
 * of each pair from search time, src/Resid.cpp:288).
 *  - FP64 form: CSR, off[n + 1] and idx (neighbour slots).
 *  - split-precision form: (slot, FP32 squared distance bits) pairs in sliced-ELL order with
 *    slices of kSlice = 32 consecutive slots and chunks of kChunk = 4 pairs per slot: pair k of
 *    slot i is entry slice[i / 32] + (k / 4) * 128 + (i % 32) * 4 + k % 4, and slot i has cnt[i]
 *    pairs.  A warp walking 32 slots' lists in step reads one 1 KB row every four pairs, and a
 *    lane writes its pairs as whole 32-byte sectors.  off is still filled (CSR offsets of the
 *    counts). */
constexpr int kSlice = 32;
constexpr int kChunk = 4;
struct DevNbr {
    const int64_t *off;
    const int32_t *idx;   /* FP64 form                                    */
    const int2 *pair;     /* split-precision form, sliced-ELL             */
    const int32_t *cnt;   /* split-precision form: pairs per slot         */
    const int64_t *slice; /* split-precision form: first entry per slice  */
    const double *xs[3];
};

/* SM-local work order of a particle sweep.  The sweep's 32-particle chunks are grouped in
 * super-chunks of kSuperChunk consecutive chunks, dealt round robin to one region per SM (%nsmid
 * regions, at most kMaxRegions): region r holds super-chunks r, r + R, r + 2R, ...  A warp takes
 * the region's next chunk of the SM it runs on, so the warps resident on an SM work on about
 * kSuperChunk * 32 consecutive particles and share their neighbours' records in L1, while all SMs
 * advance through the array together and share the rest in L2, as grid order does.  Once its
 * region is used up a warp takes a chunk of the next region that still has one (the lanes look at
 * 32 regions per round, so a warp that finds everything taken gives up after ceil(R / 32) rounds
 * of loads).  Every chunk is handed out exactly once whatever %smid reads (it only picks the
 * region tried first), and no warp waits on another. */
constexpr int kMaxRegions = 256;
constexpr int kSuperChunk = 32;
/* chunk of the t-th claim of region r (of R); past the last chunk once the region is used up */
FJSPH_HD int64_t region_chunk(int r, int R, int64_t t) {
    return ((t / kSuperChunk) * R + r) * (int64_t)kSuperChunk + t % kSuperChunk;
}
#ifdef __CUDACC__
__device__ __forceinline__ int64_t claim_chunk(int32_t *next, int64_t chunks) {
    const int lane = threadIdx.x & 31;
    unsigned sm, nsm;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
    asm("mov.u32 %0, %%nsmid;" : "=r"(nsm));
    const int R = (int)min(max(nsm, 1u), (unsigned)kMaxRegions);
    const int r0 = (int)(sm % (unsigned)R);
    int64_t got = -1;
    if (lane == 0) {
        /* counters only grow, and a region's chunks grow with its counter */
        if (region_chunk(r0, R, *(volatile int32_t *)(next + r0)) < chunks) {
            const int64_t g = region_chunk(r0, R, atomicAdd(next + r0, 1));
            if (g < chunks) got = g;
        }
    }
    got = __shfl_sync(0xffffffffu, got, 0);
    if (got >= 0) return got;
    for (int base = 1; base < R; base += 32) {
        const int k = base + lane;
        int r = 0;
        bool avail = false;
        if (k < R) {
            r = r0 + k < R ? r0 + k : r0 + k - R;
            avail = region_chunk(r, R, *(volatile int32_t *)(next + r)) < chunks;
        }
        for (unsigned m = __ballot_sync(0xffffffffu, avail); m; m &= m - 1u) {
            const int src = __ffs(m) - 1;
            int64_t g = -1;
            if (lane == src) {
                g = region_chunk(r, R, atomicAdd(next + r, 1));
                if (g >= chunks) g = -1;
            }
            g = __shfl_sync(0xffffffffu, g, src);
            if (g >= 0) return g;
        }
    }
    return -1;
}
#endif

FJSPH_HD int64_t sell_entry(int64_t slot_base, int32_t k) {
    return slot_base + (int64_t)(k / kChunk) * (kSlice * kChunk) + (k % kChunk);
}

/* The pairs of slot i: entry k at nbr_entry(R, k). */
struct NbrRange {
    int64_t base;
    int32_t n;
    bool sell;
};
__device__ __forceinline__ NbrRange nbr_range(const DevNbr &N, int64_t i) {
    if (N.pair) return NbrRange{N.slice[i / kSlice] + (i % kSlice) * kChunk, N.cnt[i], true};
    return NbrRange{N.off[i], (int32_t)(N.off[i + 1] - N.off[i]), false};
}
__device__ __forceinline__ int64_t nbr_slot(const DevNbr &N, const NbrRange &R, int32_t k) {
    return R.sell ? (int64_t)N.pair[sell_entry(R.base, k)].x : (int64_t)N.idx[R.base + k];
}

FJSPH_HD bool has(const Params &P, uint32_t bit) { return (P.variant & bit) != 0; }

/* Squared distance, accumulated as nanoflann does under -ffast-math on FMA hardware:
 * fma(dz,dz,fma(dy,dy,dx*dx)), d = query - candidate. */
template <int D>
__device__ __forceinline__ double dist2(const double *q, const double *c) {
    double d0 = q[0] - c[0];
    double r = __dmul_rn(d0, d0);
#pragma unroll
    for (int k = 1; k < D; ++k) {
        double dk = __dsub_rn(q[k], c[k]);
        r = __fma_rn(dk, dk, r);
    }
    return r;
}

template <int D, typename R>
__device__ __forceinline__ R dot(const R *a, const R *b) {
    R r = a[0] * b[0];
#pragma unroll
    for (int k = 1; k < D; ++k) r += a[k] * b[k];
    return r;
}

template <int D, typename R>
__device__ __forceinline__ R vnorm(const R *a) {
    return sqrt(dot<D, R>(a, a));
}

/* Eigen normalized(): v/|v|, zero stays zero. */
template <int D, typename R>
__device__ __forceinline__ void normalized(const R *a, R *out) {
    R z = dot<D, R>(a, a);
    if (z > R(0)) {
        R n = sqrt(z);
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = a[k] / n;
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = a[k];
    }
}

/* (1 - q/2)^n for the Wendland C2 kernel, q = r/H, formed as r (1/H): the reciprocal is the same
 * for every pair of a sweep, so the compiler forms it once per thread. */
template <typename R>
__device__ __forceinline__ R wend_base(R r, R H) {
    return R(1) - R(0.5) * (r * (R(1) / H));
}

/* Kernel.h:37-45 / :11-21 */
template <typename R>
__device__ __forceinline__ R kernel_w(R r, R H, R Wc, bool cubic) {
    if (cubic) {
        R q = r / H;
        if (q < R(1)) return Wc * (R(1) - R(1.5) * q * q * (R(1) - R(0.5) * q));
        if (q < R(2)) {
            R t = R(2) - q;
            return Wc * R(0.25) * t * t * t;
        }
        return R(0);
    }
    R b = wend_base(r, H);
    R b2 = b * b;
    return b2 * b2 * (R(2) * (r * (R(1) / H)) + R(1)) * Wc;
}

/* Kernel.h:48-61 / :23-33: gradient = Rij * (returned scalar). */
template <typename R>
__device__ __forceinline__ R gradk_scale(R r, R H, R Wc, bool cubic) {
    if (cubic) {
        R q = r / H;
        if (q < R(1)) return Wc * (R(3) * (R(0.75) * q - R(1))) / (H * H);
        if (q < R(2)) return Wc * R(-0.75) * (R(2) - q) * (R(2) - q) / (r * H);
        return R(0);
    }
    if (r * (R(1) / H) < R(1e-12)) return R(0);
    R b = wend_base(r, H);
    return R(5) / (H * H) * (b * b * b) * Wc;
}

/* (rho / rho0)^gamma of the Cole equation of state: gamma = 7 (the reference's default) by
 * three multiplications (within a few ulp of pow), any other gamma by pow. */
__device__ __forceinline__ double cole_power(double x, double gam) {
    if (gam == 7.0) {
        const double x2 = x * x, x4 = x2 * x2;
        return x4 * x2 * x;
    }
    return pow(x, gam);
}

/* FLUID::get_pressure / get_density (Var.h:203-236). */
__device__ __forceinline__ double eos_pressure(const Params &P, double rho) {
    if (P.pressure_rel == FJSPH_ISO_EOS) return P.speed_sound * P.speed_sound * (rho - P.rho_rest) + P.press_back;
    return P.B * (cole_power(rho * P.rho_rest_inv, P.gam) - 1.0) + P.press_back;
}
__device__ __forceinline__ double eos_density(const Params &P, double press) {
    if (P.pressure_rel == FJSPH_ISO_EOS) return (press - P.press_back) / (P.speed_sound * P.speed_sound) + P.rho_rest;
    return P.rho_rest * pow(((press - P.press_back) / P.B) + 1.0, 1.0 / P.gam);
}
__device__ __forceinline__ double clamp_rho(const Params &P, double lo, double v) { return fmax(lo, fmin(P.rho_max, v)); }

template <int D>
__device__ __forceinline__ void load3(double *const a[3], int64_t i, double *o) {
#pragma unroll
    for (int k = 0; k < D; ++k) o[k] = a[k][i];
}
template <int D>
__device__ __forceinline__ void store3(double *const a[3], int64_t i, const double *o) {
#pragma unroll
    for (int k = 0; k < D; ++k) a[k][i] = o[k];
}

inline unsigned grid_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

/* Device-resident scalars of the integrator (read by kernels so that a step needs no host
 * round trip). */
constexpr int32_t kStatusNbrOverflow = 1; /* DevScalars::status bit: neighbour storage too small */

struct DevScalars {
    double dt;         /* svar.integrator.delta_t                              */
    double npd;        /* numerical particle density from dSPH_PreStep         */
    double red[16];    /* reduction results                                    */
    int32_t status;    /* device-side error bits                               */
    int32_t maxcnt;    /* largest neighbour count of the last single-pass fill */
    unsigned long long pairs; /* pairs of the last single-pass fill            */
    unsigned long long tile_pairs; /* members counted by the last tile mask pass   */
    int32_t tile_maxcnt;           /* largest member count of the last mask pass    */
    int32_t pad;
};

} // namespace fjsph
