/*
 * sweeps_mixed.cu -- the neighbour sweeps of one WCSPH step in the FP32 split-precision form.
 *
 * Pair arithmetic runs on the FP32 pipe.  Quantities whose neighbour differences matter keep
 * about 48 significant bits through a hi/lo split:
 *   x = xhi + xlo, v = vhi + vlo with xhi = fl32(x), xlo = fl32(x - xhi);
 *   x_j - x_i = (xhi_j - xhi_i) + (xlo_j - xlo_i): the hi difference is exact for close values
 *   (Sterbenz) and the lo difference carries the rest, so the separation vector is accurate to
 *   FP32 rounding of the difference itself, independent of the coordinates' magnitude;
 *   rho is carried as rho - rho_rest, so density differences are exact to FP32 of the difference.
 * The squared distance at search time comes from the neighbour search (one float per pair),
 * which decided membership with the reference's FP64 test.  Density-rate and acceleration sums
 * are compensated (Kahan).  Results are written to the FP64 state, so integration, the time-step
 * reduction and global sums stay FP64.
 *
 * Packed per-slot inputs (refreshed by k_pack_state whenever x, v, rho, p, m or a flag changes):
 *   A = (xhi, m/rho)   B = (xlo, p/rho^2)   C = (vhi, rho - rho_rest)   E = (vlo, bits at packing)
 *   F = (vPert, p)     G = (gradRho, lam)   N = (surface normal, 0)     T = (normal from pass 1)
 *   bits = b | surf << 3 | surfzone << 4
 */
#include <algorithm>
#include <atomic>

#include "aero.cuh"
#include "closure.cuh"
#include "kernels.h"
#include "linalg.cuh"
#include "pack.cuh"
#include "tiles.cuh"

namespace fjsph {

namespace {

constexpr int kThreads = 128;

struct Pf { /* float copies of the constants a pair term needs */
    float H, H_sq, Wc, W_dx, rho0, Bgam, nu, alpha, dsph_cont, max_shift_vel;
    float grav[3];
    bool cubic;
};

__device__ __forceinline__ Pf make_pf(const Params &P) {
    const FConst &c = P.fc;
    Pf f;
    f.H = c.H;
    f.H_sq = c.H_sq;
    f.Wc = c.Wc;
    f.W_dx = c.W_dx;
    f.rho0 = c.rho0;
    f.Bgam = c.Bgam;
    f.nu = c.nu;
    f.alpha = c.alpha;
    f.dsph_cont = c.dsph_cont;
    f.max_shift_vel = c.max_shift_vel;
    for (int k = 0; k < 3; ++k) f.grav[k] = c.grav[k];
    f.cubic = has(P, FJSPH_VAR_CUBIC);
    return f;
}

/* Kahan-compensated FP32 accumulator */
struct KSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return to_f64(s) - to_f64(c); }
};

/* cos x for x in [0, 2 pi) on the SFU: folded into [-pi/2, pi/2] by cos x = -cos(x - pi), where
 * the hardware cosine's absolute error is about 2^-21 (the pairwise surface-tension argument
 * 3 pi r / (4 H) stays below 1.5 pi) */
__device__ __forceinline__ float cos_0_2pi(float x) {
    const float pi = 3.14159265358979f;
    return x > 0.5f * pi && x < 1.5f * pi ? -__cosf(x - pi) : (x >= 1.5f * pi ? __cosf(x - 2.f * pi) : __cosf(x));
}

__device__ __forceinline__ int bits_b(int w) { return w & 7; }
__device__ __forceinline__ int bits_surf(int w) { return (w >> 3) & 1; }
__device__ __forceinline__ int bits_zone(int w) { return (w >> 4) & 1; }

/* the pairs of slot i in the sliced-ELL list: L[k] for k < L.n */
struct SellList {
    const int2 *p;
    int32_t n;
    __device__ __forceinline__ int2 operator[](int32_t k) const { return p[sell_entry(0, k)]; }
    __device__ __forceinline__ const int2 *at(int32_t k) const { return p + sell_entry(0, k); }
};
__device__ __forceinline__ SellList sell(const DevNbr &N, int64_t i) {
    return SellList{N.pair + N.slice[i / kSlice] + (i % kSlice) * kChunk, N.cnt[i]};
}

__device__ __forceinline__ void prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

/* Pair-list rows fetched into L1 ahead of use by the residual (default; Params::list_ahead is the
 * tuned value); with the sliced-ELL order one row of a warp is one 256-byte line. */
constexpr int32_t kListAhead = 4;
/* pairs whose neighbour inputs are in flight ahead of the residual's current pair */
#ifndef FJSPH_GATHER_AHEAD
#define FJSPH_GATHER_AHEAD 1
#endif
constexpr int kGatherAhead = FJSPH_GATHER_AHEAD;

__device__ __forceinline__ void prefetch_pair_inputs(const Packed &K, int32_t j, bool f, bool g) {
    prefetch_l1(K.A + j);
    prefetch_l1(K.C + j);
    prefetch_l1(K.Lo + j);
    if (f) prefetch_l1(K.F + j);
    if (g) prefetch_l1(K.G + j);
}

/* separation x_j - x_i from the hi/lo split */

/* the compact neighbour inputs (Packed::Lo): low parts of x and v, p / rho^2 and type flags */
struct LoParts {
    float xl[3], vl[3], pr;
    uint32_t flags;
    __device__ __forceinline__ LoParts() {}
    __device__ __forceinline__ explicit LoParts(const float4 q) {
        const uint32_t a = __float_as_uint(q.x), b = __float_as_uint(q.y), c = __float_as_uint(q.z);
        xl[0] = __uint_as_float(a << 16);
        xl[1] = __uint_as_float(a & 0xFFFF0000u);
        xl[2] = __uint_as_float(b << 16);
        vl[0] = __uint_as_float(b & 0xFFFF0000u);
        vl[1] = __uint_as_float(c << 16);
        vl[2] = __uint_as_float(c & 0xFFFF0000u);
        const uint32_t w = __float_as_uint(q.w);
        pr = __uint_as_float(w & ~3u);
        flags = w & 3u;
    }
};

/* separations x_j - x_i and v_j - v_i: high parts first, then the low parts */
template <int D>
__device__ __forceinline__ void sepx(const float4 &Ai, const LoParts &Li, const float4 &Aj, const LoParts &Lj, float *R) {
    R[0] = (Aj.x - Ai.x) + (Lj.xl[0] - Li.xl[0]);
    R[1] = (Aj.y - Ai.y) + (Lj.xl[1] - Li.xl[1]);
    if (D == 3) R[2] = (Aj.z - Ai.z) + (Lj.xl[2] - Li.xl[2]);
}
template <int D>
__device__ __forceinline__ void sepv(const float4 &Ci, const LoParts &Li, const float4 &Cj, const LoParts &Lj, float *V) {
    V[0] = (Cj.x - Ci.x) + (Lj.vl[0] - Li.vl[0]);
    V[1] = (Cj.y - Ci.y) + (Lj.vl[1] - Li.vl[1]);
    if (D == 3) V[2] = (Cj.z - Ci.z) + (Lj.vl[2] - Li.vl[2]);
}

template <int D>
__device__ __forceinline__ float fdot(const float *a, const float *b) {
    float r = a[0] * b[0];
#pragma unroll
    for (int k = 1; k < D; ++k) r += a[k] * b[k];
    return r;
}

template <int D>
__device__ __forceinline__ void fnormalized(const float *a, float *o) {
    const float z = fdot<D>(a, a);
    if (z > 0.f) {
        const float n = sqrtf(z);
#pragma unroll
        for (int k = 0; k < D; ++k) o[k] = a[k] / n;
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) o[k] = a[k];
    }
}

__device__ __forceinline__ float f_kernel(const Pf &f, float r) { return kernel_w<float>(r, f.H, f.Wc, f.cubic); }
__device__ __forceinline__ float f_gscale(const Pf &f, float r) { return gradk_scale<float>(r, f.H, f.Wc, f.cubic); }

/* FP32 copy of the renormalisation matrix L (row-major D x D) in three float4 arrays */
template <int D>
__device__ __forceinline__ void store_lf(const Packed &K, int64_t i, const float *l) {
    if (D == 2) {
        K.L0[i] = make_float4(l[0], l[1], l[2], l[3]);
    } else {
        K.L0[i] = make_float4(l[0], l[1], l[2], l[3]);
        K.L1[i] = make_float4(l[4], l[5], l[6], l[7]);
        K.L2[i] = make_float4(l[8], 0.f, 0.f, 0.f);
    }
}
template <int D>
__device__ __forceinline__ void load_lf(const Packed &K, int64_t i, float *l) {
    const float4 a = K.L0[i];
    l[0] = a.x;
    l[1] = a.y;
    l[2] = a.z;
    l[3] = a.w;
    if (D == 3) {
        const float4 b = K.L1[i];
        l[4] = b.x;
        l[5] = b.y;
        l[6] = b.z;
        l[7] = b.w;
        l[8] = K.L2[i].x;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* packing                                                                                       */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void k_pack_state(Params P, DevState W, Packed K, int64_t i0, int64_t i1, int full) {
    const int64_t i = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= i1) return;
    pack_particle<D>(P, W, K, i);
    if (full) {
        K.G[i] = make_float4(to_f32(W.gradRho[0][i]), to_f32(W.gradRho[1][i]), D == 3 ? to_f32(W.gradRho[2][i]) : 0.f,
                             to_f32(W.lam[i]));
        K.N[i] = make_float4(to_f32(W.norm[0][i]), to_f32(W.norm[1][i]), D == 3 ? to_f32(W.norm[2][i]) : 0.f,
                             to_f32(W.lam_nb[i]));
        float l[9];
#pragma unroll
        for (int k = 0; k < D * D; ++k) l[k] = to_f32(W.L[k][i]);
        store_lf<D>(K, i, l);
    }
}

/* ------------------------------------------------------------------------------------------ */
/* npd alone                                                                                     */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void __launch_bounds__(kThreads) k_m_npd(Params P, DevNbr N, Packed K, double *npd_part) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const Pf f = make_pf(P);
    float npd = 0.f;
    const SellList L = sell(N, i);
    for (int32_t e = 0; e < L.n; ++e) {
        const int2 pe = L[e];
        const int32_t j = pe.x;
        if (j == i || bits_b(K.bits[j]) <= FJSPH_PISTON) continue;
        npd += f_kernel(f, sqrtf(__int_as_float(pe.y)));
    }
    npd_part[i] = npd;
}

/* ------------------------------------------------------------------------------------------ */
/* dSPH_PreStep (src/Shifting.cpp:12-123)                                                        */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void __launch_bounds__(kThreads) k_m_dsph(Params P, DevState W, DevNbr N, Packed K, double *npd_part) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const Pf f = make_pf(P);
    const float4 Ai = K.A[i];
    const LoParts Li(K.Lo[i]);
    const float drho_i = K.R[i];
    float Lm[D * D], Lnb[D * D], gR[D], nr[D];
#pragma unroll
    for (int k = 0; k < D * D; ++k) {
        Lm[k] = 0.f;
        Lnb[k] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
        gR[k] = 0.f;
        nr[k] = 0.f;
    }
    float kernsum = 0.f, colour = 0.f, npd = 0.f;
    const SellList L = sell(N, i);
    for (int32_t e = 0; e < L.n; ++e) {
        const int2 pe = L[e];
        const int32_t j = pe.x;
        if (j == i) {
            kernsum += f.Wc;
            continue;
        }
        const float4 Aj = K.A[j];
        const LoParts Lj(K.Lo[j]);
        float Rji[D];
        sepx<D>(Ai, Li, Aj, Lj, Rji);
        const float r = sqrtf(__int_as_float(pe.y));
        const float volj = Aj.w;
        const float kern = f_kernel(f, r);
        const float gs = f_gscale(f, r);
        const bool fl = (Lj.flags & kLoFluid) != 0u;
        const float drho = volj * (K.R[j] - drho_i);
        /* Lm -= volj Rji (x) Grad with Grad = -Rji gs */
        const float w = volj * gs;
#pragma unroll
        for (int a = 0; a < D; ++a) {
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const float t = w * Rji[a] * Rji[c];
                Lm[a * D + c] += t;
                if (fl) Lnb[a * D + c] += t;
            }
            gR[a] -= drho * gs * Rji[a];
        }
        if (fl) {
#pragma unroll
            for (int k = 0; k < D; ++k) nr[k] -= w * Rji[k];
            kernsum += kern;
            colour += volj * kern;
            npd += kern;
        }
    }
    float Linv[D * D];
    if (!qr_inverse<D, float>(Lm, Linv)) {
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int c = 0; c < D; ++c) Linv[a * D + c] = (a == c) ? 1.f : 0.f;
    }
    float g[D], n[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
        float sg = 0.f, sn = 0.f;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            sg += Linv[a * D + c] * gR[c];
            sn += Linv[a * D + c] * nr[c];
        }
        g[a] = sg;
        n[a] = sn;
        W.gradRho[a][i] = to_f64(sg);
        W.norm[a][i] = to_f64(sn);
    }
#pragma unroll
    for (int k = 0; k < D * D; ++k) W.L[k][i] = to_f64(Linv[k]);
    store_lf<D>(K, i, Linv);
    float lam, lam_nb;
    if (W.b[i] == FJSPH_BOUND) {
        lam = 1.f;
        lam_nb = 1.f;
    } else {
        lam = min_eig<D, float>(Lm);
        lam_nb = min_eig<D, float>(Lnb);
    }
    W.lam[i] = to_f64(lam);
    W.lam_nb[i] = to_f64(lam_nb);
    W.colourG[i] = (lam > 0.7f) ? 2.0 : 2.0 * fmax(1.0, 1.0 / (2.0 * to_f64(colour)));
    W.kernsum[i] = to_f64(kernsum);
    W.colour[i] = to_f64(colour);
    npd_part[i] = npd;
    K.G[i] = make_float4(g[0], g[1], D == 3 ? g[2] : 0.f, lam);
    K.N[i] = make_float4(n[0], n[1], D == 3 ? n[2] : 0.f, lam_nb);
}

/* ------------------------------------------------------------------------------------------ */
/* artificial viscosity scalar (src/Kernel.h:217-244)                                           */
/* ------------------------------------------------------------------------------------------ */
__device__ __forceinline__ float f_art_visc(const Pf &f, float vdotr, float idist2, float rho_i, float rho_j) {
    if (vdotr > 0.f) return 0.f;
    const float muij = f.H * vdotr * idist2;
    const float rhoij = 0.5f * (rho_i + rho_j);
    const float cbar = 0.5f * (sqrtf(f.Bgam / rho_i) + sqrtf(f.Bgam / rho_j));
    return f.alpha * cbar * muij / rhoij;
}

/* ------------------------------------------------------------------------------------------ */
/* dissipation_terms (src/Shifting.cpp:126-186)                                                  */
/* ------------------------------------------------------------------------------------------ */
/* Per-particle accumulator of the dissipation terms, shared by the stand-alone pass and the
 * surface-normal pass that carries it (both walk every neighbour j != i of a fluid particle). */
template <int D>
struct Dissip {
    bool linear, nodsph;
    float4 Ci;
    LoParts Li;
    float rho_i;
    float gRi[D], av[D];
    KSum Rrhod;
    __device__ __forceinline__ void init(const Params &P, const Pf &f, const Packed &K, int64_t i) {
        linear = has(P, FJSPH_VAR_LINEAR);
        nodsph = has(P, FJSPH_VAR_NODSPH);
        Ci = K.C[i];
        Li = LoParts(K.Lo[i]);
        const float4 Gi = K.G[i];
        rho_i = f.rho0 + Ci.w;
        gRi[0] = Gi.x;
        gRi[1] = Gi.y;
        if (D == 3) gRi[2] = Gi.z;
#pragma unroll
        for (int k = 0; k < D; ++k) av[k] = 0.f;
    }
    /* pair (i, j): Rji = x_j - x_i, rr = |Rji|^2, gs = f_gscale(r), Gj = K.G[j] */
    __device__ __forceinline__ void add(const Pf &f, const Packed &K, int32_t j, const LoParts &Lj, const float *Rji,
                                        float rr, float gs, float volj, const float4 Gj) {
        const float4 Cj = K.C[j];
        float Vji[D];
        sepv<D>(Ci, Li, Cj, Lj, Vji);
        const float idist2 = 1.f / (rr + 0.0001f * f.H_sq);
        const float rho_j = f.rho0 + Cj.w;
        float g[D];
#pragma unroll
        for (int k = 0; k < D; ++k) g[k] = Rji[k] * gs;
        const bool fl = (Lj.flags & kLoFluid) != 0u;
        if (fl) {
            const float vdotr = fdot<D>(Vji, Rji);
            const float c = linear ? volj * idist2 * vdotr : (volj * rho_j) * f_art_visc(f, vdotr, idist2, rho_i, rho_j);
#pragma unroll
            for (int k = 0; k < D; ++k) av[k] += c * g[k];
        }
        if (!nodsph) {
            const float rg = fdot<D>(Rji, g);
            float t = Cj.w - Ci.w;
            if (fl) {
                float gsum[D];
                gsum[0] = gRi[0] + Gj.x;
                gsum[1] = gRi[1] + Gj.y;
                if (D == 3) gsum[2] = gRi[2] + Gj.z;
                t += 0.5f * fdot<D>(gsum, Rji);
            }
            Rrhod.add(volj * t * rg * idist2);
        }
    }
    __device__ __forceinline__ void finish(const Params &P, const DevState &W, int64_t i) {
        if (linear) {
            const float c = (float)(P.visc_alpha * P.H * P.speed_sound * P.rho_rest) / rho_i;
#pragma unroll
            for (int k = 0; k < D; ++k) av[k] *= c;
        }
#pragma unroll
        for (int k = 0; k < D; ++k) W.aVisc[k][i] = to_f64(av[k]);
        if (!nodsph) W.deltaD[i] = P.dsph_cont * Rrhod.value();
    }
};

/* ------------------------------------------------------------------------------------------ */
/* Detect_Surface (src/Geometry.cpp:14-280)                                                      */
/* ------------------------------------------------------------------------------------------ */
/* DIS: the dissipation terms ride along in the normal's neighbour loop (one list walk and one
 * set of position gathers for both; the dissipation reads nothing this pass writes). */
template <int D, bool DIS>
__global__ void __launch_bounds__(kThreads) k_m_surface_normal(Params P, DevState W, DevNbr N, Packed K) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const Pf f = make_pf(P);
    Dissip<D> dis;
    if (DIS) dis.init(P, f, K, i);
    const float h = P.fc.surf_h;
    const float4 Ai = K.A[i];
    const LoParts Li(K.Lo[i]);
    const float4 Ni = K.N[i]; /* dSPH normal, lam_nb */
    float ni[D], nh[D];
    ni[0] = Ni.x;
    ni[1] = Ni.y;
    if (D == 3) ni[2] = Ni.z;
    fnormalized<D>(ni, nh);
    const int b = W.b[i];
    const float lam_nb = Ni.w, lam = K.G[i].w;
    const SellList L = sell(N, i);
    int surf = W.surf[i];
    /* the geometric test of the surface band runs inside the normal's walk below: a neighbour
     * inside the test region clears the flag, and once it is clear the test is skipped (the
     * flag a walk that stops at the first such neighbour would give) */
    bool test = false;
    float th[D];
    if (b < FJSPH_PIPE) {
        surf = 0;
        W.woccl[i] = 1.0;
    } else if (lam_nb < 0.2f) {
        surf = 1;
    } else if (lam_nb < 0.75f) {
        if (D == 2) {
            float tau[D];
            tau[0] = ni[1];
            tau[1] = -ni[0];
            fnormalized<D>(tau, th);
        }
        surf = 1;
        test = true;
    } else {
        surf = 0;
    }
    const float sq2h = sqrtf(2.f) * h;
    float nrm[D];
#pragma unroll
    for (int k = 0; k < D; ++k) nrm[k] = 0.f;
    const bool inside = lam > 0.7f;
    for (int32_t e = 0; e < L.n; ++e) {
        const int2 pe = L[e];
        const int32_t j = pe.x;
        if (j == i) continue;
        float Rji[D];
        const float4 Aj = K.A[j];
        const LoParts Lj(K.Lo[j]);
        sepx<D>(Ai, Li, Aj, Lj, Rji);
        const float rr = __int_as_float(pe.y);
        const float r = sqrtf(rr);
        if (test && surf) {
            /* x_j - pointT = (x_j - x_i) - h n_hat */
            float xT[D];
#pragma unroll
            for (int k = 0; k < D; ++k) xT[k] = Rji[k] - h * nh[k];
            if (r >= sq2h) {
                if (sqrtf(fdot<D>(xT, xT)) < h) surf = 0;
            } else if (D == 2) {
                if (fabsf(fdot<D>(nh, xT)) + fabsf(fdot<D>(th, xT)) < h) surf = 0;
            } else {
                float u[D];
#pragma unroll
                for (int k = 0; k < D; ++k) u[k] = Rji[k] / r;
                /* acos(c) < pi/4  <=>  c > cos(pi/4) (acos decreases on [-1, 1]) */
                if (fdot<D>(nh, u) > 0.70710678118654752f) surf = 0;
            }
        }
        const float volj = Aj.w;
        const float gs = f_gscale(f, r);
        const float4 Gj = K.G[j];
        const float lj = Gj.w;
        const float w = inside ? volj * (lj - lam) : volj * lj;
        /* GradK(Rij) with Rij = x_i - x_j = -Rji */
#pragma unroll
        for (int k = 0; k < D; ++k) nrm[k] -= w * (Rji[k] * gs);
        if (DIS) dis.add(f, K, j, Lj, Rji, rr, gs, volj, Gj);
    }
    if (DIS) dis.finish(P, W, i);
    W.surf[i] = surf;
    K.bits[i] = (K.bits[i] & ~8) | (surf << 3);
    float Lf[D * D], n2[D];
    load_lf<D>(K, i, Lf);
#pragma unroll
    for (int a = 0; a < D; ++a) {
        float s = 0.f;
#pragma unroll
        for (int c = 0; c < D; ++c) s += Lf[a * D + c] * nrm[c];
        n2[a] = s;
    }
    float out[D];
    if (sqrtf(fdot<D>(n2, n2)) > 0.1f * lam / f.H) {
        fnormalized<D>(n2, out);
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = 0.f;
    }
    K.T[i] = make_float4(out[0], out[1], D == 3 ? out[2] : 0.f, 0.f);
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_m_surface_curvature(Params P, DevState W, DevNbr N, Packed K) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const Pf f = make_pf(P);
    const bool gissler = P.acase == FJSPH_GISSLER;
    const int b = W.b[i];
    const float4 Ai = K.A[i], Ti = K.T[i];
    const LoParts Qi(K.Lo[i]);
    float ni[D], Vdiff[D];
    ni[0] = Ti.x;
    ni[1] = Ti.y;
    if (D == 3) ni[2] = Ti.z;
    const bool occl = (b == FJSPH_FREE) && gissler;
    const bool vd_on = occl && W.cellID[i] != -1;
    Vdiff[0] = vd_on ? to_f32(vinf_of(P, i, 0) - W.v[0][i]) : 0.f;
    Vdiff[1] = vd_on ? to_f32(vinf_of(P, i, 1) - W.v[1][i]) : 0.f;
    if (D == 3) Vdiff[2] = vd_on ? to_f32(vinf_of(P, i, 2) - W.v[2][i]) : 0.f;
    float Li[D * D];
    load_lf<D>(K, i, Li);
    const float nin = sqrtf(fdot<D>(ni, ni)), vdn = sqrtf(fdot<D>(Vdiff, Vdiff));
    float curve = 0.f, woccl_ = 0.f, o0 = 0.f, o1 = 0.f, o2 = 0.f;
    /* ALE/TIC builds: the surface zone (any neighbour, self included, on the surface) rides along */
    const bool zone = has(P, FJSPH_VAR_ALE) || has(P, FJSPH_VAR_TIC);
    int sz = 0;
    const SellList L = sell(N, i);
    for (int32_t e = 0; e < L.n; ++e) {
        const int2 pe = L[e];
        const int32_t j = pe.x;
        if (zone && !sz && bits_surf(K.bits[j])) sz = 1;
        if (j == i) continue;
        float Rij[D]; /* = x_j - x_i, the reference's naming in this loop */
        sepx<D>(Ai, Qi, K.A[j], LoParts(K.Lo[j]), Rij);
        const float r = sqrtf(__int_as_float(pe.y));
        /* a particle without a normal (the interior) needs no neighbour normals */
        float nj[D];
        if (nin > 0.f) {
            const float4 Tj = K.T[j];
            nj[0] = Tj.x;
            nj[1] = Tj.y;
            if (D == 3) nj[2] = Tj.z;
        }
        if (nin > 0.f && fdot<D>(nj, nj) > 0.f) {
            const float volj = K.A[j].w;
            const float gs = f_gscale(f, r);
            float s = 0.f;
#pragma unroll
            for (int a = 0; a < D; ++a) {
                float Ld = 0.f;
#pragma unroll
                for (int c = 0; c < D; ++c) Ld += Li[a * D + c] * (nj[c] - ni[c]);
                s += Ld * (Rij[a] * gs);
            }
            curve += volj * s;
        }
        if (occl) {
            const float frac = -fdot<D>(Rij, Vdiff) / (vdn * r);
            if (frac > woccl_) woccl_ = frac;
            if (vdn > 0.f) { /* inputs 0-2 of the learned closure */
                const float w = K.A[j].w * kernel_w<float>(r, f.H, f.Wc, f.cubic);
                o0 += w * fmaxf(frac, 0.f);
                o1 += w * fmaxf(-frac, 0.f);
                o2 += w * frac * frac;
            }
        }
    }
    const float lam_nb_i = K.N[i].w;
    W.woccl[i] = to_f64((lam_nb_i < P.fc.lam_cutoff) ? fmaxf(0.f, fminf(woccl_, 1.f)) : 1.0f);
    K.O[i] = make_float4(o0, o1, o2, woccl_);
#pragma unroll
    for (int k = 0; k < D; ++k) W.norm[k][i] = to_f64(ni[k]);
    const double curve_d = to_f64(curve);
    W.curve[i] = curve_d;
    W.norm_curve[i] = P.dx * curve_d;
    W.pDist[i] = W.lam[i];
    K.N[i] = make_float4(ni[0], ni[1], D == 3 ? ni[2] : 0.f, lam_nb_i);
    if (zone) { /* bit 4 of the own record; the other threads read only bit 3 of it */
        W.surfzone[i] = sz;
        atomicAnd(&K.bits[i], ~16);
        if (sz) atomicOr(&K.bits[i], 16);
    }
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_m_dissipation(Params P, DevState W, DevNbr N, Packed K) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const Pf f = make_pf(P);
    const float4 Ai = K.A[i];
    const LoParts Li(K.Lo[i]);
    Dissip<D> dis;
    dis.init(P, f, K, i);
    const SellList L = sell(N, i);
    for (int32_t e = 0; e < L.n; ++e) {
        const int2 pe = L[e];
        const int32_t j = pe.x;
        if (j == i) continue;
        const float4 Aj = K.A[j];
        const LoParts Lj(K.Lo[j]);
        float Rji[D];
        sepx<D>(Ai, Li, Aj, Lj, Rji);
        const float rr = __int_as_float(pe.y);
        dis.add(f, K, j, Lj, Rji, rr, f_gscale(f, sqrtf(rr)), Aj.w, K.G[j]);
    }
    dis.finish(P, W, i);
}

/* ------------------------------------------------------------------------------------------ */
/* particle_shift (src/Shifting.cpp:189-290, -DALE)                                              */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void __launch_bounds__(kThreads) k_m_particle_shift(Params P, DevState W, DevNbr N, Packed K) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const float lam_nb = to_f32(W.lam_nb[i]);
    if (lam_nb < 0.55f || W.b[i] == FJSPH_BUFFER) {
#pragma unroll
        for (int k = 0; k < D; ++k) W.vPert[k][i] = 0.0;
        K.F[i] = make_float4(0.f, 0.f, 0.f, K.F[i].w);
        return;
    }
    const Pf f = make_pf(P);
    const float4 Ai = K.A[i], Ci = K.C[i], Ni = K.N[i];
    const LoParts Li(K.Lo[i]);
    float ni[D], nh[D], vi[D];
    ni[0] = Ni.x;
    ni[1] = Ni.y;
    if (D == 3) ni[2] = Ni.z;
    fnormalized<D>(ni, nh);
    vi[0] = Ci.x + Li.vl[0];
    vi[1] = Ci.y + Li.vl[1];
    if (D == 3) vi[2] = Ci.z + Li.vl[2];
    float dU[D];
#pragma unroll
    for (int k = 0; k < D; ++k) dU[k] = 0.f;
    float maxUij = 0.f, woccl = 0.f;
    const SellList L = sell(N, i);
    for (int32_t e = 0; e < L.n; ++e) {
        const int2 pe = L[e];
        const int32_t j = pe.x;
        if (j == i) continue;
        float Rji[D], dv[D];
        const LoParts Lj(K.Lo[j]);
        sepx<D>(Ai, Li, K.A[j], Lj, Rji);
        sepv<D>(Ci, Li, K.C[j], Lj, dv);
        const float r = sqrtf(__int_as_float(pe.y));
        const float volj = K.A[j].w;
        const float kern = f_kernel(f, r);
        const float gs = f_gscale(f, r);
        const float q = kern / f.W_dx;
        const float q2 = q * q;
        const float c = (1.f + 0.2f * (q2 * q2)) * volj * gs;
#pragma unroll
        for (int k = 0; k < D; ++k) dU[k] += c * Rji[k];
        if (bits_b(K.bits[j]) > FJSPH_PISTON) {
            const float4 Nj = K.N[j];
            float nj[D], njh[D];
            nj[0] = Nj.x;
            nj[1] = Nj.y;
            if (D == 3) nj[2] = Nj.z;
            fnormalized<D>(nj, njh);
            const float theta = acosf(fdot<D>(nh, njh));
            if (theta > woccl) woccl = theta;
        }
        const float dvn = sqrtf(fdot<D>(dv, dv));
        if (dvn > maxUij) maxUij = dvn;
    }
    const float sc = -2.f * f.H * sqrtf(fdot<D>(vi, vi));
#pragma unroll
    for (int k = 0; k < D; ++k) dU[k] *= sc;
    const float mag = fminf(sqrtf(fdot<D>(dU, dU)), fminf(maxUij / 2.f, f.max_shift_vel));
    float dUn[D];
    fnormalized<D>(dU, dUn);
#pragma unroll
    for (int k = 0; k < D; ++k) dU[k] = mag * dUn[k];
    float out[D];
    if (W.surfzone[i] == 0 && lam_nb > 0.55f) {
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = dU[k];
    } else if (woccl < (float)(kPi / 12.0)) {
#pragma unroll
        for (int a = 0; a < D; ++a) {
            float s = 0.f;
#pragma unroll
            for (int c = 0; c < D; ++c) s += ((a == c ? 1.f : 0.f) - nh[a] * nh[c]) * dU[c];
            out[a] = s;
        }
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) W.vPert[k][i] = out[k];
    K.F[i] = make_float4(out[0], out[1], D == 3 ? out[2] : 0.f, K.F[i].w);
}

/* ------------------------------------------------------------------------------------------ */
/* boundary passes (src/Resid.cpp:21-186)                                                        */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void __launch_bounds__(kThreads) k_m_bound_pressure(Params P, DevState W, DevNbr N, Packed K) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    if (P.blocks[W.blk[i]].bound_solver != FJSPH_PRESSURE_G) return;
    const Pf f = make_pf(P);
    const float4 Ai = K.A[i];
    const LoParts Li(K.Lo[i]);
    int near = 0;
    KSum kernsum, pkern;
    float acck[D];
#pragma unroll
    for (int k = 0; k < D; ++k) acck[k] = 0.f;
    const SellList L = sell(N, i);
    for (int32_t e = 0; e < L.n; ++e) {
        const int2 pe = L[e];
        const int32_t j = pe.x;
        const int bj = K.bits[j];
        if (bits_b(bj) <= FJSPH_PISTON) continue;
        const float4 Aj = K.A[j];
        const LoParts Lj(K.Lo[j]);
        float Rji[D];
        sepx<D>(Ai, Li, Aj, Lj, Rji);
        const float r = sqrtf(__int_as_float(pe.y));
        const float rho_j = f.rho0 + K.C[j].w;
        const float kern = Aj.w * f_kernel(f, r);
        kernsum.add(kern);
        pkern.add(K.F[j].w * kern);
        /* (x_i - x_j) = -Rji */
#pragma unroll
        for (int k = 0; k < D; ++k) acck[k] -= kern * rho_j * Rji[k];
        if (bits_zone(bj)) near = 1;
    }
    double p = 0.0;
    const double ks = kernsum.value();
    if (ks > 0.0) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) s += (P.grav[k] - W.acc[k][i]) * (double)acck[k];
        p = (pkern.value() + s) / ks;
        if (near) p = fmax(0.0, p);
    }
    W.p[i] = p;
    W.rho[i] = eos_density(P, p);
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_m_bound_ghost(Params P, DevState W, DevNbr N, Packed K,
                                                              int32_t *near_inlet) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    if (P.blocks[W.blk[i]].bound_solver != FJSPH_GHOST) return;
    const Pf f = make_pf(P);
    const float4 Ai = K.A[i];
    const LoParts Li(K.Lo[i]);
    /* boundary velocity: set this stage, read from the FP64 state */
    float vi[D];
#pragma unroll
    for (int k = 0; k < D; ++k) vi[k] = to_f32(W.v[k][i]);
    KSum Rr;
    int ni = 1;
    const SellList L = sell(N, i);
    for (int32_t e = 0; e < L.n; ++e) {
        const int2 pe = L[e];
        const int32_t j = pe.x;
        if (j == i) continue;
        const int bj = bits_b(K.bits[j]);
        if (bj == FJSPH_PIPE || bj == FJSPH_FREE) ni = 0;
        float Rji[D];
        const LoParts Lj(K.Lo[j]);
        sepx<D>(Ai, Li, K.A[j], Lj, Rji);
        const float r = sqrtf(__int_as_float(pe.y));
        const float gs = f_gscale(f, r);
        const float4 Cj = K.C[j];
        float s = 0.f;
        s += ((Cj.x + Lj.vl[0]) - vi[0]) * Rji[0];
        s += ((Cj.y + Lj.vl[1]) - vi[1]) * Rji[1];
        if (D == 3) s += ((Cj.z + Lj.vl[2]) - vi[2]) * Rji[2];
        Rr.add(-K.A[j].w * s * gs);
    }
    near_inlet[i] = ni;
    W.Rrho[i] = Rr.value() * W.rho[i];
}

/* ------------------------------------------------------------------------------------------ */
/* residual (src/Resid.cpp:243-469)                                                               */
/* ------------------------------------------------------------------------------------------ */
/* Per-particle accumulator of the residual's pair sums: the same arithmetic for the pair-list
 * sweep and the shared-memory tile sweep.  Each supplies the separations x_j - x_i, v_j - v_i
 * (and the absolute velocities under ALE) in its own representation; F and G of a neighbour are
 * read by slot when a variant needs them. */
template <int D, bool ALE, bool NOFROZEN>
struct ResidAcc {
    float rho_i, m_i, pr_i, p_i, npdm2, pi3o4_H, fac_bound, drho_i;
    int b_i, sz_i;
    bool linear, nodsph, tic, st_on, csf;
    float vPi[D], gRi[D], vi[D];
    KSum acc[D];
    float acc_ale[D], visc[D], st[D], art[D];
    KSum Rrho, Rrhoc, Rrho_d;

    /* vol_i = m / rho, drho = rho - rho0, pr = p / rho^2 (packed, flags in the low bits),
     * v = absolute velocity (used under ALE) */
    __device__ __forceinline__ void init(const Params &P, const Pf &f, const Packed &K, int64_t i, float vol_i,
                                         float drho, float pr, const float *v, const double *npd_dev) {
        linear = has(P, FJSPH_VAR_LINEAR);
        nodsph = has(P, FJSPH_VAR_NODSPH);
        tic = has(P, FJSPH_VAR_TIC);
        const bool pairwise = P.st_model == FJSPH_ST_PAIRWISE;
        csf = P.st_model == FJSPH_ST_CSF;
        npdm2 = 0.f;
        if (pairwise) {
            const float npd = to_f32(npd_dev[grp_of(P, i)]);
            npdm2 = P.fc.st_coef_f / (npd * npd);
        }
        pi3o4_H = P.fc.pi3o4_H;
        fac_bound = P.fc.fac_bound;
        const float4 Fi = K.F[i];
        drho_i = drho;
        rho_i = f.rho0 + drho;
        m_i = vol_i * rho_i;
        const int bits_i = K.bits[i];
        b_i = bits_b(bits_i);
        sz_i = bits_zone(bits_i);
        pr_i = (tic && sz_i != 1) ? fabsf(pr) : pr;
        p_i = (tic && sz_i != 1) ? fabsf(Fi.w) : Fi.w;
        vPi[0] = Fi.x;
        vPi[1] = Fi.y;
        if (D == 3) vPi[2] = Fi.z;
        if (NOFROZEN) {
            const float4 Gi = K.G[i];
            gRi[0] = Gi.x;
            gRi[1] = Gi.y;
            if (D == 3) gRi[2] = Gi.z;
        }
#pragma unroll
        for (int k = 0; k < D; ++k) {
            vi[k] = v[k];
            acc_ale[k] = 0.f;
            visc[k] = 0.f;
            st[k] = 0.f;
            art[k] = 0.f;
        }
        st_on = pairwise && (!ALE || sz_i == 1);
    }

    /* slot j is read only by the variants that need F or G of the neighbour */
    __device__ __forceinline__ bool needs_slot() const { return ALE || NOFROZEN || linear; }

    /* pair (i, j), j != i: Rji = x_j - x_i, Vji = v_j - v_i, vj = v_j (ALE), rr = search-time r^2 */
    __device__ __forceinline__ void pair(const Pf &f, const Packed &K, int32_t j, const float *Rji, const float *Vji,
                                         const float *vj, float volj, float drho_j, float prj, uint32_t flags_j,
                                         float rr) {
        const float r = sqrtf(rr);
        const float idist2 = 1.f / (rr + 0.001f * f.H_sq);
        const float rho_j = f.rho0 + drho_j;
        const float m_j = volj * rho_j;
        const bool bound_j = (flags_j & kLoBound) != 0u, fluid_j = (flags_j & kLoFluid) != 0u;
        const float gs = f_gscale(f, r);
        float g[D];
#pragma unroll
        for (int k = 0; k < D; ++k) g[k] = Rji[k] * gs;
        float pc;
        if (linear)
            pc = (p_i + K.F[j].w) * volj;
        else
            pc = m_j * (pr_i + prj);
#pragma unroll
        for (int k = 0; k < D; ++k) acc[k].add(-pc * g[k]);
        const float rg = fdot<D>(Rji, g);
        const float vc = m_j * (f.nu * (rho_i + rho_j) / (rho_i * rho_j) * rg * idist2);
#pragma unroll
        for (int k = 0; k < D; ++k) visc[k] += vc * Vji[k];
        if (st_on) {
            const float fac = (b_i == FJSPH_BOUND || bound_j) ? fac_bound : 1.f;
            const float c = -npdm2 * fac * cos_0_2pi(pi3o4_H * r) / r;
#pragma unroll
            for (int k = 0; k < D; ++k) st[k] += c * Rji[k];
        }
        if (ALE) {
            const float4 Fj = K.F[j];
            float vPj[D];
            vPj[0] = Fj.x;
            vPj[1] = Fj.y;
            if (D == 3) vPj[2] = Fj.z;
            const float gj = fdot<D>(vPj, g), gi = fdot<D>(vPi, g);
            float q = 0.f, w1 = 0.f, w2 = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                q += (vPj[k] - vPi[k]) * g[k];
                w1 += (Vji[k] + (vPj[k] - vPi[k])) * g[k];
                w2 += (rho_j * vPj[k] + rho_i * vPi[k]) * g[k];
            }
#pragma unroll
            for (int a = 0; a < D; ++a) acc_ale[a] += (vj[a] * gj + vi[a] * gi - vi[a] * q) * volj;
            Rrho.add(-w1 * volj);
            Rrhoc.add(w2 * volj);
        } else {
            Rrho.add(-volj * fdot<D>(Vji, g));
        }
        if (NOFROZEN) {
            if (fluid_j) {
                if (!nodsph) {
                    const float4 Gj = K.G[j];
                    float gsum[D];
                    gsum[0] = gRi[0] + Gj.x;
                    gsum[1] = gRi[1] + Gj.y;
                    if (D == 3) gsum[2] = gRi[2] + Gj.z;
                    Rrho_d.add(volj * ((drho_j - drho_i) + 0.5f * fdot<D>(gsum, Rji)) * rg * idist2);
                }
                const float vdotr = fdot<D>(Vji, Rji);
                const float c = m_j * f_art_visc(f, vdotr, idist2, rho_i, rho_j);
#pragma unroll
                for (int k = 0; k < D; ++k) art[k] += c * g[k];
            } else if (!nodsph) {
                Rrho_d.add(volj * (drho_j - drho_i) * rg * idist2);
            }
        }
    }

    __device__ __forceinline__ void finish(const Params &P, const DevState &W, int64_t i, const double *aero,
                                           bool aero_on) {
        double accd[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            accd[k] = aero[k] + acc[k].value();
            if (linear) accd[k] /= to_f64(rho_i);
        }
        if (csf) {
            const double c = 1.0 / W.rho[i] * P.sig * W.curve[i] * W.colourG[i];
#pragma unroll
            for (int k = 0; k < D; ++k) accd[k] += c * W.norm[k][i];
        }
        const float inv_m = 1.f / m_i; /* the surface-tension sum is FP32 already */
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double av = NOFROZEN ? to_f64(art[k]) : W.aVisc[k][i];
            double t = accd[k];
            if (ALE) t += to_f64(acc_ale[k]);
            W.acc[k][i] = t + av + to_f64(visc[k]) + to_f64(st[k] * inv_m) + P.grav[k];
            if (aero_on) W.Af[k][i] = aero[k];
        }
        double R = Rrho.value() * to_f64(rho_i);
        if (ALE) R += Rrhoc.value();
        if (!nodsph) R += NOFROZEN ? P.dsph_cont * Rrho_d.value() : W.deltaD[i];
        W.Rrho[i] = R;
    }
};

/* The residual of slot i; called by whole warps (the learned closure runs on whole warps), lanes
 * with live == false contribute nothing. */
template <int D, bool ALE, bool NOFROZEN>
__device__ __forceinline__ void resid_slot(const Params &P, const DevState &W, const DevNbr &N, const Packed &K,
                                           const double *npd_dev, const Closure &C, int64_t i, bool live) {
    /* the aerodynamic term first */
    double aero[D];
    bool aero_on;
    closure_aero<D>(P, W, C, K.N, K.G, i, live, live ? double(N.cnt[i]) : 0.0, aero_on, aero);
    if (!live) return;
    const Pf f = make_pf(P);
    const bool linear = has(P, FJSPH_VAR_LINEAR);
    const float4 Ai = K.A[i], Ci = K.C[i];
    const LoParts Li(K.Lo[i]);
    ResidAcc<D, ALE, NOFROZEN> ra;
    {
        float vi[3];
        vi[0] = Ci.x + Li.vl[0];
        vi[1] = Ci.y + Li.vl[1];
        vi[2] = Ci.z + Li.vl[2];
        ra.init(P, f, K, i, Ai.w, Ci.w, Li.pr, vi, npd_dev);
    }
    const SellList L = sell(N, i);
    /* software pipeline: after this pair's own gathers are issued, the next pair is read and its
     * neighbour's packed inputs are prefetched into L1 while this pair is computed; list rows
     * are fetched kListAhead ahead */
    const int32_t ahead = P.list_ahead > 0 ? P.list_ahead : kListAhead;
    /* the next kGatherAhead pairs wait in registers; the newest one's neighbour inputs are
     * prefetched into L1 when it is read, kGatherAhead iterations before they are gathered */
    int2 q[kGatherAhead];
#pragma unroll
    for (int a = 0; a < kGatherAhead; ++a) {
        q[a] = make_int2((int32_t)i, 0);
        if (a < L.n) {
            q[a] = L[a];
            if (a > 0) prefetch_pair_inputs(K, q[a].x, linear || ALE, NOFROZEN);
        }
    }
    for (int32_t r_ = kChunk; r_ < ahead && r_ < L.n; r_ += kChunk) prefetch_l1(L.at(r_));
    for (int32_t e = 0; e < L.n; ++e) {
        const int2 pe = q[0];
        if (((e + ahead) % kChunk) == 0 && e + ahead < L.n) prefetch_l1(L.at(e + ahead)); /* next chunk */
        const int32_t j = pe.x;
        const float4 Aj = K.A[j], Cj = K.C[j], Qj = K.Lo[j];
#pragma unroll
        for (int a = 0; a + 1 < kGatherAhead; ++a) q[a] = q[a + 1];
        if (e + kGatherAhead < L.n) {
            q[kGatherAhead - 1] = L[e + kGatherAhead];
            prefetch_pair_inputs(K, q[kGatherAhead - 1].x, linear || ALE, NOFROZEN);
        }
        if (j == i) continue;
        const LoParts Lj(Qj);
        /* separations: high parts, then the (bf16) low parts */
        float Rji[D], Vji[D], vj[D];
        Rji[0] = (Aj.x - Ai.x) + (Lj.xl[0] - Li.xl[0]);
        Rji[1] = (Aj.y - Ai.y) + (Lj.xl[1] - Li.xl[1]);
        if (D == 3) Rji[2] = (Aj.z - Ai.z) + (Lj.xl[2] - Li.xl[2]);
        Vji[0] = (Cj.x - Ci.x) + (Lj.vl[0] - Li.vl[0]);
        Vji[1] = (Cj.y - Ci.y) + (Lj.vl[1] - Li.vl[1]);
        if (D == 3) Vji[2] = (Cj.z - Ci.z) + (Lj.vl[2] - Li.vl[2]);
        if (ALE) {
            vj[0] = Cj.x + Lj.vl[0];
            vj[1] = Cj.y + Lj.vl[1];
            if (D == 3) vj[2] = Cj.z + Lj.vl[2];
        }
        ra.pair(f, K, j, Rji, Vji, vj, Aj.w, Cj.w, Lj.pr, Lj.flags, __int_as_float(pe.y));
    }
    ra.finish(P, W, i, aero, aero_on);
}

template <int D, bool ALE, bool NOFROZEN>
__global__ void __launch_bounds__(kThreads, 7) k_m_resid(const __grid_constant__ Params P, const __grid_constant__ DevState W,
                                                      const __grid_constant__ DevNbr N, const __grid_constant__ Packed K,
                                                      const double *npd_dev, const __grid_constant__ Closure C) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    resid_slot<D, ALE, NOFROZEN>(P, W, N, K, npd_dev, C, i, i < P.n);
}

/* The same over one resident grid in the SM-local order (claim_chunk).  A separate kernel: the
 * compiler contracts the particle body's products and sums into fused multiply-adds per copy,
 * so the two orders agree to FP32 rounding, not bit for bit. */
template <int D, bool ALE, bool NOFROZEN>
__global__ void __launch_bounds__(kThreads, 7) k_m_resid_sm(const __grid_constant__ Params P,
                                                         const __grid_constant__ DevState W,
                                                         const __grid_constant__ DevNbr N,
                                                         const __grid_constant__ Packed K, const double *npd_dev,
                                                         const __grid_constant__ Closure C) {
    const int64_t chunks = (P.n - P.nb + 31) / 32;
    for (int64_t c = claim_chunk(P.region_next, chunks); c >= 0; c = claim_chunk(P.region_next, chunks)) {
        const int64_t i = P.nb + 32 * c + (threadIdx.x & 31);
        resid_slot<D, ALE, NOFROZEN>(P, W, N, K, npd_dev, C, i, i < P.n);
    }
}

/* The residual over shared-memory tiles: each CTA stages a tile's halo as tile-relative records
 * and every lane walks one fluid particle's members with a cursor over its mask, the lanes of a
 * warp in step through the pair arithmetic. */
template <int D, bool ALE, bool NOFROZEN>
__global__ void __launch_bounds__(kTileThreads, 3) k_t_resid(const __grid_constant__ Params P,
                                                              const __grid_constant__ DevState W, CellGrid G, TileDev T,
                                                              const __grid_constant__ Packed K, const double *npd_dev,
                                                              const __grid_constant__ Closure C) {
    using TT = Tile<D>;
    extern __shared__ __align__(16) unsigned char tsm[];
    TileSmem ts = tile_smem<D>(tsm, T.smax, kStageRel);
    const TileGrid tg = tile_grid<D>(G);
    const Pf f = make_pf(P);
    const float edge[3] = {(float)P.cell_edge[0], (float)P.cell_edge[1], (float)P.cell_edge[2]};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int ntl = *T.count;
    for (int it = blockIdx.x; it < ntl; it += gridDim.x) {
        tile_setup<D>(P, G, K, tg, T.list[it], kStageRel, kOwnFluid, ts);
        const bool over = ts.over();
        const int nown = ts.nown();
        for (int base = wid * 32; base < nown; base += kTileThreads) {
            const int k = base + lane;
            const bool live = k < nown;
            TileOwnRef o{};
            int64_t i = 0;
            int nn = 0;
            if (live) {
                o = tile_own<D>(ts, k);
                i = tile_slot(G, ts, o.e, o.hc / TT::HX);
                nn = tile_member_count(T.mask, T.stride, o.g);
            }
            double aero[D];
            bool aero_on;
            closure_aero<D>(P, W, C, K.N, K.G, i, live, double(nn), aero_on, aero);
            if (!live) continue;
            float4 Pi, Vi, Ti;
            tile_ld_rel<D>(ts, G, K, o.e, o.hc / TT::HX, over, Pi, Vi, Ti);
            const float *fr = ts.frame;
            float vi[3];
            vi[0] = fr[6] + (fr[9] + Vi.x);
            vi[1] = fr[7] + (fr[10] + Vi.y);
            vi[2] = fr[8] + (fr[11] + Vi.z);
            ResidAcc<D, ALE, NOFROZEN> ra;
            ra.init(P, f, K, i, Pi.w, Vi.w, __uint_as_float(__float_as_uint(Ti.w) & ~3u), vi, npd_dev);
            TileCursor<D> cur;
            cur.init(ts, o, T.mask, T.stride);
            TileNbr n;
            while (cur.next_member(n)) {
                if (n.e == o.e) continue;
                float4 Pj, Vj, Tj;
                tile_ld_rel<D>(ts, G, K, n.e, n.row, over, Pj, Vj, Tj);
                float Rji[D], Vji[D], vj[D];
                Rji[0] = Pj.x - Pi.x;
                Rji[1] = Pj.y - Pi.y;
                if (D == 3) Rji[2] = Pj.z - Pi.z;
                Vji[0] = Vj.x - Vi.x;
                Vji[1] = Vj.y - Vi.y;
                if (D == 3) Vji[2] = Vj.z - Vi.z;
                if (ALE) {
                    vj[0] = fr[6] + (fr[9] + Vj.x);
                    vj[1] = fr[7] + (fr[10] + Vj.y);
                    if (D == 3) vj[2] = fr[8] + (fr[11] + Vj.z);
                }
                const uint32_t tw = __float_as_uint(Tj.w);
                const int32_t j = ra.needs_slot() ? tile_slot(G, ts, n.e, n.row) : 0;
                ra.pair(f, K, j, Rji, Vji, vj, Pj.w, Vj.w, __uint_as_float(tw & ~3u), tw & 3u,
                        tile_r2<D>(Ti, Tj, n, edge));
            }
            ra.finish(P, W, i, aero, aero_on);
        }
        __syncthreads();
    }
}

__global__ void k_permute_f4(const float4 *src, float4 *dst, const int32_t *new_of_old, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && new_of_old[i] >= 0) dst[new_of_old[i]] = src[i];
}

/* block size of the pair sweeps: the tuned value (<= kThreads, the compiled maximum) */
inline int sweep_bs(const Params &P) { return P.sweep_threads > 0 ? P.sweep_threads : kThreads; }
inline int resid_bs(const Params &P) { return P.resid_threads > 0 ? P.resid_threads : kThreads; }
inline unsigned fgrid(const Params &P) { return grid_for(P.n - P.nb, sweep_bs(P)); }
inline unsigned bgrid(const Params &P) { return grid_for(P.nb, sweep_bs(P)); }
inline unsigned agrid(const Params &P) { return grid_for(P.n, sweep_bs(P)); }

} // namespace

#define FJSPH_DISPATCH_M(P, KERNEL, GRID, ...)                                             \
    do {                                                                                   \
        if ((GRID) == 0) break;                                                            \
        if ((P).D == 2)                                                                    \
            KERNEL<2><<<(GRID), sweep_bs(P), 0, s>>>(__VA_ARGS__);                         \
        else                                                                               \
            KERNEL<3><<<(GRID), sweep_bs(P), 0, s>>>(__VA_ARGS__);                         \
    } while (0)

void launch_m_pack(const Params &P, const DevState &W, const Packed &K, int64_t i0, int64_t i1, int full,
                   cudaStream_t s) {
    if (i1 <= i0) return;
    const unsigned g = grid_for(i1 - i0, 256);
    if (P.D == 2)
        k_pack_state<2><<<g, 256, 0, s>>>(P, W, K, i0, i1, full);
    else
        k_pack_state<3><<<g, 256, 0, s>>>(P, W, K, i0, i1, full);
}
void launch_m_permute_f4(const float4 *src, float4 *dst, const int32_t *new_of_old, int64_t n, cudaStream_t s) {
    if (n > 0) k_permute_f4<<<grid_for(n, 256), 256, 0, s>>>(src, dst, new_of_old, n);
}
void launch_m_npd(const Params &P, const DevNbr &N, const Packed &K, double *npd_part, cudaStream_t s) {
    FJSPH_DISPATCH_M(P, k_m_npd, agrid(P), P, N, K, npd_part);
}
void launch_m_dsph(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, double *npd_part,
                   cudaStream_t s) {
    FJSPH_DISPATCH_M(P, k_m_dsph, agrid(P), P, W, N, K, npd_part);
}
void launch_m_surface(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, bool with_dissipation,
                      cudaStream_t s) {
    if (fgrid(P) > 0) {
        if (with_dissipation) {
            if (P.D == 2)
                k_m_surface_normal<2, true><<<fgrid(P), sweep_bs(P), 0, s>>>(P, W, N, K);
            else
                k_m_surface_normal<3, true><<<fgrid(P), sweep_bs(P), 0, s>>>(P, W, N, K);
        } else {
            if (P.D == 2)
                k_m_surface_normal<2, false><<<fgrid(P), sweep_bs(P), 0, s>>>(P, W, N, K);
            else
                k_m_surface_normal<3, false><<<fgrid(P), sweep_bs(P), 0, s>>>(P, W, N, K);
        }
    }
    FJSPH_DISPATCH_M(P, k_m_surface_curvature, fgrid(P), P, W, N, K);
}
void launch_m_dissipation(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, cudaStream_t s) {
    FJSPH_DISPATCH_M(P, k_m_dissipation, fgrid(P), P, W, N, K);
}
void launch_m_particle_shift(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, cudaStream_t s) {
    FJSPH_DISPATCH_M(P, k_m_particle_shift, fgrid(P), P, W, N, K);
}
void launch_m_bound_pressure(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, cudaStream_t s) {
    FJSPH_DISPATCH_M(P, k_m_bound_pressure, bgrid(P), P, W, N, K);
}
void launch_m_bound_ghost(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, int32_t *near_inlet,
                          cudaStream_t s) {
    FJSPH_DISPATCH_M(P, k_m_bound_ghost, bgrid(P), P, W, N, K, near_inlet);
}
/* Blocks of `bs` threads of `kernel` resident on the whole device at once: the grid of the
 * SM-local order. */
template <typename F>
unsigned resident_grid(F kernel, int bs) {
    int dev = 0, sms = 1, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, bs, 0) != cudaSuccess || per < 1) per = 1;
    return (unsigned)(sms * per);
}

template <int D, bool A, bool NF>
void m_resid_launch(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, const double *npd_dev,
                    const Closure &C, unsigned g, cudaStream_t s) {
    const int bs = resid_bs(P);
    if (!P.sm_order) {
        k_m_resid<D, A, NF><<<g, bs, 0, s>>>(P, W, N, K, npd_dev, C);
        return;
    }
    /* resident blocks, computed once per instantiation and block size (64 or 128) */
    static std::atomic<unsigned> cached[2] = {0u, 0u};
    std::atomic<unsigned> &cg = cached[bs == 64 ? 0 : 1];
    unsigned rg = cg.load(std::memory_order_relaxed);
    if (rg == 0u || (bs != 64 && bs != 128)) {
        rg = resident_grid(k_m_resid_sm<D, A, NF>, bs);
        if (bs == 64 || bs == 128) cg.store(rg, std::memory_order_relaxed);
    }
    cudaMemsetAsync(P.region_next, 0, sizeof(int32_t) * kMaxRegions, s);
    k_m_resid_sm<D, A, NF><<<std::min(g, rg), bs, 0, s>>>(P, W, N, K, npd_dev, C);
}

void launch_m_resid(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, const double *npd_dev,
                    const Closure &C, cudaStream_t s) {
    const unsigned g = grid_for(P.n - P.nb, resid_bs(P));
    if (g == 0) return;
    const bool ale = has(P, FJSPH_VAR_ALE), nf = has(P, FJSPH_VAR_NOFROZEN);
#define FJSPH_RESID_M(DD, A, NF) m_resid_launch<DD, A, NF>(P, W, N, K, npd_dev, C, g, s)
    if (P.D == 2) {
        if (ale)
            nf ? FJSPH_RESID_M(2, true, true) : FJSPH_RESID_M(2, true, false);
        else
            nf ? FJSPH_RESID_M(2, false, true) : FJSPH_RESID_M(2, false, false);
    } else {
        if (ale)
            nf ? FJSPH_RESID_M(3, true, true) : FJSPH_RESID_M(3, true, false);
        else
            nf ? FJSPH_RESID_M(3, false, true) : FJSPH_RESID_M(3, false, false);
    }
#undef FJSPH_RESID_M
}

template <int D, bool A, bool NF>
void t_resid_launch(const Params &P, const DevState &W, const CellGrid &G, const TileDev &T, const Packed &K,
                    const double *npd_dev, const Closure &C, cudaStream_t s) {
    const size_t sm = tile_smem_bytes<D>(T.smax, kStageRel); /* smax is fixed for a context */
    /* the shared-memory attribute and the resident grid, set once per instantiation (a function-local
     * static is initialised exactly once, whichever host thread gets here first) */
    static const unsigned grid = [sm] {
        if (sm > 48 * 1024)
            cudaFuncSetAttribute(k_t_resid<D, A, NF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        int dev = 0, sms = 1, per = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_t_resid<D, A, NF>, kTileThreads, sm) != cudaSuccess ||
            per < 1)
            per = 1;
        return (unsigned)(sms * per);
    }();
    k_t_resid<D, A, NF><<<grid, kTileThreads, sm, s>>>(P, W, G, T, K, npd_dev, C);
}

void launch_t_resid(const Params &P, const DevState &W, const CellGrid &G, const TileDev &T, const Packed &K,
                    const double *npd_dev, const Closure &C, cudaStream_t s) {
    const bool ale = has(P, FJSPH_VAR_ALE), nf = has(P, FJSPH_VAR_NOFROZEN);
    if (P.D == 2) {
        if (ale)
            nf ? t_resid_launch<2, true, true>(P, W, G, T, K, npd_dev, C, s) : t_resid_launch<2, true, false>(P, W, G, T, K, npd_dev, C, s);
        else
            nf ? t_resid_launch<2, false, true>(P, W, G, T, K, npd_dev, C, s) : t_resid_launch<2, false, false>(P, W, G, T, K, npd_dev, C, s);
    } else {
        if (ale)
            nf ? t_resid_launch<3, true, true>(P, W, G, T, K, npd_dev, C, s) : t_resid_launch<3, true, false>(P, W, G, T, K, npd_dev, C, s);
        else
            nf ? t_resid_launch<3, false, true>(P, W, G, T, K, npd_dev, C, s) : t_resid_launch<3, false, false>(P, W, G, T, K, npd_dev, C, s);
    }
}

} // namespace fjsph
