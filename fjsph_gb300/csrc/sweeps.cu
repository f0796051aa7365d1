/*
 * sweeps.cu -- the per-particle neighbour sweeps of one WCSPH step, FP64 form.
 *
 * One thread owns one particle and walks its CSR neighbour list.  Neighbour data are gathered
 * from slot-ordered SoA arrays; slots are cell-sorted, so neighbouring threads share most of
 * their neighbours through L1/L2.  The squared distance of a pair is re-evaluated from the
 * positions frozen at search time (xs), which reproduces the reference's stored `jj.second`
 * bit for bit, while the separation vector uses current positions (src/Resid.cpp:286-290).
 */
#include "aero.cuh"
#include "kernels.h"
#include "linalg.cuh"

namespace fjsph {

namespace {

constexpr int kThreads = 128;

template <int D>
__device__ __forceinline__ double pair_rr(const DevNbr &N, int64_t i, int64_t j) {
    double a[D], b[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        a[k] = N.xs[k][i];
        b[k] = N.xs[k][j];
    }
    return dist2<D>(a, b);
}

/* ------------------------------------------------------------------------------------------ */
/* dSPH_PreStep (src/Shifting.cpp:12-123), all slots                                            */
/* ------------------------------------------------------------------------------------------ */
/* The per-particle quotients the FP64 pair sweeps take from their neighbour (ResidQuot): m / rho,
 * p / rho^2, 1 / rho and sqrt(B gamma / rho), once per particle and sweep instead of once per pair
 * (on this GPU the FP64 form is bound by its FP64 pipe, and a divide or a square root is a long
 * sequence on it).  Each is the expression the pair term evaluated, so the values are unchanged. */
__global__ void k_resid_quotients(Params P, DevState W, ResidQuot *Q) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const double rho = W.rho[i];
    Q[i] = ResidQuot{W.m[i] / rho, W.p[i] / (rho * rho), 1.0 / rho, sqrt((P.B * P.gam) / rho)};
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_dsph_prestep(Params P, DevState W, DevNbr N, double *npd_part,
                                                            const ResidQuot *Q) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const bool cubic = has(P, FJSPH_VAR_CUBIC);
    double xi[D];
    load3<D>(W.x, i, xi);
    const double rho_i = W.rho[i];
    double Lm[D * D], Lnb[D * D], gR[D], nr[D];
#pragma unroll
    for (int k = 0; k < D * D; ++k) {
        Lm[k] = 0.0;
        Lnb[k] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
        gR[k] = 0.0;
        nr[k] = 0.0;
    }
    double kernsum = 0.0, colour = 0.0, npd = 0.0;
    const int64_t e0 = N.off[i], e1 = N.off[i + 1];
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t j = N.idx[e];
        if (j == i) {
            kernsum += P.W_correc;
            continue;
        }
        double Rji[D];
#pragma unroll
        for (int k = 0; k < D; ++k) Rji[k] = W.x[k][j] - xi[k];
        const double r = sqrt(pair_rr<D>(N, i, j));
        const double volj = Q[j].vol;
        const double kern = kernel_w<double>(r, P.H, P.W_correc, cubic);
        const double gs = gradk_scale<double>(r, P.H, P.W_correc, cubic);
        double Grad[D];
#pragma unroll
        for (int k = 0; k < D; ++k) Grad[k] = -Rji[k] * gs;
        const bool fl = W.b[j] > FJSPH_PISTON;
        const double drho = volj * (W.rho[j] - rho_i);
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const double vr = volj * Rji[a];
#pragma unroll
            for (int c = 0; c < D; ++c) {
                Lm[a * D + c] -= vr * Grad[c];
                if (fl) Lnb[a * D + c] -= vr * Grad[c];
            }
            gR[a] += drho * Grad[a];
        }
        if (fl) {
#pragma unroll
            for (int k = 0; k < D; ++k) nr[k] += volj * Grad[k];
            kernsum += kern;
            colour += volj * kern;
            npd += kern;
        }
    }
    double Linv[D * D];
    if (!qr_inverse<D>(Lm, Linv)) {
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int c = 0; c < D; ++c) Linv[a * D + c] = (a == c) ? 1.0 : 0.0;
    }
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double g = 0.0, n = 0.0;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            g += Linv[a * D + c] * gR[c];
            n += Linv[a * D + c] * nr[c];
        }
        W.gradRho[a][i] = g;
        W.norm[a][i] = n;
    }
#pragma unroll
    for (int k = 0; k < D * D; ++k) W.L[k][i] = Linv[k];
    double lam, lam_nb;
    if (W.b[i] == FJSPH_BOUND) {
        lam = 1.0;
        lam_nb = 1.0;
    } else {
        lam = min_eig<D>(Lm);
        lam_nb = min_eig<D>(Lnb);
    }
    W.lam[i] = lam;
    W.lam_nb[i] = lam_nb;
    W.colourG[i] = (lam > 0.7) ? 2.0 : 2.0 * fmax(1.0, 1.0 / (2.0 * colour));
    W.kernsum[i] = kernsum;
    W.colour[i] = colour;
    npd_part[i] = npd;
}

/* Numerical particle density alone: the npd sum of dSPH_PreStep without its other outputs. */
template <int D>
__global__ void __launch_bounds__(kThreads) k_npd_only(Params P, DevState W, DevNbr N, double *npd_part) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const bool cubic = has(P, FJSPH_VAR_CUBIC);
    double npd = 0.0;
    for (int64_t e = N.off[i]; e < N.off[i + 1]; ++e) {
        const int64_t j = N.idx[e];
        if (j == i || W.b[j] <= FJSPH_PISTON) continue;
        npd += kernel_w<double>(sqrt(pair_rr<D>(N, i, j)), P.H, P.W_correc, cubic);
    }
    npd_part[i] = npd;
}

/* ------------------------------------------------------------------------------------------ */
/* get_aero_velocity, constVel source (src/Resid.cpp:569-611), fluid slots                     */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void k_aero_velocity(Params P, DevState W, DevNbr N) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    bool on;
    if (P.use_lam)
        on = W.lam_nb[i] < P.lam_cutoff && W.b[i] == FJSPH_FREE;
    else
        on = double(nbr_range(N, i).n) * P.i_n_full < P.lam_cutoff && W.b[i] == FJSPH_FREE;
#pragma unroll
    for (int k = 0; k < D; ++k) W.cellV[k][i] = on ? vinf_of(P, i, k) : 0.0;
    W.cellID[i] = on ? 1 : kNoCell;
}

/* ------------------------------------------------------------------------------------------ */
/* Detect_Surface (src/Geometry.cpp:14-280), fluid slots, three passes                         */
/* ------------------------------------------------------------------------------------------ */
/* pass 1: surface flag (Marrone et al. 2010) and the eigenvalue-gradient normal */
template <int D>
__global__ void __launch_bounds__(kThreads) k_surface_normal(Params P, DevState W, DevNbr N, double *nrm0,
                                                              double *nrm1, double *nrm2, const ResidQuot *Q) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    double *const nrm_tmp[3] = {nrm0, nrm1, nrm2};
    const bool cubic = has(P, FJSPH_VAR_CUBIC);
    const double h = 1.33 * P.particle_step;
    double xi[D], ni[D], nh[D];
    load3<D>(W.x, i, xi);
    load3<D>(W.norm, i, ni);
    normalized<D, double>(ni, nh);
    const int b = W.b[i];
    const double lam_nb = W.lam_nb[i], lam = W.lam[i];
    const int64_t e0 = N.off[i], e1 = N.off[i + 1];
    /* the geometric test of the surface band runs inside the normal's walk below: a neighbour
     * inside the test region clears the flag, and once it is clear the test is skipped (the flag
     * a walk that stops at the first such neighbour gives, src/Geometry.cpp) */
    int surf = 0;
    bool test = false;
    double pointT[D], th[D];
    if (b < FJSPH_PIPE) {
        W.woccl[i] = 1.0;
    } else if (lam_nb < 0.2) {
        surf = 1;
    } else if (lam_nb < 0.75) {
#pragma unroll
        for (int k = 0; k < D; ++k) pointT[k] = xi[k] + h * nh[k];
        if (D == 2) {
            double tau[D];
            tau[0] = ni[1];
            tau[1] = -ni[0];
            normalized<D, double>(tau, th);
        }
        surf = 1;
        test = true;
    }
    double nrm[D];
#pragma unroll
    for (int k = 0; k < D; ++k) nrm[k] = 0.0;
    const bool inside = lam > 0.7;
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t j = N.idx[e];
        if (j == i) continue;
        double xj[D], Rij[D];
        load3<D>(W.x, j, xj);
#pragma unroll
        for (int k = 0; k < D; ++k) Rij[k] = xi[k] - xj[k];
        const double r = sqrt(pair_rr<D>(N, i, j));
        if (test && surf) {
            double x_jT[D];
#pragma unroll
            for (int k = 0; k < D; ++k) x_jT[k] = xj[k] - pointT[k];
            if (r >= sqrt(2.0) * h) {
                if (vnorm<D, double>(x_jT) < h) surf = 0;
            } else if (D == 2) {
                if ((fabs(dot<D, double>(nh, x_jT)) + fabs(dot<D, double>(th, x_jT))) < h) surf = 0;
            } else {
                double u[D];
#pragma unroll
                for (int k = 0; k < D; ++k) u[k] = -(xi[k] - xj[k]) / r;
                if (acos(dot<D, double>(nh, u)) < kPi / 4.0) surf = 0;
            }
        }
        const double volj = Q[j].vol;
        const double gs = gradk_scale<double>(r, P.H, P.W_correc, cubic);
        const double w = inside ? volj * (W.lam[j] - lam) : volj * W.lam[j];
#pragma unroll
        for (int k = 0; k < D; ++k) nrm[k] += w * (Rij[k] * gs);
    }
    W.surf[i] = surf;
    double n2[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double s = 0.0;
#pragma unroll
        for (int c = 0; c < D; ++c) s += W.L[a * D + c][i] * nrm[c];
        n2[a] = s;
    }
    double out[D];
    if (vnorm<D, double>(n2) > 0.1 * lam / P.H) {
        normalized<D, double>(n2, out);
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) nrm_tmp[k][i] = out[k];
}

/* pass 2: curvature from the normals and the Gissler occlusion factor */
template <int D>
__global__ void __launch_bounds__(kThreads) k_surface_curvature(Params P, DevState W, DevNbr N, const double *nrm0,
                                                                 const double *nrm1, const double *nrm2,
                                                                 const ResidQuot *Q) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const double *const nt[3] = {nrm0, nrm1, nrm2};
    const bool cubic = has(P, FJSPH_VAR_CUBIC);
    const bool gissler = P.acase == FJSPH_GISSLER;
    const int b = W.b[i];
    double xi[D], vi[D], ni[D], Vdiff[D];
    load3<D>(W.x, i, xi);
    load3<D>(W.v, i, vi);
#pragma unroll
    for (int k = 0; k < D; ++k) ni[k] = nt[k][i];
    const bool occl = (b == FJSPH_FREE) && gissler;
#pragma unroll
    for (int k = 0; k < D; ++k) Vdiff[k] = (occl && W.cellID[i] != -1) ? vinf_of(P, i, k) - vi[k] : 0.0;
    double Li[D * D];
#pragma unroll
    for (int k = 0; k < D * D; ++k) Li[k] = W.L[k][i];
    const double nin = vnorm<D, double>(ni), vdn = vnorm<D, double>(Vdiff);
    double curve = 0.0, woccl_ = 0.0;
    /* ALE/TIC builds: the surface zone (any neighbour, self included, on the surface) rides along */
    const bool zone = has(P, FJSPH_VAR_ALE) || has(P, FJSPH_VAR_TIC);
    int sz = 0;
    const int64_t e0 = N.off[i], e1 = N.off[i + 1];
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t j = N.idx[e];
        if (zone && !sz && W.surf[j] == 1) sz = 1;
        if (j == i) continue;
        double Rij[D];
#pragma unroll
        for (int k = 0; k < D; ++k) Rij[k] = W.x[k][j] - xi[k];
        const double r = sqrt(pair_rr<D>(N, i, j));
        double nj[D];
#pragma unroll
        for (int k = 0; k < D; ++k) nj[k] = nt[k][j];
        if (nin > 0.0 && vnorm<D, double>(nj) > 0.0) {
            const double volj = Q[j].vol;
            const double gs = gradk_scale<double>(r, P.H, P.W_correc, cubic);
            double s = 0.0;
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double Ld = 0.0;
#pragma unroll
                for (int c = 0; c < D; ++c) Ld += Li[a * D + c] * (nj[c] - ni[c]);
                s += Ld * (Rij[a] * gs);
            }
            curve += volj * s;
        }
        if (occl) {
            const double frac = -dot<D, double>(Rij, Vdiff) / (vdn * r);
            if (frac > woccl_) woccl_ = frac;
        }
    }
    W.woccl[i] = (W.lam_nb[i] < P.lam_cutoff) ? fmax(0.0, fmin(woccl_, 1.0)) : 1.0;
#pragma unroll
    for (int k = 0; k < D; ++k) W.norm[k][i] = ni[k];
    W.curve[i] = curve;
    W.norm_curve[i] = P.dx * curve;
    W.pDist[i] = W.lam[i];
    if (zone) W.surfzone[i] = sz;
}

/* ------------------------------------------------------------------------------------------ */
/* Artificial viscosity (src/Kernel.h:217-244): returns the scalar multiplying gradK.           */
/* ------------------------------------------------------------------------------------------ */
/* cs_i, cs_j: sqrt(B gamma / rho) of both particles (ResidQuot::cs) */
__device__ __forceinline__ double art_visc_scale(const Params &P, double vdotr, double idist2, double rho_i,
                                                 double rho_j, double cs_i, double cs_j) {
    if (vdotr > 0.0) return 0.0;
    const double muij = P.H * vdotr * idist2;
    const double rhoij = 0.5 * (rho_i + rho_j);
    const double cbar = 0.5 * (cs_i + cs_j);
    return P.visc_alpha * cbar * muij / rhoij;
}

/* ------------------------------------------------------------------------------------------ */
/* dissipation_terms (src/Shifting.cpp:126-186), fluid slots                                   */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void __launch_bounds__(kThreads) k_dissipation(Params P, DevState W, DevNbr N, const ResidQuot *Q) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const bool cubic = has(P, FJSPH_VAR_CUBIC), linear = has(P, FJSPH_VAR_LINEAR), nodsph = has(P, FJSPH_VAR_NODSPH);
    double xi[D], vi[D], gRi[D];
    load3<D>(W.x, i, xi);
    load3<D>(W.v, i, vi);
    load3<D>(W.gradRho, i, gRi);
    const double rho_i = W.rho[i], cs_i = Q[i].cs;
    double av[D];
#pragma unroll
    for (int k = 0; k < D; ++k) av[k] = 0.0;
    double Rrhod = 0.0;
    const int64_t e0 = N.off[i], e1 = N.off[i + 1];
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t j = N.idx[e];
        if (j == i) continue;
        double Rji[D], Vji[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            Rji[k] = W.x[k][j] - xi[k];
            Vji[k] = W.v[k][j] - vi[k];
        }
        const double rr = pair_rr<D>(N, i, j);
        const double r = sqrt(rr);
        const double idist2 = 1.0 / (rr + 0.0001 * P.H_sq);
        const double rho_j = W.rho[j];
        const double volj = Q[j].vol;
        const double gs = gradk_scale<double>(r, P.H, P.W_correc, cubic);
        double g[D];
#pragma unroll
        for (int k = 0; k < D; ++k) g[k] = Rji[k] * gs;
        const bool fl = W.b[j] > FJSPH_PISTON;
        if (fl) {
            const double vdotr = dot<D, double>(Vji, Rji);
            const double c =
                linear ? volj * idist2 * vdotr : W.m[j] * art_visc_scale(P, vdotr, idist2, rho_i, rho_j, cs_i, Q[j].cs);
#pragma unroll
            for (int k = 0; k < D; ++k) av[k] += c * g[k];
        }
        if (!nodsph) {
            const double rg = dot<D, double>(Rji, g);
            double t = rho_j - rho_i;
            if (fl) {
                double gs2[D];
#pragma unroll
                for (int k = 0; k < D; ++k) gs2[k] = gRi[k] + W.gradRho[k][j];
                t += 0.5 * dot<D, double>(gs2, Rji);
            }
            Rrhod += volj * t * rg * idist2;
        }
    }
    if (linear) {
        const double c = P.visc_alpha * P.H * P.speed_sound * P.rho_rest / rho_i;
#pragma unroll
        for (int k = 0; k < D; ++k) av[k] *= c;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) W.aVisc[k][i] = av[k];
    if (!nodsph) W.deltaD[i] = P.dsph_cont * Rrhod;
}

/* ------------------------------------------------------------------------------------------ */
/* particle_shift (src/Shifting.cpp:189-290, -DALE), fluid slots                               */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void __launch_bounds__(kThreads) k_particle_shift(Params P, DevState W, DevNbr N, const ResidQuot *Q) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const double lam_nb = W.lam_nb[i];
    if (lam_nb < 0.55 || W.b[i] == FJSPH_BUFFER) {
#pragma unroll
        for (int k = 0; k < D; ++k) W.vPert[k][i] = 0.0;
        return;
    }
    const bool cubic = has(P, FJSPH_VAR_CUBIC);
    double xi[D], vi[D], ni[D], nh[D];
    load3<D>(W.x, i, xi);
    load3<D>(W.v, i, vi);
    load3<D>(W.norm, i, ni);
    normalized<D, double>(ni, nh);
    double dU[D];
#pragma unroll
    for (int k = 0; k < D; ++k) dU[k] = 0.0;
    double maxUij = 0.0, woccl = 0.0;
    const int64_t e0 = N.off[i], e1 = N.off[i + 1];
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t j = N.idx[e];
        if (j == i) continue;
        double Rji[D], dv[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            Rji[k] = W.x[k][j] - xi[k];
            dv[k] = W.v[k][j] - vi[k];
        }
        const double r = sqrt(pair_rr<D>(N, i, j));
        const double volj = Q[j].vol;
        const double kern = kernel_w<double>(r, P.H, P.W_correc, cubic);
        const double gs = gradk_scale<double>(r, P.H, P.W_correc, cubic);
        const double q = kern / P.W_dx;
        const double q2 = q * q;
        const double c = (1.0 + 0.2 * (q2 * q2));
#pragma unroll
        for (int k = 0; k < D; ++k) dU[k] += c * (Rji[k] * gs) * volj;
        if (W.b[j] > FJSPH_PISTON) {
            double nj[D], njh[D];
            load3<D>(W.norm, j, nj);
            normalized<D, double>(nj, njh);
            const double theta = acos(dot<D, double>(nh, njh));
            if (theta > woccl) woccl = theta;
        }
        const double dvn = vnorm<D, double>(dv);
        if (dvn > maxUij) maxUij = dvn;
    }
    const double sc = -2.0 * P.H * vnorm<D, double>(vi);
#pragma unroll
    for (int k = 0; k < D; ++k) dU[k] *= sc;
    const double mag = fmin(vnorm<D, double>(dU), fmin(maxUij / 2.0, P.max_shift_vel));
    double dUn[D];
    normalized<D, double>(dU, dUn);
#pragma unroll
    for (int k = 0; k < D; ++k) dU[k] = mag * dUn[k];
    double out[D];
    if (W.surfzone[i] == 0 && lam_nb > 0.55) {
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = dU[k];
    } else if (woccl < kPi / 12.0) {
        double nn[D];
#pragma unroll
        for (int k = 0; k < D; ++k) nn[k] = -nh[k];
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double s = 0.0;
#pragma unroll
            for (int c = 0; c < D; ++c) s += ((a == c ? 1.0 : 0.0) - nn[a] * nn[c]) * dU[c];
            out[a] = s;
        }
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) W.vPert[k][i] = out[k];
}

/* ------------------------------------------------------------------------------------------ */
/* Check_Pipe_Outlet (src/Containment.cpp:822-894), analytic air source                        */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void k_pipe_outlet(Params P, DevState W, int32_t *kbits) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    if (W.b[i] != FJSPH_PIPE) return;
    const DevBlock &B = P.blocks[W.blk[i]];
    double s = W.x[0][i] * B.aero_norm[0];
#pragma unroll
    for (int k = 1; k < D; ++k) s += W.x[k][i] * B.aero_norm[k];
    if (s > B.aeroconst) {
        W.b[i] = FJSPH_FREE;
        /* the packed type bits follow (the packed fluid flag is set for both types) */
        if (kbits) kbits[i] = (kbits[i] & ~7) | FJSPH_FREE;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Boundary passes (src/Resid.cpp:21-186), boundary slots [0, nb)                               */
/* ------------------------------------------------------------------------------------------ */
template <int D>
__global__ void k_bound_velocity(Params P, DevState W, int nb_rule) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    const DevBlock &B = P.blocks[W.blk[i]];
#pragma unroll
    for (int k = 0; k < D; ++k) W.v[k][i] = nb_rule ? B.vel_nb[k] : B.vel_rk[k];
}

/* Set_No_Slip: the reference applies it per block after setting the block velocity; the mirror
 * velocity reads fluid velocities only, so the blocks are independent. */
template <int D>
__global__ void k_no_slip(Params P, DevState W, DevNbr N, double *vt0, double *vt1, double *vt2) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    double *const vt[3] = {vt0, vt1, vt2};
    const DevBlock &B = P.blocks[W.blk[i]];
    double vi[D];
    load3<D>(W.v, i, vi);
    if (B.no_slip) {
        const bool cubic = has(P, FJSPH_VAR_CUBIC);
        double vs[D], ks = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) vs[k] = 0.0;
        const NbrRange R = nbr_range(N, i); /* also used by the split-precision form */
        for (int32_t k = 0; k < R.n; ++k) {
            const int64_t j = nbr_slot(N, R, k);
            if (j == i || W.b[j] <= FJSPH_PISTON) continue;
            const double r = sqrt(pair_rr<D>(N, i, j));
            const double kern = kernel_w<double>(r, P.H, P.W_correc, cubic);
            ks += kern;
#pragma unroll
            for (int k = 0; k < D; ++k) vs[k] += W.v[k][j] * kern;
        }
        if (ks > 0.0)
#pragma unroll
            for (int k = 0; k < D; ++k) vi[k] = 2.0 * vi[k] - vs[k] / ks;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) vt[k][i] = vi[k];
}

template <int D>
__global__ void k_copy_bound_v(Params P, DevState W, const double *vt0, const double *vt1, const double *vt2) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    const double *const vt[3] = {vt0, vt1, vt2};
#pragma unroll
    for (int k = 0; k < D; ++k) W.v[k][i] = vt[k][i];
}

/* Get_Boundary_Pressure (Adami, Hu & Adams 2012), src/Resid.cpp:21-76 */
template <int D>
__global__ void __launch_bounds__(kThreads) k_bound_pressure(Params P, DevState W, DevNbr N) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    if (P.blocks[W.blk[i]].bound_solver != FJSPH_PRESSURE_G) return;
    const bool cubic = has(P, FJSPH_VAR_CUBIC);
    double xi[D];
    load3<D>(W.x, i, xi);
    int near = 0;
    double kernsum = 0.0, pkern = 0.0, acck[D];
#pragma unroll
    for (int k = 0; k < D; ++k) acck[k] = 0.0;
    for (int64_t e = N.off[i]; e < N.off[i + 1]; ++e) {
        const int64_t j = N.idx[e];
        if (W.b[j] <= FJSPH_PISTON) continue;
        const double r = sqrt(pair_rr<D>(N, i, j));
        const double rho_j = W.rho[j];
        const double kern = (W.m[j] / rho_j) * kernel_w<double>(r, P.H, P.W_correc, cubic);
        kernsum += kern;
        pkern += W.p[j] * kern;
#pragma unroll
        for (int k = 0; k < D; ++k) acck[k] += kern * rho_j * (xi[k] - W.x[k][j]);
        if (W.surfzone[j]) near = 1;
    }
    double p = 0.0;
    if (kernsum > 0.0) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) s += (P.grav[k] - W.acc[k][i]) * acck[k];
        p = (pkern + s) / kernsum;
        if (near) p = fmax(0.0, p);
    }
    W.p[i] = p;
    W.rho[i] = eos_density(P, p);
}

/* Boundary_Ghost (src/Resid.cpp:122-160): density rate of ghost walls and the near-inlet flag. */
template <int D>
__global__ void __launch_bounds__(kThreads) k_bound_ghost(Params P, DevState W, DevNbr N, int32_t *near_inlet) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    if (P.blocks[W.blk[i]].bound_solver != FJSPH_GHOST) return;
    const bool cubic = has(P, FJSPH_VAR_CUBIC);
    double xi[D], vi[D];
    load3<D>(W.x, i, xi);
    load3<D>(W.v, i, vi);
    double Rr = 0.0;
    int ni = 1;
    for (int64_t e = N.off[i]; e < N.off[i + 1]; ++e) {
        const int64_t j = N.idx[e];
        if (j == i) continue;
        const int bj = W.b[j];
        if (bj == FJSPH_PIPE || bj == FJSPH_FREE) ni = 0;
        const double r = sqrt(pair_rr<D>(N, i, j));
        const double volj = W.m[j] / W.rho[j];
        const double gs = gradk_scale<double>(r, P.H, P.W_correc, cubic);
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) s += (W.v[k][j] - vi[k]) * ((W.x[k][j] - xi[k]) * gs);
        Rr -= volj * s;
    }
    near_inlet[i] = ni;
    W.Rrho[i] = Rr * W.rho[i];
}

/* Boundary_DBC (src/Resid.cpp:78-117).  The reference scatters the DBC terms into an array indexed
 * by neighbour and then copies back only the boundary range, which the scatter never touches;
 * its observable effect is a zero boundary acceleration. */
template <int D>
__global__ void k_bound_dbc(Params P, DevState W) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    if (P.blocks[W.blk[i]].bound_solver != FJSPH_DBC) return;
#pragma unroll
    for (int k = 0; k < D; ++k) W.acc[k][i] = 0.0;
}

/* ------------------------------------------------------------------------------------------ */
/* Residual (src/Resid.cpp:243-469, src/Kernel.h:153-269, src/Aero.h:10-263), fluid slots       */
/* ------------------------------------------------------------------------------------------ */
/* Wendland gradient scale of gradk_scale from q = r / H and c5 = 5 / H^2 */
__device__ __forceinline__ double wendland_gscale(double q, double c5, double Wc) {
    if (q < 1e-12) return 0.0;
    const double b = 1.0 - 0.5 * q;
    return c5 * (b * b * b) * Wc;
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_resid(Params P, DevState W, DevNbr N, const double *npd_dev,
                                                    const ResidQuot *Q) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const bool cubic = has(P, FJSPH_VAR_CUBIC), ale = has(P, FJSPH_VAR_ALE), linear = has(P, FJSPH_VAR_LINEAR),
               nofrozen = has(P, FJSPH_VAR_NOFROZEN), nodsph = has(P, FJSPH_VAR_NODSPH), tic = has(P, FJSPH_VAR_TIC);
    const bool pairwise = P.st_model == FJSPH_ST_PAIRWISE, csf = P.st_model == FJSPH_ST_CSF;
    double npdm2 = 0.0;
    if (pairwise) {
        const double npd = npd_dev[grp_of(P, i)];
        const double H2 = 2.0 * P.H;
        const double lam = (6.0 / 81.0 * (H2 * H2 * H2) / (kPi * kPi * kPi * kPi) *
                            (9.0 / 4.0 * (kPi * kPi * kPi) - 6.0 * kPi - 4.0));
        npdm2 = (0.5 * P.sig / lam) / (npd * npd);
    }
    /* uniform factors, once per thread: the pair loop multiplies instead of dividing */
    const double inv_H = 1.0 / P.H, c5 = 5.0 / (P.H * P.H), pi3o4_H = 3.0 * kPi / 4.0 * inv_H;
    double xi[D], vi[D], vPi[D], gRi[D];
    load3<D>(W.x, i, xi);
    load3<D>(W.v, i, vi);
    if (ale) load3<D>(W.vPert, i, vPi);
    if (nofrozen) load3<D>(W.gradRho, i, gRi);
    const double rho_i = W.rho[i], p_i = W.p[i], m_i = W.m[i], inv_rho_i = Q[i].inv_rho;
    const int b_i = W.b[i], sz_i = W.surfzone[i];
    const int64_t pid_i = W.part_id[i];
    const int64_t e0 = N.off[i], e1 = N.off[i + 1];
    double acc[D], acc_ale[D], visc[D], st[D], art[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        acc[k] = 0.0;
        acc_ale[k] = 0.0;
        visc[k] = 0.0;
        st[k] = 0.0;
        art[k] = 0.0;
    }
    double Rrho = 0.0, Rrhoc = 0.0, Rrho_d = 0.0;
    if (W.cellID[i] != -1) {
        double Vd[D], aero[D];
#pragma unroll
        for (int k = 0; k < D; ++k) Vd[k] = W.cellV[k][i] - vi[k];
        aero_acc<D>(P, W, i, Vd, W.lam_nb[i], double(e1 - e0), aero);
#pragma unroll
        for (int k = 0; k < D; ++k) {
            acc[k] += aero[k];
            W.Af[k][i] = aero[k];
        }
    }
    const double a_i0 = p_i / (rho_i * rho_i);
    const double a_i = (tic && sz_i != 1) ? fabs(a_i0) : a_i0;
    const double p_lin_i = (tic && sz_i != 1) ? fabs(p_i) : p_i;
    const bool st_on = pairwise && (!ale || sz_i == 1);
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t j = N.idx[e];
        if (W.part_id[j] == pid_i) continue;
        double Rji[D], Vji[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            Rji[k] = W.x[k][j] - xi[k];
            Vji[k] = W.v[k][j] - vi[k];
        }
        const double rr = pair_rr<D>(N, i, j);
        const double r = sqrt(rr);
        const double idist2 = 1.0 / (rr + 0.001 * P.H_sq);
        const double rho_j = W.rho[j], m_j = W.m[j];
        const ResidQuot qj = Q[j];
        const int b_j = W.b[j];
        const double volj = qj.vol;
        const double gs = cubic ? gradk_scale<double>(r, P.H, P.W_correc, true) : wendland_gscale(r * inv_H, c5, P.W_correc);
        double g[D];
#pragma unroll
        for (int k = 0; k < D; ++k) g[k] = Rji[k] * gs;
        /* pressure (PressureContrib, src/Resid.cpp:188-210) */
        const double pc = linear ? (p_lin_i + W.p[j]) * volj : m_j * (a_i + qj.pr);
#pragma unroll
        for (int k = 0; k < D; ++k) acc[k] -= pc * g[k];
        /* laminar viscosity (Morris), src/Kernel.h:262-269 */
        const double rg = dot<D, double>(Rji, g);
        /* (rho_i + rho_j) / (rho_i rho_j) = 1 / rho_i + 1 / rho_j */
        const double vc = m_j * (P.nu * (inv_rho_i + qj.inv_rho) * rg * idist2);
#pragma unroll
        for (int k = 0; k < D; ++k) visc[k] += vc * Vji[k];
        /* pairwise surface tension (Nair & Poeschel), src/Kernel.h:88-113 */
        if (st_on) {
            const double fac = (b_i == FJSPH_BOUND || b_j == FJSPH_BOUND) ? 1.0 + 0.5 * cos(0.5 * kPi * 7.0 / 9.0) : 1.0;
            const double c = -npdm2 * fac * cos(pi3o4_H * r) / r;
#pragma unroll
            for (int k = 0; k < D; ++k) st[k] += c * Rji[k];
        }
        if (ale) {
            double vj[D], vPj[D];
            load3<D>(W.vPert, j, vPj);
#pragma unroll
            for (int k = 0; k < D; ++k) vj[k] = W.v[k][j];
            const double gj = dot<D, double>(vPj, g), gi = dot<D, double>(vPi, g);
            double dvp[D];
#pragma unroll
            for (int k = 0; k < D; ++k) dvp[k] = vPj[k] - vPi[k];
            const double q = dot<D, double>(dvp, g);
#pragma unroll
            for (int a = 0; a < D; ++a) acc_ale[a] += (vj[a] * gj + vi[a] * gi - vi[a] * q) * volj;
            double w1 = 0.0, w2 = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                w1 += ((vj[k] + vPj[k]) - (vi[k] + vPi[k])) * g[k];
                w2 += (rho_j * vPj[k] + rho_i * vPi[k]) * g[k];
            }
            Rrho -= w1 * volj;
            Rrhoc += w2 * volj;
        } else {
            Rrho -= volj * dot<D, double>(Vji, g);
        }
        if (nofrozen) {
            if (b_j > FJSPH_PISTON) {
                if (!nodsph) {
                    double gsum[D];
#pragma unroll
                    for (int k = 0; k < D; ++k) gsum[k] = gRi[k] + W.gradRho[k][j];
                    Rrho_d += volj * ((rho_j - rho_i) + 0.5 * dot<D, double>(gsum, Rji)) * rg * idist2;
                }
                const double vdotr = dot<D, double>(Vji, Rji);
                const double c = linear ? volj * idist2 * vdotr
                                        : m_j * art_visc_scale(P, vdotr, idist2, rho_i, rho_j, Q[i].cs, qj.cs);
#pragma unroll
                for (int k = 0; k < D; ++k) art[k] += c * g[k];
            } else if (!nodsph) {
                Rrho_d += volj * (rho_j - rho_i) * rg * idist2;
            }
        }
    }
    if (linear)
#pragma unroll
        for (int k = 0; k < D; ++k) acc[k] /= rho_i;
    if (csf) {
        const double c = 1.0 / rho_i * P.sig * W.curve[i] * W.colourG[i];
#pragma unroll
        for (int k = 0; k < D; ++k) acc[k] += c * W.norm[k][i];
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const double av = nofrozen ? art[k] : W.aVisc[k][i];
        double t = acc[k];
        if (ale) t += acc_ale[k];
        W.acc[k][i] = t + av + visc[k] + st[k] / m_i + P.grav[k];
    }
    double R = Rrho * rho_i;
    if (ale) R += Rrhoc;
    if (!nodsph) R += nofrozen ? P.dsph_cont * Rrho_d : W.deltaD[i];
    W.Rrho[i] = R;
}

inline unsigned fluid_grid(const Params &P) { return grid_for(P.n - P.nb, kThreads); }
inline unsigned bound_grid(const Params &P) { return grid_for(P.nb, kThreads); }
inline unsigned all_grid(const Params &P) { return grid_for(P.n, kThreads); }

} // namespace

#define FJSPH_DISPATCH(P, KERNEL, GRID, ...)                                              \
    do {                                                                                  \
        if ((GRID) == 0) break;                                                           \
        if ((P).D == 2)                                                                   \
            KERNEL<2><<<(GRID), kThreads, 0, s>>>(__VA_ARGS__);                           \
        else                                                                              \
            KERNEL<3><<<(GRID), kThreads, 0, s>>>(__VA_ARGS__);                           \
    } while (0)

/* the quotients of every particle, before a sweep that gathers them */
inline void quotients(const Params &P, const DevState &W, ResidQuot *Q, cudaStream_t s) {
    if (all_grid(P) > 0) k_resid_quotients<<<all_grid(P), kThreads, 0, s>>>(P, W, Q);
}

void launch_dsph_prestep(const Params &P, const DevState &W, const DevNbr &N, double *npd_part, ResidQuot *Q,
                         cudaStream_t s) {
    quotients(P, W, Q, s);
    FJSPH_DISPATCH(P, k_dsph_prestep, all_grid(P), P, W, N, npd_part, Q);
}
void launch_npd_only(const Params &P, const DevState &W, const DevNbr &N, double *npd_part, cudaStream_t s) {
    FJSPH_DISPATCH(P, k_npd_only, all_grid(P), P, W, N, npd_part);
}
void launch_aero_velocity(const Params &P, const DevState &W, const DevNbr &N, cudaStream_t s) {
    FJSPH_DISPATCH(P, k_aero_velocity, fluid_grid(P), P, W, N);
}
void launch_detect_surface(const Params &P, const DevState &W, const DevNbr &N, double *const nrm_tmp[3],
                           ResidQuot *Q, cudaStream_t s) {
    quotients(P, W, Q, s);
    FJSPH_DISPATCH(P, k_surface_normal, fluid_grid(P), P, W, N, nrm_tmp[0], nrm_tmp[1], nrm_tmp[2], Q);
    FJSPH_DISPATCH(P, k_surface_curvature, fluid_grid(P), P, W, N, nrm_tmp[0], nrm_tmp[1], nrm_tmp[2], Q);
}
void launch_dissipation(const Params &P, const DevState &W, const DevNbr &N, ResidQuot *Q, cudaStream_t s) {
    quotients(P, W, Q, s);
    FJSPH_DISPATCH(P, k_dissipation, fluid_grid(P), P, W, N, Q);
}
void launch_particle_shift(const Params &P, const DevState &W, const DevNbr &N, ResidQuot *Q, cudaStream_t s) {
    quotients(P, W, Q, s);
    FJSPH_DISPATCH(P, k_particle_shift, fluid_grid(P), P, W, N, Q);
}
void launch_pipe_outlet(const Params &P, const DevState &W, int32_t *kbits, cudaStream_t s) {
    FJSPH_DISPATCH(P, k_pipe_outlet, fluid_grid(P), P, W, kbits);
}
void launch_bound_velocity(const Params &P, const DevState &W, int nb_rule, cudaStream_t s) {
    FJSPH_DISPATCH(P, k_bound_velocity, bound_grid(P), P, W, nb_rule);
}
void launch_no_slip(const Params &P, const DevState &W, const DevNbr &N, double *const vtmp[3], cudaStream_t s) {
    FJSPH_DISPATCH(P, k_no_slip, bound_grid(P), P, W, N, vtmp[0], vtmp[1], vtmp[2]);
    FJSPH_DISPATCH(P, k_copy_bound_v, bound_grid(P), P, W, vtmp[0], vtmp[1], vtmp[2]);
}
void launch_bound_pressure(const Params &P, const DevState &W, const DevNbr &N, cudaStream_t s) {
    FJSPH_DISPATCH(P, k_bound_pressure, bound_grid(P), P, W, N);
}
void launch_bound_ghost(const Params &P, const DevState &W, const DevNbr &N, int32_t *near_inlet, cudaStream_t s) {
    FJSPH_DISPATCH(P, k_bound_ghost, bound_grid(P), P, W, N, near_inlet);
}
void launch_bound_dbc(const Params &P, const DevState &W, cudaStream_t s) {
    FJSPH_DISPATCH(P, k_bound_dbc, bound_grid(P), P, W);
}
void launch_resid(const Params &P, const DevState &W, const DevNbr &N, const double *npd_dev, ResidQuot *Q,
                  cudaStream_t s) {
    quotients(P, W, Q, s);
    FJSPH_DISPATCH(P, k_resid, fluid_grid(P), P, W, N, npd_dev, Q);
}

} // namespace fjsph
