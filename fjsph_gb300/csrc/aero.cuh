/*
 * aero.cuh -- the aerodynamic closures of src/Aero.h:10-263 for one particle (FP64): Gissler's
 * sphere-plate interpolation (default), the induced-pressure model and the skin-friction model.
 * Shared by the FP64 and the FP32 split-precision residual kernels; it is evaluated once per
 * particle, not per pair.
 */
#pragma once

#include "common.cuh"
#include "split.cuh"

namespace fjsph {

__device__ __forceinline__ double get_cd(double Re) {
    return (1.0 + 0.197 * pow(Re, 0.63) + 2.6e-04 * pow(Re, 1.38)) * (24.0 / (Re + 0.00001));
}

/* Gissler drag coefficient Cd_i and un-occluded area A_i of one particle (src/Aero.h:37-98):
 * Cd_i = (1 - f) Cd_drop + f, A_i = (1 - f) A_drop + f A_plate, f from lambda or the neighbour
 * count; Cd_drop from the sphere law with the TAB deformation factor when enabled. */
template <int D>
__device__ __forceinline__ void gissler_coeff(const Params &P, double cellRho, double Vn, double V2, double lam,
                                              double nneigh, double &Cdi, double &Aun) {
    const double Re = 2.0 * cellRho * Vn * P.L / P.mu_g;
    const double frac2 = P.use_lam ? fmin(P.interp_fac * lam, 1.0) : fmin(P.interp_fac * nneigh * P.i_n_full, 1.0);
    const double frac1 = 1.0 - frac2;
    const double Cds = get_cd(Re);
    double Cdl = Cds, Adrop = P.A_sphere;
    if (P.use_TAB_def) {
        double ymax = V2 * P.ycoef;
        if (ymax > 1.0) ymax = 1.0;
        Cdl = Cds * (1 + 2.632 * ymax);
        if (D == 3) {
            const double t = P.L + P.Cb * P.L * ymax;
            Adrop = kPi * t * t;
        } else {
            Adrop = P.A_sphere + 2 * (P.Cb * P.L * ymax);
        }
    }
    Cdi = frac1 * Cdl + frac2;
    Aun = frac1 * Adrop + frac2 * P.A_plate;
}

template <int D>
__device__ __forceinline__ void aero_acc(const Params &P, const DevState &W, int64_t i, const double *Vd, double lam,
                         double nneigh, double *out) {
#pragma unroll
    for (int k = 0; k < D; ++k) out[k] = 0.0;
    if (P.acase == FJSPH_GISSLER) {
        /* fully occluded (woccl = 1): the exposed area (1 - woccl) * A is exactly zero, so the
         * force is zero for any finite relative velocity; skip the two pow() of the drag law
         * (|V| is finite exactly when its components are: they are far below overflow) */
        bool finite = true;
#pragma unroll
        for (int k = 0; k < D; ++k) finite = finite && isfinite(Vd[k]);
        if (W.woccl[i] == 1.0 && finite) return;
    }
    const double Vn = vnorm<D, double>(Vd);
    if (P.acase == FJSPH_GISSLER) {
        double Cdi, Aun;
        gissler_coeff<D>(P, W.cellRho[i], Vn, dot<D, double>(Vd, Vd), lam, nneigh, Cdi, Aun);
        const double Ai = (1.0 - W.woccl[i]) * Aun;
        const double c = 0.5 * Vn;
        const double tail = P.gamma_g * W.cellP[i] * Cdi * Ai / W.m[i];
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = c * Vd[k] / (P.sos * P.sos) * tail;
        return;
    }
    double nrm[D], nh[D];
    load3<D>(W.norm, i, nrm);
    normalized<D, double>(nrm, nh);
    const double m_i = W.m[i];
    if (P.acase == FJSPH_INDUCED_PRESSURE) {
        double vh[D], mnh[D];
        normalized<D, double>(Vd, vh);
#pragma unroll
        for (int k = 0; k < D; ++k) mnh[k] = -nh[k];
        const double theta = fabs(acos(dot<D, double>(mnh, vh)));
        double Cp_s, Cp_p, Cp_b, Cp_tot;
        if (theta < 2.4455) {
            const double s = sin(theta);
            Cp_s = 1.0 - 2.25 * s * s;
        } else
            Cp_s = 0.075;
        if (theta < 1.570797)
            Cp_p = cos(theta);
        else if (theta < 1.9918)
            Cp_p = -pow(cos(6.0 * theta + 0.5 * kPi), 1.5);
        else if (theta < 2.0838)
            Cp_p = 5.5836 * theta - 11.5601;
        else
            Cp_p = 0.075;
        if (theta < 0.7854)
            Cp_b = 1.0;
        else if (theta < 1.570797)
            Cp_b = 0.5 * (cos(4.0 * theta - kPi) + 1.0);
        else
            Cp_b = 0.0;
        const double nc = W.norm_curve[i];
        if (nc < -0.25)
            Cp_tot = Cp_b;
        else if (nc < 0.0) {
            const double fr = (nc + 0.25) * 4.0;
            Cp_tot = fr * Cp_b + (1.0 - fr) * Cp_p;
        } else if (nc < 0.25) {
            const double fr = nc * 4.0;
            Cp_tot = fr * Cp_p + (1.0 - fr) * Cp_s;
        } else
            Cp_tot = Cp_s;
        const double cellP = W.cellP[i], cellRho = W.cellRho[i];
        const double Pi = 0.5 * dot<D, double>(Vd, Vd) / (P.sos * P.sos) * P.gamma_g * cellP * Cp_tot;
        const double Cdi = get_cd(cellRho * Vn * P.L / P.mu_g);
        const double Vnorm = dot<D, double>(Vd, nh);
        double Vpar[D];
#pragma unroll
        for (int k = 0; k < D; ++k) Vpar[k] = Vd[k] - Vnorm * nh[k];
        const double Vparn = vnorm<D, double>(Vpar);
        const double Cf = 0.027 / pow(cellRho * Vparn * P.L / P.mu_g + 1e-6, 1.0 / 7.0);
        const double frac1 = P.use_lam ? fmin(P.interp_fac * lam, 1.0) : fmin(P.interp_fac * nneigh * P.i_n_full, 1.0);
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double drop = 0.5 * Vd[k] * Vn / (P.sos * P.sos) * P.gamma_g * cellP * (kPi * P.L * P.L * 0.25) * Cdi / m_i;
            const double kern = -Pi * P.A_plate * nh[k] / m_i;
            const double skin = 0.5 * Vparn * Vpar[k] / (P.sos * P.sos) * P.gamma_g * cellP * Cf * P.A_plate / m_i;
            out[k] = frac1 * (kern + skin) + (1.0 - frac1) * drop;
        }
        return;
    }
    if (P.acase == FJSPH_SKIN_FRIC) {
        const double Vnorm = dot<D, double>(Vd, nh);
        if (Vnorm > 0.001) {
            const double Re = P.rho_g * Vn * P.L / P.mu_g;
            double Vpar[D];
#pragma unroll
            for (int k = 0; k < D; ++k) Vpar[k] = Vd[k] - fabs(Vnorm) * nh[k];
            const double Cf = 0.027 / pow(Re, 1.0 / 7.0);
            const double Vparn = vnorm<D, double>(Vpar);
            const double frac2 = fmin(1.5 * lam, 1.0), frac1 = 1.0 - frac2;
            const double Cdi = get_cd(Re);
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const double press = 0.5 * P.rho_g * Vnorm * Vnorm * P.A_plate * nh[k] / m_i;
                const double skin = 0.5 * P.rho_g * Vparn * Cf * P.A_plate * Vpar[k] / m_i;
                const double drop = 0.5 * P.rho_g * Vn * Vd[k] * (kPi * P.L * P.L / 4) * Cdi / m_i;
                out[k] = frac2 * (press + skin) + frac1 * drop;
            }
        }
    }
}

/* The Gissler closure of aero_acc evaluated in FP32, for the split-precision form (whose aero
 * force is held to 1e-3 of the FP64 oracle): the same formula on FP32 operands with the
 * constants of FConst, powf for the sphere drag law.  On this GPU the FP64 pipe issues a warp
 * instruction every 16 cycles per SM, and the FP64 drag law (two pow, a square root, divides) of
 * the exposed particles kept it a third busy in the residual.  U = cellV - v; one_m_woccl =
 * 1 - woccl; nneigh the neighbour count (self included). */
template <int D>
__device__ __forceinline__ void gissler_acc_f32(const Params &P, const float *U, float cellRho, float cellP,
                                                float one_m_woccl, float m, float lam, float nneigh, float *out) {
    const FConst &c = P.fc;
    float V2 = 0.f;
#pragma unroll
    for (int k = 0; k < D; ++k) V2 += U[k] * U[k];
    const float Vn = sqrtf(V2);
    const float Re = c.re_coef * cellRho * Vn;
    const float frac2 = P.use_lam ? fminf(c.interp_fac * lam, 1.f) : fminf(c.interp_fac * nneigh * c.i_n_full, 1.f);
    const float frac1 = 1.f - frac2;
    const float Cds = (1.f + 0.197f * powf(Re, 0.63f) + 2.6e-04f * powf(Re, 1.38f)) * (24.f / (Re + 0.00001f));
    float Cdl = Cds, Adrop = c.A_sphere;
    if (P.use_TAB_def) {
        const float ymax = fminf(V2 * c.ycoef, 1.f);
        Cdl = Cds * (1.f + 2.632f * ymax);
        if (D == 3) {
            const float t = c.L + c.CbL * ymax;
            Adrop = (float)kPi * t * t;
        } else {
            Adrop = c.A_sphere + 2.f * (c.CbL * ymax);
        }
    }
    const float Cdi = frac1 * Cdl + frac2;
    const float Aun = frac1 * Adrop + frac2 * c.A_plate;
    const float tail = c.force_coef * cellP * Cdi * (one_m_woccl * Aun) / m;
    const float cc = 0.5f * Vn * tail;
#pragma unroll
    for (int k = 0; k < D; ++k) out[k] = cc * U[k];
}

} // namespace fjsph
