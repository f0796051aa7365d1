/*
 * oracle.cpp -- CPU restatement of FJSPH's WCSPH hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * Used by tests/ (parity checker), __graft_entry__.smoke() and bench.py (timed CPU baseline and
 * the `--impl reference` arm).  The product library never links it.
 *
 * Every function follows the reference function named in its comment (paths relative to the
 * FJSPH source tree) with serial semantics:
 *   - dSPH_PreStep's numerical particle density `npd` is summed in index order (the reference
 *     accumulates it in a shared variable inside an OpenMP region, which races);
 *   - Boundary_DBC's scatter is evaluated serially;
 *   - each neighbour list is ordered by neighbour index (the reference keeps nanoflann's
 *     unsorted order, which only changes floating-point summation order).
 * Third-party arithmetic is restated from its mathematics, not from library source:
 *   - nanoflann radius search (version unpinned, >= 1.5 API): squared L2 distance accumulated
 *     over dimensions in order, d2 < radius strict, self included.  The reference is compiled
 *     with -O3 -ffast-math -march=native, where GCC fuses `result += diff*diff` into fused
 *     multiply-adds; the distance here is fma(dz,dz,fma(dy,dy,dx*dx)).
 *   - Eigen ColPivHouseholderQR (3.3/3.4): Householder QR with column pivoting (Golub & Van Loan
 *     5.4.1); invertible iff every |R_kk| > dim * eps * max|R_kk|.
 *   - Eigen SelfAdjointEigenSolver::computeDirect: closed-form eigenvalues of the symmetric
 *     matrix read from its lower triangle (2x2 quadratic formula; 3x3 trigonometric method,
 *     Smith 1961), after shifting by the mean diagonal and scaling by the largest entry.
 *   - Eigen normalized(): v/|v|, and a zero vector stays zero.
 *
 * Parity status: UNPINNED (no golden vectors exist upstream and the reference cannot be built
 * here).  See the tests for the known-answer and analytic pins that are available.
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEps = std::numeric_limits<double>::epsilon(); /* MEPSILON, VarDefs.h:52 */
constexpr double kDefaultVal = 9999999.0;                       /* VarDefs.h:195 */
constexpr int64_t kNoCell = -3;                                 /* VarDefs.h:197 */
constexpr int kInletZone = 6;                                   /* shape_type inletZone */

struct Part {
    double xi[3], v[3], acc[3], Af[3], aVisc[3], cellV[3], gradRho[3], norm[3], vPert[3];
    double L[9];
    double Rrho, rho, p, m, curve, norm_curve, woccl, pDist, deltaD;
    double cellP, cellRho, colourG, colour, lam, lam_nb, kernsum;
    int64_t part_id, cellID;
    int32_t b, surf, surfzone;
};

struct Nb {
    int64_t j;
    double rr;
};

struct Block {
    fjsph_block d;
    std::vector<int64_t> back;
    std::vector<std::vector<int64_t>> buffer;
};

} // namespace

struct orc_sim {
    fjsph_settings s;
    int D = 3;
    std::vector<Block> limits;
    int64_t n_bound_blocks = 0, n_fluid_blocks = 0;
    int64_t bound_points = 0, total_points = 0, fluid_points = 0, part_id_next = 0;
    int64_t delete_count = 0;
    std::vector<Part> pn, pnp1;
    std::vector<std::vector<Nb>> outlist;
    /* Integrator members (Integration.h:52-67) */
    double safe_dt = 0, maxf = kEps, maxAf = kEps, maxRho_pc = kEps, maxRhoi = kEps, maxdrho = kEps;
    double minST = 9999999.0, maxU = kEps, maxShift = kEps;
    int64_t start_index = 0, end_index = 0;
    uint32_t iteration = 0;
    /* vortex lattice (VLM.h:31-97): panels A, B, C and normal, circulations, limit */
    std::vector<double> vlm_A, vlm_B, vlm_C, vlm_gamma;
    double vlm_vinf[3] = {0, 0, 0}, vlm_maxvel = 0.0;
    bool vlm_ready = false;
    /* analytic boundary-layer air field (a synthetic input; no reference counterpart): axis, wall,
     * thickness, exponent */
    double pl[4] = {2.0, 0.0, 1.0, 1.0 / 7.0};
    bool pl_ready = false;
    /* mesh-cell air source (MESH, Var.h:396-451) */
    std::vector<double> m_verts, m_centre, m_vel, m_p, m_rho, m_rad2;
    std::vector<int64_t> m_face_off, m_face_verts, m_cell_off, m_cell_faces;
    std::vector<int32_t> m_face_right;
    int64_t m_ncells = 0;
};

namespace {

/* ------------------------------------------------------------------------------------------ */
/* small vector helpers                                                                        */
/* ------------------------------------------------------------------------------------------ */
inline double dot(const double *a, const double *b, int D) {
    double r = a[0] * b[0];
    for (int k = 1; k < D; ++k) r += a[k] * b[k];
    return r;
}
inline double sqnorm(const double *a, int D) { return dot(a, a, D); }
inline double norm(const double *a, int D) { return std::sqrt(sqnorm(a, D)); }
inline void normalized(const double *a, int D, double *out) {
    double z = sqnorm(a, D);
    if (z > 0.0) {
        double n = std::sqrt(z);
        for (int k = 0; k < D; ++k) out[k] = a[k] / n;
    } else {
        for (int k = 0; k < D; ++k) out[k] = a[k];
    }
}
inline void sub(const double *a, const double *b, int D, double *out) {
    for (int k = 0; k < D; ++k) out[k] = a[k] - b[k];
}
inline void zero(double *a, int n) {
    for (int k = 0; k < n; ++k) a[k] = 0.0;
}

/* Squared distance as nanoflann's L2_Simple accumulates it (see the file header). */
inline double dist2(const double *q, const double *p, int D) {
    double d0 = q[0] - p[0];
    double r = d0 * d0;
    for (int k = 1; k < D; ++k) {
        double dk = q[k] - p[k];
        r = std::fma(dk, dk, r);
    }
    return r;
}

/* ------------------------------------------------------------------------------------------ */
/* Kernel.h                                                                                    */
/* ------------------------------------------------------------------------------------------ */
/* Kernel.h:37-45 (Wendland C2) and Kernel.h:11-21 (cubic, -DCUBIC). */
inline double Kernel(double dist, double H, double Wc, bool cubic) {
    if (cubic) {
        double q = dist / H;
        if (q < 1.0) return Wc * (1.0 - 1.5 * q * q * (1 - 0.5 * q));
        if (q < 2.0) return Wc * 0.25 * std::pow(2.0 - q, 3.0);
        return 0.0;
    }
    return std::pow(1 - 0.5 * dist / H, 4) * (2 * dist / H + 1) * Wc;
}

/* Kernel.h:48-61 (Wendland C2) and Kernel.h:23-33 (cubic). */
inline void GradK(const double *Rij, double dist, double H, double Wc, bool cubic, int D, double *out) {
    if (cubic) {
        double q = dist / H;
        if (q < 1.0) {
            double f = Wc * (3.0 * (0.75 * q - 1.0));
            for (int k = 0; k < D; ++k) out[k] = Rij[k] / (H * H) * f;
        } else if (q < 2.0) {
            double f = Wc * -0.75 * (2.0 - q) * (2.0 - q);
            for (int k = 0; k < D; ++k) out[k] = Rij[k] / (dist * H) * f;
        } else {
            zero(out, D);
        }
        return;
    }
    if (dist / H < 1e-12) {
        zero(out, D);
        return;
    }
    double f = std::pow(1 - 0.5 * dist / H, 3) * Wc;
    for (int k = 0; k < D; ++k) out[k] = 5.0 * (Rij[k] / (H * H)) * f;
}

/* Kernel.h:88-113 */
inline double pairwise_ST_fac(int bA, int bB) {
    if (bA == FJSPH_BOUND || bB == FJSPH_BOUND) {
        double contang = 0.5 * kPi * 7.0 / 9.0;
        return 1.0 + 0.5 * std::cos(contang);
    }
    return 1.0;
}

/* Kernel.h:217-244 */
inline void ArtVisc(const fjsph_settings &f, const Part &pi, const Part &pj, const double *Rji,
                    const double *Vji, double idist2, const double *gradK, int D, double *out) {
    double vdotr = dot(Vji, Rji, D);
    if (vdotr > 0.0) {
        zero(out, D);
        return;
    }
    double muij = f.H * vdotr * idist2;
    double rhoij = 0.5 * (pi.rho + pj.rho);
    double cbar = 0.5 * (std::sqrt((f.B * f.gam) / pi.rho) + std::sqrt((f.B * f.gam) / pj.rho));
    for (int k = 0; k < D; ++k) out[k] = gradK[k] * f.visc_alpha * cbar * muij / rhoij;
}

/* ------------------------------------------------------------------------------------------ */
/* Small dense linear algebra (restated, see file header)                                      */
/* ------------------------------------------------------------------------------------------ */
/* Householder QR with column pivoting of a DxD matrix (row-major A).  Returns 1 and the inverse
 * if the matrix has full rank under the threshold dim*eps*max|R_kk|, else 0. */
int qr_inverse(const double *Ain, int D, double *inv) {
    double A[9], vs[3][3], betas[3];
    int perm[3] = {0, 1, 2};
    std::memcpy(A, Ain, sizeof(double) * D * D);
    double maxpiv = 0.0;
    double rdiag[3] = {0, 0, 0};
    for (int k = 0; k < D; ++k) {
        /* pivot: remaining column with the largest norm (first one on ties) */
        int pc = k;
        double best = -1.0;
        for (int c = k; c < D; ++c) {
            double s = 0.0;
            for (int r = k; r < D; ++r) s += A[r * D + c] * A[r * D + c];
            if (s > best) {
                best = s;
                pc = c;
            }
        }
        if (pc != k) {
            for (int r = 0; r < D; ++r) std::swap(A[r * D + k], A[r * D + pc]);
            std::swap(perm[k], perm[pc]);
        }
        /* Householder vector for column k, rows k..D-1 */
        double xnorm2 = 0.0;
        for (int r = k; r < D; ++r) xnorm2 += A[r * D + k] * A[r * D + k];
        double xnorm = std::sqrt(xnorm2);
        double x0 = A[k * D + k];
        double alpha = (x0 >= 0.0) ? -xnorm : xnorm;
        double v[3] = {0, 0, 0};
        double beta = 0.0;
        if (xnorm > 0.0) {
            v[k] = x0 - alpha;
            for (int r = k + 1; r < D; ++r) v[r] = A[r * D + k];
            double vn2 = 0.0;
            for (int r = k; r < D; ++r) vn2 += v[r] * v[r];
            beta = (vn2 > 0.0) ? 2.0 / vn2 : 0.0;
            /* apply H = I - beta v v^T to columns k..D-1 */
            for (int c = k; c < D; ++c) {
                double s = 0.0;
                for (int r = k; r < D; ++r) s += v[r] * A[r * D + c];
                s *= beta;
                for (int r = k; r < D; ++r) A[r * D + c] -= s * v[r];
            }
        } else {
            alpha = 0.0;
        }
        for (int r = 0; r < D; ++r) vs[k][r] = v[r];
        betas[k] = beta;
        rdiag[k] = A[k * D + k];
        maxpiv = std::max(maxpiv, std::fabs(rdiag[k]));
    }
    double thr = maxpiv * kEps * double(D);
    for (int k = 0; k < D; ++k)
        if (!(std::fabs(rdiag[k]) > thr)) return 0;
    /* inverse: solve R y = Q^T e_c, then undo the column permutation */
    double Y[9];
    for (int c = 0; c < D; ++c) {
        double e[3] = {0, 0, 0};
        e[c] = 1.0;
        for (int k = 0; k < D; ++k) {
            double s = 0.0;
            for (int r = k; r < D; ++r) s += vs[k][r] * e[r];
            s *= betas[k];
            for (int r = k; r < D; ++r) e[r] -= s * vs[k][r];
        }
        double y[3];
        for (int r = D - 1; r >= 0; --r) {
            double s = e[r];
            for (int q = r + 1; q < D; ++q) s -= A[r * D + q] * y[q];
            y[r] = s / A[r * D + r];
        }
        for (int r = 0; r < D; ++r) Y[r * D + c] = y[r];
    }
    /* A P = Q R  =>  A^-1 = P R^-1 Q^T: row perm[r] of the inverse is row r of Y */
    for (int r = 0; r < D; ++r)
        for (int c = 0; c < D; ++c) inv[perm[r] * D + c] = Y[r * D + c];
    return 1;
}

/* Smallest eigenvalue of the symmetric matrix whose lower triangle is read from A. */
double min_eig(const double *A, int D) {
    if (D == 2) {
        double a00 = A[0], a10 = A[2], a11 = A[3];
        double shift = 0.5 * (a00 + a11);
        double b00 = a00 - shift, b11 = a11 - shift, b10 = a10;
        double scale = std::max(std::fabs(b00), std::max(std::fabs(b11), std::fabs(b10)));
        if (scale > 0.0) {
            b00 /= scale;
            b11 /= scale;
            b10 /= scale;
        } else {
            scale = 0.0;
        }
        double hd = 0.5 * (b00 - b11);
        double t = std::sqrt(hd * hd + b10 * b10);
        double l = 0.5 * (b00 + b11) - t;
        return l * scale + shift;
    }
    double a00 = A[0], a10 = A[3], a11 = A[4], a20 = A[6], a21 = A[7], a22 = A[8];
    double shift = (a00 + a11 + a22) / 3.0;
    double m00 = a00 - shift, m11 = a11 - shift, m22 = a22 - shift, m10 = a10, m20 = a20, m21 = a21;
    double scale = std::max({std::fabs(m00), std::fabs(m11), std::fabs(m22), std::fabs(m10),
                             std::fabs(m20), std::fabs(m21)});
    if (!(scale > 0.0)) return shift;
    m00 /= scale;
    m11 /= scale;
    m22 /= scale;
    m10 /= scale;
    m20 /= scale;
    m21 /= scale;
    /* characteristic polynomial x^3 - c2 x^2 + c1 x - c0 */
    double c0 = m00 * m11 * m22 + 2.0 * m10 * m20 * m21 - m00 * m21 * m21 - m11 * m20 * m20 -
                m22 * m10 * m10;
    double c1 = m00 * m11 - m10 * m10 + m00 * m22 - m20 * m20 + m11 * m22 - m21 * m21;
    double c2 = m00 + m11 + m22;
    /* depressed cubic via x = y + c2/3: y^3 - p y - q = 0 with p = (c2^2 - 3 c1)/3 */
    double c2o3 = c2 / 3.0;
    double p = (c2 * c2o3 - c1) / 3.0; /* = a/3 in the trigonometric form */
    if (p < 0.0) p = 0.0;
    double halfq = 0.5 * (c0 + c2o3 * (2.0 * c2o3 * c2o3 - c1));
    double disc = p * p * p - halfq * halfq;
    if (disc < 0.0) disc = 0.0;
    double rho = std::sqrt(p);
    double theta = std::atan2(std::sqrt(disc), halfq) / 3.0;
    double ct = std::cos(theta), st = std::sin(theta);
    double sqrt3 = std::sqrt(3.0);
    double r0 = c2o3 + 2.0 * rho * ct;
    double r1 = c2o3 - rho * (ct + sqrt3 * st);
    double r2 = c2o3 - rho * (ct - sqrt3 * st);
    double l = std::min(r0, std::min(r1, r2));
    return l * scale + shift;
}

/* ------------------------------------------------------------------------------------------ */
/* Aero.h                                                                                      */
/* ------------------------------------------------------------------------------------------ */
/* Aero.h:10-18 */
inline double GetCd(double Re) {
    return (1.0 + 0.197 * std::pow(Re, 0.63) + 2.6e-04 * std::pow(Re, 1.38)) * (24.0 / (Re + 0.00001));
}

/* Aero.h:37-98 */
void gissler_force(const fjsph_settings &a, const double *Vdiff, double rho, double press, double mass,
                   double lam, double nnieghb, double woccl, int D, double *out) {
    double Vn = norm(Vdiff, D);
    double Re = 2.0 * rho * Vn * a.L / a.mu_g;
    double frac2;
    if (a.use_lam)
        frac2 = std::min(a.interp_fac * lam, 1.0);
    else
        frac2 = std::min(a.interp_fac * nnieghb * a.i_n_full, 1.0);
    double frac1 = 1.0 - frac2;
    double Cds = GetCd(Re);
    double Cdl, Adrop;
    if (a.use_TAB_def) {
        double ymax = sqnorm(Vdiff, D) * a.ycoef;
        if (ymax > 1.0) ymax = 1.0;
        Cdl = Cds * (1 + 2.632 * ymax);
        if (D == 3)
            Adrop = kPi * std::pow((a.L + a.Cb * a.L * ymax), 2);
        else
            Adrop = a.A_sphere + 2 * (a.Cb * a.L * ymax);
    } else {
        Cdl = Cds;
        Adrop = a.A_sphere;
    }
    double Cdi = frac1 * Cdl + frac2;
    double Aunocc = (frac1 * Adrop + frac2 * a.A_plate);
    double Ai = (1.0 - woccl) * Aunocc;
    for (int k = 0; k < D; ++k)
        out[k] = 0.5 * Vn * Vdiff[k] / (a.sos * a.sos) * a.gamma_g * press * Cdi * Ai / mass;
}

/* Aero.h:106-202 */
void induced_pressure(const fjsph_settings &a, const double *Vdiff, const double *nrm, double lam,
                      double nnieghb, const Part &pi, int D, double *out) {
    double nh[3], vh[3];
    normalized(nrm, D, nh);
    normalized(Vdiff, D, vh);
    double mnh[3];
    for (int k = 0; k < D; ++k) mnh[k] = -nh[k];
    double theta = std::fabs(std::acos(dot(mnh, vh, D)));
    double Cp_s, Cp_p, Cp_b, Cp_tot;
    if (theta < 2.4455)
        Cp_s = 1.0 - (2.25) * std::pow(std::sin(theta), 2.0);
    else
        Cp_s = 0.075;
    if (theta < 1.570797)
        Cp_p = std::cos(theta);
    else if (theta < 1.9918)
        Cp_p = -std::pow(std::cos(6.0 * theta + 0.5 * kPi), 1.5);
    else if (theta < 2.0838)
        Cp_p = 5.5836 * theta - 11.5601;
    else
        Cp_p = 0.075;
    if (theta < 0.7854)
        Cp_b = 1.0;
    else if (theta < 1.570797)
        Cp_b = 0.5 * (std::cos(4.0 * theta - kPi) + 1.0);
    else
        Cp_b = 0.0;
    double normCurve = pi.norm_curve;
    double fac1 = 0.25, ifac1 = 1 / fac1;
    if (normCurve < -fac1)
        Cp_tot = Cp_b;
    else if (normCurve < 0.0) {
        double frac = (normCurve + fac1) * ifac1;
        Cp_tot = frac * Cp_b + (1.0 - frac) * Cp_p;
    } else if (normCurve < fac1) {
        double frac = (normCurve)*ifac1;
        Cp_tot = frac * Cp_p + (1.0 - frac) * Cp_s;
    } else
        Cp_tot = Cp_s;
    double Vsq = sqnorm(Vdiff, D), Vn = std::sqrt(Vsq);
    double Plocali = 0.5 * Vsq / (a.sos * a.sos) * a.gamma_g * pi.cellP * Cp_tot;
    double Pi = Plocali;
    double Re = pi.cellRho * Vn * a.L / a.mu_g;
    double Cdi = GetCd(Re);
    double acc_drop[3], acc_kern[3], acc_skin[3], Vpar[3];
    for (int k = 0; k < D; ++k)
        acc_drop[k] = 0.5 * Vdiff[k] * Vn / (a.sos * a.sos) * a.gamma_g * pi.cellP *
                      (kPi * a.L * a.L * 0.25) * Cdi / pi.m;
    for (int k = 0; k < D; ++k) acc_kern[k] = -Pi * a.A_plate * nh[k] / pi.m;
    double Vnorm = dot(Vdiff, nh, D);
    for (int k = 0; k < D; ++k) Vpar[k] = Vdiff[k] - Vnorm * nh[k];
    double Vparn = norm(Vpar, D);
    double Re_par = pi.cellRho * Vparn * a.L / a.mu_g;
    double Cf = 0.027 / std::pow(Re_par + 1e-6, 1.0 / 7.0);
    for (int k = 0; k < D; ++k)
        acc_skin[k] = 0.5 * Vparn * Vpar[k] / (a.sos * a.sos) * a.gamma_g * pi.cellP * Cf * a.A_plate / pi.m;
    double frac1;
    if (a.use_lam)
        frac1 = std::min(a.interp_fac * lam, 1.0);
    else
        frac1 = std::min(a.interp_fac * nnieghb * a.i_n_full, 1.0);
    for (int k = 0; k < D; ++k) out[k] = frac1 * (acc_kern[k] + acc_skin[k]) + (1.0 - frac1) * acc_drop[k];
}

/* Aero.h:204-263 */
void CalcAeroAcc(const fjsph_settings &a, const Part &pi, const double *Vdiff, const double *nrm,
                 double lam, double nneigh, int D, double *out) {
    zero(out, D);
    switch (a.acase) {
    case FJSPH_GISSLER:
        gissler_force(a, Vdiff, pi.cellRho, pi.cellP, pi.m, lam, nneigh, pi.woccl, D, out);
        break;
    case FJSPH_INDUCED_PRESSURE:
        induced_pressure(a, Vdiff, nrm, lam, nneigh, pi, D, out);
        break;
    case FJSPH_SKIN_FRIC: {
        double nh[3];
        normalized(nrm, D, nh);
        double Vnorm = dot(Vdiff, nh, D);
        if (Vnorm > 0.001) {
            double Vn = norm(Vdiff, D);
            double Re = a.rho_g * Vn * a.L / a.mu_g;
            double acc_press[3], Vpar[3], acc_skin[3], acc_drop[3];
            for (int k = 0; k < D; ++k)
                acc_press[k] = 0.5 * a.rho_g * Vnorm * Vnorm * a.A_plate * nh[k] / pi.m;
            for (int k = 0; k < D; ++k) Vpar[k] = Vdiff[k] - std::fabs(Vnorm) * nh[k];
            double Cf = 0.027 / std::pow(Re, 1.0 / 7.0);
            double Vparn = norm(Vpar, D);
            for (int k = 0; k < D; ++k) acc_skin[k] = 0.5 * a.rho_g * Vparn * Cf * a.A_plate * Vpar[k] / pi.m;
            double frac2 = std::min(1.5 * lam, 1.0);
            double frac1 = 1.0 - frac2;
            double Cdi = GetCd(Re);
            for (int k = 0; k < D; ++k)
                acc_drop[k] = 0.5 * a.rho_g * Vn * Vdiff[k] * (kPi * a.L * a.L / 4) * Cdi / pi.m;
            for (int k = 0; k < D; ++k) out[k] = frac2 * (acc_press[k] + acc_skin[k]) + frac1 * acc_drop[k];
        }
        break;
    }
    default:
        break;
    }
}

/* FLUID::get_pressure / get_density (Var.h:203-236) */
inline double get_pressure(const fjsph_settings &f, double rho) {
    if (f.pressure_rel == FJSPH_ISO_EOS) return f.speed_sound * f.speed_sound * (rho - f.rho_rest) + f.press_back;
    return f.B * (std::pow(rho / f.rho_rest, f.gam) - 1) + f.press_back;
}
inline double get_density(const fjsph_settings &f, double press) {
    if (f.pressure_rel == FJSPH_ISO_EOS) return (press - f.press_back) / (f.speed_sound * f.speed_sound) + f.rho_rest;
    return f.rho_rest * std::pow(((press - f.press_back) / f.B) + 1.0, 1.0 / f.gam);
}
inline double clamp_rho(const fjsph_settings &f, double lo, double v) { return std::max(lo, std::min(f.rho_max, v)); }

inline bool has(const orc_sim *o, uint32_t bit) { return (o->s.variant & bit) != 0; }

/* ------------------------------------------------------------------------------------------ */
/* Neighbours.cpp:7-47                                                                          */
/* ------------------------------------------------------------------------------------------ */
void find_neighbours(orc_sim *o, const std::vector<Part> &st, std::vector<std::vector<Nb>> &out) {
    const int D = o->D;
    const int64_t N = (int64_t)st.size();
    const double sr = o->s.sr;
    out.assign(N, {});
    if (N == 0) return;
    /* cell list, cell edge slightly above the search radius */
    const double cs = std::sqrt(sr) * (1.0 + 1e-6);
    double lo[3] = {0, 0, 0};
    for (int k = 0; k < D; ++k) {
        lo[k] = st[0].xi[k];
        for (int64_t i = 1; i < N; ++i) lo[k] = std::min(lo[k], st[i].xi[k]);
    }
    auto cell_of = [&](const double *x, int64_t *c) {
        for (int k = 0; k < D; ++k) c[k] = (int64_t)std::floor((x[k] - lo[k]) / cs);
        if (D == 2) c[2] = 0;
    };
    auto key = [](int64_t cx, int64_t cy, int64_t cz) -> uint64_t {
        return ((uint64_t)(cx + 1) & 0x1FFFFF) | (((uint64_t)(cy + 1) & 0x1FFFFF) << 21) |
               (((uint64_t)(cz + 1) & 0x1FFFFF) << 42);
    };
    std::unordered_map<uint64_t, std::vector<int64_t>> cells;
    cells.reserve(N);
    std::vector<int64_t> cc(3 * N);
    for (int64_t i = 0; i < N; ++i) {
        cell_of(st[i].xi, &cc[3 * i]);
        cells[key(cc[3 * i], cc[3 * i + 1], cc[3 * i + 2])].push_back(i);
    }
    const int zr = (D == 3) ? 1 : 0;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < N; ++i) {
        std::vector<Nb> &li = out[i];
        li.reserve(D == 3 ? 100 : 30);
        for (int dz = -zr; dz <= zr; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    auto it = cells.find(key(cc[3 * i] + dx, cc[3 * i + 1] + dy, cc[3 * i + 2] + dz));
                    if (it == cells.end()) continue;
                    for (int64_t j : it->second) {
                        double rr = dist2(st[i].xi, st[j].xi, D);
                        if (rr < sr) li.push_back({j, rr});
                    }
                }
        std::sort(li.begin(), li.end(), [](const Nb &a, const Nb &b) { return a.j < b.j; });
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Shifting.cpp:12-123 dSPH_PreStep                                                             */
/* ------------------------------------------------------------------------------------------ */
double dsph_prestep(orc_sim *o, int64_t end, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    const bool cubic = has(o, FJSPH_VAR_CUBIC);
    std::vector<double> npd_i(end, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < end; ++ii) {
        double Lm[9], Lnb[9], gradRho[3], nrm[3];
        zero(Lm, 9);
        zero(Lnb, 9);
        zero(gradRho, 3);
        zero(nrm, 3);
        double kernsum = 0.0, colour = 0.0, npd = 0.0;
        const Part &pi = P[ii];
        for (const Nb &jj : o->outlist[ii]) {
            if (jj.j == ii) {
                kernsum += f.W_correc;
                continue;
            }
            const Part &pj = P[jj.j];
            double Rji[3], mR[3], Grad[3];
            sub(pj.xi, pi.xi, D, Rji);
            double r = std::sqrt(jj.rr);
            double volj = pj.m / pj.rho;
            double kern = Kernel(r, f.H, f.W_correc, cubic);
            for (int k = 0; k < D; ++k) mR[k] = -Rji[k];
            GradK(mR, r, f.H, f.W_correc, cubic, D, Grad);
            for (int a = 0; a < D; ++a)
                for (int c = 0; c < D; ++c) Lm[a * D + c] -= volj * Rji[a] * Grad[c];
            for (int k = 0; k < D; ++k) gradRho[k] += volj * (pj.rho - pi.rho) * Grad[k];
            if (pj.b > FJSPH_PISTON) {
                for (int a = 0; a < D; ++a)
                    for (int c = 0; c < D; ++c) Lnb[a * D + c] -= volj * Rji[a] * Grad[c];
                for (int k = 0; k < D; ++k) nrm[k] += volj * Grad[k];
                kernsum += kern;
                colour += volj * kern;
                npd += kern;
            }
        }
        double Linv[9];
        zero(Linv, 9);
        for (int k = 0; k < D; ++k) Linv[k * D + k] = 1.0;
        double tmp[9];
        if (qr_inverse(Lm, D, tmp)) std::memcpy(Linv, tmp, sizeof(double) * D * D);
        double g2[3], n2[3];
        for (int a = 0; a < D; ++a) {
            g2[a] = 0.0;
            n2[a] = 0.0;
            for (int c = 0; c < D; ++c) {
                g2[a] += Linv[a * D + c] * gradRho[c];
                n2[a] += Linv[a * D + c] * nrm[c];
            }
        }
        Part &po = P[ii];
        if (pi.b == FJSPH_BOUND) {
            po.lam = 1.0;
            po.lam_nb = 1.0;
        } else {
            po.lam = min_eig(Lm, D);
            po.lam_nb = min_eig(Lnb, D);
        }
        std::memcpy(po.L, Linv, sizeof(double) * D * D);
        std::memcpy(po.gradRho, g2, sizeof(double) * D);
        std::memcpy(po.norm, n2, sizeof(double) * D);
        if (po.lam > 0.7)
            po.colourG = 2;
        else
            po.colourG = 2.0 * std::max(1.0, 1.0 / (2.0 * colour));
        po.kernsum = kernsum;
        po.colour = colour;
        npd_i[ii] = npd;
    }
    double npd = 0.0;
    for (int64_t ii = 0; ii < end; ++ii) npd += npd_i[ii];
    return npd / double(end);
}

/* ------------------------------------------------------------------------------------------ */
/* Resid.cpp:569-611 get_aero_velocity, constVel source                                         */
/* ------------------------------------------------------------------------------------------ */
/* ------------------------------------------------------------------------------------------ */
/* VLM.cpp: the vortex-lattice air velocity                                                      */
/* ------------------------------------------------------------------------------------------ */
inline void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

/* FindInfluence / FindInfluenceConditioned (VLM.cpp:324-430): velocity of a unit horseshoe with
 * bound vortex A-B and legs along v_inf; conditioned: zero when P is on one of its lines */
void vlm_influence(const double *A, const double *B, const double *P, const double *vinf, bool conditioned,
                   double *out) {
    const double ipi4 = 1.0 / (4.0 * kPi);
    zero(out, 3);
    double seg[3][3];
    for (int sgm = 0; sgm < 3; ++sgm) {
        double r0[3], r1[3], r2[3];
        for (int k = 0; k < 3; ++k) {
            if (sgm == 0) { /* bound */
                r0[k] = B[k] - A[k];
                r1[k] = P[k] - A[k];
                r2[k] = P[k] - B[k];
            } else if (sgm == 1) { /* A to infinity */
                const double inf = A[k] + vinf[k];
                r2[k] = P[k] - A[k];
                r1[k] = P[k] - inf;
                r0[k] = A[k] - inf;
            } else { /* B to infinity */
                const double inf = B[k] + vinf[k];
                r1[k] = P[k] - B[k];
                r2[k] = P[k] - inf;
                r0[k] = inf - B[k];
            }
        }
        double u1[3], u2[3], cu[3], c[3];
        normalized(r1, 3, u1);
        normalized(r2, 3, u2);
        if (conditioned) {
            cross3(u1, u2, cu);
            if (!(norm(cu, 3) > 1e-12)) return; /* the whole horseshoe is dropped */
        }
        cross3(r1, r2, c);
        const double den = sqnorm(c, 3);
        double f;
        if (sgm == 0) {
            double du[3];
            for (int k = 0; k < 3; ++k) du[k] = u1[k] - u2[k];
            f = ipi4 * dot(r0, du, 3) / den;
        } else if (sgm == 1) {
            f = ipi4 * norm(r0, 3) * (1.0 - dot(r0, r2, 3) / (norm(r0, 3) * norm(r2, 3))) / den;
        } else {
            f = ipi4 * norm(r0, 3) * (dot(r0, r1, 3) / (norm(r1, 3) * norm(r0, 3)) + 1.0) / den;
        }
        for (int k = 0; k < 3; ++k) seg[sgm][k] = f * c[k];
    }
    for (int k = 0; k < 3; ++k) out[k] = seg[0][k] + seg[2][k] + seg[1][k];
}

/* VLM::getVelocity (VLM.cpp:119-140) */
void vlm_velocity(const orc_sim *o, const double *P, double *vel) {
    for (int k = 0; k < 3; ++k) vel[k] = o->vlm_vinf[k];
    const size_t np = o->vlm_gamma.size();
    for (size_t q = 0; q < np; ++q) {
        double f[3];
        vlm_influence(&o->vlm_A[3 * q], &o->vlm_B[3 * q], P, o->vlm_vinf, true, f);
        for (int k = 0; k < 3; ++k) vel[k] += o->vlm_gamma[q] * f[k];
    }
    const double n = norm(vel, 3);
    double u[3];
    normalized(vel, 3, u);
    const double m = std::min(n, o->vlm_maxvel);
    for (int k = 0; k < 3; ++k) vel[k] = u[k] * m;
}

/* ------------------------------------------------------------------------------------------ */
/* Containment.cpp:385-421 CheckCell, Geometry.cpp:312-574 crossing tests, Containment.cpp:579-821 */
/* FindCell.  The candidate cells are those whose bounding sphere (largest centre-vertex        */
/* distance) holds the particle, scanned in full here; the containing one with the nearest      */
/* centre (then the lower index) is taken, as the nearest-centre walk of the reference finds.   */
/* Outside every cell, the boundary test uses the nearest centre among the cells whose doubled  */
/* sphere holds the particle.                                                                   */
/* ------------------------------------------------------------------------------------------ */
constexpr int64_t kMeshLost = -4;

bool m_cross_2d(const double *a, const double *b, double tx, double ty) {
    const bool y0 = a[1] >= ty, y1 = b[1] >= ty;
    if (y0 == y1) return false;
    return ((b[1] - ty) * (b[0] - a[0]) >= (b[0] - tx) * (b[1] - a[1])) == y1;
}

/* |p 1; a 1; b 1; c 1| < 0 */
bool m_neg_vol(const double *p, const double *a, const double *b, const double *c) {
    const double ax = a[0] - p[0], ay = a[1] - p[1], az = a[2] - p[2];
    const double bx = b[0] - p[0], by = b[1] - p[1], bz = b[2] - p[2];
    const double cx = c[0] - p[0], cy = c[1] - p[1], cz = c[2] - p[2];
    const double det = ax * (by * cz - bz * cy) - ay * (bx * cz - bz * cx) + az * (bx * cy - by * cx);
    return det > 0.0;
}

bool m_cross_3d(const orc_sim *o, int64_t f, const double *p, const double *q) {
    const int64_t f0 = o->m_face_off[f], f1 = o->m_face_off[f + 1];
    const double *v0 = &o->m_verts[3 * o->m_face_verts[f0]], *v1 = &o->m_verts[3 * o->m_face_verts[f0 + 1]];
    const double *v2 = &o->m_verts[3 * o->m_face_verts[f0 + 2]], *last = &o->m_verts[3 * o->m_face_verts[f1 - 1]];
    if (m_neg_vol(p, v0, v1, v2) == m_neg_vol(q, v0, v1, v2)) return false;
    const bool s3 = m_neg_vol(p, last, v0, q);
    if (m_neg_vol(p, v0, v1, q) != s3) return false;
    if (m_neg_vol(p, v1, v2, q) != s3) return false;
    return true;
}

bool m_check_cell(const orc_sim *o, int64_t cell, const double *p) {
    const int D = o->D;
    bool inside = false, line = false;
    const double ray[3] = {p[0] + 1e5, p[1], D == 3 ? p[2] : 0.0};
    for (int64_t e = o->m_cell_off[cell]; e < o->m_cell_off[cell + 1]; ++e) {
        const int64_t f = o->m_cell_faces[e];
        bool hit;
        if (D == 2) {
            const int64_t a = o->m_face_verts[o->m_face_off[f]], b = o->m_face_verts[o->m_face_off[f] + 1];
            hit = m_cross_2d(&o->m_verts[2 * a], &o->m_verts[2 * b], p[0], p[1]);
        } else {
            hit = m_cross_3d(o, f, p, ray);
        }
        if (hit) {
            inside = !inside;
            if (line) break;
            line = true;
        }
    }
    return inside;
}

bool m_seg_cross_2d(const orc_sim *o, int64_t f, const double *p, const double *c) {
    const int64_t a = o->m_face_verts[o->m_face_off[f]], b = o->m_face_verts[o->m_face_off[f] + 1];
    const double *e1 = &o->m_verts[2 * a], *e2 = &o->m_verts[2 * b];
    const double sx = c[0] - p[0], sy = c[1] - p[1], rx = e2[0] - e1[0], ry = e2[1] - e1[1];
    const double denom = -rx * sy + sx * ry;
    if (denom < kEps) return false;
    const double u = (-sy * (p[0] - e1[0]) + sx * (p[1] - e1[1])) / denom;
    const double t = (rx * (p[1] - e1[1]) - ry * (p[0] - e1[0])) / denom;
    return u > 0 && u < 1 && t > 0 && t < 1;
}

void find_cell(orc_sim *o, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &a = o->s;
    auto assign = [&](Part &pi, int64_t c) {
        pi.cellID = c;
        for (int k = 0; k < D; ++k) pi.cellV[k] = o->m_vel[c * D + k];
        pi.cellP = o->m_p[c];
        pi.cellRho = o->m_rho[c];
    };
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii) {
        Part &pi = P[ii];
        if (pi.b != FJSPH_FREE || pi.lam_nb > a.lam_cutoff) {
            pi.cellID = kNoCell;
            continue;
        }
        if (pi.cellID == kMeshLost) continue;
        const double p[3] = {pi.xi[0], pi.xi[1], D == 3 ? pi.xi[2] : 0.0};
        if (pi.cellID >= 0 && pi.cellID < o->m_ncells && m_check_cell(o, pi.cellID, p)) {
            assign(pi, pi.cellID);
            continue;
        }
        int64_t best = -1, nearest = -1;
        double best_d = 0.0, near_d = 0.0;
        for (int64_t c = 0; c < o->m_ncells; ++c) {
            double d2 = 0.0;
            for (int k = 0; k < D; ++k) {
                const double dd = p[k] - o->m_centre[c * D + k];
                d2 += dd * dd;
            }
            if (d2 > 4.0 * o->m_rad2[c]) continue; /* the nearest cell within twice its sphere */
            if (nearest < 0 || d2 < near_d) {
                nearest = c;
                near_d = d2;
            }
            if (d2 > o->m_rad2[c]) continue;
            if ((best < 0 || d2 < best_d) && m_check_cell(o, c, p)) {
                best = c;
                best_d = d2;
            }
        }
        if (best >= 0) {
            assign(pi, best);
        } else if (nearest >= 0) {
            const double cc[3] = {o->m_centre[nearest * D], o->m_centre[nearest * D + 1],
                                  D == 3 ? o->m_centre[nearest * D + 2] : 0.0};
            for (int64_t e = o->m_cell_off[nearest]; e < o->m_cell_off[nearest + 1]; ++e) {
                const int64_t f = o->m_cell_faces[e];
                const int32_t side = o->m_face_right[f];
                if (side >= 0) continue;
                const bool hit = D == 2 ? m_seg_cross_2d(o, f, p, cc) : m_cross_3d(o, f, p, cc);
                if (!hit) continue;
                if (side == -2) pi.cellID = kMeshLost;
                break;
            }
        }
    }
}

/* The boundary-layer air field in place of v_inf: v_inf s^n, s = (x[axis] - wall) / thickness
 * clamped to [0, 1] (n = 1/7: the turbulent power law). */
void power_law_velocity(const orc_sim *o, const double *x, double *vel) {
    const int axis = int(o->pl[0]);
    double t = (x[axis] - o->pl[1]) / o->pl[2];
    t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
    const double f = t == 1.0 ? 1.0 : std::pow(t, o->pl[3]);
    for (int k = 0; k < 3; ++k) vel[k] = o->s.v_inf[k] * f;
}

void get_aero_velocity(orc_sim *o, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &a = o->s;
    if (a.asource == FJSPH_MESH_INFL) { /* Resid.cpp:479-519: FindCell */
        find_cell(o, P);
        return;
    }
#pragma omp parallel for
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii) {
        Part &pi = P[ii];
        bool on;
        if (a.use_lam)
            on = pi.lam_nb < a.lam_cutoff && pi.b == FJSPH_FREE;
        else
            on = double(o->outlist[ii].size()) * a.i_n_full < a.lam_cutoff && pi.b == FJSPH_FREE;
        if (on) {
            if (a.asource == FJSPH_VLM_INFL)
                vlm_velocity(o, pi.xi, pi.cellV);
            else if (a.asource == FJSPH_POWER_LAW)
                power_law_velocity(o, pi.xi, pi.cellV);
            else
                for (int k = 0; k < D; ++k) pi.cellV[k] = a.v_inf[k];
            pi.cellID = 1;
        } else {
            zero(pi.cellV, D);
            pi.cellID = kNoCell;
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Geometry.cpp:14-280 Detect_Surface                                                           */
/* ------------------------------------------------------------------------------------------ */
void detect_surface(orc_sim *o, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &s = o->s;
    const bool cubic = has(o, FJSPH_VAR_CUBIC);
    const int64_t start = o->start_index, end = o->end_index;
    std::vector<double> norms(3 * end, 0.0);
    const double h = 1.33 * s.particle_step;
#pragma omp parallel for schedule(static)
    for (int64_t ii = start; ii < end; ++ii) {
        Part &pi = P[ii];
        double nrm[3] = {0, 0, 0};
        if (pi.b < FJSPH_PIPE) {
            pi.surf = 0;
            pi.woccl = 1;
        } else if (pi.lam_nb < 0.2) {
            pi.surf = 1;
        } else if (pi.lam_nb < 0.75) {
            double nh[3], pointT[3];
            normalized(pi.norm, D, nh);
            for (int k = 0; k < D; ++k) pointT[k] = pi.xi[k] + h * nh[k];
            int surf = 1;
            for (const Nb &jj : o->outlist[ii]) {
                if (jj.j == ii) continue;
                const Part &pj = P[jj.j];
                double x_jT[3];
                sub(pj.xi, pointT, D, x_jT);
                double r = std::sqrt(jj.rr);
                if (r >= std::sqrt(2.0) * h) {
                    if (norm(x_jT, D) < h) {
                        surf = 0;
                        break;
                    }
                } else {
                    if (D == 2) {
                        double tau[3] = {pi.norm[1], -pi.norm[0], 0}, th[3];
                        normalized(tau, D, th);
                        if ((std::fabs(dot(nh, x_jT, D)) + std::fabs(dot(th, x_jT, D))) < h) {
                            surf = 0;
                            break;
                        }
                    } else {
                        double Rij[3], mRr[3];
                        sub(pi.xi, pj.xi, D, Rij);
                        for (int k = 0; k < D; ++k) mRr[k] = -Rij[k] / r;
                        if (std::acos(dot(nh, mRr, D)) < kPi / 4.0) {
                            surf = 0;
                            break;
                        }
                    }
                }
            }
            pi.surf = surf;
        } else {
            pi.surf = 0;
        }
        /* normal from eigenvalue gradients */
        for (const Nb &jj : o->outlist[ii]) {
            if (jj.j == ii) continue;
            const Part &pj = P[jj.j];
            double Rij[3], g[3];
            sub(pi.xi, pj.xi, D, Rij);
            double r = std::sqrt(jj.rr);
            double volj = pj.m / pj.rho;
            GradK(Rij, r, s.H, s.W_correc, cubic, D, g);
            double w = (pi.lam > 0.7) ? volj * (pj.lam - pi.lam) : volj * pj.lam;
            for (int k = 0; k < D; ++k) nrm[k] += w * g[k];
        }
        double n2[3];
        for (int a = 0; a < D; ++a) {
            n2[a] = 0.0;
            for (int c = 0; c < D; ++c) n2[a] += pi.L[a * D + c] * nrm[c];
        }
        if (norm(n2, D) > 0.1 * pi.lam / s.H) normalized(n2, D, &norms[3 * ii]);
    }
    const bool gissler = s.acase == FJSPH_GISSLER;
#pragma omp parallel for schedule(static)
    for (int64_t ii = start; ii < end; ++ii) {
        Part &pi = P[ii];
        double woccl_ = 0.0;
        double Vdiff[3] = {0, 0, 0};
        if (pi.cellID != -1 && pi.b == FJSPH_FREE && gissler) {
            if (s.asource == FJSPH_MESH_INFL) { /* Geometry.cpp:154-157 */
                for (int k = 0; k < D; ++k) Vdiff[k] = pi.cellV[k] - pi.v[k];
            } else if (s.asource == FJSPH_VLM_INFL) { /* Geometry.cpp:158-163 */
                double vel[3];
                vlm_velocity(o, pi.xi, vel);
                for (int k = 0; k < D; ++k) Vdiff[k] = vel[k] - pi.v[k];
            } else if (s.asource == FJSPH_POWER_LAW) {
                double vel[3];
                power_law_velocity(o, pi.xi, vel);
                for (int k = 0; k < D; ++k) Vdiff[k] = vel[k] - pi.v[k];
            } else {
                for (int k = 0; k < D; ++k) Vdiff[k] = s.v_inf[k] - pi.v[k];
            }
        }
        double curve = 0.0;
        const double *ni = &norms[3 * ii];
        const double nin = norm(ni, D);
        const double vdn = norm(Vdiff, D);
        for (const Nb &jj : o->outlist[ii]) {
            if (jj.j == ii) continue;
            const Part &pj = P[jj.j];
            double Rij[3];
            sub(pj.xi, pi.xi, D, Rij);
            double r = std::sqrt(jj.rr);
            double volj = pj.m / pj.rho;
            const double *nj = (jj.j < end) ? &norms[3 * jj.j] : nullptr;
            if (nj && nin > 0 && norm(nj, D) > 0) {
                double dn[3], Ld[3], g[3];
                sub(nj, ni, D, dn);
                for (int a = 0; a < D; ++a) {
                    Ld[a] = 0.0;
                    for (int c = 0; c < D; ++c) Ld[a] += pi.L[a * D + c] * dn[c];
                }
                GradK(Rij, r, s.H, s.W_correc, cubic, D, g);
                curve += volj * dot(Ld, g, D);
            }
            if (pi.b == FJSPH_FREE && gissler) {
                double frac = -dot(Rij, Vdiff, D) / (vdn * r);
                if (frac > woccl_) woccl_ = frac;
            }
        }
        if (pi.lam_nb < s.lam_cutoff)
            pi.woccl = std::max(0.0, std::min(woccl_, 1.0));
        else
            pi.woccl = 1.0;
        for (int k = 0; k < D; ++k) pi.norm[k] = ni[k];
        pi.curve = curve;
        pi.norm_curve = s.dx * curve;
        pi.pDist = pi.lam;
    }
    if (has(o, FJSPH_VAR_ALE) || has(o, FJSPH_VAR_TIC)) {
#pragma omp parallel for schedule(static)
        for (int64_t ii = start; ii < end; ++ii) {
            int sz = 0;
            for (const Nb &jj : o->outlist[ii])
                if (P[jj.j].surf == 1) {
                    sz = 1;
                    break;
                }
            P[ii].surfzone = sz;
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Shifting.cpp:126-186 dissipation_terms                                                       */
/* ------------------------------------------------------------------------------------------ */
void dissipation_terms(orc_sim *o, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    const bool cubic = has(o, FJSPH_VAR_CUBIC), linear = has(o, FJSPH_VAR_LINEAR),
               nodsph = has(o, FJSPH_VAR_NODSPH);
#pragma omp parallel for schedule(static)
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii) {
        const Part &pi = P[ii];
        double av[3] = {0, 0, 0};
        double Rrhod = 0.0;
        for (const Nb &jj : o->outlist[ii]) {
            if (jj.j == ii) continue;
            const Part &pj = P[jj.j];
            double Rji[3], Vji[3], g[3];
            sub(pj.xi, pi.xi, D, Rji);
            sub(pj.v, pi.v, D, Vji);
            double rr = jj.rr, r = std::sqrt(rr);
            double idist2 = 1.0 / (rr + 0.0001 * f.H_sq);
            double volj = pj.m / pj.rho;
            GradK(Rji, r, f.H, f.W_correc, cubic, D, g);
            if (pj.b > FJSPH_PISTON) {
                if (linear) {
                    double c = volj * idist2 * dot(Vji, Rji, D);
                    for (int k = 0; k < D; ++k) av[k] += c * g[k];
                } else {
                    double t[3];
                    ArtVisc(f, pi, pj, Rji, Vji, idist2, g, D, t);
                    for (int k = 0; k < D; ++k) av[k] += pj.m * t[k];
                }
            }
            if (!nodsph) {
                if (pj.b > FJSPH_PISTON) {
                    double gs[3];
                    for (int k = 0; k < D; ++k) gs[k] = pi.gradRho[k] + pj.gradRho[k];
                    Rrhod += volj * ((pj.rho - pi.rho) + 0.5 * dot(gs, Rji, D)) * dot(Rji, g, D) * idist2;
                } else {
                    Rrhod += volj * (pj.rho - pi.rho) * dot(Rji, g, D) * idist2;
                }
            }
        }
        Part &po = P[ii];
        if (linear) {
            double c = f.visc_alpha * f.H * f.speed_sound * f.rho_rest / pi.rho;
            for (int k = 0; k < D; ++k) av[k] *= c;
        }
        for (int k = 0; k < D; ++k) po.aVisc[k] = av[k];
        if (!nodsph) po.deltaD = f.dsph_cont * Rrhod;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Shifting.cpp:189-290 particle_shift (-DALE)                                                  */
/* ------------------------------------------------------------------------------------------ */
void particle_shift(orc_sim *o, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &s = o->s;
    const bool cubic = has(o, FJSPH_VAR_CUBIC);
#pragma omp parallel for schedule(static)
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii) {
        if (P[ii].lam_nb < 0.55 || P[ii].b == FJSPH_BUFFER) {
            zero(P[ii].vPert, D);
            continue;
        }
        const Part &pi = P[ii];
        double dU[3] = {0, 0, 0};
        double maxUij = 0.0, woccl = 0.0;
        double ni[3];
        normalized(pi.norm, D, ni);
        for (const Nb &jj : o->outlist[ii]) {
            if (jj.j == ii) continue;
            const Part &pj = P[jj.j];
            double Rji[3], g[3];
            sub(pj.xi, pi.xi, D, Rji);
            double r = std::sqrt(jj.rr);
            double volj = pj.m / pj.rho;
            double kern = Kernel(r, s.H, s.W_correc, cubic);
            GradK(Rji, r, s.H, s.W_correc, cubic, D, g);
            double c = (1.0 + 0.2 * std::pow(kern / s.W_dx, 4.0));
            for (int k = 0; k < D; ++k) dU[k] += c * g[k] * volj;
            if (pj.b > FJSPH_PISTON) {
                double nj[3];
                normalized(pj.norm, D, nj);
                double theta = std::acos(dot(ni, nj, D));
                if (theta > woccl) woccl = theta;
            }
            double dv[3];
            sub(pj.v, pi.v, D, dv);
            double dvn = norm(dv, D);
            if (dvn > maxUij) maxUij = dvn;
        }
        double sc = -2.0 * s.H * norm(pi.v, D);
        for (int k = 0; k < D; ++k) dU[k] *= sc;
        double mag = std::min(norm(dU, D), std::min(maxUij / 2.0, s.max_shift_vel));
        double dUn[3];
        normalized(dU, D, dUn);
        for (int k = 0; k < D; ++k) dU[k] = mag * dUn[k];
        double nn[3];
        for (int k = 0; k < D; ++k) nn[k] = -ni[k];
        Part &po = P[ii];
        if (pi.surfzone == 0 && po.lam_nb > 0.55) {
            for (int k = 0; k < D; ++k) po.vPert[k] = dU[k];
        } else {
            if (woccl < kPi / 12.0) {
                for (int a = 0; a < D; ++a) {
                    double sacc = 0.0;
                    for (int c = 0; c < D; ++c) sacc += ((a == c ? 1.0 : 0.0) - nn[a] * nn[c]) * dU[c];
                    po.vPert[a] = sacc;
                }
            } else {
                zero(po.vPert, D);
            }
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Containment.cpp:822-894 Check_Pipe_Outlet (analytic air source: no cell lookup, no deletion)  */
/* ------------------------------------------------------------------------------------------ */
void check_pipe_outlet(orc_sim *o, std::vector<Part> &P) {
    const int D = o->D;
    for (int64_t blk = o->n_bound_blocks; blk < o->n_bound_blocks + o->n_fluid_blocks; ++blk) {
        const fjsph_block &B = o->limits[blk].d;
        for (int64_t ii = B.first; ii < B.second; ++ii)
            if (P[ii].b == FJSPH_PIPE && dot(P[ii].xi, B.aero_norm, D) > B.aeroconst) P[ii].b = FJSPH_FREE;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Resid.cpp:21-186 boundary passes                                                              */
/* ------------------------------------------------------------------------------------------ */
void get_boundary_pressure(orc_sim *o, int64_t start, int64_t end, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    const bool cubic = has(o, FJSPH_VAR_CUBIC);
    std::vector<double> pressure(end - start, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t ii = start; ii < end; ++ii) {
        const Part &pi = P[ii];
        int near = 0;
        double kernsum = 0.0, pkern = 0.0, acck[3] = {0, 0, 0};
        for (const Nb &jj : o->outlist[ii]) {
            const Part &pj = P[jj.j];
            if (pj.b > FJSPH_PISTON) {
                double Rji[3];
                sub(pi.xi, pj.xi, D, Rji);
                double r = std::sqrt(jj.rr);
                double volj = pj.m / pj.rho;
                double kern = volj * Kernel(r, f.H, f.W_correc, cubic);
                kernsum += kern;
                pkern += pj.p * kern;
                for (int k = 0; k < D; ++k) acck[k] += kern * pj.rho * Rji[k];
                if (pj.surfzone) near = 1;
            }
        }
        if (kernsum > 0.0) {
            double ga[3];
            for (int k = 0; k < D; ++k) ga[k] = f.grav[k] - pi.acc[k];
            double p = (pkern + dot(ga, acck, D)) / kernsum;
            pressure[ii - start] = near ? std::max(0.0, p) : p;
        }
    }
    for (int64_t ii = start; ii < end; ++ii) {
        P[ii].p = pressure[ii - start];
        P[ii].rho = get_density(f, pressure[ii - start]);
    }
}

/* Boundary_DBC: the reference scatters into RV_[neighbour] and then copies RV_ only over the
 * boundary range, where nothing was scattered; the boundary acceleration ends up zero. */
void boundary_dbc(orc_sim *o, int64_t start, int64_t end, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    const bool cubic = has(o, FJSPH_VAR_CUBIC);
    const double c2 = f.speed_sound * f.speed_sound;
    std::vector<double> RV(3 * end, 0.0);
    for (int64_t ii = start; ii < end; ++ii) {
        const Part &pi = P[ii];
        for (const Nb &jj : o->outlist[ii]) {
            const Part &pj = P[jj.j];
            if (jj.j == ii || pj.b < FJSPH_BUFFER) continue;
            if (jj.j >= end) continue; /* scattered contributions outside [0,end) are discarded */
            double Rji[3], Vji[3], g[3], av[3];
            sub(pj.xi, pi.xi, D, Rji);
            sub(pj.v, pi.v, D, Vji);
            double rr = jj.rr, r = std::sqrt(rr);
            double idist2 = 1.0 / (rr + 0.001 * f.H_sq);
            double kern = Kernel(r, f.H, f.W_correc, cubic);
            GradK(Rji, r, f.H, f.W_correc, cubic, D, g);
            ArtVisc(f, pi, pj, Rji, Vji, idist2, g, D, av);
            for (int k = 0; k < D; ++k)
                RV[3 * jj.j + k] -= 2.0 * c2 * kern / std::pow(kern + f.W_correc, 2.0) * g[k] + pj.m * av[k];
        }
    }
    for (int64_t ii = start; ii < end; ++ii)
        for (int k = 0; k < D; ++k) P[ii].acc[k] = RV[3 * ii + k];
}

void boundary_ghost(orc_sim *o, int64_t start, int64_t end, std::vector<Part> &P, std::vector<int32_t> &near_inlet) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    const bool cubic = has(o, FJSPH_VAR_CUBIC);
    std::vector<double> Rr(end - start, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t ii = start; ii < end; ++ii) {
        const Part &pi = P[ii];
        double Rrhoi = 0.0;
        int ni = 1;
        for (const Nb &jj : o->outlist[ii]) {
            const Part &pj = P[jj.j];
            if (jj.j == ii) continue;
            if (pj.b == FJSPH_PIPE || pj.b == FJSPH_FREE) ni = 0;
            double Rji[3], Vji[3], g[3];
            sub(pj.xi, pi.xi, D, Rji);
            sub(pj.v, pi.v, D, Vji);
            double r = std::sqrt(jj.rr);
            double volj = pj.m / pj.rho;
            GradK(Rji, r, f.H, f.W_correc, cubic, D, g);
            Rrhoi -= volj * dot(Vji, g, D);
        }
        near_inlet[ii] = ni;
        Rr[ii - start] = Rrhoi * pi.rho;
    }
    for (int64_t ii = start; ii < end; ++ii) P[ii].Rrho = Rr[ii - start];
}

void set_no_slip(orc_sim *o, int64_t start, int64_t end, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    const bool cubic = has(o, FJSPH_VAR_CUBIC);
    for (int64_t ii = start; ii < end; ++ii) {
        double vs[3] = {0, 0, 0}, ks = 0.0;
        for (const Nb &jj : o->outlist[ii]) {
            const Part &pj = P[jj.j];
            if (jj.j == ii || pj.b <= FJSPH_PISTON) continue;
            double r = std::sqrt(jj.rr);
            double kern = Kernel(r, f.H, f.W_correc, cubic);
            ks += kern;
            for (int k = 0; k < D; ++k) vs[k] += pj.v[k] * kern;
        }
        if (ks > 0.0)
            for (int k = 0; k < D; ++k) P[ii].v[k] = 2.0 * P[ii].v[k] - vs[k] / ks;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Resid.cpp:243-469 get_acc_and_Rrho                                                            */
/* ------------------------------------------------------------------------------------------ */
void acc_and_rrho_on_i(orc_sim *o, const std::vector<Part> &P, int64_t ii, double npdm2, double pi3o4,
                       double *acc_i, double *Af_i, double *Rrho_i) {
    const int D = o->D;
    const fjsph_settings &s = o->s;
    const bool cubic = has(o, FJSPH_VAR_CUBIC), ale = has(o, FJSPH_VAR_ALE), linear = has(o, FJSPH_VAR_LINEAR),
               nofrozen = has(o, FJSPH_VAR_NOFROZEN), nodsph = has(o, FJSPH_VAR_NODSPH), tic = has(o, FJSPH_VAR_TIC);
    const bool pairwise = s.st_model == FJSPH_ST_PAIRWISE, csf = s.st_model == FJSPH_ST_CSF;
    const Part &pi = P[ii];
    const std::vector<Nb> &li = o->outlist[ii];
    double acc[3] = {0, 0, 0}, acc_ale[3] = {0, 0, 0}, visc[3] = {0, 0, 0}, st[3] = {0, 0, 0};
    double art[3] = {0, 0, 0};
    double Rrho = 0.0, Rrhoc = 0.0, Rrho_d = 0.0;
    if (pi.cellID != -1) {
        double Vd[3], aero[3];
        sub(pi.cellV, pi.v, D, Vd);
        CalcAeroAcc(s, pi, Vd, pi.norm, pi.lam_nb, double(li.size()), D, aero);
        for (int k = 0; k < D; ++k) {
            acc[k] += aero[k];
            Af_i[k] = aero[k];
        }
    }
    for (const Nb &jj : li) {
        const Part &pj = P[jj.j];
        if (pi.part_id == pj.part_id) continue;
        double Rji[3], Vji[3], g[3];
        sub(pj.xi, pi.xi, D, Rji);
        sub(pj.v, pi.v, D, Vji);
        double rr = jj.rr, r = std::sqrt(rr);
        double idist2 = 1.0 / (rr + 0.001 * s.H_sq);
        double volj = pj.m / pj.rho;
        GradK(Rji, r, s.H, s.W_correc, cubic, D, g);
        /* PressureContrib (Resid.cpp:188-210) */
        double contrib[3];
        if (linear) {
            double pp = (tic && pi.surfzone != 1) ? (std::fabs(pi.p) + pj.p) : (pi.p + pj.p);
            for (int k = 0; k < D; ++k) contrib[k] = g[k] * pp * volj;
        } else {
            double a = pi.p / (pi.rho * pi.rho);
            if (tic && pi.surfzone != 1) a = std::fabs(a);
            double t = a + pj.p / (pj.rho * pj.rho);
            for (int k = 0; k < D; ++k) contrib[k] = pj.m * g[k] * t;
        }
        /* Viscosity (Kernel.h:262-269) */
        {
            double c = s.nu * (pi.rho + pj.rho) / (pi.rho * pj.rho) * dot(Rji, g, D) * idist2;
            for (int k = 0; k < D; ++k) visc[k] += pj.m * (c * Vji[k]);
        }
        /* SurfTenContrib (Resid.cpp:212-240) */
        if (pairwise && (!ale || pi.surfzone == 1)) {
            double fac = pairwise_ST_fac(pi.b, pj.b);
            double c = -npdm2 * fac * std::cos(pi3o4 * r / s.H);
            for (int k = 0; k < D; ++k) st[k] += c * (Rji[k] / r);
        }
        for (int k = 0; k < D; ++k) acc[k] -= contrib[k];
        if (ale) {
            /* ALEMomentum (Kernel.h:179-185) */
            double M[9];
            for (int a = 0; a < D; ++a)
                for (int c = 0; c < D; ++c) M[a * D + c] = pj.v[a] * pj.vPert[c] + pi.v[a] * pi.vPert[c];
            double dvp[3];
            sub(pj.vPert, pi.vPert, D, dvp);
            double q = dot(dvp, g, D);
            for (int a = 0; a < D; ++a) {
                double mg = 0.0;
                for (int c = 0; c < D; ++c) mg += M[a * D + c] * g[c];
                acc_ale[a] += (mg - pi.v[a] * q) * volj;
            }
            /* ALEContinuity / ALECont2ndterm (Kernel.h:187-195) */
            double w1[3], w2[3];
            for (int k = 0; k < D; ++k) {
                w1[k] = (pj.v[k] + pj.vPert[k]) - (pi.v[k] + pi.vPert[k]);
                w2[k] = pj.rho * pj.vPert[k] + pi.rho * pi.vPert[k];
            }
            Rrho -= dot(w1, g, D) * volj;
            Rrhoc += dot(w2, g, D) * volj;
        } else {
            Rrho -= volj * dot(Vji, g, D);
        }
        if (nofrozen) {
            if (pj.b > FJSPH_PISTON) {
                if (!nodsph) {
                    double gs[3];
                    for (int k = 0; k < D; ++k) gs[k] = pi.gradRho[k] + pj.gradRho[k];
                    Rrho_d += volj * ((pj.rho - pi.rho) + 0.5 * dot(gs, Rji, D)) * dot(Rji, g, D) * idist2;
                }
                if (linear) {
                    double c = volj * idist2 * dot(Vji, Rji, D);
                    for (int k = 0; k < D; ++k) art[k] += c * g[k];
                } else {
                    double t[3];
                    ArtVisc(s, pi, pj, Rji, Vji, idist2, g, D, t);
                    for (int k = 0; k < D; ++k) art[k] += pj.m * t[k];
                }
            } else if (!nodsph) {
                Rrho_d += volj * (pj.rho - pi.rho) * dot(Rji, g, D) * idist2;
            }
        }
    }
    if (linear)
        for (int k = 0; k < D; ++k) acc[k] /= pi.rho;
    if (csf)
        for (int k = 0; k < D; ++k) acc[k] += 1.0 / pi.rho * s.sig * pi.curve * pi.norm[k] * pi.colourG;
    const double *av = nofrozen ? art : pi.aVisc;
    for (int k = 0; k < D; ++k) {
        double t = acc[k];
        if (ale) t += acc_ale[k];
        acc_i[k] = t + av[k] + visc[k] + st[k] / pi.m + s.grav[k];
    }
    double R = Rrho * pi.rho;
    if (ale) R += Rrhoc;
    if (!nodsph) R += nofrozen ? s.dsph_cont * Rrho_d : pi.deltaD;
    *Rrho_i = R;
}

void get_acc_and_rrho(orc_sim *o, double npd, std::vector<Part> &P) {
    const fjsph_settings &s = o->s;
    double npdm2 = 0.0, pi3o4 = 0.0;
    if (s.st_model == FJSPH_ST_PAIRWISE) {
        double lam = (6.0 / 81.0 * std::pow((2.0 * s.H), 3.0) / std::pow(kPi, 4.0) *
                      (9.0 / 4.0 * std::pow(kPi, 3.0) - 6.0 * kPi - 4.0));
        npdm2 = (0.5 * s.sig / lam) / (npd * npd);
        pi3o4 = 3.0 * kPi / 4.0;
    }
    const int D = o->D;
    std::vector<double> out(7 * P.size(), 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii) {
        double a[3], af[3], R;
        for (int k = 0; k < D; ++k) af[k] = P[ii].Af[k];
        acc_and_rrho_on_i(o, P, ii, npdm2, pi3o4, a, af, &R);
        for (int k = 0; k < D; ++k) {
            out[7 * ii + k] = a[k];
            out[7 * ii + 3 + k] = af[k];
        }
        out[7 * ii + 6] = R;
    }
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii) {
        for (int k = 0; k < D; ++k) {
            P[ii].acc[k] = out[7 * ii + k];
            P[ii].Af[k] = out[7 * ii + 3 + k];
        }
        P[ii].Rrho = out[7 * ii + 6];
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Runge_Kutta.cpp                                                                                */
/* ------------------------------------------------------------------------------------------ */
/* Boundary velocity of a block at the current time.  Runge_Kutta.cpp:39-63 takes the last table
 * entry with time > current_time; Newmark_Beta.cpp:71-96 the last with current_time > time. */
void block_velocity(const orc_sim *o, const fjsph_block &B, bool rk, double *vel) {
    zero(vel, 3);
    if (B.n_times != 0) {
        for (int t = 0; t < B.n_times; ++t) {
            bool hit = rk ? (B.times[t] > o->s.current_time) : (o->s.current_time > B.times[t]);
            if (hit)
                for (int k = 0; k < 3; ++k) vel[k] = B.vels[t][k];
        }
    } else {
        for (int k = 0; k < 3; ++k) vel[k] = B.vels[0][k];
    }
}

/* Boundary section of do_runge_kutta_intermediate_step (:36-133) / final_step (:242-351).
 * mode 0: intermediate with dt_inter; mode 1: final, Rrho weights from the stages. */
void rk_boundaries(orc_sim *o, const std::vector<Part> &pn, std::vector<Part> &S, int mode, double dt,
                   const std::vector<Part> *st1, const std::vector<Part> *st2, const std::vector<Part> *st3) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    std::vector<int32_t> near_inlet(S.size(), 0);
    for (int64_t blk = 0; blk < o->n_bound_blocks; ++blk) {
        const fjsph_block &B = o->limits[blk].d;
        double vel[3];
        block_velocity(o, B, true, vel);
        for (int64_t jj = B.first; jj < B.second; ++jj)
            for (int k = 0; k < D; ++k) S[jj].v[k] = vel[k];
        if (B.no_slip) set_no_slip(o, B.first, B.second, S);
        auto rho_new = [&](int64_t ii) {
            if (mode == 0) return pn[ii].rho + dt * S[ii].Rrho;
            return pn[ii].rho + (dt / 6.0) * (pn[ii].Rrho + 2.0 * (*st1)[ii].Rrho + 2.0 * (*st2)[ii].Rrho +
                                              (*st3)[ii].Rrho);
        };
        switch (B.bound_solver) {
        case FJSPH_DBC:
            boundary_dbc(o, B.first, B.second, S);
            for (int64_t ii = B.first; ii < B.second; ++ii) {
                double rho = clamp_rho(f, f.rho_min, rho_new(ii));
                S[ii].rho = rho;
                S[ii].p = get_pressure(f, rho);
                if (mode == 1) S[ii].Rrho = (*st3)[ii].Rrho;
            }
            break;
        case FJSPH_PRESSURE_G:
            get_boundary_pressure(o, B.first, B.second, S);
            break;
        case FJSPH_GHOST:
            boundary_ghost(o, B.first, B.second, S, near_inlet);
            for (int64_t ii = B.first; ii < B.second; ++ii) {
                if (!near_inlet[ii]) {
                    double rho = clamp_rho(f, f.rho_min, rho_new(ii));
                    S[ii].rho = rho;
                    S[ii].p = get_pressure(f, rho);
                } else {
                    double rho = clamp_rho(f, f.rho_rest, rho_new(ii));
                    S[ii].rho = rho;
                    S[ii].p = get_pressure(f, rho);
                    S[ii].Rrho = std::fmax(0.0, S[ii].Rrho);
                }
            }
            break;
        default:
            break;
        }
    }
}

std::vector<Part> rk_intermediate(orc_sim *o, double npd, const std::vector<Part> &pn,
                                  const std::vector<Part> &prev, double dt) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    const bool ale = has(o, FJSPH_VAR_ALE);
    std::vector<Part> S = prev;
    rk_boundaries(o, pn, S, 0, dt, nullptr, nullptr, nullptr);
    get_acc_and_rrho(o, npd, S);
    for (int64_t blk = o->n_bound_blocks; blk < o->n_bound_blocks + o->n_fluid_blocks; ++blk) {
        const Block &BB = o->limits[blk];
        const fjsph_block &B = BB.d;
#pragma omp parallel for schedule(static)
        for (int64_t ii = B.first; ii < B.second; ++ii) {
            Part &q = S[ii];
            if (q.b > FJSPH_BUFFER) {
                for (int k = 0; k < D; ++k) {
                    double vv = ale ? (q.v[k] + q.vPert[k]) : q.v[k];
                    q.xi[k] = pn[ii].xi[k] + dt * vv;
                }
                for (int k = 0; k < D; ++k) q.v[k] = pn[ii].v[k] + dt * q.acc[k];
                double rho = clamp_rho(f, f.rho_min, pn[ii].rho + dt * q.Rrho);
                q.rho = rho;
                q.p = get_pressure(f, rho);
            }
        }
        if (B.block_type == kInletZone) {
            if (B.fixed_vel_or_dynamic == 1) {
                double un[3];
                normalized(B.insert_norm, D, un);
                for (size_t ii = 0; ii < BB.back.size(); ++ii) {
                    int64_t backID = BB.back[ii];
                    for (size_t jj = 0; jj < BB.buffer[ii].size(); ++jj) {
                        int64_t bid = BB.buffer[ii][jj];
                        for (int k = 0; k < D; ++k) S[bid].xi[k] = S[backID].xi[k] - f.dx * (jj + 1.0) * un[k];
                        for (int k = 0; k < D; ++k) S[bid].v[k] = S[backID].v[k];
                        S[bid].rho = S[backID].rho;
                        S[bid].p = S[backID].p;
                    }
                }
            } else {
                /* Fixed-velocity inlet.  The reference indexes limits[jj] here (an out-of-range
                 * block); the block's own buffer table is used instead. */
                for (size_t ii = 0; ii < BB.back.size(); ++ii)
                    for (size_t jj = 0; jj < BB.buffer[ii].size(); ++jj) {
                        int64_t bid = BB.buffer[ii][jj];
                        double rho = clamp_rho(f, f.rho_min, pn[bid].rho + dt * S[bid].Rrho);
                        S[bid].rho = rho;
                        S[bid].p = get_pressure(f, rho);
                        for (int k = 0; k < D; ++k) S[bid].xi[k] = pn[bid].xi[k] + dt * pn[bid].v[k];
                    }
            }
        }
    }
    return S;
}

std::vector<Part> rk_final(orc_sim *o, double npd, double dt, const std::vector<Part> &pn,
                           const std::vector<Part> &st1, const std::vector<Part> &st2,
                           const std::vector<Part> &st3) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    const bool ale = has(o, FJSPH_VAR_ALE);
    std::vector<Part> S = st3;
    rk_boundaries(o, pn, S, 1, dt, &st1, &st2, &st3);
    get_acc_and_rrho(o, npd, S);
    for (int64_t blk = o->n_bound_blocks; blk < o->n_bound_blocks + o->n_fluid_blocks; ++blk) {
        const Block &BB = o->limits[blk];
        const fjsph_block &B = BB.d;
#pragma omp parallel for schedule(static)
        for (int64_t ii = B.first; ii < B.second; ++ii) {
            Part &q = S[ii];
            if (q.b > FJSPH_BUFFER && q.b != FJSPH_OUTLET) {
                for (int k = 0; k < D; ++k) {
                    if (ale)
                        q.xi[k] = pn[ii].xi[k] + (dt / 6.0) * ((pn[ii].v[k] + pn[ii].vPert[k]) +
                                                              2.0 * (st1[ii].v[k] + st1[ii].vPert[k]) +
                                                              2.0 * (st2[ii].v[k] + st2[ii].vPert[k]) +
                                                              (st3[ii].v[k] + st3[ii].vPert[k]));
                    else
                        q.xi[k] = pn[ii].xi[k] +
                                  (dt / 6.0) * (pn[ii].v[k] + 2.0 * st1[ii].v[k] + 2.0 * st2[ii].v[k] + st3[ii].v[k]);
                }
                for (int k = 0; k < D; ++k)
                    q.v[k] = pn[ii].v[k] + (dt / 6.0) * (pn[ii].acc[k] + 2.0 * st1[ii].acc[k] +
                                                          2.0 * st2[ii].acc[k] + st3[ii].acc[k]);
                double rho = clamp_rho(f, f.rho_min,
                                       pn[ii].rho + (dt / 6.0) * (pn[ii].Rrho + 2.0 * st1[ii].Rrho +
                                                                   2.0 * st2[ii].Rrho + st3[ii].Rrho));
                q.rho = rho;
                q.p = get_pressure(f, rho);
            } else if (q.b == FJSPH_OUTLET) {
                for (int k = 0; k < D; ++k) q.xi[k] = pn[ii].xi[k] + dt * q.v[k];
            }
        }
        if (B.block_type == kInletZone) {
            if (B.fixed_vel_or_dynamic == 1) {
                double un[3];
                normalized(B.insert_norm, D, un);
                for (size_t ii = 0; ii < BB.back.size(); ++ii) {
                    int64_t backID = BB.back[ii];
                    for (size_t jj = 0; jj < BB.buffer[ii].size(); ++jj) {
                        int64_t bid = BB.buffer[ii][jj];
                        for (int k = 0; k < D; ++k) S[bid].xi[k] = S[backID].xi[k] - f.dx * (jj + 1.0) * un[k];
                        for (int k = 0; k < D; ++k) S[bid].v[k] = S[backID].v[k];
                        S[bid].rho = S[backID].rho;
                        S[bid].p = S[backID].p;
                    }
                }
            } else {
                /* The reference reads limits[jj] and the Rrho of particle ii here; the buffer
                 * particle's own stage densities are used instead. */
                for (size_t ii = 0; ii < BB.back.size(); ++ii)
                    for (size_t jj = 0; jj < BB.buffer[ii].size(); ++jj) {
                        int64_t bid = BB.buffer[ii][jj];
                        double rho = clamp_rho(
                            f, f.rho_min,
                            pn[bid].rho + (dt / 6.0) * (pn[bid].Rrho + 2.0 * st1[bid].Rrho + 2.0 * st2[bid].Rrho +
                                                         st3[bid].Rrho));
                        S[bid].rho = rho;
                        S[bid].p = get_pressure(f, rho);
                        for (int k = 0; k < D; ++k) S[bid].xi[k] = pn[bid].xi[k] + dt * pn[bid].v[k];
                    }
            }
        }
    }
    return S;
}

/* Runge_Kutta.cpp:10-26 */
double check_rk_error(const orc_sim *o, double logbase, const std::vector<Part> &a, const std::vector<Part> &b) {
    const int D = o->D;
    double errsum = 0.0;
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii) {
        double d[3];
        sub(b[ii].xi, a[ii].xi, D, d);
        errsum += sqnorm(d, D);
    }
    return std::log10(std::sqrt(errsum / double(o->end_index - o->start_index))) - logbase;
}

/* ------------------------------------------------------------------------------------------ */
/* Newmark_Beta.cpp                                                                              */
/* ------------------------------------------------------------------------------------------ */
void nb_iter(orc_sim *o, double npd, const std::vector<Part> &pn, std::vector<Part> &P) {
    const int D = o->D;
    const fjsph_settings &f = o->s;
    const bool ale = has(o, FJSPH_VAR_ALE);
    std::vector<int32_t> near_inlet(P.size(), 0);
    const double g1 = f.nb_gamma, g2 = 1 - g1, b1 = f.nb_beta, b2 = 0.5 * (1 - 2 * b1);
    for (int64_t blk = 0; blk < o->n_bound_blocks; ++blk) {
        const fjsph_block &B = o->limits[blk].d;
        double vel[3];
        block_velocity(o, B, false, vel);
        for (int64_t jj = B.first; jj < B.second; ++jj)
            for (int k = 0; k < D; ++k) P[jj].v[k] = vel[k];
        if (B.no_slip) set_no_slip(o, B.first, B.second, P);
        switch (B.bound_solver) {
        case FJSPH_DBC:
            boundary_dbc(o, B.first, B.second, P);
            break;
        case FJSPH_PRESSURE_G:
            get_boundary_pressure(o, B.first, B.second, P);
            break;
        case FJSPH_GHOST:
            boundary_ghost(o, B.first, B.second, P, near_inlet);
            break;
        default:
            break;
        }
    }
    get_acc_and_rrho(o, npd, P);
    const double dt = f.delta_t, dt2 = dt * dt;
    for (int64_t blk = 0; blk < o->n_bound_blocks; ++blk) {
        const fjsph_block &B = o->limits[blk].d;
        if (B.bound_solver == FJSPH_DBC) {
            for (int64_t ii = B.first; ii < B.second; ++ii) {
                double rho = clamp_rho(f, f.rho_min, pn[ii].rho + dt * (g1 * P[ii].Rrho + g2 * pn[ii].Rrho));
                P[ii].rho = rho;
                P[ii].p = get_pressure(f, rho);
            }
        } else if (B.bound_solver == FJSPH_GHOST) {
            for (int64_t ii = B.first; ii < B.second; ++ii) {
                if (near_inlet[ii]) {
                    double rho = clamp_rho(f, f.rho_rest, pn[ii].rho + dt * (g1 * P[ii].Rrho + g2 * pn[ii].Rrho));
                    P[ii].rho = rho;
                    P[ii].p = get_pressure(f, rho);
                    P[ii].Rrho = std::fmax(0.0, P[ii].Rrho);
                } else {
                    double rho = clamp_rho(f, f.rho_min, pn[ii].rho + dt * (g1 * P[ii].Rrho + g2 * pn[ii].Rrho));
                    P[ii].rho = rho;
                    P[ii].p = get_pressure(f, rho);
                }
            }
        }
    }
    for (int64_t blk = o->n_bound_blocks; blk < o->n_bound_blocks + o->n_fluid_blocks; ++blk) {
        const Block &BB = o->limits[blk];
        const fjsph_block &B = BB.d;
#pragma omp parallel for schedule(static)
        for (int64_t ii = B.first; ii < B.second; ++ii) {
            Part &q = P[ii];
            if (q.b > FJSPH_BUFFER && q.b != FJSPH_OUTLET) {
                for (int k = 0; k < D; ++k) {
                    if (ale)
                        q.xi[k] = pn[ii].xi[k] + dt * (pn[ii].v[k] + q.vPert[k]) + dt2 * (b1 * q.acc[k] + b2 * pn[ii].acc[k]);
                    else
                        q.xi[k] = pn[ii].xi[k] + dt * pn[ii].v[k] + dt2 * (b2 * pn[ii].acc[k] + b1 * q.acc[k]);
                }
                for (int k = 0; k < D; ++k) q.v[k] = pn[ii].v[k] + dt * (g1 * q.acc[k] + g2 * pn[ii].acc[k]);
                double rho = clamp_rho(f, f.rho_min, pn[ii].rho + dt * (g1 * q.Rrho + g2 * pn[ii].Rrho));
                q.rho = rho;
                q.p = get_pressure(f, rho);
            } else if (q.b == FJSPH_OUTLET) {
                for (int k = 0; k < D; ++k) q.xi[k] = pn[ii].xi[k] + dt * q.v[k];
            }
        }
        if (B.block_type == kInletZone) {
            if (B.fixed_vel_or_dynamic == 1) {
                double un[3];
                normalized(B.insert_norm, D, un);
                for (size_t ii = 0; ii < BB.back.size(); ++ii) {
                    int64_t backID = BB.back[ii];
                    for (size_t jj = 0; jj < BB.buffer[ii].size(); ++jj) {
                        int64_t bid = BB.buffer[ii][jj];
                        for (int k = 0; k < D; ++k) P[bid].xi[k] = P[backID].xi[k] - f.dx * (jj + 1.0) * un[k];
                        for (int k = 0; k < D; ++k) P[bid].v[k] = P[backID].v[k];
                        P[bid].rho = P[backID].rho;
                        P[bid].p = P[backID].p;
                    }
                }
            } else {
                for (size_t ii = 0; ii < BB.back.size(); ++ii)
                    for (size_t jj = 0; jj < BB.buffer[ii].size(); ++jj) {
                        int64_t bid = BB.buffer[ii][jj];
                        double rho = clamp_rho(f, f.rho_min, pn[bid].rho + dt * (g1 * P[bid].Rrho + g2 * pn[bid].Rrho));
                        P[bid].rho = rho;
                        P[bid].p = get_pressure(f, rho);
                        for (int k = 0; k < D; ++k) P[bid].xi[k] = pn[bid].xi[k] + dt * pn[bid].v[k];
                    }
            }
        }
    }
}

/* Newmark_Beta.cpp:10-52 */
int nb_check_error(orc_sim *o, double &rms_error, double &logbase, const std::vector<double> &xih) {
    const int D = o->D;
    double errsum = 0.0;
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii) {
        double d[3];
        sub(o->pnp1[ii].xi, &xih[3 * (ii - o->start_index)], D, d);
        errsum += sqnorm(d, D);
    }
    double log_error = std::log10(std::sqrt(errsum / double(o->end_index - o->start_index)));
    if (o->iteration == 0) logbase = log_error;
    rms_error = log_error - logbase;
    if ((int64_t)o->iteration > (int64_t)o->s.max_subits) {
        if (rms_error > 0.0) {
            o->pnp1 = o->pn;
            find_neighbours(o, o->pnp1, o->outlist);
            o->s.delta_t = 0.5 * o->s.delta_t;
            o->iteration = 0;
            rms_error = 0.0;
            return -1;
        }
        return 1;
    }
    return 0;
}

void save_x(const orc_sim *o, std::vector<double> &xih) {
    xih.assign(3 * (o->end_index - o->start_index), 0.0);
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii)
        for (int k = 0; k < o->D; ++k) xih[3 * (ii - o->start_index) + k] = o->pnp1[ii].xi[k];
}

double newmark_beta_loop(orc_sim *o, double npd, double &logbase) {
    double rms_error = 0.0;
    std::vector<double> xih;
    int restarts = 0;
    while (rms_error > o->s.min_residual) {
        save_x(o, xih);
        nb_iter(o, npd, o->pn, o->pnp1);
        int e = nb_check_error(o, rms_error, logbase, xih);
        if (e == 0)
            o->iteration++;
        else if (e == 1)
            break;
        else if (++restarts > 64)
            break; /* the reference would loop without bound here */
    }
    return rms_error;
}

/* ------------------------------------------------------------------------------------------ */
/* Integration.cpp                                                                               */
/* ------------------------------------------------------------------------------------------ */
double find_timestep(orc_sim *o) {
    const int D = o->D;
    const fjsph_settings &s = o->s;
    double maxf = kEps, maxAf = kEps, maxRhoi = kEps, maxdrho = kEps, maxU = kEps, minST = 9999999.0;
    double maxShift = o->maxShift;
    const std::vector<Part> &P = o->pnp1;
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii) {
        maxf = std::max(maxf, norm(P[ii].acc, D));
        maxAf = std::max(maxAf, norm(P[ii].Af, D));
        maxdrho = std::max(maxdrho, std::fabs(P[ii].Rrho));
        maxRhoi = std::max(maxRhoi, std::fabs(P[ii].rho - s.rho_rest));
        minST = std::min(minST, std::sqrt(P[ii].rho * s.dx * s.dx / (2.0 * kPi * s.sig * std::fabs(P[ii].curve))));
        maxU = std::max(maxU, norm(P[ii].v, D));
        if (o->s.variant & FJSPH_VAR_ALE) maxShift = std::max(maxShift, norm(P[ii].vPert, D));
    }
    o->maxf = maxf;
    o->maxAf = maxAf;
    o->maxRhoi = maxRhoi;
    o->maxdrho = maxdrho;
    o->maxU = maxU;
    o->minST = minST;
    o->maxShift = maxShift;
    o->maxRho_pc = 100 * maxRhoi / s.rho_rest;
    double fac[6] = {0.25 * std::sqrt(s.H / maxf), 2 * s.H / maxU, 0.125 * s.H_sq * s.rho_rest / s.mu,
                     0.067 * minST, 0.5 * std::sqrt(s.H / maxdrho), 1.5 * s.H / s.speed_sound};
    double mn = fac[0];
    for (int k = 1; k < 6; ++k)
        if (fac[k] < mn) mn = fac[k];
    o->safe_dt = 0.75 * mn;
    double dt = s.cfl * o->safe_dt;
    if (dt < s.delta_t_min)
        dt = s.delta_t_min;
    else if (dt > s.delta_t_max)
        dt = s.delta_t_max;
    if (dt > s.last_frame_time + s.frame_time_interval - s.current_time)
        dt = s.last_frame_time + s.frame_time_interval - s.current_time + s.delta_t_min;
    return dt;
}

void prestep_passes(orc_sim *o, double &npd) {
    npd = dsph_prestep(o, o->total_points, o->pnp1);
    get_aero_velocity(o, o->pnp1);
    detect_surface(o, o->pnp1);
    if (!has(o, FJSPH_VAR_NOFROZEN)) dissipation_terms(o, o->pnp1);
    if (has(o, FJSPH_VAR_ALE)) particle_shift(o, o->pnp1);
    check_pipe_outlet(o, o->pnp1);
}

double integrate_no_update(orc_sim *o) {
    o->start_index = o->bound_points;
    o->end_index = o->total_points;
    o->iteration = 0;
    double npd = 1.0, logbase = 0.0, rms_error = 0.0;
    o->s.delta_t = find_timestep(o);
    find_neighbours(o, o->pnp1, o->outlist);
    prestep_passes(o, npd);
    if (o->s.solver_type == FJSPH_RUNGE_KUTTA) {
        const double dt = 0.5 * o->s.delta_t;
        o->pnp1 = rk_intermediate(o, npd, o->pn, o->pn, dt);
        logbase = check_rk_error(o, 0.0, o->pn, o->pnp1);
    } else {
        std::vector<double> xih;
        save_x(o, xih);
        nb_iter(o, npd, o->pn, o->pnp1);
        nb_check_error(o, rms_error, logbase, xih);
        o->iteration++;
    }
    find_neighbours(o, o->pnp1, o->outlist);
    prestep_passes(o, npd);
    if (o->s.solver_type == FJSPH_RUNGE_KUTTA) {
        std::vector<Part> st1 = o->pnp1;
        const double dti = 0.5 * o->s.delta_t, dtf = o->s.delta_t;
        std::vector<Part> st2 = rk_intermediate(o, npd, o->pn, st1, dti);
        std::vector<Part> st3 = rk_intermediate(o, npd, o->pn, st2, dtf);
        o->pnp1 = rk_final(o, npd, dtf, o->pn, st1, st2, st3);
        rms_error = check_rk_error(o, logbase, st3, o->pnp1);
    } else {
        rms_error = newmark_beta_loop(o, npd, logbase);
    }
    return rms_error;
}

/* inlet.cpp:578-640 update_buffer_region */
uint32_t update_buffer_region(orc_sim *o) {
    const int D = o->D;
    uint32_t nAdd = 0;
    for (int64_t blk = o->n_bound_blocks; blk < o->n_bound_blocks + o->n_fluid_blocks; ++blk) {
        Block &BB = o->limits[blk];
        if (BB.d.block_type != kInletZone) continue;
        for (size_t ii = 0; ii < BB.back.size(); ++ii) {
            int64_t pID = BB.back[ii];
            if (dot(o->pnp1[pID].xi, BB.d.insert_norm, D) > BB.d.insconst) {
                o->pnp1[pID].b = FJSPH_PIPE;
                o->pnp1[BB.buffer[ii][0]].b = FJSPH_BACK;
                BB.back[ii] = BB.buffer[ii][0];
                for (size_t jj = 0; jj + 1 < BB.buffer[0].size(); ++jj) BB.buffer[ii][jj] = BB.buffer[ii][jj + 1];
                if (o->total_points < o->s.max_points) {
                    const Part &src = o->pnp1[BB.buffer[ii].back()];
                    Part np{};
                    for (int k = 0; k < D; ++k) np.xi[k] = src.xi[k] - o->s.dx * BB.d.insert_norm[k];
                    for (int k = 0; k < D; ++k) np.v[k] = src.v[k];
                    np.rho = src.rho;
                    np.p = src.p;
                    np.m = src.m;
                    np.cellP = src.cellP;
                    np.cellRho = src.cellRho;
                    np.cellID = kNoCell;
                    np.b = FJSPH_BUFFER;
                    np.part_id = o->part_id_next;
                    o->pnp1.insert(o->pnp1.begin() + BB.d.second, np);
                    BB.buffer[ii].back() = BB.d.second;
                    BB.d.second++;
                    for (int64_t jb = blk + 1; jb < o->n_bound_blocks + o->n_fluid_blocks; ++jb) {
                        o->limits[jb].d.first++;
                        o->limits[jb].d.second++;
                    }
                    o->fluid_points++;
                    o->total_points++;
                    o->end_index++;
                    o->part_id_next++;
                    nAdd++;
                }
            }
        }
    }
    return nAdd;
}

/* Integration.cpp:109-226 update_data (analytic air source, no particle tracking) */
void update_data(orc_sim *o) {
    const int D = o->D;
    update_buffer_region(o);
    for (int64_t ii = o->start_index; ii < o->end_index; ++ii)
        if (o->pnp1[ii].rho < 0.0001) o->pnp1[ii].rho = o->s.rho_rest;
    std::vector<int64_t> to_del;
    const int64_t nb = o->n_bound_blocks, nblk = o->n_bound_blocks + o->n_fluid_blocks;
    std::vector<int64_t> n_del(o->limits.size(), 0);
    const bool mesh = o->s.asource == FJSPH_MESH_INFL;
    for (int64_t blk = nb; blk < nblk; ++blk) {
        const fjsph_block &B = o->limits[blk].d;
        const bool plane = B.delconst != kDefaultVal;
        if (!plane && !mesh) continue;
        for (int64_t ii = B.first; ii < B.second; ++ii)
            /* plane deletion, and particles that left the mesh through its outer boundary */
            if ((plane && dot(o->pnp1[ii].xi, B.delete_norm, D) > B.delconst) ||
                (mesh && o->pnp1[ii].cellID == kMeshLost)) {
                to_del.push_back(ii);
                n_del[blk]++;
            }
    }
    if (!to_del.empty()) {
        std::sort(to_del.begin(), to_del.end());
        to_del.erase(std::unique(to_del.begin(), to_del.end()), to_del.end());
        for (auto it = to_del.rbegin(); it != to_del.rend(); ++it) {
            o->pnp1.erase(o->pnp1.begin() + *it);
            o->total_points--;
            o->fluid_points--;
            o->delete_count++;
        }
        int64_t delshift = 0;
        for (int64_t blk = nb; blk < nblk; ++blk) {
            Block &BB = o->limits[blk];
            BB.d.first -= delshift;
            delshift += n_del[blk];
            BB.d.second -= delshift;
            for (auto &bk : BB.back) bk -= delshift;
            for (auto &bf : BB.buffer)
                for (auto &p : bf) p -= delshift;
        }
    }
    o->pn = o->pnp1;
}

double integrate(orc_sim *o) {
    fjsph_settings &I = o->s;
    double step_error = integrate_no_update(o);
    update_data(o);
    if (o->pnp1.empty()) return 0;
    I.current_time += I.delta_t;
    if (step_error > I.min_residual || o->maxRho_pc > I.rho_max_iter) {
        if (step_error > 0.6 * I.min_residual) {
            I.cfl = std::max(I.cfl_min, I.cfl - I.cfl_step);
            I.n_unstable = 0;
        } else if (I.n_unstable > I.n_unstable_limit) {
            I.cfl = std::max(I.cfl_min, I.cfl - I.cfl_step);
            I.n_unstable = 0;
        } else
            I.n_unstable++;
    } else
        I.n_unstable = 0;
    if (o->iteration < I.subits_factor * I.max_subits && I.n_unstable == 0) {
        if (I.n_stable > I.n_stable_limit) {
            I.cfl = std::min(I.cfl_max, I.cfl + I.cfl_step);
            I.n_stable = 0;
        } else
            I.n_stable++;
    } else
        I.n_stable = 0;
    return step_error;
}

/* ------------------------------------------------------------------------------------------ */
/* state conversion                                                                              */
/* ------------------------------------------------------------------------------------------ */
void view_to_parts(const fjsph_state_view *v, int D, std::vector<Part> &P) {
    P.assign(v->n, Part{});
    for (int64_t i = 0; i < v->n; ++i) {
        Part &q = P[i];
        for (int k = 0; k < D; ++k) {
            q.xi[k] = v->xi[i * D + k];
            q.v[k] = v->v[i * D + k];
            q.acc[k] = v->acc[i * D + k];
            q.Af[k] = v->Af[i * D + k];
            q.aVisc[k] = v->aVisc[i * D + k];
            q.cellV[k] = v->cellV[i * D + k];
            q.gradRho[k] = v->gradRho[i * D + k];
            q.norm[k] = v->norm[i * D + k];
            q.vPert[k] = v->vPert[i * D + k];
        }
        for (int k = 0; k < D * D; ++k) q.L[k] = v->L[i * D * D + k];
        q.Rrho = v->Rrho[i];
        q.rho = v->rho[i];
        q.p = v->p[i];
        q.m = v->m[i];
        q.curve = v->curve[i];
        q.norm_curve = v->norm_curve[i];
        q.woccl = v->woccl[i];
        q.pDist = v->pDist[i];
        q.deltaD = v->deltaD[i];
        q.cellP = v->cellP[i];
        q.cellRho = v->cellRho[i];
        q.colourG = v->colourG[i];
        q.colour = v->colour[i];
        q.lam = v->lam[i];
        q.lam_nb = v->lam_nb[i];
        q.kernsum = v->kernsum[i];
        q.part_id = v->part_id[i];
        q.cellID = v->cellID[i];
        q.b = v->b[i];
        q.surf = v->surf[i];
        q.surfzone = v->surfzone[i];
    }
}

void parts_to_view(const std::vector<Part> &P, int D, fjsph_state_view *v) {
    for (int64_t i = 0; i < (int64_t)P.size() && i < v->n; ++i) {
        const Part &q = P[i];
        for (int k = 0; k < D; ++k) {
            v->xi[i * D + k] = q.xi[k];
            v->v[i * D + k] = q.v[k];
            v->acc[i * D + k] = q.acc[k];
            v->Af[i * D + k] = q.Af[k];
            v->aVisc[i * D + k] = q.aVisc[k];
            v->cellV[i * D + k] = q.cellV[k];
            v->gradRho[i * D + k] = q.gradRho[k];
            v->norm[i * D + k] = q.norm[k];
            v->vPert[i * D + k] = q.vPert[k];
        }
        for (int k = 0; k < D * D; ++k) v->L[i * D * D + k] = q.L[k];
        v->Rrho[i] = q.Rrho;
        v->rho[i] = q.rho;
        v->p[i] = q.p;
        v->m[i] = q.m;
        v->curve[i] = q.curve;
        v->norm_curve[i] = q.norm_curve;
        v->woccl[i] = q.woccl;
        v->pDist[i] = q.pDist;
        v->deltaD[i] = q.deltaD;
        v->cellP[i] = q.cellP;
        v->cellRho[i] = q.cellRho;
        v->colourG[i] = q.colourG;
        v->colour[i] = q.colour;
        v->lam[i] = q.lam;
        v->lam_nb[i] = q.lam_nb;
        v->kernsum[i] = q.kernsum;
        v->part_id[i] = q.part_id;
        v->cellID[i] = q.cellID;
        v->b[i] = q.b;
        v->surf[i] = q.surf;
        v->surfzone[i] = q.surfzone;
    }
}

void sync_counts(orc_sim *o) {
    o->total_points = (int64_t)o->pnp1.size();
    o->bound_points = 0;
    for (int64_t b = 0; b < o->n_bound_blocks; ++b) o->bound_points = std::max(o->bound_points, o->limits[b].d.second);
    o->fluid_points = o->total_points - o->bound_points;
    o->start_index = o->bound_points;
    o->end_index = o->total_points;
}

} // namespace

/* ============================================================================================ */
/* C entry points                                                                                */
/* ============================================================================================ */
extern "C" {

orc_sim *orc_create(const fjsph_settings *s) {
    orc_sim *o = new orc_sim();
    o->s = *s;
    o->D = s->dim;
    return o;
}
void orc_destroy(orc_sim *o) { delete o; }
void orc_set_settings(orc_sim *o, const fjsph_settings *s) {
    o->s = *s;
    o->D = s->dim;
}
void orc_get_settings(orc_sim *o, fjsph_settings *s) { *s = o->s; }
void orc_set_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_set_limits(orc_sim *o, const fjsph_block *blocks, int32_t nblocks, int64_t n_bound_blocks) {
    o->limits.clear();
    for (int32_t b = 0; b < nblocks; ++b) {
        Block B;
        B.d = blocks[b];
        o->limits.push_back(B);
    }
    o->n_bound_blocks = n_bound_blocks;
    o->n_fluid_blocks = nblocks - n_bound_blocks;
    return 0;
}

int orc_get_limits(orc_sim *o, fjsph_block *blocks, int32_t max_blocks, int32_t *nblocks) {
    if (nblocks) *nblocks = (int32_t)o->limits.size();
    if (!blocks) return 0;
    if (max_blocks < (int32_t)o->limits.size()) return -1;
    for (size_t b = 0; b < o->limits.size(); ++b) blocks[b] = o->limits[b].d;
    return 0;
}

int orc_update_counts(orc_sim *o, int64_t *deleted) {
    if (deleted) *deleted = o->delete_count;
    return 0;
}

int orc_set_inlet(orc_sim *o, const fjsph_inlet *in) {
    if (in->block < 0 || in->block >= (int32_t)o->limits.size()) return -1;
    Block &B = o->limits[in->block];
    B.back.assign(in->back, in->back + in->n_back);
    B.buffer.assign(in->n_back, std::vector<int64_t>(in->depth));
    for (int64_t i = 0; i < in->n_back; ++i)
        for (int64_t j = 0; j < in->depth; ++j) B.buffer[i][j] = in->buffer[i * in->depth + j];
    return 0;
}

int orc_get_inlet(orc_sim *o, fjsph_inlet *in) {
    if (in->block < 0 || in->block >= (int32_t)o->limits.size()) return -1;
    Block &B = o->limits[in->block];
    in->n_back = (int64_t)B.back.size();
    in->depth = B.buffer.empty() ? 0 : (int64_t)B.buffer[0].size();
    if (in->back)
        for (int64_t i = 0; i < in->n_back; ++i) in->back[i] = B.back[i];
    if (in->buffer)
        for (int64_t i = 0; i < in->n_back; ++i)
            for (int64_t j = 0; j < in->depth; ++j) in->buffer[i * in->depth + j] = B.buffer[i][j];
    return 0;
}

int orc_set_state(orc_sim *o, int32_t which, const fjsph_state_view *st) {
    view_to_parts(st, o->D, which == FJSPH_PN ? o->pn : o->pnp1);
    if (which == FJSPH_PNP1) {
        sync_counts(o);
        o->part_id_next = 0;
        for (const Part &q : o->pnp1) o->part_id_next = std::max<int64_t>(o->part_id_next, q.part_id + 1);
    }
    return 0;
}

int orc_get_state(orc_sim *o, int32_t which, fjsph_state_view *st) {
    parts_to_view(which == FJSPH_PN ? o->pn : o->pnp1, o->D, st);
    return 0;
}

int64_t orc_particle_count(orc_sim *o) { return (int64_t)o->pnp1.size(); }

int64_t orc_update_neighbours(orc_sim *o) {
    sync_counts(o);
    find_neighbours(o, o->pnp1, o->outlist);
    int64_t n = 0;
    for (auto &l : o->outlist) n += (int64_t)l.size();
    return n;
}

void orc_neighbours_export(orc_sim *o, int64_t *off, int64_t *idx, double *d2) {
    int64_t c = 0;
    for (size_t i = 0; i < o->outlist.size(); ++i) {
        if (off) off[i] = c;
        for (const Nb &n : o->outlist[i]) {
            if (idx) idx[c] = n.j;
            if (d2) d2[c] = n.rr;
            ++c;
        }
    }
    if (off) off[o->outlist.size()] = c;
}

double orc_dsph_prestep(orc_sim *o) {
    sync_counts(o);
    return dsph_prestep(o, o->total_points, o->pnp1);
}
void orc_get_aero_velocity(orc_sim *o) { get_aero_velocity(o, o->pnp1); }
void orc_detect_surface(orc_sim *o) { detect_surface(o, o->pnp1); }
void orc_dissipation_terms(orc_sim *o) { dissipation_terms(o, o->pnp1); }
void orc_particle_shift(orc_sim *o) { particle_shift(o, o->pnp1); }
void orc_check_pipe_outlet(orc_sim *o) { check_pipe_outlet(o, o->pnp1); }

void orc_get_boundary_pressure(orc_sim *o) {
    for (int64_t b = 0; b < o->n_bound_blocks; ++b)
        get_boundary_pressure(o, o->limits[b].d.first, o->limits[b].d.second, o->pnp1);
}
void orc_boundary_ghost(orc_sim *o, int32_t *near_inlet) {
    std::vector<int32_t> ni(o->pnp1.size(), 0);
    for (int64_t b = 0; b < o->n_bound_blocks; ++b)
        boundary_ghost(o, o->limits[b].d.first, o->limits[b].d.second, o->pnp1, ni);
    if (near_inlet)
        for (int64_t i = 0; i < o->bound_points; ++i) near_inlet[i] = ni[i];
}
void orc_boundary_dbc(orc_sim *o) {
    for (int64_t b = 0; b < o->n_bound_blocks; ++b)
        boundary_dbc(o, o->limits[b].d.first, o->limits[b].d.second, o->pnp1);
}
void orc_set_no_slip(orc_sim *o) {
    for (int64_t b = 0; b < o->n_bound_blocks; ++b)
        set_no_slip(o, o->limits[b].d.first, o->limits[b].d.second, o->pnp1);
}
void orc_get_acc_and_rrho(orc_sim *o, double npd) { get_acc_and_rrho(o, npd, o->pnp1); }

double orc_find_timestep(orc_sim *o) {
    sync_counts(o);
    return find_timestep(o);
}

double orc_get_first_rk(orc_sim *o, double npd) {
    sync_counts(o);
    const double dt = 0.5 * o->s.delta_t;
    o->pnp1 = rk_intermediate(o, npd, o->pn, o->pn, dt);
    return check_rk_error(o, 0.0, o->pn, o->pnp1);
}

double orc_runge_kutta4(orc_sim *o, double npd, double logbase) {
    sync_counts(o);
    std::vector<Part> st1 = o->pnp1;
    const double dti = 0.5 * o->s.delta_t, dtf = o->s.delta_t;
    std::vector<Part> st2 = rk_intermediate(o, npd, o->pn, st1, dti);
    std::vector<Part> st3 = rk_intermediate(o, npd, o->pn, st2, dtf);
    o->pnp1 = rk_final(o, npd, dtf, o->pn, st1, st2, st3);
    return check_rk_error(o, logbase, st3, o->pnp1);
}

void orc_nb_iter(orc_sim *o, double npd) {
    sync_counts(o);
    nb_iter(o, npd, o->pn, o->pnp1);
}

double orc_newmark_beta(orc_sim *o, double npd, double *logbase, int32_t *iteration) {
    sync_counts(o);
    o->iteration = (uint32_t)*iteration;
    double lb = *logbase;
    double r = newmark_beta_loop(o, npd, lb);
    *logbase = lb;
    *iteration = (int32_t)o->iteration;
    return r;
}

double orc_integrate_no_update(orc_sim *o) {
    sync_counts(o);
    return integrate_no_update(o);
}

double orc_integrate(orc_sim *o) {
    sync_counts(o);
    return integrate(o);
}

void orc_step_report(orc_sim *o, double *out5) {
    out5[0] = o->maxRho_pc;
    out5[1] = o->maxf;
    out5[2] = o->maxAf;
    out5[3] = o->maxShift;
    out5[4] = (double)o->iteration;
}

double orc_kernel(double r, double H, double W_correc, int32_t cubic) { return Kernel(r, H, W_correc, cubic != 0); }
void orc_gradk(const double *Rij, double r, double H, double W_correc, int32_t cubic, int32_t dim, double *out) {
    GradK(Rij, r, H, W_correc, cubic != 0, dim, out);
}
double orc_min_eig(const double *A, int32_t dim) { return min_eig(A, dim); }
int32_t orc_qr_inverse(const double *A, int32_t dim, double *inv) { return qr_inverse(A, dim, inv); }
double orc_get_cd(double Re) { return GetCd(Re); }

/* the MESH the reference's readers build (Var.h:396-451), with each cell's bounding sphere */
int orc_mesh_set(orc_sim *o, const fjsph_mesh *m) {
    const int D = o->D;
    if (!m || m->dim != D || m->n_cells <= 0) return FJSPH_E_ARG;
    const int64_t nc = m->n_cells, nf = m->n_faces;
    o->m_ncells = nc;
    o->m_verts.assign(m->verts, m->verts + D * m->n_verts);
    o->m_face_off.assign(m->face_offsets, m->face_offsets + nf + 1);
    o->m_face_verts.assign(m->face_verts, m->face_verts + m->face_offsets[nf]);
    o->m_face_right.assign(m->face_right, m->face_right + nf);
    o->m_cell_off.assign(m->cell_face_offsets, m->cell_face_offsets + nc + 1);
    o->m_cell_faces.assign(m->cell_faces, m->cell_faces + m->cell_face_offsets[nc]);
    o->m_centre.assign(m->cell_centres, m->cell_centres + D * nc);
    o->m_vel.assign(m->cell_vel, m->cell_vel + D * nc);
    o->m_p.assign(m->cell_p, m->cell_p + nc);
    o->m_rho.assign(m->cell_rho, m->cell_rho + nc);
    o->m_rad2.assign(nc, 0.0);
    for (int64_t c = 0; c < nc; ++c) {
        double r2 = 0.0;
        for (int64_t e = o->m_cell_off[c]; e < o->m_cell_off[c + 1]; ++e) {
            const int64_t f = o->m_cell_faces[e];
            for (int64_t q = o->m_face_off[f]; q < o->m_face_off[f + 1]; ++q) {
                double d2 = 0.0;
                for (int k = 0; k < D; ++k) {
                    const double dd = o->m_verts[o->m_face_verts[q] * D + k] - o->m_centre[c * D + k];
                    d2 += dd * dd;
                }
                r2 = std::max(r2, d2);
            }
        }
        r2 *= 1.0 + 1e-9;
        o->m_rad2[c] = r2 < 1e60 ? r2 : -1.0; /* a vertex at a fill value: the cell contains nothing */
    }
    return FJSPH_OK;
}

/* VLM::Init + MakeMatrix + GetGamma (VLM.cpp:14-117, 180-307) */
int orc_air_power_law(orc_sim *o, const double *params4) {
    if (!o || !params4 || o->s.asource != FJSPH_POWER_LAW) return FJSPH_E_ARG;
    for (int k = 0; k < 4; ++k) o->pl[k] = params4[k];
    o->pl_ready = true;
    return FJSPH_OK;
}

int orc_vlm_setup(orc_sim *o, const fjsph_vlm *v) {
    if (!v || o->D != 3) return -1;
    if (v->span <= 0 || v->chord <= 0 || v->panels_span <= 0 || v->panels_chord <= 0) return -1;
    const double rad = kPi / 180.0;
    const double sweep = v->sweep_deg * rad, beta = v->flap_deg * rad;
    const int NS = v->panels_span, NC = v->panels_chord;
    const double dr0 = v->chord / double(NC), dy0 = v->span / double(NS);
    std::vector<double> A, B, C;
    auto add = [&](double ax, double ay, double az, double bx, double by, double bz, double cx, double cy, double cz) {
        A.insert(A.end(), {ax, ay, az});
        B.insert(B.end(), {bx, by, bz});
        C.insert(C.end(), {cx, cy, cz});
    };
    for (int i = -NS; i < NS; ++i) {
        const double y1 = double(i) * dy0, y2 = double(i + 1) * dy0, yh = (double(i) + 0.5) * dy0;
        const double t = std::tan(sweep);
        const double fac1 = (1 - std::fabs(y1) / v->span) + v->taper * (std::fabs(y1) / v->span);
        const double fac2 = (1 - std::fabs(y2) / v->span) + v->taper * (std::fabs(y2) / v->span);
        const double fac3 = (1 - std::fabs(yh) / v->span) + v->taper * (std::fabs(yh) / v->span);
        const bool flap = (-i > v->flap_start && -i <= v->flap_width + v->flap_start) ||
                          (i >= v->flap_start && i < v->flap_width + v->flap_start);
        const int jend = flap ? NC - v->flap_depth : NC;
        for (int j = 0; j < jend; ++j)
            add(t * std::fabs(y1) + dr0 * fac1 * (0.25 + j), y1, 0.0, t * std::fabs(y2) + dr0 * fac2 * (0.25 + j), y2, 0.0,
                t * std::fabs(yh) + dr0 * fac3 * (0.75 + j), yh, 0.0);
        if (flap) {
            const double f0 = double(NC - v->flap_depth);
            for (int j = 0; j < v->flap_depth; ++j) {
                auto px = [&](double fac, double y, double w) {
                    return t * std::fabs(y) + f0 * dr0 * fac + std::cos(beta) * dr0 * fac * w;
                };
                auto pz = [&](double fac, double w) { return -std::sin(beta) * dr0 * fac * w; };
                add(px(fac1, y1, 0.25 + j), y1, pz(fac1, 0.25 + j), px(fac2, y2, 0.25 + j), y2, pz(fac2, 0.25 + j),
                    px(fac3, yh, 0.75 + j), yh, pz(fac3, 0.75 + j));
            }
        }
    }
    const int n = int(C.size() / 3);
    const double *vinf = o->s.v_inf;
    std::vector<double> nrm(3 * n);
    for (int p = 0; p < n; ++p) {
        double ca[3], cb[3], c[3];
        for (int k = 0; k < 3; ++k) {
            ca[k] = C[3 * p + k] - A[3 * p + k];
            cb[k] = C[3 * p + k] - B[3 * p + k];
        }
        cross3(ca, cb, c);
        normalized(c, 3, &nrm[3 * p]);
    }
    /* aInf(j, i) = influence of vortex i at control point j, on panel i's normal; RHS(j) = -v . n_j */
    std::vector<std::vector<double>> M(n, std::vector<double>(n + 1));
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double f[3];
            vlm_influence(&A[3 * i], &B[3 * i], &C[3 * j], vinf, false, f);
            M[j][i] = dot(f, &nrm[3 * i], 3);
        }
    for (int j = 0; j < n; ++j) M[j][n] = -dot(vinf, &nrm[3 * j], 3);
    /* Gauss-Jordan elimination with partial pivoting on the augmented matrix */
    for (int k = 0; k < n; ++k) {
        int best = k;
        for (int r = k + 1; r < n; ++r)
            if (std::fabs(M[r][k]) > std::fabs(M[best][k])) best = r;
        if (M[best][k] == 0.0) return -2;
        std::swap(M[k], M[best]);
        for (int r = 0; r < n; ++r) {
            if (r == k || M[r][k] == 0.0) continue;
            const double l = M[r][k] / M[k][k];
            for (int c2 = k; c2 <= n; ++c2) M[r][c2] -= l * M[k][c2];
        }
    }
    o->vlm_gamma.resize(n);
    for (int k = 0; k < n; ++k) o->vlm_gamma[k] = M[k][n] / M[k][k];
    o->vlm_A = A;
    o->vlm_B = B;
    o->vlm_C = C;
    for (int k = 0; k < 3; ++k) o->vlm_vinf[k] = vinf[k];
    o->vlm_maxvel = (v->max_vel == 2.0) ? v->max_vel_fac * norm(vinf, 3) : v->max_vel;
    o->vlm_ready = true;
    return n;
}

int orc_vlm_panels(orc_sim *o, double *gamma, double *abc) {
    const int n = int(o->vlm_gamma.size());
    for (int p = 0; p < n; ++p) {
        if (gamma) gamma[p] = o->vlm_gamma[p];
        if (abc)
            for (int k = 0; k < 3; ++k) {
                abc[9 * p + k] = o->vlm_A[3 * p + k];
                abc[9 * p + 3 + k] = o->vlm_B[3 * p + k];
                abc[9 * p + 6 + k] = o->vlm_C[3 * p + k];
            }
    }
    return n;
}

void orc_vlm_velocity(orc_sim *o, int64_t n, const double *pos, double *vel) {
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) vlm_velocity(o, &pos[3 * i], &vel[3 * i]);
}

} /* extern "C" */
