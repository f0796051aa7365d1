/*
 * linalg.cuh -- the small dense linear algebra of dSPH_PreStep (src/Shifting.cpp:73-100) for one
 * particle per thread, fully unrolled for D = 2, 3.
 *
 * - qr_inverse: Householder QR with column pivoting (Golub & Van Loan, alg. 5.4.1); the matrix
 *   counts as invertible iff every |R_kk| > D * eps * max|R_kk|, the rank test of a
 *   rank-revealing QR (the reference calls Eigen::ColPivHouseholderQR::isInvertible/inverse).
 * - min_eig: smallest eigenvalue of the symmetric matrix read from the lower triangle (the
 *   reference calls Eigen::SelfAdjointEigenSolver::computeDirect): shift by the mean diagonal,
 *   scale by the largest entry, then the quadratic formula (D = 2) or the trigonometric solution
 *   of the characteristic cubic (D = 3, Smith 1961).
 */
#pragma once

#include "common.cuh"

namespace fjsph {

template <int D>
__device__ __forceinline__ bool qr_inverse(const double *Ain, double *inv) {
    double A[D * D];
    double V[D][D];
    double beta[D];
    int perm[D];
#pragma unroll
    for (int k = 0; k < D * D; ++k) A[k] = Ain[k];
#pragma unroll
    for (int k = 0; k < D; ++k) perm[k] = k;
    double maxpiv = 0.0;
    double rdiag[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        int pc = k;
        double best = -1.0;
#pragma unroll
        for (int c = k; c < D; ++c) {
            double s = 0.0;
#pragma unroll
            for (int r = k; r < D; ++r) s += A[r * D + c] * A[r * D + c];
            if (s > best) {
                best = s;
                pc = c;
            }
        }
        if (pc != k) {
#pragma unroll
            for (int r = 0; r < D; ++r) {
                /* swap columns k and pc without dynamic register indexing */
#pragma unroll
                for (int c = k + 1; c < D; ++c)
                    if (c == pc) {
                        double t = A[r * D + k];
                        A[r * D + k] = A[r * D + c];
                        A[r * D + c] = t;
                    }
            }
#pragma unroll
            for (int c = k + 1; c < D; ++c)
                if (c == pc) {
                    int t = perm[k];
                    perm[k] = perm[c];
                    perm[c] = t;
                }
        }
        double xnorm2 = 0.0;
#pragma unroll
        for (int r = k; r < D; ++r) xnorm2 += A[r * D + k] * A[r * D + k];
        double xnorm = sqrt(xnorm2);
        double x0 = A[k * D + k];
        double alpha = (x0 >= 0.0) ? -xnorm : xnorm;
        double v[D];
#pragma unroll
        for (int r = 0; r < D; ++r) v[r] = 0.0;
        double bt = 0.0;
        if (xnorm > 0.0) {
            v[k] = x0 - alpha;
#pragma unroll
            for (int r = k + 1; r < D; ++r) v[r] = A[r * D + k];
            double vn2 = 0.0;
#pragma unroll
            for (int r = k; r < D; ++r) vn2 += v[r] * v[r];
            bt = (vn2 > 0.0) ? 2.0 / vn2 : 0.0;
#pragma unroll
            for (int c = k; c < D; ++c) {
                double s = 0.0;
#pragma unroll
                for (int r = k; r < D; ++r) s += v[r] * A[r * D + c];
                s *= bt;
#pragma unroll
                for (int r = k; r < D; ++r) A[r * D + c] -= s * v[r];
            }
        }
#pragma unroll
        for (int r = 0; r < D; ++r) V[k][r] = v[r];
        beta[k] = bt;
        rdiag[k] = A[k * D + k];
        maxpiv = fmax(maxpiv, fabs(rdiag[k]));
    }
    const double thr = maxpiv * kEps * double(D);
#pragma unroll
    for (int k = 0; k < D; ++k)
        if (!(fabs(rdiag[k]) > thr)) return false;
    double Y[D * D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
        double e[D];
#pragma unroll
        for (int r = 0; r < D; ++r) e[r] = (r == c) ? 1.0 : 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            double s = 0.0;
#pragma unroll
            for (int r = k; r < D; ++r) s += V[k][r] * e[r];
            s *= beta[k];
#pragma unroll
            for (int r = k; r < D; ++r) e[r] -= s * V[k][r];
        }
        double y[D];
#pragma unroll
        for (int r = D - 1; r >= 0; --r) {
            double s = e[r];
#pragma unroll
            for (int q = r + 1; q < D; ++q) s -= A[r * D + q] * y[q];
            y[r] = s / A[r * D + r];
        }
#pragma unroll
        for (int r = 0; r < D; ++r) Y[r * D + c] = y[r];
    }
    /* A P = Q R  =>  A^-1 = P R^-1 Q^T */
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int t = 0; t < D; ++t)
            if (perm[r] == t)
#pragma unroll
                for (int c = 0; c < D; ++c) inv[t * D + c] = Y[r * D + c];
    return true;
}

template <int D>
__device__ __forceinline__ double min_eig(const double *A);

template <>
__device__ __forceinline__ double min_eig<2>(const double *A) {
    double a00 = A[0], a10 = A[2], a11 = A[3];
    double shift = 0.5 * (a00 + a11);
    double b00 = a00 - shift, b11 = a11 - shift, b10 = a10;
    double scale = fmax(fabs(b00), fmax(fabs(b11), fabs(b10)));
    if (scale > 0.0) {
        b00 /= scale;
        b11 /= scale;
        b10 /= scale;
    } else {
        scale = 0.0;
    }
    double hd = 0.5 * (b00 - b11);
    double t = sqrt(hd * hd + b10 * b10);
    double l = 0.5 * (b00 + b11) - t;
    return l * scale + shift;
}

template <>
__device__ __forceinline__ double min_eig<3>(const double *A) {
    double a00 = A[0], a10 = A[3], a11 = A[4], a20 = A[6], a21 = A[7], a22 = A[8];
    double shift = (a00 + a11 + a22) / 3.0;
    double m00 = a00 - shift, m11 = a11 - shift, m22 = a22 - shift, m10 = a10, m20 = a20, m21 = a21;
    double scale = fmax(fmax(fmax(fabs(m00), fabs(m11)), fmax(fabs(m22), fabs(m10))), fmax(fabs(m20), fabs(m21)));
    if (!(scale > 0.0)) return shift;
    double is = 1.0 / scale;
    m00 *= is;
    m11 *= is;
    m22 *= is;
    m10 *= is;
    m20 *= is;
    m21 *= is;
    double c0 = m00 * m11 * m22 + 2.0 * m10 * m20 * m21 - m00 * m21 * m21 - m11 * m20 * m20 - m22 * m10 * m10;
    double c1 = m00 * m11 - m10 * m10 + m00 * m22 - m20 * m20 + m11 * m22 - m21 * m21;
    double c2 = m00 + m11 + m22;
    double c2o3 = c2 / 3.0;
    double p = (c2 * c2o3 - c1) / 3.0;
    if (p < 0.0) p = 0.0;
    double halfq = 0.5 * (c0 + c2o3 * (2.0 * c2o3 * c2o3 - c1));
    double disc = p * p * p - halfq * halfq;
    if (disc < 0.0) disc = 0.0;
    double rho = sqrt(p);
    double theta = atan2(sqrt(disc), halfq) / 3.0;
    double st, ct;
    sincos(theta, &st, &ct);
    const double sqrt3 = 1.7320508075688772935;
    double r0 = c2o3 + 2.0 * rho * ct;
    double r1 = c2o3 - rho * (ct + sqrt3 * st);
    double r2 = c2o3 - rho * (ct - sqrt3 * st);
    return fmin(r0, fmin(r1, r2)) * scale + shift;
}

} // namespace fjsph
