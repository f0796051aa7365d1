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

template <typename R>
struct RealTraits;
template <>
struct RealTraits<double> {
    static constexpr double eps = 2.220446049250313080847e-16;
};
template <>
struct RealTraits<float> {
    static constexpr float eps = 1.1920928955078125e-07f;
};

template <int D, typename R = double>
__device__ __forceinline__ bool qr_inverse(const R *Ain, R *inv) {
    R A[D * D];
    R V[D][D];
    R beta[D];
    int perm[D];
#pragma unroll
    for (int k = 0; k < D * D; ++k) A[k] = Ain[k];
#pragma unroll
    for (int k = 0; k < D; ++k) perm[k] = k;
    R maxpiv = R(0);
    R rdiag[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        int pc = k;
        R best = R(-1);
#pragma unroll
        for (int c = k; c < D; ++c) {
            R s = R(0);
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
                        R t = A[r * D + k];
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
        R xnorm2 = R(0);
#pragma unroll
        for (int r = k; r < D; ++r) xnorm2 += A[r * D + k] * A[r * D + k];
        R xnorm = sqrt(xnorm2);
        R x0 = A[k * D + k];
        R alpha = (x0 >= R(0)) ? -xnorm : xnorm;
        R v[D];
#pragma unroll
        for (int r = 0; r < D; ++r) v[r] = R(0);
        R bt = R(0);
        if (xnorm > R(0)) {
            v[k] = x0 - alpha;
#pragma unroll
            for (int r = k + 1; r < D; ++r) v[r] = A[r * D + k];
            R vn2 = R(0);
#pragma unroll
            for (int r = k; r < D; ++r) vn2 += v[r] * v[r];
            bt = (vn2 > R(0)) ? R(2) / vn2 : R(0);
#pragma unroll
            for (int c = k; c < D; ++c) {
                R s = R(0);
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
    const R thr = maxpiv * RealTraits<R>::eps * R(D);
#pragma unroll
    for (int k = 0; k < D; ++k)
        if (!(fabs(rdiag[k]) > thr)) return false;
    R Y[D * D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
        R e[D];
#pragma unroll
        for (int r = 0; r < D; ++r) e[r] = (r == c) ? R(1) : R(0);
#pragma unroll
        for (int k = 0; k < D; ++k) {
            R s = R(0);
#pragma unroll
            for (int r = k; r < D; ++r) s += V[k][r] * e[r];
            s *= beta[k];
#pragma unroll
            for (int r = k; r < D; ++r) e[r] -= s * V[k][r];
        }
        R y[D];
#pragma unroll
        for (int r = D - 1; r >= 0; --r) {
            R s = e[r];
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

template <int D, typename R = double>
struct MinEig;

template <typename R>
struct MinEig<2, R> {
    static __device__ __forceinline__ R run(const R *A) {
        R a00 = A[0], a10 = A[2], a11 = A[3];
        R shift = R(0.5) * (a00 + a11);
        R b00 = a00 - shift, b11 = a11 - shift, b10 = a10;
        R scale = fmax(fabs(b00), fmax(fabs(b11), fabs(b10)));
        if (scale > R(0)) {
            b00 /= scale;
            b11 /= scale;
            b10 /= scale;
        } else {
            scale = R(0);
        }
        R hd = R(0.5) * (b00 - b11);
        R t = sqrt(hd * hd + b10 * b10);
        R l = R(0.5) * (b00 + b11) - t;
        return l * scale + shift;
    }
};

template <typename R>
struct MinEig<3, R> {
    static __device__ __forceinline__ R run(const R *A);
};

template <int D, typename R = double>
__device__ __forceinline__ R min_eig(const R *A) {
    return MinEig<D, R>::run(A);
}

template <>
__device__ __forceinline__ double MinEig<3, double>::run(const double *A) {
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

template <>
__device__ __forceinline__ float MinEig<3, float>::run(const float *A) {
    float a00 = A[0], a10 = A[3], a11 = A[4], a20 = A[6], a21 = A[7], a22 = A[8];
    float shift = (a00 + a11 + a22) / 3.0f;
    float m00 = a00 - shift, m11 = a11 - shift, m22 = a22 - shift, m10 = a10, m20 = a20, m21 = a21;
    float scale = fmaxf(fmaxf(fmaxf(fabsf(m00), fabsf(m11)), fmaxf(fabsf(m22), fabsf(m10))), fmaxf(fabsf(m20), fabsf(m21)));
    if (!(scale > 0.0f)) return shift;
    float is = 1.0f / scale;
    m00 *= is;
    m11 *= is;
    m22 *= is;
    m10 *= is;
    m20 *= is;
    m21 *= is;
    float c0 = m00 * m11 * m22 + 2.0f * m10 * m20 * m21 - m00 * m21 * m21 - m11 * m20 * m20 - m22 * m10 * m10;
    float c1 = m00 * m11 - m10 * m10 + m00 * m22 - m20 * m20 + m11 * m22 - m21 * m21;
    float c2 = m00 + m11 + m22;
    float c2o3 = c2 / 3.0f;
    float p = (c2 * c2o3 - c1) / 3.0f;
    if (p < 0.0f) p = 0.0f;
    float halfq = 0.5f * (c0 + c2o3 * (2.0f * c2o3 * c2o3 - c1));
    float disc = p * p * p - halfq * halfq;
    if (disc < 0.0f) disc = 0.0f;
    float rho = sqrtf(p);
    float theta = atan2f(sqrtf(disc), halfq) / 3.0f;
    float st, ct;
    sincosf(theta, &st, &ct);
    const float sqrt3 = 1.7320508075688772935f;
    float r0 = c2o3 + 2.0f * rho * ct;
    float r1 = c2o3 - rho * (ct + sqrt3 * st);
    float r2 = c2o3 - rho * (ct - sqrt3 * st);
    return fminf(r0, fminf(r1, r2)) * scale + shift;
}

} // namespace fjsph
