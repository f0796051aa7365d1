/*
 * vlm.cu -- the vortex-lattice air source (src/VLM.h, src/VLM.cpp).
 *
 * Host: the wing's horseshoe vortices (VLM::MakeMatrix, src/VLM.cpp:180-307), the influence
 * matrix and the circulations (VLM::GetGamma, src/VLM.cpp:84-117).  The matrix keeps the
 * reference's formulation: row j, column i is the velocity induced at control point j by vortex
 * i, projected on the normal of panel i (the vortex's own panel; identical for a flat wing, not
 * for a deflected flap), and the right-hand side of row i is -v_inf . n_i.  It is solved by LU
 * with partial pivoting (the reference uses full pivoting; the solutions agree to round-off).
 *
 * Device: VLM::getVelocity (src/VLM.cpp:119-140) for every particle that needs the air velocity,
 * panels staged through shared memory a block-load at a time; every thread sums the induced
 * velocity of all panels for its particle.  The FP64 kernel is the parity form; the
 * split-precision form works in FP32 on separations formed from high and low parts of the point
 * and the vortex ends, sums in FP32 (the induced part is a correction to v_inf) and adds v_inf in
 * FP64.
 */
#include <cmath>
#include <vector>

#include "kernels.h"
#include "split.cuh"

namespace fjsph {

/* ---- host: geometry and circulations ----------------------------------------------------------- */
namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dotp(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 crossp(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double normp(V3 a) { return std::sqrt(dotp(a, a)); }
inline V3 unit(V3 a) {
    const double n2 = dotp(a, a);
    return n2 > 0.0 ? (1.0 / std::sqrt(n2)) * a : a;
}

/* velocity induced by a unit-strength horseshoe (bound segment A-B, legs from A and B along
 * v_inf) at P, without the conditioning of the particle evaluation (the matrix assembly) */
V3 horseshoe(V3 A, V3 B, V3 P, V3 vinf) {
    const double ipi4 = 1.0 / (4.0 * M_PI);
    V3 r0 = B - A, r1 = P - A, r2 = P - B;
    V3 c = crossp(r1, r2);
    const V3 ab = (ipi4 * dotp(r0, unit(r1) - unit(r2)) / dotp(c, c)) * c;
    V3 inf = A + vinf;
    r2 = P - A;
    r1 = P - inf;
    r0 = A - inf;
    c = crossp(r1, r2);
    const V3 la = (ipi4 * normp(r0) * (1.0 - dotp(r0, r2) / (normp(r0) * normp(r2))) / dotp(c, c)) * c;
    inf = B + vinf;
    r1 = P - B;
    r2 = P - inf;
    r0 = inf - B;
    c = crossp(r1, r2);
    const V3 lb = (ipi4 * normp(r0) * (dotp(r0, r1) / (normp(r1) * normp(r0)) + 1.0) / dotp(c, c)) * c;
    return ab + lb + la;
}

} // namespace

int vlm_build(const fjsph_vlm &v, const double *vinf3, std::vector<double> &abc, std::vector<double> &gamma) {
    if (v.span <= 0.0 || v.chord <= 0.0 || v.panels_span <= 0 || v.panels_chord <= 0) return FJSPH_E_ARG;
    if (v.flap_depth < 0 || v.flap_depth > v.panels_chord || v.flap_start < 0 || v.flap_width < 0) return FJSPH_E_ARG;
    if (v.max_vel_fac < 1.0) return FJSPH_E_ARG;
    const double d2r = M_PI / 180.0;
    const double sweep = v.sweep_deg * d2r, beta = v.flap_deg * d2r;
    const int ns = v.panels_span, nc = v.panels_chord;
    const double dr0 = v.chord / nc, dy0 = v.span / ns, dx0 = dr0, dz0 = 0.0;
    const double x0 = 0.0, y0 = 0.0, z0 = 0.0, yend = v.span;
    struct Panel {
        V3 A, B, C;
    };
    std::vector<Panel> pan;
    pan.reserve((size_t)2 * ns * nc);
    auto chord_fac = [&](double y) { /* taper: 1 at the root, taper at the tip */
        const double fr = (std::fabs(y) - y0) / (yend - y0);
        return (1.0 - fr) + v.taper * fr;
    };
    for (int i = -ns; i < ns; ++i) { /* spanwise strips */
        const double y1 = i * dy0, y2 = (i + 1) * dy0, yh = (i + 0.5) * dy0;
        const double xs1 = std::tan(sweep) * (std::fabs(y1) - y0), xs2 = std::tan(sweep) * (std::fabs(y2) - y0);
        const double xsh = std::tan(sweep) * (std::fabs(yh) - y0);
        const double f1 = chord_fac(y1), f2 = chord_fac(y2), fh = chord_fac(yh);
        const double dx1 = dx0 * f1, dz1 = dz0 * f1, dx2 = dx0 * f2, dz2 = dz0 * f2, dxh = dx0 * fh, dzh = dz0 * fh;
        const bool flap = (-i > v.flap_start && -i <= v.flap_width + v.flap_start) ||
                          (i >= v.flap_start && i < v.flap_width + v.flap_start);
        const int jend = flap ? nc - v.flap_depth : nc;
        for (int j = 0; j < jend; ++j) {
            const V3 A{x0 + xs1 + dx1 * (0.25 + j), y1, z0 + dz1 * (0.25 + j)};
            const V3 B{x0 + xs2 + dx2 * (0.25 + j), y2, z0 + dz2 * (0.25 + j)};
            const V3 C{x0 + xsh + dxh * (0.75 + j), yh, z0 + dzh * (0.75 + j)};
            pan.push_back({A, B, C});
        }
        if (flap) { /* deflected trailing-edge panels */
            const double fac = (double)(nc - v.flap_depth);
            const double dzf1 = -std::sin(beta) * dr0 * f1, dxf1 = std::cos(beta) * dr0 * f1;
            const double dzf2 = -std::sin(beta) * dr0 * f2, dxf2 = std::cos(beta) * dr0 * f2;
            const double dzfh = -std::sin(beta) * dr0 * fh, dxfh = std::cos(beta) * dr0 * fh;
            const double zf1 = z0 + fac * dz1, xf1 = x0 + xs1 + fac * dx1;
            const double zf2 = z0 + fac * dz2, xf2 = x0 + xs2 + fac * dx2;
            const double zfh = z0 + fac * dzh, xfh = x0 + xsh + fac * dxh;
            for (int j = 0; j < v.flap_depth; ++j) {
                const V3 A{xf1 + dxf1 * (0.25 + j), y1, zf1 + dzf1 * (0.25 + j)};
                const V3 B{xf2 + dxf2 * (0.25 + j), y2, zf2 + dzf2 * (0.25 + j)};
                const V3 C{xfh + dxfh * (0.75 + j), yh, zfh + dzfh * (0.75 + j)};
                pan.push_back({A, B, C});
            }
        }
    }
    const int np = (int)pan.size();
    const V3 vinf{vinf3[0], vinf3[1], vinf3[2]};
    std::vector<V3> nrm(np);
    for (int i = 0; i < np; ++i) nrm[i] = unit(crossp(pan[i].C - pan[i].A, pan[i].C - pan[i].B));
    /* M[j][i] = horseshoe_i(C_j) . n_i, rhs[j] = -v_inf . n_j */
    std::vector<double> M((size_t)np * np), rhs(np);
    for (int i = 0; i < np; ++i)
        for (int j = 0; j < np; ++j) M[(size_t)j * np + i] = dotp(horseshoe(pan[i].A, pan[i].B, pan[j].C, vinf), nrm[i]);
    for (int j = 0; j < np; ++j) rhs[j] = -dotp(vinf, nrm[j]);
    /* LU with partial pivoting, in place; singular (a zero pivot column) is an error */
    for (int k = 0; k < np; ++k) {
        int p = k;
        double best = std::fabs(M[(size_t)k * np + k]);
        for (int r = k + 1; r < np; ++r)
            if (std::fabs(M[(size_t)r * np + k]) > best) {
                best = std::fabs(M[(size_t)r * np + k]);
                p = r;
            }
        if (!(best > 0.0)) return FJSPH_E_NONFINITE;
        if (p != k) {
            for (int c = 0; c < np; ++c) std::swap(M[(size_t)k * np + c], M[(size_t)p * np + c]);
            std::swap(rhs[k], rhs[p]);
        }
        const double inv = 1.0 / M[(size_t)k * np + k];
        for (int r = k + 1; r < np; ++r) {
            double *row = &M[(size_t)r * np];
            const double l = row[k] * inv;
            if (l == 0.0) continue;
            row[k] = l;
            const double *prow = &M[(size_t)k * np];
            for (int c = k + 1; c < np; ++c) row[c] -= l * prow[c];
            rhs[r] -= l * rhs[k];
        }
    }
    gamma.assign(np, 0.0);
    for (int k = np - 1; k >= 0; --k) {
        double s = rhs[k];
        for (int c = k + 1; c < np; ++c) s -= M[(size_t)k * np + c] * gamma[c];
        gamma[k] = s / M[(size_t)k * np + k];
        if (!std::isfinite(gamma[k])) return FJSPH_E_NONFINITE;
    }
    abc.resize((size_t)9 * np);
    for (int i = 0; i < np; ++i) {
        const V3 q[3] = {pan[i].A, pan[i].B, pan[i].C};
        for (int a = 0; a < 3; ++a) {
            abc[9 * i + 3 * a + 0] = q[a].x;
            abc[9 * i + 3 * a + 1] = q[a].y;
            abc[9 * i + 3 * a + 2] = q[a].z;
        }
    }
    return FJSPH_OK;
}

/* ---- device: induced velocity ------------------------------------------------------------------ */
namespace {

constexpr int kVT = 128; /* threads per block = panels per shared-memory load */

template <typename R>
struct R3 {
    R x, y, z;
};
template <typename R>
__device__ __forceinline__ R3<R> sub(R3<R> a, R3<R> b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename R>
__device__ __forceinline__ R3<R> cr(R3<R> a, R3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename R>
__device__ __forceinline__ R dt(R3<R> a, R3<R> b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename R>
__device__ __forceinline__ R3<R> nrmz(R3<R> a) { /* normalized(), zero stays zero */
    const R n2 = dt(a, a);
    if (!(n2 > R(0))) return a;
    const R s = R(1) / sqrt(n2);
    return {a.x * s, a.y * s, a.z * s};
}

/* one segment of the conditioned horseshoe (src/VLM.cpp:371-430): returns false when the point
 * is (numerically) on the segment's line, which drops the whole horseshoe */
template <typename R>
__device__ __forceinline__ bool seg_ok(R3<R> r1, R3<R> r2) {
    const R3<R> c = cr(nrmz(r1), nrmz(r2));
    return sqrt(dt(c, c)) > R(1e-12);
}

template <typename R>
__device__ __forceinline__ void horseshoe_add(R3<R> A, R3<R> B, R3<R> P, R3<R> vinf, R g, R3<R> &acc) {
    const R ipi4 = R(0.25 / M_PI);
    /* bound vortex A -> B */
    R3<R> r0 = sub(B, A), r1 = sub(P, A), r2 = sub(P, B);
    if (!seg_ok(r1, r2)) return;
    R3<R> c = cr(r1, r2);
    const R3<R> u1 = nrmz(r1), u2 = nrmz(r2);
    const R fab = ipi4 * dt(r0, sub(u1, u2)) / dt(c, c);
    R3<R> s{fab * c.x, fab * c.y, fab * c.z};
    /* leg from A towards infinity along v_inf */
    const R3<R> ia{A.x + vinf.x, A.y + vinf.y, A.z + vinf.z};
    r2 = sub(P, A);
    r1 = sub(P, ia);
    r0 = sub(A, ia);
    if (!seg_ok(r1, r2)) return;
    c = cr(r1, r2);
    const R n0 = sqrt(dt(r0, r0));
    const R fa = ipi4 * n0 * (R(1) - dt(r0, r2) / (n0 * sqrt(dt(r2, r2)))) / dt(c, c);
    s.x += fa * c.x;
    s.y += fa * c.y;
    s.z += fa * c.z;
    /* leg from B */
    const R3<R> ib{B.x + vinf.x, B.y + vinf.y, B.z + vinf.z};
    r1 = sub(P, B);
    r2 = sub(P, ib);
    r0 = sub(ib, B);
    if (!seg_ok(r1, r2)) return;
    c = cr(r1, r2);
    const R nb0 = sqrt(dt(r0, r0));
    const R fb = ipi4 * nb0 * (dt(r0, r1) / (sqrt(dt(r1, r1)) * nb0) + R(1)) / dt(c, c);
    s.x += fb * c.x;
    s.y += fb * c.y;
    s.z += fb * c.z;
    acc.x += g * s.x;
    acc.y += g * s.y;
    acc.z += g * s.z;
}

/* The horseshoe of the FP32 form from the separations a = P - A and b = P - B, each formed as
 * (P_hi - A_hi) + (P_lo - A_lo) so that it is accurate to FP32 rounding of itself, not of the
 * coordinates (a point near the lattice sits metres from the origin but millimetres from a
 * vortex).  With the legs' vectors P - (A + v) = a - v and P - (B + v) = b - v, the three cross
 * products are a x b, (a - v) x a = a x v and b x (b - v) = v x b, and the reference's factors
 * reduce to (bound) (B - A) . (a/|a| - b/|b|), (leg A) |v| + v . a/|a|, (leg B) |v| + v . b/|b|,
 * each over the squared cross product and times 1/(4 pi).  A segment drops the horseshoe when
 * |u1 x u2| <= 1e-12 for the unit vectors of its two separations, tested as
 * |r1 x r2|^2 <= 1e-24 |r1|^2 |r2|^2. */
__device__ __forceinline__ void horseshoe_add_f32(R3<float> a, R3<float> b, R3<float> v, float vn, float g,
                                                  R3<float> &acc) {
    const float a2 = dt(a, a), b2 = dt(b, b);
    const R3<float> cab = cr(a, b), cav = cr(a, v), cvb = cr(v, b);
    const float nab = dt(cab, cab), nav = dt(cav, cav), nvb = dt(cvb, cvb);
    const R3<float> av = sub(a, v), bv = sub(b, v);
    if (!(nab > 1e-24f * a2 * b2) || !(nav > 1e-24f * dt(av, av) * a2) || !(nvb > 1e-24f * b2 * dt(bv, bv))) return;
    const float ia = rsqrtf(a2), ib = rsqrtf(b2);
    const R3<float> ab = sub(a, b); /* B - A */
    const float ipi4g = (float)(0.25 / M_PI) * g;
    const float fab = ipi4g * (dt(ab, a) * ia - dt(ab, b) * ib) / nab;
    const float fa = ipi4g * (vn + dt(v, a) * ia) / nav;
    const float fb = ipi4g * (vn + dt(v, b) * ib) / nvb;
    acc.x += fab * cab.x + fa * cav.x + fb * cvb.x;
    acc.y += fab * cab.y + fa * cav.y + fb * cvb.y;
    acc.z += fab * cab.z + fa * cav.z + fb * cvb.z;
}

/* Induced velocity at P summed over all panels (every thread of the block calls: the panels
 * pass through shared memory kVT at a time), then v = v_inf + induced limited to max_vel. */
template <typename R>
__device__ void vlm_velocity(const VlmDev &V, bool need, const double *p, double *out) {
    /* shared-memory panel records: FP64 form A, B, gamma; FP32 form (A_hi, gamma), (A_lo, 0),
     * (B_hi, 0), (B_lo, 0) as float4 (one broadcast 16-byte read each) */
    __shared__ double sd[sizeof(R) == 8 ? kVT : 1][7];
    __shared__ float4 sf[sizeof(R) == 4 ? kVT : 1][4];
    R3<R> acc{R(0), R(0), R(0)};
    const R3<R> vinf{(R)V.vinf[0], (R)V.vinf[1], (R)V.vinf[2]};
    R3<R> P{(R)p[0], (R)p[1], (R)p[2]}, Pl{R(0), R(0), R(0)};
    if constexpr (sizeof(R) == 4) {
        split_f32(p[0], P.x, Pl.x);
        split_f32(p[1], P.y, Pl.y);
        split_f32(p[2], P.z, Pl.z);
    }
    const R vn = sqrt(dt(vinf, vinf));
    for (int base = 0; base < V.np; base += kVT) {
        const int q = base + (int)threadIdx.x;
        __syncthreads();
        if (q < V.np) {
            if constexpr (sizeof(R) == 4) { /* FP32 copies made on the host */
                const float *w = V.abf + 12 * (int64_t)q;
                sf[threadIdx.x][0] = make_float4(w[0], w[1], w[2], V.gammaf[q]);
                sf[threadIdx.x][1] = make_float4(w[3], w[4], w[5], 0.f);
                sf[threadIdx.x][2] = make_float4(w[6], w[7], w[8], 0.f);
                sf[threadIdx.x][3] = make_float4(w[9], w[10], w[11], 0.f);
            } else {
#pragma unroll
                for (int k = 0; k < 6; ++k) sd[threadIdx.x][k] = V.ab[6 * (int64_t)q + k];
                sd[threadIdx.x][6] = V.gamma[q];
            }
        }
        __syncthreads();
        const int m = V.np - base < kVT ? V.np - base : kVT;
        if (need)
            for (int t = 0; t < m; ++t) {
                if constexpr (sizeof(R) == 4) {
                    const float4 ah = sf[t][0], al = sf[t][1], bh = sf[t][2], bl = sf[t][3];
                    const R3<float> rpa{(P.x - ah.x) + (Pl.x - al.x), (P.y - ah.y) + (Pl.y - al.y),
                                        (P.z - ah.z) + (Pl.z - al.z)};
                    const R3<float> rpb{(P.x - bh.x) + (Pl.x - bl.x), (P.y - bh.y) + (Pl.y - bl.y),
                                        (P.z - bh.z) + (Pl.z - bl.z)};
                    horseshoe_add_f32(rpa, rpb, vinf, vn, ah.w, acc);
                } else {
                    const R3<R> A{sd[t][0], sd[t][1], sd[t][2]}, B{sd[t][3], sd[t][4], sd[t][5]};
                    horseshoe_add<R>(A, B, P, vinf, sd[t][6], acc);
                }
            }
    }
    if (!need) return;
    const double v[3] = {V.vinf[0] + (double)acc.x, V.vinf[1] + (double)acc.y, V.vinf[2] + (double)acc.z};
    const double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const double s = n > 0.0 ? fmin(n, V.max_vel) / n : 0.0;
    for (int k = 0; k < 3; ++k) out[k] = v[k] * s;
}

/* air velocity of the fluid particles that use it: FREE particles that the aero velocity pass
 * activates, and with the Gissler closure every FREE particle (the occlusion's V_diff,
 * src/Geometry.cpp:151-164) */
template <typename R>
__global__ void __launch_bounds__(kVT) k_vlm_air(Params P, DevState W, DevNbr N, VlmDev V, double *air) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool live = i < P.n;
    bool need = false;
    double x[3] = {0, 0, 0};
    if (live && W.b[i] == FJSPH_FREE) {
        const bool active =
            P.use_lam ? W.lam_nb[i] < P.lam_cutoff : double(nbr_range(N, i).n) * P.i_n_full < P.lam_cutoff;
        need = active || P.acase == FJSPH_GISSLER;
        for (int k = 0; k < 3; ++k) x[k] = W.x[k][i];
    }
    double out[3] = {0, 0, 0};
    vlm_velocity<R>(V, need, x, out);
    if (live)
        for (int k = 0; k < 3; ++k) air[3 * i + k] = out[k];
}

template <typename R>
__global__ void __launch_bounds__(kVT) k_vlm_points(VlmDev V, int64_t n, const double *pos, double *vel) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool live = i < n;
    double x[3] = {0, 0, 0}, out[3] = {0, 0, 0};
    if (live)
        for (int k = 0; k < 3; ++k) x[k] = pos[3 * i + k];
    vlm_velocity<R>(V, live, x, out);
    if (live)
        for (int k = 0; k < 3; ++k) vel[3 * i + k] = out[k];
}

/* Boundary-layer air field: v_inf (s)^n with s = (x[axis] - wall) / thickness clamped to [0, 1];
 * the same value the oracle computes with pow in FP64 (FP32 powf in the split-precision form). */
template <typename R>
__global__ void k_power_law_air(Params P, DevState W, int axis, double wall, double inv_thick, double expo,
                                double *air) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    double t = (W.x[axis][i] - wall) * inv_thick;
    t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
    const double f = (t == 1.0) ? 1.0 : (double)pow((R)t, (R)expo);
    for (int k = 0; k < 3; ++k) air[3 * i + k] = P.v_inf[k] * f;
}

} // namespace

void launch_power_law_air(const Params &P, const DevState &W, const double *pl, double *air, bool fp32,
                          cudaStream_t s) {
    const unsigned g = grid_for(P.n - P.nb, 256);
    if (g == 0) return;
    const int axis = (int)pl[0];
    if (fp32)
        k_power_law_air<float><<<g, 256, 0, s>>>(P, W, axis, pl[1], 1.0 / pl[2], pl[3], air);
    else
        k_power_law_air<double><<<g, 256, 0, s>>>(P, W, axis, pl[1], 1.0 / pl[2], pl[3], air);
}

void launch_vlm_air(const Params &P, const DevState &W, const DevNbr &N, const VlmDev &V, double *air, bool fp32,
                    cudaStream_t s) {
    const unsigned g = grid_for(P.n - P.nb, kVT);
    if (g == 0) return;
    if (fp32)
        k_vlm_air<float><<<g, kVT, 0, s>>>(P, W, N, V, air);
    else
        k_vlm_air<double><<<g, kVT, 0, s>>>(P, W, N, V, air);
}

void launch_vlm_points(const VlmDev &V, int64_t n, const double *pos, double *vel, bool fp32, cudaStream_t s) {
    if (n <= 0) return;
    if (fp32)
        k_vlm_points<float><<<grid_for(n, kVT), kVT, 0, s>>>(V, n, pos, vel);
    else
        k_vlm_points<double><<<grid_for(n, kVT), kVT, 0, s>>>(V, n, pos, vel);
}

} // namespace fjsph
