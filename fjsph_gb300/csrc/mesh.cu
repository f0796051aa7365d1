/*
 * mesh.cu -- the mesh-cell air source: which cell of a CFD mesh each free particle is in, and
 * that cell's velocity, pressure and density (src/Containment.cpp:385-421 CheckCell,
 * :579-821 FindCell, src/Resid.cpp:477-519, src/Geometry.cpp:151-157).
 *
 * Containment is the reference's test: a ray from the particle along +x (2D: Crossings2D per
 * edge; 3D: Crossings3D per face, signed volumes of the face's first three vertices, ray end
 * point + 1e5 x) toggles an inside flag, and the second crossing ends the test (convex cells).
 * The particle's previous cell is tried first.  The reference then walks the 5 and the 500
 * nearest cell centres of a KD tree; here the candidates are the cells whose bounding sphere
 * (centre, largest centre-vertex distance) holds the particle -- every cell that can contain it
 * -- taken from a uniform grid over the spheres' boxes, and the containing candidate with the
 * nearest centre wins (ties: the lower index), which is the cell the nearest-centre walk finds.
 * A particle inside no cell is outside the mesh: the segment to the nearest centre among the
 * cells whose doubled sphere holds it (a second grid) is tested against that cell's boundary
 * faces; an outer-boundary crossing marks the particle for deletion (cellID = kMeshLost, removed
 * with the step's other deletions), an inner-boundary crossing or no crossing leaves it with its
 * previous cell values.
 */
#include <algorithm>
#include <cmath>
#include <vector>

#include "kernels.h"

namespace fjsph {

namespace {

constexpr int kT = 128;

template <int D>
__device__ __forceinline__ double vert(const MeshDev &M, int64_t v, int k) {
    return M.verts[v * D + k];
}

/* Crossings2D (src/Geometry.cpp:354-397): does the +x ray from (tx, ty) cross edge (a, b)? */
__device__ __forceinline__ bool crosses_2d(double ax, double ay, double bx, double by, double tx, double ty) {
    const bool y0 = ay >= ty, y1 = by >= ty;
    if (y0 == y1) return false;
    return ((by - ty) * (bx - ax) >= (bx - tx) * (by - ay)) == y1;
}

/* sign test of the 4x4 determinant |p 1; a 1; b 1; c 1| < 0, i.e. det(a - p, b - p, c - p) > 0 */
__device__ __forceinline__ bool neg_vol(const double *p, const double *a, const double *b, const double *c) {
    const double ax = a[0] - p[0], ay = a[1] - p[1], az = a[2] - p[2];
    const double bx = b[0] - p[0], by = b[1] - p[1], bz = b[2] - p[2];
    const double cx = c[0] - p[0], cy = c[1] - p[1], cz = c[2] - p[2];
    const double det = ax * (by * cz - bz * cy) - ay * (bx * cz - bz * cx) + az * (bx * cy - by * cx);
    return det > 0.0;
}

/* Crossings3D (src/Geometry.cpp:485-574): does segment p -> q cross the face's first triangle? */
__device__ bool crosses_3d(const MeshDev &M, int64_t f, const double *p, const double *q) {
    const int64_t f0 = M.face_off[f], f1 = M.face_off[f + 1];
    double v[3][3], last[3];
    for (int t = 0; t < 3; ++t)
        for (int k = 0; k < 3; ++k) v[t][k] = vert<3>(M, M.face_verts[f0 + t], k);
    for (int k = 0; k < 3; ++k) last[k] = vert<3>(M, M.face_verts[f1 - 1], k);
    if (neg_vol(p, v[0], v[1], v[2]) == neg_vol(q, v[0], v[1], v[2])) return false;
    /* edges (last, v0), (v0, v1), (v1, v2): the sign of every tet must agree */
    const bool s3 = neg_vol(p, last, v[0], q);
    if (neg_vol(p, v[0], v[1], q) != s3) return false;
    if (neg_vol(p, v[1], v[2], q) != s3) return false;
    return true;
}

template <int D>
__device__ bool check_cell(const MeshDev &M, int64_t cell, const double *p) {
    bool inside = false, line = false;
    double ray[3] = {p[0] + 1e5, p[1], D == 3 ? p[2] : 0.0};
    for (int64_t e = M.cell_off[cell]; e < M.cell_off[cell + 1]; ++e) {
        const int64_t f = M.cell_faces[e];
        bool hit;
        if (D == 2) {
            const int64_t a = M.face_verts[M.face_off[f]], b = M.face_verts[M.face_off[f] + 1];
            hit = crosses_2d(vert<2>(M, a, 0), vert<2>(M, a, 1), vert<2>(M, b, 0), vert<2>(M, b, 1), p[0], p[1]);
        } else {
            hit = crosses_3d(M, f, p, ray);
        }
        if (hit) {
            inside = !inside;
            if (line) break; /* convex cells: at most two crossings */
            line = true;
        }
    }
    return inside;
}

/* get_line_intersection (src/Geometry.cpp:312-343): does segment p -> c cross edge (e1, e2)?
 * Only one orientation of the pair counts (a denominator below epsilon returns "no"). */
__device__ bool seg_cross_2d(const MeshDev &M, int64_t f, const double *p, const double *c) {
    const int64_t a = M.face_verts[M.face_off[f]], b = M.face_verts[M.face_off[f] + 1];
    const double e1x = vert<2>(M, a, 0), e1y = vert<2>(M, a, 1), e2x = vert<2>(M, b, 0), e2y = vert<2>(M, b, 1);
    const double sx = c[0] - p[0], sy = c[1] - p[1], rx = e2x - e1x, ry = e2y - e1y;
    const double denom = -rx * sy + sx * ry;
    if (denom < 2.220446049250313e-16) return false;
    const double u = (-sy * (p[0] - e1x) + sx * (p[1] - e1y)) / denom;
    const double t = (rx * (p[1] - e1y) - ry * (p[0] - e1x)) / denom;
    return u > 0 && u < 1 && t > 0 && t < 1;
}

template <int D>
__device__ __forceinline__ void assign(const MeshDev &M, DevState &W, int64_t i, int64_t cell) {
    W.cellID[i] = cell;
#pragma unroll
    for (int k = 0; k < D; ++k) W.cellV[k][i] = M.cvel[cell * D + k];
    W.cellP[i] = M.cp[cell];
    W.cellRho[i] = M.crho[cell];
}

/* bucket of p in grid G, or -1 outside it (the same expression the build uses for the spans) */
template <int D>
__device__ __forceinline__ int64_t bucket_of(const MeshDev::Grid &G, const double *p) {
    int64_t q = 0, stride = 1;
    for (int k = 0; k < D; ++k) {
        const double g = floor((p[k] - G.lo[k]) * G.inv_h);
        if (!(g >= 0.0 && g < (double)G.dims[k])) return -1;
        q += (int64_t)g * stride;
        stride *= G.dims[k];
    }
    return q;
}

template <int D>
__device__ __forceinline__ double centre_d2(const MeshDev &M, int64_t c, const double *p) {
    double d2 = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const double dd = p[k] - M.centre[c * D + k];
        d2 += dd * dd;
    }
    return d2;
}

/* FindCell for one active particle (free, at or below the lambda cutoff, not lost) */
template <int D>
__device__ void find_one(const MeshDev &M, DevState &W, int64_t i) {
    double p[3] = {W.x[0][i], W.x[1][i], D == 3 ? W.x[2][i] : 0.0};
    const int64_t cur = W.cellID[i];
    if (cur >= 0 && cur < M.ncells && check_cell<D>(M, cur, p)) {
        assign<D>(M, W, i, cur);
        return;
    }
    /* the containing cell among those whose bounding sphere holds p, nearest centre first */
    int64_t best = -1;
    double best_d = 0.0;
    const int64_t q = bucket_of<D>(M.g[0], p);
    if (q >= 0)
        for (int64_t e = M.g[0].off[q]; e < M.g[0].off[q + 1]; ++e) {
            const int64_t c = M.g[0].cells[e];
            const double d2 = centre_d2<D>(M, c, p);
            if (d2 > M.rad2[c]) continue;
            if ((best < 0 || d2 < best_d || (d2 == best_d && c < best)) && check_cell<D>(M, c, p)) {
                best = c;
                best_d = d2;
            }
        }
    if (best >= 0) {
        assign<D>(M, W, i, best);
        return;
    }
    /* outside every cell: the nearest centre among the cells whose doubled sphere holds p, and
     * did the particle cross that cell's boundary? */
    int64_t nearest = -1;
    double near_d = 0.0;
    const int64_t q2 = bucket_of<D>(M.g[1], p);
    if (q2 >= 0)
        for (int64_t e = M.g[1].off[q2]; e < M.g[1].off[q2 + 1]; ++e) {
            const int64_t c = M.g[1].cells[e];
            const double d2 = centre_d2<D>(M, c, p);
            if (d2 > 4.0 * M.rad2[c]) continue;
            if (nearest < 0 || d2 < near_d || (d2 == near_d && c < nearest)) {
                nearest = c;
                near_d = d2;
            }
        }
    if (nearest < 0) return;
    double cc[3] = {M.centre[nearest * D], M.centre[nearest * D + 1], D == 3 ? M.centre[nearest * D + 2] : 0.0};
    for (int64_t e = M.cell_off[nearest]; e < M.cell_off[nearest + 1]; ++e) {
        const int64_t f = M.cell_faces[e];
        const int32_t side = M.face_right[f];
        if (side >= 0) continue;
        const bool hit = D == 2 ? seg_cross_2d(M, f, p, cc) : crosses_3d(M, f, p, cc);
        if (!hit) continue;
        if (side == -2) W.cellID[i] = kMeshLost; /* crossed the outer boundary */
        break;
    }
}

template <int D>
__device__ __forceinline__ void put_air(const DevState &W, double *air, int64_t i) {
    if (air) {
#pragma unroll
        for (int k = 0; k < 3; ++k) air[3 * i + k] = k < D ? W.cellV[k][i] : 0.0;
    }
}

/* first pass: inactive particles lose their cell; the active ones are listed (warp-aggregated
 * appends), so the containment tests run on dense warps -- their FP64 work dominates */
template <int D>
__global__ void k_mesh_mark(Params P, DevState W, double *air, int32_t *list, int32_t *count) {
    const int64_t i = P.nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool active = false;
    if (i < P.n) {
        if (W.b[i] != FJSPH_FREE || W.lam_nb[i] > P.lam_cutoff) {
            W.cellID[i] = kNoCell;
            put_air<D>(W, air, i);
        } else if (W.cellID[i] == kMeshLost) {
            put_air<D>(W, air, i);
        } else {
            active = true;
        }
    }
    const unsigned mask = __ballot_sync(0xffffffffu, active);
    if (!mask) return;
    const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (active) list[base + __popc(mask & ((1u << lane) - 1u))] = (int32_t)i;
}

template <int D>
__global__ void k_mesh_find(DevState W, MeshDev M, double *air, const int32_t *list, const int32_t *count) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= *count) return;
    const int64_t i = list[t];
    find_one<D>(M, W, i);
    put_air<D>(W, air, i);
}

} // namespace

int mesh_build(const fjsph_mesh &m, MeshHost &h) {
    const int D = m.dim;
    if ((D != 2 && D != 3) || m.n_cells <= 0 || m.n_faces <= 0 || m.n_verts <= 0) return FJSPH_E_ARG;
    if (!m.verts || !m.face_offsets || !m.face_verts || !m.face_right || !m.cell_face_offsets || !m.cell_faces ||
        !m.cell_centres || !m.cell_vel || !m.cell_p || !m.cell_rho)
        return FJSPH_E_ARG;
    const int64_t nc = m.n_cells, nf = m.n_faces;
    /* check the index arrays before anything reads through them */
    if (m.face_offsets[0] != 0 || m.cell_face_offsets[0] != 0) return FJSPH_E_ARG;
    for (int64_t f = 0; f < nf; ++f) {
        const int64_t a = m.face_offsets[f], b = m.face_offsets[f + 1];
        if (b - a < (D == 2 ? 2 : 3) || (D == 2 && b - a != 2)) return FJSPH_E_ARG;
        if (m.face_right[f] < -2 || m.face_right[f] >= nc) return FJSPH_E_ARG;
    }
    for (int64_t q = 0; q < m.face_offsets[nf]; ++q)
        if (m.face_verts[q] < 0 || m.face_verts[q] >= m.n_verts) return FJSPH_E_ARG;
    for (int64_t c = 0; c < nc; ++c)
        if (m.cell_face_offsets[c + 1] <= m.cell_face_offsets[c]) return FJSPH_E_ARG;
    for (int64_t q = 0; q < m.cell_face_offsets[nc]; ++q)
        if (m.cell_faces[q] < 0 || m.cell_faces[q] >= nf) return FJSPH_E_ARG;
    /* bounding spheres: the largest distance from a cell's centre to one of its vertices */
    h.rad2.assign((size_t)nc, 0.0);
    double rmean = 0.0;
    int64_t nvalid = 0;
    for (int64_t c = 0; c < nc; ++c) {
        double r2 = 0.0;
        for (int64_t e = m.cell_face_offsets[c]; e < m.cell_face_offsets[c + 1]; ++e) {
            const int64_t f = m.cell_faces[e];
            for (int64_t q = m.face_offsets[f]; q < m.face_offsets[f + 1]; ++q) {
                double d2 = 0.0;
                for (int k = 0; k < D; ++k) {
                    const double dd = m.verts[m.face_verts[q] * D + k] - m.cell_centres[c * D + k];
                    d2 += dd * dd;
                }
                r2 = std::max(r2, d2);
            }
        }
        r2 *= 1.0 + 1e-9; /* covers the rounding of the containment test at the sphere's edge */
        /* a cell with a vertex at a fill value (e.g. NetCDF's 9.97e36) contains nothing: no
         * candidate, no grid entry */
        if (!(r2 < 1e60)) {
            h.rad2[(size_t)c] = -1.0;
            continue;
        }
        h.rad2[(size_t)c] = r2;
        rmean += std::sqrt(r2);
        ++nvalid;
    }
    if (nvalid == 0) return FJSPH_E_ARG;
    rmean /= double(nvalid);
    /* grid g (0: spheres, 1: doubled spheres) with edge h, at most 2^22 buckets; a cell is listed
     * in every bucket its box overlaps, with the query's own bucket expression, so a point inside
     * a sphere always finds that cell in its bucket */
    for (int g = 0; g < 2; ++g) {
        const double grow = g == 0 ? 1.0 : 2.0;
        MeshHost::Grid &G = h.g[g];
        double glo[3] = {0, 0, 0}, ghi[3] = {0, 0, 0};
        for (int k = 0; k < D; ++k) {
            glo[k] = 1e300;
            ghi[k] = -1e300;
        }
        for (int64_t c = 0; c < nc; ++c)
            for (int k = 0; k < D; ++k) {
                if (h.rad2[(size_t)c] < 0.0) break;
                const double r = grow * std::sqrt(h.rad2[(size_t)c]);
                glo[k] = std::min(glo[k], m.cell_centres[c * D + k] - r);
                ghi[k] = std::max(ghi[k], m.cell_centres[c * D + k] + r);
            }
        double edge = grow * rmean;
        for (;;) {
            double nbk = 1.0;
            for (int k = 0; k < D; ++k) nbk *= std::floor((ghi[k] - glo[k]) / edge) + 1.0;
            if (nbk <= double(1 << 22)) break;
            edge *= 1.25;
        }
        G.inv_h = 1.0 / edge;
        for (int k = 0; k < 3; ++k) {
            G.lo[k] = k < D ? glo[k] : 0.0;
            G.dims[k] = k < D ? (int32_t)(std::floor((ghi[k] - glo[k]) * G.inv_h) + 1.0) : 1;
        }
        const int64_t nbk = (int64_t)G.dims[0] * G.dims[1] * G.dims[2];
        auto cellq = [&](double x, int k) {
            const double q = std::floor((x - G.lo[k]) * G.inv_h);
            return (int)std::min(std::max(q, 0.0), (double)(G.dims[k] - 1));
        };
        G.off.assign((size_t)nbk + 1, 0);
        for (int pass = 0; pass < 2; ++pass) {
            std::vector<int64_t> fill;
            if (pass == 1) {
                for (int64_t q = 0; q < nbk; ++q) G.off[(size_t)q + 1] += G.off[(size_t)q];
                G.cells.assign((size_t)G.off[(size_t)nbk], 0);
                fill.assign(G.off.begin(), G.off.end() - 1);
            }
            for (int64_t c = 0; c < nc; ++c) {
                if (h.rad2[(size_t)c] < 0.0) continue;
                int a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
                const double r = grow * std::sqrt(h.rad2[(size_t)c]);
                for (int k = 0; k < D; ++k) {
                    a[k] = cellq(m.cell_centres[c * D + k] - r, k);
                    b[k] = cellq(m.cell_centres[c * D + k] + r, k);
                }
                for (int z = a[2]; z <= b[2]; ++z)
                    for (int y = a[1]; y <= b[1]; ++y)
                        for (int x = a[0]; x <= b[0]; ++x) {
                            const int64_t q = ((int64_t)z * G.dims[1] + y) * G.dims[0] + x;
                            if (pass == 0) G.off[(size_t)q + 1]++;
                            else G.cells[(size_t)fill[(size_t)q]++] = c;
                        }
            }
        }
    }
    return FJSPH_OK;
}

void launch_mesh_find(const Params &P, const DevState &W, const MeshDev &M, double *air, int32_t *list,
                      int32_t *count, cudaStream_t s) {
    const int64_t nf = P.n - P.nb;
    if (nf <= 0) return;
    cudaMemsetAsync(count, 0, sizeof(int32_t), s);
    const unsigned g = grid_for(nf, kT);
    if (P.D == 2) {
        k_mesh_mark<2><<<g, kT, 0, s>>>(P, W, air, list, count);
        k_mesh_find<2><<<g, kT, 0, s>>>(W, M, air, list, count);
    } else {
        k_mesh_mark<3><<<g, kT, 0, s>>>(P, W, air, list, count);
        k_mesh_find<3><<<g, kT, 0, s>>>(W, M, air, list, count);
    }
}

} // namespace fjsph
