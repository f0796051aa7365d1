/*
 * neighbours.cu -- GPU cell-linked list replacing the nanoflann KD-tree radius search of
 * src/Neighbours.cpp:7-47.
 *
 * Build per search:
 *   1. bounding box of all positions and the grid over it (cell edge = search radius * (1+1e-6));
 *   2. every particle hashes its cell's linear index into a power-of-two bucket table;
 *      while the grid has no more cells than buckets the hash is the identity, so a row of three
 *      x-adjacent cells is one contiguous bucket range;
 *   3. counting sort of particles by bucket (histogram, exclusive scan, scatter, then each
 *      particle's rank in its bucket by (x, slot)), so buckets are sorted by x;
 *   4. per particle, count and then write its neighbours in CSR form.
 * Membership is the reference's test, d2 < sr with d2 = fma(dz,dz,fma(dy,dy,dx*dx)) in FP64.
 * It is decided first in FP32 on the rounded coordinates, and in FP64 only when the FP32 value
 * falls inside a band whose width bounds the FP32 rounding error; so the lists are exactly the
 * FP64 ones while the bulk of the candidate tests run on the FP32 pipe.  Candidates are read from
 * bucket-ordered copies of the coordinates (hi = fl32(x), lo = fl32(x - hi)), so a thread's walk
 * over a row of cells is a contiguous read; the lo part gives members an FP32 squared distance
 * accurate to FP32 rounding of the separation (used by the split-precision form).
 */
#include "kernels.h"
#include "split.cuh"

namespace fjsph {

namespace {

constexpr int kThreads = 128;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int64_t kMaxAxis = (int64_t)1 << 20;

/* Cells are the support radius 2H long along x (the contiguous direction of a bucket row) and
 * 2H / kCellDiv across it; the walk visits 3 cells of each of (2 kCellDiv + 1)^(D-1) rows.  With
 * kCellDiv = 2 the visited volume is 6H x 5H x 5H instead of (6H)^3 (30 % fewer candidate tests)
 * for four times the cells; halving x as well would make sparse domains (the jet's bounding box
 * is mostly air) outgrow the largest bucket table.  Cell coordinates are floor((x - lo) * inv)
 * with inv = 1 / edge from the host (Params::cell_inv), the same product everywhere. */
__device__ __forceinline__ double cell_pos(const Params &P, double x, double lo, int axis) {
    return (x - lo) * P.cell_inv[axis];
}

/* ---- bounding box ----------------------------------------------------------------------------- */
/* Order key of a coordinate: the IEEE bits mapped so that unsigned order is numeric order (a
 * total order, NaN included, so bucket ranks by key are always a permutation). */
__device__ __forceinline__ unsigned long long x_key(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_x(unsigned long long k) {
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}
__device__ __forceinline__ bool is_nan_bits(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}
__device__ __forceinline__ unsigned long long umin64(unsigned long long a, unsigned long long b) { return a < b ? a : b; }
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

/* Per-block minimum and maximum of every axis as order keys (integer compares instead of the
 * FP64 pipe); NaN coordinates are skipped, as fmin / fmax skip them. */
template <int D>
__global__ void __launch_bounds__(256) k_bbox_part(Params P, DevState W, unsigned long long *part) {
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double x = W.x[k][i];
            if (is_nan_bits(x)) continue;
            const unsigned long long q = x_key(x);
            lo[k] = umin64(lo[k], q);
            hi[k] = umax64(hi[k], q);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = umin64(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = umax64(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    __shared__ unsigned long long sh[6][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sh[k][wid] = lo[k];
            sh[3 + k][wid] = hi[k];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        unsigned long long v = sh[k][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = k < 3 ? umin64(v, sh[k][w]) : umax64(v, sh[k][w]);
        part[blockIdx.x * 6 + k] = v;
    }
}

__global__ void k_bbox_finish(Params P, const unsigned long long *part, int nblk, double *bbox, int64_t *grid,
                              int64_t table) {
    unsigned long long klo[3] = {~0ull, ~0ull, ~0ull}, khi[3] = {0ull, 0ull, 0ull};
    for (int b = threadIdx.x; b < nblk; b += 32)
        for (int k = 0; k < 3; ++k) {
            klo[k] = umin64(klo[k], part[b * 6 + k]);
            khi[k] = umax64(khi[k], part[b * 6 + 3 + k]);
        }
    for (int k = 0; k < 3; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            klo[k] = umin64(klo[k], __shfl_xor_sync(0xffffffffu, klo[k], o));
            khi[k] = umax64(khi[k], __shfl_xor_sync(0xffffffffu, khi[k], o));
        }
    if (threadIdx.x != 0) return;
    /* an axis without a finite value decodes to NaN bounds and is treated as empty below */
    double lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = klo[k] <= khi[k] ? key_x(klo[k]) : NAN;
        hi[k] = klo[k] <= khi[k] ? key_x(khi[k]) : NAN;
    }
    int64_t nc[3] = {1, 1, 1};
    double mag = 0.0;
    for (int k = 0; k < P.D; ++k) {
        if (!(lo[k] <= hi[k])) { /* empty or non-finite */
            lo[k] = 0.0;
            hi[k] = 0.0;
        }
        double c = floor(cell_pos(P, hi[k], lo[k], k)) + 1.0;
        if (!(c < (double)kMaxAxis)) c = (double)kMaxAxis;
        nc[k] = (int64_t)c;
        mag = fmax(mag, fmax(fabs(lo[k]), fabs(hi[k])));
    }
    for (int k = 0; k < 3; ++k) {
        bbox[k] = lo[k];
        bbox[3 + k] = hi[k];
    }
    /* FP32 band.  fl32(x) has |err| <= u |x| <= u M per axis (u = 2^-24, M = largest coordinate
     * magnitude), so near the sphere |d2_f32 - d2| <= D (4 u M R + 3 u R^2) + 2 u R^2 with
     * R = sqrt(sr); twice that, relative to sr, is the band inside which the FP64 test decides. */
    const double u = 5.9604644775390625e-08;
    const double R = sqrt(P.sr);
    const double rel = 2.0 * (P.D * 4.0 * u * mag / R + (3.0 * P.D + 2.0) * u) + 1e-7;
    bbox[6] = rel;
    /* the FP32 thresholds of the band, for the walk */
    float *thr = reinterpret_cast<float *>(bbox + 7);
    thr[0] = (float)(P.sr * (1.0 - rel));
    thr[1] = (float)(P.sr * (1.0 + rel));
    grid[0] = nc[0];
    grid[1] = nc[1];
    grid[2] = nc[2];
    const double ncells = (double)nc[0] * (double)nc[1] * (double)nc[2];
    grid[3] = ncells > (double)table ? 1 : 0;
    grid[4] = ncells > (double)table ? table : (int64_t)ncells; /* buckets in use */
}

/* Quarter-cell index of the occupied cells (identity hash only): bits 10 (b - 1) .. 10 b - 1 of
 * qbin[h] hold the offset from the cell's start of its first entry in x quarter b (b = 1, 2, 3),
 * kQUnknown when the offset does not fit.  Entries are sorted by x, so quarter b's entries are
 * [start + o_b, start + o_(b+1)); the walk reads the part of a row it needs from two of these
 * words instead of searching the cells.  Written by the bucket rank pass from the quarters the
 * hash pass computes. */
constexpr uint32_t kQUnknown = 1023u;
/* hash[i] holds the bucket in its low 30 bits (tables have at most 2^26 buckets) and the x
 * quarter of the particle in its cell in the top two */
constexpr int kQuarterShift = 30;
constexpr uint32_t kBucketMask = (1u << kQuarterShift) - 1u;

/* ---- hashing ---------------------------------------------------------------------------------- */
template <int D>
__device__ __forceinline__ void cell_coords(const Params &P, const double *x, const double *lo, const int64_t *nc,
                                            int64_t *c) {
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k] = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        double f = floor(cell_pos(P, x[k], lo[k], k));
        int64_t v = (f > 0.0) ? (int64_t)fmin(f, (double)(nc[k] - 1)) : 0;
        c[k] = v;
    }
}

/* cell_coords and the position inside the cell in cell edges (the same products) */
template <int D>
__device__ __forceinline__ void cell_coords_frac(const Params &P, const double *x, const double *lo, const int64_t *nc,
                                                 int64_t *c, float *t) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        c[k] = 0;
        t[k] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const double u = cell_pos(P, x[k], lo[k], k);
        const double f = floor(u);
        c[k] = (f > 0.0) ? (int64_t)fmin(f, (double)(nc[k] - 1)) : 0;
        t[k] = (float)(u - (double)c[k]);
    }
}

__device__ __forceinline__ uint64_t lin_index(const int64_t *c, const int64_t *nc) {
    return (uint64_t)c[0] + (uint64_t)nc[0] * ((uint64_t)c[1] + (uint64_t)nc[1] * (uint64_t)c[2]);
}

template <int D>
__global__ void k_hash_count(Params P, DevState W, double *xs0, double *xs1, double *xs2, CellGrid G) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    double *const xs[3] = {xs0, xs1, xs2};
    double x[3] = {0, 0, 0}, lo[3];
    int64_t nc[3], c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = G.bbox[k];
        nc[k] = G.grid[k];
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
        x[k] = W.x[k][i];
        xs[k][i] = x[k];
    }
    float t[3];
    cell_coords_frac<D>(P, x, lo, nc, c, t);
    const uint32_t h = (uint32_t)(lin_index(c, nc) & (uint64_t)(G.table_size - 1));
    const int quarter = t[0] < 0.25f ? 0 : (t[0] < 0.5f ? 1 : (t[0] < 0.75f ? 2 : 3));
    G.hash[i] = h | ((uint32_t)quarter << kQuarterShift);
    G.frac[i] = make_float4(t[0], t[1], t[2], 0.f);
    /* lanes of a warp in the same bucket (consecutive slots usually are) add once */
    const unsigned peers = __match_any_sync(__activemask(), h);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&G.count[h], (int32_t)__popc(peers));
}

/* Scatter of slots into their buckets in arrival order; each entry's (x key, slot) goes to
 * sorted_lo, which serves as scratch until the coordinates are written in bucket order. */
__global__ void k_scatter(Params P, CellGrid G, const double *xs0, int32_t *cursor) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const uint32_t hq = G.hash[i], h = hq & kBucketMask;
    const int32_t pos = G.start[h] + atomicAdd(&cursor[h], 1);
    const unsigned long long k = x_key(xs0[i]);
    reinterpret_cast<uint4 *>(G.sorted_lo)[pos] =
        make_uint4((unsigned)k, (unsigned)(k >> 32), (unsigned)i, hq >> kQuarterShift);
}

/* Each slot's rank in its bucket by (x, slot): buckets come out sorted by x, so a row of
 * x-adjacent cells is sorted by x and the walk can stop at the edges of the x range it needs;
 * the slot breaks ties, so the order is deterministic. */
__global__ void k_bucket_rank(Params P, CellGrid G, const double *xs0) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const uint32_t h = G.hash[i] & kBucketMask;
    const int32_t s0 = G.start[h], s1 = G.start[h + 1];
    const unsigned long long k = x_key(xs0[i]);
    const uint4 *ent = reinterpret_cast<const uint4 *>(G.sorted_lo);
    int32_t rank = 0;
    uint32_t below[4] = {0u, 0u, 0u, 0u}; /* entries in x quarters below 1, 2, 3 */
    for (int32_t e = s0; e < s1; ++e) {
        const uint4 q = ent[e];
        const unsigned long long ke = (unsigned long long)q.x | ((unsigned long long)q.y << 32);
        rank += (ke < k || (ke == k && (int64_t)q.z < i)) ? 1 : 0;
#pragma unroll
        for (int b = 1; b <= 3; ++b) below[b] += q.w < (uint32_t)b ? 1u : 0u;
    }
    G.sorted[s0 + rank] = (int32_t)i;
    if (rank == 0) { /* one writer per bucket: its quarter index (read by the walk when the hash
                      * is the identity, so a bucket is one cell) */
#pragma unroll
        for (int b = 1; b <= 3; ++b)
            if (below[b] > kQUnknown) below[b] = kQUnknown;
        G.qbin[h] = below[1] | (below[2] << 10) | (below[3] << 20);
    }
}

/* Coordinates in bucket order: hi = (fl32(x), slot bits), lo = fl32(x - hi). */
template <int D>
__global__ void k_sorted_pos(Params P, const double *xs0, const double *xs1, const double *xs2, CellGrid G) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= P.n) return;
    const int32_t s = G.sorted[e];
    const double x0 = xs0[s], x1 = xs1[s], x2 = D == 3 ? xs2[s] : 0.0;
    float h0, h1, h2, l0, l1, l2;
    split_f32(x0, h0, l0);
    split_f32(x1, h1, l1);
    split_f32(x2, h2, l2);
    G.sorted_hi[e] = make_float4(h0, h1, h2, __int_as_float(s));
    G.sorted_lo[e] = make_float4(l0, l1, l2, 0.f);
}

/* ---- neighbour walk --------------------------------------------------------------------------- */
/* Visits every candidate of particle i once and calls f(j) for each member (d2 < sr). */
template <int D, class F>
__device__ __forceinline__ void walk(const Params &P, double *const xs[3], const CellGrid &G, int64_t i, F &&f) {
    int64_t nc[3], c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) nc[k] = G.grid[k];
    const bool wrap = G.grid[3] != 0;
    /* the particle's cell and its position inside it, from the hash pass (for a wrapped table
     * the bucket is not the cell: recomputed) */
    float t[3];
    {
        const float4 tf = G.frac[i];
        t[0] = tf.x;
        t[1] = tf.y;
        t[2] = tf.z;
    }
    if (!wrap) {
        const uint64_t h = G.hash[i] & kBucketMask;
        c[0] = (int64_t)(h % (uint64_t)nc[0]);
        c[1] = (int64_t)((h / (uint64_t)nc[0]) % (uint64_t)nc[1]);
        c[2] = (int64_t)(h / ((uint64_t)nc[0] * (uint64_t)nc[1]));
    } else {
        double lo[3], xi[3] = {0, 0, 0};
#pragma unroll
        for (int k = 0; k < 3; ++k) lo[k] = G.bbox[k];
#pragma unroll
        for (int k = 0; k < D; ++k) xi[k] = xs[k][i];
        cell_coords<D>(P, xi, lo, nc, c);
    }
    float fi[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < D; ++k) fi[k] = to_f32(xs[k][i]);
    const float sr_lo = reinterpret_cast<const float *>(G.bbox + 7)[0];
    const float sr_hi = reinterpret_cast<const float *>(G.bbox + 7)[1];
    const uint64_t mask = (uint64_t)(G.table_size - 1);
    const int zr = (D == 3) ? kCellDiv : 0, yr = kCellDiv;
    const int64_t x0 = c[0] > 0 ? c[0] - 1 : 0;
    const int64_t x1 = c[0] + 1 < nc[0] ? c[0] + 1 : nc[0] - 1;
    /* wrapped table: true if an earlier neighbour cell of this walk hashes to bucket h */
    auto visited_before = [&](int dz, int dy, int64_t cx, uint64_t h) -> bool {
        for (int dz2 = -zr; dz2 <= zr; ++dz2) {
            const int64_t cz2 = c[2] + dz2;
            if (cz2 < 0 || cz2 >= nc[2]) continue;
            for (int dy2 = -yr; dy2 <= yr; ++dy2) {
                const int64_t cy2 = c[1] + dy2;
                if (cy2 < 0 || cy2 >= nc[1]) continue;
                for (int64_t cx2 = x0; cx2 <= x1; ++cx2) {
                    if (dz2 == dz && dy2 == dy && cx2 == cx) return false;
                    int64_t c2[3] = {cx2, cy2, cz2};
                    if ((lin_index(c2, nc) & mask) == h) return true;
                }
            }
        }
        return false;
    };
    /* FP32 test with the FP64 decision inside the rounding band */
    auto member = [&](const float4 fj) -> bool {
        const float dx = fi[0] - fj.x, dy = fi[1] - fj.y;
        float d2f = dx * dx + dy * dy;
        if (D == 3) {
            const float dz = fi[2] - fj.z;
            d2f += dz * dz;
        }
        if (d2f < sr_lo) return true;
        if (d2f > sr_hi) return false;
        const int32_t j = __float_as_int(fj.w);
        double xi[D], xj[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            xi[k] = xs[k][i];
            xj[k] = xs[k][j];
        }
        return dist2<D>(xi, xj) < P.sr;
    };
    /* Candidates [e0, e1) in batches of 32: a bit mask of the members first, then f for the
     * members only, so the lanes of a warp run the (longer) member code together instead of
     * at every candidate where some lane has a member. */
    auto range = [&](int32_t e0, int32_t e1) {
        for (int32_t b = e0; b < e1; b += 32) {
            const int32_t m = e1 - b < 32 ? e1 - b : 32;
            unsigned bits = 0u;
            for (int32_t q = 0; q < m; ++q)
                if (member(G.sorted_hi[b + q])) bits |= 1u << q;
            while (bits) {
                const int q = __ffs(bits) - 1;
                bits &= bits - 1u;
                f(__float_as_int(G.sorted_hi[b + q].w), b + q);
            }
        }
    };
    /* Identity hash: the row's x range.  Buckets are sorted by x, so a row's members lie within
     * |x_j - x_i| <= r_row with r_row^2 = R^2 - (y gap to the row)^2 - (z gap)^2: the walk tests
     * the part of the row inside that range, to the quarter cell, and skips rows beyond R.  The
     * bounds are widened by a margin that covers the FP32 rounding of both coordinates and of
     * the bound itself, so no member is ever left out. */
    const float Rf = sqrtf((float)P.sr);
    const float r2f = (float)P.sr * (1.f + 1e-5f);
    const float mx = 5e-7f * (fabsf(fi[0]) + 2.f * Rf) + 1e-5f * Rf;
    const float ey = (float)P.cell_edge[1], ez = (float)P.cell_edge[2], inv_x = (float)P.cell_inv[0];
    /* position of x_i inside its cell, in cell edges */
    const float tx = t[0], ty = t[1], tz = D == 3 ? t[2] : 0.f;
    auto gap = [](int d, float t) { /* distance to the band of row offset d, in cell edges */
        const float g = d > 0 ? (float)d - t : (d < 0 ? t - 1.f - (float)d : 0.f);
        return fmaxf(0.f, g - 1e-4f);
    };
    auto quarter = [](float u) { return u < 0.25f ? 0 : (u < 0.5f ? 1 : (u < 0.75f ? 2 : 3)); };
    const bool has_left = c[0] > 0, has_right = c[0] + 1 < nc[0];
    for (int dz = -zr; dz <= zr; ++dz) {
        const int64_t cz = c[2] + dz;
        if (cz < 0 || cz >= nc[2]) continue;
        const float gz = gap(dz, tz) * ez;
        for (int dy = -yr; dy <= yr; ++dy) {
            const int64_t cy = c[1] + dy;
            if (cy < 0 || cy >= nc[1]) continue;
            if (!wrap) {
                const float gy = gap(dy, ty) * ey;
                const float rr2 = r2f - gy * gy - gz * gz;
                if (rr2 <= 0.f) continue;
                const float rr = sqrtf(rr2);
                int64_t cc[3] = {c[0], cy, cz};
                const uint64_t hm = lin_index(cc, nc);
                /* x range in cell edges relative to x_i's cell, widened by 1e-4 edges */
                const float w = (rr + mx) * inv_x;
                const float ulo = tx - w - 1e-4f, uhi = tx + w + 1e-4f;
                /* first cell (cl) and quarter (bl) that can hold a member, last cell (ch) and
                 * quarter (bh) */
                int cl = 0, bl = 0, ch = 0, bh = 3;
                if (ulo < 0.f) {
                    if (has_left) {
                        cl = -1;
                        bl = ulo >= -1.f ? quarter(ulo + 1.f) : 0;
                    }
                } else {
                    bl = quarter(ulo);
                }
                if (uhi >= 1.f) {
                    if (has_right) {
                        ch = 1;
                        bh = uhi < 2.f ? quarter(uhi - 1.f) : 3;
                    }
                } else {
                    bh = quarter(uhi);
                }
                const int32_t sa = G.start[hm + cl], sb = G.start[hm + cl + 1];
                const int32_t sc = G.start[hm + ch], sd = G.start[hm + ch + 1];
                int32_t e0 = sa, e1 = sd;
                if (bl > 0 && sb > sa) { /* occupied cell: its quarter index is valid */
                    const uint32_t o = (G.qbin[hm + cl] >> (10 * (bl - 1))) & 1023u;
                    if (o != kQUnknown) e0 = sa + (int32_t)o;
                }
                if (bh < 3 && sd > sc) {
                    const uint32_t o = (G.qbin[hm + ch] >> (10 * bh)) & 1023u;
                    if (o != kQUnknown) e1 = sc + (int32_t)o;
                }
                range(e0, e1);
            } else {
                for (int64_t cx = x0; cx <= x1; ++cx) {
                    int64_t cc[3] = {cx, cy, cz};
                    const uint64_t h = lin_index(cc, nc) & mask;
                    if (visited_before(dz, dy, cx, h)) continue;
                    const int32_t e0 = G.start[h], e1 = G.start[h + 1];
                    range(e0, e1);
                }
            }
        }
    }
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_nbr_count(Params P, double *xs0, double *xs1, double *xs2, CellGrid G,
                                                         int32_t *counts) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    double *const xs[3] = {xs0, xs1, xs2};
    int32_t cnt = 0;
    walk<D>(P, xs, G, i, [&](int32_t, int32_t) { ++cnt; });
    counts[i] = cnt;
}

/* Entries per slice of kSlice slots: kSlice x the largest count in the slice (one warp per
 * slice; the launch covers whole warps from slot 0). */
__global__ void k_slice_width(const int32_t *counts, int64_t n, int32_t *width) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int32_t c = i < n ? counts[i] : 0;
    const int32_t m = __reduce_max_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && i < n) width[i / kSlice] = ((m + kChunk - 1) / kChunk) * kChunk * kSlice;
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_nbr_fill(Params P, double *xs0, double *xs1, double *xs2, CellGrid G,
                                                        const int64_t *off, int32_t *idx, int2 *pair,
                                                        const int64_t *slice, const int32_t *counts, int64_t cap,
                                                        int32_t *status) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    double *const xs[3] = {xs0, xs1, xs2};
    if (pair) {
        /* sliced-ELL with chunks of kChunk pairs per slot: whole chunks are written as two
         * 16-byte stores (one 32-byte sector) */
        const int64_t base = slice[i / kSlice] + (i % kSlice) * kChunk;
        const int32_t kend = counts[i];
        if (kend > 0 && sell_entry(base, ((kend - 1) / kChunk) * kChunk + kChunk - 1) >= cap) { /* too small */
            atomicOr(status, kStatusNbrOverflow);
            return;
        }
        /* (slot, FP32 squared distance from the hi/lo split, about 1e-7 relative) */
        float hi[3] = {0, 0, 0}, lo[3] = {0, 0, 0};
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double x = xs[k][i];
            split_f32(x, hi[k], lo[k]);
        }
        /* one chunk per thread staged in shared memory (registers are the walk's) */
        __shared__ __align__(16) int2 stage[kThreads][kChunk];
        int2 *buf = stage[threadIdx.x];
        int32_t k = 0;
        auto flush = [&](int32_t chunk) {
            const int4 *src = reinterpret_cast<const int4 *>(buf);
            int4 *dst = reinterpret_cast<int4 *>(pair + base + (int64_t)chunk * (kSlice * kChunk));
            dst[0] = src[0];
            dst[1] = src[1];
        };
        walk<D>(P, xs, G, i, [&](int32_t j, int32_t e) {
            if (k < kend) {
                const float4 hj = G.sorted_hi[e], lj = G.sorted_lo[e];
                const float dx = (hj.x - hi[0]) + (lj.x - lo[0]), dy = (hj.y - hi[1]) + (lj.y - lo[1]);
                float d2 = dx * dx + dy * dy;
                if (D == 3) {
                    const float dz = (hj.z - hi[2]) + (lj.z - lo[2]);
                    d2 += dz * dz;
                }
                buf[k % kChunk] = make_int2(j, __float_as_int(d2));
                if (k % kChunk == kChunk - 1) flush(k / kChunk);
            }
            ++k;
        });
        if (kend % kChunk != 0) flush(kend / kChunk);
        return;
    }
    int64_t w = off[i];
    const int64_t wend = off[i + 1];
    if (wend > cap) {
        atomicOr(status, kStatusNbrOverflow);
        return;
    }
    walk<D>(P, xs, G, i, [&](int32_t j, int32_t) {
        if (w < wend) idx[w] = j;
        ++w;
    });
}

/* Single-pass fill of the split-precision lists: every slice holds kSlice x wcap entries, so a
 * slot's storage is known before its walk and no counting walk is needed.  The walk writes up
 * to wcap pairs, records the true count, and the block's largest count and pair total go to
 * the device scalars; a count above wcap raises kStatusNbrOverflow (the caller re-runs the fill
 * with a larger wcap). */
template <int D>
__global__ void __launch_bounds__(kThreads) k_nbr_fill_fixed(Params P, double *xs0, double *xs1, double *xs2,
                                                              CellGrid G, int2 *pair, int32_t *counts, int32_t wcap,
                                                              DevScalars *dsc) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool live = i < P.n;
    __shared__ __align__(16) int2 stage[kThreads][kChunk];
    int32_t k = 0;
    if (live) {
        double *const xs[3] = {xs0, xs1, xs2};
        const int64_t base = (i / kSlice) * (int64_t)kSlice * wcap + (i % kSlice) * kChunk;
        float hi[3] = {0, 0, 0}, lo[3] = {0, 0, 0};
#pragma unroll
        for (int q = 0; q < D; ++q) {
            const double x = xs[q][i];
            split_f32(x, hi[q], lo[q]);
        }
        int2 *buf = stage[threadIdx.x];
        auto flush = [&](int32_t chunk) {
            const int4 *src = reinterpret_cast<const int4 *>(buf);
            int4 *dst = reinterpret_cast<int4 *>(pair + base + (int64_t)chunk * (kSlice * kChunk));
            dst[0] = src[0];
            dst[1] = src[1];
        };
        walk<D>(P, xs, G, i, [&](int32_t j, int32_t e) {
            if (k < wcap) {
                const float4 hj = G.sorted_hi[e], lj = G.sorted_lo[e];
                const float dx = (hj.x - hi[0]) + (lj.x - lo[0]), dy = (hj.y - hi[1]) + (lj.y - lo[1]);
                float d2 = dx * dx + dy * dy;
                if (D == 3) {
                    const float dz = (hj.z - hi[2]) + (lj.z - lo[2]);
                    d2 += dz * dz;
                }
                buf[k % kChunk] = make_int2(j, __float_as_int(d2));
                if (k % kChunk == kChunk - 1) flush(k / kChunk);
            }
            ++k;
        });
        const int32_t kw = k < wcap ? k : wcap;
        if (kw % kChunk != 0) flush(kw / kChunk);
        counts[i] = k;
    }
    const int32_t kmax = __reduce_max_sync(0xffffffffu, (unsigned)k);
    const unsigned ksum = __reduce_add_sync(0xffffffffu, (unsigned)k);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&dsc->maxcnt, kmax);
        atomicAdd(&dsc->pairs, (unsigned long long)ksum);
        if (kmax > wcap) atomicOr(&dsc->status, kStatusNbrOverflow);
    }
}

__global__ void k_slice_fixed(int64_t *slice, int64_t nslices, int64_t per) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s <= nslices) slice[s] = s * per;
}

/* ---- scans ------------------------------------------------------------------------------------ */
template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

/* exclusive scan of one block's tile of kScanThreads*kScanItems items; returns the tile total */
template <typename TI, typename TO>
__device__ TO block_tile_scan(const TI *in, TO *out, int64_t base, int64_t n, TO carry, bool write) {
    __shared__ TO wsum[kScanThreads / 32];
    TO v[kScanItems];
    TO local = 0;
    const int64_t i0 = base + (int64_t)threadIdx.x * kScanItems;
    if (sizeof(TI) == 4 && kScanItems == 8 && i0 + kScanItems <= n && (reinterpret_cast<uintptr_t>(in + i0) & 15) == 0) {
        /* whole, aligned run of 8 32-bit items: two 16-byte loads */
        const int4 a = reinterpret_cast<const int4 *>(in + i0)[0], b = reinterpret_cast<const int4 *>(in + i0)[1];
        const int32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            v[k] = (TO)(TI)w[k];
            local += v[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            const int64_t idx = i0 + k;
            v[k] = idx < n ? (TO)in[idx] : (TO)0;
            local += v[k];
        }
    }
    TO incl = warp_incl_scan<TO>(local);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        TO s = lane < kScanThreads / 32 ? wsum[lane] : (TO)0;
        s = warp_incl_scan<TO>(s);
        if (lane < kScanThreads / 32) wsum[lane] = s;
    }
    __syncthreads();
    const TO warp_off = wid > 0 ? wsum[wid - 1] : (TO)0;
    const TO total = wsum[kScanThreads / 32 - 1];
    if (write) {
        TO run = carry + warp_off + incl - local;
        if (sizeof(TO) == 4 && kScanItems == 8 && i0 + kScanItems <= n &&
            (reinterpret_cast<uintptr_t>(out + i0) & 15) == 0) {
            int32_t w[8];
#pragma unroll
            for (int k = 0; k < kScanItems; ++k) {
                w[k] = (int32_t)run;
                run += v[k];
            }
            reinterpret_cast<int4 *>(out + i0)[0] = make_int4(w[0], w[1], w[2], w[3]);
            reinterpret_cast<int4 *>(out + i0)[1] = make_int4(w[4], w[5], w[6], w[7]);
        } else {
#pragma unroll
            for (int k = 0; k < kScanItems; ++k) {
                const int64_t idx = i0 + k;
                if (idx < n) out[idx] = run;
                run += v[k];
            }
        }
    }
    __syncthreads();
    return total;
}

/* Scans take an optional device-side length n_dev (the bucket table is scanned only up to the
 * cells the grid has, which the host does not know without a round trip): the scanned length is
 * min(*n_dev, n), tiles beyond it do nothing, and out[length] receives the total. */
__device__ __forceinline__ int64_t scan_len(int64_t n, const int64_t *n_dev) {
    if (!n_dev) return n;
    const int64_t m = *n_dev;
    return m < n ? m : n;
}

template <typename TI, typename TO>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const TI *in, int64_t n, const int64_t *n_dev,
                                                               TO *tile_sums) {
    const int64_t ne = scan_len(n, n_dev);
    const int64_t base = (int64_t)blockIdx.x * kScanThreads * kScanItems;
    if (base >= ne) { /* uniform per block */
        if (threadIdx.x == 0) tile_sums[blockIdx.x] = (TO)0;
        return;
    }
    TO t = block_tile_scan<TI, TO>(in, (TO *)nullptr, base, ne, (TO)0, false);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = t;
}

template <typename TO>
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(TO *tile_sums, int64_t ntiles, TO *out, int64_t n,
                                                              const int64_t *n_dev) {
    /* exclusive scan of the tile totals, in place, one block walking tiles of the tile array */
    TO carry = 0;
    for (int64_t base = 0; base < ntiles; base += (int64_t)kScanThreads * kScanItems) {
        TO t = block_tile_scan<TO, TO>(tile_sums, tile_sums, base, ntiles, carry, true);
        carry += t;
    }
    if (threadIdx.x == 0) {
        tile_sums[ntiles] = carry;
        out[scan_len(n, n_dev)] = carry;
    }
}

template <typename TI, typename TO>
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const TI *in, TO *out, int64_t n, const int64_t *n_dev,
                                                              const TO *tile_sums) {
    const int64_t ne = scan_len(n, n_dev);
    const int64_t base = (int64_t)blockIdx.x * kScanThreads * kScanItems;
    if (base >= ne) return;
    block_tile_scan<TI, TO>(in, out, base, ne, tile_sums[blockIdx.x], true);
}

template <typename TI, typename TO>
void scan_exclusive(const TI *in, TO *out, int64_t n, TO *tmp, cudaStream_t s, const int64_t *n_dev = nullptr) {
    const int64_t tile = (int64_t)kScanThreads * kScanItems;
    const int64_t ntiles = (n + tile - 1) / tile;
    if (ntiles == 0) {
        cudaMemsetAsync(out, 0, sizeof(TO), s);
        return;
    }
    k_scan_reduce<TI, TO><<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, n_dev, tmp);
    k_scan_tiles<TO><<<1, kScanThreads, 0, s>>>(tmp, ntiles, out, n, n_dev);
    k_scan_apply<TI, TO><<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, out, n, n_dev, tmp);
}

/* zero a[0 .. min(*n_dev, nmax)] (the bucket counts the grid uses) */
__global__ void k_zero_counts(int32_t *a, int64_t nmax, const int64_t *n_dev) {
    const int64_t n = scan_len(nmax, n_dev) + 1;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        a[k] = 0;
}

/* ---- re-ordering ------------------------------------------------------------------------------ */
__global__ void k_bound_flags(Params P, const int32_t *sorted, int32_t *flag) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    flag[p] = sorted[p] < P.nb ? 1 : 0;
}

/* new slot of every particle (boundary slots first, each part in bucket order); the per-slot cell
 * data of the hash pass follow their particles into the second buffers */
__global__ void k_reorder_map(Params P, CellGrid G, const int32_t *flag, const int32_t *ex, int32_t *new_of_old) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const int32_t old = G.sorted[p];
    const int32_t ns = flag[p] ? ex[p] : (int32_t)(P.nb + p - ex[p]);
    new_of_old[old] = ns;
    G.sorted[p] = ns;
    G.hash2[ns] = G.hash[old];
    G.frac2[ns] = G.frac[old];
}

} // namespace

void launch_sorted_pos(const Params &P, double *const xs[3], CellGrid &G, cudaStream_t s) {
    if (P.n == 0) return;
    if (P.D == 2)
        k_sorted_pos<2><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, xs[0], xs[1], xs[2], G);
    else
        k_sorted_pos<3><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, xs[0], xs[1], xs[2], G);
}

void launch_bbox(const Params &P, const DevState &W, CellGrid &G, cudaStream_t s) {
    /* partials (6 keys per block) live in scan_tmp, which the bucket scan overwrites later */
    int nblk = (int)std::min<int64_t>(grid_for(P.n, 256), kBboxBlocks);
    if (nblk < 1) nblk = 1;
    unsigned long long *part = reinterpret_cast<unsigned long long *>(G.scan_tmp);
    if (P.D == 2)
        k_bbox_part<2><<<nblk, 256, 0, s>>>(P, W, part);
    else
        k_bbox_part<3><<<nblk, 256, 0, s>>>(P, W, part);
    k_bbox_finish<<<1, 32, 0, s>>>(P, part, nblk, G.bbox, G.grid, G.table_size);
}

void zero_counts(CellGrid &G, cudaStream_t s) {
    const int64_t blocks = std::min<int64_t>((G.table_size + 1 + 255) / 256, 152 * 16);
    k_zero_counts<<<(unsigned)blocks, 256, 0, s>>>(G.count, G.table_size, G.grid + 4);
}

void launch_hash_and_count(const Params &P, const DevState &W, double *const xs[3], CellGrid &G, cudaStream_t s) {
    zero_counts(G, s);
    if (P.n == 0) return;
    if (P.D == 2)
        k_hash_count<2><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, W, xs[0], xs[1], xs[2], G);
    else
        k_hash_count<3><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, W, xs[0], xs[1], xs[2], G);
}

void launch_scan_i32(const int32_t *in, int32_t *out, int64_t n, int32_t *tmp, cudaStream_t s) {
    scan_exclusive<int32_t, int32_t>(in, out, n, tmp, s);
}
void launch_scan_buckets(CellGrid &G, cudaStream_t s) {
    scan_exclusive<int32_t, int32_t>(G.count, G.start, G.table_size, G.scan_tmp, s, G.grid + 4);
}
void launch_scan_i64(const int32_t *in, int64_t *out, int64_t n, int64_t *tmp, cudaStream_t s) {
    scan_exclusive<int32_t, int64_t>(in, out, n, tmp, s);
}

void launch_scatter_sort(const Params &P, CellGrid &G, const double *xs0, cudaStream_t s) {
    /* G.count is reused as the scatter cursor */
    zero_counts(G, s);
    if (P.n == 0) return;
    k_scatter<<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, G, xs0, G.count);
    k_bucket_rank<<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, G, xs0);
}

void launch_nbr_count(const Params &P, double *const xs[3], const CellGrid &G, int32_t *counts, cudaStream_t s) {
    if (P.n == 0) return;
    if (P.D == 2)
        k_nbr_count<2><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, xs[0], xs[1], xs[2], G, counts);
    else
        k_nbr_count<3><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, xs[0], xs[1], xs[2], G, counts);
}

void launch_nbr_fill(const Params &P, double *const xs[3], const CellGrid &G, const int64_t *off, int32_t *idx,
                     int2 *pair, const int64_t *slice, const int32_t *counts, int64_t cap, int32_t *status,
                     cudaStream_t s) {
    if (P.n == 0) return;
    if (P.D == 2)
        k_nbr_fill<2><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, xs[0], xs[1], xs[2], G, off, idx, pair, slice,
                                                                   counts, cap, status);
    else
        k_nbr_fill<3><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, xs[0], xs[1], xs[2], G, off, idx, pair, slice,
                                                                   counts, cap, status);
}

void launch_nbr_fill_fixed(const Params &P, double *const xs[3], const CellGrid &G, int2 *pair, int32_t *counts,
                           int64_t *slice, int32_t wcap, DevScalars *dsc, cudaStream_t s) {
    if (P.n == 0) return;
    const int64_t nslices = (P.n + kSlice - 1) / kSlice;
    k_slice_fixed<<<grid_for(nslices + 1, kThreads), kThreads, 0, s>>>(slice, nslices, (int64_t)kSlice * wcap);
    if (P.D == 2)
        k_nbr_fill_fixed<2><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, xs[0], xs[1], xs[2], G, pair, counts,
                                                                         wcap, dsc);
    else
        k_nbr_fill_fixed<3><<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, xs[0], xs[1], xs[2], G, pair, counts,
                                                                         wcap, dsc);
}

void launch_slice_width(const int32_t *counts, int64_t n, int32_t *width, cudaStream_t s) {
    if (n > 0) k_slice_width<<<grid_for(n, kThreads), kThreads, 0, s>>>(counts, n, width);
}

void launch_reorder_map(const Params &P, const CellGrid &G, int32_t *new_of_old, int32_t *tmp, int64_t tmp_len,
                        cudaStream_t s) {
    /* tmp: [n] flags, [n+1] exclusive scan, then scan partials */
    (void)tmp_len;
    if (P.n == 0) return;
    int32_t *flag = tmp, *ex = tmp + P.n, *part = tmp + 2 * P.n + 1;
    k_bound_flags<<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, G.sorted, flag);
    scan_exclusive<int32_t, int32_t>(flag, ex, P.n, part, s);
    k_reorder_map<<<grid_for(P.n, kThreads), kThreads, 0, s>>>(P, G, flag, ex, new_of_old);
    cudaMemcpyAsync(G.hash, G.hash2, sizeof(uint32_t) * P.n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(G.frac, G.frac2, sizeof(float4) * P.n, cudaMemcpyDeviceToDevice, s);
}

} // namespace fjsph

/* ---- tiles of the split-precision sweeps (tiles.cuh) ------------------------------------------ */
#include "tiles.cuh"

namespace fjsph {

namespace {

/* Occupancy of every tile of the grid (a tile is occupied when one of its cells holds a particle);
 * a wrapped bucket table (buckets are not cells) leaves no tile and reports the overflow bit. */
template <int D>
__global__ void k_tile_flags(CellGrid G, TileDev T, int32_t *status) {
    using TT = Tile<D>;
    const TileGrid tg = tile_grid<D>(G);
    const bool wrap = G.grid[3] != 0;
    const int64_t ntiles = wrap ? 0 : tg.nt[0] * tg.nt[1] * tg.nt[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *T.ntot = ntiles;
        if (wrap) atomicOr(status, kStatusTileOverflow);
    }
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tx = t % tg.nt[0], ty = (t / tg.nt[0]) % tg.nt[1], tz = t / (tg.nt[0] * tg.nt[1]);
        const int64_t x0 = tx * TT::TX;
        const int64_t x1 = (x0 + TT::TX < tg.nc[0] ? x0 + TT::TX : tg.nc[0]) - 1;
        int occ = 0;
        for (int oz = 0; oz < TT::TZ && !occ; ++oz) {
            const int64_t cz = tz * TT::TZ + oz;
            if (cz >= tg.nc[2]) break;
            for (int oy = 0; oy < TT::TY; ++oy) {
                const int64_t cy = ty * TT::TY + oy;
                if (cy >= tg.nc[1]) break;
                const int64_t row = tg.nc[0] * (cy + tg.nc[1] * cz);
                if (G.start[row + x1 + 1] > G.start[row + x0]) {
                    occ = 1;
                    break;
                }
            }
        }
        T.flag[t] = occ;
    }
}

__global__ void k_tile_list(TileDev T) {
    const int64_t n = *T.ntot;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        if (T.flag[t]) T.list[T.scan[t]] = (int32_t)t;
    if (blockIdx.x == 0 && threadIdx.x == 0) *T.count = n > 0 ? T.scan[n] : 0;
}

/* Member masks: every own particle of every tile tests its candidates in stencil order (FP32 on
 * the in-cell positions, the FP64 test of the reference inside the rounding band) and writes one
 * bit per candidate.  A stencil row whose y/z gap alone exceeds the radius keeps zero bits without
 * tests.  One uniform loop over candidates keeps the lanes of a warp in step. */
template <int D>
__global__ void __launch_bounds__(kTileThreads) k_tile_masks(Params P, CellGrid G, TileDev T, Packed K,
                                                              const double *xs0, const double *xs1,
                                                              const double *xs2, DevScalars *dsc) {
    using TT = Tile<D>;
    extern __shared__ __align__(16) unsigned char tsm[];
    TileSmem ts = tile_smem<D>(tsm, T.smax, kStageS);
    const TileGrid tg = tile_grid<D>(G);
    const double *const xs[3] = {xs0, xs1, xs2};
    const float edge[3] = {(float)P.cell_edge[0], (float)P.cell_edge[1], (float)P.cell_edge[2]};
    const float thr_lo = (float)(P.sr * (1.0 - 2e-5)), thr_hi = (float)(P.sr * (1.0 + 2e-5));
    const float row_cut = (float)(P.sr * (1.0 + 1e-4));
    const int lane = threadIdx.x & 31;
    unsigned long long pairs = 0;
    int maxcnt = 0;
    const int ntl = *T.count;
    for (int it = blockIdx.x; it < ntl; it += gridDim.x) {
        tile_setup<D>(P, G, K, tg, T.list[it], kStageS, kOwnAll, ts);
        const bool over = ts.over();
        if (threadIdx.x == 0 && ts.head[3]) atomicOr(&dsc->status, kStatusTileOverflow);
        const int nown = ts.nown();
        for (int base = threadIdx.x - lane; base < nown; base += blockDim.x) {
            const int k = base + lane;
            if (k >= nown) continue;
            const TileOwnRef o = tile_own<D>(ts, k);
            const float4 Si = tile_ld_s(ts, G, o.e, o.hc / TT::HX, over);
            const int32_t si = __float_as_int(Si.w);
            double xi[3] = {0, 0, 0};
            bool xi_loaded = false;
            uint32_t word = 0u;
            int pos = 0, wi = 0, nm = 0;
            auto flush = [&]() {
                if (wi < kMaskWords) T.mask[wi * T.stride + o.g] = word;
                ++wi;
                word = 0u;
            };
            TileCursor<D> cur;
            cur.init(ts, o, nullptr, 0);
            for (;;) {
                while (cur.left == 0) {
                    if (!cur.open_row()) break;
                    /* the row's y/z gap from the particle, in metres */
                    const float gy = cur.dy > 0 ? (float)cur.dy - Si.y : (cur.dy < 0 ? Si.y - 1.f - (float)cur.dy : 0.f);
                    const float gz = cur.dz > 0 ? (float)cur.dz - Si.z : (cur.dz < 0 ? Si.z - 1.f - (float)cur.dz : 0.f);
                    const float a = fmaxf(gy, 0.f) * edge[1], b = D == 3 ? fmaxf(gz, 0.f) * edge[2] : 0.f;
                    if (a * a + b * b > row_cut) { /* out of reach: zero bits */
                        int n = cur.left;
                        while (n > 0) {
                            const int take = n < 32 - (pos & 31) ? n : 32 - (pos & 31);
                            pos += take;
                            n -= take;
                            if ((pos & 31) == 0) flush();
                        }
                        cur.left = 0;
                    }
                }
                if (cur.left == 0) break;
                TileNbr n;
                cur.next_cand(n);
                const float4 Sj = tile_ld_s(ts, G, n.e, n.row, over);
                const float ax = ((float)n.dc[0] + (Sj.x - Si.x)) * edge[0];
                const float ay = ((float)n.dc[1] + (Sj.y - Si.y)) * edge[1];
                float d2 = ax * ax + ay * ay;
                if (D == 3) {
                    const float az = ((float)n.dc[2] + (Sj.z - Si.z)) * edge[2];
                    d2 += az * az;
                }
                bool m = d2 < thr_lo;
                if (!m && d2 <= thr_hi) { /* inside the rounding band: the FP64 test */
                    if (!xi_loaded) {
#pragma unroll
                        for (int q = 0; q < D; ++q) xi[q] = xs[q][si];
                        xi_loaded = true;
                    }
                    const int32_t sj = __float_as_int(Sj.w);
                    double xj[3] = {0, 0, 0};
#pragma unroll
                    for (int q = 0; q < D; ++q) xj[q] = xs[q][sj];
                    m = dist2<D>(xi, xj) < P.sr;
                }
                nm += m ? 1 : 0;
                word |= (m ? 1u : 0u) << (pos & 31);
                ++pos;
                if ((pos & 31) == 0) flush();
            }
            if (pos & 31) flush();
            for (; wi < kMaskWords; ++wi) T.mask[wi * T.stride + o.g] = 0u;
            if (pos > 32 * kMaskWords) atomicOr(&dsc->status, kStatusTileOverflow);
            pairs += (unsigned long long)nm;
            maxcnt = nm > maxcnt ? nm : maxcnt;
        }
        __syncthreads();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
        const int m2 = __shfl_xor_sync(0xffffffffu, maxcnt, o);
        maxcnt = m2 > maxcnt ? m2 : maxcnt;
    }
    if (lane == 0) {
        if (pairs) atomicAdd(&dsc->tile_pairs, pairs);
        atomicMax(&dsc->tile_maxcnt, maxcnt);
    }
}

/* Members written out per slot (the neighbour export of the tile path): pass 0 counts, pass 1
 * writes the neighbour slots and their FP64 squared distances at off[slot]. */
template <int D>
__global__ void __launch_bounds__(kTileThreads) k_tile_export(Params P, CellGrid G, TileDev T, Packed K,
                                                               const double *xs0, const double *xs1,
                                                               const double *xs2, int pass, int32_t *counts,
                                                               const int64_t *off, int64_t *idx, double *d2) {
    using TT = Tile<D>;
    extern __shared__ __align__(16) unsigned char tsm[];
    TileSmem ts = tile_smem<D>(tsm, T.smax, kStageS);
    const TileGrid tg = tile_grid<D>(G);
    const double *const xs[3] = {xs0, xs1, xs2};
    const int ntl = *T.count;
    for (int it = blockIdx.x; it < ntl; it += gridDim.x) {
        tile_setup<D>(P, G, K, tg, T.list[it], kStageS, kOwnAll, ts);
        const bool over = ts.over();
        const int nown = ts.nown();
        for (int k = threadIdx.x; k < nown; k += blockDim.x) {
            const TileOwnRef o = tile_own<D>(ts, k);
            const float4 Si = tile_ld_s(ts, G, o.e, o.hc / TT::HX, over);
            const int32_t si = __float_as_int(Si.w);
            if (pass == 0) {
                counts[si] = tile_member_count(T.mask, T.stride, o.g);
                continue;
            }
            double xi[3] = {0, 0, 0};
#pragma unroll
            for (int q = 0; q < D; ++q) xi[q] = xs[q][si];
            int64_t w = off[si];
            TileCursor<D> cur;
            cur.init(ts, o, T.mask, T.stride);
            TileNbr n;
            while (cur.next_member(n)) {
                const float4 Sj = tile_ld_s(ts, G, n.e, n.row, over);
                const int32_t sj = __float_as_int(Sj.w);
                double xj[3] = {0, 0, 0};
#pragma unroll
                for (int q = 0; q < D; ++q) xj[q] = xs[q][sj];
                idx[w] = sj;
                d2[w] = dist2<D>(xi, xj);
                ++w;
            }
        }
        __syncthreads();
    }
}

/* CTAs of a persistent tile launch: the resident count per SM times the SMs */
template <class KernelT>
unsigned tile_grid_size(KernelT kernel, size_t smem) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kTileThreads, smem) != cudaSuccess || per < 1)
        per = 1;
    return (unsigned)(sms * per);
}

template <class KernelT>
void tile_attr(KernelT kernel, size_t smem) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

} // namespace

void launch_tile_build(const Params &P, CellGrid &G, TileDev &T, int32_t *status, cudaStream_t s) {
    const unsigned g = 152 * 8;
    if (P.D == 2)
        k_tile_flags<2><<<g, 256, 0, s>>>(G, T, status);
    else
        k_tile_flags<3><<<g, 256, 0, s>>>(G, T, status);
    scan_exclusive<int32_t, int32_t>(T.flag, T.scan, G.table_size, G.scan_tmp, s, T.ntot);
    k_tile_list<<<g, 256, 0, s>>>(T);
}

void launch_tile_masks(const Params &P, double *const xs[3], const CellGrid &G, const Packed &K, const TileDev &T,
                       DevScalars *dsc, cudaStream_t s) {
    if (P.D == 2) {
        const size_t sm = tile_smem_bytes<2>(T.smax, kStageS);
        tile_attr(k_tile_masks<2>, sm);
        k_tile_masks<2><<<tile_grid_size(k_tile_masks<2>, sm), kTileThreads, sm, s>>>(P, G, T, K, xs[0], xs[1], xs[2],
                                                                                       dsc);
    } else {
        const size_t sm = tile_smem_bytes<3>(T.smax, kStageS);
        tile_attr(k_tile_masks<3>, sm);
        k_tile_masks<3><<<tile_grid_size(k_tile_masks<3>, sm), kTileThreads, sm, s>>>(P, G, T, K, xs[0], xs[1], xs[2],
                                                                                       dsc);
    }
}

void launch_tile_export(const Params &P, double *const xs[3], const CellGrid &G, const Packed &K, const TileDev &T,
                        int pass, int32_t *counts, const int64_t *off, int64_t *idx, double *d2, cudaStream_t s) {
    if (P.D == 2) {
        const size_t sm = tile_smem_bytes<2>(T.smax, kStageS);
        tile_attr(k_tile_export<2>, sm);
        k_tile_export<2><<<tile_grid_size(k_tile_export<2>, sm), kTileThreads, sm, s>>>(
            P, G, T, K, xs[0], xs[1], xs[2], pass, counts, off, idx, d2);
    } else {
        const size_t sm = tile_smem_bytes<3>(T.smax, kStageS);
        tile_attr(k_tile_export<3>, sm);
        k_tile_export<3><<<tile_grid_size(k_tile_export<3>, sm), kTileThreads, sm, s>>>(
            P, G, T, K, xs[0], xs[1], xs[2], pass, counts, off, idx, d2);
    }
}

} // namespace fjsph
