/*
 * tiles.cuh -- shared-memory tiles of the cell grid for the split-precision pair sweeps.
 *
 * The neighbour search sorts particles by cell (cells are the support radius R long along x and
 * R / kCellDiv across it; the bucket of a cell is its linear index x + nx (y + ny z) while the
 * grid fits the bucket table).  A tile is a block of TX x TY x TZ cells; its halo adds the cells
 * any member of a tile particle can lie in (one cell along x, kCellDiv across).  A CTA takes one
 * occupied tile at a time: it copies the inputs of every halo particle into shared memory (each
 * halo row of cells is one contiguous range of the cell-sorted order), then every lane walks one
 * tile particle's members out of shared memory instead of gathering them through L1/L2.
 *
 * Membership is decided once per search (the reference's FP64 test, d2 < sr, as the list search
 * decides it) and kept as a bit mask per particle over its candidate sequence: the 3 x
 * (2 kCellDiv + 1)^(D-1) stencil cells visited row by row (dz, then dy), each row's three cells
 * in staged order.  A mask costs kMaskWords words per particle instead of 8 bytes per pair.
 *
 * Staged records of the sweeps (48 bytes per halo particle), in the tile's own frame:
 *   P = (x - x0, m / rho)   V = (v - v0, rho - rho0)   T = (search-time position in its cell, p / rho^2 | flags)
 * x0 and v0 are the position and velocity of one particle of the tile, both as FP32 high and low
 * parts; x - x0 = (xhi - x0hi) + (xlo - x0lo) is accurate to FP32 rounding of the offset itself
 * (a few 1e-11 m on a 50 um jet), so separations keep the accuracy of the split-precision inputs
 * whatever the coordinates' magnitude.  The search-time squared distance of a member pair is
 * the cell offset plus the difference of the in-cell positions, scaled by the cell edges.
 */
#pragma once

#include "kernels.h"

namespace fjsph {

template <int D>
struct TileShape;
template <>
struct TileShape<3> {
    static constexpr int TX = 2, TY = 4, TZ = 4, RY = kCellDiv, RZ = kCellDiv;
};
template <>
struct TileShape<2> {
    static constexpr int TX = 4, TY = 8, TZ = 1, RY = kCellDiv, RZ = 0;
};
template <int D>
struct Tile {
    using S = TileShape<D>;
    static constexpr int TX = S::TX, TY = S::TY, TZ = S::TZ, RY = S::RY, RZ = S::RZ;
    static constexpr int HX = TX + 2, HY = TY + 2 * RY, HZ = TZ + 2 * RZ;
    static constexpr int NCELL = HX * HY * HZ, NROW = HY * HZ;
    static constexpr int SY = 2 * RY + 1, NSTENCIL = (2 * RY + 1) * (2 * RZ + 1); /* stencil rows */
};

/* which particles of a tile a sweep computes */
enum TileOwn { kOwnAll = 0, kOwnFluid = 1, kOwnBound = 2 };

/* what a sweep stages per halo particle */
enum TileStage { kStageS = 1, kStageRel = 2 };

/* Shared memory of one CTA: cell table, row offsets, frame, own list, staged records. */
struct TileSmem {
    int *cs;      /* [NCELL + 1] staged start of every halo cell                          */
    int *goff;    /* [NROW] cell-sorted index g = e + goff[row] of staged entry e         */
    int *head;    /* [4] own count, staged count over smax, staged count, own list full  */
    float *frame; /* [12] x0 high, x0 low, v0 high, v0 low (3 each)                       */
    int *own;     /* [smax] own particles: staged index | halo cell << 16                 */
    float4 *S;    /* kStageS:  (in-cell position at search, slot)                         */
    float4 *P, *V, *T; /* kStageRel records                                              */
    int smax;
    __device__ __forceinline__ int nown() const { return head[0]; }
    __device__ __forceinline__ bool over() const { return head[1] != 0; }
};

template <int D>
__host__ __device__ constexpr size_t tile_head_bytes() {
    return (sizeof(int) * (size_t)(Tile<D>::NCELL + 1 + Tile<D>::NROW + 4) + sizeof(float) * 12 + 15) & ~(size_t)15;
}
template <int D>
__host__ __device__ constexpr size_t tile_smem_bytes(int smax, int stage) {
    return tile_head_bytes<D>() + sizeof(int) * (size_t)smax +
           sizeof(float4) * (size_t)smax * ((stage & kStageS) ? 1 : 0) +
           sizeof(float4) * (size_t)smax * ((stage & kStageRel) ? 3 : 0);
}

template <int D>
__device__ __forceinline__ TileSmem tile_smem(unsigned char *base, int smax, int stage) {
    using T = Tile<D>;
    TileSmem t;
    int *p = reinterpret_cast<int *>(base);
    t.cs = p;
    t.goff = p + T::NCELL + 1;
    t.head = t.goff + T::NROW;
    t.frame = reinterpret_cast<float *>(t.head + 4);
    size_t off = tile_head_bytes<D>();
    t.own = reinterpret_cast<int *>(base + off);
    off += sizeof(int) * (size_t)smax;
    float4 *f = reinterpret_cast<float4 *>(base + off);
    t.S = t.P = t.V = t.T = nullptr;
    if (stage & kStageS) {
        t.S = f;
        f += smax;
    }
    if (stage & kStageRel) {
        t.P = f;
        t.V = f + smax;
        t.T = f + 2 * smax;
    }
    t.smax = smax;
    return t;
}

/* Tile coordinates of a linear tile id and the grid in cells. */
struct TileGrid {
    int64_t nc[3];
    int64_t nt[3];
};
template <int D>
__device__ __forceinline__ TileGrid tile_grid(const CellGrid &G) {
    using T = Tile<D>;
    TileGrid g;
    g.nc[0] = G.grid[0];
    g.nc[1] = G.grid[1];
    g.nc[2] = G.grid[2];
    g.nt[0] = (g.nc[0] + T::TX - 1) / T::TX;
    g.nt[1] = (g.nc[1] + T::TY - 1) / T::TY;
    g.nt[2] = (g.nc[2] + T::TZ - 1) / T::TZ;
    return g;
}

/* The low parts of x and v from the packed Lo record (bf16 pairs). */
__device__ __forceinline__ void unpack_lo(const float4 q, float *xl, float *vl) {
    const uint32_t a = __float_as_uint(q.x), b = __float_as_uint(q.y), c = __float_as_uint(q.z);
    xl[0] = __uint_as_float(a << 16);
    xl[1] = __uint_as_float(a & 0xFFFF0000u);
    xl[2] = __uint_as_float(b << 16);
    vl[0] = __uint_as_float(b & 0xFFFF0000u);
    vl[1] = __uint_as_float(c << 16);
    vl[2] = __uint_as_float(c & 0xFFFF0000u);
}

/* Block-wide exclusive scan of a[0 .. n) in place, a[n] = total (blockDim.x <= 128: warp totals
 * in warp_tot[0 .. 3]).  All threads call it. */
__device__ __forceinline__ void block_scan_excl(int *a, int n, int *warp_tot) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int per = (n + blockDim.x - 1) / blockDim.x; /* contiguous items per thread */
    const int b = threadIdx.x * per;
    int s = 0;
    for (int k = 0; k < per; ++k)
        if (b + k < n) s += a[b + k];
    int incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int w = 0; w < nw; ++w) {
            const int t = warp_tot[w];
            warp_tot[w] = run;
            run += t;
        }
        a[n] = run;
    }
    __syncthreads();
    int run = warp_tot[wid] + incl - s;
    for (int k = 0; k < per; ++k)
        if (b + k < n) {
            const int v = a[b + k];
            a[b + k] = run;
            run += v;
        }
    __syncthreads();
}

/* Set up one tile: halo cell table, row offsets, frame, staged records (when they fit in smax)
 * and the list of own particles of kind `own_kind`.  Ends with a barrier. */
template <int D>
__device__ __forceinline__ void tile_setup(const Params &P, const CellGrid &G, const Packed &K, const TileGrid &tg,
                                           int32_t tile, int stage, int own_kind, TileSmem &ts) {
    using T = Tile<D>;
    const int64_t tx = tile % tg.nt[0], ty = (tile / tg.nt[0]) % tg.nt[1], tz = tile / (tg.nt[0] * tg.nt[1]);
    const int64_t X0 = tx * T::TX - 1, Y0 = ty * T::TY - T::RY, Z0 = tz * T::TZ - T::RZ;
    const int hx_first = X0 < 0 ? (int)(-X0) : 0; /* first halo x inside the grid */
    /* cell counts, and each row's first cell-sorted index */
    for (int c = threadIdx.x; c < T::NCELL; c += blockDim.x) {
        const int hx = c % T::HX, hy = (c / T::HX) % T::HY, hz = c / (T::HX * T::HY);
        const int64_t cx = X0 + hx, cy = Y0 + hy, cz = Z0 + hz;
        int cnt = 0;
        if (cx >= 0 && cx < tg.nc[0] && cy >= 0 && cy < tg.nc[1] && cz >= 0 && cz < tg.nc[2]) {
            const int64_t lin = cx + tg.nc[0] * (cy + tg.nc[1] * cz);
            const int32_t s0 = G.start[lin];
            cnt = G.start[lin + 1] - s0;
            if (hx == hx_first) ts.goff[c / T::HX] = s0;
        } else if (hx == hx_first) {
            ts.goff[c / T::HX] = 0;
        }
        ts.cs[c] = cnt;
    }
    __syncthreads();
    block_scan_excl(ts.cs, T::NCELL, ts.head);
    const int stot = ts.cs[T::NCELL];
    for (int r = threadIdx.x; r < T::NROW; r += blockDim.x) ts.goff[r] -= ts.cs[r * T::HX + hx_first];
    if (threadIdx.x == 0) {
        ts.head[0] = 0;
        ts.head[1] = stot > ts.smax ? 1 : 0;
        ts.head[2] = stot;
        ts.head[3] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0 && (stage & kStageRel)) {
        /* frame: the first particle of the first occupied own cell (the tile is occupied) */
        int e = 0, row = 0;
        for (int orow = 0; orow < T::TY * T::TZ; ++orow) {
            const int r = (T::RZ + orow / T::TY) * T::HY + (T::RY + orow % T::TY);
            const int c0 = r * T::HX + 1;
            if (ts.cs[c0 + T::TX] > ts.cs[c0]) {
                e = ts.cs[c0];
                row = r;
                break;
            }
        }
        const int32_t slot = G.sorted[e + ts.goff[row]];
        const float4 A = K.A[slot], C = K.C[slot], Q = K.Lo[slot];
        float xl[3], vl[3];
        unpack_lo(Q, xl, vl);
        ts.frame[0] = A.x;
        ts.frame[1] = A.y;
        ts.frame[2] = A.z;
        ts.frame[3] = xl[0];
        ts.frame[4] = xl[1];
        ts.frame[5] = xl[2];
        ts.frame[6] = C.x;
        ts.frame[7] = C.y;
        ts.frame[8] = C.z;
        ts.frame[9] = vl[0];
        ts.frame[10] = vl[1];
        ts.frame[11] = vl[2];
    }
    __syncthreads();
    const bool over = ts.head[1] != 0;
    if (!over) {
        float fr[12];
        if (stage & kStageRel)
#pragma unroll
            for (int k = 0; k < 12; ++k) fr[k] = ts.frame[k];
        /* staged entry e lies in halo row r with cs[r HX] <= e < cs[(r + 1) HX] */
        for (int e = threadIdx.x; e < stot; e += blockDim.x) {
            int lo = 0, hi = T::NROW; /* largest r with cs[r HX] <= e */
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (ts.cs[mid * T::HX] <= e)
                    lo = mid;
                else
                    hi = mid;
            }
            const int32_t slot = G.sorted[e + ts.goff[lo]];
            const float4 f = G.frac[slot];
            if (stage & kStageS) ts.S[e] = make_float4(f.x, f.y, f.z, __int_as_float(slot));
            if (stage & kStageRel) {
                const float4 A = K.A[slot], C = K.C[slot], Q = K.Lo[slot];
                float xl[3], vl[3];
                unpack_lo(Q, xl, vl);
                ts.P[e] = make_float4((A.x - fr[0]) + (xl[0] - fr[3]), (A.y - fr[1]) + (xl[1] - fr[4]),
                                      D == 3 ? (A.z - fr[2]) + (xl[2] - fr[5]) : 0.f, A.w);
                ts.V[e] = make_float4((C.x - fr[6]) + (vl[0] - fr[9]), (C.y - fr[7]) + (vl[1] - fr[10]),
                                      D == 3 ? (C.z - fr[8]) + (vl[2] - fr[11]) : 0.f, C.w);
                ts.T[e] = make_float4(f.x, f.y, f.z, Q.w);
            }
        }
    }
    /* own particles: the TX cells of each own row, filtered by kind */
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int orow = wid; orow < T::TY * T::TZ; orow += nw) {
        const int r = (T::RZ + orow / T::TY) * T::HY + (T::RY + orow % T::TY);
        const int c0 = r * T::HX + 1;
        const int e0 = ts.cs[c0], e1 = ts.cs[c0 + T::TX];
        for (int b = e0; b < e1; b += 32) {
            const int e = b + lane;
            bool keep = false;
            int hc = c0;
            if (e < e1) {
                const int32_t slot = G.sorted[e + ts.goff[r]];
                keep = own_kind == kOwnAll || (own_kind == kOwnFluid ? slot >= P.nb : slot < P.nb);
#pragma unroll
                for (int q = 1; q < T::TX; ++q) hc += e >= ts.cs[c0 + q] ? 1 : 0;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            int base = 0;
            if (lane == 0 && bal) base = atomicAdd(&ts.head[0], __popc(bal));
            base = __shfl_sync(0xffffffffu, base, 0);
            const int slot_k = base + __popc(bal & ((1u << lane) - 1u));
            if (keep) {
                if (slot_k < ts.smax && e < 0x10000 && hc < 0x8000)
                    ts.own[slot_k] = e | (hc << 16);
                else
                    ts.head[3] = 1; /* more own particles than the list holds: reported, not computed */
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && ts.head[0] > ts.smax) ts.head[0] = ts.smax;
    __syncthreads();
}

/* One own particle of a tile: staged index, halo cell, cell-sorted index. */
struct TileOwnRef {
    int e, hc, hx, hy, hz;
    int64_t g;
};
template <int D>
__device__ __forceinline__ TileOwnRef tile_own(const TileSmem &ts, int k) {
    using T = Tile<D>;
    TileOwnRef o;
    const int w = ts.own[k];
    o.e = w & 0xFFFF;
    o.hc = w >> 16;
    o.hx = o.hc % T::HX;
    o.hy = (o.hc / T::HX) % T::HY;
    o.hz = o.hc / (T::HX * T::HY);
    o.g = (int64_t)o.e + ts.goff[o.hc / T::HX];
    return o;
}

/* A member or candidate of an own particle: staged index, halo row, cell offset. */
struct TileNbr {
    int e, row;
    int dc[3];
};

/* Walks an own particle's stencil row by row.  next_member() returns its members one per call
 * (from the mask), next_cand() every candidate; a sweep loops `while (cur.next_member(n))`, so
 * the lanes of a warp run the pair arithmetic together whatever the rows hold. */
template <int D>
struct TileCursor {
    using T = Tile<D>;
    const int *cs;
    const uint32_t *mask;
    int64_t stride, g;
    int hx, hy, hz;
    int r;          /* next stencil row to open            */
    int row, dy, dz;
    int e0, cA, cB; /* next staged index of the row, x-cell boundaries */
    int left;       /* candidates of the row not taken yet */
    int base;       /* staged index of bit 0 of bits       */
    uint32_t bits;
    int pos, wi;
    uint32_t word;

    __device__ __forceinline__ void init(const TileSmem &ts, const TileOwnRef &o, const uint32_t *mask_,
                                         int64_t stride_) {
        cs = ts.cs;
        mask = mask_;
        stride = stride_;
        g = o.g;
        hx = o.hx;
        hy = o.hy;
        hz = o.hz;
        r = 0;
        left = 0;
        bits = 0u;
        pos = 0;
        wi = 0;
        word = mask ? mask[g] : 0u;
        row = dy = dz = e0 = cA = cB = base = 0;
    }
    /* opens the next stencil row; false when none is left */
    __device__ __forceinline__ bool open_row() {
        if (r == T::NSTENCIL) return false;
        dz = r / T::SY - T::RZ;
        dy = r % T::SY - T::RY;
        ++r;
        row = (hz + dz) * T::HY + (hy + dy);
        const int c0 = row * T::HX + hx - 1;
        e0 = cs[c0];
        cA = cs[c0 + 1];
        cB = cs[c0 + 2];
        left = cs[c0 + 3] - e0;
        return true;
    }
    __device__ __forceinline__ void fill(TileNbr &n, int e) const {
        n.e = e;
        n.row = row;
        n.dc[0] = (e >= cA ? 1 : 0) + (e >= cB ? 1 : 0) - 1;
        n.dc[1] = dy;
        n.dc[2] = dz;
    }
    __device__ __forceinline__ bool next_member(TileNbr &n) {
        while (bits == 0u) {
            if (left == 0) {
                if (!open_row()) return false;
                continue;
            }
            const int off = pos & 31;
            const int take = left < 32 - off ? left : 32 - off;
            bits = word >> off;
            if (take < 32) bits &= (1u << take) - 1u;
            base = e0;
            e0 += take;
            left -= take;
            pos += take;
            if ((pos & 31) == 0) {
                ++wi;
                word = wi < kMaskWords ? mask[wi * stride + g] : 0u;
            }
        }
        const int b = __ffs(bits) - 1;
        bits &= bits - 1u;
        fill(n, base + b);
        return true;
    }
    __device__ __forceinline__ bool next_cand(TileNbr &n) {
        while (left == 0)
            if (!open_row()) return false;
        fill(n, e0);
        ++e0;
        --left;
        return true;
    }
};

/* Members of the particle at cell-sorted index g (the popcount of its mask). */
__device__ __forceinline__ int tile_member_count(const uint32_t *mask, int64_t stride, int64_t g) {
    int n = 0;
#pragma unroll
    for (int w = 0; w < kMaskWords; ++w) n += __popc(mask[w * stride + g]);
    return n;
}

/* Search-time squared distance of a pair from the in-cell positions at search (FP32): the
 * separation in cells is the cell offset plus (t_j - t_i), scaled by the cell edges. */
template <int D>
__device__ __forceinline__ float tile_r2(const float4 &Ti, const float4 &Tj, const TileNbr &n, const float *edge) {
    const float ax = ((float)n.dc[0] + (Tj.x - Ti.x)) * edge[0];
    const float ay = ((float)n.dc[1] + (Tj.y - Ti.y)) * edge[1];
    float r2 = ax * ax + ay * ay;
    if (D == 3) {
        const float az = ((float)n.dc[2] + (Tj.z - Ti.z)) * edge[2];
        r2 += az * az;
    }
    return r2;
}

/* Slot of staged entry e of halo row `row`. */
__device__ __forceinline__ int32_t tile_slot(const CellGrid &G, const TileSmem &ts, int e, int row) {
    return G.sorted[e + ts.goff[row]];
}

/* kStageS record of staged entry e: shared memory, or (tile over smax) through the sort. */
__device__ __forceinline__ float4 tile_ld_s(const TileSmem &ts, const CellGrid &G, int e, int row, bool over) {
    if (!over) return ts.S[e];
    const int32_t slot = tile_slot(G, ts, e, row);
    const float4 f = G.frac[slot];
    return make_float4(f.x, f.y, f.z, __int_as_float(slot));
}

/* kStageRel records of staged entry e (shared memory, or computed from the packed arrays). */
template <int D>
__device__ __forceinline__ void tile_ld_rel(const TileSmem &ts, const CellGrid &G, const Packed &K, int e, int row,
                                            bool over, float4 &Pr, float4 &Vr, float4 &Tr) {
    if (!over) {
        Pr = ts.P[e];
        Vr = ts.V[e];
        Tr = ts.T[e];
        return;
    }
    const int32_t slot = tile_slot(G, ts, e, row);
    const float4 A = K.A[slot], C = K.C[slot], Q = K.Lo[slot], f = G.frac[slot];
    float xl[3], vl[3];
    unpack_lo(Q, xl, vl);
    const float *fr = ts.frame;
    Pr = make_float4((A.x - fr[0]) + (xl[0] - fr[3]), (A.y - fr[1]) + (xl[1] - fr[4]),
                     D == 3 ? (A.z - fr[2]) + (xl[2] - fr[5]) : 0.f, A.w);
    Vr = make_float4((C.x - fr[6]) + (vl[0] - fr[9]), (C.y - fr[7]) + (vl[1] - fr[10]),
                     D == 3 ? (C.z - fr[8]) + (vl[2] - fr[11]) : 0.f, C.w);
    Tr = make_float4(f.x, f.y, f.z, Q.w);
}

} // namespace fjsph
