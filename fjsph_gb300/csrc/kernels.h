/*
 * kernels.h -- launchers of the device kernels, grouped by translation unit.  Each launcher
 * dispatches on Params::D (2 or 3) and enqueues on the given stream; none of them synchronises.
 */
#pragma once

#include <vector>

#include "closure.cuh"
#include "common.cuh"

namespace fjsph {

/* Packed FP32 split-precision inputs of the mixed form (see sweeps_mixed.cu). */
/* ---- mesh.cu: mesh-cell air source ----------------------------------------------------------- */
struct MeshDev {
    int64_t ncells;
    const double *verts;                        /* dim per vertex                              */
    const int64_t *face_off, *face_verts;       /* CSR vertices of every face                  */
    const int32_t *face_right;                  /* right cell, -1 inner / -2 outer boundary    */
    const int64_t *cell_off, *cell_faces;       /* CSR faces of every cell                     */
    const double *centre, *cvel, *cp, *crho;    /* dim per cell for centre and velocity        */
    const double *rad2;                         /* squared bounding-sphere radius per cell     */
    /* two uniform grids listing every cell in the buckets its box overlaps: g[0] the bounding
     * sphere's box (containment candidates), g[1] the box of the doubled sphere (the nearest
     * cell of a particle outside the mesh) */
    struct Grid {
        const int64_t *off, *cells;
        double lo[3], inv_h;
        int32_t dims[3];
    } g[2];
};
struct MeshHost {
    std::vector<double> rad2;
    struct Grid {
        std::vector<int64_t> off, cells;
        double lo[3], inv_h;
        int32_t dims[3];
    } g[2];
};
/* validates the mesh's index arrays and builds the bounding spheres and the bucket grid */
int mesh_build(const fjsph_mesh &m, MeshHost &h);
/* FindCell for the fluid slots; air[3 i + k] = the resulting cellV (the occlusion's air velocity);
 * list (capacity slots) and count are scratch for the active particles */
void launch_mesh_find(const Params &P, const DevState &W, const MeshDev &M, double *air, int32_t *list,
                      int32_t *count, cudaStream_t s);

/* ---- vlm.cu: vortex-lattice air source -------------------------------------------------------- */
struct VlmDev {
    int32_t np;           /* panels                                              */
    const double *ab;     /* [6 np] vortex ends A, B of every panel (FP64)        */
    const double *gamma;  /* [np]   circulations                                  */
    const float *abf;     /* [12 np] FP32: A high, A low, B high, B low           */
    const float *gammaf;
    double vinf[3];
    double max_vel;
};
/* panels (A, B, C: 9 doubles each) and circulations of a wing for the freestream vinf */
int vlm_build(const fjsph_vlm &v, const double *vinf, std::vector<double> &abc, std::vector<double> &gamma);
/* air[3 i + k] = the VLM velocity of the fluid particles that use it (FP32 sums when fp32) */
void launch_vlm_air(const Params &P, const DevState &W, const DevNbr &N, const VlmDev &V, double *air, bool fp32,
                    cudaStream_t s);
/* air[3 i + k] = v_inf[k] f(x_i) for the fluid slots, f the boundary-layer profile of
 * pl = {axis, wall, thickness, exponent} (FP32 power in the split-precision form) */
void launch_power_law_air(const Params &P, const DevState &W, const double *pl, double *air, bool fp32,
                          cudaStream_t s);
/* vel[3 i + k] at pos[3 i + k], i < n */
void launch_vlm_points(const VlmDev &V, int64_t n, const double *pos, double *vel, bool fp32, cudaStream_t s);

struct Packed {
    float4 *A, *C, *F, *G, *N, *T;
    float4 *O; /* occlusion statistics of the surface-curvature pass (learned-closure inputs 0-3) */
    float4 *L0, *L1, *L2; /* FP32 renormalisation matrix of the dSPH pre-step (row-major, 9 of 12) */
    /* The low parts of position and velocity (x - fl32(x), v - fl32(v)) as bf16 pairs
     * (x.x|x.y, x.z|v.x, v.y|v.z) and p / rho^2 whose two lowest mantissa bits carry kLoBound
     * (type FJSPH_BOUND) and kLoFluid (type above FJSPH_PISTON): with A and C, the neighbour
     * inputs of the pair sweeps. */
    float4 *Lo;
    float *R; /* rho - rho0 of the C record, dense: the dSPH pass's one use of C */
    int32_t *bits;
};

/* ---- update.cu: particle-set changes of update_data ---------------------------------------- */
struct BlockShift {
    int64_t v[kMaxBlocks]; /* added to the key of every slot of block b */
};
struct InsertOp {
    int32_t to_pipe, to_back; /* slots whose type changes (old BACK, new BACK)      */
    int32_t src, dst;         /* copied slot and new slot (dst < 0: no new particle) */
    int32_t block, pad;
    int64_t key, part_id;     /* reference index and id of the new particle          */
    double norm[3];           /* insertion normal of the block                       */
};
struct DeletePlanes {
    int32_t lost; /* also delete particles whose cellID is kMeshLost (mesh air source) */
    int32_t on[kMaxBlocks];
    double norm[kMaxBlocks][3];
    double c[kMaxBlocks];
};
void launch_inlet_cross(const DevState &W, int D, const int32_t *back, int64_t n_back, const double *norm, double c,
                        int32_t *flag, cudaStream_t s);
void launch_shift_keys(int64_t *key, const int32_t *blk, int64_t n, const BlockShift &sh, cudaStream_t s);
void launch_insert(const DevState &W, int D, const InsertOp *ops, int64_t nops, double dx, cudaStream_t s);
void launch_delete_flags(const Params &P, const DevState &W, const DeletePlanes &DP, int32_t *flag, int32_t *keep,
                         unsigned long long *count, cudaStream_t s);
/* phase 0: by_ref[key[s]] = flag[s]; phase 1 (after the scans): new_of_old and compacted keys */
void launch_compact_map(const int32_t *flag, const int64_t *key, int64_t n, int32_t *by_ref, const int32_t *keep_ex,
                        const int64_t *ref_ex_after_scan, int32_t *new_of_old, int64_t *key_out, int phase,
                        cudaStream_t s);
void launch_permute_key_blk(const int64_t *key, const int32_t *blk, int64_t *key2, int32_t *blk2,
                            const int32_t *new_of_old, int64_t n, cudaStream_t s);

/* ---- groups.cu: independent simulations in one context --------------------------------------- */
struct GroupDev {
    double *dt, *npd, *time, *cfl, *maxShift, *maxRho_pc, *logbase, *err;
    int32_t *n_stable, *n_unstable;
    int64_t *steps, *nfluid, *count;
};
struct GroupConst {
    double rho_rest, H, H_sq, mu, speed_sound, dt_min, dt_max, last_frame_time, frame_interval;
    double min_residual, rho_max_iter, cfl_min, cfl_max, cfl_step, subits_factor;
    int32_t max_subits, n_stable_limit, n_unstable_limit, ale;
};
void launch_group_fill(double *a, int64_t n, double v, cudaStream_t s);
/* out[g] += sum of vals over slots [i0, i1) of group g (out zeroed by the caller) */
void launch_group_sum(const int32_t *grp, const double *vals, int64_t i0, int64_t i1, double *out, cudaStream_t s);
void launch_group_sq_disp(const Params &P, const DevState &W, double *const ref[3], double *out, cudaStream_t s);
/* red[g * 8 + k]: maxf, maxAf, maxdrho, maxRhoi, minST, maxU, maxShift of group g */
void launch_group_timestep(const Params &P, const DevState &W, double *red, int32_t ng, cudaStream_t s);
void launch_group_dt(const GroupDev &G, const double *red, int32_t ng, const GroupConst &K, cudaStream_t s);
void launch_group_npd(double *npd, const double *sum, const int64_t *count, int32_t ng, cudaStream_t s);
void launch_group_err(const GroupDev &G, const double *sum, int32_t ng, int mode, cudaStream_t s);
void launch_group_adapt(const GroupDev &G, int32_t ng, const GroupConst &K, cudaStream_t s);

/* ---- mlp_train.cu ------------------------------------------------------------------------- */
namespace mlp {
/* FP32 parameters (host) -> device master copy and its BF16 forward / transposed copies */
int mlp_upload(const float *host_params, float *dparams, __nv_bfloat16 *dw, __nv_bfloat16 *dwt, cudaStream_t s);
int mlp_num_bf16_t();
} // namespace mlp

/* ---- neighbours.cu ------------------------------------------------------------------------ */
struct CellGrid {
    int64_t table_size;      /* power of two                                  */
    uint32_t *hash;          /* [cap]  bucket | x quarter << 30 of each slot   */
    float4 *frac;            /* [cap]  position inside the cell, cell edges   */
    uint32_t *hash2;         /* [cap]  re-ordering buffers of hash and frac   */
    float4 *frac2;
    int32_t *count;          /* [table_size + 1]                              */
    int32_t *start;          /* [table_size + 1] exclusive scan of count      */
    int32_t *sorted;         /* [cap]  slots ordered by bucket                */
    float4 *sorted_hi;       /* [cap]  (fl32(x), slot bits) in bucket order   */
    float4 *sorted_lo;       /* [cap]  fl32(x - hi) in bucket order           */
    uint32_t *qbin;          /* [table_size] quarter-cell index of the cells  */
    double *bbox;            /* [8]    lo[3], hi[3], band, spare (device)     */
    int64_t *grid;           /* [8]    nx, ny, nz, wrap flag, buckets in use  */
    int32_t *scan_tmp;       /* scan partials                                 */
    int64_t scan_tmp_len;
};

/* blocks of the bounding-box reduction; scan_tmp holds 12 int32 words of partials per block */
constexpr int kBboxBlocks = 1216;
void launch_bbox(const Params &P, const DevState &W, CellGrid &G, cudaStream_t s);
void launch_hash_and_count(const Params &P, const DevState &W, double *const xs[3], CellGrid &G, cudaStream_t s);
void launch_scan_i32(const int32_t *in, int32_t *out, int64_t n, int32_t *tmp, cudaStream_t s);
/* exclusive scan of the bucket counts over the buckets the grid uses (G.grid[4], on the device) */
void launch_scan_buckets(CellGrid &G, cudaStream_t s);
void launch_scan_i64(const int32_t *in, int64_t *out, int64_t n, int64_t *tmp, cudaStream_t s);
void launch_scatter_sort(const Params &P, CellGrid &G, const double *xs0, cudaStream_t s);
void launch_nbr_count(const Params &P, double *const xs[3], const CellGrid &G, int32_t *counts, cudaStream_t s);
/* Writes idx (FP64 form, CSR by off) or, when pair is given, (slot, FP32 squared distance) pairs
 * in the sliced-ELL order of DevNbr (slice offsets `slice`, counts per slot `counts`). */
void launch_nbr_fill(const Params &P, double *const xs[3], const CellGrid &G, const int64_t *off, int32_t *idx,
                     int2 *pair, const int64_t *slice, const int32_t *counts, int64_t cap, int32_t *status,
                     cudaStream_t s);
/* Single-pass split-precision lists with wcap entries per slot (multiple of kChunk): sets the
 * slice offsets, the per-slot counts, dsc->maxcnt / pairs and the overflow status bit. */
void launch_nbr_fill_fixed(const Params &P, double *const xs[3], const CellGrid &G, int2 *pair, int32_t *counts,
                           int64_t *slice, int32_t wcap, DevScalars *dsc, cudaStream_t s);
/* width[s] = kSlice x the largest count of slice s (slices of kSlice slots from slot 0). */
void launch_slice_width(const int32_t *counts, int64_t n, int32_t *width, cudaStream_t s);
/* Bucket-ordered hi/lo coordinates for the neighbour walk (after any re-ordering). */
void launch_sorted_pos(const Params &P, double *const xs[3], CellGrid &G, cudaStream_t s);
/* Re-ordering: new slot of every old slot, boundary group first, each group in bucket order. */
void launch_reorder_map(const Params &P, const CellGrid &G, int32_t *new_of_old, int32_t *tmp, int64_t tmp_len,
                        cudaStream_t s);

/* candidates per particle: at most 32 kMaskWords (the search reports more as an overflow) */
constexpr int kMaskWords = 16;
constexpr int kTileThreads = 128;
constexpr int32_t kStatusTileOverflow = 2; /* DevScalars::status bit */

/* The tile structure of one search (device arrays, sized by the bucket table). */
struct TileDev {
    int32_t *list;   /* occupied tiles (linear ids over the tile grid), in id order     */
    int32_t *count;  /* [1] number of occupied tiles                                      */
    int64_t *ntot;   /* [1] tiles of the grid (the scan length)                            */
    int32_t *flag;   /* [table] occupancy flag per tile, then its exclusive scan (scratch)  */
    int32_t *scan;   /* [table + 1]                                                        */
    uint32_t *mask;  /* word w of cell-sorted entry g at mask[w * stride + g]              */
    int64_t stride;
    int32_t smax;    /* staged particles per CTA that fit the launch's shared memory      */
};

/* Tiles of the split-precision sweeps (tiles.cuh): occupancy flags, the list of occupied tiles,
 * then the member masks of every particle; a wrapped bucket table or more than 32 kMaskWords
 * candidates of a particle raise kStatusTileOverflow in *status. */
void launch_tile_build(const Params &P, CellGrid &G, TileDev &T, int32_t *status, cudaStream_t s);
void launch_tile_masks(const Params &P, double *const xs[3], const CellGrid &G, const Packed &K, const TileDev &T,
                       DevScalars *dsc, cudaStream_t s);
/* pass 0: counts[slot] = members; pass 1: idx / d2 (FP64) of the members at off[slot] */
void launch_tile_export(const Params &P, double *const xs[3], const CellGrid &G, const Packed &K, const TileDev &T,
                        int pass, int32_t *counts, const int64_t *off, int64_t *idx, double *d2, cudaStream_t s);

/* residual of the split-precision form over the tiles (sweeps_mixed.cu) */
void launch_t_resid(const Params &P, const DevState &W, const CellGrid &G, const TileDev &T, const Packed &K,
                    const double *npd_dev, const Closure &C, cudaStream_t s);

/* ---- sweeps.cu ---------------------------------------------------------------------------- */
/* Per-particle quotients the FP64 pair sweeps gather from their neighbours instead of dividing per
 * pair: m / rho, p / rho^2, 1 / rho and the artificial viscosity's sound speed sqrt(B gamma / rho)
 * (one 32-byte sector per neighbour).  The FP64 sweep launchers that take Q (scratch of the particle
 * count) fill it first. */
struct __align__(32) ResidQuot {
    double vol, pr, inv_rho, cs;
};
void launch_dsph_prestep(const Params &P, const DevState &W, const DevNbr &N, double *npd_part, ResidQuot *Q,
                         cudaStream_t s);
void launch_npd_only(const Params &P, const DevState &W, const DevNbr &N, double *npd_part, cudaStream_t s);
void launch_aero_velocity(const Params &P, const DevState &W, const DevNbr &N, cudaStream_t s);
void launch_detect_surface(const Params &P, const DevState &W, const DevNbr &N, double *const nrm_tmp[3],
                           ResidQuot *Q, cudaStream_t s);
void launch_dissipation(const Params &P, const DevState &W, const DevNbr &N, ResidQuot *Q, cudaStream_t s);
void launch_particle_shift(const Params &P, const DevState &W, const DevNbr &N, ResidQuot *Q, cudaStream_t s);
/* kbits: the packed flags to keep current (null: the caller repacks) */
void launch_pipe_outlet(const Params &P, const DevState &W, int32_t *kbits, cudaStream_t s);
/* boundary passes over slots [0, nb) */
void launch_bound_velocity(const Params &P, const DevState &W, int nb_rule, cudaStream_t s);
void launch_no_slip(const Params &P, const DevState &W, const DevNbr &N, double *const vtmp[3], cudaStream_t s);
void launch_bound_pressure(const Params &P, const DevState &W, const DevNbr &N, cudaStream_t s);
void launch_bound_ghost(const Params &P, const DevState &W, const DevNbr &N, int32_t *near_inlet, cudaStream_t s);
void launch_bound_dbc(const Params &P, const DevState &W, cudaStream_t s);
/* residual (src/Resid.cpp:426) over fluid slots */
/* Q: scratch of the particle count, filled first */
void launch_resid(const Params &P, const DevState &W, const DevNbr &N, const double *npd_dev, ResidQuot *Q,
                  cudaStream_t s);

/* ---- sweeps_mixed.cu (FP32 split-precision form) ------------------------------------------ */
void launch_m_pack(const Params &P, const DevState &W, const Packed &K, int64_t i0, int64_t i1, int full,
                   cudaStream_t s);
void launch_m_npd(const Params &P, const DevNbr &N, const Packed &K, double *npd_part, cudaStream_t s);
void launch_m_dsph(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, double *npd_part,
                   cudaStream_t s);
/* with_dissipation: the dissipation terms (launch_m_dissipation) are computed in the same walk */
void launch_m_surface(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, bool with_dissipation,
                      cudaStream_t s);
void launch_m_dissipation(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, cudaStream_t s);
void launch_m_particle_shift(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, cudaStream_t s);
void launch_m_bound_pressure(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, cudaStream_t s);
void launch_m_bound_ghost(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, int32_t *near_inlet,
                          cudaStream_t s);
void launch_m_resid(const Params &P, const DevState &W, const DevNbr &N, const Packed &K, const double *npd_dev,
                    const Closure &C, cudaStream_t s);
/* dst[new_of_old[i]] = src[i] for a per-slot float4 array (entries mapped to -1 are dropped) */
void launch_m_permute_f4(const float4 *src, float4 *dst, const int32_t *new_of_old, int64_t n, cudaStream_t s);

/* ---- integrate.cu ------------------------------------------------------------------------- */
struct RKScratch {
    double *Sx[3], *Sv[3], *Sr; /* RK4 weighted sums                                  */
    double *xsnap[3];           /* positions before the last update (error norm)      */
    int32_t *near_inlet;        /* ghost boundary flag per slot                       */
    double *part;               /* reduction partials                                 */
    int64_t part_len;
};

/* Boundary density/pressure updates.  mode 0 = RK intermediate, 1 = RK final, 2 = Newmark-Beta. */
void launch_bound_rho_update(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S, int mode,
                             double sum_w, const double *dt_dev, double dt_scale, cudaStream_t s);
/* RK4 accumulator initialisation at Runge_Kutta4 entry (st_1 = W). */
void launch_rk_init_sums(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S, cudaStream_t s);
/* Fluid stage update: stage 1..3 intermediate (weight for the sums) or final. */
/* K (may be null): also write the split-precision inputs of every particle the update moves */
void launch_rk_stage_update(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S, int stage,
                            const double *dt_dev, double dt_scale, const Packed *K, cudaStream_t s);
void launch_rk_final_update(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S,
                            const double *dt_dev, const Packed *K, cudaStream_t s);
void launch_nb_update(const Params &P, const DevState &pn, const DevState &W, const double *dt_dev, cudaStream_t s);
/* Inlet buffer particles.  mode 0 = RK intermediate, 1 = RK final, 2 = NB. */
struct DevInlet {
    int32_t block, fixed_vel_or_dynamic;
    int64_t n_back, depth;
    int32_t *back;   /* slots */
    int32_t *buffer; /* slots, n_back * depth */
    double unorm[3];
};
void launch_inlet_buffers(const Params &P, const DevState &pn, const DevState &W, const RKScratch &S,
                          const DevInlet &I, int mode, const double *dt_dev, double dt_scale, const Packed *K,
                          cudaStream_t s);
/* Sum over fluid slots of |W.x - ref|^2, written to out[0]. */
void launch_sq_disp_sum(const Params &P, const DevState &W, double *const ref[3], RKScratch &S, double *out,
                        cudaStream_t s);
/* K: packed inputs to keep current for the particles the guard resets (null: the caller repacks) */
void launch_density_guard(const Params &P, const DevState &W, const Packed *K, cudaStream_t s);
/* Sum of an array over [0, n) into out[0], deterministic (two-pass). */
void launch_sum(const double *in, int64_t n, double *part, int64_t part_len, double *out, cudaStream_t s);
/* find_timestep reductions over fluid slots: out[0..6] = maxf, maxAf, maxdrho, maxRhoi, minST, maxU,
 * maxShift (the last one only if ALE). */
/* the seven find_timestep maxima from the reduced values (the norms as their squares, the
 * surface-tension bound as its square-root argument) */
void timestep_maxima(const double *red, double *r);
void launch_timestep_reduce(const Params &P, const DevState &W, RKScratch &S, double *out, cudaStream_t s);

/* ---- state.cu ------------------------------------------------------------------------------ */
/* Field lists of a state: every array that holds per-slot data. */
constexpr int kMaxF64Fields = 64;
constexpr int kMaxI64Fields = 4;
constexpr int kMaxI32Fields = 8;
struct FieldList {
    int n64 = 0, ni64 = 0, ni32 = 0;
    double *f64[kMaxF64Fields];
    int64_t *i64[kMaxI64Fields];
    int32_t *i32[kMaxI32Fields];
};
/* Per-state fields (excludes the shared key/blk arrays). */
FieldList state_fields(const DevState &S, int D);
/* dst[new_of_old[o]] = src[o] for every field, o in [0, n); entries with new_of_old < 0 are dropped. */
void launch_permute(const FieldList &src, const FieldList &dst, const int32_t *new_of_old, int64_t n, cudaStream_t s);
/* dst = src over [0, n) for every field. */
void launch_copy(const FieldList &src, const FieldList &dst, int64_t n, cudaStream_t s);
/* Host-layout field transfer through a device staging buffer (reference order, components
 * interleaved per particle): in = stage -> slot-order arrays, out = the reverse. */
struct FieldPtrs {
    void *p[9];
};
void launch_field_in(const void *stage, int comps, int elem, const int64_t *key, const FieldPtrs &dst, int64_t n,
                     cudaStream_t s);
void launch_field_out(void *stage, int comps, int elem, const int64_t *key, const FieldPtrs &src, int64_t n,
                      cudaStream_t s);
/* a[i] = new_of_old[a[i]] */
void launch_remap_i32(int32_t *a, int64_t n, const int32_t *new_of_old, cudaStream_t s);

} // namespace fjsph
