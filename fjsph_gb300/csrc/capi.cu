/*
 * capi.cu -- the C ABI of the GB300 WCSPH hot path: device context, state hand-over, and the
 * host-side sequencing of the kernels that replaces Integrator (src/Integration.cpp) and the free
 * functions of src/Neighbours.cpp, src/Shifting.cpp, src/Geometry.cpp, src/Resid.cpp,
 * src/Runge_Kutta.cpp and src/Newmark_Beta.cpp.
 *
 * Within one step nothing returns to the host except the scalars the reference's control flow
 * branches on: the time step (find_timestep), the neighbour-list size (to size the CSR storage)
 * and, for Newmark-Beta, the residual of each sub-iteration.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "kernels.h"

using namespace fjsph;

#define CU(call)                                                                                              \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess) {                                                                              \
            std::fprintf(stderr, "fjsph: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            return FJSPH_E_CUDA;                                                                              \
        }                                                                                                     \
    } while (0)

#define TRY(call)                           \
    do {                                    \
        int r_ = (call);                    \
        if (r_ != FJSPH_OK) return r_;      \
    } while (0)

namespace {

struct HostInlet {
    int32_t block = -1, fixed_vel_or_dynamic = 0;
    int64_t n_back = 0, depth = 0;
    std::vector<int64_t> back_ref, buffer_ref; /* reference indices as given */
    int32_t *d_back = nullptr, *d_buffer = nullptr;
    double unorm[3] = {0, 0, 0};
};

} // namespace

/* Pass profiler: pairs of events around each timed section, resolved lazily. */
enum Pass {
    PASS_SEARCH = 0,
    PASS_REORDER,
    PASS_PRESTEP,
    PASS_SURFACE,
    PASS_DISSIPATION,
    PASS_SHIFT,
    PASS_BOUNDARY,
    PASS_RESID,
    PASS_UPDATE,
    PASS_REDUCE,
    PASS_COPY,
    PASS_TRANSFER,
    PASS_AIR,
    PASS_COUNT
};
static_assert(PASS_COUNT == FJSPH_NPASS, "pass table");
const char *kPassNames[PASS_COUNT] = {"neighbour_search", "reorder", "dsph_prestep", "detect_surface",
                                      "dissipation", "particle_shift", "boundary", "residual",
                                      "stage_update", "reductions", "state_copy", "host_transfer",
                                      "air_source"};

struct Profiler {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<std::pair<int, size_t>> marks; /* pass, index of start event (end = +1) */
    double ms[PASS_COUNT] = {};
    int64_t count[PASS_COUNT] = {};
};

struct fjsph_ctx {
    fjsph_settings s{};
    int D = 3;
    int64_t cap = 0, n = 0, nb = 0;
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;

    DevState st[3]{};
    int ipn = 0, iW = 1, isp = 2;
    int64_t *key = nullptr; /* reference index of each slot (shared by pn and W) */
    int32_t *blk = nullptr; /* block of each slot */

    double *xs[3] = {nullptr, nullptr, nullptr};
    CellGrid G{};
    int32_t *nbr_counts = nullptr;
    int64_t *nbr_off = nullptr;
    int32_t *nbr_idx = nullptr;
    int2 *nbr_pair = nullptr; /* split-precision form: (slot, r^2) per pair, sliced-ELL */
    int32_t *slice_w = nullptr;   /* entries per slice of kSlice slots                    */
    int64_t *slice_off = nullptr; /* first entry of each slice (exclusive scan of slice_w) */
    int64_t nbr_cap = 0, n_pairs = 0, nbr_storage = 0;
    int32_t wcap = 0;    /* split-precision single-pass lists: entries per slot (0: count first) */
    int32_t maxcnt = 0;  /* largest neighbour count of the last search                         */
    bool nbr_valid = false;
    int64_t *scan_tmp64 = nullptr;
    int64_t scan_tmp64_len = 0;
    int32_t *new_of_old = nullptr, *reorder_tmp = nullptr;
    int64_t reorder_tmp_len = 0;
    int64_t searches = 0;
    bool reorder_pending = true;
    int64_t table_want = 0;

    RKScratch S{};
    double *nrm_tmp[3] = {nullptr, nullptr, nullptr};
    double *vtmp[3] = {nullptr, nullptr, nullptr};
    double *npd_part = nullptr;
    double *stage = nullptr;   /* host-transfer staging, capacity * 9 doubles */
    double *stage2 = nullptr;  /* second staging buffer: field f + 1 moves while field f is gathered */
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t st_copied[2] = {nullptr, nullptr}, st_used[2] = {nullptr, nullptr};
    /* fjsph_step_host: input fields in flight on the copy stream, in four groups by their first
     * reader (in_grp: view_ptrs index, offset in in_stage in doubles, host array, bytes), each
     * applied by apply_in just before that reader */
    struct LateField {
        int f;
        int64_t off;
        const void *host;
        size_t bytes;
        int ev; /* input fields: index of the landing event in in_ev */
    };
    std::vector<LateField> in_grp[4];
    std::vector<cudaEvent_t> in_ev; /* one per input field: its host copy has landed */
    /* the groups are placed into pnp1 and pn on place_stream as they land (in_placed); the
     * compute stream waits for a group where it first reads it (in_wait: not waited for yet) */
    cudaStream_t place_stream = nullptr;
    cudaEvent_t place_after = nullptr; /* the compute stream's work before the placement */
    cudaEvent_t in_placed[4] = {nullptr, nullptr, nullptr, nullptr};
    bool in_wait[4] = {false, false, false, false};
    double *in_stage = nullptr;
    int64_t in_cap = 0;
    /* the scan of the uploaded ids, joined before update_data needs the next id */
    std::thread id_scan;
    int64_t id_scan_next = 0;
    /* fjsph_step_host: fields final after the second search's pre-passes, copied out while the
     * remaining stages run (offset in out_stage, host array, bytes); out_sent: the copies went
     * out for out_n particles */
    std::vector<LateField> early_out, final_out, last_out; /* after the pre-passes; after the last
                                                              * residual; after update_data */
    bool out_sent = false, final_sent = false, last_sent = false;
    int64_t out_ins0 = 0, out_del0 = 0; /* insertions and deletions before the step */
    int64_t out_n = 0;
    double *out_stage = nullptr;
    int64_t out_cap = 0;
    cudaEvent_t out_ready = nullptr;
    DevScalars *dsc = nullptr; /* device */
    DevScalars *hsc = nullptr; /* pinned host mirror */

    std::vector<fjsph_block> blocks;
    int64_t n_bound_blocks = 0;
    std::vector<HostInlet> inlets;

    bool pn_equals_W = false;
    /* Integrator members (src/Integration.h:52-67) */
    double safe_dt = 0, maxf = kEps, maxAf = kEps, maxRho_pc = kEps, maxRhoi = kEps, maxdrho = kEps;
    double minST = 9999999.0, maxU = kEps, maxShift = kEps;
    uint32_t iteration = 0;
    int64_t launches = 0;
    Profiler prof;
    cudaEvent_t user_ev[16] = {};
    /* FP32 split-precision form */
    Packed K{};
    bool packed_alloc = false;
    bool dirty_full = true, dirty_all = true, dirty_bound = true;
    /* learned aerodynamic closure */
    float *mlp_params = nullptr;
    __nv_bfloat16 *mlp_w = nullptr, *mlp_wt = nullptr;
    bool mlp_ready = false, occ_valid = false, closure_fallback = false, judge_pending = false;
    double judge_tol = 0.05;
    double *judge_dev = nullptr; /* [3] */
    double *judge_host = nullptr; /* pinned [3] */
    int64_t judged = 0, judged_particles = 0, closure_steps = 0;
    double last_rel_rms = 0.0, max_rel_rms = 0.0;
    int32_t arm = 0;             /* FJSPH_CLOSURE_ARM_* for the next residual */
    float *log_X = nullptr, *log_T = nullptr;
    unsigned long long *log_count = nullptr;
    int64_t log_cap = 0;
    int32_t log_every = 1;
    /* update_data: insertion / deletion */
    int32_t *upd_i32 = nullptr;             /* 4 * capacity + 64 scratch                 */
    unsigned long long *upd_cnt = nullptr;  /* deletions per block                       */
    int64_t part_id_next = 0, inserted = 0, deleted = 0;
    /* independent simulations sharing the context (groups) */
    int32_t ngrp = 0;
    int32_t *grp = nullptr;          /* group of every slot (permuted with the slots) */
    std::vector<int64_t> grp_first;  /* reference-index boundaries, ngrp + 1          */
    double *g_vinf = nullptr;
    GroupDev gs{};
    double *g_red = nullptr, *g_sum = nullptr;
    bool graph_mode = false;         /* steps enqueue without host round trips        */
    int32_t tune[3] = {128, 128, 4}; /* sweep block size, residual block size, list rows ahead */
    cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
    int64_t graph_launches[4] = {0, 0, 0, 0};
    int64_t graph_uses = 0;
    /* vortex-lattice air source */
    std::vector<double> vlm_abc, vlm_gamma; /* host copies: A, B, C per panel; circulations */
    double *vlm_ab = nullptr, *vlm_g = nullptr;
    float *vlm_abf = nullptr, *vlm_gf = nullptr;
    VlmDev vlm{};
    double *air_v = nullptr; /* 3 per slot */
    /* analytic boundary-layer air field (FJSPH_POWER_LAW): axis, wall, thickness, exponent */
    double power_law[4] = {2.0, 0.0, 1.0, 1.0 / 7.0};
    bool power_law_ready = false;
    /* shared-memory tiles of the split-precision sweeps (tiles.cuh) */
    TileDev T{};
    int32_t pair_mode = FJSPH_PAIRS_LISTS; /* FJSPH_PAIRS_*                               */
    int32_t sweep_order = FJSPH_ORDER_GRID; /* FJSPH_ORDER_*                              */
    int32_t *region_next = nullptr;         /* kMaxRegions chunk counters of the SM order */
    ResidQuot *resid_q = nullptr;           /* FP64 residual: per-particle quotients      */
    bool tiles_valid = false;              /* the last search built the tile masks        */
    int64_t tiles_table = 0;               /* bucket table size the tile arrays fit       */
    /* mesh-cell air source */
    MeshDev mesh{};
    bool mesh_ready = false;
    int32_t *mesh_list = nullptr, *mesh_count = nullptr; /* active particles of FindCell */
    std::vector<void *> mesh_allocs;
};

namespace {

DevState &PN(fjsph_ctx *c) { return c->st[c->ipn]; }
DevState &WS(fjsph_ctx *c) { return c->st[c->iW]; }

template <typename T>
int dalloc(fjsph_ctx *c, T **p, int64_t count) {
    *p = nullptr;
    if (count <= 0) count = 1;
    void *q = nullptr;
    CU(cudaMalloc(&q, sizeof(T) * (size_t)count));
    c->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return FJSPH_OK;
}

int alloc_state(fjsph_ctx *c, DevState &S) {
    const int D = c->D;
    const int64_t cap = c->cap;
    std::memset(&S, 0, sizeof(S));
    auto vec = [&](double **a) -> int {
        for (int k = 0; k < D; ++k) TRY(dalloc(c, &a[k], cap));
        return FJSPH_OK;
    };
    TRY(vec(S.x));
    TRY(vec(S.v));
    TRY(vec(S.acc));
    TRY(vec(S.Af));
    TRY(vec(S.aVisc));
    TRY(vec(S.cellV));
    TRY(vec(S.gradRho));
    TRY(vec(S.norm));
    TRY(vec(S.vPert));
    for (int k = 0; k < D * D; ++k) TRY(dalloc(c, &S.L[k], cap));
    double **sc[] = {&S.Rrho, &S.rho,    &S.p,       &S.m,       &S.curve,  &S.norm_curve, &S.woccl,  &S.pDist,
                     &S.deltaD, &S.cellP, &S.cellRho, &S.colourG, &S.colour, &S.lam,        &S.lam_nb, &S.kernsum};
    for (double **a : sc) TRY(dalloc(c, a, cap));
    TRY(dalloc(c, &S.part_id, cap));
    TRY(dalloc(c, &S.cellID, cap));
    TRY(dalloc(c, &S.b, cap));
    TRY(dalloc(c, &S.surf, cap));
    TRY(dalloc(c, &S.surfzone, cap));
    S.key = c->key;
    S.blk = c->blk;
    return FJSPH_OK;
}

int64_t next_pow2(int64_t v) {
    int64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

template <typename T>
int dfree(fjsph_ctx *c, T *&p) {
    if (p) {
        CU(cudaFree(p));
        c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), (void *)p), c->allocs.end());
        p = nullptr;
    }
    return FJSPH_OK;
}

/* Bucket table of the cell list: while the grid over the particles' bounding box has no more
 * cells than buckets, the hash is the identity and rows of cells are contiguous. */
constexpr int64_t kMinTable = (int64_t)1 << 22;
constexpr int64_t kMaxTable = (int64_t)1 << 26;

int graph_release(fjsph_ctx *c);

int alloc_table(fjsph_ctx *c, int64_t size) {
    TRY(graph_release(c)); /* captured launches hold the old arrays */
    if (size > ((int64_t)1 << 30)) return FJSPH_E_CAPACITY; /* bucket ids use 30 bits */
    CellGrid &G = c->G;
    TRY(dfree(c, G.count));
    TRY(dfree(c, G.start));
    TRY(dfree(c, G.scan_tmp));
    TRY(dfree(c, G.qbin));
    G.table_size = size;
    TRY(dalloc(c, &G.count, G.table_size + 1));
    TRY(dalloc(c, &G.start, G.table_size + 1));
    TRY(dalloc(c, &G.qbin, G.table_size));
    G.scan_tmp_len = std::max<int64_t>(G.table_size / 2048 + 16, (int64_t)kBboxBlocks * 12 + 16);
    TRY(dalloc(c, &G.scan_tmp, G.scan_tmp_len));
    return FJSPH_OK;
}

int validate_settings(const fjsph_settings *s) {
    if (!s) return FJSPH_E_ARG;
    if (s->dim != 2 && s->dim != 3) return FJSPH_E_ARG;
    if (!(s->H > 0) || !(s->sr > 0) || !(s->W_correc > 0)) return FJSPH_E_ARG;
    if (s->st_model < FJSPH_ST_PAIRWISE || s->st_model > FJSPH_ST_CSF) return FJSPH_E_ARG;
    /* -DNOFROZEN -DLINEAR does not compile upstream (src/Resid.cpp:381 uses fluid.rho0) */
    if ((s->variant & FJSPH_VAR_NOFROZEN) && (s->variant & FJSPH_VAR_LINEAR)) return FJSPH_E_UNSUPPORTED;
    if (s->precision != FJSPH_PREC_FP64 && s->precision != FJSPH_PREC_MIXED) return FJSPH_E_UNSUPPORTED;
    if (s->asource != FJSPH_CONST_VEL && s->asource != FJSPH_MESH_INFL && s->asource != FJSPH_POWER_LAW &&
        !(s->asource == FJSPH_VLM_INFL && s->dim == 3))
        return FJSPH_E_UNSUPPORTED;
    if (s->aero_closure != FJSPH_CLOSURE_PLAIN && s->aero_closure != FJSPH_CLOSURE_LEARNED) return FJSPH_E_ARG;
    /* the learned closure lives in the split-precision residual */
    if (s->aero_closure == FJSPH_CLOSURE_LEARNED && s->precision != FJSPH_PREC_MIXED) return FJSPH_E_UNSUPPORTED;
    return FJSPH_OK;
}

/* Boundary velocity at the current time: RK rule (src/Runge_Kutta.cpp:39-63) and NB rule
 * (src/Newmark_Beta.cpp:71-96). */
void block_velocities(const fjsph_ctx *c, const fjsph_block &B, double *vrk, double *vnb) {
    for (int k = 0; k < 3; ++k) vrk[k] = vnb[k] = 0.0;
    if (B.n_times != 0) {
        for (int t = 0; t < B.n_times && t < FJSPH_MAX_TIMES; ++t) {
            if (B.times[t] > c->s.current_time)
                for (int k = 0; k < 3; ++k) vrk[k] = B.vels[t][k];
            if (c->s.current_time > B.times[t])
                for (int k = 0; k < 3; ++k) vnb[k] = B.vels[t][k];
        }
    } else {
        for (int k = 0; k < 3; ++k) vrk[k] = vnb[k] = B.vels[0][k];
    }
}

Params make_params(const fjsph_ctx *c) {
    Params P;
    std::memset(&P, 0, sizeof(P));
    const fjsph_settings &s = c->s;
    P.D = c->D;
    P.variant = s.variant;
    P.st_model = s.st_model;
    P.pressure_rel = s.pressure_rel;
    P.acase = s.acase;
    P.use_lam = s.use_lam;
    P.use_TAB_def = s.use_TAB_def;
    P.H = s.H;
    P.H_sq = s.H_sq;
    P.sr = s.sr;
    for (int k = 0; k < 3; ++k) {
        P.cell_edge[k] = std::sqrt(s.sr) / (k == 0 ? 1 : kCellDiv) * (1.0 + 1e-6);
        P.cell_inv[k] = 1.0 / P.cell_edge[k];
    }
    P.W_correc = s.W_correc;
    P.W_dx = s.W_dx;
    P.dx = s.dx;
    P.particle_step = s.particle_step;
    P.rho_rest = s.rho_rest;
    P.rho_rest_inv = 1.0 / s.rho_rest;
    P.B = s.B;
    P.gam = s.gam;
    P.speed_sound = s.speed_sound;
    P.press_back = s.press_back;
    P.rho_min = s.rho_min;
    P.rho_max = s.rho_max;
    P.visc_alpha = s.visc_alpha;
    P.mu = s.mu;
    P.nu = s.nu;
    P.sig = s.sig;
    P.dsph_cont = s.dsph_cont;
    P.max_shift_vel = s.max_shift_vel;
    for (int k = 0; k < 3; ++k) {
        P.grav[k] = s.grav[k];
        P.v_inf[k] = s.v_inf[k];
    }
    P.grp = c->ngrp > 0 ? c->grp : nullptr;
    P.g_vinf = c->g_vinf;
    P.air_v = ((s.asource == FJSPH_VLM_INFL && c->vlm.np > 0) || (s.asource == FJSPH_MESH_INFL && c->mesh_ready) ||
               (s.asource == FJSPH_POWER_LAW && c->power_law_ready))
                  ? c->air_v
                  : nullptr;
    P.sweep_threads = c->tune[0];
    P.resid_threads = c->tune[1];
    P.list_ahead = c->tune[2];
    P.sm_order = (c->sweep_order == FJSPH_ORDER_SM && c->region_next) ? 1 : 0;
    P.region_next = c->region_next;
    {
        FConst &f = P.fc;
        f.H = (float)s.H;
        f.H_sq = (float)s.H_sq;
        f.Wc = (float)s.W_correc;
        f.W_dx = (float)s.W_dx;
        f.rho0 = (float)s.rho_rest;
        f.Bgam = (float)(s.B * s.gam);
        f.nu = (float)s.nu;
        f.alpha = (float)s.visc_alpha;
        f.dsph_cont = (float)s.dsph_cont;
        f.max_shift_vel = (float)s.max_shift_vel;
        for (int k = 0; k < 3; ++k) f.grav[k] = (float)s.grav[k];
        const double pi = 3.14159265358979323846;
        f.pi3o4_H = (float)(3.0 * pi / 4.0 / s.H);
        f.fac_bound = (float)(1.0 + 0.5 * std::cos(0.5 * pi * 7.0 / 9.0));
        const double H2 = 2.0 * s.H;
        const double lam = (6.0 / 81.0 * (H2 * H2 * H2) / (pi * pi * pi * pi) * (9.0 / 4.0 * (pi * pi * pi) - 6.0 * pi - 4.0));
        f.st_coef = 0.5 * s.sig / lam;
        f.st_coef_f = (float)f.st_coef;
        f.re_coef = (float)(2.0 * s.L / s.mu_g);
        f.interp_fac = (float)s.interp_fac;
        f.i_n_full = (float)s.i_n_full;
        f.ycoef = (float)s.ycoef;
        f.L = (float)s.L;
        f.CbL = (float)(s.Cb * s.L);
        f.A_sphere = (float)s.A_sphere;
        f.A_plate = (float)s.A_plate;
        f.force_coef = (float)(s.gamma_g / (s.sos * s.sos));
        f.we_coef = s.sig > 0.0 ? (float)(s.L / s.sig) : 0.f;
        f.surf_h = (float)(1.33 * s.particle_step);
        f.lam_cutoff = (float)s.lam_cutoff;
    }
    P.L = s.L;
    P.A_sphere = s.A_sphere;
    P.A_plate = s.A_plate;
    P.mu_g = s.mu_g;
    P.sos = s.sos;
    P.gamma_g = s.gamma_g;
    P.lam_cutoff = s.lam_cutoff;
    P.interp_fac = s.interp_fac;
    P.i_n_full = s.i_n_full;
    P.ycoef = s.ycoef;
    P.Cb = s.Cb;
    P.rho_g = s.rho_g;
    P.nb_beta = s.nb_beta;
    P.nb_gamma = s.nb_gamma;
    P.n = c->n;
    P.nb = c->nb;
    P.nblocks = (int32_t)std::min<size_t>(c->blocks.size(), kMaxBlocks);
    for (int b = 0; b < P.nblocks; ++b) {
        const fjsph_block &B = c->blocks[b];
        DevBlock &d = P.blocks[b];
        d.is_fluid = B.is_fluid;
        d.bound_solver = B.bound_solver;
        d.no_slip = B.no_slip;
        d.block_type = B.block_type;
        d.fixed_vel_or_dynamic = B.fixed_vel_or_dynamic;
        d.n_times = B.n_times;
        block_velocities(c, B, d.vel_rk, d.vel_nb);
        for (int k = 0; k < 3; ++k) d.aero_norm[k] = B.aero_norm[k];
        d.aeroconst = B.aeroconst;
        double nrm = 0.0;
        for (int k = 0; k < c->D; ++k) nrm += B.insert_norm[k] * B.insert_norm[k];
        nrm = std::sqrt(nrm);
        for (int k = 0; k < 3; ++k) d.insert_unorm[k] = nrm > 0 ? B.insert_norm[k] / nrm : B.insert_norm[k];
    }
    return P;
}

DevNbr make_nbr(const fjsph_ctx *c) {
    DevNbr N;
    N.off = c->nbr_off;
    const bool m = c->s.precision == FJSPH_PREC_MIXED;
    N.idx = m ? nullptr : c->nbr_idx;
    N.pair = m ? c->nbr_pair : nullptr;
    N.cnt = m ? c->nbr_counts : nullptr;
    N.slice = m ? c->slice_off : nullptr;
    for (int k = 0; k < 3; ++k) N.xs[k] = c->xs[k];
    return N;
}

bool mixed(const fjsph_ctx *c) { return c->s.precision == FJSPH_PREC_MIXED; }
bool grouped(const fjsph_ctx *c) { return c->ngrp > 0; }
/* time step and npd as the kernels read them: one scalar, or one per group */
const double *dt_ptr(const fjsph_ctx *c) { return grouped(c) ? c->gs.dt : &c->dsc->dt; }
const double *npd_ptr(const fjsph_ctx *c) { return grouped(c) ? c->gs.npd : &c->dsc->npd; }

int alloc_packed(fjsph_ctx *c) {
    if (c->packed_alloc) return FJSPH_OK;
    Packed &K = c->K;
    float4 **arrs[] = {&K.A, &K.C, &K.F, &K.G, &K.N, &K.T, &K.O, &K.L0, &K.L1, &K.L2, &K.Lo};
    for (float4 **a : arrs) TRY(dalloc(c, a, c->cap));
    TRY(dalloc(c, &K.R, c->cap));
    TRY(dalloc(c, &K.bits, c->cap));
    TRY(dalloc(c, &c->nbr_pair, c->nbr_cap));
    TRY(dalloc(c, &c->T.mask, (int64_t)kMaskWords * c->cap));
    TRY(dalloc(c, &c->T.count, 4));
    TRY(dalloc(c, &c->T.ntot, 2));
    c->T.stride = c->cap;
    c->T.smax = 1280;
    c->packed_alloc = true;
    c->dirty_full = true;
    return FJSPH_OK;
}

/* The FP64 pair sweeps' per-particle quotients (ResidQuot), allocated with the first FP64 sweep;
 * quot() after ensure_quot(). */
int ensure_quot(fjsph_ctx *c) {
    if (!c->resid_q) TRY(dalloc(c, &c->resid_q, c->cap));
    return FJSPH_OK;
}
ResidQuot *quot(fjsph_ctx *c) { return c->resid_q; }

void mark_full(fjsph_ctx *c) { c->dirty_full = true; }
void mark_all(fjsph_ctx *c) { c->dirty_all = true; }
void mark_bound(fjsph_ctx *c) { c->dirty_bound = true; }

/* Refresh the packed FP32 inputs of the mixed form where the FP64 state changed. */
void ensure_pack(fjsph_ctx *c) {
    if (!mixed(c) || !c->packed_alloc || c->n == 0) return;
    Params P = make_params(c);
    if (c->dirty_full) {
        launch_m_pack(P, WS(c), c->K, 0, c->n, 1, c->stream);
        c->launches++;
    } else if (c->dirty_all) {
        launch_m_pack(P, WS(c), c->K, 0, c->n, 0, c->stream);
        c->launches++;
    } else if (c->dirty_bound) {
        launch_m_pack(P, WS(c), c->K, 0, c->nb, 0, c->stream);
        c->launches++;
    }
    c->dirty_full = c->dirty_all = c->dirty_bound = false;
}

/* The stage updates write the split-precision inputs of the fluid particles they move, and the
 * inlet buffer moves those of the buffer particles they place, when the packed arrays are current
 * apart from that; the packed state is then complete again without a packing pass. */
const Packed *fused_pack(const fjsph_ctx *c) {
    return (mixed(c) && c->packed_alloc && !c->dirty_full && !c->dirty_all) ? &c->K : nullptr;
}
void after_update(fjsph_ctx *c) {
    if (!fused_pack(c)) mark_all(c);
}

int sync(fjsph_ctx *c) {
    CU(cudaStreamSynchronize(c->stream));
    CU(cudaGetLastError());
    return FJSPH_OK;
}

/* Scoped profiling section: records a start event on construction and an end event on
 * destruction when the profiler is on. */
struct Section {
    fjsph_ctx *c;
    int pass;
    size_t idx = (size_t)-1;
    Section(fjsph_ctx *c_, int pass_) : c(c_), pass(pass_) {
        Profiler &p = c->prof;
        if (!p.on) return;
        if (p.used + 2 > p.pool.size()) {
            for (int k = 0; k < 64; ++k) {
                cudaEvent_t e;
                if (cudaEventCreate(&e) != cudaSuccess) return;
                p.pool.push_back(e);
            }
        }
        idx = p.used;
        p.used += 2;
        cudaEventRecord(p.pool[idx], c->stream);
    }
    ~Section() {
        if (idx == (size_t)-1) return;
        Profiler &p = c->prof;
        cudaEventRecord(p.pool[idx + 1], c->stream);
        p.marks.push_back({pass, idx});
    }
};

int profile_collect(fjsph_ctx *c) {
    Profiler &p = c->prof;
    if (p.marks.empty()) return FJSPH_OK;
    CU(cudaStreamSynchronize(c->stream));
    for (auto &m : p.marks) {
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, p.pool[m.second], p.pool[m.second + 1]));
        p.ms[m.first] += ms;
        p.count[m.first] += 1;
    }
    p.marks.clear();
    p.used = 0;
    return FJSPH_OK;
}

/* ---- slot <-> reference index --------------------------------------------------------------- */
int download_keys(fjsph_ctx *c, std::vector<int64_t> &keys) {
    keys.resize(c->n);
    if (c->n) CU(cudaMemcpyAsync(keys.data(), c->key, sizeof(int64_t) * c->n, cudaMemcpyDeviceToHost, c->stream));
    return sync(c);
}

int block_of_ref(const fjsph_ctx *c, int64_t r) {
    for (size_t b = 0; b < c->blocks.size(); ++b)
        if (r >= c->blocks[b].first && r < c->blocks[b].second) return (int)b;
    return -1;
}

int upload_blk(fjsph_ctx *c, const std::vector<int64_t> &keys) {
    std::vector<int32_t> hb(c->n);
    for (int64_t s = 0; s < c->n; ++s) {
        int b = block_of_ref(c, keys[s]);
        if (b < 0) return FJSPH_E_ARG;
        hb[s] = b;
    }
    if (c->n) CU(cudaMemcpyAsync(c->blk, hb.data(), sizeof(int32_t) * c->n, cudaMemcpyHostToDevice, c->stream));
    return sync(c);
}

int upload_inlets(fjsph_ctx *c, const std::vector<int64_t> &keys) {
    if (c->inlets.empty()) return FJSPH_OK;
    std::vector<int32_t> slot_of_ref(c->n, -1);
    for (int64_t s = 0; s < c->n; ++s)
        if (keys[s] >= 0 && keys[s] < c->n) slot_of_ref[keys[s]] = (int32_t)s;
    for (HostInlet &I : c->inlets) {
        std::vector<int32_t> b(I.n_back), f(I.n_back * I.depth);
        for (int64_t i = 0; i < I.n_back; ++i) {
            if (I.back_ref[i] < 0 || I.back_ref[i] >= c->n) return FJSPH_E_ARG;
            b[i] = slot_of_ref[I.back_ref[i]];
        }
        for (int64_t i = 0; i < I.n_back * I.depth; ++i) {
            if (I.buffer_ref[i] < 0 || I.buffer_ref[i] >= c->n) return FJSPH_E_ARG;
            f[i] = slot_of_ref[I.buffer_ref[i]];
        }
        if (!b.empty()) CU(cudaMemcpyAsync(I.d_back, b.data(), sizeof(int32_t) * b.size(), cudaMemcpyHostToDevice, c->stream));
        if (!f.empty())
            CU(cudaMemcpyAsync(I.d_buffer, f.data(), sizeof(int32_t) * f.size(), cudaMemcpyHostToDevice, c->stream));
    }
    return sync(c);
}

/* ---- host <-> device state transfer ----------------------------------------------------------- */
struct HostField {
    const char *name;
    int comps; /* 1, D or D*D */
    int type;  /* 0 double, 1 int64, 2 int32 */
};

void view_ptrs(const fjsph_state_view *v, std::vector<void *> &ptr) {
    ptr = {v->xi,         v->v,      v->acc,   v->Af,      v->aVisc,   v->cellV,  v->gradRho, v->norm,
           v->vPert,      v->L,      v->Rrho,  v->rho,     v->p,       v->m,      v->curve,   v->norm_curve,
           v->woccl,      v->pDist,  v->deltaD, v->cellP,  v->cellRho, v->colourG, v->colour, v->lam,
           v->lam_nb,     v->kernsum, v->part_id, v->cellID, v->b,      v->surf,   v->surfzone};
}

/* Device arrays in the same order as view_ptrs, with component counts. */
void dev_ptrs(const DevState &S, int D, std::vector<std::vector<void *>> &ptr, std::vector<int> &type) {
    ptr.clear();
    type.clear();
    auto vec = [&](double *const a[3]) {
        std::vector<void *> p;
        for (int k = 0; k < D; ++k) p.push_back(a[k]);
        ptr.push_back(p);
        type.push_back(0);
    };
    vec(S.x);
    vec(S.v);
    vec(S.acc);
    vec(S.Af);
    vec(S.aVisc);
    vec(S.cellV);
    vec(S.gradRho);
    vec(S.norm);
    vec(S.vPert);
    {
        std::vector<void *> p;
        for (int k = 0; k < D * D; ++k) p.push_back(S.L[k]);
        ptr.push_back(p);
        type.push_back(0);
    }
    double *sc[] = {S.Rrho, S.rho,     S.p,       S.m,      S.curve, S.norm_curve, S.woccl,  S.pDist,
                    S.deltaD, S.cellP, S.cellRho, S.colourG, S.colour, S.lam,      S.lam_nb, S.kernsum};
    for (double *a : sc) {
        ptr.push_back({a});
        type.push_back(0);
    }
    ptr.push_back({S.part_id});
    type.push_back(1);
    ptr.push_back({S.cellID});
    type.push_back(1);
    ptr.push_back({S.b});
    type.push_back(2);
    ptr.push_back({S.surf});
    type.push_back(2);
    ptr.push_back({S.surfzone});
    type.push_back(2);
}

/* Host <-> device state transfer, field by field through two staging buffers: the copy of one
 * field (copy stream) overlaps the reference-order gather / scatter of the previous one (context
 * stream); events order the reuse of each buffer. */
/* Host <-> device copy of a state view through two staging buffers.  mirror (upload only):
 * a second state that receives each field by a device copy right after it arrives. */
int transfer(fjsph_ctx *c, DevState &S, const fjsph_state_view *v, bool up, DevState *mirror = nullptr) {
    Section sec(c, PASS_TRANSFER);
    std::vector<void *> hp;
    view_ptrs(v, hp);
    std::vector<std::vector<void *>> dp, dp2;
    std::vector<int> type, type2;
    dev_ptrs(S, c->D, dp, type);
    if (mirror) dev_ptrs(*mirror, c->D, dp2, type2);
    const int64_t n = c->n;
    bool any = false;
    for (void *p : hp) any = any || p != nullptr;
    if (!any) return FJSPH_E_ARG;
    if (!c->copy_stream) {
        CU(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            CU(cudaEventCreateWithFlags(&c->st_copied[b], cudaEventDisableTiming));
            CU(cudaEventCreateWithFlags(&c->st_used[b], cudaEventDisableTiming));
        }
    }
    double *stage[2] = {c->stage, c->stage2};
    int moved = 0; /* fields copied so far: null host arrays are skipped */
    for (size_t f = 0; f < dp.size(); ++f) {
        if (!hp[f]) continue;
        const int b = moved & 1;
        const bool reuse = moved >= 2;
        ++moved;
        const int comps = (int)dp[f].size();
        const int es = type[f] == 2 ? 4 : 8;
        const size_t bytes = (size_t)es * comps * n;
        FieldPtrs fp{};
        for (int k = 0; k < comps; ++k) fp.p[k] = dp[f][k];
        if (up) {
            if (reuse) CU(cudaStreamWaitEvent(c->copy_stream, c->st_used[b], 0));
            CU(cudaMemcpyAsync(stage[b], hp[f], bytes, cudaMemcpyHostToDevice, c->copy_stream));
            CU(cudaEventRecord(c->st_copied[b], c->copy_stream));
            CU(cudaStreamWaitEvent(c->stream, c->st_copied[b], 0));
            launch_field_in(stage[b], comps, es, c->key, fp, n, c->stream);
            CU(cudaEventRecord(c->st_used[b], c->stream));
            if (mirror)
                for (int k = 0; k < comps; ++k)
                    CU(cudaMemcpyAsync(dp2[f][k], dp[f][k], (size_t)es * n, cudaMemcpyDeviceToDevice, c->stream));
        } else {
            if (reuse) CU(cudaStreamWaitEvent(c->stream, c->st_copied[b], 0));
            launch_field_out(stage[b], comps, es, c->key, fp, n, c->stream);
            CU(cudaEventRecord(c->st_used[b], c->stream));
            CU(cudaStreamWaitEvent(c->copy_stream, c->st_used[b], 0));
            CU(cudaMemcpyAsync(hp[f], stage[b], bytes, cudaMemcpyDeviceToHost, c->copy_stream));
            CU(cudaEventRecord(c->st_copied[b], c->copy_stream));
        }
    }
    CU(cudaStreamSynchronize(c->copy_stream));
    return sync(c);
}

/* bytes per particle of field f (view_ptrs order) */
int64_t es_bytes_of(fjsph_ctx *c, int f) {
    std::vector<std::vector<void *>> dp;
    std::vector<int> type;
    dev_ptrs(WS(c), c->D, dp, type);
    return (int64_t)(type[f] == 2 ? 4 : 8) * (int64_t)dp[f].size();
}

/* The input groups of fjsph_step_host, by the first pass that reads them (view_ptrs order):
 *   kInPos    the neighbour search: the positions;
 *   kInStep   the time-step reduction: acc, Af, v, Rrho, rho, curve (and vPert under ALE);
 *   kInPack   the npd pass and the packing of the split-precision inputs: p, m, type, surface flags
 *             (and the fields the pre-passes recompute before reading, when given);
 *   kInLate   the first stage: the frozen dissipation terms, the air cell values, the previous
 *             surface detection, the particle id and cell. */
enum { kInPos = 0, kInStep = 1, kInPack = 2, kInLate = 3 }; /* the order they travel in */
int in_group(size_t f, int32_t variant) {
    switch (f) {
    case 2: case 3: case 1: case 10: case 11: case 14: /* acc Af v Rrho rho curve */
        return kInStep;
    case 8: /* vPert: the time-step reduction reads it under ALE, the packing always */
        return (variant & FJSPH_VAR_ALE) ? kInStep : kInPack;
    case 0: /* xi */
        return kInPos;
    case 4: case 5: case 7: case 15: case 16: case 18: case 19: case 20: case 23: case 24: case 26: case 27:
        /* aVisc cellV norm norm_curve woccl deltaD cellP cellRho lam lam_nb part_id cellID */
        return kInLate;
    default:
        return kInPack;
    }
}

/* One input group of fjsph_step_host into pnp1 and pn on place_stream, each field once its host
 * copy has landed (enqueued at once for every group). */
int place_in(fjsph_ctx *c, int g) {
    if (c->in_grp[g].empty()) return FJSPH_OK;
    cudaStream_t s = c->place_stream;
    std::vector<std::vector<void *>> dp, dp2;
    std::vector<int> type, type2;
    dev_ptrs(WS(c), c->D, dp, type);
    dev_ptrs(PN(c), c->D, dp2, type2);
    for (const auto &L : c->in_grp[g]) {
        CU(cudaStreamWaitEvent(s, c->in_ev[L.ev], 0)); /* each field as it lands */
        const size_t f = (size_t)L.f;
        const int comps = (int)dp[f].size();
        const int es = type[f] == 2 ? 4 : 8;
        FieldPtrs fp{};
        for (int k = 0; k < comps; ++k) fp.p[k] = dp[f][k];
        launch_field_in(c->in_stage + L.off, comps, es, c->key, fp, c->n, s);
        for (int k = 0; k < comps; ++k)
            CU(cudaMemcpyAsync(dp2[f][k], dp[f][k], (size_t)es * c->n, cudaMemcpyDeviceToDevice, s));
        c->launches++;
    }
    CU(cudaEventRecord(c->in_placed[g], s));
    c->in_grp[g].clear();
    c->in_wait[g] = true;
    return FJSPH_OK;
}

/* The compute stream waits for input group g of fjsph_step_host (before its first reader). */
int apply_in(fjsph_ctx *c, int g) {
    if (!c->in_wait[g]) return FJSPH_OK;
    CU(cudaStreamWaitEvent(c->stream, c->in_placed[g], 0));
    c->in_wait[g] = false;
    return FJSPH_OK;
}

int apply_all_in(fjsph_ctx *c) {
    for (int g = 0; g < 4; ++g) TRY(apply_in(c, g));
    return FJSPH_OK;
}

/* the ids of fjsph_step_host's upload, scanned on a host thread during the step */
void join_id_scan(fjsph_ctx *c) {
    if (!c->id_scan.joinable()) return;
    c->id_scan.join();
    c->part_id_next = c->id_scan_next;
}

/* The fields a Runge-Kutta step does not write after the pre-passes of its second search (view_ptrs
 * order): the surface detection, the dSPH eigenvalues, the air cell values, the shifting velocity,
 * mass, id and type (the pipe-outlet pass is a pre-pass) and, with frozen dissipation, the
 * dissipation terms.  The stages and the final update leave them; an insertion or a deletion
 * moves the slots (and retypes the inlet's particles), after which they are copied out again
 * with the rest. */
bool early_out_field(size_t f, int32_t variant) {
    static const int kOut[] = {5 /* cellV */, 7 /* norm */, 8 /* vPert */, 13 /* m */, 14 /* curve */,
                               15 /* norm_curve */, 16 /* woccl */, 19 /* cellP */, 20 /* cellRho */, 23 /* lam */,
                               24 /* lam_nb */, 26 /* part_id */, 27 /* cellID */, 28 /* b */, 29 /* surf */,
                               30 /* surfzone */};
    for (int k : kOut)
        if ((size_t)k == f) return true;
    if (!(variant & FJSPH_VAR_NOFROZEN) && (f == 4 /* aVisc */ || f == 18 /* deltaD */)) return true;
    return false;
}

/* The fields a Runge-Kutta step writes last in its final residual (acceleration and density
 * rate): sent while the final update, the inlet and update_data run. */
bool final_out_field(size_t f) { return f == 2 /* acc */ || f == 10 /* Rrho */; }

/* fjsph_step_host: fields gathered into reference order and sent to the host on the copy stream
 * (list: the early fields once the second search's pre-passes are enqueued, the final ones after
 * the last residual) */
int send_out(fjsph_ctx *c, const std::vector<fjsph_ctx::LateField> &list) {
    cudaStream_t s = c->stream;
    std::vector<std::vector<void *>> dp;
    std::vector<int> type;
    dev_ptrs(WS(c), c->D, dp, type);
    for (const auto &E : list) {
        const size_t f = (size_t)E.f;
        const int comps = (int)dp[f].size();
        const int es = type[f] == 2 ? 4 : 8;
        FieldPtrs fp{};
        for (int k = 0; k < comps; ++k) fp.p[k] = dp[f][k];
        launch_field_out(c->out_stage + E.off, comps, es, c->key, fp, c->n, s);
        c->launches++;
    }
    CU(cudaEventRecord(c->out_ready, s));
    CU(cudaStreamWaitEvent(c->copy_stream, c->out_ready, 0));
    for (const auto &E : list)
        CU(cudaMemcpyAsync(const_cast<void *>(E.host), c->out_stage + E.off, (size_t)es_bytes_of(c, E.f) * c->n,
                           cudaMemcpyDeviceToHost, c->copy_stream));
    return FJSPH_OK;
}

int send_early_out(fjsph_ctx *c) {
    if (c->early_out.empty() || c->out_sent) return FJSPH_OK;
    TRY(send_out(c, c->early_out));
    c->out_sent = true;
    c->out_n = c->n;
    return FJSPH_OK;
}

/* The fields update_data writes last (positions, velocities, density, pressure): sent when it has
 * run without inserting or deleting, while the state is copied to pn. */
bool last_out_field(size_t f) { return f == 0 || f == 1 || f == 11 || f == 12; }

int send_last_out(fjsph_ctx *c) {
    if (c->last_out.empty() || !c->out_sent || c->last_sent || c->n != c->out_n || c->inserted != c->out_ins0 ||
        c->deleted != c->out_del0)
        return FJSPH_OK;
    TRY(send_out(c, c->last_out));
    c->last_sent = true;
    return FJSPH_OK;
}

int send_final_out(fjsph_ctx *c) {
    if (c->final_out.empty() || !c->out_sent || c->final_sent || c->n != c->out_n) return FJSPH_OK;
    TRY(send_out(c, c->final_out));
    c->final_sent = true;
    return FJSPH_OK;
}

/* ---- neighbour search --------------------------------------------------------------------------- */
int reorder_states(fjsph_ctx *c, const Params &P) {
    TRY(apply_all_in(c)); /* the permutation moves every field */
    cudaStream_t s = c->stream;
    launch_reorder_map(P, c->G, c->new_of_old, c->reorder_tmp, c->reorder_tmp_len, s);
    c->launches += 5;
    /* permute pn and W through the spare state (in graph mode the result is copied back, so
     * that every captured launch keeps addressing the same buffers) */
    for (int which = 0; which < 2; ++which) {
        int &role = which == 0 ? c->ipn : c->iW;
        launch_permute(state_fields(c->st[role], c->D), state_fields(c->st[c->isp], c->D), c->new_of_old, c->n, s);
        if (c->graph_mode)
            launch_copy(state_fields(c->st[c->isp], c->D), state_fields(c->st[role], c->D), c->n, s);
        else
            std::swap(role, c->isp);
        c->launches += c->graph_mode ? 2 : 1;
    }
    /* shared per-slot arrays: key and blk (through the spare state's i64/i32 scratch) */
    {
        FieldList a, b;
        a.i64[a.ni64++] = c->key;
        b.i64[b.ni64++] = c->st[c->isp].part_id;
        a.i32[a.ni32++] = c->blk;
        b.i32[b.ni32++] = c->st[c->isp].b;
        if (grouped(c)) {
            a.i32[a.ni32++] = c->grp;
            b.i32[b.ni32++] = c->st[c->isp].surf;
        }
        launch_permute(a, b, c->new_of_old, c->n, s);
        CU(cudaMemcpyAsync(c->key, c->st[c->isp].part_id, sizeof(int64_t) * c->n, cudaMemcpyDeviceToDevice, s));
        CU(cudaMemcpyAsync(c->blk, c->st[c->isp].b, sizeof(int32_t) * c->n, cudaMemcpyDeviceToDevice, s));
        if (grouped(c))
            CU(cudaMemcpyAsync(c->grp, c->st[c->isp].surf, sizeof(int32_t) * c->n, cudaMemcpyDeviceToDevice, s));
        c->launches += 1;
    }
    for (HostInlet &I : c->inlets) {
        launch_remap_i32(I.d_back, I.n_back, c->new_of_old, s);
        launch_remap_i32(I.d_buffer, I.n_back * I.depth, c->new_of_old, s);
        c->launches += 2;
    }
    for (int k = 0; k < c->D; ++k)
        CU(cudaMemcpyAsync(c->xs[k], WS(c).x[k], sizeof(double) * c->n, cudaMemcpyDeviceToDevice, s));
    if (c->packed_alloc && c->occ_valid) { /* occlusion statistics follow their particles */
        float4 *tmp = reinterpret_cast<float4 *>(c->stage);
        launch_m_permute_f4(c->K.O, tmp, c->new_of_old, c->n, s);
        CU(cudaMemcpyAsync(c->K.O, tmp, sizeof(float4) * c->n, cudaMemcpyDeviceToDevice, s));
        c->launches += 1;
    }
    mark_full(c);
    return FJSPH_OK;
}

int32_t wcap_for(int64_t maxcnt) {
    const int64_t w = maxcnt + maxcnt / 4 + kChunk;
    return (int32_t)(((w + kChunk - 1) / kChunk) * kChunk);
}

int grow_pairs(fjsph_ctx *c, int64_t need) {
    if (need <= c->nbr_cap) return FJSPH_OK;
    TRY(graph_release(c));
    const int64_t ncap = need + need / 8;
    if (ncap >= ((int64_t)1 << 31) * 4) return FJSPH_E_NEIGHBOUR;
    TRY(dfree(c, c->nbr_pair));
    TRY(dalloc(c, &c->nbr_pair, ncap));
    if (c->nbr_idx) {
        TRY(dfree(c, c->nbr_idx));
        TRY(dalloc(c, &c->nbr_idx, ncap));
    }
    c->nbr_cap = ncap;
    return FJSPH_OK;
}

/* Tiles and member masks of the split-precision sweeps for this search.  A grid that outgrew the
 * bucket table or a particle with more candidates than a mask holds leaves the sweeps on the pair
 * lists for this search (tiles_valid false). */
int tile_search(fjsph_ctx *c, const Params &P) {
    cudaStream_t s = c->stream;
    TRY(alloc_packed(c));
    if (c->tiles_table != c->G.table_size) {
        TRY(dfree(c, c->T.list));
        TRY(dfree(c, c->T.scan));
        TRY(dalloc(c, &c->T.list, c->G.table_size + 1));
        TRY(dalloc(c, &c->T.scan, c->G.table_size + 1));
        c->tiles_table = c->G.table_size;
    }
    c->T.flag = c->G.count; /* free after the scatter */
    if (!c->graph_mode) CU(cudaMemsetAsync(&c->dsc->status, 0, sizeof(int32_t), s));
    CU(cudaMemsetAsync(&c->dsc->tile_pairs, 0, sizeof(unsigned long long) + sizeof(int32_t), s));
    launch_tile_build(P, c->G, c->T, &c->dsc->status, s);
    launch_tile_masks(P, c->xs, c->G, c->K, c->T, c->dsc, s);
    c->launches += 6;
    if (!c->graph_mode) {
        CU(cudaMemcpyAsync(&c->hsc->status, &c->dsc->status, sizeof(DevScalars) - offsetof(DevScalars, status),
                           cudaMemcpyDeviceToHost, s));
        TRY(sync(c));
        if (c->hsc->status & kStatusTileOverflow) {
            CU(cudaMemsetAsync(&c->dsc->status, 0, sizeof(int32_t), s));
            c->hsc->status = 0;
            c->tiles_valid = false;
            return FJSPH_OK;
        }
    }
    c->tiles_valid = true;
    return FJSPH_OK;
}

/* Split-precision lists in one walk: wcap entries of storage per slot, a re-run with a larger
 * wcap if any slot has more neighbours. */
int search_fixed(fjsph_ctx *c, const Params &P) {
    cudaStream_t s = c->stream;
    const int64_t nslices = (c->n + kSlice - 1) / kSlice;
    for (int attempt = 0;; ++attempt) {
        const int64_t need = nslices * kSlice * (int64_t)c->wcap;
        if (need > c->nbr_cap) {
            if (c->graph_mode) return FJSPH_E_NEIGHBOUR; /* sized before capture */
            TRY(grow_pairs(c, need));
        }
        CU(cudaMemsetAsync(&c->dsc->maxcnt, 0, sizeof(int32_t) + sizeof(unsigned long long), s));
        launch_nbr_fill_fixed(P, c->xs, c->G, c->nbr_pair, c->nbr_counts, c->slice_off, c->wcap, c->dsc, s);
        c->launches += 3;
        c->nbr_storage = need;
        if (c->graph_mode) {
            c->nbr_valid = true;
            return FJSPH_OK;
        }
        int64_t grid[4];
        CU(cudaMemcpyAsync(&c->hsc->status, &c->dsc->status, sizeof(DevScalars) - offsetof(DevScalars, status),
                           cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(&c->hsc->red[10], c->G.grid, 4 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        TRY(sync(c));
        std::memcpy(grid, &c->hsc->red[10], 4 * sizeof(int64_t));
        if (grid[3]) {
            const double ncells = (double)grid[0] * (double)grid[1] * (double)grid[2];
            if (ncells <= (double)kMaxTable) c->table_want = next_pow2((int64_t)ncells);
        }
        c->maxcnt = c->hsc->maxcnt;
        if (c->hsc->status & kStatusNbrOverflow) {
            CU(cudaMemsetAsync(&c->dsc->status, 0, sizeof(int32_t), s));
            c->hsc->status = 0;
            if (attempt >= 3) return FJSPH_E_NEIGHBOUR;
            c->wcap = wcap_for(c->maxcnt);
            continue;
        }
        c->n_pairs = (int64_t)c->hsc->pairs;
        c->nbr_valid = true;
        return FJSPH_OK;
    }
}

int search(fjsph_ctx *c) {
    if (c->n == 0) return FJSPH_E_STATE;
    TRY(apply_in(c, kInPos));
    if (c->pair_mode == FJSPH_PAIRS_TILES) TRY(apply_in(c, kInPack)); /* the masks read packed inputs */
    if (c->table_want > c->G.table_size) {
        TRY(sync(c));
        TRY(alloc_table(c, c->table_want));
    }
    if (c->prof.on && c->prof.used > 4096) TRY(profile_collect(c));
    cudaStream_t s = c->stream;
    Params P = make_params(c);
    Section sec(c, PASS_SEARCH);
    launch_bbox(P, WS(c), c->G, s);
    if (!c->graph_mode && (c->searches == 0 || c->reorder_pending)) {
        /* a new particle set: size the bucket table for its grid before the first walk (a
         * wrapped table makes the walk check every earlier cell for a shared bucket) */
        int64_t grid[4];
        CU(cudaMemcpyAsync(&c->hsc->red[10], c->G.grid, 4 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        TRY(sync(c));
        std::memcpy(grid, &c->hsc->red[10], 4 * sizeof(int64_t));
        const double ncells = (double)grid[0] * (double)grid[1] * (double)grid[2];
        if (grid[3] && ncells <= (double)kMaxTable) {
            TRY(alloc_table(c, next_pow2((int64_t)ncells)));
            launch_bbox(P, WS(c), c->G, s);
        }
    }
    launch_hash_and_count(P, WS(c), c->xs, c->G, s);
    launch_scan_buckets(c->G, s);
    launch_scatter_sort(P, c->G, c->xs[0], s);
    c->launches += 2 + 1 + 3 + 2;
    const bool due = c->s.reorder_interval > 0 && (c->reorder_pending || (c->searches % c->s.reorder_interval) == 0);
    if (due) {
        Section sr(c, PASS_REORDER);
        TRY(reorder_states(c, P));
        c->reorder_pending = false;
    }
    c->searches++;
    launch_sorted_pos(P, c->xs, c->G, s);
    c->tiles_valid = false;
    if (mixed(c) && c->pair_mode == FJSPH_PAIRS_TILES && c->D >= 2) TRY(tile_search(c, P));
    if (mixed(c) && c->wcap > 0) return search_fixed(c, P);
    launch_nbr_count(P, c->xs, c->G, c->nbr_counts, s);
    launch_scan_i64(c->nbr_counts, c->nbr_off, c->n, c->scan_tmp64, s);
    c->launches += 4;
    const int64_t nslices = (c->n + kSlice - 1) / kSlice;
    if (mixed(c)) {
        launch_slice_width(c->nbr_counts, c->n, c->slice_w, s);
        launch_scan_i64(c->slice_w, c->slice_off, nslices, c->scan_tmp64, s);
        c->launches += 4;
    }
    if (c->graph_mode) {
        /* no host round trip: the lists must fit the storage sized before capture; the fill
         * raises a device status bit otherwise */
        launch_nbr_fill(P, c->xs, c->G, c->nbr_off, c->nbr_idx, mixed(c) ? c->nbr_pair : nullptr, c->slice_off,
                        c->nbr_counts, c->nbr_cap, &c->dsc->status, s);
        c->launches += 1;
        c->nbr_valid = true;
        return FJSPH_OK;
    }
    if (mixed(c))
        CU(cudaMemcpyAsync(&c->hsc->red[14], c->slice_off + nslices, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    int64_t total = 0, storage = 0, grid[4] = {0, 0, 0, 0};
    CU(cudaMemcpyAsync(&c->hsc->red[15], c->nbr_off + c->n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(&c->hsc->red[10], c->G.grid, 4 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    TRY(sync(c));
    std::memcpy(&total, &c->hsc->red[15], sizeof(int64_t));
    std::memcpy(grid, &c->hsc->red[10], 4 * sizeof(int64_t));
    if (mixed(c)) std::memcpy(&storage, &c->hsc->red[14], sizeof(int64_t));
    const int64_t need = std::max(total, storage);
    if (grid[3]) {
        /* the grid outgrew the table: this search used the wrapped (slower) walk; grow the table
         * for the next one when the grid is of a reasonable size */
        const double ncells = (double)grid[0] * (double)grid[1] * (double)grid[2];
        if (ncells <= (double)kMaxTable) c->table_want = next_pow2((int64_t)ncells);
    }
    if (need > c->nbr_cap) {
        int64_t ncap = std::max<int64_t>(need + need / 4, c->nbr_cap * 2);
        if (ncap >= ((int64_t)1 << 31)) return FJSPH_E_NEIGHBOUR;
        CU(cudaFree(c->nbr_idx));
        c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), (void *)c->nbr_idx), c->allocs.end());
        TRY(dalloc(c, &c->nbr_idx, ncap));
        if (c->packed_alloc) {
            CU(cudaFree(c->nbr_pair));
            c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), (void *)c->nbr_pair), c->allocs.end());
            TRY(dalloc(c, &c->nbr_pair, ncap));
        }
        c->nbr_cap = ncap;
    }
    if (mixed(c)) TRY(alloc_packed(c));
    launch_nbr_fill(P, c->xs, c->G, c->nbr_off, c->nbr_idx, mixed(c) ? c->nbr_pair : nullptr, c->slice_off,
                    c->nbr_counts, c->nbr_cap, &c->dsc->status, s);
    c->launches += 1;
    c->n_pairs = total;
    c->nbr_storage = mixed(c) ? storage : total;
    if (mixed(c) && c->n > 0) { /* later searches: one walk with room for 1.6x the mean count */
        const int64_t mean = (total + c->n - 1) / c->n;
        c->wcap = wcap_for(mean + mean / 3);
    }
    c->nbr_valid = true;
    return FJSPH_OK;
}

/* ---- passes ----------------------------------------------------------------------------------------- */
__global__ void k_finish_npd(DevScalars *d, double inv_n) { d->npd = d->red[0] * inv_n; }
__global__ void k_set_scalar(double *dst, double v) { *dst = v; }

/* npd = mean kernel sum over all particles (per group when the context holds several) */
int finish_npd(fjsph_ctx *c) {
    if (grouped(c)) {
        CU(cudaMemsetAsync(c->g_sum, 0, sizeof(double) * c->ngrp, c->stream));
        launch_group_sum(c->grp, c->npd_part, 0, c->n, c->g_sum, c->stream);
        launch_group_npd(c->gs.npd, c->g_sum, c->gs.count, c->ngrp, c->stream);
        c->launches += 3;
        return FJSPH_OK;
    }
    launch_sum(c->npd_part, c->n, c->S.part, c->S.part_len, &c->dsc->red[0], c->stream);
    k_finish_npd<<<1, 1, 0, c->stream>>>(c->dsc, 1.0 / double(c->n));
    c->launches += 4;
    return FJSPH_OK;
}

int prestep_npd(fjsph_ctx *c, const Params &P) {
    Section sec(c, PASS_PRESTEP);
    if (mixed(c)) {
        ensure_pack(c);
        launch_m_dsph(P, WS(c), make_nbr(c), c->K, c->npd_part, c->stream);
    } else {
        TRY(ensure_quot(c));
        launch_dsph_prestep(P, WS(c), make_nbr(c), c->npd_part, quot(c), c->stream);
    }
    return finish_npd(c);
}

/* npd only (Runge-Kutta first pre-pass, see integrate_no_update) */
int npd_only(fjsph_ctx *c, const Params &P) {
    Section sec(c, PASS_PRESTEP);
    if (mixed(c)) {
        ensure_pack(c);
        launch_m_npd(P, make_nbr(c), c->K, c->npd_part, c->stream);
    } else {
        launch_npd_only(P, WS(c), make_nbr(c), c->npd_part, c->stream);
    }
    return finish_npd(c);
}

/* the position-dependent air velocity of the particles that use it (before the aero velocity
 * pass): the vortex lattice or the analytic boundary layer */
int vlm_air(fjsph_ctx *c, const Params &P, const DevNbr &N) {
    if (c->s.asource == FJSPH_POWER_LAW) {
        if (!c->power_law_ready) return FJSPH_E_STATE; /* fjsph_air_power_law has not run */
        Section sec(c, PASS_AIR);
        launch_power_law_air(P, WS(c), c->power_law, c->air_v, mixed(c), c->stream);
        c->launches++;
        return FJSPH_OK;
    }
    if (c->s.asource != FJSPH_VLM_INFL) return FJSPH_OK;
    if (c->vlm.np == 0) return FJSPH_E_STATE; /* fjsph_vlm_setup has not run */
    Section sec(c, PASS_AIR);
    launch_vlm_air(P, WS(c), N, c->vlm, c->air_v, mixed(c), c->stream);
    c->launches++;
    return FJSPH_OK;
}

/* get_aero_velocity: the uniform / vortex-lattice source, or FindCell for the mesh source */
int aero_velocity(fjsph_ctx *c, const Params &P, const DevNbr &N) {
    if (c->s.asource == FJSPH_MESH_INFL) {
        if (!c->mesh_ready) return FJSPH_E_STATE; /* fjsph_mesh_set has not run */
        launch_mesh_find(P, WS(c), c->mesh, c->air_v, c->mesh_list, c->mesh_count, c->stream);
        c->launches++; /* two launches: mark, then the listed particles */
    } else {
        launch_aero_velocity(P, WS(c), N, c->stream);
    }
    c->launches++;
    return FJSPH_OK;
}

int prestep_passes(fjsph_ctx *c) {
    if (!c->nbr_valid) return FJSPH_E_STATE;
    Params P = make_params(c);
    DevNbr N = make_nbr(c);
    cudaStream_t s = c->stream;
    TRY(prestep_npd(c, P));
    const bool dissipation = !(c->s.variant & FJSPH_VAR_NOFROZEN);
    TRY(vlm_air(c, P, N)); /* position-dependent air velocity, its own section */
    {
        /* split-precision form: the dissipation terms are computed in the surface-normal walk
         * (they read nothing the surface passes write), timed with the surface section */
        Section sec(c, PASS_SURFACE);
        TRY(aero_velocity(c, P, N));
        if (mixed(c)) {
            launch_m_surface(P, WS(c), N, c->K, dissipation, s);
            c->occ_valid = true;
        } else {
            TRY(ensure_quot(c));
            launch_detect_surface(P, WS(c), N, c->nrm_tmp, quot(c), s);
        }
        c->launches += 3; /* plus the aero velocity pass, counted by aero_velocity */
    }
    if (dissipation && !mixed(c)) {
        Section sec(c, PASS_DISSIPATION);
        TRY(ensure_quot(c));
        launch_dissipation(P, WS(c), N, quot(c), s);
        c->launches++;
    }
    if (c->s.variant & FJSPH_VAR_ALE) {
        Section sec(c, PASS_SHIFT);
        if (mixed(c)) {
            launch_m_particle_shift(P, WS(c), N, c->K, s);
        } else {
            TRY(ensure_quot(c));
            launch_particle_shift(P, WS(c), N, quot(c), s);
        }
        c->launches++;
    }
    {
        Section sec(c, PASS_UPDATE);
        const Packed *K = fused_pack(c);
        launch_pipe_outlet(P, WS(c), K ? K->bits : nullptr, s);
        c->launches++;
        if (!K) mark_all(c);
    }
    c->pn_equals_W = false;
    return FJSPH_OK;
}

bool has_solver(const fjsph_ctx *c, int solver) {
    for (int64_t b = 0; b < c->n_bound_blocks; ++b)
        if (c->blocks[b].bound_solver == solver) return true;
    return false;
}
bool has_no_slip(const fjsph_ctx *c) {
    for (int64_t b = 0; b < c->n_bound_blocks; ++b)
        if (c->blocks[b].no_slip) return true;
    return false;
}

/* Boundary section of a stage: velocities, no-slip mirror, solver pass. */
int boundary_section(fjsph_ctx *c, const Params &P, int nb_rule) {
    if (c->nb == 0) return FJSPH_OK;
    Section sec(c, PASS_BOUNDARY);
    DevNbr N = make_nbr(c);
    cudaStream_t s = c->stream;
    launch_bound_velocity(P, WS(c), nb_rule, s);
    c->launches++;
    if (has_no_slip(c)) {
        launch_no_slip(P, WS(c), N, c->vtmp, s);
        c->launches += 2;
    }
    if (has_solver(c, FJSPH_DBC)) {
        launch_bound_dbc(P, WS(c), s);
        c->launches++;
    }
    if (mixed(c)) {
        mark_bound(c); /* boundary velocities changed */
        ensure_pack(c);
    }
    if (has_solver(c, FJSPH_PRESSURE_G)) {
        if (mixed(c))
            launch_m_bound_pressure(P, WS(c), N, c->K, s);
        else
            launch_bound_pressure(P, WS(c), N, s);
        c->launches++;
    }
    if (has_solver(c, FJSPH_GHOST)) {
        if (mixed(c))
            launch_m_bound_ghost(P, WS(c), N, c->K, c->S.near_inlet, s);
        else
            launch_bound_ghost(P, WS(c), N, c->S.near_inlet, s);
        c->launches++;
    }
    mark_bound(c);
    return FJSPH_OK;
}

bool learned_wanted(const fjsph_ctx *c) { return c->s.aero_closure == FJSPH_CLOSURE_LEARNED; }
bool learned_active(const fjsph_ctx *c) {
    return learned_wanted(c) && mixed(c) && c->s.acase == FJSPH_GISSLER && c->mlp_ready && !c->closure_fallback;
}

/* Closure of the next residual: plain, learned, or a one-shot judge / log call.  The learned
 * closure needs the occlusion statistics of a surface pass on the current particle set; until
 * one has run the residual uses the plain closure. */
Closure next_closure(fjsph_ctx *c) {
    Closure C{};
    C.mode = kClosurePlain;
    C.occ = c->K.O;
    C.M = mlp::DevMlp{c->mlp_params, c->mlp_w, c->mlp_wt};
    C.judge = c->judge_dev;
    C.logX = c->log_X;
    C.logT = c->log_T;
    C.log_count = c->log_count;
    C.log_cap = c->log_cap;
    /* an armed judge / log waits for the first residual that can honour it */
    if (!mixed(c) || c->s.acase != FJSPH_GISSLER || !c->occ_valid) return C;
    if (learned_active(c)) {
        C.mode = kClosureLearned;
        if (c->arm == FJSPH_CLOSURE_ARM_JUDGE && c->judge_dev) {
            C.mode = kClosureJudge;
            c->arm = 0;
        }
    } else if (c->arm == FJSPH_CLOSURE_ARM_LOG && c->log_cap > 0) {
        C.mode = kClosureLog;
        c->arm = 0;
    }
    return C;
}

/* Judge result of the last judge residual (after the stream reached it). */
int closure_collect(fjsph_ctx *c) {
    if (!c->judge_pending) return FJSPH_OK;
    TRY(sync(c));
    c->judge_pending = false;
    const double d2 = c->judge_host[0], p2 = c->judge_host[1];
    c->judged_particles = (int64_t)c->judge_host[2];
    c->last_rel_rms = p2 > 0.0 ? std::sqrt(d2 / p2) : (d2 > 0.0 ? INFINITY : 0.0);
    c->max_rel_rms = std::max(c->max_rel_rms, c->last_rel_rms);
    c->judged++;
    if (!(c->last_rel_rms <= c->judge_tol)) c->closure_fallback = true;
    return FJSPH_OK;
}

/* The residual in the configured form. */
int resid(fjsph_ctx *c, const Params &P) {
    if (learned_wanted(c) && !(mixed(c) && c->mlp_ready)) return FJSPH_E_STATE;
    Section sec(c, PASS_RESID);
    if (mixed(c)) {
        ensure_pack(c);
        const Closure C = next_closure(c);
        if (C.mode == kClosureJudge) CU(cudaMemsetAsync(c->judge_dev, 0, 3 * sizeof(double), c->stream));
        if (c->tiles_valid)
            launch_t_resid(P, WS(c), c->G, c->T, c->K, npd_ptr(c), C, c->stream);
        else
            launch_m_resid(P, WS(c), make_nbr(c), c->K, npd_ptr(c), C, c->stream);
        if (C.mode == kClosureJudge) {
            CU(cudaMemcpyAsync(c->judge_host, c->judge_dev, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
            c->judge_pending = true;
        }
    } else {
        TRY(ensure_quot(c));
        launch_resid(P, WS(c), make_nbr(c), npd_ptr(c), quot(c), c->stream);
        c->launches++;
    }
    return FJSPH_OK;
}

DevInlet dev_inlet(const fjsph_ctx *c, const HostInlet &I) {
    DevInlet d;
    d.block = I.block;
    d.fixed_vel_or_dynamic = I.fixed_vel_or_dynamic;
    d.n_back = I.n_back;
    d.depth = I.depth;
    d.back = I.d_back;
    d.buffer = I.d_buffer;
    for (int k = 0; k < 3; ++k) d.unorm[k] = I.unorm[k];
    (void)c;
    return d;
}

void inlet_buffers(fjsph_ctx *c, const Params &P, int mode, double dt_scale) {
    for (const HostInlet &I : c->inlets) {
        if (I.n_back == 0 || I.depth == 0) continue;
        launch_inlet_buffers(P, PN(c), WS(c), c->S, dev_inlet(c, I), mode, dt_ptr(c), dt_scale, fused_pack(c),
                             c->stream);
        c->launches++;
    }
}

/* do_runge_kutta_intermediate_step on W (W already holds part_prev). stage 1, 2, 3. */
int rk_intermediate(fjsph_ctx *c, int stage, double dt_scale) {
    Params P = make_params(c);
    cudaStream_t s = c->stream;
    TRY(boundary_section(c, P, 0));
    const double sum_w = stage == 2 ? 2.0 : (stage == 3 ? 1.0 : 0.0);
    if (has_solver(c, FJSPH_DBC) || has_solver(c, FJSPH_GHOST)) {
        launch_bound_rho_update(P, PN(c), WS(c), c->S, 0, sum_w, dt_ptr(c), dt_scale, s);
        c->launches++;
    }
    TRY(resid(c, P));
    {
        Section sec(c, PASS_UPDATE);
        launch_rk_stage_update(P, PN(c), WS(c), c->S, stage, dt_ptr(c), dt_scale, fused_pack(c), s);
    }
    c->launches += 2;
    inlet_buffers(c, P, 0, dt_scale);
    after_update(c);
    c->pn_equals_W = false;
    return FJSPH_OK;
}

int rk_final(fjsph_ctx *c) {
    Params P = make_params(c);
    cudaStream_t s = c->stream;
    TRY(boundary_section(c, P, 0));
    if (has_solver(c, FJSPH_DBC) || has_solver(c, FJSPH_GHOST)) {
        launch_bound_rho_update(P, PN(c), WS(c), c->S, 1, 0.0, dt_ptr(c), 1.0, s);
        c->launches++;
    }
    TRY(resid(c, P));
    TRY(send_final_out(c));
    {
        Section sec(c, PASS_UPDATE);
        for (int k = 0; k < c->D; ++k)
            CU(cudaMemcpyAsync(c->S.xsnap[k], WS(c).x[k], sizeof(double) * c->n, cudaMemcpyDeviceToDevice, s));
        launch_rk_final_update(P, PN(c), WS(c), c->S, dt_ptr(c), fused_pack(c), s);
    }
    c->launches += 2;
    inlet_buffers(c, P, 1, 1.0);
    after_update(c);
    c->pn_equals_W = false;
    return FJSPH_OK;
}

int sq_disp(fjsph_ctx *c, double *const ref[3], double *out_host) {
    Params P = make_params(c);
    Section sec(c, PASS_REDUCE);
    launch_sq_disp_sum(P, WS(c), ref, c->S, &c->dsc->red[1], c->stream);
    c->launches += 2;
    CU(cudaMemcpyAsync(&c->hsc->red[1], &c->dsc->red[1], sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    TRY(sync(c));
    *out_host = c->hsc->red[1];
    return FJSPH_OK;
}

int set_dt_device(fjsph_ctx *c) {
    k_set_scalar<<<1, 1, 0, c->stream>>>(&c->dsc->dt, c->s.delta_t);
    c->launches++;
    return FJSPH_OK;
}
int set_npd_device(fjsph_ctx *c, double npd) {
    k_set_scalar<<<1, 1, 0, c->stream>>>(&c->dsc->npd, npd);
    c->launches++;
    return FJSPH_OK;
}

int copy_state(fjsph_ctx *c, int from, int to) {
    Section sec(c, PASS_COPY);
    launch_copy(state_fields(c->st[from], c->D), state_fields(c->st[to], c->D), c->n, c->stream);
    c->launches++;
    if (to == c->iW) mark_full(c);
    return FJSPH_OK;
}

/* find_timestep (src/Integration.cpp:370-443): reductions on the device, the scalar tail here. */
int find_timestep(fjsph_ctx *c, double *dt_out) {
    Params P = make_params(c);
    Section sec(c, PASS_REDUCE);
    launch_timestep_reduce(P, WS(c), c->S, &c->dsc->red[2], c->stream);
    c->launches += 2;
    CU(cudaMemcpyAsync(&c->hsc->red[2], &c->dsc->red[2], sizeof(double) * 7, cudaMemcpyDeviceToHost, c->stream));
    TRY(sync(c));
    double r[7];
    timestep_maxima(&c->hsc->red[2], r);
    const fjsph_settings &s = c->s;
    const bool any = c->n > c->nb;
    c->maxf = any ? r[0] : kEps;
    c->maxAf = any ? r[1] : kEps;
    c->maxdrho = any ? r[2] : kEps;
    c->maxRhoi = any ? r[3] : kEps;
    c->minST = any ? r[4] : 9999999.0;
    c->maxU = any ? r[5] : kEps;
    if ((s.variant & FJSPH_VAR_ALE) && any) c->maxShift = std::max(c->maxShift, r[6]);
    c->maxRho_pc = 100 * c->maxRhoi / s.rho_rest;
    const double kPi_ = 3.14159265358979323846;
    (void)kPi_;
    double fac[6] = {0.25 * std::sqrt(s.H / c->maxf), 2 * s.H / c->maxU, 0.125 * s.H_sq * s.rho_rest / s.mu,
                     0.067 * c->minST, 0.5 * std::sqrt(s.H / c->maxdrho), 1.5 * s.H / s.speed_sound};
    double mn = fac[0];
    for (int k = 1; k < 6; ++k)
        if (fac[k] < mn) mn = fac[k];
    c->safe_dt = 0.75 * mn;
    double dt = s.cfl * c->safe_dt;
    if (dt < s.delta_t_min)
        dt = s.delta_t_min;
    else if (dt > s.delta_t_max)
        dt = s.delta_t_max;
    if (dt > s.last_frame_time + s.frame_time_interval - s.current_time)
        dt = s.last_frame_time + s.frame_time_interval - s.current_time + s.delta_t_min;
    *dt_out = dt;
    return FJSPH_OK;
}

/* Newmark_Beta::Do_NB_Iter on W. */
int nb_iter(fjsph_ctx *c) {
    Params P = make_params(c);
    cudaStream_t s = c->stream;
    TRY(boundary_section(c, P, 1));
    TRY(resid(c, P));
    c->launches++;
    if (has_solver(c, FJSPH_DBC) || has_solver(c, FJSPH_GHOST)) {
        launch_bound_rho_update(P, PN(c), WS(c), c->S, 2, 0.0, dt_ptr(c), 1.0, s);
        c->launches++;
    }
    launch_nb_update(P, PN(c), WS(c), dt_ptr(c), s);
    c->launches++;
    inlet_buffers(c, P, 2, 1.0);
    mark_all(c);
    c->pn_equals_W = false;
    return FJSPH_OK;
}

/* Newmark_Beta::Check_Error (src/Newmark_Beta.cpp:10-52); xih is S.xsnap. */
int nb_check_error(fjsph_ctx *c, double &rms_error, double &logbase, int &state) {
    double errsum = 0.0;
    TRY(sq_disp(c, c->S.xsnap, &errsum));
    const double nf = double(c->n - c->nb);
    const double log_error = std::log10(std::sqrt(errsum / nf));
    if (c->iteration == 0) logbase = log_error;
    rms_error = log_error - logbase;
    state = 0;
    if ((int64_t)c->iteration > (int64_t)c->s.max_subits) {
        if (rms_error > 0.0) {
            TRY(copy_state(c, c->ipn, c->iW));
            TRY(search(c));
            c->s.delta_t = 0.5 * c->s.delta_t;
            TRY(set_dt_device(c));
            c->iteration = 0;
            rms_error = 0.0;
            state = -1;
            return FJSPH_OK;
        }
        state = 1;
    }
    return FJSPH_OK;
}

int save_xsnap(fjsph_ctx *c) {
    for (int k = 0; k < c->D; ++k)
        CU(cudaMemcpyAsync(c->S.xsnap[k], WS(c).x[k], sizeof(double) * c->n, cudaMemcpyDeviceToDevice, c->stream));
    return FJSPH_OK;
}

int newmark_beta_loop(fjsph_ctx *c, double &logbase, double &rms_error) {
    rms_error = 0.0;
    int restarts = 0;
    while (rms_error > c->s.min_residual) {
        TRY(save_xsnap(c));
        TRY(nb_iter(c));
        int st = 0;
        TRY(nb_check_error(c, rms_error, logbase, st));
        if (st == 0)
            c->iteration++;
        else if (st == 1)
            break;
        else if (++restarts > 64)
            return FJSPH_E_NONFINITE; /* the reference would halve dt without bound here */
    }
    return FJSPH_OK;
}

int get_first_rk(fjsph_ctx *c, double &logbase) {
    TRY(set_dt_device(c));
    if (!c->pn_equals_W) TRY(copy_state(c, c->ipn, c->iW));
    TRY(rk_intermediate(c, 1, 0.5));
    double e = 0.0;
    TRY(sq_disp(c, PN(c).x, &e));
    logbase = std::log10(std::sqrt(e / double(c->n - c->nb)));
    return FJSPH_OK;
}

int runge_kutta4(fjsph_ctx *c, double logbase, double &rms) {
    TRY(set_dt_device(c));
    Params P = make_params(c);
    launch_rk_init_sums(P, PN(c), WS(c), c->S, c->stream);
    c->launches++;
    TRY(rk_intermediate(c, 2, 0.5));
    TRY(rk_intermediate(c, 3, 1.0));
    TRY(rk_final(c));
    double e = 0.0;
    TRY(sq_disp(c, c->S.xsnap, &e));
    rms = std::log10(std::sqrt(e / double(c->n - c->nb))) - logbase;
    return FJSPH_OK;
}


/* Integrator::integrate_no_update (src/Integration.cpp:27-107).  skip_dead: under Runge-Kutta the
 * first pre-pass results on pnp1 are overwritten by Get_First_RK's copy of pn before anything
 * reads them, except npd; the whole-step path then only computes npd. */
int integrate_no_update(fjsph_ctx *c, double &rms_error, bool skip_dead) {
    c->iteration = 0;
    double logbase = 0.0;
    rms_error = 0.0;
    double dt = 0.0;
    if (c->in_wait[kInPos]) {
        /* a fjsph_step_host upload in flight: its positions land first, so the search runs while
         * the time-step reduction's inputs travel.  The search reads neither the time step nor
         * those inputs, and the reduction (maxima and a minimum) gives the same bits in any
         * particle order, so the results are those of the reference order. */
        TRY(search(c));
        TRY(apply_in(c, kInStep));
        TRY(find_timestep(c, &dt));
        c->s.delta_t = dt;
        TRY(set_dt_device(c));
    } else {
        TRY(apply_in(c, kInStep));
        TRY(find_timestep(c, &dt));
        c->s.delta_t = dt;
        TRY(set_dt_device(c));
        TRY(search(c));
    }
    TRY(apply_in(c, kInPack));
    const bool rk = c->s.solver_type == FJSPH_RUNGE_KUTTA;
    if (rk && skip_dead) {
        if (c->s.st_model == FJSPH_ST_PAIRWISE) {
            Params P = make_params(c);
            TRY(npd_only(c, P));
        }
        TRY(apply_in(c, kInLate));
    } else {
        TRY(apply_in(c, kInLate));
        TRY(prestep_passes(c));
    }
    if (rk) {
        TRY(get_first_rk(c, logbase));
    } else {
        TRY(save_xsnap(c));
        TRY(nb_iter(c));
        int st = 0;
        TRY(nb_check_error(c, rms_error, logbase, st));
        c->iteration++;
    }
    TRY(search(c));
    TRY(prestep_passes(c));
    if (rk) {
        TRY(send_early_out(c));
        TRY(runge_kutta4(c, logbase, rms_error));
    } else {
        TRY(newmark_beta_loop(c, logbase, rms_error));
    }
    return FJSPH_OK;
}

/* update_buffer_region (src/shapes/inlet.cpp:578-640) for every inlet block, in block and
 * column order: a BACK particle past the insertion plane becomes PIPE, the column's first
 * BUFFER particle becomes BACK and the column shifts; while the particle count is below
 * max_points (and the context capacity), a new BUFFER particle one dx upstream of the column's
 * last one is inserted at the end of the block's reference range. */
int inlet_advance(fjsph_ctx *c, bool &moved) {
    moved = false;
    if (c->inlets.empty()) return FJSPH_OK;
    const int64_t limit = std::min<int64_t>(c->s.max_points, c->cap);
    const int64_t n_old = c->n;
    int64_t n_new = c->n;
    std::vector<InsertOp> ops;
    std::vector<int64_t> ins(c->blocks.size(), 0);
    std::vector<HostInlet *> order;
    for (HostInlet &I : c->inlets) order.push_back(&I);
    std::sort(order.begin(), order.end(), [](HostInlet *a, HostInlet *b) { return a->block < b->block; });
    int32_t *flag = c->upd_i32;
    for (HostInlet *Ip : order) {
        HostInlet &I = *Ip;
        fjsph_block &B = c->blocks[I.block];
        if (B.block_type != kInletZone || I.n_back == 0 || I.depth == 0) continue;
        launch_inlet_cross(WS(c), c->D, I.d_back, I.n_back, B.insert_norm, B.insconst, flag, c->stream);
        c->launches++;
        std::vector<int32_t> f(I.n_back), back(I.n_back), buf(I.n_back * I.depth);
        CU(cudaMemcpyAsync(f.data(), flag, sizeof(int32_t) * I.n_back, cudaMemcpyDeviceToHost, c->stream));
        CU(cudaMemcpyAsync(back.data(), I.d_back, sizeof(int32_t) * I.n_back, cudaMemcpyDeviceToHost, c->stream));
        CU(cudaMemcpyAsync(buf.data(), I.d_buffer, sizeof(int32_t) * buf.size(), cudaMemcpyDeviceToHost, c->stream));
        TRY(sync(c));
        bool changed = false;
        for (int64_t ii = 0; ii < I.n_back; ++ii) {
            if (!f[ii]) continue;
            changed = true;
            int32_t *col = &buf[ii * I.depth];
            InsertOp op{};
            op.to_pipe = back[ii];
            op.to_back = col[0];
            back[ii] = col[0];
            for (int64_t jj = 0; jj + 1 < I.depth; ++jj) col[jj] = col[jj + 1];
            op.dst = -1;
            if (n_new < limit) {
                op.src = col[I.depth - 1]; /* the column's last particle before the shift */
                op.dst = (int32_t)n_new;
                op.block = I.block;
                op.key = B.second;
                op.part_id = c->part_id_next++;
                for (int k = 0; k < 3; ++k) op.norm[k] = B.insert_norm[k];
                col[I.depth - 1] = (int32_t)n_new;
                ++n_new;
                ++ins[I.block];
                B.second++;
                for (size_t jb = I.block + 1; jb < c->blocks.size(); ++jb) {
                    c->blocks[jb].first++;
                    c->blocks[jb].second++;
                }
            }
            ops.push_back(op);
        }
        if (changed) {
            CU(cudaMemcpyAsync(I.d_back, back.data(), sizeof(int32_t) * I.n_back, cudaMemcpyHostToDevice, c->stream));
            CU(cudaMemcpyAsync(I.d_buffer, buf.data(), sizeof(int32_t) * buf.size(), cudaMemcpyHostToDevice, c->stream));
        }
    }
    if (ops.empty()) return FJSPH_OK;
    moved = true;
    /* existing particles of later blocks move up by the insertions before them */
    BlockShift sh{};
    int64_t acc = 0;
    for (size_t b = 0; b < c->blocks.size() && b < (size_t)kMaxBlocks; ++b) {
        sh.v[b] = acc;
        acc += ins[b];
    }
    if (acc > 0) {
        launch_shift_keys(c->key, c->blk, n_old, sh, c->stream);
        c->launches++;
    }
    InsertOp *d_ops = reinterpret_cast<InsertOp *>(c->stage);
    CU(cudaMemcpyAsync(d_ops, ops.data(), sizeof(InsertOp) * ops.size(), cudaMemcpyHostToDevice, c->stream));
    c->n = n_new;
    launch_insert(WS(c), c->D, d_ops, (int64_t)ops.size(), c->s.dx, c->stream);
    c->launches++;
    if (c->packed_alloc && n_new > n_old) /* new BUFFER particles carry no occlusion inputs */
        CU(cudaMemsetAsync(c->K.O + n_old, 0, sizeof(float4) * (n_new - n_old), c->stream));
    c->inserted += n_new - n_old;
    TRY(sync(c)); /* the host vector `ops` is released on return */
    return FJSPH_OK;
}

/* Deletion past the fluid blocks' deletion planes (src/Integration.cpp:127-205, analytic air
 * source): deleted slots are compacted out in slot order and the remaining reference indices
 * close up. */
int delete_particles(fjsph_ctx *c) {
    DeletePlanes DP{};
    DP.lost = c->s.asource == FJSPH_MESH_INFL ? 1 : 0;
    bool any = DP.lost != 0;
    for (size_t b = c->n_bound_blocks; b < c->blocks.size() && b < (size_t)kMaxBlocks; ++b) {
        const fjsph_block &B = c->blocks[b];
        if (B.delconst == kDefaultVal) continue;
        DP.on[b] = 1;
        for (int k = 0; k < 3; ++k) DP.norm[b][k] = B.delete_norm[k];
        DP.c[b] = B.delconst;
        any = true;
    }
    if (!any || c->n == 0) return FJSPH_OK;
    const int64_t n = c->n;
    cudaStream_t s = c->stream;
    int32_t *flag = c->upd_i32, *keep = flag + n, *keep_ex = keep + n, *by_ref = keep_ex + n + 1;
    CU(cudaMemsetAsync(c->upd_cnt, 0, sizeof(unsigned long long) * kMaxBlocks, s));
    Params P = make_params(c);
    launch_delete_flags(P, WS(c), DP, flag, keep, c->upd_cnt, s);
    std::vector<unsigned long long> cnt(kMaxBlocks);
    CU(cudaMemcpyAsync(cnt.data(), c->upd_cnt, sizeof(unsigned long long) * kMaxBlocks, cudaMemcpyDeviceToHost, s));
    TRY(sync(c));
    int64_t total = 0;
    for (unsigned long long v : cnt) total += (int64_t)v;
    c->launches++;
    if (total == 0) return FJSPH_OK;
    /* new slots (stable order of the kept ones) and closed-up reference indices */
    int64_t *ref_ex = c->nbr_off; /* the lists are rebuilt at the next search */
    launch_scan_i32(keep, keep_ex, n, c->G.scan_tmp, s);
    launch_compact_map(flag, c->key, n, by_ref, nullptr, nullptr, nullptr, nullptr, 0, s);
    launch_scan_i64(by_ref, ref_ex, n, c->scan_tmp64, s);
    launch_compact_map(flag, c->key, n, by_ref, keep_ex, ref_ex, c->new_of_old, c->key, 1, s);
    c->launches += 8;
    launch_permute(state_fields(WS(c), c->D), state_fields(c->st[c->isp], c->D), c->new_of_old, n, s);
    std::swap(c->iW, c->isp);
    DevState &spare = c->st[c->isp];
    launch_permute_key_blk(c->key, c->blk, spare.part_id, spare.b, c->new_of_old, n, s);
    const int64_t n2 = n - total;
    CU(cudaMemcpyAsync(c->key, spare.part_id, sizeof(int64_t) * n2, cudaMemcpyDeviceToDevice, s));
    CU(cudaMemcpyAsync(c->blk, spare.b, sizeof(int32_t) * n2, cudaMemcpyDeviceToDevice, s));
    if (c->packed_alloc && c->occ_valid) {
        float4 *tmp = reinterpret_cast<float4 *>(c->stage);
        launch_m_permute_f4(c->K.O, tmp, c->new_of_old, n, s);
        CU(cudaMemcpyAsync(c->K.O, tmp, sizeof(float4) * n2, cudaMemcpyDeviceToDevice, s));
    }
    for (HostInlet &I : c->inlets) {
        launch_remap_i32(I.d_back, I.n_back, c->new_of_old, s);
        launch_remap_i32(I.d_buffer, I.n_back * I.depth, c->new_of_old, s);
    }
    c->launches += 4;
    int64_t shift = 0;
    for (size_t b = c->n_bound_blocks; b < c->blocks.size(); ++b) {
        fjsph_block &B = c->blocks[b];
        B.first -= shift;
        if (b < (size_t)kMaxBlocks) shift += (int64_t)cnt[b];
        B.second -= shift;
    }
    c->n = n2;
    c->deleted += total;
    return sync(c);
}

/* Integrator::update_data (src/Integration.cpp:109-226): insertion, zero-density guard
 * (:116-124), deletion; the neighbour lists and packed inputs are stale afterwards. */
int update_data(fjsph_ctx *c) {
    const int64_t n0 = c->n;
    bool moved = false;
    TRY(inlet_advance(c, moved));
    launch_density_guard(make_params(c), WS(c), fused_pack(c), c->stream);
    c->launches++;
    TRY(delete_particles(c));
    if (c->n != n0) {
        c->nbr_valid = false;
        mark_full(c);
    }
    if (moved) mark_all(c); /* inlet columns advanced: types changed, particles inserted */
    return FJSPH_OK;
}

/* Integrator::integrate (src/Integration.cpp:233-303). */
int integrate(fjsph_ctx *c, double &step_error) {
    /* judge / log schedule of the closure: the first residual of every n-th step */
    const int64_t k = c->closure_steps++;
    if (learned_active(c) && c->s.learned_judge_interval > 0 && k % c->s.learned_judge_interval == 0)
        c->arm = FJSPH_CLOSURE_ARM_JUDGE;
    else if (!learned_active(c) && c->log_cap > 0 && c->log_every > 0 && k % c->log_every == 0)
        c->arm = FJSPH_CLOSURE_ARM_LOG;
    else
        c->arm = 0;
    TRY(integrate_no_update(c, step_error, true));
    c->arm = 0;
    TRY(closure_collect(c));
    join_id_scan(c); /* insertion numbers new particles from the uploaded ids */
    TRY(update_data(c));
    TRY(send_last_out(c));
    TRY(copy_state(c, c->iW, c->ipn));
    c->pn_equals_W = true;
    fjsph_settings &I = c->s;
    I.current_time += I.delta_t;
    if (step_error > I.min_residual || c->maxRho_pc > I.rho_max_iter) {
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
    if (c->iteration < I.subits_factor * I.max_subits && I.n_unstable == 0) {
        if (I.n_stable > I.n_stable_limit) {
            I.cfl = std::min(I.cfl_max, I.cfl + I.cfl_step);
            I.n_stable = 0;
        } else
            I.n_stable++;
    } else
        I.n_stable = 0;
    return FJSPH_OK;
}

/* ---- independent simulations sharing the context (groups) ------------------------------------ */
GroupConst group_const(const fjsph_ctx *c) {
    const fjsph_settings &s = c->s;
    GroupConst K;
    K.rho_rest = s.rho_rest;
    K.H = s.H;
    K.H_sq = s.H_sq;
    K.mu = s.mu;
    K.speed_sound = s.speed_sound;
    K.dt_min = s.delta_t_min;
    K.dt_max = s.delta_t_max;
    K.last_frame_time = s.last_frame_time;
    K.frame_interval = s.frame_time_interval;
    K.min_residual = s.min_residual;
    K.rho_max_iter = s.rho_max_iter;
    K.cfl_min = s.cfl_min;
    K.cfl_max = s.cfl_max;
    K.cfl_step = s.cfl_step;
    K.subits_factor = s.subits_factor;
    K.max_subits = s.max_subits;
    K.n_stable_limit = s.n_stable_limit;
    K.n_unstable_limit = s.n_unstable_limit;
    K.ale = (s.variant & FJSPH_VAR_ALE) ? 1 : 0;
    return K;
}

/* find_timestep per group: reductions and the scalar tail on the device */
int group_timestep(fjsph_ctx *c) {
    Params P = make_params(c);
    Section sec(c, PASS_REDUCE);
    launch_group_timestep(P, WS(c), c->g_red, c->ngrp, c->stream);
    launch_group_dt(c->gs, c->g_red, c->ngrp, group_const(c), c->stream);
    c->launches += 3;
    return FJSPH_OK;
}

/* log10 RMS position change per group against ref: mode 0 sets logbase, mode 1 the error */
int group_err(fjsph_ctx *c, double *const ref[3], int mode) {
    Params P = make_params(c);
    Section sec(c, PASS_REDUCE);
    CU(cudaMemsetAsync(c->g_sum, 0, sizeof(double) * c->ngrp, c->stream));
    launch_group_sq_disp(P, WS(c), ref, c->g_sum, c->stream);
    launch_group_err(c->gs, c->g_sum, c->ngrp, mode, c->stream);
    c->launches += 3;
    return FJSPH_OK;
}

/* One Integrator::integrate of every group (Runge-Kutta, no insertion or deletion): the same
 * pass sequence as the single-simulation step, with every scalar decision made per group on the
 * device, so nothing waits for the host. */
int group_step(fjsph_ctx *c) {
    TRY(group_timestep(c));
    TRY(search(c));
    if (c->s.st_model == FJSPH_ST_PAIRWISE) TRY(npd_only(c, make_params(c)));
    if (!c->pn_equals_W) TRY(copy_state(c, c->ipn, c->iW));
    TRY(rk_intermediate(c, 1, 0.5));
    TRY(group_err(c, PN(c).x, 0));
    TRY(search(c));
    TRY(prestep_passes(c));
    launch_rk_init_sums(make_params(c), PN(c), WS(c), c->S, c->stream);
    c->launches++;
    TRY(rk_intermediate(c, 2, 0.5));
    TRY(rk_intermediate(c, 3, 1.0));
    TRY(rk_final(c));
    TRY(group_err(c, c->S.xsnap, 1));
    launch_density_guard(make_params(c), WS(c), nullptr, c->stream);
    c->launches++;
    mark_all(c);
    TRY(copy_state(c, c->iW, c->ipn));
    c->pn_equals_W = true;
    launch_group_adapt(c->gs, c->ngrp, group_const(c), c->stream);
    c->launches++;
    return FJSPH_OK;
}

/* group of every slot from its reference index */
int upload_groups(fjsph_ctx *c) {
    if (!grouped(c) || c->n == 0) return FJSPH_OK;
    std::vector<int64_t> keys;
    TRY(download_keys(c, keys));
    std::vector<int32_t> g(c->n);
    for (int64_t s = 0; s < c->n; ++s) {
        const auto it = std::upper_bound(c->grp_first.begin(), c->grp_first.end(), keys[s]);
        g[s] = (int32_t)(it - c->grp_first.begin()) - 1;
    }
    CU(cudaMemcpy(c->grp, g.data(), sizeof(int32_t) * c->n, cudaMemcpyHostToDevice));
    return FJSPH_OK;
}

int graph_release(fjsph_ctx *c) {
    for (cudaGraphExec_t &g : c->graph)
        if (g) {
            CU(cudaGraphExecDestroy(g));
            g = nullptr;
        }
    return FJSPH_OK;
}

/* which searches of the next step re-order the particles (bit 0: first, bit 1: second) */
int graph_variant(const fjsph_ctx *c) {
    const int64_t iv = c->s.reorder_interval;
    if (iv <= 0) return 0;
    return ((c->searches % iv) == 0 ? 1 : 0) | (((c->searches + 1) % iv) == 0 ? 2 : 0);
}

int check_ctx(fjsph_ctx *c) { return c ? FJSPH_OK : FJSPH_E_ARG; }
int need_state(fjsph_ctx *c) { return (c && c->n > 0) ? FJSPH_OK : FJSPH_E_STATE; }
int need_nbr(fjsph_ctx *c) {
    if (!c || c->n == 0) return FJSPH_E_STATE;
    return c->nbr_valid ? FJSPH_OK : FJSPH_E_STATE;
}

} // namespace

/* ================================================================================================ */
extern "C" {

const char *fjsph_status_string(int status) {
    switch (status) {
    case FJSPH_OK:
        return "ok";
    case FJSPH_E_ARG:
        return "invalid argument";
    case FJSPH_E_CUDA:
        return "CUDA runtime error";
    case FJSPH_E_CAPACITY:
        return "particle count above context capacity";
    case FJSPH_E_NEIGHBOUR:
        return "neighbour list storage exhausted";
    case FJSPH_E_NONFINITE:
        return "non-finite values or divergent integration";
    case FJSPH_E_UNSUPPORTED:
        return "unsupported option or variant combination";
    case FJSPH_E_STATE:
        return "call order error";
    default:
        return "unknown status";
    }
}

int fjsph_ctx_create(const fjsph_settings *s, int64_t capacity, fjsph_ctx **out) {
    if (!out) return FJSPH_E_ARG;
    *out = nullptr;
    TRY(validate_settings(s));
    if (capacity <= 0 || capacity >= ((int64_t)1 << 31)) return FJSPH_E_ARG;
    fjsph_ctx *c = new fjsph_ctx();
    c->s = *s;
    c->D = s->dim;
    c->cap = capacity;
    auto fail = [&](int r) {
        fjsph_ctx_destroy(c);
        return r;
    };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(FJSPH_E_CUDA);
    int r = FJSPH_OK;
#define A(call)                  \
    do {                         \
        r = (call);              \
        if (r != FJSPH_OK) return fail(r); \
    } while (0)
    A(dalloc(c, &c->key, capacity));
    A(dalloc(c, &c->blk, capacity));
    for (int i = 0; i < 3; ++i) A(alloc_state(c, c->st[i]));
    for (int k = 0; k < c->D; ++k) {
        A(dalloc(c, &c->xs[k], capacity));
        A(dalloc(c, &c->nrm_tmp[k], capacity));
        A(dalloc(c, &c->vtmp[k], capacity));
        A(dalloc(c, &c->S.Sx[k], capacity));
        A(dalloc(c, &c->S.Sv[k], capacity));
        A(dalloc(c, &c->S.xsnap[k], capacity));
    }
    A(dalloc(c, &c->S.Sr, capacity));
    A(dalloc(c, &c->S.near_inlet, capacity));
    c->S.part_len = 16 * 1216;
    A(dalloc(c, &c->S.part, c->S.part_len));
    A(dalloc(c, &c->npd_part, capacity));
    A(dalloc(c, &c->stage, capacity * 9));
    A(dalloc(c, &c->stage2, capacity * 9));
    CellGrid &G = c->G;
    A(dalloc(c, &G.hash, capacity));
    A(dalloc(c, &G.frac, capacity));
    A(dalloc(c, &G.hash2, capacity));
    A(dalloc(c, &G.frac2, capacity));
    A(alloc_table(c, next_pow2(std::max<int64_t>(2 * capacity, kMinTable))));
    A(dalloc(c, &G.sorted, capacity));
    A(dalloc(c, &G.sorted_hi, capacity));
    A(dalloc(c, &G.sorted_lo, capacity));
    A(dalloc(c, &G.bbox, 8));
    A(dalloc(c, &G.grid, 8));
    A(dalloc(c, &c->nbr_counts, capacity));
    A(dalloc(c, &c->nbr_off, capacity + 1));
    A(dalloc(c, &c->slice_w, capacity / kSlice + 2));
    A(dalloc(c, &c->slice_off, capacity / kSlice + 3));
    c->scan_tmp64_len = capacity / 2048 + 16;
    A(dalloc(c, &c->scan_tmp64, c->scan_tmp64_len));
    c->nbr_cap = capacity * (c->D == 3 ? 96 : 28);
    A(dalloc(c, &c->nbr_idx, c->nbr_cap));
    A(dalloc(c, &c->new_of_old, capacity));
    c->reorder_tmp_len = 2 * capacity + 1 + capacity / 2048 + 16;
    A(dalloc(c, &c->reorder_tmp, c->reorder_tmp_len));
    A(dalloc(c, &c->dsc, 1));
    A(dalloc(c, &c->upd_i32, 4 * capacity + 64));
    A(dalloc(c, &c->upd_cnt, kMaxBlocks));
    if (s->precision == FJSPH_PREC_MIXED) A(alloc_packed(c));
#undef A
    if (cudaMallocHost(&c->hsc, sizeof(DevScalars)) != cudaSuccess) return fail(FJSPH_E_CUDA);
    std::memset(c->hsc, 0, sizeof(DevScalars));
    if (cudaMemsetAsync(c->dsc, 0, sizeof(DevScalars), c->stream) != cudaSuccess) return fail(FJSPH_E_CUDA);
    if (cudaMemsetAsync(c->S.near_inlet, 0, sizeof(int32_t) * capacity, c->stream) != cudaSuccess)
        return fail(FJSPH_E_CUDA);
    for (int k = 0; k < c->D; ++k)
        if (cudaMemsetAsync(c->nrm_tmp[k], 0, sizeof(double) * capacity, c->stream) != cudaSuccess)
            return fail(FJSPH_E_CUDA);
    if (sync(c) != FJSPH_OK) return fail(FJSPH_E_CUDA);
    *out = c;
    return FJSPH_OK;
}

int fjsph_ctx_destroy(fjsph_ctx *c) {
    if (!c) return FJSPH_E_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    graph_release(c);
    for (HostInlet &I : c->inlets) {
        if (I.d_back) cudaFree(I.d_back);
        if (I.d_buffer) cudaFree(I.d_buffer);
    }
    for (void *p : c->allocs) cudaFree(p);
    for (cudaEvent_t e : c->prof.pool) cudaEventDestroy(e);
    for (cudaEvent_t e : c->user_ev)
        if (e) cudaEventDestroy(e);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    for (int b = 0; b < 2; ++b) {
        if (c->st_copied[b]) cudaEventDestroy(c->st_copied[b]);
        if (c->st_used[b]) cudaEventDestroy(c->st_used[b]);
    }
    join_id_scan(c);
    for (cudaEvent_t e : c->in_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : c->in_placed)
        if (e) cudaEventDestroy(e);
    if (c->place_after) cudaEventDestroy(c->place_after);
    if (c->place_stream) {
        cudaStreamSynchronize(c->place_stream);
        cudaStreamDestroy(c->place_stream);
    }
    if (c->out_ready) cudaEventDestroy(c->out_ready);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->hsc) cudaFreeHost(c->hsc);
    if (c->judge_host) cudaFreeHost(c->judge_host);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FJSPH_OK;
}

int fjsph_set_settings(fjsph_ctx *c, const fjsph_settings *s) {
    TRY(check_ctx(c));
    TRY(validate_settings(s));
    if (s->dim != c->D) return FJSPH_E_ARG;
    const bool was_mixed = mixed(c);
    c->s = *s;
    if (mixed(c)) {
        TRY(alloc_packed(c));
        if (!was_mixed) {
            mark_full(c);
            c->nbr_valid = false; /* the lists need their FP32 squared distances */
        }
    }
    return FJSPH_OK;
}

int fjsph_get_settings(fjsph_ctx *c, fjsph_settings *s) {
    TRY(check_ctx(c));
    if (!s) return FJSPH_E_ARG;
    *s = c->s;
    return FJSPH_OK;
}

int fjsph_set_limits(fjsph_ctx *c, const fjsph_block *blocks, int32_t nblocks, int64_t n_bound_blocks) {
    TRY(check_ctx(c));
    if (!blocks || nblocks <= 0 || nblocks > kMaxBlocks || n_bound_blocks < 0 || n_bound_blocks > nblocks)
        return FJSPH_E_ARG;
    std::vector<fjsph_block> b(blocks, blocks + nblocks);
    int64_t expect = 0;
    for (int32_t i = 0; i < nblocks; ++i) {
        if (b[i].first != expect || b[i].second < b[i].first) return FJSPH_E_ARG;
        if ((i < n_bound_blocks) == (b[i].is_fluid != 0)) return FJSPH_E_ARG;
        if (b[i].n_times < 0 || b[i].n_times > FJSPH_MAX_TIMES) return FJSPH_E_ARG;
        expect = b[i].second;
    }
    c->blocks = b;
    c->n_bound_blocks = n_bound_blocks;
    c->nb = n_bound_blocks > 0 ? b[n_bound_blocks - 1].second : 0;
    if (c->n > 0) {
        if (expect != c->n) return FJSPH_E_ARG;
        std::vector<int64_t> keys;
        TRY(download_keys(c, keys));
        TRY(upload_blk(c, keys));
    }
    return FJSPH_OK;
}

int fjsph_set_inlet(fjsph_ctx *c, const fjsph_inlet *in) {
    TRY(check_ctx(c));
    if (!in || in->block < 0 || in->block >= (int32_t)c->blocks.size() || in->n_back < 0 || in->depth < 0)
        return FJSPH_E_ARG;
    if ((in->n_back > 0 && !in->back) || (in->n_back * in->depth > 0 && !in->buffer)) return FJSPH_E_ARG;
    HostInlet I;
    for (HostInlet &old : c->inlets)
        if (old.block == in->block) {
            if (old.d_back) cudaFree(old.d_back);
            if (old.d_buffer) cudaFree(old.d_buffer);
            old.d_back = old.d_buffer = nullptr;
            old.block = -1;
        }
    c->inlets.erase(std::remove_if(c->inlets.begin(), c->inlets.end(), [](const HostInlet &h) { return h.block < 0; }),
                    c->inlets.end());
    const fjsph_block &B = c->blocks[in->block];
    I.block = in->block;
    I.fixed_vel_or_dynamic = B.fixed_vel_or_dynamic;
    I.n_back = in->n_back;
    I.depth = in->depth;
    I.back_ref.assign(in->back, in->back + in->n_back);
    I.buffer_ref.assign(in->buffer, in->buffer + in->n_back * in->depth);
    double nrm = 0.0;
    for (int k = 0; k < c->D; ++k) nrm += B.insert_norm[k] * B.insert_norm[k];
    nrm = std::sqrt(nrm);
    for (int k = 0; k < 3; ++k) I.unorm[k] = nrm > 0 ? B.insert_norm[k] / nrm : B.insert_norm[k];
    CU(cudaMalloc(&I.d_back, sizeof(int32_t) * std::max<int64_t>(I.n_back, 1)));
    CU(cudaMalloc(&I.d_buffer, sizeof(int32_t) * std::max<int64_t>(I.n_back * I.depth, 1)));
    c->inlets.push_back(I);
    if (c->n > 0) {
        std::vector<int64_t> keys;
        TRY(download_keys(c, keys));
        TRY(upload_inlets(c, keys));
    }
    return FJSPH_OK;
}

int fjsph_get_inlet(fjsph_ctx *c, fjsph_inlet *in) {
    TRY(check_ctx(c));
    if (!in) return FJSPH_E_ARG;
    for (HostInlet &I : c->inlets)
        if (I.block == in->block) {
            in->n_back = I.n_back;
            in->depth = I.depth;
            if (!in->back && !in->buffer) return FJSPH_OK;
            if (c->n == 0) { /* no state yet: the tables as given */
                if (in->back) std::copy(I.back_ref.begin(), I.back_ref.end(), in->back);
                if (in->buffer) std::copy(I.buffer_ref.begin(), I.buffer_ref.end(), in->buffer);
                return FJSPH_OK;
            }
            /* current tables: device slots -> reference indices */
            TRY(sync(c));
            std::vector<int64_t> keys;
            TRY(download_keys(c, keys));
            std::vector<int32_t> b(I.n_back), f(I.n_back * I.depth);
            if (!b.empty()) CU(cudaMemcpy(b.data(), I.d_back, sizeof(int32_t) * b.size(), cudaMemcpyDeviceToHost));
            if (!f.empty()) CU(cudaMemcpy(f.data(), I.d_buffer, sizeof(int32_t) * f.size(), cudaMemcpyDeviceToHost));
            for (size_t k = 0; k < b.size(); ++k)
                if (in->back) in->back[k] = (b[k] >= 0 && b[k] < c->n) ? keys[b[k]] : -1;
            for (size_t k = 0; k < f.size(); ++k)
                if (in->buffer) in->buffer[k] = (f[k] >= 0 && f[k] < c->n) ? keys[f[k]] : -1;
            return FJSPH_OK;
        }
    return FJSPH_E_ARG;
}

int fjsph_get_limits(fjsph_ctx *c, fjsph_block *blocks, int32_t max_blocks, int32_t *nblocks) {
    TRY(check_ctx(c));
    if (nblocks) *nblocks = (int32_t)c->blocks.size();
    if (!blocks) return FJSPH_OK;
    if (max_blocks < (int32_t)c->blocks.size()) return FJSPH_E_ARG;
    std::copy(c->blocks.begin(), c->blocks.end(), blocks);
    return FJSPH_OK;
}

int fjsph_update_counts(fjsph_ctx *c, int64_t *inserted, int64_t *deleted) {
    TRY(check_ctx(c));
    if (inserted) *inserted = c->inserted;
    if (deleted) *deleted = c->deleted;
    return FJSPH_OK;
}

/* The bookkeeping of an upload before its fields move: checks, a new particle set's keys, block
 * and inlet tables, and the scan of the ids (on a second thread while the fields transfer). */
int upload_begin(fjsph_ctx *c, const fjsph_state_view *st, std::thread &ids, int64_t &id_next, bool scan_ids = true) {
    TRY(sync(c));
    if (st->n < 0) return FJSPH_E_ARG;
    if (st->n > c->cap) return FJSPH_E_CAPACITY;
    if (c->blocks.empty()) return FJSPH_E_STATE;
    if (c->blocks.back().second != st->n) return FJSPH_E_ARG;
    c->occ_valid = false; /* occlusion statistics belong to the previous state */
    TRY(graph_release(c));
    std::vector<int64_t> keys;
    if (st->n != c->n || c->n == 0) {
        /* new particle set: identity mapping, re-sort at the next search */
        c->n = st->n;
        keys.resize(c->n);
        for (int64_t i = 0; i < c->n; ++i) keys[i] = i;
        if (c->n) CU(cudaMemcpy(c->key, keys.data(), sizeof(int64_t) * c->n, cudaMemcpyHostToDevice));
        TRY(upload_blk(c, keys));
        TRY(upload_inlets(c, keys));
        c->reorder_pending = true;
    }
    /* ids of inserted particles continue from the largest uploaded one */
    if (scan_ids && st->part_id)
        ids = std::thread([&id_next, st] {
            int64_t m = 0;
            for (int64_t i = 0; i < st->n; ++i) m = std::max<int64_t>(m, st->part_id[i] + 1);
            id_next = m;
        });
    return FJSPH_OK;
}

/* The bookkeeping after the fields of an upload are enqueued. */
int upload_end(fjsph_ctx *c, int32_t which, const fjsph_state_view *st, std::thread *ids, int64_t id_next) {
    if (ids && ids->joinable()) ids->join();
    if (grouped(c)) TRY(upload_groups(c));
    if (ids && which != FJSPH_PN && st->part_id) c->part_id_next = id_next;
    if (which != FJSPH_PN) {
        c->nbr_valid = false;
        mark_full(c);
    }
    c->pn_equals_W = which == FJSPH_BOTH;
    return FJSPH_OK;
}

int fjsph_state_upload(fjsph_ctx *c, int32_t which, const fjsph_state_view *st) {
    TRY(check_ctx(c));
    if (!st || (which != FJSPH_PN && which != FJSPH_PNP1 && which != FJSPH_BOTH)) return FJSPH_E_ARG;
    int64_t id_next = 0;
    std::thread ids;
    TRY(upload_begin(c, st, ids, id_next, which != FJSPH_PN));
    /* FJSPH_BOTH: pn = pnp1 = the uploaded state: one host transfer, each field copied on the
     * device as it arrives */
    const int rc_t = transfer(c, which == FJSPH_PN ? PN(c) : WS(c), st, true, which == FJSPH_BOTH ? &PN(c) : nullptr);
    if (rc_t != FJSPH_OK) {
        if (ids.joinable()) ids.join();
        return rc_t;
    }
    TRY(upload_end(c, which, st, &ids, id_next));
    return sync(c);
}

int fjsph_state_download(fjsph_ctx *c, int32_t which, fjsph_state_view *st) {
    TRY(need_state(c));
    if (!st || (which != FJSPH_PN && which != FJSPH_PNP1)) return FJSPH_E_ARG;
    if (st->n != c->n) return FJSPH_E_ARG;
    TRY(sync(c));
    return transfer(c, which == FJSPH_PN ? PN(c) : WS(c), st, false);
}

int fjsph_step_host(fjsph_ctx *c, const fjsph_state_view *in, fjsph_state_view *out, double *rms_error) {
    TRY(check_ctx(c));
    if (!in || !out) return FJSPH_E_ARG;
    if (c->ngrp > 0) return FJSPH_E_STATE; /* independent simulations step through the groups */
    for (const auto &g : c->in_grp)
        if (!g.empty()) return FJSPH_E_STATE;
    std::vector<void *> hp;
    view_ptrs(in, hp);
    if (!in->xi) return FJSPH_E_ARG; /* positions at least */
    /* pn = pnp1 = in: the bookkeeping of an upload now, the fields on the copy stream in four
     * groups, each applied just before the pass that first reads it */
    join_id_scan(c);
    TRY(upload_begin(c, in, c->id_scan, c->id_scan_next));
    std::vector<std::vector<void *>> dp;
    std::vector<int> type;
    dev_ptrs(WS(c), c->D, dp, type);
    const int64_t n = c->n;
    int64_t need = 0;
    for (size_t f = 0; f < hp.size(); ++f)
        if (hp[f]) need += ((type[f] == 2 ? 4 : 8) * (int64_t)dp[f].size() * n + 15) / 16 * 2;
    int rc_up = FJSPH_OK;
    if (need > c->in_cap) {
        rc_up = dfree(c, c->in_stage);
        if (rc_up == FJSPH_OK) rc_up = dalloc(c, &c->in_stage, need);
        c->in_cap = rc_up == FJSPH_OK ? need : 0;
    }
    /* the output fields that go out before the step ends (Runge-Kutta; room for the particles
     * the state holds now): after the second search's pre-passes, after the last residual, after
     * update_data */
    std::vector<void *> op;
    view_ptrs(out, op);
    c->early_out.clear();
    c->final_out.clear();
    c->last_out.clear();
    c->out_sent = c->final_sent = c->last_sent = false;
    c->out_ins0 = c->inserted;
    c->out_del0 = c->deleted;
    if (rc_up == FJSPH_OK && c->s.solver_type == FJSPH_RUNGE_KUTTA && out->n >= n) {
        int64_t oneed = 0;
        for (size_t f = 0; f < op.size(); ++f) {
            const bool e = early_out_field(f, c->s.variant), fi = final_out_field(f), la = last_out_field(f);
            if (!op[f] || !(e || fi || la)) continue;
            (e ? c->early_out : (fi ? c->final_out : c->last_out))
                .push_back({(int)f, oneed, op[f], (size_t)es_bytes_of(c, (int)f) * n, -1});
            oneed += (es_bytes_of(c, (int)f) * c->cap + 15) / 16 * 2;
        }
        if (oneed > c->out_cap) {
            rc_up = dfree(c, c->out_stage);
            if (rc_up == FJSPH_OK) rc_up = dalloc(c, &c->out_stage, oneed);
            c->out_cap = rc_up == FJSPH_OK ? oneed : 0;
        }
        if (rc_up == FJSPH_OK && !c->out_ready &&
            cudaEventCreateWithFlags(&c->out_ready, cudaEventDisableTiming) != cudaSuccess)
            rc_up = FJSPH_E_CUDA;
        if (rc_up != FJSPH_OK) {
            c->early_out.clear();
            c->final_out.clear();
            c->last_out.clear();
        }
    }
    if (!c->copy_stream && rc_up == FJSPH_OK) {
        if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) rc_up = FJSPH_E_CUDA;
        for (int b = 0; b < 2 && rc_up == FJSPH_OK; ++b)
            if (cudaEventCreateWithFlags(&c->st_copied[b], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&c->st_used[b], cudaEventDisableTiming) != cudaSuccess)
                rc_up = FJSPH_E_CUDA;
    }
    if (!c->place_stream && rc_up == FJSPH_OK) {
        /* the highest priority: the placement's blocks go ahead of the search's waiting ones */
        int lo = 0, hi = 0;
        if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess ||
            cudaStreamCreateWithPriority(&c->place_stream, cudaStreamNonBlocking, hi) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->place_after, cudaEventDisableTiming) != cudaSuccess)
            rc_up = FJSPH_E_CUDA;
    }
    /* the placement reads the keys and writes pnp1 and pn after everything the compute stream
     * has enqueued so far */
    if (rc_up == FJSPH_OK && (cudaEventRecord(c->place_after, c->stream) != cudaSuccess ||
                              cudaStreamWaitEvent(c->place_stream, c->place_after, 0) != cudaSuccess))
        rc_up = FJSPH_E_CUDA;
    int64_t off = 0;
    int nev = 0;
    for (int g = 0; g < 4 && rc_up == FJSPH_OK; ++g) {
        if (!c->in_placed[g] && cudaEventCreateWithFlags(&c->in_placed[g], cudaEventDisableTiming) != cudaSuccess) {
            rc_up = FJSPH_E_CUDA;
            break;
        }
        for (size_t f = 0; f < hp.size(); ++f) {
            if (!hp[f] || in_group(f, c->s.variant) != g) continue;
            if ((size_t)nev == c->in_ev.size()) {
                cudaEvent_t e = nullptr;
                if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                    rc_up = FJSPH_E_CUDA;
                    break;
                }
                c->in_ev.push_back(e);
            }
            const size_t bytes = (size_t)(type[f] == 2 ? 4 : 8) * dp[f].size() * n;
            if (cudaMemcpyAsync(c->in_stage + off, hp[f], bytes, cudaMemcpyHostToDevice, c->copy_stream) !=
                    cudaSuccess ||
                cudaEventRecord(c->in_ev[nev], c->copy_stream) != cudaSuccess) {
                rc_up = FJSPH_E_CUDA;
                break;
            }
            c->in_grp[g].push_back({(int)f, off, hp[f], bytes, nev});
            ++nev;
            off += ((int64_t)bytes + 15) / 16 * 2;
        }
    }
    for (int g = 0; g < 4 && rc_up == FJSPH_OK; ++g) rc_up = place_in(c, g);
    const int rc_end = upload_end(c, FJSPH_BOTH, in, nullptr, 0);
    if (rc_up != FJSPH_OK || rc_end != FJSPH_OK) {
        for (auto &g : c->in_grp) g.clear();
        for (bool &w : c->in_wait) w = false;
        c->early_out.clear();
        c->final_out.clear();
        c->last_out.clear();
        if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
        if (c->place_stream) cudaStreamSynchronize(c->place_stream);
        join_id_scan(c);
        return rc_up != FJSPH_OK ? rc_up : rc_end;
    }
    const int64_t ins0 = c->inserted, del0 = c->deleted;
    double r = 0.0;
    const int rc = integrate(c, r);
    const int rc_late = apply_all_in(c); /* a step that stopped early */
    join_id_scan(c);
    const bool sent = c->out_sent, fsent = c->final_sent, lsent = c->last_sent;
    c->early_out.clear();
    c->final_out.clear();
    c->last_out.clear();
    c->out_sent = c->final_sent = c->last_sent = false;
    if (rc != FJSPH_OK || rc_late != FJSPH_OK) { /* no copy into the caller's arrays outlives the call */
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamSynchronize(c->stream);
        return rc != FJSPH_OK ? rc : rc_late;
    }
    if (rms_error) *rms_error = r;
    if (out->n < c->n) {
        TRY(sync(c));
        CU(cudaStreamSynchronize(c->copy_stream));
        return FJSPH_E_CAPACITY;
    }
    out->n = c->n;
    TRY(sync(c));
    fjsph_state_view rest = *out;
    if (sent && c->n == c->out_n && c->inserted == ins0 && c->deleted == del0) {
        /* the early fields are on their way: the rest only */
        double **f64[] = {&rest.xi,     &rest.v,     &rest.acc,    &rest.Af,     &rest.aVisc,  &rest.cellV,
                          &rest.gradRho, &rest.norm, &rest.vPert,  &rest.L,      &rest.Rrho,   &rest.rho,
                          &rest.p,      &rest.m,     &rest.curve,  &rest.norm_curve, &rest.woccl, &rest.pDist,
                          &rest.deltaD, &rest.cellP, &rest.cellRho, &rest.colourG, &rest.colour, &rest.lam,
                          &rest.lam_nb, &rest.kernsum};
        for (size_t f = 0; f < 26; ++f)
            if (early_out_field(f, c->s.variant)) *f64[f] = nullptr;
        if (early_out_field(26, c->s.variant)) rest.part_id = nullptr;
        if (early_out_field(27, c->s.variant)) rest.cellID = nullptr;
        if (early_out_field(28, c->s.variant)) rest.b = nullptr;
        if (early_out_field(29, c->s.variant)) rest.surf = nullptr;
        if (early_out_field(30, c->s.variant)) rest.surfzone = nullptr;
        if (fsent) {
            rest.acc = nullptr;
            rest.Rrho = nullptr;
        }
        if (lsent) {
            rest.xi = nullptr;
            rest.v = nullptr;
            rest.rho = nullptr;
            rest.p = nullptr;
        }
    }
    std::vector<void *> rp;
    view_ptrs(&rest, rp);
    bool any = false;
    for (void *q : rp) any = any || q != nullptr;
    const int rc_t = any ? transfer(c, WS(c), &rest, false) : FJSPH_OK;
    CU(cudaStreamSynchronize(c->copy_stream)); /* the early copies too */
    return rc_t;
}

int fjsph_particle_count(fjsph_ctx *c, int64_t *n_total, int64_t *n_bound) {
    TRY(check_ctx(c));
    if (n_total) *n_total = c->n;
    if (n_bound) *n_bound = c->nb;
    return FJSPH_OK;
}

int fjsph_update_neighbours(fjsph_ctx *c, int64_t *n_pairs) {
    TRY(need_state(c));
    TRY(search(c));
    if (n_pairs) *n_pairs = c->n_pairs;
    return FJSPH_OK;
}

int fjsph_neighbours_export(fjsph_ctx *c, int64_t *offsets, int64_t *idx, double *d2) {
    TRY(need_nbr(c));
    TRY(sync(c));
    const int64_t n = c->n;
    std::vector<int64_t> keys;
    TRY(download_keys(c, keys));
    std::vector<int64_t> off(n + 1);
    std::vector<int32_t> id(c->n_pairs);
    std::vector<double> xs(c->D * n);
    if (mixed(c) && c->tiles_valid) { /* the member masks of the tiles, decoded on the device */
        const Params P = make_params(c);
        std::vector<int32_t> cnt(n);
        launch_tile_export(P, c->xs, c->G, c->K, c->T, 0, c->nbr_counts, nullptr, nullptr, nullptr, c->stream);
        CU(cudaMemcpyAsync(cnt.data(), c->nbr_counts, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream));
        TRY(sync(c));
        off[0] = 0;
        for (int64_t i = 0; i < n; ++i) off[i + 1] = off[i] + cnt[i];
        const int64_t total = off[n];
        /* the caller sized its buffers from the pair count the search reported */
        if (total != c->n_pairs) return FJSPH_E_NEIGHBOUR;
        id.assign(total, 0);
        int64_t *didx = nullptr, *doff = nullptr;
        double *dd2 = nullptr;
        if (total > 0) {
            CU(cudaMalloc(&didx, sizeof(int64_t) * total));
            CU(cudaMalloc(&dd2, sizeof(double) * total));
            CU(cudaMalloc(&doff, sizeof(int64_t) * (n + 1)));
            CU(cudaMemcpy(doff, off.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
            launch_tile_export(P, c->xs, c->G, c->K, c->T, 1, nullptr, doff, didx, dd2, c->stream);
            std::vector<int64_t> id64(total);
            const cudaError_t e1 = cudaMemcpyAsync(id64.data(), didx, sizeof(int64_t) * total, cudaMemcpyDeviceToHost,
                                                   c->stream);
            const cudaError_t e2 = cudaStreamSynchronize(c->stream);
            cudaFree(didx);
            cudaFree(dd2);
            cudaFree(doff);
            if (e1 != cudaSuccess || e2 != cudaSuccess) return FJSPH_E_CUDA;
            for (int64_t k = 0; k < total; ++k) id[k] = (int32_t)id64[k];
        }
    } else if (mixed(c)) { /* offsets from the per-slot counts (single-pass lists keep no CSR) */
        std::vector<int32_t> cnt(n);
        CU(cudaMemcpy(cnt.data(), c->nbr_counts, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
        off[0] = 0;
        for (int64_t i = 0; i < n; ++i) off[i + 1] = off[i] + cnt[i];
    } else {
        CU(cudaMemcpy(off.data(), c->nbr_off, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost));
    }
    if (c->n_pairs && !(mixed(c) && c->tiles_valid)) {
        if (mixed(c)) { /* sliced-ELL -> CSR */
            const int64_t nslices = (n + kSlice - 1) / kSlice;
            std::vector<int2> pr(c->nbr_storage);
            std::vector<int64_t> so(nslices + 1);
            CU(cudaMemcpy(pr.data(), c->nbr_pair, sizeof(int2) * c->nbr_storage, cudaMemcpyDeviceToHost));
            CU(cudaMemcpy(so.data(), c->slice_off, sizeof(int64_t) * (nslices + 1), cudaMemcpyDeviceToHost));
            for (int64_t i = 0; i < n; ++i)
                for (int64_t k = 0; k < off[i + 1] - off[i]; ++k)
                    id[off[i] + k] = pr[sell_entry(so[i / kSlice] + (i % kSlice) * kChunk, (int32_t)k)].x;
        } else {
            CU(cudaMemcpy(id.data(), c->nbr_idx, sizeof(int32_t) * c->n_pairs, cudaMemcpyDeviceToHost));
        }
    }
    for (int k = 0; k < c->D; ++k) CU(cudaMemcpy(&xs[k * n], c->xs[k], sizeof(double) * n, cudaMemcpyDeviceToHost));
    std::vector<int64_t> slot_of_ref(n);
    for (int64_t s = 0; s < n; ++s) slot_of_ref[keys[s]] = s;
    int64_t w = 0;
    std::vector<std::pair<int64_t, double>> row;
    for (int64_t r = 0; r < n; ++r) {
        const int64_t s = slot_of_ref[r];
        if (offsets) offsets[r] = w;
        row.clear();
        for (int64_t e = off[s]; e < off[s + 1]; ++e) {
            const int64_t j = id[e];
            double d0 = xs[s] - xs[j];
            double rr = d0 * d0;
            for (int k = 1; k < c->D; ++k) {
                double dk = xs[k * n + s] - xs[k * n + j];
                rr = std::fma(dk, dk, rr);
            }
            row.push_back({keys[j], rr});
        }
        std::sort(row.begin(), row.end());
        for (auto &p : row) {
            if (idx) idx[w] = p.first;
            if (d2) d2[w] = p.second;
            ++w;
        }
    }
    if (offsets) offsets[n] = w;
    return FJSPH_OK;
}

int fjsph_dsph_prestep(fjsph_ctx *c, double *npd) {
    TRY(need_nbr(c));
    Params P = make_params(c);
    TRY(prestep_npd(c, P));
    c->pn_equals_W = false;
    if (npd) {
        CU(cudaMemcpyAsync(&c->hsc->npd, &c->dsc->npd, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        TRY(sync(c));
        *npd = c->hsc->npd;
    }
    return FJSPH_OK;
}

int fjsph_get_aero_velocity(fjsph_ctx *c) {
    TRY(need_nbr(c));
    TRY(vlm_air(c, make_params(c), make_nbr(c)));
    TRY(aero_velocity(c, make_params(c), make_nbr(c)));
    c->pn_equals_W = false;
    return sync(c);
}

int fjsph_detect_surface(fjsph_ctx *c) {
    TRY(need_nbr(c));
    if (mixed(c)) {
        ensure_pack(c);
        launch_m_surface(make_params(c), WS(c), make_nbr(c), c->K, false, c->stream);
        c->occ_valid = true;
    } else {
        TRY(ensure_quot(c));
        launch_detect_surface(make_params(c), WS(c), make_nbr(c), c->nrm_tmp, quot(c), c->stream);
    }
    c->pn_equals_W = false;
    return sync(c);
}

int fjsph_dissipation_terms(fjsph_ctx *c) {
    TRY(need_nbr(c));
    if (mixed(c)) {
        ensure_pack(c);
        launch_m_dissipation(make_params(c), WS(c), make_nbr(c), c->K, c->stream);
    } else {
        TRY(ensure_quot(c));
        launch_dissipation(make_params(c), WS(c), make_nbr(c), quot(c), c->stream);
    }
    c->pn_equals_W = false;
    return sync(c);
}

int fjsph_particle_shift(fjsph_ctx *c) {
    TRY(need_nbr(c));
    if (!(c->s.variant & FJSPH_VAR_ALE)) return FJSPH_E_UNSUPPORTED;
    if (mixed(c)) {
        ensure_pack(c);
        launch_m_particle_shift(make_params(c), WS(c), make_nbr(c), c->K, c->stream);
    } else {
        TRY(ensure_quot(c));
        launch_particle_shift(make_params(c), WS(c), make_nbr(c), quot(c), c->stream);
    }
    c->pn_equals_W = false;
    return sync(c);
}

int fjsph_check_pipe_outlet(fjsph_ctx *c) {
    TRY(need_state(c));
    launch_pipe_outlet(make_params(c), WS(c), nullptr, c->stream);
    c->pn_equals_W = false;
    mark_all(c);
    return sync(c);
}

int fjsph_get_boundary_pressure(fjsph_ctx *c) {
    TRY(need_nbr(c));
    if (mixed(c)) {
        ensure_pack(c);
        launch_m_bound_pressure(make_params(c), WS(c), make_nbr(c), c->K, c->stream);
    } else {
        launch_bound_pressure(make_params(c), WS(c), make_nbr(c), c->stream);
    }
    mark_bound(c);
    c->pn_equals_W = false;
    return sync(c);
}

int fjsph_boundary_ghost(fjsph_ctx *c, int32_t *near_inlet) {
    TRY(need_nbr(c));
    if (mixed(c)) {
        ensure_pack(c);
        launch_m_bound_ghost(make_params(c), WS(c), make_nbr(c), c->K, c->S.near_inlet, c->stream);
    } else {
        launch_bound_ghost(make_params(c), WS(c), make_nbr(c), c->S.near_inlet, c->stream);
    }
    c->pn_equals_W = false;
    TRY(sync(c));
    if (near_inlet && c->nb > 0) {
        std::vector<int64_t> keys;
        TRY(download_keys(c, keys));
        std::vector<int32_t> tmp(c->nb);
        CU(cudaMemcpy(tmp.data(), c->S.near_inlet, sizeof(int32_t) * c->nb, cudaMemcpyDeviceToHost));
        for (int64_t s = 0; s < c->nb; ++s) near_inlet[keys[s]] = tmp[s];
    }
    return FJSPH_OK;
}

int fjsph_boundary_dbc(fjsph_ctx *c) {
    TRY(need_nbr(c));
    launch_bound_dbc(make_params(c), WS(c), c->stream);
    c->pn_equals_W = false;
    return sync(c);
}

int fjsph_set_no_slip(fjsph_ctx *c) {
    TRY(need_nbr(c));
    launch_no_slip(make_params(c), WS(c), make_nbr(c), c->vtmp, c->stream);
    c->pn_equals_W = false;
    mark_bound(c);
    return sync(c);
}

int fjsph_get_acc_and_rrho(fjsph_ctx *c, double npd) {
    TRY(need_nbr(c));
    TRY(set_npd_device(c, npd));
    TRY(resid(c, make_params(c)));
    c->pn_equals_W = false;
    return sync(c);
}

int fjsph_find_timestep(fjsph_ctx *c, double *dt) {
    TRY(need_state(c));
    double d = 0.0;
    TRY(find_timestep(c, &d));
    if (dt) *dt = d;
    return FJSPH_OK;
}

int fjsph_get_first_rk(fjsph_ctx *c, double npd, double *logbase) {
    TRY(need_nbr(c));
    TRY(set_npd_device(c, npd));
    double lb = 0.0;
    c->pn_equals_W = false; /* the caller may have changed W since the last copy */
    TRY(get_first_rk(c, lb));
    if (logbase) *logbase = lb;
    return FJSPH_OK;
}

int fjsph_runge_kutta4(fjsph_ctx *c, double npd, double logbase, double *rms_error) {
    TRY(need_nbr(c));
    TRY(set_npd_device(c, npd));
    double r = 0.0;
    TRY(runge_kutta4(c, logbase, r));
    if (rms_error) *rms_error = r;
    return FJSPH_OK;
}

int fjsph_nb_iter(fjsph_ctx *c, double npd) {
    TRY(need_nbr(c));
    TRY(set_npd_device(c, npd));
    TRY(set_dt_device(c));
    TRY(nb_iter(c));
    return sync(c);
}

int fjsph_newmark_beta(fjsph_ctx *c, double npd, double *logbase, int32_t *iteration, double *rms_error) {
    TRY(need_nbr(c));
    if (!logbase || !iteration) return FJSPH_E_ARG;
    TRY(set_npd_device(c, npd));
    TRY(set_dt_device(c));
    c->iteration = (uint32_t)*iteration;
    double r = 0.0;
    TRY(newmark_beta_loop(c, *logbase, r));
    *iteration = (int32_t)c->iteration;
    if (rms_error) *rms_error = r;
    return FJSPH_OK;
}

int fjsph_integrate_no_update(fjsph_ctx *c, double *rms_error) {
    TRY(need_state(c));
    double r = 0.0;
    TRY(integrate_no_update(c, r, false));
    if (rms_error) *rms_error = r;
    return sync(c);
}

int fjsph_integrate(fjsph_ctx *c, double *rms_error) {
    TRY(need_state(c));
    double r = 0.0;
    TRY(integrate(c, r));
    if (rms_error) *rms_error = r;
    return sync(c);
}

int fjsph_integrate_n(fjsph_ctx *c, int32_t n_steps, double *last_error) {
    TRY(need_state(c));
    double r = 0.0;
    for (int32_t k = 0; k < n_steps; ++k) TRY(integrate(c, r));
    if (last_error) *last_error = r;
    return sync(c);
}

int fjsph_step_report(fjsph_ctx *c, double *out5) {
    TRY(check_ctx(c));
    if (!out5) return FJSPH_E_ARG;
    out5[0] = c->maxRho_pc;
    out5[1] = c->maxf;
    out5[2] = c->maxAf;
    out5[3] = c->maxShift;
    out5[4] = (double)c->iteration;
    return FJSPH_OK;
}

int fjsph_air_power_law(fjsph_ctx *c, const double *params4) {
    TRY(check_ctx(c));
    if (!params4 || c->s.asource != FJSPH_POWER_LAW) return FJSPH_E_ARG;
    const double axis = params4[0];
    if (!(axis == 0.0 || axis == 1.0 || axis == 2.0) || axis >= c->D) return FJSPH_E_ARG;
    if (!(params4[2] > 0.0) || !(params4[3] > 0.0) || !std::isfinite(params4[1])) return FJSPH_E_ARG;
    for (int k = 0; k < 4; ++k) c->power_law[k] = params4[k];
    if (!c->air_v) TRY(dalloc(c, &c->air_v, 3 * c->cap));
    c->power_law_ready = true;
    return FJSPH_OK;
}

int fjsph_set_pair_mode(fjsph_ctx *c, int32_t mode) {
    TRY(check_ctx(c));
    if (mode != FJSPH_PAIRS_TILES && mode != FJSPH_PAIRS_LISTS) return FJSPH_E_ARG;
    if (mode != c->pair_mode) {
        TRY(graph_release(c));
        c->pair_mode = mode;
        c->nbr_valid = false; /* the next sweep needs a search in the new mode */
        c->tiles_valid = false;
    }
    return FJSPH_OK;
}

int fjsph_get_pair_mode(fjsph_ctx *c, int32_t *mode, int32_t *tiles_in_use) {
    TRY(check_ctx(c));
    if (mode) *mode = c->pair_mode;
    if (tiles_in_use) *tiles_in_use = c->tiles_valid ? 1 : 0;
    return FJSPH_OK;
}

int fjsph_set_sweep_order(fjsph_ctx *c, int32_t order) {
    TRY(check_ctx(c));
    if (order != FJSPH_ORDER_GRID && order != FJSPH_ORDER_SM) return FJSPH_E_ARG;
    if (order == FJSPH_ORDER_SM && !c->region_next) TRY(dalloc(c, &c->region_next, kMaxRegions));
    if (order != c->sweep_order) {
        TRY(graph_release(c)); /* captured launches carry the order */
        c->sweep_order = order;
    }
    return FJSPH_OK;
}

int fjsph_get_sweep_order(fjsph_ctx *c, int32_t *order) {
    TRY(check_ctx(c));
    if (!order) return FJSPH_E_ARG;
    *order = c->sweep_order;
    return FJSPH_OK;
}

int fjsph_neighbour_counts(fjsph_ctx *c, int32_t *counts) {
    TRY(need_nbr(c));
    if (!counts) return FJSPH_E_ARG;
    TRY(sync(c));
    const int64_t n = c->n;
    std::vector<int32_t> cnt(n);
    if (mixed(c)) {
        CU(cudaMemcpy(cnt.data(), c->nbr_counts, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    } else {
        std::vector<int64_t> off(n + 1);
        CU(cudaMemcpy(off.data(), c->nbr_off, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < n; ++i) cnt[i] = (int32_t)(off[i + 1] - off[i]);
    }
    std::vector<int64_t> keys;
    TRY(download_keys(c, keys));
    for (int64_t s = 0; s < n; ++s) counts[keys[s]] = cnt[s];
    return FJSPH_OK;
}

int fjsph_timestep_maxima(fjsph_ctx *c, double *out7) {
    TRY(check_ctx(c));
    if (!out7) return FJSPH_E_ARG;
    out7[0] = c->maxf;
    out7[1] = c->maxAf;
    out7[2] = c->maxdrho;
    out7[3] = c->maxRhoi;
    out7[4] = c->minST;
    out7[5] = c->maxU;
    out7[6] = c->maxShift;
    return FJSPH_OK;
}

int fjsph_launch_stats(fjsph_ctx *c, int64_t *n_launches, int32_t reset) {
    TRY(check_ctx(c));
    if (n_launches) *n_launches = c->launches;
    if (reset) c->launches = 0;
    return FJSPH_OK;
}

int fjsph_ctx_stream(fjsph_ctx *c, void **stream) {
    TRY(check_ctx(c));
    if (!stream) return FJSPH_E_ARG;
    *stream = (void *)c->stream;
    return FJSPH_OK;
}

int fjsph_event_record(fjsph_ctx *c, int32_t slot) {
    TRY(check_ctx(c));
    if (slot < 0 || slot >= 16) return FJSPH_E_ARG;
    if (!c->user_ev[slot]) CU(cudaEventCreate(&c->user_ev[slot]));
    CU(cudaEventRecord(c->user_ev[slot], c->stream));
    return FJSPH_OK;
}

int fjsph_event_elapsed(fjsph_ctx *c, int32_t a, int32_t b, double *ms) {
    TRY(check_ctx(c));
    if (a < 0 || a >= 16 || b < 0 || b >= 16 || !ms || !c->user_ev[a] || !c->user_ev[b]) return FJSPH_E_ARG;
    CU(cudaEventSynchronize(c->user_ev[b]));
    float f = 0.f;
    CU(cudaEventElapsedTime(&f, c->user_ev[a], c->user_ev[b]));
    *ms = f;
    return FJSPH_OK;
}

int fjsph_profile_enable(fjsph_ctx *c, int32_t on) {
    TRY(check_ctx(c));
    if (!on) TRY(profile_collect(c));
    c->prof.on = on != 0;
    return FJSPH_OK;
}

int fjsph_profile_read(fjsph_ctx *c, double *ms, int64_t *launches) {
    TRY(check_ctx(c));
    TRY(profile_collect(c));
    for (int k = 0; k < PASS_COUNT; ++k) {
        if (ms) ms[k] = c->prof.ms[k];
        if (launches) launches[k] = c->prof.count[k];
        c->prof.ms[k] = 0.0;
        c->prof.count[k] = 0;
    }
    return FJSPH_OK;
}

const char *fjsph_profile_pass_name(int32_t k) {
    if (k < 0 || k >= PASS_COUNT) return "";
    return kPassNames[k];
}

/* ---- independent simulations (groups) -------------------------------------------------------- */
int fjsph_set_groups(fjsph_ctx *c, int32_t ngroups, const int64_t *first, const double *v_inf) {
    TRY(check_ctx(c));
    if (ngroups <= 0 || !first || !v_inf || c->blocks.empty()) return FJSPH_E_ARG;
    const int64_t n_ref = c->blocks.back().second;
    if (first[0] != 0 || first[ngroups] != n_ref) return FJSPH_E_ARG;
    for (int32_t g = 0; g < ngroups; ++g)
        if (first[g + 1] <= first[g]) return FJSPH_E_ARG;
    /* the device step of groups covers Runge-Kutta without insertion or deletion, with each
     * group's uniform v_inf as the air source */
    if (c->s.solver_type != FJSPH_RUNGE_KUTTA || !c->inlets.empty()) return FJSPH_E_UNSUPPORTED;
    if (c->s.asource != FJSPH_CONST_VEL) return FJSPH_E_UNSUPPORTED;
    for (const fjsph_block &B : c->blocks)
        if (B.delconst != kDefaultVal || B.block_type == kInletZone) return FJSPH_E_UNSUPPORTED;
    TRY(sync(c));
    TRY(graph_release(c));
    if (c->ngrp != ngroups) {
        TRY(dfree(c, c->g_vinf));
        TRY(dfree(c, c->g_red));
        TRY(dfree(c, c->g_sum));
        double **d8[] = {&c->gs.dt, &c->gs.npd, &c->gs.time, &c->gs.cfl, &c->gs.maxShift, &c->gs.maxRho_pc, &c->gs.logbase,
                         &c->gs.err};
        for (double **a : d8) TRY(dfree(c, *a));
        TRY(dfree(c, c->gs.n_stable));
        TRY(dfree(c, c->gs.n_unstable));
        TRY(dfree(c, c->gs.steps));
        TRY(dfree(c, c->gs.nfluid));
        TRY(dfree(c, c->gs.count));
        TRY(dalloc(c, &c->g_vinf, 3 * ngroups));
        TRY(dalloc(c, &c->g_red, 8 * ngroups));
        TRY(dalloc(c, &c->g_sum, ngroups));
        for (double **a : d8) TRY(dalloc(c, a, ngroups));
        TRY(dalloc(c, &c->gs.n_stable, ngroups));
        TRY(dalloc(c, &c->gs.n_unstable, ngroups));
        TRY(dalloc(c, &c->gs.steps, ngroups));
        TRY(dalloc(c, &c->gs.nfluid, ngroups));
        TRY(dalloc(c, &c->gs.count, ngroups));
    }
    if (!c->grp) TRY(dalloc(c, &c->grp, c->cap));
    c->ngrp = ngroups;
    c->grp_first.assign(first, first + ngroups + 1);
    const int64_t nb_ref = c->n_bound_blocks > 0 ? c->blocks[c->n_bound_blocks - 1].second : 0;
    std::vector<int64_t> cnt(ngroups), nf(ngroups), zero(ngroups, 0);
    std::vector<int32_t> ns(ngroups, c->s.n_stable), nu(ngroups, c->s.n_unstable);
    std::vector<double> dt(ngroups, c->s.delta_t), t(ngroups, c->s.current_time), cfl(ngroups, c->s.cfl),
        shift(ngroups, kEps), z(ngroups, 0.0);
    for (int32_t g = 0; g < ngroups; ++g) {
        cnt[g] = first[g + 1] - first[g];
        nf[g] = std::max<int64_t>(0, first[g + 1] - std::max(first[g], nb_ref));
        if (nf[g] == 0) return FJSPH_E_ARG;
    }
    cudaStream_t s = c->stream;
    CU(cudaMemcpyAsync(c->g_vinf, v_inf, sizeof(double) * 3 * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.dt, dt.data(), sizeof(double) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.time, t.data(), sizeof(double) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.cfl, cfl.data(), sizeof(double) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.maxShift, shift.data(), sizeof(double) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.maxRho_pc, z.data(), sizeof(double) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.logbase, z.data(), sizeof(double) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.err, z.data(), sizeof(double) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.npd, z.data(), sizeof(double) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.n_stable, ns.data(), sizeof(int32_t) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.n_unstable, nu.data(), sizeof(int32_t) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.steps, zero.data(), sizeof(int64_t) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.nfluid, nf.data(), sizeof(int64_t) * ngroups, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(c->gs.count, cnt.data(), sizeof(int64_t) * ngroups, cudaMemcpyHostToDevice, s));
    TRY(sync(c));
    return upload_groups(c);
}

int fjsph_integrate_groups(fjsph_ctx *c, int32_t n_steps, int32_t use_graph) {
    TRY(need_state(c));
    if (!grouped(c)) return FJSPH_E_STATE;
    if (n_steps < 0) return FJSPH_E_ARG;
    int32_t k = 0;
    if (use_graph) {
        /* the captured step replays the host decisions of a steady step: settle the lists, the
         * table size and the first re-ordering with one ordinary step first */
        if (c->reorder_pending || !c->nbr_valid || c->table_want > c->G.table_size || c->graph_uses == 0) {
            if (k < n_steps) {
                TRY(group_step(c));
                ++k;
            }
        }
        /* neighbour storage with room for the lists to grow while the graphs run */
        TRY(sync(c));
        if (mixed(c) && c->wcap > 0) {
            const int32_t w = wcap_for(c->maxcnt + c->maxcnt / 4);
            if (w > c->wcap) {
                TRY(graph_release(c));
                c->wcap = w;
            }
            c->nbr_storage = ((c->n + kSlice - 1) / kSlice) * kSlice * (int64_t)c->wcap;
        }
        const int64_t want = c->nbr_storage + c->nbr_storage / 2;
        if (want > c->nbr_cap && want < ((int64_t)1 << 31)) {
            TRY(graph_release(c));
            TRY(dfree(c, c->nbr_idx));
            TRY(dalloc(c, &c->nbr_idx, want));
            if (c->packed_alloc) {
                TRY(dfree(c, c->nbr_pair));
                TRY(dalloc(c, &c->nbr_pair, want));
            }
            c->nbr_cap = want;
        }
        c->hsc->status = 0;
        CU(cudaMemsetAsync(&c->dsc->status, 0, sizeof(int32_t), c->stream));
        const bool prof = c->prof.on;
        c->prof.on = false;
        c->graph_mode = true;
        int rc = FJSPH_OK;
        for (; k < n_steps && rc == FJSPH_OK; ++k) {
            const int v = graph_variant(c);
            if (!c->graph[v]) {
                const int64_t searches = c->searches, launches = c->launches;
                cudaGraph_t g = nullptr;
                if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                    rc = FJSPH_E_CUDA;
                    break;
                }
                rc = group_step(c);
                const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
                if (rc == FJSPH_OK && e != cudaSuccess) rc = FJSPH_E_CUDA;
                if (rc == FJSPH_OK && cudaGraphInstantiate(&c->graph[v], g, 0) != cudaSuccess) rc = FJSPH_E_CUDA;
                if (g) cudaGraphDestroy(g);
                if (rc != FJSPH_OK) break;
                c->graph_launches[v] = c->launches - launches;
                c->searches = searches;
                c->launches = launches;
            }
            if (cudaGraphLaunch(c->graph[v], c->stream) != cudaSuccess) {
                rc = FJSPH_E_CUDA;
                break;
            }
            c->searches += 2;
            c->launches += c->graph_launches[v];
            c->graph_uses++;
        }
        c->graph_mode = false;
        c->prof.on = prof;
        TRY(rc);
        CU(cudaMemcpyAsync(&c->hsc->status, &c->dsc->status, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
        TRY(sync(c));
        if (c->hsc->status & kStatusNbrOverflow) return FJSPH_E_NEIGHBOUR;
        return FJSPH_OK;
    }
    for (; k < n_steps; ++k) TRY(group_step(c));
    return sync(c);
}

int fjsph_group_report(fjsph_ctx *c, double *time, double *dt, double *cfl, double *err, int64_t *steps) {
    TRY(check_ctx(c));
    if (!grouped(c)) return FJSPH_E_STATE;
    TRY(sync(c));
    const size_t g = (size_t)c->ngrp;
    if (time) CU(cudaMemcpy(time, c->gs.time, sizeof(double) * g, cudaMemcpyDeviceToHost));
    if (dt) CU(cudaMemcpy(dt, c->gs.dt, sizeof(double) * g, cudaMemcpyDeviceToHost));
    if (cfl) CU(cudaMemcpy(cfl, c->gs.cfl, sizeof(double) * g, cudaMemcpyDeviceToHost));
    if (err) CU(cudaMemcpy(err, c->gs.err, sizeof(double) * g, cudaMemcpyDeviceToHost));
    if (steps) CU(cudaMemcpy(steps, c->gs.steps, sizeof(int64_t) * g, cudaMemcpyDeviceToHost));
    return FJSPH_OK;
}

/* ---- launch-configuration autotuner ---------------------------------------------------------- */
} /* extern "C" */
namespace {
bool valid_tune(const int32_t *t) {
    auto bs = [](int32_t v) { return v == 32 || v == 64 || v == 96 || v == 128; };
    return bs(t[0]) && bs(t[1]) && t[2] >= 1 && t[2] <= 16;
}

/* mean milliseconds of `repeats` runs of fn on the context's stream */
template <class F>
int time_ms(fjsph_ctx *c, int repeats, F &&fn, double *ms) {
    cudaEvent_t a, b;
    CU(cudaEventCreate(&a));
    CU(cudaEventCreate(&b));
    int rc = fn(); /* warm-up */
    if (rc == FJSPH_OK && cudaEventRecord(a, c->stream) != cudaSuccess) rc = FJSPH_E_CUDA;
    for (int r = 0; r < repeats && rc == FJSPH_OK; ++r) rc = fn();
    if (rc == FJSPH_OK && cudaEventRecord(b, c->stream) != cudaSuccess) rc = FJSPH_E_CUDA;
    float f = 0.f;
    if (rc == FJSPH_OK && (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&f, a, b) != cudaSuccess))
        rc = FJSPH_E_CUDA;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = f / repeats;
    return rc;
}
} // namespace
extern "C" {

int fjsph_set_tuning(fjsph_ctx *c, const int32_t *cfg3) {
    TRY(check_ctx(c));
    if (!cfg3 || !valid_tune(cfg3)) return FJSPH_E_ARG;
    TRY(sync(c));
    TRY(graph_release(c)); /* captured launches carry the old configuration */
    std::copy(cfg3, cfg3 + 3, c->tune);
    return FJSPH_OK;
}

int fjsph_get_tuning(fjsph_ctx *c, int32_t *cfg3) {
    TRY(check_ctx(c));
    if (!cfg3) return FJSPH_E_ARG;
    std::copy(c->tune, c->tune + 3, cfg3);
    return FJSPH_OK;
}

/* Times the pre-passes under each sweep block size and the residual under each residual block
 * size and list prefetch distance on the context's current state (all of them recompute the same
 * outputs from the same inputs, so the state is unchanged) and keeps the fastest.  times_ms, if
 * given, receives the 2 + 2 * 3 measured configurations in the order tried. */
int fjsph_autotune(fjsph_ctx *c, int32_t repeats, int32_t *chosen3, double *times_ms) {
    TRY(need_state(c));
    if (!mixed(c)) return FJSPH_E_UNSUPPORTED;
    if (repeats <= 0) return FJSPH_E_ARG;
    if (!c->nbr_valid) TRY(search(c));
    TRY(sync(c));
    TRY(graph_release(c));
    const bool prof = c->prof.on;
    c->prof.on = false;
    int k = 0, rc = FJSPH_OK;
    const int32_t bs[2] = {64, 128}, la[3] = {2, 4, 8};
    double best = 1e300;
    int32_t best_sweep = c->tune[0];
    for (int32_t v : bs) {
        c->tune[0] = v;
        double ms = 0.0;
        rc = time_ms(c, repeats, [&] { return prestep_passes(c); }, &ms);
        if (rc != FJSPH_OK) break;
        if (times_ms) times_ms[k] = ms;
        ++k;
        if (ms < best) {
            best = ms;
            best_sweep = v;
        }
    }
    c->tune[0] = best_sweep;
    best = 1e300;
    int32_t best_res = c->tune[1], best_la = c->tune[2];
    for (int32_t v : bs)
        for (int32_t a : la) {
            if (rc != FJSPH_OK) break;
            c->tune[1] = v;
            c->tune[2] = a;
            double ms = 0.0;
            rc = time_ms(c, repeats, [&] { return resid(c, make_params(c)); }, &ms);
            if (rc != FJSPH_OK) break;
            if (times_ms) times_ms[k] = ms;
            ++k;
            if (ms < best) {
                best = ms;
                best_res = v;
                best_la = a;
            }
        }
    c->tune[1] = best_res;
    c->tune[2] = best_la;
    c->prof.on = prof;
    TRY(rc);
    if (chosen3) std::copy(c->tune, c->tune + 3, chosen3);
    return sync(c);
}

int fjsph_autotune_order(fjsph_ctx *c, int32_t repeats, int32_t *chosen, double *times_ms) {
    TRY(need_state(c));
    if (!mixed(c)) return FJSPH_E_UNSUPPORTED;
    if (repeats <= 0) return FJSPH_E_ARG;
    if (!c->nbr_valid) TRY(search(c));
    if (!c->region_next) TRY(dalloc(c, &c->region_next, kMaxRegions));
    TRY(sync(c));
    TRY(graph_release(c));
    const bool prof = c->prof.on;
    c->prof.on = false;
    const int32_t orders[2] = {FJSPH_ORDER_GRID, FJSPH_ORDER_SM};
    double ms[2] = {0.0, 0.0};
    int rc = FJSPH_OK;
    for (int k = 0; k < 2 && rc == FJSPH_OK; ++k) {
        c->sweep_order = orders[k];
        rc = time_ms(c, repeats, [&] { return resid(c, make_params(c)); }, &ms[k]);
    }
    c->sweep_order = (rc == FJSPH_OK && ms[1] < ms[0]) ? FJSPH_ORDER_SM : FJSPH_ORDER_GRID;
    c->prof.on = prof;
    TRY(rc);
    if (chosen) *chosen = c->sweep_order;
    if (times_ms) std::copy(ms, ms + 2, times_ms);
    return sync(c);
}

/* ---- learned aerodynamic closure ------------------------------------------------------------ */
int fjsph_closure_set_weights(fjsph_ctx *c, const float *params, double judge_tol) {
    TRY(check_ctx(c));
    if (!params || !(judge_tol > 0.0)) return FJSPH_E_ARG;
    for (int k = 0; k < mlp::kNumParams; ++k)
        if (!std::isfinite(params[k])) return FJSPH_E_NONFINITE;
    if (!c->mlp_params) {
        TRY(dalloc(c, &c->mlp_params, mlp::kNumParams));
        TRY(dalloc(c, &c->mlp_w, mlp::kNumBf16));
        TRY(dalloc(c, &c->mlp_wt, mlp::mlp_num_bf16_t()));
        TRY(dalloc(c, &c->judge_dev, 3));
        if (!c->judge_host) CU(cudaMallocHost(&c->judge_host, 3 * sizeof(double)));
    }
    TRY(sync(c));
    TRY(mlp::mlp_upload(params, c->mlp_params, c->mlp_w, c->mlp_wt, c->stream));
    TRY(sync(c));
    c->mlp_ready = true;
    c->judge_tol = judge_tol;
    return FJSPH_OK;
}

int fjsph_closure_get_weights(fjsph_ctx *c, float *params) {
    TRY(check_ctx(c));
    if (!params) return FJSPH_E_ARG;
    if (!c->mlp_ready) return FJSPH_E_STATE;
    TRY(sync(c));
    CU(cudaMemcpy(params, c->mlp_params, sizeof(float) * mlp::kNumParams, cudaMemcpyDeviceToHost));
    return FJSPH_OK;
}

int fjsph_closure_log(fjsph_ctx *c, int64_t capacity, int32_t every_n_steps) {
    TRY(check_ctx(c));
    if (capacity < 0 || every_n_steps <= 0) return FJSPH_E_ARG;
    TRY(sync(c));
    if (capacity != c->log_cap) {
        TRY(dfree(c, c->log_X));
        TRY(dfree(c, c->log_T));
        TRY(dfree(c, c->log_count));
        c->log_cap = 0;
        if (capacity > 0) {
            TRY(dalloc(c, &c->log_X, capacity * mlp::kIn));
            TRY(dalloc(c, &c->log_T, capacity * mlp::kOut));
            TRY(dalloc(c, &c->log_count, 1));
            CU(cudaMemset(c->log_count, 0, sizeof(unsigned long long)));
            c->log_cap = capacity;
        }
    }
    c->log_every = every_n_steps;
    return FJSPH_OK;
}

int64_t log_held(fjsph_ctx *c) {
    if (c->log_cap == 0) return 0;
    unsigned long long n = 0;
    if (cudaMemcpy(&n, c->log_count, sizeof(n), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return std::min<int64_t>((int64_t)n, c->log_cap);
}

int fjsph_closure_log_read(fjsph_ctx *c, float *X, float *T, int64_t max_samples, int64_t *count, int32_t reset) {
    TRY(check_ctx(c));
    if (max_samples < 0 || (max_samples > 0 && (!X || !T))) return FJSPH_E_ARG;
    TRY(sync(c));
    const int64_t held = log_held(c);
    if (held < 0) return FJSPH_E_CUDA;
    const int64_t m = std::min(held, max_samples);
    if (m > 0) {
        CU(cudaMemcpy(X, c->log_X, sizeof(float) * mlp::kIn * m, cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(T, c->log_T, sizeof(float) * mlp::kOut * m, cudaMemcpyDeviceToHost));
    }
    if (count) *count = m;
    if (reset && c->log_cap > 0) CU(cudaMemset(c->log_count, 0, sizeof(unsigned long long)));
    return FJSPH_OK;
}

int fjsph_closure_arm(fjsph_ctx *c, int32_t what) {
    TRY(check_ctx(c));
    if (what != 0 && what != FJSPH_CLOSURE_ARM_JUDGE && what != FJSPH_CLOSURE_ARM_LOG) return FJSPH_E_ARG;
    c->arm = what;
    return FJSPH_OK;
}

int fjsph_closure_report_get(fjsph_ctx *c, fjsph_closure_report *out) {
    TRY(check_ctx(c));
    if (!out) return FJSPH_E_ARG;
    TRY(closure_collect(c));
    TRY(sync(c));
    std::memset(out, 0, sizeof(*out));
    out->judged = c->judged;
    out->judged_particles = c->judged_particles;
    out->last_rel_rms = c->last_rel_rms;
    out->max_rel_rms = c->max_rel_rms;
    out->judge_tol = c->judge_tol;
    out->logged = log_held(c);
    if (out->logged < 0) return FJSPH_E_CUDA;
    out->log_capacity = c->log_cap;
    out->steps = c->closure_steps;
    out->learned_active = learned_active(c) ? 1 : 0;
    out->fallback = c->closure_fallback ? 1 : 0;
    return FJSPH_OK;
}

int fjsph_closure_reset(fjsph_ctx *c) {
    TRY(check_ctx(c));
    TRY(closure_collect(c));
    c->closure_fallback = false;
    c->judged = c->judged_particles = 0;
    c->last_rel_rms = c->max_rel_rms = 0.0;
    return FJSPH_OK;
}

/* ---- vortex-lattice air source ---------------------------------------------------------------- */
int fjsph_vlm_defaults(fjsph_vlm *v) {
    if (!v) return FJSPH_E_ARG;
    std::memset(v, 0, sizeof(*v));
    v->span = v->chord = -1.0;
    v->panels_span = v->panels_chord = -1;
    v->max_vel_fac = 2.0;
    v->max_vel = 2.0; /* maxVelFac x |(1, 0, 0)|, the reference's constructor value */
    return FJSPH_OK;
}

int fjsph_mesh_set(fjsph_ctx *c, const fjsph_mesh *m) {
    if (!c || !m) return FJSPH_E_ARG;
    if (c->s.asource != FJSPH_MESH_INFL || m->dim != c->D) return FJSPH_E_ARG;
    MeshHost h;
    TRY(mesh_build(*m, h));
    TRY(sync(c));
    TRY(graph_release(c));
    for (void *q : c->mesh_allocs) {
        char *qq = static_cast<char *>(q);
        TRY(dfree(c, qq));
    }
    c->mesh_allocs.clear();
    c->mesh_ready = false;
    const int D = c->D;
    const int64_t nc = m->n_cells, nf = m->n_faces;
    auto put = [&](auto **dst, const auto *src, int64_t count) -> int {
        TRY(dalloc(c, dst, count));
        c->mesh_allocs.push_back((void *)*dst);
        if (count > 0) CU(cudaMemcpy((void *)*dst, src, sizeof(**dst) * (size_t)count, cudaMemcpyHostToDevice));
        return FJSPH_OK;
    };
    double *verts, *centre, *cvel, *cp, *crho, *rad2;
    int64_t *face_off, *face_verts, *cell_off, *cell_faces;
    int32_t *face_right;
    TRY(put(&verts, m->verts, D * m->n_verts));
    TRY(put(&face_off, m->face_offsets, nf + 1));
    TRY(put(&face_verts, m->face_verts, m->face_offsets[nf]));
    TRY(put(&face_right, m->face_right, nf));
    TRY(put(&cell_off, m->cell_face_offsets, nc + 1));
    TRY(put(&cell_faces, m->cell_faces, m->cell_face_offsets[nc]));
    TRY(put(&centre, m->cell_centres, D * nc));
    TRY(put(&cvel, m->cell_vel, D * nc));
    TRY(put(&cp, m->cell_p, nc));
    TRY(put(&crho, m->cell_rho, nc));
    TRY(put(&rad2, h.rad2.data(), nc));
    MeshDev &M = c->mesh;
    for (int g = 0; g < 2; ++g) {
        int64_t *off, *cells;
        TRY(put(&off, h.g[g].off.data(), (int64_t)h.g[g].off.size()));
        TRY(put(&cells, h.g[g].cells.data(), (int64_t)h.g[g].cells.size()));
        M.g[g].off = off;
        M.g[g].cells = cells;
        M.g[g].inv_h = h.g[g].inv_h;
        for (int k = 0; k < 3; ++k) {
            M.g[g].lo[k] = h.g[g].lo[k];
            M.g[g].dims[k] = h.g[g].dims[k];
        }
    }
    if (!c->air_v) TRY(dalloc(c, &c->air_v, 3 * c->cap));
    if (!c->mesh_list) TRY(dalloc(c, &c->mesh_list, c->cap));
    if (!c->mesh_count) TRY(dalloc(c, &c->mesh_count, 1));
    M.ncells = nc;
    M.verts = verts;
    M.face_off = face_off;
    M.face_verts = face_verts;
    M.face_right = face_right;
    M.cell_off = cell_off;
    M.cell_faces = cell_faces;
    M.centre = centre;
    M.cvel = cvel;
    M.cp = cp;
    M.crho = crho;
    M.rad2 = rad2;
    c->mesh_ready = true;
    return FJSPH_OK;
}

int fjsph_vlm_setup(fjsph_ctx *c, const fjsph_vlm *v, int32_t *npanels) {
    TRY(check_ctx(c));
    if (!v) return FJSPH_E_ARG;
    if (c->D != 3) return FJSPH_E_UNSUPPORTED;
    std::vector<double> abc, gamma;
    TRY(vlm_build(*v, c->s.v_inf, abc, gamma));
    const int32_t np = (int32_t)gamma.size();
    TRY(sync(c));
    TRY(graph_release(c));
    TRY(dfree(c, c->vlm_ab));
    TRY(dfree(c, c->vlm_g));
    TRY(dfree(c, c->vlm_abf));
    TRY(dfree(c, c->vlm_gf));
    TRY(dalloc(c, &c->vlm_ab, 6 * (int64_t)np));
    TRY(dalloc(c, &c->vlm_g, np));
    TRY(dalloc(c, &c->vlm_abf, 12 * (int64_t)np));
    TRY(dalloc(c, &c->vlm_gf, np));
    if (!c->air_v) TRY(dalloc(c, &c->air_v, 3 * c->cap));
    std::vector<double> ab(6 * (size_t)np);
    std::vector<float> abf(12 * (size_t)np), gf(np); /* FP32: A hi, A lo, B hi, B lo */
    for (int32_t q = 0; q < np; ++q) {
        for (int k = 0; k < 6; ++k) ab[6 * q + k] = abc[9 * q + k];
        for (int e = 0; e < 2; ++e)
            for (int k = 0; k < 3; ++k) {
                const double x = abc[9 * q + 3 * e + k];
                const float hi = (float)x;
                abf[12 * q + 6 * e + k] = hi;
                abf[12 * q + 6 * e + 3 + k] = (float)(x - (double)hi);
            }
        gf[q] = (float)gamma[q];
    }
    CU(cudaMemcpy(c->vlm_ab, ab.data(), sizeof(double) * ab.size(), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(c->vlm_g, gamma.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(c->vlm_abf, abf.data(), sizeof(float) * abf.size(), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(c->vlm_gf, gf.data(), sizeof(float) * np, cudaMemcpyHostToDevice));
    VlmDev &V = c->vlm;
    V.np = np;
    V.ab = c->vlm_ab;
    V.gamma = c->vlm_g;
    V.abf = c->vlm_abf;
    V.gammaf = c->vlm_gf;
    for (int k = 0; k < 3; ++k) V.vinf[k] = c->s.v_inf[k];
    const double vn = std::sqrt(V.vinf[0] * V.vinf[0] + V.vinf[1] * V.vinf[1] + V.vinf[2] * V.vinf[2]);
    /* src/VLM.cpp:89-90: a velocity limit still at the constructor value becomes the factor
     * times the freestream speed */
    V.max_vel = (v->max_vel == 2.0) ? v->max_vel_fac * vn : v->max_vel;
    c->vlm_abc = std::move(abc);
    c->vlm_gamma = std::move(gamma);
    if (npanels) *npanels = np;
    return FJSPH_OK;
}

int fjsph_vlm_panels(fjsph_ctx *c, double *gamma, double *abc, int32_t *npanels) {
    TRY(check_ctx(c));
    if (npanels) *npanels = c->vlm.np;
    if (gamma) std::copy(c->vlm_gamma.begin(), c->vlm_gamma.end(), gamma);
    if (abc) std::copy(c->vlm_abc.begin(), c->vlm_abc.end(), abc);
    return FJSPH_OK;
}

int fjsph_vlm_velocity(fjsph_ctx *c, int64_t n, const double *pos, double *vel) {
    TRY(check_ctx(c));
    if (c->vlm.np == 0) return FJSPH_E_STATE;
    if (n < 0 || (n > 0 && (!pos || !vel))) return FJSPH_E_ARG;
    if (n == 0) return FJSPH_OK;
    TRY(sync(c));
    double *d = nullptr;
    CU(cudaMalloc(&d, sizeof(double) * 6 * (size_t)n));
    int rc = FJSPH_OK;
    if (cudaMemcpy(d, pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) rc = FJSPH_E_CUDA;
    if (rc == FJSPH_OK) {
        {
            Section sec(c, PASS_AIR);
            launch_vlm_points(c->vlm, n, d, d + 3 * n, mixed(c), c->stream);
        }
        if (cudaStreamSynchronize(c->stream) != cudaSuccess ||
            cudaMemcpy(vel, d + 3 * n, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = FJSPH_E_CUDA;
    }
    cudaFree(d);
    return rc;
}

} /* extern "C" */
