/*
 * update.cu -- the particle-set changes of Integrator::update_data on the device
 * (src/Integration.cpp:109-226 with the analytic air source):
 *   - inlet buffer advance and insertion (src/shapes/inlet.cpp:578-640): a BACK particle past
 *     its block's insertion plane becomes PIPE, the column's first BUFFER particle becomes BACK,
 *     and a new BUFFER particle is created one dx upstream of the column's last one;
 *   - deletion of fluid particles past their block's deletion plane.
 * Slots are not reference indices: every slot carries its reference index in `key`, so the
 * reference's shifting of indices becomes arithmetic on `key` and compaction of the slots.
 */
#include "kernels.h"

namespace fjsph {

namespace {

constexpr int kT = 256;

/* x . n accumulated as the reference's dot (products then sums, no fused multiply-add) */
__device__ __forceinline__ double plane_dot(const DevState &W, int D, int64_t s, const double *n) {
    double r = __dmul_rn(W.x[0][s], n[0]);
    r = __dadd_rn(r, __dmul_rn(W.x[1][s], n[1]));
    if (D == 3) r = __dadd_rn(r, __dmul_rn(W.x[2][s], n[2]));
    return r;
}

__global__ void k_inlet_cross(DevState W, int D, const int32_t *back, int64_t n_back, double n0, double n1, double n2,
                              double c, int32_t *flag) {
    const int64_t ii = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (ii >= n_back) return;
    const double n[3] = {n0, n1, n2};
    flag[ii] = plane_dot(W, D, back[ii], n) > c ? 1 : 0;
}

__global__ void k_shift_keys(int64_t *key, const int32_t *blk, int64_t n, BlockShift sh) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    key[s] += sh.v[blk[s]];
}

__global__ void k_insert(DevState W, FieldList F, int D, const InsertOp *ops, int64_t nops, double dx) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= nops) return;
    const InsertOp op = ops[q];
    W.b[op.to_pipe] = FJSPH_PIPE;
    W.b[op.to_back] = FJSPH_BACK;
    if (op.dst < 0) return;
    const int64_t d = op.dst, s = op.src;
    for (int k = 0; k < F.n64; ++k) F.f64[k][d] = 0.0;
    for (int k = 0; k < F.ni64; ++k) F.i64[k][d] = 0;
    for (int k = 0; k < F.ni32; ++k) F.i32[k][d] = 0;
    for (int k = 0; k < D; ++k) {
        W.x[k][d] = __dsub_rn(W.x[k][s], __dmul_rn(dx, op.norm[k]));
        W.v[k][d] = W.v[k][s];
    }
    W.rho[d] = W.rho[s];
    W.p[d] = W.p[s];
    W.m[d] = W.m[s];
    W.cellP[d] = W.cellP[s];
    W.cellRho[d] = W.cellRho[s];
    W.cellID[d] = kNoCell;
    W.b[d] = FJSPH_BUFFER;
    W.part_id[d] = op.part_id;
    W.key[d] = op.key;
    W.blk[d] = op.block;
}

__global__ void k_delete_flags(Params P, DevState W, DeletePlanes DP, int32_t *flag, int32_t *keep,
                               unsigned long long *count) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= P.n) return;
    int f = 0;
    if (s >= P.nb) {
        const int b = W.blk[s];
        if (DP.on[b] && plane_dot(W, P.D, s, DP.norm[b]) > DP.c[b]) f = 1;
        if (DP.lost && W.cellID[s] == kMeshLost) f = 1;
    }
    flag[s] = f;
    keep[s] = 1 - f;
    if (f) atomicAdd(&count[W.blk[s]], 1ull);
}

/* deleted[key[s]] = flag[s] */
__global__ void k_scatter_by_key(const int32_t *flag, const int64_t *key, int64_t n, int32_t *by_ref) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    by_ref[key[s]] = flag[s];
}

/* new slot of each kept slot (-1 for deleted), new key = key - deleted references below it */
__global__ void k_compact_map(const int32_t *flag, const int32_t *keep_ex, const int64_t *ref_ex, int64_t n,
                              int32_t *new_of_old, int64_t *key) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    new_of_old[s] = flag[s] ? -1 : keep_ex[s];
    key[s] -= ref_ex[key[s]];
}

__global__ void k_permute_pair(const int64_t *key, const int32_t *blk, int64_t *key2, int32_t *blk2,
                               const int32_t *new_of_old, int64_t n) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int32_t t = new_of_old[s];
    if (t < 0) return;
    key2[t] = key[s];
    blk2[t] = blk[s];
}

} // namespace

void launch_inlet_cross(const DevState &W, int D, const int32_t *back, int64_t n_back, const double *norm, double c,
                        int32_t *flag, cudaStream_t s) {
    if (n_back > 0)
        k_inlet_cross<<<grid_for(n_back, kT), kT, 0, s>>>(W, D, back, n_back, norm[0], norm[1], D == 3 ? norm[2] : 0.0,
                                                          c, flag);
}

void launch_shift_keys(int64_t *key, const int32_t *blk, int64_t n, const BlockShift &sh, cudaStream_t s) {
    if (n > 0) k_shift_keys<<<grid_for(n, kT), kT, 0, s>>>(key, blk, n, sh);
}

void launch_insert(const DevState &W, int D, const InsertOp *ops, int64_t nops, double dx, cudaStream_t s) {
    if (nops > 0) k_insert<<<grid_for(nops, 64), 64, 0, s>>>(W, state_fields(W, D), D, ops, nops, dx);
}

void launch_delete_flags(const Params &P, const DevState &W, const DeletePlanes &DP, int32_t *flag, int32_t *keep,
                         unsigned long long *count, cudaStream_t s) {
    if (P.n > 0) k_delete_flags<<<grid_for(P.n, kT), kT, 0, s>>>(P, W, DP, flag, keep, count);
}

void launch_compact_map(const int32_t *flag, const int64_t *key, int64_t n, int32_t *by_ref, const int32_t *keep_ex,
                        const int64_t *ref_ex_after_scan, int32_t *new_of_old, int64_t *key_out, int phase,
                        cudaStream_t s) {
    if (n == 0) return;
    if (phase == 0)
        k_scatter_by_key<<<grid_for(n, kT), kT, 0, s>>>(flag, key, n, by_ref);
    else
        k_compact_map<<<grid_for(n, kT), kT, 0, s>>>(flag, keep_ex, ref_ex_after_scan, n, new_of_old, key_out);
}

void launch_permute_key_blk(const int64_t *key, const int32_t *blk, int64_t *key2, int32_t *blk2,
                            const int32_t *new_of_old, int64_t n, cudaStream_t s) {
    if (n > 0) k_permute_pair<<<grid_for(n, kT), kT, 0, s>>>(key, blk, key2, blk2, new_of_old, n);
}

} // namespace fjsph
