/*
 * state.cu -- whole-state data movement: slot re-ordering (gather into cell order) and state
 * copies.  Each kernel moves one particle's fields per thread, field by field, so that every load
 * and store of a field array is coalesced on one side.
 */
#include "kernels.h"

namespace fjsph {

FieldList state_fields(const DevState &S, int D) {
    FieldList f;
    auto add_vec = [&](double *const a[3]) {
        for (int k = 0; k < D; ++k) f.f64[f.n64++] = a[k];
    };
    add_vec(S.x);
    add_vec(S.v);
    add_vec(S.acc);
    add_vec(S.Af);
    add_vec(S.aVisc);
    add_vec(S.cellV);
    add_vec(S.gradRho);
    add_vec(S.norm);
    add_vec(S.vPert);
    for (int k = 0; k < D * D; ++k) f.f64[f.n64++] = S.L[k];
    double *sc[] = {S.Rrho, S.rho,     S.p,       S.m,      S.curve, S.norm_curve, S.woccl,  S.pDist,
                    S.deltaD, S.cellP, S.cellRho, S.colourG, S.colour, S.lam,      S.lam_nb, S.kernsum};
    for (double *a : sc) f.f64[f.n64++] = a;
    f.i64[f.ni64++] = S.part_id;
    f.i64[f.ni64++] = S.cellID;
    f.i32[f.ni32++] = S.b;
    f.i32[f.ni32++] = S.surf;
    f.i32[f.ni32++] = S.surfzone;
    return f;
}

namespace {

constexpr int kThreads = 256;

__global__ void k_permute(FieldList src, FieldList dst, const int32_t *new_of_old, int64_t n) {
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int64_t t = new_of_old ? new_of_old[o] : o;
    if (t < 0) return; /* deleted */
    for (int k = 0; k < src.n64; ++k) dst.f64[k][t] = src.f64[k][o];
    for (int k = 0; k < src.ni64; ++k) dst.i64[k][t] = src.i64[k][o];
    for (int k = 0; k < src.ni32; ++k) dst.i32[k][t] = src.i32[k][o];
}

__global__ void k_remap(int32_t *a, int64_t n, const int32_t *new_of_old) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = new_of_old[a[i]];
}

} // namespace

void launch_permute(const FieldList &src, const FieldList &dst, const int32_t *new_of_old, int64_t n, cudaStream_t s) {
    if (n == 0) return;
    k_permute<<<grid_for(n, kThreads), kThreads, 0, s>>>(src, dst, new_of_old, n);
}

void launch_copy(const FieldList &src, const FieldList &dst, int64_t n, cudaStream_t s) {
    if (n == 0) return;
    k_permute<<<grid_for(n, kThreads), kThreads, 0, s>>>(src, dst, nullptr, n);
}

namespace {

/* dst_k[s] = stage[key[s] * comps + k]: reference-order, component-interleaved host layout to
 * slot-order structure of arrays (and the reverse for download). */
template <typename T>
__global__ void k_field_in(const T *stage, int comps, const int64_t *key, FieldPtrs dst, int64_t n) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int64_t r = key[s];
    for (int k = 0; k < comps; ++k) static_cast<T *>(dst.p[k])[s] = stage[r * comps + k];
}

template <typename T>
__global__ void k_field_out(T *stage, int comps, const int64_t *key, FieldPtrs src, int64_t n) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int64_t r = key[s];
    for (int k = 0; k < comps; ++k) stage[r * comps + k] = static_cast<const T *>(src.p[k])[s];
}

} // namespace

void launch_field_in(const void *stage, int comps, int elem, const int64_t *key, const FieldPtrs &dst, int64_t n,
                     cudaStream_t s) {
    if (n == 0) return;
    const unsigned g = grid_for(n, kThreads);
    if (elem == 8)
        k_field_in<int64_t><<<g, kThreads, 0, s>>>(static_cast<const int64_t *>(stage), comps, key, dst, n);
    else
        k_field_in<int32_t><<<g, kThreads, 0, s>>>(static_cast<const int32_t *>(stage), comps, key, dst, n);
}

void launch_field_out(void *stage, int comps, int elem, const int64_t *key, const FieldPtrs &src, int64_t n,
                      cudaStream_t s) {
    if (n == 0) return;
    const unsigned g = grid_for(n, kThreads);
    if (elem == 8)
        k_field_out<int64_t><<<g, kThreads, 0, s>>>(static_cast<int64_t *>(stage), comps, key, src, n);
    else
        k_field_out<int32_t><<<g, kThreads, 0, s>>>(static_cast<int32_t *>(stage), comps, key, src, n);
}

void launch_remap_i32(int32_t *a, int64_t n, const int32_t *new_of_old, cudaStream_t s) {
    if (n == 0) return;
    k_remap<<<grid_for(n, kThreads), kThreads, 0, s>>>(a, n, new_of_old);
}

} // namespace fjsph
