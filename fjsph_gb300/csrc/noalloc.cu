/*
 * noalloc.cu -- the CFL time-step bound of find_timestep (src/Integration.cpp:370-443) for callers
 * that cannot allocate device memory.
 *
 * fjsph_find_timestep reduces inside a context, whose creation allocated its scratch with
 * cudaMalloc.  Some callers own all of the GPU's memory through their own allocator or memory
 * pool (a coupled solver that reserves HBM up front, a host code embedding this library next to
 * another framework's caching allocator) and may not call cudaMalloc at all, or want no
 * allocation on their time-step path.  fjsph_find_timestep_noalloc serves them: it reads the
 * caller's device arrays, reduces with the same block-then-final scheme, and keeps its scratch in
 * a fixed file-scope __device__ array that every GPU loading this library holds until exit.
 *
 * Scratch: one row of partial results per block (at most kMaxRows) plus one result row.  Every
 * call writes every row it later reads, so no row needs clearing between calls.  All calls share
 * the one array: calls whose kernels overlap on the GPU (different streams, or different host
 * threads, on the same device) race and must be serialised by the caller.
 */
#include <cmath>
#include <mutex>

#include "common.cuh"

namespace {

using fjsph::kEps;
using fjsph::kPi;

constexpr int kThreads = 256;
constexpr int kItems = 16;                 /* particles per thread                  */
constexpr int kVals = 8;                   /* 7 reduced values, padded              */
constexpr int kMaxRows = 4096;             /* partial rows = blocks per call        */
constexpr int64_t kMaxParticles = (int64_t)kMaxRows * kThreads * kItems; /* 16,777,216 */
constexpr int kMaxDevices = 64;

/* 4097 rows x 8 doubles = 262,208 bytes per device. */
static __device__ __align__(256) double g_timestep_scratch[(kMaxRows + 1) * kVals];

struct Fields {
    const double *acc[3], *Af[3], *Rrho, *rho, *curve, *v[3], *vPert[3];
};

/* max/min over one block's chunk of kThreads*kItems particles; ops: max,max,max,max,min,max,max.
 * The squared norms are formed exactly as the context's reduction forms them (fjsph::dot over
 * loaded components, compile-time D), so both give bit-identical maxima. */
template <int D>
__global__ void __launch_bounds__(kThreads) k_partial(int64_t n, int ale, double rho_rest, double dx, double sig,
                                                       Fields f, double *rows) {
    double v[7] = {kEps, kEps, kEps, kEps, 9999999.0, kEps, 0.0};
    const int64_t base = (int64_t)blockIdx.x * kThreads * kItems;
    for (int it = 0; it < kItems; ++it) {
        const int64_t i = base + (int64_t)it * kThreads + threadIdx.x;
        if (i >= n) break;
        double a[D], af[D], vv[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            a[k] = f.acc[k][i];
            af[k] = f.Af[k][i];
            vv[k] = f.v[k][i];
        }
        v[0] = fmax(v[0], sqrt(fjsph::dot<D, double>(a, a)));
        v[1] = fmax(v[1], sqrt(fjsph::dot<D, double>(af, af)));
        v[2] = fmax(v[2], fabs(f.Rrho[i]));
        const double rho = f.rho[i];
        v[3] = fmax(v[3], fabs(rho - rho_rest));
        v[4] = fmin(v[4], sqrt(rho * dx * dx / (2.0 * kPi * sig * fabs(f.curve[i]))));
        v[5] = fmax(v[5], sqrt(fjsph::dot<D, double>(vv, vv)));
        if (ale) {
            double vp[D];
#pragma unroll
            for (int k = 0; k < D; ++k) vp[k] = f.vPert[k][i];
            v[6] = fmax(v[6], sqrt(fjsph::dot<D, double>(vp, vp)));
        }
    }
    __shared__ double sh[7][kThreads];
    for (int k = 0; k < 7; ++k) sh[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int st = kThreads / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int k = 0; k < 7; ++k) {
                const double o = sh[k][threadIdx.x + st];
                sh[k][threadIdx.x] = (k == 4) ? fmin(sh[k][threadIdx.x], o) : fmax(sh[k][threadIdx.x], o);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 7; ++k) rows[blockIdx.x * kVals + k] = sh[k][0];
}

/* one block: reduce nrows partial rows into the result row kMaxRows */
__global__ void __launch_bounds__(kThreads) k_final(int nrows, double *rows) {
    __shared__ double sh[7][kThreads];
    for (int k = 0; k < 7; ++k) {
        double t = (k == 4) ? INFINITY : -INFINITY;
        for (int r = threadIdx.x; r < nrows; r += kThreads) {
            const double x = rows[r * kVals + k];
            t = (k == 4) ? fmin(t, x) : fmax(t, x);
        }
        sh[k][threadIdx.x] = t;
    }
    __syncthreads();
    for (int st = kThreads / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int k = 0; k < 7; ++k) {
                const double o = sh[k][threadIdx.x + st];
                sh[k][threadIdx.x] = (k == 4) ? fmin(sh[k][threadIdx.x], o) : fmax(sh[k][threadIdx.x], o);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 7; ++k) rows[kMaxRows * kVals + k] = sh[k][0];
}

std::mutex g_setup_mutex;
double *g_scratch_addr[kMaxDevices] = {};

/* Device address of the scratch array on the current device.  The array's name in host code is
 * only a host-side stand-in: handing it to a kernel would fault, or on a GPU that can reach host
 * memory silently use the wrong memory, so the address comes from cudaGetSymbolAddress, once per
 * device, with that device current. */
int scratch_address(double **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FJSPH_E_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return FJSPH_E_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_timestep_scratch) != cudaSuccess) return FJSPH_E_CUDA;
        g_scratch_addr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_addr[dev];
    return FJSPH_OK;
}

} // namespace

extern "C" int fjsph_find_timestep_noalloc(const fjsph_settings *s, int64_t n_fluid, const double *const acc[3],
                                           const double *const Af[3], const double *Rrho, const double *rho,
                                           const double *curve, const double *const v[3],
                                           const double *const vPert[3], void *stream, double *dt,
                                           double *maxima7) {
    if (!s || !dt || !maxima7 || n_fluid < 0 || (s->dim != 2 && s->dim != 3)) return FJSPH_E_ARG;
    if (n_fluid > kMaxParticles) return FJSPH_E_CAPACITY;
    const int D = s->dim;
    const int ale = (s->variant & FJSPH_VAR_ALE) ? 1 : 0;
    Fields f{};
    if (n_fluid > 0) {
        if (!acc || !Af || !Rrho || !rho || !curve || !v || (ale && !vPert)) return FJSPH_E_ARG;
        for (int k = 0; k < D; ++k) {
            if (!acc[k] || !Af[k] || !v[k] || (ale && !vPert[k])) return FJSPH_E_ARG;
            f.acc[k] = acc[k];
            f.Af[k] = Af[k];
            f.v[k] = v[k];
            f.vPert[k] = ale ? vPert[k] : nullptr;
        }
        f.Rrho = Rrho;
        f.rho = rho;
        f.curve = curve;
    }
    double *rows = nullptr;
    int r = scratch_address(&rows);
    if (r != FJSPH_OK) return r;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nrows = n_fluid > 0 ? (int)((n_fluid + (int64_t)kThreads * kItems - 1) / ((int64_t)kThreads * kItems)) : 1;
    /* a launch that fails (no kernel image for this device, an invalid stream) leaves the result
     * row holding an earlier call's values or zeros: report it instead of returning them */
    if (D == 2)
        k_partial<2><<<nrows, kThreads, 0, st>>>(n_fluid, ale, s->rho_rest, s->dx, s->sig, f, rows);
    else
        k_partial<3><<<nrows, kThreads, 0, st>>>(n_fluid, ale, s->rho_rest, s->dx, s->sig, f, rows);
    if (cudaGetLastError() != cudaSuccess) return FJSPH_E_CUDA;
    k_final<<<1, kThreads, 0, st>>>(nrows, rows);
    if (cudaGetLastError() != cudaSuccess) return FJSPH_E_CUDA;
    double red[kVals];
    if (cudaMemcpyAsync(red, rows + (size_t)kMaxRows * kVals, sizeof(double) * 7, cudaMemcpyDeviceToHost, st) !=
        cudaSuccess)
        return FJSPH_E_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return FJSPH_E_CUDA;
    for (int k = 0; k < 7; ++k) maxima7[k] = red[k];
    /* the scalar tail of find_timestep */
    const double maxf = red[0], maxU = red[5], maxdrho = red[2], minST = red[4];
    double fac[6] = {0.25 * std::sqrt(s->H / maxf), 2 * s->H / maxU, 0.125 * s->H_sq * s->rho_rest / s->mu,
                     0.067 * minST, 0.5 * std::sqrt(s->H / maxdrho), 1.5 * s->H / s->speed_sound};
    double mn = fac[0];
    for (int k = 1; k < 6; ++k)
        if (fac[k] < mn) mn = fac[k];
    /* cfl * (0.75 * min), in the reference's order (src/Integration.cpp:427-428) */
    const double safe_dt = 0.75 * mn;
    double d = s->cfl * safe_dt;
    if (d < s->delta_t_min)
        d = s->delta_t_min;
    else if (d > s->delta_t_max)
        d = s->delta_t_max;
    if (d > s->last_frame_time + s->frame_time_interval - s->current_time)
        d = s->last_frame_time + s->frame_time_interval - s->current_time + s->delta_t_min;
    *dt = d;
    return FJSPH_OK;
}
