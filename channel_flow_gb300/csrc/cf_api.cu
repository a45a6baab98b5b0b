// C-ABI of the GB300 channel-flow hot path: context, device mirrors of host
// arrays, argument resolution and one entry point per reference routine
// (declarations and contracts: include/channel_flow_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/channel_flow_gb300.h"
#include "cf_common.cuh"
#include "cf_launch.h"

#define CF_VERSION 100

struct cf_ctx {
    cf_dims d;
    int prec = CF_PREC_FP64;
    cudaStream_t stream = nullptr;
    double gamma = 1.5;
    double q0 = 20.464969232814912;   // target bulk flux Q0 (prm.h)
    std::string out_dir = ".";        // where Statistic / Output / Initial_condition put their files
    double *stat_acc = nullptr;       // Statistic accumulators, 17 rows of Y_m (device)
    double sxy_bottom = 0, sxy_up = 0;
    double E[5] = {0, 0, 0, 0, 0};    // running maxima of the residual norms (main.cpp:63, 387-391)
    std::vector<double> er_hist;      // normalised er1..er5 of every iteration of the last cf_step
    std::unordered_map<const double *, float *> met32;   // FP32 copies of fixed metric arrays (cf_step)
    const double *shadow_j = nullptr;   // the fixed J whose FP32 J, 1/J the flux shadow holds (cf_step)
    std::unordered_map<const double *, double *> mirrors;
    std::unordered_map<std::string, std::pair<double *, size_t>> scratch;
    std::vector<int> nijk;            // plane tables, Hyperplane layout (host)
    std::vector<int> ijk;
    int *ijk_dev = nullptr;
    bool tables_checked = false;
    double *er_dev = nullptr;         // 5 doubles + device counter space
    double *er_host = nullptr;        // pinned
    cudaStream_t cap = nullptr;       // private stream for graph capture
    cudaStream_t side = nullptr;      // cf_step: Flux_Y/Z beside the viscous terms
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // cf_step's Statistic: its kernels on a stream of their own, from a copy
    // of the step's final U_, beside the next call's work; the host part
    // (accumulators to the host, the files) of step stat_step is pending
    cudaStream_t stat_stream = nullptr;
    cudaEvent_t ev_stat = nullptr;
    bool stat_pending = false;
    int stat_step = 0, stat_every = 0;
    int lu_schedule = CF_LU_WAVEFRONT;                // hyperplane sweep schedule
    unsigned wait_limit = CF_WAVE_SPIN_LIMIT;         // polls of a wavefront dependency wait
    int *tile_order = nullptr;        // wavefront tiles sorted by plane (device)
    int *pencil_order = nullptr;      // pencils sorted by pj + pk (device)
    long long *trace = nullptr;       // wavefront trace: [2 sweeps][tiles][4] stamps, when enabled
    size_t trace_tiles = 0;
    cudaGraphExec_t dts_exec = nullptr;               // Dual_time_stepping as one graph
    std::vector<unsigned char> dts_key;               // arguments it was captured with
    std::string err;
};

namespace {

int fail(cf_ctx *c, int code, const char *fmt, ...)
{
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

int cuda_check(cf_ctx *c, cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return CF_OK;
    return fail(c, CF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// field pointer of an argument: the device mirror of a registered host
// array, or the pointer itself (a device pointer)
inline double *R(cf_ctx *c, const double *p)
{
    auto it = c->mirrors.find(p);
    return it == c->mirrors.end() ? const_cast<double *>(p) : it->second;
}

int check_ptrs(cf_ctx *c, const double *const *p, int n, const char *who)
{
    for (int i = 0; i < n; i++)
        if (!p[i]) return fail(c, CF_ERR_ARG, "%s: array argument %d is NULL", who, i);
    return CF_OK;
}

// scratch of a number of bytes, owned by the context (allocated on first use)
void *scratch_bytes(cf_ctx *c, const char *key, size_t bytes)
{
    auto &e = c->scratch[key];
    if (e.first && e.second >= bytes) return e.first;
    if (e.first) cudaFree(e.first);
    e.first = nullptr;
    e.second = 0;
    if (cudaMalloc(&e.first, bytes) != cudaSuccess) {
        e.first = nullptr;
        return nullptr;
    }
    e.second = bytes;
    return e.first;
}

// scratch of nfields fields
double *scratch(cf_ctx *c, const char *key, int nfields)
{
    return static_cast<double *>(scratch_bytes(c, key, (size_t)nfields * c->d.total() * sizeof(double)));
}

// cells of plane m = i+j+k in i-major order, exactly the tables of
// Hyperplane.cpp:50-78 (ijk 1-based, Nijk[m] = {last index, count})
void build_tables(cf_ctx *c)
{
    const cf_dims &d = c->d;
    const int nplanes = (d.X_out + 3) + d.ny + d.nz + 7;
    c->nijk.assign((size_t)nplanes * 2, 0);
    c->ijk.assign(((size_t)d.X_out * d.Y_out * d.Z_out * 3 + 1) * 3, 0);
    int ii = 0;
    for (int m = 7; m <= d.gend + d.ny + d.nz; m++) {
        int mi = 0;
        for (int i = 3; i <= d.gend; i++)
            for (int j = 2; j <= d.ny; j++) {
                const int k = m - i - j;
                if (k >= 2 && k <= d.nz) {
                    mi++;
                    ii++;
                    c->ijk[3 * (size_t)ii] = i;
                    c->ijk[3 * (size_t)ii + 1] = j;
                    c->ijk[3 * (size_t)ii + 2] = k;
                }
            }
        c->nijk[2 * (size_t)m] = ii;
        c->nijk[2 * (size_t)m + 1] = mi;
    }
}

__global__ void k_count_nonfinite(cf_dims d, const double *f, unsigned long long *bad)
{
    const int k = 2 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 2 + (int)blockIdx.y;
    const int i = 3 + (int)blockIdx.z;
    if (k > d.nz) return;
    const double v = f[d.ix(i, j, k)];
    if (!isfinite(v)) atomicAdd(bad, 1ull);
}

// FP64 rate probe: sixteen independent FMA chains per thread, the loop
// unrolled four times, so the FP64 pipe, not the FMA latency or the loop
// control, bounds the kernel; the sum keeps the chains live.  a < 1 and b
// small keep every value bounded.
constexpr int CF_PROBE_CHAINS = 16;
__global__ void __launch_bounds__(256) k_fp64_fma_chains(int iters, double a, double b, double *out)
{
    double x[CF_PROBE_CHAINS];
#pragma unroll
    for (int c = 0; c < CF_PROBE_CHAINS; c++) x[c] = 1e-3 * (threadIdx.x + c);
#pragma unroll 4
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int c = 0; c < CF_PROBE_CHAINS; c++) x[c] = fma(x[c], a, b);
    double s = 0;
#pragma unroll
    for (int c = 0; c < CF_PROBE_CHAINS; c++) s += x[c];
    if (s == 12345.678) out[blockIdx.x] = s;   // never true; keeps the chains
}

// the contracted build's reciprocal (frcp<double> of cf_common.cuh) of n values
__global__ void __launch_bounds__(256) k_reciprocal(const double *d, double *out, size_t n)
{
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) out[q] = frcp<double>(d[q]);
}

inline bool exact(const cf_ctx *c) { return c->prec == CF_PREC_FP64_EXACT; }
inline int kprec(const cf_ctx *c) { return c->prec == CF_PREC_FP32 ? 1 : 0; }

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

int cf_library_version(void) { return CF_VERSION; }

int cf_fp64_peak_probe(void *stream, int blocks, int iters, double *scratch_dev)
{
    if (blocks <= 0 || iters <= 0 || !scratch_dev) return CF_ERR_ARG;
    k_fp64_fma_chains<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(iters, 0.9999999, 1e-9, scratch_dev);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

int cf_reciprocal_check(void *stream, const double *d_dev, double *out_dev, size_t n)
{
    if (!d_dev || !out_dev) return CF_ERR_ARG;
    if (n == 0) return CF_OK;
    k_reciprocal<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_dev, out_dev, n);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

const char *cf_error_string(int code)
{
    switch (code) {
    case CF_OK: return "ok";
    case CF_ERR_ARG: return "invalid argument";
    case CF_ERR_CUDA: return "CUDA error";
    case CF_ERR_NONFINITE: return "non-finite value";
    case CF_ERR_NOMEM: return "device allocation failed";
    case CF_ERR_STATE: return "call out of order";
    case CF_ERR_TIMEOUT: return "a bounded device wait ran out";
    default: return "unknown error";
    }
}

const char *cf_last_error(const cf_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int cf_grid_reference(cf_grid *g, int cells_x, int cells_y, int cells_z)
{
    if (!g) return CF_ERR_ARG;
    const double h = 0.5 * 0.005;
    const double pi = 3.14159265358979323846;
    g->cells_x = cells_x; g->cells_y = cells_y; g->cells_z = cells_z;
    g->d_xi = 4 * pi * h / cells_x;
    g->d_eta = 1.0 / cells_y;
    g->d_zeta = 2 * pi * h / cells_z;
    g->gamma_gas = 1.4; g->r_gas = 287; g->beta_min = 0.0001;
    g->cv = 717.5; g->mu = 0.0000185; g->prandtl = 0.72;
    g->body_force = 599.29876710; g->height = 0.005;
    g->bulk_flux = 20.464969232814912;
    return CF_OK;
}

int cf_create(const cf_grid *g, int precision, cf_ctx **out)
{
    if (!g || !out) return CF_ERR_ARG;
    *out = nullptr;
    if (g->cells_x < 6 || g->cells_y < 6 || g->cells_z < 6) return CF_ERR_ARG;
    if (precision < CF_PREC_FP64_EXACT || precision > CF_PREC_FP32) return CF_ERR_ARG;
    cf_ctx *c = new cf_ctx();
    cf_dims &d = c->d;
    d.X_out = g->cells_x; d.Y_out = g->cells_y; d.Z_out = g->cells_z;
    d.Ym = g->cells_y + 4; d.Zm = g->cells_z + 4;
    d.gend = g->cells_x + 2; d.ny = g->cells_y + 1; d.nz = g->cells_z + 1;
    d.dXI = g->d_xi; d.dET = g->d_eta; d.dZT = g->d_zeta;
    d.K = g->gamma_gas; d.R = g->r_gas; d.e = g->beta_min; d.Cv = g->cv; d.mu_L = g->mu; d.Pr_L = g->prandtl;
    d.f = g->body_force; d.high = g->height;
    d.scheme = CF_SCHEME_REFERENCE;
    cf_dims_fill_f32(d);
    c->q0 = g->bulk_flux;
    c->prec = precision;
    build_tables(c);
    cudaError_t e = cudaMalloc(&c->ijk_dev, c->ijk.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(c->ijk_dev, c->ijk.data(), c->ijk.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&c->er_dev, 16 * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&c->er_host, 16 * sizeof(double));
    if (e != cudaSuccess) {
        cf_destroy(c);
        return CF_ERR_CUDA;
    }
    *out = c;
    return CF_OK;
}

void cf_destroy(cf_ctx *c)
{
    if (!c) return;
    cf_statistic_flush(c);
    for (auto &m : c->mirrors) cudaFree(m.second);
    for (auto &s : c->scratch) cudaFree(s.second.first);
    if (c->ijk_dev) cudaFree(c->ijk_dev);
    if (c->er_dev) cudaFree(c->er_dev);
    if (c->er_host) cudaFreeHost(c->er_host);
    if (c->dts_exec) cudaGraphExecDestroy(c->dts_exec);
    if (c->stat_acc) cudaFree(c->stat_acc);
    if (c->tile_order) cudaFree(c->tile_order);
    if (c->pencil_order) cudaFree(c->pencil_order);
    if (c->trace) cudaFree(c->trace);
    if (c->cap) cudaStreamDestroy(c->cap);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->stat_stream) cudaStreamDestroy(c->stat_stream);
    if (c->ev_stat) cudaEventDestroy(c->ev_stat);
    for (auto &m : c->met32) cudaFree(m.second);
    delete c;
}

int cf_set_precision(cf_ctx *c, int precision)
{
    if (!c || precision < CF_PREC_FP64_EXACT || precision > CF_PREC_FP32) return CF_ERR_ARG;
    c->prec = precision;
    return CF_OK;
}

int cf_set_stream(cf_ctx *c, void *stream)
{
    if (!c) return CF_ERR_ARG;
    c->stream = (cudaStream_t)stream;
    return CF_OK;
}

int cf_set_scheme(cf_ctx *c, int scheme)
{
    if (!c || (scheme != CF_SCHEME_REFERENCE && scheme != CF_SCHEME_CONSISTENT)) return CF_ERR_ARG;
    c->d.scheme = scheme;
    return CF_OK;
}

int cf_set_wait_limit(cf_ctx *c, unsigned polls)
{
    if (!c) return CF_ERR_ARG;
    c->wait_limit = polls ? polls : CF_WAVE_SPIN_LIMIT;
    return CF_OK;
}

int cf_set_lu_schedule(cf_ctx *c, int schedule)
{
    if (!c || (schedule != CF_LU_WAVEFRONT && schedule != CF_LU_PLANES && schedule != CF_LU_PENCIL))
        return CF_ERR_ARG;
    c->lu_schedule = schedule;
    return CF_OK;
}

int cf_lu_trace(cf_ctx *c, int enable)
{
    if (!c) return CF_ERR_ARG;
    if (!enable) {
        if (c->trace) cudaFree(c->trace);
        c->trace = nullptr;
        c->trace_tiles = 0;
    } else if (!c->trace_tiles) {
        c->trace_tiles = 1;     // sized by the next Dual_time_stepping call
    }
    return CF_OK;
}

int cf_lu_trace_read(cf_ctx *c, long long *out, size_t count)
{
    if (!c || !out) return CF_ERR_ARG;
    if (!c->trace) return fail(c, CF_ERR_STATE, "cf_lu_trace_read: no trace recorded");
    const size_t n = 2 * 4 * c->trace_tiles;
    if (count < n) return fail(c, CF_ERR_ARG, "cf_lu_trace_read: %zu values needed", n);
    if (int rc = cuda_check(c, cudaStreamSynchronize(c->stream), "cf_lu_trace_read")) return rc;
    return cuda_check(c, cudaMemcpy(out, c->trace, n * sizeof(long long), cudaMemcpyDeviceToHost),
                      "cf_lu_trace_read");
}

int cf_set_stretching(cf_ctx *c, double gamma)
{
    if (!c || !(gamma > 0)) return CF_ERR_ARG;
    c->gamma = gamma;
    return CF_OK;
}

int cf_synchronize(cf_ctx *c)
{
    if (!c) return CF_ERR_ARG;
    return cuda_check(c, cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
}

size_t cf_field_count(const cf_ctx *c) { return c ? c->d.total() : 0; }

int cf_register(cf_ctx *c, double *host)
{
    if (!c || !host) return CF_ERR_ARG;
    if (c->mirrors.count(host)) return CF_OK;
    double *dev = nullptr;
    if (cudaMalloc(&dev, c->d.total() * sizeof(double)) != cudaSuccess)
        return fail(c, CF_ERR_NOMEM, "cf_register: cudaMalloc of %zu doubles failed", c->d.total());
    c->mirrors[host] = dev;
    return CF_OK;
}

int cf_unregister(cf_ctx *c, double *host)
{
    if (!c) return CF_ERR_ARG;
    auto it = c->mirrors.find(host);
    if (it == c->mirrors.end()) return fail(c, CF_ERR_ARG, "cf_unregister: pointer not registered");
    cudaFree(it->second);
    c->mirrors.erase(it);
    return CF_OK;
}

int cf_upload(cf_ctx *c, const double *host)
{
    if (!c) return CF_ERR_ARG;
    auto it = c->mirrors.find(host);
    if (it == c->mirrors.end()) return fail(c, CF_ERR_ARG, "cf_upload: pointer not registered");
    return cuda_check(c, cudaMemcpyAsync(it->second, host, c->d.total() * sizeof(double), cudaMemcpyHostToDevice,
                                         c->stream), "cf_upload");
}

int cf_download(cf_ctx *c, double *host)
{
    if (!c) return CF_ERR_ARG;
    auto it = c->mirrors.find(host);
    if (it == c->mirrors.end()) return fail(c, CF_ERR_ARG, "cf_download: pointer not registered");
    int rc = cuda_check(c, cudaMemcpyAsync(host, it->second, c->d.total() * sizeof(double), cudaMemcpyDeviceToHost,
                                           c->stream), "cf_download");
    if (rc) return rc;
    return cuda_check(c, cudaStreamSynchronize(c->stream), "cf_download sync");
}

int cf_upload_async(cf_ctx *c, const double *host, void *stream)
{
    if (!c) return CF_ERR_ARG;
    auto it = c->mirrors.find(host);
    if (it == c->mirrors.end()) return fail(c, CF_ERR_ARG, "cf_upload_async: pointer not registered");
    return cuda_check(c, cudaMemcpyAsync(it->second, host, c->d.total() * sizeof(double), cudaMemcpyHostToDevice,
                                         (cudaStream_t)stream), "cf_upload_async");
}

int cf_download_async(cf_ctx *c, double *host, void *stream)
{
    if (!c) return CF_ERR_ARG;
    auto it = c->mirrors.find(host);
    if (it == c->mirrors.end()) return fail(c, CF_ERR_ARG, "cf_download_async: pointer not registered");
    return cuda_check(c, cudaMemcpyAsync(host, it->second, c->d.total() * sizeof(double), cudaMemcpyDeviceToHost,
                                         (cudaStream_t)stream), "cf_download_async");
}

double *cf_device_ptr(cf_ctx *c, const double *p) { return c ? R(c, p) : nullptr; }

int cf_check_finite(cf_ctx *c, const double *field)
{
    if (!c || !field) return CF_ERR_ARG;
    const cf_dims &d = c->d;
    unsigned long long *bad = reinterpret_cast<unsigned long long *>(c->er_dev + 8);
    cudaMemsetAsync(bad, 0, sizeof *bad, c->stream);
    dim3 g((unsigned)((d.Z_out + 127) / 128), (unsigned)d.Y_out, (unsigned)d.X_out);
    k_count_nonfinite<<<g, 128, 0, c->stream>>>(d, R(c, field), bad);
    unsigned long long h = 0;
    int rc = cuda_check(c, cudaMemcpyAsync(&h, bad, sizeof h, cudaMemcpyDeviceToHost, c->stream), "cf_check_finite");
    if (rc) return rc;
    rc = cuda_check(c, cudaStreamSynchronize(c->stream), "cf_check_finite sync");
    if (rc) return rc;
    return h ? fail(c, CF_ERR_NONFINITE, "%llu non-finite interior values", h) : CF_OK;
}

// ---------------------------------------------------------------------------
// boundary conditions

int cf_Y_boundary_condition(cf_ctx *c, int, double *U1_, double *U2_, double *U3_, double *U4_, double *U5_,
                            double *J)
{
    if (!c) return CF_ERR_ARG;
    const double *p[6] = {U1_, U2_, U3_, U4_, U5_, J};
    if (int rc = check_ptrs(c, p, 6, "Y_boundary_condition")) return rc;
    cf_ptr5 U{{R(c, U1_), R(c, U2_), R(c, U3_), R(c, U4_), R(c, U5_)}};
    cudaError_t e = exact(c) ? cf_exact::y_wall(c->d, U, R(c, J), c->stream)
                             : cf_fast::y_wall(c->d, U, R(c, J), c->stream);
    return cuda_check(c, e, "Y_boundary_condition");
}

int cf_Z_boundary_condition(cf_ctx *c, int, double *U1_, double *U2_, double *U3_, double *U4_, double *U5_,
                            double *J)
{
    if (!c) return CF_ERR_ARG;
    const double *p[5] = {U1_, U2_, U3_, U4_, U5_};
    if (int rc = check_ptrs(c, p, 5, "Z_boundary_condition")) return rc;
    (void)J;
    cf_ptr5 U{{R(c, U1_), R(c, U2_), R(c, U3_), R(c, U4_), R(c, U5_)}};
    return cuda_check(c, cf_exact::z_periodic(c->d, U, c->stream), "Z_boundary_condition");
}

int cf_X_periodic(cf_ctx *c, int, double *U1_, double *U2_, double *U3_, double *U4_, double *U5_)
{
    if (!c) return CF_ERR_ARG;
    const double *p[5] = {U1_, U2_, U3_, U4_, U5_};
    if (int rc = check_ptrs(c, p, 5, "X_periodic")) return rc;
    cf_ptr5 U{{R(c, U1_), R(c, U2_), R(c, U3_), R(c, U4_), R(c, U5_)}};
    return cuda_check(c, cf_exact::x_periodic(c->d, U, c->stream), "X_periodic");
}

// ---------------------------------------------------------------------------
// fluxes

// The FP32 copy of a metric array that the caller keeps fixed across
// cf_step calls (cf_step_params.static_metrics), made on first use; null
// when it cannot be made (the kernels then read the FP64 array)
static const float *met32_get(cf_ctx *c, const double *p)
{
    if (!p) return nullptr;
    auto it = c->met32.find(p);
    if (it != c->met32.end()) return it->second;
    float *f = nullptr;
    const size_t n = c->d.total();
    if (cudaMalloc(&f, n * sizeof(float)) != cudaSuccess) return nullptr;
    if (cf_fast::to_f32(n, p, f, c->stream) != cudaSuccess) {
        cudaFree(f);
        return nullptr;
    }
    c->met32[p] = f;
    return f;
}

// reuse_shadow: the FP32 copies of U and J made by the previous FP32 flux
// call are still current (the step driver's y and z fluxes after x)
// f32_out: in FP32 mode, write inF as FP32 values into their FP64 arrays
// (only the step driver, whose own Dual_time_stepping reads them)
static int flux_common(cf_ctx *c, const char *who, int dir, bool limited, double *const *p32,
                       bool reuse_shadow = false, bool f32_out = false, bool static_metrics = false)
{
    if (!c) return CF_ERR_ARG;
    // arrays 5..14 (ML/MR) are the reference's scratch and are not needed
    for (int i = 0; i < 32; i++) {
        if (i >= 5 && i < 15) continue;
        if (i == 15 && dir == 0 && limited) continue;       // X limiter does not read J
        if (i == 31 && !limited) continue;                  // unlimited fluxes do not read Ep
        if (!p32[i]) return fail(c, CF_ERR_ARG, "%s: array argument %d is NULL", who, i);
    }
    cf_flux_args a;
    for (int n = 0; n < 5; n++) a.U[n] = R(c, p32[n]);
    a.J = p32[15] ? R(c, p32[15]) : nullptr;
    a.Jf = R(c, p32[16]);
    for (int n = 0; n < 9; n++) a.m[n] = R(c, p32[17 + n]);
    for (int n = 0; n < 5; n++) a.F[n] = R(c, p32[26 + n]);
    a.Ep = p32[31] ? R(c, p32[31]) : nullptr;
    a.wz[0] = a.wz[1] = nullptr;
    a.f32_out = (f32_out && kprec(c) == 1) ? 1 : 0;
    a.reserved = 0;
    if (dir == 2 && limited) {
        double *wz = scratch(c, "flux_zweights", 2);
        if (!wz) return fail(c, CF_ERR_NOMEM, "%s: scratch allocation failed", who);
        a.wz[0] = wz;
        a.wz[1] = wz + c->d.total();
    }
    if (kprec(c) == 1) {
        // FP32: the stencils read FP32 copies of U, J, 1/J (7 fields)
        double *sh = scratch(c, "flux_f32", 4);
        if (!sh) return fail(c, CF_ERR_NOMEM, "%s: scratch allocation failed", who);
        if (!a.J && dir != 0) return fail(c, CF_ERR_ARG, "%s: J is NULL", who);
        const float *m32[10] = {nullptr};
        if (static_metrics) {
            m32[0] = met32_get(c, a.Jf);
            for (int n = 0; n < 9; n++) m32[1 + n] = met32_get(c, a.m[n]);
            for (int n = 0; n < 10; n++)
                if (!m32[n]) return fail(c, CF_ERR_NOMEM, "%s: FP32 metric copy allocation failed", who);
        }
        // with fixed metrics the shadow's J and 1/J, once made from this J,
        // stay current: only U is converted again (a null J skips them)
        const double *J_in = a.J;
        if (static_metrics && !reuse_shadow && a.J && c->shadow_j == a.J) a.J = nullptr;
        // the step driver's layout (FP32 outputs, FP32 metric copies): the
        // variant compiled for it
        auto fn = (a.f32_out && static_metrics) ? cf_drv::flux_f32 : cf_fast::flux_f32;
        const int rc = cuda_check(c, fn(c->d, a, reinterpret_cast<float *>(sh), !reuse_shadow,
                                        static_metrics ? m32 : nullptr, dir, limited, c->stream), who);
        if (!reuse_shadow) c->shadow_j = (rc == CF_OK && static_metrics) ? J_in : nullptr;
        return rc;
    }
    cudaError_t e = exact(c) ? cf_exact::flux(c->d, a, dir, limited, 0, c->stream)
                             : cf_fast::flux(c->d, a, dir, limited, 0, c->stream);
    return cuda_check(c, e, who);
}

#define CF_FLUX_LIST                                                                                  \
    U1_, U2_, U3_, U4_, U5_, MR1, MR2, MR3, MR4, MR5, ML1, ML2, ML3, ML4, ML5, J, J_f, xidx_f, xidy_f, \
        xidz_f, etdx_f, etdy_f, etdz_f, ztdx_f, ztdy_f, ztdz_f, inF1, inF2, inF3, inF4, inF5, Ep

#define CF_FLUX_ENTRY(name, dir, lim)                                   \
    int cf_##name(cf_ctx *c, int, CF_FLUX_ARRAYS)                       \
    {                                                                   \
        double *const p[32] = {CF_FLUX_LIST};                           \
        return flux_common(c, #name, dir, lim, p);                      \
    }

CF_FLUX_ENTRY(Flux_X_limiter, 0, true)
CF_FLUX_ENTRY(Flux_Y_limiter, 1, true)
CF_FLUX_ENTRY(Flux_Z_limiter, 2, true)
CF_FLUX_ENTRY(Flux_X, 0, false)
CF_FLUX_ENTRY(Flux_Y, 1, false)
CF_FLUX_ENTRY(Flux_Z, 2, false)

// ---------------------------------------------------------------------------
// viscous terms

// f32_io: in FP32 mode, LL/ML/NL and vF hold FP32 values (the step driver)
// step_copies: the FP32 step driver's copies of U_ and J for this
// sub-iteration are current (the viscous terms then run as one pass that
// writes vF only)
static int viscous_common(cf_ctx *c, double **p, bool f32_io, bool static_metrics = false,
                          bool step_copies = false)
{
    if (!c || !p) return CF_ERR_ARG;
    // read: U (0-4), J (9), face metric sets (19-48); written: vF (5-8),
    // LL2..5 (55-58), ML2..5 (65-68), NL2..5 (75-78)
    static const int need[] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30,
                               31, 32, 33, 34, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48,
                               55, 56, 57, 58, 65, 66, 67, 68, 75, 76, 77, 78};
    for (int i : need)
        if (!p[i]) return fail(c, CF_ERR_ARG, "Viscous_terms: array argument %d is NULL", i);
    cf_visc_args a;
    for (int n = 0; n < 5; n++) a.U[n] = R(c, p[n]);
    for (int n = 0; n < 4; n++) a.vF[n] = R(c, p[5 + n]);
    a.J = R(c, p[9]);
    for (int f = 0; f < 3; f++) {
        a.Jf[f] = R(c, p[19 + 10 * f]);
        for (int n = 0; n < 9; n++) a.mf[f][n] = R(c, p[20 + 10 * f + n]);
    }
    for (int n = 0; n < 4; n++) {
        a.LL[n] = R(c, p[55 + n]);
        a.ML[n] = R(c, p[65 + n]);
        a.NL[n] = R(c, p[75 + n]);
    }
    double *prim = scratch(c, "visc_prim", 4);
    if (!prim) return fail(c, CF_ERR_NOMEM, "Viscous_terms: scratch allocation failed");
    for (int n = 0; n < 4; n++) a.prim[n] = prim + (size_t)n * c->d.total();
    a.f32_io = (f32_io && kprec(c) == 1) ? 1 : 0;
    a.reserved = 0;
    const bool m32 = static_metrics && kprec(c) == 1;
    for (int f = 0; f < 3; f++) {
        a.Jf32[f] = m32 ? met32_get(c, a.Jf[f]) : nullptr;
        for (int n = 0; n < 9; n++) a.mf32[f][n] = m32 ? met32_get(c, a.mf[f][n]) : nullptr;
        if (m32 && !a.Jf32[f]) return fail(c, CF_ERR_NOMEM, "Viscous_terms: FP32 metric copy allocation failed");
        for (int n = 0; n < 9; n++)
            if (m32 && !a.mf32[f][n]) return fail(c, CF_ERR_NOMEM, "Viscous_terms: FP32 metric copy allocation failed");
    }
    for (int n = 0; n < 5; n++) a.U32[n] = nullptr;
    a.J32 = nullptr;
    if (step_copies && a.f32_io && m32) {
        // the sub-iteration's FP32 copies of U_ and J (made by Flux_X)
        const float *sh = reinterpret_cast<const float *>(scratch(c, "flux_f32", 4));
        if (!sh) return fail(c, CF_ERR_NOMEM, "Viscous_terms: scratch allocation failed");
        const size_t n = c->d.total();
        for (int v = 0; v < 5; v++) a.U32[v] = sh + v * n;
        a.J32 = sh + 5 * n;
    }
    cudaError_t e = exact(c) ? cf_exact::viscous(c->d, a, 0, c->stream)
                    : (a.f32_io && m32) ? cf_drv::viscous(c->d, a, kprec(c), c->stream)
                                        : cf_fast::viscous(c->d, a, kprec(c), c->stream);
    return cuda_check(c, e, "Viscous_terms");
}

int cf_Viscous_terms(cf_ctx *c, int, double **p) { return viscous_common(c, p, false); }

// ---------------------------------------------------------------------------
// sensor

int cf_Filter(cf_ctx *c, int, double Roe_criterion, double E_high, double E_low, double *U1_, double *U2_,
              double *U3_, double *U4_, double *U5_, double *Y_point, double *EpX, double *EpY, double *EpZ,
              double *J)
{
    if (!c) return CF_ERR_ARG;
    const double *p[10] = {U1_, U2_, U3_, U4_, U5_, Y_point, EpX, EpY, EpZ, J};
    if (int rc = check_ptrs(c, p, 10, "Filter")) return rc;
    cf_filter_args a;
    for (int n = 0; n < 5; n++) a.U[n] = R(c, p[n]);
    a.Yp = R(c, Y_point);
    a.J = R(c, J);
    a.Ep[0] = R(c, EpX); a.Ep[1] = R(c, EpY); a.Ep[2] = R(c, EpZ);
    double *s = scratch(c, "filter", 17);
    if (!s) return fail(c, CF_ERR_NOMEM, "Filter: scratch allocation failed");
    const size_t n = c->d.total();
    int f = 0;
    for (int l = 0; l < 2; l++)
        for (int v = 0; v < 4; v++) a.lev[l][v] = s + n * f++;
    for (int v = 0; v < 4; v++) a.acc[v] = s + n * f++;
    a.cA = s + n * f++;
    a.cC = s + n * f++;
    a.cB = s + n * f++;
    a.Eh = s + n * f++;
    a.E2h = s + n * f++;
    // FP64 exact: the reference's expression trees (no FMA), so the switch
    // takes the reference's decisions; FP64: contracted, reciprocal weights;
    // FP32: float arithmetic and float scratch levels
    cudaError_t e = c->prec == CF_PREC_FP64_EXACT
                        ? cf_exact::filter(c->d, a, Roe_criterion, E_high, E_low, 0, c->stream)
                        : cf_fast::filter(c->d, a, Roe_criterion, E_high, E_low, kprec(c), c->stream);
    return cuda_check(c, e, "Filter");
}

// ---------------------------------------------------------------------------
// time integration

int cf_RK3NODT(cf_ctx *c, int, int RK, double deltaT, double *, double *, double *, double *, double *,
               double **p)
{
    if (!c || !p) return CF_ERR_ARG;
    if (RK < 1 || RK > 3) return fail(c, CF_ERR_ARG, "RK3NODT: RK must be 1, 2 or 3");
    static const int need[] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 15, 25, 26, 27, 28, 29, 30, 31, 32, 33, 34,
                               35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48};
    for (int i : need)
        if (!p[i]) return fail(c, CF_ERR_ARG, "RK3NODT: array argument %d is NULL", i);
    cf_rk3_args a;
    for (int n = 0; n < 5; n++) {
        a.U_[n] = R(c, p[n]);
        a.U[n] = R(c, p[5 + n]);
        a.Fx[n] = R(c, p[25 + n]);
        a.Fy[n] = R(c, p[30 + n]);
        a.Fz[n] = R(c, p[35 + n]);
        a.MR[n] = R(c, p[44 + n]);
    }
    a.J = R(c, p[15]);
    for (int n = 0; n < 4; n++) a.vF[n] = R(c, p[40 + n]);
    cudaError_t e = exact(c) ? cf_exact::rk3(c->d, a, RK, deltaT, 0, c->stream)
                             : cf_fast::rk3(c->d, a, RK, deltaT, kprec(c), c->stream);
    return cuda_check(c, e, "RK3NODT");
}

int cf_Hyperplane(cf_ctx *c, int, int *Nijk, int *ijk)
{
    if (!c || !Nijk || !ijk) return CF_ERR_ARG;
    std::memcpy(Nijk, c->nijk.data(), c->nijk.size() * sizeof(int));
    std::memcpy(ijk, c->ijk.data(), c->ijk.size() * sizeof(int));
    return CF_OK;
}

static int lu_args(cf_ctx *c, double **p, const char *who, cf_lu_args &a)
{
    static const int skip_lo = 44;  // everything up to MR is read or written
    (void)skip_lo;
    for (int i = 0; i < 64; i++)
        if (!p[i]) return fail(c, CF_ERR_ARG, "%s: array argument %d is NULL", who, i);
    for (int n = 0; n < 5; n++) {
        a.U_[n] = R(c, p[n]);
        a.U[n] = R(c, p[5 + n]);
        a.Uq[n] = R(c, p[10 + n]);
        a.Fx[n] = R(c, p[25 + n]);
        a.Fy[n] = R(c, p[30 + n]);
        a.Fz[n] = R(c, p[35 + n]);
        a.MR[n] = R(c, p[44 + n]);
        a.NR[n] = R(c, p[49 + n]);
        a.NL[n] = R(c, p[54 + n]);
        a.Res[n] = R(c, p[59 + n]);
    }
    a.J = R(c, p[15]);
    for (int n = 0; n < 9; n++) a.m[n] = R(c, p[16 + n]);
    for (int n = 0; n < 4; n++) a.vF[n] = R(c, p[40 + n]);
    a.f32_rhs = 0;
    a.f32_lu = 0;
    for (int n = 0; n < 9; n++) a.m32[n] = nullptr;
    for (int n = 0; n < 5; n++) a.U32[n] = a.dUq32[n] = nullptr;
    a.J32 = nullptr;
    cf_dims &d = c->d;
    const size_t np = cf_fast::lu_partial_count(d);
    auto &e = c->scratch["lu_partial"];
    if (!e.first || e.second < 5 * np * sizeof(double)) {
        if (e.first) cudaFree(e.first);
        e.first = nullptr;
        if (cudaMalloc(&e.first, 5 * np * sizeof(double)) != cudaSuccess) {
            e.first = nullptr;
            return fail(c, CF_ERR_NOMEM, "%s: scratch allocation failed", who);
        }
        e.second = 5 * np * sizeof(double);
    }
    a.partial = e.first;
    return CF_OK;
}

static int lu_read_norms(cf_ctx *c, double *er[5], const char *who)
{
    if (int rc = cuda_check(c, cudaMemcpyAsync(c->er_host, c->er_dev, 5 * sizeof(double), cudaMemcpyDeviceToHost,
                                               c->stream), who)) return rc;
    if (int rc = cuda_check(c, cudaStreamSynchronize(c->stream), who)) return rc;
    for (int n = 0; n < 5; n++)
        if (er[n]) *er[n] = c->er_host[n];
    return CF_OK;
}

static int lu_finish_host(cf_ctx *c, const cf_lu_args &a, double *er[5], const char *who)
{
    cudaError_t e = exact(c) ? cf_exact::lu_finish(c->d, a, c->er_dev, 0, c->stream)
                             : cf_fast::lu_finish(c->d, a, c->er_dev, kprec(c), c->stream);
    if (int rc = cuda_check(c, e, who)) return rc;
    return lu_read_norms(c, er, who);
}

// tiling and scratch of the wavefront sweeps (cf_wave.cuh)
static int wave_setup(cf_ctx *c, cf_wave_args &w)
{
    const cf_dims &d = c->d;
    w.d = d;
    w.nti = (d.X_out + CF_WAVE_TI - 1) / CF_WAVE_TI;
    w.ntj = (d.Y_out + CF_WAVE_TJ - 1) / CF_WAVE_TJ;
    w.ntk = (d.Z_out + CF_WAVE_TK - 1) / CF_WAVE_TK;
    w.ntiles = w.nti * w.ntj * w.ntk;
    if (!c->tile_order) {
        // topological order of both sweeps: tiles by ti + tj + tk
        std::vector<int> order;
        order.reserve((size_t)w.ntiles);
        for (int p = 0; p <= w.nti + w.ntj + w.ntk - 3; p++)
            for (int a = 0; a < w.nti; a++)
                for (int b = 0; b < w.ntj; b++) {
                    const int k = p - a - b;
                    if (k >= 0 && k < w.ntk) order.push_back((a * w.ntj + b) * w.ntk + k);
                }
        if (cudaMalloc(&c->tile_order, order.size() * sizeof(int)) != cudaSuccess) {
            c->tile_order = nullptr;
            return fail(c, CF_ERR_NOMEM, "Dual_time_stepping: tile table allocation failed");
        }
        if (int rc = cuda_check(c, cudaMemcpy(c->tile_order, order.data(), order.size() * sizeof(int),
                                              cudaMemcpyHostToDevice), "tile table")) return rc;
    }
    w.order = c->tile_order;
    const size_t cells = (size_t)CF_WAVE_TI * CF_WAVE_TJ * CF_WAVE_TK;
    const size_t T8 = sizeof(double);       // sized for double; the FP32 kernels use half
    const size_t pack = (size_t)w.ntiles * cells * CF_WAVE_PACK * T8;
    const size_t fx = (size_t)w.ntiles * 5 * CF_WAVE_TJ * CF_WAVE_TK * T8;
    const size_t fy = (size_t)w.ntiles * 5 * CF_WAVE_TI * CF_WAVE_TK * T8;
    const size_t fz = (size_t)w.ntiles * 5 * CF_WAVE_TI * CF_WAVE_TJ * T8;
    const size_t nl = (size_t)w.ntiles * 5 * cells * T8;
    const size_t flags = (((size_t)w.ntiles + 2) * sizeof(int) + 255) / 256 * 256;
    unsigned char *base = static_cast<unsigned char *>(
        scratch_bytes(c, "lu_wave", pack + fx + fy + fz + nl + flags));
    if (!base) return fail(c, CF_ERR_NOMEM, "Dual_time_stepping: wavefront scratch allocation failed");
    w.pack = base;
    w.inx = base + pack;
    w.iny = base + pack + fx;
    w.inz = base + pack + fx + fy;
    w.nl = base + pack + fx + fy + fz;
    unsigned char *f = base + pack + fx + fy + fz + nl;
    w.flags = reinterpret_cast<int *>(f);
    w.counter = w.flags + w.ntiles;
    w.err = w.flags + w.ntiles + 1;
    w.dep_limit = c->wait_limit;
    w.trace = nullptr;
    if (c->trace_tiles) {
        if (c->trace_tiles != (size_t)w.ntiles) {
            if (c->trace) cudaFree(c->trace);
            c->trace = nullptr;
            if (cudaMalloc(&c->trace, 2 * 4 * (size_t)w.ntiles * sizeof(long long)) != cudaSuccess) {
                c->trace = nullptr;
                c->trace_tiles = 0;
                return fail(c, CF_ERR_NOMEM, "Dual_time_stepping: trace allocation failed");
            }
            c->trace_tiles = (size_t)w.ntiles;
        }
        w.trace = c->trace;
    }
    return CF_OK;
}

// pencils and scratch of the pencil sweeps (cf_pencil.cuh)
static int pencil_setup(cf_ctx *c, cf_wave_args &w)
{
    const cf_dims &d = c->d;
    w.d = d;
    w.npj = (d.Y_out + CF_PENCIL_TJ - 1) / CF_PENCIL_TJ;
    w.npk = (d.Z_out + CF_PENCIL_TK - 1) / CF_PENCIL_TK;
    w.npencils = w.npj * w.npk;
    w.nplanes = d.X_out + (CF_PENCIL_TJ - 1) + (CF_PENCIL_TK - 1);
    w.ntiles = w.npencils;
    if (!c->pencil_order) {
        // topological order of both sweeps: pencils by pj + pk
        std::vector<int> order;
        order.reserve((size_t)w.npencils);
        for (int p = 0; p <= w.npj + w.npk - 2; p++)
            for (int b = 0; b < w.npj; b++) {
                const int k = p - b;
                if (k >= 0 && k < w.npk) order.push_back(b * w.npk + k);
            }
        if (cudaMalloc(&c->pencil_order, order.size() * sizeof(int)) != cudaSuccess) {
            c->pencil_order = nullptr;
            return fail(c, CF_ERR_NOMEM, "Dual_time_stepping: pencil table allocation failed");
        }
        if (int rc = cuda_check(c, cudaMemcpy(c->pencil_order, order.data(), order.size() * sizeof(int),
                                              cudaMemcpyHostToDevice), "pencil table")) return rc;
    }
    w.order = c->pencil_order;
    const size_t T8 = sizeof(double);       // sized for double; the FP32 kernels use half
    const size_t np = (size_t)w.npencils;
    const size_t pack = np * w.nplanes * CF_WAVE_PACK * 32 * T8;
    const size_t nl = np * w.nplanes * 5 * 32 * T8;
    const size_t xg = np * 5 * 32 * T8;
    // exchange words: 64 bits per 32-bit part of a value (two parts for double)
    const size_t yex = np * d.X_out * 5 * CF_PENCIL_TK * 2 * sizeof(unsigned long long);
    const size_t zex = np * d.X_out * 5 * CF_PENCIL_TJ * 2 * sizeof(unsigned long long);
    const size_t flags = ((np + 3) * sizeof(int) + 255) / 256 * 256;
    const size_t total = pack + nl + xg + yex + zex + flags;
    const bool fresh = !c->scratch["lu_pencil"].first || c->scratch["lu_pencil"].second < total;
    unsigned char *base = static_cast<unsigned char *>(scratch_bytes(c, "lu_pencil", total));
    if (!base) return fail(c, CF_ERR_NOMEM, "Dual_time_stepping: pencil scratch allocation failed");
    // a new buffer: exchange tags and the epoch start at zero (the first
    // call's tags are 2 and 3)
    if (fresh)
        if (int rc = cuda_check(c, cudaMemset(base + pack + nl + xg, 0, yex + zex + flags), "pencil scratch"))
            return rc;
    w.pack = base;
    w.nl = base + pack;
    w.xg = base + pack + nl;
    w.yex = base + pack + nl + xg;
    w.zex = base + pack + nl + xg + yex;
    w.flags = reinterpret_cast<int *>(base + pack + nl + xg + yex + zex);
    w.counter = w.flags + w.npencils;
    w.err = w.flags + w.npencils + 1;
    w.dep_limit = c->wait_limit;
    w.trace = nullptr;
    if (c->trace_tiles) {
        // per sweep and pencil: the claim, then the end of each block wait
        const size_t per = (size_t)w.npencils * ((w.nplanes + CF_PENCIL_PUB - 1) / CF_PENCIL_PUB + 1);
        const size_t units = (per + 3) / 4;
        if (c->trace_tiles != units) {
            if (c->trace) cudaFree(c->trace);
            c->trace = nullptr;
            if (cudaMalloc(&c->trace, 2 * 4 * units * sizeof(long long)) != cudaSuccess) {
                c->trace = nullptr;
                c->trace_tiles = 0;
                return fail(c, CF_ERR_NOMEM, "Dual_time_stepping: trace allocation failed");
            }
            c->trace_tiles = units;
        }
        w.trace = c->trace;
    }
    return CF_OK;
}

// The whole Dual_time_stepping call on stream s: assembly, one forward and
// one backward hyperplane sweep, NL <- NR, update and norms into er_dev.
//
// The reference runs the forward/backward pair twice
// (Dual_time_stepping.cpp:563-1275) so that, with several ranks, the
// second pass sees the neighbours' interface planes of the first.  On one
// domain the second pass reproduces the first bit for bit: the sweeps read
// N only at ghost cells (zero, never written) and at cells the same sweep
// has already recomputed from MR and fixed coefficients.  It is run once.
//
// Schedules: CF_LU_WAVEFRONT, one persistent tiled launch per sweep
// (cf_wave.cuh); CF_LU_PENCIL, one persistent launch per sweep of warps
// sweeping 4x8 pencils (cf_pencil.cuh); CF_LU_PLANES, one launch per
// hyperplane from a per-cell coefficient pack.  All give the same bits.
static cudaError_t enqueue_dts(cf_ctx *c, const cf_lu_args &a, double *pack, const cf_wave_args &w, double dt,
                               cudaStream_t s)
{
    const cf_dims &d = c->d;
    const bool ex = exact(c);
    const int pr = ex ? 0 : kprec(c);
    cudaError_t e = cudaSuccess;
    if (c->lu_schedule == CF_LU_PENCIL) {
        // as the tiled wavefront below: FP64 assembles inside the pack
        const bool asm_in_pack = pr != 1;
        const bool st = pr == 1 && a.f32_rhs && a.f32_lu && a.m32[0] && a.U32[0] && a.J32 && a.dUq32[0];
        auto prepare = st ? cf_drv::lu_prepare : cf_fast::lu_prepare;
        auto ppack = st ? cf_drv::lu_pencil_pack : cf_fast::lu_pencil_pack;
        auto psweep = st ? cf_drv::lu_pencil_sweep : cf_fast::lu_pencil_sweep;
        e = asm_in_pack ? (ex ? cf_exact::lu_zero(d, a, s) : cf_fast::lu_zero(d, a, s))
                        : prepare(d, a, dt, true, pr, s);
        const size_t fl = ((size_t)w.npencils + 1) * sizeof(int);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.err, 0, sizeof(int), s);
        if (e == cudaSuccess) e = ex ? cf_exact::lu_pencil_pack(d, a, w, dt, false, true, 0, s)
                                     : ppack(d, a, w, dt, false, asm_in_pack, pr, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.flags, 0, fl, s);
        if (e == cudaSuccess) e = ex ? cf_exact::lu_pencil_sweep(a, w, true, 0, s) : psweep(a, w, true, pr, s);
        if (e == cudaSuccess) e = ex ? cf_exact::lu_pencil_pack(d, a, w, dt, true, false, 0, s)
                                     : ppack(d, a, w, dt, true, false, pr, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.flags, 0, fl, s);
        cf_wave_args wb = w;
        if (w.trace) wb.trace = w.trace + 4 * c->trace_tiles;
        if (e == cudaSuccess) e = ex ? cf_exact::lu_pencil_sweep(a, wb, false, 0, s) : psweep(a, wb, false, pr, s);
        if (pr == 1) {
            auto finish = st ? cf_drv::lu_finish : cf_fast::lu_finish;
            if (e == cudaSuccess) e = finish(d, a, c->er_dev, pr, s);
            return e;
        }
    } else if (c->lu_schedule == CF_LU_WAVEFRONT) {
        // FP64: the assembly happens inside the forward tile pack (one pass
        // over the cells less); FP32: its own box kernel, which measured
        // faster than the heavier FP32 pack kernel doing both
        const bool asm_in_pack = pr != 1;
        // the step driver's FP32 layout (every FP32 copy set up): the kernels
        // compiled for it
        const bool st = pr == 1 && a.f32_rhs && a.f32_lu && a.m32[0] && a.U32[0] && a.J32 && a.dUq32[0];
        auto prepare = st ? cf_drv::lu_prepare : cf_fast::lu_prepare;
        auto wpack = st ? cf_drv::lu_wave_pack : cf_fast::lu_wave_pack;
        auto wsweep = st ? cf_drv::lu_wave_sweep : cf_fast::lu_wave_sweep;
        e = asm_in_pack ? (ex ? cf_exact::lu_zero(d, a, s) : cf_fast::lu_zero(d, a, s))
                        : prepare(d, a, dt, true, pr, s);
        const size_t fl = ((size_t)w.ntiles + 1) * sizeof(int);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.err, 0, sizeof(int), s);
        if (e == cudaSuccess) e = ex ? cf_exact::lu_wave_pack(d, a, w, dt, false, true, 0, s)
                                     : wpack(d, a, w, dt, false, asm_in_pack, pr, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.flags, 0, fl, s);
        if (e == cudaSuccess) e = ex ? cf_exact::lu_wave_sweep(a, w, true, 0, s)
                                     : wsweep(a, w, true, pr, s);
        cf_wave_args wb = w;
        if (w.trace) wb.trace = w.trace + 4 * (size_t)w.ntiles;
        if (e == cudaSuccess) e = ex ? cf_exact::lu_wave_pack(d, a, w, dt, true, false, 0, s)
                                     : wpack(d, a, w, dt, true, false, pr, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.flags, 0, fl, s);
        if (e == cudaSuccess) e = ex ? cf_exact::lu_wave_sweep(a, wb, false, 0, s)
                                     : wsweep(a, wb, false, pr, s);
        // the state update and the norms as their own pass over the cells
        // (in FP32 it also copies NL <- NR; fused into the backward sweep's
        // tiles it took the blocks' time between tiles, which at
        // 256x192x192 cost more than the pass)
        if (pr == 1) {
            auto finish = st ? cf_drv::lu_finish : cf_fast::lu_finish;
            if (e == cudaSuccess) e = finish(d, a, c->er_dev, pr, s);
            return e;
        }
    } else {
        e = ex ? cf_exact::lu_prepare(d, a, dt, true, 0, s) : cf_fast::lu_prepare(d, a, dt, true, pr, s);
        if (e == cudaSuccess) e = ex ? cf_exact::lu_pack(d, a, pack, dt, 0, s) : cf_fast::lu_pack(d, a, pack, dt, pr, s);
        const int mlast = d.gend + d.ny + d.nz;
        for (int m = 7; m <= mlast && e == cudaSuccess; m++) {
            const int cnt = c->nijk[2 * (size_t)m + 1], first = c->nijk[2 * (size_t)m] - cnt + 1;
            e = ex ? cf_exact::lu_plane_packed(d, a, pack, c->ijk_dev, first, cnt, true, 0, s)
                   : cf_fast::lu_plane_packed(d, a, pack, c->ijk_dev, first, cnt, true, pr, s);
        }
        for (int m = mlast; m >= 7 && e == cudaSuccess; m--) {
            const int cnt = c->nijk[2 * (size_t)m + 1], first = c->nijk[2 * (size_t)m] - cnt + 1;
            e = ex ? cf_exact::lu_plane_packed(d, a, pack, c->ijk_dev, first, cnt, false, 0, s)
                   : cf_fast::lu_plane_packed(d, a, pack, c->ijk_dev, first, cnt, false, pr, s);
        }
    }
    if (e == cudaSuccess) e = cf_fast::lu_copy(d, a, s);
    if (e == cudaSuccess) e = ex ? cf_exact::lu_finish(d, a, c->er_dev, 0, s) : cf_fast::lu_finish(d, a, c->er_dev, pr, s);
    return e;
}

// capture enqueue_dts into c->dts_exec (kept while the arguments repeat)
static int capture_dts(cf_ctx *c, const cf_lu_args &a, double *pack, const cf_wave_args &w, double dt)
{
    if (!c->cap) {
        if (int rc = cuda_check(c, cudaStreamCreateWithFlags(&c->cap, cudaStreamNonBlocking), "capture stream"))
            return rc;
    }
    if (c->dts_exec) {
        cudaGraphExecDestroy(c->dts_exec);
        c->dts_exec = nullptr;
    }
    c->dts_key.clear();
    if (int rc = cuda_check(c, cudaStreamBeginCapture(c->cap, cudaStreamCaptureModeThreadLocal), "graph capture"))
        return rc;
    const cudaError_t le = enqueue_dts(c, a, pack, w, dt, c->cap);
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(c->cap, &g);
    if (le != cudaSuccess || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_check(c, le != cudaSuccess ? le : ee, "Dual_time_stepping capture");
    }
    const cudaError_t ie = cudaGraphInstantiate(&c->dts_exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        c->dts_exec = nullptr;
        return cuda_check(c, ie, "Dual_time_stepping graph");
    }
    return CF_OK;
}

// f32_rhs: in FP32 mode, Fx/Fy/Fz and vF hold FP32 values (the step driver)
// step_copies (FP32 step driver): the FP32 copies of U_ and J that this
// sub-iteration's fluxes made, and float(U - Uq) of the physical step, are
// current; the LU-SGS kernels read them instead of converting
static int dts_common(cf_ctx *c, double deltaT, double *er1, double *er2, double *er3, double *er4, double *er5,
                      int *Nijk, int *ijk, double **p, bool f32_rhs, bool static_metrics = false,
                      bool step_copies = false)
{
    if (!c || !p) return CF_ERR_ARG;
    // the plane tables are a fixed function of the grid; the context holds
    // them already.  Tables handed in are checked once against them.
    if (Nijk && ijk && !c->tables_checked) {
        if (std::memcmp(Nijk, c->nijk.data(), c->nijk.size() * sizeof(int)) != 0)
            return fail(c, CF_ERR_ARG, "Dual_time_stepping: Nijk differs from the Hyperplane tables of this grid");
        c->tables_checked = true;
    }
    cf_lu_args a{};
    if (int rc = lu_args(c, p, "Dual_time_stepping", a)) return rc;
    a.f32_rhs = (f32_rhs && kprec(c) == 1) ? 1 : 0;
    // with the wavefront, MR, NL and NR pass between the step driver's own
    // FP32 kernels only
    a.f32_lu = (a.f32_rhs && c->lu_schedule != CF_LU_PLANES) ? 1 : 0;
    if (static_metrics && kprec(c) == 1)
        for (int n = 0; n < 9; n++) {
            a.m32[n] = met32_get(c, a.m[n]);
            if (!a.m32[n]) return fail(c, CF_ERR_NOMEM, "Dual_time_stepping: FP32 metric copy allocation failed");
        }
    if (step_copies && kprec(c) == 1) {
        const float *sh = reinterpret_cast<const float *>(scratch(c, "flux_f32", 4));
        const float *dq = reinterpret_cast<const float *>(scratch(c, "step_duq", 3));
        if (!sh || !dq) return fail(c, CF_ERR_NOMEM, "Dual_time_stepping: scratch allocation failed");
        const size_t n = c->d.total();
        for (int v = 0; v < 5; v++) {
            a.U32[v] = sh + v * n;
            a.dUq32[v] = dq + v * n;
        }
        a.J32 = sh + 5 * n;
    }
    double *pack = nullptr;
    cf_wave_args w{};
    if (c->lu_schedule == CF_LU_WAVEFRONT) {
        if (int rc = wave_setup(c, w)) return rc;
    } else if (c->lu_schedule == CF_LU_PENCIL) {
        if (int rc = pencil_setup(c, w)) return rc;
    } else {
        pack = scratch(c, "lu_pack", CF_LU_PACK);
        if (!pack) return fail(c, CF_ERR_NOMEM, "Dual_time_stepping: coefficient pack allocation failed");
    }
    // the graph bakes in every pointer and scalar: recapture when they change
    std::vector<unsigned char> key(sizeof(cf_lu_args) + sizeof(double *) + sizeof(void *) + sizeof(double) +
                                   2 * sizeof(int), 0);
    unsigned char *kp = key.data();
    std::memcpy(kp, &a, sizeof a);
    kp += sizeof a;
    std::memcpy(kp, &pack, sizeof pack);
    kp += sizeof pack;
    std::memcpy(kp, &w.pack, sizeof w.pack);
    kp += sizeof w.pack;
    std::memcpy(kp, &deltaT, sizeof deltaT);
    kp += sizeof deltaT;
    std::memcpy(kp, &c->prec, sizeof c->prec);
    kp += sizeof c->prec;
    std::memcpy(kp, &c->lu_schedule, sizeof c->lu_schedule);
    key.insert(key.end(), reinterpret_cast<const unsigned char *>(&w.trace),
               reinterpret_cast<const unsigned char *>(&w.trace) + sizeof w.trace);
    key.insert(key.end(), reinterpret_cast<const unsigned char *>(&w.dep_limit),
               reinterpret_cast<const unsigned char *>(&w.dep_limit) + sizeof w.dep_limit);
    if (!c->dts_exec || key != c->dts_key) {
        if (int rc = capture_dts(c, a, pack, w, deltaT)) return rc;
        c->dts_key = key;
    }
    if (int rc = cuda_check(c, cudaGraphLaunch(c->dts_exec, c->stream), "Dual_time_stepping")) return rc;
    int *err_host = reinterpret_cast<int *>(c->er_host + 12);
    *err_host = 0;
    if (c->lu_schedule != CF_LU_PLANES)
        if (int rc = cuda_check(c, cudaMemcpyAsync(err_host, w.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream),
                                "Dual_time_stepping")) return rc;
    double *er[5] = {er1, er2, er3, er4, er5};
    if (int rc = lu_read_norms(c, er, "Dual_time_stepping")) return rc;
    if (*err_host)
        return fail(c, CF_ERR_TIMEOUT, "Dual_time_stepping: a wavefront wait ran out (code %d)", *err_host);
    return CF_OK;
}

int cf_Dual_time_stepping(cf_ctx *c, int, double deltaT, double *er1, double *er2, double *er3, double *er4,
                          double *er5, int *Nijk, int *ijk, double **p)
{
    return dts_common(c, deltaT, er1, er2, er3, er4, er5, Nijk, ijk, p, false);
}

int cf_DPLUSGS(cf_ctx *c, int, double deltaT, double *er1, double *er2, double *er3, double *er4, double *er5,
               double **p)
{
    if (!c || !p) return CF_ERR_ARG;
    cf_lu_args a{};
    if (int rc = lu_args(c, p, "DPLUSGS", a)) return rc;
    const cf_dims &d = c->d;
    const bool ex = exact(c);
    const int pr = ex ? 0 : kprec(c);
    cudaError_t e = ex ? cf_exact::lu_prepare(d, a, deltaT, false, 0, c->stream)
                       : cf_fast::lu_prepare(d, a, deltaT, false, pr, c->stream);
    if (int rc = cuda_check(c, e, "DPLUSGS")) return rc;
    for (int sweep = 1; sweep <= 4; sweep++) {
        e = ex ? cf_exact::lu_jacobi(d, a, deltaT, 0, c->stream) : cf_fast::lu_jacobi(d, a, deltaT, pr, c->stream);
        if (int rc = cuda_check(c, e, "DPLUSGS sweep")) return rc;
        e = cf_fast::lu_copy(d, a, c->stream);
        if (int rc = cuda_check(c, e, "DPLUSGS copy")) return rc;
    }
    double *er[5] = {er1, er2, er3, er4, er5};
    return lu_finish_host(c, a, er, "DPLUSGS");
}

// ---------------------------------------------------------------------------
// face metrics

static int jacobian_common(cf_ctx *c, double **p, int which, const char *who)
{
    if (!c || !p) return CF_ERR_ARG;
    const int n = which == 1 ? 20 : 10;
    for (int i = 0; i < n; i++)
        if (!p[i]) return fail(c, CF_ERR_ARG, "%s: array argument %d is NULL", who, i);
    cf_metric_args a;
    a.Jf = R(c, p[0]);
    for (int t = 0; t < 9; t++) a.m[t] = R(c, p[1 + t]);
    a.Jc = which == 1 ? R(c, p[10]) : nullptr;
    for (int t = 0; t < 9; t++) a.mc[t] = which == 1 ? R(c, p[11 + t]) : nullptr;
    return cuda_check(c, cf_fast::face_metrics(c->d, a, which, c->gamma, c->stream), who);
}

int cf_Jacobian_u(cf_ctx *c, int, double **p) { return jacobian_common(c, p, 0, "Jacobian_u"); }
int cf_Jacobian_v(cf_ctx *c, int, double **p) { return jacobian_common(c, p, 1, "Jacobian_v"); }
int cf_Jacobian_w(cf_ctx *c, int, double **p) { return jacobian_common(c, p, 2, "Jacobian_w"); }

// ---------------------------------------------------------------------------
// reductions and IO around the step (FP64 in every precision mode)

static std::string out_path(const cf_ctx *c, const char *name)
{
    return c->out_dir.empty() ? std::string(name) : c->out_dir + "/" + name;
}

int cf_set_output_dir(cf_ctx *c, const char *dir)
{
    if (!c) return CF_ERR_ARG;
    c->out_dir = dir ? dir : "";
    return CF_OK;
}

int cf_Driven_force(cf_ctx *c, int, double *U2_, double *J, double *Q, double *ER_Q)
{
    if (!c || !U2_ || !J) return CF_ERR_ARG;
    const cf_dims &d = c->d;
    double *rows = scratch(c, "bulk_rows", 1);            // Y_m row sums + Jsum, inside one field
    // (its own partials: cf_step's Statistic may still be running beside it)
    const size_t plen = (size_t)4 * 152 * 9 + (size_t)d.Ym * 64;
    double *partial = static_cast<double *>(scratch_bytes(c, "bulk_partial", plen * sizeof(double)));
    if (!rows || !partial) return fail(c, CF_ERR_NOMEM, "Driven_force: scratch allocation failed");
    double *jsum = rows + d.Ym;
    cudaError_t e = cf_fast::bulk_rows(d, R(c, U2_), R(c, J), jsum, rows, partial, plen, c->stream);
    if (int rc = cuda_check(c, e, "Driven_force")) return rc;
    std::vector<double> h((size_t)d.Ym);
    if (int rc = cuda_check(c, cudaMemcpyAsync(h.data(), rows, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                               c->stream), "Driven_force")) return rc;
    if (int rc = cuda_check(c, cudaStreamSynchronize(c->stream), "Driven_force")) return rc;
    double q = 0;
    for (int j = 2; j <= d.ny; j++) q += h[(size_t)j];
    q = q / d.X_out / d.Z_out;
    if (Q) *Q = q;
    if (ER_Q) *ER_Q = std::fabs(c->q0 - q) / c->q0;
    return CF_OK;
}

static int stat_alloc(cf_ctx *c)
{
    if (c->stat_acc) return CF_OK;
    const size_t n = (size_t)17 * c->d.Ym;
    if (cudaMalloc(&c->stat_acc, n * sizeof(double)) != cudaSuccess) {
        c->stat_acc = nullptr;
        return fail(c, CF_ERR_NOMEM, "Statistic: accumulator allocation failed");
    }
    // cleared on the context's stream: whatever reads the accumulators
    // next is ordered after it (cf_step's Statistic stream by its event)
    return cuda_check(c, cudaMemsetAsync(c->stat_acc, 0, n * sizeof(double), c->stream), "Statistic");
}

int cf_statistic_reset(cf_ctx *c)
{
    if (!c) return CF_ERR_ARG;
    if (int rc = cf_statistic_flush(c)) return rc;
    if (int rc = stat_alloc(c)) return rc;
    c->sxy_bottom = c->sxy_up = 0;
    return cuda_check(c, cudaMemsetAsync(c->stat_acc, 0, (size_t)17 * c->d.Ym * sizeof(double), c->stream),
                      "cf_statistic_reset");
}

int cf_statistic_read(cf_ctx *c, double *out)
{
    if (!c || !out) return CF_ERR_ARG;
    if (int rc = cf_statistic_flush(c)) return rc;
    if (int rc = stat_alloc(c)) return rc;
    const size_t n = (size_t)17 * c->d.Ym;
    if (int rc = cuda_check(c, cudaMemcpyAsync(out, c->stat_acc, n * sizeof(double), cudaMemcpyDeviceToHost,
                                               c->stream), "cf_statistic_read")) return rc;
    if (int rc = cuda_check(c, cudaStreamSynchronize(c->stream), "cf_statistic_read")) return rc;
    out[n] = c->sxy_bottom;
    out[n + 1] = c->sxy_up;
    return CF_OK;
}

namespace {

// The Statistic's kernels (row sums added to the accumulators) on stream s
static int stat_launch(cf_ctx *c, double **p, cudaStream_t s)
{
    if (int rc = stat_alloc(c)) return rc;
    const cf_dims &d = c->d;
    cf_stat_args a;
    for (int n = 0; n < 5; n++) a.U[n] = R(c, p[n]);
    a.J = R(c, p[5]);
    a.Jv = R(c, p[6]);
    for (int n = 0; n < 9; n++) a.m[n] = R(c, p[7 + n]);
    // row partials: up to Y_m rows x (X_out/4 + 1) chunks x 9 sums
    const size_t plen = (size_t)d.Ym * (size_t)(d.X_out / 4 + 1) * 9;
    double *partial = static_cast<double *>(scratch_bytes(c, "stat_partial", plen * sizeof(double)));
    if (!partial) return fail(c, CF_ERR_NOMEM, "Statistic: scratch allocation failed");
    cudaError_t e = exact(c) ? cf_exact::statistic(d, a, c->stat_acc, partial, plen, s)
                             : cf_fast::statistic(d, a, c->stat_acc, partial, plen, s);
    return cuda_check(c, e, "Statistic");
}

// The Statistic's host part after its kernels on stream s (Statistic.cpp:
// 900-1068): the accumulators to the host, the wall shear increments to
// Shear_stress.dat and, when step % statistic_step == 0, ND%05d.dat,
// st%05d.dat and cleared accumulators
static int stat_host(cf_ctx *c, int step, int statistic_step, cudaStream_t s)
{
    const cf_dims &d = c->d;
    const int Ym = d.Ym, ny = d.ny;
    std::vector<double> h((size_t)17 * Ym);
    if (int rc = cuda_check(c, cudaMemcpyAsync(h.data(), c->stat_acc, h.size() * sizeof(double),
                                               cudaMemcpyDeviceToHost, s), "Statistic")) return rc;
    if (int rc = cuda_check(c, cudaStreamSynchronize(s), "Statistic")) return rc;
    const double XZ = (double)d.X_out, ZZ = (double)d.Z_out;
    // wall shear-stress increments (Statistic.cpp:900-920)
    const double s1 = h[(size_t)7 * Ym + 1] / XZ / ZZ, sn = h[(size_t)7 * Ym + ny] / XZ / ZZ;
    {
        FILE *f = std::fopen(out_path(c, "Shear_stress.dat").c_str(), "a");
        if (!f) return fail(c, CF_ERR_ARG, "Statistic: cannot open Shear_stress.dat in '%s'", c->out_dir.c_str());
        std::fprintf(f, "%f\t%f\n", s1 - c->sxy_bottom, sn - c->sxy_up);
        std::fclose(f);
    }
    c->sxy_bottom = s1;
    c->sxy_up = sn;
    if (step % statistic_step == 0) {
        const double inv = 1. / statistic_step / XZ / ZZ;
        char name[64];
        std::snprintf(name, sizeof name, "ND%05d.dat", step);
        FILE *f = std::fopen(out_path(c, name).c_str(), "w");
        if (!f) return fail(c, CF_ERR_ARG, "Statistic: cannot write %s", name);
        for (int r = 0; r < 10; r++)
            for (int j = 1; j <= ny; j++) std::fprintf(f, "%.16f\n", h[(size_t)r * Ym + j] * inv);
        std::fclose(f);
        std::snprintf(name, sizeof name, "st%05d.dat", step);
        f = std::fopen(out_path(c, name).c_str(), "w");
        if (!f) return fail(c, CF_ERR_ARG, "Statistic: cannot write %s", name);
        for (int r = 10; r < 17; r++)
            for (int j = 2; j <= ny; j++) std::fprintf(f, "%.16f\n", h[(size_t)r * Ym + j] * inv);
        std::fclose(f);
        c->sxy_bottom = c->sxy_up = 0;
        if (int rc = cuda_check(c, cudaMemsetAsync(c->stat_acc, 0, h.size() * sizeof(double), s), "Statistic"))
            return rc;
        if (int rc = cuda_check(c, cudaStreamSynchronize(s), "Statistic")) return rc;
    }
    return CF_OK;
}

}  // namespace

// completes the pending Statistic of the last cf_step (its host part)
int cf_statistic_flush(cf_ctx *c)
{
    if (!c) return CF_ERR_ARG;
    if (!c->stat_pending) return CF_OK;
    c->stat_pending = false;
    return stat_host(c, c->stat_step, c->stat_every, c->stat_stream);
}

namespace {

// cf_step's Statistic of the final U_: the pending one completed, U_ copied
// (ghosts included) on the step's stream, the kernels on the Statistic's
// stream after that copy; the host part waits for the next flush
static int stat_overlapped(cf_ctx *c, int step, int statistic_step, double **st)
{
    if (int rc = cf_statistic_flush(c)) return rc;
    if (!c->stat_stream) {
        // the least priority: a caller that runs its steps on a stream of
        // higher priority keeps the block scheduler's preference
        int least = 0, greatest = 0;
        if (int rc = cuda_check(c, cudaDeviceGetStreamPriorityRange(&least, &greatest), "cf_step stream")) return rc;
        if (int rc = cuda_check(c, cudaStreamCreateWithPriority(&c->stat_stream, cudaStreamNonBlocking, least),
                                "cf_step stream")) return rc;
        if (int rc = cuda_check(c, cudaEventCreateWithFlags(&c->ev_stat, cudaEventDisableTiming), "cf_step event"))
            return rc;
    }
    if (int rc = stat_alloc(c)) return rc;                 // before the event the kernels wait on
    const size_t n = c->d.total();
    double *snap = scratch(c, "stat_state", 5);
    if (!snap) return fail(c, CF_ERR_NOMEM, "cf_step: Statistic state copy allocation failed");
    double *p[16];
    for (int v = 0; v < 5; v++) {
        if (int rc = cuda_check(c, cudaMemcpyAsync(snap + v * n, R(c, st[v]), n * sizeof(double),
                                                   cudaMemcpyDeviceToDevice, c->stream), "cf_step")) return rc;
        p[v] = snap + v * n;
    }
    for (int v = 5; v < 16; v++) p[v] = st[v];
    if (int rc = cuda_check(c, cudaEventRecord(c->ev_stat, c->stream), "cf_step")) return rc;
    if (int rc = cuda_check(c, cudaStreamWaitEvent(c->stat_stream, c->ev_stat, 0), "cf_step")) return rc;
    if (int rc = stat_launch(c, p, c->stat_stream)) return rc;
    c->stat_pending = true;
    c->stat_step = step;
    c->stat_every = statistic_step;
    return CF_OK;
}

}  // namespace

int cf_Statistic(cf_ctx *c, int, int step, int, int statistic_step, double **p)
{
    if (!c || !p) return CF_ERR_ARG;
    if (statistic_step <= 0) return fail(c, CF_ERR_ARG, "Statistic: statistic_step must be positive");
    for (int i = 0; i < 16; i++)
        if (!p[i]) return fail(c, CF_ERR_ARG, "Statistic: array argument %d is NULL", i);
    if (int rc = cf_statistic_flush(c)) return rc;
    if (int rc = stat_launch(c, p, c->stream)) return rc;
    return stat_host(c, step, statistic_step, c->stream);
}

static int restart_args(cf_ctx *c, double *const *U, double *const *Uq, const double *J, cf_ptr5 &u, cf_ptr5 &uq,
                        const char *who)
{
    for (int n = 0; n < 5; n++) {
        if (!U[n] || !Uq[n]) return fail(c, CF_ERR_ARG, "%s: NULL array", who);
        u.p[n] = R(c, U[n]);
        uq.p[n] = R(c, Uq[n]);
    }
    if (!J) return fail(c, CF_ERR_ARG, "%s: NULL J", who);
    return CF_OK;
}

int cf_Output(cf_ctx *c, int step, int, double *U1, double *U2, double *U3, double *U4, double *U5, double *U1q,
              double *U2q, double *U3q, double *U4q, double *U5q, double *J)
{
    if (!c) return CF_ERR_ARG;
    double *U[5] = {U1, U2, U3, U4, U5}, *Uq[5] = {U1q, U2q, U3q, U4q, U5q};
    cf_ptr5 u, uq;
    if (int rc = restart_args(c, U, Uq, J, u, uq, "Output")) return rc;
    const cf_dims &d = c->d;
    const size_t N = (size_t)d.X_out * d.Y_out * d.Z_out;
    double *img = static_cast<double *>(scratch_bytes(c, "restart", 10 * N * sizeof(double)));
    if (!img) return fail(c, CF_ERR_NOMEM, "Output: scratch allocation failed");
    if (int rc = cuda_check(c, cf_fast::restart_pack(d, u, uq, R(c, J), img, c->stream), "Output")) return rc;
    std::vector<double> h(10 * N);
    if (int rc = cuda_check(c, cudaMemcpyAsync(h.data(), img, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                               c->stream), "Output")) return rc;
    if (int rc = cuda_check(c, cudaStreamSynchronize(c->stream), "Output")) return rc;
    char name[64];
    std::snprintf(name, sizeof name, "LES%05d.bin", step);
    FILE *f = std::fopen(out_path(c, name).c_str(), "wb");
    if (!f) return fail(c, CF_ERR_ARG, "Output: cannot write %s", name);
    const size_t w = std::fwrite(h.data(), sizeof(double), h.size(), f);
    std::fclose(f);
    return w == h.size() ? CF_OK : fail(c, CF_ERR_ARG, "Output: short write of %s", name);
}

int cf_Initial_condition(cf_ctx *c, int, double *, double *, double *, double *, double *, double *U1, double *U2,
                         double *U3, double *U4, double *U5, double *U1q, double *U2q, double *U3q, double *U4q,
                         double *U5q, double *J)
{
    if (!c) return CF_ERR_ARG;
    double *U[5] = {U1, U2, U3, U4, U5}, *Uq[5] = {U1q, U2q, U3q, U4q, U5q};
    cf_ptr5 u, uq;
    if (int rc = restart_args(c, U, Uq, J, u, uq, "Initial_condition")) return rc;
    const cf_dims &d = c->d;
    const size_t N = (size_t)d.X_out * d.Y_out * d.Z_out;
    std::vector<double> h(10 * N);
    FILE *f = std::fopen(out_path(c, "initial.bin").c_str(), "rb");
    if (!f) return fail(c, CF_ERR_ARG, "Initial_condition: cannot open initial.bin in '%s'", c->out_dir.c_str());
    const size_t r = std::fread(h.data(), sizeof(double), h.size(), f);
    std::fclose(f);
    if (r != h.size()) return fail(c, CF_ERR_ARG, "Initial_condition: initial.bin holds %zu of %zu values", r, h.size());
    double *img = static_cast<double *>(scratch_bytes(c, "restart", 10 * N * sizeof(double)));
    if (!img) return fail(c, CF_ERR_NOMEM, "Initial_condition: scratch allocation failed");
    if (int rc = cuda_check(c, cudaMemcpyAsync(img, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice,
                                               c->stream), "Initial_condition")) return rc;
    if (int rc = cuda_check(c, cf_fast::restart_unpack(d, img, u, uq, R(c, J), c->stream), "Initial_condition"))
        return rc;
    return cuda_check(c, cudaStreamSynchronize(c->stream), "Initial_condition");
}

// ---------------------------------------------------------------------------
// physical time step driver (main.cpp:143-480)

int cf_step_reset(cf_ctx *c)
{
    if (!c) return CF_ERR_ARG;
    for (double &e : c->E) e = 0;
    if (!c->met32.empty()) {
        cudaStreamSynchronize(c->stream);
        for (auto &m : c->met32) cudaFree(m.second);
        c->met32.clear();
    }
    c->shadow_j = nullptr;
    return CF_OK;
}

int cf_step_scale(cf_ctx *c, double *E, int set)
{
    if (!c || !E) return CF_ERR_ARG;
    for (int n = 0; n < 5; n++) {
        if (set) {
            if (!(E[n] >= 0)) return fail(c, CF_ERR_ARG, "cf_step_scale: E[%d] must be >= 0", n);
            c->E[n] = E[n];
        } else {
            E[n] = c->E[n];
        }
    }
    return CF_OK;
}

int cf_step_residuals(cf_ctx *c, double *out, int cap, int *count)
{
    if (!c || !count || (cap > 0 && !out)) return CF_ERR_ARG;
    const int n = (int)(c->er_hist.size() / 5);
    *count = n;
    const int m = std::min(n, std::max(cap, 0));
    for (int t = 0; t < 5 * m; t++) out[t] = c->er_hist[t];
    return CF_OK;
}

int cf_step(cf_ctx *c, const cf_step_params *pp, int step, const cf_fields *f, int *iterations, double *er_out,
            double *Q)
{
    if (!c || !pp || !f) return CF_ERR_ARG;
    if (pp->max_iterations < 1) return fail(c, CF_ERR_ARG, "cf_step: max_iterations must be >= 1");
    double *const *U_ = f->U_;
    double *visc[79] = {nullptr};
    for (int n = 0; n < 5; n++) visc[n] = U_[n];
    for (int n = 0; n < 4; n++) visc[5 + n] = f->vF[n];
    visc[9] = f->J;
    for (int n = 0; n < 9; n++) visc[10 + n] = f->cell_metric[n];
    for (int s = 0; s < 3; s++) {
        visc[19 + 10 * s] = f->face_J[s];
        for (int n = 0; n < 9; n++) visc[20 + 10 * s + n] = f->face_metric[s][n];
    }
    for (int n = 0; n < 4; n++) {
        visc[55 + n] = f->LL[n];
        visc[65 + n] = f->ML[n];
        visc[75 + n] = f->NL[1 + n];
    }
    double *dts[64];
    for (int n = 0; n < 5; n++) {
        dts[n] = U_[n];
        dts[5 + n] = f->U[n];
        dts[10 + n] = f->Uq[n];
        dts[25 + n] = f->inF[0][n];
        dts[30 + n] = f->inF[1][n];
        dts[35 + n] = f->inF[2][n];
        dts[44 + n] = f->MR[n];
        dts[49 + n] = f->NR[n];
        dts[54 + n] = f->NL[n];
        dts[59 + n] = f->Residual[n];
    }
    dts[15] = f->J;
    for (int n = 0; n < 9; n++) dts[16 + n] = f->cell_metric[n];
    for (int n = 0; n < 4; n++) dts[40 + n] = f->vF[n];
    double er[5] = {0, 0, 0, 0, 0};
    // FP32: the fluxes, viscous terms and Dual_time_stepping of the loop
    // pass the right-hand-side arrays as FP32 values (the caller's inF, vF,
    // LL/ML/NL are the loop's own scratch here)
    const bool f32_rhs = kprec(c) == 1;
    // fixed metric arrays: their FP32 copies are made once and kept
    const bool static_m = f32_rhs && pp->static_metrics != 0;
    c->er_hist.clear();
    if (!c->side) {
        if (int rc = cuda_check(c, cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking), "cf_step stream"))
            return rc;
        if (int rc = cuda_check(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "cf_step event"))
            return rc;
        if (int rc = cuda_check(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "cf_step event"))
            return rc;
    }
    if (static_m) {
        // every FP32 metric copy the loop reads, made here on the main
        // stream: Flux_Y and Flux_Z run on the side stream and the viscous
        // terms on the main one, and both read the y- and z-face copies, so
        // a copy made by whichever comes first would be read unordered by
        // the other
        for (int s = 0; s < 3; s++) {
            if (!met32_get(c, R(c, f->face_J[s])))
                return fail(c, CF_ERR_NOMEM, "cf_step: FP32 metric copy allocation failed");
            for (int n = 0; n < 9; n++)
                if (!met32_get(c, R(c, f->face_metric[s][n])))
                    return fail(c, CF_ERR_NOMEM, "cf_step: FP32 metric copy allocation failed");
        }
        for (int n = 0; n < 9; n++)
            if (!met32_get(c, R(c, f->cell_metric[n])))
                return fail(c, CF_ERR_NOMEM, "cf_step: FP32 metric copy allocation failed");
    }
    if (f32_rhs) {
        // U - Uq is fixed over the step: its FP32 value once, for the BDF2 term
        float *dq = reinterpret_cast<float *>(scratch(c, "step_duq", 3));
        if (!dq) return fail(c, CF_ERR_NOMEM, "cf_step: scratch allocation failed");
        cf_ptr5 u, uq;
        for (int n = 0; n < 5; n++) {
            u.p[n] = R(c, f->U[n]);
            uq.p[n] = R(c, f->Uq[n]);
        }
        if (int rc = cuda_check(c, cf_fast::diff_f32(c->d.total(), u, uq, dq, c->stream), "cf_step")) return rc;
    }
    int it = 1;
    for (;; it++) {
        if (int rc = cf_X_periodic(c, 0, U_[0], U_[1], U_[2], U_[3], U_[4])) return rc;
        if (int rc = cf_Y_boundary_condition(c, 0, U_[0], U_[1], U_[2], U_[3], U_[4], f->J)) return rc;
        if (int rc = cf_Z_boundary_condition(c, 0, U_[0], U_[1], U_[2], U_[3], U_[4], f->J)) return rc;
        if (pp->filter == 1 || (pp->filter == 2 && it == 1))
            if (int rc = cf_Filter(c, 0, pp->roe_criterion, pp->e_high, pp->e_low, U_[0], U_[1], U_[2], U_[3],
                                   U_[4], f->Y_point, f->Ep[0], f->Ep[1], f->Ep[2], f->J)) return rc;
        // Flux_X on the stream (in FP32 it makes the copies of U and J the
        // others read), then Flux_Y and Flux_Z on a side stream while the
        // viscous terms run: independent kernels that are each bound by
        // latency fill the GPU together
        const cudaStream_t main = c->stream;
        for (int dir = 0; dir < 3; dir++) {
            double *p32[32] = {nullptr};
            for (int n = 0; n < 5; n++) {
                p32[n] = U_[n];
                p32[26 + n] = f->inF[dir][n];
            }
            p32[15] = f->J;
            p32[16] = f->face_J[dir];
            for (int n = 0; n < 9; n++) p32[17 + n] = f->face_metric[dir][n];
            p32[31] = f->Ep[dir];
            static const char *names[2][3] = {{"Flux_X", "Flux_Y", "Flux_Z"},
                                              {"Flux_X_limiter", "Flux_Y_limiter", "Flux_Z_limiter"}};
            if (dir == 1) {
                if (int rc = cuda_check(c, cudaEventRecord(c->ev_fork, main), "cf_step")) return rc;
                if (int rc = cuda_check(c, cudaStreamWaitEvent(c->side, c->ev_fork, 0), "cf_step")) return rc;
                c->stream = c->side;
            }
            const int rc = flux_common(c, names[pp->limiter ? 1 : 0][dir], dir, pp->limiter != 0, p32, dir > 0,
                                       f32_rhs, static_m);
            if (rc) {
                c->stream = main;
                return rc;
            }
        }
        c->stream = main;
        if (int rc = cuda_check(c, cudaEventRecord(c->ev_join, c->side), "cf_step")) return rc;
        if (int rc = viscous_common(c, visc, f32_rhs, static_m, f32_rhs)) return rc;
        if (int rc = cuda_check(c, cudaStreamWaitEvent(main, c->ev_join, 0), "cf_step")) return rc;
        if (int rc = dts_common(c, pp->deltaT, &er[0], &er[1], &er[2], &er[3], &er[4], nullptr, nullptr, dts,
                                f32_rhs, static_m, f32_rhs)) return rc;
        for (int n = 0; n < 5; n++)
            if (!std::isfinite(er[n]))
                return fail(c, CF_ERR_NONFINITE, "cf_step: residual norm er%d is not finite at iteration %d", n + 1,
                            it);
        for (int n = 0; n < 5; n++) {
            c->E[n] = std::max(c->E[n], er[n]);
            er[n] = er[n] / c->E[n];
            c->er_hist.push_back(er[n]);
        }
        const double tol = pp->tolerance;
        if ((er[0] < tol && er[1] < tol && er[2] < tol && er[3] < tol) || it >= pp->max_iterations) break;
    }
    if (int rc = cf_Driven_force(c, 0, f->U[1], f->J, Q, nullptr)) return rc;
    if (pp->statistic_step > 0) {
        double *st[27] = {nullptr};
        for (int n = 0; n < 5; n++) st[n] = U_[n];
        st[5] = f->J;
        st[6] = f->face_J[1];
        for (int n = 0; n < 9; n++) st[7 + n] = f->face_metric[1][n];
        st[26] = f->Ep[1];
        if (int rc = stat_overlapped(c, step, pp->statistic_step, st)) return rc;
    }
    cf_ptr5 u_, u, uq;
    for (int n = 0; n < 5; n++) {
        u_.p[n] = R(c, U_[n]);
        u.p[n] = R(c, f->U[n]);
        uq.p[n] = R(c, f->Uq[n]);
    }
    if (int rc = cuda_check(c, cf_fast::advance_levels(c->d, u_, u, uq, c->stream), "cf_step")) return rc;
    if (iterations) *iterations = it;
    if (er_out)
        for (int n = 0; n < 5; n++) er_out[n] = er[n];
    return CF_OK;
}

}  // extern "C"
