// One build variant of the hot-path kernels (see cf_launch.h).  The build
// compiles this file twice, with -DCF_NS=cf_exact --fmad=false and with
// -DCF_NS=cf_fast -DCF_WITH_FLOAT.
#include <algorithm>

#include "cf_flux.cuh"
#include "cf_bc.cuh"
#include "cf_visc.cuh"
#include "cf_filter.cuh"
#include "cf_lusgs.cuh"
#include "cf_wave.cuh"
#include "cf_pencil.cuh"
#include "cf_stats.cuh"
#include "cf_launch.h"

#ifdef CF_WITH_FLOAT
#define CF_DISPATCH(prec, call_double, call_float) ((prec) == 1 ? (call_float) : (call_double))
#else
#define CF_DISPATCH(prec, call_double, call_float) ((prec) == 1 ? cudaErrorNotSupported : (call_double))
#endif

namespace CF_NS {

cudaError_t x_periodic(const cf_dims &d, const cf_ptr5 &U, cudaStream_t s)
{
    const size_t n = d.plane() * 6;
    k_x_periodic<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, U);
    return cudaGetLastError();
}

cudaError_t y_wall(const cf_dims &d, const cf_ptr5 &U, const double *J, cudaStream_t s)
{
    // Y_boundary_condition.cpp:41-50: i = 2..gend+1, k = 2..nz, both walls
    cf_box b = make_box(2, d.gend + 1, 0, 1, 2, d.nz);
    k_y_wall<double><<<box_grid(b), box_block(), 0, s>>>(d, U, J, b);
    return cudaGetLastError();
}

cudaError_t z_periodic(const cf_dims &d, const cf_ptr5 &U, cudaStream_t s)
{
    // Z_boundary_condition.cpp:162-188: i = 2..gend+1, j = 0..nyyy
    cf_box b = make_box(2, d.gend + 1, 0, d.ny + 2, 0, 0);
    dim3 g((unsigned)((b.nj + 127) / 128), (unsigned)b.ni);
    k_z_periodic<<<g, 128, 0, s>>>(d, U, b);
    return cudaGetLastError();
}

// FP64 fluxes; the FP32 ones go through flux_f32 (they need the FP32 copies)
cudaError_t flux(const cf_dims &d, const cf_flux_args &a, int dir, bool limited, int prec, cudaStream_t s)
{
    return prec == 1 ? cudaErrorNotSupported : launch_flux<double>(d, a, dir, limited, s);
}

// shadow: 7 FP32 fields (U1..U5, J, 1/J) of d.total() values each; met32:
// FP32 copies of J_f and the 9 face metrics, or null
cudaError_t flux_f32(const cf_dims &d, const cf_flux_args &a, float *shadow, bool convert, const float *const *met32,
                     int dir, bool limited, cudaStream_t s)
{
#ifdef CF_WITH_FLOAT
    return launch_flux_f32(d, a, shadow, convert, met32, dir, limited, s);
#else
    (void)d; (void)a; (void)shadow; (void)convert; (void)met32; (void)dir; (void)limited; (void)s;
    return cudaErrorNotSupported;
#endif
}

__global__ void k_to_f32(size_t n, const double *__restrict__ src, float *__restrict__ dst)
{
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) dst[q] = float(src[q]);
}

// dst[0..n) = src rounded to FP32
cudaError_t to_f32(size_t n, const double *src, float *dst, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, src, dst);
    return cudaGetLastError();
}

__global__ void k_diff_f32(size_t n, cf_ptr5 a, cf_ptr5 b, float *__restrict__ dst)
{
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
#pragma unroll
    for (int v = 0; v < 5; v++) dst[v * n + q] = float(a.p[v][q] - b.p[v][q]);
}

// dst[v * n + q] = float(a[v][q] - b[v][q]), five fields of n values
cudaError_t diff_f32(size_t n, const cf_ptr5 &a, const cf_ptr5 &b, float *dst, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_diff_f32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, a, b, dst);
    return cudaGetLastError();
}

cudaError_t viscous(const cf_dims &d, const cf_visc_args &a, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, launch_viscous<double>(d, a, s), launch_viscous<float>(d, a, s));
}

cudaError_t filter(const cf_dims &d, const cf_filter_args &a, double crit, double hi, double lo, int prec,
                   cudaStream_t s)
{
#ifdef CF_FAST_MATH
    constexpr bool exact = false;
#else
    constexpr bool exact = true;
#endif
    return CF_DISPATCH(prec, (launch_filter<double, double, exact>(d, a, crit, hi, lo, s)),
                       (launch_filter<float, float, false>(d, a, crit, hi, lo, s)));
}

template <typename T>
static cudaError_t rk3_t(const cf_dims &d, const cf_rk3_args &a, int RK, double dt, cudaStream_t s)
{
    cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    k_rk3<T><<<box_grid(b), box_block(), 0, s>>>(d, a, b, RK, dt);
    return cudaGetLastError();
}
cudaError_t rk3(const cf_dims &d, const cf_rk3_args &a, int RK, double dt, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, rk3_t<double>(d, a, RK, dt, s), rk3_t<float>(d, a, RK, dt, s));
}

template <typename T>
static cudaError_t lu_prepare_t(const cf_dims &d, const cf_lu_args &a, double dt, bool copy_nr, cudaStream_t s)
{
    const size_t n = d.total();
    // the FP32 step driver's sweeps read N at no ghost cell (their ghost
    // terms take N = 0 as a constant): no zeroing
    if (!(sizeof(T) == 4 && cf_step_layout)) k_lu_zero<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, a, n);
    cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    k_lu_assemble<T><<<box_grid(b), box_block(), 0, s>>>(d, a, b, T(dt), copy_nr ? 1 : 0);
    return cudaGetLastError();
}
cudaError_t lu_prepare(const cf_dims &d, const cf_lu_args &a, double dt, bool copy_nr, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, lu_prepare_t<double>(d, a, dt, copy_nr, s), lu_prepare_t<float>(d, a, dt, copy_nr, s));
}

template <typename T>
static cudaError_t lu_plane_t(const cf_dims &d, const cf_lu_args &a, const int *ijk, int first, int count,
                              bool forward, double dt, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((count + 127) / 128);
    if (forward) k_lu_forward<T><<<blocks, 128, 0, s>>>(d, a, ijk, first, count, dt);
    else k_lu_backward<T><<<blocks, 128, 0, s>>>(d, a, ijk, first, count, dt);
    return cudaGetLastError();
}
cudaError_t lu_plane(const cf_dims &d, const cf_lu_args &a, const int *ijk, int first, int count, bool forward,
                     double dt, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, lu_plane_t<double>(d, a, ijk, first, count, forward, dt, s),
                       lu_plane_t<float>(d, a, ijk, first, count, forward, dt, s));
}

template <typename T>
static cudaError_t lu_pack_t(const cf_dims &d, const cf_lu_args &a, double *pack, double dt, cudaStream_t s)
{
    // every interior cell and its face-neighbour ghosts
    cf_box b = make_box(2, d.gend + 1, 1, d.ny + 1, 1, d.nz + 1);
    k_lu_pack<T><<<box_grid(b), box_block(), 0, s>>>(d, a, pack, b, dt);
    return cudaGetLastError();
}
cudaError_t lu_pack(const cf_dims &d, const cf_lu_args &a, double *pack, double dt, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, lu_pack_t<double>(d, a, pack, dt, s), lu_pack_t<float>(d, a, pack, dt, s));
}

template <typename T>
static cudaError_t lu_plane_packed_t(const cf_dims &d, const cf_lu_args &a, const double *pack, const int *ijk,
                                     int first, int count, bool forward, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((count + 127) / 128);
    if (forward) k_lu_forward_packed<T><<<blocks, 128, 0, s>>>(d, a, pack, ijk, first, count);
    else k_lu_backward_packed<T><<<blocks, 128, 0, s>>>(d, a, pack, ijk, first, count);
    return cudaGetLastError();
}
cudaError_t lu_plane_packed(const cf_dims &d, const cf_lu_args &a, const double *pack, const int *ijk, int first,
                            int count, bool forward, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, lu_plane_packed_t<double>(d, a, pack, ijk, first, count, forward, s),
                       lu_plane_packed_t<float>(d, a, pack, ijk, first, count, forward, s));
}

template <typename T>
static cudaError_t lu_wave_pack_t(const cf_dims &d, const cf_lu_args &a, const cf_wave_args &w, double dt,
                                  bool upper, bool assemble, cudaStream_t s)
{
    if (upper) {
        cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
        k_lu_tile_ghost_upper<T><<<box_grid(b), box_block(), 0, s>>>(a, w, b);
        return cudaGetLastError();
    }
    void (*kf)(cf_lu_args, wave_args, T) = assemble ? k_lu_tile_pack<T, true> : k_lu_tile_pack<T, false>;
    kf<<<w.ntiles, WV_CELLS, 0, s>>>(a, w, T(dt));
    return cudaGetLastError();
}
// assemble: the forward pack also assembles MR (no lu_prepare assembly pass)
cudaError_t lu_wave_pack(const cf_dims &d, const cf_lu_args &a, const cf_wave_args &w, double dt, bool upper,
                         bool assemble, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, lu_wave_pack_t<double>(d, a, w, dt, upper, assemble, s),
                       lu_wave_pack_t<float>(d, a, w, dt, upper, assemble, s));
}

template <typename T>
static cudaError_t lu_pencil_pack_t(const cf_dims &d, const cf_lu_args &a, const cf_wave_args &w, double dt,
                                    bool upper, bool assemble, cudaStream_t s)
{
    if (upper) {
        cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
        k_lu_pencil_ghost_upper<T><<<box_grid(b), box_block(), 0, s>>>(a, w, b);
        return cudaGetLastError();
    }
    k_lu_wave_epoch<<<1, 1, 0, s>>>(w, w.npencils);
    const size_t smem = (size_t)WV_PACK * 256 * sizeof(T);
    void (*kf)(cf_lu_args, wave_args, T) = assemble ? k_lu_pencil_pack<T, true> : k_lu_pencil_pack<T, false>;
    cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)w.npencils * (unsigned)((d.X_out + 7) / 8);
    kf<<<blocks, 256, smem, s>>>(a, w, T(dt));
    return cudaGetLastError();
}
// pencil packs (forward, with the assembly when asked) or the backward
// sweep's upper ghost terms
cudaError_t lu_pencil_pack(const cf_dims &d, const cf_lu_args &a, const cf_wave_args &w, double dt, bool upper,
                           bool assemble, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, lu_pencil_pack_t<double>(d, a, w, dt, upper, assemble, s),
                       lu_pencil_pack_t<float>(d, a, w, dt, upper, assemble, s));
}

template <typename T>
static cudaError_t lu_pencil_sweep_t(const cf_lu_args &a, const cf_wave_args &w, bool fwd, cudaStream_t s)
{
    const size_t smem = pc_smem_bytes<T>(fwd);
    void (*kf)(cf_lu_args, wave_args) = fwd ? k_lu_pencil<T, true> : k_lu_pencil<T, false>;
    cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, occ = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    constexpr int warps = pc_geom<T>::WARPS;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kf, 32 * warps, smem)) != cudaSuccess) return e;
    const int blocks = std::min((w.npencils + warps - 1) / warps, std::max(1, occ) * sms);
    kf<<<blocks, 32 * warps, smem, s>>>(a, w);
    return cudaGetLastError();
}
cudaError_t lu_pencil_sweep(const cf_lu_args &a, const cf_wave_args &w, bool fwd, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, lu_pencil_sweep_t<double>(a, w, fwd, s), lu_pencil_sweep_t<float>(a, w, fwd, s));
}

// the zeroing of lu_prepare alone (NL, NR of every index, ghosts included)
cudaError_t lu_zero(const cf_dims &d, const cf_lu_args &a, cudaStream_t s)
{
    const size_t n = d.total();
    k_lu_zero<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, a, n);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t lu_wave_sweep_t(const cf_lu_args &a, const cf_wave_args &w, bool fwd, cudaStream_t s)
{
    const size_t smem = (size_t)WV_SM_TOTAL * sizeof(T);
    void (*kf)(cf_lu_args, wave_args) = fwd ? k_lu_wave<T, true> : k_lu_wave<T, false>;
    cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, occ = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const int threads = 32 * WV_WARPS;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kf, threads, smem)) != cudaSuccess) return e;
    const int blocks = std::min(w.ntiles, std::max(1, occ) * sms);
    kf<<<blocks, threads, smem, s>>>(a, w);
    return cudaGetLastError();
}
cudaError_t lu_wave_sweep(const cf_lu_args &a, const cf_wave_args &w, bool fwd, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, lu_wave_sweep_t<double>(a, w, fwd, s), lu_wave_sweep_t<float>(a, w, fwd, s));
}

template <typename T>
static cudaError_t lu_jacobi_t(const cf_dims &d, const cf_lu_args &a, double dt, cudaStream_t s)
{
    cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    k_lu_jacobi<T><<<box_grid(b), box_block(), 0, s>>>(d, a, b, dt);
    return cudaGetLastError();
}
cudaError_t lu_jacobi(const cf_dims &d, const cf_lu_args &a, double dt, int prec, cudaStream_t s)
{
    return CF_DISPATCH(prec, lu_jacobi_t<double>(d, a, dt, s), lu_jacobi_t<float>(d, a, dt, s));
}

cudaError_t lu_copy(const cf_dims &d, const cf_lu_args &a, cudaStream_t s)
{
    cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    k_lu_copy<<<box_grid(b), box_block(), 0, s>>>(d, a, b);
    return cudaGetLastError();
}

size_t lu_partial_count(const cf_dims &d)
{
    cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    dim3 g = box_grid(b);
    return (size_t)g.x * g.y * g.z;
}

cudaError_t lu_finish(const cf_dims &d, const cf_lu_args &a, double *er_dev, int prec, cudaStream_t s)
{
    cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    dim3 g = box_grid(b);
#ifdef CF_WITH_FLOAT
    if (prec == 1) {
        // FP32: four planes per thread (fewer partial sums to reduce)
        g.z = (unsigned)((b.ni + 3) / 4);
        k_lu_update<float><<<g, box_block(), 0, s>>>(d, a, b);
    } else
#endif
        k_lu_update<double><<<g, box_block(), 0, s>>>(d, a, b);
    const double DN = 1. / (d.X_out * d.Y_out * d.Z_out);
    k_lu_norm<<<1, 256, 0, s>>>(a.partial, (size_t)g.x * g.y * g.z, DN, er_dev);
    return cudaGetLastError();
}

template <int KIND>
static cudaError_t stat_kind(const cf_dims &d, const cf_stat_args &a, double *partial, size_t partial_len,
                             double *out, int Ym, st_qmap qm, int j0, int nrows, int accumulate,
                             const double *jsum, cudaStream_t s)
{
    constexpr int NQ = st_kind<KIND>::NQ;
    if (nrows <= 0) return cudaSuccess;
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 132;
    }
    // chunks of about four x planes (short blocks, which share the SMs
    // well with kernels of other streams), at least four blocks per SM
    int nchunk = std::max(1, std::min(d.X_out, std::max((4 * sms + nrows - 1) / nrows, (d.X_out + 3) / 4)));
    while ((size_t)nrows * nchunk * NQ > partial_len && nchunk > 1) nchunk--;
    if ((size_t)nrows * nchunk * NQ > partial_len) return cudaErrorInvalidValue;
    k_stat_rows<KIND><<<dim3((unsigned)nrows, (unsigned)nchunk), ST_THREADS, 0, s>>>(d, a, partial, nchunk, jsum);
    const int n = nrows * NQ;
    k_stat_finish<NQ><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(partial, nrows, nchunk, j0, out, Ym, qm, accumulate);
    return cudaGetLastError();
}

// Statistic's per-call accumulation into acc (17 rows of Ym): y-face Roe
// quantities (rows 0..6, 8, 9), wall-normal shear (row 7), cell moments
// (rows 10..16)
cudaError_t statistic(const cf_dims &d, const cf_stat_args &a, double *acc, double *partial, size_t partial_len,
                      cudaStream_t s)
{
    const int Ym = d.Ym;
    st_qmap qf{{0, 1, 2, 3, 4, 5, 6, 8, 9}}, qs{{7}}, qm{{10, 11, 12, 13, 14, 15, 16}};
    cudaError_t e = stat_kind<ST_FACE>(d, a, partial, partial_len, acc, Ym, qf, 1, d.ny, 1, nullptr, s);
    if (e == cudaSuccess) e = stat_kind<ST_SHEAR>(d, a, partial, partial_len, acc, Ym, qs, 1, d.ny, 1, nullptr, s);
    if (e == cudaSuccess)
        e = stat_kind<ST_MOMENT>(d, a, partial, partial_len, acc, Ym, qm, 2, d.ny - 1, 1, nullptr, s);
    return e;
}

// Driven_force's bulk-flow integral: rows[j] = row sums (j = 2..ny) into
// out (Ym doubles), jsum_dev receives Jsum
cudaError_t bulk_rows(const cf_dims &d, const double *U2, const double *J, double *jsum_dev, double *rows,
                      double *partial, size_t partial_len, cudaStream_t s)
{
    k_bulk_jsum<<<1, 256, 0, s>>>(d, J, jsum_dev);
    cf_stat_args a{};
    a.U[1] = U2;
    a.J = J;
    st_qmap q0{{0}};
    return stat_kind<ST_BULK>(d, a, partial, partial_len, rows, d.Ym, q0, 2, d.ny - 1, 0, jsum_dev, s);
}

cudaError_t restart_pack(const cf_dims &d, const cf_ptr5 &U, const cf_ptr5 &Uq, const double *J, double *img,
                         cudaStream_t s)
{
    const size_t N = (size_t)d.X_out * d.Y_out * d.Z_out;
    k_restart_pack<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(d, U, Uq, J, img);
    return cudaGetLastError();
}

cudaError_t restart_unpack(const cf_dims &d, const double *img, const cf_ptr5 &U, const cf_ptr5 &Uq,
                           const double *J, cudaStream_t s)
{
    const size_t N = (size_t)d.X_out * d.Y_out * d.Z_out;
    k_restart_unpack<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(d, img, U, Uq, J);
    return cudaGetLastError();
}

cudaError_t advance_levels(const cf_dims &d, const cf_ptr5 &U_, const cf_ptr5 &U, const cf_ptr5 &Uq,
                           cudaStream_t s)
{
    cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    k_advance_levels<<<box_grid(b), box_block(), 0, s>>>(d, U_, U, Uq, b);
    return cudaGetLastError();
}

cudaError_t face_metrics(const cf_dims &d, const cf_metric_args &a, int which, double gamma, cudaStream_t s)
{
    cf_box b;
    double joff;
    if (which == 0) { b = make_box(2, d.gend, 1, d.ny - 1, 1, d.nz - 1); joff = 0.5; }       // Jacobian_u
    else if (which == 1) { b = make_box(2, d.gend - 1, 1, d.ny, 1, d.nz - 1); joff = 1.0; }  // Jacobian_v
    else { b = make_box(2, d.gend - 1, 1, d.ny - 1, 1, d.nz); joff = 0.5; }                  // Jacobian_w
    k_face_metrics<<<box_grid(b), box_block(), 0, s>>>(d, a, b, gamma, joff);
    if (which == 1) {
        cf_box w = make_box(2, d.gend - 1, 0, 0, 1, d.nz - 1);
        dim3 g((unsigned)((w.nk + 127) / 128), (unsigned)w.ni);
        k_v_wall_rows<<<g, 128, 0, s>>>(d, a, w);
    }
    return cudaGetLastError();
}

}  // namespace CF_NS
