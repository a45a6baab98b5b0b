// Host launchers of one build variant of the kernels.  cf_variant.cu is
// compiled three times: namespace cf_exact with --fmad=false (every FP64
// result equals the reference's bit for bit), namespace cf_fast with fused
// multiply-add (FP64 within 1e-12; also the FP32 instantiations), and
// namespace cf_drv, the cf_fast kernels with the step driver's FP32 array
// layout fixed at compile time (CF_STEP_LAYOUT, cf_common.cuh).
// prec: 0 = double, 1 = float arithmetic inside the kernel.
#pragma once
#include "cf_types.h"

constexpr int CF_LU_PACK = 52;   // doubles per cell of the sweep coefficient pack

#define CF_DECLARE_LAUNCHERS(NS)                                                                        \
    namespace NS {                                                                                      \
    cudaError_t x_periodic(const cf_dims &d, const cf_ptr5 &U, cudaStream_t s);                         \
    cudaError_t y_wall(const cf_dims &d, const cf_ptr5 &U, const double *J, cudaStream_t s);            \
    cudaError_t z_periodic(const cf_dims &d, const cf_ptr5 &U, cudaStream_t s);                         \
    cudaError_t flux(const cf_dims &d, const cf_flux_args &a, int dir, bool limited, int prec,          \
                     cudaStream_t s);                                                                   \
    cudaError_t flux_f32(const cf_dims &d, const cf_flux_args &a, float *shadow, bool convert,           \
                         const float *const *met32, int dir, bool limited, cudaStream_t s);             \
    cudaError_t to_f32(size_t n, const double *src, float *dst, cudaStream_t s);                        \
    cudaError_t diff_f32(size_t n, const cf_ptr5 &a, const cf_ptr5 &b, float *dst, cudaStream_t s);    \
    cudaError_t viscous(const cf_dims &d, const cf_visc_args &a, int prec, cudaStream_t s);            \
    cudaError_t filter(const cf_dims &d, const cf_filter_args &a, double crit, double hi, double lo,   \
                       int prec, cudaStream_t s);                                                       \
    cudaError_t rk3(const cf_dims &d, const cf_rk3_args &a, int RK, double dt, int prec,               \
                    cudaStream_t s);                                                                    \
    cudaError_t lu_prepare(const cf_dims &d, const cf_lu_args &a, double dt, bool copy_nr, int prec,   \
                           cudaStream_t s);                                                             \
    cudaError_t lu_plane(const cf_dims &d, const cf_lu_args &a, const int *ijk, int first, int count,  \
                         bool forward, double dt, int prec, cudaStream_t s);                            \
    cudaError_t lu_pack(const cf_dims &d, const cf_lu_args &a, double *pack, double dt, int prec,       \
                        cudaStream_t s);                                                                \
    cudaError_t lu_plane_packed(const cf_dims &d, const cf_lu_args &a, const double *pack, const int *ijk, \
                                int first, int count, bool forward, int prec, cudaStream_t s);          \
    cudaError_t lu_wave_pack(const cf_dims &d, const cf_lu_args &a, const cf_wave_args &w, double dt,  \
                             bool upper, bool assemble, int prec, cudaStream_t s);                      \
    cudaError_t lu_zero(const cf_dims &d, const cf_lu_args &a, cudaStream_t s);                         \
    cudaError_t lu_pencil_pack(const cf_dims &d, const cf_lu_args &a, const cf_wave_args &w, double dt, \
                               bool upper, bool assemble, int prec, cudaStream_t s);                    \
    cudaError_t lu_pencil_sweep(const cf_lu_args &a, const cf_wave_args &w, bool fwd, int prec,         \
                                cudaStream_t s);                                                        \
    cudaError_t lu_wave_sweep(const cf_lu_args &a, const cf_wave_args &w, bool fwd, int prec,           \
                              cudaStream_t s);                                                          \
    cudaError_t lu_jacobi(const cf_dims &d, const cf_lu_args &a, double dt, int prec, cudaStream_t s); \
    cudaError_t lu_copy(const cf_dims &d, const cf_lu_args &a, cudaStream_t s);                        \
    cudaError_t lu_finish(const cf_dims &d, const cf_lu_args &a, double *er_dev, int prec, cudaStream_t s);     \
    size_t lu_partial_count(const cf_dims &d);                                                          \
    cudaError_t statistic(const cf_dims &d, const cf_stat_args &a, double *acc, double *partial,         \
                          size_t partial_len, cudaStream_t s);                                          \
    cudaError_t bulk_rows(const cf_dims &d, const double *U2, const double *J, double *jsum_dev,        \
                          double *rows, double *partial, size_t partial_len, cudaStream_t s);           \
    cudaError_t restart_pack(const cf_dims &d, const cf_ptr5 &U, const cf_ptr5 &Uq, const double *J,   \
                             double *img, cudaStream_t s);                                              \
    cudaError_t restart_unpack(const cf_dims &d, const double *img, const cf_ptr5 &U, const cf_ptr5 &Uq, \
                               const double *J, cudaStream_t s);                                        \
    cudaError_t advance_levels(const cf_dims &d, const cf_ptr5 &U_, const cf_ptr5 &U, const cf_ptr5 &Uq, \
                               cudaStream_t s);                                                         \
    cudaError_t face_metrics(const cf_dims &d, const cf_metric_args &a, int which, double gamma,       \
                             cudaStream_t s);                                                           \
    }

CF_DECLARE_LAUNCHERS(cf_exact)
CF_DECLARE_LAUNCHERS(cf_fast)
CF_DECLARE_LAUNCHERS(cf_drv)
