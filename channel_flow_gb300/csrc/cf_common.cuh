// Shared device-side definitions of the channel-flow hot path.
//
// Layout (the reference's single-rank layout, Array.h:7): every field is one
// double[X_out+6][Y_out+4][Z_out+4] array with z fastest.  Interior cells are
// i = 3..gend (gend = X_out+2), j = 2..ny (ny = Y_out+1), k = 2..nz
// (nz = Z_out+1).  Face arrays use the same extents with one index shifted
// by -1 (x faces inFx[i][j-1][k-1] between cells i and i+1, and so on).
#pragma once

#include "cf_types.h"

#ifndef CF_NS
#error "CF_NS (the build-variant namespace) must be defined by the including translation unit"
#endif



// The reference's min/max macros (Flux_X_limiter.cpp:13-14): plain
// comparisons, so NaN and signed zeros resolve as they do there.
template <typename T>
__device__ __forceinline__ T rmin(T a, T b) { return (a < b) ? a : b; }
template <typename T>
__device__ __forceinline__ T rmax(T a, T b) { return (a > b) ? a : b; }


// Arrays of the right-hand side that the step driver passes between its own
// FP32 kernels (face fluxes, viscous face fluxes and divergence) can hold
// FP32 values in their FP64 allocation (flag f32, warp-uniform): no FP64 ->
// FP32 conversion, which issues to GB300's slow FP64 pipe, on either side.
// In the FP64 kernels (T = double) the flag is ignored.
//
// The choice must not be a runtime branch in the kernels the step driver
// runs: the compiler turns such short branches into predicated code, and a
// predicated-off conversion still issues to the FP64 pipe (measured: 60-87 %
// FP64-pipe activity in FP32 kernels that convert nothing).  The build
// therefore compiles the kernels a third time with CF_STEP_LAYOUT (namespace
// cf_drv), where the FP32 intermediates and the FP32 copies of metrics, U_
// and J are known at compile time to be present; the step driver calls that
// variant when it has set all of them up.
#ifdef CF_STEP_LAYOUT
constexpr bool cf_step_layout = true;
#else
constexpr bool cf_step_layout = false;
#endif

template <typename T>
__device__ __forceinline__ void rhs_put(double *p, size_t q, T v, int f32)
{
    if (sizeof(T) == 4 && (cf_step_layout || f32)) reinterpret_cast<float *>(p)[q] = float(v);
    else p[q] = double(v);
}
template <typename T>
__device__ __forceinline__ T rhs_get(const double *p, size_t q, int f32)
{
    if (sizeof(T) == 4 && (cf_step_layout || f32)) return T(reinterpret_cast<const float *>(p)[q]);
    return T(p[q]);
}


// a metric value in the compute type: from its FP32 copy when the caller
// has one (the step driver's cache of the fixed metric arrays, FP32 build),
// else from the FP64 array
template <typename T>
__device__ __forceinline__ T met_ld(const double *p, const float *p32, size_t q)
{
    if (sizeof(T) == 4 && (cf_step_layout || p32)) return T(p32[q]);
    return T(p[q]);
}

// 1/d for the contracted builds.  FP64: the hardware's approximate
// reciprocal (about 20 correct bits) refined by two Newton-Raphson steps
// x <- x + x (1 - d x), each doubling the correct bits, so the result lies
// within about one unit in the last place of the rounded quotient, in fewer
// FP64-pipe operations than an IEEE-rounded division.  d = 0 gives NaN
// (callers guard ties), and so does a subnormal d (|d| < 2.2e-308, flushed
// to zero on input); a quotient below the normal range (|d| > 4.5e307)
// flushes to zero.  The solver's divisors (densities, Jacobians, metric
// norms, sound speeds) lie far inside these limits.  FP32: the approximate
// division of the FP32 build.
template <typename T>
__device__ __forceinline__ T frcp(T d);
template <>
__device__ __forceinline__ float frcp<float>(float d) { return 1.0f / d; }
template <>
__device__ __forceinline__ double frcp<double>(double d)
{
    double x;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(x) : "d"(d));
    double e = fma(-d, x, 1.0);
    x = fma(x, e, x);
    e = fma(-d, x, 1.0);
    return fma(x, e, x);
}

// float -> double on the integer pipe (the conversion instruction issues
// to GB300's slow FP64 pipe): exact for normal values and signed zeros,
// infinities and NaNs stay infinities and NaNs, FP32 subnormals (below
// 1.2e-38) become signed zeros
__device__ __forceinline__ double f2d(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u, ex = (u >> 23) & 0xffu, man = u & 0x7fffffu;
    const unsigned exd = ex == 0xffu ? 0x7ffu : ex + 896u;      // 1023 - 127
    const unsigned hi = ex == 0u ? sign : (sign | (exd << 20) | (man >> 3));
    const unsigned lo = ex == 0u ? 0u : (man << 29);
    return __hiloint2double((int)hi, (int)lo);
}

// a grid constant of cf_dims in the compute type T (its FP32 copy for float)
#define CF_DC(T, d, x) (sizeof(T) == 4 ? (T)((d).f_##x) : (T)((d).x))
// 1/x of a grid constant (dXI, dET, dZT, Pr): in the contracted FP64 build
// the host's correctly rounded value (the same bits a device division
// gives, without one per thread), else the division
#ifdef CF_FAST_MATH
#define CF_DINV(T, d, x, ix) (sizeof(T) == 8 ? (T)((d).ix) : T(1) / CF_DC(T, d, x))
#else
#define CF_DINV(T, d, x, ix) (T(1) / CF_DC(T, d, x))
#endif


#define CF_BOX_INDEX(b, i, j, k)                                    \
    const int k = (b).k0 + (int)(blockIdx.x * blockDim.x + threadIdx.x); \
    const int j = (b).j0 + (int)(blockIdx.y * blockDim.y + threadIdx.y); \
    const int i = (b).i0 + (int)blockIdx.z;                         \
    if (k >= (b).k0 + (b).nk || j >= (b).j0 + (b).nj) return
