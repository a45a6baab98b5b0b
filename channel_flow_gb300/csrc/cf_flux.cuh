// Inviscid face fluxes: limited MUSCL-5 + low-Mach preconditioned Roe
// (Flux_X/Y/Z_limiter.cpp) and linear MUSCL-5 + Roe (Flux_X/Y/Z.cpp).
//
// One thread per face.  The reference first writes every face's left and
// right states into ML/MR scratch arrays and then runs a face loop; each
// reconstructed state is used by exactly one face, so here the two states of
// a face are formed in registers by the thread that evaluates the face, with
// the same branch the reference's reconstruction loop takes for that state
// (3rd order near the x seam and the walls, boundary averages, ...).  The
// arithmetic follows the reference's expression trees, so the --fmad=false
// build reproduces it bit for bit.
#pragma once
#include "cf_common.cuh"


namespace CF_NS {

// face metrics and face Jacobian of a flux kernel's arguments
template <typename T>
__device__ __forceinline__ T fmet(const cf_flux_args &a, int n, size_t q) { return T(a.m[n][q]); }
template <typename T>
__device__ __forceinline__ T fmet(const cf_flux_args_f &a, int n, size_t q) { return met_ld<T>(a.m[n], a.m32[n], q); }
template <typename T>
__device__ __forceinline__ T fjf(const cf_flux_args &a, size_t q) { return T(a.Jf[q]); }
template <typename T>
__device__ __forceinline__ T fjf(const cf_flux_args_f &a, size_t q) { return met_ld<T>(a.Jf, a.Jf32, q); }


// ---------------------------------------------------------------------------
// limiter pieces (Flux_X_limiter.cpp:149-159, 247-262)
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T lim3(T r)
{
    T b = T(1.) / T(3) * (T(1) + T(2) * r);
    return rmin(T(2), rmin(T(2) * r, b));
}
template <typename T>
__device__ __forceinline__ T lim5(T a, T r, T c)
{
    T b = T(1.) / T(30) * (T(-2.) / a + T(11) + T(24) * r - T(3) * r * c);
    return rmin(T(2), rmin(T(2) * r, b));
}
// left state of a cell, 3rd / 5th order, slope sign s (+ in x, y; - in z)
template <typename T, int S>
__device__ __forceinline__ T left3(T iu, T u, T ui)
{
    T rL = (ui - u) / (u - iu);
    T m = lim3(rL);
    return S > 0 ? (u + T(0.5) * rmax(T(0), m) * (u - iu)) : (u - T(0.5) * rmax(T(0), m) * (u - iu));
}
template <typename T>
__device__ __forceinline__ T right3(T iu, T u, T ui)
{
    T rR = (u - iu) / (ui - u);
    T m = lim3(rR);
    return u - T(0.5) * rmax(T(0), m) * (ui - u);
}
template <typename T, int S>
__device__ __forceinline__ T left5(T iiu, T iu, T u, T ui, T uii)
{
    T irL = (u - iu) / (iu - iiu);
    T rL = (ui - u) / (u - iu);
    T rLi = (uii - ui) / (ui - u);
    T m = lim5(irL, rL, rLi);
    return S > 0 ? (u + T(0.5) * rmax(T(0), m) * (u - iu)) : (u - T(0.5) * rmax(T(0), m) * (u - iu));
}
template <typename T>
__device__ __forceinline__ T right5(T iiu, T iu, T u, T ui, T uii)
{
    T rRi = (ui - u) / (uii - ui);
    T rR = (u - iu) / (ui - u);
    T irR = (iu - iiu) / (u - iu);
    T m = lim5(rRi, rR, irR);
    return u - T(0.5) * rmax(T(0), m) * (ui - u);
}

// linear states of the unlimited scheme (Flux_X.cpp:108-122, 138-162)
template <typename T, typename SP>
__device__ __forceinline__ T lin5L(const SP *U, const SP *J, size_t q, ptrdiff_t s)
{
    T temp = T(1.) / (T(2) / T(J[q - 2 * s]) - T(13) / T(J[q - s]) + T(47) / T(J[q]) + T(27) / T(J[q + s]) - T(3) / T(J[q + 2 * s]));
    return temp * (T(2) * T(U[q - 2 * s]) - T(13) * T(U[q - s]) + T(47) * T(U[q]) + T(27) * T(U[q + s]) - T(3) * T(U[q + 2 * s]));
}
template <typename T, typename SP>
__device__ __forceinline__ T lin5R(const SP *U, const SP *J, size_t q, ptrdiff_t s)
{
    T temp = T(1.) / (T(-3) / T(J[q - 2 * s]) + T(27) / T(J[q - s]) + T(47) / T(J[q]) - T(13) / T(J[q + s]) + T(2) / T(J[q + 2 * s]));
    return temp * (T(-3) * T(U[q - 2 * s]) + T(27) * T(U[q - s]) + T(47) * T(U[q]) - T(13) * T(U[q + s]) + T(2) * T(U[q + 2 * s]));
}
template <typename T, typename SP>
__device__ __forceinline__ T lin3L(const SP *U, const SP *J, size_t q, ptrdiff_t s)
{
    T temp = T(1.) / (T(-1) / T(J[q - s]) + T(5) / T(J[q]) + T(2) / T(J[q + s]));
    return temp * (-T(U[q - s]) + T(5) * T(U[q]) + T(2) * T(U[q + s]));
}
template <typename T, typename SP>
__device__ __forceinline__ T lin3R(const SP *U, const SP *J, size_t q, ptrdiff_t s)
{
    T temp = T(1.) / (T(2) / T(J[q - s]) + T(5) / T(J[q]) - T(1) / T(J[q + s]));
    return temp * (T(2) * T(U[q - s]) + T(5) * T(U[q]) - T(U[q + s]));
}
// two-cell average of cells q and q+s (Flux_X.cpp:138-144)
template <typename T, typename SP>
__device__ __forceinline__ T avg2(const SP *U, const SP *J, size_t q, ptrdiff_t s)
{
    T temp = T(1.) / (T(1) / T(J[q]) + T(1) / T(J[q + s]));
    return temp * (T(U[q]) + T(U[q + s]));
}
// same pair taken high cell first (Flux_Y.cpp:206-219)
template <typename T, typename SP>
__device__ __forceinline__ T avg2hi(const SP *U, const SP *J, size_t q, ptrdiff_t s)
{
    T temp = T(1.) / (T(1) / T(J[q]) + T(1) / T(J[q - s]));
    return temp * (T(U[q]) + T(U[q - s]));
}

// ---------------------------------------------------------------------------
// face states
// ---------------------------------------------------------------------------
// DIR 0/1/2 = x/y/z.  (i,j,k) is the face index; the left state belongs to
// cell cL and the right state to cell cR of the reference's reconstruction
// loops:  x: cL = (i, j+1, k+1), cR = (i+1, j+1, k+1);  y: cL = (i+1, j, k+1),
// cR = (i+1, j+1, k+1);  z: cL = (i+1, j+1, k), cR = (i+1, j+1, k+1).

// Flux_X_limiter.cpp:113-341: 3rd order where the cell index is <= 3 or >= gend
template <typename T, typename A>
__device__ __forceinline__ void states_x_limited(const cf_dims &d, const A &a, int i, int j,
                                                 int k, T *mL, T *mR)
{
    const ptrdiff_t s = (ptrdiff_t)d.plane();
    const T jf = fjf<T>(a, d.ix(i, j, k));
    const size_t qL = d.ix(i, j + 1, k + 1), qR = d.ix(i + 1, j + 1, k + 1);
    const bool lo3 = (i <= 3) || (i >= d.gend);
    const bool hi3 = (i + 1 <= 3) || (i + 1 >= d.gend);
#pragma unroll
    for (int n = 0; n < 5; n++) {
        const auto *U = a.U[n];
        if (lo3) mL[n] = left3<T, 1>(T(U[qL - s]), T(U[qL]), T(U[qL + s])) * jf;
        else mL[n] = left5<T, 1>(T(U[qL - 2 * s]), T(U[qL - s]), T(U[qL]), T(U[qL + s]), T(U[qL + 2 * s])) * jf;
        if (hi3) mR[n] = right3<T>(T(U[qR - s]), T(U[qR]), T(U[qR + s])) * jf;
        else mR[n] = right5<T>(T(U[qR - 2 * s]), T(U[qR - s]), T(U[qR]), T(U[qR + s]), T(U[qR + 2 * s])) * jf;
    }
}

// Flux_Y_limiter.cpp:115-477.  Near-wall branch (cell j <= 2 or >= ny-1):
// variable 1 uses ratios guarded by 1e-7 and the cell value times J; the
// reference's jL/jR there are uninitialised, here they are the face J_v, as
// in the interior branch.  Face 1 takes its left state and face ny its right
// state from the wall averages (Flux_Y_limiter.cpp:365-477).
template <typename T, typename SP>
__device__ __forceinline__ T ywall_var1_left(const SP *U, const SP *J, size_t q, ptrdiff_t s)
{
    T iu = T(U[q - s]), u = T(U[q]), ui = T(U[q + s]);
    T rL = (ui - u) / ((u - iu) + T(0.0000001));
    T m = lim3(rL);
    return (u * T(J[q]) + T(0.5) * rmax(T(0), m) * (u - iu));
}
template <typename T, typename SP>
__device__ __forceinline__ T ywall_var1_right(const SP *U, const SP *J, size_t q, ptrdiff_t s)
{
    T iu = T(U[q - s]), u = T(U[q]), ui = T(U[q + s]);
    T rR = (u - iu) / ((ui - u) + T(0.0000001));
    T m = lim3(rR);
    return (u * T(J[q]) - T(0.5) * rmax(T(0), m) * (ui - u));
}

// CF_SCHEME_CONSISTENT, near-wall rows: the limited 3rd-order states of the
// conserved variables q = U_*J of cells q-s, q, q+s themselves (the
// reference's variable-1 line with every cell value scaled by its own J),
// variable 1 with the reference's 1e-7 ratio guard
template <typename T, typename SP>
__device__ __forceinline__ T ywall_q_left(const SP *U, const SP *J, size_t q, ptrdiff_t s, bool guard)
{
    T iu = T(U[q - s]) * T(J[q - s]), u = T(U[q]) * T(J[q]), ui = T(U[q + s]) * T(J[q + s]);
    T rL = guard ? (ui - u) / ((u - iu) + T(0.0000001)) : (ui - u) / (u - iu);
    T m = lim3(rL);
    return u + T(0.5) * rmax(T(0), m) * (u - iu);
}
template <typename T, typename SP>
__device__ __forceinline__ T ywall_q_right(const SP *U, const SP *J, size_t q, ptrdiff_t s, bool guard)
{
    T iu = T(U[q - s]) * T(J[q - s]), u = T(U[q]) * T(J[q]), ui = T(U[q + s]) * T(J[q + s]);
    T rR = guard ? (u - iu) / ((ui - u) + T(0.0000001)) : (u - iu) / (ui - u);
    T m = lim3(rR);
    return u - T(0.5) * rmax(T(0), m) * (ui - u);
}

template <typename T, typename A>
__device__ __forceinline__ void states_y_limited(const cf_dims &d, const A &a, int i, int j,
                                                 int k, T *mL, T *mR)
{
    const ptrdiff_t s = d.Zm;
    const int ny = d.ny;
    const T jf = fjf<T>(a, d.ix(i, j, k));
    const size_t qL = d.ix(i + 1, j, k + 1), qR = d.ix(i + 1, j + 1, k + 1);
    // left state: cell j (face 1 is the wall average of cells 1, 2)
    if (j == 1) {
        T temp = T(1.) / (T(1) / T(a.J[qL]) + T(1) / T(a.J[qL + s]));
#pragma unroll
        for (int n = 0; n < 5; n++) mL[n] = temp * (T(a.U[n][qL]) + T(a.U[n][qL + s]));
    } else if ((j <= 2 || j >= ny - 1) && d.scheme) {
#pragma unroll
        for (int n = 0; n < 5; n++) mL[n] = ywall_q_left<T>(a.U[n], a.J, qL, s, n == 0);
    } else if (j <= 2 || j >= ny - 1) {
        mL[0] = ywall_var1_left<T>(a.U[0], a.J, qL, s);
#pragma unroll
        for (int n = 1; n < 5; n++)
            mL[n] = left3<T, 1>(T(a.U[n][qL - s]), T(a.U[n][qL]), T(a.U[n][qL + s])) * jf;
    } else {
#pragma unroll
        for (int n = 0; n < 5; n++) {
            const auto *U = a.U[n];
            mL[n] = left5<T, 1>(T(U[qL - 2 * s]), T(U[qL - s]), T(U[qL]), T(U[qL + s]), T(U[qL + 2 * s])) * jf;
        }
    }
    // right state: cell j+1 (face ny is the wall average of cells ny, ny+1)
    const int jc = j + 1;
    if (j == ny) {
        const size_t q = d.ix(i + 1, ny, k + 1);
        T temp = T(1.) / (T(1) / T(a.J[q]) + T(1) / T(a.J[q + s]));
#pragma unroll
        for (int n = 0; n < 5; n++) mR[n] = temp * (T(a.U[n][q]) + T(a.U[n][q + s]));
    } else if ((jc <= 2 || jc >= ny - 1) && d.scheme) {
#pragma unroll
        for (int n = 0; n < 5; n++) mR[n] = ywall_q_right<T>(a.U[n], a.J, qR, s, n == 0);
    } else if (jc <= 2 || jc >= ny - 1) {
        mR[0] = ywall_var1_right<T>(a.U[0], a.J, qR, s);
#pragma unroll
        for (int n = 1; n < 5; n++)
            mR[n] = right3<T>(T(a.U[n][qR - s]), T(a.U[n][qR]), T(a.U[n][qR + s])) * jf;
    } else {
#pragma unroll
        for (int n = 0; n < 5; n++) {
            const auto *U = a.U[n];
            mR[n] = right5<T>(T(U[qR - 2 * s]), T(U[qR - s]), T(U[qR]), T(U[qR + s]), T(U[qR + 2 * s])) * jf;
        }
    }
}

// Flux_Z_limiter.cpp:120-520.  Faces 1, 2, nz-1, nz use the boundary rows
// (average, linear 3rd order); interior cells k = 3..nz-1 the limited states
// scaled by 1/sum(w/J) with the reference's unnormalised weights, and the
// 3rd-order branch where k >= ny (the reference compares with the y extent).
// CF_SCHEME_CONSISTENT: numerators 60 and 6 (the weights' sums) and the
// upwind left slope.
template <typename T, typename SP>
__device__ __forceinline__ T zjL5(const SP *J, size_t q, int scheme = 0)
{
    return T(scheme ? 60. : 1.) / (T(2) / T(J[q - 2]) - T(13) / T(J[q - 1]) + T(47) / T(J[q]) + T(27) / T(J[q + 1]) - T(3) / T(J[q + 2]));
}
template <typename T, typename SP>
__device__ __forceinline__ T zjR5(const SP *J, size_t q, int scheme = 0)
{
    return T(scheme ? 60. : 1.) / (T(-3) / T(J[q - 2]) + T(27) / T(J[q - 1]) + T(47) / T(J[q]) - T(13) / T(J[q + 1]) + T(2) / T(J[q + 2]));
}
template <typename T, typename SP>
__device__ __forceinline__ T zjL3(const SP *J, size_t q, int scheme = 0)
{
    return T(scheme ? 6. : 1.) / (T(-1) / T(J[q - 1]) + T(5) / T(J[q]) + T(2) / T(J[q + 1]));
}
template <typename T, typename SP>
__device__ __forceinline__ T zjR3(const SP *J, size_t q, int scheme = 0)
{
    return T(scheme ? 6. : 1.) / (T(2) / T(J[q - 1]) + T(5) / T(J[q]) - T(1) / T(J[q + 1]));
}

template <typename T, typename A>
__device__ __forceinline__ void states_z_limited(const cf_dims &d, const A &a, int i, int j,
                                                 int k, T *mL, T *mR)
{
    const int nz = d.nz, ny = d.ny;
    const size_t qL = d.ix(i + 1, j + 1, k), qR = d.ix(i + 1, j + 1, k + 1);
    // left state of face k from cell k
    if (k == 1) {
#pragma unroll
        for (int n = 0; n < 5; n++) mL[n] = avg2<T>(a.U[n], a.J, qL, 1);
    } else if (k == 2 || k == nz) {
#pragma unroll
        for (int n = 0; n < 5; n++) mL[n] = lin3L<T>(a.U[n], a.J, qL, 1);
    } else if (k >= ny) {
        T jl = T(a.wz[0][qL]);
#pragma unroll
        for (int n = 0; n < 5; n++)
            mL[n] = (d.scheme ? left3<T, 1>(T(a.U[n][qL - 1]), T(a.U[n][qL]), T(a.U[n][qL + 1]))
                              : left3<T, -1>(T(a.U[n][qL - 1]), T(a.U[n][qL]), T(a.U[n][qL + 1]))) * jl;
    } else {
        T jl = T(a.wz[0][qL]);
#pragma unroll
        for (int n = 0; n < 5; n++) {
            const auto *U = a.U[n];
            mL[n] = (d.scheme ? left5<T, 1>(T(U[qL - 2]), T(U[qL - 1]), T(U[qL]), T(U[qL + 1]), T(U[qL + 2]))
                              : left5<T, -1>(T(U[qL - 2]), T(U[qL - 1]), T(U[qL]), T(U[qL + 1]), T(U[qL + 2]))) * jl;
        }
    }
    // right state of face k from cell k+1
    const int kc = k + 1;
    if (k == nz) {
#pragma unroll
        for (int n = 0; n < 5; n++) mR[n] = avg2<T>(a.U[n], a.J, qL, 1);
    } else if (kc == 2 || kc == nz) {
#pragma unroll
        for (int n = 0; n < 5; n++) mR[n] = lin3R<T>(a.U[n], a.J, qR, 1);
    } else if (kc >= ny) {
        T jr = T(a.wz[1][qR]);
#pragma unroll
        for (int n = 0; n < 5; n++)
            mR[n] = right3<T>(T(a.U[n][qR - 1]), T(a.U[n][qR]), T(a.U[n][qR + 1])) * jr;
    } else {
        T jr = T(a.wz[1][qR]);
#pragma unroll
        for (int n = 0; n < 5; n++) {
            const auto *U = a.U[n];
            mR[n] = right5<T>(T(U[qR - 2]), T(U[qR - 1]), T(U[qR]), T(U[qR + 1]), T(U[qR + 2])) * jr;
        }
    }
}

// Flux_X.cpp:102-215 (5-point for cells 4..gend-1; seam rows 2, 3, gend)
template <typename T, typename A>
__device__ __forceinline__ void states_x_linear(const cf_dims &d, const A &a, int i, int j,
                                                int k, T *mL, T *mR)
{
    const ptrdiff_t s = (ptrdiff_t)d.plane();
    const int gend = d.gend;
    const size_t qL = d.ix(i, j + 1, k + 1), qR = d.ix(i + 1, j + 1, k + 1);
#pragma unroll
    for (int n = 0; n < 5; n++) {
        const auto *U = a.U[n];
        if (i == 2) mL[n] = avg2<T>(U, a.J, qL, s);
        else if (i == 3 || i == gend) mL[n] = lin3L<T>(U, a.J, qL, s);
        else mL[n] = lin5L<T>(U, a.J, qL, s);
        if (i == gend) mR[n] = avg2<T>(U, a.J, qL, s);
        else if (i + 1 == 3 || i + 1 == gend) mR[n] = lin3R<T>(U, a.J, qR, s);
        else mR[n] = lin5R<T>(U, a.J, qR, s);
    }
}

// Flux_Y.cpp:100-240 (5-point for cells 4..ny-2; rows 1, 2, 3, ny-1, ny)
template <typename T, typename A>
__device__ __forceinline__ void states_y_linear(const cf_dims &d, const A &a, int i, int j,
                                                int k, T *mL, T *mR)
{
    const ptrdiff_t s = d.Zm;
    const int ny = d.ny;
    const size_t qL = d.ix(i + 1, j, k + 1), qR = d.ix(i + 1, j + 1, k + 1);
#pragma unroll
    for (int n = 0; n < 5; n++) {
        const auto *U = a.U[n];
        if (j == 1 || j == 2) mL[n] = avg2<T>(U, a.J, qL, s);
        else if (j == 3 || j == ny - 1) mL[n] = lin3L<T>(U, a.J, qL, s);
        else if (j == ny) mL[n] = avg2hi<T>(U, a.J, qL, s);
        else mL[n] = lin5L<T>(U, a.J, qL, s);
        if (j == 1) mR[n] = avg2<T>(U, a.J, qR, s);
        else if (j == 2 || j == ny - 2) mR[n] = lin3R<T>(U, a.J, qR, s);
        else if (j == ny - 1) mR[n] = avg2hi<T>(U, a.J, qR, s);
        else if (j == ny) mR[n] = avg2<T>(U, a.J, qL, s);
        else mR[n] = lin5R<T>(U, a.J, qR, s);
    }
}

// Flux_Z.cpp:104-300 (5-point for cells 3..nz-1; rows 1, 2, nz)
template <typename T, typename A>
__device__ __forceinline__ void states_z_linear(const cf_dims &d, const A &a, int i, int j,
                                                int k, T *mL, T *mR)
{
    const int nz = d.nz;
    const size_t qL = d.ix(i + 1, j + 1, k), qR = d.ix(i + 1, j + 1, k + 1);
#pragma unroll
    for (int n = 0; n < 5; n++) {
        const auto *U = a.U[n];
        if (k == 1) mL[n] = avg2<T>(U, a.J, qL, 1);
        else if (k == 2 || k == nz) mL[n] = lin3L<T>(U, a.J, qL, 1);
        else mL[n] = lin5L<T>(U, a.J, qL, 1);
        if (k == nz) mR[n] = avg2<T>(U, a.J, qL, 1);
        else if (k == 1 || k == nz - 1) mR[n] = lin3R<T>(U, a.J, qR, 1);
        else mR[n] = lin5R<T>(U, a.J, qR, 1);
    }
}

// ---------------------------------------------------------------------------
// face fluxes
// ---------------------------------------------------------------------------
// Preconditioned Roe (Flux_X_limiter.cpp:382-536).  n0..n2: normal metric
// row.  F[5] receives the wall-face form of the normal-momentum flux.
template <typename T>
__device__ __forceinline__ void flux_precond_roe(const T *mL, const T *mR, const T *m, int dir, T Ep,
                                                 T Jf, T K, T e, T *F)
{
    const T n0 = m[3 * dir], n1 = m[3 * dir + 1], n2 = m[3 * dir + 2];
    T NX = n0 / (sqrt(n0 * n0 + n1 * n1 + n2 * n2));
    T NY = n1 / (sqrt(n0 * n0 + n1 * n1 + n2 * n2));
    T NZ = n2 / (sqrt(n0 * n0 + n1 * n1 + n2 * n2));

    T _rho = mL[0];
    T _u = mL[1] / _rho;
    T _v = mL[2] / _rho;
    T _w = mL[3] / _rho;
    T _U = n0 * _u + n1 * _v + n2 * _w;
    T __U = NX * _u + NY * _v + NZ * _w;
    T _VV = _u * _u + _v * _v + _w * _w;
    T _P = (mL[4] - T(0.5) * _rho * _VV) * (K - T(1));
    T _T = _P / _rho;
    T _C = K * _P / _rho;
    T _H = T(0.5) * _VV + _C / (K - T(1));

    T rho_ = mR[0];
    T u_ = mR[1] / rho_;
    T v_ = mR[2] / rho_;
    T w_ = mR[3] / rho_;
    T U_ = n0 * u_ + n1 * v_ + n2 * w_;
    T U__ = NX * u_ + NY * v_ + NZ * w_;
    T VV_ = u_ * u_ + v_ * v_ + w_ * w_;
    T P_ = (mR[4] - T(0.5) * rho_ * VV_) * (K - T(1));
    T T_ = P_ / rho_;
    T C_ = K * P_ / rho_;
    T H_ = T(0.5) * VV_ + C_ / (K - T(1));

    T rho = T(0.5) * (_rho + rho_);
    T u = T(0.5) * (_u + u_);
    T v = T(0.5) * (_v + v_);
    T w = T(0.5) * (_w + w_);
    T U = T(0.5) * (_U + U_);
    T _U_ = T(0.5) * (__U + U__);
    T VV = u * u + v * v + w * w;
    T H = T(0.5) * (_H + H_);
    T C = (H - T(0.5) * VV) * (K - T(1));
    T P = rho * C / K;
    T Tm = P / rho;

    T dU1 = P_ - _P, dU2 = u_ - _u, dU3 = v_ - _v, dU4 = w_ - _w, dU5 = T_ - _T;

    T beta = rmax(VV / C, e);
    T S = sqrt(U * U * (beta - T(1)) * (beta - T(1)) + T(4) * beta * C * (n0 * n0 + n1 * n1 + n2 * n2));
    T _S_ = sqrt(_U_ * _U_ * (beta - T(1)) * (beta - T(1)) + T(4) * beta * C * (NX * NX + NY * NY + NZ * NZ));

    T temp = T(4) * K * _S_ * Tm * beta;
    T temp1 = S + U + U * beta;
    T temp2 = -S + U + U * beta;
    T temp3 = _S_ - _U_ + _U_ * beta;
    T temp4 = _S_ + _U_ - _U_ * beta;
    T temp5 = _S_ * _S_ - (beta - T(1)) * (beta - T(1)) * _U_ * _U_;
    T tempu1 = T(2) * Tm * NX * K * beta + u * _S_ + u * (beta - T(1)) * _U_;
    T tempu2 = T(2) * Tm * NX * K * beta - u * _S_ + u * (beta - T(1)) * _U_;
    T tempv1 = T(2) * Tm * NY * K * beta + v * _S_ + v * (beta - T(1)) * _U_;
    T tempv2 = T(2) * Tm * NY * K * beta - v * _S_ + v * (beta - T(1)) * _U_;
    T tempw1 = T(2) * Tm * NZ * K * beta + w * _S_ + w * (beta - T(1)) * _U_;
    T tempw2 = T(2) * Tm * NZ * K * beta - w * _S_ + w * (beta - T(1)) * _U_;
    T tempuvw = T(2) * Tm * K * beta * (u * NX + v * NY + w * NZ);
    T temph1 = tempuvw + H * _S_ + H * _U_ * beta - H * _U_;
    T temph2 = tempuvw - H * _S_ + H * _U_ * beta - H * _U_;
    T aU = fabs(U), a1 = fabs(temp1), a2 = fabs(temp2);

    T d11 = T(1) / temp * (T(4) * (K - T(1)) * _S_ * beta * aU + temp3 * a1 + temp4 * a2);
    T d12 = T(-1) / (T(2) * temp) * (NX * rho * (a2 - a1) * temp5);
    T d13 = T(-1) / (T(2) * temp) * (NY * rho * (a2 - a1) * temp5);
    T d14 = T(-1) / (T(2) * temp) * (NZ * rho * (a2 - a1) * temp5);
    T d15 = -rho * aU / Tm;

    T d21 = T(1) / temp * (u * _S_ * (T(4) * (K - T(1)) * beta * aU + a2 + a1) - (a2 - a1) * (T(2) * Tm * NX * K * beta + u * _U_ * (beta - T(1))));
    T d22 = T(1) / (T(2) * temp) * (rho * (T(8) * Tm * K * _S_ * beta * (NY * NY + NZ * NZ) * aU + NX * (temp3 * tempu2 * a2 + temp4 * tempu1 * a1)));
    T d23 = T(1) / (T(2) * temp) * (rho * NY * (T(-8) * Tm * K * _S_ * beta * NX * aU + temp3 * tempu2 * a2 + temp4 * tempu1 * a1));
    T d24 = T(1) / (T(2) * temp) * (rho * NZ * (T(-8) * Tm * K * _S_ * beta * NX * aU + temp3 * tempu2 * a2 + temp4 * tempu1 * a1));
    T d25 = -u * rho * aU / Tm;

    T d31 = T(1) / temp * (v * _S_ * (T(4) * (K - T(1)) * beta * aU + a2 + a1) - (a2 - a1) * (T(2) * Tm * NY * K * beta + v * _U_ * (beta - T(1))));
    T d32 = T(1) / (T(2) * temp) * (rho * NX * (T(-8) * Tm * K * _S_ * beta * NY * aU + temp3 * tempv2 * a2 + temp4 * tempv1 * a1));
    T d33 = T(1) / (T(2) * temp) * (rho * (T(8) * Tm * K * _S_ * beta * (NX * NX + NZ * NZ) * aU + NY * (temp3 * tempv2 * a2 + temp4 * tempv1 * a1)));
    T d34 = T(1) / (T(2) * temp) * (rho * NZ * (T(-8) * Tm * K * _S_ * beta * NY * aU + temp3 * tempv2 * a2 + temp4 * tempv1 * a1));
    T d35 = -v * rho * aU / Tm;

    T d41 = T(1) / temp * (w * _S_ * (T(4) * (K - T(1)) * beta * aU + a2 + a1) - (a2 - a1) * (T(2) * Tm * NZ * K * beta + w * _U_ * (beta - T(1))));
    T d42 = T(1) / (T(2) * temp) * (rho * NX * (T(-8) * Tm * K * _S_ * beta * NZ * aU + temp3 * tempw2 * a2 + temp4 * tempw1 * a1));
    T d43 = T(1) / (T(2) * temp) * (rho * NY * (T(-8) * Tm * K * _S_ * beta * NZ * aU + temp3 * tempw2 * a2 + temp4 * tempw1 * a1));
    T d44 = T(1) / (T(2) * temp) * (rho * (T(8) * Tm * K * _S_ * beta * (NX * NX + NY * NY) * aU + NZ * (temp3 * tempw2 * a2 + temp4 * tempw1 * a1)));
    T d45 = -w * rho * aU / Tm;

    T d51 = T(1) / temp * (_S_ * (T(4) * beta * (H * K - H - Tm * K) * aU + H * (a2 + a1)) - (a2 - a1) * (tempuvw + H * _U_ * beta - H * _U_));
    T d52 = T(1) / (T(2) * temp) * (rho * (T(8) * Tm * K * _S_ * beta * (-v * NX * NY - w * NX * NZ + u * (NY * NY + NZ * NZ) * aU) + NX * (temph2 * temp3 * a2 + temph1 * temp4 * a1)));
    T d53 = T(1) / (T(2) * temp) * (rho * (T(8) * Tm * K * _S_ * beta * (-u * NX * NY - w * NY * NZ + v * (NX * NX + NZ * NZ) * aU) + NY * (temph2 * temp3 * a2 + temph1 * temp4 * a1)));
    T d54 = T(1) / (T(2) * temp) * (rho * (T(8) * Tm * K * _S_ * beta * (-u * NX * NZ - v * NY * NZ + w * (NX * NX + NY * NY) * aU) + NZ * (temph2 * temp3 * a2 + temph1 * temp4 * a1)));
    T d55 = (-H / Tm + K / (K - T(1))) * rho * aU;

    T Fav1 = d11 * dU1 + d12 * dU2 + d13 * dU3 + d14 * dU4 + d15 * dU5;
    T Fav2 = d21 * dU1 + d22 * dU2 + d23 * dU3 + d24 * dU4 + d25 * dU5;
    T Fav3 = d31 * dU1 + d32 * dU2 + d33 * dU3 + d34 * dU4 + d35 * dU5;
    T Fav4 = d41 * dU1 + d42 * dU2 + d43 * dU3 + d44 * dU4 + d45 * dU5;
    T Fav5 = d51 * dU1 + d52 * dU2 + d53 * dU3 + d54 * dU4 + d55 * dU5;

    F[0] = T(0.5) * ((_rho * _U + rho_ * U_) - Ep * Fav1) / Jf;
    F[1] = T(0.5) * ((_rho * _u * _U + rho_ * u_ * U_ + n0 * (_P + P_)) - Ep * Fav2) / Jf;
    F[2] = T(0.5) * ((_rho * _v * _U + rho_ * v_ * U_ + n1 * (_P + P_)) - Ep * Fav3) / Jf;
    F[3] = T(0.5) * ((_rho * _w * _U + rho_ * w_ * U_ + n2 * (_P + P_)) - Ep * Fav4) / Jf;
    F[4] = T(0.5) * ((_U * (T(3.5) * _P + T(0.5) * _rho * _VV) + U_ * (T(3.5) * P_ + T(0.5) * rho_ * VV_)) - Ep * Fav5) / Jf;
    F[5] = T(0.5) * (n1 * (_P + P_) - Ep * Fav3) / Jf;
}

// Roe, ROE == 1 (Flux_X.cpp:247-420); energy term deltaP*U in x and z,
// deltaP*V*insqr in y (Flux_Y.cpp:383).
template <typename T>
__device__ __forceinline__ void flux_roe(const T *mL, const T *mR, const T *m, int dir, T Jf, T K, T *F)
{
    const T n0 = m[3 * dir], n1 = m[3 * dir + 1], n2 = m[3 * dir + 2];
    T insqr = T(1.0) / sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    T NX = n0 * insqr, NY = n1 * insqr, NZ = n2 * insqr;

    T _rho = mL[0];
    T _u = mL[1] / _rho;
    T _v = mL[2] / _rho;
    T _w = mL[3] / _rho;
    T _U = n0 * _u + n1 * _v + n2 * _w;
    T _VV = _u * _u + _v * _v + _w * _w;
    T _P = (mL[4] - T(0.5) * _rho * _VV) * (K - T(1));
    T _C = K * _P / _rho;
    T _H = T(0.5) * _VV + _C / (K - T(1));

    T rho_ = mR[0];
    T u_ = mR[1] / rho_;
    T v_ = mR[2] / rho_;
    T w_ = mR[3] / rho_;
    T U_ = n0 * u_ + n1 * v_ + n2 * w_;
    T VV_ = u_ * u_ + v_ * v_ + w_ * w_;
    T P_ = (mR[4] - T(0.5) * rho_ * VV_) * (K - T(1));
    T C_ = K * P_ / rho_;
    T H_ = T(0.5) * VV_ + C_ / (K - T(1));

    T temp5 = sqrt(_rho);
    T temp6 = sqrt(rho_);
    T temp4 = temp5 + temp6;
    T rho = sqrt(_rho * rho_);
    T u = (temp5 * _u + temp6 * u_) / temp4;
    T v = (temp5 * _v + temp6 * v_) / temp4;
    T w = (temp5 * _w + temp6 * w_) / temp4;
    T U = (temp5 * _U + temp6 * U_) / temp4;
    T VV = u * u + v * v + w * w;
    T H = (temp5 * _H + temp6 * H_) / temp4;
    T C = (H - T(0.5) * VV) * (K - T(1));

    T dU1 = rho_ - _rho;
    T dU2 = rho_ * u_ - _rho * _u;
    T dU3 = rho_ * v_ - _rho * _v;
    T dU4 = rho_ * w_ - _rho * _w;
    T dU5 = (P_ / (K - T(1)) + T(0.5) * rho_ * VV_) - (_P / (K - T(1)) + T(0.5) * _rho * _VV);

    T S = sqrt(C);
    T temp1 = (P_ - _P) / rho / C;
    T temp2 = U * insqr / S * (U_ - _U) * insqr;
    T deltaU = (S - fabs(U * insqr)) * temp1 + temp2;
    T deltaP = U * insqr / S * (P_ - _P) + (S - fabs(U * insqr)) * rho * (U_ - _U) * insqr;

    T Fav1 = fabs(U * insqr) * dU1 + deltaU * rho;
    T Fav2 = fabs(U * insqr) * dU2 + deltaU * rho * u + deltaP * NX;
    T Fav3 = fabs(U * insqr) * dU3 + deltaU * rho * v + deltaP * NY;
    T Fav4 = fabs(U * insqr) * dU4 + deltaU * rho * w + deltaP * NZ;
    T Fav5 = dir == 1 ? fabs(U * insqr) * dU5 + deltaU * rho * H + deltaP * U * insqr
                      : fabs(U * insqr) * dU5 + deltaU * rho * H + deltaP * U;

    F[0] = T(0.5) * ((_rho * _U + rho_ * U_) - Fav1 / insqr) / Jf;
    F[1] = T(0.5) * ((_rho * _u * _U + rho_ * u_ * U_ + n0 * (_P + P_)) - Fav2 / insqr) / Jf;
    F[2] = T(0.5) * ((_rho * _v * _U + rho_ * v_ * U_ + n1 * (_P + P_)) - Fav3 / insqr) / Jf;
    F[3] = T(0.5) * ((_rho * _w * _U + rho_ * w_ * U_ + n2 * (_P + P_)) - Fav4 / insqr) / Jf;
    F[4] = T(0.5) * ((_U * (T(3.5) * _P + T(0.5) * _rho * _VV) + U_ * (T(3.5) * P_ + T(0.5) * rho_ * VV_)) - Fav5 / insqr) / Jf;
    F[5] = T(0.5) * (n1 * (_P + P_) - Fav3 / insqr) / Jf;
}

}  // namespace CF_NS

#ifdef CF_FAST_MATH
#include "cf_flux_fast.cuh"
#endif

namespace CF_NS {

// One thread per face of the box; DIR 0/1/2, LIMITED selects the scheme.
// A is cf_flux_args (FP64 cell arrays) or, in the FP32 build,
// cf_flux_args_f (FP32 copies of U, J and 1/J made once per call, so the
// stencil reads convert nothing; the face arrays stay FP64).
// FP32: at least four blocks per SM (64 registers; a few bytes of spill,
// measured 15 % faster than three blocks without)
//
// ZP (z faces only): 0 every face of the box; 1 the interior faces k =
// 3..nz-2 of the box (their warps never take the edge branches); 2 the four
// edge faces k = 1, 2, nz-1, nz of every (i, j) of the box, four lanes per
// row.  A warp of the z box spans 32 consecutive k, so with ZP 0 the warps
// holding a row's edges execute the edge and the interior code one after
// the other.
template <int DIR, bool LIMITED, typename T, typename A = cf_flux_args, int ZP = 0>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) k_flux(cf_dims d, A a, cf_box b)
{
    int i, j, k;
    if (ZP == 2) {
        const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        const int e = (int)(t & 3);
        const long long r = t >> 2;
        j = b.j0 + (int)(r % b.nj);
        i = b.i0 + (int)(r / b.nj);
        if (i >= b.i0 + b.ni) return;
        k = e < 2 ? 1 + e : d.nz - 3 + e;
    } else {
        k = b.k0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
        j = b.j0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
        i = b.i0 + (int)blockIdx.z;
        if (k >= b.k0 + b.nk || j >= b.j0 + b.nj) return;
    }
    T mL[5], mR[5], m[9], F[6];
#ifdef CF_FAST_MATH
    if (DIR == 0) {
        if (LIMITED) fast_states_x_limited<T>(d, a, i, j, k, mL, mR);
        else fast_states_x_linear<T>(d, a, i, j, k, mL, mR);
    } else if (DIR == 1) {
        if (LIMITED) fast_states_y_limited<T>(d, a, i, j, k, mL, mR);
        else fast_states_y_linear<T>(d, a, i, j, k, mL, mR);
    } else {
        if (LIMITED) fast_states_z_limited<T, A, ZP == 1>(d, a, i, j, k, mL, mR);
        else fast_states_z_linear<T, A, ZP == 1>(d, a, i, j, k, mL, mR);
    }
    const size_t q = d.ix(i, j, k);
#pragma unroll
    for (int n = 0; n < 9; n++) m[n] = fmet<T>(a, n, q);
    if (LIMITED)
        fast_flux_precond_roe<T>(mL, mR, m, DIR, T(a.Ep[q]), fjf<T>(a, q), CF_DC(T, d, K), CF_DC(T, d, e), F);
    else
        fast_flux_roe<T>(mL, mR, m, DIR, fjf<T>(a, q), CF_DC(T, d, K), F);
#else
    if (DIR == 0) {
        if (LIMITED) states_x_limited<T>(d, a, i, j, k, mL, mR);
        else states_x_linear<T>(d, a, i, j, k, mL, mR);
    } else if (DIR == 1) {
        if (LIMITED) states_y_limited<T>(d, a, i, j, k, mL, mR);
        else states_y_linear<T>(d, a, i, j, k, mL, mR);
    } else {
        if (LIMITED) states_z_limited<T>(d, a, i, j, k, mL, mR);
        else states_z_linear<T>(d, a, i, j, k, mL, mR);
    }
    const size_t q = d.ix(i, j, k);
#pragma unroll
    for (int n = 0; n < 9; n++) m[n] = fmet<T>(a, n, q);
    if (LIMITED)
        flux_precond_roe<T>(mL, mR, m, DIR, T(a.Ep[q]), fjf<T>(a, q), CF_DC(T, d, K), CF_DC(T, d, e), F);
    else
        flux_roe<T>(mL, mR, m, DIR, fjf<T>(a, q), CF_DC(T, d, K), F);
#endif
    const int f32 = a.f32_out;
    if (DIR == 1 && (j == 1 || j == d.ny)) {
        // wall faces keep the pressure term of the normal momentum only
        rhs_put<T>(a.F[0], q, T(0), f32);
        rhs_put<T>(a.F[1], q, T(0), f32);
        rhs_put<T>(a.F[2], q, F[5], f32);
        rhs_put<T>(a.F[3], q, T(0), f32);
        rhs_put<T>(a.F[4], q, T(0), f32);
    } else {
#pragma unroll
        for (int n = 0; n < 5; n++) rhs_put<T>(a.F[n], q, F[n], f32);
    }
}

#ifdef CF_WITH_FLOAT
// FP32 x faces marching along x.  Each thread owns one (j, k) face column
// of the box and walks a chunk of its x faces in order, keeping the six
// cells i-2..i+3 of the current face's stencil for each variable in
// registers: one new cell per variable and face instead of six, and the
// next face's cell, metrics and sensor requested before the current face
// is evaluated, so the loads of one face overlap the arithmetic of the
// previous one.  (One thread per face reads six cells one x plane apart,
// which L1 never reuses; those faces wait on L2.)  The arithmetic is
// fast_states_x_limited / fast_lin_pair on the same values, so the fluxes
// equal the per-face kernel's bit for bit.
template <bool LIMITED>
__global__ void __launch_bounds__(256, 3) k_flux_x_march(cf_dims d, cf_flux_args_f a, cf_box b, int chunk)
{
    const int k = b.k0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = b.j0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (k >= b.k0 + b.nk || j >= b.j0 + b.nj) return;
    const int ia = b.i0 + (int)blockIdx.z * chunk;
    const int ib = min(ia + chunk, b.i0 + b.ni);
    if (ia >= ib) return;
    const ptrdiff_t s = (ptrdiff_t)d.plane();
    const int f32 = a.f32_out;
    // window: cells ia-2 .. ia+3 of row (j+1, k+1)
    float u[5][6];
    const size_t c0 = d.ix(ia, j + 1, k + 1);
#pragma unroll
    for (int n = 0; n < 5; n++)
#pragma unroll
        for (int t = 0; t < 6; t++) u[n][t] = a.U[n][c0 + (t - 2) * s];
    float iJw[6];
    if (!LIMITED) {
#pragma unroll
        for (int t = 0; t < 6; t++) iJw[t] = frcp<float>(a.J[c0 + (t - 2) * s]);
    }
    for (int i = ia; i < ib; i++) {
        const size_t q = d.ix(i, j, k);
        float m[9], mL[5], mR[5], F[6];
#pragma unroll
        for (int n = 0; n < 9; n++) m[n] = fmet<float>(a, n, q);
        const float jf = fjf<float>(a, q);
        const float ep = LIMITED ? float(a.Ep[q]) : 0.f;
        // next face's new cell (i+4), requested before this face's arithmetic
        float nx[5], nj = 0.f;
        const bool more = i + 1 < ib;
        const size_t cn = d.ix(i + 4, j + 1, k + 1);
#pragma unroll
        for (int n = 0; n < 5; n++) nx[n] = more ? a.U[n][cn] : 0.f;
        if (!LIMITED && more) nj = a.J[cn];
        if (LIMITED) {
            const bool lo3 = (i <= 3) || (i >= d.gend);
            const bool hi3 = (i + 1 <= 3) || (i + 1 >= d.gend);
#pragma unroll
            for (int n = 0; n < 5; n++) fast_pair<float, 1>(u[n], lo3, hi3, jf, jf, mL[n], mR[n]);
            fast_flux_precond_roe<float>(mL, mR, m, 0, ep, jf, CF_DC(float, d, K), CF_DC(float, d, e), F);
        } else {
            if (i <= 3 || i >= d.gend - 1) {
                states_x_linear<float>(d, a, i, j, k, mL, mR);
            } else {
                const float tl = frcp<float>(2.f * iJw[0] - 13.f * iJw[1] + 47.f * iJw[2] + 27.f * iJw[3] - 3.f * iJw[4]);
                const float tr = frcp<float>(-3.f * iJw[1] + 27.f * iJw[2] + 47.f * iJw[3] - 13.f * iJw[4] + 2.f * iJw[5]);
#pragma unroll
                for (int n = 0; n < 5; n++) {
                    const float *w = u[n];
                    mL[n] = tl * (2.f * w[0] - 13.f * w[1] + 47.f * w[2] + 27.f * w[3] - 3.f * w[4]);
                    mR[n] = tr * (-3.f * w[1] + 27.f * w[2] + 47.f * w[3] - 13.f * w[4] + 2.f * w[5]);
                }
            }
            fast_flux_roe<float>(mL, mR, m, 0, jf, CF_DC(float, d, K), F);
        }
#pragma unroll
        for (int n = 0; n < 5; n++) rhs_put<float>(a.F[n], q, F[n], f32);
#pragma unroll
        for (int n = 0; n < 5; n++) {
#pragma unroll
            for (int t = 0; t < 5; t++) u[n][t] = u[n][t + 1];
            u[n][5] = nx[n];
        }
        if (!LIMITED) {
#pragma unroll
            for (int t = 0; t < 5; t++) iJw[t] = iJw[t + 1];
            iJw[5] = more ? frcp<float>(nj) : 0.f;
        }
    }
}

// chunk of x faces per block: enough blocks for four per SM
inline int flux_x_chunk(const cf_box &b)
{
    const long long cols = (long long)((b.nk + 31) / 32) * ((b.nj + 7) / 8);
    const long long want = 152LL * 8;
    long long nch = (want + cols - 1) / cols;
    if (nch < 1) nch = 1;
    int chunk = (int)((b.ni + nch - 1) / nch);
    return chunk < 8 ? 8 : chunk;
}
#endif

// face boxes of the reference's flux loops
static inline cf_box flux_box(const cf_dims &d, int dir)
{
    if (dir == 0) return make_box(2, d.gend, 1, d.ny - 1, 1, d.nz - 1);      // Flux_X*.cpp face loop
    if (dir == 1) return make_box(2, d.gend - 1, 1, d.ny, 1, d.nz - 1);      // Flux_Y*.cpp
    return make_box(2, d.gend - 1, 1, d.ny - 1, 1, d.nz);                    // Flux_Z*.cpp
}

// The z limiter's state weights 1/sum(w/J) depend on J alone.  The no-FMA
// build forms them once per cell with the reference's expressions
// (Flux_Z_limiter.cpp:190-196, 3rd order where k >= ny) into wz[0], wz[1];
// the contracted and FP32 builds store 1/J in wz[0] and form the weights
// from it in the flux kernel (two divisions per face instead of eight).
__global__ void __launch_bounds__(256) k_flux_zweights(cf_dims d, const double *__restrict__ J, double *wl,
                                                       double *wr, cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
#ifdef CF_FAST_MATH
    (void)wr;
    wl[q] = 1.0 / J[q];
#else
    const bool o3 = k >= d.ny;
    wl[q] = o3 ? zjL3<double>(J, q, d.scheme) : zjL5<double>(J, q, d.scheme);
    wr[q] = o3 ? zjR3<double>(J, q, d.scheme) : zjR5<double>(J, q, d.scheme);
#endif
}

// the z faces of box b: interior faces k = 3..nz-2 in one launch, the four
// edge faces of every row in another (small grids: one launch of all)
template <bool LIM, typename T, typename A>
cudaError_t launch_flux_z(const cf_dims &d, const A &a, const cf_box &b, cudaStream_t s)
{
    if (d.nz < 6 || b.k0 != 1 || b.nk != d.nz) {
        k_flux<2, LIM, T, A><<<box_grid(b), box_block(), 0, s>>>(d, a, b);
        return cudaGetLastError();
    }
    cf_box bi = b;
    bi.k0 = 3;
    bi.nk = d.nz - 4;
    k_flux<2, LIM, T, A, 1><<<box_grid(bi), box_block(), 0, s>>>(d, a, bi);
    const long long n = 4LL * b.ni * b.nj;
    k_flux<2, LIM, T, A, 2><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, a, b);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_flux(const cf_dims &d, const cf_flux_args &a, int dir, bool limited, cudaStream_t s)
{
    cf_box b = flux_box(d, dir);
    if (b.ni == 0 || b.nj == 0 || b.nk == 0) return cudaSuccess;
    dim3 g = box_grid(b), t = box_block();
    if (dir == 2 && limited) {
        if (!a.wz[0] || !a.wz[1]) return cudaErrorInvalidValue;
#ifdef CF_FAST_MATH
        cf_box bw = make_box(3, d.gend, 2, d.ny, 1, d.nz + 1);      // 1/J of every cell a stencil reads
#else
        cf_box bw = make_box(3, d.gend, 2, d.ny, 3, d.nz - 1);
#endif
        if (bw.nk > 0) k_flux_zweights<<<box_grid(bw), t, 0, s>>>(d, a.J, a.wz[0], a.wz[1], bw);
    }
    if (dir == 2) return limited ? launch_flux_z<true, T>(d, a, b, s) : launch_flux_z<false, T>(d, a, b, s);
    if (limited) {
        if (dir == 0) k_flux<0, true, T><<<g, t, 0, s>>>(d, a, b);
        else k_flux<1, true, T><<<g, t, 0, s>>>(d, a, b);
    } else {
        if (dir == 0) k_flux<0, false, T><<<g, t, 0, s>>>(d, a, b);
        else k_flux<1, false, T><<<g, t, 0, s>>>(d, a, b);
    }
    return cudaGetLastError();
}


#ifdef CF_WITH_FLOAT
// FP32 copies of the cell arrays the stencils read: U1..U5, J and 1/J over
// every index of the array (one FP64 -> FP32 conversion per value instead
// of one per stencil read)
__global__ void __launch_bounds__(256) k_flux_shadow(size_t n, cf_ptr5 U, const double *__restrict__ J, float *u0,
                                                     float *u1, float *u2, float *u3, float *u4, float *jf,
                                                     float *ij)
{
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    u0[q] = float(U.p[0][q]);
    u1[q] = float(U.p[1][q]);
    u2[q] = float(U.p[2][q]);
    u3[q] = float(U.p[3][q]);
    u4[q] = float(U.p[4][q]);
    if (J) {
        const float j = float(J[q]);
        jf[q] = j;
        ij[q] = 1.0f / j;
    }
}

// FP32 fluxes from the FP32 copies in sh (7 fields: U1..U5, J, 1/J);
// convert = false reuses copies made by an earlier call for the same U, J
inline cudaError_t launch_flux_f32(const cf_dims &d, const cf_flux_args &a, float *sh, bool convert,
                                   const float *const *met32, int dir, bool limited, cudaStream_t s)
{
    const size_t n = d.total();
    if (convert) {
        cf_ptr5 U;
        for (int v = 0; v < 5; v++) U.p[v] = const_cast<double *>(a.U[v]);
        k_flux_shadow<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, U, a.J, sh, sh + n, sh + 2 * n, sh + 3 * n,
                                                                  sh + 4 * n, sh + 5 * n, sh + 6 * n);
    }
    cf_flux_args_f fa;
    for (int v = 0; v < 5; v++) fa.U[v] = sh + v * n;
    fa.J = sh + 5 * n;
    fa.wz[0] = sh + 6 * n;
    fa.wz[1] = nullptr;
    fa.Jf = a.Jf;
    for (int v = 0; v < 9; v++) fa.m[v] = a.m[v];
    fa.Jf32 = met32 ? met32[0] : nullptr;
    for (int v = 0; v < 9; v++) fa.m32[v] = met32 ? met32[1 + v] : nullptr;
    fa.Ep = a.Ep;
    for (int v = 0; v < 5; v++) fa.F[v] = a.F[v];
    fa.f32_out = a.f32_out;
    cf_box b = flux_box(d, dir);
    if (b.ni == 0 || b.nj == 0 || b.nk == 0) return cudaGetLastError();
    dim3 g = box_grid(b), t = box_block();
    if (dir == 2)
        return limited ? launch_flux_z<true, float>(d, fa, b, s) : launch_flux_z<false, float>(d, fa, b, s);
    if (dir == 0) {
        const int chunk = flux_x_chunk(b);
        const dim3 gx = dim3(g.x, g.y, (unsigned)((b.ni + chunk - 1) / chunk));
        if (limited) k_flux_x_march<true><<<gx, t, 0, s>>>(d, fa, b, chunk);
        else k_flux_x_march<false><<<gx, t, 0, s>>>(d, fa, b, chunk);
        return cudaGetLastError();
    }
    if (limited) k_flux<1, true, float, cf_flux_args_f><<<g, t, 0, s>>>(d, fa, b);
    else k_flux<1, false, float, cf_flux_args_f><<<g, t, 0, s>>>(d, fa, b);
    return cudaGetLastError();
}
#endif

}  // namespace CF_NS
