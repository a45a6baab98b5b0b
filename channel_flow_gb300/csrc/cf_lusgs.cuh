// Dual-time LU-SGS: hyperplane Gauss-Seidel (Dual_time_stepping.cpp) and
// the data-parallel Jacobi variant (DPLUSGS.cpp).
//
// Plane m of the hyperplane sweep holds the cells with i + j + k = m; every
// cell of a plane depends only on cells of the previous plane, so one
// launch per plane processes it in parallel and the result equals the
// reference's plane-ordered loop.  Cells come from the reference's own
// plane tables (Hyperplane.cpp), uploaded once per context.
#pragma once
#include "cf_common.cuh"


namespace CF_NS {

template <typename T>
struct lstate {
    T rho, u, v, w, VV, P, C, Tt, H, beta;
    T irho;      // 1/rho (contracted builds)
};

// Dual_time_stepping.cpp:344-363
template <typename T>
__device__ __forceinline__ lstate<T> lu_state(const cf_dims &d, const cf_lu_args &a, size_t q)
{
    lstate<T> s;
    const T K = CF_DC(T, d, K);
    // FP32 build: the step driver's FP32 copies of U_ and J when it has
    // them (the same values as converting here, without the conversions)
    const bool cp = sizeof(T) == 4 && (cf_step_layout || a.U32[0]);
    T u[5], Jq;
#pragma unroll
    for (int n = 0; n < 5; n++) u[n] = cp ? T(a.U32[n][q]) : T(a.U_[n][q]);
    Jq = cp ? T(a.J32[q]) : T(a.J[q]);
    const T u1 = u[0];
    s.rho = u1 * Jq;
#ifdef CF_FAST_MATH
    // three reciprocals instead of seven divisions
    const T iu1 = frcp<T>(u1), irho = frcp<T>(s.rho);
    s.irho = irho;
    const T ikm1 = sizeof(T) == 8 ? T(d.ikm1) : T(1) / (K - T(1));
    s.u = u[1] * iu1;
    s.v = u[2] * iu1;
    s.w = u[3] * iu1;
    s.VV = s.u * s.u + s.v * s.v + s.w * s.w;
    s.P = (u[4] * Jq - T(0.5) * s.rho * s.VV) * (K - T(1));
    s.C = K * s.P * irho;
    s.Tt = s.P * irho;
    s.H = T(0.5) * s.VV + s.C * ikm1;
    s.beta = rmax(s.VV * frcp<T>(s.C), CF_DC(T, d, e));
#else
    s.irho = T(0);
    s.u = u[1] / u1;
    s.v = u[2] / u1;
    s.w = u[3] / u1;
    s.VV = s.u * s.u + s.v * s.v + s.w * s.w;
    s.P = (u[4] * Jq - T(0.5) * s.rho * s.VV) * (K - T(1));
    s.C = K * s.P / s.rho;
    s.Tt = s.P / s.rho;
    s.H = T(0.5) * s.VV + s.C / (K - T(1));
    s.beta = rmax(s.VV / s.C, CF_DC(T, d, e));
#endif
    return s;
}

// split Jacobian of one neighbour cell along metric row m0..m2
// (Dual_time_stepping.cpp:619-651 x, 669-700 y/z; entries 52-54 associate
// differently in x than in y and z, kept as written)
template <typename T>
struct lsplit {
    T p11, p12, p13, p14, p21, p22, p31, p33, p41, p44, p51, p52, p53, p54, p55, m11, m22;
};
template <typename T>
__device__ __forceinline__ lsplit<T> lu_split(lstate<T> s, T m0, T m1, T m2, bool xform, T K)
{
    lsplit<T> A;
    T U = m0 * s.u + m1 * s.v + m2 * s.w;
    T S = sqrt(U * U * (s.beta - T(1)) * (s.beta - T(1)) + T(4) * s.beta * s.C * (m0 * m0 + m1 * m1 + m2 * m2));
    T lambda = ((s.beta + T(1)) * fabs(U) + S) / T(2);
    T dd = fabs(lambda);
    A.p11 = T(0.5) * (s.beta * U + dd);
    A.p12 = T(0.5) * s.P * K * s.beta * m0;
    A.p13 = T(0.5) * s.P * K * s.beta * m1;
    A.p14 = T(0.5) * s.P * K * s.beta * m2;
#ifdef CF_FAST_MATH
    A.p21 = T(0.5) * m0 * s.irho;
    A.p22 = T(0.5) * (U + dd);
    A.p31 = T(0.5) * m1 * s.irho;
    A.p33 = A.p22;
    A.p41 = T(0.5) * m2 * s.irho;
    A.p44 = A.p22;
    A.p51 = T(0.5) * U * (K - T(1)) * (s.beta - T(1)) * s.irho * frcp<T>(K);
#else
    A.p21 = T(0.5) * m0 / s.rho;
    A.p22 = T(0.5) * (U + dd);
    A.p31 = T(0.5) * m1 / s.rho;
    A.p33 = A.p22;
    A.p41 = T(0.5) * m2 / s.rho;
    A.p44 = A.p22;
    A.p51 = T(0.5) * U * (K - T(1)) * (s.beta - T(1)) / s.rho / K;
#endif
    if (xform) {
        A.p52 = T(0.5) * m0 * s.beta * s.Tt * (K - T(1));
        A.p53 = T(0.5) * m1 * s.beta * s.Tt * (K - T(1));
        A.p54 = T(0.5) * m2 * s.beta * s.Tt * (K - T(1));
    } else {
        A.p52 = T(0.5) * s.beta * s.Tt * (K - T(1)) * m0;
        A.p53 = T(0.5) * s.beta * s.Tt * (K - T(1)) * m1;
        A.p54 = T(0.5) * s.beta * s.Tt * (K - T(1)) * m2;
    }
    A.p55 = A.p22;
    A.m11 = T(0.5) * (s.beta * U - dd);
    A.m22 = T(0.5) * (U - dd);
    return A;
}

template <typename T>
struct ldiag {
    T d11, d22, d51;
};
// Dual_time_stepping.cpp:447-489
template <typename T>
__device__ __forceinline__ ldiag<T> lu_diag(const cf_dims &d, const cf_lu_args &a, size_t q, lstate<T> s,
                                            T deltaT)
{
    const T K = CF_DC(T, d, K);
    T xix = met_ld<T>(a.m[0], a.m32[0], q), xiy = met_ld<T>(a.m[1], a.m32[1], q), xiz = met_ld<T>(a.m[2], a.m32[2], q);
    T etx = met_ld<T>(a.m[3], a.m32[3], q), ety = met_ld<T>(a.m[4], a.m32[4], q), etz = met_ld<T>(a.m[5], a.m32[5], q);
    T ztx = met_ld<T>(a.m[6], a.m32[6], q), zty = met_ld<T>(a.m[7], a.m32[7], q), ztz = met_ld<T>(a.m[8], a.m32[8], q);
    T beta = s.beta, C = s.C;
    T U = xix * s.u + xiy * s.v + xiz * s.w;
    T V = etx * s.u + ety * s.v + etz * s.w;
    T W = ztx * s.u + zty * s.v + ztz * s.w;
    T Sx = sqrt(U * U * (beta - T(1)) * (beta - T(1)) + T(4) * beta * C * (xix * xix + xiy * xiy + xiz * xiz));
    T Sy = sqrt(V * V * (beta - T(1)) * (beta - T(1)) + T(4) * beta * C * (etx * etx + ety * ety + etz * etz));
    T Sz = sqrt(W * W * (beta - T(1)) * (beta - T(1)) + T(4) * beta * C * (ztx * ztx + zty * zty + ztz * ztz));
    T lambdaX = ((beta + T(1)) * fabs(U) + Sx) / T(2);
    T lambdaY = ((beta + T(1)) * fabs(V) + Sy) / T(2);
    T lambdaZ = ((beta + T(1)) * fabs(W) + Sz) / T(2);
    ldiag<T> g;
#ifdef CF_FAST_MATH
    T lambda = lambdaX * CF_DINV(T, d, dXI, idXI) + lambdaY * CF_DINV(T, d, dET, idET) +
               lambdaZ * CF_DINV(T, d, dZT, idZT);
    g.d11 = T(2) * deltaT * frcp<T>(T(3) * beta + T(2) * lambda * deltaT);
    g.d22 = T(2) * deltaT * frcp<T>(T(3) + T(2) * lambda * deltaT);
    T temp1 = T(6) * (K - T(1)) * (beta - T(1)) * deltaT;
    T temp2 = K * (T(3) + T(2) * lambda * deltaT) * (T(3) * beta + T(2) * lambda * deltaT) * s.rho;
    g.d51 = -temp1 * frcp<T>(temp2);
#else
    T lambda = lambdaX / CF_DC(T, d, dXI) + lambdaY / CF_DC(T, d, dET) + lambdaZ / CF_DC(T, d, dZT);
    g.d11 = T(2) * deltaT / (T(3) * beta + T(2) * lambda * deltaT);
    g.d22 = T(2) * deltaT / (T(3) + T(2) * lambda * deltaT);
    T temp1 = T(6) * (K - T(1)) * (beta - T(1)) * deltaT;
    T temp2 = K * (T(3) + T(2) * lambda * deltaT) * (T(3) * beta + T(2) * lambda * deltaT) * s.rho;
    g.d51 = -temp1 / temp2;
#endif
    return g;
}

// NL/NR ghost shell = 0 (Dual_time_stepping.cpp:195-316)
__global__ void k_lu_zero(cf_dims d, cf_lu_args a, size_t n)
{
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const size_t plane = d.plane();
    const int i = (int)(q / plane);
    const size_t r = q - (size_t)i * plane;
    const int j = (int)(r / (size_t)d.Zm);
    const int k = (int)(r - (size_t)j * (size_t)d.Zm);
    const int nyy = d.ny + 1, nzz = d.nz + 1;
    const bool xpl = (i == 2 || i == d.gend + 1) && j >= 1 && j <= nyy && k >= 1 && k <= nzz;
    const bool in_x = i >= 2 && i <= d.gend + 1;
    const bool yrow = in_x && (j == 1 || j == nyy) && k >= 1 && k <= nzz;
    const bool zcol = in_x && (k == 1 || k == nzz) && j >= 1 && j <= nyy;
    if (!(xpl || yrow || zcol)) return;
#pragma unroll
    for (int v = 0; v < 5; v++) {
        a.NL[v][q] = 0;
        a.NR[v][q] = 0;
    }
}

// BDF2 residual R and MR = Gamma^-1 R of cell (i, j, k) at q, from its
// state s (Dual_time_stepping.cpp:339-490)
template <typename T>
__device__ __forceinline__ void lu_mr(const cf_dims &d, const cf_lu_args &a, int i, int j, int k, size_t q,
                                      T dt, const lstate<T> &s, T *MR)
{
    const T K = CF_DC(T, d, K);
    T rho = s.rho, u = s.u, v = s.v, w = s.w, VV = s.VV, Tt = s.Tt, H = s.H, beta = s.beta;
    T temp = rho * K;
    T d11 = -(H * (K - T(1)) + VV - K * (Tt + VV)) * beta;
    T d12 = -(K - T(1)) * u * beta;
    T d13 = -(K - T(1)) * v * beta;
    T d14 = -(K - T(1)) * w * beta;
    T d15 = (K - T(1)) * beta;
#ifdef CF_FAST_MATH
    // reciprocals of rho, K rho, J and the spacings instead of 26 divisions
    const T irho = frcp<T>(rho), itemp = frcp<T>(temp);
#define CF_LDIV(x, y, iy) ((x) * (iy))
#else
#define CF_LDIV(x, y, iy) ((x) / (y))
#endif
    T d21 = CF_LDIV(-u, rho, irho), d22 = CF_LDIV(T(1), rho, irho);
    T d31 = CF_LDIV(-v, rho, irho);
    T d41 = CF_LDIV(-w, rho, irho);
    T d51 = CF_LDIV((K - T(1)) * (VV + K * Tt * beta + (K - T(1)) * VV * beta + H * (T(-1) + beta - K * beta)), temp, itemp);
    T d52 = CF_LDIV(-(K - T(1)) * u * (T(1) + (K - T(1)) * beta), temp, itemp);
    T d53 = CF_LDIV(-(K - T(1)) * v * (T(1) + (K - T(1)) * beta), temp, itemp);
    T d54 = CF_LDIV(-(K - T(1)) * w * (T(1) + (K - T(1)) * beta), temp, itemp);
    T d55 = CF_LDIV((K - T(1)) * (T(1) + (K - T(1)) * beta), temp, itemp);
    const size_t fx = d.ix(i, j - 1, k - 1), f0 = d.ix(i - 1, j - 1, k - 1);
    const size_t fy = d.ix(i - 1, j, k - 1), fz = d.ix(i - 1, j - 1, k);
    const T dXI = CF_DC(T, d, dXI), dET = CF_DC(T, d, dET), dZT = CF_DC(T, d, dZT);
#ifdef CF_FAST_MATH
    const T iXI = CF_DINV(T, d, dXI, idXI), iET = CF_DINV(T, d, dET, idET), iZT = CF_DINV(T, d, dZT, idZT);
#endif
    T Rk[5];
#ifdef CF_FAST_MATH
    const double rdt2 = sizeof(T) == 4 ? 0.0 : 0.5 / dt;   // one FP64 division per cell instead of five
#endif
#pragma unroll
    for (int n = 0; n < 5; n++) {
        // the BDF2 time term combines three nearly equal FP64 states: their
        // differences are formed in FP64 in every build (the reference's
        // expression when T is double) before any rounding to FP32, so an
        // FP32 build keeps the digits that the difference resolves
#ifdef CF_FAST_MATH
        T Rp;
        if (sizeof(T) == 4) {
            // FP32 build: 3 U_ - 4 U + Uq = 3 (U_ - U) - (U - Uq), the two
            // differences formed in FP64 (nearly equal states: exact) and
            // combined in FP32; U - Uq is fixed over a physical step, the
            // step driver keeps it in FP32
            const float d1 = float(a.U_[n][q] - a.U[n][q]);
            const float d2 = (cf_step_layout || a.dUq32[0]) ? a.dUq32[n][q] : float(a.U[n][q] - a.Uq[n][q]);
            Rp = T(-(3.0f * d1 - d2) * (0.5f / float(dt)));   // dt is FP32 here
        } else {
            Rp = T(-(3.0 * a.U_[n][q] - 4.0 * a.U[n][q] + a.Uq[n][q]) * rdt2);
        }
#else
        T Rp = T(-(3.0 * a.U_[n][q] - 4.0 * a.U[n][q] + a.Uq[n][q]) / (2.0 * dt));
#endif
        const int f32 = a.f32_rhs;
        T Rf = -(CF_LDIV(rhs_get<T>(a.Fx[n], fx, f32) - rhs_get<T>(a.Fx[n], f0, f32), dXI, iXI) +
                 CF_LDIV(rhs_get<T>(a.Fy[n], fy, f32) - rhs_get<T>(a.Fy[n], f0, f32), dET, iET) +
                 CF_LDIV(rhs_get<T>(a.Fz[n], fz, f32) - rhs_get<T>(a.Fz[n], f0, f32), dZT, iZT));
        Rk[n] = Rp + Rf;
    }
    const T f = CF_DC(T, d, f), Jq = (sizeof(T) == 4 && (cf_step_layout || a.J32)) ? T(a.J32[q]) : T(a.J[q]);
#ifdef CF_FAST_MATH
    const T iJq = frcp<T>(Jq);
#endif
    Rk[1] = Rk[1] + rhs_get<T>(a.vF[0], q, a.f32_rhs) + CF_LDIV(f, Jq, iJq);
    Rk[2] = Rk[2] + rhs_get<T>(a.vF[1], q, a.f32_rhs);
    Rk[3] = Rk[3] + rhs_get<T>(a.vF[2], q, a.f32_rhs);
    Rk[4] = Rk[4] + rhs_get<T>(a.vF[3], q, a.f32_rhs) + CF_LDIV(f * u, Jq, iJq);
#undef CF_LDIV
    MR[0] = (d11 * Rk[0] + d12 * Rk[1] + d13 * Rk[2] + d14 * Rk[3] + d15 * Rk[4]);
    MR[1] = (d21 * Rk[0] + d22 * Rk[1]);
    MR[2] = (d31 * Rk[0] + d22 * Rk[2]);
    MR[3] = (d41 * Rk[0] + d22 * Rk[3]);
    MR[4] = (d51 * Rk[0] + d52 * Rk[1] + d53 * Rk[2] + d54 * Rk[3] + d55 * Rk[4]);
}

// BDF2 residual, Gamma^-1 R and the diagonal solve (Dual_time_stepping.cpp:339-506)
template <typename T>
__global__ void __launch_bounds__(256) k_lu_assemble(cf_dims d, cf_lu_args a, cf_box b, T dt, int copy_nr)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
    const T deltaT = dt;
    lstate<T> s = lu_state<T>(d, a, q);
    T MR[5];
    lu_mr<T>(d, a, i, j, k, q, dt, s, MR);
    const int f32 = a.f32_lu;
#pragma unroll
    for (int n = 0; n < 5; n++) rhs_put<T>(a.MR[n], q, MR[n], f32);
    // the FP32 step driver's sweeps overwrite N at every interior cell, so
    // its build forms no initial NL, NR
    if (sizeof(T) == 4 && cf_step_layout) return;
    ldiag<T> g = lu_diag<T>(d, a, q, s, deltaT);
    T nl[5] = {g.d11 * MR[0], g.d22 * MR[1], g.d22 * MR[2], g.d22 * MR[3], g.d51 * MR[0] + g.d22 * MR[4]};
#pragma unroll
    for (int n = 0; n < 5; n++) {
        rhs_put<T>(a.NL[n], q, nl[n], f32);
        if (copy_nr) rhs_put<T>(a.NR[n], q, nl[n], f32);
    }
}

// x / den of the sweep sums: the division itself in the no-FMA build,
// a multiplication by the reciprocal in the contracted and FP32 builds
template <typename T>
struct lu_den {
    T den, rden;
    __device__ __forceinline__ explicit lu_den(T d) : den(d), rden(T(1) / d) {}
};
template <typename T>
__device__ __forceinline__ T lu_div(T x, const lu_den<T> &d)
{
#ifdef CF_FAST_MATH
    return x * d.rden;
#else
    return x / d.den;
#endif
}

// L*N from the split Jacobians A, B, C of cells i-1, j-1, k-1 and their
// N values a, b, c (Dual_time_stepping.cpp:751-811)
template <typename T>
__device__ __forceinline__ void lu_lower_sum(const lsplit<T> &A, const lsplit<T> &B, const lsplit<T> &C,
                                             const T *a, const T *b, const T *c, T dXI_, T dET_, T dZT_, T *LL)
{
    const lu_den<T> dXI(dXI_), dET(dET_), dZT(dZT_);
    LL[0] = lu_div(-A.p11 * a[0] - A.p12 * a[1] - A.p13 * a[2] - A.p14 * a[3], dXI) +
            lu_div(-B.p11 * b[0] - B.p12 * b[1] - B.p13 * b[2] - B.p14 * b[3], dET) +
            lu_div(-C.p11 * c[0] - C.p12 * c[1] - C.p13 * c[2] - C.p14 * c[3], dZT);
    LL[1] = lu_div(-A.p21 * a[0] - A.p22 * a[1], dXI) + lu_div(-B.p21 * b[0] - B.p22 * b[1], dET) +
            lu_div(-C.p21 * c[0] - C.p22 * c[1], dZT);
    LL[2] = lu_div(-A.p31 * a[0] - A.p33 * a[2], dXI) + lu_div(-B.p31 * b[0] - B.p33 * b[2], dET) +
            lu_div(-C.p31 * c[0] - C.p33 * c[2], dZT);
    LL[3] = lu_div(-A.p41 * a[0] - A.p44 * a[3], dXI) + lu_div(-B.p41 * b[0] - B.p44 * b[3], dET) +
            lu_div(-C.p41 * c[0] - C.p44 * c[3], dZT);
    LL[4] = lu_div(-A.p51 * a[0] - A.p52 * a[1] - A.p53 * a[2] - A.p54 * a[3] - A.p55 * a[4], dXI) +
            lu_div(-B.p51 * b[0] - B.p52 * b[1] - B.p53 * b[2] - B.p54 * b[3] - B.p55 * b[4], dET) +
            lu_div(-C.p51 * c[0] - C.p52 * c[1] - C.p53 * c[2] - C.p54 * c[3] - C.p55 * c[4], dZT);
}

// U*N from the split Jacobians of cells i+1, j+1, k+1 (Dual_time_stepping.cpp:1116-1177)
template <typename T>
__device__ __forceinline__ void lu_upper_sum(const lsplit<T> &A, const lsplit<T> &B, const lsplit<T> &C,
                                             const T *a, const T *b, const T *c, T dXI_, T dET_, T dZT_, T *UU)
{
    const lu_den<T> dXI(dXI_), dET(dET_), dZT(dZT_);
    UU[0] = lu_div(+A.m11 * a[0] + A.p12 * a[1] + A.p13 * a[2] + A.p14 * a[3], dXI) +
            lu_div(+B.m11 * b[0] + B.p12 * b[1] + B.p13 * b[2] + B.p14 * b[3], dET) +
            lu_div(+C.m11 * c[0] + C.p12 * c[1] + C.p13 * c[2] + C.p14 * c[3], dZT);
    UU[1] = lu_div(+A.p21 * a[0] + A.m22 * a[1], dXI) + lu_div(+B.p21 * b[0] + B.m22 * b[1], dET) +
            lu_div(+C.p21 * c[0] + C.m22 * c[1], dZT);
    UU[2] = lu_div(+A.p31 * a[0] + A.m22 * a[2], dXI) + lu_div(+B.p31 * b[0] + B.m22 * b[2], dET) +
            lu_div(+C.p31 * c[0] + C.m22 * c[2], dZT);
    UU[3] = lu_div(+A.p41 * a[0] + A.m22 * a[3], dXI) + lu_div(+B.p41 * b[0] + B.m22 * b[3], dET) +
            lu_div(+C.p41 * c[0] + C.m22 * c[3], dZT);
    UU[4] = lu_div(+A.p51 * a[0] + A.p52 * a[1] + A.p53 * a[2] + A.p54 * a[3] + A.m22 * a[4], dXI) +
            lu_div(+B.p51 * b[0] + B.p52 * b[1] + B.p53 * b[2] + B.p54 * b[3] + B.m22 * b[4], dET) +
            lu_div(+C.p51 * c[0] + C.p52 * c[1] + C.p53 * c[2] + C.p54 * c[3] + C.m22 * c[4], dZT);
}

template <typename T>
__device__ __forceinline__ void lu_load5(double *const *N, size_t q, T *v)
{
#pragma unroll
    for (int n = 0; n < 5; n++) v[n] = T(N[n][q]);
}

// L*N with the splits formed from the neighbours' states
template <typename T>
__device__ __forceinline__ void lu_lower(const cf_dims &d, const cf_lu_args &a, double *const *N, int i, int j,
                                         int k, T *LL)
{
    const T K = CF_DC(T, d, K);
    const size_t qa = d.ix(i - 1, j, k), qb = d.ix(i, j - 1, k), qc = d.ix(i, j, k - 1);
    lsplit<T> A = lu_split<T>(lu_state<T>(d, a, qa), met_ld<T>(a.m[0], a.m32[0], qa), met_ld<T>(a.m[1], a.m32[1], qa), met_ld<T>(a.m[2], a.m32[2], qa), true, K);
    lsplit<T> B = lu_split<T>(lu_state<T>(d, a, qb), met_ld<T>(a.m[3], a.m32[3], qb), met_ld<T>(a.m[4], a.m32[4], qb), met_ld<T>(a.m[5], a.m32[5], qb), false, K);
    lsplit<T> C = lu_split<T>(lu_state<T>(d, a, qc), met_ld<T>(a.m[6], a.m32[6], qc), met_ld<T>(a.m[7], a.m32[7], qc), met_ld<T>(a.m[8], a.m32[8], qc), false, K);
    T va[5], vb[5], vc[5];
    lu_load5<T>(N, qa, va);
    lu_load5<T>(N, qb, vb);
    lu_load5<T>(N, qc, vc);
    lu_lower_sum<T>(A, B, C, va, vb, vc, CF_DC(T, d, dXI), CF_DC(T, d, dET), CF_DC(T, d, dZT), LL);
}

// U*N with the splits formed from the neighbours' states
template <typename T>
__device__ __forceinline__ void lu_upper(const cf_dims &d, const cf_lu_args &a, double *const *N, int i, int j,
                                         int k, T *UU)
{
    const T K = CF_DC(T, d, K);
    const size_t qa = d.ix(i + 1, j, k), qb = d.ix(i, j + 1, k), qc = d.ix(i, j, k + 1);
    lsplit<T> A = lu_split<T>(lu_state<T>(d, a, qa), met_ld<T>(a.m[0], a.m32[0], qa), met_ld<T>(a.m[1], a.m32[1], qa), met_ld<T>(a.m[2], a.m32[2], qa), true, K);
    lsplit<T> B = lu_split<T>(lu_state<T>(d, a, qb), met_ld<T>(a.m[3], a.m32[3], qb), met_ld<T>(a.m[4], a.m32[4], qb), met_ld<T>(a.m[5], a.m32[5], qb), false, K);
    lsplit<T> C = lu_split<T>(lu_state<T>(d, a, qc), met_ld<T>(a.m[6], a.m32[6], qc), met_ld<T>(a.m[7], a.m32[7], qc), met_ld<T>(a.m[8], a.m32[8], qc), false, K);
    T va[5], vb[5], vc[5];
    lu_load5<T>(N, qa, va);
    lu_load5<T>(N, qb, vb);
    lu_load5<T>(N, qc, vc);
    lu_upper_sum<T>(A, B, C, va, vb, vc, CF_DC(T, d, dXI), CF_DC(T, d, dET), CF_DC(T, d, dZT), UU);
}

// ---------------------------------------------------------------------------
// coefficient pack of the hyperplane sweeps
// ---------------------------------------------------------------------------
// The split Jacobians and the diagonal inverse of a cell depend only on its
// own state and metrics, which the sweeps do not change.  k_lu_pack forms
// them once per call for every cell and its ghost neighbours, so a plane
// step only gathers them.  Per cell LU_PACK doubles: for x, y, z (16 each)
// p11 p22 m11 m22 p12 p13 p14 p21 p31 p41 p51 p52 p53 p54 (2 unused), then
// d11 d22 d51 (1 unused).  Same expressions as the unpacked path, so the
// values are the same bits.
constexpr int LU_PACK = 52;

template <typename T>
__global__ void __launch_bounds__(256) k_lu_pack(cf_dims d, cf_lu_args a, double *__restrict__ pack, cf_box b,
                                                 double dt)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
    const T K = CF_DC(T, d, K);
    const lstate<T> s = lu_state<T>(d, a, q);
    double *P = pack + q * LU_PACK;
#pragma unroll
    for (int dir = 0; dir < 3; dir++) {
        const lsplit<T> A = lu_split<T>(s, met_ld<T>(a.m[3 * dir], a.m32[3 * dir], q), met_ld<T>(a.m[3 * dir + 1], a.m32[3 * dir + 1], q), met_ld<T>(a.m[3 * dir + 2], a.m32[3 * dir + 2], q),
                                        dir == 0, K);
        double2 *o = reinterpret_cast<double2 *>(P + 16 * dir);
        o[0] = make_double2(double(A.p11), double(A.p22));
        o[1] = make_double2(double(A.m11), double(A.m22));
        o[2] = make_double2(double(A.p12), double(A.p13));
        o[3] = make_double2(double(A.p14), double(A.p21));
        o[4] = make_double2(double(A.p31), double(A.p41));
        o[5] = make_double2(double(A.p51), double(A.p52));
        o[6] = make_double2(double(A.p53), double(A.p54));
    }
    const ldiag<T> g = lu_diag<T>(d, a, q, s, T(dt));
    double2 *o = reinterpret_cast<double2 *>(P + 48);
    o[0] = make_double2(double(g.d11), double(g.d22));
    o[1] = make_double2(double(g.d51), 0.0);
}

// split of one direction from the pack; UPPER selects m11/m22 in place of p11/p22
template <typename T, bool UPPER>
__device__ __forceinline__ lsplit<T> lu_unpack(const double *__restrict__ P)
{
    const double2 *v = reinterpret_cast<const double2 *>(P);
    lsplit<T> A;
    const double2 d0 = UPPER ? v[1] : v[0], d2 = v[2], d3 = v[3], d4 = v[4], d5 = v[5], d6 = v[6];
    if (UPPER) {
        A.m11 = T(d0.x); A.m22 = T(d0.y);
    } else {
        A.p11 = T(d0.x); A.p22 = T(d0.y);
        A.p33 = A.p22; A.p44 = A.p22; A.p55 = A.p22;
    }
    A.p12 = T(d2.x); A.p13 = T(d2.y); A.p14 = T(d3.x); A.p21 = T(d3.y);
    A.p31 = T(d4.x); A.p41 = T(d4.y); A.p51 = T(d5.x); A.p52 = T(d5.y);
    A.p53 = T(d6.x); A.p54 = T(d6.y);
    return A;
}

template <typename T>
__device__ __forceinline__ ldiag<T> lu_unpack_diag(const double *__restrict__ P)
{
    const double2 *v = reinterpret_cast<const double2 *>(P + 48);
    const double2 a0 = v[0], a1 = v[1];
    ldiag<T> g;
    g.d11 = T(a0.x); g.d22 = T(a0.y); g.d51 = T(a1.x);
    return g;
}

// forward plane from the pack: NL = D^-1 (MR - L NL)
template <typename T>
__global__ void k_lu_forward_packed(cf_dims d, cf_lu_args a, const double *__restrict__ pack,
                                    const int *__restrict__ ijk, int first, int count)
{
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= count) return;
    const int *c = ijk + 3 * (size_t)(first + t);
    const size_t q = d.ix(c[0], c[1], c[2]);
    const size_t qa = q - d.plane(), qb = q - (size_t)d.Zm, qc = q - 1;
    const lsplit<T> A = lu_unpack<T, false>(pack + qa * LU_PACK);
    const lsplit<T> B = lu_unpack<T, false>(pack + qb * LU_PACK + 16);
    const lsplit<T> C = lu_unpack<T, false>(pack + qc * LU_PACK + 32);
    const ldiag<T> g = lu_unpack_diag<T>(pack + q * LU_PACK);
    T va[5], vb[5], vc[5], LL[5];
    lu_load5<T>(a.NL, qa, va);
    lu_load5<T>(a.NL, qb, vb);
    lu_load5<T>(a.NL, qc, vc);
    lu_lower_sum<T>(A, B, C, va, vb, vc, CF_DC(T, d, dXI), CF_DC(T, d, dET), CF_DC(T, d, dZT), LL);
    T r0 = T(a.MR[0][q]) - LL[0];
    a.NL[0][q] = double(g.d11 * r0);
    a.NL[1][q] = double(g.d22 * (T(a.MR[1][q]) - LL[1]));
    a.NL[2][q] = double(g.d22 * (T(a.MR[2][q]) - LL[2]));
    a.NL[3][q] = double(g.d22 * (T(a.MR[3][q]) - LL[3]));
    a.NL[4][q] = double(g.d51 * r0 + g.d22 * (T(a.MR[4][q]) - LL[4]));
}

// backward plane from the pack: NR = NL - D^-1 U NR
template <typename T>
__global__ void k_lu_backward_packed(cf_dims d, cf_lu_args a, const double *__restrict__ pack,
                                     const int *__restrict__ ijk, int first, int count)
{
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= count) return;
    const int *c = ijk + 3 * (size_t)(first + t);
    const size_t q = d.ix(c[0], c[1], c[2]);
    const size_t qa = q + d.plane(), qb = q + (size_t)d.Zm, qc = q + 1;
    const lsplit<T> A = lu_unpack<T, true>(pack + qa * LU_PACK);
    const lsplit<T> B = lu_unpack<T, true>(pack + qb * LU_PACK + 16);
    const lsplit<T> C = lu_unpack<T, true>(pack + qc * LU_PACK + 32);
    const ldiag<T> g = lu_unpack_diag<T>(pack + q * LU_PACK);
    T va[5], vb[5], vc[5], UU[5];
    lu_load5<T>(a.NR, qa, va);
    lu_load5<T>(a.NR, qb, vb);
    lu_load5<T>(a.NR, qc, vc);
    lu_upper_sum<T>(A, B, C, va, vb, vc, CF_DC(T, d, dXI), CF_DC(T, d, dET), CF_DC(T, d, dZT), UU);
    a.NR[0][q] = double(T(a.NL[0][q]) - g.d11 * UU[0]);
    a.NR[1][q] = double(T(a.NL[1][q]) - g.d22 * UU[1]);
    a.NR[2][q] = double(T(a.NL[2][q]) - g.d22 * UU[2]);
    a.NR[3][q] = double(T(a.NL[3][q]) - g.d22 * UU[3]);
    a.NR[4][q] = double(T(a.NL[4][q]) - (g.d51 * UU[0] + g.d22 * UU[4]));
}

// forward plane: NL = D^-1 (MR - L NL) (Dual_time_stepping.cpp:594-877)
template <typename T>
__global__ void k_lu_forward(cf_dims d, cf_lu_args a, const int *__restrict__ ijk, int first, int count, double dt)
{
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= count) return;
    const int *c = ijk + 3 * (size_t)(first + t);
    const int i = c[0], j = c[1], k = c[2];
    const size_t q = d.ix(i, j, k);
    T LL[5];
    lu_lower<T>(d, a, a.NL, i, j, k, LL);
    ldiag<T> g = lu_diag<T>(d, a, q, lu_state<T>(d, a, q), T(dt));
    T r0 = T(a.MR[0][q]) - LL[0];
    a.NL[0][q] = double(g.d11 * r0);
    a.NL[1][q] = double(g.d22 * (T(a.MR[1][q]) - LL[1]));
    a.NL[2][q] = double(g.d22 * (T(a.MR[2][q]) - LL[2]));
    a.NL[3][q] = double(g.d22 * (T(a.MR[3][q]) - LL[3]));
    a.NL[4][q] = double(g.d51 * r0 + g.d22 * (T(a.MR[4][q]) - LL[4]));
}

// backward plane: NR = NL - D^-1 U NR (Dual_time_stepping.cpp:926-1245)
template <typename T>
__global__ void k_lu_backward(cf_dims d, cf_lu_args a, const int *__restrict__ ijk, int first, int count, double dt)
{
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= count) return;
    const int *c = ijk + 3 * (size_t)(first + t);
    const int i = c[0], j = c[1], k = c[2];
    const size_t q = d.ix(i, j, k);
    T UU[5];
    lu_upper<T>(d, a, a.NR, i, j, k, UU);
    ldiag<T> g = lu_diag<T>(d, a, q, lu_state<T>(d, a, q), T(dt));
    a.NR[0][q] = double(T(a.NL[0][q]) - g.d11 * UU[0]);
    a.NR[1][q] = double(T(a.NL[1][q]) - g.d22 * UU[1]);
    a.NR[2][q] = double(T(a.NL[2][q]) - g.d22 * UU[2]);
    a.NR[3][q] = double(T(a.NL[3][q]) - g.d22 * UU[3]);
    a.NR[4][q] = double(T(a.NL[4][q]) - (g.d51 * UU[0] + g.d22 * UU[4]));
}

// Jacobi sweep: NR = D^-1 (MR - L NL - U NL) (DPLUSGS.cpp:573-1121, with the
// upper neighbours at j+1, k+1)
template <typename T>
__global__ void __launch_bounds__(256) k_lu_jacobi(cf_dims d, cf_lu_args a, cf_box b, double dt)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
    T LL[5], UU[5];
    lu_lower<T>(d, a, a.NL, i, j, k, LL);
    lu_upper<T>(d, a, a.NL, i, j, k, UU);
    ldiag<T> g = lu_diag<T>(d, a, q, lu_state<T>(d, a, q), T(dt));
    T r0 = T(a.MR[0][q]) - LL[0] - UU[0];
    a.NR[0][q] = double(g.d11 * r0);
    a.NR[1][q] = double(g.d22 * (T(a.MR[1][q]) - LL[1] - UU[1]));
    a.NR[2][q] = double(g.d22 * (T(a.MR[2][q]) - LL[2] - UU[2]));
    a.NR[3][q] = double(g.d22 * (T(a.MR[3][q]) - LL[3] - UU[3]));
    a.NR[4][q] = double(g.d51 * r0 + g.d22 * (T(a.MR[4][q]) - LL[4] - UU[4]));
}

// interior copy NL <- NR (Dual_time_stepping.cpp:1261-1274)
__global__ void k_lu_copy(cf_dims d, cf_lu_args a, cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
#pragma unroll
    for (int v = 0; v < 5; v++) a.NL[v][q] = a.NR[v][q];
}

// primitive update of one cell from its NR and the squared changes
// (Dual_time_stepping.cpp:1290-1326), FP64 in every precision mode; r2
// gets the squares of the five squared changes (the terms of the
// reference's Sum(Delta^2)^2 norm)
__device__ __forceinline__ void lu_update_cell(const cf_dims &d, const cf_lu_args &a, size_t q, const double *nr,
                                               double *r2)
{
    const double K = d.K, Jq = a.J[q];
    double rhoold = a.U_[0][q] * Jq;
#ifdef CF_FAST_MATH
    // FP64 with three divisions instead of ten (reciprocals of U1 and J,
    // 1/(K-1) from the host, 1/rho_old = (1/U1)(1/J))
    const double iu1 = frcp<double>(a.U_[0][q]), iJ = frcp<double>(Jq);
    double Uold = a.U_[1][q] * iu1;
    double Vold = a.U_[2][q] * iu1;
    double Wold = a.U_[3][q] * iu1;
#else
    double Uold = a.U_[1][q] / a.U_[0][q];
    double Vold = a.U_[2][q] / a.U_[0][q];
    double Wold = a.U_[3][q] / a.U_[0][q];
#endif
    double VVold = Uold * Uold + Vold * Vold + Wold * Wold;
    double Pold = (a.U_[4][q] * Jq - 0.5 * rhoold * VVold) * (K - 1);
#ifdef CF_FAST_MATH
    double Told = Pold * (iu1 * iJ);
#else
    double Told = Pold / rhoold;
#endif
    double P = Pold + nr[0] * Jq;
    double U = Uold + nr[1] * Jq;
    double V = Vold + nr[2] * Jq;
    double W = Wold + nr[3] * Jq;
    double Tt = Told + nr[4] * Jq;
#ifdef CF_FAST_MATH
    const double rho = P * frcp<double>(Tt);
    const double rJ = rho * iJ;
    a.U_[0][q] = rJ;
    a.U_[1][q] = rJ * U;
    a.U_[2][q] = rJ * V;
    a.U_[3][q] = rJ * W;
    a.U_[4][q] = (P * d.ikm1 + 0.5 * rho * (U * U + V * V + W * W)) * iJ;
#else
    const double rho = P / Tt;
    a.U_[0][q] = rho / Jq;
    a.U_[1][q] = rho * U / Jq;
    a.U_[2][q] = rho * V / Jq;
    a.U_[3][q] = rho * W / Jq;
    a.U_[4][q] = (P / (K - 1) + 0.5 * rho * (U * U + V * V + W * W)) / Jq;
#endif
    double r[5] = {(P - Pold) * (P - Pold), (U - Uold) * (U - Uold), (V - Vold) * (V - Vold),
                   (W - Wold) * (W - Wold), (Tt - Told) * (Tt - Told)};
#pragma unroll
    for (int n = 0; n < 5; n++) {
        a.Res[n][q] = r[n];
        r2[n] = r[n] * r[n];
    }
}

// FP32 build: the change of the cell's state formed in FP32 and added to
// the FP64 state in FP64.  The old primitives p = (P, u, v, w, T) come
// from the state rounded to FP32, their changes dp = NR J from the FP32
// sweeps, and the conserved change g(p + dp) - g(p) is written in products
// of the changes, free of cancellation:
//   drho     = (dP T - P dT) / ((T + dT) T)           (rho = P / T)
//   d(rho u) = drho u + rho' du                       (rho' = rho + drho)
//   d(e)     = dP / (K - 1) + (drho |u|^2 + rho' (du (2u + du) + ...)) / 2
// Its FP32 rounding is relative to the change, which vanishes as the
// sub-iterations converge, so the FP64 state keeps the digits that the
// FP32 sweeps resolve; per cell this is about a third of the FP64
// operations of the FP64 update.  The squared changes and their squares
// (the norm terms) are formed and summed in FP64; acc[n] += Residual^2.
__device__ __forceinline__ void lu_update_cell_f32(const cf_dims &d, const cf_lu_args &a, size_t q, const float *nr,
                                                   double *acc)
{
    double u[5];
    float f[5];
    const bool cp = cf_step_layout || a.U32[0] != nullptr;     // the step driver's FP32 copies of U_ and J
#pragma unroll
    for (int n = 0; n < 5; n++) {
        u[n] = a.U_[n][q];
        f[n] = cp ? a.U32[n][q] : float(u[n]);
    }
    const float Km1 = d.f_K - 1.0f;
    const float J = cp ? a.J32[q] : float(a.J[q]), iJ = 1.0f / J, iu0 = 1.0f / f[0];
    const float rho = f[0] * J;
    const float uo = f[1] * iu0, vo = f[2] * iu0, wo = f[3] * iu0;
    const float VV = uo * uo + vo * vo + wo * wo;
    const float P = (f[4] * J - 0.5f * rho * VV) * Km1;
    const float T = P * (iu0 * iJ);
    const float e[5] = {nr[0] * J, nr[1] * J, nr[2] * J, nr[3] * J, nr[4] * J};
    const float drho = (e[0] * T - P * e[4]) / ((T + e[4]) * T);
    const float rn = rho + drho;
    const float dE = e[0] / Km1 + 0.5f * (drho * VV + rn * (e[1] * (2.0f * uo + e[1]) + e[2] * (2.0f * vo + e[2]) +
                                                          e[3] * (2.0f * wo + e[3])));
    const float dc[5] = {drho, drho * uo + rn * e[1], drho * vo + rn * e[2], drho * wo + rn * e[3], dE};
    // FP32 -> FP64 on the integer pipe (f2d): the FP64 pipe keeps the
    // additions and the norm terms only
#pragma unroll
    for (int n = 0; n < 5; n++) {
        a.U_[n][q] = u[n] + f2d(dc[n] * iJ);
        const double x = f2d(e[n]), r = x * x;
        // the step driver reads no Residual array: only the drop-in writes it
        if (!cf_step_layout) a.Res[n][q] = r;
        acc[n] = fma(r, r, acc[n]);
    }
}

// the update over the interior box (blocks of 32 x 8 cells of a plane,
// grid-stride over the planes: gridDim.z may be smaller than the box); each
// block also writes its partial sums of Residual^2
template <typename T>
__global__ void __launch_bounds__(256) k_lu_update(cf_dims d, cf_lu_args a, cf_box b)
{
    const int k = b.k0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = b.j0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    double r2[5] = {0, 0, 0, 0, 0};
    if (k < b.k0 + b.nk && j < b.j0 + b.nj)
        for (int i = b.i0 + (int)blockIdx.z; i < b.i0 + b.ni; i += (int)gridDim.z) {
            const size_t q = d.ix(i, j, k);
            if (sizeof(T) == 4) {
                // FP32: also NL <- NR here (the arrays may hold FP32 values,
                // which the FP64 copy kernel would pair up wrongly)
                // (the step driver reads neither NL nor Residual afterwards:
                // its build writes neither)
                float nr[5];
#pragma unroll
                for (int n = 0; n < 5; n++) {
                    nr[n] = rhs_get<float>(a.NR[n], q, a.f32_lu);
                    if (!cf_step_layout) rhs_put<float>(a.NL[n], q, nr[n], a.f32_lu);
                }
                lu_update_cell_f32(d, a, q, nr, r2);
            } else {
                double nr[5];
#pragma unroll
                for (int n = 0; n < 5; n++) nr[n] = a.NR[n][q];
                lu_update_cell(d, a, q, nr, r2);
            }
        }
    // block reduction in a fixed order (deterministic): each warp by
    // shuffles, then the eight warp sums by the first warp
    __shared__ double sh[5][8];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int n = 0; n < 5; n++) {
        double v = r2[n];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) sh[n][warp] = v;
    }
    __syncthreads();
    if (warp == 0) {
        const size_t blk = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
#pragma unroll
        for (int n = 0; n < 5; n++) {
            double v = lane < 8 ? sh[n][lane] : 0.0;
#pragma unroll
            for (int off = 4; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
            if (lane == 0) a.partial[5 * blk + n] = v;
        }
    }
}

// final reduction of the block partial sums, one block, fixed order;
// er[n] = sqrt(sum) * DN (Dual_time_stepping.cpp:1348-1352).  Thread t sums
// partials t, t + 256, ... in order, eight of them in flight (coalesced).
__global__ void k_lu_norm(const double *partial, size_t nblk, double DN, double *er)
{
    __shared__ double sh[5][256];
    const int tid = threadIdx.x;
    double s[5] = {0, 0, 0, 0, 0};
    size_t b = tid;
    for (; b + 7 * 256 < nblk; b += 8 * 256) {
        double v[8][5];
#pragma unroll
        for (int m = 0; m < 8; m++)
#pragma unroll
            for (int n = 0; n < 5; n++) v[m][n] = partial[5 * (b + 256 * m) + n];
#pragma unroll
        for (int m = 0; m < 8; m++)
#pragma unroll
            for (int n = 0; n < 5; n++) s[n] += v[m][n];
    }
    for (; b < nblk; b += 256)
#pragma unroll
        for (int n = 0; n < 5; n++) s[n] += partial[5 * b + n];
#pragma unroll
    for (int n = 0; n < 5; n++) sh[n][tid] = s[n];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (tid < w)
#pragma unroll
            for (int n = 0; n < 5; n++) sh[n][tid] += sh[n][tid + w];
        __syncthreads();
    }
    if (tid < 5) er[tid] = sqrt(sh[tid][0]) * DN;
}

}  // namespace CF_NS
