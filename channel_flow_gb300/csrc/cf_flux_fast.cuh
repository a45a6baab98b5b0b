// Reduced-division forms of the face states and face fluxes, used by the
// contracted FP64 build and the FP32 build (CF_FAST_MATH).  Same mathematics
// as cf_flux.cuh, evaluated with fewer divisions, each reciprocal by frcp
// (cf_common.cuh: Newton-refined hardware reciprocal in FP64):
//
// * limited states: every ratio of the MUSCL-5 limiter is a quotient of two
//   neighbouring differences D_k = u_{k+1} - u_k, so the ten states of a
//   face need the reciprocals of three differences per variable instead of
//   eight divisions;
// * the Jacobian weights 1/sum(w/J) share the reciprocals of J of the six
//   stencil cells;
// * the Roe and preconditioned-Roe matrices reuse the reciprocals of rho,
//   C, T, the metric norm, the matrix denominator and the face Jacobian.
//
// Results differ from the reference only by rounding (tests: within 1e-12
// normwise in FP64), except where two neighbouring values tie: the
// reference's ratio is then 0/0 or x/0 and its state NaN; here the
// reciprocal of a zero difference is taken as 0, which gives the limit
// (no slope on that side).  Ties are rare in FP64 but frequent in FP32.
#pragma once
#include "cf_common.cuh"

namespace CF_NS {

// The limiter's comparisons in FP64 on the integer pipe: the contracted
// FP64 build is bound by the FP64 pipe, which would also issue every FP64
// compare.  fkey orders doubles as signed integers (the sign-magnitude bit
// pattern turned two's complement); the order is the floating-point order
// except that -0 < +0 (the limiter then returns -0 for 0, the same state)
// and NaN (which these limiters are not given).  FP32 keeps its compares.
__device__ __forceinline__ long long fkey(double x)
{
    const long long b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
template <typename T>
__device__ __forceinline__ T lmin(T a, T b) { return rmin(a, b); }
template <>
__device__ __forceinline__ double lmin<double>(double a, double b) { return fkey(a) < fkey(b) ? a : b; }
template <typename T>
__device__ __forceinline__ T lmax(T a, T b) { return rmax(a, b); }
template <>
__device__ __forceinline__ double lmax<double>(double a, double b) { return fkey(a) > fkey(b) ? a : b; }
template <typename T>
__device__ __forceinline__ bool nonzero(T D) { return D != T(0); }
template <>
__device__ __forceinline__ bool nonzero<double>(double D) { return (__double_as_longlong(D) << 1) != 0; }

// reciprocal of a neighbour difference, 0 for a tie
template <typename T>
__device__ __forceinline__ T ginv(T D)
{
    return nonzero(D) ? frcp<T>(D) : T(0);
}

// u[0..5] = cells c-2 .. c+3 of the face's stencil line; left state of cell
// c (3rd or 5th order, slope sign S) and right state of cell c+1
// (S = 0: the sign of the left slope term is that of hs = +-0.5, chosen at
// run time)
template <typename T, int S>
__device__ __forceinline__ void fast_pair(const T *u, bool lo3, bool hi3, T jL, T jR, T &mL, T &mR,
                                          T hs = T(0.5))
{
    const T D1 = u[2] - u[1], D2 = u[3] - u[2], D3 = u[4] - u[3];
    const T inv1 = ginv(D1), inv2 = ginv(D2), inv3 = ginv(D3);
    const T rL = D2 * inv1;
    T bL;
    if (lo3) {
        bL = T(1.) / T(3) * (T(1) + T(2) * rL);
    } else {
        const T rLi = (u[4] - u[3]) * inv2;
        bL = T(1.) / T(30) * (T(-2) * (u[1] - u[0]) * inv1 + T(11) + T(24) * rL - T(3) * rL * rLi);
    }
    const T phiL = lmax(T(0), lmin(T(2), lmin(T(2) * rL, bL)));
    mL = (S > 0 ? u[2] + T(0.5) * phiL * D1 : S < 0 ? u[2] - T(0.5) * phiL * D1 : u[2] + hs * phiL * D1) * jL;
    const T rR = D2 * inv3;
    T bR;
    if (hi3) {
        bR = T(1.) / T(3) * (T(1) + T(2) * rR);
    } else {
        const T irR = D1 * inv2;
        bR = T(1.) / T(30) * (T(-2) * (u[5] - u[4]) * inv3 + T(11) + T(24) * rR - T(3) * rR * irR);
    }
    const T phiR = lmax(T(0), lmin(T(2), lmin(T(2) * rR, bR)));
    mR = (u[3] - T(0.5) * phiR * D3) * jR;
}

// left state alone: u[0..4] = cells c-2 .. c+2 (u[0] unused at 3rd order)
template <typename T, int S>
__device__ __forceinline__ T fast_left(const T *u, bool o3, T hs = T(0.5))
{
    const T D1 = u[2] - u[1], D2 = u[3] - u[2];
    const T inv1 = ginv(D1);
    const T rL = D2 * inv1;
    T b;
    if (o3) {
        b = T(1.) / T(3) * (T(1) + T(2) * rL);
    } else {
        const T rLi = (u[4] - u[3]) * ginv(D2);
        b = T(1.) / T(30) * (T(-2) * (u[1] - u[0]) * inv1 + T(11) + T(24) * rL - T(3) * rL * rLi);
    }
    const T phi = lmax(T(0), lmin(T(2), lmin(T(2) * rL, b)));
    return S > 0 ? u[2] + T(0.5) * phi * D1 : S < 0 ? u[2] - T(0.5) * phi * D1 : u[2] + hs * phi * D1;
}

// right state alone: w[0..4] = cells c-2 .. c+2 of the right cell c
// (w[4] unused at 3rd order)
template <typename T>
__device__ __forceinline__ T fast_right(const T *w, bool o3)
{
    const T Dm = w[2] - w[1], Dp = w[3] - w[2];
    const T invp = ginv(Dp);
    const T rR = Dm * invp;
    T b;
    if (o3) {
        b = T(1.) / T(3) * (T(1) + T(2) * rR);
    } else {
        const T irR = (w[1] - w[0]) * ginv(Dm);
        b = T(1.) / T(30) * (T(-2) * (w[4] - w[3]) * invp + T(11) + T(24) * rR - T(3) * rR * irR);
    }
    const T phi = lmax(T(0), lmin(T(2), lmin(T(2) * rR, b)));
    return w[2] - T(0.5) * phi * Dp;
}

template <typename T, typename SP>
__device__ __forceinline__ void load5(const SP *U, size_t qc, ptrdiff_t s, T *u)
{
#pragma unroll
    for (int t = 0; t < 5; t++) u[t] = T(U[qc + (t - 2) * s]);
}

// loads the cells the selected orders need (others stay 0)
template <typename T, typename SP>
__device__ __forceinline__ void load6(const SP *U, size_t qc, ptrdiff_t s, bool lo3, bool hi3, T *u)
{
    u[0] = lo3 ? T(0) : T(U[qc - 2 * s]);
    u[1] = T(U[qc - s]);
    u[2] = T(U[qc]);
    u[3] = T(U[qc + s]);
    u[4] = T(U[qc + 2 * s]);
    u[5] = hi3 ? T(0) : T(U[qc + 3 * s]);
}

template <typename T, typename A>
__device__ __forceinline__ void fast_states_x_limited(const cf_dims &d, const A &a, int i, int j,
                                                      int k, T *mL, T *mR)
{
    const ptrdiff_t s = (ptrdiff_t)d.plane();
    const T jf = fjf<T>(a, d.ix(i, j, k));
    const size_t qc = d.ix(i, j + 1, k + 1);
    const bool lo3 = (i <= 3) || (i >= d.gend);
    const bool hi3 = (i + 1 <= 3) || (i + 1 >= d.gend);
#pragma unroll
    for (int n = 0; n < 5; n++) {
        T u[6];
        load6<T>(a.U[n], qc, s, lo3, hi3, u);
        fast_pair<T, 1>(u, lo3, hi3, jf, jf, mL[n], mR[n]);
    }
}

template <typename T, typename A>
__device__ __forceinline__ void fast_states_y_limited(const cf_dims &d, const A &a, int i, int j,
                                                      int k, T *mL, T *mR)
{
    const ptrdiff_t s = d.Zm;
    const int ny = d.ny;
    const T jf = fjf<T>(a, d.ix(i, j, k));
    const size_t qL = d.ix(i + 1, j, k + 1), qR = qL + s;
    const bool wallL = (j <= 2) || (j >= ny - 1);
    const bool wallR = (j + 1 <= 2) || (j + 1 >= ny - 1);
    if (j != 1 && j != ny && !wallL && !wallR) {
#pragma unroll
        for (int n = 0; n < 5; n++) {
            T u[6];
            load6<T>(a.U[n], qL, s, false, false, u);
            fast_pair<T, 1>(u, false, false, jf, jf, mL[n], mR[n]);
        }
        return;
    }
    // rows next to a wall (Flux_Y_limiter.cpp:115-477): wall averages on
    // faces 1 and ny, the guarded ratio of variable 1 and 3rd order
    if (j == 1) {
        T temp = frcp<T>(frcp<T>(T(a.J[qL])) + frcp<T>(T(a.J[qL + s])));
#pragma unroll
        for (int n = 0; n < 5; n++) mL[n] = temp * (T(a.U[n][qL]) + T(a.U[n][qL + s]));
    } else if (wallL && d.scheme) {
#pragma unroll
        for (int n = 0; n < 5; n++) mL[n] = ywall_q_left<T>(a.U[n], a.J, qL, s, n == 0);
    } else if (wallL) {
        mL[0] = ywall_var1_left<T>(a.U[0], a.J, qL, s);
#pragma unroll
        for (int n = 1; n < 5; n++) {
            T u[5];
            u[0] = T(0);
            u[1] = T(a.U[n][qL - s]); u[2] = T(a.U[n][qL]); u[3] = T(a.U[n][qL + s]); u[4] = T(0);
            mL[n] = fast_left<T, 1>(u, true) * jf;
        }
    } else {
#pragma unroll
        for (int n = 0; n < 5; n++) {
            T u[5];
            load5<T>(a.U[n], qL, s, u);
            mL[n] = fast_left<T, 1>(u, false) * jf;
        }
    }
    if (j == ny) {
        const size_t q = d.ix(i + 1, ny, k + 1);
        T temp = frcp<T>(frcp<T>(T(a.J[q])) + frcp<T>(T(a.J[q + s])));
#pragma unroll
        for (int n = 0; n < 5; n++) mR[n] = temp * (T(a.U[n][q]) + T(a.U[n][q + s]));
    } else if (wallR && d.scheme) {
#pragma unroll
        for (int n = 0; n < 5; n++) mR[n] = ywall_q_right<T>(a.U[n], a.J, qR, s, n == 0);
    } else if (wallR) {
        mR[0] = ywall_var1_right<T>(a.U[0], a.J, qR, s);
#pragma unroll
        for (int n = 1; n < 5; n++) {
            T w[5];
            w[0] = T(0);
            w[1] = T(a.U[n][qR - s]); w[2] = T(a.U[n][qR]); w[3] = T(a.U[n][qR + s]); w[4] = T(0);
            mR[n] = fast_right<T>(w, true) * jf;
        }
    } else {
#pragma unroll
        for (int n = 0; n < 5; n++) {
            T w[5];
            load5<T>(a.U[n], qR, s, w);
            mR[n] = fast_right<T>(w, false) * jf;
        }
    }
}

// INTERIOR: the caller launches faces k = 3..nz-2 only, where both states
// are limited (the edge branches are then not compiled in)
template <typename T, typename A, bool INTERIOR = false>
__device__ __forceinline__ void fast_states_z_limited(const cf_dims &d, const A &a, int i, int j,
                                                      int k, T *mL, T *mR)
{
    const int nz = d.nz, ny = d.ny;
    const size_t qL = d.ix(i + 1, j + 1, k), qR = qL + 1;
    const bool limL = INTERIOR || (k >= 3 && k <= nz - 1);          // cell k takes a limited state
    const bool limR = INTERIOR || (k + 1 >= 3 && k + 1 <= nz - 1);  // cell k+1 takes a limited state
    const bool lo3 = k >= ny, hi3 = k + 1 >= ny;      // the reference compares with the y extent
    const auto *iJp = a.wz[0];      // 1/J per cell
    // CF_SCHEME_CONSISTENT: normalised weights (the sums 60 and 6) and the
    // upwind left slope; the reference's: unnormalised, downwind
    const T w5 = T(d.scheme ? 60 : 1), w3 = T(d.scheme ? 6 : 1), hs = T(d.scheme ? 0.5 : -0.5);
    if (limL && limR) {
        T iJ[6];
        iJ[0] = lo3 ? T(0) : T(iJp[qL - 2]);
        iJ[1] = T(iJp[qL - 1]);
        iJ[2] = T(iJp[qL]);
        iJ[3] = T(iJp[qL + 1]);
        iJ[4] = T(iJp[qL + 2]);
        iJ[5] = hi3 ? T(0) : T(iJp[qL + 3]);
        const T jl = frcp<T>(lo3 ? (T(-1) * iJ[1] + T(5) * iJ[2] + T(2) * iJ[3])
                                 : (T(2) * iJ[0] - T(13) * iJ[1] + T(47) * iJ[2] + T(27) * iJ[3] - T(3) * iJ[4])) *
                     (lo3 ? w3 : w5);
        const T jr = frcp<T>(hi3 ? (T(2) * iJ[2] + T(5) * iJ[3] - T(1) * iJ[4])
                                 : (T(-3) * iJ[1] + T(27) * iJ[2] + T(47) * iJ[3] - T(13) * iJ[4] + T(2) * iJ[5])) *
                     (hi3 ? w3 : w5);
#pragma unroll
        for (int n = 0; n < 5; n++) {
            T u[6];
            load6<T>(a.U[n], qL, 1, lo3, hi3, u);
            fast_pair<T, 0>(u, lo3, hi3, jl, jr, mL[n], mR[n], hs);
        }
        return;
    }
    // left state of face k from cell k (Flux_Z_limiter.cpp:120-330)
    if (k == 1) {
#pragma unroll
        for (int n = 0; n < 5; n++) mL[n] = avg2<T>(a.U[n], a.J, qL, 1);
    } else if (!limL) {
#pragma unroll
        for (int n = 0; n < 5; n++) mL[n] = lin3L<T>(a.U[n], a.J, qL, 1);
    } else {
        const T jl = frcp<T>(lo3 ? (T(-1) * T(iJp[qL - 1]) + T(5) * T(iJp[qL]) + T(2) * T(iJp[qL + 1]))
                                 : (T(2) * T(iJp[qL - 2]) - T(13) * T(iJp[qL - 1]) + T(47) * T(iJp[qL]) +
                                    T(27) * T(iJp[qL + 1]) - T(3) * T(iJp[qL + 2]))) * (lo3 ? w3 : w5);
#pragma unroll
        for (int n = 0; n < 5; n++) {
            T u[5];
            load5<T>(a.U[n], qL, 1, u);
            mL[n] = fast_left<T, 0>(u, lo3, hs) * jl;
        }
    }
    // right state of face k from cell k+1
    if (k == nz) {
#pragma unroll
        for (int n = 0; n < 5; n++) mR[n] = avg2<T>(a.U[n], a.J, qL, 1);
    } else if (!limR) {
#pragma unroll
        for (int n = 0; n < 5; n++) mR[n] = lin3R<T>(a.U[n], a.J, qR, 1);
    } else {
        const T jr = frcp<T>(hi3 ? (T(2) * T(iJp[qR - 1]) + T(5) * T(iJp[qR]) - T(1) * T(iJp[qR + 1]))
                                 : (T(-3) * T(iJp[qR - 2]) + T(27) * T(iJp[qR - 1]) + T(47) * T(iJp[qR]) -
                                    T(13) * T(iJp[qR + 1]) + T(2) * T(iJp[qR + 2]))) * (hi3 ? w3 : w5);
#pragma unroll
        for (int n = 0; n < 5; n++) {
            T w[5];
            load5<T>(a.U[n], qR, 1, w);
            mR[n] = fast_right<T>(w, hi3) * jr;
        }
    }
}

// linear 5-point states of the unlimited scheme with shared 1/J (Flux_X.cpp:108-122)
template <typename T, typename A>
__device__ __forceinline__ void fast_lin_pair(const A &a, size_t qc, ptrdiff_t s, T *mL, T *mR)
{
    T iJ[6];
#pragma unroll
    for (int t = 0; t < 6; t++) iJ[t] = frcp<T>(T(a.J[qc + (t - 2) * s]));
    const T tl = frcp<T>(T(2) * iJ[0] - T(13) * iJ[1] + T(47) * iJ[2] + T(27) * iJ[3] - T(3) * iJ[4]);
    const T tr = frcp<T>(T(-3) * iJ[1] + T(27) * iJ[2] + T(47) * iJ[3] - T(13) * iJ[4] + T(2) * iJ[5]);
#pragma unroll
    for (int n = 0; n < 5; n++) {
        const auto *U = a.U[n];
        T u0 = T(U[qc - 2 * s]), u1 = T(U[qc - s]), u2 = T(U[qc]), u3 = T(U[qc + s]), u4 = T(U[qc + 2 * s]),
          u5 = T(U[qc + 3 * s]);
        mL[n] = tl * (T(2) * u0 - T(13) * u1 + T(47) * u2 + T(27) * u3 - T(3) * u4);
        mR[n] = tr * (T(-3) * u1 + T(27) * u2 + T(47) * u3 - T(13) * u4 + T(2) * u5);
    }
}

template <typename T, typename A>
__device__ __forceinline__ void fast_states_x_linear(const cf_dims &d, const A &a, int i, int j,
                                                     int k, T *mL, T *mR)
{
    if (i <= 3 || i >= d.gend - 1) {
        states_x_linear<T>(d, a, i, j, k, mL, mR);
        return;
    }
    fast_lin_pair<T>(a, d.ix(i, j + 1, k + 1), (ptrdiff_t)d.plane(), mL, mR);
}

template <typename T, typename A>
__device__ __forceinline__ void fast_states_y_linear(const cf_dims &d, const A &a, int i, int j,
                                                     int k, T *mL, T *mR)
{
    if (j <= 3 || j >= d.ny - 2) {
        states_y_linear<T>(d, a, i, j, k, mL, mR);
        return;
    }
    fast_lin_pair<T>(a, d.ix(i + 1, j, k + 1), d.Zm, mL, mR);
}

template <typename T, typename A, bool INTERIOR = false>
__device__ __forceinline__ void fast_states_z_linear(const cf_dims &d, const A &a, int i, int j,
                                                     int k, T *mL, T *mR)
{
    if (!INTERIOR && (k <= 2 || k >= d.nz - 1)) {
        states_z_linear<T>(d, a, i, j, k, mL, mR);
        return;
    }
    fast_lin_pair<T>(a, d.ix(i + 1, j + 1, k), 1, mL, mR);
}

// Preconditioned Roe with shared reciprocals (Flux_X_limiter.cpp:382-536)
template <typename T>
__device__ __forceinline__ void fast_flux_precond_roe(const T *mL, const T *mR, const T *m, int dir, T Ep, T Jf,
                                                      T K, T e, T *F)
{
    const T n0 = m[3 * dir], n1 = m[3 * dir + 1], n2 = m[3 * dir + 2];
    const T nn = n0 * n0 + n1 * n1 + n2 * n2;
    const T inorm = frcp<T>(sqrt(nn));
    const T NX = n0 * inorm, NY = n1 * inorm, NZ = n2 * inorm;
    const T Km1 = K - T(1), iKm1 = frcp<T>(Km1), iK = frcp<T>(K);

    const T _rho = mL[0], irL = frcp<T>(_rho);
    const T _u = mL[1] * irL, _v = mL[2] * irL, _w = mL[3] * irL;
    const T _U = n0 * _u + n1 * _v + n2 * _w;
    const T __U = NX * _u + NY * _v + NZ * _w;
    const T _VV = _u * _u + _v * _v + _w * _w;
    const T _P = (mL[4] - T(0.5) * _rho * _VV) * Km1;
    const T _T = _P * irL;
    const T _H = T(0.5) * _VV + K * _T * iKm1;

    const T rho_ = mR[0], irR = frcp<T>(rho_);
    const T u_ = mR[1] * irR, v_ = mR[2] * irR, w_ = mR[3] * irR;
    const T U_ = n0 * u_ + n1 * v_ + n2 * w_;
    const T U__ = NX * u_ + NY * v_ + NZ * w_;
    const T VV_ = u_ * u_ + v_ * v_ + w_ * w_;
    const T P_ = (mR[4] - T(0.5) * rho_ * VV_) * Km1;
    const T T_ = P_ * irR;
    const T H_ = T(0.5) * VV_ + K * T_ * iKm1;

    const T rho = T(0.5) * (_rho + rho_);
    const T u = T(0.5) * (_u + u_), v = T(0.5) * (_v + v_), w = T(0.5) * (_w + w_);
    const T U = T(0.5) * (_U + U_);
    const T _U_ = T(0.5) * (__U + U__);
    const T VV = u * u + v * v + w * w;
    const T H = T(0.5) * (_H + H_);
    const T C = (H - T(0.5) * VV) * Km1;
    const T Tm = C * iK;                 // P/rho with P = rho*C/K
    const T iC = frcp<T>(C), iT = K * iC;

    const T dU1 = P_ - _P, dU2 = u_ - _u, dU3 = v_ - _v, dU4 = w_ - _w, dU5 = T_ - _T;

    const T beta = rmax(VV * iC, e);
    const T bm1 = beta - T(1);
    const T S = sqrt(U * U * bm1 * bm1 + T(4) * beta * C * nn);
    const T _S_ = sqrt(_U_ * _U_ * bm1 * bm1 + T(4) * beta * C * (NX * NX + NY * NY + NZ * NZ));

    const T TKb = Tm * K * beta;
    const T temp = T(4) * _S_ * TKb;
    const T it = frcp<T>(temp), ih = T(0.5) * it;
    const T temp1 = S + U + U * beta;
    const T temp2 = -S + U + U * beta;
    const T temp3 = _S_ - _U_ + _U_ * beta;
    const T temp4 = _S_ + _U_ - _U_ * beta;
    const T temp5 = _S_ * _S_ - bm1 * bm1 * _U_ * _U_;
    const T bU = bm1 * _U_;
    const T tempu1 = T(2) * TKb * NX + u * _S_ + u * bU;
    const T tempu2 = T(2) * TKb * NX - u * _S_ + u * bU;
    const T tempv1 = T(2) * TKb * NY + v * _S_ + v * bU;
    const T tempv2 = T(2) * TKb * NY - v * _S_ + v * bU;
    const T tempw1 = T(2) * TKb * NZ + w * _S_ + w * bU;
    const T tempw2 = T(2) * TKb * NZ - w * _S_ + w * bU;
    const T tempuvw = T(2) * TKb * (u * NX + v * NY + w * NZ);
    const T HbU = H * bU;
    const T temph1 = tempuvw + H * _S_ + HbU;
    const T temph2 = tempuvw - H * _S_ + HbU;
    const T aU = fabs(U), a1 = fabs(temp1), a2 = fabs(temp2);
    const T sa = a2 + a1, da = a2 - a1;
    const T k8 = T(8) * TKb * _S_ * aU;          // 8 T K S beta |U|
    const T c4 = T(4) * Km1 * beta * aU;
    const T t32u = temp3 * tempu2 * a2 + temp4 * tempu1 * a1;
    const T t32v = temp3 * tempv2 * a2 + temp4 * tempv1 * a1;
    const T t32w = temp3 * tempw2 * a2 + temp4 * tempw1 * a1;
    const T t32h = temph2 * temp3 * a2 + temph1 * temp4 * a1;
    const T rih = rho * ih;
    const T rhoT = rho * aU * iT;

    const T d11 = it * (_S_ * c4 + temp3 * a1 + temp4 * a2);
    const T c1 = -rih * da * temp5;
    const T d12 = NX * c1, d13 = NY * c1, d14 = NZ * c1;
    const T d15 = -rhoT;

    const T d21 = it * (u * _S_ * (c4 + sa) - da * (T(2) * TKb * NX + u * bU));
    const T d22 = rih * (k8 * (NY * NY + NZ * NZ) + NX * t32u);
    const T d23 = rih * NY * (-k8 * NX + t32u);
    const T d24 = rih * NZ * (-k8 * NX + t32u);
    const T d25 = -u * rhoT;

    const T d31 = it * (v * _S_ * (c4 + sa) - da * (T(2) * TKb * NY + v * bU));
    const T d32 = rih * NX * (-k8 * NY + t32v);
    const T d33 = rih * (k8 * (NX * NX + NZ * NZ) + NY * t32v);
    const T d34 = rih * NZ * (-k8 * NY + t32v);
    const T d35 = -v * rhoT;

    const T d41 = it * (w * _S_ * (c4 + sa) - da * (T(2) * TKb * NZ + w * bU));
    const T d42 = rih * NX * (-k8 * NZ + t32w);
    const T d43 = rih * NY * (-k8 * NZ + t32w);
    const T d44 = rih * (k8 * (NX * NX + NY * NY) + NZ * t32w);
    const T d45 = -w * rhoT;

    const T k8n = T(8) * TKb * _S_;
    const T d51 = it * (_S_ * (T(4) * beta * (H * K - H - Tm * K) * aU + H * sa) - da * (tempuvw + HbU));
    const T d52 = rih * (k8n * (-v * NX * NY - w * NX * NZ + u * (NY * NY + NZ * NZ) * aU) + NX * t32h);
    const T d53 = rih * (k8n * (-u * NX * NY - w * NY * NZ + v * (NX * NX + NZ * NZ) * aU) + NY * t32h);
    const T d54 = rih * (k8n * (-u * NX * NZ - v * NY * NZ + w * (NX * NX + NY * NY) * aU) + NZ * t32h);
    const T d55 = (-H * iT + K * iKm1) * rho * aU;

    const T Fav1 = d11 * dU1 + d12 * dU2 + d13 * dU3 + d14 * dU4 + d15 * dU5;
    const T Fav2 = d21 * dU1 + d22 * dU2 + d23 * dU3 + d24 * dU4 + d25 * dU5;
    const T Fav3 = d31 * dU1 + d32 * dU2 + d33 * dU3 + d34 * dU4 + d35 * dU5;
    const T Fav4 = d41 * dU1 + d42 * dU2 + d43 * dU3 + d44 * dU4 + d45 * dU5;
    const T Fav5 = d51 * dU1 + d52 * dU2 + d53 * dU3 + d54 * dU4 + d55 * dU5;

    const T hJ = T(0.5) * frcp<T>(Jf);
    const T Ps = _P + P_;
    F[0] = ((_rho * _U + rho_ * U_) - Ep * Fav1) * hJ;
    F[1] = ((_rho * _u * _U + rho_ * u_ * U_ + n0 * Ps) - Ep * Fav2) * hJ;
    F[2] = ((_rho * _v * _U + rho_ * v_ * U_ + n1 * Ps) - Ep * Fav3) * hJ;
    F[3] = ((_rho * _w * _U + rho_ * w_ * U_ + n2 * Ps) - Ep * Fav4) * hJ;
    F[4] = ((_U * (T(3.5) * _P + T(0.5) * _rho * _VV) + U_ * (T(3.5) * P_ + T(0.5) * rho_ * VV_)) - Ep * Fav5) * hJ;
    F[5] = (n1 * Ps - Ep * Fav3) * hJ;
}

// Roe (ROE == 1) with shared reciprocals (Flux_X.cpp:247-420)
template <typename T>
__device__ __forceinline__ void fast_flux_roe(const T *mL, const T *mR, const T *m, int dir, T Jf, T K, T *F)
{
    const T n0 = m[3 * dir], n1 = m[3 * dir + 1], n2 = m[3 * dir + 2];
    const T insqr = frcp<T>(sqrt(n0 * n0 + n1 * n1 + n2 * n2));
    const T NX = n0 * insqr, NY = n1 * insqr, NZ = n2 * insqr;
    const T Km1 = K - T(1), iKm1 = frcp<T>(Km1);

    const T _rho = mL[0], irL = frcp<T>(_rho);
    const T _u = mL[1] * irL, _v = mL[2] * irL, _w = mL[3] * irL;
    const T _U = n0 * _u + n1 * _v + n2 * _w;
    const T _VV = _u * _u + _v * _v + _w * _w;
    const T _P = (mL[4] - T(0.5) * _rho * _VV) * Km1;
    const T _H = T(0.5) * _VV + K * _P * irL * iKm1;

    const T rho_ = mR[0], irR = frcp<T>(rho_);
    const T u_ = mR[1] * irR, v_ = mR[2] * irR, w_ = mR[3] * irR;
    const T U_ = n0 * u_ + n1 * v_ + n2 * w_;
    const T VV_ = u_ * u_ + v_ * v_ + w_ * w_;
    const T P_ = (mR[4] - T(0.5) * rho_ * VV_) * Km1;
    const T H_ = T(0.5) * VV_ + K * P_ * irR * iKm1;

    const T temp5 = sqrt(_rho), temp6 = sqrt(rho_);
    const T it4 = frcp<T>(temp5 + temp6);
    const T rho = temp5 * temp6;
    const T u = (temp5 * _u + temp6 * u_) * it4;
    const T v = (temp5 * _v + temp6 * v_) * it4;
    const T w = (temp5 * _w + temp6 * w_) * it4;
    const T U = (temp5 * _U + temp6 * U_) * it4;
    const T VV = u * u + v * v + w * w;
    const T H = (temp5 * _H + temp6 * H_) * it4;
    const T C = (H - T(0.5) * VV) * Km1;

    const T dU1 = rho_ - _rho;
    const T dU2 = rho_ * u_ - _rho * _u;
    const T dU3 = rho_ * v_ - _rho * _v;
    const T dU4 = rho_ * w_ - _rho * _w;
    const T dU5 = (P_ * iKm1 + T(0.5) * rho_ * VV_) - (_P * iKm1 + T(0.5) * _rho * _VV);

    const T S = sqrt(C), iS = frcp<T>(S);
    const T Un = U * insqr, aUn = fabs(Un);
    const T dP = P_ - _P, dUn = (U_ - _U) * insqr;
    const T deltaU = (S - aUn) * dP * frcp<T>(rho * C) + Un * iS * dUn;
    const T deltaP = Un * iS * dP + (S - aUn) * rho * dUn;

    const T Fav1 = aUn * dU1 + deltaU * rho;
    const T Fav2 = aUn * dU2 + deltaU * rho * u + deltaP * NX;
    const T Fav3 = aUn * dU3 + deltaU * rho * v + deltaP * NY;
    const T Fav4 = aUn * dU4 + deltaU * rho * w + deltaP * NZ;
    const T Fav5 = dir == 1 ? aUn * dU5 + deltaU * rho * H + deltaP * Un : aUn * dU5 + deltaU * rho * H + deltaP * U;

    const T sq = frcp<T>(insqr), hJ = T(0.5) * frcp<T>(Jf);
    const T Ps = _P + P_;
    F[0] = ((_rho * _U + rho_ * U_) - Fav1 * sq) * hJ;
    F[1] = ((_rho * _u * _U + rho_ * u_ * U_ + n0 * Ps) - Fav2 * sq) * hJ;
    F[2] = ((_rho * _v * _U + rho_ * v_ * U_ + n1 * Ps) - Fav3 * sq) * hJ;
    F[3] = ((_rho * _w * _U + rho_ * w_ * U_ + n2 * Ps) - Fav4 * sq) * hJ;
    F[4] = ((_U * (T(3.5) * _P + T(0.5) * _rho * _VV) + U_ * (T(3.5) * P_ + T(0.5) * rho_ * VV_)) - Fav5 * sq) * hJ;
    F[5] = (n1 * Ps - Fav3 * sq) * hJ;
}

}  // namespace CF_NS
