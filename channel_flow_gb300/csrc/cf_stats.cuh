// FP64 reductions and IO staging around the step: Driven_force
// (Driven_force.cpp:38-62), Statistic (Statistic.cpp:139-1068) and the
// restart image of Output / Initial_condition (Output.cpp:43-70,
// Initial_condition.cpp:64-95).
//
// Row sums are deterministic: a block sums a fixed part of one y row in a
// fixed order and a fixed tree; a second kernel adds the parts of a row in
// order.  The per-element quantities follow the reference's expressions
// (identical bits in the no-FMA build); the sums differ from the
// reference's serial loops only by summation order.  Always FP64.
#pragma once
#include "cf_flux.cuh"

namespace CF_NS {

constexpr int ST_THREADS = 256;

// Statistic row quantity sets
enum { ST_FACE = 0, ST_SHEAR = 1, ST_MOMENT = 2, ST_BULK = 3 };

template <int KIND>
struct st_kind;
template <> struct st_kind<ST_FACE> { static constexpr int NQ = 9; };
template <> struct st_kind<ST_SHEAR> { static constexpr int NQ = 1; };
template <> struct st_kind<ST_MOMENT> { static constexpr int NQ = 7; };
template <> struct st_kind<ST_BULK> { static constexpr int NQ = 1; };

// y-face Roe quantities (Statistic.cpp:292-489, ROE == 1) of face (i, j, k)
// from the linear MUSCL states (Statistic.cpp:139-290 = Flux_Y.cpp's states):
// u_L, u_R, v_L, v_R, rho_L, rho_R, 0.5 (rho u V)/J_v, 0.5 Fav2/insqr/J_v, d(rho u)
#ifdef CF_FAST_MATH
// The contracted build: the face states with the 1/J of the stencil shared
// by the five variables, every quotient by a Newton-refined reciprocal
// (one per divisor) and the square roots of the Roe weights reused; within
// about 1e-13 of the expressions below, at a fraction of their FP64-pipe
// operations (the kernel is bound by that pipe).
__device__ __forceinline__ void st_face(const cf_dims &d, const cf_stat_args &a, int i, int j, int k, double *o)
{
    cf_flux_args fa;
    for (int n = 0; n < 5; n++) fa.U[n] = a.U[n];
    fa.J = a.J;
    double ML[5], MR[5];
    fast_states_y_linear<double>(d, fa, i, j, k, ML, MR);
    const double K = d.K, km1 = K - 1, ikm1 = d.ikm1;
    const size_t q = d.ix(i, j, k);
    const double etx = a.m[3][q], ety = a.m[4][q], etz = a.m[5][q];
    const double sq = sqrt(etx * etx + ety * ety + etz * etz);
    const double insqr = frcp(sq);
    const double ETx = etx * insqr;
    const double _rho = ML[0], ir_ = frcp(_rho);
    const double _u = ML[1] * ir_, _v = ML[2] * ir_, _w = ML[3] * ir_;
    const double _V = etx * _u + ety * _v + etz * _w;
    const double _VV = _u * _u + _v * _v + _w * _w;
    const double _P = (ML[4] - 0.5 * _rho * _VV) * km1;
    const double _H = 0.5 * _VV + K * _P * ir_ * ikm1;
    const double rho_ = MR[0], ir2 = frcp(rho_);
    const double u_ = MR[1] * ir2, v_ = MR[2] * ir2, w_ = MR[3] * ir2;
    const double V_ = etx * u_ + ety * v_ + etz * w_;
    const double VV_ = u_ * u_ + v_ * v_ + w_ * w_;
    const double P_ = (MR[4] - 0.5 * rho_ * VV_) * km1;
    const double H_ = 0.5 * VV_ + K * P_ * ir2 * ikm1;
    const double dU2 = rho_ * u_ - _rho * _u;
    const double temp5 = sqrt(_rho), temp6 = sqrt(rho_);
    const double it4 = frcp(temp5 + temp6);
    const double rho = temp5 * temp6;
    const double u = (temp5 * _u + temp6 * u_) * it4;
    const double v = (temp5 * _v + temp6 * v_) * it4;
    const double w = (temp5 * _w + temp6 * w_) * it4;
    const double V = (temp5 * _V + temp6 * V_) * it4;
    const double VV = u * u + v * v + w * w;
    const double H = (temp5 * _H + temp6 * H_) * it4;
    const double C = (H - 0.5 * VV) * km1;
    const double S = sqrt(C), iS = frcp(S);
    const double Vn = V * insqr;
    const double temp1 = (P_ - _P) * frcp(rho * C);
    const double temp2 = Vn * iS * (V_ - _V) * insqr;
    const double deltaU = (S - fabs(Vn)) * temp1 + temp2;
    const double deltaP = Vn * iS * (P_ - _P) + (S - fabs(Vn)) * rho * (V_ - _V) * insqr;
    // the reference takes the Cartesian Roe v here, not the contravariant V
    const double Fav2 = fabs(v * insqr) * dU2 + deltaU * rho * u + deltaP * ETx;
    const double iJv = frcp(a.Jv[q]);
    o[0] = _u;
    o[1] = u_;
    o[2] = _v;
    o[3] = v_;
    o[4] = _rho;
    o[5] = rho_;
    o[6] = 0.5 * (_rho * _u * _V + rho_ * u_ * V_) * iJv;
    o[7] = 0.5 * Fav2 * sq * iJv;
    o[8] = dU2;
}
#else
__device__ __forceinline__ void st_face(const cf_dims &d, const cf_stat_args &a, int i, int j, int k, double *o)
{
    cf_flux_args fa;
    for (int n = 0; n < 5; n++) fa.U[n] = a.U[n];
    fa.J = a.J;
    double ML[5], MR[5];
    states_y_linear<double>(d, fa, i, j, k, ML, MR);
    const double K = d.K;
    const size_t q = d.ix(i, j, k);
    double etx = a.m[3][q], ety = a.m[4][q], etz = a.m[5][q];
    double insqr = 1.0 / sqrt(etx * etx + ety * ety + etz * etz);
    double ETx = etx * insqr;
    double _rho = ML[0];
    double _u = ML[1] / _rho;
    double _v = ML[2] / _rho;
    double _w = ML[3] / _rho;
    double _V = etx * _u + ety * _v + etz * _w;
    double _VV = _u * _u + _v * _v + _w * _w;
    double _P = (ML[4] - 0.5 * _rho * _VV) * (K - 1);
    double _C = K * _P / _rho;
    double _H = 0.5 * _VV + _C / (K - 1);
    double rho_ = MR[0];
    double u_ = MR[1] / rho_;
    double v_ = MR[2] / rho_;
    double w_ = MR[3] / rho_;
    double V_ = etx * u_ + ety * v_ + etz * w_;
    double VV_ = u_ * u_ + v_ * v_ + w_ * w_;
    double P_ = (MR[4] - 0.5 * rho_ * VV_) * (K - 1);
    double C_ = K * P_ / rho_;
    double H_ = 0.5 * VV_ + C_ / (K - 1);
    double dU2 = rho_ * u_ - _rho * _u;
    double temp5 = sqrt(_rho);
    double temp6 = sqrt(rho_);
    double temp4 = temp5 + temp6;
    double rho = sqrt(_rho * rho_);
    double u = (temp5 * _u + temp6 * u_) / temp4;
    double v = (temp5 * _v + temp6 * v_) / temp4;
    double w = (temp5 * _w + temp6 * w_) / temp4;
    double V = (temp5 * _V + temp6 * V_) / temp4;
    double VV = u * u + v * v + w * w;
    double H = (temp5 * _H + temp6 * H_) / temp4;
    double C = (H - 0.5 * VV) * (K - 1);
    double S = sqrt(C);
    double temp1 = (P_ - _P) / rho / C;
    double temp2 = V * insqr / S * (V_ - _V) * insqr;
    double deltaU = (S - fabs(V * insqr)) * temp1 + temp2;
    double deltaP = V * insqr / S * (P_ - _P) + (S - fabs(V * insqr)) * rho * (V_ - _V) * insqr;
    // the reference takes the Cartesian Roe v here, not the contravariant V
    double Fav2 = fabs(v * insqr) * dU2 + deltaU * rho * u + deltaP * ETx;
    const double Jv = a.Jv[q];
    o[0] = _u;
    o[1] = u_;
    o[2] = _v;
    o[3] = v_;
    o[4] = _rho;
    o[5] = rho_;
    o[6] = 0.5 * (_rho * _u * _V + rho_ * u_ * V_) / Jv;
    o[7] = 0.5 * Fav2 / insqr / Jv;
    o[8] = dU2;
}
#endif

__device__ __forceinline__ void st_vel(const cf_stat_args &a, size_t q, double &u, double &v, double &w)
{
    const double rho = a.U[0][q];
#ifdef CF_FAST_MATH
    const double ir = frcp(rho);
    u = a.U[1][q] * ir;
    v = a.U[2][q] * ir;
    w = a.U[3][q] * ir;
#else
    u = a.U[1][q] / rho;
    v = a.U[2][q] / rho;
    w = a.U[3][q] / rho;
#endif
}

// viscous x-momentum flux of the low y face of cell (i, j, k)
// (Statistic.cpp:592-840): only the velocity gradients enter
__device__ __forceinline__ double st_shear(const cf_dims &d, const cf_stat_args &a, int i, int j, int k)
{
    double U, V, W, iU, iV, iW, jU, jV, jW, kU, kV, kW, ijU, ijV, ijW, jkU, jkV, jkW;
    double Ui, Vi, Wi, Uk, Vk, Wk, jUi, jVi, jWi, jUk, jVk, jWk;
    st_vel(a, d.ix(i, j, k), U, V, W);
    st_vel(a, d.ix(i - 1, j, k), iU, iV, iW);
    st_vel(a, d.ix(i, j - 1, k), jU, jV, jW);
    st_vel(a, d.ix(i, j, k - 1), kU, kV, kW);
    st_vel(a, d.ix(i - 1, j - 1, k), ijU, ijV, ijW);
    st_vel(a, d.ix(i, j - 1, k - 1), jkU, jkV, jkW);
    st_vel(a, d.ix(i + 1, j, k), Ui, Vi, Wi);
    st_vel(a, d.ix(i, j, k + 1), Uk, Vk, Wk);
    st_vel(a, d.ix(i + 1, j - 1, k), jUi, jVi, jWi);
    st_vel(a, d.ix(i, j - 1, k + 1), jUk, jVk, jWk);
    const double invET = 1. / (d.dET);
    const double inv4XI = 1. / (4 * d.dXI), inv4ZT = 1. / (4 * d.dZT);
    const size_t f = d.ix(i - 1, j - 1, k - 1);
    double xix = a.m[0][f], xiy = a.m[1][f], xiz = a.m[2][f];
    double etx = a.m[3][f], ety = a.m[4][f], etz = a.m[5][f];
    double ztx = a.m[6][f], zty = a.m[7][f], ztz = a.m[8][f];
    double du_dx = (Ui + jUi - iU - ijU) * inv4XI;
    double dv_dx = (Vi + jVi - iV - ijV) * inv4XI;
    double dw_dx = (Wi + jWi - iW - ijW) * inv4XI;
    double du_dy = (U - jU) * invET;
    double dv_dy = (V - jV) * invET;
    double dw_dy = (W - jW) * invET;
    double du_dz = (Uk + jUk - kU - jkU) * inv4ZT;
    double dv_dz = (Vk + jVk - kV - jkV) * inv4ZT;
    double dw_dz = (Wk + jWk - kW - jkW) * inv4ZT;
    double b1 = (4. / 3) * etx * etx + ety * ety + etz * etz;
    double b5 = (1. / 3) * etx * ety;
    double b7 = (1. / 3) * etx * etz;
    double d1 = (4. / 3) * xix * etx + xiy * ety + xiz * etz;
    double d5 = xix * ety - (2. / 3) * xiy * etx;
    double d6 = xix * etz - (2. / 3) * xiz * etx;
    double f1 = (4. / 3) * etx * ztx + ety * zty + etz * ztz;
    double f7 = ety * ztx - (2. / 3) * etx * zty;
    double f9 = etz * ztx - (2. / 3) * etx * ztz;
#ifdef CF_FAST_MATH
    return d.mu_L * (d1 * du_dx + d5 * dv_dx + d6 * dw_dx + b1 * du_dy + b5 * dv_dy + b7 * dw_dy + f1 * du_dz +
                     f7 * dv_dz + f9 * dw_dz) * frcp(a.Jv[f]);
#else
    return d.mu_L * (d1 * du_dx + d5 * dv_dx + d6 * dw_dx + b1 * du_dy + b5 * dv_dy + b7 * dw_dy + f1 * du_dz +
                     f7 * dv_dz + f9 * dw_dz) / a.Jv[f];
#endif
}

// Jsum = sum over j of 1/J[3][j][3] in the reference's order (Driven_force.cpp:38-42):
// the quotients in parallel, then one thread adds them in order (one block
// of 256 threads, rows in chunks of 256)
__global__ void __launch_bounds__(256) k_bulk_jsum(cf_dims d, const double *J, double *jsum)
{
    __shared__ double q[256];
    double s = 0;
    for (int j0 = 2; j0 <= d.ny; j0 += 256) {
        const int j = j0 + (int)threadIdx.x;
        if (j <= d.ny) q[threadIdx.x] = 1. / J[d.ix(3, j, 3)];
        __syncthreads();
        if (threadIdx.x == 0) {
            const int n = min(256, d.ny - j0 + 1);
            for (int t = 0; t < n; t++) s = s + q[t];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *jsum = s;
}

// Partial row sums: block (r, c) sums the elements of row r in i-chunk c.
// Rows and element ranges per kind (j: row, i, k: elements):
//   FACE   j = 1..ny,   i = 2..gend-1, k = 1..nz-1
//   SHEAR  j = 1..ny,   i = 3..gend,   k = 2..nz   (flux of the face below cell j+1)
//   MOMENT j = 2..ny,   i = 3..gend,   k = 2..nz
//   BULK   j = 2..ny,   i = 3..gend,   k = 2..nz
template <int KIND>
__global__ void __launch_bounds__(ST_THREADS) k_stat_rows(cf_dims d, cf_stat_args a, double *partial, int nchunk,
                                                          const double *jsum)
{
    constexpr int NQ = st_kind<KIND>::NQ;
    const int r = blockIdx.x, c = blockIdx.y;
    const int j = (KIND == ST_FACE || KIND == ST_SHEAR) ? 1 + r : 2 + r;
    const int ilo = KIND == ST_FACE ? 2 : 3, ihi = KIND == ST_FACE ? d.gend - 1 : d.gend;
    const int klo = KIND == ST_FACE ? 1 : 2, khi = KIND == ST_FACE ? d.nz - 1 : d.nz;
    const int ni = ihi - ilo + 1, nk = khi - klo + 1;
    const int i0 = ilo + (int)(((long long)ni * c) / nchunk), i1 = ilo + (int)(((long long)ni * (c + 1)) / nchunk);
    double s[NQ];
#pragma unroll
    for (int n = 0; n < NQ; n++) s[n] = 0;
    const long long count = (long long)(i1 - i0) * nk;
    for (long long e = threadIdx.x; e < count; e += ST_THREADS) {
        const int i = i0 + (int)(e / nk), k = klo + (int)(e % nk);
        if constexpr (KIND == ST_FACE) {
            double o[9];
            st_face(d, a, i, j, k, o);
#pragma unroll
            for (int n = 0; n < NQ; n++) s[n] += o[n];
        } else if constexpr (KIND == ST_SHEAR) {
            s[0] += st_shear(d, a, i, j + 1, k);
        } else if constexpr (KIND == ST_MOMENT) {
            double U, V, W;
            st_vel(a, d.ix(i, j, k), U, V, W);
            s[0] += U; s[1] += V; s[2] += W;
            s[3] += U * U; s[4] += V * V; s[5] += W * W; s[6] += U * V;
        } else {
            const size_t q = d.ix(i, j, k);
            s[0] += (a.U[1][q] * a.J[q]) * 1. / a.J[q] / *jsum;
        }
    }
    __shared__ double sh[NQ][ST_THREADS];
#pragma unroll
    for (int n = 0; n < NQ; n++) sh[n][threadIdx.x] = s[n];
    __syncthreads();
    for (int wdt = ST_THREADS / 2; wdt > 0; wdt >>= 1) {
        if ((int)threadIdx.x < wdt)
#pragma unroll
            for (int n = 0; n < NQ; n++) sh[n][threadIdx.x] += sh[n][threadIdx.x + wdt];
        __syncthreads();
    }
    if (threadIdx.x == 0)
#pragma unroll
        for (int n = 0; n < NQ; n++) partial[((size_t)r * nchunk + c) * NQ + n] = sh[n][0];
}

// out[qmap[n]][j0 + r] (+)= sum over the chunks of row r, in chunk order
struct st_qmap {
    int q[9];
};
template <int NQ>
__global__ void k_stat_finish(const double *partial, int nrows, int nchunk, int j0, double *out, int Ym, st_qmap qm,
                              int accumulate)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nrows * NQ) return;
    const int r = t / NQ, n = t % NQ;
    double s = 0;
    for (int c = 0; c < nchunk; c++) s += partial[((size_t)r * nchunk + c) * NQ + n];
    double &dst = out[(size_t)qm.q[n] * Ym + j0 + r];
    dst = accumulate ? dst + s : s;
}

// restart image (Output.cpp:43-70): ten blocks [i][j][k] of U*J
__global__ void k_restart_pack(cf_dims d, cf_ptr5 U, cf_ptr5 Uq, const double *J, double *img)
{
    const size_t N = (size_t)d.X_out * d.Y_out * d.Z_out;
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N) return;
    const int k = (int)(e % d.Z_out), j = (int)((e / d.Z_out) % d.Y_out), i = (int)(e / ((size_t)d.Z_out * d.Y_out));
    const size_t q = d.ix(i + 3, j + 2, k + 2);
    const double Jq = J[q];
#pragma unroll
    for (int f = 0; f < 5; f++) {
        img[f * N + e] = U.p[f][q] * Jq;
        img[(5 + f) * N + e] = Uq.p[f][q] * Jq;
    }
}

// Initial_condition.cpp:77-95: U = image / J on the interior
__global__ void k_restart_unpack(cf_dims d, const double *img, cf_ptr5 U, cf_ptr5 Uq, const double *J)
{
    const size_t N = (size_t)d.X_out * d.Y_out * d.Z_out;
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N) return;
    const int k = (int)(e % d.Z_out), j = (int)((e / d.Z_out) % d.Y_out), i = (int)(e / ((size_t)d.Z_out * d.Y_out));
    const size_t q = d.ix(i + 3, j + 2, k + 2);
    const double Jq = J[q];
#pragma unroll
    for (int f = 0; f < 5; f++) {
        U.p[f][q] = img[f * N + e] / Jq;
        Uq.p[f][q] = img[(5 + f) * N + e] / Jq;
    }
}

// U_q <- U, U <- U_ on the interior (main.cpp:443-462)
__global__ void k_advance_levels(cf_dims d, cf_ptr5 U_, cf_ptr5 U, cf_ptr5 Uq, cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
#pragma unroll
    for (int f = 0; f < 5; f++) {
        Uq.p[f][q] = U.p[f][q];
        U.p[f][q] = U_.p[f][q];
    }
}

}  // namespace CF_NS
