// Boundary conditions, the explicit RK3 update and the flat-wall face
// metrics (small element-wise kernels).
#pragma once
#include "cf_common.cuh"

namespace CF_NS {

// x ghost planes 0..2 <- gend-2..gend and gend+1..gend+3 <- 3..5: the whole
// domain is on one device, so the reference's halo exchange and periodic
// seam (main.cpp:156-244) become a periodic image of every ghost plane.
__global__ void k_x_periodic(cf_dims d, cf_ptr5 U)
{
    const size_t plane = d.plane();
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= plane * 6) return;
    const int s = (int)(t / plane);
    const size_t r = t - (size_t)s * plane;
    const int dst = s < 3 ? s : d.gend + 1 + (s - 3);
    const int src = s < 3 ? d.gend - 2 + s : 3 + (s - 3);
#pragma unroll
    for (int n = 0; n < 5; n++) U.p[n][(size_t)dst * plane + r] = U.p[n][(size_t)src * plane + r];
}

// Y_boundary_condition.cpp:48-120: isothermal no-slip wall ghosts (rows 1
// and nyy) from rows 2 and ny, i = 2..gend+1, k = 2..nz.
template <typename T>
__global__ void k_y_wall(cf_dims d, cf_ptr5 U, const double *__restrict__ J, cf_box b)
{
    CF_BOX_INDEX(b, i, side, k);
    const int js = side == 0 ? 2 : d.ny;
    const int jg = side == 0 ? 1 : d.ny + 1;
    const size_t s = d.ix(i, js, k), q = d.ix(i, jg, k);
    const T K = CF_DC(T, d, K), R = CF_DC(T, d, R);
    T u1 = T(U.p[0][s]);
    T rho = u1 * T(J[s]);
    T Uu = T(U.p[1][s]) / u1;
    T V = T(U.p[2][s]) / u1;
    T W = T(U.p[3][s]) / u1;
    T VV = Uu * Uu + V * V + W * W;
    T P = (T(U.p[4][s]) * T(J[s]) - T(0.5) * rho * VV) * (K - T(1));
    T temp = P / rho / R;
    T Tg = T(2) * T(298.0592) - temp;
    rho = P / R / Tg;
    const T Jq = T(J[q]);
    U.p[0][q] = P / R / Tg / Jq;
    U.p[1][q] = -P / R / Tg * Uu / Jq;
    U.p[2][q] = -P / R / Tg * V / Jq;
    U.p[3][q] = -P / R / Tg * W / Jq;
    U.p[4][q] = (rho * R * Tg / (K - T(1)) + T(0.5) * P / R / Tg * VV) / Jq;
}

// Z_boundary_condition.cpp:48-67: one-deep periodic copy in z for rows
// j = 0..nyyy of planes i = 2..gend+1.
__global__ void k_z_periodic(cf_dims d, cf_ptr5 U, cf_box b)
{
    const int j = b.j0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int i = b.i0 + (int)blockIdx.y;
    if (j >= b.j0 + b.nj) return;
#pragma unroll
    for (int n = 0; n < 5; n++) {
        double *u = U.p[n];
        u[d.ix(i, j, 1)] = u[d.ix(i, j, d.nz)];
        u[d.ix(i, j, d.nz + 1)] = u[d.ix(i, j, 2)];
    }
}

// RK3NODT.cpp:130-184: flux divergence + viscous + body force, SSP-RK3 stage.

template <typename T>
__global__ void k_rk3(cf_dims d, cf_rk3_args a, cf_box b, int RK, double deltaT)
{
    CF_BOX_INDEX(b, i, j, k);
    const double c1[3] = {1.0, 0.75, 1.0 / 3.0};
    const double c2[3] = {0.0, 0.25, 2.0 / 3.0};
    const double c3[3] = {1.0, 0.25, 2.0 / 3.0};
    const size_t q = d.ix(i, j, k);
    const size_t fx = d.ix(i, j - 1, k - 1), f0 = d.ix(i - 1, j - 1, k - 1);
    const size_t fy = d.ix(i - 1, j, k - 1), fz = d.ix(i - 1, j - 1, k);
    const T dXI = CF_DC(T, d, dXI), dET = CF_DC(T, d, dET), dZT = CF_DC(T, d, dZT);
    T tmp = T(a.U_[1][q]) / T(a.U_[0][q]);
    T Rk[5];
#pragma unroll
    for (int n = 0; n < 5; n++)
        Rk[n] = -((T(a.Fx[n][fx]) - T(a.Fx[n][f0])) / dXI + (T(a.Fy[n][fy]) - T(a.Fy[n][f0])) / dET +
                  (T(a.Fz[n][fz]) - T(a.Fz[n][f0])) / dZT);
    const T f = CF_DC(T, d, f), Jq = T(a.J[q]);
    Rk[1] = Rk[1] + T(a.vF[0][q]) + f / Jq;
    Rk[2] = Rk[2] + T(a.vF[1][q]);
    Rk[3] = Rk[3] + T(a.vF[2][q]);
    Rk[4] = Rk[4] + T(a.vF[3][q]) + f * tmp / Jq;
#pragma unroll
    for (int n = 0; n < 5; n++) {
        double mr = deltaT * double(Rk[n]);
        a.MR[n][q] = mr;
        a.U_[n][q] = c1[RK - 1] * double(a.U[n][q]) + c2[RK - 1] * a.U_[n][q] + c3[RK - 1] * mr;
    }
}

// Flat-wall analytic face metrics (Jacobian_u.cpp:27-68, Jacobian_v.cpp:
// 40-141, Jacobian_w.cpp:26-67) with stretching parameter gamma and the
// wall-normal offset joff (0.5 for x/z faces, 1.0 for y faces).

__global__ void k_face_metrics(cf_dims d, cf_metric_args a, cf_box b, double gamma, double joff)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
    const double high = d.high;
    double temp = (0.5 * high) * (1 - 1. / tanh(gamma) * tanh(gamma * (1 - 2 * (j - joff) * d.dET)));
    double temp1 = (1 - temp / (0.5 * high)) * tanh(gamma);
    double etdy = tanh(gamma) / (2 * (0.5 * high) * gamma * (1 - temp1 * temp1));
    double temp2 = 1 / cosh(gamma * (1 - 2 * (j - joff) * d.dET));
    double ydet = high * gamma * 1. / tanh(gamma) * temp2 * temp2;
    a.m[0][q] = 1; a.m[1][q] = 0; a.m[2][q] = 0;
    a.m[3][q] = 0; a.m[4][q] = etdy; a.m[5][q] = 0;
    a.m[6][q] = 0; a.m[7][q] = 0; a.m[8][q] = 1;
    a.Jf[q] = 1. / (1 * ydet * 1);
}

// Jacobian_v.cpp:124-141: wall rows of the y-face metrics from the cell
// metrics' ghost rows
__global__ void k_v_wall_rows(cf_dims d, cf_metric_args a, cf_box b)
{
    const int k = b.k0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int i = b.i0 + (int)blockIdx.y;
    if (k >= b.k0 + b.nk) return;
    const int ny = d.ny;
#pragma unroll
    for (int t = 0; t < 3; t++) {
        a.m[3 + t][d.ix(i, 1, k)] = a.mc[3 + t][d.ix(i, 1, k)];
        a.m[3 + t][d.ix(i, ny, k)] = a.mc[3 + t][d.ix(i, ny + 1, k)];
    }
    a.Jf[d.ix(i, ny, k)] = a.Jc[d.ix(i, ny + 1, k)];
    a.Jf[d.ix(i, 1, k)] = a.Jc[d.ix(i, 1, k)];
}

}  // namespace CF_NS
