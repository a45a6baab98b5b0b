// Metrics of a channel whose lower wall undulates in x: the general
// curvilinear set-up that the reference lacks (its Grid.cpp:49-141 and
// Jacobian*.cpp build analytic flat-wall metrics only).
//
// Mapping of the computational coordinates (xi = x, eta in [0, 1], zeta = z):
//
//     y(xi, eta) = y_w(xi) + Y0(eta) (1 - y_w(xi) / high)
//     y_w(xi)    = A sin(2 pi xi / lambda)                        (lower wall)
//     Y0(eta)    = high/2 (1 - tanh(g (1 - 2 eta)) / tanh(g))    (Jacobian.cpp:73)
//
// so the upper wall stays at y = high and A = 0 gives the reference's
// flat channel.  At every point the forward derivative matrix
// d(x, y, z)/d(xi, eta, zeta) is formed, either analytically or (the
// conservative form) from differences of the mapping across the cell, half
// a spacing to each side; the Jacobian J = 1/det and the nine metrics
// xidx..ztdz are its inverse.  In the conservative form the x-face value of
// dy/deta and the y-face value of dy/dxi are differences between the same
// cell-corner points, so the finite-volume divergence of a constant flux
// vanishes to rounding (the discrete geometric conservation law); the
// analytic form leaves a truncation-sized residual.
//
// Every index of the array (ghosts included) is written, with the
// positions of the reference's index conventions: cells at
// xi = (i - 1.5) dXI (Grid.cpp X_point), eta = (j - 1.5) dET; x faces
// (face between cells i and i+1, stored at [i][j-1][k-1]) at
// xi = (i - 1) dXI, eta = (j - 0.5) dET; y faces ([i-1][j][k-1]) at
// xi = (i - 0.5) dXI, eta = (j - 1) dET; z faces ([i-1][j-1][k]) at
// xi = (i - 0.5) dXI, eta = (j - 0.5) dET.  Compiled without FMA
// contraction (set-up, not on the timed path).
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>

#include "../../include/channel_flow_gb300.h"

namespace {

struct wv {
    int X, Y, Z;              // interior cells
    double dXI, dET, dZT, high;
    double A, k_wave, g, tg;  // amplitude, 2 pi / lambda, stretching, tanh(g)
    int conservative;
    __host__ __device__ size_t Ym() const { return (size_t)Y + 4; }
    __host__ __device__ size_t Zm() const { return (size_t)Z + 4; }
};

__device__ __forceinline__ double wall(const wv &w, double xi) { return w.A * sin(w.k_wave * xi); }

__device__ __forceinline__ double y0(const wv &w, double eta)
{
    return 0.5 * w.high * (1.0 - tanh(w.g * (1.0 - 2.0 * eta)) / w.tg);
}

__device__ __forceinline__ double ymap(const wv &w, double xi, double eta)
{
    const double yw = wall(w, xi);
    return yw + y0(w, eta) * (1.0 - yw / w.high);
}

// dy/dxi and dy/deta at (xi, eta)
__device__ __forceinline__ void yderiv(const wv &w, double xi, double eta, double &y_xi, double &y_eta)
{
    if (w.conservative) {
        y_xi = (ymap(w, xi + 0.5 * w.dXI, eta) - ymap(w, xi - 0.5 * w.dXI, eta)) / w.dXI;
        y_eta = (ymap(w, xi, eta + 0.5 * w.dET) - ymap(w, xi, eta - 0.5 * w.dET)) / w.dET;
    } else {
        // the flat-wall factor in the reference's order (Jacobian.cpp:82-84)
        const double s = 1.0 / cosh(w.g * (1.0 - 2.0 * eta));
        const double ydet0 = w.high * w.g * 1. / w.tg * s * s;
        const double yw = wall(w, xi);
        y_xi = w.A * w.k_wave * cos(w.k_wave * xi) * (1.0 - y0(w, eta) / w.high);
        y_eta = ydet0 * (1.0 - yw / w.high);
    }
}

__global__ void k_wavy_metrics(wv w, int where, double *J, double *m0, double *m1, double *m2, double *m3,
                               double *m4, double *m5, double *m6, double *m7, double *m8)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= (int)w.Zm() || j >= (int)w.Ym()) return;
    // position of this index (reference index conventions)
    const double ci[4] = {1.5, 1.0, 0.5, 0.5}, cj[4] = {1.5, 0.5, 1.0, 0.5};
    const double xi = (i - ci[where]) * w.dXI, eta = (j - cj[where]) * w.dET;
    double y_xi, y_eta;
    yderiv(w, xi, eta, y_xi, y_eta);
    // forward matrix a[r][c] = d(x, y, z)_r / d(xi, eta, zeta)_c and its inverse
    const double a00 = 1, a01 = 0, a02 = 0;
    const double a10 = y_xi, a11 = y_eta, a12 = 0;
    const double a20 = 0, a21 = 0, a22 = 1;
    const double c00 = a11 * a22 - a12 * a21, c01 = a12 * a20 - a10 * a22, c02 = a10 * a21 - a11 * a20;
    const double det = a00 * c00 + a01 * c01 + a02 * c02;
    const double Jq = 1.0 / det;
    const size_t q = ((size_t)i * w.Ym() + j) * w.Zm() + k;
    J[q] = Jq;
    // row r of the inverse = d(xi, eta, zeta)_r / d(x, y, z)
    m0[q] = c00 * Jq;                                   // xidx
    m1[q] = (a02 * a21 - a01 * a22) * Jq;               // xidy
    m2[q] = (a01 * a12 - a02 * a11) * Jq;               // xidz
    m3[q] = c01 * Jq;                                   // etdx
    m4[q] = (a00 * a22 - a02 * a20) * Jq;               // etdy
    m5[q] = (a02 * a10 - a00 * a12) * Jq;               // etdz
    m6[q] = c02 * Jq;                                   // ztdx
    m7[q] = (a01 * a20 - a00 * a21) * Jq;               // ztdy
    m8[q] = (a00 * a11 - a01 * a10) * Jq;               // ztdz
}

// cell-centre y with the ghost rows of Grid.cpp:49-108 taken about the
// local wall: Y[1] = 2 y_w - Y[2], Y[nyy] = Y[ny] + 2 (Y[2] - y_w), and
// linear continuation into rows 0 and nyy+1
__global__ void k_wavy_ypoint(wv w, double *Yp)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= (int)w.Zm() || j >= (int)w.Ym()) return;
    const int ny = w.Y + 1;
    const double xi = (i - 1.5) * w.dXI, yw = wall(w, xi);
    const double y2 = ymap(w, xi, 0.5 * w.dET), yny = ymap(w, xi, (ny - 1.5) * w.dET);
    const double y1 = 2.0 * yw - y2, ynyy = yny + 2.0 * (y2 - yw);
    double v;
    if (j == 0) v = 2.0 * y1 - y2;
    else if (j == 1) v = y1;
    else if (j == ny + 1) v = ynyy;
    else if (j == ny + 2) v = 2.0 * ynyy - yny;
    else v = ymap(w, xi, (j - 1.5) * w.dET);
    Yp[((size_t)i * w.Ym() + j) * w.Zm() + k] = v;
}

int make(const cf_grid *g, const cf_wavy_wall *ww, wv &w)
{
    if (!g || !ww) return CF_ERR_ARG;
    if (g->cells_x < 1 || g->cells_y < 1 || g->cells_z < 1) return CF_ERR_ARG;
    if (!(ww->wavelength > 0) || !(ww->stretching > 0) || !(g->height > 0)) return CF_ERR_ARG;
    if (!(std::fabs(ww->amplitude) < 0.5 * g->height)) return CF_ERR_ARG;   // the wall stays below mid-channel
    w.X = g->cells_x;
    w.Y = g->cells_y;
    w.Z = g->cells_z;
    w.dXI = g->d_xi;
    w.dET = g->d_eta;
    w.dZT = g->d_zeta;
    w.high = g->height;
    w.A = ww->amplitude;
    w.k_wave = 2.0 * M_PI / ww->wavelength;
    w.g = ww->stretching;
    w.tg = std::tanh(ww->stretching);
    w.conservative = ww->conservative ? 1 : 0;
    return CF_OK;
}

dim3 grid_of(const wv &w) { return dim3((unsigned)((w.Zm() + 31) / 32), (unsigned)((w.Ym() + 7) / 8), (unsigned)(w.X + 6)); }

}  // namespace

extern "C" {

int cf_wavy_metrics(const cf_grid *g, void *cuda_stream, const cf_wavy_wall *wall_, int where,
                    double *const *J_and_metrics10)
{
    wv w;
    if (int rc = make(g, wall_, w)) return rc;
    if (where < CF_AT_CELL || where > CF_AT_ZFACE || !J_and_metrics10) return CF_ERR_ARG;
    for (int n = 0; n < 10; n++)
        if (!J_and_metrics10[n]) return CF_ERR_ARG;
    double *const *p = J_and_metrics10;
    k_wavy_metrics<<<grid_of(w), dim3(32, 8), 0, static_cast<cudaStream_t>(cuda_stream)>>>(
        w, where, p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9]);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

int cf_wavy_y_point(const cf_grid *g, void *cuda_stream, const cf_wavy_wall *wall_, double *Y_point)
{
    wv w;
    if (int rc = make(g, wall_, w)) return rc;
    if (!Y_point) return CF_ERR_ARG;
    k_wavy_ypoint<<<grid_of(w), dim3(32, 8), 0, static_cast<cudaStream_t>(cuda_stream)>>>(w, Y_point);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

}  // extern "C"
