// Approximate-deconvolution sensor Filter (Filter.cpp:12-1720).
//
// Per filter width (h: [1 6 1]/8, 2h: [1 2 1]/4) six levels, each an x pass,
// a stretched-y pass and a z pass over the interior box i = 3..gend,
// j = 2..ny, k = 2..nz.  Values read outside that box are the copies of U
// the reference puts into every temporary (Filter.cpp:121-136): the shell
// of each scratch field is filled with U once per call.  The deconvolved
// field 6 G1p - 15 G1 + 20 GG - 15 GGG + 6 GGGG - GGGGG is accumulated in
// the z pass level by level in the reference's summation order (the
// roundings are identical), which replaces the reference's 55 temporaries
// by 5 ping-pong level fields, the x/y pass fields and one accumulator.
#pragma once
#include "cf_common.cuh"


namespace CF_NS {

// copy U into every scratch field outside the interior box
__global__ void k_filter_shell(cf_dims d, cf_filter_args a, size_t n)
{
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const size_t plane = d.plane();
    const int i = (int)(q / plane);
    const size_t r = q - (size_t)i * plane;
    const int j = (int)(r / (size_t)d.Zm);
    const int k = (int)(r - (size_t)j * (size_t)d.Zm);
    if (i >= 3 && i <= d.gend && j >= 2 && j <= d.ny && k >= 2 && k <= d.nz) return;
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const double u = a.U[v][q];
        a.gx[v][q] = u;
        a.gy[v][q] = u;
        a.lev[0][v][q] = u;
        a.lev[1][v][q] = u;
    }
}

// x pass (Filter.cpp:156-170, 835-849): level L -> gx
template <typename T, bool WIDE>
__global__ void k_filter_x(cf_dims d, cf_ptr5 src, cf_ptr5 dst, cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k), s = d.plane();
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const double *g = src.p[v];
        T r = WIDE ? T(0.25) * (T(g[q - s]) + T(2) * T(g[q]) + T(g[q + s]))
                   : T(0.125) * (T(g[q - s]) + T(6) * T(g[q]) + T(g[q + s]));
        dst.p[v][q] = double(r);
    }
}

// stretched y pass (Filter.cpp:186-208, 863-883): gx -> gy
template <typename T, bool WIDE>
__global__ void k_filter_y(cf_dims d, cf_ptr5 src, cf_ptr5 dst, const double *__restrict__ J,
                           const double *__restrict__ Yp, cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k), s = d.Zm;
    T a_ = T(Yp[q + s]) - T(Yp[q - s]);
    T b_ = T(Yp[q + s]) - T(Yp[q]);
    T c_ = T(Yp[q]) - T(Yp[q - s]);
    const T Jm = T(J[q - s]), J0 = T(J[q]), Jp = T(J[q + s]);
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const double *G = src.p[v];
        T r = WIDE ? T(0.5) * (b_ / a_ * T(G[q - s]) * Jm + T(G[q]) * J0 + c_ / a_ * T(G[q + s]) * Jp) / J0
                   : T(0.125) * (T(2) * b_ / a_ * T(G[q - s]) * Jm + T(6) * T(G[q]) * J0 + T(2) * c_ / a_ * T(G[q + s]) * Jp) / J0;
        dst.p[v][q] = double(r);
    }
}

// z pass (Filter.cpp:224-239, 896-910): gy -> level L+1, and the running
// deconvolution sum of Filter.cpp:769 (weights 6, -15, 20, -15, 6, -1)
template <typename T, bool WIDE>
__global__ void k_filter_z(cf_dims d, cf_ptr5 src, cf_ptr5 dst, cf_ptr5 acc, cf_box b, int level)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const double *G = src.p[v];
        T r = WIDE ? T(0.25) * (T(G[q - 1]) + T(2) * T(G[q]) + T(G[q + 1]))
                   : T(0.125) * (T(G[q - 1]) + T(6) * T(G[q]) + T(G[q + 1]));
        dst.p[v][q] = double(r);
        T s;
        switch (level) {
        case 0: s = T(6) * r; break;
        case 1: s = T(acc.p[v][q]) - T(15) * r; break;
        case 2: s = T(acc.p[v][q]) + T(20) * r; break;
        case 3: s = T(acc.p[v][q]) - T(15) * r; break;
        case 4: s = T(acc.p[v][q]) + T(6) * r; break;
        default: s = T(acc.p[v][q]) - r; break;
        }
        acc.p[v][q] = double(s);
    }
}

// E = |u - u_deconvolved|^2 (Filter.cpp:790-804, 1465-1479)
template <typename T>
__global__ void k_filter_energy(cf_dims d, cf_filter_args a, double *E, cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
    T u1 = T(a.U[0][q]), f1 = T(a.acc[0][q]);
    T Ue = T(a.U[1][q]) / u1 - T(a.acc[1][q]) / f1;
    T Ve = T(a.U[2][q]) / u1 - T(a.acc[2][q]) / f1;
    T We = T(a.U[3][q]) / u1 - T(a.acc[3][q]) / f1;
    E[q] = double(Ue * Ue + Ve * Ve + We * We);
}

// ghost copies of E_h and E_2h (Filter.cpp:1487-1555): x planes 2, gend+1
// for j = 2..ny, k = 2..nz; then rows 1, nyy and columns 1, nzz of the
// interior planes.  One thread per (plane, row) pair of the fill boxes.
__global__ void k_filter_efill_x(cf_dims d, double *Eh, double *E2h, cf_box b)
{
    CF_BOX_INDEX(b, side, j, k);
    const int dst = side == 0 ? 2 : d.gend + 1;
    const int src = side == 0 ? 3 : d.gend;
    Eh[d.ix(dst, j, k)] = Eh[d.ix(src, j, k)];
    E2h[d.ix(dst, j, k)] = E2h[d.ix(src, j, k)];
}
__global__ void k_filter_efill_y(cf_dims d, double *Eh, double *E2h, cf_box b)
{
    CF_BOX_INDEX(b, i, side, k);
    const int dst = side == 0 ? 1 : d.ny + 1;
    const int src = side == 0 ? 2 : d.ny;
    Eh[d.ix(i, dst, k)] = Eh[d.ix(i, src, k)];
    E2h[d.ix(i, dst, k)] = E2h[d.ix(i, src, k)];
}
__global__ void k_filter_efill_z(cf_dims d, double *Eh, double *E2h, cf_box b)
{
    CF_BOX_INDEX(b, i, j, side);
    const int dst = side == 0 ? 1 : d.nz + 1;
    const int src = side == 0 ? 2 : d.nz;
    Eh[d.ix(i, j, dst)] = Eh[d.ix(i, j, src)];
    E2h[d.ix(i, j, dst)] = E2h[d.ix(i, j, src)];
}

// Ep thresholds (Filter.cpp:1568-1645): Ep = E_high where
// (E_h + E_h')/(E_2h + E_2h') >= Roe_criterion over the face's two cells
template <typename T, int DIR>
__global__ void k_filter_ep(cf_dims d, const double *__restrict__ Eh, const double *__restrict__ E2h,
                            double *Ep, cf_box b, double crit, double hi, double lo)
{
    CF_BOX_INDEX(b, i, j, k);
    size_t qa, qb;
    if (DIR == 0) { qa = d.ix(i, j + 1, k + 1); qb = d.ix(i + 1, j + 1, k + 1); }
    else if (DIR == 1) { qa = d.ix(i + 1, j, k + 1); qb = d.ix(i + 1, j + 1, k + 1); }
    else { qa = d.ix(i + 1, j + 1, k); qb = d.ix(i + 1, j + 1, k + 1); }
    T Emax = (T(Eh[qa]) + T(Eh[qb])) / (T(E2h[qa]) + T(E2h[qb]));
    Ep[d.ix(i, j, k)] = Emax >= T(crit) ? hi : lo;
}

template <typename T>
cudaError_t launch_filter(const cf_dims &d, const cf_filter_args &a, double crit, double hi, double lo,
                          cudaStream_t s)
{
    const size_t n = d.total();
    k_filter_shell<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, a, n);
    const cf_box bi = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    const dim3 g = box_grid(bi), t = box_block();
    cf_ptr5 gx, gy, acc, l0, l1, U;
    for (int v = 0; v < 5; v++) {
        gx.p[v] = a.gx[v]; gy.p[v] = a.gy[v]; acc.p[v] = a.acc[v];
        l0.p[v] = a.lev[0][v]; l1.p[v] = a.lev[1][v]; U.p[v] = const_cast<double *>(a.U[v]);
    }
    for (int wide = 0; wide < 2; wide++) {
        cf_ptr5 src = U, dst = l0, other = l1;
        for (int lev = 0; lev < 6; lev++) {
            if (wide) {
                k_filter_x<T, true><<<g, t, 0, s>>>(d, src, gx, bi);
                k_filter_y<T, true><<<g, t, 0, s>>>(d, gx, gy, a.J, a.Yp, bi);
                k_filter_z<T, true><<<g, t, 0, s>>>(d, gy, dst, acc, bi, lev);
            } else {
                k_filter_x<T, false><<<g, t, 0, s>>>(d, src, gx, bi);
                k_filter_y<T, false><<<g, t, 0, s>>>(d, gx, gy, a.J, a.Yp, bi);
                k_filter_z<T, false><<<g, t, 0, s>>>(d, gy, dst, acc, bi, lev);
            }
            src = dst;
            cf_ptr5 tmp = dst; dst = other; other = tmp;
        }
        k_filter_energy<T><<<g, t, 0, s>>>(d, a, wide ? a.E2h : a.Eh, bi);
    }
    cf_box bx = make_box(0, 1, 2, d.ny, 2, d.nz);
    k_filter_efill_x<<<box_grid(bx), t, 0, s>>>(d, a.Eh, a.E2h, bx);
    cf_box by = make_box(3, d.gend, 0, 1, 2, d.nz);
    k_filter_efill_y<<<box_grid(by), t, 0, s>>>(d, a.Eh, a.E2h, by);
    cf_box bz = make_box(3, d.gend, 2, d.ny, 0, 1);
    k_filter_efill_z<<<box_grid(bz), t, 0, s>>>(d, a.Eh, a.E2h, bz);
    cf_box ex = make_box(2, d.gend, 1, d.ny - 1, 1, d.nz - 1);
    k_filter_ep<T, 0><<<box_grid(ex), t, 0, s>>>(d, a.Eh, a.E2h, a.Ep[0], ex, crit, hi, lo);
    cf_box ey = make_box(2, d.gend - 1, 1, d.ny, 1, d.nz - 1);
    k_filter_ep<T, 1><<<box_grid(ey), t, 0, s>>>(d, a.Eh, a.E2h, a.Ep[1], ey, crit, hi, lo);
    cf_box ez = make_box(2, d.gend - 1, 1, d.ny - 1, 1, d.nz);
    k_filter_ep<T, 2><<<box_grid(ez), t, 0, s>>>(d, a.Eh, a.E2h, a.Ep[2], ez, crit, hi, lo);
    return cudaGetLastError();
}

}  // namespace CF_NS
