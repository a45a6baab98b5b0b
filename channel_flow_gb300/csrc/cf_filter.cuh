// Approximate-deconvolution sensor Filter (Filter.cpp:12-1720).
//
// Per filter width (h: [1 6 1]/8, 2h: [1 2 1]/4) six levels, each an x pass,
// a stretched-y pass and a z pass over the interior box i = 3..gend,
// j = 2..ny, k = 2..nz.  Every value a pass reads outside that box is the
// cell's U: the reference fills each temporary with U before the passes
// (Filter.cpp:121-136) and the passes write only the box.  The deconvolved
// field 6 G1p - 15 G1 + 20 GG - 15 GGG + 6 GGGG - GGGGG (Filter.cpp:769) is
// accumulated level by level in the reference's summation order.
//
// One launch per level (k_filter_level) runs the three passes in shared
// memory: a block owns a 8 x 32 (j, k) tile and marches through a chunk of
// x planes, holding the level's input on three planes in registers; x-pass
// and y-pass results live in shared memory only.  Of the five variables
// only rho, rho u, rho v, rho w are filtered: the sensor E (Filter.cpp:
// 790-804) never reads the filtered energy.
//
// The FP32 build uses the high-pass form instead: with G the three passes
// (values outside the box read as U), the deconvolution residual is
// u - u* = (I - G~)^5 (I - G) u, where G~ is G on fields that are zero
// outside the box (1 - (6x - 15x^2 + 20x^3 - 15x^4 + 6x^5 - x^6) =
// (1 - x)^6, and the affine level map splits into U + the linear part).  So
// each level stores h_(l+1) = -(G - I) h_l, formed from differences of
// neighbouring values, pass by pass ((G - I) = (Gz - I) + Gz (Gy - I) +
// Gz Gy (Gx - I)), and the sixth is u - u* itself: the FP32 rounding is
// then relative to the small high-pass values rather than to u, which is
// what the sensor's energy |u - u*|^2 resolves, and no sum is carried.
//
// EXACT (no-FMA build) keeps the reference's expression trees, with the
// metric ratios b/a and c/a of the y pass formed once per call; otherwise
// the y pass uses per-cell weights A = (b/a) J(j-1)/J(j), C = (c/a)
// J(j+1)/J(j) and no division, and the passes carry their normalisations
// forward (x: NX = 4 or 8 times the filtered value, y: 1/c0 more, z: NX
// more) to one exact scaling by c0/NX^2 at the end: two FP64 (or FP32)
// operations per value and pass instead of three or four.  ST is the
// storage type of the level and accumulator fields (float in the FP32
// build).
#pragma once
#include <algorithm>

#include "cf_common.cuh"


namespace CF_NS {

constexpr int FT_J = 8, FT_K = 32;    // tile rows (j), columns (k); planes per block set at launch
constexpr int FT_HJ = FT_J + 2, FT_HK = FT_K + 2, FT_HALO = FT_HJ * FT_HK;

template <typename ST>
struct filt_fields {
    const double *U[4];
    const void *src[4];     // level input: U (level 0) or the previous level (ST)
    ST *dst[4];             // level output (unused at the last level)
    ST *acc[4];             // deconvolution sum
    ST *lev[2][4];          // both level fields: level 0 copies U into their ghost ring
    const ST *cA, *cC;      // y-pass coefficients (b/a, c/a when EXACT)
    const ST *cB;           // high-pass form: A + C - 1 of the per-cell weights
    const double *J;
};

__device__ __forceinline__ bool filt_inside(const cf_dims &d, int i, int j, int k)
{
    return i >= 3 && i <= d.gend && j >= 2 && j <= d.ny && k >= 2 && k <= d.nz;
}

// y-pass coefficients, once per call (Filter.cpp:186-208)
template <typename T, typename ST, bool EXACT>
__global__ void __launch_bounds__(256) k_filter_coef(cf_dims d, const double *__restrict__ Yp,
                                                     const double *__restrict__ J, ST *cA, ST *cC, ST *cB,
                                                     cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k), s = d.Zm;
    if (EXACT) {
        T a_ = T(Yp[q + s]) - T(Yp[q - s]);
        T b_ = T(Yp[q + s]) - T(Yp[q]);
        T c_ = T(Yp[q]) - T(Yp[q - s]);
        cA[q] = ST(b_ / a_);
        cC[q] = ST(c_ / a_);
    } else if (sizeof(T) == 4) {
        // FP32 build: the differences of Y_point in FP64 (they cancel), the
        // ratios in FP32 (FP64 divisions would dominate this kernel)
        const float a_ = float(Yp[q + s] - Yp[q - s]);
        const float b_ = float(Yp[q + s] - Yp[q]);
        const float c_ = float(Yp[q] - Yp[q - s]);
        const float ia = 1.0f / a_, iJ = 1.0f / float(J[q]);
        cA[q] = ST(b_ * ia * (float(J[q - s]) * iJ));
        cC[q] = ST(c_ * ia * (float(J[q + s]) * iJ));
        // A + C - 1 = (b (J(j-1) - J(j)) + c (J(j+1) - J(j))) / (a J(j)),
        // with the J differences formed in FP64 (they cancel)
        cB[q] = ST((b_ * float(J[q - s] - J[q]) + c_ * float(J[q + s] - J[q])) * ia * iJ);
    } else {
        const double a_ = Yp[q + s] - Yp[q - s];
        const double b_ = Yp[q + s] - Yp[q];
        const double c_ = Yp[q] - Yp[q - s];
        const double iJ = frcp<double>(J[q]), ia = frcp<double>(a_);
        cA[q] = ST(b_ * ia * (J[q - s] * iJ));
        cC[q] = ST(c_ * ia * (J[q + s] * iJ));
    }
}

// Every value a pass reads outside the box is the cell's U.  Level 0 reads
// U itself and copies the values it reads outside the box into the ghost
// ring of both level fields (as ST), so the later levels read their input
// field alone, with no per-load choice between two arrays.  Offsets are
// 32-bit (the launcher checks the array size).
template <typename T, typename SRC, typename ST, bool L0, bool HF>
__device__ __forceinline__ void filt_load4(const filt_fields<ST> &f, bool ghost, unsigned q, T *x)
{
#pragma unroll
    for (int v = 0; v < 4; v++) x[v] = T(static_cast<const SRC *>(f.src[v])[q]);
    if (L0 && ghost) {
        // the high-pass levels are zero outside the box
#pragma unroll
        for (int v = 0; v < 4; v++) {
            f.lev[0][v][q] = HF ? ST(0) : ST(x[v]);
            f.lev[1][v][q] = HF ? ST(0) : ST(x[v]);
        }
    }
}

// One filter level.  The block's input planes roll through registers: at
// plane i the thread holds planes i-1, i, i+1 of its halo positions and
// has plane i+2 in flight, and the y-pass coefficients and the
// deconvolution sum of plane i are requested before the x pass, so the
// passes wait on no global load.
template <typename T, typename SRC, typename ST, bool WIDE, bool EXACT, bool L0, bool HF>
__global__ void __launch_bounds__(256, HF ? 3 : sizeof(T) == 4 ? 4 : 2) k_filter_level(cf_dims d, filt_fields<ST> f, int level, int fti)
{
    __shared__ T sgx[4][FT_HJ][FT_HK];     // x pass, rows j0-1..j0+8, columns k0-1..k0+32
    __shared__ T sgy[4][FT_J][FT_HK];      // y pass, rows j0..j0+7
    __shared__ T sfv[HF ? 4 : 1][FT_HJ][FT_HK];   // high-pass form: the level's input on the halo
    constexpr T cxz = T(WIDE ? 0.25 : 0.125), cy = T(WIDE ? 0.5 : 0.25);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
    const int k0 = 2 + (int)blockIdx.x * FT_K, j0 = 2 + (int)blockIdx.y * FT_J;
    const int i0 = 3 + (int)blockIdx.z * fti;
    const int i1 = min(i0 + fti - 1, d.gend);
    const bool level0 = L0;
    const unsigned P = (unsigned)d.plane(), Zm = (unsigned)d.Zm;
    // halo positions owned by this thread: tid and tid + 256; qh = offset
    // in plane 0, hin = inside the box in (j, k)
    bool pv[2], hin[2];
    unsigned qh[2];
#pragma unroll
    for (int o = 0; o < 2; o++) {
        const int p = tid + 256 * o;
        const int pj = j0 - 1 + p / FT_HK, pk = k0 - 1 + p % FT_HK;
        pv[o] = p < FT_HALO && pj <= d.ny + 1 && pk <= d.nz + 1;
        hin[o] = pj >= 2 && pj <= d.ny && pk >= 2 && pk <= d.nz;
        qh[o] = (unsigned)pj * Zm + (unsigned)pk;
    }
    // level 0 copies the values outside the box (outside in (j, k), or on
    // the planes 2 and gend+1) into the level fields' ghost ring
    T sm[2][4], s0[2][4], sp[2][4], sn[2][4];
#pragma unroll
    for (int o = 0; o < 2; o++) {
#pragma unroll
        for (int v = 0; v < 4; v++) sm[o][v] = s0[o][v] = sp[o][v] = sn[o][v] = T(0);
        if (pv[o]) {
            filt_load4<T, SRC, ST, L0, HF>(f, level0 && (!hin[o] || i0 - 1 < 3), (unsigned)(i0 - 1) * P + qh[o], sm[o]);
            filt_load4<T, SRC, ST, L0, HF>(f, level0 && !hin[o], (unsigned)i0 * P + qh[o], s0[o]);
            filt_load4<T, SRC, ST, L0, HF>(f, level0 && (!hin[o] || i0 + 1 > d.gend), (unsigned)(i0 + 1) * P + qh[o], sp[o]);
        }
    }
    const int jy = j0 + ty;                  // y-pass / output row of this thread
    const int kz = k0 + tx;                  // z-pass / output column
    const bool last = level == 5;
    const bool outp = jy <= d.ny && kz <= d.nz;
    const bool rowp = jy <= d.ny;
    const unsigned qy = (unsigned)jy * Zm + (unsigned)(k0 - 1 + tx);   // y-pass column tx (plane 0)
    const unsigned qz = (unsigned)jy * Zm + (unsigned)kz;              // output cell (plane 0)
    bool ycol[2];
#pragma unroll
    for (int o = 0; o < 2; o++) {
        const int kk = k0 - 1 + tx + 32 * o;
        ycol[o] = rowp && tx + 32 * o < FT_HK && kk >= 2 && kk <= d.nz;
    }
    for (int i = i0; i <= i1; i++) {
        const unsigned qi = (unsigned)i * P;
        // requests for this plane's y-pass coefficients and sum, and the
        // input plane i+2
        T cAv[2] = {T(0), T(0)}, cCv[2] = {T(0), T(0)}, cBv[2] = {T(0), T(0)}, ac[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int o = 0; o < 2; o++)
            if (ycol[o]) {
                cAv[o] = T(f.cA[qi + qy + 32 * o]);
                cCv[o] = T(f.cC[qi + qy + 32 * o]);
                if (HF) cBv[o] = T(f.cB[qi + qy + 32 * o]);
            }
        if (!HF && outp && level > 0) {
#pragma unroll
            for (int v = 0; v < 4; v++) ac[v] = T(f.acc[v][qi + qz]);
        }
        if (i + 2 <= i1 + 1) {
#pragma unroll
            for (int o = 0; o < 2; o++)
                if (pv[o])
                    filt_load4<T, SRC, ST, L0, HF>(f, level0 && (!hin[o] || i + 2 > d.gend), qi + 2 * P + qh[o], sn[o]);
        }
        // x pass (Filter.cpp:156-170, 835-849); plane i lies inside the box
#pragma unroll
        for (int o = 0; o < 2; o++) {
            if (!pv[o]) continue;
            const bool in = hin[o];
            const int r = (tid + 256 * o) / FT_HK, c = (tid + 256 * o) % FT_HK;
#pragma unroll
            for (int v = 0; v < 4; v++) {
                T g = s0[o][v];
                if (HF) {
                    // (Gx - I) f: differences of neighbours, zero outside the box
                    sfv[v][r][c] = s0[o][v];
                    sgx[v][r][c] = in ? cxz * ((sm[o][v] - s0[o][v]) + (sp[o][v] - s0[o][v])) : T(0);
                    continue;
                }
                if (EXACT) {
                    if (in)
                        g = WIDE ? T(0.25) * (sm[o][v] + T(2) * s0[o][v] + sp[o][v])
                                 : T(0.125) * (sm[o][v] + T(6) * s0[o][v] + sp[o][v]);
                } else {
                    // NX times the filtered value (cells outside the box:
                    // NX times the cell's value), one add and one FMA
                    g = (in ? T(WIDE ? 2 : 6) : T(WIDE ? 4 : 8)) * s0[o][v] + (in ? sm[o][v] + sp[o][v] : T(0));
                }
                sgx[v][r][c] = g;
            }
        }
        __syncthreads();
        // stretched y pass (Filter.cpp:186-208, 863-883)
        if (rowp) {
#pragma unroll
            for (int o = 0; o < 2; o++) {
                const int c = tx + 32 * o;
                const int kk = k0 - 1 + c;
                if (c >= FT_HK || kk > d.nz + 1) continue;
                if (!ycol[o]) {
#pragma unroll
                    for (int v = 0; v < 4; v++)
                        sgy[v][ty][c] = HF ? T(0)
                                           : EXACT ? sgx[v][ty + 1][c] : T(WIDE ? 2.0 : 4.0 / 3.0) * sgx[v][ty + 1][c];
                    continue;
                }
                const T A = cAv[o], C = cCv[o];
                if (HF) {
                    // (Gy Gx - I) f = (Gy - I) f + Gy (Gx - I) f, with
                    // (Gy - I) g = cy (A (g(j-1) - g) + C (g(j+1) - g) + B g)
                    const T B = cBv[o];
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const T fm = sfv[v][ty][c], f0 = sfv[v][ty + 1][c], fp = sfv[v][ty + 2][c];
                        const T em = sgx[v][ty][c], e0 = sgx[v][ty + 1][c], ep = sgx[v][ty + 2][c];
                        sgy[v][ty][c] = e0 + cy * (A * ((fm - f0) + (em - e0)) + C * ((fp - f0) + (ep - e0)) +
                                                   B * (f0 + e0));
                    }
                } else if (EXACT) {
                    const size_t q = d.ix(i, jy, kk);
                    const size_t s = d.Zm;
                    const T Jm = T(f.J[q - s]), J0 = T(f.J[q]), Jp = T(f.J[q + s]);
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const T gm = sgx[v][ty][c], g0 = sgx[v][ty + 1][c], gp = sgx[v][ty + 2][c];
                        sgy[v][ty][c] = WIDE ? T(0.5) * (A * gm * Jm + g0 * J0 + C * gp * Jp) / J0
                                             : T(0.125) * (T(2) * A * gm * Jm + T(6) * g0 * J0 + T(2) * C * gp * Jp) / J0;
                    }
                } else {
                    // cw (A gm + C gp) + c0 g0 over c0: two FMAs per value
                    // (cw/c0 = 1 wide, 1/3 narrow)
                    const T As = WIDE ? A : A * T(1.0 / 3.0), Cs = WIDE ? C : C * T(1.0 / 3.0);
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const T gm = sgx[v][ty][c], g0 = sgx[v][ty + 1][c], gp = sgx[v][ty + 2][c];
                        sgy[v][ty][c] = As * gm + (Cs * gp + g0);
                    }
                }
            }
        }
        // high-pass form: the z pass's input values, read before the barrier
        // after which the next plane's x pass rewrites sfv
        T zfm[4], zf0[4], zfp[4];
        if (HF && outp) {
#pragma unroll
            for (int v = 0; v < 4; v++) {
                zfm[v] = sfv[v][ty + 1][tx];
                zf0[v] = sfv[v][ty + 1][tx + 1];
                zfp[v] = sfv[v][ty + 1][tx + 2];
            }
        }
        __syncthreads();
        // z pass (Filter.cpp:224-239, 896-910) and the deconvolution sum
        if (outp) {
            const unsigned q = qi + qz;
#pragma unroll
            for (int v = 0; v < 4; v++) {
                const T gm = sgy[v][ty][tx], g0 = sgy[v][ty][tx + 1], gp = sgy[v][ty][tx + 2];
                if (HF) {
                    // next high-pass level h <- h - G h = -(G - I) h, with
                    // (G - I) f = (Gz - I) f + Gz (Gy Gx - I) f; the last
                    // level's h is u - u* and goes to acc
                    const T dev = g0 + cxz * (((zfm[v] - zf0[v]) + (zfp[v] - zf0[v])) + ((gm - g0) + (gp - g0)));
                    (last ? f.acc[v] : f.dst[v])[q] = ST(-dev);
                    continue;
                }
                // the contracted build's passes carry the factors NX (x),
                // NX / c0 (y) and NX (z); c0 / NX^2 is 1/32 (wide) or 3/256
                // (narrow), both exact
                const T r = EXACT ? (WIDE ? T(0.25) * (gm + T(2) * g0 + gp) : T(0.125) * (gm + T(6) * g0 + gp))
                                  : T(WIDE ? 1.0 / 32.0 : 3.0 / 256.0) * (T(WIDE ? 2 : 6) * g0 + (gm + gp));
                if (!last) f.dst[v][q] = ST(r);
                T s;
                switch (level) {
                case 0: s = T(6) * r; break;
                case 1: s = ac[v] - T(15) * r; break;
                case 2: s = ac[v] + T(20) * r; break;
                case 3: s = ac[v] - T(15) * r; break;
                case 4: s = ac[v] + T(6) * r; break;
                default: s = ac[v] - r; break;
                }
                f.acc[v][q] = ST(s);
            }
        }
#pragma unroll
        for (int o = 0; o < 2; o++)
#pragma unroll
            for (int v = 0; v < 4; v++) {
                sm[o][v] = s0[o][v];
                s0[o][v] = sp[o][v];
                sp[o][v] = sn[o][v];
            }
        // sgx is rewritten next plane only after every thread passed the
        // second barrier (y pass done); sgy after the next first barrier
    }
}

// E = |u - u_deconvolved|^2 (Filter.cpp:790-804, 1465-1479)
template <typename ST>
struct filt_ptr4 {
    ST *p[4];
};
// HF (high-pass form): acc holds h = u - u*, and with velocity V = m/rho
// of the state, m/rho - (m - h_m)/(rho - h_rho) = (h_m - V h_rho)/(rho - h_rho)
template <typename T, typename ST, bool HF>
__global__ void k_filter_energy4(cf_dims d, cf_ptr5 U, filt_ptr4<ST> acc, double *E, cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
    if (HF) {
        const T rho = T(U.p[0][q]), hr = T(acc.p[0][q]);
        const T irho = frcp<T>(rho), iden = frcp<T>(rho - hr);
        const T Ue = (T(acc.p[1][q]) - T(U.p[1][q]) * irho * hr) * iden;
        const T Ve = (T(acc.p[2][q]) - T(U.p[2][q]) * irho * hr) * iden;
        const T We = (T(acc.p[3][q]) - T(U.p[3][q]) * irho * hr) * iden;
        E[q] = double(Ue * Ue + Ve * Ve + We * We);
        return;
    }
    T u1 = T(U.p[0][q]), f1 = T(acc.p[0][q]);
#ifdef CF_FAST_MATH
    // two reciprocals instead of six divisions
    const T iu = frcp<T>(u1), iff = frcp<T>(f1);
    T Ue = T(U.p[1][q]) * iu - T(acc.p[1][q]) * iff;
    T Ve = T(U.p[2][q]) * iu - T(acc.p[2][q]) * iff;
    T We = T(U.p[3][q]) * iu - T(acc.p[3][q]) * iff;
#else
    T Ue = T(U.p[1][q]) / u1 - T(acc.p[1][q]) / f1;
    T Ve = T(U.p[2][q]) / u1 - T(acc.p[2][q]) / f1;
    T We = T(U.p[3][q]) / u1 - T(acc.p[3][q]) / f1;
#endif
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

template <typename T, typename SRC, typename ST, bool EXACT, bool HF>
static cudaError_t filter_level_launch(const cf_dims &d, const filt_fields<ST> &f, bool wide, int level,
                                       cudaStream_t s)
{
    // planes per block: one wave of the resident blocks (3 per SM in the
    // FP32 high-pass form, 2 in FP64), x cut into as many chunks as fill it
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 132;
    }
    const int tk = (d.Z_out + FT_K - 1) / FT_K, tj = (d.Y_out + FT_J - 1) / FT_J;
    if (d.total() >= (size_t(1) << 31)) return cudaErrorInvalidValue;   // 32-bit offsets
    // chunks minimising (waves of resident blocks) x (planes per block +
    // the two extra planes a block loads before its first)
    const int slots = sms * (HF ? 3 : sizeof(T) == 4 ? 4 : 2);
    int chunks = 1;
    long best = -1;
    for (int c = 1; c <= d.X_out; c++) {
        const long waves = ((long)tk * tj * c + slots - 1) / slots, planes = (d.X_out + c - 1) / c;
        if (best < 0 || waves * (planes + 2) < best) { best = waves * (planes + 2); chunks = c; }
    }
    const int fti = (d.X_out + chunks - 1) / chunks;
    const dim3 g((unsigned)tk, (unsigned)tj, (unsigned)((d.X_out + fti - 1) / fti));
    const dim3 t(32, 8);
    if (level == 0) {
        if (wide) k_filter_level<T, SRC, ST, true, EXACT, true, HF><<<g, t, 0, s>>>(d, f, level, fti);
        else k_filter_level<T, SRC, ST, false, EXACT, true, HF><<<g, t, 0, s>>>(d, f, level, fti);
    } else {
        if (wide) k_filter_level<T, SRC, ST, true, EXACT, false, HF><<<g, t, 0, s>>>(d, f, level, fti);
        else k_filter_level<T, SRC, ST, false, EXACT, false, HF><<<g, t, 0, s>>>(d, f, level, fti);
    }
    return cudaSuccess;
}

// T: arithmetic type, ST: storage of the scratch levels, EXACT: reference
// expression trees.  Scratch (cf_filter_args): lev[2][4], acc[4], cA, cC
// hold ST values; Eh, E2h doubles.
template <typename T, typename ST, bool EXACT>
cudaError_t launch_filter(const cf_dims &d, const cf_filter_args &a, double crit, double hi, double lo,
                          cudaStream_t s)
{
    const cf_box bi = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    const dim3 g = box_grid(bi), t = box_block();
    ST *cA = static_cast<ST *>(a.cA), *cC = static_cast<ST *>(a.cC);
    // FP32: the high-pass form (each level holds h_(l+1) = (I - G) h_l, h_0 = u,
    // and h_6 = u - u*), whose FP32 rounding is relative to the small
    // high-pass values instead of to u
    constexpr bool HF = sizeof(T) == 4 && !EXACT;
    ST *cB = static_cast<ST *>(a.cB);
    k_filter_coef<T, ST, EXACT><<<g, t, 0, s>>>(d, a.Yp, a.J, cA, cC, cB, bi);
    filt_fields<ST> f;
    for (int v = 0; v < 4; v++) {
        f.U[v] = a.U[v];
        f.acc[v] = static_cast<ST *>(a.acc[v]);
    }
    f.cA = cA;
    f.cC = cC;
    f.cB = cB;
    f.J = a.J;
    cf_ptr5 U;
    filt_ptr4<ST> acc;
    for (int v = 0; v < 5; v++) U.p[v] = const_cast<double *>(a.U[v]);
    for (int v = 0; v < 4; v++) acc.p[v] = static_cast<ST *>(a.acc[v]);
    for (int l = 0; l < 2; l++)
        for (int v = 0; v < 4; v++) f.lev[l][v] = static_cast<ST *>(a.lev[l][v]);
    for (int wide = 0; wide < 2; wide++) {
        for (int lev = 0; lev < 6; lev++) {
            for (int v = 0; v < 4; v++) {
                f.src[v] = lev == 0 ? static_cast<const void *>(a.U[v]) : a.lev[(lev - 1) & 1][v];
                f.dst[v] = static_cast<ST *>(a.lev[lev & 1][v]);
            }
            const cudaError_t e = lev == 0 ? filter_level_launch<T, double, ST, EXACT, HF>(d, f, wide != 0, lev, s)
                                           : filter_level_launch<T, ST, ST, EXACT, HF>(d, f, wide != 0, lev, s);
            if (e != cudaSuccess) return e;
        }
        k_filter_energy4<T, ST, HF><<<g, t, 0, s>>>(d, U, acc, wide ? a.E2h : a.Eh, bi);
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
