/*
 * CPU oracle (test infrastructure): the reference's approximate-
 * deconvolution sensor Filter (Filter.cpp:12-1720), restated in C.
 *
 * Per filter width (h: weights [1 6 1]/8, 2h: [1 2 1]/4) six nested
 * applications of an x pass, a stretched-y pass and a z pass give the
 * levels G1p, G1, GG, GGG, GGGG, GGGGG; the deconvolved field is
 * 6 G1p - 15 G1 + 20 GG - 15 GGG + 6 GGGG - GGGGG (Filter.cpp:769), summed
 * here level by level in that same order (identical rounding).  Every pass
 * covers the interior i = 3..gend, j = 2..ny, k = 2..nz; values it reads
 * outside that box are the copies of U made when the temporaries are
 * initialised (Filter.cpp:121-136), i.e. the caller's ghost cells.  The
 * resolved kinetic-energy differences E_h, E_2h then decide the switch
 * Ep = E_high where E_h/E_2h >= Roe_criterion (Filter.cpp:1568-1645).
 */
#include "cf_oracle_common.h"

typedef struct { double *v[5]; } fields5;

static fields5 alloc5(size_t n)
{
    fields5 f;
    for (int q = 0; q < 5; q++) f.v[q] = (double *)malloc(n * sizeof(double));
    return f;
}
static void free5(fields5 f)
{
    for (int q = 0; q < 5; q++) free(f.v[q]);
}
static void copy5(fields5 d, double **src, size_t n)
{
    for (int q = 0; q < 5; q++) {
        double *dst = d.v[q];
        const double *s = src[q];
        #pragma omp parallel for
        for (size_t x = 0; x < n; x++) dst[x] = s[x];
    }
}

/* one x, y and z pass: dst = Z(Y(X(src))), using gx, gy as the
 * intermediate arrays (their out-of-box values are U copies).  The x and
 * z passes run variable by variable with k innermost (contiguous,
 * vectorisable); every value is the reference's expression, so the order of
 * the loops does not change a bit. */
static void level(const cfo_grid *g, double *const *src, fields5 gx, fields5 gy, fields5 dst,
                  const double *J, const double *Yp, int wide)
{
    GRID_LOCALS(g);
    const ptrdiff_t sx = (ptrdiff_t)Ym * Zm, sy = Zm;
    /* x pass (Filter.cpp:156-170 / 835-849) */
    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j <= ny; j++)
            for (int n = 0; n < 5; n++) {
                const double *s = src[n];
                double *d = gx.v[n];
                const size_t q0 = IX(i, j, 0);
                if (wide)
                    for (int k = 2; k <= nz; k++) {
                        const size_t q = q0 + k;
                        d[q] = 0.25 * (s[q - sx] + 2 * s[q] + s[q + sx]);
                    }
                else
                    for (int k = 2; k <= nz; k++) {
                        const size_t q = q0 + k;
                        d[q] = 0.125 * (s[q - sx] + 6 * s[q] + s[q + sx]);
                    }
            }
    /* stretched y pass (Filter.cpp:186-208 / 863-883): the spacings a, b,
     * c once per cell for the five variables, as the reference forms them */
    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j <= ny; j++)
            for (int k = 2; k <= nz; k++) {
                const size_t q = IX(i, j, k);
                double a = Yp[q + sy] - Yp[q - sy];
                double b = Yp[q + sy] - Yp[q];
                double c = Yp[q] - Yp[q - sy];
                for (int n = 0; n < 5; n++) {
                    const double *G = gx.v[n];
                    gy.v[n][q] = wide
                        ? 0.5 * (b / a * G[q - sy] * J[q - sy] + G[q] * J[q] + c / a * G[q + sy] * J[q + sy]) / J[q]
                        : 0.125 * (2 * b / a * G[q - sy] * J[q - sy] + 6 * G[q] * J[q] + 2 * c / a * G[q + sy] * J[q + sy]) / J[q];
                }
            }
    /* z pass (Filter.cpp:224-239 / 896-910) */
    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j <= ny; j++)
            for (int n = 0; n < 5; n++) {
                const double *G = gy.v[n];
                double *d = dst.v[n];
                const size_t q0 = IX(i, j, 0);
                if (wide)
                    for (int k = 2; k <= nz; k++) {
                        const size_t q = q0 + k;
                        d[q] = 0.25 * (G[q - 1] + 2 * G[q] + G[q + 1]);
                    }
                else
                    for (int k = 2; k <= nz; k++) {
                        const size_t q = q0 + k;
                        d[q] = 0.125 * (G[q - 1] + 6 * G[q] + G[q + 1]);
                    }
            }
}

/* deconvolved field of one filter width and its energy difference E */
static void sensor_energy(const cfo_grid *g, double **U, const double *J, const double *Yp,
                          int wide, double *E, size_t n)
{
    GRID_LOCALS(g);
    static const double wgt[6] = {6, -15, 20, -15, 6, -1};
    fields5 gx = alloc5(n), gy = alloc5(n), l0 = alloc5(n), l1 = alloc5(n), acc = alloc5(n);
    /* the reference initialises every temporary to U (Filter.cpp:121-136);
     * acc is written on the whole interior before it is read and read only
     * there, so its copy is left out */
    copy5(gx, U, n); copy5(gy, U, n); copy5(l0, U, n); copy5(l1, U, n);
    fields5 prev = {{U[0], U[1], U[2], U[3], U[4]}};
    fields5 cur = l0, nxt = l1;
    for (int lev = 0; lev < 6; lev++) {
        level(g, prev.v, gx, gy, cur, J, Yp, wide);
        const double w = wgt[lev];
        #pragma omp parallel for collapse(2)
        for (int i = 3; i <= gend; i++)
            for (int j = 2; j <= ny; j++)
                for (int v = 0; v < 5; v++) {
                    const double *x = cur.v[v];
                    double *s = acc.v[v];
                    const size_t q0 = IX(i, j, 0);
                    if (lev == 0)
                        for (int k = 2; k <= nz; k++) s[q0 + k] = 6 * x[q0 + k];
                    else if (lev == 5)
                        for (int k = 2; k <= nz; k++) s[q0 + k] = s[q0 + k] - x[q0 + k];
                    else
                        for (int k = 2; k <= nz; k++) s[q0 + k] = s[q0 + k] + w * x[q0 + k];
                }
        prev = cur;
        fields5 t = cur; cur = nxt; nxt = t;
    }
    /* E = |u - u_f|^2 (Filter.cpp:796-800 / 1471-1475) */
    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j <= ny; j++)
            for (int k = 2; k <= nz; k++) {
                const size_t q = IX(i, j, k);
                double Ue = U[1][q] / U[0][q] - acc.v[1][q] / acc.v[0][q];
                double Ve = U[2][q] / U[0][q] - acc.v[2][q] / acc.v[0][q];
                double We = U[3][q] / U[0][q] - acc.v[3][q] / acc.v[0][q];
                E[q] = Ue * Ue + Ve * Ve + We * We;
            }
    free5(gx); free5(gy); free5(l0); free5(l1); free5(acc);
}

/* ghost copies of E (Filter.cpp:1487-1555) */
static void fill_E(const cfo_grid *g, double *E)
{
    GRID_LOCALS(g);
    for (int j = 2; j <= ny; j++)
        for (int k = 2; k <= nz; k++) {
            E[IX(2, j, k)] = E[IX(3, j, k)];
            E[IX(gend + 1, j, k)] = E[IX(gend, j, k)];
        }
    for (int i = 3; i <= gend; i++)
        for (int k = 2; k <= nz; k++) {
            E[IX(i, 1, k)] = E[IX(i, 2, k)];
            E[IX(i, nyy, k)] = E[IX(i, ny, k)];
        }
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j <= ny; j++) {
            E[IX(i, j, 1)] = E[IX(i, j, 2)];
            E[IX(i, j, nzz)] = E[IX(i, j, nz)];
        }
}

/* arrays: U1_..U5_ (0-4), Y_point (5), EpX (6), EpY (7), EpZ (8), J (9) */
void cfo_Filter(const cfo_grid *g, double Roe_criterion, double E_high, double E_low, double **a)
{
    GRID_LOCALS(g);
    const size_t n = (size_t)(g->X_out + 6) * Ym * Zm;
    const double *Yp = a[5], *J = a[9];
    double *Eh = (double *)calloc(n, sizeof(double));
    double *E2h = (double *)calloc(n, sizeof(double));
    sensor_energy(g, a, J, Yp, 0, Eh, n);
    sensor_energy(g, a, J, Yp, 1, E2h, n);
    fill_E(g, Eh);
    fill_E(g, E2h);
    double *EpX = a[6], *EpY = a[7], *EpZ = a[8];
    #pragma omp parallel for collapse(2)
    for (int i = 2; i <= gend; i++)
        for (int j = 1; j < ny; j++)
            for (int k = 1; k < nz; k++) {
                double Emax = (Eh[IX(i, j + 1, k + 1)] + Eh[IX(i + 1, j + 1, k + 1)]) /
                              (E2h[IX(i, j + 1, k + 1)] + E2h[IX(i + 1, j + 1, k + 1)]);
                EpX[IX(i, j, k)] = Emax >= Roe_criterion ? E_high : E_low;
            }
    #pragma omp parallel for collapse(2)
    for (int i = 2; i <= gend - 1; i++)
        for (int j = 1; j < nyy; j++)
            for (int k = 1; k < nz; k++) {
                double Emax = (Eh[IX(i + 1, j, k + 1)] + Eh[IX(i + 1, j + 1, k + 1)]) /
                              (E2h[IX(i + 1, j, k + 1)] + E2h[IX(i + 1, j + 1, k + 1)]);
                EpY[IX(i, j, k)] = Emax >= Roe_criterion ? E_high : E_low;
            }
    #pragma omp parallel for collapse(2)
    for (int i = 2; i <= gend - 1; i++)
        for (int j = 1; j < ny; j++)
            for (int k = 1; k < nzz; k++) {
                double Emax = (Eh[IX(i + 1, j + 1, k)] + Eh[IX(i + 1, j + 1, k + 1)]) /
                              (E2h[IX(i + 1, j + 1, k)] + E2h[IX(i + 1, j + 1, k + 1)]);
                EpZ[IX(i, j, k)] = Emax >= Roe_criterion ? E_high : E_low;
            }
    free(Eh);
    free(E2h);
}
