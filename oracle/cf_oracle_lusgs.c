/*
 * CPU oracle (test infrastructure): the reference's dual-time LU-SGS
 * (Dual_time_stepping.cpp:18-1364, hyperplane Gauss-Seidel), its Jacobi
 * variant (DPLUSGS.cpp:18-1238), the plane tables (Hyperplane.cpp:18-81),
 * the flat-wall face metrics (Jacobian_u/v/w.cpp) and the bulk-flow
 * integral (Driven_force.cpp:38-62), restated in C.  See cf_oracle.h.
 */
#include "cf_oracle_common.h"

/* slots of the 64-array dual-time signature (main.h:653) */
enum { D_U_ = 0, D_U = 5, D_UQ = 10, D_J = 15, D_M = 16, D_FX = 25, D_FY = 30, D_FZ = 35,
       D_VF = 40, D_MR = 44, D_NR = 49, D_NL = 54, D_RES = 59 };

/* ------------------------------------------------------------------------ */
/* Plane tables                                                              */
/* ------------------------------------------------------------------------ */

/* Hyperplane.cpp:50-78: cells of plane m = i+j+k listed i-major, ijk[]
 * 1-based; Nijk[m] = {index of the plane's last entry, plane size}. */
void cfo_Hyperplane(const cfo_grid *g, int *Nijk, int *ijk)
{
    GRID_LOCALS(g);
    int ii = 0;
    for (int m = 7; m <= gend + ny + nz; m++) {
        int mi = 0;
        for (int i = 3; i <= gend; i++)
            for (int j = 2; j < nyy; j++) {
                int k = m - i - j;
                if (k >= 2 && k < nzz) {
                    mi = mi + 1;
                    ii = ii + 1;
                    ijk[3 * ii] = i;
                    ijk[3 * ii + 1] = j;
                    ijk[3 * ii + 2] = k;
                }
            }
        Nijk[2 * m] = ii;
        Nijk[2 * m + 1] = mi;
    }
}

/* ------------------------------------------------------------------------ */
/* Pieces shared by both LU-SGS variants                                      */
/* ------------------------------------------------------------------------ */

typedef struct { double rho, u, v, w, VV, P, C, T, H, beta; } cstate;

/* primitive state of one cell (Dual_time_stepping.cpp:344-363) */
static inline cstate cell_state(double **a, size_t q, double K, double e)
{
    cstate s;
    const double *J = a[D_J];
    s.rho = a[D_U_][q] * J[q];
    s.u = a[D_U_ + 1][q] / a[D_U_][q];
    s.v = a[D_U_ + 2][q] / a[D_U_][q];
    s.w = a[D_U_ + 3][q] / a[D_U_][q];
    s.VV = s.u * s.u + s.v * s.v + s.w * s.w;
    s.P = (a[D_U_ + 4][q] * J[q] - 0.5 * s.rho * s.VV) * (K - 1);
    s.C = K * s.P / s.rho;
    s.T = s.P / s.rho;
    s.H = 0.5 * s.VV + s.C / (K - 1);
    s.beta = RMAX(s.VV / s.C, e);
    return s;
}

/* Split flux Jacobian of one neighbour cell along metric row (m0,m1,m2)
 * (Dual_time_stepping.cpp:619-651 for A, 669-700 for B and C).  The
 * x-direction entries 52..54 associate as 0.5*m*beta*T*(K-1), the y and z
 * ones as 0.5*beta*T*(K-1)*m, kept as written.  pl = "plus" entries,
 * mi = the five "minus" diagonal entries of the backward sweep. */
typedef struct { double p11, p12, p13, p14, p21, p22, p31, p33, p41, p44, p51, p52, p53, p54, p55;
                 double m11, m22, m33, m44, m55; } splitjac;

static inline splitjac split_jacobian(cstate s, double m0, double m1, double m2, int xform, double K)
{
    splitjac A;
    double U = m0 * s.u + m1 * s.v + m2 * s.w;
    double S = sqrt(U * U * (s.beta - 1) * (s.beta - 1) + 4 * s.beta * s.C * (m0 * m0 + m1 * m1 + m2 * m2));
    double lambda = ((s.beta + 1) * fabs(U) + S) / 2;
    double d = fabs(lambda);
    A.p11 = 0.5 * (s.beta * U + d);
    A.p12 = 0.5 * s.P * K * s.beta * m0;
    A.p13 = 0.5 * s.P * K * s.beta * m1;
    A.p14 = 0.5 * s.P * K * s.beta * m2;
    A.p21 = 0.5 * m0 / s.rho;
    A.p22 = 0.5 * (U + d);
    A.p31 = 0.5 * m1 / s.rho;
    A.p33 = 0.5 * (U + d);
    A.p41 = 0.5 * m2 / s.rho;
    A.p44 = 0.5 * (U + d);
    A.p51 = 0.5 * U * (K - 1) * (s.beta - 1) / s.rho / K;
    if (xform) {
        A.p52 = 0.5 * m0 * s.beta * s.T * (K - 1);
        A.p53 = 0.5 * m1 * s.beta * s.T * (K - 1);
        A.p54 = 0.5 * m2 * s.beta * s.T * (K - 1);
    } else {
        A.p52 = 0.5 * s.beta * s.T * (K - 1) * m0;
        A.p53 = 0.5 * s.beta * s.T * (K - 1) * m1;
        A.p54 = 0.5 * s.beta * s.T * (K - 1) * m2;
    }
    A.p55 = 0.5 * (U + d);
    A.m11 = 0.5 * (s.beta * U - d);
    A.m22 = 0.5 * (U - d);
    A.m33 = 0.5 * (U - d);
    A.m44 = 0.5 * (U - d);
    A.m55 = 0.5 * (U - d);
    return A;
}

/* diagonal of the preconditioned implicit operator at one cell
 * (Dual_time_stepping.cpp:447-489): d11, d22(=d33=d44=d55), d51 */
typedef struct { double d11, d22, d51; } diag;

static inline diag cell_diag(const cfo_grid *g, double **a, size_t q, cstate s, double deltaT)
{
    const double K = g->K;
    const double *m[9];
    for (int t = 0; t < 9; t++) m[t] = &a[D_M + t][q];
    double xix = *m[0], xiy = *m[1], xiz = *m[2], etx = *m[3], ety = *m[4], etz = *m[5];
    double ztx = *m[6], zty = *m[7], ztz = *m[8];
    double beta = s.beta, C = s.C;
    double U = xix * s.u + xiy * s.v + xiz * s.w;
    double V = etx * s.u + ety * s.v + etz * s.w;
    double W = ztx * s.u + zty * s.v + ztz * s.w;
    double Sx = sqrt(U * U * (beta - 1) * (beta - 1) + 4 * beta * C * (xix * xix + xiy * xiy + xiz * xiz));
    double Sy = sqrt(V * V * (beta - 1) * (beta - 1) + 4 * beta * C * (etx * etx + ety * ety + etz * etz));
    double Sz = sqrt(W * W * (beta - 1) * (beta - 1) + 4 * beta * C * (ztx * ztx + zty * zty + ztz * ztz));
    double lambdaX = ((beta + 1) * fabs(U) + Sx) / 2;
    double lambdaY = ((beta + 1) * fabs(V) + Sy) / 2;
    double lambdaZ = ((beta + 1) * fabs(W) + Sz) / 2;
    double lambda = lambdaX / g->deltaXI + lambdaY / g->deltaET + lambdaZ / g->deltaZT;
    diag d;
    d.d11 = 2 * deltaT / (3 * beta + 2 * lambda * deltaT);
    d.d22 = 2 * deltaT / (3 + 2 * lambda * deltaT);
    double temp1 = 6 * (K - 1) * (beta - 1) * deltaT;
    double temp2 = K * (3 + 2 * lambda * deltaT) * (3 * beta + 2 * lambda * deltaT) * s.rho;
    d.d51 = -temp1 / temp2;
    return d;
}

/* ghost planes of NL/NR set to zero: x planes 2 and gend+1, y rows 1 and
 * nyy, z columns 1 and nzz (Dual_time_stepping.cpp:195-316) */
static void zero_ghosts(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    for (int v = 0; v < 5; v++) {
        double *NL = a[D_NL + v], *NR = a[D_NR + v];
        for (int j = 1; j <= nyy; j++)
            for (int k = 1; k <= nzz; k++) {
                NL[IX(2, j, k)] = 0; NR[IX(2, j, k)] = 0;
                NL[IX(gend + 1, j, k)] = 0; NR[IX(gend + 1, j, k)] = 0;
            }
        for (int i = 2; i <= gend + 1; i++)
            for (int k = 1; k <= nzz; k++) {
                NL[IX(i, 1, k)] = 0; NR[IX(i, 1, k)] = 0;
                NL[IX(i, nyy, k)] = 0; NR[IX(i, nyy, k)] = 0;
            }
        for (int i = 2; i <= gend + 1; i++)
            for (int j = 1; j <= nyy; j++) {
                NL[IX(i, j, 1)] = 0; NR[IX(i, j, 1)] = 0;
                NL[IX(i, j, nzz)] = 0; NR[IX(i, j, nzz)] = 0;
            }
    }
}

/* BDF2 residual, Gamma^-1 and the first diagonal solve
 * (Dual_time_stepping.cpp:339-506; copy_nr: also NR = NL) */
static void assemble(const cfo_grid *g, double deltaT, double **a, int copy_nr)
{
    GRID_LOCALS(g);
    const double K = g->K, e = g->e, f = g->f;
    const double dXI = g->deltaXI, dET = g->deltaET, dZT = g->deltaZT;
    const double *J = a[D_J];
    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j < nyy; j++)
            for (int k = 2; k < nzz; k++) {
                const size_t q = IX(i, j, k);
                cstate s = cell_state(a, q, K, e);
                double rho = s.rho, u = s.u, v = s.v, w = s.w, VV = s.VV, T = s.T, H = s.H, beta = s.beta;
                double temp = rho * K;
                double d11 = -(H * (K - 1) + VV - K * (T + VV)) * beta;
                double d12 = -(K - 1) * u * beta;
                double d13 = -(K - 1) * v * beta;
                double d14 = -(K - 1) * w * beta;
                double d15 = (K - 1) * beta;
                double d21 = -u / rho, d22 = 1 / rho;
                double d31 = -v / rho, d33 = 1 / rho;
                double d41 = -w / rho, d44 = 1 / rho;
                double d51 = (K - 1) * (VV + K * T * beta + (K - 1) * VV * beta + H * (-1 + beta - K * beta)) / temp;
                double d52 = -(K - 1) * u * (1 + (K - 1) * beta) / temp;
                double d53 = -(K - 1) * v * (1 + (K - 1) * beta) / temp;
                double d54 = -(K - 1) * w * (1 + (K - 1) * beta) / temp;
                double d55 = (K - 1) * (1 + (K - 1) * beta) / temp;
                const size_t fx = IX(i, j - 1, k - 1), fx0 = IX(i - 1, j - 1, k - 1);
                const size_t fy = IX(i - 1, j, k - 1), fz = IX(i - 1, j - 1, k);
                double Rk[5];
                for (int n = 0; n < 5; n++) {
                    double Rp = -(3 * a[D_U_ + n][q] - 4 * a[D_U + n][q] + a[D_UQ + n][q]) / (2 * deltaT);
                    const double *Fx = a[D_FX + n], *Fy = a[D_FY + n], *Fz = a[D_FZ + n];
                    double Rf = -((Fx[fx] - Fx[fx0]) / dXI + (Fy[fy] - Fy[fx0]) / dET + (Fz[fz] - Fz[fx0]) / dZT);
                    Rk[n] = Rp + Rf;
                }
                Rk[1] = Rk[1] + a[D_VF][q] + f / J[q];
                Rk[2] = Rk[2] + a[D_VF + 1][q];
                Rk[3] = Rk[3] + a[D_VF + 2][q];
                Rk[4] = Rk[4] + a[D_VF + 3][q] + f * u / J[q];
                /* Gamma^-1 R with the structurally zero entries of the
                 * reference's full 5x5 product left out */
                double MR1 = (d11 * Rk[0] + d12 * Rk[1] + d13 * Rk[2] + d14 * Rk[3] + d15 * Rk[4]);
                double MR2 = (d21 * Rk[0] + d22 * Rk[1]);
                double MR3 = (d31 * Rk[0] + d33 * Rk[2]);
                double MR4 = (d41 * Rk[0] + d44 * Rk[3]);
                double MR5 = (d51 * Rk[0] + d52 * Rk[1] + d53 * Rk[2] + d54 * Rk[3] + d55 * Rk[4]);
                a[D_MR][q] = MR1; a[D_MR + 1][q] = MR2; a[D_MR + 2][q] = MR3;
                a[D_MR + 3][q] = MR4; a[D_MR + 4][q] = MR5;
                diag dg = cell_diag(g, a, q, s, deltaT);
                double nl[5] = {dg.d11 * MR1, dg.d22 * MR2, dg.d22 * MR3, dg.d22 * MR4,
                                dg.d51 * MR1 + dg.d22 * MR5};
                for (int n = 0; n < 5; n++) {
                    a[D_NL + n][q] = nl[n];
                    if (copy_nr) a[D_NR + n][q] = nl[n];
                }
            }
}

/* lower-neighbour product L*N of one cell (Dual_time_stepping.cpp:751-811):
 * A+ of cell i-1, B+ of cell j-1, C+ of cell k-1 applied to N there */
static inline void lower_product(const cfo_grid *g, double **a, double *const *N, int i, int j, int k,
                                 double *LL)
{
    GRID_LOCALS(g);
    const double K = g->K, e = g->e;
    const size_t qa = IX(i - 1, j, k), qb = IX(i, j - 1, k), qc = IX(i, j, k - 1);
    splitjac A = split_jacobian(cell_state(a, qa, K, e), a[D_M][qa], a[D_M + 1][qa], a[D_M + 2][qa], 1, K);
    splitjac B = split_jacobian(cell_state(a, qb, K, e), a[D_M + 3][qb], a[D_M + 4][qb], a[D_M + 5][qb], 0, K);
    splitjac Cc = split_jacobian(cell_state(a, qc, K, e), a[D_M + 6][qc], a[D_M + 7][qc], a[D_M + 8][qc], 0, K);
    const double dXI = g->deltaXI, dET = g->deltaET, dZT = g->deltaZT;
    LL[0] = (-A.p11 * N[0][qa] - A.p12 * N[1][qa] - A.p13 * N[2][qa] - A.p14 * N[3][qa]) / dXI +
            (-B.p11 * N[0][qb] - B.p12 * N[1][qb] - B.p13 * N[2][qb] - B.p14 * N[3][qb]) / dET +
            (-Cc.p11 * N[0][qc] - Cc.p12 * N[1][qc] - Cc.p13 * N[2][qc] - Cc.p14 * N[3][qc]) / dZT;
    LL[1] = (-A.p21 * N[0][qa] - A.p22 * N[1][qa]) / dXI +
            (-B.p21 * N[0][qb] - B.p22 * N[1][qb]) / dET +
            (-Cc.p21 * N[0][qc] - Cc.p22 * N[1][qc]) / dZT;
    LL[2] = (-A.p31 * N[0][qa] - A.p33 * N[2][qa]) / dXI +
            (-B.p31 * N[0][qb] - B.p33 * N[2][qb]) / dET +
            (-Cc.p31 * N[0][qc] - Cc.p33 * N[2][qc]) / dZT;
    LL[3] = (-A.p41 * N[0][qa] - A.p44 * N[3][qa]) / dXI +
            (-B.p41 * N[0][qb] - B.p44 * N[3][qb]) / dET +
            (-Cc.p41 * N[0][qc] - Cc.p44 * N[3][qc]) / dZT;
    LL[4] = (-A.p51 * N[0][qa] - A.p52 * N[1][qa] - A.p53 * N[2][qa] - A.p54 * N[3][qa] - A.p55 * N[4][qa]) / dXI +
            (-B.p51 * N[0][qb] - B.p52 * N[1][qb] - B.p53 * N[2][qb] - B.p54 * N[3][qb] - B.p55 * N[4][qb]) / dET +
            (-Cc.p51 * N[0][qc] - Cc.p52 * N[1][qc] - Cc.p53 * N[2][qc] - Cc.p54 * N[3][qc] - Cc.p55 * N[4][qc]) / dZT;
}

/* upper-neighbour product U*N (Dual_time_stepping.cpp:1116-1177): the
 * split Jacobians of cells i+1, j+1, k+1 with their minus diagonals */
static inline void upper_product(const cfo_grid *g, double **a, double *const *N, int i, int j, int k,
                                 double *UU)
{
    GRID_LOCALS(g);
    const double K = g->K, e = g->e;
    const size_t qa = IX(i + 1, j, k), qb = IX(i, j + 1, k), qc = IX(i, j, k + 1);
    splitjac A = split_jacobian(cell_state(a, qa, K, e), a[D_M][qa], a[D_M + 1][qa], a[D_M + 2][qa], 1, K);
    splitjac B = split_jacobian(cell_state(a, qb, K, e), a[D_M + 3][qb], a[D_M + 4][qb], a[D_M + 5][qb], 0, K);
    splitjac Cc = split_jacobian(cell_state(a, qc, K, e), a[D_M + 6][qc], a[D_M + 7][qc], a[D_M + 8][qc], 0, K);
    const double dXI = g->deltaXI, dET = g->deltaET, dZT = g->deltaZT;
    UU[0] = (+A.m11 * N[0][qa] + A.p12 * N[1][qa] + A.p13 * N[2][qa] + A.p14 * N[3][qa]) / dXI +
            (+B.m11 * N[0][qb] + B.p12 * N[1][qb] + B.p13 * N[2][qb] + B.p14 * N[3][qb]) / dET +
            (+Cc.m11 * N[0][qc] + Cc.p12 * N[1][qc] + Cc.p13 * N[2][qc] + Cc.p14 * N[3][qc]) / dZT;
    UU[1] = (+A.p21 * N[0][qa] + A.m22 * N[1][qa]) / dXI +
            (+B.p21 * N[0][qb] + B.m22 * N[1][qb]) / dET +
            (+Cc.p21 * N[0][qc] + Cc.m22 * N[1][qc]) / dZT;
    UU[2] = (+A.p31 * N[0][qa] + A.m33 * N[2][qa]) / dXI +
            (+B.p31 * N[0][qb] + B.m33 * N[2][qb]) / dET +
            (+Cc.p31 * N[0][qc] + Cc.m33 * N[2][qc]) / dZT;
    UU[3] = (+A.p41 * N[0][qa] + A.m44 * N[3][qa]) / dXI +
            (+B.p41 * N[0][qb] + B.m44 * N[3][qb]) / dET +
            (+Cc.p41 * N[0][qc] + Cc.m44 * N[3][qc]) / dZT;
    UU[4] = (+A.p51 * N[0][qa] + A.p52 * N[1][qa] + A.p53 * N[2][qa] + A.p54 * N[3][qa] + A.m55 * N[4][qa]) / dXI +
            (+B.p51 * N[0][qb] + B.p52 * N[1][qb] + B.p53 * N[2][qb] + B.p54 * N[3][qb] + B.m55 * N[4][qb]) / dET +
            (+Cc.p51 * N[0][qc] + Cc.p52 * N[1][qc] + Cc.p53 * N[2][qc] + Cc.p54 * N[3][qc] + Cc.m55 * N[4][qc]) / dZT;
}

/* primitive update, residual arrays and the Sum(Delta^2)^2 norms
 * (Dual_time_stepping.cpp:1288-1352); the sums run serially in the
 * reference's i, j, k order */
static void update_and_norm(const cfo_grid *g, double **a, double *er)
{
    GRID_LOCALS(g);
    const double K = g->K;
    const double *J = a[D_J];
    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j < nyy; j++)
            for (int k = 2; k < nzz; k++) {
                const size_t q = IX(i, j, k);
                double rhoold = a[D_U_][q] * J[q];
                double Uold = a[D_U_ + 1][q] / a[D_U_][q];
                double Vold = a[D_U_ + 2][q] / a[D_U_][q];
                double Wold = a[D_U_ + 3][q] / a[D_U_][q];
                double VVold = Uold * Uold + Vold * Vold + Wold * Wold;
                double Pold = (a[D_U_ + 4][q] * J[q] - 0.5 * rhoold * VVold) * (K - 1);
                double Told = Pold / rhoold;
                double P = Pold + a[D_NR][q] * J[q];
                double U = Uold + a[D_NR + 1][q] * J[q];
                double V = Vold + a[D_NR + 2][q] * J[q];
                double W = Wold + a[D_NR + 3][q] * J[q];
                double T = Told + a[D_NR + 4][q] * J[q];
                double rho = P / T;
                a[D_U_][q] = rho / J[q];
                a[D_U_ + 1][q] = rho * U / J[q];
                a[D_U_ + 2][q] = rho * V / J[q];
                a[D_U_ + 3][q] = rho * W / J[q];
                a[D_U_ + 4][q] = (P / (K - 1) + 0.5 * rho * (U * U + V * V + W * W)) / J[q];
                a[D_RES][q] = (P - Pold) * (P - Pold);
                a[D_RES + 1][q] = (U - Uold) * (U - Uold);
                a[D_RES + 2][q] = (V - Vold) * (V - Vold);
                a[D_RES + 3][q] = (W - Wold) * (W - Wold);
                a[D_RES + 4][q] = (T - Told) * (T - Told);
            }
    double e[5] = {0, 0, 0, 0, 0};
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j <= ny; j++)
            for (int k = 2; k <= nz; k++)
                for (int n = 0; n < 5; n++) {
                    double r = a[D_RES + n][IX(i, j, k)];
                    e[n] = e[n] + r * r;
                }
    double DN = 1. / (g->X_out * g->Y_out * g->Z_out);
    for (int n = 0; n < 5; n++) er[n] = sqrt(e[n]) * DN;
}

static void copy_interior(const cfo_grid *g, double *const *dst, double *const *src)
{
    GRID_LOCALS(g);
    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j <= ny; j++)
            for (int v = 0; v < 5; v++)
                memcpy(&dst[v][IX(i, j, 2)], &src[v][IX(i, j, 2)], (size_t)(nz - 1) * sizeof(double));
}

/* ------------------------------------------------------------------------ */
/* Hyperplane LU-SGS                                                        */
/* ------------------------------------------------------------------------ */

void cfo_Dual_time_stepping(const cfo_grid *g, double deltaT, double *er,
                            const int *Nijk, const int *ijk, double **a)
{
    GRID_LOCALS(g);
    const double K = g->K, e = g->e;
    zero_ghosts(g, a);
    assemble(g, deltaT, a, 1);
    double *const *NL = &a[D_NL];
    double *const *NR = &a[D_NR];
    for (int sweep = 1; sweep <= 2; sweep++) {
        /* forward planes (Dual_time_stepping.cpp:563-881) */
        for (int m = 7; m <= gend + ny + nz; m++) {
            const int first = Nijk[2 * m] - Nijk[2 * m + 1] + 1, last = Nijk[2 * m];
            #pragma omp parallel for
            for (int mi = first; mi <= last; mi++) {
                const int i = ijk[3 * mi], j = ijk[3 * mi + 1], k = ijk[3 * mi + 2];
                const size_t q = IX(i, j, k);
                double LL[5];
                lower_product(g, a, NL, i, j, k, LL);
                cstate s = cell_state(a, q, K, e);
                diag dg = cell_diag(g, a, q, s, deltaT);
                const double *MR0 = a[D_MR], *MR1 = a[D_MR + 1], *MR2 = a[D_MR + 2];
                const double *MR3 = a[D_MR + 3], *MR4 = a[D_MR + 4];
                NL[0][q] = dg.d11 * (MR0[q] - LL[0]);
                NL[1][q] = dg.d22 * (MR1[q] - LL[1]);
                NL[2][q] = dg.d22 * (MR2[q] - LL[2]);
                NL[3][q] = dg.d22 * (MR3[q] - LL[3]);
                NL[4][q] = dg.d51 * (MR0[q] - LL[0]) + dg.d22 * (MR4[q] - LL[4]);
            }
        }
        /* backward planes (Dual_time_stepping.cpp:890-1250) */
        for (int m = gend + ny + nz; m >= 7; m--) {
            const int first = Nijk[2 * m] - Nijk[2 * m + 1] + 1, last = Nijk[2 * m];
            #pragma omp parallel for
            for (int mi = first; mi <= last; mi++) {
                const int i = ijk[3 * mi], j = ijk[3 * mi + 1], k = ijk[3 * mi + 2];
                const size_t q = IX(i, j, k);
                double UU[5];
                upper_product(g, a, NR, i, j, k, UU);
                cstate s = cell_state(a, q, K, e);
                diag dg = cell_diag(g, a, q, s, deltaT);
                NR[0][q] = NL[0][q] - dg.d11 * UU[0];
                NR[1][q] = NL[1][q] - dg.d22 * UU[1];
                NR[2][q] = NL[2][q] - dg.d22 * UU[2];
                NR[3][q] = NL[3][q] - dg.d22 * UU[3];
                NR[4][q] = NL[4][q] - (dg.d51 * UU[0] + dg.d22 * UU[4]);
            }
        }
        copy_interior(g, NL, NR);
    }
    update_and_norm(g, a, er);
}

/* ------------------------------------------------------------------------ */
/* Data-parallel (Jacobi) LU-SGS (DPLUSGS.cpp:313-1235)                      */
/* ------------------------------------------------------------------------ */

void cfo_DPLUSGS(const cfo_grid *g, double deltaT, double *er, double **a)
{
    GRID_LOCALS(g);
    const double K = g->K, e = g->e;
    zero_ghosts(g, a);
    assemble(g, deltaT, a, 0);
    double *const *NL = &a[D_NL];
    double *const *NR = &a[D_NR];
    for (int sweep = 1; sweep <= 4; sweep++) {
        #pragma omp parallel for collapse(2)
        for (int i = 3; i <= gend; i++)
            for (int j = 2; j < nyy; j++)
                for (int k = 2; k < nzz; k++) {
                    const size_t q = IX(i, j, k);
                    double LL[5], UU[5];
                    lower_product(g, a, NL, i, j, k, LL);
                    upper_product(g, a, NL, i, j, k, UU);
                    cstate s = cell_state(a, q, K, e);
                    diag dg = cell_diag(g, a, q, s, deltaT);
                    const double *MR0 = a[D_MR], *MR1 = a[D_MR + 1], *MR2 = a[D_MR + 2];
                    const double *MR3 = a[D_MR + 3], *MR4 = a[D_MR + 4];
                    NR[0][q] = dg.d11 * (MR0[q] - LL[0] - UU[0]);
                    NR[1][q] = dg.d22 * (MR1[q] - LL[1] - UU[1]);
                    NR[2][q] = dg.d22 * (MR2[q] - LL[2] - UU[2]);
                    NR[3][q] = dg.d22 * (MR3[q] - LL[3] - UU[3]);
                    NR[4][q] = dg.d51 * (MR0[q] - LL[0] - UU[0]) + dg.d22 * (MR4[q] - LL[4] - UU[4]);
                }
        copy_interior(g, NL, NR);
    }
    update_and_norm(g, a, er);
}

/* ------------------------------------------------------------------------ */
/* Face metrics and the bulk-flow integral                                   */
/* ------------------------------------------------------------------------ */

/* analytic flat-wall metrics at wall-normal index j with offset joff
 * (Jacobian_u.cpp:57-97): writes etdy and J of one face */
static inline void stretch_metric(const cfo_grid *g, double gamma, double joff, int j,
                                  double *etdy, double *Jf)
{
    const double high = g->high;
    double temp = (0.5 * high) * (1 - 1. / tanh(gamma) * tanh(gamma * (1 - 2 * (j - joff) * g->deltaET)));
    double temp1 = (1 - temp / (0.5 * high)) * tanh(gamma);
    *etdy = tanh(gamma) / (2 * (0.5 * high) * gamma * (1 - temp1 * temp1));
    double temp2 = 1 / cosh(gamma * (1 - 2 * (j - joff) * g->deltaET));
    double ydet = high * gamma * 1. / tanh(gamma) * temp2 * temp2;
    *Jf = 1. / (1 * ydet * 1);
}

/* arrays: J_f, xidx..ztdz of the face set */
static void face_metrics(const cfo_grid *g, double gamma, double joff, double **a,
                         int i0, int i1, int j0, int j1, int k0, int k1)
{
    GRID_LOCALS(g);
    for (int i = i0; i <= i1; i++)
        for (int j = j0; j <= j1; j++)
            for (int k = k0; k <= k1; k++) {
                const size_t q = IX(i, j, k);
                double etdy, Jf;
                stretch_metric(g, gamma, joff, j, &etdy, &Jf);
                a[1][q] = 1; a[2][q] = 0; a[3][q] = 0;
                a[4][q] = 0; a[5][q] = etdy; a[6][q] = 0;
                a[7][q] = 0; a[8][q] = 0; a[9][q] = 1;
                a[0][q] = Jf;
            }
}

/* Jacobian_u.cpp:27-68: faces i = 2..gend, j = 1..ny-1, k = 1..nz-1, j-0.5 */
void cfo_Jacobian_u(const cfo_grid *g, double gamma, double **a)
{
    GRID_LOCALS(g);
    face_metrics(g, gamma, 0.5, a, 2, gend, 1, ny - 1, 1, nz - 1);
}

/* Jacobian_w.cpp:26-67: faces i = 2..gend-1, j = 1..ny-1, k = 1..nz, j-0.5 */
void cfo_Jacobian_w(const cfo_grid *g, double gamma, double **a)
{
    GRID_LOCALS(g);
    face_metrics(g, gamma, 0.5, a, 2, gend - 1, 1, ny - 1, 1, nz);
}

/* Jacobian_v.cpp:77-141: faces i = 2..gend-1, j = 1..ny, k = 1..nz-1 at
 * j-1.0, then the wall rows take the cell metrics' ghost rows
 * (etd* of rows 1 and nyy, J of rows 1 and nyy).  Arrays 0-9: J_v + 9 face
 * metrics, 10-19: J + 9 cell metrics. */
void cfo_Jacobian_v(const cfo_grid *g, double gamma, double **a)
{
    GRID_LOCALS(g);
    face_metrics(g, gamma, 1.0, a, 2, gend - 1, 1, ny, 1, nz - 1);
    for (int i = 2; i <= gend - 1; i++)
        for (int k = 1; k < nz; k++) {
            for (int t = 0; t < 3; t++) {
                a[4 + t][IX(i, 1, k)] = a[14 + t][IX(i, 1, k)];
                a[4 + t][IX(i, ny, k)] = a[14 + t][IX(i, nyy, k)];
            }
            a[0][IX(i, ny, k)] = a[10][IX(i, nyy, k)];
            a[0][IX(i, 1, k)] = a[10][IX(i, 1, k)];
        }
}

/* Driven_force.cpp:38-62: Q = sum over the interior of (U2_*J)/J/Jsum,
 * divided by X_out*Z_out (serial sum in i, j, k order) */
double cfo_Driven_force(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    const double *U2 = a[0], *J = a[1];
    double Jsum = 0, Q = 0;
    for (int j = 2; j <= ny; j++) Jsum = Jsum + 1. / J[IX(3, j, 3)];
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j < nyy; j++)
            for (int k = 2; k < nzz; k++) {
                double temp = (U2[IX(i, j, k)] * J[IX(i, j, k)]) * 1. / J[IX(i, j, k)] / Jsum;
                Q = Q + temp;
            }
    Q = Q / g->X_out / g->Z_out;
    return Q;
}
