/*
 * CPU oracle (test infrastructure): the reference's viscous terms
 * (Viscous_terms.cpp:15-886), restated in C.  See cf_oracle.h.
 *
 * Structure kept from the reference: for every cell (i,j,k) with
 * i = 3..gend+1, j = 2..nyy, k = 2..nzz the three face fluxes on its low
 * x, y and z faces are formed (LL*, ML*, NL* = x, y, z faces) from
 * primitive values of a 13-cell neighbourhood; then the divergence gives
 * vF2..vF5 on the interior.  The primitive conversion of each cell is done
 * once into scratch arrays here; the reference repeats it per neighbour
 * with the same expression, so the values are identical.
 */
#include "cf_oracle_common.h"

/* slots of the 79-array signature (main.h:525) */
enum { V_U = 0, V_VF = 5, V_J = 9, V_M = 10, V_JU = 19, V_MU = 20, V_JV = 29, V_MV = 30,
       V_JW = 39, V_MW = 40, V_LR = 49, V_LL = 54, V_MR = 59, V_ML = 64, V_NR = 69, V_NL = 74 };

/* symmetric and cross coefficient sets of one face (Viscous_terms.cpp:471-526) */
typedef struct { double s1, s2, s3, s4, s5, s6, s7; } symc;
typedef struct { double x1, x2, x3, x4, x5, x6, x7, x8, x9, x10; } crossc;

static inline symc sym_coef(double p0, double p1, double p2)
{
    symc c;
    c.s1 = (4. / 3) * p0 * p0 + p1 * p1 + p2 * p2;
    c.s2 = p0 * p0 + (4. / 3) * p1 * p1 + p2 * p2;
    c.s3 = p0 * p0 + p1 * p1 + (4. / 3) * p2 * p2;
    c.s4 = p0 * p0 + p1 * p1 + p2 * p2;
    c.s5 = (1. / 3) * p0 * p1;
    c.s6 = (1. / 3) * p1 * p2;
    c.s7 = (1. / 3) * p0 * p2;
    return c;
}

static inline crossc cross_coef(double p0, double p1, double p2, double q0, double q1, double q2)
{
    crossc c;
    c.x1 = (4. / 3) * p0 * q0 + p1 * q1 + p2 * q2;
    c.x2 = p0 * q0 + (4. / 3) * p1 * q1 + p2 * q2;
    c.x3 = p0 * q0 + p1 * q1 + (4. / 3) * p2 * q2;
    c.x4 = p0 * q0 + p1 * q1 + p2 * q2;
    c.x5 = p0 * q1 - (2. / 3) * p1 * q0;
    c.x6 = p0 * q2 - (2. / 3) * p2 * q0;
    c.x7 = p1 * q0 - (2. / 3) * p0 * q1;
    c.x8 = p1 * q2 - (2. / 3) * p2 * q1;
    c.x9 = p2 * q0 - (2. / 3) * p0 * q2;
    c.x10 = p2 * q1 - (2. / 3) * p1 * q2;
    return c;
}

/* gradients along one computational direction */
typedef struct { double du, dv, dw, du2, dv2, dw2, duv, dvw, duw, dT; } grad;

/* one-sided difference between cell c and its low neighbour n */
static inline grad grad2(const double *c, const double *n, double inv)
{
    grad d;
    d.du = (c[0] - n[0]) * inv;
    d.dv = (c[1] - n[1]) * inv;
    d.dw = (c[2] - n[2]) * inv;
    d.du2 = (c[0] * c[0] - n[0] * n[0]) * inv;
    d.dv2 = (c[1] * c[1] - n[1] * n[1]) * inv;
    d.dw2 = (c[2] * c[2] - n[2] * n[2]) * inv;
    d.duv = (c[0] * c[1] - n[0] * n[1]) * inv;
    d.dvw = (c[1] * c[2] - n[1] * n[2]) * inv;
    d.duw = (c[0] * c[2] - n[0] * n[2]) * inv;
    d.dT = (c[3] - n[3]) * inv;
    return d;
}

/* four-point tangential difference (p + q - r - s) * inv; the mixed
 * products use the second factor from p2/q2/r2/s2, which lets the
 * reference's z-face y-derivative (Viscous_terms.cpp:728-730: kUj*iVj
 * where kUj*kVj is meant) be expressed with q2 = the (i-1,j+1,k) cell. */
static inline grad grad4(const double *p, const double *q, const double *r, const double *s,
                         const double *q2, double inv)
{
    grad d;
    d.du = (p[0] + q[0] - r[0] - s[0]) * inv;
    d.dv = (p[1] + q[1] - r[1] - s[1]) * inv;
    d.dw = (p[2] + q[2] - r[2] - s[2]) * inv;
    d.du2 = (p[0] * p[0] + q[0] * q[0] - r[0] * r[0] - s[0] * s[0]) * inv;
    d.dv2 = (p[1] * p[1] + q[1] * q[1] - r[1] * r[1] - s[1] * s[1]) * inv;
    d.dw2 = (p[2] * p[2] + q[2] * q[2] - r[2] * r[2] - s[2] * s[2]) * inv;
    d.duv = (p[0] * p[1] + q[0] * q2[1] - r[0] * r[1] - s[0] * s[1]) * inv;
    d.dvw = (p[1] * p[2] + q[1] * q2[2] - r[1] * r[2] - s[1] * s[2]) * inv;
    d.duw = (p[0] * p[2] + q[0] * q2[2] - r[0] * r[2] - s[0] * s[2]) * inv;
    d.dT = (p[3] + q[3] - r[3] - s[3]) * inv;
    return d;
}

/* Primitive (u, v, w, T) of every cell (Viscous_terms.cpp:261-267). */
static void primitives(const cfo_grid *g, double **a, double *pr)
{
    GRID_LOCALS(g);
    const double K = g->K, R = g->R;
    const double *J = a[V_J];
    const size_t n = (size_t)(g->X_out + 6) * Ym * Zm;
    #pragma omp parallel for
    for (size_t q = 0; q < n; q++) {
        double rho = a[V_U][q];
        double U = a[V_U + 1][q] / rho;
        double V = a[V_U + 2][q] / rho;
        double W = a[V_U + 3][q] / rho;
        double VV = U * U + V * V + W * W;
        double P = (a[V_U + 4][q] - 0.5 * rho * VV) * (K - 1) * J[q];
        double T = P / (rho * R) / J[q];
        pr[4 * q] = U; pr[4 * q + 1] = V; pr[4 * q + 2] = W; pr[4 * q + 3] = T;
    }
}

void cfo_Viscous_terms(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    const double K = g->K, Cv = g->Cv, mu_E = g->mu_L, Pr_E = g->Pr_L;
    const double invXI = 1. / (g->deltaXI), invET = 1. / (g->deltaET), invZT = 1. / (g->deltaZT);
    const double inv4XI = 1. / (4 * g->deltaXI), inv4ET = 1. / (4 * g->deltaET), inv4ZT = 1. / (4 * g->deltaZT);
    const size_t n = (size_t)(g->X_out + 6) * Ym * Zm;
    double *pr = (double *)malloc(4 * n * sizeof(double));
    primitives(g, a, pr);
#define PR(i, j, k) (pr + 4 * IX(i, j, k))

    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend + 1; i++)
        for (int j = 2; j <= nyy; j++)
            for (int k = 2; k <= nzz; k++) {
                const double *c = PR(i, j, k);
                const double *im = PR(i - 1, j, k), *jm = PR(i, j - 1, k), *km = PR(i, j, k - 1);
                const double *ip = PR(i + 1, j, k), *jp = PR(i, j + 1, k), *kp = PR(i, j, k + 1);
                const double *imjp = PR(i - 1, j + 1, k), *imkp = PR(i - 1, j, k + 1);
                const double *ipjm = PR(i + 1, j - 1, k), *ipkm = PR(i + 1, j, k - 1);
                const double *jmkp = PR(i, j - 1, k + 1), *jpkm = PR(i, j + 1, k - 1);
                const double *imjm = PR(i - 1, j - 1, k), *jmkm = PR(i, j - 1, k - 1), *imkm = PR(i - 1, j, k - 1);
                const size_t q = IX(i, j, k), f = IX(i - 1, j - 1, k - 1);

                /* ---- x face (Viscous_terms.cpp:400-547) ---- */
                {
                    grad X = grad2(c, im, invXI);
                    grad Y = grad4(jp, imjp, jm, imjm, imjp, inv4ET);
                    grad Z = grad4(kp, imkp, km, imkm, imkp, inv4ZT);
                    const double *m[9];
                    for (int t = 0; t < 9; t++) m[t] = &a[V_MU + t][f];
                    symc A = sym_coef(*m[0], *m[1], *m[2]);
                    crossc D = cross_coef(*m[0], *m[1], *m[2], *m[3], *m[4], *m[5]);
                    crossc E = cross_coef(*m[0], *m[1], *m[2], *m[6], *m[7], *m[8]);
                    double Ux = 0.5 * (c[0] + im[0]), Vx = 0.5 * (c[1] + im[1]), Wx = 0.5 * (c[2] + im[2]);
                    double Jf = a[V_JU][f];
                    a[V_LL + 1][q] = mu_E * (A.s1 * X.du + A.s5 * X.dv + A.s7 * X.dw +
                        D.x1 * Y.du + D.x7 * Y.dv + D.x9 * Y.dw +
                        E.x1 * Z.du + E.x7 * Z.dv + E.x9 * Z.dw) / Jf;
                    a[V_LL + 2][q] = mu_E * (A.s5 * X.du + A.s2 * X.dv + A.s6 * X.dw +
                        D.x5 * Y.du + D.x2 * Y.dv + D.x10 * Y.dw +
                        E.x5 * Z.du + E.x2 * Z.dv + E.x10 * Z.dw) / Jf;
                    a[V_LL + 3][q] = mu_E * (A.s7 * X.du + A.s6 * X.dv + A.s3 * X.dw +
                        D.x6 * Y.du + D.x8 * Y.dv + D.x3 * Y.dw +
                        E.x6 * Z.du + E.x8 * Z.dv + E.x3 * Z.dw) / Jf;
                    a[V_LL + 4][q] = mu_E * (0.5 * A.s1 * X.du2 + 0.5 * A.s2 * X.dv2 + 0.5 * A.s3 * X.dw2 + A.s5 * X.duv + A.s6 * X.dvw + A.s7 * X.duw + Cv * K * A.s4 * X.dT / (Pr_E) +
                        0.5 * D.x1 * Y.du2 + 0.5 * D.x2 * Y.dv2 + 0.5 * D.x3 * Y.dw2 + D.x5 * Vx * Y.du + D.x6 * Wx * Y.du + D.x7 * Ux * Y.dv + D.x8 * Wx * Y.dv + D.x9 * Ux * Y.dw + D.x10 * Vx * Y.dw + Cv * K * D.x4 * Y.dT / (Pr_E) +
                        0.5 * E.x1 * Z.du2 + 0.5 * E.x2 * Z.dv2 + 0.5 * E.x3 * Z.dw2 + E.x5 * Vx * Z.du + E.x6 * Wx * Z.du + E.x7 * Ux * Z.dv + E.x8 * Wx * Z.dv + E.x9 * Ux * Z.dw + E.x10 * Vx * Z.dw + Cv * K * E.x4 * Z.dT / (Pr_E)) / Jf;
                }
                /* ---- y face (Viscous_terms.cpp:550-695) ---- */
                {
                    grad X = grad4(ip, ipjm, im, imjm, ipjm, inv4XI);
                    grad Y = grad2(c, jm, invET);
                    grad Z = grad4(kp, jmkp, km, jmkm, jmkp, inv4ZT);
                    const double *m[9];
                    for (int t = 0; t < 9; t++) m[t] = &a[V_MV + t][f];
                    symc B = sym_coef(*m[3], *m[4], *m[5]);
                    crossc D = cross_coef(*m[0], *m[1], *m[2], *m[3], *m[4], *m[5]);
                    crossc F = cross_coef(*m[3], *m[4], *m[5], *m[6], *m[7], *m[8]);
                    double Uy = 0.5 * (c[0] + jm[0]), Vy = 0.5 * (c[1] + jm[1]), Wy = 0.5 * (c[2] + jm[2]);
                    double Jf = a[V_JV][f];
                    a[V_ML + 1][q] = mu_E * (D.x1 * X.du + D.x5 * X.dv + D.x6 * X.dw +
                        B.s1 * Y.du + B.s5 * Y.dv + B.s7 * Y.dw +
                        F.x1 * Z.du + F.x7 * Z.dv + F.x9 * Z.dw) / Jf;
                    a[V_ML + 2][q] = mu_E * (D.x7 * X.du + D.x2 * X.dv + D.x8 * X.dw +
                        B.s5 * Y.du + B.s2 * Y.dv + B.s6 * Y.dw +
                        F.x5 * Z.du + F.x2 * Z.dv + F.x10 * Z.dw) / Jf;
                    a[V_ML + 3][q] = mu_E * (D.x9 * X.du + D.x10 * X.dv + D.x3 * X.dw +
                        B.s7 * Y.du + B.s6 * Y.dv + B.s3 * Y.dw +
                        F.x6 * Z.du + F.x8 * Z.dv + F.x3 * Z.dw) / Jf;
                    a[V_ML + 4][q] = mu_E * (0.5 * B.s1 * Y.du2 + 0.5 * B.s2 * Y.dv2 + 0.5 * B.s3 * Y.dw2 + B.s5 * Y.duv + B.s6 * Y.dvw + B.s7 * Y.duw + Cv * K * B.s4 * Y.dT / (Pr_E) +
                        0.5 * D.x1 * X.du2 + 0.5 * D.x2 * X.dv2 + 0.5 * D.x3 * X.dw2 + D.x5 * Uy * X.dv + D.x6 * Uy * X.dw + D.x7 * Vy * X.du + D.x8 * Vy * X.dw + D.x9 * Wy * X.du + D.x10 * Wy * X.dv + Cv * K * D.x4 * X.dT / (Pr_E) +
                        0.5 * F.x1 * Z.du2 + 0.5 * F.x2 * Z.dv2 + 0.5 * F.x3 * Z.dw2 + F.x5 * Vy * Z.du + F.x6 * Wy * Z.du + F.x7 * Uy * Z.dv + F.x8 * Wy * Z.dv + F.x9 * Uy * Z.dw + F.x10 * Vy * Z.dw + Cv * K * F.x4 * Z.dT / (Pr_E)) / Jf;
                }
                /* ---- z face (Viscous_terms.cpp:698-841) ---- */
                {
                    grad X = grad4(ip, ipkm, im, imkm, ipkm, inv4XI);
                    /* kUj*iVj: the second factor of the (i,j+1,k-1) products
                     * is taken from the (i-1,j+1,k) cell (Viscous_terms.cpp:728-730) */
                    grad Y = grad4(jp, jpkm, jm, jmkm, imjp, inv4ET);
                    grad Z = grad2(c, km, invZT);
                    const double *m[9];
                    for (int t = 0; t < 9; t++) m[t] = &a[V_MW + t][f];
                    symc Cc = sym_coef(*m[6], *m[7], *m[8]);
                    crossc E = cross_coef(*m[0], *m[1], *m[2], *m[6], *m[7], *m[8]);
                    crossc F = cross_coef(*m[3], *m[4], *m[5], *m[6], *m[7], *m[8]);
                    double Uz = 0.5 * (c[0] + km[0]), Vz = 0.5 * (c[1] + km[1]), Wz = 0.5 * (c[2] + km[2]);
                    double Jf = a[V_JW][f];
                    a[V_NL + 1][q] = mu_E * (E.x1 * X.du + E.x5 * X.dv + E.x6 * X.dw +
                        F.x1 * Y.du + F.x5 * Y.dv + F.x6 * Y.dw +
                        Cc.s1 * Z.du + Cc.s5 * Z.dv + Cc.s7 * Z.dw) / Jf;
                    a[V_NL + 2][q] = mu_E * (E.x7 * X.du + E.x2 * X.dv + E.x8 * X.dw +
                        F.x7 * Y.du + F.x2 * Y.dv + F.x8 * Y.dw +
                        Cc.s5 * Z.du + Cc.s2 * Z.dv + Cc.s6 * Z.dw) / Jf;
                    a[V_NL + 3][q] = mu_E * (E.x9 * X.du + E.x10 * X.dv + E.x3 * X.dw +
                        F.x9 * Y.du + F.x10 * Y.dv + F.x3 * Y.dw +
                        Cc.s7 * Z.du + Cc.s6 * Z.dv + Cc.s3 * Z.dw) / Jf;
                    a[V_NL + 4][q] = mu_E * (0.5 * Cc.s1 * Z.du2 + 0.5 * Cc.s2 * Z.dv2 + 0.5 * Cc.s3 * Z.dw2 + Cc.s5 * Z.duv + Cc.s6 * Z.dvw + Cc.s7 * Z.duw + Cv * K * Cc.s4 * Z.dT / (Pr_E) +
                        0.5 * E.x1 * X.du2 + 0.5 * E.x2 * X.dv2 + 0.5 * E.x3 * X.dw2 + E.x5 * Uz * X.dv + E.x6 * Uz * X.dw + E.x7 * Vz * X.du + E.x8 * Vz * X.dw + E.x9 * Wz * X.du + E.x10 * Wz * X.dv + Cv * K * E.x4 * X.dT / (Pr_E) +
                        0.5 * F.x1 * Y.du2 + 0.5 * F.x2 * Y.dv2 + 0.5 * F.x3 * Y.dw2 + F.x5 * Uz * Y.dv + F.x6 * Uz * Y.dw + F.x7 * Vz * Y.du + F.x8 * Vz * Y.dw + F.x9 * Wz * Y.du + F.x10 * Wz * Y.dv + Cv * K * F.x4 * Y.dT / (Pr_E)) / Jf;
                }
            }
#undef PR
    free(pr);

    /* divergence (Viscous_terms.cpp:854-883) */
    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j <= ny; j++)
            for (int k = 2; k <= nz; k++) {
                const size_t q = IX(i, j, k);
                for (int v = 1; v < 5; v++) {
                    const double *LL = a[V_LL + v], *ML = a[V_ML + v], *NL = a[V_NL + v];
                    a[V_VF + v - 1][q] = (LL[IX(i + 1, j, k)] - LL[q]) * invXI +
                                         (ML[IX(i, j + 1, k)] - ML[q]) * invET +
                                         (NL[IX(i, j, k + 1)] - NL[q]) * invZT;
                }
            }
}
