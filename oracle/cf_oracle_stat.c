/*
 * CPU oracle (test infrastructure): the reference's Statistic routine
 * (Statistic.cpp:16-1159), restated in C.
 *
 * Per call it forms, on the y faces, the linear MUSCL states
 * (Statistic.cpp:139-290), the Roe averages of the ROE == 1 scheme and the
 * face quantities u_L, u_R, v_L, v_R, rho_L, rho_R, rho u V / J_v, the x
 * momentum Roe dissipation and the jump d(rho u) (:292-489), the viscous x
 * momentum flux of the y faces (:560-840), and the cell moments U, V, W,
 * UU, VV, WW, UV (:1053-1068); it adds their y-row sums to accumulators
 * that persist across calls (the reference's static arrays), reports the
 * wall shear-stress increments (:900-920), and every statistic_step steps
 * returns the averages of the ND and st files (:940-1140) and clears the
 * accumulators.  Sums run in the reference's loop order.
 *
 * Accumulator layout acc[]: 17 rows of Y_m doubles, rows 0..9 = ULm, URm,
 * VLm, VRm, rhoLm, rhoRm, RUVm, SXYm, Roe_Dm, dRLm (the ND file order),
 * rows 10..16 = Um, Vm, Wm, UUm, VVm, WWm, UVm (the st file order), then
 * SXY_bottom, SXY_up.
 */
#include "cf_oracle_common.h"

enum { S_U_ = 0, S_J = 5, S_JV = 6, S_M = 7, S_MR = 16, S_ML = 21, S_EPY = 26 };

/* primitive u, v, w, T of a cell (Statistic.cpp:598-735) */
static void prim(const cfo_grid *g, double **a, size_t q, double *u, double *v, double *w, double *T)
{
    const double K = g->K, R = g->R;
    const double *J = a[S_J];
    double rho = a[S_U_][q];
    double U = a[S_U_ + 1][q] / rho;
    double V = a[S_U_ + 2][q] / rho;
    double W = a[S_U_ + 3][q] / rho;
    double P = (a[S_U_ + 4][q] - 0.5 * rho * (U * U + V * V + W * W)) * (K - 1) * J[q];
    *u = U;
    *v = V;
    *w = W;
    *T = P / (rho * R) / J[q];
}

int cfo_Statistic(const cfo_grid *g, double *acc, int step, int iteration, int statistic_step, double **a,
                  double *shear, double *nd, double *st)
{
    GRID_LOCALS(g);
    (void)iteration;
    const double K = g->K;
    const size_t n = (size_t)(g->X_out + 6) * Ym * Zm;
    double *U1 = a[S_U_], *U2 = a[S_U_ + 1], *U3 = a[S_U_ + 2], *U4 = a[S_U_ + 3], *U5 = a[S_U_ + 4];
    double **Uv = a + S_U_;
    const double *J = a[S_J], *Jv = a[S_JV];
    double **MR = a + S_MR, **ML = a + S_ML;
    double *row[17];
    for (int r = 0; r < 17; r++) row[r] = acc + (size_t)r * Ym;
    double *SXY_bottom = acc + 17 * (size_t)Ym, *SXY_up = SXY_bottom + 1;
    (void)U2;
    (void)U3;
    (void)U4;
    (void)U5;

    /* linear MUSCL states of the y faces (Statistic.cpp:139-290), i = 2..gend */
    for (int i = 2; i <= gend; i++)
        for (int j = 4; j <= ny - 2; j++)
            for (int k = 2; k <= nz; k++) {
                double temp = 1. / (2 / J[IX(i, j - 2, k)] - 13 / J[IX(i, j - 1, k)] + 47 / J[IX(i, j, k)] +
                                    27 / J[IX(i, j + 1, k)] - 3 / J[IX(i, j + 2, k)]);
                for (int v = 0; v < 5; v++) {
                    const double *U = Uv[v];
                    ML[v][IX(i - 1, j, k - 1)] = temp * (2 * U[IX(i, j - 2, k)] - 13 * U[IX(i, j - 1, k)] +
                                                         47 * U[IX(i, j, k)] + 27 * U[IX(i, j + 1, k)] -
                                                         3 * U[IX(i, j + 2, k)]);
                }
                temp = 1. / (-3 / J[IX(i, j - 2, k)] + 27 / J[IX(i, j - 1, k)] + 47 / J[IX(i, j, k)] -
                             13 / J[IX(i, j + 1, k)] + 2 / J[IX(i, j + 2, k)]);
                for (int v = 0; v < 5; v++) {
                    const double *U = Uv[v];
                    MR[v][IX(i - 1, j - 1, k - 1)] = temp * (-3 * U[IX(i, j - 2, k)] + 27 * U[IX(i, j - 1, k)] +
                                                             47 * U[IX(i, j, k)] - 13 * U[IX(i, j + 1, k)] +
                                                             2 * U[IX(i, j + 2, k)]);
                }
            }
    for (int i = 2; i <= gend; i++)
        for (int k = 2; k <= nz; k++) {
            double temp;
            int j = 1;
            temp = 1. / (1 / J[IX(i, j, k)] + 1 / J[IX(i, j + 1, k)]);
            for (int v = 0; v < 5; v++) ML[v][IX(i - 1, j, k - 1)] = temp * (Uv[v][IX(i, j, k)] + Uv[v][IX(i, j + 1, k)]);
            j = 2;
            temp = 1. / (1 / J[IX(i, j, k)] + 1 / J[IX(i, j + 1, k)]);
            for (int v = 0; v < 5; v++) ML[v][IX(i - 1, j, k - 1)] = temp * (Uv[v][IX(i, j, k)] + Uv[v][IX(i, j + 1, k)]);
            temp = 1. / (1 / J[IX(i, j, k)] + 1 / J[IX(i, j + 1, k)]);
            for (int v = 0; v < 5; v++)
                MR[v][IX(i - 1, j - 1, k - 1)] = temp * (Uv[v][IX(i, j, k)] + Uv[v][IX(i, j + 1, k)]);
            j = 3;
            temp = 1. / (-1 / J[IX(i, j - 1, k)] + 5 / J[IX(i, j, k)] + 2 / J[IX(i, j + 1, k)]);
            for (int v = 0; v < 5; v++)
                ML[v][IX(i - 1, j, k - 1)] = temp * (-Uv[v][IX(i, j - 1, k)] + 5 * Uv[v][IX(i, j, k)] + 2 * Uv[v][IX(i, j + 1, k)]);
            temp = 1. / (2 / J[IX(i, j - 1, k)] + 5 / J[IX(i, j, k)] - 1 / J[IX(i, j + 1, k)]);
            for (int v = 0; v < 5; v++)
                MR[v][IX(i - 1, j - 1, k - 1)] = temp * (2 * Uv[v][IX(i, j - 1, k)] + 5 * Uv[v][IX(i, j, k)] - Uv[v][IX(i, j + 1, k)]);
            j = ny - 1;
            temp = 1. / (-1 / J[IX(i, j - 1, k)] + 5 / J[IX(i, j, k)] + 2 / J[IX(i, j + 1, k)]);
            for (int v = 0; v < 5; v++)
                ML[v][IX(i - 1, j, k - 1)] = temp * (-Uv[v][IX(i, j - 1, k)] + 5 * Uv[v][IX(i, j, k)] + 2 * Uv[v][IX(i, j + 1, k)]);
            temp = 1. / (2 / J[IX(i, j - 1, k)] + 5 / J[IX(i, j, k)] - 1 / J[IX(i, j + 1, k)]);
            for (int v = 0; v < 5; v++)
                MR[v][IX(i - 1, j - 1, k - 1)] = temp * (2 * Uv[v][IX(i, j - 1, k)] + 5 * Uv[v][IX(i, j, k)] - Uv[v][IX(i, j + 1, k)]);
            j = ny;
            temp = 1. / (1 / J[IX(i, j, k)] + 1 / J[IX(i, j - 1, k)]);
            for (int v = 0; v < 5; v++) ML[v][IX(i - 1, j, k - 1)] = temp * (Uv[v][IX(i, j, k)] + Uv[v][IX(i, j - 1, k)]);
            temp = 1. / (1 / J[IX(i, j, k)] + 1 / J[IX(i, j - 1, k)]);
            for (int v = 0; v < 5; v++)
                MR[v][IX(i - 1, j - 1, k - 1)] = temp * (Uv[v][IX(i, j, k)] + Uv[v][IX(i, j - 1, k)]);
            j = ny;
            temp = 1. / (1 / J[IX(i, j, k)] + 1 / J[IX(i, j + 1, k)]);
            for (int v = 0; v < 5; v++) MR[v][IX(i - 1, j, k - 1)] = temp * (Uv[v][IX(i, j, k)] + Uv[v][IX(i, j + 1, k)]);
        }

    /* y-face Roe quantities (Statistic.cpp:292-489, ROE == 1), i = 2..gend-1 */
    double *face = (double *)calloc(9 * n, sizeof(double));   /* MUL MUR MVL MVR MrhoL MrhoR MRUV MRoe_D MdRL */
    for (int i = 2; i <= gend - 1; i++)
        for (int j = 1; j < nyy; j++)
            for (int k = 1; k < nz; k++) {
                const size_t q = IX(i, j, k);
                double etx = a[S_M + 3][q], ety = a[S_M + 4][q], etz = a[S_M + 5][q];
                double insqr = 1.0 / sqrt(etx * etx + ety * ety + etz * etz);
                double ETx = etx * insqr;
                double _rho = ML[0][q];
                double _u = ML[1][q] / _rho;
                double _v = ML[2][q] / _rho;
                double _w = ML[3][q] / _rho;
                double _V = etx * _u + ety * _v + etz * _w;
                double _VV = _u * _u + _v * _v + _w * _w;
                double _P = (ML[4][q] - 0.5 * _rho * _VV) * (K - 1);
                double _C = K * _P / _rho;
                double _H = 0.5 * _VV + _C / (K - 1);
                double rho_ = MR[0][q];
                double u_ = MR[1][q] / rho_;
                double v_ = MR[2][q] / rho_;
                double w_ = MR[3][q] / rho_;
                double V_ = etx * u_ + ety * v_ + etz * w_;
                double VV_ = u_ * u_ + v_ * v_ + w_ * w_;
                double P_ = (MR[4][q] - 0.5 * rho_ * VV_) * (K - 1);
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
                double Fav2 = fabs(v * insqr) * dU2 + deltaU * rho * u + deltaP * ETx;
                face[0 * n + q] = _u;
                face[1 * n + q] = u_;
                face[2 * n + q] = _v;
                face[3 * n + q] = v_;
                face[4 * n + q] = _rho;
                face[5 * n + q] = rho_;
                face[6 * n + q] = 0.5 * (_rho * _u * _V + rho_ * u_ * V_) / Jv[q];
                face[7 * n + q] = 0.5 * Fav2 / insqr / Jv[q];
                face[8 * n + q] = dU2;
            }

    /* viscous x-momentum flux of the y faces (Statistic.cpp:560-840): MSXY[i][j-1][k] */
    double *msxy = (double *)calloc(n, sizeof(double));
    const double mu_E = g->mu_L;
    const double invET = 1. / (g->deltaET);
    const double inv4XI = 1. / (4 * g->deltaXI), inv4ZT = 1. / (4 * g->deltaZT);
    for (int i = 3; i <= gend + 1; i++)
        for (int j = 2; j <= nyy; j++)
            for (int k = 2; k <= nzz; k++) {
                double U, V, W, T, iU, iV, iW, iT, jU, jV, jW, jT, kU, kV, kW, kT, ijU, ijV, ijW, ijT;
                double jkU, jkV, jkW, jkT, Ui, Vi, Wi, Ti, Uk, Vk, Wk, Tk, jUi, jVi, jWi, jTi, jUk, jVk, jWk, jTk;
                prim(g, a, IX(i, j, k), &U, &V, &W, &T);
                prim(g, a, IX(i - 1, j, k), &iU, &iV, &iW, &iT);
                prim(g, a, IX(i, j - 1, k), &jU, &jV, &jW, &jT);
                prim(g, a, IX(i, j, k - 1), &kU, &kV, &kW, &kT);
                prim(g, a, IX(i - 1, j - 1, k), &ijU, &ijV, &ijW, &ijT);
                prim(g, a, IX(i, j - 1, k - 1), &jkU, &jkV, &jkW, &jkT);
                prim(g, a, IX(i + 1, j, k), &Ui, &Vi, &Wi, &Ti);
                prim(g, a, IX(i, j, k + 1), &Uk, &Vk, &Wk, &Tk);
                prim(g, a, IX(i + 1, j - 1, k), &jUi, &jVi, &jWi, &jTi);
                prim(g, a, IX(i, j - 1, k + 1), &jUk, &jVk, &jWk, &jTk);
                const size_t f = IX(i - 1, j - 1, k - 1);
                double xix = a[S_M + 0][f], xiy = a[S_M + 1][f], xiz = a[S_M + 2][f];
                double etx = a[S_M + 3][f], ety = a[S_M + 4][f], etz = a[S_M + 5][f];
                double ztx = a[S_M + 6][f], zty = a[S_M + 7][f], ztz = a[S_M + 8][f];
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
                double ML2 = mu_E * (d1 * du_dx + d5 * dv_dx + d6 * dw_dx + b1 * du_dy + b5 * dv_dy + b7 * dw_dy +
                                     f1 * du_dz + f7 * dv_dz + f9 * dw_dz) / Jv[f];
                ML[1][IX(i, j, k)] = ML2;
                msxy[IX(i, j - 1, k)] = ML2;
            }

    /* y-row sums (Statistic.cpp:843-885) */
    for (int j = 1; j < nyy; j++)
        for (int i = 2; i <= gend - 1; i++)
            for (int k = 1; k < nz; k++) {
                const size_t q = IX(i, j, k);
                row[0][j] = row[0][j] + face[0 * n + q];
                row[1][j] = row[1][j] + face[1 * n + q];
                row[2][j] = row[2][j] + face[2 * n + q];
                row[3][j] = row[3][j] + face[3 * n + q];
                row[4][j] = row[4][j] + face[4 * n + q];
                row[5][j] = row[5][j] + face[5 * n + q];
                row[6][j] = row[6][j] + face[6 * n + q];
                row[8][j] = row[8][j] + face[7 * n + q];
                row[9][j] = row[9][j] + face[8 * n + q];
            }
    for (int j = 1; j < nyy; j++)
        for (int i = 3; i <= gend; i++)
            for (int k = 2; k <= nz; k++) row[7][j] = row[7][j] + msxy[IX(i, j, k)];
    free(face);
    free(msxy);

    /* wall shear-stress increments (Statistic.cpp:900-920) */
    const double XZ = (double)g->X_out, ZZ = (double)g->Z_out;
    shear[0] = row[7][1] / XZ / ZZ - *SXY_bottom;
    shear[1] = row[7][ny] / XZ / ZZ - *SXY_up;
    *SXY_bottom = row[7][1] / XZ / ZZ;
    *SXY_up = row[7][ny] / XZ / ZZ;

    int wrote = 0;
    if (step % statistic_step == 0) {
        double inv = 1. / statistic_step / XZ / ZZ;
        for (int r = 0; r < 10; r++)
            for (int j = 0; j < Ym; j++) nd[(size_t)r * Ym + j] = j >= 1 && j <= ny ? row[r][j] * inv : 0.0;
        for (int r = 0; r < 10; r++)
            for (int j = 1; j <= ny; j++) row[r][j] = 0;
        *SXY_bottom = *SXY_up = 0;
        wrote = 1;
    }

    /* mean profile and turbulence intensities (Statistic.cpp:1053-1068) */
    for (int j = 2; j <= ny; j++)
        for (int i = 3; i <= gend; i++)
            for (int k = 2; k <= nz; k++) {
                const size_t q = IX(i, j, k);
                double U = a[S_U_ + 1][q] / U1[q];
                double V = a[S_U_ + 2][q] / U1[q];
                double W = a[S_U_ + 3][q] / U1[q];
                row[10][j] = row[10][j] + U;
                row[11][j] = row[11][j] + V;
                row[12][j] = row[12][j] + W;
                row[13][j] = row[13][j] + U * U;
                row[14][j] = row[14][j] + V * V;
                row[15][j] = row[15][j] + W * W;
                row[16][j] = row[16][j] + U * V;
            }
    if (step % statistic_step == 0) {
        double inv = 1. / statistic_step / XZ / ZZ;
        for (int r = 0; r < 7; r++)
            for (int j = 0; j < Ym; j++) st[(size_t)r * Ym + j] = j >= 2 && j <= ny ? row[10 + r][j] * inv : 0.0;
        for (int r = 10; r < 17; r++)
            for (int j = 2; j <= ny; j++) row[r][j] = 0;
    }
    return wrote;
}
