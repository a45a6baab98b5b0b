/*
 * CPU oracle (test infrastructure): boundary conditions, the six inviscid
 * flux routines and the explicit RK3 update of the reference solver,
 * restated in C.  See cf_oracle.h for the layout and the bit-exactness rule.
 */
#include "cf_oracle_common.h"

/* ------------------------------------------------------------------------ */
/* Boundary conditions                                                       */
/* ------------------------------------------------------------------------ */

/* x ghost planes, periodic and 3 deep: planes 0..2 take the last interior
 * planes gend-2..gend, planes gend+1..gend+3 take the first interior planes
 * 3..5.  This is the single-domain form of the reference's halo exchange
 * plus periodic seam (main.cpp:156-244): with the whole domain on one
 * device every ghost plane is the periodic image. */
void cfo_x_periodic(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    const size_t plane = (size_t)Ym * Zm;
    for (int n = 0; n < 5; n++) {
        double *U = a[n];
        for (int s = 0; s < 3; s++) {
            memcpy(U + (size_t)s * plane, U + (size_t)(gend - 2 + s) * plane, plane * sizeof(double));
            memcpy(U + (size_t)(gend + 1 + s) * plane, U + (size_t)(3 + s) * plane, plane * sizeof(double));
        }
    }
}

/* Y_boundary_condition.cpp:48-120: isothermal no-slip wall ghosts j=1 and
 * j=nyy from the first interior rows j=2 and j=ny (pressure copied,
 * T_ghost = 2*298.0592 - T, velocity reversed). */
void cfo_Y_boundary_condition(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    double *U1 = a[0], *U2 = a[1], *U3 = a[2], *U4 = a[3], *U5 = a[4];
    const double *J = a[5];
    const double K = g->K, R = g->R;
    #pragma omp parallel for
    for (int i = 2; i <= gend + 1; i++) {
        for (int k = 2; k <= nz; k++) {
            for (int side = 0; side < 2; side++) {
                const int js = side == 0 ? 2 : ny;      /* interior row */
                const int jg = side == 0 ? 1 : nyy;     /* ghost row */
                const size_t s = IX(i, js, k), q = IX(i, jg, k);
                double rho = U1[s] * J[s];
                double U = U2[s] / U1[s];
                double V = U3[s] / U1[s];
                double W = U4[s] / U1[s];
                double VV = U * U + V * V + W * W;
                double P = (U5[s] * J[s] - 0.5 * rho * VV) * (K - 1);
                double temp = P / rho / R;
                double T = 2 * 298.0592 - temp;
                rho = P / R / T;
                U1[q] = P / R / T / J[q];
                U2[q] = -P / R / T * U / J[q];
                U3[q] = -P / R / T * V / J[q];
                U4[q] = -P / R / T * W / J[q];
                U5[q] = (rho * R * T / (K - 1) + 0.5 * P / R / T * VV) / J[q];
            }
        }
    }
}

/* Z_boundary_condition.cpp:48-67: one-deep periodic copy in z for every
 * row j = 0..nyyy of planes i = 2..gend+1. */
void cfo_Z_boundary_condition(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    for (int i = 2; i <= gend + 1; i++)
        for (int j = 0; j <= nyy + 1; j++)
            for (int n = 0; n < 5; n++) {
                double *U = a[n];
                U[IX(i, j, 1)] = U[IX(i, j, nz)];
                U[IX(i, j, nzz)] = U[IX(i, j, 2)];
            }
}

/* ------------------------------------------------------------------------ */
/* MUSCL reconstruction helpers                                             */
/* ------------------------------------------------------------------------ */

/* 3rd-order limiter value min(2, min(2r, (1+2r)/3)) (Flux_X_limiter.cpp:152-156) */
static inline double lim3(double r)
{
    double b = 1. / 3 * (1 + 2 * r);
    return RMIN(2, RMIN(2 * r, b));
}

/* 5th-order limiter value min(2, min(2r, b)), b = (-2/a + 11 + 24r - 3rc)/30
 * (Flux_X_limiter.cpp:255-259; for the left state a = r_{i-1}, c = r_{i+1},
 * for the right state a = 1/.. ratios as written there). */
static inline double lim5(double a_, double r, double c_)
{
    double b = 1. / 30 * (-2. / a_ + 11 + 24 * r - 3 * r * c_);
    return RMIN(2, RMIN(2 * r, b));
}

/* Limited left/right states from five cells iiu, iu, u, ui, uii (5th order)
 * with sign s of the left-state slope term (+1 in x and y, -1 in z:
 * Flux_Z_limiter.cpp:271 writes u - 0.5*phi*(u-iu)). */
static inline void muscl5(double iiu, double iu, double u, double ui, double uii, int s,
                          double jL, double jR, double *mL, double *mR)
{
    double irL = (u - iu) / (iu - iiu);
    double rL = (ui - u) / (u - iu);
    double rLi = (uii - ui) / (ui - u);
    double rRi = (ui - u) / (uii - ui);
    double rR = (u - iu) / (ui - u);
    double irR = (iu - iiu) / (u - iu);
    double minL3 = lim5(irL, rL, rLi);
    double minR3 = lim5(rRi, rR, irR);
    if (s > 0)
        *mL = (u + 0.5 * RMAX(0, minL3) * (u - iu)) * jL;
    else
        *mL = (u - 0.5 * RMAX(0, minL3) * (u - iu)) * jL;
    *mR = (u - 0.5 * RMAX(0, minR3) * (ui - u)) * jR;
}

static inline void muscl3(double iu, double u, double ui, int s, double jL, double jR,
                          double *mL, double *mR)
{
    double rL = (ui - u) / (u - iu);
    double rR = (u - iu) / (ui - u);
    double minL3 = lim3(rL);
    double minR3 = lim3(rR);
    if (s > 0)
        *mL = (u + 0.5 * RMAX(0, minL3) * (u - iu)) * jL;
    else
        *mL = (u - 0.5 * RMAX(0, minL3) * (u - iu)) * jL;
    *mR = (u - 0.5 * RMAX(0, minR3) * (ui - u)) * jR;
}

/* ------------------------------------------------------------------------ */
/* Face flux kernels                                                        */
/* ------------------------------------------------------------------------ */

/* Low-Mach preconditioned Roe flux of one face (Flux_X_limiter.cpp:373-536).
 * m[0..8] = xix,xiy,xiz,etx,ety,etz,ztx,zty,ztz at the face, dir selects the
 * normal metric row (0: xi, 1: eta, 2: zeta).  Writes the five fluxes. */
static void flux_precond_roe(const double *mL, const double *mR, const double *m, int dir,
                             double Ep, double Jf, double K, double e, double *F)
{
    const double n0 = m[3 * dir], n1 = m[3 * dir + 1], n2 = m[3 * dir + 2];
    double NX = n0 / (sqrt(n0 * n0 + n1 * n1 + n2 * n2));
    double NY = n1 / (sqrt(n0 * n0 + n1 * n1 + n2 * n2));
    double NZ = n2 / (sqrt(n0 * n0 + n1 * n1 + n2 * n2));

    double _rho = mL[0];
    double _u = mL[1] / _rho;
    double _v = mL[2] / _rho;
    double _w = mL[3] / _rho;
    double _U = n0 * _u + n1 * _v + n2 * _w;
    double __U = NX * _u + NY * _v + NZ * _w;
    double _VV = _u * _u + _v * _v + _w * _w;
    double _P = (mL[4] - 0.5 * _rho * _VV) * (K - 1);
    double _T = _P / _rho;
    double _C = K * _P / _rho;
    double _H = 0.5 * _VV + _C / (K - 1);

    double rho_ = mR[0];
    double u_ = mR[1] / rho_;
    double v_ = mR[2] / rho_;
    double w_ = mR[3] / rho_;
    double U_ = n0 * u_ + n1 * v_ + n2 * w_;
    double U__ = NX * u_ + NY * v_ + NZ * w_;
    double VV_ = u_ * u_ + v_ * v_ + w_ * w_;
    double P_ = (mR[4] - 0.5 * rho_ * VV_) * (K - 1);
    double T_ = P_ / rho_;
    double C_ = K * P_ / rho_;
    double H_ = 0.5 * VV_ + C_ / (K - 1);

    double rho = 0.5 * (_rho + rho_);
    double u = 0.5 * (_u + u_);
    double v = 0.5 * (_v + v_);
    double w = 0.5 * (_w + w_);
    double U = 0.5 * (_U + U_);
    double _U_ = 0.5 * (__U + U__);
    double VV = u * u + v * v + w * w;
    double H = 0.5 * (_H + H_);
    double C = (H - 0.5 * VV) * (K - 1);
    double P = rho * C / K;
    double T = P / rho;

    double dU1 = P_ - _P, dU2 = u_ - _u, dU3 = v_ - _v, dU4 = w_ - _w, dU5 = T_ - _T;

    double beta = RMAX(VV / C, e);
    double S = sqrt(U * U * (beta - 1) * (beta - 1) + 4 * beta * C * (n0 * n0 + n1 * n1 + n2 * n2));
    double _S_ = sqrt(_U_ * _U_ * (beta - 1) * (beta - 1) + 4 * beta * C * (NX * NX + NY * NY + NZ * NZ));

    double temp = 4 * K * _S_ * T * beta;
    double temp1 = S + U + U * beta;
    double temp2 = -S + U + U * beta;
    double temp3 = _S_ - _U_ + _U_ * beta;
    double temp4 = _S_ + _U_ - _U_ * beta;
    double temp5 = _S_ * _S_ - (beta - 1) * (beta - 1) * _U_ * _U_;
    double tempu1 = 2 * T * NX * K * beta + u * _S_ + u * (beta - 1) * _U_;
    double tempu2 = 2 * T * NX * K * beta - u * _S_ + u * (beta - 1) * _U_;
    double tempv1 = 2 * T * NY * K * beta + v * _S_ + v * (beta - 1) * _U_;
    double tempv2 = 2 * T * NY * K * beta - v * _S_ + v * (beta - 1) * _U_;
    double tempw1 = 2 * T * NZ * K * beta + w * _S_ + w * (beta - 1) * _U_;
    double tempw2 = 2 * T * NZ * K * beta - w * _S_ + w * (beta - 1) * _U_;
    double tempuvw = 2 * T * K * beta * (u * NX + v * NY + w * NZ);
    double temph1 = tempuvw + H * _S_ + H * _U_ * beta - H * _U_;
    double temph2 = tempuvw - H * _S_ + H * _U_ * beta - H * _U_;
    double aU = fabs(U), a1 = fabs(temp1), a2 = fabs(temp2);

    double d11 = 1 / temp * (4 * (K - 1) * _S_ * beta * aU + temp3 * a1 + temp4 * a2);
    double d12 = -1 / (2 * temp) * (NX * rho * (a2 - a1) * temp5);
    double d13 = -1 / (2 * temp) * (NY * rho * (a2 - a1) * temp5);
    double d14 = -1 / (2 * temp) * (NZ * rho * (a2 - a1) * temp5);
    double d15 = -rho * aU / T;

    double d21 = 1 / temp * (u * _S_ * (4 * (K - 1) * beta * aU + a2 + a1) - (a2 - a1) * (2 * T * NX * K * beta + u * _U_ * (beta - 1)));
    double d22 = 1 / (2 * temp) * (rho * (8 * T * K * _S_ * beta * (NY * NY + NZ * NZ) * aU + NX * (temp3 * tempu2 * a2 + temp4 * tempu1 * a1)));
    double d23 = 1 / (2 * temp) * (rho * NY * (-8 * T * K * _S_ * beta * NX * aU + temp3 * tempu2 * a2 + temp4 * tempu1 * a1));
    double d24 = 1 / (2 * temp) * (rho * NZ * (-8 * T * K * _S_ * beta * NX * aU + temp3 * tempu2 * a2 + temp4 * tempu1 * a1));
    double d25 = -u * rho * aU / T;

    double d31 = 1 / temp * (v * _S_ * (4 * (K - 1) * beta * aU + a2 + a1) - (a2 - a1) * (2 * T * NY * K * beta + v * _U_ * (beta - 1)));
    double d32 = 1 / (2 * temp) * (rho * NX * (-8 * T * K * _S_ * beta * NY * aU + temp3 * tempv2 * a2 + temp4 * tempv1 * a1));
    double d33 = 1 / (2 * temp) * (rho * (8 * T * K * _S_ * beta * (NX * NX + NZ * NZ) * aU + NY * (temp3 * tempv2 * a2 + temp4 * tempv1 * a1)));
    double d34 = 1 / (2 * temp) * (rho * NZ * (-8 * T * K * _S_ * beta * NY * aU + temp3 * tempv2 * a2 + temp4 * tempv1 * a1));
    double d35 = -v * rho * aU / T;

    double d41 = 1 / temp * (w * _S_ * (4 * (K - 1) * beta * aU + a2 + a1) - (a2 - a1) * (2 * T * NZ * K * beta + w * _U_ * (beta - 1)));
    double d42 = 1 / (2 * temp) * (rho * NX * (-8 * T * K * _S_ * beta * NZ * aU + temp3 * tempw2 * a2 + temp4 * tempw1 * a1));
    double d43 = 1 / (2 * temp) * (rho * NY * (-8 * T * K * _S_ * beta * NZ * aU + temp3 * tempw2 * a2 + temp4 * tempw1 * a1));
    double d44 = 1 / (2 * temp) * (rho * (8 * T * K * _S_ * beta * (NX * NX + NY * NY) * aU + NZ * (temp3 * tempw2 * a2 + temp4 * tempw1 * a1)));
    double d45 = -w * rho * aU / T;

    double d51 = 1 / temp * (_S_ * (4 * beta * (H * K - H - T * K) * aU + H * (a2 + a1)) - (a2 - a1) * (tempuvw + H * _U_ * beta - H * _U_));
    double d52 = 1 / (2 * temp) * (rho * (8 * T * K * _S_ * beta * (-v * NX * NY - w * NX * NZ + u * (NY * NY + NZ * NZ) * aU) + NX * (temph2 * temp3 * a2 + temph1 * temp4 * a1)));
    double d53 = 1 / (2 * temp) * (rho * (8 * T * K * _S_ * beta * (-u * NX * NY - w * NY * NZ + v * (NX * NX + NZ * NZ) * aU) + NY * (temph2 * temp3 * a2 + temph1 * temp4 * a1)));
    double d54 = 1 / (2 * temp) * (rho * (8 * T * K * _S_ * beta * (-u * NX * NZ - v * NY * NZ + w * (NX * NX + NY * NY) * aU) + NZ * (temph2 * temp3 * a2 + temph1 * temp4 * a1)));
    double d55 = (-H / T + K / (K - 1)) * rho * aU;

    double Fav1 = d11 * dU1 + d12 * dU2 + d13 * dU3 + d14 * dU4 + d15 * dU5;
    double Fav2 = d21 * dU1 + d22 * dU2 + d23 * dU3 + d24 * dU4 + d25 * dU5;
    double Fav3 = d31 * dU1 + d32 * dU2 + d33 * dU3 + d34 * dU4 + d35 * dU5;
    double Fav4 = d41 * dU1 + d42 * dU2 + d43 * dU3 + d44 * dU4 + d45 * dU5;
    double Fav5 = d51 * dU1 + d52 * dU2 + d53 * dU3 + d54 * dU4 + d55 * dU5;

    F[0] = 0.5 * ((_rho * _U + rho_ * U_) - Ep * Fav1) / Jf;
    F[1] = 0.5 * ((_rho * _u * _U + rho_ * u_ * U_ + n0 * (_P + P_)) - Ep * Fav2) / Jf;
    F[2] = 0.5 * ((_rho * _v * _U + rho_ * v_ * U_ + n1 * (_P + P_)) - Ep * Fav3) / Jf;
    F[3] = 0.5 * ((_rho * _w * _U + rho_ * w_ * U_ + n2 * (_P + P_)) - Ep * Fav4) / Jf;
    F[4] = 0.5 * ((_U * (3.5 * _P + 0.5 * _rho * _VV) + U_ * (3.5 * P_ + 0.5 * rho_ * VV_)) - Ep * Fav5) / Jf;
    /* the wall faces of Flux_Y_limiter (j = 1, ny) keep only the pressure
     * term of the wall-normal momentum flux (Flux_Y_limiter.cpp:658-666) */
    F[5] = 0.5 * (n1 * (_P + P_) - Ep * Fav3) / Jf;
}

/* Roe flux (ROE == 1, Pre_selection.h:6) of one face (Flux_X.cpp:247-420).
 * The energy dissipation term differs per direction: deltaP*U in x and z,
 * deltaP*V*insqr in y (Flux_Y.cpp:383). */
static void flux_roe(const double *mL, const double *mR, const double *m, int dir,
                     double Jf, double K, double *F)
{
    const double n0 = m[3 * dir], n1 = m[3 * dir + 1], n2 = m[3 * dir + 2];
    double insqr = 1.0 / sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    double NX = n0 * insqr, NY = n1 * insqr, NZ = n2 * insqr;

    double _rho = mL[0];
    double _u = mL[1] / _rho;
    double _v = mL[2] / _rho;
    double _w = mL[3] / _rho;
    double _U = n0 * _u + n1 * _v + n2 * _w;
    double _VV = _u * _u + _v * _v + _w * _w;
    double _P = (mL[4] - 0.5 * _rho * _VV) * (K - 1);
    double _C = K * _P / _rho;
    double _H = 0.5 * _VV + _C / (K - 1);

    double rho_ = mR[0];
    double u_ = mR[1] / rho_;
    double v_ = mR[2] / rho_;
    double w_ = mR[3] / rho_;
    double U_ = n0 * u_ + n1 * v_ + n2 * w_;
    double VV_ = u_ * u_ + v_ * v_ + w_ * w_;
    double P_ = (mR[4] - 0.5 * rho_ * VV_) * (K - 1);
    double C_ = K * P_ / rho_;
    double H_ = 0.5 * VV_ + C_ / (K - 1);

    double temp5 = sqrt(_rho);
    double temp6 = sqrt(rho_);
    double temp4 = temp5 + temp6;
    double rho = sqrt(_rho * rho_);
    double u = (temp5 * _u + temp6 * u_) / temp4;
    double v = (temp5 * _v + temp6 * v_) / temp4;
    double w = (temp5 * _w + temp6 * w_) / temp4;
    double U = (temp5 * _U + temp6 * U_) / temp4;
    double VV = u * u + v * v + w * w;
    double H = (temp5 * _H + temp6 * H_) / temp4;
    double C = (H - 0.5 * VV) * (K - 1);

    double dU1 = rho_ - _rho;
    double dU2 = rho_ * u_ - _rho * _u;
    double dU3 = rho_ * v_ - _rho * _v;
    double dU4 = rho_ * w_ - _rho * _w;
    double dU5 = (P_ / (K - 1) + 0.5 * rho_ * VV_) - (_P / (K - 1) + 0.5 * _rho * _VV);

    double S = sqrt(C);
    double temp1 = (P_ - _P) / rho / C;
    double temp2 = U * insqr / S * (U_ - _U) * insqr;
    double deltaU = (S - fabs(U * insqr)) * temp1 + temp2;
    double deltaP = U * insqr / S * (P_ - _P) + (S - fabs(U * insqr)) * rho * (U_ - _U) * insqr;

    double Fav1 = fabs(U * insqr) * dU1 + deltaU * rho;
    double Fav2 = fabs(U * insqr) * dU2 + deltaU * rho * u + deltaP * NX;
    double Fav3 = fabs(U * insqr) * dU3 + deltaU * rho * v + deltaP * NY;
    double Fav4 = fabs(U * insqr) * dU4 + deltaU * rho * w + deltaP * NZ;
    double Fav5 = dir == 1 ? fabs(U * insqr) * dU5 + deltaU * rho * H + deltaP * U * insqr
                           : fabs(U * insqr) * dU5 + deltaU * rho * H + deltaP * U;

    F[0] = 0.5 * ((_rho * _U + rho_ * U_) - Fav1 / insqr) / Jf;
    F[1] = 0.5 * ((_rho * _u * _U + rho_ * u_ * U_ + n0 * (_P + P_)) - Fav2 / insqr) / Jf;
    F[2] = 0.5 * ((_rho * _v * _U + rho_ * v_ * U_ + n1 * (_P + P_)) - Fav3 / insqr) / Jf;
    F[3] = 0.5 * ((_rho * _w * _U + rho_ * w_ * U_ + n2 * (_P + P_)) - Fav4 / insqr) / Jf;
    F[4] = 0.5 * ((_U * (3.5 * _P + 0.5 * _rho * _VV) + U_ * (3.5 * P_ + 0.5 * rho_ * VV_)) - Fav5 / insqr) / Jf;
    F[5] = 0.5 * (n1 * (_P + P_) - Fav3 / insqr) / Jf;   /* Flux_Y.cpp:455-463 wall faces */
}

/* argument slots of the 32-array flux signature (main.h) */
enum { A_U = 0, A_MR = 5, A_ML = 10, A_J = 15, A_JF = 16, A_M = 17, A_F = 26, A_EP = 31 };

/* face loop shared by all six routines: for each face index in the given
 * box, gather ML/MR and the 9 metrics, evaluate, store. */
static void face_loop(const cfo_grid *g, double **a, int dir, int limited,
                      int i0, int i1, int j0, int j1, int k0, int k1, int ywall)
{
    GRID_LOCALS(g);
    const double K = g->K, e = g->e;
    #pragma omp parallel for collapse(2)
    for (int i = i0; i <= i1; i++)
        for (int j = j0; j <= j1; j++)
            for (int k = k0; k <= k1; k++) {
                const size_t q = IX(i, j, k);
                double mL[5], mR[5], m[9], F[6];
                for (int n = 0; n < 5; n++) { mL[n] = a[A_ML + n][q]; mR[n] = a[A_MR + n][q]; }
                for (int n = 0; n < 9; n++) m[n] = a[A_M + n][q];
                if (limited)
                    flux_precond_roe(mL, mR, m, dir, a[A_EP][q], a[A_JF][q], K, e, F);
                else
                    flux_roe(mL, mR, m, dir, a[A_JF][q], K, F);
                if (ywall && (j == 1 || j == ny)) {
                    a[A_F + 0][q] = 0;
                    a[A_F + 1][q] = 0;
                    a[A_F + 2][q] = F[5];
                    a[A_F + 3][q] = 0;
                    a[A_F + 4][q] = 0;
                } else {
                    for (int n = 0; n < 5; n++) a[A_F + n][q] = F[n];
                }
            }
}

/* ------------------------------------------------------------------------ */
/* Limited fluxes                                                            */
/* ------------------------------------------------------------------------ */

/* Flux_X_limiter.cpp:113-341 (reconstruction, i = 2..gend+1, 3rd order at
 * i <= 3 and i >= gend) and 369-547 (faces i = 2..gend, j,k = 1..n-1). */
void cfo_Flux_X_limiter(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    const double *J_u = a[A_JF];
    #pragma omp parallel for collapse(2)
    for (int i = 2; i <= gend + 1; i++)
        for (int j = 2; j <= ny; j++)
            for (int n = 0; n < 5; n++) {
                const double *U = a[A_U + n];
                for (int k = 2; k <= nz; k++) {
                    const double jL = J_u[IX(i, j - 1, k - 1)];
                    const double jR = J_u[IX(i - 1, j - 1, k - 1)];
                    double *ML = &a[A_ML + n][IX(i, j - 1, k - 1)];
                    double *MR = &a[A_MR + n][IX(i - 1, j - 1, k - 1)];
                    if (i <= 3 || i >= gend)
                        muscl3(U[IX(i - 1, j, k)], U[IX(i, j, k)], U[IX(i + 1, j, k)], +1, jL, jR, ML, MR);
                    else
                        muscl5(U[IX(i - 2, j, k)], U[IX(i - 1, j, k)], U[IX(i, j, k)], U[IX(i + 1, j, k)],
                               U[IX(i + 2, j, k)], +1, jL, jR, ML, MR);
                }
            }
    face_loop(g, a, 0, 1, 2, gend, 1, ny - 1, 1, nz - 1, 0);
}

/* Flux_Y_limiter.cpp:115-361 (reconstruction, i = 2..gend, j = 1..ny, with
 * the near-wall branch at j <= 2 or j >= ny-1), 365-477 (wall-face averages)
 * and 504-688 (faces i = 2..gend-1, j = 1..ny, k = 1..nz-1).
 *
 * Reference defect, replaced by a defined value: in the near-wall branch the
 * states of variables 2..5 are scaled by jL/jR, which that branch never sets
 * (private, uninitialised OpenMP variables at Flux_Y_limiter.cpp:120).  Here
 * they are the face Jacobians J_v of the same face, exactly as the interior
 * branch sets them (Flux_Y_limiter.cpp:231-232).  Faces j = 1, 2, ny-2,
 * ny-1 and ny depend on this choice.
 *
 * g->scheme == 1 (the consistent variant, not the reference): in the
 * near-wall branch every variable is reconstructed from the conserved values
 * q = U_*J of cells j-1, j, j+1 (each scaled by its own J) with the same
 * 3rd-order limiter - the reference's variable-1 line with its slope scaled
 * like its cell value - variable 1 keeping the 1e-7 ratio guard. */
static inline void ywall_q(double iq, double q, double qi, int guard, double *mL, double *mR)
{
    double rL = guard ? (qi - q) / ((q - iq) + 0.0000001) : (qi - q) / (q - iq);
    double rR = guard ? (q - iq) / ((qi - q) + 0.0000001) : (q - iq) / (qi - q);
    double minL3 = lim3(rL), minR3 = lim3(rR);
    *mL = q + 0.5 * RMAX(0, minL3) * (q - iq);
    *mR = q - 0.5 * RMAX(0, minR3) * (qi - q);
}

void cfo_Flux_Y_limiter(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    const double *J = a[A_J], *J_v = a[A_JF];
    #pragma omp parallel for collapse(2)
    for (int i = 2; i <= gend; i++)
        for (int j = 1; j <= ny; j++)
            for (int k = 2; k <= nz; k++) {
                const double jL = J_v[IX(i - 1, j, k - 1)];
                const double jR = J_v[IX(i - 1, j - 1, k - 1)];
                const size_t qL = IX(i - 1, j, k - 1), qR = IX(i - 1, j - 1, k - 1);
                if ((j <= 2 || j >= ny - 1) && g->scheme) {
                    const double Jm = J[IX(i, j - 1, k)], J0 = J[IX(i, j, k)], Jp = J[IX(i, j + 1, k)];
                    for (int n = 0; n < 5; n++) {
                        const double *Un = a[A_U + n];
                        ywall_q(Un[IX(i, j - 1, k)] * Jm, Un[IX(i, j, k)] * J0, Un[IX(i, j + 1, k)] * Jp, n == 0,
                                &a[A_ML + n][qL], &a[A_MR + n][qR]);
                    }
                } else if (j <= 2 || j >= ny - 1) {
                    /* variable 1: ratios guarded by +1e-7 and the cell value
                     * scaled by the cell Jacobian (Flux_Y_limiter.cpp:153-168) */
                    const double *U = a[A_U];
                    double iu1 = U[IX(i, j - 1, k)], u1 = U[IX(i, j, k)], u1i = U[IX(i, j + 1, k)];
                    double rL = (u1i - u1) / ((u1 - iu1) + 0.0000001);
                    double rR = (u1 - iu1) / ((u1i - u1) + 0.0000001);
                    double minL3 = lim3(rL), minR3 = lim3(rR);
                    a[A_ML][qL] = (u1 * J[IX(i, j, k)] + 0.5 * RMAX(0, minL3) * (u1 - iu1));
                    a[A_MR][qR] = (u1 * J[IX(i, j, k)] - 0.5 * RMAX(0, minR3) * (u1i - u1));
                    for (int n = 1; n < 5; n++) {
                        const double *Un = a[A_U + n];
                        muscl3(Un[IX(i, j - 1, k)], Un[IX(i, j, k)], Un[IX(i, j + 1, k)], +1, jL, jR,
                               &a[A_ML + n][qL], &a[A_MR + n][qR]);
                    }
                } else {
                    for (int n = 0; n < 5; n++) {
                        const double *Un = a[A_U + n];
                        muscl5(Un[IX(i, j - 2, k)], Un[IX(i, j - 1, k)], Un[IX(i, j, k)], Un[IX(i, j + 1, k)],
                               Un[IX(i, j + 2, k)], +1, jL, jR, &a[A_ML + n][qL], &a[A_MR + n][qR]);
                    }
                }
            }
    for (int i = 2; i <= gend; i++)
        for (int k = 2; k <= nz; k++) {
            double temp = 1. / (1 / J[IX(i, 1, k)] + 1 / J[IX(i, 2, k)]);
            for (int n = 0; n < 5; n++)
                a[A_ML + n][IX(i - 1, 1, k - 1)] = temp * (a[A_U + n][IX(i, 1, k)] + a[A_U + n][IX(i, 2, k)]);
            temp = 1. / (1 / J[IX(i, ny, k)] + 1 / J[IX(i, ny + 1, k)]);
            for (int n = 0; n < 5; n++)
                a[A_MR + n][IX(i - 1, ny, k - 1)] = temp * (a[A_U + n][IX(i, ny, k)] + a[A_U + n][IX(i, ny + 1, k)]);
        }
    face_loop(g, a, 1, 1, 2, gend - 1, 1, ny, 1, nz - 1, 1);
}

/* Flux_Z_limiter.cpp:120-352 (reconstruction, i = 2..gend, j = 2..ny,
 * k = 3..nz-1; the 3rd-order branch is taken for k >= ny, a comparison with
 * the y extent kept as written), 354-520 (rows k = 1, 2, nz) and 548-712
 * (faces i = 2..gend-1, j = 1..ny-1, k = 1..nz).  The reconstructed states
 * are scaled by 1/sum(w/J) with the unnormalised 5-point (sum 60) and
 * 3-point (sum 6) weights, as the reference does.
 *
 * g->scheme == 1 (the consistent variant, not the reference): the weights
 * are normalised (60/sum(w/J), 6/sum(w/J)) and the left state takes the
 * upwind slope u + 0.5*phi*(u-iu), as in x and y. */
void cfo_Flux_Z_limiter(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    const double *J = a[A_J];
    const double w5 = g->scheme ? 60. : 1., w3 = g->scheme ? 6. : 1.;
    const int sL = g->scheme ? +1 : -1;
    #pragma omp parallel for collapse(2)
    for (int i = 2; i <= gend; i++)
        for (int j = 2; j <= ny; j++)
            for (int k = 3; k <= nz - 1; k++) {
                const size_t qL = IX(i - 1, j - 1, k), qR = IX(i - 1, j - 1, k - 1);
                if (k <= 2 || k >= ny) {
                    double jL = w3 / (-1 / J[IX(i, j, k - 1)] + 5 / J[IX(i, j, k)] + 2 / J[IX(i, j, k + 1)]);
                    double jR = w3 / (2 / J[IX(i, j, k - 1)] + 5 / J[IX(i, j, k)] - 1 / J[IX(i, j, k + 1)]);
                    for (int n = 0; n < 5; n++) {
                        const double *U = a[A_U + n];
                        muscl3(U[IX(i, j, k - 1)], U[IX(i, j, k)], U[IX(i, j, k + 1)], sL, jL, jR,
                               &a[A_ML + n][qL], &a[A_MR + n][qR]);
                    }
                } else {
                    double jL = w5 / (2 / J[IX(i, j, k - 2)] - 13 / J[IX(i, j, k - 1)] + 47 / J[IX(i, j, k)] + 27 / J[IX(i, j, k + 1)] - 3 / J[IX(i, j, k + 2)]);
                    double jR = w5 / (-3 / J[IX(i, j, k - 2)] + 27 / J[IX(i, j, k - 1)] + 47 / J[IX(i, j, k)] - 13 / J[IX(i, j, k + 1)] + 2 / J[IX(i, j, k + 2)]);
                    for (int n = 0; n < 5; n++) {
                        const double *U = a[A_U + n];
                        muscl5(U[IX(i, j, k - 2)], U[IX(i, j, k - 1)], U[IX(i, j, k)], U[IX(i, j, k + 1)],
                               U[IX(i, j, k + 2)], sL, jL, jR, &a[A_ML + n][qL], &a[A_MR + n][qR]);
                    }
                }
            }
    #pragma omp parallel for collapse(2)
    for (int i = 2; i <= gend; i++)
        for (int j = 2; j <= ny; j++) {
            double temp;
            int k = 1;
            temp = 1. / (1 / J[IX(i, j, k)] + 1 / J[IX(i, j, k + 1)]);
            for (int n = 0; n < 5; n++)
                a[A_ML + n][IX(i - 1, j - 1, k)] = temp * (a[A_U + n][IX(i, j, k)] + a[A_U + n][IX(i, j, k + 1)]);
            for (int pass = 0; pass < 2; pass++) {
                k = pass == 0 ? 2 : nz;
                temp = 1. / (-1 / J[IX(i, j, k - 1)] + 5 / J[IX(i, j, k)] + 2 / J[IX(i, j, k + 1)]);
                for (int n = 0; n < 5; n++) {
                    const double *U = a[A_U + n];
                    a[A_ML + n][IX(i - 1, j - 1, k)] = temp * (-U[IX(i, j, k - 1)] + 5 * U[IX(i, j, k)] + 2 * U[IX(i, j, k + 1)]);
                }
                temp = 1. / (2 / J[IX(i, j, k - 1)] + 5 / J[IX(i, j, k)] - 1 / J[IX(i, j, k + 1)]);
                for (int n = 0; n < 5; n++) {
                    const double *U = a[A_U + n];
                    a[A_MR + n][IX(i - 1, j - 1, k - 1)] = temp * (2 * U[IX(i, j, k - 1)] + 5 * U[IX(i, j, k)] - U[IX(i, j, k + 1)]);
                }
            }
            k = nz;
            temp = 1. / (1 / J[IX(i, j, k)] + 1 / J[IX(i, j, k + 1)]);
            for (int n = 0; n < 5; n++)
                a[A_MR + n][IX(i - 1, j - 1, k)] = temp * (a[A_U + n][IX(i, j, k)] + a[A_U + n][IX(i, j, k + 1)]);
        }
    face_loop(g, a, 2, 1, 2, gend - 1, 1, ny - 1, 1, nz, 0);
}

/* ------------------------------------------------------------------------ */
/* Unlimited (linear MUSCL-5) fluxes                                         */
/* ------------------------------------------------------------------------ */

/* Linear 5-point face states: temp = 1/sum(w/J), state = temp*sum(w*U)
 * (Flux_X.cpp:108-122), written through a stride s along the sweep axis. */
static inline double lin5L(const double *U, const double *J, size_t q, ptrdiff_t s)
{
    double temp = 1. / (2 / J[q - 2 * s] - 13 / J[q - s] + 47 / J[q] + 27 / J[q + s] - 3 / J[q + 2 * s]);
    return temp * (2 * U[q - 2 * s] - 13 * U[q - s] + 47 * U[q] + 27 * U[q + s] - 3 * U[q + 2 * s]);
}
static inline double lin5R(const double *U, const double *J, size_t q, ptrdiff_t s)
{
    double temp = 1. / (-3 / J[q - 2 * s] + 27 / J[q - s] + 47 / J[q] - 13 / J[q + s] + 2 / J[q + 2 * s]);
    return temp * (-3 * U[q - 2 * s] + 27 * U[q - s] + 47 * U[q] - 13 * U[q + s] + 2 * U[q + 2 * s]);
}
/* 3rd-order (Flux_X.cpp:148-162) and two-cell (Flux_X.cpp:138-144) states */
static inline double lin3L(const double *U, const double *J, size_t q, ptrdiff_t s)
{
    double temp = 1. / (-1 / J[q - s] + 5 / J[q] + 2 / J[q + s]);
    return temp * (-U[q - s] + 5 * U[q] + 2 * U[q + s]);
}
static inline double lin3R(const double *U, const double *J, size_t q, ptrdiff_t s)
{
    double temp = 1. / (2 / J[q - s] + 5 / J[q] - 1 / J[q + s]);
    return temp * (2 * U[q - s] + 5 * U[q] - U[q + s]);
}
/* average of cells q and q+s with the weights in the order written */
static inline double avg2(const double *U, const double *J, size_t q, ptrdiff_t s)
{
    double temp = 1. / (1 / J[q] + 1 / J[q + s]);
    return temp * (U[q] + U[q + s]);
}

/* Flux_X.cpp:102-215 (np = 1: 5-point for i = 4..gend-1, seam rows i = 2, 3,
 * gend) and 228-424 (faces i = 2..gend). */
void cfo_Flux_X(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    const double *J = a[A_J];
    const ptrdiff_t s = (ptrdiff_t)Ym * Zm;
    #pragma omp parallel for collapse(2)
    for (int i = 4; i <= gend - 1; i++)
        for (int j = 2; j <= ny; j++)
            for (int k = 2; k <= nz; k++)
                for (int n = 0; n < 5; n++) {
                    a[A_ML + n][IX(i, j - 1, k - 1)] = lin5L(a[A_U + n], J, IX(i, j, k), s);
                    a[A_MR + n][IX(i - 1, j - 1, k - 1)] = lin5R(a[A_U + n], J, IX(i, j, k), s);
                }
    for (int j = 2; j <= ny; j++)
        for (int k = 2; k <= nz; k++)
            for (int n = 0; n < 5; n++) {
                const double *U = a[A_U + n];
                a[A_ML + n][IX(2, j - 1, k - 1)] = avg2(U, J, IX(2, j, k), s);
                a[A_ML + n][IX(3, j - 1, k - 1)] = lin3L(U, J, IX(3, j, k), s);
                a[A_MR + n][IX(2, j - 1, k - 1)] = lin3R(U, J, IX(3, j, k), s);
                a[A_ML + n][IX(gend, j - 1, k - 1)] = lin3L(U, J, IX(gend, j, k), s);
                a[A_MR + n][IX(gend - 1, j - 1, k - 1)] = lin3R(U, J, IX(gend, j, k), s);
                a[A_MR + n][IX(gend, j - 1, k - 1)] = avg2(U, J, IX(gend, j, k), s);
            }
    face_loop(g, a, 0, 0, 2, gend, 1, ny - 1, 1, nz - 1, 0);
}

/* Flux_Y.cpp:100-240 (5-point for j = 4..ny-2, near-wall rows j = 1, 2, 3,
 * ny-1, ny) and 254-467 (faces i = 2..gend-1, j = 1..ny, wall faces keep
 * the pressure term only). */
void cfo_Flux_Y(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    const double *J = a[A_J];
    const ptrdiff_t s = Zm;
    #pragma omp parallel for collapse(2)
    for (int i = 2; i <= gend; i++)
        for (int j = 4; j <= ny - 2; j++)
            for (int k = 2; k <= nz; k++)
                for (int n = 0; n < 5; n++) {
                    a[A_ML + n][IX(i - 1, j, k - 1)] = lin5L(a[A_U + n], J, IX(i, j, k), s);
                    a[A_MR + n][IX(i - 1, j - 1, k - 1)] = lin5R(a[A_U + n], J, IX(i, j, k), s);
                }
    for (int i = 2; i <= gend; i++)
        for (int k = 2; k <= nz; k++)
            for (int n = 0; n < 5; n++) {
                const double *U = a[A_U + n];
                double *ML = a[A_ML + n], *MR = a[A_MR + n];
                ML[IX(i - 1, 1, k - 1)] = avg2(U, J, IX(i, 1, k), s);
                ML[IX(i - 1, 2, k - 1)] = avg2(U, J, IX(i, 2, k), s);
                MR[IX(i - 1, 1, k - 1)] = avg2(U, J, IX(i, 2, k), s);
                ML[IX(i - 1, 3, k - 1)] = lin3L(U, J, IX(i, 3, k), s);
                MR[IX(i - 1, 2, k - 1)] = lin3R(U, J, IX(i, 3, k), s);
                ML[IX(i - 1, ny - 1, k - 1)] = lin3L(U, J, IX(i, ny - 1, k), s);
                MR[IX(i - 1, ny - 2, k - 1)] = lin3R(U, J, IX(i, ny - 1, k), s);
                /* j = ny: the pair (ny, ny-1) taken in that order (Flux_Y.cpp:206-219) */
                {
                    const size_t q = IX(i, ny, k);
                    double temp = 1. / (1 / J[q] + 1 / J[q - s]);
                    ML[IX(i - 1, ny, k - 1)] = temp * (U[q] + U[q - s]);
                    temp = 1. / (1 / J[q] + 1 / J[q - s]);
                    MR[IX(i - 1, ny - 1, k - 1)] = temp * (U[q] + U[q - s]);
                }
                MR[IX(i - 1, ny, k - 1)] = avg2(U, J, IX(i, ny, k), s);
            }
    face_loop(g, a, 1, 0, 2, gend - 1, 1, ny, 1, nz - 1, 1);
}

/* Flux_Z.cpp:104-300 (5-point for k = 3..nz-1, rows k = 1, 2, nz) and
 * 308-512 (faces i = 2..gend-1, j = 1..ny-1, k = 1..nz). */
void cfo_Flux_Z(const cfo_grid *g, double **a)
{
    GRID_LOCALS(g);
    const double *J = a[A_J];
    const ptrdiff_t s = 1;
    #pragma omp parallel for collapse(2)
    for (int i = 2; i <= gend; i++)
        for (int j = 2; j <= ny; j++) {
            for (int k = 3; k <= nz - 1; k++)
                for (int n = 0; n < 5; n++) {
                    a[A_ML + n][IX(i - 1, j - 1, k)] = lin5L(a[A_U + n], J, IX(i, j, k), s);
                    a[A_MR + n][IX(i - 1, j - 1, k - 1)] = lin5R(a[A_U + n], J, IX(i, j, k), s);
                }
            for (int n = 0; n < 5; n++) {
                const double *U = a[A_U + n];
                double *ML = a[A_ML + n], *MR = a[A_MR + n];
                ML[IX(i - 1, j - 1, 1)] = avg2(U, J, IX(i, j, 1), s);
                ML[IX(i - 1, j - 1, 2)] = lin3L(U, J, IX(i, j, 2), s);
                MR[IX(i - 1, j - 1, 1)] = lin3R(U, J, IX(i, j, 2), s);
                ML[IX(i - 1, j - 1, nz)] = lin3L(U, J, IX(i, j, nz), s);
                MR[IX(i - 1, j - 1, nz - 1)] = lin3R(U, J, IX(i, j, nz), s);
                MR[IX(i - 1, j - 1, nz)] = avg2(U, J, IX(i, j, nz), s);
            }
        }
    face_loop(g, a, 2, 0, 2, gend - 1, 1, ny - 1, 1, nz, 0);
}

/* ------------------------------------------------------------------------ */
/* Explicit SSP-RK3 (RK3NODT.cpp:115-184)                                    */
/* ------------------------------------------------------------------------ */

/* 49-array signature; slots: U_ 0-4, U 5-9, Uq 10-14, J 15, metrics 16-24,
 * inFx 25-29, inFy 30-34, inFz 35-39, vF2..5 40-43, MR 44-48 */
void cfo_RK3NODT(const cfo_grid *g, int RK, double deltaT, double *er, double **a)
{
    GRID_LOCALS(g);
    (void)er;
    const double c1[3] = {1.0, 0.75, 1.0 / 3.0};
    const double c2[3] = {0.0, 0.25, 2.0 / 3.0};
    const double c3[3] = {1.0, 0.25, 2.0 / 3.0};
    const double f = g->f;
    const double dXI = g->deltaXI, dET = g->deltaET, dZT = g->deltaZT;
    const double *J = a[15];
    #pragma omp parallel for collapse(2)
    for (int i = 3; i <= gend; i++)
        for (int j = 2; j < nyy; j++)
            for (int k = 2; k < nzz; k++) {
                const size_t q = IX(i, j, k);
                const size_t fx = IX(i, j - 1, k - 1), fx0 = IX(i - 1, j - 1, k - 1);
                const size_t fy = IX(i - 1, j, k - 1), fz = IX(i - 1, j - 1, k);
                double tmp = a[1][q] / a[0][q];
                double Rk[5];
                for (int n = 0; n < 5; n++) {
                    const double *Fx = a[25 + n], *Fy = a[30 + n], *Fz = a[35 + n];
                    Rk[n] = -((Fx[fx] - Fx[fx0]) / dXI + (Fy[fy] - Fy[fx0]) / dET + (Fz[fz] - Fz[fx0]) / dZT);
                }
                Rk[1] = Rk[1] + a[40][q] + f / J[q];
                Rk[2] = Rk[2] + a[41][q];
                Rk[3] = Rk[3] + a[42][q];
                Rk[4] = Rk[4] + a[43][q] + f * tmp / J[q];
                for (int n = 0; n < 5; n++) {
                    a[44 + n][q] = deltaT * Rk[n];
                    a[n][q] = c1[RK - 1] * a[5 + n][q] + c2[RK - 1] * a[n][q] + c3[RK - 1] * a[44 + n][q];
                }
            }
}
