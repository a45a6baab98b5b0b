/*
 * CPU oracle for the channel-flow hot path: a plain-C restatement of the
 * reference solver's per-step routines (ricklee209/Channel_Flow).
 *
 * TEST INFRASTRUCTURE.  Only the tests, the smoke check and the bench's CPU
 * baseline load this library, and only as the checker / timed CPU arm.  The
 * GPU product never links or calls it.
 *
 * Layout: every field is one double[X_np][Y_m][Z_m] array, z fastest, with
 * X_np = X_out+6, Y_m = Y_out+4, Z_m = Z_out+4 (the reference's single-rank
 * layout, Array.h:7).  Routines take the grid description plus an array of
 * field pointers in the reference routine's argument order (main.h), so a
 * test can hand the same pointer list to this library and to the compiled
 * reference.
 *
 * Arithmetic follows the reference's expression trees operation for
 * operation, and the library is built with -ffp-contract=off, so on the same
 * inputs its results equal the reference's bit for bit (checked by
 * tests/test_oracle_vs_reference.py on x86 where the reference compiles).
 */
#ifndef CF_ORACLE_H
#define CF_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int X_out, Y_out, Z_out;          /* interior cells (Resolution.h:1-3) */
    double deltaXI, deltaET, deltaZT; /* computational spacings (Resolution.h:13-15) */
    double K, R, e;                   /* gamma, gas constant, preconditioning floor (prm.h:7-11) */
    double Cv, mu_L, Pr_L;            /* Viscous_terms.h:3-5 */
    double f, high;                   /* body force, channel height 2h (prm.h:14,19) */
    int scheme;                       /* limited-flux face-state scaling: 0 the reference's,
                                       * 1 consistent (cfo_Flux_Y_limiter, cfo_Flux_Z_limiter) */
} cfo_grid;

/* boundary conditions */
void cfo_x_periodic(const cfo_grid *g, double **a);          /* U1_..U5_ */
void cfo_Y_boundary_condition(const cfo_grid *g, double **a); /* U1_..U5_, J */
void cfo_Z_boundary_condition(const cfo_grid *g, double **a); /* U1_..U5_, J */

/* inviscid fluxes: 32 arrays U1_..5, MR1..5, ML1..5, J, J_f, 9 metrics, inF1..5, Ep */
void cfo_Flux_X(const cfo_grid *g, double **a);
void cfo_Flux_Y(const cfo_grid *g, double **a);
void cfo_Flux_Z(const cfo_grid *g, double **a);
void cfo_Flux_X_limiter(const cfo_grid *g, double **a);
void cfo_Flux_Y_limiter(const cfo_grid *g, double **a);
void cfo_Flux_Z_limiter(const cfo_grid *g, double **a);

/* viscous terms: 79 arrays in Viscous_terms' argument order */
void cfo_Viscous_terms(const cfo_grid *g, double **a);

/* ADM sensor: U1_..5, Y_point, EpX, EpY, EpZ, J */
void cfo_Filter(const cfo_grid *g, double Roe_criterion, double E_high, double E_low, double **a);

/* time integration: 49 (RK3NODT) / 64 (dual time) arrays, see main.h */
void cfo_RK3NODT(const cfo_grid *g, int RK, double deltaT, double *er, double **a);
void cfo_Dual_time_stepping(const cfo_grid *g, double deltaT, double *er,
                            const int *Nijk, const int *ijk, double **a);
void cfo_DPLUSGS(const cfo_grid *g, double deltaT, double *er, double **a);
void cfo_Hyperplane(const cfo_grid *g, int *Nijk, int *ijk);

/* face metrics (flat-wall analytic, stretching gamma): J_f + 9 metrics,
 * Jacobian_v also reads J + 9 cell metrics for its wall rows */
void cfo_Jacobian_u(const cfo_grid *g, double gamma, double **a);
void cfo_Jacobian_v(const cfo_grid *g, double gamma, double **a);
void cfo_Jacobian_w(const cfo_grid *g, double gamma, double **a);

/* bulk flow integral Q (Driven_force.cpp:38-62): U2_, J */
double cfo_Driven_force(const cfo_grid *g, double **a);

/* Statistic (Statistic.cpp): 27 arrays U1_..5, J, J_v, 9 metrics _v,
 * MR1..5, ML1..5, EpY; acc = 17*Y_m + 2 accumulators kept across calls;
 * shear[2] = wall shear-stress increments; when step % statistic_step == 0
 * nd[10][Y_m] and st[7][Y_m] receive the averages (returns 1) */
int cfo_Statistic(const cfo_grid *g, double *acc, int step, int iteration, int statistic_step, double **a,
                  double *shear, double *nd, double *st);

/* restart image of Output / Initial_condition (cf_oracle_io.c) */
void cfo_restart_pack(const cfo_grid *g, double **a, double *out);
void cfo_restart_unpack(const cfo_grid *g, const double *img, double **a);

#ifdef __cplusplus
}
#endif

#endif
