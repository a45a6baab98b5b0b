/*
 * extern "C" entry points around the reference solver's own routines
 * (ricklee209/Channel_Flow, compiled unmodified from its sources with the
 * single-rank headers in oracle/ref_overrides and a generated Resolution.h).
 *
 * TEST INFRASTRUCTURE ONLY: this library is the checker that pins the C
 * restatement in oracle/cf_oracle.c; nothing in the product links it.
 *
 * Every array argument is passed as a flat pointer in the reference's
 * argument order (prototypes: main.h); the wrapper casts each one to the
 * reference's double (*)[Y_m][Z_m] row type.  Grid extents are the
 * compile-time macros of the generated Resolution.h, reported back by
 * ref_grid() so the caller can check it loaded the right build.
 */
#include <mpi.h>
#include "main.h"

typedef double (*A)[Y_m][Z_m];
#define P(n) ((A)a[n])

int X_np = X_out + 6;

/* DPLUSGS.cpp compiled a second time with j_ = j+1, k_ = k+1 defined
 * (ref_overrides/dplusgs_defined.h); same C++ signature as DPLUSGS */
decltype(DPLUSGS) DPLUSGS_defined;

extern "C" {

void ref_grid(int *dims, double *deltas)
{
    dims[0] = X_out; dims[1] = Y_out; dims[2] = Z_out;
    dims[3] = X_np;  dims[4] = Y_m;   dims[5] = Z_m;
    deltas[0] = deltaXI; deltas[1] = deltaET; deltas[2] = deltaZT;
}

/* Y_boundary_condition.cpp:14 (U1_..U5_, J) */
void ref_Y_boundary_condition(double **a)
{
    Y_boundary_condition(0, P(0), P(1), P(2), P(3), P(4), P(5));
}

/* Z_boundary_condition.cpp:15 (U1_..U5_, J) */
void ref_Z_boundary_condition(double **a)
{
    Z_boundary_condition(0, P(0), P(1), P(2), P(3), P(4), P(5));
}

#define FLUX_ARGS P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9), P(10), P(11), \
    P(12), P(13), P(14), P(15), P(16), P(17), P(18), P(19), P(20), P(21), P(22), P(23), P(24), \
    P(25), P(26), P(27), P(28), P(29), P(30), P(31)

/* 32 arrays: U1_..U5_, MR1..5, ML1..5, J, J_f, 9 face metrics, inF1..5, Ep */
void ref_Flux_X(double **a) { Flux_X(0, FLUX_ARGS); }
void ref_Flux_Y(double **a) { Flux_Y(0, FLUX_ARGS); }
void ref_Flux_Z(double **a) { Flux_Z(0, FLUX_ARGS); }
void ref_Flux_X_limiter(double **a) { Flux_X_limiter(0, FLUX_ARGS); }
void ref_Flux_Y_limiter(double **a) { Flux_Y_limiter(0, FLUX_ARGS); }
void ref_Flux_Z_limiter(double **a) { Flux_Z_limiter(0, FLUX_ARGS); }

/* Viscous_terms.cpp:15, 79 arrays in prototype order */
void ref_Viscous_terms(double **a)
{
    Viscous_terms(0,
        P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9),
        P(10), P(11), P(12), P(13), P(14), P(15), P(16), P(17), P(18), P(19),
        P(20), P(21), P(22), P(23), P(24), P(25), P(26), P(27), P(28), P(29),
        P(30), P(31), P(32), P(33), P(34), P(35), P(36), P(37), P(38), P(39),
        P(40), P(41), P(42), P(43), P(44), P(45), P(46), P(47), P(48), P(49),
        P(50), P(51), P(52), P(53), P(54), P(55), P(56), P(57), P(58), P(59),
        P(60), P(61), P(62), P(63), P(64), P(65), P(66), P(67), P(68), P(69),
        P(70), P(71), P(72), P(73), P(74), P(75), P(76), P(77), P(78));
}

/* Filter.cpp:12 (U1_..U5_, Y_point, EpX, EpY, EpZ, J) */
void ref_Filter(double Roe_criterion, double E_high, double E_low, double **a)
{
    Filter(0, Roe_criterion, E_high, E_low, P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7),
           P(8), P(9));
}

#define DT_ARGS P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9), \
    P(10), P(11), P(12), P(13), P(14), P(15), P(16), P(17), P(18), P(19), \
    P(20), P(21), P(22), P(23), P(24), P(25), P(26), P(27), P(28), P(29), \
    P(30), P(31), P(32), P(33), P(34), P(35), P(36), P(37), P(38), P(39), \
    P(40), P(41), P(42), P(43), P(44), P(45), P(46), P(47), P(48)

/* The 15 trailing arrays of the dual-time routines: NR1..5, NL1..5, Residual1..5 */
#define LU_ARGS P(49), P(50), P(51), P(52), P(53), P(54), P(55), P(56), P(57), P(58), \
    P(59), P(60), P(61), P(62), P(63)

/* RK3NODT.cpp:18: 49 arrays U1_..5, U1..5, U1q..5, J, 9 metrics, inFx/y/z 1..5, vF2..5, MR1..5 */
void ref_RK3NODT(int RK, double deltaT, double *er, double **a)
{
    RK3NODT(0, RK, deltaT, &er[0], &er[1], &er[2], &er[3], &er[4], DT_ARGS);
}

/* Dual_time_stepping.cpp:18: as RK3NODT plus NR1..5, NL1..5, Residual1..5 */
void ref_Dual_time_stepping(double deltaT, double *er, int *Nijk, int *ijk, double **a)
{
    Dual_time_stepping(0, deltaT, &er[0], &er[1], &er[2], &er[3], &er[4],
                       (int (*)[2])Nijk, (int (*)[3])ijk, DT_ARGS, LU_ARGS);
}

/* DPLUSGS.cpp:18: same arrays as Dual_time_stepping without the plane tables */
void ref_DPLUSGS(double deltaT, double *er, double **a)
{
    DPLUSGS(0, deltaT, &er[0], &er[1], &er[2], &er[3], &er[4], DT_ARGS, LU_ARGS);
}

void ref_DPLUSGS_defined(double deltaT, double *er, double **a)
{
    DPLUSGS_defined(0, deltaT, &er[0], &er[1], &er[2], &er[3], &er[4], DT_ARGS, LU_ARGS);
}

/* Hyperplane.cpp:18 */
void ref_Hyperplane(int *Nijk, int *ijk)
{
    Hyperplane(0, (int (*)[2])Nijk, (int (*)[3])ijk);
}

/* Grid.cpp:11 (X_point, Y_point, Z_point) */
void ref_Grid(double **a) { Grid(0, P(0), P(1), P(2)); }

/* Jacobian.cpp:16 (J + 9 cell metrics) */
void ref_Jacobian(double **a)
{
    Jacobian(0, P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9));
}
void ref_Jacobian_u(double **a)
{
    Jacobian_u(0, P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9));
}
void ref_Jacobian_w(double **a)
{
    Jacobian_w(0, P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9));
}
/* Jacobian_v.cpp:17: 10 face arrays then J + 9 cell metrics */
void ref_Jacobian_v(double **a)
{
    Jacobian_v(0, P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9),
               P(10), P(11), P(12), P(13), P(14), P(15), P(16), P(17), P(18), P(19));
}

/* Driven_force.cpp:14 (U2_, J); prints the bulk-flux line */
void ref_Driven_force(double **a) { Driven_force(0, P(0), P(1)); }

/* Statistic.cpp:16 (U1_..U5_, J, J_v, 9 metrics _v, MR1..5, ML1..5, EpY);
 * appends Shear_stress.dat and writes ND%05d.dat / st%05d.dat in the
 * current directory every statistic_step steps */
void ref_Statistic(int step, int iteration, int statistic_step, double **a)
{
    Statistic(0, step, iteration, statistic_step, P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9),
              P(10), P(11), P(12), P(13), P(14), P(15), P(16), P(17), P(18), P(19), P(20), P(21), P(22), P(23),
              P(24), P(25), P(26));
}

/* Output.cpp:15 (U1..U5, U1q..U5q, J): writes LES%05d.bin */
void ref_Output(int step, double **a)
{
    Output(step, 0, P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9), P(10));
}

/* Initial_condition.cpp:10 (U1_..U5_, U1..U5, U1q..U5q, J): reads initial.bin */
void ref_Initial_condition(double **a)
{
    Initial_condition(0, P(0), P(1), P(2), P(3), P(4), P(5), P(6), P(7), P(8), P(9), P(10), P(11), P(12), P(13),
                      P(14), P(15));
}

} /* extern "C" */
