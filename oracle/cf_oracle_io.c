/*
 * CPU oracle (test infrastructure): the restart image of the reference's
 * Output (Output.cpp:43-190) and Initial_condition (Initial_condition.cpp:
 * 64-116), restated in C.
 *
 * The image is ten float64 blocks of X_out*Y_out*Z_out values in C order
 * ([i][j][k] over the interior, k fastest): U1..U5 then U1q..U5q, each
 * multiplied by J (Output); Initial_condition divides by J again into the
 * interior of U1..U5 and U1q..U5q.
 */
#include "cf_oracle_common.h"

/* arrays: U1..U5, U1q..U5q, J */
void cfo_restart_pack(const cfo_grid *g, double **a, double *out)
{
    GRID_LOCALS(g);
    const size_t N = (size_t)g->X_out * g->Y_out * g->Z_out;
    const double *J = a[10];
    for (int f = 0; f < 10; f++) {
        const double *U = a[f];
        double *o = out + f * N;
        for (int i = 0; i < g->X_out; i++)
            for (int j = 0; j < ny - 1; j++)
                for (int k = 0; k < nz - 1; k++) {
                    const size_t q = IX(i + 3, j + 2, k + 2);
                    o[((size_t)i * g->Y_out + j) * g->Z_out + k] = U[q] * J[q];
                }
    }
}

/* arrays: U1_..U5_, U1..U5, U1q..U5q, J (Initial_condition's order); only
 * U1..U5 and U1q..U5q are written */
void cfo_restart_unpack(const cfo_grid *g, const double *img, double **a)
{
    GRID_LOCALS(g);
    const size_t N = (size_t)g->X_out * g->Y_out * g->Z_out;
    const double *J = a[15];
    for (int f = 0; f < 10; f++) {
        double *U = a[5 + f];
        const double *s = img + f * N;
        for (int i = 0; i < g->X_out; i++)
            for (int j = 2; j < nyy; j++)
                for (int k = 2; k < nzz; k++) {
                    const size_t q = IX(i + 3, j, k);
                    U[q] = s[((size_t)i * g->Y_out + (j - 2)) * g->Z_out + (k - 2)] / J[q];
                }
    }
}
