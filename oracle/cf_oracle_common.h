/* Shared definitions of the CPU oracle's translation units (test infrastructure). */
#ifndef CF_ORACLE_COMMON_H
#define CF_ORACLE_COMMON_H

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "cf_oracle.h"

/* The reference's min/max macros (Flux_X_limiter.cpp:13-14): comparisons as
 * written, so NaN and signed-zero cases resolve the same way. */
#define RMIN(a, b) (((a) < (b)) ? (a) : (b))
#define RMAX(a, b) (((a) > (b)) ? (a) : (b))

/* Index helpers of the single-rank layout: gend = X_out+2 is the last
 * interior x plane, ny = Y_out+1 and nz = Z_out+1 the last interior rows. */
#define GRID_LOCALS(g)                                  \
    const int Ym = (g)->Y_out + 4, Zm = (g)->Z_out + 4; \
    const int gend = (g)->X_out + 2;                    \
    const int ny = (g)->Y_out + 1, nz = (g)->Z_out + 1; \
    const int nyy = ny + 1, nzz = nz + 1;               \
    (void)Ym; (void)Zm; (void)gend; (void)ny; (void)nz; (void)nyy; (void)nzz

#define IX(i, j, k) (((size_t)(i) * (size_t)Ym + (size_t)(j)) * (size_t)Zm + (size_t)(k))

#endif
