/*
 * Forced include for the defined-index build of the reference's DPLUSGS.cpp
 * (CPU oracle only).  DPLUSGS.cpp indexes the upper neighbours as
 * NL*[i][j_][k] and NL*[i][j][k_] but never assigns j_ or k_ (they are
 * OpenMP-private and uninitialised, DPLUSGS.cpp:569), so its result is
 * undefined.  Defining them as the neighbour indices j+1 and k+1, as
 * Dual_time_stepping.cpp uses (j+1, k+1 at 1121-1129), gives the intended
 * Jacobi sweep; the function is renamed so both builds can be linked
 * together.  Compiled without OpenMP (the renamed indices cannot appear in
 * a private clause); the Jacobi sweep does not depend on the loop order.
 */
#define j_ (j + 1)
#define k_ (k + 1)
#define DPLUSGS DPLUSGS_defined
