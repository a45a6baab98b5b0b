/* Loop-index declarations of the reference (ijk.h) without j_ and k_, which
 * dplusgs_defined.h turns into the expressions (j+1) and (k+1).  Used only
 * for the second, defined-index build of DPLUSGS.cpp in the CPU oracle. */
int i, j, k, i_, i__, j__, k__, _i, _j, _k, __i, __j, __k;
