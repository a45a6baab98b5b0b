/*
 * Drop-in binding for the reference solver's C++ driver (ricklee209/
 * Channel_Flow main.cpp): functions with the reference's exact signatures
 * (main.h) that forward to the C-ABI of channel_flow_gb300.h.
 *
 * Include it instead of main.h in the driver, after the reference's
 * Resolution.h (Y_m and Z_m must be defined), and call cfdrop::init() once
 * after the arrays of Array.h are allocated.  init() creates the device
 * context, registers every array the hot path touches as a device mirror
 * (cfdrop::track) and uploads it; from then on the routine calls of the
 * step loop run on the GPU on those mirrors.  Download what the host reads
 * (Driven_force, Statistic, Output) with cfdrop::to_host().
 *
 * One rank covers the whole x extent (X_np = X_out+6): the halo exchange
 * and periodic seam of main.cpp:156-244 become cfdrop::x_halo().
 */
#ifndef CHANNEL_FLOW_GB300_DROPIN_HPP
#define CHANNEL_FLOW_GB300_DROPIN_HPP

#include <cstdio>
#include <cstdlib>

#include "channel_flow_gb300.h"

#ifndef Y_m
#error "include the reference's Resolution.h before channel_flow_gb300_dropin.hpp"
#endif

typedef double (*cf_field)[Y_m][Z_m];

namespace cfdrop {

inline cf_ctx *&ctx()
{
    static cf_ctx *c = nullptr;
    return c;
}

inline double &q0()
{
    static double q = 0;
    return q;
}

inline void check(int rc, const char *what)
{
    if (rc != CF_OK) {
        std::fprintf(stderr, "channel_flow_gb300: %s failed: %s\n", what, cf_last_error(ctx()));
        std::abort();
    }
}

/* create the context: grid of Resolution.h, reference constants */
inline void init(int precision = CF_PREC_FP64)
{
    cf_grid g;
    cf_grid_reference(&g, X_out, Y_out, Z_out);
    g.d_xi = deltaXI;
    g.d_eta = deltaET;
    g.d_zeta = deltaZT;
    q0() = g.bulk_flux;
    check(cf_create(&g, precision, &ctx()), "cf_create");
}

/* register a host array as a device mirror and upload its contents */
inline void track(cf_field a)
{
    check(cf_register(ctx(), &a[0][0][0]), "cf_register");
    check(cf_upload(ctx(), &a[0][0][0]), "cf_upload");
}
inline void to_host(cf_field a) { check(cf_download(ctx(), &a[0][0][0]), "cf_download"); }
inline void to_device(cf_field a) { check(cf_upload(ctx(), &a[0][0][0]), "cf_upload"); }

inline void x_halo(int myid, cf_field U1_, cf_field U2_, cf_field U3_, cf_field U4_, cf_field U5_)
{
    check(cf_X_periodic(ctx(), myid, &U1_[0][0][0], &U2_[0][0][0], &U3_[0][0][0], &U4_[0][0][0],
                        &U5_[0][0][0]), "X_periodic");
}

}  // namespace cfdrop

#define CF_P(a) (&(a)[0][0][0])

inline void Y_boundary_condition(int myid, cf_field U1_, cf_field U2_, cf_field U3_, cf_field U4_,
                                 cf_field U5_, cf_field J)
{
    cfdrop::check(cf_Y_boundary_condition(cfdrop::ctx(), myid, CF_P(U1_), CF_P(U2_), CF_P(U3_),
                                          CF_P(U4_), CF_P(U5_), CF_P(J)), "Y_boundary_condition");
}

inline void Z_boundary_condition(int myid, cf_field U1_, cf_field U2_, cf_field U3_, cf_field U4_,
                                 cf_field U5_, cf_field J)
{
    cfdrop::check(cf_Z_boundary_condition(cfdrop::ctx(), myid, CF_P(U1_), CF_P(U2_), CF_P(U3_),
                                          CF_P(U4_), CF_P(U5_), CF_P(J)), "Z_boundary_condition");
}

#define CF_DROPIN_FLUX(NAME)                                                                            \
    inline void NAME(int myid, cf_field U1_, cf_field U2_, cf_field U3_, cf_field U4_, cf_field U5_,    \
                     cf_field MR1, cf_field MR2, cf_field MR3, cf_field MR4, cf_field MR5, cf_field ML1, \
                     cf_field ML2, cf_field ML3, cf_field ML4, cf_field ML5, cf_field J, cf_field J_f,   \
                     cf_field xidx, cf_field xidy, cf_field xidz, cf_field etdx, cf_field etdy,          \
                     cf_field etdz, cf_field ztdx, cf_field ztdy, cf_field ztdz, cf_field F1,            \
                     cf_field F2, cf_field F3, cf_field F4, cf_field F5, cf_field Ep)                    \
    {                                                                                                   \
        cfdrop::check(cf_##NAME(cfdrop::ctx(), myid, CF_P(U1_), CF_P(U2_), CF_P(U3_), CF_P(U4_),        \
                                CF_P(U5_), CF_P(MR1), CF_P(MR2), CF_P(MR3), CF_P(MR4), CF_P(MR5),       \
                                CF_P(ML1), CF_P(ML2), CF_P(ML3), CF_P(ML4), CF_P(ML5), CF_P(J),         \
                                CF_P(J_f), CF_P(xidx), CF_P(xidy), CF_P(xidz), CF_P(etdx), CF_P(etdy),  \
                                CF_P(etdz), CF_P(ztdx), CF_P(ztdy), CF_P(ztdz), CF_P(F1), CF_P(F2),     \
                                CF_P(F3), CF_P(F4), CF_P(F5), CF_P(Ep)),                                \
                      #NAME);                                                                           \
    }

CF_DROPIN_FLUX(Flux_X_limiter)
CF_DROPIN_FLUX(Flux_Y_limiter)
CF_DROPIN_FLUX(Flux_Z_limiter)
CF_DROPIN_FLUX(Flux_X)
CF_DROPIN_FLUX(Flux_Y)
CF_DROPIN_FLUX(Flux_Z)

inline void Filter(int myid, double Roe_criterion, double E_high, double E_low, cf_field U1_, cf_field U2_,
                   cf_field U3_, cf_field U4_, cf_field U5_, cf_field Y_point, cf_field EpX, cf_field EpY,
                   cf_field EpZ, cf_field J)
{
    cfdrop::check(cf_Filter(cfdrop::ctx(), myid, Roe_criterion, E_high, E_low, CF_P(U1_), CF_P(U2_),
                            CF_P(U3_), CF_P(U4_), CF_P(U5_), CF_P(Y_point), CF_P(EpX), CF_P(EpY),
                            CF_P(EpZ), CF_P(J)), "Filter");
}

/* the routines with long argument lists collect their arrays in the
 * reference's order and pass the list */
template <typename... A>
inline void cf_collect(double **out, A... a)
{
    double *v[] = {CF_P(a)...};
    for (size_t i = 0; i < sizeof...(A); i++) out[i] = v[i];
}

template <typename... A>
inline void Viscous_terms(int myid, A... a)
{
    static_assert(sizeof...(A) == 79, "Viscous_terms takes 79 arrays");
    double *p[79];
    cf_collect(p, a...);
    cfdrop::check(cf_Viscous_terms(cfdrop::ctx(), myid, p), "Viscous_terms");
}

template <typename... A>
inline void RK3NODT(int myid, int RK, double deltaT, double *er1, double *er2, double *er3, double *er4,
                    double *er5, A... a)
{
    static_assert(sizeof...(A) == 49, "RK3NODT takes 49 arrays");
    double *p[49];
    cf_collect(p, a...);
    cfdrop::check(cf_RK3NODT(cfdrop::ctx(), myid, RK, deltaT, er1, er2, er3, er4, er5, p), "RK3NODT");
}

inline void Hyperplane(int myid, int (*Nijk)[2], int (*ijk)[3])
{
    cfdrop::check(cf_Hyperplane(cfdrop::ctx(), myid, &Nijk[0][0], &ijk[0][0]), "Hyperplane");
}

template <typename... A>
inline void Dual_time_stepping(int myid, double deltaT, double *er1, double *er2, double *er3, double *er4,
                               double *er5, int (*Nijk)[2], int (*ijk)[3], A... a)
{
    static_assert(sizeof...(A) == 64, "Dual_time_stepping takes 64 arrays");
    double *p[64];
    cf_collect(p, a...);
    cfdrop::check(cf_Dual_time_stepping(cfdrop::ctx(), myid, deltaT, er1, er2, er3, er4, er5, &Nijk[0][0],
                                        &ijk[0][0], p), "Dual_time_stepping");
}

template <typename... A>
inline void DPLUSGS(int myid, double deltaT, double *er1, double *er2, double *er3, double *er4, double *er5,
                    A... a)
{
    static_assert(sizeof...(A) == 64, "DPLUSGS takes 64 arrays");
    double *p[64];
    cf_collect(p, a...);
    cfdrop::check(cf_DPLUSGS(cfdrop::ctx(), myid, deltaT, er1, er2, er3, er4, er5, p), "DPLUSGS");
}

template <typename... A>
inline void Jacobian_u(int myid, A... a)
{
    static_assert(sizeof...(A) == 10, "Jacobian_u takes 10 arrays");
    double *p[10];
    cf_collect(p, a...);
    cfdrop::check(cf_Jacobian_u(cfdrop::ctx(), myid, p), "Jacobian_u");
}
template <typename... A>
inline void Jacobian_w(int myid, A... a)
{
    static_assert(sizeof...(A) == 10, "Jacobian_w takes 10 arrays");
    double *p[10];
    cf_collect(p, a...);
    cfdrop::check(cf_Jacobian_w(cfdrop::ctx(), myid, p), "Jacobian_w");
}
template <typename... A>
inline void Jacobian_v(int myid, A... a)
{
    static_assert(sizeof...(A) == 20, "Jacobian_v takes 20 arrays");
    double *p[20];
    cf_collect(p, a...);
    cfdrop::check(cf_Jacobian_v(cfdrop::ctx(), myid, p), "Jacobian_v");
}

/* Driven_force.cpp:14: prints the bulk flux as the reference does */
inline void Driven_force(int myid, cf_field U2_, cf_field J)
{
    double Q = 0, ER_Q = 0;
    cfdrop::check(cf_Driven_force(cfdrop::ctx(), myid, CF_P(U2_), CF_P(J), &Q, &ER_Q), "Driven_force");
    if (myid == 0) std::printf("Q0=%f\tQall=%f\tER_Q=%f\n", cfdrop::q0(), Q, ER_Q);
}

template <typename... A>
inline void Statistic(int myid, int step, int iteration, int statistic_step, A... a)
{
    static_assert(sizeof...(A) == 27, "Statistic takes 27 arrays");
    double *p[27];
    cf_collect(p, a...);
    cfdrop::check(cf_Statistic(cfdrop::ctx(), myid, step, iteration, statistic_step, p), "Statistic");
}

inline void Output(int step, int myid, cf_field U1, cf_field U2, cf_field U3, cf_field U4, cf_field U5,
                   cf_field U1q, cf_field U2q, cf_field U3q, cf_field U4q, cf_field U5q, cf_field J)
{
    cfdrop::check(cf_Output(cfdrop::ctx(), step, myid, CF_P(U1), CF_P(U2), CF_P(U3), CF_P(U4), CF_P(U5),
                            CF_P(U1q), CF_P(U2q), CF_P(U3q), CF_P(U4q), CF_P(U5q), CF_P(J)), "Output");
}

template <typename... A>
inline void Initial_condition(int myid, A... a)
{
    static_assert(sizeof...(A) == 16, "Initial_condition takes 16 arrays");
    double *p[16];
    cf_collect(p, a...);
    cfdrop::check(cf_Initial_condition(cfdrop::ctx(), myid, p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8],
                                       p[9], p[10], p[11], p[12], p[13], p[14], p[15]), "Initial_condition");
}

#undef CF_P
#endif
