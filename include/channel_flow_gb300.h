/*
 * channel_flow_gb300: C ABI of the GB300 (sm_103a) implementation of the
 * channel-flow solver's per-step hot path.
 *
 * Each routine entry point replaces one free function of the reference
 * solver (ricklee209/Channel_Flow, prototypes in main.h) and keeps its
 * argument order and meaning: the reference passes `double (*)[Y_m][Z_m]`
 * rows, here every field is a plain `double *` to X_np*Y_m*Z_m contiguous
 * doubles (z fastest, X_np = X_out+6, Y_m = Y_out+4, Z_m = Z_out+4), the
 * reference's single-rank layout (Array.h:7).  Scalars keep their meaning.
 *
 * Field pointers are either device pointers or host arrays registered with
 * cf_register() (the routine then works on the registered device mirror;
 * cf_upload()/cf_download() move the data at IO points).  All work is
 * queued on the context's stream; routines that return scalars (the
 * residual norms) synchronise that stream.
 *
 * Every function returns CF_OK or an error code; cf_last_error() gives the
 * message.  The reference's routines return void and check nothing.
 *
 * A context is not thread-safe: one host thread drives one context, as one
 * MPI rank drives its routines in the reference.
 */
#ifndef CHANNEL_FLOW_GB300_H
#define CHANNEL_FLOW_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define CF_OK 0
#define CF_ERR_ARG 1         /* bad argument, unknown pointer, grid too small */
#define CF_ERR_CUDA 2        /* a CUDA call failed (message in cf_last_error) */
#define CF_ERR_NONFINITE 3   /* cf_check_finite found a NaN or Inf */
#define CF_ERR_NOMEM 4       /* device allocation failed */
#define CF_ERR_STATE 5       /* call out of order (e.g. sweep before Hyperplane) */
#define CF_ERR_TIMEOUT 6     /* a bounded device-side wait ran out (results invalid) */

/* arithmetic modes of the flux, viscous, filter and LU-SGS kernels */
#define CF_PREC_FP64_EXACT 0 /* FP64, no fused multiply-add: equals the reference bit for bit */
#define CF_PREC_FP64 1       /* FP64 with fused multiply-add (within 1e-12 of the reference) */
#define CF_PREC_FP32 2       /* FP32 kernels; the FP64 state accumulates their changes; FP64 norms */

typedef struct cf_ctx cf_ctx;

/* Grid and constants.  The reference fixes these at compile time:
 * Resolution.h (cell counts X_out, Y_out, Z_out and spacings deltaXI,
 * deltaET, deltaZT), prm.h (K = 1.4, R = 287, e = 1e-4, f = 599.29876710,
 * high = 0.005, Q0 = 20.464969232814912) and Viscous_terms.h (Cv = 717.5, mu_L = 1.85e-5,
 * Pr_L = 0.72).  The field names differ from those macro names so that this
 * header can be included after the reference's headers. */
typedef struct {
    int cells_x, cells_y, cells_z;          /* X_out, Y_out, Z_out */
    double d_xi, d_eta, d_zeta;             /* deltaXI, deltaET, deltaZT */
    double gamma_gas, r_gas, beta_min;      /* K, R, e */
    double cv, mu, prandtl;                 /* Cv, mu_L, Pr_L */
    double body_force, height;              /* f, high */
    double bulk_flux;                       /* Q0 (prm.h), the Driven_force target */
} cf_grid;

/* ------------------------------------------------------------------ */
/* context                                                              */
/* ------------------------------------------------------------------ */

/* Fill g with the reference's constants and its 4*pi*h x 2h x 2*pi*h
 * domain for the given cell counts. */
int cf_grid_reference(cf_grid *g, int cells_x, int cells_y, int cells_z);

/* Create a context on the current CUDA device.  Each extent must be >= 6. */
int cf_create(const cf_grid *g, int precision, cf_ctx **out);
void cf_destroy(cf_ctx *ctx);
int cf_set_precision(cf_ctx *ctx, int precision);
int cf_set_stream(cf_ctx *ctx, void *cuda_stream); /* cudaStream_t; NULL = legacy default */
/* Wall-normal stretching parameter of the analytic metrics (Jacobian_u/v/w):
 * the reference hard-codes 1.5 (Jacobian_u.cpp:19). */
int cf_set_stretching(cf_ctx *ctx, double gamma);
/* Schedule of the hyperplane sweeps of Dual_time_stepping (same results):
 * CF_LU_WAVEFRONT (default) runs each sweep as one persistent launch over
 * 4x8x8-cell tiles; CF_LU_PLANES launches one kernel per hyperplane;
 * CF_LU_PENCIL runs each sweep as one persistent launch in which a warp
 * sweeps a 4x8 (j, k) pencil through every x plane, one cell per lane and
 * step. */
#define CF_LU_WAVEFRONT 0
#define CF_LU_PLANES 1
#define CF_LU_PENCIL 2
int cf_set_lu_schedule(cf_ctx *ctx, int schedule);
/* Polls of a wavefront dependency wait (a tile waiting for the done flags
 * of its upstream tiles) before it gives up, sets the error word and the
 * call returns CF_ERR_TIMEOUT; 0 restores the default (2^22 polls of
 * about 20 ns).  A test hook: a short limit makes a wait run out on
 * purpose, without a fault or a hang (the tile's own copy waits keep the
 * default limit, so no copy is left in flight). */
int cf_set_wait_limit(cf_ctx *ctx, unsigned polls);
/* Face-state scaling of the limited fluxes.  CF_SCHEME_REFERENCE (default)
 * is the reference's, bit for bit in CF_PREC_FP64_EXACT.  Two of its
 * scalings are inconsistent, and the assembled limited loop diverges on
 * channel states at the configuration time step:
 *   - Flux_Y_limiter's rows next to a wall (cells j <= 2, j >= ny-1) scale
 *     the density by the cell J and leave its slope unscaled, and scale the
 *     other four variables by jL/jR, which that branch never sets
 *     (Flux_Y_limiter.cpp:115-232; here the face J_v);
 *   - Flux_Z_limiter scales its limited states by 1/sum(w/J) with weights
 *     summing to 60 (5-point) and 6 (3-point), so interior z faces carry
 *     1/60 of the state, and its left state takes the downwind slope
 *     (Flux_Z_limiter.cpp:131-272).
 * CF_SCHEME_CONSISTENT reconstructs the conserved variables U_*J of the
 * three cells with the same limiter in Flux_Y_limiter's near-wall rows,
 * normalises the z weights (60/sum(w/J), 6/sum(w/J)) and takes the upwind
 * left slope in z.  Every other face and routine is unchanged. */
#define CF_SCHEME_REFERENCE 0
#define CF_SCHEME_CONSISTENT 1
int cf_set_scheme(cf_ctx *ctx, int scheme);
/* Wavefront trace (profiling): when enabled, each Dual_time_stepping call
 * records per tile four device global-timer stamps in ns (claimed, inputs
 * ready, coefficients staged, done), forward sweep then backward sweep.
 * cf_lu_trace_read copies 2*4*tiles values, tiles = ceil(cells_x/4) *
 * ceil(cells_y/8) * ceil(cells_z/8), tile id (ti*ntj + tj)*ntk + tk. */
int cf_lu_trace(cf_ctx *ctx, int enable);
int cf_lu_trace_read(cf_ctx *ctx, long long *out, size_t count);
int cf_synchronize(cf_ctx *ctx);
const char *cf_last_error(const cf_ctx *ctx);
const char *cf_error_string(int code);
size_t cf_field_count(const cf_ctx *ctx); /* doubles per field: X_np*Y_m*Z_m */
int cf_library_version(void);
/* Measurement helper (no counterpart in the reference): FP64 rate probe.
 * Launches `blocks` blocks of 256 threads, each running sixteen independent
 * chains of `iters` FP64 fused multiply-adds (2 * 16 * 256 * iters * blocks
 * floating-point operations), on cuda_stream; time it with events around
 * the call.  scratch_dev: `blocks` doubles the kernel may write. */
int cf_fp64_peak_probe(void *cuda_stream, int blocks, int iters, double *scratch_dev);
/* No counterpart in the reference: a check of the contracted FP64 build's
 * reciprocal (the hardware's approximate FP64 reciprocal refined by two
 * Newton-Raphson steps, used in place of divisions): out_dev[q] = 1/d_dev[q]
 * as the kernels form it, for n device doubles, on cuda_stream.  Normal
 * inputs only: subnormal d flush to zero and, like d = 0, give NaN. */
int cf_reciprocal_check(void *cuda_stream, const double *d_dev, double *out_dev, size_t n);

/* ------------------------------------------------------------------ */
/* host arrays and device mirrors                                        */
/* ------------------------------------------------------------------ */
int cf_register(cf_ctx *ctx, double *host);   /* allocate the device mirror of one field */
int cf_unregister(cf_ctx *ctx, double *host);
int cf_upload(cf_ctx *ctx, const double *host);
int cf_download(cf_ctx *ctx, double *host);
double *cf_device_ptr(cf_ctx *ctx, const double *host_or_device);
/* The same copies queued on cuda_stream (cudaStream_t, NULL = legacy
 * default) without waiting for them: with pinned host arrays a caller can
 * overlap the copies of one step with the routines of another, ordering
 * the two streams with CUDA events.  The host array must stay untouched
 * until the copy has completed. */
int cf_upload_async(cf_ctx *ctx, const double *host, void *cuda_stream);
int cf_download_async(cf_ctx *ctx, double *host, void *cuda_stream);

/* 0 if every interior value of the field is finite, else CF_ERR_NONFINITE
 * (synchronises the stream). */
int cf_check_finite(cf_ctx *ctx, const double *field);

/* ------------------------------------------------------------------ */
/* boundary conditions                                                  */
/* ------------------------------------------------------------------ */

/* replaces Y_boundary_condition (Y_boundary_condition.cpp:14) */
int cf_Y_boundary_condition(cf_ctx *ctx, int myid, double *U1_, double *U2_, double *U3_,
                            double *U4_, double *U5_, double *J);
/* replaces Z_boundary_condition (Z_boundary_condition.cpp:15) */
int cf_Z_boundary_condition(cf_ctx *ctx, int myid, double *U1_, double *U2_, double *U3_,
                            double *U4_, double *U5_, double *J);
/* replaces the x halo exchange and periodic seam of the step loop
 * (main.cpp:156-244): fills the three ghost planes on each side with the
 * periodic image of the interior */
int cf_X_periodic(cf_ctx *ctx, int myid, double *U1_, double *U2_, double *U3_, double *U4_,
                  double *U5_);

/* ------------------------------------------------------------------ */
/* inviscid fluxes                                                      */
/* ------------------------------------------------------------------ */
/* All six take the reference's 32 arrays: U1_..U5_, MR1..MR5, ML1..ML5
 * (reference scratch; not touched here), J, the face Jacobian, the nine face
 * metrics, the five face fluxes inF1..inF5 (written) and the sensor Ep (read
 * by the limited fluxes only). */
#define CF_FLUX_ARRAYS                                                                          \
    double *U1_, double *U2_, double *U3_, double *U4_, double *U5_, double *MR1, double *MR2,  \
        double *MR3, double *MR4, double *MR5, double *ML1, double *ML2, double *ML3,            \
        double *ML4, double *ML5, double *J, double *J_f, double *xidx_f, double *xidy_f,        \
        double *xidz_f, double *etdx_f, double *etdy_f, double *etdz_f, double *ztdx_f,          \
        double *ztdy_f, double *ztdz_f, double *inF1, double *inF2, double *inF3, double *inF4,  \
        double *inF5, double *Ep

/* replaces Flux_X_limiter (Flux_X_limiter.cpp:17) */
int cf_Flux_X_limiter(cf_ctx *ctx, int myid, CF_FLUX_ARRAYS);
/* replaces Flux_Y_limiter (Flux_Y_limiter.cpp:16) */
int cf_Flux_Y_limiter(cf_ctx *ctx, int myid, CF_FLUX_ARRAYS);
/* replaces Flux_Z_limiter (Flux_Z_limiter.cpp:16) */
int cf_Flux_Z_limiter(cf_ctx *ctx, int myid, CF_FLUX_ARRAYS);
/* replace Flux_X / Flux_Y / Flux_Z (Flux_X.cpp:18, Flux_Y.cpp:17, Flux_Z.cpp:17) */
int cf_Flux_X(cf_ctx *ctx, int myid, CF_FLUX_ARRAYS);
int cf_Flux_Y(cf_ctx *ctx, int myid, CF_FLUX_ARRAYS);
int cf_Flux_Z(cf_ctx *ctx, int myid, CF_FLUX_ARRAYS);

/* ------------------------------------------------------------------ */
/* viscous terms and sensor                                             */
/* ------------------------------------------------------------------ */

/* replaces Viscous_terms (Viscous_terms.cpp:15): 79 arrays U1_..U5_,
 * vF2..vF5, J, 9 cell metrics, J_u + 9, J_v + 9, J_w + 9, then the scratch
 * LR1..5, LL1..5, MR1..5, ML1..5, NR1..5, NL1..5 (LL2..5, ML2..5, NL2..5
 * receive the face fluxes as in the reference) */
int cf_Viscous_terms(cf_ctx *ctx, int myid, double **arrays79);

/* replaces Filter (Filter.cpp:12): U1_..U5_, Y_point, EpX, EpY, EpZ, J */
int cf_Filter(cf_ctx *ctx, int myid, double Roe_criterion, double E_high, double E_low,
              double *U1_, double *U2_, double *U3_, double *U4_, double *U5_, double *Y_point,
              double *EpX, double *EpY, double *EpZ, double *J);

/* ------------------------------------------------------------------ */
/* time integration                                                     */
/* ------------------------------------------------------------------ */

/* replaces RK3NODT (RK3NODT.cpp:18): 49 arrays U1_..5, U1..5, U1q..5, J,
 * 9 cell metrics, inFx1..5, inFy1..5, inFz1..5, vF2..5, MR1..5; er1..er5
 * are not written (as in the reference) */
int cf_RK3NODT(cf_ctx *ctx, int myid, int RK, double deltaT, double *er1, double *er2,
               double *er3, double *er4, double *er5, double **arrays49);

/* replaces Hyperplane (Hyperplane.cpp:18): fills the host plane tables
 * Nijk[(X_np-3)+ny+nz+7][2] and ijk[(X_np-6)*Y_out*Z_out*3][3] and keeps a
 * device copy for the sweeps */
int cf_Hyperplane(cf_ctx *ctx, int myid, int *Nijk, int *ijk);

/* replaces Dual_time_stepping (Dual_time_stepping.cpp:18): 64 arrays as
 * RK3NODT plus NR1..5, NL1..5, Residual1..5; writes er1..er5 */
int cf_Dual_time_stepping(cf_ctx *ctx, int myid, double deltaT, double *er1, double *er2,
                          double *er3, double *er4, double *er5, int *Nijk, int *ijk,
                          double **arrays64);

/* replaces DPLUSGS (DPLUSGS.cpp:18): same arrays, 4 Jacobi sweeps */
int cf_DPLUSGS(cf_ctx *ctx, int myid, double deltaT, double *er1, double *er2, double *er3,
               double *er4, double *er5, double **arrays64);

/* Allocation-free DPLUSGS: no counterpart in the reference.  Same arrays,
 * arithmetic and results as cf_DPLUSGS in CF_PREC_FP64_EXACT mode, but it
 * needs no context and calls no cudaMalloc/cudaFree, for callers that may
 * not allocate device memory: a host application whose memory manager owns
 * all device memory (the HBM reserved up front for its grids), or a loop
 * that cannot absorb the device-wide synchronisation an allocation
 * implies.  Its only scratch, the
 * residual-norm partial sums, is a fixed 10 MB file-scope device array per
 * GPU, so grids needing more than 262144 reduction blocks
 * (ceil(cells_z/32) * ceil(cells_y/8) * cells_x) are rejected with CF_ERR_ARG.
 * All calls share that array: calls overlapping on the GPU race.  The first
 * call on a device looks the array's address up (cudaGetSymbolAddress).
 * er1..er5 are host pointers; the call synchronises the stream. */
int cf_DPLUSGS_noalloc(const cf_grid *g, void *cuda_stream, double deltaT, double *er1, double *er2,
                       double *er3, double *er4, double *er5, double **arrays64);

/* ------------------------------------------------------------------ */
/* face metrics                                                         */
/* ------------------------------------------------------------------ */
/* replace Jacobian_u / Jacobian_w (Jacobian_u.cpp:15, Jacobian_w.cpp:14):
 * J_f then xidx_f..ztdz_f (10 arrays) */
int cf_Jacobian_u(cf_ctx *ctx, int myid, double **arrays10);
int cf_Jacobian_w(cf_ctx *ctx, int myid, double **arrays10);
/* replaces Jacobian_v (Jacobian_v.cpp:17): J_v + 9 face metrics, then J +
 * 9 cell metrics (read for the wall rows) */
int cf_Jacobian_v(cf_ctx *ctx, int myid, double **arrays20);

/* Metrics of a channel whose lower wall undulates in x, y_w(x) =
 * amplitude * sin(2 pi x / wavelength), with the upper wall flat at y =
 * height and the tanh wall-normal stretching of Jacobian.cpp:73-84 (the
 * reference builds flat-wall metrics only: Grid.cpp:49-141, Jacobian*.cpp).
 * conservative = 1 forms dy/dxi and dy/deta from differences of the mapping
 * half a spacing to each side, so face values are differences between cell
 * corners and the finite-volume divergence of a constant flux vanishes to
 * rounding; 0 uses the analytic derivatives (amplitude 0 then gives the
 * reference's flat-wall values).  Needs |amplitude| < height / 2. */
typedef struct {
    double amplitude, wavelength;
    double stretching;          /* gamma of the tanh stretching */
    int conservative;
} cf_wavy_wall;

enum { CF_AT_CELL = 0, CF_AT_XFACE = 1, CF_AT_YFACE = 2, CF_AT_ZFACE = 3 };

/* J and xidx, xidy, xidz, etdx, etdy, etdz, ztdx, ztdy, ztdz (device arrays
 * in the reference layout, every index written) at the cells or one face
 * set, in the reference's face indexing (x face between cells i and i+1 at
 * [i][j-1][k-1], and so on).  Stream-ordered; no allocation. */
int cf_wavy_metrics(const cf_grid *g, void *cuda_stream, const cf_wavy_wall *wall, int where,
                    double *const *J_and_metrics10);
/* cell-centre y (Y_point, read by Filter) with the ghost rows of
 * Grid.cpp:49-108 taken about the local wall */
int cf_wavy_y_point(const cf_grid *g, void *cuda_stream, const cf_wavy_wall *wall, double *Y_point);


/* ------------------------------------------------------------------ */
/* reductions and IO around the step (FP64 in every precision mode)      */
/* ------------------------------------------------------------------ */

/* Directory for the files of Statistic (Shear_stress.dat, ND%05d.dat,
 * st%05d.dat), Output (LES%05d.bin) and Initial_condition (initial.bin);
 * default ".", the reference's current directory. */
int cf_set_output_dir(cf_ctx *ctx, const char *dir);

/* Driven_force.cpp:14 (U2_, J): the bulk-flow integral Q and
 * ER_Q = |Q0 - Q| / Q0 (the reference prints them; either pointer may be
 * NULL).  Deterministic FP64 reduction. */
int cf_Driven_force(cf_ctx *ctx, int myid, double *U2_, double *J, double *Q, double *ER_Q);

/* Statistic.cpp:16.  Arrays in the reference's order (27): U1_..U5_, J,
 * J_v, xidx_v..ztdz_v, MR1..5, ML1..5, EpY; only the first 16 are read (the
 * MR/ML scratch the reference overwrites is left untouched).  Adds this
 * call's y-row sums to accumulators kept in the context, appends the wall
 * shear increments to Shear_stress.dat and, when step % statistic_step == 0,
 * writes ND%05d.dat and st%05d.dat in the reference's format and clears the
 * accumulators. */
int cf_Statistic(cf_ctx *ctx, int myid, int step, int iteration, int statistic_step, double **arrays27);
/* accumulators: 17 rows of Y_m doubles (ULm URm VLm VRm rhoLm rhoRm RUVm
 * SXYm Roe_Dm dRLm Um Vm Wm UUm VVm WWm UVm, raw sums) then SXY_bottom,
 * SXY_up: 17*Y_m + 2 values */
int cf_statistic_read(cf_ctx *ctx, double *out);
int cf_statistic_reset(cf_ctx *ctx);
/* Completes the Statistic that the last cf_step left running (its
 * accumulators to the host, the Shear_stress.dat line, at the output steps
 * ND/st files and cleared accumulators); nothing when none is pending.
 * cf_step, cf_Statistic, cf_statistic_read, cf_statistic_reset and
 * cf_destroy call it first. */
int cf_statistic_flush(cf_ctx *ctx);

/* Output.cpp:14 / Initial_condition.cpp:10: the restart image LES%05d.bin
 * (ten float64 blocks [X_out][Y_out][Z_out] of U1..U5, U1q..U5q times J)
 * written from, and initial.bin read into, the device fields.
 * Initial_condition fills U1..U5 and U1q..U5q; U1_..U5_ are not read. */
int cf_Output(cf_ctx *ctx, int step, int myid, double *U1, double *U2, double *U3, double *U4, double *U5,
              double *U1q, double *U2q, double *U3q, double *U4q, double *U5q, double *J);
int cf_Initial_condition(cf_ctx *ctx, int myid, double *U1_, double *U2_, double *U3_, double *U4_, double *U5_,
                         double *U1, double *U2, double *U3, double *U4, double *U5, double *U1q, double *U2q,
                         double *U3q, double *U4q, double *U5q, double *J);


/* ------------------------------------------------------------------ */
/* physical time step driver (main.cpp:143-480)                          */
/* ------------------------------------------------------------------ */

/* The device fields of a run (one per reference array; arrays the
 * routines treat as scratch may be shared). */
typedef struct {
    double *U_[5], *U[5], *Uq[5];      /* pseudo-time state, level n, level n-1 */
    double *J, *Y_point;
    double *cell_metric[9];            /* xidx..ztdz */
    double *face_J[3];                 /* J_u, J_v, J_w */
    double *face_metric[3][9];         /* xidx_u..ztdz_u, then _v, then _w */
    double *Ep[3];                     /* EpX, EpY, EpZ */
    double *inF[3][5];                 /* inFx1..5, inFy1..5, inFz1..5 */
    double *vF[4];                     /* vF2..vF5 */
    double *LL[4], *ML[4];             /* viscous face-flux scratch LL2..5, ML2..5 */
    double *MR[5], *NR[5], *NL[5], *Residual[5];
} cf_fields;

typedef struct {
    double deltaT;
    int max_iterations;        /* pseudo-time iterations at most (iteration_end_step, main.cpp:48) */
    double tolerance;          /* er_n / max(er_n) of fields 1-4 below this ends the step (main.cpp:406) */
    int limiter;               /* 1: Flux_X/Y/Z_limiter, 0: Flux_X/Y/Z */
    int filter;                /* 1: Filter every sub-iteration (its Ep switches the limited fluxes'
                                  dissipation), 2: Filter at the first sub-iteration of the step only
                                  (the sensor then stays fixed while the sub-iterations converge),
                                  0: no Filter (Ep as given) */
    double roe_criterion, e_high, e_low;
    int statistic_step;        /* > 0: Statistic after the step (its host part deferred, see cf_step) */
    int static_metrics;        /* 1: the metric arrays (J, cell and face metrics) stay unchanged between
                                  cf_step calls, so the FP32 path converts them to FP32 once and keeps
                                  the copies (cf_step_reset drops them) */
} cf_step_params;

/* One physical time step: pseudo-time iterations of x halo, wall and
 * periodic ghosts, [Filter], three fluxes, viscous terms and
 * Dual_time_stepping until the normalised residuals of fields 1-4 drop
 * below the tolerance (the maxima persist across steps, main.cpp:63, 387)
 * or max_iterations; then Driven_force (Q), Statistic when
 * statistic_step > 0, and Uq <- U, U <- U_.  The Statistic adds the rows of
 * a copy of the final U_ on a stream of its own, beside whatever the caller
 * enqueues next; its host part (the Shear_stress.dat line, the ND/st files
 * at the output steps) follows at the next cf_statistic_flush, which the
 * next cf_step, cf_Statistic, cf_statistic_read/reset and cf_destroy make
 * first.  Returns the iteration count,
 * the last normalised er1..er5 and Q (pointers may be NULL).  In
 * CF_PREC_FP32 the loop's intermediate arrays (inF, vF, LL, ML, MR, NR, NL)
 * are its scratch and hold FP32 values in their FP64 allocation afterwards.
 * A residual norm that is not finite (a NaN or Inf in the state) ends the
 * step with CF_ERR_NONFINITE. */
int cf_step(cf_ctx *ctx, const cf_step_params *params, int step, const cf_fields *fields, int *iterations,
            double *er, double *Q);
/* forget the running residual maxima and the FP32 metric copies */
int cf_step_reset(cf_ctx *ctx);
/* read (set = 0) or replace (set = 1) the running residual maxima E1..E5 */
int cf_step_scale(cf_ctx *ctx, double *E, int set);
/* the normalised er1..er5 of each pseudo-time iteration of the last cf_step,
 * row-major [iteration][5]; *count = that step's iterations, at most cap
 * rows are copied */
int cf_step_residuals(cf_ctx *ctx, double *out, int cap, int *count);


/* ------------------------------------------------------------------ */
/* learned initial guess: tensor-core building blocks (cf_mlp.cu)         */
/* ------------------------------------------------------------------ */

/* C = A B^T on the tcgen05 tensor cores: A [M x K] and B [N x K] row-major
 * BF16 device matrices (16-byte aligned), FP32 accumulation.  M multiple
 * of 128, K multiple of 64, N multiple of 16, ldo >= N and a multiple of 8.
 * epilogue 0: out = C (float); 1: z = C + bias, out = SiLU(z) (bf16), zout
 * (float, optional) = z; 2: out = C + bias (float).  err_dev (device int)
 * gets a nonzero bit if a bounded device wait ran out. */
int cf_gemm_bf16(void *cuda_stream, const void *A, const void *B, int M, int N, int K, int epilogue,
                 const float *bias, void *out, float *zout, int ldo, int *err_dev);
/* C = A B^T in FP32 (out [M x N], row-major) with the reduction dimension
 * split over `splits` CTAs per 128-row output tile, for products whose
 * output has few tiles and whose K is long (the weight gradients, K =
 * rows): each split writes its partial product to partial (splits x M x N
 * floats), then the partials are summed in split order.  1 <= splits <=
 * K / 64; the other constraints as cf_gemm_bf16's. */
int cf_gemm_bf16_splitk(void *cuda_stream, const void *A, const void *B, int M, int N, int K, int splits,
                        float *partial, float *out, int *err_dev);


/* The per-cell MLP of the learned initial guess (270 -> 128 -> 128 -> 5,
 * SiLU; training by Adam).  Grids are given by their interior extents; a
 * row r is interior cell (i, j, k) = (3 + r / (Y*Z), 2 + (r / Z) % Y,
 * 2 + r % Z), or rows[r] of that numbering when rows is not NULL; Mpad
 * (multiple of 128) rows are written, rows >= M zero.  Fields are FP64
 * device arrays in the reference layout; levels arrays list U^n,
 * U^(n-1)[, U^(n-2)] (five fields each).  scale10 (device floats) holds the
 * interior RMS of the first time difference U^n - U^(n-1) per variable
 * ([0..4]) and of the second, U^n - 2 U^(n-1) + U^(n-2) ([5..9]).
 * features: column 135 l + 27 v + s of a row is the first (l = 0) or
 * second (l = 1) difference of variable v at neighbour s = 9 (di+1) +
 * 3 (dj+1) + (dk+1) of the 3x3x3 stencil, over its scale. */
int cf_mlp_features(void *cuda_stream, int X, int Y, int Z, const double *const *levels15, const float *scale10,
                    const int *rows, long long M, long long Mpad, void *X_bf16_Mpad_x_320);
/* the same rows for every interior cell (M = X*Y*Z, rows M..Mpad-1 zero),
 * equal bit for bit, through diff_scratch: 10 * (X+6)*(Y+4)*(Z+4) floats
 * that receive the FP32 time differences of every array index first */
int cf_mlp_features_grid(void *cuda_stream, int X, int Y, int Z, const double *const *levels15,
                         const float *scale10, long long Mpad, float *diff_scratch, void *X_bf16_Mpad_x_320);
/* The network corrects the linear predictor P = U^n + a_v dU^n + b_v d2U of
 * U^(n+1), with dU^n = U^n - U^(n-1), d2U = U^n - 2 U^(n-1) + U^(n-2) and
 * coef10_host = a[0..4], b[5..9] (NULL: a = b = 1, the quadratic
 * extrapolation U^n + 2 dU^n - dU^(n-1)).
 * targets: (U^(n+1) - P) over scale10[5 + v] * oscale5[v] (levels20 =
 * U^(n+1), U^n, U^(n-1), U^(n-2)) */
int cf_mlp_targets(void *cuda_stream, int X, int Y, int Z, const double *const *levels20, const double *coef10_host,
                   const float *scale10, const float *oscale5, const int *rows, long long M, long long Mpad,
                   float *T_Mpad_x_16);
/* the guess on every interior cell: out = P + scale10[5 + v] * oscale5[v] *
 * Y (levels15 = U^n, U^(n-1), U^(n-2)); Y = NULL gives P alone (scale10,
 * oscale5 may then be NULL) */
int cf_mlp_apply(void *cuda_stream, int X, int Y, int Z, const double *const *levels15, const double *coef10_host,
                 const float *scale10, const float *oscale5, const float *Y_M_x_16, double *const *out5);
/* interior sums per variable v for the least-squares fit of P: with
 * d1 = dU^n, d2 = d2U, t = U^(n+1) - U^n, sums30_host[6 v + 0..5] =
 * sum d1 d1, d1 d2, d2 d2, t d1, t d2, t t (levels20 = U^(n+1), U^n, U^(n-1),
 * U^(n-2)); partial_dev holds 30 * nblocks doubles */
int cf_mlp_base_sums(void *cuda_stream, int X, int Y, int Z, const double *const *levels20, double *partial_dev,
                     int nblocks, double *sums30_host);
/* interior RMS per variable of the first and second time differences
 * (rms10_host[0..4], [5..9]); levels15 = U^n, U^(n-1), U^(n-2); partial_dev
 * holds 10 * nblocks doubles */
int cf_mlp_rms(void *cuda_stream, int X, int Y, int Z, const double *const *levels15, double *partial_dev,
               int nblocks, double *rms10_host);
/* the same ten RMS values as FP32 feature scales written to scale10_dev on
 * the device (0 becomes 1), stream-ordered, without a host round trip */
int cf_mlp_scale(void *cuda_stream, int X, int Y, int Z, const double *const *levels15, double *partial_dev,
                 int nblocks, float *scale10_dev);
/* interior RMS per variable of U^(n+1) - 3 U^n + 3 U^(n-1) - U^(n-2) (levels20 in that order) */
int cf_mlp_rms3(void *cuda_stream, int X, int Y, int Z, const double *const *levels20, double *partial_dev,
                int nblocks, double *rms5_host);
/* sums over M rows of T.Y, Y.Y, T.T per output (FP64) into sums15_host[0..4], [5..9], [10..14];
 * partial_dev holds 15 * nblocks doubles */
int cf_mlp_dot(void *cuda_stream, const float *Y, const float *T, long long M, double *partial_dev, int nblocks,
               double *sums15_host);
int cf_mlp_loss_grad(void *cuda_stream, const float *Y, const float *T, long long M, long long Mpad,
                     void *dY_bf16_Mpad_x_64, void *dYT_bf16_16_x_Mpad, float *partial);
int cf_mlp_silu_bwd(void *cuda_stream, const float *dH, const float *Z, long long Mpad, void *dZ_bf16,
                    void *dZT_bf16);
int cf_transpose_bf16(void *cuda_stream, const void *src, long long rows, int cols, void *dst);
int cf_colsum_bf16(void *cuda_stream, const void *src, long long rows, int cols, float *out);
int cf_adam(void *cuda_stream, float *param, const float *grad, float *m, float *v, long long n, float lr,
            float beta1, float beta2, float eps, int step);
int cf_mlp_pack(void *cuda_stream, const float *W1, const float *W2, const float *W3T, void *W1b, void *W2b,
                void *W3b, void *W2T, void *W3p);

#ifdef __cplusplus
}
#endif

#endif
