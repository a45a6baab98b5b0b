// Plain data types shared by the kernels and the C-ABI layer (no device code).
//
// Layout (the reference's single-rank layout, Array.h:7): every field is one
// double[X_out+6][Y_out+4][Z_out+4] array with z fastest.  Interior cells are
// i = 3..gend (gend = X_out+2), j = 2..ny (ny = Y_out+1), k = 2..nz
// (nz = Z_out+1).  Face arrays use the same extents with one index shifted
// by -1 (x faces inFx[i][j-1][k-1] between cells i and i+1, and so on).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

struct cf_dims {
    int X_out, Y_out, Z_out;
    int Ym, Zm;               // Y_out+4, Z_out+4: row and plane strides
    int gend, ny, nz;         // X_out+2, Y_out+1, Z_out+1
    double dXI, dET, dZT;     // computational spacings
    double K, R, e;           // gamma, gas constant, preconditioning floor
    double Cv, mu_L, Pr_L;
    double f, high;           // body force, channel height 2h
    // the same constants rounded to FP32, for the FP32 kernels (a per-thread
    // FP64 -> FP32 conversion of a kernel parameter issues to the FP64 pipe)
    float f_dXI, f_dET, f_dZT, f_K, f_R, f_e, f_Cv, f_mu_L, f_Pr_L, f_f, f_high;
    double ikm1;              // 1 / (K - 1), for the contracted build's state update
    double idXI, idET, idZT, iPr;   // 1/dXI, 1/dET, 1/dZT, 1/Pr_L (correctly rounded, host)
    // face-state scaling of the limited fluxes: 0 = the reference's
    // (CF_SCHEME_REFERENCE), 1 = consistently scaled (CF_SCHEME_CONSISTENT:
    // Flux_Y_limiter's near-wall rows reconstruct the conserved variables
    // themselves, Flux_Z_limiter's weights are normalised and its left
    // state takes the upwind slope as in x and y)
    int scheme;

    __host__ __device__ __forceinline__ size_t ix(int i, int j, int k) const
    {
        return ((size_t)i * (size_t)Ym + (size_t)j) * (size_t)Zm + (size_t)k;
    }
    __host__ __device__ __forceinline__ size_t plane() const { return (size_t)Ym * (size_t)Zm; }
    __host__ __device__ __forceinline__ size_t total() const { return (size_t)(X_out + 6) * plane(); }
};

// the FP32 copies of a cf_dims' constants
static inline void cf_dims_fill_f32(cf_dims &d)
{
    d.f_dXI = (float)d.dXI; d.f_dET = (float)d.dET; d.f_dZT = (float)d.dZT;
    d.f_K = (float)d.K; d.f_R = (float)d.R; d.f_e = (float)d.e; d.f_Cv = (float)d.Cv;
    d.f_mu_L = (float)d.mu_L; d.f_Pr_L = (float)d.Pr_L; d.f_f = (float)d.f; d.f_high = (float)d.high;
    d.ikm1 = 1.0 / (d.K - 1.0);
    d.idXI = 1.0 / d.dXI; d.idET = 1.0 / d.dET; d.idZT = 1.0 / d.dZT; d.iPr = 1.0 / d.Pr_L;
}

struct cf_ptr5 {
    double *p[5];
};

// Launch geometry of one index box [i0,i0+ni) x [j0,j0+nj) x [k0,k0+nk):
// 32 consecutive z indices per warp (coalesced), 8 rows per block,
// one x plane per grid layer.
struct cf_box {
    int i0, j0, k0, ni, nj, nk;
};

static inline dim3 box_block() { return dim3(32, 8, 1); }
static inline dim3 box_grid(const cf_box &b)
{
    return dim3((unsigned)((b.nk + 31) / 32), (unsigned)((b.nj + 7) / 8), (unsigned)b.ni);
}
static inline cf_box make_box(int i0, int i1, int j0, int j1, int k0, int k1)
{
    cf_box b{i0, j0, k0, i1 - i0 + 1, j1 - j0 + 1, k1 - k0 + 1};
    if (b.ni < 0) b.ni = 0;
    if (b.nj < 0) b.nj = 0;
    if (b.nk < 0) b.nk = 0;
    return b;
}

struct cf_flux_args {
    const double *U[5];   // U1_..U5_ (conserved / J)
    const double *J;      // cell Jacobian
    const double *Jf;     // face Jacobian J_u / J_v / J_w
    const double *m[9];   // face metrics xidx..ztdz of the same face set
    const double *Ep;     // sensor EpX / EpY / EpZ (limited fluxes only)
    double *F[5];         // inF1..inF5
    double *wz[2];        // scratch of the z limiter: per-cell 1/sum(w/J) of the left and right states
    int f32_out;          // FP32 build: inF hold FP32 values (the step driver's internal use)
    int reserved;
};

// the FP32 flux kernels' view: FP32 copies of the cell arrays, FP64 face arrays
struct cf_flux_args_f {
    const float *U[5];
    const float *J;
    const double *Jf;
    const double *m[9];
    const double *Ep;
    double *F[5];
    const float *wz[2];   // wz[0]: 1/J per cell
    int f32_out;          // inF hold FP32 values
    int reserved;
    const float *Jf32, *m32[9];   // FP32 copies of Jf and m (or null)
};

struct cf_visc_args {
    const double *U[5];
    double *vF[4];
    const double *J;
    const double *Jf[3];       // J_u, J_v, J_w
    const double *mf[3][9];    // x-, y-, z-face metrics
    double *LL[4], *ML[4], *NL[4];   // x/y/z face fluxes of variables 2..5
    double *prim[4];           // scratch: u, v, w, T of every cell
    int f32_io;                // FP32 build: LL/ML/NL and vF hold FP32 values (the step driver's internal use)
    int reserved;
    const float *Jf32[3], *mf32[3][9];   // FP32 copies of the face sets (or null)
    // FP32 step driver: this sub-iteration's FP32 copies of U_ and J (or null)
    const float *U32[5], *J32;
};

struct cf_filter_args {
    const double *U[5];
    const double *Yp;       // Y_point
    const double *J;
    double *Ep[3];          // EpX, EpY, EpZ
    // scratch: two level fields and the deconvolution sum per filtered
    // variable, the y-pass coefficients (double, or float in the FP32
    // build; cB only in the FP32 build), and the sensor energies
    void *lev[2][4], *acc[4], *cA, *cC, *cB;
    double *Eh, *E2h;
};

struct cf_lu_args {
    double *U_[5];
    const double *U[5], *Uq[5];
    const double *J;
    const double *m[9];      // cell metrics xidx..ztdz
    const double *Fx[5], *Fy[5], *Fz[5];
    const double *vF[4];
    double *MR[5], *NR[5], *NL[5], *Res[5];
    double *partial;         // scratch: per-block partial norm sums (5 per block)
    int f32_rhs;             // FP32 build: Fx/Fy/Fz and vF hold FP32 values (the step driver's internal use)
    int f32_lu;              // FP32 build, wavefront: MR, NL, NR hold FP32 values (the step driver)
    const float *m32[9];     // FP32 copies of the cell metrics (or null)
    // FP32 build, step driver only (null otherwise): FP32 copies of U_ and J
    // made for this sub-iteration's fluxes, and float(U - Uq) of the step
    const float *U32[5], *J32;
    const float *dUq32[5];
};

// tiled wavefront of the hyperplane sweeps (cf_wave.cuh)
constexpr int CF_WAVE_TI = 4, CF_WAVE_TJ = 8, CF_WAVE_TK = 8, CF_WAVE_PACK = 50;
constexpr unsigned CF_WAVE_SPIN_LIMIT = 1u << 22;   // default polls before a wavefront wait gives up
struct cf_wave_args {
    cf_dims d;
    int nti, ntj, ntk, ntiles;
    const int *order;        // tile ids sorted by ti + tj + tk
    void *pack;              // [ntiles][CF_WAVE_PACK][tile cells] of the kernel's type (cf_wave.cuh)
    void *inx, *iny, *inz;   // terms arriving at a tile's x, y, z face: [ntiles][5][64 | 32 | 32]
    void *nl;                // forward N of every tile, [ntiles][5][tile cells]
    int *flags;              // per tile: 1 when done; [ntiles] = claim counter, [ntiles+1] = error word
    int *counter;
    int *err;                // bit 0: dependency wait ran out, bit 1: pack copy wait ran out
    unsigned dep_limit;      // polls of a dependency-flag wait before it gives up (the tile's own
                             // copy waits keep CF_WAVE_SPIN_LIMIT)
    long long *trace;        // optional: per tile 4 global-timer stamps (claimed, inputs ready,
                             // pack landed, done); NULL when tracing is off
    // pencil schedule (cf_pencil.cuh): 4 x 8 (j, k) pencils through every x
    // plane; order, pack, nl, flags (steps done per pencil), counter, err and
    // dep_limit take the pencil meaning, the face fields are these
    int npj, npk, npencils, nplanes;
    void *xg;                // terms from the x ghost cells: [npencils][5][32]
    void *yex, *zex;         // terms crossing pencil faces: [npencils][X_out][5][8], [npencils][X_out][5][4]
};
constexpr int CF_PENCIL_TJ = 4, CF_PENCIL_TK = 8;
constexpr int CF_PENCIL_PUB = 4;    // steps between two publications of a pencil's count

struct cf_stat_args {
    const double *U[5];      // U1_..U5_
    const double *J;         // cell Jacobian
    const double *Jv;        // y-face Jacobian J_v
    const double *m[9];      // y-face metrics xidx_v..ztdz_v
};

struct cf_rk3_args {
    double *U_[5];
    const double *U[5];
    const double *J;
    const double *Fx[5], *Fy[5], *Fz[5];
    const double *vF[4];
    double *MR[5];
};

struct cf_metric_args {
    double *Jf;
    double *m[9];
    const double *Jc;       // cell J (Jacobian_v wall rows)
    const double *mc[9];    // cell metrics (Jacobian_v wall rows)
};

