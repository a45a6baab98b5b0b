// Allocation-free entry point: the data-parallel LU-SGS (DPLUSGS) without a
// context.
//
// Who needs it: a host solver that drives the pseudo-time iterations but may
// not allocate device memory itself - because a memory manager of the host
// application owns every device byte (it reserves the HBM for the large
// grids up front and forbids a library from taking more), or because its
// loop cannot absorb the device-wide synchronisation that cudaMalloc and
// cudaFree imply.  Such a caller passes all inputs and outputs; this file
// keeps the only scratch the routine needs (per-block partial sums of the
// residual norms and the five norms themselves) in file-scope device
// arrays of fixed size, which every GPU that loads the library holds until
// the process exits.
//
// Limits and rules:
// * at most CF_NOALLOC_MAX_BLOCKS reduction blocks, i.e. ceil(Z_out/32) *
//   ceil(Y_out/8) * X_out <= 262144 (a 512 x 256 x 384 grid needs 196608);
//   larger grids are rejected with CF_ERR_ARG before anything is launched;
// * the scratch is shared by every call on a device and keeps the last
//   call's contents; every value the routine reads from it is written
//   earlier in the same call, so nothing needs clearing, but calls that
//   overlap on the GPU (different streams or host threads at the same time)
//   race on it and must not be issued;
// * the device address of the scratch is looked up once per device
//   (cudaGetSymbolAddress), on the first call made with that device
//   current;
// * the call ends by copying the five norms to the caller's host doubles and
//   synchronising the stream.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/channel_flow_gb300.h"
#include "cf_lusgs.cuh"
#include "cf_launch.h"

#define CF_NOALLOC_MAX_BLOCKS 262144
#define CF_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double cf_noalloc_partial[5 * CF_NOALLOC_MAX_BLOCKS];
static __device__ __align__(256) double cf_noalloc_er[8];

namespace {

struct scratch_ptrs {
    double *partial = nullptr;
    double *er = nullptr;
};

scratch_ptrs g_scratch[CF_NOALLOC_MAX_DEVICES];
std::mutex g_scratch_mutex;

// device addresses of the two file-scope arrays for the current device
int scratch_for_current_device(scratch_ptrs &out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= CF_NOALLOC_MAX_DEVICES) return CF_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    scratch_ptrs &s = g_scratch[dev];
    if (!s.partial) {
        void *p = nullptr, *e = nullptr;
        if (cudaGetSymbolAddress(&p, cf_noalloc_partial) != cudaSuccess) return CF_ERR_CUDA;
        if (cudaGetSymbolAddress(&e, cf_noalloc_er) != cudaSuccess) return CF_ERR_CUDA;
        s.partial = static_cast<double *>(p);
        s.er = static_cast<double *>(e);
    }
    out = s;
    return CF_OK;
}

}  // namespace

extern "C" int cf_DPLUSGS_noalloc(const cf_grid *g, void *stream, double deltaT, double *er1, double *er2,
                                  double *er3, double *er4, double *er5, double **p)
{
    if (!g || !p) return CF_ERR_ARG;
    if (g->cells_x < 6 || g->cells_y < 6 || g->cells_z < 6) return CF_ERR_ARG;
    for (int i = 0; i < 64; i++)
        if (!p[i]) return CF_ERR_ARG;
    cf_dims d{};
    d.X_out = g->cells_x; d.Y_out = g->cells_y; d.Z_out = g->cells_z;
    d.Ym = g->cells_y + 4; d.Zm = g->cells_z + 4;
    d.gend = g->cells_x + 2; d.ny = g->cells_y + 1; d.nz = g->cells_z + 1;
    d.dXI = g->d_xi; d.dET = g->d_eta; d.dZT = g->d_zeta;
    d.K = g->gamma_gas; d.R = g->r_gas; d.e = g->beta_min; d.Cv = g->cv; d.mu_L = g->mu; d.Pr_L = g->prandtl;
    d.f = g->body_force; d.high = g->height;
    d.scheme = CF_SCHEME_REFERENCE;
    cf_dims_fill_f32(d);

    const cf_box b = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    const dim3 grid = box_grid(b), block = box_block();
    const size_t nblk = (size_t)grid.x * grid.y * grid.z;
    if (nblk > CF_NOALLOC_MAX_BLOCKS) return CF_ERR_ARG;

    scratch_ptrs s;
    if (int rc = scratch_for_current_device(s)) return rc;

    cf_lu_args a{};   // FP32-only fields stay null
    for (int n = 0; n < 5; n++) {
        a.U_[n] = p[n];
        a.U[n] = p[5 + n];
        a.Uq[n] = p[10 + n];
        a.Fx[n] = p[25 + n];
        a.Fy[n] = p[30 + n];
        a.Fz[n] = p[35 + n];
        a.MR[n] = p[44 + n];
        a.NR[n] = p[49 + n];
        a.NL[n] = p[54 + n];
        a.Res[n] = p[59 + n];
    }
    a.J = p[15];
    for (int n = 0; n < 9; n++) a.m[n] = p[16 + n];
    for (int n = 0; n < 4; n++) a.vF[n] = p[40 + n];
    a.partial = s.partial;

    cudaStream_t st = (cudaStream_t)stream;
    const size_t total = d.total();
    CF_NS::k_lu_zero<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(d, a, total);
    CF_NS::k_lu_assemble<double><<<grid, block, 0, st>>>(d, a, b, deltaT, 0);
    for (int sweep = 1; sweep <= 4; sweep++) {
        CF_NS::k_lu_jacobi<double><<<grid, block, 0, st>>>(d, a, b, deltaT);
        CF_NS::k_lu_copy<<<grid, block, 0, st>>>(d, a, b);
    }
    CF_NS::k_lu_update<double><<<grid, block, 0, st>>>(d, a, b);
    const double DN = 1. / (d.X_out * d.Y_out * d.Z_out);
    CF_NS::k_lu_norm<<<1, 256, 0, st>>>(s.partial, nblk, DN, s.er);
    if (cudaGetLastError() != cudaSuccess) return CF_ERR_CUDA;

    double *er[5] = {er1, er2, er3, er4, er5};
    for (int n = 0; n < 5; n++)
        if (er[n] && cudaMemcpyAsync(er[n], s.er + n, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return CF_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return CF_ERR_CUDA;
    return CF_OK;
}
