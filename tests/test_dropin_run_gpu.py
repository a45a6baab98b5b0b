"""The C++ drop-in binding run as a reference-style driver on the GPU.

A driver written like the reference's main.cpp (main.cpp:143-480, the
dual-time path with the limited fluxes and the Filter) includes
include/channel_flow_gb300_dropin.hpp after a generated Resolution.h,
allocates its arrays as the reference does (double[X_np][Y_m][Z_m]),
registers them with cfdrop::track, calls the routines with the reference's
own signatures in the reference's order for two physical steps (with the
level shift Uq <- U <- U_ done on the host arrays, as main.cpp does) and
writes the final state.  In the no-FMA build that state equals the same two
steps of the C oracle (tests/cases.py port_step) bit for bit.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
DIMS = (12, 10, 8)
STEPS, MAX_IT, TOL = 2, 2, 1e-3

DRIVER = r'''
#include <cstdio>
#include <cstdlib>
#include <initializer_list>
#include "Resolution.h"
#include "channel_flow_gb300_dropin.hpp"

int X_np = X_out + 6;

static cf_field field() { return new double[X_np][Y_m][Z_m]; }

int main(int argc, char **argv)
{
    if (argc != 5) return 2;
    const int steps = std::atoi(argv[3]), iteration_end_step = std::atoi(argv[4]);
    const double deltaT = 0.00000005, tolerance = 0.001;
    const size_t n = (size_t)X_np * Y_m * Z_m;
    // inputs, in the file's order: U1_..U5_, U1..U5, U1q..U5q, J, Y_point,
    // xidx..ztdz, J_u + 9, J_v + 9, J_w + 9
    cf_field in[56];
    for (int a = 0; a < 56; a++) in[a] = field();
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    for (int a = 0; a < 56; a++)
        if (std::fread(&in[a][0][0][0], sizeof(double), n, f) != n) return 4;
    std::fclose(f);
    cf_field *U_ = in, *U = in + 5, *Uq = in + 10, J = in[15], Y_point = in[16], *m = in + 17;
    cf_field *mu = in + 27, *mv = in + 37, *mw = in + 47, J_u = in[26], J_v = in[36], J_w = in[46];
    // outputs and scratch of the routines (Array.h)
    cf_field Ep[3], inFx[5], inFy[5], inFz[5], vF[4], MR[5], ML[5], NR[5], NL[5], LR[5], LL[5], Res[5];
    for (int a = 0; a < 3; a++) Ep[a] = field();
    for (int a = 0; a < 4; a++) vF[a] = field();
    for (int a = 0; a < 5; a++) {
        inFx[a] = field(); inFy[a] = field(); inFz[a] = field();
        MR[a] = field(); ML[a] = field(); NR[a] = field(); NL[a] = field(); LR[a] = field(); LL[a] = field();
        Res[a] = field();
    }
    int (*Nijk)[2] = new int[(X_np - 3) + ny + nz + 7][2];
    int (*ijk)[3] = new int[(X_np - 6) * Y_out * Z_out * 3 + 1][3];

    cfdrop::init(CF_PREC_FP64_EXACT);
    for (int a = 0; a < 56; a++) cfdrop::track(in[a]);
    for (int a = 0; a < 3; a++) cfdrop::track(Ep[a]);
    for (int a = 0; a < 4; a++) cfdrop::track(vF[a]);
    for (int a = 0; a < 5; a++)
        for (cf_field x : {inFx[a], inFy[a], inFz[a], MR[a], ML[a], NR[a], NL[a], LR[a], LL[a], Res[a]})
            cfdrop::track(x);

    Hyperplane(0, Nijk, ijk);
    double er1, er2, er3, er4, er5, E1 = 0, E2 = 0, E3 = 0, E4 = 0, E5 = 0;
    for (int step = 1; step <= steps; step++) {
        for (int iteration = 1; iteration < 50000; iteration++) {
            cfdrop::x_halo(0, U_[0], U_[1], U_[2], U_[3], U_[4]);
            Y_boundary_condition(0, U_[0], U_[1], U_[2], U_[3], U_[4], J);
            Z_boundary_condition(0, U_[0], U_[1], U_[2], U_[3], U_[4], J);
            Filter(0, 0.007, 1., 0., U_[0], U_[1], U_[2], U_[3], U_[4], Y_point, Ep[0], Ep[1], Ep[2], J);
            Flux_X_limiter(0, U_[0], U_[1], U_[2], U_[3], U_[4], MR[0], MR[1], MR[2], MR[3], MR[4],
                           ML[0], ML[1], ML[2], ML[3], ML[4], J, J_u,
                           mu[0], mu[1], mu[2], mu[3], mu[4], mu[5], mu[6], mu[7], mu[8],
                           inFx[0], inFx[1], inFx[2], inFx[3], inFx[4], Ep[0]);
            Flux_Y_limiter(0, U_[0], U_[1], U_[2], U_[3], U_[4], MR[0], MR[1], MR[2], MR[3], MR[4],
                           ML[0], ML[1], ML[2], ML[3], ML[4], J, J_v,
                           mv[0], mv[1], mv[2], mv[3], mv[4], mv[5], mv[6], mv[7], mv[8],
                           inFy[0], inFy[1], inFy[2], inFy[3], inFy[4], Ep[1]);
            Flux_Z_limiter(0, U_[0], U_[1], U_[2], U_[3], U_[4], MR[0], MR[1], MR[2], MR[3], MR[4],
                           ML[0], ML[1], ML[2], ML[3], ML[4], J, J_w,
                           mw[0], mw[1], mw[2], mw[3], mw[4], mw[5], mw[6], mw[7], mw[8],
                           inFz[0], inFz[1], inFz[2], inFz[3], inFz[4], Ep[2]);
            Viscous_terms(0, U_[0], U_[1], U_[2], U_[3], U_[4], vF[0], vF[1], vF[2], vF[3], J,
                          m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8],
                          J_u, mu[0], mu[1], mu[2], mu[3], mu[4], mu[5], mu[6], mu[7], mu[8],
                          J_v, mv[0], mv[1], mv[2], mv[3], mv[4], mv[5], mv[6], mv[7], mv[8],
                          J_w, mw[0], mw[1], mw[2], mw[3], mw[4], mw[5], mw[6], mw[7], mw[8],
                          LR[0], LR[1], LR[2], LR[3], LR[4], LL[0], LL[1], LL[2], LL[3], LL[4],
                          MR[0], MR[1], MR[2], MR[3], MR[4], ML[0], ML[1], ML[2], ML[3], ML[4],
                          NR[0], NR[1], NR[2], NR[3], NR[4], NL[0], NL[1], NL[2], NL[3], NL[4]);
            Dual_time_stepping(0, deltaT, &er1, &er2, &er3, &er4, &er5, Nijk, ijk,
                               U_[0], U_[1], U_[2], U_[3], U_[4], U[0], U[1], U[2], U[3], U[4],
                               Uq[0], Uq[1], Uq[2], Uq[3], Uq[4], J,
                               m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8],
                               inFx[0], inFx[1], inFx[2], inFx[3], inFx[4], inFy[0], inFy[1], inFy[2], inFy[3], inFy[4],
                               inFz[0], inFz[1], inFz[2], inFz[3], inFz[4], vF[0], vF[1], vF[2], vF[3],
                               MR[0], MR[1], MR[2], MR[3], MR[4], NR[0], NR[1], NR[2], NR[3], NR[4],
                               NL[0], NL[1], NL[2], NL[3], NL[4], Res[0], Res[1], Res[2], Res[3], Res[4]);
            E1 = E1 > er1 ? E1 : er1; E2 = E2 > er2 ? E2 : er2; E3 = E3 > er3 ? E3 : er3;
            E4 = E4 > er4 ? E4 : er4; E5 = E5 > er5 ? E5 : er5;
            er1 /= E1; er2 /= E2; er3 /= E3; er4 /= E4; er5 /= E5;
            if ((er1 < tolerance && er2 < tolerance && er3 < tolerance && er4 < tolerance) ||
                iteration == iteration_end_step) {
                Driven_force(0, U[1], J);
                // the level shift of main.cpp:440-455 on the host arrays
                for (int a = 0; a < 5; a++) {
                    cfdrop::to_host(U_[a]);
                    cfdrop::to_host(U[a]);
                }
                for (int a = 0; a < 5; a++)
                    for (int i = 3; i <= X_out + 2; i++)
                        for (int j = 2; j < ny + 1; j++)
                            for (int k = 2; k < nz + 1; k++) {
                                Uq[a][i][j][k] = U[a][i][j][k];
                                U[a][i][j][k] = U_[a][i][j][k];
                            }
                for (int a = 0; a < 5; a++) {
                    cfdrop::to_device(U[a]);
                    cfdrop::to_device(Uq[a]);
                }
                break;
            }
        }
    }
    f = std::fopen(argv[2], "wb");
    if (!f) return 5;
    for (int a = 0; a < 15; a++) {
        cfdrop::to_host(in[a]);
        std::fwrite(&in[a][0][0][0], sizeof(double), n, f);
    }
    std::fclose(f);
    return 0;
}
'''


def _build(tmp_path, g):
    from channel_flow_gb300 import _lib
    from oracle import build_ref
    (tmp_path / "Resolution.h").write_text(build_ref.resolution_header(g.X_out, g.Y_out, g.Z_out, g.deltaXI,
                                                                       g.deltaET, g.deltaZT))
    (tmp_path / "driver.cpp").write_text(DRIVER)
    cuda = Path("/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O1", f"-I{tmp_path}", f"-I{ROOT / 'include'}", str(tmp_path / "driver.cpp"),
           "-o", str(tmp_path / "driver"), f"-L{_lib.LIB_PATH.parent}", "-lcfgb300",
           f"-Wl,-rpath,{_lib.LIB_PATH.parent}"]
    for libdir in (cuda / "lib64", cuda / "targets" / "sbsa-linux" / "lib", cuda / "targets" / "x86_64-linux" / "lib"):
        if libdir.exists():
            cmd += [f"-L{libdir}", f"-Wl,-rpath,{libdir}"]
    cmd += ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return tmp_path / "driver"


def test_dropin_driver_runs_physical_steps(tmp_path, port, cuda_lib):
    g = cases.grid(DIMS)
    f = cases.step_case(g, seed=2)
    inputs = f["U_"] + f["U"] + f["Uq"] + [f["J"], f["Y_point"]] + f["cell_metric"]
    for d in range(3):
        inputs += [f["face_J"][d]] + f["face_metric"][d]
    assert len(inputs) == 56
    with open(tmp_path / "in.bin", "wb") as fh:
        for a in inputs:
            np.ascontiguousarray(a, dtype=np.float64).tofile(fh)
    exe = _build(tmp_path, g)
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(STEPS), str(MAX_IT)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])
    assert r.stdout.count("Q0=") == STEPS          # Driven_force prints once per step, as the reference does
    got = np.fromfile(tmp_path / "out.bin", dtype=np.float64).reshape(15, *g.shape)
    E = [0.0] * 5
    for _ in range(STEPS):
        cases.port_step(port, g, f, cases.DELTA_T, MAX_IT, TOL, E)
    want = f["U_"] + f["U"] + f["Uq"]
    for a in range(15):
        assert np.array_equal(got[a], want[a], equal_nan=True), a
