"""The C++ drop-in binding (include/channel_flow_gb300_dropin.hpp) compiles
with the reference's grid header and links against libcfgb300.so: a driver
written like main.cpp, calling every routine with the reference's
signatures, builds without the reference's own routine sources."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

DRIVER = r'''
#include "Resolution.h"
#include "channel_flow_gb300_dropin.hpp"
int X_np = X_out + 6;
int main(int argc, char **)
{
    if (argc > 99) {   /* compiled and linked, never run here */
        cf_field a = new double[X_np][Y_m][Z_m];
        int (*Nijk)[2] = new int[(X_np - 3) + ny + nz + 7][2];
        int (*ijk)[3] = new int[(X_np - 6) * Y_out * Z_out * 3][3];
        double er1, er2, er3, er4, er5;
        cfdrop::init();
        cfdrop::track(a);
        cfdrop::x_halo(0, a, a, a, a, a);
        Y_boundary_condition(0, a, a, a, a, a, a);
        Z_boundary_condition(0, a, a, a, a, a, a);
        Filter(0, 0.007, 1., 0., a, a, a, a, a, a, a, a, a, a);
        Flux_X_limiter(0, a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a, a,a,a,a,a,a,a,a,a, a,a,a,a,a, a);
        Flux_Y_limiter(0, a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a, a,a,a,a,a,a,a,a,a, a,a,a,a,a, a);
        Flux_Z_limiter(0, a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a, a,a,a,a,a,a,a,a,a, a,a,a,a,a, a);
        Flux_X(0, a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a, a,a,a,a,a,a,a,a,a, a,a,a,a,a, a);
        Viscous_terms(0, a,a,a,a,a, a,a,a,a, a, a,a,a,a,a,a,a,a,a, a,a,a,a,a,a,a,a,a,a,
                      a,a,a,a,a,a,a,a,a,a, a,a,a,a,a,a,a,a,a,a,
                      a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a,a,a,a);
        RK3NODT(0, 1, 5e-8, &er1, &er2, &er3, &er4, &er5,
                a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a, a,a,a,a,a,a,a,a,a,
                a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a,a,a, a,a,a,a,a);
        Hyperplane(0, Nijk, ijk);
        Driven_force(0, a, a);
        Statistic(0, 1, 1, 5000, a,a,a,a,a, a, a, a,a,a,a,a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a);
        Output(10, 0, a,a,a,a,a, a,a,a,a,a, a);
        Initial_condition(0, a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a);
        Dual_time_stepping(0, 5e-8, &er1, &er2, &er3, &er4, &er5, Nijk, ijk,
                a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a, a,a,a,a,a,a,a,a,a,
                a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a,a,a, a,a,a,a,a,
                a,a,a,a,a, a,a,a,a,a, a,a,a,a,a);
        DPLUSGS(0, 5e-8, &er1, &er2, &er3, &er4, &er5,
                a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a, a,a,a,a,a,a,a,a,a,
                a,a,a,a,a, a,a,a,a,a, a,a,a,a,a, a,a,a,a, a,a,a,a,a,
                a,a,a,a,a, a,a,a,a,a, a,a,a,a,a);
        Jacobian_u(0, a,a,a,a,a,a,a,a,a,a);
        Jacobian_v(0, a,a,a,a,a,a,a,a,a,a, a,a,a,a,a,a,a,a,a,a);
        Jacobian_w(0, a,a,a,a,a,a,a,a,a,a);
        cfdrop::to_host(a);
    }
    return 0;
}
'''


def test_dropin_header_compiles_and_links(tmp_path, cuda_lib):
    from channel_flow_gb300 import _lib
    from oracle import build_ref
    (tmp_path / "Resolution.h").write_text(build_ref.resolution_header(16, 12, 10, 0.001, 1 / 12, 0.001))
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
