"""The C-ABI library builds for sm_103a, loads, and exports every function
the public header declares (no GPU needed: nothing is called)."""
import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "channel_flow_gb300.h"


def declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cf_[A-Za-z0-9_]+)\s*\(", text)))


def test_header_declares_all_routines():
    names = declared()
    for routine in ("Y_boundary_condition", "Z_boundary_condition", "Flux_X_limiter", "Flux_Y_limiter",
                    "Flux_Z_limiter", "Flux_X", "Flux_Y", "Flux_Z", "Viscous_terms", "Filter", "RK3NODT",
                    "Hyperplane", "Dual_time_stepping", "DPLUSGS", "Jacobian_u", "Jacobian_v", "Jacobian_w"):
        assert "cf_" + routine in names


def test_library_exports_header(cuda_lib):
    from channel_flow_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\s[TW]\s+(cf_\w+)$", out, flags=re.M))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    # the Python binding covers every exported entry point
    assert set(declared()) <= set(_lib.EXPORTED)


def test_library_is_sm103a(cuda_lib):
    from channel_flow_gb300 import _lib
    out = subprocess.run(["cuobjdump", "--list-elf", str(_lib.LIB_PATH)], capture_output=True, text=True)
    if out.returncode == 0:
        assert "sm_103a" in out.stdout


def test_version_and_errors(cuda_lib):
    assert cuda_lib.cf_library_version() >= 100
    assert cuda_lib.cf_error_string(0) == b"ok"
