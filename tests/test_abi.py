"""The C-ABI library loads and exports every entry point of include/hcc.h; host-side checks that need no GPU."""
import ctypes as C
import re
import sys

import pytest

from conftest import ROOT


def _declared_symbols():
    text = (ROOT / "include" / "hcc.h").read_text()
    # function declarations: a line that starts with a return type and names an hcc_ function
    return sorted(set(re.findall(r"(?m)^(?:const\s+)?[a-z_]+\s*\**\s*(hcc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_entry_points():
    names = _declared_symbols()
    for required in ("hcc_create", "hcc_destroy", "hcc_upload_cloud", "hcc_build_neighbours", "hcc_prepare_geometry",
                     "hcc_upload_state", "hcc_time_step", "hcc_step", "hcc_download_state", "hcc_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(cuda_lib):
    for name in _declared_symbols():
        assert hasattr(cuda_lib, name), name


def test_status_strings_and_defaults(hcc, cuda_lib):
    assert cuda_lib.hcc_status_string(0) == b"HCC_OK"
    assert cuda_lib.hcc_status_string(2) == b"HCC_ERR_CAPACITY"
    assert cuda_lib.hcc_last_error(None) == b"null context"
    cfg_c = hcc.HccConfig()
    cuda_lib.hcc_config_defaults(C.byref(cfg_c))
    cfg_py = hcc.config_defaults()
    assert bytes(cfg_c) == bytes(cfg_py)        # the Python twin matches the C defaults field for field


@pytest.mark.parametrize("field,value,status", [
    ("dim", 4, 1), ("n_vars", 0, 1), ("muscl_order", 5, 7), ("radius", 0.0, 1), ("abi_version", 99, 1),
])
def test_create_rejects_bad_configs_before_touching_the_gpu(hcc, cuda_lib, field, value, status):
    cfg = hcc.config_defaults()
    cfg.radius = 0.025
    setattr(cfg, field, value)
    h = C.c_void_p()
    st = cuda_lib.hcc_create(C.byref(cfg), 0, C.byref(h))
    assert st == status
    assert cuda_lib.hcc_last_error(h)            # a message is available
    cuda_lib.hcc_destroy(h)


def test_euler_needs_matching_n_vars(hcc, cuda_lib):
    cfg = hcc.config_defaults()
    cfg.radius, cfg.pde, cfg.dim, cfg.n_vars = 0.025, 1, 2, 3
    h = C.c_void_p()
    assert cuda_lib.hcc_create(C.byref(cfg), 0, C.byref(h)) == 1
    assert b"n_vars" in cuda_lib.hcc_last_error(h)
    cuda_lib.hcc_destroy(h)


def test_missing_library_fails_loudly(hcc, tmp_path):
    with pytest.raises(hcc.HCCError):
        hcc.load_library(tmp_path / "nope.so")


def test_upwind_is_first_order_muscl(hcc):
    """UpwindDivergence(:Classic) is the first-order MUSCL scheme (unit_core.jl:937-945)."""
    cl = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), 0.05, 0.125, periodic=True)
    a = hcc.make_config(hcc.LinearAdvection(((1.0,), (1.0,))), cl, scheme=hcc.Upwind(2))
    b = hcc.make_config(hcc.LinearAdvection(((1.0,), (1.0,))), cl, scheme=hcc.MUSCL(1, 2))
    assert bytes(a) == bytes(b)


def test_struct_layouts_match_the_header(hcc, tmp_path):
    """Every struct of include/hcc.h has the size and field offsets of its ctypes mirror (compiled with the host C
    compiler against the header; no GPU)."""
    import ctypes as C
    import shutil
    import subprocess
    import sys
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    abi = sys.modules["hcc_gb300._abi"]
    pairs = {"hcc_config": abi.HccConfig, "hcc_counters": abi.HccCounters, "hcc_mover": abi.HccMover,
             "hcc_kernel_times": abi.HccKernelTimes, "hcc_mlp_config": abi.HccMlpConfig,
             "hcc_tuning": abi.HccTuning, "hcc_tune_report": abi.HccTuneReport}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "hcc.h"', "int main(void) {"]
    for cname, cls in pairs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = ROOT / "include"
    subprocess.run([cc, "-std=c11", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, cls in pairs.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_build_info_names_the_launch_bounds(cuda_lib):
    info = cuda_lib.hcc_build_info().decode()
    keys = dict(kv.split("=") for kv in info.split())
    assert set(keys) == {"flux_block", "flux_minb", "flux_minb_wide", "flux_minb64", "flux_minb_many", "fp32_packed",
                         "tile_flux_pf", "tile_stage_unroll", "flux_kahan_block",
                         "tile_flux_group", "tile_gather_group"}
    assert all(v.isdigit() for v in keys.values()) and keys["flux_block"] == "128"


def test_bindings_call_only_declared_entry_points():
    """The Julia shim's ccalls and the ctypes prototype table name only entry points of include/hcc.h, and the
    ctypes table covers all of them."""
    import importlib.util
    names = set(_declared_symbols())
    jl = (ROOT / "hypercloudcore.jl_gb300" / "julia" / "HCCGB300.jl").read_text()
    called = set(re.findall(r"ccall\(\(:(hcc_[a-z0-9_]+),", jl))
    assert called and called <= names, called - names
    spec = importlib.util.spec_from_file_location("_abi_only", ROOT / "hypercloudcore.jl_gb300" / "_abi.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    bound = {p[0] for p in mod.PROTOTYPES}
    assert bound == names, (bound ^ names)
