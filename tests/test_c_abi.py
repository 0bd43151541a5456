"""The C ABI library (no GPU needed): libuds.so builds for sm_103a, loads,
and exports every entry point include/uds.h declares; the ctypes table
covers exactly those."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "uds.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(uds_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_header():
    from unbiased_differentiable_splatting_gb300 import _build, _lib
    _build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", _build.LIB], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (uds_[a-z0-9_]+)", out))
    names = declared()
    assert names, "no declarations parsed"
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert sorted(_lib.exported_symbols()) == names


def test_library_loads_without_gpu():
    from unbiased_differentiable_splatting_gb300 import _lib
    L = _lib.load()
    assert L.uds_version() == 100
    assert L.uds_status_string(2).decode() == "workspace too small"
    # size queries are host-only
    prm = _lib.SampleParams(B=1, N=1000, W=64, H=64, K=8, focal=50.0, smoothing=0.0, precision=0.01, max_degree=16,
                            std_batch=1, coef_pool=0, seed=0)
    assert L.uds_sample_workspace_size(prm) > 1000 * 64
    prm.K = 65
    assert L.uds_sample_workspace_size(prm) == 0
    assert L.uds_splat_workspace_size(2, 100) >= 2 * 100 * 64


def test_invalid_arguments_are_rejected_on_the_host():
    from unbiased_differentiable_splatting_gb300 import _lib
    L = _lib.load()
    # B = 0 and NULL pointers are refused before anything is enqueued
    assert L.uds_transform_forward(1, 0, None, 1, 10, None, None, None) == 1
    assert L.uds_filter_forward(1, 4, 4, 99, None, None, 1.0, 1, 10, None, None, None, None) == 1
    prm = _lib.SampleParams(B=1, N=10, W=8, H=8, K=4, focal=8.0, smoothing=0.0, precision=0.01, max_degree=16,
                            std_batch=1, coef_pool=0, seed=0)
    assert L.uds_sample(prm, None, None, None, None, None, None, None, None, 0, None) == 1


def test_sm103a_code_object():
    """The build targets sm_103a only (checked from the build flags)."""
    from unbiased_differentiable_splatting_gb300 import _build
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.ARCH)


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of uds_sample_params and uds_view_desc have the C
    header's size and field offsets (compiled with the host C compiler)."""
    import shutil
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no host C compiler")
    from unbiased_differentiable_splatting_gb300._lib import SampleParams, ViewDesc
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    structs = {"uds_sample_params": SampleParams, "uds_view_desc": ViewDesc}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "uds.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = str(tmp_path / "layout")
    subprocess.run([cc, "-std=c11", "-I", inc, str(src), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
