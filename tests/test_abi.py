"""The C-ABI library loads and exports every symbol the public header declares."""

import ctypes
import os
import re

import pytest

from conftest import ROOT


def _header_symbols():
    src = open(os.path.join(ROOT, "include", "l3es_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(l3es_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = _header_symbols()
    for s in ("l3es_plan_create", "l3es_step", "l3es_rhs", "l3es_rfftn", "l3es_irfftn",
              "l3es_last_error"):
        assert s in syms


def test_library_exports_all_header_symbols():
    from l3es import _native

    if not os.path.exists(_native.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    lib = _native.load()
    for s in _header_symbols():
        assert hasattr(lib, s), f"{s} missing from {_native.LIB_PATH}"
        assert s in _native._SIGNATURES, f"{s} has no ctypes signature"
    assert lib.l3es_version().decode().startswith("l3es_gb300")


def test_invalid_arguments_fail_without_gpu():
    """Argument validation runs before any device work and reports a message."""
    from l3es import _native

    if not os.path.exists(_native.LIB_PATH):
        pytest.skip("library not built")
    lib = _native.load()
    h = ctypes.c_void_p()
    d = _native.PlanDesc(dim=4, n=64, batch=1, nu=0.01, dt=0.01)
    assert lib.l3es_plan_create(ctypes.byref(d), ctypes.byref(h)) == -1
    assert b"dim" in lib.l3es_last_error()
    d = _native.PlanDesc(dim=3, n=100, batch=1, nu=0.01, dt=0.01)
    assert lib.l3es_plan_create(ctypes.byref(d), ctypes.byref(h)) == -1
    assert b"not supported" in lib.l3es_last_error()
    assert lib.l3es_step(None, None, None, 1, None, None) == -1
    assert lib.l3es_plan_check(None) == -1
    form = ctypes.c_int32()
    assert lib.l3es_plan_get_step_form(None, ctypes.byref(form)) == -1
    assert b"null" in lib.l3es_last_error()
    assert lib.l3es_plan_set_step_form(None, 1) == -1
    assert b"step_form" in lib.l3es_last_error()
    sched = (ctypes.c_int32 * 4)()
    assert lib.l3es_plan_get_schedule(None, sched) == -1
    assert lib.l3es_plan_autotune(None, None, None) == -1


def test_header_is_plain_c99(tmp_path):
    """The public header compiles as C99 (what a cgo / FFI / C caller includes): a
    translation unit that takes the address of every declared entry point."""
    import shutil
    import subprocess

    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    syms = _header_symbols()
    src = tmp_path / "use_header.c"
    src.write_text('#include "l3es_gb300.h"\n#include <stddef.h>\ntypedef void (*l3es_fn)(void);\n'
                   "l3es_fn l3es_entry_points[] = {\n" + "".join(f"    (l3es_fn)&{s},\n" for s in syms)
                   + "    NULL};\n")
    res = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-fsyntax-only",
                          "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


def test_noalloc_wrapper_rejects_bad_inputs_before_launching():
    """The Python wrapper of the allocation-free entry point validates shapes, dtypes
    and sizes on the host and raises before anything reaches the library (CPU tensors:
    a launch would fail differently)."""
    import torch

    from l3es import _native

    n, c = 16, 8
    uh3 = torch.zeros(3, n, n, n // 2 + 1, dtype=torch.complex64)
    r3 = torch.zeros(10, 3, dtype=torch.float64)
    bad = [
        # positions of the wrong dimension (reads past the end of r in the kernel)
        dict(dim=3, uh=uh3, r=torch.zeros(10, 2, dtype=torch.float64)),
        # spectrum of a larger grid than n_fine says, and of a smaller one
        dict(dim=3, uh=torch.zeros(3, 2 * n, 2 * n, n + 1, dtype=torch.complex64), r=r3),
        dict(dim=3, uh=torch.zeros(3, n, n, n // 2, dtype=torch.complex64), r=r3),
        # wrong dtype of the spectrum
        dict(dim=3, uh=torch.zeros(3, n, n, n // 2 + 1, dtype=torch.complex128), r=r3),
        # non-contiguous spectrum
        dict(dim=3, uh=torch.zeros(3, n, n, n + 2, dtype=torch.complex64)[..., ::2], r=r3),
        # a 2D call with a 3D spectrum
        dict(dim=2, uh=uh3, r=torch.zeros(10, 2, dtype=torch.float64)),
        # float32 positions
        dict(dim=3, uh=uh3, r=torch.zeros(10, 3, dtype=torch.float32)),
    ]
    for case in bad:
        out = torch.zeros(case["r"].shape, dtype=torch.float64)
        with pytest.raises(ValueError):
            _native.interp_dft_noalloc(case["dim"], n, c, case["uh"], case["r"], out)
