"""libbtgpu.so loads and exports every function include/btgpu.h declares (no
compute calls: these run without a GPU)."""

import ctypes
import os
import re

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "btgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*int\s+(bt_\w+)\s*\(", src, flags=re.M)))


def test_header_and_binding_agree(pkg):
    assert declared_functions() == sorted(pkg._native.EXPORTS)


def test_library_exports_every_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.bt_version() == 100


def test_null_arguments_are_rejected(lib):
    assert lib.bt_create(None, 0) == 1          # BT_ERR_INVALID, no device touched
    assert lib.bt_destroy(None) == 0
    assert lib.bt_assemble(None) == 1
    assert lib.bt_solve(None, 1, None, None, None, None, 0, 1e-9, 10, None, None, None, None) == 1
    buf = ctypes.create_string_buffer(8)
    assert lib.bt_last_error(None, buf, 8) == 1
    assert lib.bt_set_periodic(None, None) == 1
    assert lib.bt_periodic_info(None, None) == 1
    assert lib.bt_set_schedule_phase(None, None, 1, 1) == 1
    assert lib.bt_adjoint_batch(None, 1, None, None, None, 1e-9, 10, 0, None, None, None, None, None) == 1
    assert lib.bt_adjoint_multi(None, 1, None, None, None, None, 1e-9, 10, 0, None, None, None, None, None) == 1
    assert lib.bt_set_kappa_mode(None, 1) == 1
    assert lib.bt_set_periodic_mode(None, 1) == 1
    assert lib.bt_set_schedule_integral(None, None, None, 1, 1) == 1
    assert lib.bt_strong_periodic_info(None, None, None, None) == 1
    assert lib.bt_adjoint_cells(None, 1.0, None, 0, None, 1e-9, 10, 0, None, None, None, None, None) == 1
    assert lib.bt_adjoint_batch_cells(None, 1, None, None, None, None, 1e-9, 10, 0, None, None, None, None,
                                      None) == 1
    assert lib.bt_solve_dev(None, 1, None, None, None, None, 0, 1e-9, 10, None, None, None, None) == 1


def test_no_cpu_fallback_without_library(pkg, tmp_path, monkeypatch):
    import importlib
    nat = importlib.import_module(pkg.__name__ + "._native")
    saved = nat._lib
    try:
        nat._lib = None
        try:
            nat.load(str(tmp_path / "missing.so"))
        except RuntimeError as e:
            assert "no CPU fallback" in str(e)
        else:
            raise AssertionError("loading a missing library must fail")
    finally:
        nat._lib = saved
