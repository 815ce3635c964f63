"""Host-side checks of the native library that need no GPU.

The C-ABI library must load and export every entry point include/amfls_gpu.h
declares; argument errors that are caught before any CUDA call must come back
as error codes with a message.  No compute call is made here.
"""
import ctypes
import re
from pathlib import Path

import pytest

from amfls_solver_gb300 import _native
from amfls_solver_gb300.build import LIB

HEADER = Path(__file__).resolve().parents[1] / "include" / "amfls_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(amfls_gpu_[a-z_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not LIB.exists():
        from amfls_solver_gb300 import build
        build.build()
    return _native.load()


def test_header_declares_the_exported_list():
    assert declared_functions() == sorted(_native.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_default_options_match_reference_defaults(lib):
    o = _native.default_options()
    assert o.regularization == 0.0
    assert o.tolerance == 1e-8
    assert o.failure_probability == 1e-6
    assert (o.maximum_epochs, o.maximum_depth, o.maximum_auxiliary_width,
            o.maximum_basis_size) == (0, 0, 0, 0)
    assert (o.seed, o.stream) == (0, 0)
    assert o.auxiliary_width == 4 and o.stop_early == 1


def test_null_arguments_are_errors_not_crashes(lib):
    res = _native.Result()
    o = _native.default_options()
    rc = lib.amfls_gpu_solve_amfls(None, None, ctypes.byref(o), None, ctypes.byref(res), None,
                                   None, 0, None)
    assert rc == 1
    assert b"solution must not be null" in lib.amfls_gpu_last_error()
    assert lib.amfls_gpu_operator_rows(None) == -1
    assert lib.amfls_gpu_operator_cols(None) == -1
    handle = ctypes.c_void_p()
    rc = lib.amfls_gpu_csr_operator_create(0, 5, None, None, None, 0, None, ctypes.byref(handle))
    assert rc == 1 and handle.value is None
    assert b"dimensions are invalid" in lib.amfls_gpu_last_error()


def test_status_constants_match_reference():
    text = HEADER.read_text()
    for name, value in [("SUCCESS", 0), ("WORK_LIMIT", 1), ("BASIS_LIMIT", 2),
                        ("PRECISION_LIMIT", 3), ("NUMERICAL_BREAKDOWN", 4)]:
        assert re.search(rf"AMFLS_STATUS_{name} = {value}\b", text)


def test_mixed_entry_points_reject_bad_arguments(lib):
    handle = ctypes.c_void_p()
    rc = lib.amfls_gpu_reduced_operator_create(None, 3, None, ctypes.byref(handle))
    assert rc == 1 and b"FP32 (1) or BF16 (2)" in lib.amfls_gpu_last_error()
    rc = lib.amfls_gpu_reduced_operator_create(None, 1, None, ctypes.byref(handle))
    assert rc == 1 and b"operator must not be null" in lib.amfls_gpu_last_error()
    assert handle.value is None
    res = _native.Result()
    o = _native.default_options()
    rc = lib.amfls_gpu_solve_amfls_mixed(None, None, None, ctypes.byref(o), 1e-6, 4, None,
                                         ctypes.byref(res), None, None, 0, None)
    assert rc == 1 and b"operator must not be null" in lib.amfls_gpu_last_error()


def test_lsqr_lsmr_entry_points_reject_bad_arguments(lib):
    o = _native.BaselineOptions()
    lib.amfls_gpu_default_baseline_options(ctypes.byref(o))
    assert (o.regularization, o.tolerance, o.maximum_iterations) == (0.0, 1e-8, 0)
    res = _native.Result()
    for name in ("amfls_gpu_solve_lsqr", "amfls_gpu_solve_lsmr"):
        fn = getattr(lib, name)
        rc = fn(None, None, ctypes.byref(o), None, ctypes.byref(res), None, None, 0, None)
        assert rc == 1 and b"solution must not be null" in lib.amfls_gpu_last_error()
        rc = fn(None, None, None, ctypes.c_void_p(16), ctypes.byref(res), None, None, 0, None)
        assert rc == 1 and b"must not be null" in lib.amfls_gpu_last_error()


def test_callback_operator_needs_both_products(lib):
    cb = _native.Callbacks()
    handle = ctypes.c_void_p()
    rc = lib.amfls_gpu_callback_operator_create(10, 5, ctypes.byref(cb), None, ctypes.byref(handle))
    assert rc == 1 and b"apply and apply_transpose" in lib.amfls_gpu_last_error()
    rc = lib.amfls_gpu_callback_operator_create(10, 5, None, None, ctypes.byref(handle))
    assert rc == 1 and handle.value is None


def test_schedule_query_rejects_null_buffers(lib):
    rc = lib.amfls_gpu_csr_operator_schedule(None, None, None)
    assert rc == 1


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the C structs against the header itself: a C
    program compiled from include/amfls_gpu.h prints every field's offset
    and each struct's size."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"amfls_gpu_options": _native.Options, "amfls_gpu_result": _native.Result,
               "amfls_gpu_baseline_options": _native.BaselineOptions,
               "amfls_gpu_validation_error_model": _native.ValidationModel,
               "amfls_gpu_operator_callbacks": _native.Callbacks}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "amfls_gpu.h"',
             'int main(void) {']
    for cname, mirror in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in mirror._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(HEADER.parent), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, mirror in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(mirror), cname
        for field, _ in mirror._fields_:
            assert got[(cname, field)] == getattr(mirror, field).offset, (cname, field)


def test_reduced_basis_defaults_off_and_probe_checks_sizes(lib):
    o = _native.default_options()
    assert o.reduced_basis == 0 and o.use_graphs == 1
    sec = (ctypes.c_double * 2)()
    rc = lib.amfls_gpu_probe_reorthogonalization_reduced(0, 10, 1, 1, None, sec, None)
    assert rc == 1 and b"probe sizes must be positive" in lib.amfls_gpu_last_error()
    rc = lib.amfls_gpu_probe_reorthogonalization_reduced(10, 10, 1, 3, None, sec, None)
    assert rc == 1 and b"probe storage must be 1 (FP32) or 2 (FP16)" in lib.amfls_gpu_last_error()


def test_invalid_reduced_basis_is_rejected_before_device_work(lib):
    """Every solve entry point converts its options first: an out-of-range
    reduced_basis is an argument error, reported before the operator is
    looked at or anything is allocated."""
    o = _native.default_options()
    o.reduced_basis = 3
    res = _native.Result()
    dummy = ctypes.c_void_p(16)
    expect = b"options.reduced_basis must be 0 (off), 1 (FP32) or 2 (FP16)"
    calls = {
        "solve_amfls": lambda: lib.amfls_gpu_solve_amfls(
            None, None, ctypes.byref(o), dummy, ctypes.byref(res), None, None, 0, None),
        "solve_fixed_rbgk": lambda: lib.amfls_gpu_solve_fixed_rbgk(
            None, None, ctypes.byref(o), dummy, ctypes.byref(res), None, None, 0, None),
        "solve_amfls_mixed": lambda: lib.amfls_gpu_solve_amfls_mixed(
            None, None, None, ctypes.byref(o), 1e-6, 4, dummy, ctypes.byref(res), None, None, 0,
            None),
        "solve_amfls_controlled": lambda: lib.amfls_gpu_solve_amfls_controlled(
            None, None, ctypes.byref(o), None, 0.0, 0, None, 0, None, dummy, ctypes.byref(res),
            None, None, 0, None),
        "solve_amfls_replay": lambda: lib.amfls_gpu_solve_amfls_replay(
            None, None, ctypes.byref(o), None, 0, None, 0, None, None, dummy,
            ctypes.byref(res), None, None, 0, None),
    }
    for name, call in calls.items():
        assert call() == 1, name
        assert expect in lib.amfls_gpu_last_error(), name
    ops = (ctypes.c_void_p * 1)(None)
    bs = (ctypes.c_void_p * 1)(16)
    xs = (ctypes.c_void_p * 1)(16)
    rc = lib.amfls_gpu_solve_amfls_batch(1, ops, bs, ctypes.byref(o), xs, ctypes.byref(res),
                                         None, 1, None)
    assert rc == 1 and expect in lib.amfls_gpu_last_error()
    o.reduced_basis = -1
    assert calls["solve_amfls"]() == 1 and expect in lib.amfls_gpu_last_error()


def test_reduced_basis_argument_mapping():
    from amfls_solver_gb300 import binding

    assert [binding._reduced_storage(v) for v in (False, None, 0, True, 1, "fp32", 2, "fp16")] == \
        [0, 0, 0, 1, 1, 1, 2, 2]
    for bad in ("bf16", 3, 1.5):
        with pytest.raises(ValueError):
            binding._reduced_storage(bad)
