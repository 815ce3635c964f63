"""The allocation-free dense transpose product against the regular one.

amfls_gpu_dense_apply_transpose_noalloc serves callers that cannot allocate
device memory (inside CUDA stream capture, in loops that must not synchronise
the device, under a host memory manager that owns all device memory).  It
keeps its partial sums in a fixed device array shared by all calls, so this
test runs it twice in a row (the second call sees the first call's leftover
partials) and compares both results with the regular entry point,
amfls_gpu_operator_apply_transpose on a dense operator, and with a float64
numpy product A^T y, to the product's rounding model.  A third call is
captured into a CUDA graph (capture fails if the call allocates or
synchronises) and the graph replayed on a new y.  This file sorts last so a
stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def native():
    import amfls_solver_gb300 as amfls
    from amfls_solver_gb300 import _native

    amfls.load_library()
    return amfls, _native.load()


def noalloc_transpose(lib, a, y):
    x = torch.empty(a.shape[1], dtype=torch.float64, device=a.device)
    rc = lib.amfls_gpu_dense_apply_transpose_noalloc(
        a.shape[0], a.shape[1], a.data_ptr(), y.data_ptr(), x.data_ptr(),
        torch.cuda.current_stream(a.device).cuda_stream)
    assert rc == 0, lib.amfls_gpu_last_error()
    return x


def test_noalloc_matches_regular_entry_point_twice(native):
    amfls, lib = native
    rng = np.random.default_rng(7)
    a_host = rng.standard_normal((3000, 700))
    a = torch.from_numpy(a_host).cuda()
    op = amfls.DeviceOperator(a)
    for seed in (1, 2):  # two calls in a row share the scratch array
        y_host = np.random.default_rng(seed).standard_normal(3000)
        y = torch.from_numpy(y_host).cuda()
        ref = op.apply(y, transpose=True).cpu().numpy()
        got = noalloc_transpose(lib, a, y).cpu().numpy()
        exact = a_host.T @ y_host
        # gamma_{2 rows + 2} |A|^T |y|: the reference's rounding model for A^T y
        k = 2 * 3000 + 2
        u = np.finfo(np.float64).eps / 2
        bound = (np.abs(a_host).T @ np.abs(y_host)) * (k * u / (1 - k * u))
        assert np.all(np.abs(got - ref) <= 2 * bound)
        assert np.all(np.abs(got - exact) <= 2 * bound)


def test_noalloc_call_is_captured_into_a_graph(native):
    """The call the entry point exists for: inside stream capture, after a
    first call on the device outside capture."""
    amfls, lib = native
    rows, cols = 2500, 900
    a_host = np.random.default_rng(8).standard_normal((rows, cols))
    a = torch.from_numpy(a_host).cuda()
    y = torch.from_numpy(np.random.default_rng(3).standard_normal(rows)).cuda()
    x = torch.empty(cols, dtype=torch.float64, device=a.device)

    def call():
        rc = lib.amfls_gpu_dense_apply_transpose_noalloc(
            rows, cols, a.data_ptr(), y.data_ptr(), x.data_ptr(),
            torch.cuda.current_stream(a.device).cuda_stream)
        assert rc == 0, lib.amfls_gpu_last_error()

    call()  # the first call on the device, outside capture
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        call()
    y_host = np.random.default_rng(12).standard_normal(rows)
    y.copy_(torch.from_numpy(y_host))
    x.fill_(np.nan)
    graph.replay()
    torch.cuda.synchronize()
    got = x.cpu().numpy()
    k = 2 * rows + 2
    u = np.finfo(np.float64).eps / 2
    bound = (np.abs(a_host).T @ np.abs(y_host)) * (k * u / (1 - k * u))
    assert np.all(np.abs(got - a_host.T @ y_host) <= 2 * bound)
    ref = amfls.DeviceOperator(a).apply(y, transpose=True).cpu().numpy()
    assert np.all(np.abs(got - ref) <= 2 * bound)


def test_noalloc_rejects_oversized_input(native):
    _, lib = native
    rc = lib.amfls_gpu_dense_apply_transpose_noalloc(2, (1 << 20) + 1, ctypes.c_void_p(8),
                                                     ctypes.c_void_p(8), ctypes.c_void_p(8), None)
    assert rc == 2
    assert b"exceeds the fixed scratch" in lib.amfls_gpu_last_error()
