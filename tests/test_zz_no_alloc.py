"""The allocation-free compliance dot product (anl_dot_static) against anl_dot.

anl_dot_static exists for callers that cannot allocate device memory (memory-pool hooks
and allocator callbacks, frameworks that own the whole pool): it keeps its reduction scratch in
a fixed array inside the library. This test calls it through the C ABI twice in a row on
different data and compares each result with the context-based anl_dot, at the FP64
tolerance the other dot-product tests use. It sits in its own file, collected last."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_static_dot_matches_context_dot_on_two_calls():
    from anneal_gb300 import _native as N
    from anneal_gb300.context import Context
    lib = N.load()
    shape = (96, 48, 48)                    # 698,691 values: 11 chunks of 65,536 per CTA
    ctx = Context(shape, 1.0, 0.3)
    n = ctx.ndof
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(1234)
    for call in range(2):
        a = torch.randn(n, dtype=torch.float64, device="cuda", generator=g) * (1 + call)
        b = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
        want = ctx.dot(a, b)
        st = lib.anl_dot_static(_ptr(a), _ptr(b), n, _ptr(out), stream)
        assert st == N.ANL_OK, N.last_error()
        torch.cuda.synchronize()
        got = float(out.item())
        scale = float((a.abs() * b.abs()).sum())
        assert abs(got - want) <= 1e-12 * scale, (call, got, want)
    ctx.close()


def test_static_dot_rejects_oversized_and_handles_empty():
    from anneal_gb300 import _native as N
    lib = N.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    a = torch.ones(8, dtype=torch.float64, device="cuda")
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    st = lib.anl_dot_static(_ptr(a), _ptr(a), (1 << 28) + 1, _ptr(out), stream)
    assert st == N.ANL_ERR_BADARG and "exceed the maximum" in N.last_error()
    assert lib.anl_dot_static(_ptr(a), _ptr(a), 0, _ptr(out), stream) == N.ANL_OK
    torch.cuda.synchronize()
    assert float(out.item()) == 0.0
    assert lib.anl_dot_static(_ptr(a), _ptr(a), 8, _ptr(out), stream) == N.ANL_OK
    torch.cuda.synchronize()
    assert float(out.item()) == 8.0
