"""ug4gb_vector_dot_noalloc, the dot product that allocates no device memory,
called through the C ABI and checked against ug4gb_vector_dot.

Callers that cannot allocate (an application whose allocator owns the GPU's
memory, or a phase where cudaMalloc/cudaFree must not run) use it; besides
the values, the tests check that a warmed call leaves the device's free
memory unchanged and that the largest n the static scratch allows works.

The two entry points sum the same products in a different order, so they
are compared within 1e-12 * sum_i |a_i b_i| (rounding of an FP64 sum of up to
67 million terms, summed in blocks of 8192).  Two calls in a row must give bit-identical results:
the static scratch has to be left clean by the first call.  This file runs
last so that it also sees the library after every other test has used it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12
MAX_N = 67108864


def _noalloc(L, a, b, n, res, stream):
    buf = ctypes.create_string_buffer(256)
    rc = L.ug4gb_vector_dot_noalloc(ctypes.c_void_p(a.data_ptr() if a is not None else 0),
                                    ctypes.c_void_p(b.data_ptr() if b is not None else 0),
                                    n, ctypes.c_void_p(res.data_ptr()), ctypes.c_void_p(stream), buf, 256)
    return rc, buf.value.decode()


def _reference_dot(L, ctx, a, b):
    from ugcore_gb300 import _lib
    va, vb = ctypes.c_void_p(), ctypes.c_void_p()
    n = a.numel()
    assert L.ug4gb_vector_wrap(ctx.h, ctypes.c_void_p(a.data_ptr()), n, ctypes.byref(va)) == _lib.OK
    assert L.ug4gb_vector_wrap(ctx.h, ctypes.c_void_p(b.data_ptr()), n, ctypes.byref(vb)) == _lib.OK
    out = ctypes.c_double()
    rc = L.ug4gb_vector_dot(va, vb, ctypes.byref(out))
    L.ug4gb_vector_destroy(va)
    L.ug4gb_vector_destroy(vb)
    assert rc == _lib.OK, L.ug4gb_last_error(ctx.h)
    return out.value


@pytest.mark.parametrize("n", [1, 31, 8192, 8193, 1_000_003, 2_146_689])
def test_noalloc_dot_matches_vector_dot(ctx, n):
    import torch
    from ugcore_gb300 import _lib
    L = _lib.lib()
    g = torch.Generator(device="cpu").manual_seed(1234 + n)
    a = (torch.rand(n, dtype=torch.float64, generator=g) * 2 - 1).cuda()
    b = (torch.rand(n, dtype=torch.float64, generator=g) * 2 - 1).cuda()
    res = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    ref = _reference_dot(L, ctx, a, b)
    rc0, msg0 = _noalloc(L, a, b, n, res[0:1], stream)
    rc1, msg1 = _noalloc(L, a, b, n, res[1:2], stream)
    assert rc0 == _lib.OK, msg0
    assert rc1 == _lib.OK, msg1
    torch.cuda.synchronize()
    r = res.cpu().numpy()
    scale = float((a * b).abs().sum())
    assert abs(r[0] - ref) <= TOL * scale, (r[0], ref)
    assert r[0] == r[1]                      # second call: scratch left clean
    exact = float(np.dot(a.cpu().numpy().astype(np.longdouble), b.cpu().numpy().astype(np.longdouble)))
    assert abs(r[0] - exact) <= TOL * scale


def test_noalloc_dot_edge_cases(ctx):
    import torch
    from ugcore_gb300 import _lib
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    res = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    a = torch.ones(16, dtype=torch.float64, device="cuda")
    # n = 0: result is 0, nothing read
    rc, msg = _noalloc(L, None, None, 0, res, stream)
    assert rc == _lib.OK, msg
    torch.cuda.synchronize()
    assert res.item() == 0.0
    # beyond the static scratch: rejected before any launch, with a message
    rc, msg = _noalloc(L, a, a, MAX_N + 1, res, stream)
    assert rc == _lib.ERR_INVALID and "outside" in msg
    rc, msg = _noalloc(L, a, a, -1, res, stream)
    assert rc == _lib.ERR_INVALID
    # host memory is not accepted
    host = torch.ones(16, dtype=torch.float64)
    rc, msg = _noalloc(L, host, host, 16, res, stream)
    assert rc == _lib.ERR_INVALID and "device memory" in msg
    # still correct after the rejected calls
    rc, msg = _noalloc(L, a, a, 16, res, stream)
    assert rc == _lib.OK, msg
    torch.cuda.synchronize()
    assert res.item() == 16.0


def test_noalloc_dot_at_the_scratch_limit_allocates_nothing(ctx):
    """n = UG4GB_DOT_NOALLOC_MAX_N (every partial slot of the scratch in use,
    two vectors of 512 MiB): matches ug4gb_vector_dot, two calls in a row are
    bit-identical, and the device's free memory is the same before and after
    the (warmed) calls"""
    import torch
    from ugcore_gb300 import _lib
    L = _lib.lib()
    n = MAX_N
    g = torch.Generator(device="cuda").manual_seed(99)
    a = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    b = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    res = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc, msg = _noalloc(L, a, b, 1, res[0:1], stream)            # warm-up call (module load, look-up)
    assert rc == _lib.OK, msg
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc0, msg0 = _noalloc(L, a, b, n, res[0:1], stream)
    rc1, msg1 = _noalloc(L, a, b, n, res[1:2], stream)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert rc0 == _lib.OK, msg0
    assert rc1 == _lib.OK, msg1
    assert free1 == free0, (free0, free1)
    r = res.cpu().numpy()
    assert r[0] == r[1]
    ref = _reference_dot(L, ctx, a, b)
    scale = float((a * b).abs().sum())
    assert abs(r[0] - ref) <= TOL * scale, (r[0], ref)
