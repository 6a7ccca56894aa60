"""stz_mg_const_residual_sumsq_noalloc: the allocation-free residual check.

It must give the same |b - A x|^2 as the handle-based stz_mg_residual_norm on
the same operator and fields, on two calls in a row (the second reusing the
static scratch the first left behind), refuse grids beyond its scratch, and
leave the device's free memory unchanged across repeated calls.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRIDS = [((16, 16, 17), (True, True, False)),
         ((12, 10, 9), (False, False, False)),
         ((16, 12, 11), (True, False, False)),
         ((8, 6, 10), (False, True, True))]


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from stzpp_gb300 import build, mg
    build.build()
    return mg.load_library()


def handle_norm(dims, per, st, fix, x, b):
    import stzpp_gb300 as sg
    with sg.Multigrid(dims, per, precision="fp64") as h:
        h.setup_matrices(stencil=st, fix=fix)
        h.setup_fields(x=x, r=b)
        rn, bn = h.residual_norm()
    return rn


def call(lib, dims, per, st, fix, xd, bd, out, stream):
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    return lib.stz_mg_const_residual_sumsq_noalloc(
        *dims, *[int(v) for v in per], st.ctypes.data_as(ctypes.c_void_p), fix.ctypes.data_as(ctypes.c_void_p),
        p(xd), p(bd), p(out), 0, ctypes.c_void_p(stream))


@pytest.mark.parametrize("dims,per", GRIDS)
def test_matches_handle_residual_norm_twice(lib, dims, per):
    import torch
    from oracle import problem as P
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    st, fix = P.elastic_stencil_const(1.0, 2.0, *h)
    st = np.ascontiguousarray(st, dtype=np.float64)
    fix = np.ascontiguousarray(fix, dtype=np.float64)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((m * n * o, 3))
    b = rng.standard_normal((m * n * o, 3))
    want = handle_norm(dims, per, st, fix, x, b) ** 2
    xd = torch.from_numpy(x).cuda()
    bd = torch.from_numpy(b).cuda()
    # garbage in the output on purpose: the result is stored, not accumulated
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert call(lib, dims, per, st, fix, xd, bd, out[0:], stream) == 0, lib.stz_mg_last_error()
    assert call(lib, dims, per, st, fix, xd, bd, out[1:], stream) == 0, lib.stz_mg_last_error()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert got[0] == got[1]   # same scratch, same order of summation
    assert abs(got[0] - want) <= 1e-12 * want, (got, want)


def test_refuses_grids_beyond_the_scratch(lib):
    import torch
    from stzpp_gb300 import mg
    st = np.zeros(243)
    fix = np.eye(3).ravel()
    t = torch.zeros(3, dtype=torch.float64, device="cuda")
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    dims = (1024, 1024, 129)   # 135,266,304 nodes > 1024 * 131072
    rc = call(lib, dims, (True, True, False), st, fix, t, t, out, torch.cuda.current_stream().cuda_stream)
    assert rc == mg.ERR_ARG
    msg = lib.stz_mg_last_error().decode()
    assert "too large" in msg and "stz_mg_residual_norm" in msg
    torch.cuda.synchronize()
    assert out.item() == 7.0
    rc = call(lib, (0, 4, 4), (True, True, False), st, fix, t, t, out, torch.cuda.current_stream().cuda_stream)
    assert rc == mg.ERR_ARG


def test_repeated_calls_leave_free_memory_unchanged(lib):
    import torch
    from oracle import problem as P
    dims, per = (64, 64, 65), (True, True, False)
    st, fix = P.elastic_stencil_const(1.0, 2.0, *P.grid_spacing(*dims, per))
    st = np.ascontiguousarray(st, dtype=np.float64)
    fix = np.ascontiguousarray(fix, dtype=np.float64)
    N = dims[0] * dims[1] * dims[2]
    xd = torch.randn(N, 3, dtype=torch.float64, device="cuda")
    bd = torch.randn(N, 3, dtype=torch.float64, device="cuda")
    out = torch.empty(6, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert call(lib, dims, per, st, fix, xd, bd, out[0:], stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    # nothing else allocates between the two readings of free memory
    for c in range(1, 6):
        assert call(lib, dims, per, st, fix, xd, bd, out[c:], stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    vals = out.cpu().numpy()
    assert (vals == vals[0]).all()
