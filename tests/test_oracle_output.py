"""The numpy restatements of the reference's output formats (oracle/outfmt.py,
oracle/advect.cube_values) against the files the reference's own writers
produce: shear_sim_3d::output_cube for every Field member and the x, r and
residual z-slices of region::output_internal, byte for byte, from the golden
fixture (tests/golden/output_files.npz) and live where the reference is built."""
import os
import tempfile

import numpy as np
import pytest

from oracle import advect as A
from oracle import outfmt, refpy
from oracle import problem as P

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "output_files.npz")
CUBE = (6, 5, 4)
SLICE_DIMS, SLICE_PER, SLICE_K = (8, 6, 5), (True, True, False), 2
BOXES = [(0.0, 7.0, 0.0, 5.0), (0.0, 1.0, -0.5, 0.5)]
OUT_COLS = list(range(10)) + [20, 21, 22]


def cube_fields():
    d = np.load(GOLD)
    F = np.zeros((d["cube/in"].shape[0], A.NFIELD))
    F[:, OUT_COLS] = d["cube/in"]
    return F


def slice_residual(x, r):
    """b - A x of the fixture's level with the oracle (its box stencil)."""
    from oracle import port
    m, n, o = SLICE_DIMS
    st, fix = P.elastic_stencil_const(1.0, 2.0, 1 / m, 1 / n, 1 / (o - 1))
    Q = port.PortMultigrid(SLICE_DIMS, SLICE_PER, stencil=st, fix=fix, max_coarse=16)
    Q.set_field(0, "x", x)
    Q.set_field(0, "r", r)
    res, _ = Q.residual(0)
    Q.close()
    return res


@pytest.mark.parametrize("mode", range(16))
def test_cube_bytes_match_reference(mode):
    d = np.load(GOLD)
    assert outfmt.cube_file(cube_fields(), *CUBE, mode) == d[f"cube/{mode}"].tobytes()


@pytest.mark.parametrize("which", ["x", "r", "residual"])
@pytest.mark.parametrize("b", [0, 1])
def test_slice_bytes_match_reference(which, b):
    d = np.load(GOLD)
    x, r = d["slice/x"], d["slice/r"]
    if which == "residual":
        mine = outfmt.slice_file(slice_residual(x, r), SLICE_DIMS, SLICE_K, BOXES[b], quartic=True)
    else:
        mine = outfmt.slice_file(x if which == "x" else r, SLICE_DIMS, SLICE_K, BOXES[b])
    assert mine == d[f"slice/{which}/{b}"].tobytes()


@pytest.mark.skipif(not (A.reference_available() and refpy.available()),
                    reason="oracle/_ref not built (no reference checkout)")
def test_live_reference_writers():
    tmp = tempfile.mkdtemp()
    nx, ny, nz = 7, 3, 5
    F = A.random_fields(31, nx, ny, nz)
    F[:, 20:23] = np.random.default_rng(32).normal(size=(F.shape[0], 3))
    for mode in (0, 5, 9, 10, 11, 12, 15):
        A.reference_cube(F, nx, ny, nz, A.driver_params(nx), mode, os.path.join(tmp, "c"), "f", mode)
        A.reference_cube(F, nx, ny, nz, A.driver_params(nx), mode, os.path.join(tmp, "c"), "f", mode)
        got = open(os.path.join(tmp, "c", f"f_grid.{mode}"), "rb").read()
        assert got == 2 * outfmt.cube_file(F, nx, ny, nz, mode)   # output_cube appends
    dims, per = (6, 4, 7), (True, False, False)
    st, fix = P.elastic_stencil_const(1.0, 2.0, 1 / 6, 1 / 3, 1 / 6)
    R = refpy.RefMultigrid(dims, per, stencil=st, fix=fix, max_coarse=16)
    rng = np.random.default_rng(33)
    x = rng.normal(size=(6 * 4 * 7, 3))
    R.set_field(0, "x", x)
    fn = os.path.join(tmp, "sx")
    R.output_slice("x", 6, (0.0, 5.0, 0.0, 3.0), fn)
    assert open(fn, "rb").read() == outfmt.slice_file(x, dims, 6, (0.0, 5.0, 0.0, 3.0))
    R.close()
