"""The GPU file output against the files of the reference's own writers
(tests/golden/output_files.npz): shear_sim_3d::output_cube for every Field
member and the x and r z-slices of region::output_internal byte for byte; the
residual slice (the GPU's FP64 residual rounds its fused multiply-adds
differently from the host) value by value within 1e-6."""
import os

import numpy as np
import pytest

from oracle import advect as A
from test_oracle_output import BOXES, CUBE, GOLD, SLICE_DIMS, SLICE_K, SLICE_PER, cube_fields

pytestmark = pytest.mark.gpu

CUBE_COLS = {"u": 0, "v": 1, "w": 2, "s11": 3, "s12": 4, "s13": 5, "s22": 6, "s23": 7, "s33": 8, "chi": 9,
             "xi_x": 20, "xi_y": 21, "xi_z": 22}


def device_fields(F):
    import torch
    return {k: torch.tensor(np.ascontiguousarray(F[:, c]), dtype=torch.float64, device="cuda")
            for k, c in CUBE_COLS.items()}


@pytest.mark.parametrize("mode", range(16))
def test_cube_file_is_the_reference_file(mode, tmp_path):
    from stzpp_gb300 import advect
    d = np.load(GOLD)
    f = device_fields(cube_fields())
    advect.output_cube(f, CUBE, mode, str(tmp_path / "out"), "field", 3)
    path = tmp_path / "out" / "field_grid.3"
    assert path.read_bytes() == d[f"cube/{mode}"].tobytes()
    advect.output_cube(f, CUBE, mode, str(tmp_path / "out"), "field", 3)   # appends, as the reference
    assert path.read_bytes() == 2 * d[f"cube/{mode}"].tobytes()


def test_cube_values_on_a_larger_grid():
    from stzpp_gb300 import advect
    nx, ny, nz = 40, 24, 17
    F = A.random_fields(41, nx, ny, nz, plastic_bias=0.3)
    F[:, 20:23] = np.random.default_rng(42).normal(size=(F.shape[0], 3))
    f = device_fields(F)
    for mode in range(16):
        got = advect.cube_values(f, (nx, ny, nz), mode).cpu().numpy()
        assert np.array_equal(got, A.cube_values(F, nx, ny, nz, mode)), mode


def test_cube_rejects_missing_members():
    from stzpp_gb300 import advect, mg
    f = device_fields(cube_fields())
    del f["xi_y"]
    with pytest.raises(mg.StzMgError):
        advect.cube_values(f, CUBE, 14)


def slice_handle(d):
    import stzpp_gb300 as sg
    m, n, o = SLICE_DIMS
    h = sg.Multigrid(SLICE_DIMS, SLICE_PER, precision="fp64")   # 240 nodes: a single level
    h.setup_matrices(*sg.elastic_stencil(1.0, 2.0, 1 / m, 1 / n, 1 / (o - 1)))
    h.setup_fields(x=d["slice/x"], r=d["slice/r"])
    return h


@pytest.mark.parametrize("b", [0, 1])
def test_slices_are_the_reference_files(b, tmp_path):
    d = np.load(GOLD)
    h = slice_handle(d)
    for which in ("x", "r"):
        fn = str(tmp_path / f"{which}{b}")
        h.output_slice(which, SLICE_K, fn, box=BOXES[b])
        assert open(fn, "rb").read() == d[f"slice/{which}/{b}"].tobytes(), which
    fn = str(tmp_path / f"res{b}")
    h.output_slice("residual", SLICE_K, fn, box=BOXES[b])
    got = np.frombuffer(open(fn, "rb").read(), np.float32)
    ref = np.frombuffer(d[f"slice/residual/{b}"].tobytes(), np.float32)
    m = SLICE_DIMS[0]
    assert got.shape == ref.shape
    assert np.array_equal(got[:m + 1], ref[:m + 1])   # header row
    rows_g, rows_r = got[m + 1:].reshape(-1, m + 1), ref[m + 1:].reshape(-1, m + 1)
    assert np.array_equal(rows_g[:, 0], rows_r[:, 0])
    assert np.allclose(rows_g[:, 1:], rows_r[:, 1:], rtol=1e-6, atol=0)
    h.close()


def test_slice_rejects_bad_arguments(tmp_path):
    from stzpp_gb300 import mg
    d = np.load(GOLD)
    h = slice_handle(d)
    with pytest.raises(mg.StzMgError):
        h.output_slice("x", SLICE_DIMS[2], str(tmp_path / "s"))
    with pytest.raises(mg.StzMgError):
        h.output_slice("x", 0, str(tmp_path / "no" / "such" / "dir" / "s"))
    h.close()
