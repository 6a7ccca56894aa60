"""Failure reporting of the C-ABI on the GPU: every failure is a status code
and a message, never a fault (the reference aborts the MPI job instead)."""
import numpy as np
import pytest

from oracle import problem as P

pytestmark = pytest.mark.gpu


def make(dims=(8, 8, 9), per=(True, True, False), **kw):
    import stzpp_gb300 as sg
    mg = sg.Multigrid(dims, per, **kw)
    m, n, o = dims
    st, fix = sg.elastic_stencil(1.0, 2.0, *P.grid_spacing(m, n, o, per))
    return mg, st, fix


def test_call_order_and_arguments():
    import stzpp_gb300 as sg
    mg, st, fix = make()
    with pytest.raises(sg.StzMgError) as e:
        mg.v_cycle()
    assert e.value.code == sg.mg.ERR_ARG
    with pytest.raises(sg.StzMgError):
        mg.level_dims(99)
    mg.close()


def test_odd_periodic_size_is_unsupported():
    import stzpp_gb300 as sg
    with pytest.raises(sg.StzMgError) as e:
        sg.Multigrid((9, 8, 9), (True, True, False))
    assert e.value.code == sg.mg.ERR_UNSUPPORTED


def test_nonfinite_inputs():
    import stzpp_gb300 as sg
    mg, st, fix = make()
    bad = st.copy()
    bad[13, 0] = np.nan
    with pytest.raises(sg.StzMgError) as e:
        mg.setup_matrices(stencil=bad, fix=fix)
    assert e.value.code in (sg.mg.ERR_NONFINITE, sg.mg.ERR_SINGULAR)
    mu = np.ones(8 * 8 * 9)
    mu[5] = np.inf
    with pytest.raises(sg.StzMgError) as e:
        mg.set_coeffs_lame(mu, 2 * np.ones_like(mu), 0.1, 0.1, 0.1)
    assert e.value.code == sg.mg.ERR_NONFINITE
    mg.setup_matrices(stencil=st, fix=fix)
    b = np.ones((8 * 8 * 9, 3))
    b[7, 1] = np.nan
    mg.setup_fields(r=b)
    with pytest.raises(sg.StzMgError) as e:
        mg.solve(1e-10, 10)
    assert e.value.code == sg.mg.ERR_NONFINITE
    mg.close()


def test_singular_centre_block():
    import stzpp_gb300 as sg
    mg, st, fix = make()
    bad = st.copy()
    bad[13] = 0
    with pytest.raises(sg.StzMgError) as e:
        mg.setup_matrices(stencil=bad, fix=fix)
    assert e.value.code == sg.mg.ERR_SINGULAR
    mg.close()


def test_cycle_cap_reports_noconv():
    import stzpp_gb300 as sg
    for prec in ("fp64", "mixed"):
        mg, st, fix = make((16, 16, 17), precision=prec)
        mg.setup_matrices(stencil=st, fix=fix)
        rng = np.random.default_rng(0)
        mg.setup_fields(r=rng.standard_normal((16 * 16 * 17, 3)))
        with pytest.raises(sg.StzMgError) as e:
            mg.solve(1e-10, 1)
        assert e.value.code == sg.mg.ERR_NOCONV
        cycles, rel = mg.solve(1e-10, 1, check=False)
        assert cycles == 1 and rel > 1e-10
        mg.close()


def test_handle_survives_errors_and_solves():
    import stzpp_gb300 as sg
    mg, st, fix = make((16, 16, 17))
    with pytest.raises(sg.StzMgError):
        mg.solve(1e-10, 5)
    mg.setup_matrices(stencil=st, fix=fix)
    rng = np.random.default_rng(1)
    mg.setup_fields(r=rng.standard_normal((16 * 16 * 17, 3)))
    cycles, rel = mg.solve(1e-10, 100)
    assert rel <= 1e-10
    c, nres, launches = mg.solve_stats()
    assert c == cycles and nres >= 2 and launches > 8 * cycles
    mg.close()
