"""GPU right-hand side assembly (node divergence of the cell tensor field)
against the oracle's restatement of calculate_first_order_stresses:
bit-identical (same operation order, no FMA contraction)."""
import numpy as np
import pytest

from oracle import problem as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,per", [((16, 16, 17), (True, True, False)), ((12, 10, 9), (False, False, False)),
                                      ((8, 6, 10), (True, False, True)), ((32, 32, 33), (True, True, False))])
def test_rhs_divergence_bit_exact(dims, per):
    import stzpp_gb300 as sg
    from stzpp_gb300 import problems
    m, n, o = dims
    h = P.grid_spacing(m, n, o, per)
    eps = problems.random_strain(3, dims, per)
    ref = P.rhs_divergence(eps, m, n, o, per, *h)
    with sg.Multigrid(dims, per, max_coarse=10**9) as mg:
        mg.set_rhs_divergence(eps, h)
        got = mg.get_rhs()
    assert np.array_equal(got, ref), np.abs(got - ref).max()
