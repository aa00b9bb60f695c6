"""Host logic of the LP layer (sih_pdhg.layer), no GPU: which point each
instance returns.  A polished vertex is returned only when the polish
certified its basis optimal; otherwise the instance keeps its PDHG point
(feasible to the solve's tolerance) and is reported."""
from types import SimpleNamespace

import numpy as np

from sih_pdhg.layer import choose_outputs


def _info(status=0, pv=0.0, dv=0.0):
    return {"status": status, "primal_violation": pv, "dual_violation": dv}


def test_certified_instances_return_the_vertex_others_the_pdhg_point():
    sols = [SimpleNamespace(x=np.full(3, 10.0 + i), row_duals=np.full(2, -1.0 - i)) for i in range(4)]
    xs = [np.full(3, float(i)) for i in range(4)]
    ys = [np.full(2, float(i)) for i in range(4)]
    infos = [_info(), _info(pv=2e-3), _info(dv=5e-4), _info(status=1)]
    xo, yo, bad = choose_outputs(sols, xs, ys, infos, 1e-6)
    assert bad == [1, 2, 3]
    assert np.array_equal(xo[0], xs[0]) and np.array_equal(yo[0], ys[0])
    for i in bad:
        assert xo[i] is sols[i].x and yo[i] is sols[i].row_duals


def test_certify_tolerance_is_inclusive():
    sols = [SimpleNamespace(x=np.zeros(1), row_duals=np.zeros(1))]
    _, _, bad = choose_outputs(sols, [np.ones(1)], [np.ones(1)], [_info(pv=1e-6, dv=1e-6)], 1e-6)
    assert bad == []
