"""The CPU oracle reproduces the reference's own PDHG code bit for bit.

The golden vectors were produced by the reference driver and kernels
(core/src/gpu/gpu_solver.cpp:60-307, core/src/gpu/cuda_pdhg.cu:14-151) run on
the CPU with the intended int32 index copy (tests/golden/make_golden.py).
"""
import numpy as np
import pytest

from conftest import golden_case, golden_config, golden_index

CASES = [(name, cname) for name, e in sorted(golden_index()["cases"].items()) for cname in sorted(e["pdhg"])]


@pytest.mark.parametrize("name,cname", CASES)
def test_plain_oracle_matches_reference_code(oracle_lib, name, cname):
    prob, entry, vec = golden_case(name)
    if "sha256" in entry:
        from make_golden_digest import problem_digest
        assert problem_digest(prob) == entry["sha256"], "generator output changed"
    ref = entry["pdhg"][cname]
    x, y, info = oracle_lib.plain_pdhg(prob, golden_config(cname))
    assert info["status"] == ref["status"]
    assert info["iterations"] == ref["iterations"]
    np.testing.assert_array_equal(x, vec[f"pdhg/{cname}/x"])
    np.testing.assert_array_equal(y, vec[f"pdhg/{cname}/row_duals"])
    assert info["primal_objective"] == pytest.approx(ref["primal_objective"], rel=1e-14, abs=1e-14)


@pytest.mark.parametrize("name", sorted(n for n, e in golden_index()["cases"].items() if e["kind"] == "toy"))
def test_toy_known_answers(oracle_lib, name):
    """Converged plain PDHG meets the toy suite's expected objective and primal
    (data/toy/toy_suite_metadata.json) to the FP32 path's 1e-3 accuracy."""
    prob, entry, _ = golden_case(name)
    x, y, info = oracle_lib.plain_pdhg(prob, golden_config("default"))
    assert info["status"] == 0
    assert info["primal_objective"] == pytest.approx(entry["expected_objective"], rel=1e-4, abs=1e-4)
    np.testing.assert_allclose(x, entry["expected_primal"], atol=2e-3)


def test_highs_and_reference_simplex_agree():
    for name, e in golden_index()["cases"].items():
        if "simplex" in e:
            assert e["simplex"]["primal_objective"] == pytest.approx(e["highs_objective"], rel=1e-9, abs=1e-9)


def test_kkt_certificate_at_highs_optimum(oracle_lib):
    """The FP64 KKT certificate reads ~0 at HiGHS's optimum (duals flipped to the PDHG sign)."""
    for name in ("toy01_lp_simple", "rand_50x120_k4_s1", "rand_2000x5000_k8_s0"):
        prob, entry, vec = golden_case(name)
        k = oracle_lib.kkt(prob, vec["highs/x"], -vec["highs/row_duals"])
        assert k["rel_primal"] < 1e-7 and k["rel_dual"] < 1e-7 and k["rel_gap"] < 1e-7, (name, k)
        assert k["primal_obj"] == pytest.approx(entry["highs_objective"], rel=1e-9)
