"""The FP64 oracle of the mixed algorithm (oracle/pdlp_oracle.c) solves the
golden LPs to the requested relative KKT tolerance, and its objective matches
the FP64 simplex / HiGHS objective of the golden vectors."""
import pytest

from conftest import golden_case, golden_index

NAMES = sorted(golden_index()["cases"])


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("tol", [1e-4, 1e-6])
def test_pdlp_oracle_reaches_tolerance(oracle_lib, name, tol):
    prob, entry, _ = golden_case(name)
    x, y, info = oracle_lib.pdlp_solve(prob, tol=tol)
    assert info["status"] == 0
    k = oracle_lib.kkt(prob, x, y)
    assert k["rel_primal"] <= tol * 1.01 and k["rel_dual"] <= tol * 1.01 and k["rel_gap"] <= tol * 1.01
    ref = entry["highs_objective"]
    assert abs(k["primal_obj"] - ref) <= 20 * tol * (1 + abs(ref))
