"""The engine is a drop-in for the reference's GPU path: the reference's own
pybind module, built with refinery-optimizer_gb300/host/gpu_solver_adapter.cpp
in place of core/src/gpu/gpu_solver.cpp (oracle/ref_build.sh), loads and
dispatches GpuSolver calls to this engine.  Needs the reference sources (this
container), so it is skipped where they are absent."""
import os
import subprocess
import sys

import pytest

import oracle  # test infrastructure: locates the reference sources
from conftest import REPO

REF = oracle.reference_dir() or ""  # the reference sources, where present (located by oracle/ref_build.sh)
ENGINE_CORE = os.path.join(REPO, "oracle", "_ref", "engine")


@pytest.fixture(scope="module")
def engine_core():
    if not os.path.isdir(os.path.join(REF, "core", "src")):
        pytest.skip("reference sources not present")
    lib = os.path.join(REPO, "refinery-optimizer_gb300", "_build", "libsih_pdhg.so")
    if not os.path.exists(lib):
        pytest.skip("engine library not built")
    subprocess.run(["bash", os.path.join(REPO, "oracle", "ref_build.sh"), REF], check=True, capture_output=True)
    if not any(f.startswith("_core") for f in os.listdir(ENGINE_CORE)):
        pytest.fail("drop-in build did not produce the reference module")
    return ENGINE_CORE


def run_child(core_dir, code):
    return subprocess.run([sys.executable, "-c", f"import sys; sys.path.insert(0, {core_dir!r})\n" + code],
                          capture_output=True, text=True, timeout=300)


def test_reference_bindings_call_the_engine(engine_core):
    code = f"""
import _core
p = _core.read_mps({os.path.join(REF, 'data', 'toy', 'toy01_lp_simple.mps')!r})
cfg = _core.GpuPdhgConfig()
avail = _core.GpuSolver.is_cuda_available()
s = _core.GpuSolver.solve_pdhg(p, cfg)
if avail:
    assert s.is_optimal() and abs(s.primal_objective + 6.5) < 1e-3, (s.status, s.primal_objective)
    print('engine-ok', s.simplex_iterations)
else:
    assert s.status == _core.SolutionStatus.NumericalFailure, s.status
    assert 'no CUDA device' in s.in_solve_log
    print('engine-no-device')
h = _core.GpuSolver.solve_hybrid(p, cfg)
print('hybrid', h.status, h.primal_objective)
"""
    out = run_child(engine_core, code)
    assert out.returncode == 0, out.stderr
    assert "engine-" in out.stdout


def test_adapter_config_fields_match_reference_header():
    """GpuPdhgConfig fields in the reference header are the ones the C struct mirrors."""
    hdr = os.path.join(REF, "core", "include", "sih", "gpu", "gpu_solver.hpp")
    if not os.path.exists(hdr):
        pytest.skip("reference sources not present")
    text = open(hdr).read()
    from sih_pdhg.config import GpuPdhgConfig

    pos = [text.index(f" {name}{{") for name, _ in GpuPdhgConfig._fields_]
    assert pos == sorted(pos), "field order differs from the reference struct"
