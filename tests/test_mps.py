"""MPS ingest (sih_pdhg_read_mps / sih_pdhg.read_mps) on the CPU.

* golden: on MPS texts written for these tests (tests/golden/mps/*.mps:
  sections, comments, unknown headers, every row and bound type, ranges,
  markers, duplicate and cancelling entries, unknown rows, number forms), the
  reader gives exactly the arrays that the reference's own reader
  (core/src/io/mps_io.cpp:63-323) gave (tests/golden/mps_golden.npz, made by
  tests/golden/make_mps_golden.py), and fails where it failed;
* round trips: write_mps then read_mps gives back the generators' LPs;
* with the reference build present (this container): the reference's toy LP
  and MILP files, generated LPs and 200 seeded random MPS texts read the same
  through both readers (or fail in both).
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle  # test infrastructure: locates the reference sources
from conftest import GOLDEN, REPO

MPS_DIR = os.path.join(GOLDEN, "mps")
REF = oracle.reference_dir() or ""  # the reference sources, where present (located by oracle/ref_build.sh)
REF_CORE = os.path.join(REPO, "oracle", "_ref", "intended")
ARRAYS = ("csc_col_ptr", "csc_row_ind", "csc_values", "csr_row_ptr", "csr_col_ind", "csr_values", "c", "col_lower",
          "col_upper", "row_lower", "row_upper")


def _index():
    with open(os.path.join(GOLDEN, "mps_golden.json")) as f:
        return json.load(f)


def _arrays(p):
    A = p.A
    return {"csc_col_ptr": A.csc_col_ptr(), "csc_row_ind": A.csc_row_ind(), "csc_values": A.csc_values(),
            "csr_row_ptr": A.csr_row_ptr(), "csr_col_ind": A.csr_col_ind(), "csr_values": A.csr_values(),
            "c": p.c, "col_lower": p.col_lower, "col_upper": p.col_upper, "row_lower": p.row_lower,
            "row_upper": p.row_upper}


def _assert_same(p, ref, prefix=""):
    for k in ARRAYS:
        np.testing.assert_array_equal(_arrays(p)[k], ref[prefix + k], err_msg=k)
    assert int(p.sense) == int(ref[prefix + "sense"])
    assert float(p.obj_offset) == float(ref[prefix + "obj_offset"])
    assert p.integer_columns == int(ref[prefix + "integer_columns"])


@pytest.fixture(scope="module")
def sih():
    import sih_pdhg

    return sih_pdhg


@pytest.mark.parametrize("name", sorted(k for k, v in _index().items() if v["reference"] == "reads"
                                        and k != "quadratic"))
def test_reader_matches_the_reference_reader(sih, name):
    g = np.load(os.path.join(GOLDEN, "mps_golden.npz"))
    p = sih.read_mps(os.path.join(MPS_DIR, name + ".mps"))
    _assert_same(p, g, f"{name}/")
    assert p.name == _index()[name]["name"]


@pytest.mark.parametrize("name", sorted(k for k, v in _index().items() if v["reference"] == "raises"))
def test_reader_fails_where_the_reference_raises(sih, name):
    with pytest.raises(sih.SihPdhgError) as e:
        sih.read_mps(os.path.join(MPS_DIR, name + ".mps"))
    assert e.value.code == 1


def test_quadratic_objective_is_rejected(sih):
    assert _index()["quadratic"]["reference"] == "reads"  # the reference reads QPs; this LP engine does not
    with pytest.raises(sih.SihPdhgError) as e:
        sih.read_mps(os.path.join(MPS_DIR, "quadratic.mps"))
    assert e.value.code == 5


def test_text_equals_file_and_missing_file_is_an_error(sih):
    path = os.path.join(MPS_DIR, "edge_sections.mps")
    a = sih.read_mps(path)
    with open(path, "rb") as f:
        b = sih.read_mps_text(f.read())
    for k in ARRAYS:
        np.testing.assert_array_equal(_arrays(a)[k], _arrays(b)[k])
    with pytest.raises(sih.SihPdhgError) as e:
        sih.read_mps(os.path.join(MPS_DIR, "no_such_file.mps"))
    assert e.value.code == 1
    with pytest.raises(sih.SihPdhgError) as e:  # a directory: an error, not a crash
        sih.read_mps(MPS_DIR)
    assert e.value.code == 1 and "directory" in str(e.value)
    empty = sih.read_mps_text(b"")  # no records: the empty problem, as the reference reads it
    assert empty.num_rows() == 0 and empty.num_cols() == 0 and empty.name == "problem"


def _generated():
    from sih_pdhg.generators import mixed_bounds_lp, refinery_lp, small_random_lp
    from sih_pdhg.problem import ObjectiveSense, Problem

    probs = [mixed_bounds_lp(seed=0), small_random_lp(200, 500, 8, 1), refinery_lp(2, 0)]
    q = probs[1]
    probs.append(Problem.from_arrays(q.A, q.c, q.col_lower, q.col_upper, q.row_lower, q.row_upper,
                                     ObjectiveSense.Maximize, 3.25, "max_with_offset"))
    return probs


def test_write_then_read_gives_the_problem_back(sih, tmp_path):
    from sih_pdhg.mps import same_problem

    for k, p in enumerate(_generated()):
        path = tmp_path / f"p{k}.mps"
        sih.write_mps(p, path)
        q = sih.read_mps(path)
        # ranged rows come back as lower + (upper - lower)
        same_problem(q, p, bound_rtol=1e-15)
        # the reader's CSR is the CSC's transpose with columns ascending in each row
        np.testing.assert_array_equal(q.A.csr_row_ptr(), p.A.csr_row_ptr())
        np.testing.assert_array_equal(q.A.csr_col_ind(), p.A.csr_col_ind())
        np.testing.assert_array_equal(q.A.csr_values(), p.A.csr_values())


def _reference_read(paths, out):
    code = ("import sys, numpy as np\n"
            f"sys.path.insert(0, {REF_CORE!r})\n"
            "import _core\n"
            "arr = {}\n"
            f"for i, path in enumerate({list(paths)!r}):\n"
            "    r = _core.read_mps(path); A = r.A\n"
            "    for k in ('csc_col_ptr', 'csc_row_ind', 'csc_values', 'csr_row_ptr', 'csr_col_ind', 'csr_values'):\n"
            "        arr[f'{i}/{k}'] = np.asarray(getattr(A, k)())\n"
            "    for k in ('c', 'col_lower', 'col_upper', 'row_lower', 'row_upper'):\n"
            "        arr[f'{i}/{k}'] = np.asarray(getattr(r, k), dtype=np.float64)\n"
            "    arr[f'{i}/sense'] = np.int64(int(r.sense)); arr[f'{i}/obj_offset'] = np.float64(r.obj_offset)\n"
            "    arr[f'{i}/integer_columns'] = np.int64(sum(int(t) != 0 for t in r.var_types))\n"
            f"np.savez({out!r}, **arr)\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(out)


@pytest.mark.skipif(not (os.path.isdir(os.path.join(REF, "data", "toy")) and os.path.isdir(REF_CORE)
                         and any(f.startswith("_core") for f in os.listdir(REF_CORE))),
                    reason="reference build (oracle/ref_build.sh) and data not present")
def test_reference_files_and_generated_lps_read_the_same(sih, tmp_path):
    toy = sorted(os.path.join(REF, "data", "toy", f) for f in os.listdir(os.path.join(REF, "data", "toy"))
                 if f.endswith(".mps") and "_qp_" not in f)
    gen = []
    for k, p in enumerate(_generated()):
        gen.append(str(tmp_path / f"g{k}.mps"))
        sih.write_mps(p, gen[-1])
    paths = toy + gen
    ref = _reference_read(paths, str(tmp_path / "ref.npz"))
    for i, path in enumerate(paths):
        _assert_same(sih.read_mps(path), ref, f"{i}/")


def _random_mps(rng) -> str:
    """A seeded random MPS text mixing every record form the readers handle:
    row kinds (some lower case, repeated, unknown), entries to unknown and to
    extra N rows, duplicates, odd RHS / RANGES token counts, every bound type,
    value-less bounds, number forms, tabs, CRLF endings, comments, unknown
    headers and integer markers."""
    nr, nc = int(rng.integers(1, 9)), int(rng.integers(1, 9))
    rows = [f"r{i}" for i in range(nr)]
    cols = [f"x{j}" for j in range(nc)]
    num_forms = ["{:.17g}", "{:.3e}", "{:.2f}", "{:.1f}abc", "+{:.4g}"]

    def num():
        v = float(rng.choice([0.0, 1e-16, 1.0, -2.5, 3.0])) if rng.random() < 0.3 else float(rng.normal(0, 5))
        s = str(rng.choice(num_forms)).format(v)
        return s.replace("+-", "-")

    sep = lambda: str(rng.choice([" ", "  ", "\t", "    "]))
    out = ["* random MPS", f"NAME{sep()}rand{int(rng.integers(1000))}"]
    if rng.random() < 0.5:
        out += ["OBJSENSE", f"    {rng.choice(['MAX', 'MIN', 'max', 'MAXIMIZE'])}"]
    out.append("ROWS")
    out.append(f" N{sep()}obj")
    for r in rows:
        out.append(f" {rng.choice(['E', 'L', 'G', 'e', 'l', 'g'])}{sep()}{r}")
    if rng.random() < 0.3:
        out.append(f" N{sep()}obj2")
    if rng.random() < 0.3:
        out.append(f" L{sep()}{rows[0]}")  # repeated definition: the first one stays
    if rng.random() < 0.2:
        out.append(f" X{sep()}odd")
    if rng.random() < 0.2:
        out.append("UNKNOWNSECTION")
    out.append("COLUMNS")
    marker = False
    for j, cname in enumerate(cols):
        if rng.random() < 0.2:
            out.append(f"    M{sep()}'MARKER'{sep()}{'INTEND' if marker else 'INTORG'}")
            marker = not marker
        targets = ["obj"] + list(rng.choice(rows + ["nowhere", "obj2"], size=int(rng.integers(0, 4))))
        for t in targets:
            if rng.random() < 0.5:
                out.append(f"    {cname}{sep()}{t}{sep()}{num()}")
            else:
                t2 = str(rng.choice(rows))
                out.append(f"    {cname}{sep()}{t}{sep()}{num()}{sep()}{t2}{sep()}{num()}")
    out.append("RHS")
    for r in list(rng.choice(rows + ["obj"], size=int(rng.integers(0, nr + 2)))):
        if rng.random() < 0.5:
            out.append(f"    rhs{sep()}{r}{sep()}{num()}")
        else:
            out.append(f"    {r}{sep()}{num()}")
    if rng.random() < 0.6:
        out.append("RANGES")
        for r in list(rng.choice(rows, size=int(rng.integers(1, nr + 1)))):
            out.append(f"    rng{sep()}{r}{sep()}{num()}")
    out.append("BOUNDS")
    for cname in list(rng.choice(cols + ["newcol"], size=int(rng.integers(0, 2 * nc + 1)))):
        bt = str(rng.choice(["UP", "LO", "FX", "FR", "MI", "PL", "BV", "UI", "LI", "SC", "up"]))
        if bt in ("FR", "MI", "PL", "BV") and rng.random() < 0.5:
            out.append(f" {bt}{sep()}bnd{sep()}{cname}")
        else:
            v = abs(float(rng.normal(0, 4))) + (0.0 if bt in ("LO", "LI") else 1.0)
            out.append(f" {bt}{sep()}bnd{sep()}{cname}{sep()}{v:.6g}")
    out.append("ENDATA")
    eol = "\r\n" if rng.random() < 0.3 else "\n"
    return eol.join(out) + eol


@pytest.mark.skipif(not (os.path.isdir(REF_CORE) and any(f.startswith("_core") for f in os.listdir(REF_CORE))),
                    reason="reference build (oracle/ref_build.sh) not present")
def test_random_mps_texts_read_like_the_reference(sih, tmp_path):
    """200 seeded random MPS texts: wherever the reference reader returns a
    problem this reader returns the same arrays; wherever it raises, this one
    reports an error."""
    rng = np.random.default_rng(20261204)
    paths = []
    for k in range(200):
        path = tmp_path / f"r{k}.mps"
        path.write_bytes(_random_mps(rng).encode())
        paths.append(str(path))
    code = ("import sys, json, numpy as np\n"
            f"sys.path.insert(0, {REF_CORE!r})\n"
            "import _core\n"
            "arr, ok = {}, []\n"
            f"for i, path in enumerate({paths!r}):\n"
            "    try:\n"
            "        r = _core.read_mps(path)\n"
            "    except Exception:\n"
            "        ok.append(False); continue\n"
            "    ok.append(True); A = r.A\n"
            "    for k in ('csc_col_ptr', 'csc_row_ind', 'csc_values'):\n"
            "        arr[f'{i}/{k}'] = np.asarray(getattr(A, k)())\n"
            "    for k in ('c', 'col_lower', 'col_upper', 'row_lower', 'row_upper'):\n"
            "        arr[f'{i}/{k}'] = np.asarray(getattr(r, k), dtype=np.float64)\n"
            "    arr[f'{i}/sense'] = np.int64(int(r.sense)); arr[f'{i}/obj_offset'] = np.float64(r.obj_offset)\n"
            "    arr[f'{i}/integer_columns'] = np.int64(sum(int(t) != 0 for t in r.var_types))\n"
            f"np.savez({str(tmp_path / 'ref.npz')!r}, **arr)\n"
            "print(json.dumps(ok))\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    ok = json.loads(r.stdout.strip().splitlines()[-1])
    ref = np.load(tmp_path / "ref.npz")
    reads = 0
    for i, path in enumerate(paths):
        if not ok[i]:
            with pytest.raises(sih.SihPdhgError):
                sih.read_mps(path)
            continue
        p = sih.read_mps(path)
        reads += 1
        for k in ("csc_col_ptr", "csc_row_ind", "csc_values", "c", "col_lower", "col_upper", "row_lower",
                  "row_upper"):
            np.testing.assert_array_equal(_arrays(p)[k], ref[f"{i}/{k}"], err_msg=f"{path}: {k}")
        assert int(p.sense) == int(ref[f"{i}/sense"]) and float(p.obj_offset) == float(ref[f"{i}/obj_offset"])
        assert p.integer_columns == int(ref[f"{i}/integer_columns"])
    assert reads >= 50  # most texts are valid problems


def test_sliced_columns_parse_equals_the_sequential_parse(sih, monkeypatch):
    """COLUMNS bodies cut into per-thread slices (forced here for small texts)
    give the same problem and the same error messages as the one-thread pass."""
    rng = np.random.default_rng(7)
    texts = [_random_mps(rng) for _ in range(60)]
    texts += [open(os.path.join(MPS_DIR, f)).read() for f in sorted(os.listdir(MPS_DIR)) if f.endswith(".mps")]

    def read_all():
        out = []
        for t in texts:
            try:
                out.append(("ok", _arrays(sih.read_mps_text(t))))
            except sih.SihPdhgError as e:
                out.append(("err", str(e)))
        return out

    monkeypatch.setenv("SIH_PDHG_MPS_PARALLEL_BYTES", str(1 << 40))
    seq = read_all()
    monkeypatch.setenv("SIH_PDHG_MPS_PARALLEL_BYTES", "0")
    par = read_all()
    for (ka, a), (kb, b) in zip(seq, par):
        assert ka == kb
        if ka == "err":
            assert a == b
        else:
            for k in ARRAYS:
                np.testing.assert_array_equal(a[k], b[k])
