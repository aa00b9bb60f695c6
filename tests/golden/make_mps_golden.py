"""Writes the MPS ingest fixtures: MPS texts that exercise the reader's record
semantics (tests/golden/mps/*.mps, written here, not taken from the reference)
and, for each, what the reference's own reader (sih_solver.read_mps,
core/src/io/mps_io.cpp:63-323) makes of it: the problem's arrays in
tests/golden/mps_golden.npz, or the fact that it raises.

Run in a container that has the reference build of oracle/ref_build.sh
(oracle/_ref/intended/_core*.so):

    python tests/golden/make_mps_golden.py
"""
import glob
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
MPS_DIR = os.path.join(HERE, "mps")

# Sections, comments, headers, row kinds, duplicates, markers, ranges and every bound type.
EDGE_SECTIONS = """* comment line, then a blank line

NAME          edge_sections  extra_token
OBJSENSE
    MAX
ROWS
 N  COST
 E  BAL1
 l  CAP2
 G  DEM3
 E  RNG4
 E  RNG5
 G  RNG6
 L  RNG7
 N  SECOND_OBJ
 E  BAL1
 X  ODD8
COLUMNS
    X1        COST       1.5   BAL1       1.0
    X1        CAP2       2.0   DEM3       1e-17
    X1        NOWHERE    9.0   SECOND_OBJ 4.0
    X2        COST      -2.0   CAP2       1.0
    X2        BAL1       0.5   BAL1       0.25
    MARKER                 'MARKER'                 'INTORG'
    X3        COST       3.0   DEM3       1.0
    X3        RNG4       1.0   RNG5       1.0
    MARKER                 'MARKER'                 'INTEND'
    X4        RNG6       1.0   RNG7       1.0
    X4        ODD8       2.0   COST       0.5
    X1        RNG4       -1.0
    X2        DEM3       7.0   DEM3      -7.0
    X5        COST       0.0
FOOBAR
RHS
    RHS1      BAL1       4.0   CAP2      10.0
    DEM3       2.0
    RHS1      COST      12.5
    RHS1      RNG4       1.0   RNG5       2.0
    RHS1      RNG6       3.0   RNG7       4.0
RANGES
    RNG1      RNG4       2.0   RNG5      -3.0
    RNG1      RNG6      -1.5   RNG7      -2.5
BOUNDS
 UP BND       X1         4.0
 LO BND       X2        -1.0
 UP BND       X2         3.0
 FX BND       X3         0.5
 FR BND       X4
 MI BND       X5
 PL BND       X6
 BV BND       X7
 UI BND       X8         9.0
 LI BND       X8         2.0
ENDATA
    X9        COST       1.0
"""

# Number forms strtod reads (as std::stod does): exponents, signs, leading dot,
# hexadecimal, trailing characters ignored, infinity.
EDGE_VALUES = """NAME          edge_values
ROWS
 N  OBJ
 L  R1
 G  R2
COLUMNS
    A         OBJ        1.5e+2   R1         -.5
    B         OBJ        +3       R2         0x10
    C         OBJ        2.5abc   R1         1D2
    C         R2         -0.0
RHS
    RHS       R1         inf      R2         -1E-3
BOUNDS
 UP BND       A          1e300
 LO BND       B          -inf
ENDATA
"""

# Free-format lines without section names where the reader takes the first token as a set name.
EDGE_FREE = """NAME
ROWS
 N obj
 E c1
 L c2
COLUMNS
 x obj 1 c1 1
 y obj 2 c1 1
 y c2 3
RHS
 c1 5 c2 6
RANGES
 c2 2
BOUNDS
 UP x 4
 LO BND y 1
ENDATA
"""

BAD_NUMBER = """NAME bad_number
ROWS
 N  OBJ
 L  R1
COLUMNS
    A         OBJ        abc      R1         1.0
ENDATA
"""

OUT_OF_RANGE = """NAME out_of_range
ROWS
 N  OBJ
 L  R1
COLUMNS
    A         OBJ        1.0      R1         1e400
ENDATA
"""

CONTRADICTORY = """NAME contradictory
ROWS
 N  OBJ
 L  R1
COLUMNS
    A         OBJ        1.0      R1         1.0
RHS
    RHS       R1         1.0
BOUNDS
 UP BND       A          -1.0
ENDATA
"""

QUADRATIC = """NAME quadratic
ROWS
 N  OBJ
 L  R1
COLUMNS
    A         OBJ        1.0      R1         1.0
RHS
    RHS       R1         1.0
QUADOBJ
    A         A          2.0
ENDATA
"""

FILES = {"edge_sections": EDGE_SECTIONS, "edge_values": EDGE_VALUES, "edge_free": EDGE_FREE,
         "bad_number": BAD_NUMBER, "out_of_range": OUT_OF_RANGE, "contradictory": CONTRADICTORY,
         "quadratic": QUADRATIC}


def reference_arrays(core, path):
    r = core.read_mps(path)
    A = r.A
    types = [int(t) for t in r.var_types]
    return {"m": np.int64(r.num_rows()), "n": np.int64(r.num_cols()),
            "csc_col_ptr": np.asarray(A.csc_col_ptr(), np.int64), "csc_row_ind": np.asarray(A.csc_row_ind(), np.int64),
            "csc_values": np.asarray(A.csc_values(), np.float64), "csr_row_ptr": np.asarray(A.csr_row_ptr(), np.int64),
            "csr_col_ind": np.asarray(A.csr_col_ind(), np.int64), "csr_values": np.asarray(A.csr_values(), np.float64),
            "c": np.asarray(r.c, np.float64), "col_lower": np.asarray(r.col_lower, np.float64),
            "col_upper": np.asarray(r.col_upper, np.float64), "row_lower": np.asarray(r.row_lower, np.float64),
            "row_upper": np.asarray(r.row_upper, np.float64), "sense": np.int64(int(r.sense)),
            "obj_offset": np.float64(r.obj_offset), "integer_columns": np.int64(sum(t != 0 for t in types)),
            "has_quadratic": np.int64(bool(r.has_quadratic()))}, r.name


def main():
    sys.path.insert(0, glob.glob(os.path.join(REPO, "oracle", "_ref", "intended"))[0])
    import _core

    os.makedirs(MPS_DIR, exist_ok=True)
    arrays, index = {}, {}
    for name, text in FILES.items():
        path = os.path.join(MPS_DIR, name + ".mps")
        with open(path, "w") as f:
            f.write(text)
        try:
            arr, pname = reference_arrays(_core, path)
        except Exception as e:  # the reference raises: record the exception type
            index[name] = {"reference": "raises", "exception": type(e).__name__}
            continue
        index[name] = {"reference": "reads", "name": pname}
        for k, v in arr.items():
            arrays[f"{name}/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "mps_golden.npz"), **arrays)
    with open(os.path.join(HERE, "mps_golden.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)
    print(json.dumps(index, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
