"""SHA-256 of a problem's arrays (the digest tests/golden/make_golden.py records)."""
import hashlib

import numpy as np


def problem_digest(p) -> str:
    h = hashlib.sha256()
    A = p.A
    for a in (A.csc_col_ptr(), A.csc_row_ind(), A.csc_values(), p.c, p.col_lower, p.col_upper, p.row_lower,
              p.row_upper):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()
