"""Generate the golden fixtures in tests/golden/golden.npz.

The reference (Fortran 90 + MPI) cannot be built or run on the machines this
project uses, and it ships no test vectors, so these fixtures are outputs of
the FP64 C oracle (oracle/mgbf_oracle.c) on small seeded cases.  They pin the
oracle against regressions and give the GPU tests fixed targets; they do not
pin parity with the reference itself.

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from tests.golden.cases import CASES, case_input, case_oracle_cfg  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main():
    out = {}
    for name in CASES:
        x = case_input(name)
        out[name] = O.filter_compact(case_oracle_cfg(name), x)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
