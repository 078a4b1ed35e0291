"""Generates tests/golden/momentum.npz from the reference's own momentum code.

Run in a tree where the reference is checked out (it reads
src/olcao/gaussIntegrals.f90 through oracle/fexpr_eval.py, which executes the
generated Fortran statements of momentum2CIntg verbatim in binary64):

    python tests/golden/make_momentum_goldens.py [path/to/gaussIntegrals.f90]

The fixture holds, for every (lmAlpha1, lmAlpha2) block the reference
generates (s/p/d/f), seeded exponent pairs and centres plus edge cases
(coincident centres, very unequal and very large exponents, a large
separation), as sh(16,16,3): the x, y, z components of <a| d/dr |b>.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import fexpr_eval as fe  # noqa: E402

LMS = (1, 4, 9, 16)


def main(path=None):
    path = path or fe.default_path()
    F = fe.FortranIntegrals(path)
    rng = np.random.default_rng(20261204)
    params, lmal, outs = [], [], []

    def add(a1, a2, A, B, l1, l2):
        outs.append(F.momentum(a1, a2, A, B, fe.l1l2switch(l1, l2)))
        params.append([a1, a2, 0.0, *A, *B, 0.0, 0.0, 0.0])
        lmal.append([l1, l2])

    for l1 in LMS:
        for l2 in LMS:
            for t in range(6):
                a1, a2 = np.exp(rng.uniform(np.log(0.12), np.log(1.0e4), 2))
                A = rng.normal(size=3) * 2.0
                B = A + rng.normal(size=3) * (0.5 if t < 4 else 3.0)
                add(a1, a2, A, B, l1, l2)
            A = rng.normal(size=3)
            add(0.3, 2.0, A, A.copy(), l1, l2)                     # coincident centres
            add(0.15, 5.0e5, A, A + [0.2, -0.1, 0.05], l1, l2)     # very unequal exponents
            add(2.0e3, 3.0e3, A, A + [0.01, 0.02, -0.01], l1, l2)  # large exponents, near centres
            add(0.12, 0.2, A, A + [6.0, -4.0, 3.0], l1, l2)        # diffuse, far apart
    out = os.path.join(HERE, "momentum.npz")
    np.savez_compressed(out, params=np.array(params), lmalpha=np.array(lmal, np.int32),
                        sh=np.array(outs))
    print(f"wrote {out}: {len(outs)} momentum blocks (x, y, z)")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
