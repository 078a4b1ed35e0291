"""Generates tests/golden/primitives.npz from the reference's own integral code.

Run in a tree where the reference is checked out (it reads
src/olcao/gaussIntegrals.f90 through oracle/fexpr_eval.py, which executes the
generated Fortran statements verbatim in binary64):

    python tests/golden/make_primitive_goldens.py [path/to/gaussIntegrals.f90]

The fixture holds, for overlap2CIntg (kind 1), kinetic2CIntg (2),
nuclear3CIntg (3), electron3CIntg (4) and massvel2CIntg (5), seeded inputs
for every (lmAlpha1, lmAlpha2) block the reference generates (s/p/d/f, the
f-f block being each routine's final `else`) plus edge cases (coincident
centres, Boys argument at and around the reference's 0.1
series/closed-form switch, extreme exponents, large separations), and the
Boys values F_0..F_6 on a grid.  The f-f blocks of kinds 1-4 come last
(drawn after everything else, so the earlier entries keep their inputs).  For kind 5 it also stores the rounding
scale of each block (oracle.massvel_scale): with very unequal exponents the
nabla^4 expansion cancels to many digits and both the reference's and any
other FP64 evaluation are only accurate relative to that scale.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import fexpr_eval as fe  # noqa: E402
import oracle as orc  # noqa: E402

LMS = (1, 4, 9, 16)


def main(path=None):
    path = path or fe.default_path()
    F = fe.FortranIntegrals(path)
    rng = np.random.default_rng(20261203)
    params, lmal, kinds, outs, scales = [], [], [], [], []

    def add(kind, a1, a2, a3, A, B, Cc, l1, l2):
        sw = fe.l1l2switch(l1, l2)
        if kind == 1:
            sh = F.overlap(a1, a2, A, B, sw)
        elif kind == 2:
            sh = F.kinetic(a1, a2, A, B, sw)
        elif kind == 3:
            sh = F.nuclear3c(a1, a2, a3, A, B, Cc, sw)
        elif kind == 4:
            sh = F.electron3c(a1, a2, a3, A, B, Cc, sw)
        else:
            sh = F.massvel(a1, a2, A, B, sw)
        lof = {1: 0, 4: 1, 9: 2, 16: 3}
        scales.append(orc.massvel_scale(a1, a2, A, B, lof[l1], lof[l2]) if kind == 5 else np.nan)
        block = np.full((16, 16), np.nan)
        block[:l1, :l2] = sh[:l1, :l2]
        params.append([a1, a2, a3, *A, *B, *Cc])
        lmal.append([l1, l2])
        kinds.append(kind)
        outs.append(block)

    for kind in (1, 2, 3, 4, 5):
        for l1 in LMS:
            for l2 in LMS:
                if l1 == 16 and l2 == 16 and kind != 5:
                    continue
                for t in range(8):
                    a1, a2, a3 = np.exp(rng.uniform(np.log(0.12), np.log(80.0), 3))
                    A, B, Cc = rng.uniform(-2.0, 2.0, (3, 3))
                    if t == 0:
                        B = A.copy()            # on-site pair
                    if t == 1:
                        Cc = A.copy()
                    if t == 2 and kind == 3:
                        # Boys argument close to the 0.1 switch
                        z3 = a1 + a2 + a3
                        G = (a1 * A + a2 * B + a3 * Cc) / z3
                        d = rng.standard_normal(3)
                        d /= np.linalg.norm(d)
                        Cc = G - d * np.sqrt(0.1 / z3) * (1.0 + rng.uniform(-1e-3, 1e-3))
                        # re-centre: G moves with C; iterate twice
                        for _ in range(3):
                            G = (a1 * A + a2 * B + a3 * Cc) / z3
                            Cc = G - d * np.sqrt(0.1 * 1.01 / z3)
                    if t == 3:
                        a1, a2 = 0.12, 1.0e6    # extreme exponents
                    if t == 4:
                        B = A + rng.standard_normal(3) * 4.0
                    add(kind, a1, a2, a3, A, B, Cc, l1, l2)
    # f-f blocks of kinds 1-4 (`else ! switch 136` of each routine)
    for kind in (1, 2, 3, 4):
        for t in range(6):
            a1, a2, a3 = np.exp(rng.uniform(np.log(0.12), np.log(80.0), 3))
            A, B, Cc = rng.uniform(-2.0, 2.0, (3, 3))
            if t == 0:
                B = A.copy()
            if t == 1:
                Cc = A.copy()
            add(kind, a1, a2, a3, A, B, Cc, 16, 16)
    grid = np.concatenate([[0.0, 1e-12, 1e-6, 0.05, 0.0999999, 0.1, 0.10000001,
                            0.1000001, 0.2], np.geomspace(0.3, 80.0, 40)])
    boys = np.array([F.boys(T) for T in grid])
    out = os.path.join(HERE, "primitives.npz")
    np.savez_compressed(out, params=np.array(params), lmalpha=np.array(lmal, np.int32),
                        kind=np.array(kinds, np.int32), sh=np.array(outs),
                        scale=np.array(scales),
                        boys_T=grid, boys_F=boys,
                        source=np.array(os.path.relpath(path, os.path.dirname(path) + "/../..")))
    print(f"wrote {out}: {len(kinds)} primitive blocks, {len(grid)} Boys points")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
