"""Regenerate the golden fixtures from the ASTR reference tree.

The only numeric golden artefact ASTR ships for this path is the 100-step
kinetic-energy / enstrophy history of the 128^3 Taylor-Green vortex written
by the compact-scheme mini-app (``miniapps/tgv_solver_3d/state.ref_128``,
columns nstep, time, KE, enstrophy).  This script copies its numbers into
``tgv128_state_ref.txt`` so the tests can run where the reference tree is
absent.  Usage: ``python tests/golden/make_golden.py /path/to/astr`` (the root of
the ASTR source tree; required).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(root: str) -> None:
    src = os.path.join(root, "miniapps", "tgv_solver_3d", "state.ref_128")
    rows = np.loadtxt(src)
    out = os.path.join(HERE, "tgv128_state_ref.txt")
    with open(out, "w") as f:
        f.write("# nstep time kinetic_energy enstrophy  "
                "(ASTR miniapps/tgv_solver_3d/state.ref_128)\n")
        for r in rows:
            f.write(f"{int(r[0])} {float(r[1])!r} {float(r[2])!r} {float(r[3])!r}\n")
    print(f"wrote {out} ({len(rows)} rows)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/astr")
    main(sys.argv[1])
