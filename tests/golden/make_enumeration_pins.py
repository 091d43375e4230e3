"""Writes tests/golden/enumeration_pins.json: the oracle's full enumeration of large sectors,
as a count and a SHA-256 of the sorted little-endian uint64 representatives.

The oracle's threaded enumeration (oracle/ls_oracle.c lso_enumerate_projected_par: Benes orbit
scan in the reference's chunk order, StatesEnumeration.chpl:242-268) takes minutes on a few
cores for these sectors, so the GPU tests compare against these pins instead of enumerating
again.  Run from the repository root:

    python tests/golden/make_enumeration_pins.py
"""

from __future__ import annotations

import hashlib
import importlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for p in (REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402


def sectors():
    ls = importlib.import_module("lattice-symmetries_gb300")
    lat = importlib.import_module("lattice-symmetries_gb300.lattices")
    return {
        # the bench's default workload: J1-J2 6x6 torus, (pi, pi), T x C4v x Z2, Sz = 0
        "square6_pipi_z1": ls.SpinBasis(36, 18, 1, ls.Symmetries(lat.square_symmetries(6, 3, 3))),
        # triangular 6x6 torus, T x C6v x Z2, Sz = 0 (16 group elements per lane)
        "triangular6_c6v_z1": ls.SpinBasis(36, 18, 1, ls.Symmetries(lat.triangular_symmetries(6, 0, 0, 0, 0))),
    }


def main():
    from ls_helpers import oracle_group
    O.build()
    out = {}
    for name, basis in sectors().items():
        g = oracle_group(basis.symmetries, basis._c.spin_inversion)
        lo, hi = basis._estimates()
        t0 = time.time()
        reps = O.enumerate_projected_par(g, lo, hi, lane_width=8, use_benes=True)
        out[name] = {"count": int(len(reps)), "sha256": hashlib.sha256(reps.astype("<u8").tobytes()).hexdigest(),
                     "first": [int(v) for v in reps[:4]], "last": [int(v) for v in reps[-4:]]}
        print(name, out[name]["count"], "{:.1f} s".format(time.time() - t0), flush=True)
    with open(os.path.join(HERE, "enumeration_pins.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
