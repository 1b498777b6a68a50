"""Regenerate tests/golden/sample_deck.json from the PLES sample deck.

Run where the PLES sources are mounted:
    python tests/golden/make_golden.py /path/to/PLES

The deck gri3dp_in.dat (read by fsrc/stratiParticle.f03:365-423) is a 32^3
tensor-product grid: x depends on i only, y on j only, z on k only.  The
fixture keeps the lengths, the cell counts, the three 1-D node arrays, the
periodicity and solver settings of Aboundary.in / Agenerale.in, and a
checksum of the full coordinate set so the reconstruction can be verified.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from ples_gb300.synthetic import read_gri3dp  # noqa: E402


def main(root):
    lengths, dims, (x, y, z) = read_gri3dp(os.path.join(root, "gri3dp_in.dat"))
    xs, ys, zs = x[:, 0, 0], y[0, :, 0], z[0, 0, :]
    assert np.all(x == xs[:, None, None]) and np.all(y == ys[None, :, None])
    assert np.all(z == zs[None, None, :])
    h = hashlib.sha256()
    for a in (x, y, z):
        h.update(np.ascontiguousarray(a.ravel(order="F")).tobytes())
    out = {
        "source": "gri3dp_in.dat, Aboundary.in:6-8, Agenerale.in:41-52",
        "lengths": list(lengths),
        "dims": list(dims),
        "x": xs.tolist(),
        "y": ys.tolist(),
        "z": zs.tolist(),
        "coords_sha256": h.hexdigest(),
        "periodicity": {"ip": 0, "jp": 1, "kp": 0},
        "solver": {"omega": 1.6, "islor": 0, "nlevmultimax": 4, "eps": 1e-8, "ficycle": 1000},
    }
    with open(os.path.join(HERE, "sample_deck.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of the PLES sources>")
    main(sys.argv[1])
