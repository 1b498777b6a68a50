"""PLES's grid file (gri3dp_in.dat, read by fsrc/stratiParticle.f03:364-412)
through the native reader ples_mg_read_grid: no device needed.

The reader follows Fortran list-directed input: the header READs take their
values from as many records as they need, each coordinate READ starts a new
record and takes its first value, and D exponents read as E.  Checked
bit-for-bit against numpy's parse of files written by synthetic.write_gri3dp
and against the committed sample-deck fixture.
"""
import json
import os

import numpy as np
import pytest

from ples_gb300 import mg
from ples_gb300 import synthetic as S

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_read_grid_matches_numpy(tmp_path):
    x, y, z = S.wavy_channel_grid(12, 6, 10, 0.1, 2.5)
    path = tmp_path / "gri3dp_in.dat"
    S.write_gri3dp(str(path), (2 * np.pi, 2.0, np.pi), x, y, z)
    lengths, dims, (gx, gy, gz) = mg.read_grid(str(path))
    rl, rd, (rx, ry, rz) = S.read_gri3dp(str(path))
    assert dims == rd == (12, 6, 10)
    assert lengths == rl
    for a, b in ((gx, rx), (gy, ry), (gz, rz)):
        assert a.flags.f_contiguous and np.array_equal(a, b)


def test_read_grid_sample_deck(tmp_path):
    """The 32^3 sample deck of the reference, rewritten from the committed
    fixture in the reference's own line layout."""
    d = json.load(open(os.path.join(GOLDEN, "sample_deck.json")))
    xs, ys, zs = (np.array(d[c]) for c in "xyz")
    shp = (xs.size, ys.size, zs.size)
    x = np.asfortranarray(np.broadcast_to(xs[:, None, None], shp))
    y = np.asfortranarray(np.broadcast_to(ys[None, :, None], shp))
    z = np.asfortranarray(np.broadcast_to(zs[None, None, :], shp))
    path = tmp_path / "gri3dp_in.dat"
    S.write_gri3dp(str(path), (xs[-1], ys[-1], zs[-1]), x, y, z)
    _, dims, (gx, gy, gz) = mg.read_grid(str(path))
    assert dims == (32, 32, 32)
    assert np.array_equal(gx, x) and np.array_equal(gy, y) and np.array_equal(gz, z)


def test_read_grid_fortran_records(tmp_path):
    """Header values spread over records, D exponents, trailing values on a
    coordinate record ignored, blank records skipped."""
    jx, jy, jz = 1, 1, 1
    n = (jx + 1) * (jy + 1) * (jz + 1)
    lines = ["6.283185307179586D+00", "2.0d0, 3.1415926535897931", "1 1", "1"]
    want = np.arange(3 * n, dtype=np.float64) * 0.25 - 1.0
    for q in range(n):
        for c in range(3):
            v = float(want[3 * q + c])
            lines.append(f"{v:.17e}   99.0  junk" if c == 1 else f" {v!r}")
            if q == 2 and c == 0:
                lines.append("")
    path = tmp_path / "gri3dp_in.dat"
    path.write_text("\r\n".join(lines) + "\r\n")
    lengths, dims, (x, y, z) = mg.read_grid(str(path))
    assert dims == (1, 1, 1)
    assert lengths == (6.283185307179586, 2.0, 3.1415926535897931)
    got = np.stack([x.ravel(order="F"), y.ravel(order="F"), z.ravel(order="F")], axis=1).ravel()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("text", ["", "1.0 2.0 3.0\n4 4\n", "1 2 3\n2 2 2\n0.5\n0.5\n"])
def test_read_grid_rejects_malformed(tmp_path, text):
    path = tmp_path / "bad.dat"
    path.write_text(text)
    with pytest.raises(mg.PlesMGError) as e:
        mg.read_grid(str(path))
    assert e.value.code == mg.BAD_ARG


def test_read_grid_missing_file(tmp_path):
    with pytest.raises(mg.PlesMGError):
        mg.read_grid(str(tmp_path / "absent.dat"))
