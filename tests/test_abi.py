"""The C ABI library: builds for sm_103a, loads, exports every symbol the
public header declares, and rejects bad descriptors before touching a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from ples_gb300 import build, mg
from ples_gb300 import synthetic as S

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ples_mg.h")


def declared_functions():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ples_(?:mg|srv)_\w+)\s*\(", txt)))


def test_library_builds_and_loads():
    path = build.build()
    assert os.path.exists(path)
    lib = mg.load()
    assert lib is not None


def test_every_declared_symbol_is_exported():
    lib = C.CDLL(build.build())
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(mg.EXPORTS)


def test_strerror_covers_codes():
    lib = mg.load()
    msgs = {lib.ples_mg_strerror(c).decode() for c in range(8)}
    assert len(msgs) == 8
    assert lib.ples_mg_strerror(99).decode() == "unknown status"


def _desc(**kw):
    x, y, z = S.wavy_channel_grid(16, 8, 16, 0.05, 2.0)
    keep = (np.asfortranarray(x), np.asfortranarray(y), np.asfortranarray(z))
    d = mg.Desc()
    d.jx, d.jy, d.jz, d.ip, d.jp, d.kp = 16, 8, 16, 0, 1, 0
    d.precision, d.coords_layout, d.dt = mg.PREC_MIXED, mg.COORDS_NODES, 1.0
    dp = C.POINTER(C.c_double)
    d.x, d.y, d.z = (a.ctypes.data_as(dp) for a in keep)
    for k, v in kw.items():
        setattr(d, k, v)
    return d, keep


@pytest.mark.parametrize("fields", [{"jp": 0}, {"ip": 2}, {"kp": -1}, {"jx": 4}, {"precision": 7},
                                    {"coords_layout": 5}, {"dt": 0.0}, {"smoother": 4}, {"jz": 15},
                                    {"freesurface": 2}, {"freesurface": 1, "smoother": 0}],
                         ids=lambda f: ",".join(f"{k}={v}" for k, v in f.items()))
def test_bad_descriptor_rejected_without_device(fields):
    """Including a free surface without the point smoother: the reference's
    line SOR keeps the wall relation (multigrid.f03:2019)."""
    lib = mg.load()
    d, keep = _desc(**fields)
    h = C.c_void_p()
    rc = lib.ples_mg_create(C.byref(d), C.byref(h))
    assert rc == mg.BAD_ARG
    assert not h.value


def test_null_arguments():
    lib = mg.load()
    assert lib.ples_mg_create(None, None) == mg.BAD_ARG
    h = C.c_void_p()
    assert lib.ples_mg_create(None, C.byref(h)) == mg.BAD_ARG
    lib.ples_mg_destroy(None)
    assert lib.ples_mg_set_line_threads(None, 1, 256) == mg.BAD_ARG


def test_no_device_reported_on_cpu_host():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = mg.load()
    d, keep = _desc()
    h = C.c_void_p()
    assert lib.ples_mg_create(C.byref(d), C.byref(h)) == mg.NO_DEVICE
    with pytest.raises(mg.PlesMGError):
        mg.Multigrid(*S.wavy_channel_grid(16, 8, 16, 0.05, 2.0))
