"""The C ABI library: it loads without a GPU, exports every symbol the
public headers declare, and its compute entry points report an error
(never a silent host result) when no device is present."""
import ctypes
import os
import re

import numpy as np

from gplum_gb300 import _lib
from tests.conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(p3t_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported():
    lib = _lib.host_lib()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if getattr(lib, n, None) is None]
    assert not missing, missing
    assert names <= set(_lib.SIGNATURES), sorted(names - set(_lib.SIGNATURES))


def test_compute_without_device_fails_loudly():
    if gpu_available():
        return
    lib = _lib.host_lib()
    assert lib.p3t_init(0) < 0
    assert lib.p3t_soft_run(0) < 0
    f = np.zeros(4, np.uint8)
    assert lib.p3t_epep(f.ctypes.data_as(ctypes.c_void_p), 0, None, 0, None) < 0
