"""CPU checks of the C ABI boundary: the library builds for sm_103a, loads,
and exports every symbol include/*.h declares; the Python binding covers them
all.  No compute call is made (there is no GPU here)."""
import ctypes
import glob
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from isosurface_gb300 import _capi
from isosurface_gb300 import source as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names |= set(re.findall(r"^ISO_API[^(]*?\b(iso_\w+)\s*\(", text, re.M))
    return sorted(names)


def _built_lib():
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not available")
    from isosurface_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "iso_mc_extract" in names and "iso_ctx_create" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    path = _built_lib()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (iso_\w+)", out))
    missing = [n for n in declared_symbols() if n not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(path)  # loads without a GPU
    for n in declared_symbols():
        assert hasattr(lib, n)


def test_binding_covers_header():
    assert sorted(_capi.SIGNATURES) == declared_symbols()


def test_status_strings_without_gpu():
    _built_lib()
    L = _capi.lib()
    assert L.iso_status_str(0) == b"ISO_OK"
    assert L.iso_status_str(5) == b"ISO_ERR_BAD_PROGRAM"
    # no device in this container: context creation reports it, never aborts
    h = ctypes.c_void_p()
    st = L.iso_ctx_create(0, ctypes.byref(h))
    assert st in (0, 6)
    if st == 0:
        L.iso_ctx_destroy(h)


def test_lowering_layout():
    prog = S.lower(S.unit_to_cube(S.Sphere(0.75)))
    magic, n_ops, n_consts, flags = np.frombuffer(prog[:16], np.uint32)
    assert magic == 0x314F5349 and flags == 0
    ops = np.frombuffer(prog[16:16 + 4 * n_ops], np.uint32)
    assert [o & 0xFF for o in ops] == [0x01, 0x10, 0x04]
    consts = np.frombuffer(prog[16 + 4 * n_ops:], np.float32)
    assert len(consts) == n_consts == 7
    assert consts[6] == np.float32(0.75)
