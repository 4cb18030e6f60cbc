"""CPU-only checks of the C ABI: the in-tree library loads and exports every
symbol include/fest_gpu.h declares; argument validation happens before any
device work."""
import ctypes as C
import os
import re

import pytest

from fest3d import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "fest_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fest_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    return C.CDLL(abi.LIB_PATH)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    assert set(declared_functions()) <= set(abi.EXPORTED) | {
        "fest_array_size", "fest_set_array", "fest_get_array"}


def test_argument_validation_without_device(lib):
    L = abi.load()
    h = C.c_void_p()
    ext = abi.Extent(1, 5, 5, 5)  # imx < 2
    rc = L.fest_create(C.byref(ext), C.byref(abi.make_flow()), C.byref(abi.make_scheme()),
                       C.byref(abi.make_bc([-5] * 6)), C.byref(h))
    assert rc == abi.FEST_ERR_ARG
    ext = abi.Extent(9, 7, 6, 5)
    # interface partners: a face number outside 0..5, a negative block, an
    # orientation outside 0..7, a self pair whose columns do not match
    for partners in ({0: (1, 6), 1: (0, 0)}, {0: (-1, 1), 1: (0, 0)}, {0: (0, 1, 8), 1: (0, 0)},
                     {0: (0, 2), 1: (0, 0)}):
        bc = abi.make_bc([-10, -10, -5, -5, -5, -5], partners=partners)
        rc = L.fest_create(C.byref(ext), C.byref(abi.make_flow()), C.byref(abi.make_scheme()),
                           C.byref(bc), C.byref(h))
        assert rc == abi.FEST_ERR_ARG, partners
    for fn in ("fest_destroy", "fest_find_resnorm", "fest_step"):
        assert getattr(L, fn)(None, *([None] if fn == "fest_find_resnorm" else
                                       [0, 0, 0.5, None] if fn == "fest_step" else [])) in (0, 1)


def test_handle_refuses_short_host_arrays():
    """Host arrays shorter than what a C call reads are refused before the
    call (no device needed: the object is built without fest_create)."""
    import numpy as np
    from fest3d.handle import Handle
    ext = abi.Extent(9, 7, 5, 5)
    sh = abi.shapes(ext)
    h = Handle.__new__(Handle)
    h.h = None
    h.shape = {"qp": sh["qp"], "residue": sh["residue"], "cells": sh["cells"],
               "Ifaces": sh["Ifaces"], "Jfaces": sh["Jfaces"], "Kfaces": sh["Kfaces"]}
    ok = h._input(np.zeros(sh["qp"], order="C"), "qp")
    assert ok.flags.f_contiguous and ok.dtype == np.float64 and ok.shape == sh["qp"]
    with pytest.raises(ValueError):
        h._input(np.zeros(sh["qp"])[..., :4], "qp")
    with pytest.raises(ValueError):
        h._input(np.zeros(sh["residue"][:3]), "residue", copy=False)
    # set_metrics checks each of its four arrays before the call
    full = [np.zeros(sh[n], order="F") for n in ("cells", "Ifaces", "Jfaces", "Kfaces")]
    for bad in range(4):
        args = list(full)
        args[bad] = args[bad].ravel(order="F")[:-1]
        with pytest.raises(ValueError):
            h.set_metrics(*args)
