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
    assert L.fest_snapshot_begin(None, None) == abi.FEST_ERR_ARG
    assert L.fest_snapshot_wait(None) == abi.FEST_ERR_ARG
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


class _StreamStandIn:
    """The calls Handle.iterate makes, on a state that is the number of
    iterations done: work runs at once, which is the order the handle's
    stream runs it in."""

    def __init__(self, ext, first):
        self.shape = {"qp": abi.shapes(ext)["qp"]}
        self.done, self.log = first - 1, []

    def step_async(self, n, first, CFL):
        assert first == self.done + 1
        self.done += n
        self.log.append(("step", first, n))

    def snapshot_begin(self, q):
        q[...] = self.done
        self.log.append(("begin", self.done))

    def snapshot_wait(self):
        self.log.append(("wait",))

    def last_device_error(self):
        self.log.append(("sync",))


@pytest.mark.parametrize("max_iters,every,first", [(10, 3, 1), (9, 3, 1), (7, 0, 1), (12, 5, 4),
                                                   (3, 10, 1)])
def test_iterate_follows_the_reference_checkpoint_schedule(max_iters, every, first):
    """Handle.iterate hands on_checkpoint the states of the iterations
    dump_solution.f90:40-43 dumps (every checkpoint_iter-th and the last;
    none when checkpoint_iter is 0), and enqueues the next iterations before
    it waits for a snapshot."""
    import numpy as np
    from fest3d.handle import Handle
    h = _StreamStandIn(abi.Extent(9, 7, 5, 5), first)
    got = []
    nxt = Handle.iterate(h, max_iters, 0.5, every, lambda it, q: got.append((it, float(q.flat[0]))),
                         first_iter=first)
    want = [] if every == 0 else [it for it in range(first, max_iters + 1)
                                  if it % every == 0 or it == max_iters]
    assert [it for it, _ in got] == want
    assert all(v == it for it, v in got)  # each snapshot holds its own iteration's state
    assert nxt == max_iters + 1 and h.done == max_iters and h.log[-1] == ("sync",)
    # overlap: between a snapshot's begin and its wait, the next stretch of
    # iterations is already enqueued
    for a, b in zip(want, want[1:]):
        i = h.log.index(("begin", a))
        assert h.log[i + 1][0] == "step" and h.log[i + 2] == ("wait",)
    assert np.all(np.isfinite([v for _, v in got]))


def test_struct_layouts_match_the_header(tmp_path):
    """Every field of fest_extent, fest_flow, fest_scheme and fest_bc sits
    at the same offset in the ctypes mirrors as the C compiler places it
    from include/fest_gpu.h (tests/abi_layout.c prints the C side)."""
    import subprocess
    exe = tmp_path / "abi_layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_layout.c"), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                              text=True).stdout.split("\n") if line)
    want = {}
    for T, n in ((abi.Extent, "fest_extent"), (abi.Flow, "fest_flow"), (abi.Scheme, "fest_scheme"),
                 (abi.BC, "fest_bc")):
        want[n] = str(C.sizeof(T))
        for f, _ in T._fields_:
            want[f"{n}.{f}"] = str(getattr(T, f).offset)
    assert got == want
