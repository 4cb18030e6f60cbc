"""The reference's SmoothBump case (tests/SmoothBump of FEST-3D: two
48x48x1-cell blocks joined by an interface, mapping.txt) run unmerged on
the GPU, both blocks in one batch.

* The reference's own run (system/fvscheme.md "implicit", control.md CFL
  1000 and 3000 iterations from the free stream), LU-SGS in FP64: the
  relative entropy change of SmoothBump/pp/entropy.py is the 7.883E-07 of
  tests/Report.txt to the four digits the report prints; and the first 20
  iterations within 1e-11 of the oracle's two-block LU-SGS run.
* Explicit RK4 at CFL 1.5 with local time steps for the 10^5 iterations of
  the committed steady state (tests/golden/smoothbump_converged.npz: the
  oracle's run on the merged grid, whose entropy change is the report's):
  FP64 and mixed precision, each block through its fused sweep.  The
  interior state against the fixture: FP64 within 1e-9 of each variable's
  scale, mixed within 1e-5 (the FP32 stencil's steady state differs from
  the FP64 one by the rounding of the flux balance), and both entropy
  changes to the report's 7.883E-07 (FP64 to its four digits, mixed to
  1e-9 absolute)."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

import oracle as O
from fest3d import abi, post
from fest3d.handle import Handle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_smoothbump as MS  # noqa: E402

pytestmark = pytest.mark.gpu

REPORT_DS = 7.883e-07  # tests/Report.txt: "Calculated relative change in entropy: 7.883E-07"
P_INF, RHO_INF = 101325.0, 1.225


def two_blocks(integrator):
    """The case's two blocks as (ext, flow, scheme, bc, nodes, qp): block 0
    (far field at imin) and block 1 (subsonic outlet at imax) share the node
    plane i = 49 of the merged grid; block 0's imax pairs with block 1's
    imin column for column (mapping.txt: "0 2 1 49 1 2 1 1 1 49 1 2 0")."""
    nodes = np.load(os.path.join(HERE, "golden", "smoothbump_nodes.npz"))["nodes"]
    out = []
    for b, sl in enumerate((slice(0, 49), slice(48, 97))):
        ext, flow, scheme, _, nd, qp = MS.smoothbump_case(nodes[sl])
        scheme = abi.Scheme.from_buffer_copy(scheme)
        scheme.time_step_accuracy = abi.TIME[integrator]
        ids = [-8, 1, -6, -6, -6, -6] if b == 0 else [0, -4, -6, -6, -6, -6]
        partners = {1: (1, 0)} if b == 0 else {0: (0, 1)}
        bc = abi.make_bc(ids, partners=partners, block_id=b, fixed_pressure=[P_INF] * 6)
        out.append((ext, flow, scheme, bc, nd, qp))
    return out


def _interior(ext):
    return (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))


def merged(qs, exts):
    return np.concatenate([q[_interior(e)] for q, e in zip(qs, exts)], axis=0)


def entropy(parts, qs):
    """entropy.py over both blocks' interior cells"""
    vols = []
    for ext, flow, scheme, bc, nodes, qp in parts:
        blk = O.Block(ext, flow, scheme, bc)
        blk["nodes"] = nodes
        blk.setup_geometry()
        vols.append(np.array(blk["cells"][0][_interior(ext)]))
    q = merged(qs, [p[0] for p in parts])
    return post.entropy_change(q, np.concatenate(vols, axis=0), P_INF, RHO_INF, 1.4)


def run_batch(lib, parts, precision, iters, CFL):
    hs = []
    for ext, flow, scheme, bc, nodes, qp in parts:
        h = Handle(ext, flow, scheme, bc, lib=lib)
        h.setup_geometry(nodes)
        h.upload_state(qp)
        h.set_precision(precision)
        hs.append(h)
    arr = (C.c_void_p * len(hs))(*[h.h.value for h in hs])
    b = C.c_void_p()
    abi.check(lib.fest_batch_create(arr, len(hs), C.byref(b)), "fest_batch_create")
    try:
        abi.check(lib.fest_batch_step(b, iters, 1, CFL), "fest_batch_step")
        return [h.download_state() for h in hs]
    finally:
        lib.fest_batch_destroy(b)
        for h in hs:
            h.close()


def _scale(q):
    V = 170.14  # the free-stream speed (w stays 0 in the one-cell-thick case)
    return [np.abs(q[..., 0]).max(), V, V, V, np.abs(q[..., 4]).max()]


def test_reference_smoothbump_run_lusgs_on_gpu(gpu_lib):
    parts = two_blocks("implicit")
    qs = run_batch(gpu_lib, parts, abi.FEST_FP64, 3000, 1000.0)
    ds = entropy(parts, qs)
    assert abs(ds - REPORT_DS) <= 0.5e-10, ds


def test_smoothbump_lusgs_matches_oracle(gpu_lib):
    parts = two_blocks("implicit")
    qs = run_batch(gpu_lib, parts, abi.FEST_FP64, 20, 1000.0)
    blocks = []
    for ext, flow, scheme, bc, nodes, qp in parts:
        blk = O.Block(ext, flow, scheme, bc)
        blk["nodes"] = nodes
        blk.setup_geometry()
        blk["qp"] = qp
        blocks.append(blk)
    for it in range(1, 21):
        assert O.lusgs_next_solution(blocks, it, 1000.0) == 0
    for n, (q, blk) in enumerate(zip(qs, blocks)):
        e = blk.ext
        a, r = post.interior(q, e), post.interior(blk["qp"], e)
        sc = _scale(r)
        err = max(np.abs(a[..., l] - r[..., l]).max() / sc[l] for l in range(5))
        assert err <= 1e-11, f"block {n}: {err:.3e}"


@pytest.mark.parametrize("precision", [abi.FEST_FP64, abi.FEST_MIXED], ids=["fp64", "mixed"])
def test_smoothbump_rk4_steady_state_unmerged(gpu_lib, precision):
    parts = two_blocks("RK4")
    fx = np.load(os.path.join(HERE, "golden", "smoothbump_converged.npz"))
    qs = run_batch(gpu_lib, parts, precision, 100000, 1.5)
    q = merged(qs, [p[0] for p in parts])
    ref = fx["q"]
    sc = _scale(ref)
    errs = [float(np.abs(q[..., l] - ref[..., l]).max() / sc[l]) for l in range(5)]
    ds = entropy(parts, qs)
    if precision == abi.FEST_FP64:
        assert max(errs) <= 1e-9, errs
        assert abs(ds - REPORT_DS) <= 0.5e-10, ds
    else:
        assert max(errs) <= 1e-5, errs
        assert abs(ds - REPORT_DS) <= 1e-9, ds
