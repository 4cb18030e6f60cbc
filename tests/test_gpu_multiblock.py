"""Interface exchange between the blocks of a batch, on the GPU, against the
oracle's multiblock run on the same blocks.

Two blocks cut from one (tests/multiblock.py): the halves side by side
(aligned columns) and with the second half turned a quarter turn (the
interface maps columns with a swap and a reversal).  Both advance in one
batch: FP64 (each block's own fused sweeps, stage by stage) within 1e-11 of
each variable's magnitude after three iterations; mixed precision (one
batched ghost launch and sweep launch per stage from iteration 3) within
2e-5 after six.  A handle whose face pairs with another block refuses to
step on its own."""
import ctypes as C

import numpy as np
import pytest

import multiblock as MB
import oracle as O
from fest3d import abi, post
from fest3d.handle import Handle

pytestmark = pytest.mark.gpu

SCHEMES = {"muscl-ausm-tvdrk3": dict(interpolant="muscl", scheme_name="ausm", time_step_accuracy="TVDRK3"),
           "weno-slau-rk4": dict(interpolant="weno", scheme_name="slau", time_step_accuracy="RK4")}
SPLITS = {"aligned": MB.split_aligned, "rotated": MB.split_rotated}


def _handles(lib, parts, flow, scheme, precision):
    hs = []
    for ext, bc, nodes, qp in parts:
        h = Handle(ext, flow, scheme, bc, lib=lib)
        h.setup_geometry(nodes)
        h.upload_state(qp)
        h.set_precision(precision)
        hs.append(h)
    return hs


def _batch(lib, hs):
    arr = (C.c_void_p * len(hs))(*[h.h.value for h in hs])
    b = C.c_void_p()
    abi.check(lib.fest_batch_create(arr, len(hs), C.byref(b)), "fest_batch_create")
    return b


def _oracle(parts, flow, scheme, iters, CFL):
    blocks = []
    for ext, bc, nodes, qp in parts:
        b = O.Block(ext, flow, scheme, bc)
        b["nodes"] = nodes
        b.setup_geometry()
        b["qp"] = qp
        blocks.append(b)
    for it in range(1, iters + 1):
        assert O.get_next_solution(blocks, it, CFL) == 0
    return blocks


@pytest.mark.parametrize("split", list(SPLITS))
@pytest.mark.parametrize("name", list(SCHEMES))
@pytest.mark.parametrize("precision", [abi.FEST_FP64, abi.FEST_MIXED], ids=["fp64", "mixed"])
def test_batch_interface_exchange_matches_oracle(gpu_lib, split, name, precision):
    ext, flow, scheme, bc, nodes, qp = MB.single_block(scheme_kw=SCHEMES[name])
    parts = SPLITS[split](ext, flow, scheme, nodes, qp)
    iters = 3 if precision == abi.FEST_FP64 else 6
    tol = 1e-11 if precision == abi.FEST_FP64 else 2e-5
    hs = _handles(gpu_lib, parts, flow, scheme, precision)
    b = _batch(gpu_lib, hs)
    try:
        abi.check(gpu_lib.fest_batch_step(b, 2, 1, 0.5), "fest_batch_step")
        abi.check(gpu_lib.fest_batch_step(b, iters - 2, 3, 0.5), "fest_batch_step")
        ref = _oracle(parts, flow, scheme, iters, 0.5)
        for n, (h, r) in enumerate(zip(hs, ref)):
            e = h.ext
            got, want = post.interior(h.download_state(), e), post.interior(r["qp"], e)
            V = flow.vel_mag
            sc = [np.abs(want[..., 0]).max(), V, V, V, np.abs(want[..., 4]).max()]
            err = max(np.abs(got[..., l] - want[..., l]).max() / sc[l] for l in range(5))
            assert err <= tol, f"block {n}: {err:.3e}"
    finally:
        gpu_lib.fest_batch_destroy(b)
        for h in hs:
            h.close()


def test_handle_with_partner_block_steps_only_in_its_batch(gpu_lib):
    ext, flow, scheme, bc, nodes, qp = MB.single_block(scheme_kw=SCHEMES["muscl-ausm-tvdrk3"])
    parts = MB.split_aligned(ext, flow, scheme, nodes, qp)
    hs = _handles(gpu_lib, parts, flow, scheme, abi.FEST_FP64)
    try:
        rc = gpu_lib.fest_step(hs[0].h, 1, 1, 0.5, None)
        assert rc == abi.FEST_ERR_ARG
        # a batch without the partner cannot resolve it either
        arr = (C.c_void_p * 1)(hs[0].h.value)
        b = C.c_void_p()
        assert gpu_lib.fest_batch_create(arr, 1, C.byref(b)) == abi.FEST_ERR_ARG
    finally:
        for h in hs:
            h.close()
