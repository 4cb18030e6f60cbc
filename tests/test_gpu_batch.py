"""Batched multiblock stepping (fest_batch_*): one ghost launch and one sweep
launch per stage for all blocks (or, when the blocks share no sweep kernel,
each block's own launches stage by stage).

The batched sweep runs the same per-CTA code as the single-block sweep, so
every block's state must equal, bit for bit, the state its own handle
reaches with fest_step; and the blocks (periodic or extrapolated faces,
thin ones included) follow the FP64 oracle to the mixed-precision bound of
2e-5 of each variable's magnitude over six iterations."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from fest3d import abi, cases
from fest3d.handle import Handle

pytestmark = pytest.mark.gpu


def small_blocks(n=6, seed=3, viscous=True):
    return cases.batch_blocks(n=n, seed=seed, dims_lo=(8, 8, 1), dims_hi=(40, 30, 8), viscous=viscous)


def handle_of(c, lib):
    h = Handle(c["ext"], c["flow"], c["scheme"], c["bc"], lib=lib)
    h.setup_geometry(c["nodes"])
    h.upload_state(c["qp"])
    h.set_precision(abi.FEST_MIXED)
    return h


def make_batch(lib, handles):
    arr = (C.c_void_p * len(handles))(*[h.h.value for h in handles])
    b = C.c_void_p()
    abi.check(lib.fest_batch_create(arr, len(handles), C.byref(b)), "fest_batch_create")
    return b


@pytest.mark.parametrize("viscous", [False, True])
def test_batch_equals_single_blocks(gpu_lib, viscous):
    blocks = small_blocks(viscous=viscous)
    single = [handle_of(c, gpu_lib) for c in blocks]
    batched = [handle_of(c, gpu_lib) for c in blocks]
    b = make_batch(gpu_lib, batched)
    try:
        for h, c in zip(single, blocks):
            h.step(6, 1, c["CFL"], with_norm=False)
        abi.check(gpu_lib.fest_batch_step(b, 3, 1, 0.5), "fest_batch_step")
        abi.check(gpu_lib.fest_batch_step(b, 3, 4, 0.5), "fest_batch_step")
        for n, (hs, hb) in enumerate(zip(single, batched)):
            qs, qb = hs.download_state(), hb.download_state()
            ext = blocks[n]["ext"]
            sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
            assert np.array_equal(qs[sl], qb[sl]), f"block {n} differs"
            # each handle still answers for its own block
            assert np.all(np.isfinite(hb.resnorm()))
    finally:
        gpu_lib.fest_batch_destroy(b)


@pytest.mark.parametrize("viscous", [False, True])
def test_batch_follows_oracle(gpu_lib, viscous):
    blocks = small_blocks(n=4, seed=5, viscous=viscous)
    hs = [handle_of(c, gpu_lib) for c in blocks]
    b = make_batch(gpu_lib, hs)
    try:
        abi.check(gpu_lib.fest_batch_step(b, 6, 1, 0.5), "fest_batch_step")
    finally:
        gpu_lib.fest_batch_destroy(b)
    for n, (c, h) in enumerate(zip(blocks, hs)):
        blk = O.Block(c["ext"], c["flow"], c["scheme"], c["bc"])
        blk["nodes"] = c["nodes"]
        blk.setup_geometry()
        blk["qp"] = c["qp"]
        for it in range(1, 7):
            assert O.get_next_solution([blk], it, c["CFL"]) == 0
        ext = c["ext"]
        sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
        q, ref = h.download_state()[sl], blk["qp"][sl]
        for l in range(5):
            e = np.abs(q[..., l] - ref[..., l]).max() / np.abs(ref[..., l]).max()
            assert e <= 2e-5, (n, l, e, (ext.imx - 1, ext.jmx - 1, ext.kmx - 1))


def test_batch_of_different_schemes_steps_block_by_block(gpu_lib):
    """blocks with different flux schemes share no sweep kernel: the batch
    launches each block's own sweeps, stage by stage, which gives the states
    stepping them alone gives; different integrators share no stages and are
    refused"""
    blocks = small_blocks(n=2)
    blocks[1]["scheme"] = abi.make_scheme(scheme_name="slau", interpolant="muscl",
                                          time_step_accuracy="TVDRK3", time_stepping_method="l")
    single = [handle_of(c, gpu_lib) for c in blocks]
    batched = [handle_of(c, gpu_lib) for c in blocks]
    b = make_batch(gpu_lib, batched)
    try:
        for h, c in zip(single, blocks):
            h.step(6, 1, c["CFL"], with_norm=False)
        abi.check(gpu_lib.fest_batch_step(b, 6, 1, 0.5), "fest_batch_step")
        for n, (hs, hb) in enumerate(zip(single, batched)):
            ext = blocks[n]["ext"]
            sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
            assert np.array_equal(hs.download_state()[sl], hb.download_state()[sl]), f"block {n} differs"
    finally:
        gpu_lib.fest_batch_destroy(b)
    blocks[1]["scheme"] = abi.make_scheme(scheme_name="slau", interpolant="muscl",
                                          time_step_accuracy="RK4", time_stepping_method="l")
    hs = [handle_of(c, gpu_lib) for c in blocks]
    arr = (C.c_void_p * 2)(*[h.h.value for h in hs])
    b = C.c_void_p()
    assert gpu_lib.fest_batch_create(arr, 2, C.byref(b)) == abi.FEST_ERR_ARG


def sst_blocks():
    """three k-omega SST blocks of different sizes and walls (wall distances
    from their -5 faces' nodes)"""
    from parity import small_case
    out = []
    for nc, ids in (((14, 9, 5), (-3, -4, -5, -4, -10, -10)),
                    ((21, 7, 6), (-3, -4, -5, -6, -10, -10)),
                    ((9, 12, 4), (-2, -4, -5, -5, -6, -6))):
        ext, flow, scheme, bc, nodes, qp = small_case(
            nc=nc, ids=ids, turb=True, scheme_kw=dict(interpolant="muscl", scheme_name="ausmUP",
                                                      time_step_accuracy="RK4"),
            flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law", MInf=0.2))
        out.append(dict(ext=ext, flow=flow, scheme=scheme, bc=bc, nodes=nodes, qp=qp, CFL=0.5,
                        wall=cases.wall_nodes_of(nodes, ext, bc)))
    return out


def sst_handle(c, lib):
    h = Handle(c["ext"], c["flow"], c["scheme"], c["bc"], lib=lib)
    h.setup_geometry(c["nodes"])
    h.find_wall_dist(c["wall"])
    h.upload_state(c["qp"])
    h.set_precision(abi.FEST_MIXED)
    return h


def test_sst_batch_equals_single_blocks_and_follows_oracle(gpu_lib):
    blocks = sst_blocks()
    single = [sst_handle(c, gpu_lib) for c in blocks]
    batched = [sst_handle(c, gpu_lib) for c in blocks]
    b = make_batch(gpu_lib, batched)
    try:
        for h, c in zip(single, blocks):
            h.step(6, 1, c["CFL"], with_norm=False)
        abi.check(gpu_lib.fest_batch_step(b, 6, 1, 0.5), "fest_batch_step")
    finally:
        gpu_lib.fest_batch_destroy(b)
    for n, (hs, hb, c) in enumerate(zip(single, batched, blocks)):
        ext = c["ext"]
        sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
        qb = hb.download_state()
        assert np.array_equal(hs.download_state()[sl], qb[sl]), f"block {n} differs"
        blk = O.Block(ext, c["flow"], c["scheme"], c["bc"])
        blk["nodes"] = c["nodes"]
        blk.setup_geometry()
        blk.find_wall_dist(c["wall"])
        blk["qp"] = c["qp"]
        for it in range(1, 7):
            assert O.get_next_solution([blk], it, c["CFL"]) == 0
        ref = blk["qp"][sl]
        for l in range(ext.n_var):
            e = np.abs(qb[sl][..., l] - ref[..., l]).max() / np.abs(ref[..., l]).max()
            assert e <= 2e-5, (n, l, e)
