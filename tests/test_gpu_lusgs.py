"""The implicit integrators (LU-SGS, lusgs.f90:134-1196, and its low-Mach
preconditioned form PLU-SGS, plusgs.f90:139-1431) on the GPU against the
oracle's restatement of them, and the reference's own laminar flat-plate
run replayed on the GPU.

* Single blocks, laminar and k-omega SST, both integrators, three implicit
  iterations at CFL 200 (PLU-SGS at free-stream Mach 0.2, so that the
  preconditioner acts): interior state within 1e-11 of each variable's
  magnitude.  The hyperplane sweeps do per cell the reference's arithmetic
  in an order the data dependencies allow, so the result is the
  sequential sweep's.
* The reference's laminar flat plate (tests/Lfp: two blocks joined by an
  interface) in one batch: three iterations within 1e-11 of the oracle's
  two-block run, with either integrator; and the case's own run, 5000 iterations at CFL 2000 from
  the free stream, whose drag coefficient (Lfp/pp/Surface.py on the
  gradients of the last residual evaluation) is the reference's reported
  1.32933e-3 (tests/Report.txt) to 3e-5, as the oracle's replay is."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

import oracle as O
from fest3d import abi, cases, post
from fest3d.handle import Handle
from parity import make_pair, small_case

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_flatplate as MF  # noqa: E402

pytestmark = pytest.mark.gpu


def _err(q, ref, ext, speed=None):
    """max over variables of max|q - ref| / scale: each variable's magnitude,
    with `speed` for the velocity components (the two-dimensional plate's w
    is zero)"""
    a, b = post.interior(q, ext), post.interior(ref, ext)
    sc = [np.abs(b[..., l]).max() for l in range(ext.n_var)]
    if speed is not None:
        sc[1:4] = [speed] * 3
    return max(np.abs(a[..., l] - b[..., l]).max() / sc[l] for l in range(ext.n_var))


@pytest.mark.parametrize("integ", ["implicit", "plusgs"])
@pytest.mark.parametrize("turb", [False, True], ids=["laminar", "sst"])
def test_lusgs_single_block_matches_oracle(gpu_lib, turb, integ):
    kw = dict(nc=(19, 13, 6), ids=(-3, -4, -5, -4, -10, -10),
              scheme_kw=dict(interpolant="muscl", scheme_name="ausm", time_step_accuracy=integ),
              flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law", MInf=0.2))
    if turb:
        kw["turb"] = True
        kw["scheme_kw"] = dict(kw["scheme_kw"], scheme_name="ausmUP")
    ext, flow, scheme, bc, nodes, qp = small_case(**kw)
    wall = cases.wall_nodes_of(nodes, ext, bc) if turb else None
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp, wall=wall)
    h.step(3, 1, 200.0, with_norm=False)
    step = O.plusgs_next_solution if integ == "plusgs" else O.lusgs_next_solution
    for it in (1, 2, 3):
        assert step([blk], it, 200.0) == 0
    e = _err(h.download_state(), blk["qp"], ext)
    assert e <= 1e-11, f"LU-SGS interior state differs by {e:.3e}"
    assert np.abs(post.interior(blk["qp"], ext)[..., 4] - post.interior(qp, ext)[..., 4]).max() > 1.0
    h.close()


def _lfp(lib, integ="implicit"):
    fx = np.load(os.path.join(HERE, "golden", "flatplate_laminar.npz"))
    parts = MF.flatplate_case([fx["nodes0"], fx["nodes1"]])
    hs, blocks = [], []
    for ext, flow, scheme, bc, nodes, qp in parts:
        # the case's own integrator (Lfp/system/fvscheme.md: "implicit")
        scheme = abi.Scheme.from_buffer_copy(scheme)
        scheme.time_step_accuracy = abi.TIME[integ]
        h = Handle(ext, flow, scheme, bc, lib=lib)
        h.setup_geometry(nodes)
        h.upload_state(qp)
        hs.append(h)
        blk = O.Block(ext, flow, scheme, bc)
        blk["nodes"] = nodes
        blk.setup_geometry()
        blk["qp"] = qp
        blocks.append(blk)
    arr = (C.c_void_p * len(hs))(*[h.h.value for h in hs])
    b = C.c_void_p()
    abi.check(lib.fest_batch_create(arr, len(hs), C.byref(b)), "fest_batch_create")
    return hs, blocks, b


@pytest.mark.parametrize("integ", ["implicit", "plusgs"])
def test_lusgs_two_block_flat_plate_matches_oracle(gpu_lib, integ):
    hs, blocks, b = _lfp(gpu_lib, integ)
    step = O.plusgs_next_solution if integ == "plusgs" else O.lusgs_next_solution
    try:
        abi.check(gpu_lib.fest_batch_step(b, 3, 1, 2000.0), "fest_batch_step")
        for it in (1, 2, 3):
            assert step(blocks, it, 2000.0) == 0
        for n, (h, blk) in enumerate(zip(hs, blocks)):
            e = _err(h.download_state(), blk["qp"], h.ext, speed=MF.U_INF)
            assert e <= 1e-11, f"block {n}: LU-SGS state differs by {e:.3e}"
    finally:
        gpu_lib.fest_batch_destroy(b)
        for h in hs:
            h.close()


def drag_coefficient(h, length_span=0.05):
    """Lfp/pp/Surface.py on the wall (j = 1) faces of the plate block, from
    the gradients the handle holds from its last residual evaluation (the
    ones the reference's output carries) and the case's constant viscosity"""
    ext = h.ext
    gx, gy, gz = h.get("gradqp_x"), h.get("gradqp_y"), h.get("gradqp_z")
    c = (slice(1, ext.imx), 1, 1)
    dudx, dudy, dudz = gx[c + (0,)], gy[c + (0,)], gz[c + (0,)]
    dvdx, dvdy, dwdz = gx[c + (1,)], gy[c + (1,)], gz[c + (2,)]
    dwdx = gx[c + (2,)]
    delv = dudx + dvdy + dwdz
    m = MF.MU
    txx = m * (2.0 * dudx - 2.0 * delv / 3.0)
    txy = m * (dudy + dvdx)
    txz = m * (dudz + dwdx)
    Jf = h.get("Jfaces")[:, 3:ext.imx + 2, 3, 3]
    Fx = txx * Jf[1] + txy * Jf[2] + txz * Jf[3]
    q_inf = 0.5 * MF.RHO_INF * MF.U_INF ** 2
    return float(np.sum(Fx * Jf[0] / q_inf) / length_span)


# tests/Report.txt, laminar case: "Difference 5.001E-02 %" from the expected 1.330E-03
REFERENCE_RUN_CD = 1.330e-03 * (1.0 - 5.001e-4)


def test_reference_laminar_flat_plate_run_on_gpu(gpu_lib):
    hs, blocks, b = _lfp(gpu_lib)
    try:
        abi.check(gpu_lib.fest_batch_step(b, 5000, 1, 2000.0), "fest_batch_step")
        cd = drag_coefficient(hs[1])
        assert abs(cd - REFERENCE_RUN_CD) <= 3e-5 * REFERENCE_RUN_CD, (cd, REFERENCE_RUN_CD)
    finally:
        gpu_lib.fest_batch_destroy(b)
        for h in hs:
            h.close()
