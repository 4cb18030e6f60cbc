"""Parity at the benchmark configurations' own sizes, on the GPU, against the
oracle on the same inputs.

* Smooth bump, 256x96x4 cells, WENO5 + SLAU, TVD-RK3, CFL 0.8 (the workload
  bench.py times, built by the same function): FP64 through the fused sweep,
  three iterations, residual of the last stage within 1e-12 flux-scaled
  (and in global L2) and the interior state within 1e-11 of each variable's
  magnitude (the free-stream speed for the velocity components); mixed
  precision, twenty iterations, interior state within 5e-5 (measured 2.2e-5
  on v: in FP32 the WENO weights respond to the rounding of the pressure
  differences of nearly uniform regions, about 0.01 Pa at 1e5 Pa, an effect
  that grows with the iteration count from the uniform start).
* Lid-driven cavity, 64x64x4 cells, MUSCL (van Albada) + AUSM, laminar,
  forward Euler, CFL 0.5: all 2000 iterations of the configuration,
  field-wise (every interior cell, every variable) against the oracle's
  2000 iterations, FP64 within 1e-9 and mixed precision within 2e-5 of
  each variable's magnitude.  The cavity starts at rest, so its velocities
  are judged against the lid speed.
* Turbulent flat plate with k-omega SST, 192x128x2 cells as two blocks (the
  0.33 m symmetry run-in and the 2 m plate, joined by an interface, the
  reference's own Tfp layout), first cell 1e-6 m: both blocks in one batch,
  FP64 within 1e-11 after three RK4 iterations and mixed precision within
  2e-5 after six, against the oracle's two-block run."""
import numpy as np
import pytest

import oracle as O
from fest3d import abi, cases, post
from parity import assert_residual, make_pair

pytestmark = pytest.mark.gpu


def _oracle_run(blk, first, n, CFL):
    for it in range(first, first + n):
        assert O.get_next_solution([blk], it, CFL) == 0


def _field_err(q, ref, ext, scale=None):
    """max over variables of max|q - ref| / scale_l over interior cells
    (scale_l: max|ref_l| unless given)."""
    a, b = post.interior(q, ext), post.interior(ref, ext)
    errs = []
    for l in range(ext.n_var):
        s = scale[l] if scale is not None else np.abs(b[..., l]).max()
        errs.append(np.abs(a[..., l] - b[..., l]).max() / s)
    return max(errs), errs


def _bump_scale(case, ref):
    """per-variable scales: density and pressure magnitudes, the free-stream
    speed for the velocity components (w stays ~0 in the extruded bump)"""
    ext, flow = case["ext"], case["flow"]
    r = post.interior(ref, ext)
    V = flow.vel_mag
    return [np.abs(r[..., 0]).max(), V, V, V, np.abs(r[..., 4]).max()]


def test_bump_256x96x4_fp64_residual_and_state(gpu_lib):
    case = cases.bump_case()
    ext = case["ext"]
    blk, h = make_pair(ext, case["flow"], case["scheme"], case["bc"], case["nodes"], case["qp"])
    h.set_precision(abi.FEST_FP64)
    h.step(3, 1, case["CFL"])
    q = h.download_state()
    res = h.get("residue")  # the last stage's residual, kept by the fused sweep
    _oracle_run(blk, 1, 3, case["CFL"])
    assert_residual(res, blk, rtol=1e-12, what="bump 256x96x4 FP64 residual, iteration 3 stage 3")
    e, errs = _field_err(q, blk["qp"], ext, _bump_scale(case, blk["qp"]))
    assert e <= 1e-11, f"bump FP64 interior state after 3 iterations differs by {errs}"
    h.close()


def test_bump_256x96x4_mixed_twenty_iterations(gpu_lib):
    case = cases.bump_case()
    ext = case["ext"]
    blk, h = make_pair(ext, case["flow"], case["scheme"], case["bc"], case["nodes"], case["qp"])
    h.set_precision(abi.FEST_MIXED)
    norm = h.step(20, 1, case["CFL"])
    q = h.download_state()
    _oracle_run(blk, 1, 20, case["CFL"])
    # the flow has left the uniform start: compare the departure from it too
    dep = np.abs(post.interior(blk["qp"], ext)[..., 4] - case["flow"].pressure_inf).max()
    assert dep > 10.0, dep
    e, errs = _field_err(q, blk["qp"], ext, _bump_scale(case, blk["qp"]))
    assert e <= 5e-5, f"bump mixed interior state after 20 iterations differs by {errs}"
    ref = O.find_resnorm([blk])
    assert np.allclose(norm[1:], ref[1:], rtol=2e-2), (norm, ref)
    h.close()


@pytest.mark.parametrize("precision", [abi.FEST_FP64, abi.FEST_MIXED], ids=["fp64", "mixed"])
def test_cavity_64x64x4_all_2000_iterations(gpu_lib, precision):
    case = cases.ldc_case()
    ext = case["ext"]
    iters = 2000
    blk, h = make_pair(ext, case["flow"], case["scheme"], case["bc"], case["nodes"], case["qp"])
    h.set_precision(precision)
    h.step(iters, 1, case["CFL"], with_norm=False)
    q = h.download_state()
    _oracle_run(blk, 1, iters, case["CFL"])
    ref = blk["qp"]
    lid = 34.7
    rho_s, p_s = np.abs(post.interior(ref, ext)[..., 0]).max(), np.abs(post.interior(ref, ext)[..., 4]).max()
    scale = [rho_s, lid, lid, lid, p_s]
    # the lid has set the cavity in motion
    assert np.abs(post.interior(ref, ext)[..., 1]).max() > 0.05 * lid
    tol = 1e-9 if precision == abi.FEST_FP64 else 2e-5
    e, errs = _field_err(q, ref, ext, scale)
    assert e <= tol, f"cavity after {iters} iterations differs by {errs} (tolerance {tol})"
    h.close()


def _plate_handles(lib, case, precision):
    from fest3d.handle import Handle
    hs = []
    for b in case["blocks"]:
        h = Handle(b["ext"], b["flow"], b["scheme"], b["bc"], lib=lib)
        h.setup_geometry(b["nodes"])
        h.find_wall_dist(case["wall"])
        h.upload_state(b["qp"])
        h.set_precision(precision)
        hs.append(h)
    return hs


@pytest.mark.parametrize("precision", [abi.FEST_FP64, abi.FEST_MIXED], ids=["fp64", "mixed"])
def test_sst_plate_two_blocks_192x128x2(gpu_lib, precision):
    import ctypes as C
    case = cases.plate_case()
    iters = 3 if precision == abi.FEST_FP64 else 6
    tol = 1e-11 if precision == abi.FEST_FP64 else 2e-5
    hs = _plate_handles(gpu_lib, case, precision)
    arr = (C.c_void_p * 2)(*[h.h.value for h in hs])
    b = C.c_void_p()
    abi.check(gpu_lib.fest_batch_create(arr, 2, C.byref(b)), "fest_batch_create")
    try:
        abi.check(gpu_lib.fest_batch_step(b, iters, 1, case["CFL"]), "fest_batch_step")
        blks = []
        for blk in case["blocks"]:
            o = O.Block(blk["ext"], blk["flow"], blk["scheme"], blk["bc"])
            o["nodes"] = blk["nodes"]
            o.setup_geometry()
            o.find_wall_dist(case["wall"])
            o["qp"] = blk["qp"]
            blks.append(o)
        _oracle_run_blocks(blks, iters, case["CFL"])
        flow = case["flow"]
        for n, (h, o) in enumerate(zip(hs, blks)):
            ext = h.ext
            ref = post.interior(o["qp"], ext)
            V = flow.vel_mag
            scale = [np.abs(ref[..., 0]).max(), V, V, V, np.abs(ref[..., 4]).max(),
                     np.abs(ref[..., 5]).max(), np.abs(ref[..., 6]).max()]
            e, errs = _field_err(h.download_state(), o["qp"], ext, scale)
            assert e <= tol, f"plate block {n} after {iters} iterations differs by {errs}"
    finally:
        gpu_lib.fest_batch_destroy(b)
        for h in hs:
            h.close()


def _oracle_run_blocks(blocks, n, CFL):
    for it in range(1, n + 1):
        assert O.get_next_solution(blocks, it, CFL) == 0
