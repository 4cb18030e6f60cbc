"""The fused stage sweep (fest_step) against the oracle's get_next_solution.

FP64: interior state after three iterations within 1e-11 of each variable's
magnitude (ghost layers of the returned state are those of the last BC
application, not the reference's blended copies; the next iteration's BCs
rewrite them, so only interior cells are compared).
FEST_MIXED: FP32 stencil arithmetic (ghost cells in FP32 from iteration 3 on)
with FP64 accumulation, inviscid and laminar viscous; the interior state
stays within 2e-5 of each variable's magnitude over six iterations."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from fest3d import abi, cases
from parity import assert_residual, make_pair, rel_err, small_case

pytestmark = pytest.mark.gpu

COMBOS = {
    "weno-slau": dict(scheme_kw=dict(interpolant="weno", scheme_name="slau"),
                      ids=(-11, -4, -6, -6, -10, -10)),
    "muscl-ausm": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausm"),
                       ids=(-5, -4, -6, -3, -10, -10)),
    "ppm-ausmP": dict(scheme_kw=dict(interpolant="ppm", scheme_name="ausmP", iPB_switch=1),
                      ids=(-3, -4, -5, -6, -6, -6)),
    "wenoNM-ausmUP": dict(scheme_kw=dict(interpolant="weno_NM", scheme_name="ausmUP"),
                          ids=(-8, -2, -6, -6, -10, -10), flow_kw=dict(MInf=0.3)),
    "none-vanleer": dict(scheme_kw=dict(interpolant="none", scheme_name="van_leer"),
                         ids=(-1, -4, -6, -6, -10, -10)),
    "muscl-ldfss-vanalbada": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ldfss0",
                                                 limiter="van_albada"),
                                  ids=(-3, -4, -6, -5, -10, -10)),
}


# laminar viscous terms: the FP32 sweep evaluates the temperature gradient
# from the current stage's state where the reference (and the FP64 sweep)
# uses the iteration's first
VISC_COMBOS = {
    "lam-muscl-ausm-cavity": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausm"),
                                  ids=(-5, -5, -5, -3, -10, -10),
                                  flow_kw=dict(mu_ref=5e-2, mu_variation="constant")),
    "suth-weno-slau": dict(scheme_kw=dict(interpolant="weno", scheme_name="slau"),
                           ids=(-3, -4, -5, -6, -10, -10),
                           flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law")),
    "suth-ppm-ausmP-slip": dict(scheme_kw=dict(interpolant="ppm", scheme_name="ausmP"),
                                ids=(-3, -4, -5, -6, -6, -6),
                                flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law")),
    "lam-none-vanleer": dict(scheme_kw=dict(interpolant="none", scheme_name="van_leer"),
                             ids=(-1, -4, -5, -6, -10, -10),
                             flow_kw=dict(mu_ref=5e-2, mu_variation="constant")),
}
# k-omega SST in the FP32 sweep: seven variables, eddy viscosity and F1 per
# cell, SST face, source and time-step terms, point-implicit destruction;
# wall distances from the -5 faces' nodes
SST_COMBOS = {
    "sst-muscl-ausmUP": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausmUP"),
                             ids=(-3, -4, -5, -4, -10, -10),
                             flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law", MInf=0.2)),
    "sst2003-weno-slau": dict(scheme_kw=dict(interpolant="weno", scheme_name="slau", turbulence="sst2003"),
                              ids=(-11, -4, -5, -6, -10, -10),
                              flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law")),
    "sst-ppm-ausmP-slip": dict(scheme_kw=dict(interpolant="ppm", scheme_name="ausmP"),
                               ids=(-3, -4, -5, -6, -6, -6),
                               flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law")),
    "sst-none-vanleer-farfield": dict(scheme_kw=dict(interpolant="none", scheme_name="van_leer"),
                                      ids=(-8, -4, -5, -6, -10, -10),
                                      flow_kw=dict(mu_ref=5e-2, mu_variation="constant")),
    "sst-wenoNM-ldfss-walls": dict(scheme_kw=dict(interpolant="weno_NM", scheme_name="ldfss0"),
                                   ids=(-5, -4, -5, -5, -10, -10),
                                   flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law")),
}
COMBOS_ALL = dict(COMBOS, **VISC_COMBOS)


def interior(q, ext):
    return q[3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2, :]


def run_pair(name, acc, precision, iters=3, nc=(37, 14, 5)):
    kw = dict(COMBOS_ALL[name])
    sk = dict(kw.pop("scheme_kw"))
    sk["time_step_accuracy"] = acc
    kw.setdefault("nc", nc)
    ext, flow, scheme, bc, nodes, qp = small_case(scheme_kw=sk, **kw)
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    h.set_precision(precision)
    norm = h.step(iters, 1, 0.5)
    for it in range(1, iters + 1):
        assert O.get_next_solution([blk], it, 0.5) == 0
    return ext, blk, h, h.download_state(), norm


@pytest.mark.parametrize("name", list(COMBOS))
@pytest.mark.parametrize("acc", ["none", "RK2", "RK4", "TVDRK2", "TVDRK3"])
def test_fused_fp64(gpu_lib, name, acc):
    ext, blk, h, q, norm = run_pair(name, acc, abi.FEST_FP64)
    e = rel_err(interior(q, ext), interior(blk["qp"], ext))
    assert e <= 1e-11, f"fused FP64 interior state differs by {e:.3e}"
    ref = O.find_resnorm([blk])
    assert np.allclose(norm, ref, rtol=1e-9, atol=1e-300), (norm, ref)


@pytest.mark.parametrize("name", list(COMBOS))
@pytest.mark.parametrize("acc", ["none", "TVDRK3", "RK4"])
def test_fused_mixed(gpu_lib, name, acc):
    ext, blk, h, q, norm = run_pair(name, acc, abi.FEST_MIXED, iters=6)
    e = rel_err(interior(q, ext), interior(blk["qp"], ext))
    assert e <= 2e-5, f"mixed interior state differs by {e:.3e}"
    ref = O.find_resnorm([blk])
    assert np.allclose(norm[1:], ref[1:], rtol=2e-2), (norm, ref)


@pytest.mark.parametrize("name", list(VISC_COMBOS))
@pytest.mark.parametrize("acc", ["none", "TVDRK3", "RK4"])
def test_fused_mixed_viscous(gpu_lib, name, acc):
    ext, blk, h, q, norm = run_pair(name, acc, abi.FEST_MIXED, iters=6)
    e = rel_err(interior(q, ext), interior(blk["qp"], ext))
    assert e <= 2e-5, f"mixed viscous interior state differs by {e:.3e}"


def run_sst_pair(name, acc, precision, iters=6, nc=(37, 14, 5), ids=None):
    kw = dict(SST_COMBOS[name])
    sk = dict(kw.pop("scheme_kw"))
    sk["time_step_accuracy"] = acc
    if ids is not None:
        kw["ids"] = ids
    ext, flow, scheme, bc, nodes, qp = small_case(scheme_kw=sk, turb=True, nc=nc, **kw)
    wall = cases.wall_nodes_of(nodes, ext, bc)
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp, wall=wall)
    h.set_precision(precision)
    norm = h.step(iters, 1, 0.5)
    for it in range(1, iters + 1):
        assert O.get_next_solution([blk], it, 0.5) == 0
    return ext, blk, h, h.download_state(), norm


@pytest.mark.parametrize("name", list(SST_COMBOS))
@pytest.mark.parametrize("acc", ["none", "TVDRK3", "RK4"])
def test_fused_mixed_sst(gpu_lib, name, acc):
    ext, blk, h, q, norm = run_sst_pair(name, acc, abi.FEST_MIXED)
    e = rel_err(interior(q, ext), interior(blk["qp"], ext))
    assert e <= 2e-5, f"mixed SST interior state differs by {e:.3e}"
    ref = O.find_resnorm([blk])
    assert np.allclose(norm[1:], ref[1:], rtol=2e-2), (norm, ref)


def test_fused_mixed_sst_single_plane(gpu_lib):
    """a flat-plate-like single-plane block (kmx = 2, slip k faces): the
    mixed sweep reads ghost layer 1 only, and makes the symmetric faces'
    ghosts in the reference's face order"""
    ext, blk, h, q, norm = run_sst_pair("sst-muscl-ausmUP", "RK4", abi.FEST_MIXED, nc=(40, 9, 1),
                                        ids=(-3, -4, -5, -4, -6, -6))
    e = rel_err(interior(q, ext), interior(blk["qp"], ext))
    assert e <= 2e-5, f"mixed SST single-plane interior state differs by {e:.3e}"


@pytest.mark.parametrize("name", list(VISC_COMBOS))
@pytest.mark.parametrize("acc", ["none", "TVDRK3", "RK4"])
def test_fused_fp64_viscous(gpu_lib, name, acc):
    """FP64 laminar blocks in the fused sweep: the gradients take the
    temperature of the iteration's start, as the reference's do"""
    ext, blk, h, q, norm = run_pair(name, acc, abi.FEST_FP64, iters=3)
    e = rel_err(interior(q, ext), interior(blk["qp"], ext))
    assert e <= 1e-11, f"fused FP64 viscous interior state differs by {e:.3e}"
    assert_residual(h.get("residue"), blk, rtol=1e-12, what="fused FP64 viscous residual")
    ref = O.find_resnorm([blk])
    assert np.allclose(norm, ref, rtol=1e-9, atol=1e-300), (norm, ref)


@pytest.mark.parametrize("name", list(SST_COMBOS))
@pytest.mark.parametrize("acc", ["none", "TVDRK3", "RK4"])
def test_fused_fp64_sst(gpu_lib, name, acc):
    """FP64 k-omega SST blocks in the fused sweep"""
    ext, blk, h, q, norm = run_sst_pair(name, acc, abi.FEST_FP64, iters=3)
    e = rel_err(interior(q, ext), interior(blk["qp"], ext))
    assert e <= 1e-11, f"fused FP64 SST interior state differs by {e:.3e}"
    assert_residual(h.get("residue"), blk, rtol=1e-12, what="fused FP64 SST residual")


@pytest.mark.parametrize("nc,ids,acc,mixed_runs", [((40, 9, 1), (-3, -4, -6, -5, -6, -6), "RK4", True),
                                                   ((40, 9, 1), (-3, -4, -6, -5, -6, -6), "TVDRK3", False),
                                                   ((37, 14, 5), (-1, -4, -6, -6, -9, -9), "TVDRK3", False)])
def test_in_place_cases_use_module_path(gpu_lib, nc, ids, acc, mixed_runs):
    """thin blocks and -9 faces read other faces' ghosts: FP64 fest_step
    runs the in-place module path (exact).  FEST_MIXED runs the thin block
    with the reference's face order (its interior updates read ghost layer
    1 only, the symmetric faces the opposite face's layer 1) unless a TVD
    integrator blends those ghosts between fills; it refuses -9."""
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=nc, ids=ids, scheme_kw=dict(interpolant="muscl", scheme_name="ausm",
                                       time_step_accuracy=acc))
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    h.step(3, 1, 0.5)
    for it in (1, 2, 3):
        assert O.get_next_solution([blk], it, 0.5) == 0
    assert rel_err(h.download_state(), blk["qp"]) <= 1e-11
    h.set_precision(abi.FEST_MIXED)
    if mixed_runs:
        h.step(3, 4, 0.5)
        for it in (4, 5, 6):
            assert O.get_next_solution([blk], it, 0.5) == 0
        assert rel_err(interior(h.download_state(), ext), interior(blk["qp"], ext)) <= 2e-5
    else:
        with pytest.raises(abi.FestError):
            h.step(1, 4, 0.5)


def test_fused_state_roundtrip_and_module_interplay(gpu_lib):
    """after fused steps the module entry points see the fused state."""
    ext, blk, h, q, norm = run_pair("weno-slau", "TVDRK3", abi.FEST_FP64, iters=2)
    q2 = h.get_next_solution(q, 3, 0.5)  # module path continues from the fused state
    assert O.get_next_solution([blk], 3, 0.5) == 0
    assert rel_err(interior(q2, ext), interior(blk["qp"], ext)) <= 1e-11


def test_profile_counts_stage_launches(gpu_lib):
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(37, 14, 5), scheme_kw=dict(interpolant="weno", scheme_name="slau",
                                       time_step_accuracy="TVDRK3"),
        ids=(-11, -4, -6, -6, -10, -10))
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    h.set_precision(abi.FEST_MIXED)
    L = h.lib
    abi.check(L.fest_profile(h.h, 1), "profile")
    h.step(4, 1, 0.5, with_norm=False)
    n = C.c_longlong()
    ms = C.c_double()
    abi.check(L.fest_profile_read(h.h, C.byref(n), C.byref(ms)), "profile_read")
    assert n.value == 12 and ms.value > 0


def test_mixed_block_with_many_rows(gpu_lib):
    """a block whose padded rows (j, k, variable) outnumber 65535: the FP32
    mirror's conversion covers every row"""
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(16, 200, 64), ids=(-3, -4, -6, -6, -10, -10),
        scheme_kw=dict(interpolant="muscl", scheme_name="ausm", time_step_accuracy="TVDRK3"))
    assert (ext.jmx + 5) * (ext.kmx + 5) * ext.n_var > 65535
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    h.set_precision(abi.FEST_MIXED)
    h.step(3, 1, 0.5, with_norm=False)
    for it in (1, 2, 3):
        assert O.get_next_solution([blk], it, 0.5) == 0
    e = rel_err(interior(h.download_state(), ext), interior(blk["qp"], ext))
    assert e <= 2e-5, f"mixed interior state differs by {e:.3e}"


@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
@pytest.mark.parametrize("precision", [abi.FEST_FP64, abi.FEST_MIXED], ids=["fp64", "mixed"])
def test_step_host_equals_upload_step_download(gpu_lib, precision, pinned):
    """fest_step_host (one synchronisation) leaves in the caller's array the
    state that upload + fest_step + download leave, bit for bit, and the
    same norm; pinned host memory moves through the host-link copy kernel
    (the bump block's state is above its 1 MiB threshold)."""
    import torch
    case = cases.bump_case(nc=(64, 24, 4))
    ext = case["ext"]
    _, h1 = make_pair(ext, case["flow"], case["scheme"], case["bc"], case["nodes"], case["qp"])
    _, h2 = make_pair(ext, case["flow"], case["scheme"], case["bc"], case["nodes"], case["qp"])
    for h in (h1, h2):
        h.set_precision(precision)
    if pinned:
        buf = torch.empty(abi.shapes(ext)["qp"][::-1], dtype=torch.float64, pin_memory=True)
        q = buf.numpy().T
    else:
        q = np.zeros(abi.shapes(ext)["qp"], order="F")
    q[...] = case["qp"]
    it = 1
    for _ in range(3):
        n2 = h2.step_host(q, 2, it, case["CFL"])
        h1.upload_state(h1.download_state())  # the same invalidation as an upload
        n1 = h1.step(2, it, case["CFL"])
        it += 2
        ref = h1.download_state()
        assert np.array_equal(q, ref)
        assert np.allclose(n1, n2, rtol=1e-13, atol=0)
    h1.close()
    h2.close()


@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
def test_step_host_interior_equals_device_steps(gpu_lib, pinned):
    """fest_step_host_interior on the interior cells (ghost cells kept on
    the device) leaves the interior that fest_step leaves, bit for bit,
    over calls that start in iterations 1-2 (fix() ghosts) and after: once
    the fused path holds a state, a call writes the interior into its
    current buffer and FP32 mirror in place (the values the mirror already
    holds, when the host array is unchanged), so the sweeps continue as if
    no call had been made."""
    import torch
    case = cases.bump_case(nc=(64, 24, 4))
    ext = case["ext"]
    _, h1 = make_pair(ext, case["flow"], case["scheme"], case["bc"], case["nodes"], case["qp"])
    _, h2 = make_pair(ext, case["flow"], case["scheme"], case["bc"], case["nodes"], case["qp"])
    for h in (h1, h2):
        h.set_precision(abi.FEST_MIXED)
    shape = (ext.imx - 1, ext.jmx - 1, ext.kmx - 1, ext.n_var)
    if pinned:
        buf = torch.empty(shape[::-1], dtype=torch.float64, pin_memory=True)
        q = buf.numpy().T
    else:
        q = np.zeros(shape, order="F")
    sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
    q[...] = case["qp"][sl]
    it = 1
    for n in (1, 2, 3):
        n2 = h2.step_host_interior(q, n, it, case["CFL"])
        n1 = h1.step(n, it, case["CFL"])
        it += n
        assert np.array_equal(q, h1.download_state()[sl])
        assert np.allclose(n1, n2, rtol=1e-13, atol=0)
    h1.close()
    h2.close()


@pytest.mark.parametrize("precision", [abi.FEST_FP64, abi.FEST_MIXED], ids=["fp64", "mixed"])
def test_checkpoint_snapshots_while_stepping(gpu_lib, precision):
    """Handle.iterate with the reference's checkpoint schedule (every third
    iteration and the last): each snapshot, copied into pinned memory while
    the next iterations are already enqueued, is bit for bit the state that
    synchronous steps and fest_download_state give at that iteration, and
    stepping after the snapshots continues unchanged; one snapshot at a
    time."""
    import torch
    case = cases.bump_case(nc=(64, 24, 4))
    ext = case["ext"]
    _, h1 = make_pair(ext, case["flow"], case["scheme"], case["bc"], case["nodes"], case["qp"])
    _, h2 = make_pair(ext, case["flow"], case["scheme"], case["bc"], case["nodes"], case["qp"])
    for h in (h1, h2):
        h.set_precision(precision)
    buf = torch.empty(abi.shapes(ext)["qp"][::-1], dtype=torch.float64, pin_memory=True)
    q = buf.numpy().T
    got = []
    nxt = h1.iterate(7, case["CFL"], 3, lambda it, qp: got.append((it, qp.copy(order="F"))), q=q)
    assert nxt == 8 and [it for it, _ in got] == [3, 6, 7]
    it = 1
    for d, snap in got:
        h2.step(d - it + 1, it, case["CFL"], with_norm=False)
        it = d + 1
        assert np.array_equal(snap, h2.download_state()), d
    h1.step(2, 8, case["CFL"], with_norm=False)
    h2.step(2, 8, case["CFL"], with_norm=False)
    assert np.array_equal(h1.download_state(), h2.download_state())
    h1.snapshot_begin(q)
    with pytest.raises(abi.FestError):
        h1.snapshot_begin(q)
    h1.snapshot_wait()
    assert np.array_equal(q, h2.download_state())
    h1.close()
    h2.close()
