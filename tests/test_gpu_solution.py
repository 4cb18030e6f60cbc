"""Whole-iteration parity: get_total_conservative_Residue and
get_next_solution of every explicit integrator (update.f90:129-226), plus
find_resnorm (resnorm.f90:62) and the reference's abort conditions."""
import numpy as np
import pytest

import oracle as O
from fest3d import abi, cases
from parity import assert_close, assert_residual, make_pair, small_case

pytestmark = pytest.mark.gpu

PHYSICS = {
    "euler-weno-slau": dict(scheme_kw=dict(interpolant="weno", scheme_name="slau"),
                            ids=(-11, -4, -6, -6, -10, -10)),
    "laminar-muscl-ausm": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausm"),
                               ids=(-5, -5, -5, -3, -10, -10),
                               flow_kw=dict(mu_ref=5e-2, mu_variation="constant")),
    "sutherland-ppm-ausmP": dict(scheme_kw=dict(interpolant="ppm", scheme_name="ausmP"),
                                 ids=(-3, -4, -5, -6, -10, -10),
                                 flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law")),
    "sst-muscl-ausmUP": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausmUP"),
                             ids=(-3, -4, -5, -4, -10, -10), turb=True,
                             flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law", MInf=0.2)),
    "euler-wenoNM-ldfss": dict(scheme_kw=dict(interpolant="weno_NM", scheme_name="ldfss0"),
                               ids=(-8, -2, -6, -6, -9, -9)),
    "euler-none-vanleer": dict(scheme_kw=dict(interpolant="none", scheme_name="van_leer"),
                               ids=(-1, -4, -6, -6, -10, -10)),
}


def build(name, **extra):
    kw = dict(PHYSICS[name])
    kw.update(extra)
    ext, flow, scheme, bc, nodes, qp = small_case(**kw)
    wall = cases.wall_nodes_of(nodes, ext, bc) if ext.n_var == 7 else None
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp, wall=wall)
    return ext, blk, h


@pytest.mark.parametrize("name", list(PHYSICS))
def test_total_residual(gpu_lib, name):
    """get_total_conservative_Residue (update.f90:495-547), flux-scaled."""
    ext, blk, h = build(name)
    blk.compute_temperature()
    h.set("Temp", blk["Temp"])
    q, res = h.residual(blk["qp"].copy(order="F"), 1)
    assert O.get_total_conservative_residue([blk], 1) == 0
    assert_close(q, blk["qp"], 1e-13, "qp ghosts")
    assert_residual(res, blk)


@pytest.mark.parametrize("name", list(PHYSICS))
@pytest.mark.parametrize("acc", ["none", "RK2", "RK4", "TVDRK2", "TVDRK3"])
def test_next_solution(gpu_lib, name, acc):
    """three iterations of get_next_solution; the state (ghosts included)
    follows the oracle to 1e-11 of each variable's magnitude."""
    sk = dict(PHYSICS[name]["scheme_kw"])
    sk["time_step_accuracy"] = acc
    ext, blk, h = build(name, scheme_kw=sk)
    q = blk["qp"].copy(order="F")
    for it in (1, 2, 3):
        q = h.get_next_solution(q, it, 0.5)
        assert O.get_next_solution([blk], it, 0.5) == 0
        assert_close(q, blk["qp"], 1e-11, f"qp after iteration {it}")
    res = h.get("residue")
    assert_residual(res, blk, 1e-10, "last-stage residue")
    norm = h.resnorm()
    ref = O.find_resnorm([blk])
    assert np.allclose(norm, ref, rtol=1e-10, atol=0), (norm, ref)


def test_negative_state_is_reported(gpu_lib):
    """update.f90:448: rho or p < 0 after an update aborts the reference; the
    ABI returns FEST_ERR_NEGATIVE_STATE.  Injected on the host with an
    over-large CFL (the oracle reports the same); no device fault."""
    ext, blk, h = build("euler-none-vanleer")
    q = blk["qp"].copy(order="F")
    assert O.get_next_solution([blk], 1, 200.0) == abi.FEST_ERR_NEGATIVE_STATE
    with pytest.raises(abi.FestError) as e:
        h.get_next_solution(q, 1, 200.0)
    assert e.value.code == abi.FEST_ERR_NEGATIVE_STATE
    # the handle stays usable afterwards
    ext, blk, h2 = build("euler-none-vanleer")
    q2 = h.get_next_solution(blk["qp"].copy(order="F"), 1, 0.5)
    assert np.all(np.isfinite(q2))


def test_nan_state_is_reported(gpu_lib):
    """ausm.f90:195: a NaN flux aborts the reference; here FEST_ERR_NAN."""
    ext, blk, h = build("laminar-muscl-ausm")
    q = blk["qp"].copy(order="F")
    q[5, 5, 4, 1] = np.nan
    with pytest.raises(abi.FestError) as e:
        h.get_next_solution(q, 1, 0.5)
    assert e.value.code in (abi.FEST_ERR_NAN, abi.FEST_ERR_NEGATIVE_STATE)
