"""The Spalart-Allmaras model (FEST_TURB_SA, six variables) on the GPU
against the oracle's restatement (tests/test_sa_cpu.py checks the oracle's
SA terms against a second restatement):

* module by module, as the reference calls them: gradients with tv
  (gradients.f90:165-169), the eddy viscosity and its ghost copies
  (viscosity.f90:149-213), the laminar terms with mu_t and the tv diffusion
  (viscous.f90:570-656), the residue with the SA source
  (source.f90:845-983), the local time step with the turbulent term;
* whole iterations of get_next_solution (update.f90:129-226) with the
  point-implicit destruction and the tv floor (update.f90:405-419,
  474-475), through fest_get_next_solution and through fest_step, and the
  residual norm with tv_inf's scale;
* what is refused: the mixed sweep and the implicit integrators for SA."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from fest3d import abi, cases
from parity import assert_close, assert_residual, make_pair, small_case

pytestmark = pytest.mark.gpu

FLOW = dict(mu_ref=2e-2, mu_variation="sutherland_law", tv_inf=1.2e-4)


def sa_pair(nc=(8, 6, 5), ids=(-3, -4, -5, -6, -10, -10), **kw):
    ext, flow, scheme, bc, nodes, qp = small_case(nc=nc, ids=ids, turb="sa", flow_kw=FLOW,
                                                  fixed={"fixed_wall_temperature": [0] * 6}, **kw)
    wall = cases.wall_nodes_of(nodes, ext, bc)
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp, wall=wall)
    return ext, flow, scheme, bc, blk, h


@pytest.mark.parametrize("thin", [False, True])
def test_sa_modules(gpu_lib, thin):
    nc = (8, 6, 1) if thin else (8, 6, 5)
    ids = (-3, -4, -5, -4, -6, -6) if thin else (-3, -4, -5, -6, -10, -10)
    ext, flow, scheme, bc, blk, h = sa_pair(nc=nc, ids=ids)
    assert ext.n_var == 6 and blk.n_grad == 5
    blk.compute_temperature()
    O.apply_interface([blk])
    blk.populate_ghost_primitive(1)
    blk.compute_face_interpolant()
    blk.reconstruct_boundary_state()
    blk.compute_fluxes()
    q = np.asfortranarray(blk["qp"].copy())
    T = np.asfortranarray(blk["Temp"].copy())
    g = [np.zeros(abi.shapes(ext, 5)["grad"], order="F") for _ in range(3)]
    abi.check(h.lib.fest_evaluate_all_gradients(h.h, abi.ptr(q), abi.ptr(T), *[abi.ptr(a) for a in g]),
              "gradients")
    assert blk.evaluate_all_gradients() == 0
    for c, a in enumerate(g):
        assert_close(a, blk["gradqp_" + "xyz"[c]], 1e-11, "gradqp_" + "xyz"[c])
    mu, mut, F1 = (np.zeros(abi.shapes(ext)["pad"], order="F") for _ in range(3))
    abi.check(h.lib.fest_calculate_viscosity(h.h, abi.ptr(q), abi.ptr(mu), abi.ptr(mut), abi.ptr(F1)),
              "viscosity")
    assert blk.calculate_viscosity() == 0
    assert_close(mu, blk["mu"], 1e-12, "mu")
    assert_close(mut, blk["mu_t"], 1e-11, "mu_t")
    F, G, H = (np.asfortranarray(blk[n].copy()) for n in ("F", "G", "H"))
    abi.check(h.lib.fest_compute_viscous_fluxes(h.h, abi.ptr(q), abi.ptr(F), abi.ptr(G), abi.ptr(H)),
              "viscous")
    assert blk.compute_viscous_fluxes() == 0
    for a, n in ((F, "F"), (G, "G"), (H, "H")):
        assert_close(a, blk[n], 1e-11, n + " viscous")
    res = np.zeros(abi.shapes(ext)["residue"], order="F")
    abi.check(h.lib.fest_compute_residue(h.h, abi.ptr(F), abi.ptr(G), abi.ptr(H), abi.ptr(res)),
              "residue")
    blk.compute_residue()
    assert_residual(res, blk)
    abi.check(h.lib.fest_add_source_term_residue(h.h, abi.ptr(q), abi.ptr(res)), "source")
    blk.add_source_term_residue()
    assert_close(res, blk["residue"], 1e-10, "residue + SA source")
    assert np.abs(res[..., 5]).max() > 0.0
    dt = np.zeros(abi.shapes(ext)["delta_t"], order="F")
    for n in ("x_qp_left", "x_qp_right", "y_qp_left", "y_qp_right", "z_qp_left", "z_qp_right"):
        h.set(n, blk[n])
    abi.check(h.lib.fest_compute_time_step(h.h, abi.ptr(q), 0.7, abi.ptr(dt)), "time step")
    blk.compute_time_step(0.7)
    assert_close(dt, blk["delta_t"], 1e-12, "delta_t")
    h.close()


@pytest.mark.parametrize("acc", ["none", "RK4", "TVDRK3"])
@pytest.mark.parametrize("case", ["muscl-ausm-walls", "weno-slau-farfield"])
def test_sa_next_solution(gpu_lib, acc, case):
    kw = dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausm", time_step_accuracy=acc),
              ids=(-3, -4, -5, -6, -10, -10))
    if case == "weno-slau-farfield":
        kw = dict(scheme_kw=dict(interpolant="weno", scheme_name="slau", time_step_accuracy=acc),
                  ids=(-8, -2, -5, -6, -10, -10))
    ext, flow, scheme, bc, blk, h = sa_pair(**kw)
    q = blk["qp"].copy(order="F")
    for it in (1, 2, 3):
        q = h.get_next_solution(q, it, 0.5)
        assert O.get_next_solution([blk], it, 0.5) == 0
        assert_close(q, blk["qp"], 1e-11, f"qp after iteration {it}")
    assert_residual(h.get("residue"), blk, 1e-10, "last-stage residue")
    assert np.allclose(h.resnorm(), O.find_resnorm([blk]), rtol=1e-10, atol=0)
    h.close()


def test_sa_step_and_refusals(gpu_lib):
    """fest_step (the module path for SA blocks) over five iterations
    matches the oracle's; FEST_MIXED steps are refused (the fused sweep has
    no SA variant), and so are SA blocks with the implicit integrators."""
    ext, flow, scheme, bc, blk, h = sa_pair(scheme_kw=dict(time_step_accuracy="RK4"))
    norm = h.step(5, 1, 0.5)
    for it in range(1, 6):
        assert O.get_next_solution([blk], it, 0.5) == 0
    assert_close(h.download_state(), blk["qp"], 1e-11, "qp after five steps")
    assert np.allclose(norm, O.find_resnorm([blk]), rtol=1e-10, atol=0)
    h.set_precision(abi.FEST_MIXED)
    with pytest.raises(abi.FestError) as e:
        h.step(1, 6, 0.5)
    assert e.value.code == abi.FEST_ERR_ARG
    h.close()
    for integ in ("implicit", "plusgs"):
        s2 = abi.Scheme.from_buffer_copy(scheme)
        s2.time_step_accuracy = abi.TIME[integ]
        hh = C.c_void_p()
        assert gpu_lib.fest_create(C.byref(ext), C.byref(flow), C.byref(s2), C.byref(bc),
                                   C.byref(hh)) == abi.FEST_ERR_ARG
