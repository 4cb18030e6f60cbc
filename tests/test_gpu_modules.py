"""Module-by-module parity of the CUDA path (through the C ABI) against the
oracle, on small seeded blocks.  Each test names the reference procedure it
covers."""
import numpy as np
import pytest

import oracle as O
from fest3d import abi, cases
from fest3d.handle import Handle
from parity import (assert_close, assert_residual, face_slice, make_pair, small_case)

pytestmark = pytest.mark.gpu


def test_geometry(gpu_lib):
    """ghost_grid (grid.f90:137-236) + setup_geometry (geometry.f90:548-580)."""
    ext, flow, scheme, bc, nodes, qp = small_case()
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    assert_close(h.setup_geometry(nodes), blk["nodes"], 1e-15, "nodes")
    for name in ("cells", "Ifaces", "Jfaces", "Kfaces"):
        g, r = h.get(name), blk[name]
        for c in range(4):
            assert_close(g[c], r[c], 1e-13, f"{name}[{c}]")


BC_SETS = [
    ("ldc", (-5, -5, -5, -3, -10, -10), {}),
    ("bump", (-11, -4, -6, -6, -10, -10), {}),
    ("mixed", (-1, -2, -7, -4, -6, -5), {"fixed_wall_temperature": [0, 0, 0, 0, 0, 350.0]}),
    ("walls", (-5, -5, -6, -5, -10, -10), {"fixed_wall_temperature": [-1.0, 320.0, 0, 0.5, 0, 0]}),
    ("farfield", (-8, -4, -6, -6, -10, -10), {}),
    ("periodic", (-9, -9, -5, -6, -10, -10), {}),
    ("two_riemann", (-11, -8, -6, -6, -10, -10), {}),
]


@pytest.mark.parametrize("name,ids,fixed", BC_SETS, ids=[b[0] for b in BC_SETS])
@pytest.mark.parametrize("it", [1, 5])
def test_ghost_cells(gpu_lib, name, ids, fixed, it):
    """apply_interface + populate_ghost_primitive (bc_primitive.f90:55-226)."""
    ext, flow, scheme, bc, nodes, qp = small_case(ids=ids, fixed=fixed)
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    q = h.populate_ghost_primitive(qp, it)
    O.apply_interface([blk])
    blk.populate_ghost_primitive(it)
    assert_close(q, blk["qp"], 1e-13, f"qp after BCs ({name})")


@pytest.mark.parametrize("thin", [False, True])
def test_ghost_cells_sst(gpu_lib, thin):
    """SST ghosts incl. set_omega_at_wall (bc_primitive.f90:564-643); a thin
    block (kmx=2) runs the faces in the reference's order."""
    nc = (8, 6, 1) if thin else (8, 6, 5)
    ids = (-3, -4, -5, -4, -6, -6) if thin else (-3, -11, -5, -4, -10, -10)
    ext, flow, scheme, bc, nodes, qp = small_case(nc=nc, ids=ids, turb=True,
                                                  flow_kw=dict(mu_ref=1.8e-5, mu_variation="sutherland_law"))
    wall = cases.wall_nodes_of(nodes, ext, bc)
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp, wall=wall)
    assert_close(h.get("dist"), blk["dist"], 1e-13, "wall distance")
    q = h.populate_ghost_primitive(qp, 1)
    O.apply_interface([blk])
    blk.populate_ghost_primitive(1)
    assert_close(q, blk["qp"], 1e-13, "qp after SST BCs")


INTERPS = [("none", {}), ("muscl", {}), ("muscl", {"limiter": "van_albada"}),
           ("muscl", {"iPB_switch": 1, "jPB_switch": 1, "kPB_switch": 1}),
           ("muscl", {"ilimiter_switch": 0, "jlimiter_switch": 0, "klimiter_switch": 0}),
           ("ppm", {}), ("ppm", {"iPB_switch": 1}), ("weno", {}), ("weno_NM", {})]


@pytest.mark.parametrize("interp,kw", INTERPS, ids=[f"{a}-{i}" for i, (a, _) in enumerate(INTERPS)])
@pytest.mark.parametrize("ids", [(-5, -8, -6, -3, -10, -10), (-9, -9, -7, -4, -5, -6)])
def test_face_states(gpu_lib, interp, kw, ids):
    """compute_face_interpolant (face_interpolant.f90:79) then
    reconstruct_boundary_state (boundary_state_reconstruction.f90:28)."""
    sk = dict(interpolant=interp)
    sk.update(kw)
    ext, flow, scheme, bc, nodes, qp = small_case(ids=ids, scheme_kw=sk)
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    q = h.populate_ghost_primitive(qp, 3)
    O.apply_interface([blk])
    blk.populate_ghost_primitive(3)
    names = ("x_qp_left", "x_qp_right", "y_qp_left", "y_qp_right", "z_qp_left", "z_qp_right")
    outs = [np.zeros(abi.shapes(ext)[n[0] + "_qp"], order="F") for n in names]
    abi.check(h.lib.fest_compute_face_interpolant(h.h, abi.ptr(q), *[abi.ptr(a) for a in outs]),
              "face_interpolant")
    blk.compute_face_interpolant()
    for n, a in zip(names, outs):
        d = "xyz".index(n[0])
        assert_close(a[face_slice(ext, d)], blk[n][face_slice(ext, d)], 1e-13, n)
    abi.check(h.lib.fest_reconstruct_boundary_state(h.h, abi.ptr(q), *[abi.ptr(a) for a in outs]),
              "boundary_state")
    blk.reconstruct_boundary_state()
    for n, a in zip(names, outs):
        d = "xyz".index(n[0])
        assert_close(a[face_slice(ext, d)], blk[n][face_slice(ext, d)], 1e-13, n + " (bnd)")


@pytest.mark.parametrize("scheme_name", list(abi.FLUX))
@pytest.mark.parametrize("thin", [False, True])
def test_fluxes(gpu_lib, scheme_name, thin):
    """compute_fluxes (scheme.f90:68) with every scheme; kmx=2 zeroes H."""
    nc = (8, 6, 1) if thin else (8, 6, 5)
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=nc, ids=(-5, -4, -6, -3, -6, -6), scheme_kw=dict(scheme_name=scheme_name),
        flow_kw=dict(MInf=0.3))
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    blk.populate_ghost_primitive(1)
    blk.compute_face_interpolant()
    blk.reconstruct_boundary_state()
    for n in ("x_qp_left", "x_qp_right", "y_qp_left", "y_qp_right", "z_qp_left", "z_qp_right"):
        h.set(n, blk[n])
    F = np.zeros(abi.shapes(ext)["F"], order="F")
    G = np.zeros(abi.shapes(ext)["G"], order="F")
    H = np.zeros(abi.shapes(ext)["H"], order="F")
    abi.check(h.lib.fest_compute_fluxes(h.h, abi.ptr(F), abi.ptr(G), abi.ptr(H)), "fluxes")
    assert blk.compute_fluxes() == 0
    for a, n in ((F, "F"), (G, "G"), (H, "H")):
        assert_close(a, blk[n], 1e-12, n)


@pytest.mark.parametrize("turb,mu_var", [(False, "constant"), (False, "sutherland_law"),
                                         (True, "sutherland_law")])
@pytest.mark.parametrize("thin", [False, True])
def test_viscous_modules(gpu_lib, turb, mu_var, thin):
    """evaluate_all_gradients (gradients.f90:276), calculate_viscosity
    (viscosity.f90:52), compute_viscous_fluxes (viscous.f90:55),
    add_source_term_residue (source.f90:94), compute_time_step (time.f90:291)."""
    nc = (8, 6, 1) if thin else (8, 6, 5)
    ids = (-3, -4, -5, -4, -6, -6) if thin else (-3, -4, -5, -6, -10, -10)
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=nc, ids=ids, turb=turb, flow_kw=dict(mu_ref=2e-2, mu_variation=mu_var),
        fixed={"fixed_wall_temperature": [0, 0, 0, 0, 0, 0]})
    wall = cases.wall_nodes_of(nodes, ext, bc)
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp, wall=wall if turb else None)
    # reference sequence up to the viscous fluxes on the oracle
    blk.compute_temperature()
    O.apply_interface([blk])
    blk.populate_ghost_primitive(1)
    blk.compute_face_interpolant()
    blk.reconstruct_boundary_state()
    blk.compute_fluxes()
    q = np.asfortranarray(blk["qp"].copy())
    T = np.asfortranarray(blk["Temp"].copy())
    ng = blk.n_grad
    g = [np.zeros(abi.shapes(ext, ng)["grad"], order="F") for _ in range(3)]
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
    if turb:
        assert_close(mut, blk["mu_t"], 1e-11, "mu_t")
        assert_close(F1, blk["sst_F1"], 1e-11, "sst_F1")
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
    assert_close(res, blk["residue"], 1e-10, "residue + SST source")
    dt = np.zeros(abi.shapes(ext)["delta_t"], order="F")
    for n in ("x_qp_left", "x_qp_right", "y_qp_left", "y_qp_right", "z_qp_left", "z_qp_right"):
        h.set(n, blk[n])
    abi.check(h.lib.fest_compute_time_step(h.h, abi.ptr(q), 0.7, abi.ptr(dt)), "time step")
    blk.compute_time_step(0.7)
    assert_close(dt, blk["delta_t"], 1e-12, "delta_t")


@pytest.mark.parametrize("method,gdt", [("l", -1.0), ("g", -1.0), ("g", 1e-6)])
def test_time_step_global(gpu_lib, method, gdt):
    """compute_global_time_step (time.f90:248-289): per-block minval."""
    ext, flow, scheme, bc, nodes, qp = small_case(
        scheme_kw=dict(time_stepping_method=method, global_time_step=gdt))
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    blk.populate_ghost_primitive(1)
    blk.compute_face_interpolant()
    blk.reconstruct_boundary_state()
    for n in ("x_qp_left", "x_qp_right", "y_qp_left", "y_qp_right", "z_qp_left", "z_qp_right"):
        h.set(n, blk[n])
    q = np.asfortranarray(blk["qp"].copy())
    dt = np.zeros(abi.shapes(ext)["delta_t"], order="F")
    abi.check(h.lib.fest_compute_time_step(h.h, abi.ptr(q), 0.9, abi.ptr(dt)), "time step")
    blk.compute_time_step(0.9)
    assert_close(dt, blk["delta_t"], 1e-12, "delta_t")


def test_c_abi_rejects_bad_arguments(gpu_lib):
    ext, flow, scheme, bc, nodes, qp = small_case()
    bad = abi.Extent(ext.imx, ext.jmx, ext.kmx, 7)  # n_var 7 without a turbulence model
    import ctypes as C
    hh = C.c_void_p()
    assert gpu_lib.fest_create(C.byref(bad), C.byref(flow), C.byref(scheme), C.byref(bc),
                               C.byref(hh)) == abi.FEST_ERR_ARG
    assert gpu_lib.fest_find_resnorm(None, None) == abi.FEST_ERR_ARG
