"""Pin the oracle against the reference's own known-answer unit tests.

Each test restates one ``tests/test_*.f90`` of FEST-3D (inputs and pass
bands copied from those files, cited per test) and runs it on the C
restatement.  No GPU."""
import numpy as np
import pytest

import oracle as O
from fest3d import abi


def tiny_block(imx, jmx, kmx, n_var=5, **scheme_kw):
    ext = abi.Extent(imx, jmx, kmx, n_var)
    flow = abi.make_flow()
    sch = abi.make_scheme(**scheme_kw)
    bc = abi.make_bc([3, 3, 3, 3, 3, 3])  # interfaces everywhere: no BC override
    return O.Block(ext, flow, sch, bc)


def unit_faces(blk):
    """Ifaces/Jfaces/Kfaces with unit Cartesian normals and A=1
    (tests/test_ausm.f90:33-44)."""
    for name, c in (("Ifaces", 1), ("Jfaces", 2), ("Kfaces", 3)):
        f = blk[name]
        f[...] = 0.0
        f[0] = 1.0
        f[c] = 1.0


@pytest.mark.parametrize("scheme,band", [
    ("ausm", (4.48, 4.5)),       # tests/test_ausm.f90:54-55
    ("slau", (4.5, 4.7)),        # tests/test_slau.f90:55
    ("ausmP", (4.5, 4.6)),       # tests/test_ausmp.f90:55
    ("ausmUP", (5.0, 5.2)),      # tests/test_ausmUP.f90:55
    ("ldfss0", (4.9, 5.1)),      # tests/test_ldfss.f90:55
    ("van_leer", (4.9, 5.1)),    # tests/test_van_leer.f90:55
])
def test_flux_known_answer(scheme, band):
    """Face pairs L=(1,2,3,4,5)/R=(1,2,3,4,5) and L=(1,2,0,0,1)/R=(.125,0,0,0,.1)
    (tests/test_ausm.f90:45-50), flow defaults (gamma 1.4, MInf 0)."""
    blk = tiny_block(2, 2, 2, scheme_name=scheme)
    blk.flow.MInf = 0.0
    unit_faces(blk)
    xl, xr = blk["x_qp_left"], blk["x_qp_right"]
    xl[1, 0, 0, :] = [1.0, 2.0, 3.0, 4.0, 5.0]   # x_qp_left(1,1,1,:)
    xl[2, 0, 0, :] = [1.0, 2.0, 0.0, 0.0, 1.0]   # x_qp_left(2,1,1,:)
    xr[1, 0, 0, :] = [1.0, 2.0, 3.0, 4.0, 5.0]
    xr[2, 0, 0, :] = [0.125, 0.0, 0.0, 0.0, 0.1]
    for n in ("y_qp_left", "y_qp_right", "z_qp_left", "z_qp_right"):
        blk[n][...] = 1.0
    # MInf is read from the flow struct the block was created with
    blk2 = O.Block(blk.ext, abi.make_flow(MInf=0.0), blk.scheme, blk.bc)
    for n in ("Ifaces", "Jfaces", "Kfaces", "x_qp_left", "x_qp_right", "y_qp_left",
              "y_qp_right", "z_qp_left", "z_qp_right"):
        blk2[n] = blk[n]
    assert blk2.compute_fluxes() == 0
    F = blk2["F"]
    assert 8.9 < F[0, 0, 0, 1] < 9.1
    assert band[0] < F[1, 0, 0, 1] < band[1]


RAMP = [-2.0, -1.0, 0.0, 1.0, 2.0, 3.0, 5.0, 7.0, 7.0, 7.0]  # tests/test_muscl.f90:27-36


def ramp_block(**kw):
    blk = tiny_block(5, 2, 2, **kw)
    qp = blk["qp"]
    qp[...] = 0.0
    for i, v in zip(range(-2, 8), RAMP):
        qp[i + 2, 1 + 2, 1 + 2, :] = v
    return blk


def x_states(blk):
    L, R = blk["x_qp_left"], blk["x_qp_right"]
    return [(L[f, 0, 0, 0], R[f, 0, 0, 0]) for f in range(1, 6)]


def test_muscl_limiter_off_exact():
    """tests/test_muscl.f90:17-50 (limiters off)."""
    blk = ramp_block(interpolant="muscl", ilimiter_switch=0, jlimiter_switch=0, klimiter_switch=0)
    blk.compute_face_interpolant()
    s = x_states(blk)
    assert s[0] == (0.5, 0.5)
    assert s[1] == (1.5, 1.5)
    assert s[2][0] == 2.5 and 2.3 < s[2][1] < 2.4
    assert 3.82 < s[3][0] < 3.85 and s[3][1] == 4.0
    assert s[4][0] == 6.0 and 6.32 < s[4][1] < 6.35


@pytest.mark.parametrize("interp", ["weno", "weno_NM"])
def test_weno_bands(interp):
    """tests/test_weno.f90:28-35 and tests/test_weno_NM.f90:30-37 (volumes 1)."""
    blk = ramp_block(interpolant=interp)
    blk["cells"][0] = 1.0
    blk.compute_face_interpolant()
    s = x_states(blk)
    assert 0.48 <= s[0][0] < 0.52 and 0.48 < s[0][1] < 0.52
    assert 1.48 <= s[1][0] < 1.52 and 1.48 < s[1][1] < 1.52
    assert 2.4 <= s[2][0] < 2.5 and 2.4 < s[2][1] < 2.5
    assert 3.6 <= s[3][0] < 3.7 and 3.8 < s[3][1] < 4.1
    assert 5.9 <= s[4][0] < 6.1 and 6.9 < s[4][1] < 7.1


def test_ppm_bands():
    """tests/test_ppm.f90:22-45 (limiter on)."""
    blk = ramp_block(interpolant="ppm")
    blk.compute_face_interpolant()
    s = x_states(blk)
    assert 0.48 < s[0][0] < 0.52 and 0.48 < s[0][1] < 0.52
    assert 1.48 < s[1][0] < 1.52 and 1.48 < s[1][1] < 1.52
    assert 2.3 < s[2][0] < 2.5 and 2.3 < s[2][1] < 2.5
    assert 3.8 < s[3][0] < 4.0 and 3.8 < s[3][1] < 4.0
    assert 6.0 < s[4][0] < 6.2 and 6.5 < s[4][1] < 6.7


def test_first_order_exact():
    """tests/test_first_order.f90:26-46."""
    blk = ramp_block(interpolant="none", ilimiter_switch=0, jlimiter_switch=0, klimiter_switch=0)
    blk.compute_face_interpolant()
    assert x_states(blk) == [(0, 1), (1, 2), (2, 3), (3, 5), (5, 7)]


def test_residue_exact():
    """tests/test_residue.f90:17-31."""
    blk = tiny_block(2, 2, 2)
    blk["F"][0, 0, 0, :] = [1.0, 2.0, 3.0, 4.0, 5.0]
    blk["F"][1, 0, 0, :] = [2.0, 2.0, 9.0, 0.0, 5.1]
    blk["G"][...] = 1.0
    blk["H"][...] = 1.0
    blk.compute_residue()
    r = blk["residue"][0, 0, 0]
    assert r[0] == 1.0 and r[1] == 0.0 and r[2] == 6.0
    assert 0.09 < r[4] < 1.1


def test_gradient_exact():
    """tests/test_gradient.f90:27-58: qp doubling along i, cell volume 2,
    I-face area 2, J/K area 1; gradqp_x(0:2,1,1,1) = 1.5, 3, 6."""
    ext = abi.Extent(2, 2, 2, 5)
    blk = O.Block(ext, abi.make_flow(mu_ref=1.0), abi.make_scheme(), abi.make_bc([3] * 6))
    blk["cells"][0] = 2.0
    for name, c, A in (("Ifaces", 1, 2.0), ("Jfaces", 2, 1.0), ("Kfaces", 3, 1.0)):
        f = blk[name]
        f[...] = 0.0
        f[0] = A
        f[c] = 1.0
    qp = blk["qp"]
    qp[...] = 1.0
    for i, v in ((0, 2.0), (1, 4.0), (2, 8.0), (3, 16.0)):
        qp[i + 2] = v
    blk["Temp"][...] = 1.0
    assert blk.evaluate_all_gradients() == 0
    g = blk["gradqp_x"]
    assert g[0, 1, 1, 0] == 1.5 and g[1, 1, 1, 0] == 3.0 and g[2, 1, 1, 0] == 6.0


def test_time_step_band():
    """tests/test_time.f90:19-50: unit faces, face states 1.0, CFL 1,
    volumes 1; qp (left uninitialised there) set to rest."""
    blk = tiny_block(2, 2, 2)
    unit_faces(blk)
    for n in ("x_qp_left", "x_qp_right", "y_qp_left", "y_qp_right", "z_qp_left", "z_qp_right"):
        blk[n][...] = 1.0
    blk["cells"][0] = 1.0
    blk["qp"][...] = 0.0
    blk.compute_time_step(1.0)
    dt = blk["delta_t"][0, 0, 0]
    assert 0.135 < dt < 0.145


def test_sutherland_viscosity():
    """tests/test_viscosity.f90:20-40: T = 103320/(1.2*287) = 300 K -> mu = 1."""
    ext = abi.Extent(2, 2, 2, 7)
    blk = O.Block(ext, abi.make_flow(mu_ref=1.0, mu_variation="sutherland_law"),
                  abi.make_scheme(turbulence="sst"), abi.make_bc([3] * 6))
    qp = blk["qp"]
    qp[...] = 1.0
    qp[1 + 2, 1 + 2, 1 + 2, :] = [1.2, 1.0, 1.0, 0.0, 103320.0, 1.0, 1.0]
    blk["dist"][...] = 1.0
    assert blk.calculate_viscosity() == 0
    assert 0.99 < blk["mu"][3, 3, 3] < 1.01


def test_geometry_unit_faces_and_cube():
    """tests/test_geometry.f90:14-47: the face vector of the quad
    (0,0,0),(0,1,1),(0,0,1),(0,1,0) is (1,0,0); a unit cube has volume 1."""
    ext = abi.Extent(2, 2, 2, 5)
    blk = O.Block(ext, abi.make_flow(), abi.make_scheme(), abi.make_bc([3] * 6))
    nd = blk["nodes"]
    for i in (1, 2):
        for j in (1, 2):
            for k in (1, 2):
                nd[:, i + 2, j + 2, k + 2] = [i - 1.0, j - 1.0, k - 1.0]
    blk.setup_geometry()
    If = blk["Ifaces"]
    assert tuple(If[:, 1 + 2, 1 + 2, 1 + 2]) == (1.0, 1.0, 0.0, 0.0)
    assert blk["cells"][0, 1 + 2, 1 + 2, 1 + 2] == pytest.approx(1.0, abs=1e-15)
    assert np.allclose(blk["cells"][1:, 3, 3, 3], [0.5, 0.5, 0.5])
    # ghost nodes are linear extrapolations (grid.f90:137-236)
    assert nd[0, 0, 3, 3] == -3.0 and nd[0, 7, 3, 3] == 4.0


@pytest.mark.parametrize("scheme", ["ausm", "slau", "ausmP", "ausmUP", "ldfss0", "van_leer"])
def test_wall_faces_carry_no_mass_flux(scheme):
    """tests/test_bc.f90: setup_bc with a wall at jmin gives
    make_G_flux_zero(1) == 0 (bc.f90:53-66): wall (-5), slip (-6) and pole
    (-7) faces get a zero mass flux in every scheme (ausm.f90:103-108,
    slau.f90:166-168, ausmP.f90:160-162, ausmUP.f90:178-180,
    ldfss0.f90:110-115, van_leer.f90:95-100), hence a zero energy flux;
    other faces keep theirs.  Random face states, unit normals."""
    ext = abi.Extent(5, 5, 5, 5)
    ids = [-3, -6, -5, -4, -7, -11]  # imin, imax (slip), jmin (wall), jmax, kmin (pole), kmax
    blk = O.Block(ext, abi.make_flow(), abi.make_scheme(scheme_name=scheme), abi.make_bc(ids))
    unit_faces(blk)
    rng = np.random.default_rng(7)
    for n in ("x_qp_left", "x_qp_right", "y_qp_left", "y_qp_right", "z_qp_left", "z_qp_right"):
        a = blk[n]
        a[..., 0] = rng.uniform(0.8, 1.4, a.shape[:-1])
        a[..., 1:4] = rng.uniform(-0.5, 0.5, a.shape[:-1] + (3,))
        a[..., 4] = rng.uniform(0.6, 1.2, a.shape[:-1])
    assert blk.compute_fluxes() == 0
    F, G, H = blk["F"], blk["G"], blk["H"]  # face index 1 at position 0
    for masked, normal in ((F[ext.imx - 1], 1), (G[:, 0], 2), (H[:, :, 0], 3)):
        assert np.all(masked[..., 0] == 0.0) and np.all(masked[..., 4] == 0.0)
        # only the pressure force remains: along the normal, none tangentially
        assert np.all(masked[..., normal] != 0.0)
        assert np.all(np.delete(masked[..., 1:4], normal - 1, axis=-1) == 0.0)
    for open_face in (F[0], G[:, ext.jmx - 1], H[:, :, ext.kmx - 1]):
        assert np.all(open_face[..., 0] != 0.0)
    # control: the same face states without walls carry mass through those faces
    ctl = O.Block(ext, abi.make_flow(), abi.make_scheme(scheme_name=scheme), abi.make_bc([-3] * 6))
    for n in ("Ifaces", "Jfaces", "Kfaces", "x_qp_left", "x_qp_right", "y_qp_left", "y_qp_right",
              "z_qp_left", "z_qp_right"):
        ctl[n] = blk[n]
    assert ctl.compute_fluxes() == 0
    for face in (ctl["F"][ext.imx - 1], ctl["G"][:, 0], ctl["H"][:, :, 0]):
        assert np.all(face[..., 0] != 0.0)


def test_sst_free_stream_values():
    """tests/test_state.f90: with the flow defaults, SST and mu_ref = 1,
    init_infinity_values gives Turb_intensity_inf 0.01, tk_inf 1.5 (and a
    7-variable state, which fest_create requires for SST blocks)."""
    flow = abi.make_flow(mu_ref=1.0)
    tk, tw = abi.sst_free_stream(flow)
    assert tk == 1.5
    assert tw == flow.density_inf * 1.5 / 1.0
    # the turbulent flat plate's free stream (tests/Tfp/system/flow.md)
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_flatplate as MF
    f = abi.make_flow(density_inf=MF.T_RHO, x_speed_inf=MF.T_U, mu_ref=MF.T_MU)
    tk, tw = abi.sst_free_stream(f, tu_inf=0.03873, mu_ratio_inf=0.01)
    assert tk == pytest.approx(MF.T_TK, rel=1e-15) and tw == pytest.approx(MF.T_TW, rel=1e-15)
