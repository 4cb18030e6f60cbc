"""The oracle's LCTM2015 transition model (FEST_TRANSITION_LCTM2015 on
k-omega SST, eight variables) against a second, independent numpy
restatement of the same reference lines, on a small block with a smooth
random state, an intermittency in (0.1, 0.9) and wall distances:

* the source (source.f90:273-465): SST's with the production by vorticity
  times strain scaled by the intermittency, the limited extra production
  and the floored destruction, and the intermittency's own source; the
  pressure-gradient parameter from the wall distance's Green-Gauss gradient
  dotted with its unit vector (CC.f90:56-92);
* F1 raised to exp(-(var1/120)^8) (viscosity.f90:390-405), with the
  density and k of the cell (imx, jmx, kmx) that the reference's loop
  carries over;
* the intermittency's diffusion flux (viscous.f90:658-749);
* the updates: the explicit ones leave the intermittency as it is (the
  reference's update_with writes variables 1-7 only, update.f90:448-480),
  LU-SGS moves it and floors it at zero (lusgs.f90:2685-2687).

No case of the reference runs LCTM2015, so this pins the restatement's
arithmetic; the GPU tests then compare the CUDA path with this oracle."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from fest3d import abi
from parity import small_case

SIGMA_W1, SIGMA_W2, BETA1, BETA2, BSTAR, KAP = 0.5, 0.856, 0.075, 0.0828, 0.09, 0.41


def P(a, i, j, k):
    """a padded array's (i, j, k) entry (lower bound -2)"""
    return a[i + 2, j + 2, k + 2]


def lctm_block(turb="sst", transition="lctm2015", acc="RK4"):
    sk = dict(transition=transition, time_step_accuracy=acc)
    if turb != "sst":
        sk["turbulence"] = turb
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(9, 7, 6), turb=True, ids=(-3, -4, -5, -6, -10, -10), scheme_kw=sk,
        flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law", tk_inf=1.0, tw_inf=1000.0))
    if transition != "lctm2015":
        qp = np.asfortranarray(qp[..., :7])
    blk = O.Block(ext, flow, scheme, bc)
    blk["nodes"] = nodes
    blk.setup_geometry()
    blk["dist"] = 0.02 + np.abs(blk["cells"][2])  # a wall at y = 0
    blk["qp"] = qp
    return ext, flow, blk


def residual_parts(blk):
    assert O.get_total_conservative_residue([blk], 3) == 0
    blk.compute_temperature()
    assert O.get_total_conservative_residue([blk], 3) == 0
    blk.compute_residue()
    r0 = np.array(blk["residue"])
    blk.add_source_term_residue()
    return blk["residue"] - r0, 4e-16 * np.abs(r0)


@pytest.mark.parametrize("turb", ["sst", "sst2003"])
def test_lctm_source(turb):
    ext, flow, blk = lctm_block(turb)
    dS, rnd = residual_parts(blk)
    q, mu, mut, dist, cells, F1s = blk["qp"], blk["mu"], blk["mu_t"], blk["dist"], blk["cells"], blk["sst_F1"]
    fa = [blk["Ifaces"], blk["Jfaces"], blk["Kfaces"]]
    g = [blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]]
    s2003 = turb == "sst2003"
    lim = 10 if s2003 else 20
    g1 = 5 / 9 if s2003 else BETA1 / BSTAR - SIGMA_W1 * KAP * KAP / np.sqrt(BSTAR)
    g2 = 0.44 if s2003 else BETA2 / BSTAR - SIGMA_W2 * KAP * KAP / np.sqrt(BSTAR)
    onset = []
    for k in range(1, ext.kmx):
        for j in range(1, ext.jmx):
            for i in range(1, ext.imx):
                rho, tk, tw, gm = (P(q, i, j, k)[c] for c in (0, 5, 6, 7))
                G = lambda c, l: g[c][i, j, k, l - 1]  # noqa: E731
                vort = np.sqrt((G(1, 3) - G(2, 2)) ** 2 + (G(2, 1) - G(0, 3)) ** 2 + (G(0, 2) - G(1, 1)) ** 2)
                strain = np.sqrt((G(1, 3) + G(2, 2)) ** 2 + (G(2, 1) + G(0, 3)) ** 2 + (G(0, 2) + G(1, 1)) ** 2
                                 + 2 * G(0, 1) ** 2 + 2 * G(1, 2) ** 2 + 2 * G(2, 3) ** 2)
                cd = max(2 * rho * SIGMA_W2 * sum(G(c, 5) * G(c, 6) for c in range(3)) / tw, 10.0 ** -lim)
                F1 = P(F1s, i, j, k)
                gama, beta = g1 * F1 + g2 * (1 - F1), BETA1 * F1 + BETA2 * (1 - F1)
                Dk, Dw = BSTAR * rho * tw * tk, beta * rho * tw * tw
                mt, m, d = P(mut, i, j, k), P(mu, i, j, k), P(dist, i, j, k)
                Pk = min(mt * vort * strain - 2 / 3 * rho * tk * (G(0, 1) + G(1, 2) + G(2, 3)), lim * Dk)
                Pw = rho * gama / mt * Pk
                # CC.f90: the distance's gradient and its unit vector
                nb = [(i - 1, j, k), (i, j - 1, k), (i, j, k - 1), (i + 1, j, k), (i, j + 1, k), (i, j, k + 1)]
                fr = [fa[f % 3][:, i + 2 + (f == 3), j + 2 + (f == 4), k + 2 + (f == 5)] for f in range(6)]
                vol = cells[0, i + 2, j + 2, k + 2]
                gd = np.array([sum((1 if f >= 3 else -1) * (P(dist, *nb[f]) + d) * fr[f][1 + c] * fr[f][0]
                                   for f in range(6)) / (2 * vol) for c in range(3)])
                dvdy = float(gd @ (gd / (np.linalg.norm(gd) + 1e-12)))
                lamd = min(max(-7.57e-3 * dvdy * d * d * rho / m + 0.0128, -1.0), 1.0)
                fpg = max(min(1 + 14.68 * lamd, 1.5) if lamd >= 0 else min(1 - 7.34 * lamd, 3.0), 0.0)
                tul = min(100 * np.sqrt(2 * tk / 3) / (tw * d), 100.0)
                ret = 100 + 1000 * np.exp(-tul * fpg)
                rev = rho * d * d * strain / m
                rt = rho * tk / (m * tw)
                fturb = np.exp(-(0.5 * rt) ** 4)
                fon = max(min(rev / (2.2 * ret), 2.0) - max(1 - (rt / 3.5) ** 3, 0.0), 0.0)
                onset.append(fon)
                Pg = 100 * rho * strain * gm * (1 - gm) * fon
                Dg = 0.06 * rho * vort * gm * fturb * (50 * gm - 1)
                flim = min(max(rev / 2420.0 - 1, 0.0), 3.0)
                Pkl = 5 * max(gm - 0.2, 0) * (1 - gm) * flim * max(3 * m - mt, 0) * strain * vort
                want = [-(gm * Pk - max(gm, 0.1) * Dk + Pkl) * vol, -(Pw - Dw + (1 - F1) * cd) * vol,
                        -(Pg - Dg) * vol]
                scale = [max(abs(gm * Pk), Dk, abs(Pkl)), max(abs(Pw), Dw, cd), max(abs(Pg), abs(Dg))]
                got, e = dS[i - 1, j - 1, k - 1], rnd[i - 1, j - 1, k - 1]
                for n, l in enumerate((5, 6, 7)):
                    assert abs(got[l] - want[n]) <= 1e-11 * scale[n] * vol + e[l], (l, i, j, k, got[l], want[n])
    assert max(onset) > 0.0  # the onset term acts somewhere in the block


def test_lctm_blending_and_diffusion():
    """F1 and the fluxes of an LCTM2015 block against the same state's SST
    block: F1 = max(F1_sst, exp(-(var1/120)^8)) with the corner cell's
    density and k; the fluxes of variables 1-7 unchanged where F1 is, and
    the eighth the intermittency's convection less its diffusion."""
    ext, flow, blk = lctm_block()
    ext7, _, sst = lctm_block(transition="none")
    sst["qp"] = np.asfortranarray(blk["qp"][..., :7])
    for b in (blk, sst):
        assert O.get_total_conservative_residue([b], 3) == 0
        b.compute_temperature()
        assert O.get_total_conservative_residue([b], 3) == 0
    q, mu, dist = blk["qp"], blk["mu"], blk["dist"]
    rc, tc = q[ext.imx + 2, ext.jmx + 2, ext.kmx + 2, 0], q[ext.imx + 2, ext.jmx + 2, ext.kmx + 2, 5]
    sl = (slice(2, ext.imx + 3), slice(2, ext.jmx + 3), slice(2, ext.kmx + 3))  # cells 0..imx
    var1 = rc * dist[sl] * np.sqrt(tc) / mu[sl]
    want = np.maximum(sst["sst_F1"][sl], np.exp(-(var1 / 120) ** 8))
    inner = (slice(1, -1),) * 3
    assert np.allclose(blk["sst_F1"][sl][inner], want[inner], rtol=1e-13, atol=0)
    changed = np.abs(blk["sst_F1"][sl][inner] - sst["sst_F1"][sl][inner]).max()
    assert changed > 1e-3  # the blending acts in this block
    # the eighth flux: convection (the scheme's) minus the diffusion
    g = [blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]]
    cells, mut = blk["cells"], blk["mu_t"]
    blk.compute_face_interpolant()
    blk.reconstruct_boundary_state()
    assert blk.compute_fluxes() == 0
    F0 = np.array(blk["F"][..., 7])
    assert blk.compute_viscous_fluxes() == 0
    dF = blk["F"][..., 7] - F0
    fa = blk["Ifaces"]
    for k in range(1, ext.kmx):
        for j in range(1, ext.jmx):
            for i in range(1, ext.imx + 1):
                gt = np.array([0.5 * (g[c][i - 1, j, k, 6] + g[c][i, j, k, 6]) for c in range(3)])
                dl = cells[1:, i + 2, j + 2, k + 2] - cells[1:, i + 1, j + 2, k + 2]
                dlr = np.sqrt(dl @ dl)
                nc = (P(q, i, j, k)[7] - P(q, i - 1, j, k)[7] - gt @ dl) / dlr
                gt = gt + nc * dl / dlr
                muf = 0.5 * (P(mu, i - 1, j, k) + P(mu, i, j, k)) + 0.5 * (P(mut, i - 1, j, k) + P(mut, i, j, k))
                A, nx, ny, nz = fa[:, i + 2, j + 2, k + 2]
                want = -A * muf * (gt @ np.array([nx, ny, nz]))
                tol = 1e-12 * abs(want) + 4e-16 * abs(F0[i - 1, j - 1, k - 1])
                assert abs(dF[i - 1, j - 1, k - 1] - want) <= tol, (i, j, k)


def test_lctm_updates():
    sl = lambda e: (slice(3, e.imx + 2), slice(3, e.jmx + 2), slice(3, e.kmx + 2))  # noqa: E731
    ext, flow, blk = lctm_block(acc="RK4")
    q0 = np.array(blk["qp"])
    assert O.get_next_solution([blk], 1, 0.5) == 0
    assert np.array_equal(blk["qp"][sl(ext) + (7,)], q0[sl(ext) + (7,)])
    assert np.abs(blk["qp"][sl(ext) + (5,)] - q0[sl(ext) + (5,)]).max() > 0
    ext, flow, blk = lctm_block(acc="implicit")
    q0 = np.array(blk["qp"])
    for it in (1, 2):
        assert O.lusgs_next_solution([blk], it, 20.0) == 0
    g = blk["qp"][sl(ext) + (7,)]
    assert np.abs(g - q0[sl(ext) + (7,)]).max() > 1e-3 and g.min() >= 0.0
    # PLU-SGS (plusgs.f90:2130-2624): the same sweeps, preconditioned, the
    # intermittency in x and a zero in c
    ext, flow, blk = lctm_block(acc="plusgs")
    q0 = np.array(blk["qp"])
    for it in (1, 2):
        assert O.plusgs_next_solution([blk], it, 20.0) == 0
    g = blk["qp"][sl(ext) + (7,)]
    assert np.abs(g - q0[sl(ext) + (7,)]).max() > 1e-3 and g.min() >= 0.0


def test_create_checks_lctm():
    """fest_create checks the scheme before it touches a device: LCTM2015
    needs k-omega SST, eight variables and a viscosity; with SST and
    either implicit integrator it passes the checks."""
    L = abi.load()

    def create(turb, n_var, acc="RK4", mu_ref=1e-3):
        h = C.c_void_p()
        scheme = abi.make_scheme(turbulence=turb, transition="lctm2015", time_step_accuracy=acc)
        rc = L.fest_create(C.byref(abi.Extent(5, 5, 5, n_var)), C.byref(abi.make_flow(mu_ref=mu_ref)),
                           C.byref(scheme), C.byref(abi.make_bc([-3, -4, -5, -6, -5, -5])), C.byref(h))
        if rc == abi.FEST_OK:
            L.fest_destroy(h)
        return rc

    assert create("none", 6) == abi.FEST_ERR_ARG
    assert create("sa", 7) == abi.FEST_ERR_ARG
    assert create("kkl", 8) == abi.FEST_ERR_ARG
    assert create("sst", 7) == abi.FEST_ERR_ARG  # the intermittency is the eighth variable
    assert create("sst", 8, mu_ref=0.0) == abi.FEST_ERR_ARG
    assert create("sst", 8, acc="plusgs") != abi.FEST_ERR_ARG
    assert create("sst", 8) != abi.FEST_ERR_ARG
    assert create("sst2003", 8, acc="implicit") != abi.FEST_ERR_ARG
