"""The oracle's 'bc' transition models (FEST_TRANSITION_BC: saBC and
SST-BC) against a second, independent numpy restatement of the same
reference lines, on a small block with a smooth random state and wall
distances:

* saBC (source.f90:985-1194): the SA source with S-hat floored at 1e-10,
  the production scaled by the intermittency and not by density;
* SST-BC (source.f90:467-604): production mu_t Omega^2 limited by 20 D_k,
  P_w taken from it before the intermittency scales P_k, the cross
  diffusion unfloored, the SST constants for sst2003 too;
* the intermittency itself (source.f90:571-589): from the momentum-
  thickness Reynolds number against 803.73 (Tu + 0.6067)^-1.027 and the
  eddy viscosity against 5/Re, Re the free stream's per unit length
  (state.f90:89).

The flows are set so that the intermittency takes values across (0, 1) in
the block, not only its limits.  No case of the reference runs either
model, so this pins the restatement's arithmetic; the GPU tests then
compare the CUDA path with this oracle."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from fest3d import abi
from parity import small_case

CB1, CB2, CW2, CW3, CV1, SIG, KAP = 0.1355, 0.6220, 0.3, 2.0, 7.1, 2. / 3., 0.41
CW1 = (CB1 / (KAP * KAP)) + ((1 + CB2) / SIG)
SIGMA_W1, SIGMA_W2, BETA1, BETA2, BSTAR = 0.5, 0.856, 0.075, 0.0828, 0.09
GAMA1 = BETA1 / BSTAR - SIGMA_W1 * KAP * KAP / np.sqrt(BSTAR)
GAMA2 = BETA2 / BSTAR - SIGMA_W2 * KAP * KAP / np.sqrt(BSTAR)


def pow6(x):
    x2 = x * x
    return (x2 * x2) * x2


def P(a, i, j, k):
    """a padded array's (i, j, k) entry (lower bound -2)"""
    return a[i + 2, j + 2, k + 2]


def gamma_bc(re_v, nu_bc, flow):
    Re = flow.density_inf * flow.vel_mag / flow.mu_ref
    nu_cr = 5.0 / Re
    rt = 803.73 * (flow.tu_inf + 0.6067) ** -1.027
    t1 = np.sqrt(max(re_v / 2.193 - rt, 0.0) / (0.002 * rt))
    t2 = np.sqrt(max(nu_bc - nu_cr, 0.0) / nu_cr)
    return 1.0 - np.exp(-(t1 + t2))


def bc_block(turb, tu_inf, mu_ref, tv_inf=None):
    fk = dict(mu_ref=mu_ref, mu_variation="constant", tu_inf=tu_inf)
    if tv_inf is not None:
        fk["tv_inf"] = tv_inf
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(9, 7, 6), turb=turb, ids=(-3, -4, -5, -6, -10, -10),
        scheme_kw=dict(transition="bc", **({} if turb == "sa" else dict(turbulence=turb))), flow_kw=fk)
    if turb == "sa":
        qp[..., 5] *= tv_inf / 1.2e-4  # the state's tv around the free stream's
    blk = O.Block(ext, flow, scheme, bc)
    blk["nodes"] = nodes
    blk.setup_geometry()
    blk["dist"] = 0.02 + np.abs(blk["cells"][2])  # a wall at y = 0
    blk["qp"] = qp
    assert O.get_total_conservative_residue([blk], 3) == 0
    blk.compute_temperature()
    assert O.get_total_conservative_residue([blk], 3) == 0
    blk.compute_residue()
    r0 = np.array(blk["residue"])
    blk.add_source_term_residue()
    # the source's share of the residual, and the rounding of the residual
    # it was added to
    return ext, flow, blk, blk["residue"] - r0, 4e-16 * np.abs(r0)


def test_sa_bc_source():
    # mu 2e-3: Re = 3.6e4 per unit length; nu_t around 5/Re
    ext, flow, blk, dS, rnd = bc_block("sa", tu_inf=1.0, mu_ref=2e-3, tv_inf=2e-4)
    q, mu, dist, cells = blk["qp"], blk["mu"], blk["dist"], blk["cells"]
    If, Jf, Kf = blk["Ifaces"], blk["Jfaces"], blk["Kfaces"]
    g = [blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]]
    gams = []
    for k in range(1, ext.kmx):
        for j in range(1, ext.jmx):
            for i in range(1, ext.imx):
                rho, u, v, w, tv = (P(q, i, j, k)[c] for c in (0, 1, 2, 3, 5))
                nb = [(i - 1, j, k), (i, j - 1, k), (i, j, k - 1), (i + 1, j, k), (i, j + 1, k), (i, j, k + 1)]
                rf = [P(q, *c)[0] + rho for c in nb]
                fr = [If[:, i + 2, j + 2, k + 2], Jf[:, i + 2, j + 2, k + 2], Kf[:, i + 2, j + 2, k + 2],
                      If[:, i + 3, j + 2, k + 2], Jf[:, i + 2, j + 3, k + 2], Kf[:, i + 2, j + 2, k + 3]]
                nrm = [f[1:4] for f in fr]
                nrm[2] = np.array([fr[2][1]] * 3)  # source.f90:1084
                vol = cells[0, i + 2, j + 2, k + 2]
                gr = [sum((1 if f >= 3 else -1) * rf[f] * nrm[f][c] * fr[f][0] for f in range(6)) / (2.0 * vol)
                      for c in range(3)]
                G = lambda c, l: g[c][i, j, k, l - 1]  # noqa: E731
                om = np.sqrt((G(1, 3) - G(2, 2)) ** 2 + (G(2, 1) - G(0, 3)) ** 2 + (G(0, 2) - G(1, 1)) ** 2)
                cd1 = CB2 * (G(0, 5) ** 2 + G(1, 5) ** 2 + G(2, 5) ** 2)
                cd2 = gr[0] * G(0, 5) + gr[1] * G(1, 5) + gr[2] * G(2, 5)
                d = P(dist, i, j, k)
                nu = P(mu, i, j, k) / rho
                chi = tv / nu
                fv1 = chi ** 3 / (chi ** 3 + CV1 ** 3)
                fv2 = 1.0 - chi / (1.0 + chi * fv1)
                shat = max(om + tv * fv2 / (KAP * KAP * d * d), 1e-10)
                gam = gamma_bc(d * d * om / nu, tv * fv1 / (np.sqrt(u * u + v * v + w * w) * d), flow)
                gams.append(gam)
                prod = gam * CB1 * shat * tv * vol
                rr = min(tv / (shat * KAP * KAP * d * d), 10.0)
                gg = rr + CW2 * (pow6(rr) - rr)
                fw = gg * ((1.0 + pow6(CW3)) / (pow6(gg) + pow6(CW3))) ** (1.0 / 6.0)
                dest = CW1 * fw * tv * tv / (d * d) * vol
                lam1, lam2 = rho * cd1 / SIG * vol, cd2 * (nu + tv) / SIG * vol
                want = -(prod - dest + (lam1 - lam2))
                got = dS[i - 1, j - 1, k - 1, 5]
                tol = 1e-12 * max(abs(prod), abs(dest), abs(lam1), abs(lam2)) + rnd[i - 1, j - 1, k - 1, 5]
                assert abs(got - want) <= tol, (i, j, k, got, want)
    gams = np.array(gams)
    assert gams.min() < 0.5 and gams.max() > 0.9 and np.sum((gams > 0.05) & (gams < 0.95)) >= 1


@pytest.mark.parametrize("turb", ["sst", "sst2003"])
def test_sst_bc_source(turb):
    # mu 0.1: nu_t / (|u| d) near 5/Re = 7e-3 in the block
    ext, flow, blk, dS, rnd = bc_block(turb, tu_inf=3.0, mu_ref=0.1)
    q, mu, mut, dist, cells, F1s = blk["qp"], blk["mu"], blk["mu_t"], blk["dist"], blk["cells"], blk["sst_F1"]
    g = [blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]]
    gams = []
    for k in range(1, ext.kmx):
        for j in range(1, ext.jmx):
            for i in range(1, ext.imx):
                rho, u, v, w, tk, tw = (P(q, i, j, k)[c] for c in (0, 1, 2, 3, 5, 6))
                G = lambda c, l: g[c][i, j, k, l - 1]  # noqa: E731
                om = np.sqrt((G(1, 3) - G(2, 2)) ** 2 + (G(2, 1) - G(0, 3)) ** 2 + (G(0, 2) - G(1, 1)) ** 2)
                cd = 2 * rho * SIGMA_W2 * (G(0, 5) * G(0, 6) + G(1, 5) * G(1, 6) + G(2, 5) * G(2, 6)) / tw
                F1 = P(F1s, i, j, k)
                gama = GAMA1 * F1 + GAMA2 * (1 - F1)
                beta = BETA1 * F1 + BETA2 * (1 - F1)
                Dk, Dw = BSTAR * rho * tw * tk, beta * rho * tw * tw
                mt = P(mut, i, j, k)
                Pk = min(mt * om * om, 20.0 * Dk)
                Pw = rho * gama / mt * Pk
                d = P(dist, i, j, k)
                gam = gamma_bc(rho * d * d * om / P(mu, i, j, k), mt / rho / (np.sqrt(u * u + v * v + w * w) * d), flow)
                gams.append(gam)
                vol = cells[0, i + 2, j + 2, k + 2]
                want_k = -(gam * Pk - Dk) * vol
                want_w = -(Pw - Dw + (1 - F1) * cd) * vol
                got, e = dS[i - 1, j - 1, k - 1], rnd[i - 1, j - 1, k - 1]
                assert abs(got[5] - want_k) <= 1e-12 * max(abs(Pk), abs(Dk)) * vol + e[5], (i, j, k, got[5], want_k)
                assert abs(got[6] - want_w) <= 1e-12 * max(abs(Pw), abs(Dw), abs(cd)) * vol + e[6], \
                    (i, j, k, got[6], want_w)
    gams = np.array(gams)
    assert gams.min() < 0.5 and gams.max() > 0.9 and np.sum((gams > 0.05) & (gams < 0.95)) >= 1


def test_transition_is_a_source_only_change():
    """Away from the source the 'bc' models leave the residual alone: the
    SST-BC and SST residuals before the source are identical, and so are
    the k and omega rows' differences after it wherever the intermittency
    is 1 and the production is unlimited with no divergence (here: the
    mass, momentum and energy rows everywhere)."""
    base = bc_block("sst", tu_inf=3.0, mu_ref=0.1)
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(9, 7, 6), turb=True, ids=(-3, -4, -5, -6, -10, -10),
        flow_kw=dict(mu_ref=0.1, mu_variation="constant", tu_inf=3.0))
    blk = O.Block(ext, flow, scheme, bc)
    blk["nodes"] = nodes
    blk.setup_geometry()
    blk["dist"] = 0.02 + np.abs(blk["cells"][2])
    blk["qp"] = qp
    assert O.get_total_conservative_residue([blk], 3) == 0
    blk.compute_temperature()
    assert O.get_total_conservative_residue([blk], 3) == 0
    blk.compute_residue()
    blk.add_source_term_residue()
    assert np.array_equal(blk["residue"][..., :5], base[2]["residue"][..., :5])
    assert not np.array_equal(blk["residue"][..., 5], base[2]["residue"][..., 5])


def test_create_refuses_transition_outside_sa_and_sst():
    """fest_create checks the scheme before it touches a device: 'bc' with
    no model or k-kL, an unknown transition model (lctm2015 is not built),
    and 'bc' without a viscosity are FEST_ERR_ARG; 'bc' with SA and SST
    passes the checks."""
    L = abi.load()

    def create(turb, n_var, transition, mu_ref=1e-3):
        h = C.c_void_p()
        scheme = abi.make_scheme(turbulence=turb)
        scheme.transition = transition
        rc = L.fest_create(C.byref(abi.Extent(5, 5, 5, n_var)), C.byref(abi.make_flow(mu_ref=mu_ref)),
                           C.byref(scheme), C.byref(abi.make_bc([-3, -4, -5, -6, -5, -5])), C.byref(h))
        if rc == abi.FEST_OK:
            L.fest_destroy(h)
        return rc

    assert create("none", 5, abi.TRANSITION["bc"]) == abi.FEST_ERR_ARG
    assert create("kkl", 7, abi.TRANSITION["bc"]) == abi.FEST_ERR_ARG
    assert create("sst", 7, 2) == abi.FEST_ERR_ARG
    assert create("sst", 7, abi.TRANSITION["bc"], mu_ref=0.0) == abi.FEST_ERR_ARG
    assert create("sst", 7, abi.TRANSITION["bc"]) != abi.FEST_ERR_ARG
    assert create("sa", 6, abi.TRANSITION["bc"]) != abi.FEST_ERR_ARG


def test_sst_bc_runs_with_lusgs():
    """The implicit integrators update SST-BC blocks as SST ones
    (lusgs.f90:161-164): LU-SGS takes them, and its iterations differ from
    plain SST's only through the source."""
    out = []
    for transition in ("bc", "none"):
        ext, flow, scheme, bc, nodes, qp = small_case(
            nc=(9, 7, 6), turb=True, ids=(-3, -4, -5, -6, -10, -10),
            scheme_kw=dict(transition=transition, time_step_accuracy="implicit", scheme_name="ausmUP"),
            flow_kw=dict(mu_ref=0.1, mu_variation="constant", tu_inf=3.0, tk_inf=1.0, tw_inf=1000.0))
        blk = O.Block(ext, flow, scheme, bc)
        blk["nodes"] = nodes
        blk.setup_geometry()
        blk["dist"] = 0.02 + np.abs(blk["cells"][2])
        blk["qp"] = qp
        for it in (1, 2):
            assert O.lusgs_next_solution([blk], it, 20.0) == 0
        out.append(np.array(blk["qp"]))
    sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
    assert np.all(np.isfinite(out[0][sl]))
    assert np.abs(out[0][sl + (5,)] - out[1][sl + (5,)]).max() > 0.0
