"""The oracle's Spalart-Allmaras terms (FEST_TURB_SA) against a second,
independent numpy restatement of the same reference lines, on a small
block with a smooth random state and wall distances:

* the eddy viscosity mu_t = rho tv fv1 over the gradient range and its
  ghost copies (viscosity.f90:149-213);
* the tv diffusion flux of every face (viscous.f90:570-656);
* the source, with the density gradient from the cell's face sums and the
  k faces' (nx, nx, nx) normal (source.f90:845-983);
* the point-implicit destruction and the tv floor of the update
  (update.f90:405-419, 474-475) and the residual-norm scale
  (resnorm.f90:157-158).

No case of the reference runs SA, so this pins the restatement's
arithmetic (a slip in either version shows), not the reference's numbers;
the GPU tests then compare the CUDA path with this oracle."""
import numpy as np

import oracle as O
from fest3d import abi
from parity import small_case

CB1, CB2, CW2, CW3, CV1, SIG, KAP = 0.1355, 0.6220, 0.3, 2.0, 7.1, 2. / 3., 0.41
CW1 = (CB1 / (KAP * KAP)) + ((1 + CB2) / SIG)


def pow6(x):
    x2 = x * x
    return (x2 * x2) * x2


def sa_block():
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(9, 7, 6), turb="sa", ids=(-3, -4, -5, -6, -10, -10),
        flow_kw=dict(mu_ref=1.8e-5, mu_variation="sutherland_law", T_ref=273.0))
    blk = O.Block(ext, flow, scheme, bc)
    blk["nodes"] = nodes
    blk.setup_geometry()
    cells = blk["cells"]
    blk["dist"] = 0.02 + np.abs(cells[2])  # a wall at y = 0
    blk["qp"] = qp
    assert O.get_total_conservative_residue([blk], 3) == 0
    blk.compute_temperature()
    assert O.get_total_conservative_residue([blk], 3) == 0
    return ext, flow, blk


def P(a, i, j, k):
    """a padded array's (i, j, k) entry (lower bound -2)"""
    return a[i + 2, j + 2, k + 2]


def test_sa_eddy_viscosity_and_ghost_copies():
    ext, flow, blk = sa_block()
    q, mu, mut = blk["qp"], blk["mu"], blk["mu_t"]
    imx, jmx, kmx = ext.imx, ext.jmx, ext.kmx
    sl = (slice(3, imx + 2), slice(3, jmx + 2), slice(3, kmx + 2))
    tv, rho = q[sl + (5,)], q[sl + (0,)]
    xi = tv * rho / mu[sl]
    x3 = xi * xi * xi
    want = rho * tv * (x3 / (x3 + CV1 ** 3))
    assert np.allclose(mut[sl], want, rtol=1e-14, atol=0)
    # ghost layer of the imin face (-3): a copy; of the jmin wall (-5): negated
    assert np.array_equal(mut[2, 3:jmx + 2, 3:kmx + 2], mut[3, 3:jmx + 2, 3:kmx + 2])
    assert np.array_equal(mut[3:imx + 2, 2, 3:kmx + 2], -mut[3:imx + 2, 3, 3:kmx + 2])


def test_sa_diffusion_flux():
    ext, flow, blk = sa_block()
    blk.compute_face_interpolant()
    blk.reconstruct_boundary_state()
    assert blk.compute_fluxes() == 0
    F0 = {n: np.array(blk[n]) for n in "FGH"}
    assert blk.compute_viscous_fluxes() == 0
    q, mu, cells = blk["qp"], blk["mu"], blk["cells"]
    g = [blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]]
    imx, jmx, kmx = ext.imx, ext.jmx, ext.kmx
    for d, (n, faces) in enumerate(zip("FGH", ("Ifaces", "Jfaces", "Kfaces"))):
        fa = blk[faces]
        e = np.eye(3, dtype=int)[d]
        dF = blk[n][..., 5] - F0[n][..., 5]
        for k in range(1, kmx + e[2]):
            for j in range(1, jmx + e[1]):
                for i in range(1, imx + e[0]):
                    im, jm, km = i - e[0], j - e[1], k - e[2]
                    gt = [0.5 * (g[c][im, jm, km, 4] + g[c][i, j, k, 4]) for c in range(3)]
                    c1, c0 = cells[:, i + 2, j + 2, k + 2], cells[:, im + 2, jm + 2, km + 2]
                    dl = c1[1:] - c0[1:]
                    dlr = np.sqrt(dl[0] * dl[0] + dl[1] * dl[1] + dl[2] * dl[2])
                    dtv = P(q, i, j, k)[5] - P(q, im, jm, km)[5]
                    nc = (dtv - (gt[0] * dl[0] + gt[1] * dl[1] + gt[2] * dl[2])) / dlr
                    gt = [gt[c] + (nc * dl[c] / dlr) for c in range(3)]
                    rhof = 0.5 * (P(q, im, jm, km)[0] + P(q, i, j, k)[0])
                    muf = 0.5 * (P(mu, im, jm, km) + P(mu, i, j, k))
                    mutf = 0.5 * (P(q, im, jm, km)[5] + P(q, i, j, k)[5]) * rhof
                    A, nx, ny, nz = fa[:, i + 2, j + 2, k + 2]
                    want = -(A * ((muf + mutf) * (gt[0] * nx + gt[1] * ny + gt[2] * nz))) / SIG
                    got = dF[i - 1, j - 1, k - 1]
                    # dF is a difference of the whole flux: its rounding
                    tol = 1e-12 * abs(want) + 4e-16 * abs(F0[n][i - 1, j - 1, k - 1, 5])
                    assert abs(got - want) <= tol, (n, i, j, k, got, want)


def test_sa_source():
    ext, flow, blk = sa_block()
    blk.compute_residue()
    r0 = np.array(blk["residue"][..., 5])
    blk.add_source_term_residue()
    dS = blk["residue"][..., 5] - r0
    q, mu, dist, cells = blk["qp"], blk["mu"], blk["dist"], blk["cells"]
    If, Jf, Kf = blk["Ifaces"], blk["Jfaces"], blk["Kfaces"]
    g = [blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]]
    for k in range(1, ext.kmx):
        for j in range(1, ext.jmx):
            for i in range(1, ext.imx):
                rho, tv = P(q, i, j, k)[0], P(q, i, j, k)[5]
                nb = [(i - 1, j, k), (i, j - 1, k), (i, j, k - 1), (i + 1, j, k), (i, j + 1, k), (i, j, k + 1)]
                rf = [P(q, *c)[0] + rho for c in nb]
                fr = [If[:, i + 2, j + 2, k + 2], Jf[:, i + 2, j + 2, k + 2], Kf[:, i + 2, j + 2, k + 2],
                      If[:, i + 3, j + 2, k + 2], Jf[:, i + 2, j + 3, k + 2], Kf[:, i + 2, j + 2, k + 3]]
                nrm = [f[1:4] for f in fr]
                nrm[2] = np.array([fr[2][1]] * 3)  # source.f90:913
                vol = cells[0, i + 2, j + 2, k + 2]
                gr = [(-rf[0] * nrm[0][c] * fr[0][0] - rf[1] * nrm[1][c] * fr[1][0] - rf[2] * nrm[2][c] * fr[2][0]
                       + rf[3] * nrm[3][c] * fr[3][0] + rf[4] * nrm[4][c] * fr[4][0] + rf[5] * nrm[5][c] * fr[5][0])
                      / (2.0 * vol) for c in range(3)]
                G = lambda c, l: g[c][i, j, k, l - 1]  # noqa: E731
                vort = np.sqrt((G(1, 3) - G(2, 2)) ** 2 + (G(2, 1) - G(0, 3)) ** 2 + (G(0, 2) - G(1, 1)) ** 2)
                cd1 = CB2 * (G(0, 5) * G(0, 5) + G(1, 5) * G(1, 5) + G(2, 5) * G(2, 5))
                cd2 = gr[0] * G(0, 5) + gr[1] * G(1, 5) + gr[2] * G(2, 5)
                d = P(dist, i, j, k)
                kd2 = (KAP * d) * (KAP * d)
                nu = P(mu, i, j, k) / rho
                xi = tv / nu
                fv1 = xi ** 3 / (xi ** 3 + CV1 ** 3)
                fv2 = 1.0 - xi / (1.0 + xi * fv1)
                scap = max(vort + tv * fv2 / kd2, 0.3 * vort)
                rr = min(tv / (scap * kd2), 10.0)
                gg = rr + CW2 * (pow6(rr) - rr)
                fw = gg * ((1.0 + pow6(CW3)) / (pow6(gg) + pow6(CW3))) ** (1.0 / 6.0)
                Dv = rho * CW1 * fw * (tv / d) ** 2
                Pv = rho * CB1 * scap * tv
                lam = rho * cd1 / SIG - cd2 * (nu + tv) / SIG
                want = -(Pv - Dv + lam) * vol
                got = dS[i - 1, j - 1, k - 1]
                assert abs(got - want) <= 1e-12 * max(abs(Pv * vol), abs(Dv * vol), abs(lam * vol)), \
                    (i, j, k, got, want)


def test_sa_point_implicit_update_and_norm():
    ext, flow, blk = sa_block()
    blk.compute_time_step(0.5)
    q0 = np.array(blk["qp"])
    R = np.array(blk["residue"])
    mu, dist, cells, dt = blk["mu"], blk["dist"], blk["cells"], blk["delta_t"]
    g = [blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]]
    assert blk.update_with(1.0, 0.0) == 0
    q1 = blk["qp"]
    for k in range(1, ext.kmx):
        for j in range(1, ext.jmx):
            for i in range(1, ext.imx):
                rho, tv = P(q0, i, j, k)[0], P(q0, i, j, k)[5]
                u6 = tv * rho
                G = lambda c, l: g[c][i, j, k, l - 1]  # noqa: E731
                vort = np.sqrt((G(1, 3) - G(2, 2)) ** 2 + (G(2, 1) - G(0, 3)) ** 2 + (G(0, 2) - G(1, 1)) ** 2)
                d = P(dist, i, j, k)
                kd2 = (KAP * d) * (KAP * d)
                xi = u6 * rho / P(mu, i, j, k)  # update.f90:412, as written
                fv1 = xi ** 3 / (xi ** 3 + CV1 ** 3)
                fv2 = 1.0 - xi / (1 + xi * fv1)
                scap = vort + u6 * fv2 / kd2
                rsa = min(u6 / (scap * kd2), 10.0)
                gg = rsa + CW2 * (pow6(rsa) - rsa)
                fw = gg * ((1.0 + pow6(CW3)) / (pow6(gg) + pow6(CW3))) ** (1.0 / 6.0)
                dtc = dt[i - 1, j - 1, k - 1]
                R6 = R[i - 1, j - 1, k - 1, 5] / (1. + ((-rho * CB1 * scap) + (2.0 * rho * CW1 * fw * u6 / (d * d))) * dtc)
                fac = dtc / cells[0, i + 2, j + 2, k + 2]
                r2 = rho - R[i - 1, j - 1, k - 1, 0] * fac
                want = max((u6 - R6 * fac) / r2, 1e-12)
                got = P(q1, i, j, k)[5]
                assert abs(got - want) <= 1e-12 * abs(want), (i, j, k, got, want)
    norm = O.find_resnorm([blk])
    sl = (slice(0, ext.imx - 1), slice(0, ext.jmx - 1), slice(0, ext.kmx - 1))
    scale = flow.density_inf * flow.vel_mag * flow.tv_inf
    assert abs(norm[6] - np.sqrt(np.sum((blk["residue"][sl + (5,)] / scale) ** 2))) <= 1e-12 * norm[6]
