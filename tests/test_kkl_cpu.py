"""The oracle's k-kL terms (FEST_TURB_KKL) against a second, independent
numpy restatement of the same reference lines, on a small block with a
smooth random state and wall distances:

* the eddy viscosity mu_t = cmu^0.25 rho kL / max(sqrt(k), 1e-20) over the
  gradient range and its ghost copies on faces -1..-4, -6, -8, -9
  (viscosity.f90:469-533);
* the k and kL diffusion and the -2/3 rho k normal stress of every face
  (viscous.f90:450-567);
* the source, with the von Karman length from the Green-Gauss second
  derivatives of the velocity (source.f90:607-832);
* the point-implicit destruction of the update (update.f90:399-404) and
  the residual-norm scales (resnorm.f90:151-153).

No case of the reference runs k-kL: this pins the restatement's
arithmetic, not the reference's numbers."""
import numpy as np

import oracle as O
from parity import small_case

Z1, Z2, Z3, SK, SP, CMU, KAP, C11, C12, CD1 = 1.2, 0.97, 0.13, 1.0, 1.0, 0.09, 0.41, 10.0, 1.3, 4.7


def kkl_block():
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(9, 7, 6), turb="kkl", ids=(-3, -4, -5, -6, -10, -10),
        flow_kw=dict(mu_ref=1.8e-5, mu_variation="sutherland_law", T_ref=273.0))
    blk = O.Block(ext, flow, scheme, bc)
    blk["nodes"] = nodes
    blk.setup_geometry()
    cells = blk["cells"]
    blk["dist"] = 0.02 + np.abs(cells[2])
    blk["qp"] = qp
    assert O.get_total_conservative_residue([blk], 3) == 0
    blk.compute_temperature()
    assert O.get_total_conservative_residue([blk], 3) == 0
    return ext, flow, blk


def P(a, i, j, k):
    return a[i + 2, j + 2, k + 2]


def test_kkl_eddy_viscosity_and_ghost_copies():
    ext, flow, blk = kkl_block()
    q, mut = blk["qp"], blk["mu_t"]
    imx, jmx, kmx = ext.imx, ext.jmx, ext.kmx
    sl = (slice(3, imx + 2), slice(3, jmx + 2), slice(3, kmx + 2))
    rho, tk, tkl = q[sl + (0,)], q[sl + (5,)], q[sl + (6,)]
    want = CMU ** 0.25 * rho * tkl / np.maximum(np.sqrt(tk), 1e-20)
    want = np.where((tkl < 1e-14) | (tk < 1e-14), 0.0, want)
    assert np.allclose(mut[sl], want, rtol=1e-14, atol=0)
    assert np.array_equal(mut[2, 3:jmx + 2, 3:kmx + 2], mut[3, 3:jmx + 2, 3:kmx + 2])      # -3 copy
    assert np.array_equal(mut[3:imx + 2, 2, 3:kmx + 2], -mut[3:imx + 2, 3, 3:kmx + 2])     # -5 negated


def test_kkl_diffusion_flux():
    ext, flow, blk = kkl_block()
    blk.compute_face_interpolant()
    blk.reconstruct_boundary_state()
    assert blk.compute_fluxes() == 0
    F0 = {n: np.array(blk[n]) for n in "FGH"}
    assert blk.compute_viscous_fluxes() == 0
    q, mu, mut, cells = blk["qp"], blk["mu"], blk["mu_t"], blk["cells"]
    g = [blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]]
    imx, jmx, kmx = ext.imx, ext.jmx, ext.kmx
    for d, (n, faces) in enumerate(zip("FGH", ("Ifaces", "Jfaces", "Kfaces"))):
        fa = blk[faces]
        e = np.eye(3, dtype=int)[d]
        for k in range(1, kmx + e[2]):
            for j in range(1, jmx + e[1]):
                for i in range(1, imx + e[0]):
                    im, jm, km = i - e[0], j - e[1], k - e[2]
                    c1, c0 = cells[:, i + 2, j + 2, k + 2], cells[:, im + 2, jm + 2, km + 2]
                    dl = c1[1:] - c0[1:]
                    dlr = np.sqrt(dl[0] * dl[0] + dl[1] * dl[1] + dl[2] * dl[2])
                    G = []
                    for lv, l in ((4, 5), (5, 6)):
                        gt = [0.5 * (g[c][im, jm, km, lv] + g[c][i, j, k, lv]) for c in range(3)]
                        dv = P(q, i, j, k)[l] - P(q, im, jm, km)[l]
                        nc = (dv - (gt[0] * dl[0] + gt[1] * dl[1] + gt[2] * dl[2])) / dlr
                        G.append([gt[c] + (nc * dl[c] / dlr) for c in range(3)])
                    muf = 0.5 * (P(mu, im, jm, km) + P(mu, i, j, k))
                    mutf = 0.5 * (P(mut, im, jm, km) + P(mut, i, j, k))
                    A, nx, ny, nz = fa[:, i + 2, j + 2, k + 2]
                    dk = G[0][0] * nx + G[0][1] * ny + G[0][2] * nz
                    dkl = G[1][0] * nx + G[1][1] * ny + G[1][2] * nz
                    want6 = -(A * ((muf + SK * mutf) * dk))
                    want7 = -(A * ((muf + SP * mutf) * dkl))
                    for l, want in ((5, want6), (6, want7)):
                        got = blk[n][i - 1, j - 1, k - 1, l] - F0[n][i - 1, j - 1, k - 1, l]
                        tol = 1e-12 * abs(want) + 4e-16 * abs(F0[n][i - 1, j - 1, k - 1, l])
                        assert abs(got - want) <= tol, (n, l, i, j, k, got, want)


def test_kkl_source():
    ext, flow, blk = kkl_block()
    blk.compute_residue()
    r0 = np.array(blk["residue"][..., 5:7])
    blk.add_source_term_residue()
    dS = blk["residue"][..., 5:7] - r0
    q, mu, mut, dist, cells = blk["qp"], blk["mu"], blk["mu_t"], blk["dist"], blk["cells"]
    If, Jf, Kf = blk["Ifaces"], blk["Jfaces"], blk["Kfaces"]
    g = [blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]]
    for k in range(1, ext.kmx):
        for j in range(1, ext.jmx):
            for i in range(1, ext.imx):
                rho, tk, tkl = P(q, i, j, k)[0], P(q, i, j, k)[5], P(q, i, j, k)[6]
                gv = np.array([[g[c][i, j, k, a] for c in range(3)] for a in range(3)])  # gv[a, c] = d u_a / d x_c
                S = 0.5 * (gv + gv.T)
                delv = gv[0, 0] + gv[1, 1] + gv[2, 2]
                mt = P(mut, i, j, k)
                Tau = mt * 2 * S
                for a in range(3):
                    Tau[a, a] = mt * (2 * S[a, a] - (2.0 / 3.0) * delv) - (2.0 / 3.0) * rho * tk
                Pk = float(np.sum(Tau * gv))
                Dk = CMU ** 0.75 * rho * tk ** 2.5 / max(tkl, 1e-20)
                Pk = min(Pk, 20 * Dk)
                fr = [If[:, i + 2, j + 2, k + 2], Jf[:, i + 2, j + 2, k + 2], Kf[:, i + 2, j + 2, k + 2],
                      If[:, i + 3, j + 2, k + 2], Jf[:, i + 2, j + 3, k + 2], Kf[:, i + 2, j + 2, k + 3]]
                nb = [(i - 1, j, k), (i, j - 1, k), (i, j, k - 1), (i + 1, j, k), (i, j + 1, k), (i, j, k + 1)]
                vol = cells[0, i + 2, j + 2, k + 2]
                lap = []
                for a in range(3):
                    tot = 0.0
                    for c in range(3):
                        gc = g[c][i, j, k, a]
                        t = sum((1 if f >= 3 else -1) * (g[c][nb[f] + (a,)] + gc) * fr[f][1 + c] * fr[f][0]
                                for f in range(6))
                        tot += t / (2 * vol)
                    lap.append(tot)
                udd = np.sqrt(lap[0] ** 2 + lap[1] ** 2 + lap[2] ** 2)
                ud = np.sqrt(2 * np.sum(S * S))
                lvk = KAP * abs(ud / max(udd, 1e-20))
                fp = min(max(Pk / Dk, 0.5), 1.0)
                d, m = P(dist, i, j, k), P(mu, i, j, k)
                lvk = max(lvk, tkl / max(tk * C11, 1e-20))
                lvk = min(lvk, C12 * KAP * d * fp)
                eta = rho * d * np.sqrt(0.3 * tk) / (20 * m)
                fphi = (1 + CD1 * eta) / (1 + eta ** 4)
                cphi1 = Z1 - Z2 * (tkl / max(tk * lvk, 1e-20)) ** 2
                Pkl = cphi1 * tkl * Pk / max(tk, 1e-20)
                Dkl = Z3 * rho * tk ** 1.5
                Sk = (Pk - Dk - 2 * m * tk / d ** 2) * vol
                Skl = (Pkl - Dkl - 6 * m * tkl * fphi / d ** 2) * vol
                scale_k = max(abs(Pk), abs(Dk), abs(2 * m * tk / d ** 2)) * vol
                scale_l = max(abs(Pkl), abs(Dkl), abs(6 * m * tkl * fphi / d ** 2)) * vol
                assert abs(dS[i - 1, j - 1, k - 1, 0] + Sk) <= 1e-11 * scale_k, (i, j, k, dS[i - 1, j - 1, k - 1, 0], -Sk)
                assert abs(dS[i - 1, j - 1, k - 1, 1] + Skl) <= 1e-11 * scale_l, (i, j, k, dS[i - 1, j - 1, k - 1, 1], -Skl)


def test_kkl_point_implicit_update_and_norm():
    ext, flow, blk = kkl_block()
    blk.compute_time_step(0.5)
    q0 = np.array(blk["qp"])
    R = np.array(blk["residue"])
    mu, dist, cells, dt = blk["mu"], blk["dist"], blk["cells"], blk["delta_t"]
    assert blk.update_with(1.0, 0.0) == 0
    q1 = blk["qp"]
    for k in range(1, ext.kmx):
        for j in range(1, ext.jmx):
            for i in range(1, ext.imx):
                rho = P(q0, i, j, k)[0]
                u6, u7 = P(q0, i, j, k)[5] * rho, P(q0, i, j, k)[6] * rho
                d, m = P(dist, i, j, k), P(mu, i, j, k)
                dtc = dt[i - 1, j - 1, k - 1]
                eta = rho * d * (np.sqrt(0.3 * u6) / (20 * m))
                fphi = (1 + CD1 * eta) / (1 + eta ** 4)
                R6 = R[i - 1, j - 1, k - 1, 5] / (1. + ((2.5 * (CMU ** 0.75 * np.sqrt(rho) * u6 ** 1.5 / max(u7, 1e-20)))
                                                       + (2 * m / d ** 2)) * dtc)
                R7 = R[i - 1, j - 1, k - 1, 6] / (1. + (6 * m * fphi / d ** 2) * dtc)
                fac = dtc / cells[0, i + 2, j + 2, k + 2]
                r2 = rho - R[i - 1, j - 1, k - 1, 0] * fac
                for l, uu, RR in ((5, u6, R6), (6, u7, R7)):
                    new = (uu - RR * fac) / r2
                    want = new if new >= 0 else P(q0, i, j, k)[l]
                    got = P(q1, i, j, k)[l]
                    assert abs(got - want) <= 1e-12 * abs(want), (l, i, j, k, got, want)
    norm = O.find_resnorm([blk])
    sl = (slice(0, ext.imx - 1), slice(0, ext.jmx - 1), slice(0, ext.kmx - 1))
    for l, inf in ((6, flow.tk_inf), (7, flow.tkl_inf)):
        scale = flow.density_inf * flow.vel_mag * inf
        want = np.sqrt(np.sum((blk["residue"][sl + (l - 1,)] / scale) ** 2))
        assert abs(norm[l] - want) <= 1e-12 * want
