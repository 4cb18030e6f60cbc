"""fest_residual_vjp: the transposed-Jacobian product of the inviscid and
laminar residual, checked against central finite differences of the oracle's FP64
residual (get_total_conservative_Residue, update.f90:495-547, at iteration 3
so that no fix() BC writes), and wrapped in a torch.autograd.Function for
torch.autograd.gradcheck.

Finite-difference directions perturb 24 random interior cells (the ghost
cells follow through the BCs in both codes) with steps of 1e-6 and 2e-7 of
each variable's magnitude in a fourth-order central stencil.  Limited MUSCL
(Koren) and PPM are piecewise: a direction whose two difference quotients
disagree has a limiter kink within the step and says nothing about the
derivative, so it is skipped; every other direction must match the adjoint
to 1e-5, and at least three of six must be usable."""
import numpy as np
import pytest

import oracle as O
from fest3d import abi
from parity import make_pair, small_case

pytestmark = pytest.mark.gpu

CASES = {
    "weno-slau": dict(scheme_kw=dict(interpolant="weno", scheme_name="slau"),
                      ids=(-11, -4, -6, -6, -10, -10)),
    "muscl-slau": dict(scheme_kw=dict(interpolant="muscl", scheme_name="slau"),
                       ids=(-11, -4, -6, -6, -10, -10)),
    # speeds up to 1.6 c: the capped Mach number and the supersonic
    # branches of the SLAU reverse sweep
    "muscl-slau-supersonic": dict(scheme_kw=dict(interpolant="muscl", scheme_name="slau"),
                                  ids=(-1, -2, -6, -5, -10, -10), state_mach=1.6),
    "muscl-ausm-wall": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausm"),
                            ids=(-3, -4, -5, -6, -10, -10)),
    "ppm-ausmP": dict(scheme_kw=dict(interpolant="ppm", scheme_name="ausmP"),
                      ids=(-3, -4, -5, -6, -6, -6)),
    "wenoNM-ausmUP": dict(scheme_kw=dict(interpolant="weno_NM", scheme_name="ausmUP"),
                          ids=(-8, -2, -6, -6, -10, -10), flow_kw=dict(MInf=0.3)),
    "none-vanleer": dict(scheme_kw=dict(interpolant="none", scheme_name="van_leer"),
                         ids=(-1, -4, -6, -6, -10, -10)),
    "muscl-ldfss-vanalbada": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ldfss0",
                                                 limiter="van_albada"),
                                  ids=(-3, -4, -6, -5, -10, -10)),
}
IT = 3


def interior_mask(ext):
    m = np.zeros((ext.imx + 5, ext.jmx + 5, ext.kmx + 5, 1))
    m[3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2] = 1.0
    return m


def var_scale(qp, ext):
    inner = qp[3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2]
    s = np.abs(inner).reshape(-1, ext.n_var).max(axis=0)
    s[1:4] = max(s[1:4].max(), 1.0)  # velocities share one scale
    return s


@pytest.mark.parametrize("name", list(CASES))
def test_vjp_matches_oracle_finite_differences(gpu_lib, name):
    ext, flow, scheme, bc, nodes, qp = small_case(nc=(12, 9, 7), **CASES[name])
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    rng = np.random.default_rng(11)
    lam = np.asfortranarray(rng.standard_normal((ext.imx - 1, ext.jmx - 1, ext.kmx - 1, ext.n_var)))
    dq = h.residual_vjp(qp, IT, lam)
    mask = interior_mask(ext)
    assert np.all(dq * (1 - mask) == 0), "ghost entries of dq must be zero"
    scale = var_scale(qp, ext)

    def phi(q):
        blk["qp"] = np.asfortranarray(q)
        assert O.get_total_conservative_residue([blk], IT) == 0
        return float(np.sum(lam * blk["residue"]))

    def fd(v, e):
        return (8 * (phi(qp + e * v) - phi(qp - e * v)) - (phi(qp + 2 * e * v) - phi(qp - 2 * e * v))) / (12 * e)

    inner = np.argwhere(mask[..., 0] > 0)
    usable = 0
    for trial in range(6):
        v = np.zeros(qp.shape)
        for i, j, k in inner[rng.choice(len(inner), 24, replace=False)]:
            v[i, j, k] = rng.standard_normal(ext.n_var) * scale
        f1, f2 = fd(v, 1e-6), fd(v, 2e-7)
        if abs(f1 - f2) > 1e-6 * max(abs(f1), abs(f2)):
            continue  # a limiter kink inside the step
        ad = float(np.sum(dq * v))
        assert abs(f1 - ad) <= 1e-5 * max(abs(f1), abs(ad)), (name, trial, f1, f2, ad)
        usable += 1
    assert usable >= 3, f"{name}: only {usable} kink-free directions"


# laminar blocks: the viscous face terms (viscous.f90:144-325) through the
# Green-Gauss gradients and their BCs (gradients.f90:276-676) and the
# viscosity (viscosity.f90:109-136), with the temperature p/(rho R) of the
# state; viscosities large enough that the viscous terms are a sizeable
# part of the residual
VISC_CASES = {
    "lam-muscl-ausm-walls": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausm"),
                                 ids=(-3, -4, -5, -6, -10, -10),
                                 flow_kw=dict(mu_ref=1.0, mu_variation="constant")),
    "suth-weno-slau-riemann": dict(scheme_kw=dict(interpolant="weno", scheme_name="slau"),
                                   ids=(-11, -4, -5, -5, -10, -10),
                                   flow_kw=dict(mu_ref=0.5, mu_variation="sutherland_law")),
    "suth-none-vanleer-farfield": dict(scheme_kw=dict(interpolant="none", scheme_name="van_leer"),
                                       ids=(-8, -2, -6, -5, -6, -6),
                                       flow_kw=dict(mu_ref=0.5, mu_variation="sutherland_law")),
}


@pytest.mark.parametrize("name", list(VISC_CASES))
def test_viscous_vjp_matches_oracle_finite_differences(gpu_lib, name):
    ext, flow, scheme, bc, nodes, qp = small_case(nc=(10, 8, 6), **VISC_CASES[name])
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    rng = np.random.default_rng(13)
    lam = np.asfortranarray(rng.standard_normal((ext.imx - 1, ext.jmx - 1, ext.kmx - 1, ext.n_var)))
    dq = h.residual_vjp(qp, IT, lam)
    mask = interior_mask(ext)
    assert np.all(dq * (1 - mask) == 0), "ghost entries of dq must be zero"
    scale = var_scale(qp, ext)

    def phi(q):
        # ghosts of this state first, then its temperature, then the residual
        blk["qp"] = np.asfortranarray(q)
        assert O.get_total_conservative_residue([blk], IT) == 0
        blk.compute_temperature()
        assert O.get_total_conservative_residue([blk], IT) == 0
        return float(np.sum(lam * blk["residue"]))

    def fd(v, e):
        return (8 * (phi(qp + e * v) - phi(qp - e * v)) - (phi(qp + 2 * e * v) - phi(qp - 2 * e * v))) / (12 * e)

    inner = np.argwhere(mask[..., 0] > 0)
    usable = 0
    for trial in range(6):
        v = np.zeros(qp.shape)
        for i, j, k in inner[rng.choice(len(inner), 24, replace=False)]:
            v[i, j, k] = rng.standard_normal(ext.n_var) * scale
        f1, f2 = fd(v, 1e-6), fd(v, 2e-7)
        if abs(f1 - f2) > 1e-6 * max(abs(f1), abs(f2)):
            continue  # a limiter kink inside the step
        ad = float(np.sum(dq * v))
        assert abs(f1 - ad) <= 1e-5 * max(abs(f1), abs(ad)), (name, trial, f1, f2, ad)
        usable += 1
    assert usable >= 3, f"{name}: only {usable} kink-free directions"


# k-omega SST blocks: convective fluxes of seven variables, the viscous
# terms with the eddy viscosity and the k, omega diffusion (viscous.f90:
# 144-447), the eddy viscosity and F1 of every cell from its state and
# gradient (viscosity.f90:215-546), the source (source.f90:158-270), the
# gradients of u, v, w, T, k, omega with their BCs, and the ghost cells of
# k and omega (wall omega of bc_primitive.f90:564-643); wall distances of a
# wall face, molecular viscosity large enough that every term counts
SST_CASES = {
    "sst-muscl-ausmUP-walls": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausmUP",
                                                  turbulence="sst"),
                                   ids=(-3, -4, -5, -6, -10, -10),
                                   flow_kw=dict(mu_ref=0.3, mu_variation="sutherland_law", MInf=0.3)),
    "sst-weno-slau-outlets": dict(scheme_kw=dict(interpolant="weno", scheme_name="slau", turbulence="sst"),
                                  ids=(-3, -4, -6, -5, -10, -10),
                                  flow_kw=dict(mu_ref=0.3, mu_variation="constant")),
    "sst2003-none-ausm-supersonic": dict(scheme_kw=dict(interpolant="none", scheme_name="ausm",
                                                        turbulence="sst2003"),
                                         ids=(-1, -2, -5, -5, -6, -6),
                                         flow_kw=dict(mu_ref=0.3, mu_variation="sutherland_law")),
}


@pytest.mark.parametrize("name", list(SST_CASES))
def test_sst_vjp_matches_oracle_finite_differences(gpu_lib, name):
    from fest3d import cases
    kw = dict(SST_CASES[name])
    ext, flow, scheme, bc, nodes, qp = small_case(nc=(10, 8, 6), turb=True, **kw)
    wall = cases.wall_nodes_of(nodes, ext, bc)
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp, wall=wall)
    rng = np.random.default_rng(17)
    lam = np.asfortranarray(rng.standard_normal((ext.imx - 1, ext.jmx - 1, ext.kmx - 1, ext.n_var)))
    dq = h.residual_vjp(qp, IT, lam)
    mask = interior_mask(ext)
    assert np.all(dq * (1 - mask) == 0), "ghost entries of dq must be zero"
    scale = var_scale(qp, ext)

    def phi(q):
        blk["qp"] = np.asfortranarray(q)
        assert O.get_total_conservative_residue([blk], IT) == 0
        blk.compute_temperature()
        assert O.get_total_conservative_residue([blk], IT) == 0
        return float(np.sum(lam * blk["residue"]))

    def fd(v, e):
        return (8 * (phi(qp + e * v) - phi(qp - e * v)) - (phi(qp + 2 * e * v) - phi(qp - 2 * e * v))) / (12 * e)

    inner = np.argwhere(mask[..., 0] > 0)
    usable = 0
    for trial in range(8):
        v = np.zeros(qp.shape)
        for i, j, k in inner[rng.choice(len(inner), 24, replace=False)]:
            v[i, j, k] = rng.standard_normal(ext.n_var) * scale
        f1, f2 = fd(v, 1e-6), fd(v, 2e-7)
        if abs(f1 - f2) > 1e-6 * max(abs(f1), abs(f2)):
            continue  # a min/max switch inside the step
        ad = float(np.sum(dq * v))
        assert abs(f1 - ad) <= 1e-5 * max(abs(f1), abs(ad)), (name, trial, f1, f2, ad)
        usable += 1
    assert usable >= 3, f"{name}: only {usable} kink-free directions"


def test_vjp_rejects_unsupported_blocks(gpu_lib):
    """SST blocks with far-field faces have no residual VJP; SST blocks no
    metric VJP."""
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(12, 9, 7), ids=(-8, -4, -5, -6, -10, -10), turb=True,
        flow_kw=dict(mu_ref=1e-2, mu_variation="constant"))
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    lam = np.zeros((ext.imx - 1, ext.jmx - 1, ext.kmx - 1, ext.n_var), order="F")
    with pytest.raises(abi.FestError) as e:
        h.residual_vjp(qp, IT, lam)
    assert e.value.code == abi.FEST_ERR_ARG
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(12, 9, 7), ids=(-3, -4, -5, -6, -10, -10), turb=True,
        flow_kw=dict(mu_ref=1e-2, mu_variation="constant"))
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    lam = np.zeros((ext.imx - 1, ext.jmx - 1, ext.kmx - 1, ext.n_var), order="F")
    with pytest.raises(abi.FestError) as e:
        h.residual_vjp_nodes(qp, IT, lam)
    assert e.value.code == abi.FEST_ERR_ARG


def test_autograd_function_gradcheck(gpu_lib):
    """the residual (fest_get_total_conservative_residue) and its VJP as a
    torch.autograd.Function over the scaled interior state; verification
    only - nothing in the library goes through torch.  The adjoint sums face
    contributions with FP64 atomic adds, whose order varies from run to run:
    repeated backward passes agree to rounding (nondet_tol).  fast_mode
    compares u^T J v for random u, v (one backward, one directional
    difference), which keeps the O(eps^2) truncation of the difference
    quotient relative to the whole product rather than to single small
    Jacobian entries."""
    import torch
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(5, 4, 4), scheme_kw=dict(interpolant="weno", scheme_name="slau"),
        ids=(-11, -4, -6, -6, -10, -10))
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    scale = var_scale(qp, ext)
    sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
    base = np.array(qp, order="F")

    def full_state(x):  # scaled interior -> padded state
        q = base.copy(order="F")
        q[sl] = x * scale
        return q

    class Residual(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            xn = x.detach().cpu().numpy()
            q, r = h.residual(full_state(xn), IT)
            ctx.save_for_backward(x)
            return torch.from_numpy(np.ascontiguousarray(r))

        @staticmethod
        def backward(ctx, g):
            (x,) = ctx.saved_tensors
            lam = np.asfortranarray(g.detach().cpu().numpy())
            dq = h.residual_vjp(full_state(x.detach().cpu().numpy()), IT, lam)
            return torch.from_numpy(np.ascontiguousarray(dq[sl] * scale))

    x0 = torch.tensor(np.ascontiguousarray(qp[sl] / scale), dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(Residual.apply, (x0,), eps=1e-6, atol=1e-6, rtol=1e-4,
                                     nondet_tol=1e-9, fast_mode=True)


NODE_CASES = {
    "weno-slau": CASES["weno-slau"],
    "muscl-ausm-wall-nolim": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausm",
                                                 ilimiter_switch=0, jlimiter_switch=0,
                                                 klimiter_switch=0),
                                  ids=(-3, -4, -5, -6, -10, -10)),
    "none-vanleer": CASES["none-vanleer"],
    # laminar: face records, volumes and centres in the Green-Gauss
    # gradients, their wall and outlet BCs and the viscous fluxes
    "lam-muscl-ausm-walls-nolim": dict(scheme_kw=dict(interpolant="muscl", scheme_name="ausm",
                                                      ilimiter_switch=0, jlimiter_switch=0,
                                                      klimiter_switch=0),
                                       ids=(-3, -4, -5, -6, -10, -10),
                                       flow_kw=dict(mu_ref=1.0, mu_variation="constant")),
    "suth-none-vanleer-farfield": VISC_CASES["suth-none-vanleer-farfield"],
}


@pytest.mark.parametrize("name", list(NODE_CASES))
def test_node_vjp_matches_oracle_finite_differences(gpu_lib, name):
    """(dR/dnodes)^T lambda + (dfaces/dnodes)^T w against central
    differences of the oracle (geometry rebuilt from perturbed interior
    nodes, residual at fixed state) for random lambda and face weights w;
    laminar blocks with the temperature of the state, as the state VJP."""
    ext, flow, scheme, bc, nodes, qp = small_case(nc=(12, 9, 7), **NODE_CASES[name])
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    rng = np.random.default_rng(5)
    lam = np.asfortranarray(rng.standard_normal((ext.imx - 1, ext.jmx - 1, ext.kmx - 1, ext.n_var)))
    w = [np.asfortranarray(rng.standard_normal(blk[nm].shape)) for nm in ("Ifaces", "Jfaces", "Kfaces")]
    dn = h.residual_vjp_nodes(qp, IT, lam, w)
    inner = np.zeros(nodes.shape)
    inner[:, 3:ext.imx + 3, 3:ext.jmx + 3, 3:ext.kmx + 3] = 1.0
    assert np.all(dn * (1 - inner) == 0), "ghost nodes carry no adjoint"

    def phi(nd):
        blk["nodes"] = np.asfortranarray(nd)
        blk.setup_geometry()
        blk["qp"] = qp
        assert O.get_total_conservative_residue([blk], IT) == 0
        if flow.mu_ref != 0.0:
            blk.compute_temperature()
            assert O.get_total_conservative_residue([blk], IT) == 0
        return float(np.sum(lam * blk["residue"])) + sum(
            float(np.sum(wf * blk[nm])) for wf, nm in zip(w, ("Ifaces", "Jfaces", "Kfaces")))

    spacing = 1.0 / max(ext.imx, ext.jmx, ext.kmx)
    for trial in range(3):
        v = rng.standard_normal(nodes.shape) * inner * spacing
        e = 1e-6
        fd = (8 * (phi(nodes + e * v) - phi(nodes - e * v)) - (phi(nodes + 2 * e * v) - phi(nodes - 2 * e * v))) / (12 * e)
        ad = float(np.sum(dn * v))
        assert abs(fd - ad) <= 1e-5 * max(abs(fd), abs(ad)), (name, trial, fd, ad)
