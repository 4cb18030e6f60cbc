"""The fixed-point adjoint (fest_adjoint_solve) on the smooth-bump channel:
wall-force sensitivities to the inflow Mach number and angle against
central finite differences of re-converged FP64 primal solutions.

Reduced grid (64x24x4 cells) and the first-order scheme, whose explicit
iteration converges to a 1e-10 drop within seconds (the second-order
scheme's explicit iteration needs far longer on this case; its residual
Jacobian is checked against finite differences in test_gpu_adjoint.py).
Nine primal solves and one adjoint solve, each to a 1e-10 drop; agreement
to 1e-4 relative for the inflow Mach number, the inflow angle and two
lower-wall node displacements (grid deformed by linear blending to the top
wall)."""
import numpy as np
import pytest

from fest3d import adjoint as A

pytestmark = pytest.mark.gpu


def test_wall_force_study_at_the_configuration_size(gpu_lib):
    """The configuration itself: the 128x48x4 bump with unlimited MUSCL +
    SLAU, the primal converged to a 1e-12 drop (Anderson-accelerated
    explicit iterations), the adjoint to a 1e-10 drop (GMRES over the
    fixed-point adjoint iteration); the inflow Mach number and the two
    largest wall-node gradients (the inlet corner and the bump's flank)
    against central differences (step 1e-6) of re-converged primal
    solutions, to 2e-4.  The full run over all 128 nodes is committed with
    its command line (bench.py --adjoint-study)."""
    out = A.wall_force_study(gpu_lib, wall_nodes=(1, 65), params=("mach",), threads=3)
    assert out["primal"]["drop"] <= 1e-12
    assert out["adjoint"]["drop"] <= 1e-10
    for r in out["rows"]:
        assert r["rel_diff"] <= 2e-4, r


def test_bump_wall_force_sensitivities(gpu_lib):
    case = A.adjoint_case(nc=(64, 24, 4), interpolant="none")
    h = A.make_handle(case, lib=gpu_lib)
    q, it, drop, ref = A.converge(h, case["qp"], case["CFL"], tol=1e-10)
    assert drop <= 1e-10
    wall_nodes = (20, 33)  # on the bump's flank and near its crest
    grads, J, n, adrop = A.sensitivities(case, q, it, wall_nodes=wall_nodes, tol=1e-10, lib=gpu_lib)
    assert adrop <= 1e-10, (n, adrop)
    Jf = h.get("Jfaces")
    for param, step in (("mach", 1e-4), ("angle", 1e-2)):
        vals = []
        for sgn in (1, -1):
            c2 = dict(case)
            c2[param] = case[param] + sgn * step
            c2["flow"] = A.bump_flow(c2["mach"], c2["angle"])
            c2["bc"] = A.bump_bc(c2["mach"])
            hp = A.make_handle(c2, lib=gpu_lib)
            qs, _, d2, _ = A.converge(hp, q, case["CFL"], first_iter=it, tol=1e-10, ref=ref)
            assert d2 <= 1e-10
            vals.append(A.wall_force(qs, case["ext"], Jf)[0])
            hp.close()
        fd = (vals[0] - vals[1]) / (2 * step)
        assert abs(fd - grads[param]) <= 1e-4 * max(abs(fd), 1e-6 * abs(J)), (param, fd, grads[param])
    # lower-wall node displacements (grid deformed by linear blending)
    for i in wall_nodes:
        step = 1e-6
        vals = []
        for sgn in (1, -1):
            c2 = dict(case)
            c2["nodes"] = A.displaced_nodes(case, i, sgn * step)
            hp = A.make_handle(c2, lib=gpu_lib)
            qs, _, d2, _ = A.converge(hp, q, case["CFL"], first_iter=it, tol=1e-10, ref=ref)
            assert d2 <= 1e-10
            vals.append(A.wall_force(qs, case["ext"], hp.get("Jfaces"))[0])
            hp.close()
        fd = (vals[0] - vals[1]) / (2 * step)
        g = grads[f"wall_node_{i}"]
        assert abs(fd - g) <= 1e-4 * max(abs(fd), 1e-3 * abs(J)), (i, fd, g)


def test_laminar_adjoint_solve_satisfies_the_adjoint_equation(gpu_lib):
    """fest_adjoint_solve on a laminar bump (no-slip adiabatic walls,
    Reynolds number ~ 2000 on the channel height, first-order SLAU, forward
    Euler) after 3000 primal iterations: the fixed point psi satisfies
    (dR/dq)^T psi = -dJ/dq, checked with fest_residual_vjp on every
    interior cell (the iteration needs a contractive linearised step, not a
    converged primal)."""
    case = A.adjoint_case(nc=(48, 16, 4), interpolant="none", mu_ref=0.1, integrator="none", CFL=0.5)
    h = A.make_handle(case, lib=gpu_lib)
    h.upload_state(case["qp"])
    h.step(3000, 1, case["CFL"], with_norm=False)
    q = h.download_state()
    ext = case["ext"]
    J, dJ = A.wall_force(q, ext, h.get("Jfaces"))
    psi, n, drop = h.adjoint_solve(dJ, case["CFL"], max_iters=100000, tol=1e-10)
    assert drop <= 1e-10, (n, drop)
    back = h.residual_vjp(q, 3, psi)
    sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
    err = np.abs(back[sl] + dJ[sl]).max() / np.abs(dJ[sl]).max()
    assert err <= 1e-6, (err, n)


def test_sst_adjoint_solve_satisfies_the_adjoint_equation(gpu_lib):
    """fest_adjoint_solve on a k-omega SST block (no-slip wall, slip wall,
    subsonic inlet and outlet, periodic k faces; first-order AUSM, forward
    Euler, local time steps) after 300 primal iterations from a random
    state: the pseudo-time preconditioner maps all seven variables (k and
    omega through U/rho, divided by the update's point-implicit destruction
    factors), and the fixed point psi satisfies (dR/dq)^T psi = -dJ/dq for
    a random dJ/dq, checked with fest_residual_vjp on every interior cell."""
    from parity import make_pair, small_case
    from fest3d import cases
    ext, flow, scheme, bc, nodes, qp = small_case(
        nc=(12, 8, 6), turb=True, ids=(-3, -4, -5, -6, -10, -10),
        scheme_kw=dict(interpolant="none", scheme_name="ausm"),
        flow_kw=dict(mu_ref=0.3, mu_variation="sutherland_law"))
    _, h = make_pair(ext, flow, scheme, bc, nodes, qp, wall=cases.wall_nodes_of(nodes, ext, bc))
    CFL = 0.5
    h.step(300, 1, CFL, with_norm=False)
    q = h.download_state()
    dJ = np.zeros(q.shape, order="F")
    sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
    dJ[sl] = np.random.default_rng(21).standard_normal(q[sl].shape)
    psi, n, drop = h.adjoint_solve(dJ, CFL, max_iters=100000, tol=1e-10)
    assert drop <= 1e-10, (n, drop)
    back = h.residual_vjp(q, 3, psi)
    err = np.abs(back[sl] + dJ[sl]).max() / np.abs(dJ[sl]).max()
    assert err <= 1e-6, (err, n)
    h.close()
