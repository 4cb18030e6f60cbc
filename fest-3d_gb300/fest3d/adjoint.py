"""Wall-force sensitivities of the smooth-bump channel by the discrete adjoint.

The objective is the x-component of the pressure force on the lower wall,
J = sum over the j=1 J-faces of p(i,1,k) * nx * A (the first cell row's
pressure, as the reference's post-processing reads wall pressure).  With the
primal converged (R(q*, alpha) = 0), fest_adjoint_solve returns psi with
(dR/dq)^T psi = -dJ/dq, and dJ/dalpha = psi . dR/dalpha at fixed q* for a
flow parameter alpha (inflow Mach number, inflow angle).  dR/dalpha is the
residual's change through the inlet BC; it is taken here by a central
difference of two residual evaluations at the frozen state.

Everything runs through the C ABI (include/fest_gpu.h) in FP64.
"""
import numpy as np

from . import abi, cases
from .handle import Handle


def bump_flow(mach, angle_deg=0.0, p0=101325.0, rho0=1.2, gm=1.4):
    c = np.sqrt(gm * p0 / rho0)
    a = np.deg2rad(angle_deg)
    return abi.make_flow(density_inf=rho0, x_speed_inf=mach * c * np.cos(a),
                         y_speed_inf=mach * c * np.sin(a), pressure_inf=p0, mu_ref=0.0)


def bump_bc(mach, p0=101325.0, gm=1.4):
    pt = p0 * (1 + 0.5 * (gm - 1) * mach * mach) ** (gm / (gm - 1))
    fixed = {k: [0.0] * 6 for k in ("fixed_pressure", "fixed_Tpressure")}
    fixed["fixed_pressure"][1] = p0
    fixed["fixed_Tpressure"][0] = pt
    return abi.make_bc([-11, -4, -6, -6, -10, -10], partners={4: (0, 5), 5: (0, 4)}, **fixed)


def adjoint_case(nc=(128, 48, 4), mach=0.5, angle_deg=0.0, interpolant="muscl"):
    """The bump at 128x48x4 cells, Euler, unlimited MUSCL (kappa 1/3) + SLAU,
    TVD-RK3 with local time steps at CFL 0.8 (the smooth subsonic flow needs
    no limiter, which keeps the residual differentiable; forward Euler is
    unstable with unlimited MUSCL).  interpolant="none" gives the
    first-order scheme, whose explicit iteration converges to round-off
    within a few 10^4 iterations (the second-order one drops by only ~20
    in 4*10^4 on this grid, identically in the oracle)."""
    ext = abi.Extent(nc[0] + 1, nc[1] + 1, nc[2] + 1, 5)
    scheme = abi.make_scheme(scheme_name="slau", interpolant=interpolant, time_step_accuracy="TVDRK3",
                             time_stepping_method="l", ilimiter_switch=0, jlimiter_switch=0,
                             klimiter_switch=0)
    flow = bump_flow(mach, angle_deg)
    return dict(ext=ext, flow=flow, scheme=scheme, bc=bump_bc(mach), nodes=cases.bump_nodes(ext),
                qp=cases.uniform_state(ext, flow), CFL=0.8, mach=mach, angle=angle_deg)


def make_handle(case, flow=None, bc=None, lib=None):
    h = Handle(case["ext"], flow or case["flow"], case["scheme"], bc or case["bc"], lib=lib)
    h.setup_geometry(case["nodes"])
    h.set_precision(abi.FEST_FP64)
    return h


def converge(h, q, CFL, first_iter=1, tol=1e-12, max_iters=200000, chunk=500, ref=None):
    """Iterate from state q until the L2 norm of the mass residual has
    dropped by tol relative to ref (default: its value after the first
    chunk); returns the state, the next iteration number, the achieved drop
    and ref."""
    h.upload_state(q)
    it = first_iter
    drop = 1.0
    while it - first_iter < max_iters:
        norm = h.step(chunk, it, CFL)
        it += chunk
        r = float(norm[1])
        ref = r if ref is None else ref
        drop = r / ref if ref > 0 else 0.0
        if not np.isfinite(r):
            raise FloatingPointError("primal diverged")
        if drop <= tol:
            break
    return h.download_state(), it, drop, ref


def wall_force(q, ext, Jfaces):
    """J = sum_{i,k} p(i,1,k) nx A over the lower-wall J-faces, and dJ/dq
    in the qp layout."""
    p = q[3:ext.imx + 2, 3, 3:ext.kmx + 2, 4]            # cells (1..imx-1, 1, 1..kmx-1)
    jf = Jfaces[:, 3:ext.imx + 2, 3, 3:ext.kmx + 2]      # faces (i, 1, k): {A, nx, ny, nz}
    w = jf[1] * jf[0]
    dJ = np.zeros_like(q)
    dJ[3:ext.imx + 2, 3, 3:ext.kmx + 2, 4] = w
    return float(np.sum(p * w)), dJ


def residual_param_derivative(case, q, it, param, h_rel=1e-6, lib=None):
    """dR/dalpha at fixed q by a central difference over the flow parameter
    (param 'mach' or 'angle', in the units of the case)."""
    a0 = case[param]
    step = h_rel * max(abs(a0), 1.0)
    out = []
    for a in (a0 + step, a0 - step):
        mach = a if param == "mach" else case["mach"]
        ang = a if param == "angle" else case["angle"]
        hp = make_handle(case, flow=bump_flow(mach, ang), bc=bump_bc(mach), lib=lib)
        _, r = hp.residual(q, it)
        out.append(r)
        hp.close()
    return (out[0] - out[1]) / (2 * step)


def wall_force_faces_bar(q, ext, Jfaces):
    """dJ/dJfaces of J = sum p nx A (J-face layout, zero elsewhere)."""
    bar = np.zeros_like(Jfaces)
    p = q[3:ext.imx + 2, 3, 3:ext.kmx + 2, 4]
    bar[0, 3:ext.imx + 2, 3, 3:ext.kmx + 2] = p * Jfaces[1, 3:ext.imx + 2, 3, 3:ext.kmx + 2]
    bar[1, 3:ext.imx + 2, 3, 3:ext.kmx + 2] = p * Jfaces[0, 3:ext.imx + 2, 3, 3:ext.kmx + 2]
    return bar


def wall_blend(ext):
    """Weight (1 - t_j) of a lower-wall node displacement at node row j
    (linear blending to the fixed top wall in the bump grid's j spacing)."""
    r = 1.02 ** np.arange(ext.jmx - 1)
    t = np.concatenate([[0.0], np.cumsum(r)])
    return 1.0 - t / t[-1]


def displaced_nodes(case, i, delta):
    """The bump grid with lower-wall node i (1..imx) moved by delta in y,
    blended linearly to the top wall."""
    ext = case["ext"]
    nodes = np.array(case["nodes"], order="F")
    nodes[1, i + 2, 3:ext.jmx + 3, 3:ext.kmx + 3] += delta * wall_blend(ext)[:, None]
    return nodes


def sensitivities(case, q, it, params=("mach", "angle"), wall_nodes=(), tol=1e-10,
                  max_iters=200000, lib=None):
    """dJ/dalpha for each flow parameter and dJ/d(delta_i) for each listed
    lower-wall node i from one adjoint solve at the converged state q;
    returns ({name: derivative}, J, adjoint iterations, drop)."""
    h = make_handle(case, lib=lib)
    h.upload_state(q)
    Jf = h.get("Jfaces")
    J, dJ = wall_force(q, case["ext"], Jf)
    psi, n, drop = h.adjoint_solve(dJ, case["CFL"], max_iters, tol)
    grads = {pname: float(np.sum(psi * residual_param_derivative(case, q, it, pname, lib=lib)))
             for pname in params}
    if len(wall_nodes):
        ext = case["ext"]
        dn = h.residual_vjp_nodes(q, it, psi, (None, wall_force_faces_bar(q, ext, Jf), None))
        wgt = wall_blend(ext)
        for i in wall_nodes:
            grads[f"wall_node_{i}"] = float(np.sum(dn[1, i + 2, 3:ext.jmx + 3, 3:ext.kmx + 3] * wgt[:, None]))
    h.close()
    return grads, J, n, drop
