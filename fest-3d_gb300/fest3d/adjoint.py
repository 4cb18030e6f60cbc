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

from . import abi, cases, krylov
from .handle import Handle


def bump_flow(mach, angle_deg=0.0, p0=101325.0, rho0=1.2, gm=1.4, mu_ref=0.0):
    """Free stream of the bump channel; mu_ref > 0: laminar, constant
    viscosity."""
    c = np.sqrt(gm * p0 / rho0)
    a = np.deg2rad(angle_deg)
    return abi.make_flow(density_inf=rho0, x_speed_inf=mach * c * np.cos(a),
                         y_speed_inf=mach * c * np.sin(a), pressure_inf=p0, mu_ref=mu_ref,
                         mu_variation="constant")


def bump_bc(mach, p0=101325.0, gm=1.4, wall=-6):
    """Total-pressure inlet, pressure outlet, lower and upper walls of type
    wall (-6 slip, -5 no-slip adiabatic), periodic k faces."""
    pt = p0 * (1 + 0.5 * (gm - 1) * mach * mach) ** (gm / (gm - 1))
    fixed = {k: [0.0] * 6 for k in ("fixed_pressure", "fixed_Tpressure")}
    fixed["fixed_pressure"][1] = p0
    fixed["fixed_Tpressure"][0] = pt
    return abi.make_bc([-11, -4, wall, wall, -10, -10], partners={4: (0, 5), 5: (0, 4)}, **fixed)


def adjoint_case(nc=(128, 48, 4), mach=0.5, angle_deg=0.0, interpolant="muscl", mu_ref=0.0,
                 integrator="TVDRK3", CFL=0.8):
    """The bump at 128x48x4 cells, Euler, unlimited MUSCL (kappa 1/3) + SLAU,
    TVD-RK3 with local time steps at CFL 0.8 (the smooth subsonic flow needs
    no limiter, which keeps the residual differentiable; forward Euler is
    unstable with unlimited MUSCL).  interpolant="none" gives the
    first-order scheme, whose explicit iteration converges to round-off
    within a few 10^4 iterations (the second-order one drops by only ~20
    in 4*10^4 on this grid, identically in the oracle).  mu_ref > 0: laminar
    with no-slip adiabatic walls."""
    ext = abi.Extent(nc[0] + 1, nc[1] + 1, nc[2] + 1, 5)
    scheme = abi.make_scheme(scheme_name="slau", interpolant=interpolant, time_step_accuracy=integrator,
                             time_stepping_method="l", ilimiter_switch=0, jlimiter_switch=0,
                             klimiter_switch=0)
    flow = bump_flow(mach, angle_deg, mu_ref=mu_ref)
    wall = -5 if mu_ref > 0 else -6
    return dict(ext=ext, flow=flow, scheme=scheme, bc=bump_bc(mach, wall=wall), nodes=cases.bump_nodes(ext),
                qp=cases.uniform_state(ext, flow), CFL=CFL, mach=mach, angle=angle_deg, mu_ref=mu_ref,
                wall=wall)


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


def _flat(a, sl):
    return np.asarray(a[sl]).reshape(-1, order="F")


def state_scale(flow, ext):
    """Per-entry weights of the interior state vector: the free-stream
    density, speed (three components) and pressure."""
    sc = np.array([flow.density_inf, flow.vel_mag, flow.vel_mag, flow.vel_mag, flow.pressure_inf])
    shape = (ext.imx - 1, ext.jmx - 1, ext.kmx - 1, 5)
    return np.broadcast_to(sc, shape).reshape(-1, order="F").copy()


def converge_accelerated(h, q, CFL, first_iter=3, tol=1e-12, ref=None, k=50, m=20, max_maps=4000,
                         flow=None):
    """The steady state from q by Anderson acceleration (fest3d.krylov) of
    k solver iterations (fest_step, the handle's own integrator and
    precision) as the fixed-point map, until the mass-residual norm the
    step reports has dropped by tol relative to ref (default: the norm
    of the first map).  Returns (state, next iteration, drop, ref, maps,
    iterations)."""
    ext = h.ext
    sl = _interior(ext)
    shape = q[sl].shape
    cur = np.array(q, order="F")
    state = {"it": first_iter, "ref": ref}

    def phi(x):
        cur[sl] = x.reshape(shape, order="F")
        h.upload_state(cur)
        norm = h.step(k, state["it"], CFL)
        state["it"] += k
        r = float(norm[1])
        if not np.isfinite(r):
            raise FloatingPointError("primal diverged")
        if state["ref"] is None:
            state["ref"] = r
        cur[...] = h.download_state()
        return _flat(cur, sl), r / state["ref"] if state["ref"] > 0 else 0.0

    scale = state_scale(flow or h.flow, ext)
    x, drop, maps = krylov.anderson(phi, _flat(cur, sl), m=m, maxiter=max_maps,
                                    done=lambda d, n: d <= tol, scale=scale)
    cur[sl] = x.reshape(shape, order="F")
    return cur, state["it"], drop, state["ref"], maps, maps * k


def adjoint_krylov(h, dJ, CFL, tol=1e-10, k=20, restart=100, max_products=8000, it=3, history=None):
    """psi with (dR/dq)^T psi = -dJ/dq at the device state by GMRES
    (fest3d.krylov) on (I - G^k) psi = S_k(g): S_k is k steps of the
    fixed-point adjoint iteration from zero (fest_adjoint_solve), G its
    iteration matrix, and (I - G^k) v = -S_k((dR/dq)^T v), one residual VJP
    and k adjoint steps per product.  GMRES cycles of `restart` products
    until the true residual ||(dR/dq)^T psi + dJ/dq|| / ||dJ/dq|| over the
    interior cells is at most tol (checked after every cycle; history, a
    list, receives (products, drop)).  Returns (psi in the residue layout,
    GMRES products, drop, residual-VJP calls)."""
    ext = h.ext
    sl = _interior(ext)
    shape = (ext.imx - 1, ext.jmx - 1, ext.kmx - 1, 5)
    pad = np.zeros(h.shape["qp"], order="F")
    calls = [0]

    def S(b):
        pad[sl] = b.reshape(shape, order="F")
        psi, _, _ = h.adjoint_solve(pad, CFL, k, 0.0)
        calls[0] += 3 * k
        return psi.reshape(-1, order="F")

    def AT(v):
        dq = h.residual_vjp(None, it, np.asfortranarray(v.reshape(shape, order="F")))
        calls[0] += 1
        return _flat(dq, sl)

    g = _flat(dJ, sl)
    gn = np.linalg.norm(g)
    rhs = S(g)
    x, products, drop = None, 0, np.inf
    while products < max_products:
        # one cycle (the preconditioned system's own tolerance is far below
        # what the true residual needs: the true residual decides)
        x, n, _ = krylov.gmres(lambda v: -S(AT(v)), rhs, x0=x, tol=1e-16, restart=restart,
                               maxiter=min(restart + 1, max_products - products))
        products += n
        drop = float(np.linalg.norm(AT(x) + g) / gn)
        if history is not None:
            history.append((products, drop))
        if drop <= tol:
            break
    return np.asfortranarray(x.reshape(shape, order="F")), products, drop, calls[0]


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
        hp = make_handle(case, flow=bump_flow(mach, ang, mu_ref=case.get("mu_ref", 0.0)),
                         bc=bump_bc(mach, wall=case.get("wall", -6)), lib=lib)
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
                  max_iters=200000, lib=None, krylov_solve=False):
    """dJ/dalpha for each flow parameter and dJ/d(delta_i) for each listed
    lower-wall node i from one adjoint solve at the converged state q (the
    fixed-point iteration, or with krylov_solve its GMRES acceleration,
    adjoint_krylov); returns ({name: derivative}, J, adjoint iterations or
    GMRES products, drop)."""
    h = make_handle(case, lib=lib)
    h.upload_state(q)
    Jf = h.get("Jfaces")
    J, dJ = wall_force(q, case["ext"], Jf)
    if krylov_solve:
        psi, n, drop, _ = adjoint_krylov(h, dJ, case["CFL"], tol=tol, max_products=max_iters)
    else:
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


def perturbed_case(case, param, delta):
    """The case with flow parameter param ('mach', 'angle') moved by delta,
    or with lower-wall node param (an int) moved by delta in y."""
    c = dict(case)
    if isinstance(param, str):
        c[param] = case[param] + delta
        c["flow"] = bump_flow(c["mach"], c["angle"], mu_ref=case.get("mu_ref", 0.0))
        c["bc"] = bump_bc(c["mach"], wall=case.get("wall", -6))
    else:
        c["nodes"] = displaced_nodes(case, param, delta)
    return c


def wall_force_study(lib, wall_nodes=tuple(range(1, 129)), params=("mach", "angle"), fd_step=1e-6,
                     fd_steps=None, primal_tol=1e-12, adjoint_tol=1e-10, threads=4, log=None, progress=None,
                     fd_tol=None):
    """The bump's wall-force sensitivities at 128x48x4 cells (Euler,
    unlimited MUSCL + SLAU, FP64): the primal converged to a primal_tol
    drop (Anderson-accelerated explicit iterations from the free stream),
    one adjoint solve to an adjoint_tol drop (GMRES over the fixed-point
    adjoint iteration), gradients with respect to the inflow Mach number and
    angle and the y-displacements of the listed lower-wall nodes; each
    checked by a central difference of two re-converged primal solutions
    (step fd_step, or fd_steps[param]; each re-solve from the converged
    state to the same drop, or to fd_tol), the re-solves spread over
    `threads` handles.
    Returns a dict of everything measured; progress(dict), if given, sees
    it after every stage and every checked parameter."""
    import time
    from concurrent.futures import ThreadPoolExecutor
    say = log or (lambda *a: None)
    case = adjoint_case()
    ext, CFL = case["ext"], case["CFL"]
    out = {"workload": "smooth bump 128x48x4, Euler, MUSCL (unlimited) + SLAU, TVD-RK3 CFL 0.8, FP64",
           "objective": "x-force of the first-cell pressure on the lower wall J-faces"}
    t0 = time.perf_counter()
    h = make_handle(case, lib=lib)
    h.upload_state(case["qp"])
    ref = float(h.step(1, 1, CFL)[1])
    q, it, drop, ref, maps, iters = converge_accelerated(h, h.download_state(), CFL, first_iter=2,
                                                         tol=primal_tol, ref=ref)
    out["primal"] = {"drop": drop, "ref_norm": ref, "anderson_maps": maps, "iterations": iters + 1,
                     "seconds": time.perf_counter() - t0}
    say("primal", out["primal"])
    if progress:
        progress(out)
    t1 = time.perf_counter()
    Jf = h.get("Jfaces")
    J, dJ = wall_force(q, ext, Jf)
    h.upload_state(q)
    ahist = []
    psi, products, adrop, vjps = adjoint_krylov(h, dJ, CFL, tol=adjoint_tol, history=ahist)
    grads = {p: float(np.sum(psi * residual_param_derivative(case, q, it, p, lib=lib))) for p in params}
    if len(wall_nodes):
        dn = h.residual_vjp_nodes(q, it, psi, (None, wall_force_faces_bar(q, ext, Jf), None))
        wgt = wall_blend(ext)
        for i in wall_nodes:
            grads[i] = float(np.sum(dn[1, i + 2, 3:ext.jmx + 3, 3:ext.kmx + 3] * wgt[:, None]))
    h.close()
    out["adjoint"] = {"drop": adrop, "gmres_products": products, "residual_vjp_calls": vjps,
                      "seconds": time.perf_counter() - t1, "J": J, "history": ahist}
    say("adjoint", out["adjoint"])
    if progress:
        progress(out)
    steps = dict(fd_steps or {})

    def fd(param):
        """J at +step and -step, each from a primal re-converged to the same
        drop; the -step solve starts from 2 q* - q(+step), whose error is
        second order in the step"""
        step = steps.get(param, fd_step)
        vals, info, start = [], [], q
        for sgn in (1.0, -1.0):
            c = perturbed_case(case, param, sgn * step)
            hp = make_handle(c, lib=lib)
            qs, _, d, _, m, n = converge_accelerated(hp, start, CFL, first_iter=it, tol=fd_tol or primal_tol,
                                                     ref=ref, max_maps=6000)
            vals.append(wall_force(qs, ext, hp.get("Jfaces"))[0])
            info.append({"drop": d, "iterations": n})
            hp.close()
            start = np.asfortranarray(2.0 * q - qs)
        return param, (vals[0] - vals[1]) / (2 * step), step, info

    t2 = time.perf_counter()
    rows = []
    out["rows"] = rows
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for param, g_fd, step, info in ex.map(fd, list(params) + list(wall_nodes)):
            g = grads[param]
            rel = abs(g - g_fd) / max(abs(g_fd), 1e-300)
            rows.append({"param": param if isinstance(param, str) else f"wall_node_{param}",
                         "node": None if isinstance(param, str) else int(param),
                         "adjoint": g, "fd": g_fd, "rel_diff": rel, "fd_step": step,
                         "fd_drops": [i["drop"] for i in info],
                         "fd_iterations": [i["iterations"] for i in info]})
            say(rows[-1]["param"], g, g_fd, rel)
            if progress:
                progress(out)
    out["fd_seconds"] = time.perf_counter() - t2
    out["rows"] = rows
    out["max_rel_diff"] = max(r["rel_diff"] for r in rows) if rows else None
    nodes = [r for r in rows if r["node"] is not None]
    if nodes:
        big = max(abs(r["fd"]) for r in nodes)
        for r in nodes:
            r["abs_diff_over_max_node_gradient"] = abs(r["adjoint"] - r["fd"]) / big
        out["wall_nodes_max_abs_diff_over_max_gradient"] = max(r["abs_diff_over_max_node_gradient"] for r in nodes)
    return out


# ---- unsteady adjoint with checkpointing -------------------------------------
# N time-accurate TVD-RK3 steps with a fixed global time step (schemetype
# 'g' with global_time_step > 0, time.f90:248-289) on the FP64 module path
# (fest_get_next_solution).  One step: q1 = M(q0), q2 = 3/4 q0 + 1/4 M(q1),
# q3 = 1/3 q0 + 2/3 M(q2) (update.f90:196-206) with the stage update
# M(q) = prim(cons(q) - (dt/V) R(q)) (update.f90:367-485).  The adjoint runs
# the steps backwards: M'(q)^T v = C'(q)^T w - (dR/dq)^T ((dt/V) w),
# w = P'(M(q))^T v, C = cons, P = prim, the residual part by
# fest_residual_vjp.  States are kept at every `every`-th step and each
# segment is recomputed forwards before it is reversed.

GM = 1.4


def _interior(ext):
    return (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))


def _cons_T(q, w, gm=GM):
    """C'(q)^T w for U = (rho, rho u, rho v, rho w, E) of q = (rho,u,v,w,p)."""
    r, u, v, x = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    out = np.empty_like(w)
    out[..., 0] = w[..., 0] + u * w[..., 1] + v * w[..., 2] + x * w[..., 3] + 0.5 * (u * u + v * v + x * x) * w[..., 4]
    out[..., 1] = r * w[..., 1] + r * u * w[..., 4]
    out[..., 2] = r * w[..., 2] + r * v * w[..., 4]
    out[..., 3] = r * w[..., 3] + r * x * w[..., 4]
    out[..., 4] = w[..., 4] / (gm - 1.0)
    return out


def _prim_T(q, v, gm=GM):
    """P'(U)^T v at the primitive state q = P(U)."""
    r, u, vv, x = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    g1 = gm - 1.0
    out = np.empty_like(v)
    out[..., 0] = v[..., 0] - (u * v[..., 1] + vv * v[..., 2] + x * v[..., 3]) / r + 0.5 * g1 * (u * u + vv * vv + x * x) * v[..., 4]
    out[..., 1] = v[..., 1] / r - g1 * u * v[..., 4]
    out[..., 2] = v[..., 2] / r - g1 * vv * v[..., 4]
    out[..., 3] = v[..., 3] / r - g1 * x * v[..., 4]
    out[..., 4] = g1 * v[..., 4]
    return out


def _stage_update(q, R, dtv, gm=GM):
    """M(q) on interior cells: prim(cons(q) - dt/V R), FP64."""
    r, u, v, x, p = (q[..., l] for l in range(5))
    U = np.stack([r, r * u, r * v, r * x, p / (gm - 1.0) + 0.5 * r * (u * u + v * v + x * x)], axis=-1)
    U = U - R * dtv[..., None]
    rn = U[..., 0]
    un, vn, xn = U[..., 1] / rn, U[..., 2] / rn, U[..., 3] / rn
    pn = (gm - 1.0) * (U[..., 4] - 0.5 * rn * (un * un + vn * vn + xn * xn))
    return np.stack([rn, un, vn, xn, pn], axis=-1)


def _stages(h, q0, it, dtv, ext):
    """The three stage inputs of one step from q0 (padded, ghosts as the
    step starts) and the step's result; each with its ghosts as filled by
    its own residual evaluation."""
    sl = _interior(ext)
    qs, Rs = [], []
    q = np.array(q0, order="F")
    for k in range(3):
        qf, R = h.residual(q, it)
        qs.append(qf)
        Rs.append(R)
        m = _stage_update(qf[sl], R, dtv)
        nxt = np.array(qf, order="F")
        if k == 0:
            nxt[sl] = m
        elif k == 1:
            nxt[sl] = 0.75 * qs[0][sl] + 0.25 * m
        else:
            nxt[sl] = qs[0][sl] / 3.0 + 2.0 / 3.0 * m
        q = nxt
    return qs, Rs, q


def _stage_vjp(h, qf, R, it, dtv, v, ext):
    """M'(q)^T v on interior cells (v and the result: (nI,nJ,nK,5))."""
    sl = _interior(ext)
    qn = _stage_update(qf[sl], R, dtv)
    w = _prim_T(qn, v)
    lam = np.asfortranarray(w * dtv[..., None])
    dq = h.residual_vjp(qf, it, lam)[sl]
    return _cons_T(qf[sl], w) - dq


def unsteady_case(nc=(64, 24, 4), dt=2e-5, steps=100, mach=0.5):
    """The bump run time-accurately: unlimited MUSCL + SLAU, TVD-RK3 with a
    fixed global time step dt, from the uniform inflow plus a pressure pulse
    (the perturbation direction dq0, 1000 Pa Gaussian in the channel)."""
    ext = abi.Extent(nc[0] + 1, nc[1] + 1, nc[2] + 1, 5)
    scheme = abi.make_scheme(scheme_name="slau", interpolant="muscl", time_step_accuracy="TVDRK3",
                             time_stepping_method="g", global_time_step=dt, ilimiter_switch=0,
                             jlimiter_switch=0, klimiter_switch=0)
    flow = bump_flow(mach)
    nodes = cases.bump_nodes(ext)
    qp = cases.uniform_state(ext, flow)
    X = 0.125 * (nodes[0, 3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2] + nodes[0, 4:ext.imx + 3, 3:ext.jmx + 2, 3:ext.kmx + 2]
                 + nodes[0, 3:ext.imx + 2, 4:ext.jmx + 3, 3:ext.kmx + 2] + nodes[0, 4:ext.imx + 3, 4:ext.jmx + 3, 3:ext.kmx + 2]) * 2
    Y = 0.125 * (nodes[1, 3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2] + nodes[1, 4:ext.imx + 3, 3:ext.jmx + 2, 3:ext.kmx + 2]
                 + nodes[1, 3:ext.imx + 2, 4:ext.jmx + 3, 3:ext.kmx + 2] + nodes[1, 4:ext.imx + 3, 4:ext.jmx + 3, 3:ext.kmx + 2]) * 2
    dq0 = np.zeros_like(qp)
    dq0[3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2, 4] = 1000.0 * np.exp(-((X + 0.5) ** 2 + (Y - 0.4) ** 2) / 0.02)
    return dict(ext=ext, flow=flow, scheme=scheme, bc=bump_bc(mach), nodes=nodes, qp=qp, dq0=dq0,
                dt=dt, steps=steps, CFL=0.8, mach=mach, angle=0.0)


def run_primal(h, q0, steps, first_iter=1, keep_every=0):
    """`steps` steps of fest_get_next_solution from q0; returns the final
    state and, with keep_every, the states at steps 0, keep_every, ..."""
    q = np.array(q0, order="F")
    kept = {}
    for n in range(steps):
        if keep_every and n % keep_every == 0:
            kept[n] = q.copy(order="F")
        q = h.get_next_solution(q, first_iter + n, 0.8)
    return q, kept


def unsteady_sensitivity(case, eps=0.0, every=10, lib=None):
    """dJ/d(eps) of J = wall_force(q_N) for q_0 = qp + eps dq0 by the
    discrete adjoint of the N steps, states checkpointed every `every`
    steps and recomputed segment by segment.  Returns (J, dJ/deps,
    residual-VJP calls)."""
    ext = case["ext"]
    sl = _interior(ext)
    h = make_handle(case, lib=lib)
    vol = h.get("cells")[0][sl]
    dtv = case["dt"] / vol
    q0 = case["qp"] + eps * case["dq0"]
    N = case["steps"]
    qN, ckpt = run_primal(h, q0, N, keep_every=every)
    J, dJ = wall_force(qN, ext, h.get("Jfaces"))
    lam = np.array(dJ[sl])
    calls = 0
    for seg in range(((N - 1) // every) * every, -1, -every):
        # recompute the segment's step-start states
        states = [ckpt[seg]]
        for n in range(seg, min(seg + every, N) - 1):
            states.append(h.get_next_solution(states[-1], n + 1, 0.8))
        for n in range(min(seg + every, N) - 1, seg - 1, -1):
            it = n + 1
            qs, Rs, _ = _stages(h, states[n - seg], it, dtv, ext)
            # q3 = q0/3 + 2/3 M(q2); q2 = 3/4 q0 + 1/4 M(q1); q1 = M(q0)
            l2 = _stage_vjp(h, qs[2], Rs[2], it, dtv, (2.0 / 3.0) * lam, ext)
            l0 = lam / 3.0 + 0.75 * l2
            l1 = _stage_vjp(h, qs[1], Rs[1], it, dtv, 0.25 * l2, ext)
            l0 = l0 + _stage_vjp(h, qs[0], Rs[0], it, dtv, l1, ext)
            lam = l0
            calls += 3
    h.close()
    return J, float(np.sum(lam * case["dq0"][sl])), calls
