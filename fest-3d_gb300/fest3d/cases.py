"""Synthetic, seeded inputs in the reference's own layouts.

No dataset is involved: every workload is analytic or drawn from a fixed
seed.  Node arrays hold interior nodes (1:imx,1:jmx,1:kmx) as FEST-3D's grid
reader fills them (grid.f90:110-127); ghost nodes are left to
``setup_geometry``.  States fill the whole padded block, ghosts included, as
init_state_with_infinity_values does (state.f90:195-278).
"""
import numpy as np

from . import abi


def empty_nodes(ext):
    return np.zeros((3, ext.imx + 6, ext.jmx + 6, ext.kmx + 6), order="F")


def set_interior_nodes(nodes, x, y, z):
    """x,y,z of shape (imx,jmx,kmx) -> nodes(1:imx,1:jmx,1:kmx)."""
    imx, jmx, kmx = x.shape
    nodes[0, 3:3 + imx, 3:3 + jmx, 3:3 + kmx] = x
    nodes[1, 3:3 + imx, 3:3 + jmx, 3:3 + kmx] = y
    nodes[2, 3:3 + imx, 3:3 + jmx, 3:3 + kmx] = z
    return nodes


def box_nodes(ext, L=(1.0, 1.0, 1.0), perturb=0.0, seed=0, stretch_j=1.0):
    """Cartesian box, optional wall-normal stretching in j and a smooth
    sinusoidal node perturbation of amplitude perturb x local spacing."""
    imx, jmx, kmx = ext.imx, ext.jmx, ext.kmx
    s = np.linspace(0.0, 1.0, imx)
    if stretch_j != 1.0:
        r = stretch_j ** np.arange(jmx - 1)
        t = np.concatenate([[0.0], np.cumsum(r)])
        t = t / t[-1]
    else:
        t = np.linspace(0.0, 1.0, jmx)
    u = np.linspace(0.0, 1.0, kmx)
    X, Y, Z = np.meshgrid(s * L[0], t * L[1], u * L[2], indexing="ij")
    if perturb:
        rng = np.random.default_rng(seed)
        dx, dy, dz = L[0] / (imx - 1), L[1] / (jmx - 1), L[2] / (kmx - 1)
        ph = rng.uniform(0, 2 * np.pi, 6)
        fx = np.sin(2 * np.pi * Y / L[1] + ph[0]) * np.sin(2 * np.pi * Z / L[2] + ph[1])
        fy = np.sin(2 * np.pi * X / L[0] + ph[2]) * np.sin(2 * np.pi * Z / L[2] + ph[3])
        fz = np.sin(2 * np.pi * X / L[0] + ph[4]) * np.sin(2 * np.pi * Y / L[1] + ph[5])
        X = X + perturb * dx * fx
        Y = Y + perturb * dy * fy
        Z = Z + perturb * dz * fz
    return set_interior_nodes(empty_nodes(ext), X, Y, Z)


def bump_nodes(ext, x0=-1.5, x1=1.5, top=0.8, stretch=1.02, depth=0.1):
    """Channel over y_b = 0.0625 exp(-25 x^2), geometric stretching in j."""
    imx, jmx, kmx = ext.imx, ext.jmx, ext.kmx
    x = np.linspace(x0, x1, imx)
    yb = 0.0625 * np.exp(-25.0 * x * x)
    r = stretch ** np.arange(jmx - 1)
    t = np.concatenate([[0.0], np.cumsum(r)])
    t = t / t[-1]
    z = np.linspace(0.0, depth, kmx)
    X = np.repeat(np.repeat(x[:, None, None], jmx, 1), kmx, 2)
    Y = yb[:, None, None] + (top - yb)[:, None, None] * t[None, :, None]
    Y = np.repeat(Y, kmx, 2)
    Z = np.broadcast_to(z[None, None, :], (imx, jmx, kmx)).copy()
    return set_interior_nodes(empty_nodes(ext), X, Y, Z)


def wall_spacing(n, dy1=1e-6, stretch=1.12, height=1.0):
    """Wall-normal node coordinates of n cells: the first cell dy1, each next
    one stretch times longer, the growth capped at the spacing that puts the
    last node at height (geometric near the wall, uniform beyond)."""
    def top(cap):
        return np.minimum(dy1 * stretch ** np.arange(n), cap).sum()
    lo, hi = dy1, height
    for _ in range(200):  # bisection on the cap
        mid = 0.5 * (lo + hi)
        if top(mid) < height:
            lo = mid
        else:
            hi = mid
    dy = np.minimum(dy1 * stretch ** np.arange(n), 0.5 * (lo + hi))
    y = np.concatenate([[0.0], np.cumsum(dy)])
    return y * (height / y[-1])  # the cap's last bit; dy1 moves by ~1e-12 relative


def plate_block_nodes(ext, x, y, depth):
    """Cartesian block of node lines x, y and kmx nodes over depth in z."""
    z = np.linspace(0.0, depth, ext.kmx)
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    return set_interior_nodes(empty_nodes(ext), X, Y, Z)


def uniform_state(ext, flow, tk=0.0, tw=0.0):
    qp = abi.farray(ext, "qp")
    qp[..., 0] = flow.density_inf
    qp[..., 1] = flow.x_speed_inf
    qp[..., 2] = flow.y_speed_inf
    qp[..., 3] = flow.z_speed_inf
    qp[..., 4] = flow.pressure_inf
    if ext.n_var > 5:
        qp[..., 5] = tk
        qp[..., 6] = tw
    return qp


def random_state(ext, seed=0, mach=0.3, amp=0.1, p0=101325.0, rho0=1.2, tk=1.0, tw=1000.0,
                 rho_amp=None, tv=1e-4):
    """Smooth 3-mode Fourier field over the padded block: rho in
    rho0*(1 +- amp), |u| up to mach*c, p0*(1 +- amp), positive tk/tw
    (seven variables) or tv (six, Spalart-Allmaras), and an intermittency in
    (0.1, 0.9) (eight, LCTM2015)."""
    rng = np.random.default_rng(seed)
    ni, nj, nk = ext.imx + 5, ext.jmx + 5, ext.kmx + 5
    I, J, K = np.meshgrid(np.arange(ni) / ni, np.arange(nj) / nj, np.arange(nk) / nk, indexing="ij")

    def field():
        f = np.zeros_like(I)
        for _ in range(3):
            a = rng.uniform(-1, 1)
            kx, ky, kz = rng.integers(1, 4, 3)
            ph = rng.uniform(0, 2 * np.pi, 3)
            f += a * np.sin(2 * np.pi * kx * I + ph[0]) * np.sin(2 * np.pi * ky * J + ph[1]) * \
                np.cos(2 * np.pi * kz * K + ph[2])
        return f / 3.0

    c = np.sqrt(1.4 * p0 / rho0)
    qp = abi.farray(ext, "qp")
    qp[..., 0] = rho0 * (1 + (amp if rho_amp is None else rho_amp) * field())
    for l in (1, 2, 3):
        qp[..., l] = mach * c * field()
    qp[..., 4] = p0 * (1 + amp * field())
    if ext.n_var == 6:
        qp[..., 5] = tv * (1 + 0.5 * field())
    elif ext.n_var > 5:
        qp[..., 5] = tk * (1 + 0.5 * field())
        qp[..., 6] = tw * (1 + 0.5 * field())
    if ext.n_var == 8:  # LCTM2015's intermittency, inside (0, 1)
        qp[..., 7] = 0.5 + 0.4 * field()
    return qp


# ---------------------------------------------------------------------------
# the benchmark configurations (one structured block each)
def ldc_case(nc=(64, 64, 4)):
    """Laminar lid-driven cavity: 64x64x4 cells over 1 x 1 x 0.0625 m,
    gamma 1.4, R 287, rho 1.2, p 101325, lid at jmax moving +x at 34.7 m/s
    (id -3, FIX_DENSITY/X_SPEED, COPY_PRESSURE), other x/y faces adiabatic
    no-slip walls (-5), z faces periodic (-10, kmin<->kmax); constant mu for
    Re=100 on the lid; MUSCL (van Albada limiter) + AUSM, local time step,
    forward Euler, CFL 0.5."""
    ext = abi.Extent(nc[0] + 1, nc[1] + 1, nc[2] + 1, 5)
    flow = abi.make_flow(density_inf=1.2, x_speed_inf=0.0, pressure_inf=101325.0,
                         mu_ref=1.2 * 34.7 * 1.0 / 100.0, mu_variation="constant")
    scheme = abi.make_scheme(scheme_name="ausm", interpolant="muscl", time_step_accuracy="none",
                             time_stepping_method="l", limiter="van_albada")
    fixed = {k: [0.0] * 6 for k in ("fixed_density", "fixed_x_speed", "fixed_y_speed",
                                    "fixed_z_speed", "fixed_wall_temperature")}
    fixed["fixed_density"][3] = 1.2
    fixed["fixed_x_speed"][3] = 34.7
    bc = abi.make_bc([-5, -5, -5, -3, -10, -10], partners={4: (0, 5), 5: (0, 4)}, **fixed)
    nodes = box_nodes(ext, L=(1.0, 1.0, 0.0625))
    qp = uniform_state(ext, flow)
    return dict(name="lid-driven cavity 64x64x4, MUSCL+AUSM, laminar, forward Euler",
                ext=ext, flow=flow, scheme=scheme, bc=bc, nodes=nodes, qp=qp, CFL=0.5)


def bump_case(nc=(256, 96, 4), mach=0.5):
    """Inviscid channel over a smooth bump: 256x96x4 cells, subsonic total
    pressure inlet (-11) for Mach 0.5, back-pressure outlet (-4), slip walls
    (-6) top and bottom, periodic z (-10); WENO5 + SLAU, TVD-RK3, CFL 0.8."""
    ext = abi.Extent(nc[0] + 1, nc[1] + 1, nc[2] + 1, 5)
    p0, rho0, gm = 101325.0, 1.2, 1.4
    c = np.sqrt(gm * p0 / rho0)
    flow = abi.make_flow(density_inf=rho0, x_speed_inf=mach * c, pressure_inf=p0, mu_ref=0.0)
    scheme = abi.make_scheme(scheme_name="slau", interpolant="weno", time_step_accuracy="TVDRK3",
                             time_stepping_method="l")
    pt = p0 * (1 + 0.5 * (gm - 1) * mach * mach) ** (gm / (gm - 1))
    fixed = {k: [0.0] * 6 for k in ("fixed_pressure", "fixed_Tpressure")}
    fixed["fixed_pressure"][1] = p0
    fixed["fixed_Tpressure"][0] = pt
    bc = abi.make_bc([-11, -4, -6, -6, -10, -10], partners={4: (0, 5), 5: (0, 4)}, **fixed)
    nodes = bump_nodes(ext)
    qp = uniform_state(ext, flow)
    return dict(name=f"smooth bump {nc[0]}x{nc[1]}x{nc[2]}, WENO5+SLAU, inviscid, TVD-RK3", ext=ext, flow=flow,
                scheme=scheme, bc=bc, nodes=nodes, qp=qp, CFL=0.8)


def plate_case(n_run=32, n_plate=160, nj=128, nk=2, mach=0.2, Re_per_m=5e6, Tu=0.1, mut_ratio=0.01,
               run_in=0.33, length=2.0, depth=0.01):
    """Turbulent zero-pressure-gradient flat plate with k-omega SST, laid out
    as the reference's own Tfp case (tests/Tfp/system/mesh/layout): block 0
    the symmetry run-in x in [-0.33, 0] (far field -8 at imin, symmetry -6
    below), block 1 the plate x in [0, 2] (no-slip adiabatic wall -5 below,
    outlet -4 at imax), joined by an interface (block 0's imax = block 1's
    imin), slip top and k faces (-6).  192x128x2 cells in all (32 + 160 in
    i); first wall-normal cell 1e-6 m, stretched by 1.12 up to the spacing
    that reaches the 1 m top; nodes clustered at the leading edge.  Mach
    0.2, Re 5e6 per metre, Tu 0.1%, mu_t/mu 0.01; MUSCL + AUSM-UP, RK4,
    local time steps, CFL 1.0.  Returns dict(name, blocks=[per-block dicts
    of ext, flow, scheme, bc, nodes, qp], wall, CFL)."""
    p0, T0, gm, R = 101325.0, 300.0, 1.4, 287.0
    rho0 = p0 / (R * T0)
    c = np.sqrt(gm * p0 / rho0)
    U = mach * c
    mu_ref = rho0 * U / Re_per_m
    tk = 1.5 * (U * Tu / 100.0) ** 2
    tw = rho0 * tk / (mu_ref * mut_ratio)
    flow = abi.make_flow(density_inf=rho0, x_speed_inf=U, pressure_inf=p0, mu_ref=mu_ref,
                         mu_variation="sutherland_law", T_ref=T0, tk_inf=tk, tw_inf=tw)
    scheme = abi.make_scheme(scheme_name="ausmUP", interpolant="muscl", time_step_accuracy="RK4",
                             time_stepping_method="l", turbulence="sst")
    fixed = {k: [0.0] * 6 for k in ("fixed_density", "fixed_x_speed", "fixed_y_speed",
                                    "fixed_z_speed", "fixed_pressure", "fixed_tk", "fixed_tw",
                                    "fixed_wall_temperature")}
    for f in range(6):
        fixed["fixed_density"][f] = rho0
        fixed["fixed_x_speed"][f] = U
        fixed["fixed_pressure"][f] = p0
        fixed["fixed_tk"][f] = tk
        fixed["fixed_tw"][f] = tw
    y = wall_spacing(nj, height=1.0)
    s_run = np.linspace(0.0, 1.0, n_run + 1)
    s_pl = np.linspace(0.0, 1.0, n_plate + 1)
    x_run = -run_in * (1.0 - s_run) ** 1.5
    x_pl = length * s_pl ** 1.5
    blocks = []
    for b, (x, ids, partners) in enumerate(((x_run, [-8, 1, -6, -6, -6, -6], {1: (1, 0)}),
                                            (x_pl, [0, -4, -5, -6, -6, -6], {0: (0, 1)}))):
        ext = abi.Extent(len(x), nj + 1, nk + 1, 7)
        bc = abi.make_bc(ids, partners=partners, block_id=b, **fixed)
        blocks.append(dict(ext=ext, flow=flow, scheme=scheme, bc=bc,
                           nodes=plate_block_nodes(ext, x, y, depth),
                           qp=uniform_state(ext, flow, tk=tk, tw=tw)))
    wall = wall_nodes_of(blocks[1]["nodes"], blocks[1]["ext"], blocks[1]["bc"])
    return dict(name=f"SST flat plate {n_run + n_plate}x{nj}x{nk} (run-in {n_run} + plate {n_plate}), "
                     "MUSCL+AUSM-UP, RK4", blocks=blocks, wall=wall, CFL=1.0, flow=flow)


def wall_nodes_of(nodes, ext, bc):
    """Wall node list (surface_points, wall.f90:200-286): every node of a
    face with id -5, in the reference's face order."""
    pts = []
    imx, jmx, kmx = ext.imx, ext.jmx, ext.kmx
    rng = {0: ((1, 1), (1, jmx), (1, kmx)), 1: ((imx, imx), (1, jmx), (1, kmx)),
           2: ((1, imx), (1, 1), (1, kmx)), 3: ((1, imx), (jmx, jmx), (1, kmx)),
           4: ((1, imx), (1, jmx), (1, 1)), 5: ((1, imx), (1, jmx), (kmx, kmx))}
    for f in range(6):
        if bc.id[f] != -5:
            continue
        (i0, i1), (j0, j1), (k0, k1) = rng[f]
        for k in range(k0, k1 + 1):
            for j in range(j0, j1 + 1):
                for i in range(i0, i1 + 1):
                    pts.append(nodes[:, i + 2, j + 2, k + 2])
    return np.array(pts, dtype=np.float64)


def batch_blocks(n=96, seed=0, dims_lo=(16, 16, 2), dims_hi=(160, 96, 16), mach=0.8,
                 scheme_name="ausmP", interpolant="muscl", integrator="TVDRK3", viscous=True):
    """Independent blocks of a batched multiblock case: cell dimensions drawn
    uniformly from [16,160]x[16,96]x[2,16] (numpy default_rng(seed)),
    Cartesian grids with a sinusoidal node perturbation of 5% of the local
    spacing, smooth random fields (rho in [0.9,1.3], velocity components up
    to Mach 0.8 from 3 Fourier modes, p = 101325 +- 10%).  Each direction is
    periodic (a self-paired interface, when the block has >= 4 cells there)
    or extrapolated (-2: ghost = first interior cell), by a fair coin.
    Laminar Navier-Stokes with Sutherland viscosity (viscous=False: Euler),
    MUSCL + AUSM+ with TVD-RK3, CFL 0.5."""
    rng = np.random.default_rng(seed)
    out = []
    c = np.sqrt(1.4 * 101325.0 / 1.1)
    for b in range(n):
        nc = [int(rng.integers(lo, hi + 1)) for lo, hi in zip(dims_lo, dims_hi)]
        ext = abi.Extent(nc[0] + 1, nc[1] + 1, nc[2] + 1, 5)
        ids, partners = [], {}
        for d in range(3):
            periodic = nc[d] >= 4 and rng.random() < 0.5
            ids += [-10, -10] if periodic else [-2, -2]
            if periodic:
                partners[2 * d] = (0, 2 * d + 1)
                partners[2 * d + 1] = (0, 2 * d)
        bc = abi.make_bc(ids, partners=partners)
        flow = abi.make_flow(density_inf=1.1, x_speed_inf=0.3 * c, pressure_inf=101325.0,
                             mu_ref=1.716e-5 if viscous else 0.0, mu_variation="sutherland_law")
        scheme = abi.make_scheme(scheme_name=scheme_name, interpolant=interpolant,
                                 time_step_accuracy=integrator, time_stepping_method="l")
        h = 1.0 / 64
        nodes = box_nodes(ext, L=(nc[0] * h, nc[1] * h, nc[2] * h), perturb=0.05, seed=seed * 1000 + b)
        qp = random_state(ext, seed=seed * 1000 + b + 7, mach=mach, amp=0.1, p0=101325.0, rho0=1.1,
                          rho_amp=0.2 / 1.1)
        out.append(dict(ext=ext, flow=flow, scheme=scheme, bc=bc, nodes=nodes, qp=qp, CFL=0.5, cells=int(np.prod(nc))))
    return out
