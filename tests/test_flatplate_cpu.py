"""The reference's laminar and turbulent flat-plate test cases (tests/Lfp
and tests/Tfp of FEST-3D) as integration checks of the viscous and SST
paths.

Turbulent (k-omega SST): the report expects 2.900E-03 within 2 % (the
reference computed 2.872E-03); the oracle's steady state on the case's two
blocks gives 2.880E-03 (0.3 % above the reference's figure).  That figure
too is the state after a fixed implicit run, one that restarts from the
case's stored solution: replayed from it, the oracle's LU-SGS gives
2.8686E-03 (0.13 % below it).

Laminar:

Its report (tests/Report.txt) compares the plate's drag coefficient with
the Blasius value 1.330E-03 and passes within 1 % (the reference computed
1.329E-03).  The fixture (tests/golden/make_flatplate.py) holds the case's
two blocks and the oracle's steady state on them; the drag coefficient is
evaluated as the reference's post-processing does (Lfp/pp/Surface.py: wall
shear from the first cells' Green-Gauss velocity gradients and viscosity on
the wall faces, divided by the dynamic pressure and the span 0.05).  The
oracle's steady-state value, 1.3194E-03, passes the report's 1 % band; it
is 0.75 % below the reference's own figure because that figure is not a
steady state but the state after the case's 5000 implicit iterations,
which the oracle's restatement of the reference's LU-SGS integrator
replays to 1.4e-5 relative.  No GPU."""
import os
import sys

import numpy as np

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_flatplate as MF  # noqa: E402

BLASIUS_CD = 1.330e-03  # tests/Report.txt, "Expected drag coeffcient", allowed tolerance 1 %


def drag_coefficient(blk, length_span=0.05, rho=None, u=None, mu=None, recompute=True):
    """Lfp/pp/Surface.py (Tfp/pp/Surface.py: length x span 2 x 0.04) on the
    wall (j = 1) faces of the plate block; mu: the first cells' laminar
    viscosity (default the laminar case's constant).  recompute=False uses
    the gradients held from the last residual evaluation, as the reference's
    output files hold them (update.f90:540 is their only evaluation)."""
    ext = blk.ext
    rho = MF.RHO_INF if rho is None else rho
    u = MF.U_INF if u is None else u
    if recompute:
        blk.compute_temperature()
        blk.evaluate_all_gradients()
    gx, gy, gz = blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]
    c = (slice(1, ext.imx), 1, 1)  # first cell row, (0:imx, 0:jmx, 0:kmx) layout
    dudx, dudy, dudz = gx[c + (0,)], gy[c + (0,)], gz[c + (0,)]
    dvdx, dvdy, dwdz = gx[c + (1,)], gy[c + (1,)], gz[c + (2,)]
    dwdx = gx[c + (2,)]
    delv = dudx + dvdy + dwdz
    m = MF.MU if mu is None else mu
    txx = m * (2.0 * dudx - 2.0 * delv / 3.0)
    txy = m * (dudy + dvdx)
    txz = m * (dudz + dwdx)
    Jf = blk["Jfaces"][:, 3:ext.imx + 2, 3, 3]  # faces (i, 1, 1): {A, nx, ny, nz}
    Fx = txx * Jf[1] + txy * Jf[2] + txz * Jf[3]
    q_inf = 0.5 * rho * u ** 2
    return float(np.sum(Fx * Jf[0] / q_inf) / length_span)


def test_oracle_flat_plate_drag_passes_the_reference_test():
    fx = np.load(os.path.join(HERE, "golden", "flatplate_laminar.npz"))
    grids = [fx["nodes0"], fx["nodes1"]]
    blocks = []
    for ext, flow, scheme, bc, nodes, qp in MF.flatplate_case(grids):
        blk = O.Block(ext, flow, scheme, bc)
        blk["nodes"] = nodes
        blk.setup_geometry()
        blk["qp"] = qp
        blocks.append(blk)
    assert O.get_total_conservative_residue(blocks, 1) == 0
    r0 = O.find_resnorm(blocks)
    for blk, q in zip(blocks, (fx["q0"], fx["q1"])):
        full = np.array(blk["qp"], order="F")
        full[3:blk.ext.imx + 2, 3:blk.ext.jmx + 2, 3:blk.ext.kmx + 2] = q
        blk["qp"] = full
    assert O.get_total_conservative_residue(blocks, 1) == 0
    r = O.find_resnorm(blocks)
    # a steady state: the x-momentum residual (the free stream's comes from
    # the wall shear; its mass residual vanishes) dropped by 10^-3 and more
    assert r[2] < 1e-3 * r0[2], (r, r0)
    cd = drag_coefficient(blocks[1])
    assert abs(cd - BLASIUS_CD) <= 0.01 * BLASIUS_CD, cd


# Report.txt, laminar case: "Difference 5.001E-02 %" from the expected
# 1.330E-03, i.e. the reference computed 1.330e-3 * (1 - 5.001e-4)
REFERENCE_RUN_CD = BLASIUS_CD * (1.0 - 5.001e-4)


def test_oracle_replays_the_reference_implicit_run():
    """The reference's own figure is not a steady state: its case runs the
    implicit LU-SGS integrator (Lfp/system/fvscheme.md "implicit") for 5000
    iterations at CFL 2000 from the free stream (control.md) and stops
    there.  The oracle's restatement of that integrator, run the same way
    on the same two blocks, gives the reference's drag coefficient to
    1.4e-5 relative (the reference's value lies between the oracle's
    iterations 5001 and 5002, where the drag still falls by 7e-6 relative
    per iteration), while its converged value is 0.75 % lower."""
    fx = np.load(os.path.join(HERE, "golden", "flatplate_laminar.npz"))
    blocks = []
    for ext, flow, scheme, bc, nodes, qp in MF.flatplate_case([fx["nodes0"], fx["nodes1"]]):
        blk = O.Block(ext, flow, scheme, bc)
        blk["nodes"] = nodes
        blk.setup_geometry()
        blk["qp"] = qp  # the free stream, as the reference starts (restart level 0)
        blocks.append(blk)
    O.set_threads(min(4, os.cpu_count() or 1))
    for it in range(1, 5001):
        assert O.lusgs_next_solution(blocks, it, 2000.0) == 0
    # the gradients of the last residual evaluation, as the reference writes them
    cd = drag_coefficient(blocks[1], recompute=False)
    assert abs(cd - REFERENCE_RUN_CD) <= 3e-5 * REFERENCE_RUN_CD, (cd, REFERENCE_RUN_CD)


def _sst_blocks(fx, steady):
    case = MF.flatplate_sst_case([fx["nodes0"], fx["nodes1"]])
    wall = MF.wall_nodes(case)
    blocks = []
    for n, (ext, flow, scheme, bc, nodes, qp) in enumerate(case):
        blk = O.Block(ext, flow, scheme, bc)
        blk["nodes"] = nodes
        blk.setup_geometry()
        blk.find_wall_dist(wall)
        if steady:
            qp = np.array(qp, order="F")
            qp[3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2] = fx["q%d" % n]
        blk["qp"] = qp
        blocks.append(blk)
    return blocks


def test_lusgs_sst_holds_the_explicit_steady_state():
    """The SST branch of the LU-SGS restatement (lusgs.f90:686-1196) solves
    the same residual: started on the explicit integrator's steady state it
    stays there (drag within 2e-4, the fixture's own convergence level: run
    from the free stream it settles at 2.8801e-3 against the fixture's
    2.8805e-3; x-momentum residual not growing)."""
    fx = np.load(os.path.join(HERE, "golden", "flatplate_sst.npz"))
    blocks = _sst_blocks(fx, steady=True)
    plate = blocks[1]

    def cd():
        mu = plate["mu"][3:plate.ext.imx + 2, 3, 3]
        return drag_coefficient(plate, length_span=2 * 0.04, rho=MF.T_RHO, u=MF.T_U, mu=mu,
                                recompute=False)

    assert O.lusgs_next_solution(blocks, 1, 3000.0) == 0
    cd0, r0 = cd(), O.find_resnorm(blocks)[2]
    for it in range(2, 201):
        assert O.lusgs_next_solution(blocks, it, 3000.0) == 0
    assert abs(cd() - cd0) <= 2e-4 * cd0, (cd(), cd0)
    assert O.find_resnorm(blocks)[2] <= r0, (O.find_resnorm(blocks)[2], r0)


SST_CD = 2.900e-03  # tests/Report.txt, turbulent case, "Expected drag coeffcient", tolerance 2 %
# Report.txt, turbulent case: "Difference 9.586E-01 %" from the expected 2.900E-03
REFERENCE_SST_RUN_CD = SST_CD * (1.0 - 9.586e-3)


def test_oracle_replays_the_reference_turbulent_restart_run():
    """The turbulent case's figure is not a steady state either: the case
    restarts (control.md "Restart level 2") from its stored solution
    (density, velocity, pressure; k and omega at free stream), runs 10000
    LU-SGS iterations at CFL 3000 and writes what it has.  Replayed from
    that state (tests/golden/flatplate_sst_restart.npz) the oracle's LU-SGS
    gives 2.8686e-3, 0.13 % below the reported 2.8722e-3 and approaching
    it from below, the way the reported figure lies below the steady state
    (2.8801e-3); from the free stream instead it gives 2.952e-3.  The
    remaining 0.13 % (about 700 iterations of progress at that point) is
    not explained; the replay is insensitive to 1e-12 perturbations of the
    start, so it is not rounding."""
    fx = np.load(os.path.join(HERE, "golden", "flatplate_sst.npz"))
    rs = np.load(os.path.join(HERE, "golden", "flatplate_sst_restart.npz"))
    blocks = _sst_blocks(fx, steady=False)
    for n, blk in enumerate(blocks):
        ext = blk.ext
        qp = np.array(blk["qp"], order="F")  # the free stream, ghosts included
        qp[3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2, :5] = rs["q%d" % n]
        blk["qp"] = qp
    O.set_threads(min(4, os.cpu_count() or 1))
    for it in range(1, 10001):
        assert O.lusgs_next_solution(blocks, it, 3000.0) == 0
    plate = blocks[1]
    mu = plate["mu"][3:plate.ext.imx + 2, 3, 3]
    cd = drag_coefficient(plate, length_span=2 * 0.04, rho=MF.T_RHO, u=MF.T_U, mu=mu, recompute=False)
    assert cd < REFERENCE_SST_RUN_CD and abs(cd - REFERENCE_SST_RUN_CD) <= 2e-3 * REFERENCE_SST_RUN_CD, cd


def test_oracle_sst_flat_plate_drag_passes_the_reference_test():
    fx = np.load(os.path.join(HERE, "golden", "flatplate_sst.npz"))
    case = MF.flatplate_sst_case([fx["nodes0"], fx["nodes1"]])
    wall = MF.wall_nodes(case)
    blocks = []
    for ext, flow, scheme, bc, nodes, qp in case:
        blk = O.Block(ext, flow, scheme, bc)
        blk["nodes"] = nodes
        blk.setup_geometry()
        blk.find_wall_dist(wall)
        blk["qp"] = qp
        blocks.append(blk)
    assert O.get_total_conservative_residue(blocks, 1) == 0
    r0 = O.find_resnorm(blocks)
    for blk, q in zip(blocks, (fx["q0"], fx["q1"])):
        full = np.array(blk["qp"], order="F")
        full[3:blk.ext.imx + 2, 3:blk.ext.jmx + 2, 3:blk.ext.kmx + 2] = q
        blk["qp"] = full
    assert O.get_total_conservative_residue(blocks, 1) == 0
    r = O.find_resnorm(blocks)
    assert r[2] < 1e-3 * r0[2], (r, r0)  # a steady state (x momentum)
    plate = blocks[1]
    plate.compute_temperature()
    plate.calculate_viscosity()
    mu = plate["mu"][3:plate.ext.imx + 2, 3, 3]  # the first cells' laminar viscosity
    cd = drag_coefficient(plate, length_span=2 * 0.04, rho=MF.T_RHO, u=MF.T_U, mu=mu)
    assert abs(cd - SST_CD) <= 0.02 * SST_CD, cd


def test_plusgs_restatement_properties():
    """The oracle's PLU-SGS (plusgs.f90:191-577, 779-1256) where its
    preconditioner is the identity: with every cell's Mach number capped
    from below by a free-stream Mach number of 1.2, eps = 1, P = I and the
    preconditioned spectral radius (0.5 (2 |Vn| + sqrt(4 c^2))) equals
    LU-SGS's |Vn| + c, so an inviscid block advances as LU-SGS advances it,
    bit for bit; at Mach 0.2 the preconditioner acts and the iterates
    differ."""
    import numpy as np
    from fest3d import post
    from parity import small_case

    def run(fn, n, CFL, mach):
        kw = dict(nc=(9, 7, 6), ids=(-3, -4, -6, -6, -10, -10),
                  scheme_kw=dict(interpolant="muscl", scheme_name="ausm"), flow_kw=dict(MInf=mach))
        ext, flow, scheme, bc, nodes, qp = small_case(**kw)
        b = O.Block(ext, flow, scheme, bc)
        b["nodes"] = nodes
        b.setup_geometry()
        b["qp"] = qp
        for it in range(1, n + 1):
            assert fn([b], it, CFL) == 0
        return np.array(b["qp"]), ext

    a, ext = run(O.lusgs_next_solution, 3, 50.0, 1.2)
    b, _ = run(O.plusgs_next_solution, 3, 50.0, 1.2)
    assert np.array_equal(post.interior(a, ext), post.interior(b, ext))
    a, _ = run(O.lusgs_next_solution, 3, 50.0, 0.2)
    b, _ = run(O.plusgs_next_solution, 3, 50.0, 0.2)
    assert np.abs(post.interior(a, ext) - post.interior(b, ext)).max() > 1e-3
