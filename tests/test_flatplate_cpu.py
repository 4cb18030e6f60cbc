"""The reference's laminar and turbulent flat-plate test cases (tests/Lfp
and tests/Tfp of FEST-3D) as integration checks of the viscous and SST
paths.

Turbulent (k-omega SST): the report expects 2.900E-03 within 2 % (the
reference computed 2.872E-03); the oracle's steady state on the case's two
blocks gives 2.880E-03 (0.3 % above the reference's figure).

Laminar:

Its report (tests/Report.txt) compares the plate's drag coefficient with
the Blasius value 1.330E-03 and passes within 1 % (the reference computed
1.329E-03).  The fixture (tests/golden/make_flatplate.py) holds the case's
two blocks and the oracle's steady state on them; the drag coefficient is
evaluated as the reference's post-processing does (Lfp/pp/Surface.py: wall
shear from the first cells' Green-Gauss velocity gradients and viscosity on
the wall faces, divided by the dynamic pressure and the span 0.05).  The
oracle's value, 1.3195E-03, passes the report's 1 % band; it is 0.7 % below
the reference's own figure, a difference not yet explained.  No GPU."""
import os
import sys

import numpy as np

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_flatplate as MF  # noqa: E402

BLASIUS_CD = 1.330e-03  # tests/Report.txt, "Expected drag coeffcient", allowed tolerance 1 %


def drag_coefficient(blk, length_span=0.05, rho=None, u=None, mu=None):
    """Lfp/pp/Surface.py (Tfp/pp/Surface.py: length x span 2 x 0.04) on the
    wall (j = 1) faces of the plate block; mu: the first cells' laminar
    viscosity (default the laminar case's constant)."""
    ext = blk.ext
    rho = MF.RHO_INF if rho is None else rho
    u = MF.U_INF if u is None else u
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


SST_CD = 2.900e-03  # tests/Report.txt, turbulent case, "Expected drag coeffcient", tolerance 2 %


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
