"""The reference's laminar flat-plate test case (tests/Lfp of FEST-3D) as an
integration check of the viscous path.

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


def drag_coefficient(blk, span=0.05):
    """Lfp/pp/Surface.py on the wall (j = 1) faces of the plate block."""
    ext = blk.ext
    blk.compute_temperature()
    blk.evaluate_all_gradients()
    gx, gy, gz = blk["gradqp_x"], blk["gradqp_y"], blk["gradqp_z"]
    c = (slice(1, ext.imx), 1, 1)  # first cell row, (0:imx, 0:jmx, 0:kmx) layout
    dudx, dudy, dudz = gx[c + (0,)], gy[c + (0,)], gz[c + (0,)]
    dvdx, dvdy, dwdz = gx[c + (1,)], gy[c + (1,)], gz[c + (2,)]
    dwdx = gx[c + (2,)]
    delv = dudx + dvdy + dwdz
    txx = MF.MU * (2.0 * dudx - 2.0 * delv / 3.0)
    txy = MF.MU * (dudy + dvdx)
    txz = MF.MU * (dudz + dwdx)
    Jf = blk["Jfaces"][:, 3:ext.imx + 2, 3, 3]  # faces (i, 1, 1): {A, nx, ny, nz}
    Fx = txx * Jf[1] + txy * Jf[2] + txz * Jf[3]
    q_inf = 0.5 * MF.RHO_INF * MF.U_INF ** 2
    return float(np.sum(Fx * Jf[0] / q_inf) / span)


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
