"""The reference's own SmoothBump test case as an integration anchor.

FEST-3D's tests/Report.txt records, for its inviscid smooth-bump case (AUSM,
MUSCL without limiter, 2 x 48x48x1 cells), a converged relative entropy
change of 7.883E-07 (entropy measure of SmoothBump/pp/entropy.py). The
fixtures (tests/golden/make_smoothbump.py) hold that case's grid and the
oracle's steady state on it after 10^5 explicit RK4 iterations.  Checked
here: the state is a steady state of the oracle's discretisation, and its
entropy change equals the reference's reported value to the four digits
the report prints, i.e. the oracle converges to the reference's solution.
No GPU."""
import os
import sys

import numpy as np

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_smoothbump as MS  # noqa: E402
from fest3d import post as P  # noqa: E402

REPORT_DS = 7.883e-07  # tests/Report.txt: "Calculated relative change in entropy: 7.883E-07"


def entropy_change(q, vol, p_inf=101325.0, rho_inf=1.225, gm=1.4):
    """SmoothBump/pp/entropy.py at the case's free stream."""
    return P.entropy_change(q, vol, p_inf, rho_inf, gm)


def test_oracle_steady_state_matches_reference_entropy_change():
    nodes_ijk = np.load(os.path.join(HERE, "golden", "smoothbump_nodes.npz"))["nodes"]
    fx = np.load(os.path.join(HERE, "golden", "smoothbump_converged.npz"))
    ext, flow, scheme, bc, nodes, qp = MS.smoothbump_case(nodes_ijk)
    blk = O.Block(ext, flow, scheme, bc)
    blk["nodes"] = nodes
    blk.setup_geometry()
    sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
    # the free stream's residual, for scale
    blk["qp"] = qp
    assert O.get_total_conservative_residue([blk], 1) == 0
    r0 = O.find_resnorm([blk])
    # the fixture state: interior from the fixture, ghosts from the BCs
    q = np.array(qp, order="F")
    q[sl] = fx["q"]
    blk["qp"] = q
    assert O.get_total_conservative_residue([blk], 1) == 0
    r = O.find_resnorm([blk])
    assert r[1] < 1e-3 * r0[1], (r, r0)  # continuity residual: a steady state
    vol = blk["cells"][0][sl]
    ds = entropy_change(fx["q"], vol)
    assert abs(ds - REPORT_DS) <= 0.5e-10, ds  # equal to the report's 4 digits
