"""Make the SmoothBump fixtures from the reference's SmoothBump test case
(tests/SmoothBump of FEST-3D):

* smoothbump_nodes.npz: the grid.  The case's two 49x49x2-node blocks
  (system/mesh/gridfiles/grid_0{0,1}.txt) abut in i (layout.md,
  mapping.txt: block 0 imax = block 1 imin); they are written as one
  97x49x2-node block, whose stencil reads across the seam exactly what the
  interface exchange copies into the ghost cells.
* smoothbump_converged.npz (with --converge N): the oracle's steady state
  on that grid after N RK4 iterations (CFL 1.5, local time steps) from the
  free stream, interior cells only, with the case's scheme and BCs
  (system/fvscheme.md, flow.md, bc_0{0,1}.md): AUSM, MUSCL without limiter
  or pressure switch, first-order ghost cells; far field (-8) at imin,
  subsonic outlet (-4, pressure 101325) at imax, slip walls (-6) elsewhere.
  The reference solved the same discretisation implicitly; its entropy
  error (tests/Report.txt) is the test's reference value.

Run in the container that holds the reference:

    python tests/golden/make_smoothbump.py /root/reference/tests/SmoothBump --converge 100000
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def read_grid(path):
    """FEST-3D grid file as (imx, jmx, kmx, 3) nodes (fest3d.files)."""
    sys.path.insert(0, os.path.join(ROOT, "fest-3d_gb300"))
    from fest3d.files import read_grid as read
    return read(path)


def smoothbump_case(nodes_ijk):
    """The reference SmoothBump configuration on the merged grid."""
    sys.path.insert(0, os.path.join(ROOT, "fest-3d_gb300"))
    from fest3d import abi, cases
    imx, jmx, kmx = nodes_ijk.shape[:3]
    ext = abi.Extent(imx, jmx, kmx, 5)
    flow = abi.make_flow(density_inf=1.225, x_speed_inf=170.14, pressure_inf=101325.0, mu_ref=0.0,
                         gm=1.4, R_gas=287.0)
    scheme = abi.make_scheme(scheme_name="ausm", interpolant="muscl", time_step_accuracy="RK4",
                             time_stepping_method="l", ilimiter_switch=0, jlimiter_switch=0,
                             klimiter_switch=0, accur=0)
    bc = abi.make_bc([-8, -4, -6, -6, -6, -6], fixed_pressure=[101325.0] * 6)
    nodes = cases.set_interior_nodes(cases.empty_nodes(ext), nodes_ijk[..., 0], nodes_ijk[..., 1],
                                     nodes_ijk[..., 2])
    return ext, flow, scheme, bc, nodes, cases.uniform_state(ext, flow)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case_dir", help="the reference's SmoothBump case directory")
    ap.add_argument("--converge", type=int, default=0, metavar="N")
    args = ap.parse_args()
    g = os.path.join(args.case_dir, "system", "mesh", "gridfiles")
    b0 = read_grid(os.path.join(g, "grid_00.txt"))
    b1 = read_grid(os.path.join(g, "grid_01.txt"))
    assert np.array_equal(b0[-1], b1[0]), "blocks must share their interface node plane"
    nodes_ijk = np.concatenate([b0, b1[1:]], axis=0)
    np.savez_compressed(os.path.join(HERE, "smoothbump_nodes.npz"), nodes=nodes_ijk)
    print("smoothbump_nodes.npz", nodes_ijk.shape)
    if not args.converge:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    ext, flow, scheme, bc, nodes, qp = smoothbump_case(nodes_ijk)
    blk = O.Block(ext, flow, scheme, bc)
    blk["nodes"] = nodes
    blk.setup_geometry()
    blk["qp"] = qp
    O.set_threads(os.cpu_count() or 1)
    for it in range(1, args.converge + 1):
        assert O.get_next_solution([blk], it, 1.5) == 0
    q = blk["qp"][3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2, :]
    np.savez_compressed(os.path.join(HERE, "smoothbump_converged.npz"), q=q, iterations=args.converge,
                        resnorm=O.find_resnorm([blk]))
    print("smoothbump_converged.npz", q.shape)


if __name__ == "__main__":
    main()
