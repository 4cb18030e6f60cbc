"""Make tests/golden/flatplate_laminar.npz from the reference's laminar
flat-plate test case (tests/Lfp of FEST-3D) and, with --turbulent,
tests/golden/flatplate_sst.npz from its turbulent one (tests/Tfp: k-omega
SST, Sutherland viscosity 1.63416585e-5 at 300 K, free stream 69.445 m/s,
turbulence intensity 0.03873 % and viscosity ratio 0.01 turned into k and
omega as state.f90:98-99 does, a 2 m plate; blocks of 7x49x2 and 29x49x2
nodes; wall distances from the plate's nodes; CFL 1.0).

Laminar case: its two blocks (grid_00.txt,
21x41x2 nodes, the run-in with a slip floor; grid_01.txt, 37x41x2 nodes, the
no-slip adiabatic plate from x = 0 to 1), joined at an interface (layout.md,
mapping.txt), and the oracle's steady state on them after N RK4 iterations
(CFL 1.5, local time steps) from the free stream, with the case's scheme,
flow and BCs (system/fvscheme.md, flow.md, bc_0{0,1}.md): AUSM, MUSCL
without limiter or pressure switch, first-order ghost cells, constant
viscosity 2.12653e-4 (Re 10^6 on the plate), far field (-8) at the inlet,
subsonic outlet (-4, pressure 105472.5), slip (-6) and wall (-5) faces.
Saved: both blocks' nodes and interior states.  Run in the container that
holds the reference:

    python tests/golden/make_flatplate.py /root/reference/tests/Lfp --converge 60000
    python tests/golden/make_flatplate.py /root/reference/tests/Tfp --turbulent --converge 150000
    python tests/golden/make_flatplate.py /root/reference/tests/Tfp --restart

The last writes tests/golden/flatplate_sst_restart.npz: the turbulent
case's own starting state, which its run restarts from (see
restart_states).
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from make_smoothbump import read_grid  # noqa: E402

U_INF, RHO_INF, P_INF, MU = 173.5943, 1.225, 105472.5, 2.12653e-4


def flatplate_case(grids):
    """The reference laminar flat-plate configuration on its two blocks:
    (ext, flow, scheme, bc, nodes, qp) per block."""
    sys.path.insert(0, os.path.join(ROOT, "fest-3d_gb300"))
    from fest3d import abi, cases
    flow = abi.make_flow(density_inf=RHO_INF, x_speed_inf=U_INF, pressure_inf=P_INF, mu_ref=MU,
                         mu_variation="constant", T_ref=300.0, Sutherland_temp=110.5, Pr=0.72, tPr=0.9,
                         gm=1.4, R_gas=287.0)
    scheme = abi.make_scheme(scheme_name="ausm", interpolant="muscl", time_step_accuracy="RK4",
                             time_stepping_method="l", ilimiter_switch=0, jlimiter_switch=0,
                             klimiter_switch=0, accur=0)
    fixed = dict(fixed_pressure=[P_INF] * 6, fixed_wall_temperature=[0.0] * 6)
    bcs = [abi.make_bc([-8, 1, -6, -6, -6, -6], partners={1: (1, 0)}, **fixed),
           abi.make_bc([0, -4, -5, -6, -6, -6], partners={0: (0, 1)}, block_id=1, **fixed)]
    out = []
    for n, bc in zip(grids, bcs):
        ext = abi.Extent(*n.shape[:3], 5)
        nodes = cases.set_interior_nodes(cases.empty_nodes(ext), n[..., 0], n[..., 1], n[..., 2])
        out.append((ext, flow, scheme, bc, nodes, cases.uniform_state(ext, flow)))
    return out


# the turbulent case (tests/Tfp/system/flow.md)
T_RHO, T_U, T_P, T_MU = 1.17659, 69.445, 101325.0, 1.63416585e-05
T_TK = 1.5 * (T_U * 0.03873 / 100.0) ** 2
T_TW = T_RHO * T_TK / (T_MU * 0.01)


def flatplate_sst_case(grids):
    """The reference turbulent flat-plate configuration on its two blocks:
    (ext, flow, scheme, bc, nodes, qp) per block; wall distances from
    wall_nodes()."""
    sys.path.insert(0, os.path.join(ROOT, "fest-3d_gb300"))
    from fest3d import abi, cases
    flow = abi.make_flow(density_inf=T_RHO, x_speed_inf=T_U, pressure_inf=T_P, mu_ref=T_MU,
                         mu_variation="sutherland_law", T_ref=300.0, Sutherland_temp=110.5, Pr=0.72, tPr=0.9,
                         gm=1.4, R_gas=287.0, tk_inf=T_TK, tw_inf=T_TW)
    scheme = abi.make_scheme(scheme_name="ausm", interpolant="muscl", time_step_accuracy="RK4",
                             time_stepping_method="l", ilimiter_switch=0, jlimiter_switch=0,
                             klimiter_switch=0, accur=0, turbulence="sst")
    fixed = dict(fixed_pressure=[T_P] * 6, fixed_wall_temperature=[0.0] * 6, fixed_tk=[T_TK] * 6,
                 fixed_tw=[T_TW] * 6, fixed_density=[T_RHO] * 6, fixed_x_speed=[T_U] * 6,
                 fixed_y_speed=[0.0] * 6, fixed_z_speed=[0.0] * 6)
    bcs = [abi.make_bc([-8, 1, -6, -6, -6, -6], partners={1: (1, 0)}, **fixed),
           abi.make_bc([0, -4, -5, -6, -6, -6], partners={0: (0, 1)}, block_id=1, **fixed)]
    out = []
    for n, bc in zip(grids, bcs):
        ext = abi.Extent(*n.shape[:3], 7)
        nodes = cases.set_interior_nodes(cases.empty_nodes(ext), n[..., 0], n[..., 1], n[..., 2])
        out.append((ext, flow, scheme, bc, nodes, cases.uniform_state(ext, flow, tk=T_TK, tw=T_TW)))
    return out


def wall_nodes(case):
    """the plate's nodes (block 1, jmin) in the reference's surface order"""
    sys.path.insert(0, os.path.join(ROOT, "fest-3d_gb300"))
    from fest3d import cases
    ext, flow, scheme, bc, nodes, qp = case[1]
    return cases.wall_nodes_of(nodes, ext, bc)


def read_tecplot_block(path, nodes_shape, n_cell_vars):
    """A block-packed Tecplot dump as the reference writes it
    (write_output_tec.f90): x, y, z at the nodes, then n_cell_vars
    cell-centred scalars over the interior cells, one value per line after
    a header of variable names and zone records."""
    vals, started = [], False
    for line in open(path):
        t = line.split()
        if not t:
            continue
        if not started:
            try:
                float(t[0])
                started = True
            except ValueError:
                continue
        vals.extend(float(x) for x in t)
    v = np.array(vals)
    ni, nj, nk = nodes_shape
    nn, nc = ni * nj * nk, (ni - 1) * (nj - 1) * (nk - 1)
    assert v.size == 3 * nn + n_cell_vars * nc, (path, v.size)
    xyz = np.stack([v[m * nn:(m + 1) * nn].reshape(nodes_shape, order="F") for m in range(3)], axis=-1)
    cc = [v[3 * nn + m * nc:3 * nn + (m + 1) * nc].reshape((ni - 1, nj - 1, nk - 1), order="F")
          for m in range(n_cell_vars)]
    return xyz, cc


def restart_states(case_dir, grids):
    """The turbulent case's starting state (control.md "Restart level 2"):
    its dumps time_directories/0002/process_0{0,1}.dat hold u, v, w,
    density, pressure and Mu; the reference reads velocity, density and
    pressure (output_control.md read list) into the interior cells over a
    free-stream state (state.f90:181-187), so k and omega start at their
    free-stream values.  Returns per block the interior (rho, u, v, w, p)."""
    out = []
    for b, g in enumerate(grids):
        path = os.path.join(case_dir, "time_directories", "0002", f"process_0{b}.dat")
        xyz, (u, v, w, rho, p, _mu) = read_tecplot_block(path, g.shape[:3], 6)
        assert np.array_equal(xyz, g), "the restart dump must be on the case's grid"
        out.append(np.stack([rho, u, v, w, p], axis=-1))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case_dir", help="the reference's Lfp or Tfp case directory")
    ap.add_argument("--converge", type=int, default=60000, metavar="N")
    ap.add_argument("--turbulent", action="store_true")
    ap.add_argument("--restart", action="store_true",
                    help="write the turbulent case's restart state (flatplate_sst_restart.npz) and stop")
    args = ap.parse_args()
    g = os.path.join(args.case_dir, "system", "mesh", "gridfiles")
    grids = [read_grid(os.path.join(g, f"grid_0{b}.txt")) for b in (0, 1)]
    assert np.array_equal(grids[0][-1], grids[1][0]), "blocks must share their interface node plane"
    if args.restart:
        qs = restart_states(args.case_dir, grids)
        np.savez_compressed(os.path.join(HERE, "flatplate_sst_restart.npz"), q0=qs[0], q1=qs[1])
        print("flatplate_sst_restart.npz", [q.shape for q in qs])
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    case = flatplate_sst_case(grids) if args.turbulent else flatplate_case(grids)
    blocks = []
    for ext, flow, scheme, bc, nodes, qp in case:
        blk = O.Block(ext, flow, scheme, bc)
        blk["nodes"] = nodes
        blk.setup_geometry()
        blk["qp"] = qp
        blocks.append(blk)
    if args.turbulent:
        wall = wall_nodes(case)
        for blk in blocks:
            blk.find_wall_dist(wall)
    cfl = 1.0 if args.turbulent else 1.5
    O.set_threads(os.cpu_count() or 1)
    for it in range(1, args.converge + 1):
        assert O.get_next_solution(blocks, it, cfl) == 0
    qs = [b["qp"][3:b.ext.imx + 2, 3:b.ext.jmx + 2, 3:b.ext.kmx + 2, :] for b in blocks]
    name = "flatplate_sst.npz" if args.turbulent else "flatplate_laminar.npz"
    np.savez_compressed(os.path.join(HERE, name), nodes0=grids[0], nodes1=grids[1],
                        q0=qs[0], q1=qs[1], iterations=args.converge, resnorm=O.find_resnorm(blocks))
    print(name, [q.shape for q in qs])


if __name__ == "__main__":
    main()
