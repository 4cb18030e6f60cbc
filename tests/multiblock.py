"""A two-block case cut from one block, for the interface exchange tests.

The block (Ni x Nj x Nk cells) is cut at i = Ni/2.  Block 0 keeps the low
half as it is.  Block 1 holds the high half with its indices rotated a
quarter turn about the i axis: its j runs along the original k and its k
against the original j, so the interface pairs columns with a swap of the
two tangential directions and one reversal, as a mapping-file line with
dir_switch 1 and one backwards range describes it (mapping.f90:64-236).
The rotation keeps the index system right-handed, so volumes and face
normals keep their sign.  The state and nodes are the same physical
fields, so the two-block case has the same residual as the single block
(up to rounding: fluxes of rotated faces are summed in another order).
Its time steps differ: the reference's local time step takes the high
face's term with the neighbour cell's velocity (time.f90:199-223), which a
reversed direction turns into the low face.  split_aligned cuts without
rotating, which advances the same flow.

Faces (imin, imax, jmin, jmax, kmin, kmax) of the single block: inlet -3,
outlet -4, no-slip wall -5 at jmin, extrapolation -2 at jmax, periodic k.
In block 1 the periodic pair becomes its j faces and the wall its kmax.
"""
import numpy as np

from fest3d import abi, cases


def _bc(ids, partners, block_id, fixed):
    return abi.make_bc(ids, partners=partners, block_id=block_id, **fixed)


def single_block(nc=(16, 10, 6), scheme_kw=None, flow_kw=None, seed=3):
    """(ext, flow, scheme, bc, nodes, qp) of the uncut block."""
    Ni, Nj, Nk = nc
    ext = abi.Extent(Ni + 1, Nj + 1, Nk + 1, 5)
    fk = dict(density_inf=1.2, x_speed_inf=60.0, y_speed_inf=4.0, pressure_inf=101325.0)
    fk.update(flow_kw or {})
    flow = abi.make_flow(**fk)
    sk = dict(scheme_name="ausm", interpolant="muscl")
    sk.update(scheme_kw or {})
    scheme = abi.make_scheme(**sk)
    fixed = fixed_values()
    bc = _bc([-3, -4, -5, -2, -10, -10], {4: (0, 5), 5: (0, 4)}, 0, fixed)
    nodes = cases.box_nodes(ext, L=(1.6, 1.0, 0.6), perturb=0.12, seed=seed)
    qp = cases.random_state(ext, seed=seed + 11, mach=0.3)
    return ext, flow, scheme, bc, nodes, qp


def fixed_values():
    fx = {k: [0.0] * 6 for k in ("fixed_density", "fixed_x_speed", "fixed_y_speed",
                                 "fixed_z_speed", "fixed_pressure", "fixed_wall_temperature")}
    fx["fixed_density"][0] = 1.18
    fx["fixed_x_speed"][0] = 55.0
    fx["fixed_y_speed"][0] = 3.0
    fx["fixed_pressure"][1] = 101000.0
    return fx


# Block 1's indices (i', j', k') from the original (i, j, k) of its half:
# i' = i - Ni/2, j' = k, k' = Nj + 1 - j (cells; nodes: k' = Nj + 2 - j).
def _rotate_cells(a, Nj):
    """padded cell array (i, j, k, ...) -> block 1 order (i, k, reversed j)."""
    b = np.swapaxes(a, 1, 2)          # (i, k, j)
    return np.ascontiguousarray(b[:, :, ::-1]).copy(order="F")  # j reversed: k' = Nj+1-j


def split_aligned(ext, flow, scheme, nodes, qp):
    """The two halves without rotation: list of (ext, bc, nodes, qp), block
    0's imax paired with block 1's imin column for column."""
    Ni, Nj, Nk = ext.imx - 1, ext.jmx - 1, ext.kmx - 1
    h = Ni // 2
    fixed = fixed_values()
    out = []
    for b, (lo, n) in enumerate(((0, h), (h, Ni - h))):
        e = abi.Extent(n + 1, Nj + 1, Nk + 1, 5)
        nd = cases.empty_nodes(e)
        nd[:, 3:3 + n + 1] = nodes[:, 3 + lo:3 + lo + n + 1]
        q = np.asfortranarray(qp[lo:lo + n + 6].copy())
        ids = [-3, 1, -5, -2, -10, -10] if b == 0 else [0, -4, -5, -2, -10, -10]
        partners = {4: (b, 5), 5: (b, 4)}
        partners[1 if b == 0 else 0] = (1 - b, 0 if b == 0 else 1, 0)
        out.append((e, _bc(ids, partners, b, fixed), nd, q))
    return out


def merge_aligned(ext, q0, q1):
    """The two halves' padded states back in the single block's frame."""
    h = (ext.imx - 1) // 2
    q = np.zeros(abi.shapes(ext)["qp"], order="F")
    q[0:h + 3] = q0[0:h + 3]
    q[h + 3:] = q1[3:]
    return q


def split_rotated(ext, flow, scheme, nodes, qp):
    """The two blocks: list of (ext, bc, nodes, qp), the interface pairs
    block 0's imax with block 1's imin."""
    Ni, Nj, Nk = ext.imx - 1, ext.jmx - 1, ext.kmx - 1
    h = Ni // 2
    fixed = fixed_values()
    # block 0: cells 1..h (padded -2..h+3), nodes 1..h+1 (padded -2..h+4)
    e0 = abi.Extent(h + 1, Nj + 1, Nk + 1, 5)
    n0 = cases.empty_nodes(e0)
    n0[:, 3:3 + h + 1] = nodes[:, 3:3 + h + 1]
    q0 = np.asfortranarray(qp[0:h + 6].copy())
    # block 1: original cells h+1..Ni; its imin face (original i = h+1) pairs
    # with block 0's imax.  Swap (j', k') = (k, reversed j): dir_switch, and
    # block 1's second tangential direction runs against block 0's first.
    e1 = abi.Extent(Ni - h + 1, Nk + 1, Nj + 1, 5)
    n1 = cases.empty_nodes(e1)
    interior = nodes[:, 3 + h:3 + Ni + 1, 3:3 + Nj + 1, 3:3 + Nk + 1]  # (3, i, j, k) interior nodes
    n1[:, 3:3 + Ni - h + 1, 3:3 + Nk + 1, 3:3 + Nj + 1] = np.swapaxes(interior, 2, 3)[:, :, :, ::-1]
    q1 = _rotate_cells(qp[h:Ni + 6], Nj)
    # block 0's imax ghost column (ta=j, tb=k) reads block 1 at (j'=k, k'=Nj+1-j):
    # swap, and the first direction (j) reversed into block 1's second: orient 1|4
    # block 1's imin column (ta=j', tb=k') reads block 0 at (j=Nj+1-k', k=j'):
    # swap, second direction reversed: orient 2|4
    bc0 = _bc([-3, 1, -5, -2, -10, -10], {1: (1, 0, 5), 4: (0, 5), 5: (0, 4)}, 0, fixed)
    # block 1 faces: imin interface, imax outlet, j faces the periodic pair,
    # kmin (k'=1: original j = Nj) extrapolation, kmax (original j = 1) wall
    f1 = {k: [0.0] * 6 for k in fixed}
    for k in fixed:
        f1[k][0] = fixed[k][0]
        f1[k][1] = fixed[k][1]
    bc1 = _bc([0, -4, -10, -10, -2, -5], {0: (0, 1, 6), 2: (1, 3), 3: (1, 2)}, 1, f1)
    return [(e0, bc0, n0, q0), (e1, bc1, n1, q1)]


def merge_rotated(ext, q0, q1):
    """The two blocks' padded states back in the single block's frame
    (interior cells only are meaningful)."""
    Ni, Nj = ext.imx - 1, ext.jmx - 1
    h = Ni // 2
    q = np.zeros(abi.shapes(ext)["qp"], order="F")
    q[0:h + 3] = q0[0:h + 3]
    back = np.swapaxes(q1[:, :, ::-1], 1, 2)  # (i', k', j') -> (i, j, k)
    q[h + 3:] = back[3:]
    return q
