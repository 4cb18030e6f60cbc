"""The interface exchange between blocks, in the oracle (no GPU).

A block cut in two (tests/multiblock.py) advances the same flow as the
uncut block; with the second half's indices turned a quarter turn, the
interface maps its columns with the swap and the reversal of the
reference's mapping file (interface1.f90:96-464, mapping.f90:64-236) and
the residual equals the uncut block's.  This pins the oracle's interface
handling, which the GPU batch tests then check against.  Also: partner
orientations from mapping-file lines, and block numbers resolving
partners."""
import numpy as np
import pytest

import oracle as O
from fest3d import abi, post
import multiblock as MB


def _run(blocks, iters, CFL=0.5):
    for it in range(1, iters + 1):
        assert O.get_next_solution(blocks, it, CFL) == 0


def _oracle_blocks(parts, flow, scheme):
    out = []
    for ext, bc, nodes, qp in parts:
        b = O.Block(ext, flow, scheme, bc)
        b["nodes"] = nodes
        b.setup_geometry()
        b["qp"] = qp
        out.append(b)
    return out


SCHEMES = [dict(interpolant="muscl", scheme_name="ausm", time_step_accuracy="TVDRK3"),
           dict(interpolant="weno", scheme_name="slau", time_step_accuracy="RK4")]
SCHEME_IDS = ["muscl-ausm-tvdrk3", "weno-slau-rk4"]


def _scale(ref, flow):
    V = flow.vel_mag
    return [np.abs(ref[..., 0]).max(), V, V, V, np.abs(ref[..., 4]).max()]


@pytest.mark.parametrize("scheme_kw", SCHEMES, ids=SCHEME_IDS)
def test_aligned_two_block_cut_advances_like_the_uncut_block(scheme_kw):
    ext, flow, scheme, bc, nodes, qp = MB.single_block(scheme_kw=scheme_kw)
    one = _oracle_blocks([(ext, bc, nodes, qp)], flow, scheme)
    two = _oracle_blocks(MB.split_aligned(ext, flow, scheme, nodes, qp), flow, scheme)
    _run(one, 3)
    _run(two, 3)
    ref = post.interior(one[0]["qp"], ext)
    got = post.interior(MB.merge_aligned(ext, two[0]["qp"], two[1]["qp"]), ext)
    sc = _scale(ref, flow)
    err = max(np.abs(got[..., l] - ref[..., l]).max() / sc[l] for l in range(5))
    assert err <= 1e-12, err
    assert np.abs(ref[..., 4] - post.interior(qp, ext)[..., 4]).max() > 1.0  # the flow moved


@pytest.mark.parametrize("scheme_kw", SCHEMES, ids=SCHEME_IDS)
def test_rotated_two_block_cut_has_the_uncut_residual(scheme_kw):
    """the swap and the reversal of the interface map: the residual of every
    cell, the cut's included, equals the uncut block's"""
    ext, flow, scheme, bc, nodes, qp = MB.single_block(scheme_kw=scheme_kw)
    one = _oracle_blocks([(ext, bc, nodes, qp)], flow, scheme)
    parts = MB.split_rotated(ext, flow, scheme, nodes, qp)
    two = _oracle_blocks(parts, flow, scheme)
    # the cut's geometry: the rotated half's cells have the same volumes
    v1 = MB.merge_rotated(ext, two[0]["cells"][0][..., None], two[1]["cells"][0][..., None])[..., 0]
    assert np.allclose(post.interior(v1, ext), post.interior(one[0]["cells"][0], ext), rtol=1e-13, atol=0)
    assert O.get_total_conservative_residue(one, 1) == 0
    assert O.get_total_conservative_residue(two, 1) == 0
    h = (ext.imx - 1) // 2
    r = one[0]["residue"]
    r0 = two[0]["residue"]
    r1 = np.swapaxes(two[1]["residue"][:, :, ::-1], 1, 2)  # block 1's (i, k, reversed j) back
    scale = np.abs(r).max(axis=(0, 1, 2))
    assert np.all(np.abs(r0 - r[:h]).max(axis=(0, 1, 2)) <= 1e-13 * scale)
    assert np.all(np.abs(r1 - r[h:]).max(axis=(0, 1, 2)) <= 1e-13 * scale)


def test_orientation_from_mapping_lines():
    # the reference's own two-block cases: aligned ranges, no switch
    # (tests/SmoothBump/system/mesh/layout/mapping.txt: "0 2 1 49 1 2 1 1 1 49 1 2 0")
    assert abi.orient_from_mapping(2, 1, 49, 1, 2, 0) == 0
    assert abi.orient_from_mapping(1, 49, 1, 1, 2, 0) == 1
    assert abi.orient_from_mapping(3, 1, 9, 17, 1, 1) == 6


def test_partner_by_block_number():
    """a face pairs with the block whose block_id is its partner_block; with
    its own number, with the block itself"""
    ext, flow, scheme, bc, nodes, qp = MB.single_block(nc=(8, 6, 6))
    parts = MB.split_rotated(ext, flow, scheme, nodes, qp)
    # list order does not matter: block numbers do
    two = _oracle_blocks(parts[::-1], flow, scheme)
    ref = _oracle_blocks(parts, flow, scheme)
    _run(two, 2)
    _run(ref, 2)
    for a, b in zip(two[::-1], ref):
        assert np.array_equal(post.interior(a["qp"], a.ext), post.interior(b["qp"], b.ext))
