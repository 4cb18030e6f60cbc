"""Helpers shared by the parity tests: one oracle block and one CUDA handle
built from identical inputs, and the comparison rules.

Tolerances (FP64): module outputs agree to 1e-12 relative to the array's
per-variable magnitude (the GPU contracts a*b+c into FMA, the oracle does
not, so bitwise equality is not expected); the residual agrees to 1e-12 of
the sum of |face flux| around each cell (the flux-scaled criterion), plus
1e-12 in global L2."""
import numpy as np

import oracle as O
from fest3d import abi, cases
from fest3d.handle import Handle

RTOL = 1e-12


def make_pair(ext, flow, scheme, bc, nodes, qp, wall=None):
    blk = O.Block(ext, flow, scheme, bc)
    blk["nodes"] = nodes
    blk.setup_geometry()
    h = Handle(ext, flow, scheme, bc)
    h.setup_geometry(nodes)
    if wall is not None and len(wall):
        blk.find_wall_dist(wall)
        h.find_wall_dist(wall)
    elif ext.n_var > 5:
        d = np.full(abi.shapes(ext)["pad"], 0.05, order="F")
        blk["dist"] = d
        h.set("dist", d)
    blk["qp"] = qp
    h.upload_state(qp)
    return blk, h


def rel_err(gpu, ref, axis_last_is_var=True):
    """max |gpu-ref| / max|ref|, per trailing variable when the array has one."""
    gpu = np.asarray(gpu)
    ref = np.asarray(ref)
    assert gpu.shape == ref.shape, (gpu.shape, ref.shape)
    if axis_last_is_var and ref.ndim == 4:
        errs = []
        for l in range(ref.shape[-1]):
            s = np.abs(ref[..., l]).max()
            e = np.abs(gpu[..., l] - ref[..., l]).max()
            errs.append(e / s if s > 0 else e)
        return max(errs)
    s = np.abs(ref).max()
    e = np.abs(gpu - ref).max()
    return e / s if s > 0 else e


def assert_close(gpu, ref, rtol=RTOL, what=""):
    assert np.all(np.isfinite(gpu)) == np.all(np.isfinite(ref)), f"{what}: finiteness differs"
    e = rel_err(gpu, ref)
    assert e <= rtol, f"{what}: relative error {e:.3e} > {rtol:.1e}"
    return e


def face_slice(ext, dir):
    """the faces the reference consumes: 1..n along dir (all tangential)."""
    n = (ext.imx, ext.jmx, ext.kmx)[dir]
    s = [slice(None)] * 4
    s[dir] = slice(1, n + 1)  # x_qp arrays start at face 0 along dir
    return tuple(s)


def flux_scale(blk):
    """sum over the six faces of |F| for every interior cell and variable"""
    F, G, H = blk["F"], blk["G"], blk["H"]
    return (np.abs(F[1:]) + np.abs(F[:-1]) + np.abs(G[:, 1:]) + np.abs(G[:, :-1]) +
            np.abs(H[:, :, 1:]) + np.abs(H[:, :, :-1]))


def assert_residual(gpu_res, blk, rtol=RTOL, what="residue"):
    ref = blk["residue"]
    S = flux_scale(blk)
    floor = 1e-300 + S.max(axis=(0, 1, 2)) * 1e-3
    cell = np.abs(gpu_res - ref) / np.maximum(S, floor)
    e_cell = cell.max()
    l2 = np.sqrt(((gpu_res - ref) ** 2).sum()) / max(np.sqrt((ref ** 2).sum()), 1e-300)
    assert e_cell <= rtol, f"{what}: flux-scaled error {e_cell:.3e} > {rtol:.1e}"
    assert l2 <= rtol, f"{what}: relative L2 {l2:.3e} > {rtol:.1e}"
    return e_cell, l2


def small_case(nc=(9, 7, 6), ids=(-5, -5, -5, -3, -10, -10), scheme_kw=None, flow_kw=None,
               turb=False, perturb=0.15, seed=1, partners=None, fixed=None, state_mach=0.3):
    # turb: False, True (k-omega SST, seven variables), "sa" (six) or
    # "kkl" (seven: k and kL)
    sa, kkl = turb == "sa", turb == "kkl"
    lctm = (scheme_kw or {}).get("transition") == "lctm2015"
    ext = abi.Extent(nc[0] + 1, nc[1] + 1, nc[2] + 1, 6 if sa else 8 if lctm else 7 if turb else 5)
    fk = dict(density_inf=1.2, x_speed_inf=60.0, y_speed_inf=5.0, pressure_inf=101325.0)
    if sa:
        fk["tv_inf"] = 1.2e-4
    if kkl:
        fk["tk_inf"], fk["tkl_inf"] = 1.0, 2e-3
    fk.update(flow_kw or {})
    flow = abi.make_flow(**fk)
    sk = dict(scheme_name="ausm", interpolant="muscl")
    if turb:
        sk["turbulence"] = "sa" if sa else "kkl" if kkl else "sst"
    sk.update(scheme_kw or {})
    scheme = abi.make_scheme(**sk)
    fx = {k: [0.0] * 6 for k in ("fixed_density", "fixed_x_speed", "fixed_y_speed",
                                 "fixed_z_speed", "fixed_pressure", "fixed_tk", "fixed_tw",
                                 "fixed_wall_temperature", "fixed_Tpressure", "fixed_tv", "fixed_tkl",
                                 "fixed_tgm")}
    for f in range(6):
        fx["fixed_density"][f] = 1.15 + 0.01 * f
        fx["fixed_x_speed"][f] = 40.0 + f
        fx["fixed_y_speed"][f] = 2.0 * f
        fx["fixed_z_speed"][f] = -1.0 * f
        fx["fixed_pressure"][f] = 101000.0 + 100 * f
        fx["fixed_tk"][f] = 0.8 + 0.05 * f
        fx["fixed_tw"][f] = 900.0 + 10 * f
        fx["fixed_Tpressure"][f] = 104000.0 + 50 * f
        fx["fixed_tv"][f] = 1.1e-4 + 1e-6 * f
        fx["fixed_tkl"][f] = 1.9e-3 + 2e-5 * f
        fx["fixed_tgm"][f] = 0.9 + 0.01 * f
    for k, v in (fixed or {}).items():
        fx[k] = list(v)
    if partners is None:
        partners = {}
        for f in range(6):
            if ids[f] == -10:
                partners[f] = (0, f ^ 1)
    bc = abi.make_bc(list(ids), partners=partners, **fx)
    nodes = cases.box_nodes(ext, L=(1.0, 0.8, 0.6), perturb=perturb, seed=seed)
    qp = cases.random_state(ext, seed=seed + 7, mach=state_mach, tw=2e-3 if kkl else 1000.0)
    return ext, flow, scheme, bc, nodes, qp
