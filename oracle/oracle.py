"""Python handle on the C restatement (fest_oracle.c) of FEST-3D's explicit path.

TEST INFRASTRUCTURE ONLY.  The parity tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` use it as the checker; the product never
imports it.  ``build()`` compiles the restatement with gcc into
``oracle/_build/libfest_oracle.so`` (parity build: ``-ffp-contract=off`` so no
FMA contraction changes the reference's rounding).
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "fest-3d_gb300"))
from fest3d import abi  # noqa: E402  (parameter structs only)

LIB = os.path.join(HERE, "_build", "libfest_oracle.so")
SRC = os.path.join(HERE, "fest_oracle.c")

(FO_QP, FO_TEMP, FO_NODES, FO_CELLS, FO_IFACES, FO_JFACES, FO_KFACES, FO_XL, FO_XR, FO_YL,
 FO_YR, FO_ZL, FO_ZR, FO_PDIF, FO_F, FO_G, FO_H, FO_RES, FO_GX, FO_GY, FO_GZ, FO_MU, FO_MUT,
 FO_F1, FO_DIST, FO_DT, FO_USTORE, FO_RSTORE) = range(28)

NAMES = {"qp": FO_QP, "Temp": FO_TEMP, "nodes": FO_NODES, "cells": FO_CELLS,
         "Ifaces": FO_IFACES, "Jfaces": FO_JFACES, "Kfaces": FO_KFACES,
         "x_qp_left": FO_XL, "x_qp_right": FO_XR, "y_qp_left": FO_YL, "y_qp_right": FO_YR,
         "z_qp_left": FO_ZL, "z_qp_right": FO_ZR, "pdif": FO_PDIF, "F": FO_F, "G": FO_G,
         "H": FO_H, "residue": FO_RES, "gradqp_x": FO_GX, "gradqp_y": FO_GY, "gradqp_z": FO_GZ,
         "mu": FO_MU, "mu_t": FO_MUT, "sst_F1": FO_F1, "dist": FO_DIST, "delta_t": FO_DT,
         "U_store": FO_USTORE, "R_store": FO_RSTORE}


def build(force=False):
    """Compile the restatement (gcc, OpenMP, no FMA contraction)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "fest_oracle.h"))):
        return LIB
    cmd = ["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           SRC, "-o", LIB, "-lm"]
    subprocess.check_call(cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, ip, dp = C.c_void_p, C.c_int, C.POINTER(C.c_double)
        L.fo_create.argtypes = [C.POINTER(abi.Extent), C.POINTER(abi.Flow),
                                C.POINTER(abi.Scheme), C.POINTER(abi.BC)]
        L.fo_create.restype = vp
        L.fo_destroy.argtypes = [vp]
        L.fo_ptr.argtypes = [vp, ip]
        L.fo_ptr.restype = dp
        L.fo_size.argtypes = [vp, ip]
        L.fo_size.restype = C.c_long
        L.fo_n_grad.argtypes = [vp]
        L.fo_set_threads.argtypes = [ip]
        for name in ("fo_setup_geometry", "fo_compute_temperature", "fo_reconstruct_boundary_state",
                     "fo_compute_residue", "fo_add_source_term_residue"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = None
        for name in ("fo_compute_face_interpolant", "fo_compute_fluxes",
                     "fo_evaluate_all_gradients", "fo_calculate_viscosity",
                     "fo_compute_viscous_fluxes"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = ip
        L.fo_find_wall_dist.argtypes = [vp, dp, ip]
        L.fo_find_wall_dist.restype = None
        L.fo_populate_ghost_primitive.argtypes = [vp, ip]
        L.fo_compute_time_step.argtypes = [vp, C.c_double]
        L.fo_compute_time_step.restype = None
        L.fo_update_with.argtypes = [vp, C.c_double, C.c_double, ip, ip]
        pvp = C.POINTER(vp)
        L.fo_apply_interface.argtypes = [pvp, ip]
        L.fo_apply_interface.restype = None
        L.fo_get_total_conservative_residue.argtypes = [pvp, ip, ip]
        L.fo_get_next_solution.argtypes = [pvp, ip, ip, C.c_double]
        L.fo_lusgs_next_solution.argtypes = [pvp, ip, ip, C.c_double]
        L.fo_plusgs_next_solution.argtypes = [pvp, ip, ip, C.c_double]
        L.fo_find_resnorm.argtypes = [pvp, ip, dp]
        L.fo_find_resnorm.restype = None
        _lib = L
    return _lib


def set_threads(n):
    return lib().fo_set_threads(int(n))


class Block:
    """One block of the reference (one MPI rank) held by the restatement.

    ``blk["qp"]`` etc. are zero-copy numpy views with the reference's
    Fortran shapes (order='F'); index ``qp[i+2, j+2, k+2, l-1]``."""

    def __init__(self, ext, flow, scheme, bc):
        self.ext, self.flow, self.scheme, self.bc = ext, flow, scheme, bc
        self.h = lib().fo_create(C.byref(ext), C.byref(flow), C.byref(scheme), C.byref(bc))
        self.n_grad = lib().fo_n_grad(self.h)
        sh = abi.shapes(ext, self.n_grad)
        self._shape = {"qp": sh["qp"], "Temp": sh["pad"], "nodes": sh["nodes"],
                       "cells": sh["cells"], "Ifaces": sh["Ifaces"], "Jfaces": sh["Jfaces"],
                       "Kfaces": sh["Kfaces"], "x_qp_left": sh["x_qp"], "x_qp_right": sh["x_qp"],
                       "y_qp_left": sh["y_qp"], "y_qp_right": sh["y_qp"],
                       "z_qp_left": sh["z_qp"], "z_qp_right": sh["z_qp"],
                       "pdif": (ext.imx + 1, ext.jmx + 1, ext.kmx + 1), "F": sh["F"],
                       "G": sh["G"], "H": sh["H"], "residue": sh["residue"],
                       "gradqp_x": sh["grad"], "gradqp_y": sh["grad"], "gradqp_z": sh["grad"],
                       "mu": sh["pad"], "mu_t": sh["pad"], "sst_F1": sh["pad"],
                       "dist": sh["pad"], "delta_t": sh["delta_t"], "U_store": sh["qp"],
                       "R_store": sh["residue"]}

    def __del__(self):
        try:
            if self.h:
                lib().fo_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def __getitem__(self, name):
        aid = NAMES[name]
        n = lib().fo_size(self.h, aid)
        p = lib().fo_ptr(self.h, aid)
        flat = np.ctypeslib.as_array(p, shape=(n,))
        return flat.reshape(self._shape[name], order="F")

    def __setitem__(self, name, value):
        self[name][...] = value

    # ---- one call per reference procedure ----
    def setup_geometry(self):
        lib().fo_setup_geometry(self.h)

    def find_wall_dist(self, wall_xyz):
        w = np.ascontiguousarray(wall_xyz, dtype=np.float64)
        lib().fo_find_wall_dist(self.h, w.ctypes.data_as(C.POINTER(C.c_double)), len(w))

    def populate_ghost_primitive(self, it):
        return lib().fo_populate_ghost_primitive(self.h, int(it))

    def compute_temperature(self):
        lib().fo_compute_temperature(self.h)

    def compute_face_interpolant(self):
        return lib().fo_compute_face_interpolant(self.h)

    def reconstruct_boundary_state(self):
        lib().fo_reconstruct_boundary_state(self.h)

    def compute_fluxes(self):
        return lib().fo_compute_fluxes(self.h)

    def evaluate_all_gradients(self):
        return lib().fo_evaluate_all_gradients(self.h)

    def calculate_viscosity(self):
        return lib().fo_calculate_viscosity(self.h)

    def compute_viscous_fluxes(self):
        return lib().fo_compute_viscous_fluxes(self.h)

    def compute_residue(self):
        lib().fo_compute_residue(self.h)

    def add_source_term_residue(self):
        lib().fo_add_source_term_residue(self.h)

    def compute_time_step(self, CFL):
        lib().fo_compute_time_step(self.h, float(CFL))

    def update_with(self, TF, SF, TU=False, use_store=False):
        return lib().fo_update_with(self.h, float(TF), float(SF), int(TU), int(use_store))


def _arr(blocks):
    return (C.c_void_p * len(blocks))(*[b.h for b in blocks])


def apply_interface(blocks):
    lib().fo_apply_interface(_arr(blocks), len(blocks))


def get_total_conservative_residue(blocks, it):
    return lib().fo_get_total_conservative_residue(_arr(blocks), len(blocks), int(it))


def get_next_solution(blocks, it, CFL):
    return lib().fo_get_next_solution(_arr(blocks), len(blocks), int(it), float(CFL))


def lusgs_next_solution(blocks, it, CFL):
    """one iteration of the reference's implicit LU-SGS integrator (laminar
    blocks), for replaying the reference's implicit test runs"""
    return lib().fo_lusgs_next_solution(_arr(blocks), len(blocks), int(it), float(CFL))


def plusgs_next_solution(blocks, it, CFL):
    """one iteration of the reference's low-Mach preconditioned PLU-SGS
    integrator (plusgs.f90, laminar and k-omega SST blocks)"""
    return lib().fo_plusgs_next_solution(_arr(blocks), len(blocks), int(it), float(CFL))


def find_resnorm(blocks):
    out = np.zeros(blocks[0].ext.n_var + 1)
    lib().fo_find_resnorm(_arr(blocks), len(blocks), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out
