"""ctypes mirror of include/fest_gpu.h and loader of the in-tree CUDA library.

The structs follow the Fortran derived types of the reference
(``src/vartypes.f90:21-367``): ``fest_extent`` <- ``extent``,
``fest_flow`` <- ``flowtype``, ``fest_scheme`` <- ``schemetype``,
``fest_bc`` <- ``boundarytype``.  Nothing here computes: it only binds the
C ABI so tests and the benchmark can call it.
"""
import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
LIB_PATH = os.path.join(ROOT, "_build", "libfest_gpu.so")

FEST_OK = 0
FEST_ERR_ARG = 1
FEST_ERR_CUDA = 2
FEST_ERR_NAN = 3
FEST_ERR_NEGATIVE_STATE = 4
FEST_ERR_TIMEOUT = 5
FEST_ERR_NOMEM = 6
FEST_ERR_NO_DEVICE = 7
FEST_ERR_SCRATCH = 8
ERR_NAMES = {0: "FEST_OK", 1: "FEST_ERR_ARG", 2: "FEST_ERR_CUDA", 3: "FEST_ERR_NAN",
             4: "FEST_ERR_NEGATIVE_STATE", 5: "FEST_ERR_TIMEOUT", 6: "FEST_ERR_NOMEM",
             7: "FEST_ERR_NO_DEVICE", 8: "FEST_ERR_SCRATCH"}

FLUX = {"ausm": 0, "ausmP": 1, "ausmUP": 2, "slau": 3, "ldfss0": 4, "van_leer": 5}
INTERP = {"none": 0, "muscl": 1, "ppm": 2, "weno": 3, "weno_NM": 4}
TIME = {"none": 0, "RK2": 1, "RK4": 2, "TVDRK2": 3, "TVDRK3": 4, "implicit": 5, "plusgs": 6}
TURB = {"none": 0, "sst": 1, "sst2003": 2, "sa": 3, "kkl": 4}
TRANSITION = {"none": 0, "bc": 1, "lctm2015": 2}
MU = {"constant": 0, "sutherland_law": 1}
LIMITER = {"koren": 0, "van_albada": 1}
FEST_FP64, FEST_MIXED = 0, 1
FACES = ("imin", "imax", "jmin", "jmax", "kmin", "kmax")


class Extent(C.Structure):
    _fields_ = [("imx", C.c_int), ("jmx", C.c_int), ("kmx", C.c_int), ("n_var", C.c_int)]


class Flow(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "density_inf", "x_speed_inf", "y_speed_inf", "z_speed_inf", "pressure_inf",
        "tk_inf", "tw_inf", "vel_mag", "MInf", "gm", "R_gas", "mu_ref", "T_ref",
        "Sutherland_temp", "Pr", "tPr")] + [("mu_variation", C.c_int), ("reserved", C.c_int),
                                            ("tv_inf", C.c_double), ("tkl_inf", C.c_double),
                                            ("tu_inf", C.c_double), ("tgm_inf", C.c_double)]


class Scheme(C.Structure):
    _fields_ = [("scheme_name", C.c_int), ("interpolant", C.c_int),
                ("time_stepping_method", C.c_int), ("time_step_accuracy", C.c_int),
                ("global_time_step", C.c_double)] + [(n, C.c_int) for n in (
                    "ilimiter_switch", "jlimiter_switch", "klimiter_switch",
                    "itlimiter_switch", "jtlimiter_switch", "ktlimiter_switch",
                    "iPB_switch", "jPB_switch", "kPB_switch", "turbulence", "accur", "limiter",
                    "transition")]


D6 = C.c_double * 6
I6 = C.c_int * 6


class BC(C.Structure):
    _fields_ = [("id", I6), ("partner_block", I6), ("partner_face", I6)] + [(n, D6) for n in (
        "fixed_density", "fixed_pressure", "fixed_x_speed", "fixed_y_speed", "fixed_z_speed",
        "fixed_tk", "fixed_tw", "fixed_wall_temperature", "fixed_Tpressure", "fixed_Ttemperature")] + [
        ("block_id", C.c_int), ("partner_orient", I6), ("fixed_tv", D6), ("fixed_tkl", D6),
        ("fixed_tgm", D6)]


def make_flow(**kw):
    """flowtype with the reference defaults (vartypes.f90:236-285) and the
    derived vel_mag / MInf of init_infinity_values (state.f90:87-88)."""
    d = dict(density_inf=1.2, x_speed_inf=100.0, y_speed_inf=0.0, z_speed_inf=0.0,
             pressure_inf=101325.0, tk_inf=0.0, tw_inf=0.0, tv_inf=0.0, tkl_inf=0.0, tu_inf=1.0, tgm_inf=1.0, gm=1.4,
             R_gas=287.0,
             mu_ref=0.0, T_ref=300.0, Sutherland_temp=110.0, Pr=0.7, tPr=0.9,
             mu_variation="constant")
    d.update(kw)
    f = Flow()
    for k, v in d.items():
        if k == "mu_variation":
            f.mu_variation = MU[v] if isinstance(v, str) else int(v)
        elif k in ("vel_mag", "MInf"):
            continue
        else:
            setattr(f, k, float(v))
    f.vel_mag = np.sqrt(f.x_speed_inf ** 2 + f.y_speed_inf ** 2 + f.z_speed_inf ** 2)
    f.MInf = f.vel_mag / np.sqrt(f.gm * f.pressure_inf / f.density_inf)
    if "vel_mag" in kw:
        f.vel_mag = kw["vel_mag"]
    if "MInf" in kw:
        f.MInf = kw["MInf"]
    return f


def sst_free_stream(flow, tu_inf=1.0, mu_ratio_inf=1.0):
    """Free-stream k and omega of the SST models from the turbulence
    intensity tu_inf (percent) and the eddy-to-laminar viscosity ratio, as
    init_infinity_values derives them (state.f90:90, 98-99; defaults of
    vartypes.f90:256, 266): returns (tk_inf, tw_inf) for make_flow."""
    intensity = tu_inf / 100
    tk = 1.5 * ((flow.vel_mag * intensity) ** 2)
    tw = flow.density_inf * tk / (flow.mu_ref * mu_ratio_inf)
    return tk, tw


def make_scheme(**kw):
    """schemetype with the reference defaults (vartypes.f90:198-231)."""
    d = dict(scheme_name="ausm", interpolant="muscl", time_stepping_method="l",
             time_step_accuracy="none", global_time_step=-1.0, ilimiter_switch=1,
             jlimiter_switch=1, klimiter_switch=1, itlimiter_switch=1, jtlimiter_switch=1,
             ktlimiter_switch=1, iPB_switch=0, jPB_switch=0, kPB_switch=0, turbulence="none",
             accur=1, limiter="koren", transition="none")
    d.update(kw)
    s = Scheme()
    s.scheme_name = FLUX[d["scheme_name"]]
    s.interpolant = INTERP[d["interpolant"]]
    s.time_stepping_method = ord(d["time_stepping_method"])
    s.time_step_accuracy = TIME[d["time_step_accuracy"]]
    s.global_time_step = float(d["global_time_step"])
    for k in ("ilimiter_switch", "jlimiter_switch", "klimiter_switch", "itlimiter_switch",
              "jtlimiter_switch", "ktlimiter_switch", "iPB_switch", "jPB_switch", "kPB_switch",
              "accur"):
        setattr(s, k, int(d[k]))
    s.turbulence = TURB[d["turbulence"]]
    s.limiter = LIMITER[d["limiter"]]
    s.transition = TRANSITION[d["transition"]]
    return s


def make_bc(ids, partners=None, block_id=0, **fixed):
    """boundarytype: ids per face (imin..kmax); partners maps face index ->
    (block, face) or (block, face, orient) for interface faces (orient:
    bit 0/1 the partner's first/second tangential range reversed, bit 2 the
    two swapped); block_id: this block's number in its case; fixed_* arrays
    of 6 values."""
    b = BC()
    b.block_id = int(block_id)
    for f in range(6):
        b.id[f] = int(ids[f])
        b.partner_block[f] = int(block_id)
        b.partner_face[f] = f
        b.partner_orient[f] = 0
    for f, v in (partners or {}).items():
        b.partner_block[f] = int(v[0])
        b.partner_face[f] = int(v[1])
        b.partner_orient[f] = int(v[2]) if len(v) > 2 else 0
    for k, v in fixed.items():
        arr = getattr(b, k)
        for f in range(6):
            arr[f] = float(v[f])
    return b


def n_var_for(scheme):
    """set_n_var_value (state.f90:280-320): 5, 6 for Spalart-Allmaras, 7 for
    the two-equation models, one more with LCTM2015's intermittency"""
    n = {0: 5, TURB["sa"]: 6}.get(scheme.turbulence, 7)
    return n + (scheme.transition == TRANSITION["lctm2015"])


def n_grad_for(n_var):
    """get_n_grad (gradients.f90:229-270): u, v, w, T and the turbulence
    (and LCTM2015's intermittency) variables"""
    return {5: 4, 6: 5, 8: 7}.get(n_var, 6)


# ---- Fortran-shaped array helpers ----------------------------------------
def shapes(ext, n_grad=None):
    """Fortran shapes (numpy, order='F') of every array the C ABI exchanges."""
    i, j, k, n = ext.imx, ext.jmx, ext.kmx, ext.n_var
    ng = n_grad if n_grad is not None else n_grad_for(n)
    return {
        "qp": (i + 5, j + 5, k + 5, n), "pad": (i + 5, j + 5, k + 5),
        "cells": (4, i + 5, j + 5, k + 5), "Ifaces": (4, i + 6, j + 5, k + 5),
        "Jfaces": (4, i + 5, j + 6, k + 5), "Kfaces": (4, i + 5, j + 5, k + 6),
        "nodes": (3, i + 6, j + 6, k + 6),
        "x_qp": (i + 2, j - 1, k - 1, n), "y_qp": (i - 1, j + 2, k - 1, n),
        "z_qp": (i - 1, j - 1, k + 2, n),
        "F": (i, j - 1, k - 1, n), "G": (i - 1, j, k - 1, n), "H": (i - 1, j - 1, k, n),
        "residue": (i - 1, j - 1, k - 1, n), "grad": (i + 1, j + 1, k + 1, ng),
        "delta_t": (i - 1, j - 1, k - 1),
    }


def farray(ext, name, fill=0.0, n_grad=None):
    return np.full(shapes(ext, n_grad)[name], fill, dtype=np.float64, order="F")


def ptr(a):
    """double* of a Fortran-ordered float64 array (None -> NULL)."""
    if a is None:
        return None
    if not (a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim == 1)):
        raise TypeError(f"need an F-contiguous float64 array, got {a.dtype} {a.shape}")
    return a.ctypes.data_as(C.POINTER(C.c_double))


# ---- the CUDA library --------------------------------------------------------
_lib = None
_DP = C.POINTER(C.c_double)
_SIGS = {
    "fest_create": [C.POINTER(Extent), C.POINTER(Flow), C.POINTER(Scheme), C.POINTER(BC),
                    C.POINTER(C.c_void_p)],
    "fest_destroy": [C.c_void_p],
    "fest_set_precision": [C.c_void_p, C.c_int],
    "fest_last_device_error": [C.c_void_p],
    "fest_setup_geometry": [C.c_void_p, _DP, _DP, _DP, _DP, _DP],
    "fest_set_metrics": [C.c_void_p, _DP, _DP, _DP, _DP],
    "fest_find_wall_dist": [C.c_void_p, _DP, C.c_int, _DP],
    "fest_set_wall_dist": [C.c_void_p, _DP],
    "fest_upload_state": [C.c_void_p, _DP],
    "fest_download_state": [C.c_void_p, _DP],
    "fest_snapshot_begin": [C.c_void_p, _DP],
    "fest_snapshot_wait": [C.c_void_p],
    "fest_populate_ghost_primitive": [C.c_void_p, _DP, C.c_int],
    "fest_compute_temperature": [C.c_void_p, _DP, _DP],
    "fest_compute_face_interpolant": [C.c_void_p, _DP, _DP, _DP, _DP, _DP, _DP, _DP],
    "fest_reconstruct_boundary_state": [C.c_void_p, _DP, _DP, _DP, _DP, _DP, _DP, _DP],
    "fest_compute_fluxes": [C.c_void_p, _DP, _DP, _DP],
    "fest_evaluate_all_gradients": [C.c_void_p, _DP, _DP, _DP, _DP, _DP],
    "fest_calculate_viscosity": [C.c_void_p, _DP, _DP, _DP, _DP],
    "fest_compute_viscous_fluxes": [C.c_void_p, _DP, _DP, _DP, _DP],
    "fest_compute_residue": [C.c_void_p, _DP, _DP, _DP, _DP],
    "fest_add_source_term_residue": [C.c_void_p, _DP, _DP],
    "fest_compute_time_step": [C.c_void_p, _DP, C.c_double, _DP],
    "fest_get_total_conservative_residue": [C.c_void_p, _DP, C.c_int, _DP],
    "fest_get_next_solution": [C.c_void_p, _DP, C.c_int, C.c_double, _DP, _DP],
    "fest_find_resnorm": [C.c_void_p, _DP],
    "fest_step": [C.c_void_p, C.c_int, C.c_int, C.c_double, _DP],
    "fest_step_async": [C.c_void_p, C.c_int, C.c_int, C.c_double],
    "fest_step_host": [C.c_void_p, _DP, C.c_int, C.c_int, C.c_double, _DP],
    "fest_step_host_interior": [C.c_void_p, _DP, C.c_int, C.c_int, C.c_double, _DP],
    "fest_set_stream": [C.c_void_p, C.c_void_p],
    "fest_profile": [C.c_void_p, C.c_int],
    "fest_profile_read": [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_double)],
    "fest_batch_create": [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)],
    "fest_batch_destroy": [C.c_void_p],
    "fest_batch_step": [C.c_void_p, C.c_int, C.c_int, C.c_double],
    "fest_batch_step_async": [C.c_void_p, C.c_int, C.c_int, C.c_double],
    "fest_residual_vjp": [C.c_void_p, _DP, C.c_int, _DP, _DP],
    "fest_residual_vjp_nodes": [C.c_void_p, _DP, C.c_int, _DP, _DP, _DP, _DP, _DP, _DP],
    "fest_adjoint_solve": [C.c_void_p, _DP, C.c_double, C.c_int, C.c_double, _DP,
                           C.POINTER(C.c_int), _DP],
    "fest_last_kernel_ms": [C.c_void_p, _DP],
    "fest_measure_peak": [C.c_int, _DP],
    "fest_find_resnorm_noalloc": [C.POINTER(Extent), C.POINTER(Flow), C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, _DP, C.c_void_p],
}
EXPORTED = tuple(_SIGS) + ("fest_kernel_launches", "fest_array_size", "fest_set_array",
                          "fest_get_array")


def load(path=None):
    """Load the in-tree libfest_gpu.so (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"CUDA library not built: {p} (run __graft_entry__.build())")
    lib = C.CDLL(p)
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.fest_kernel_launches.argtypes = [C.c_void_p]
    lib.fest_kernel_launches.restype = C.c_longlong
    if path is None:
        _lib = lib
    return lib


class FestError(RuntimeError):
    def __init__(self, code, where):
        super().__init__(f"{where} returned {ERR_NAMES.get(code, code)}")
        self.code = code


def check(code, where):
    if code != FEST_OK:
        raise FestError(code, where)
    return code


def orient_from_mapping(f1, s21, e21, s22, e22, dir_switch):
    """partner_orient of face f1 (1..6) from its line of the reference's
    mapping file (b1 f1 s11 e11 s12 e12 b2 f2 s21 e21 s22 e22 dir_switch):
    the partner's ranges along this face's tangential directions, reversed
    where they run backwards (mapping.f90:159-236)."""
    del f1  # the same two columns describe every face's tangential directions
    return (1 if s21 > e21 else 0) | (2 if s22 > e22 else 0) | (4 if dir_switch else 0)
