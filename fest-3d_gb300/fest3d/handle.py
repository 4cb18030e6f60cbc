"""A Python object over one ``fest_handle`` of the C ABI.

Every method is one C call (include/fest_gpu.h) with the reference's
Fortran-shaped arrays; ``None`` passes NULL (keep the device-resident copy).
"""
import ctypes as C

import numpy as np

from . import abi

ARR = {"qp": 0, "Temp": 1, "cells": 2, "Ifaces": 3, "Jfaces": 4, "Kfaces": 5, "nodes": 6,
       "x_qp_left": 7, "x_qp_right": 8, "y_qp_left": 9, "y_qp_right": 10, "z_qp_left": 11,
       "z_qp_right": 12, "F": 13, "G": 14, "H": 15, "residue": 16, "gradqp_x": 17,
       "gradqp_y": 18, "gradqp_z": 19, "mu": 20, "mu_t": 21, "sst_F1": 22, "dist": 23,
       "delta_t": 24}


class Handle:
    def __init__(self, ext, flow, scheme, bc, lib=None):
        self.lib = lib or abi.load()
        self.ext, self.flow, self.scheme, self.bc = ext, flow, scheme, bc
        self.h = C.c_void_p()
        abi.check(self.lib.fest_create(C.byref(ext), C.byref(flow), C.byref(scheme), C.byref(bc),
                                       C.byref(self.h)), "fest_create")
        ng = abi.n_grad_for(ext.n_var)
        sh = abi.shapes(ext, ng)
        self.shape = {"qp": sh["qp"], "Temp": sh["pad"], "cells": sh["cells"],
                      "Ifaces": sh["Ifaces"], "Jfaces": sh["Jfaces"], "Kfaces": sh["Kfaces"],
                      "nodes": sh["nodes"], "x_qp_left": sh["x_qp"], "x_qp_right": sh["x_qp"],
                      "y_qp_left": sh["y_qp"], "y_qp_right": sh["y_qp"], "z_qp_left": sh["z_qp"],
                      "z_qp_right": sh["z_qp"], "F": sh["F"], "G": sh["G"], "H": sh["H"],
                      "residue": sh["residue"], "gradqp_x": sh["grad"], "gradqp_y": sh["grad"],
                      "gradqp_z": sh["grad"], "mu": sh["pad"], "mu_t": sh["pad"],
                      "sst_F1": sh["pad"], "dist": sh["pad"], "delta_t": sh["delta_t"]}

    def close(self):
        if self.h:
            self.lib.fest_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        return abi.check(getattr(self.lib, name)(self.h, *args), name)

    def _input(self, a, name, copy=True):
        """a as a Fortran-ordered float64 array for an argument in the
        layout of array `name`; ValueError if it holds fewer values than the
        C call reads (which would read past the end of it)."""
        a = np.array(a, order="F", dtype=np.float64) if copy else np.asfortranarray(a, dtype=np.float64)
        need = int(np.prod(self.shape[name]))
        if a.size < need:
            raise ValueError(f"{name} argument of shape {a.shape}: {a.size} values, the call reads {need}")
        return a

    def get(self, name):
        a = np.empty(self.shape[name], order="F")
        self._call("fest_get_array", ARR[name], abi.ptr(a))
        return a

    def set(self, name, a):
        a = self._input(a, name, copy=False)
        self._call("fest_set_array", ARR[name], abi.ptr(a))

    @property
    def launches(self):
        return self.lib.fest_kernel_launches(self.h)

    def set_precision(self, p):
        self._call("fest_set_precision", int(p))

    def setup_geometry(self, nodes):
        nodes = self._input(nodes, "nodes")
        self._call("fest_setup_geometry", abi.ptr(nodes), None, None, None, None)
        return nodes

    def set_metrics(self, cells, If, Jf, Kf):
        args = [self._input(a, n, copy=False) for a, n in
                ((cells, "cells"), (If, "Ifaces"), (Jf, "Jfaces"), (Kf, "Kfaces"))]
        self._call("fest_set_metrics", *[abi.ptr(a) for a in args])

    def find_wall_dist(self, wall_xyz):
        w = np.ascontiguousarray(wall_xyz, dtype=np.float64)
        d = np.empty(self.shape["dist"], order="F")
        self._call("fest_find_wall_dist", w.ctypes.data_as(C.POINTER(C.c_double)), len(w),
                   abi.ptr(d))
        return d

    def upload_state(self, qp):
        self._call("fest_upload_state", abi.ptr(self._input(qp, "qp", copy=False)))

    def download_state(self):
        q = np.empty(self.shape["qp"], order="F")
        self._call("fest_download_state", abi.ptr(q))
        return q

    def snapshot_begin(self, q):
        """Start copying the current state into q (padded shape, F-ordered
        float64; pinned memory lets later steps overlap the copy) and return
        at once (fest_snapshot_begin); q is complete when snapshot_wait
        returns."""
        if not (isinstance(q, np.ndarray) and q.dtype == np.float64 and q.flags.f_contiguous
                and q.shape == tuple(self.shape["qp"])):
            raise ValueError(f"q must be an F-ordered float64 array of shape {self.shape['qp']}")
        self._call("fest_snapshot_begin", abi.ptr(q))
        self._snap = q

    def snapshot_wait(self):
        """Wait for the snapshot begun last; FestError if the state it holds
        comes from a failed step."""
        try:
            self._call("fest_snapshot_wait")
        finally:
            self._snap = None

    def step_async(self, n, first_iter, CFL):
        """Enqueue n iterations and return; errors surface at the next
        synchronous call (last_device_error)."""
        self._call("fest_step_async", int(n), int(first_iter), float(CFL))

    def last_device_error(self):
        self._call("fest_last_device_error")

    def iterate(self, max_iters, CFL, checkpoint_iter, on_checkpoint, first_iter=1, q=None):
        """Iterations first_iter..max_iters with the reference's checkpoint
        schedule (dump_solution.f90:40-43: with checkpoint_iter != 0, every
        checkpoint_iter-th iteration and the last one; none with 0):
        on_checkpoint(iteration, qp) gets each of those states on the host
        while the device steps on toward the next one.  q: the host buffer
        the snapshots land in (pinned memory for the overlap; a new pageable
        array if None).  on_checkpoint must be done with qp when it returns:
        the next snapshot reuses it.  Returns the next iteration number."""
        if checkpoint_iter < 0 or first_iter < 1:
            raise ValueError("checkpoint_iter >= 0 and first_iter >= 1")
        if q is None:
            q = np.zeros(self.shape["qp"], order="F")
        if checkpoint_iter == 0:
            if max_iters >= first_iter:
                self.step_async(max_iters - first_iter + 1, first_iter, CFL)
            self.last_device_error()
            return max(first_iter, max_iters + 1)
        dumps = [it for it in range(first_iter, max_iters + 1)
                 if it % checkpoint_iter == 0 or it == max_iters]
        it, pending = first_iter, None
        for d in dumps + [None]:
            if d is not None:
                self.step_async(d - it + 1, it, CFL)
                it = d + 1
            if pending is not None:
                self.snapshot_wait()
                on_checkpoint(pending, q)
            if d is not None:
                self.snapshot_begin(q)
                pending = d
        self.last_device_error()
        return it

    def populate_ghost_primitive(self, qp, it):
        q = self._input(qp, "qp")
        self._call("fest_populate_ghost_primitive", abi.ptr(q), int(it))
        return q

    def compute_temperature(self, qp=None):
        T = np.empty(self.shape["Temp"], order="F")
        self._call("fest_compute_temperature", abi.ptr(qp), abi.ptr(T))
        return T

    def get_next_solution(self, qp, it, CFL):
        q = self._input(qp, "qp")
        self._call("fest_get_next_solution", abi.ptr(q), int(it), float(CFL), None, None)
        return q

    def residual(self, qp, it):
        q = self._input(qp, "qp")
        r = np.empty(self.shape["residue"], order="F")
        self._call("fest_get_total_conservative_residue", abi.ptr(q), int(it), abi.ptr(r))
        return q, r

    def step(self, n, first_iter, CFL, with_norm=True):
        out = np.zeros(8) if with_norm else None
        self._call("fest_step", int(n), int(first_iter), float(CFL),
                   out.ctypes.data_as(C.POINTER(C.c_double)) if with_norm else None)
        return out[:self.ext.n_var + 1] if with_norm else None

    def step_host(self, qp, n, first_iter, CFL, with_norm=True):
        """n iterations on the host state qp (padded, F-ordered float64),
        updated in place; one synchronisation (fest_step_host)."""
        if not (isinstance(qp, np.ndarray) and qp.dtype == np.float64 and qp.flags.f_contiguous
                and qp.shape == self.shape["qp"]):
            raise ValueError(f"qp must be an F-ordered float64 array of shape {self.shape['qp']}")
        out = np.zeros(8) if with_norm else None
        self._call("fest_step_host", abi.ptr(qp), int(n), int(first_iter), float(CFL),
                   out.ctypes.data_as(C.POINTER(C.c_double)) if with_norm else None)
        return out[:self.ext.n_var + 1] if with_norm else None

    def step_host_interior(self, q, n, first_iter, CFL, with_norm=True):
        """n iterations on the interior-cell state q ((imx-1, jmx-1, kmx-1,
        n_var), F-ordered float64), updated in place; ghost cells stay on
        the device (fest_step_host_interior)."""
        e = self.ext
        shape = (e.imx - 1, e.jmx - 1, e.kmx - 1, e.n_var)
        if not (isinstance(q, np.ndarray) and q.dtype == np.float64 and q.flags.f_contiguous
                and q.shape == shape):
            raise ValueError(f"q must be an F-ordered float64 array of shape {shape}")
        out = np.zeros(8) if with_norm else None
        self._call("fest_step_host_interior", abi.ptr(q), int(n), int(first_iter), float(CFL),
                   out.ctypes.data_as(C.POINTER(C.c_double)) if with_norm else None)
        return out[:self.ext.n_var + 1] if with_norm else None

    def residual_vjp(self, qp, it, lam):
        """(dR/dq)^T lam for the residual of iteration it at state qp."""
        q = None if qp is None else self._input(qp, "qp")
        lam = self._input(lam, "residue", copy=False)
        dq = np.empty(self.shape["qp"], order="F")
        self._call("fest_residual_vjp", abi.ptr(q), int(it), abi.ptr(lam), abi.ptr(dq))
        return dq

    def residual_vjp_nodes(self, qp, it, lam=None, faces_bar=(None, None, None)):
        """(dR/dnodes)^T lam + (dfaces/dnodes)^T faces_bar (nodes layout)."""
        q = None if qp is None else self._input(qp, "qp")
        lam = None if lam is None else self._input(lam, "residue", copy=False)
        fb = [None if f is None else self._input(f, n, copy=False)
              for f, n in zip(faces_bar, ("Ifaces", "Jfaces", "Kfaces"))]
        dn = np.empty(self.shape["nodes"], order="F")
        self._call("fest_residual_vjp_nodes", abi.ptr(q), int(it), abi.ptr(lam), abi.ptr(fb[0]),
                   abi.ptr(fb[1]), abi.ptr(fb[2]), None, abi.ptr(dn))
        return dn

    def adjoint_solve(self, dJdq, CFL, max_iters, tol):
        """psi with (dR/dq)^T psi = -dJ/dq at the device state; returns
        (psi, iterations, drop)."""
        dj = self._input(dJdq, "qp", copy=False)
        psi = np.empty(self.shape["residue"], order="F")
        n = C.c_int()
        drop = C.c_double()
        self._call("fest_adjoint_solve", abi.ptr(dj), float(CFL), int(max_iters), float(tol),
                   abi.ptr(psi), C.byref(n), C.byref(drop))
        return psi, n.value, drop.value

    def resnorm(self):
        out = np.zeros(8)
        self._call("fest_find_resnorm", out.ctypes.data_as(C.POINTER(C.c_double)))
        return out[:self.ext.n_var + 1]
