"""Host logic of the checkpointed unsteady adjoint (fest3d/adjoint.py) on
the CPU: the transposed Jacobians of the conservative/primitive maps, and
the reverse sweep over checkpointed segments, with a stand-in for the
device handle whose residual has a known exact VJP.  The device residual
and its VJP are covered by the GPU adjoint tests; here the stand-in lets the
segment bookkeeping (a partial last segment included) and the TVD-RK3 stage
transposes be checked against central finite differences without a GPU.
No GPU."""
import numpy as np

import oracle as O
from fest3d import adjoint as A


def _fd_vjp(fn, q, v, h=1e-7):
    """v^T (d fn / d q) by central differences, per cell (last axis = 5)."""
    out = np.zeros_like(q)
    for m in range(q.shape[-1]):
        dq = np.zeros_like(q)
        step = h * np.maximum(np.abs(q[..., m]), 1.0)
        dq[..., m] = step
        jp, jm = fn(q + dq), fn(q - dq)
        out[..., m] = np.sum((jp - jm) * v, axis=-1) / (2 * step)
    return out


def _state(rng, n=7):
    q = np.empty((n, 5))
    q[:, 0] = rng.uniform(0.8, 1.5, n)
    q[:, 1:4] = rng.uniform(-200.0, 200.0, (n, 3))
    q[:, 4] = rng.uniform(5e4, 2e5, n)
    return q


def _cons(q, gm=A.GM):
    r, u, v, w, p = (q[..., l] for l in range(5))
    return np.stack([r, r * u, r * v, r * w, p / (gm - 1.0) + 0.5 * r * (u * u + v * v + w * w)], axis=-1)


def _prim(U, gm=A.GM):
    r = U[..., 0]
    u, v, w = U[..., 1] / r, U[..., 2] / r, U[..., 3] / r
    return np.stack([r, u, v, w, (gm - 1.0) * (U[..., 4] - 0.5 * r * (u * u + v * v + w * w))], axis=-1)


def test_transposed_jacobians_of_the_state_maps():
    rng = np.random.default_rng(5)
    q = _state(rng)
    v = rng.standard_normal(q.shape)
    got = A._cons_T(q, v)
    want = _fd_vjp(_cons, q, v)
    assert np.allclose(got, want, rtol=1e-6, atol=1e-9 * np.abs(want).max())
    U = _cons(q)
    got = A._prim_T(q, v)  # P'(U)^T v at q = P(U)
    want = _fd_vjp(_prim, U, v)
    assert np.allclose(got, want, rtol=1e-6, atol=1e-9 * np.abs(want).max())


class _StandIn:
    """The calls the unsteady adjoint makes on a handle, for a per-cell
    residual R = V s (K d/s + b (d_p/s_p)^2), d = q - q_ref, with its exact
    VJP; the primal step is the TVD-RK3 step of the stage map."""

    def __init__(self, case, q_ref, K, b):
        ext = case["ext"]
        blk = O.Block(ext, case["flow"], case["scheme"], case["bc"])
        blk["nodes"] = case["nodes"]
        blk.setup_geometry()
        self.arrays = {"cells": np.array(blk["cells"], order="F"), "Jfaces": np.array(blk["Jfaces"], order="F")}
        self.ext, self.sl = ext, A._interior(ext)
        self.vol = self.arrays["cells"][0][self.sl]
        self.dtv = case["dt"] / self.vol
        self.q_ref = q_ref[self.sl]
        self.s = np.array([1.2, 170.0, 170.0, 170.0, 1e5])
        self.K, self.b = K, b
        self.vjp_calls = 0

    def get(self, name):
        return self.arrays[name]

    def close(self):
        pass

    def residual(self, qp, it):
        q = np.array(qp, order="F")
        d = (q[self.sl] - self.q_ref) / self.s
        R = (d @ self.K.T + self.b * (d[..., 4:5] ** 2)) * self.s * self.vol[..., None]
        return q, np.asfortranarray(R)

    def residual_vjp(self, qp, it, lam):
        d = (qp[self.sl] - self.q_ref) / self.s
        w = lam * self.s * self.vol[..., None]
        g = (w @ self.K) / self.s
        g[..., 4] += 2.0 * d[..., 4] * np.sum(w * self.b, axis=-1) / self.s[4]
        out = np.zeros_like(qp)
        out[self.sl] = g
        self.vjp_calls += 1
        return out

    def get_next_solution(self, qp, it, CFL):
        _, _, q = A._stages(self, qp, it, self.dtv, self.ext)
        return q


def test_checkpointed_reverse_sweep_matches_finite_differences(monkeypatch):
    case = A.unsteady_case(nc=(12, 6, 2), steps=12)
    rng = np.random.default_rng(11)
    q_ref = case["qp"].copy(order="F")
    q_ref[..., 0] *= 1.01
    q_ref[..., 4] *= 0.99
    K = 2000.0 * (np.eye(5) + 0.3 * rng.standard_normal((5, 5)))
    b = 500.0 * rng.standard_normal(5)
    stand_in = _StandIn(case, q_ref, K, b)
    monkeypatch.setattr(A, "make_handle", lambda case, lib=None, **kw: stand_in)

    J, dJ, calls = A.unsteady_sensitivity(case, eps=0.0, every=5)  # segments 10 (two steps), 5, 0
    assert calls == 3 * case["steps"]
    assert stand_in.vjp_calls == 3 * case["steps"]

    def objective(eps):
        q, _ = A.run_primal(stand_in, case["qp"] + eps * case["dq0"], case["steps"])
        return A.wall_force(q, case["ext"], stand_in.get("Jfaces"))[0]

    assert objective(0.0) == J
    h = 1e-3
    fd = (objective(h) - objective(-h)) / (2 * h)
    assert abs(fd) > 0
    assert abs(dJ - fd) <= 1e-6 * abs(fd), (dJ, fd)

    # the checkpoint spacing must not change the result
    _, dJ1, _ = A.unsteady_sensitivity(case, eps=0.0, every=1)
    _, dJ12, _ = A.unsteady_sensitivity(case, eps=0.0, every=12)
    assert abs(dJ1 - dJ) <= 1e-12 * abs(dJ) and abs(dJ12 - dJ) <= 1e-12 * abs(dJ)
