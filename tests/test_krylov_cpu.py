"""Convergence acceleration (fest3d.krylov) and its use on the solver's
fixed-point iterations (fest3d.adjoint.converge_accelerated,
adjoint_krylov), on the CPU: GMRES and Anderson acceleration on model
problems, the accelerated flow solve on a small bump driven by the oracle's
own iterations, and the GMRES adjoint on a dense model of the linearised
residual with a stationary pseudo-time iteration as preconditioner."""
import numpy as np

import oracle as O
from fest3d import adjoint as A
from fest3d import krylov as K


def test_gmres_solves_a_nonsymmetric_system():
    rng = np.random.default_rng(1)
    n = 300
    M = np.eye(n) * 3 + rng.standard_normal((n, n)) * 0.3 / np.sqrt(n)
    b = rng.standard_normal(n)
    x, products, hist = K.gmres(lambda v: M @ v, b, tol=1e-12, restart=30)
    assert np.linalg.norm(M @ x - b) <= 1e-12 * np.linalg.norm(b) * 10
    assert products < 40
    # restarts: a tiny restart length still gets there
    x2, p2, _ = K.gmres(lambda v: M @ v, b, tol=1e-10, restart=3, maxiter=500)
    assert np.linalg.norm(M @ x2 - b) <= 1e-10 * np.linalg.norm(b) * 10


def test_anderson_removes_the_slow_modes_of_a_contraction():
    """x <- Gx + c with five eigenvalues within 2e-3 of 1: plain iteration
    needs ~10^5 maps for 1e-10, Anderson (m=10) under 100."""
    rng = np.random.default_rng(2)
    n = 300
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = np.full(n, 0.5)
    ev[:5] = [0.9999, 0.9998, 0.9995, 0.999, 0.998]
    G = Q @ np.diag(ev) @ Q.T
    c = rng.standard_normal(n)
    xs = np.linalg.solve(np.eye(n) - G, c)

    def phi(x):
        y = G @ x + c
        return y, np.linalg.norm(y - x)

    x, info, maps = K.anderson(phi, np.zeros(n), m=10, maxiter=200, done=lambda r, k: r < 1e-12)
    assert maps < 100
    assert np.linalg.norm(x - xs) <= 1e-9 * np.linalg.norm(xs)


class OracleStepper:
    """The oracle behind the few handle calls converge_accelerated makes."""

    def __init__(self, case):
        self.ext, self.flow = case["ext"], case["flow"]
        self.blk = O.Block(case["ext"], case["flow"], case["scheme"], case["bc"])
        self.blk["nodes"] = case["nodes"]
        self.blk.setup_geometry()
        self.blk["qp"] = case["qp"]
        self.iterations = 0

    def upload_state(self, q):
        self.blk["qp"] = q

    def download_state(self):
        return np.array(self.blk["qp"], order="F")

    def step(self, n, first, CFL):
        for it in range(first, first + n):
            assert O.get_next_solution([self.blk], it, CFL) == 0
        self.iterations += n
        return O.find_resnorm([self.blk])


def test_accelerated_flow_solve_on_the_bump_channel():
    """The second-order bump channel (unlimited MUSCL + SLAU, TVD-RK3, total
    pressure inlet, pressure outlet) at 24x8x2 cells: plain iteration drops
    the mass residual by ~20 in 2000 iterations; Anderson acceleration
    (m = 20) of 50-iteration maps reaches a 1e-10 drop within 5000
    iterations, and the state it returns is a fixed point of the solver."""
    case = A.adjoint_case(nc=(24, 8, 2))
    plain = OracleStepper(case)
    r0 = plain.step(1, 1, case["CFL"])[1]
    r = plain.step(2000, 2, case["CFL"])[1]
    assert r / r0 > 1e-3  # slow
    acc = OracleStepper(case)
    ref = acc.step(1, 1, case["CFL"])[1]
    q, it, drop, ref2, maps, iters = A.converge_accelerated(acc, acc.download_state(), case["CFL"], first_iter=2,
                                                            tol=1e-10, ref=ref, k=50, m=20, max_maps=200)
    assert drop <= 1e-10, (drop, maps)
    assert iters <= 5000
    acc.upload_state(q)
    r1 = acc.step(1, it, case["CFL"])[1]
    assert r1 / ref <= 1e-9


class DenseAdjointModel:
    """A handle stand-in for adjoint_krylov: the interior-cell Jacobian A of
    a model residual (dense, n = cells x 5), residual_vjp = A^T lam, and
    adjoint_solve = k steps from zero of psi <- psi - D (A^T psi + dJ), a
    stationary iteration with slow modes."""

    def __init__(self, ext, seed=3):
        self.ext = ext
        sh = (ext.imx + 5, ext.jmx + 5, ext.kmx + 5, 5)
        self.shape = {"qp": sh, "residue": (ext.imx - 1, ext.jmx - 1, ext.kmx - 1, 5)}
        self.sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
        n = int(np.prod(self.shape["residue"]))
        rng = np.random.default_rng(seed)
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        ev = np.concatenate([[1e-4, 3e-4, 1e-3], rng.uniform(0.2, 1.5, n - 3)])
        self.A = (Q * ev) @ Q.T + 0.05 * rng.standard_normal((n, n)) / np.sqrt(n)
        self.D = 0.6
        self.n = n

    def _vec(self, a):
        return np.asarray(a).reshape(-1, order="F")

    def residual_vjp(self, q, it, lam):
        out = np.zeros(self.shape["qp"], order="F")
        out[self.sl] = (self.A.T @ self._vec(lam)).reshape(self.shape["residue"], order="F")
        return out

    def adjoint_solve(self, dJ, CFL, k, tol):
        g = self._vec(dJ[self.sl])
        psi = np.zeros(self.n)
        for _ in range(k):
            psi = psi - self.D * (self.A.T @ psi + g)
        return psi.reshape(self.shape["residue"], order="F"), k, 1.0


def test_gmres_adjoint_on_a_stationary_iteration():
    from fest3d import abi
    ext = abi.Extent(7, 5, 4, 5)  # 6x4x3 cells
    h = DenseAdjointModel(ext)
    dJ = np.zeros(h.shape["qp"], order="F")
    dJ[h.sl] = np.random.default_rng(4).standard_normal(h.shape["residue"])
    psi, products, drop, calls = A.adjoint_krylov(h, dJ, 1.0, tol=1e-10, k=5, restart=30, max_products=600)
    g = h._vec(dJ[h.sl])
    assert drop <= 1e-10
    assert np.linalg.norm(h.A.T @ h._vec(psi) + g) <= 1e-10 * np.linalg.norm(g) * 1.01
    # the stationary iteration alone: slow modes with rates 1 - 0.6e-4
    assert products < 300
