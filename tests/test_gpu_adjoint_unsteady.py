"""Checkpointed discrete adjoint of a time-accurate run: 500 TVD-RK3 steps
with a fixed global time step (1e-5 s) on the 128x48x4 bump from a
perturbed start (uniform inflow + eps * pressure pulse), states kept every
50 steps and recomputed per segment.  dJ/deps of the final wall force
against a central difference of two full primal runs (eps = +-1e-2, i.e.
+-10 Pa), to 1e-4."""
import numpy as np
import pytest

from fest3d import adjoint as A

pytestmark = pytest.mark.gpu


def test_unsteady_checkpointed_adjoint(gpu_lib):
    case = A.unsteady_case(nc=(128, 48, 4), dt=1e-5, steps=500)
    J, g, calls = A.unsteady_sensitivity(case, eps=0.0, every=50, lib=gpu_lib)
    assert calls == 3 * case["steps"]
    vals = []
    for e in (1e-2, -1e-2):
        h = A.make_handle(case, lib=gpu_lib)
        qN, _ = A.run_primal(h, case["qp"] + e * case["dq0"], case["steps"])
        vals.append(A.wall_force(qN, case["ext"], h.get("Jfaces"))[0])
        h.close()
    fd = (vals[0] - vals[1]) / 2e-2
    assert np.isfinite(J) and abs(fd) > 0
    assert abs(fd - g) <= 1e-4 * abs(fd), (fd, g, J)
