"""Post-processing of block states, as the reference's test scripts do it.

Host-side numpy on Fortran-shaped arrays (qp(-2:imx+2,-2:jmx+2,-2:kmx+2,n_var)
as returned by ``Handle.download_state``), used by the bench and the tests to
report the quantities the reference's own cases report.
"""
import numpy as np


def interior(a, ext):
    """Interior cells (1:imx-1, 1:jmx-1, 1:kmx-1) of a padded cell array."""
    return a[3:ext.imx + 2, 3:ext.jmx + 2, 3:ext.kmx + 2]


def entropy_change(q, vol, p_inf, rho_inf, gm=1.4):
    """Relative entropy change of SmoothBump/pp/entropy.py:23-28:
    sqrt(sum(((s - s_inf) V / s_inf)^2) / sum V) with s = p / rho^gamma,
    over the cells of q (interior cells, last axis the variables) and their
    volumes vol."""
    s_inf = p_inf / rho_inf ** gm
    s = q[..., 4] / q[..., 0] ** gm
    err2 = np.sum(((s - s_inf) * vol / s_inf) ** 2)
    return float(np.sqrt(err2 / np.sum(vol)))


def entropy_field(q, p_inf, rho_inf, gm=1.4):
    """(s - s_inf) / s_inf per cell, the field entropy.py sums."""
    s_inf = p_inf / rho_inf ** gm
    return q[..., 4] / q[..., 0] ** gm / s_inf - 1.0


def wall_cp(q, ext, flow, j=1, k=1):
    """Pressure coefficient (p - p_inf) / (rho_inf V_inf^2 / 2) on the first
    cell row above the jmin wall (cell row j, plane k), all i, as
    Lfp/pp/Surface.py:95,132 takes the wall pressure from the first cells."""
    p = q[3:ext.imx + 2, j + 2, k + 2, 4]
    qinf = 0.5 * flow.density_inf * flow.vel_mag ** 2
    return (p - flow.pressure_inf) / qinf
