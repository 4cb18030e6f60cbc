"""The reference's case files on the host: grid files, Tecplot and legacy
VTK block output, restart logs and residual-norm lines, in the formats
FEST-3D's own readers and writers use, so that a run of this library starts
from, and leaves behind, files the reference's driver and post-processing
read.

Arrays are in the C ABI's layouts (fest_gpu.h): the state ``qp`` is
Fortran-ordered ``(imx+5, jmx+5, kmx+5, n_var)`` with Fortran index -2 at
0, so interior cell ``i = 1..imx-1`` is ``qp[i + 2]``; ``nodes`` is
``(3, imx+6, jmx+6, kmx+6)`` with node ``i = 1..imx`` at ``nodes[:, i + 2]``.

Number formats follow the Fortran edit descriptors the reference writes
with (ES28.15E4, Ew.dE2, F0.16, I0): the decimal digits are the correctly
rounded digits of the binary value (round half to even, as the C library's
printf that gfortran formats through).  Grid files, Tecplot output and
restart logs are checked byte for byte against files the reference wrote;
the legacy VTK format, of which the reference ships no sample, against
known answers.
"""
import math
import os

import numpy as np

# Tecplot output variables (write_output_tec.f90:127-197): output-control
# name -> (header label(s), state variable index(es), 0-based).  Names
# outside the state (Mu, Mu_t, F1, Wall_distance, gradients) are written
# from arrays passed in `extra`.
_STATE_VARS = {
    "Velocity": ((" u v w ",), (1, 2, 3)),
    "Density": (("Density ",), (0,)),
    "Pressure": (("Pressure ",), (4,)),
    "TKE": (("TKE ",), (5,)),
    "Omega": (("Omega ",), (6,)),
}
_TURB_WITH_K_OMEGA = ("sst", "sst2003", "bsl", "des-sst", "kw")


# ---- Fortran number formats -------------------------------------------------
def _nonfinite(x):
    if math.isnan(x):
        return "NaN"
    return "Infinity" if x > 0 else "-Infinity"


def fortran_es(x, w=28, d=15, e=4):
    """x under the edit descriptor ESw.dEe: one nonzero digit before the
    point, d after it, an exponent of e digits; right-justified in w."""
    x = float(x)
    if not math.isfinite(x):
        return _nonfinite(x).rjust(w)
    s = "%.*E" % (d, x)
    mant, ex = s.split("E")
    ex = int(ex)
    if len(str(abs(ex))) > e:
        return "*" * w
    out = "%sE%s%0*d" % (mant, "-" if ex < 0 else "+", e, abs(ex))
    return "*" * w if len(out) > w else out.rjust(w)


def fortran_e(x, w, d, e=2):
    """x under Ew.dEe: mantissa 0.ddd (d digits), exponent of e digits,
    right-justified in w (gfortran prints the optional leading zero when
    the width leaves room for it).  e=None is Ew.d: a two-digit exponent
    after 'E', or a sign and three digits without the 'E' beyond 99."""
    x = float(x)
    if not math.isfinite(x):
        return _nonfinite(x).rjust(w)
    if x == 0.0:
        digits, ex, neg = "0" * d, 0, math.copysign(1.0, x) < 0
    else:
        s = "%.*e" % (d - 1, abs(x))  # d significant digits, correctly rounded
        mant, ex = s.split("e")
        digits, ex, neg = mant.replace(".", ""), int(ex) + 1, x < 0
    sign = "-" if ex < 0 else "+"
    if e is None:
        if abs(ex) > 999:
            return "*" * w
        body = "0.%s%s%s%0*d" % (digits, "E" if abs(ex) <= 99 else "", sign, 2 if abs(ex) <= 99 else 3, abs(ex))
    elif len(str(abs(ex))) > e:
        return "*" * w
    else:
        body = "0.%sE%s%0*d" % (digits, sign, e, abs(ex))
    if neg:
        body = "-" + body
    if len(body) > w:
        body = body.replace("0.", ".", 1)  # drop the optional zero first
    return "*" * w if len(body) > w else body.rjust(w)


def fortran_f0(x, d=16):
    """x under F0.d: the minimal width, d digits after the point, no
    leading zero before the point (gfortran: 0 -> '.0000000000000000')."""
    x = float(x)
    if not math.isfinite(x):
        return _nonfinite(x)
    s = "%.*f" % (d, x)
    if s.startswith("0."):
        s = s[1:]
    elif s.startswith("-0."):
        s = "-" + s[2:]
    return s


# ---- grid files (grid.f90:72-127) -------------------------------------------
def read_grid(path):
    """A FEST-3D grid file: a header line 'imx jmx kmx', then one node
    'x y z' per line with i fastest, then j, then k (grid.f90:86-127).
    Returns the nodes as an array of shape (imx, jmx, kmx, 3)."""
    with open(path) as f:
        header = f.readline().split()
        if len(header) < 3:
            raise ValueError(f"{path}: grid header needs imx jmx kmx, got {header!r}")
        imx, jmx, kmx = (int(v) for v in header[:3])
        xyz = np.loadtxt(f, ndmin=2)
    if xyz.shape != (imx * jmx * kmx, 3):
        raise ValueError(f"{path}: {xyz.shape[0]} nodes for a {imx}x{jmx}x{kmx} grid")
    return np.ascontiguousarray(xyz.reshape(kmx, jmx, imx, 3).transpose(2, 1, 0, 3))


def write_grid(path, nodes_ijk):
    """Write nodes of shape (imx, jmx, kmx, 3) as a FEST-3D grid file, in
    the layout of the reference's test-case grids ('%.18e' columns
    separated by tabs)."""
    nodes_ijk = np.asarray(nodes_ijk, dtype=np.float64)
    imx, jmx, kmx = nodes_ijk.shape[:3]
    xyz = nodes_ijk.transpose(2, 1, 0, 3).reshape(-1, 3)
    with open(path, "w") as f:
        f.write(f"{imx} {jmx} {kmx}\n")
        np.savetxt(f, xyz, fmt="%.18e", delimiter="\t")


def nodes_from_grid(nodes_ijk):
    """(imx, jmx, kmx, 3) nodes -> the ABI's (3, imx+6, jmx+6, kmx+6)
    array (ghost nodes zero; fest_setup_geometry makes them)."""
    imx, jmx, kmx = nodes_ijk.shape[:3]
    out = np.zeros((3, imx + 6, jmx + 6, kmx + 6), order="F")
    for c in range(3):
        out[c, 3:3 + imx, 3:3 + jmx, 3:3 + kmx] = nodes_ijk[..., c]
    return out


# ---- Tecplot block output (write_output_tec.f90, read_output_tec.f90) ------
def _tec_labels(variables):
    labels = []
    for v in variables:
        if v == "do not write":
            continue
        labels.extend(_STATE_VARS[v][0] if v in _STATE_VARS else (v + " ",))
    return labels


def tecplot_text(qp, nodes, variables=("Velocity", "Density", "Pressure"), block=0,
                 solution_time=0, turbulence="none", extra=None):
    """The text write_file (write_output_tec.f90:58-200) writes for one
    block: the header (write_header, :202-232), the interior nodes x, y, z
    (write_grid, :235-249), then each listed variable over the interior
    cells (write_scalar, :252-268), one ES28.15E4 value per line, i
    fastest.  `variables` is the output-control list (Velocity, Density,
    Pressure, TKE, Omega, or any name found in `extra`, a dict of arrays
    over the padded cells -2..imx+2 or, for gradients, 0..imx)."""
    qp = np.asarray(qp)
    if qp.ndim != 4 or nodes.shape[0] != 3:
        raise ValueError("qp must be (imx+5, jmx+5, kmx+5, n_var) and nodes (3, imx+6, jmx+6, kmx+6)")
    imx, jmx, kmx = qp.shape[0] - 5, qp.shape[1] - 5, qp.shape[2] - 5
    if nodes.shape[1:] != (imx + 6, jmx + 6, kmx + 6):
        raise ValueError(f"nodes {nodes.shape} do not match a {imx}x{jmx}x{kmx} block")
    extra = extra or {}
    k_omega = turbulence in _TURB_WITH_K_OMEGA
    labels = _tec_labels(variables)
    total = 3 + sum(len(lb.split()) for lb in labels)
    out = ["variables = x y z "]
    out += [lb for lb in labels]
    out.append("zone T=block%04d  i=%05d j=%05d k=%05d Datapacking=Block" % (block, imx, jmx, kmx))
    out.append(" Varlocation=([1-3]=Nodal)")
    out.append("Varlocation=([4-%02d]=CELLCENTERED)" % total)
    out.append("STRANDID=%04d" % 1)
    out.append("SOLUTIONTIME=%04d" % solution_time)

    def column(a):  # Fortran order over the block, one value per record
        return [fortran_es(v) for v in np.asarray(a).ravel(order="F")]

    for c in range(3):
        out += column(nodes[c, 3:3 + imx, 3:3 + jmx, 3:3 + kmx])
    cells = (slice(3, imx + 2), slice(3, jmx + 2), slice(3, kmx + 2))
    for v in variables:
        if v == "do not write":
            continue
        if v in _STATE_VARS:
            if v in ("TKE", "Omega") and not k_omega:
                raise ValueError(f"{v} needs a k-omega turbulence model, not {turbulence!r}")
            for l in _STATE_VARS[v][1]:
                out += column(qp[cells + (l,)])
        elif v in extra:
            a = np.asarray(extra[v])
            off = 3 if a.shape[0] == imx + 5 else 1  # padded (-2:) or gradient (0:) lower bound
            out += column(a[off:off + imx - 1, off:off + jmx - 1, off:off + kmx - 1])
        else:
            raise ValueError(f"no data for output variable {v!r}")
    return "\n".join(out) + "\n"


def tecplot_nodal_text(qp, nodes, variables=("Velocity", "Density", "Pressure"), block=0,
                       solution_time=0, turbulence="none", extra=None):
    """The text of the 'tecplot_nodal' output (write_output_tec_node.f90):
    every field at the nodes i = 1..imx, j = 1..jmx of the node planes
    k = 1..kmx-1, a node's value the mean 0.25*(v(i,j)+v(i-1,j)+v(i,j-1)+
    v(i-1,j-1)) of the four cells around it in its i-j plane (ghost cells
    included, summed in that order), written 35 values per record under
    E25.15.  Arguments as tecplot_text."""
    qp = np.asarray(qp)
    imx, jmx, kmx = qp.shape[0] - 5, qp.shape[1] - 5, qp.shape[2] - 5
    if nodes.shape != (3, imx + 6, jmx + 6, kmx + 6):
        raise ValueError(f"nodes {nodes.shape} do not match a {imx}x{jmx}x{kmx} block")
    extra = extra or {}
    k_omega = turbulence in _TURB_WITH_K_OMEGA
    labels = _tec_labels(variables)
    total = 3 + sum(len(lb.split()) for lb in labels)
    out = ["variables = x y z "] + labels
    out.append("zone T=block%04d  i=%05d j=%05d k=%05d Datapacking=Block" % (block, imx, jmx, kmx - 1))
    out.append(" Varlocation=([1-3]=Nodal)")
    out.append("Varlocation=([4-%02d]=Nodal)" % total)
    out.append("STRANDID=%04d" % 1)
    out.append("SOLUTIONTIME=%04d" % solution_time)

    def records(a):  # one write statement: 35 values per record
        v = [fortran_e(x, 25, 15, None) for x in np.asarray(a).ravel(order="F")]
        return ["".join(v[n:n + 35]) for n in range(0, len(v), 35)]

    def at_nodes(a, off):  # a over cells, Fortran index -off at 0
        i0, j0 = off + 1, off + 1  # cell 1 (the cell after node 1)
        k = slice(off + 1, off + kmx)  # k = 1..kmx-1
        return 0.25 * (a[i0:i0 + imx, j0:j0 + jmx, k] + a[i0 - 1:i0 - 1 + imx, j0:j0 + jmx, k]
                       + a[i0:i0 + imx, j0 - 1:j0 - 1 + jmx, k] + a[i0 - 1:i0 - 1 + imx, j0 - 1:j0 - 1 + jmx, k])

    for c in range(3):
        out += records(nodes[c, 3:3 + imx, 3:3 + jmx, 3:3 + kmx - 1])
    for v in variables:
        if v == "do not write":
            continue
        if v in _STATE_VARS:
            if v in ("TKE", "Omega") and not k_omega:
                raise ValueError(f"{v} needs a k-omega turbulence model, not {turbulence!r}")
            for l in _STATE_VARS[v][1]:
                out += records(at_nodes(qp[..., l], 2))
        elif v in extra:
            a = np.asarray(extra[v])
            out += records(at_nodes(a, 2 if a.shape[0] == imx + 5 else 0))
        else:
            raise ValueError(f"no data for output variable {v!r}")
    return "\n".join(out) + "\n"


def write_tecplot(path, qp, nodes, **kw):
    """tecplot_text(qp, nodes, **kw) written to `path`."""
    with open(path, "w") as f:
        f.write(tecplot_text(qp, nodes, **kw))


def read_tecplot(path, qp, variables=("Velocity", "Density", "Pressure"), turbulence="none"):
    """Fill the interior cells of qp (in place; also returned) from a
    Tecplot block file as read_file (read_output_tec.f90:48-140) does:
    skip the header (one line per listed variable, read_header :143-160)
    and the three node coordinates, then read each listed variable over
    the interior cells.  'do not read' skips one field; any other name the
    reference cannot read (Mu, gradients, ...) reads nothing, as in the
    reference, which only prints a message for it."""
    imx, jmx, kmx = qp.shape[0] - 5, qp.shape[1] - 5, qp.shape[2] - 5
    nc = (imx - 1) * (jmx - 1) * (kmx - 1)
    nn = imx * jmx * kmx
    with open(path) as f:
        lines = f.read().split("\n")
    n_head = 1 + len(variables) + 5
    vals = np.array(" ".join(lines[n_head:]).split(), dtype=np.float64)
    fields = {v: (_STATE_VARS[v][1] if v in _STATE_VARS else (None,) if v == "do not read" else ())
              for v in variables}
    need = 3 * nn + nc * sum(len(f) for f in fields.values())
    if vals.size < need:
        raise ValueError(f"{path}: {vals.size} values, a {imx}x{jmx}x{kmx} block with "
                         f"{list(variables)} needs {need}")
    pos = 3 * nn
    cells = (slice(3, imx + 2), slice(3, jmx + 2), slice(3, kmx + 2))
    shape = (imx - 1, jmx - 1, kmx - 1)
    for v in variables:
        if v in ("TKE", "Omega") and turbulence not in _TURB_WITH_K_OMEGA:
            raise ValueError(f"{v} needs a k-omega turbulence model, not {turbulence!r}")
        for l in fields[v]:
            field = vals[pos:pos + nc].reshape(shape, order="F")
            pos += nc
            if l is not None:
                qp[cells + (l,)] = field
    return qp


# ---- legacy VTK output (write_output_vtk.f90, read_output_vtk.f90) ---------
# scalar names in the file (write_output_vtk.f90:131-199); trailing blanks
# of the gradient names are trimmed by the writer
_VTK_SCALAR = {"Density": "Density", "Pressure": "Pressure", "Mu": "Mu", "Mu_t": "Mu_t",
               "TKE": "TKE", "Omega": "Omega", "Kl": "Kl", "tv": "tv", "tgm": "tgm",
               "Dissipation": "Dissipation", "Wall_distance": "dist", "F1": "F1"}
for _g in ("u", "v", "w", "T", "tk", "tw"):
    for _c in "xyz":
        _VTK_SCALAR["D%sd%s" % (_g, _c)] = "d%sd%s" % (_g, _c)


def vtk_text(qp, nodes, variables=("Velocity", "Density", "Pressure"), turbulence="none",
             extra=None, data_format="ASCII"):
    """The text write_file (write_output_vtk.f90:46-163) writes for one
    block: the header (write_header), the nodes as F0.16 triples
    (write_grid), the velocity as ES27.16E4 triples (write_velocity) and
    each scalar as one ES25.16E4 value per line (write_scalar), every
    section closed by an empty record.  Arguments as tecplot_text.  The
    reference ships no VTK output of its own, so this format is restated
    from the writer's edit descriptors and checked by known answers and
    round trips, not against reference bytes."""
    qp = np.asarray(qp)
    imx, jmx, kmx = qp.shape[0] - 5, qp.shape[1] - 5, qp.shape[2] - 5
    if nodes.shape != (3, imx + 6, jmx + 6, kmx + 6):
        raise ValueError(f"nodes {nodes.shape} do not match a {imx}x{jmx}x{kmx} block")
    extra = extra or {}
    nc = (imx - 1) * (jmx - 1) * (kmx - 1)
    out = ["# vtk DataFile Version 3.1", "cfd-iitm output", data_format, "DATASET STRUCTURED_GRID",
           "DIMENSIONS %d %d %d" % (imx, jmx, kmx), "POINTS %d DOUBLE" % (imx * jmx * kmx)]
    xyz = [nodes[c, 3:3 + imx, 3:3 + jmx, 3:3 + kmx].ravel(order="F") for c in range(3)]
    out += ["%s %s %s" % (fortran_f0(x), fortran_f0(y), fortran_f0(z)) for x, y, z in zip(*xyz)]
    out.append("")
    cells = (slice(3, imx + 2), slice(3, jmx + 2), slice(3, kmx + 2))
    k_omega = turbulence in _TURB_WITH_K_OMEGA
    for v in variables:
        if v == "do not write":
            continue
        if v == "Velocity":
            out += ["CELL_DATA %d" % nc, "VECTORS Velocity FLOAT"]
            uvw = [qp[cells + (l,)].ravel(order="F") for l in (1, 2, 3)]
            out += ["%s %s %s" % (fortran_es(u, 27, 16), fortran_es(vv, 27, 16), fortran_es(w, 27, 16))
                    for u, vv, w in zip(*uvw)]
        elif v in _VTK_SCALAR:
            if v in ("Density", "Pressure"):
                a = qp[cells + (0 if v == "Density" else 4,)]
            elif v in ("TKE", "Omega"):
                if not k_omega:
                    raise ValueError(f"{v} needs a k-omega turbulence model, not {turbulence!r}")
                a = qp[cells + (5 if v == "TKE" else 6,)]
            elif v in extra:
                e = np.asarray(extra[v])
                off = 3 if e.shape[0] == imx + 5 else 1
                a = e[off:off + imx - 1, off:off + jmx - 1, off:off + kmx - 1]
            else:
                raise ValueError(f"no data for output variable {v!r}")
            out += ["SCALARS %s FLOAT" % _VTK_SCALAR[v], "LOOKUP_TABLE default"]
            out += [fortran_es(x, 25, 16) for x in np.asarray(a).ravel(order="F")]
        else:
            continue  # the reference prints a message and writes nothing
        out.append("")
    return "\n".join(out) + "\n"


def write_vtk(path, qp, nodes, **kw):
    """vtk_text(qp, nodes, **kw) written to `path`."""
    with open(path, "w") as f:
        f.write(vtk_text(qp, nodes, **kw))


def read_vtk(path, qp, variables=("Velocity", "Density", "Pressure"), turbulence="none"):
    """Fill the interior cells of qp (in place; also returned) from a
    legacy VTK block file as read_file (read_output_vtk.f90:24-92) reads
    it, one record per line: header, grid, then each listed variable
    (Velocity as one vector field, Density, Pressure, TKE, Omega); 'do not
    read' skips a scalar field and other names read nothing."""
    imx, jmx, kmx = qp.shape[0] - 5, qp.shape[1] - 5, qp.shape[2] - 5
    nc, nn = (imx - 1) * (jmx - 1) * (kmx - 1), imx * jmx * kmx
    with open(path) as f:
        lines = f.read().split("\n")
    pos = 4 + 2 + nn + 1  # header, DIMENSIONS/POINTS, the points, the empty record
    cells = (slice(3, imx + 2), slice(3, jmx + 2), slice(3, kmx + 2))
    shape = (imx - 1, jmx - 1, kmx - 1)

    def block(n_cols):
        nonlocal pos
        rows = lines[pos + 2:pos + 2 + nc]
        if len(rows) < nc:
            raise ValueError(f"{path}: the file ends inside a field of {nc} cells")
        pos += 2 + nc + 1
        a = np.array(" ".join(rows).split(), dtype=np.float64)
        if a.size != nc * n_cols:
            raise ValueError(f"{path}: {a.size} values where {nc * n_cols} belong")
        return a.reshape(nc, n_cols)

    for v in variables:
        if v in ("TKE", "Omega") and turbulence not in _TURB_WITH_K_OMEGA:
            raise ValueError(f"{v} needs a k-omega turbulence model, not {turbulence!r}")
        if v == "Velocity":
            a = block(3)
            for c, l in enumerate((1, 2, 3)):
                qp[cells + (l,)] = a[:, c].reshape(shape, order="F")
        elif v in ("Density", "Pressure", "TKE", "Omega"):
            l = {"Density": 0, "Pressure": 4, "TKE": 5, "Omega": 6}[v]
            qp[cells + (l,)] = block(1)[:, 0].reshape(shape, order="F")
        elif v == "do not read":
            pos += 2 + nc + 1
    return qp


# ---- restart log (dump_solution.f90:120-153, read_output.f90:103-117) -------
def write_restart_log(path, turbulence, iteration, previous_res):
    """The restart log write_restart_log writes: the flow type ('viscous'
    for no turbulence model, else the model's name), the iteration count
    (I0), then the reference residual norms, one F0.16 value per line."""
    kind = "viscous" if turbulence == "none" else turbulence
    with open(path, "w") as f:
        f.write(kind + "\n")
        f.write("%d\n" % int(iteration))
        for r in previous_res:
            f.write(fortran_f0(r) + "\n")


def read_restart_log(path):
    """(flow type, last iteration, reference residual norms) from a
    restart log, as read_restart_file reads it."""
    with open(path) as f:
        rows = [ln.strip() for ln in f if ln.strip()]
    if len(rows) < 2:
        raise ValueError(f"{path}: a restart log holds the flow type and the iteration count")
    return rows[0], int(rows[1]), np.array([float(r) for r in rows[2:]])


# ---- residual-norm file (resnorm.f90:94-114, 241-377) -----------------------
def resnorm_header(res_list):
    """The first line setup_file writes: 'Iteration' and each listed norm,
    each followed by two spaces."""
    return "".join(name + "  " for name in ("Iteration",) + tuple(res_list)) + "\n"


def resnorm_line(iteration, res_abs, res_rel, res_list, turbulence="none", precision=6):
    """One line of the residual-norm file (write_resnorm): the iteration
    (I0, 4x), then each listed norm as E(p+8).pE2 followed by four spaces.
    res_abs and res_rel hold n_var+1 values, index 0 the boundary mass
    imbalance and 1..n_var the per-variable norms (fest_find_resnorm's
    output for res_abs; res_abs / the saved reference norms for res_rel).
    Norms of a turbulence model the run does not have are left out, as the
    reference does."""
    ra = np.asarray(res_abs, dtype=np.float64)
    rr = np.asarray(res_rel, dtype=np.float64)
    w = precision + 8

    def nrm(a, lo, hi=None):
        return math.sqrt(float(np.sum(a[lo:hi] ** 2)))

    k_any = ("sst", "kkl", "sst2003")
    table = {
        "Mass_abs": lambda: ra[0], "Resnorm_abs": lambda: nrm(ra, 1),
        "Viscous_abs": lambda: nrm(ra, 1, 6),
        "Turbulent_abs": lambda: nrm(ra, 6) if turbulence != "none" else None,
        "Continuity_abs": lambda: ra[1], "X_mom_abs": lambda: ra[2], "Y_mom_abs": lambda: ra[3],
        "Z_mom_abs": lambda: ra[4], "Energy_abs": lambda: ra[5],
        "Mass_rel": lambda: rr[0], "Resnorm_rel": lambda: nrm(rr, 1),
        "Viscous_rel": lambda: nrm(rr, 1, 6),
        "Turbulent_rel": lambda: nrm(rr, 6) if turbulence != "none" else None,
        "Continuity_rel": lambda: rr[1], "X-mom_rel": lambda: rr[2], "Y-mom_rel": lambda: rr[3],
        "Z-mom_rel": lambda: rr[4], "Energy_rel": lambda: rr[5],
        "TKE_abs": lambda: ra[6] if turbulence in k_any else None,
        "Tv_abs": lambda: ra[6] if turbulence in ("sa", "saBC") else None,
        "Dissipation_abs": lambda: ra[7] if turbulence == "ke" else None,
        "Omega_abs": lambda: ra[7] if turbulence in ("sst", "sst2003") else None,
        "Kl_abs": lambda: ra[7] if turbulence == "kkl" else None,
        "TKE_rel": lambda: rr[6] if turbulence in k_any else None,
        "Tv_rel": lambda: rr[6] if turbulence in ("sa", "saBC") else None,
        "Dissipation_rel": lambda: rr[7] if turbulence == "ke" else None,
        "Omega_rel": lambda: rr[7] if turbulence in ("sst", "sst2003") else None,
        "Kl_rel": lambda: rr[7] if turbulence == "kkl" else None,
    }
    parts = ["%d    " % int(iteration)]
    for name in res_list:
        v = table.get(name, lambda: nrm(ra, 1))()  # unknown names: the total norm, as the reference
        if v is not None:
            parts.append(fortran_e(v, w, precision) + "    ")
    return "".join(parts) + "\n"


class ResnormLog:
    """The reference's residual-norm bookkeeping (resnorm.f90:62-91,
    226-238): relative norms are the absolute norms over those of the
    first three iterations' last (or, on a restart, the restart log's),
    and a line is written at iteration 1, 3 and every `interval`-th."""

    SAVE_ITERS = 3  # Res_itr (resnorm.f90:29)

    def __init__(self, path, res_list, interval=100, turbulence="none", precision=6,
                 previous_res=None, last_iter=0):
        self.res_list, self.interval = tuple(res_list), int(interval)
        self.turbulence, self.precision = turbulence, int(precision)
        self.restart = previous_res is not None
        self.saved = None if previous_res is None else np.asarray(previous_res, dtype=np.float64)
        self.last_iter = int(last_iter)
        self.f = open(path, "a" if self.restart and os.path.exists(path) else "w")
        self.f.write(resnorm_header(self.res_list))

    def record(self, current_iter, res_abs):
        """Norms of iteration current_iter (1-based, counted from this
        run's start); returns the relative norms."""
        ra = np.asarray(res_abs, dtype=np.float64)
        if current_iter <= self.SAVE_ITERS and not self.restart:
            self.saved = ra.copy()
        with np.errstate(divide="ignore", invalid="ignore"):  # IEEE results, as in the reference
            rr = ra / self.saved
        if current_iter % self.interval == 0 or current_iter in (1, self.SAVE_ITERS):
            self.f.write(resnorm_line(current_iter + self.last_iter, ra, rr, self.res_list,
                                      self.turbulence, self.precision))
        return rr

    def close(self):
        if self.f:
            self.f.close()
            self.f = None
