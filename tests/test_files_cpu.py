"""The reference's file formats on the host (fest3d.files), pinned byte for
byte to files the reference wrote in its own test cases
(tests/golden/reference_files.npz, made by make_reference_files.py):
Tecplot block output of the SmoothBump and turbulent flat-plate runs, their
restart logs and the SmoothBump grid file; plus known answers for the
Fortran edit descriptors and the residual-norm file."""
import hashlib
import os

import numpy as np
import pytest

from fest3d import abi, cases
from fest3d import files as FI

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF = np.load(os.path.join(GOLD, "reference_files.npz"))
VARS = {"bump": ("Velocity", "Density", "Pressure"), "tfp": ("Velocity", "Density", "Pressure", "Mu")}


def sha(text):
    return hashlib.sha256(text.encode()).hexdigest()


def block_arrays(key, n_var):
    """qp, nodes (ABI layouts) and the Mu array of a stored output block."""
    nodes_ijk, fields = REF[key + "_nodes"], REF[key + "_fields"]
    imx, jmx, kmx = nodes_ijk.shape[:3]
    qp = np.zeros((imx + 5, jmx + 5, kmx + 5, n_var), order="F")
    cells = (slice(3, imx + 2), slice(3, jmx + 2), slice(3, kmx + 2))
    for l, var in enumerate((1, 2, 3, 0, 4)):  # u v w, density, pressure
        qp[cells + (var,)] = fields[..., l]
    mu = np.zeros(qp.shape[:3], order="F")
    if fields.shape[-1] > 5:
        mu[cells] = fields[..., 5]
    return qp, FI.nodes_from_grid(nodes_ijk), mu


@pytest.mark.parametrize("key", ["bump0", "bump1", "tfp0", "tfp1"])
def test_tecplot_output_matches_the_reference_bytes(key):
    """write_file (write_output_tec.f90:58-200) text for the block equals the
    file the reference wrote, byte for byte."""
    kind = key[:-1]
    turb = "sst" if kind == "tfp" else "none"
    qp, nodes, mu = block_arrays(key, 7 if turb == "sst" else 5)
    block, t = (int(v) for v in REF[key + "_meta"])
    txt = FI.tecplot_text(qp, nodes, variables=VARS[kind], block=block, solution_time=t,
                          turbulence=turb, extra={"Mu": mu})
    assert sha(txt) == str(REF[key + "_sha256"])


@pytest.mark.parametrize("key", ["bump0", "tfp1"])
def test_tecplot_read_returns_the_written_fields(key, tmp_path):
    """read_file (read_output_tec.f90:48-140) of the written file recovers
    the interior fields exactly (16 significant digits of these values
    parse back to the same doubles) and leaves the ghost cells alone; a
    name the reference cannot read (Mu) reads nothing."""
    kind = key[:-1]
    turb = "sst" if kind == "tfp" else "none"
    qp, nodes, mu = block_arrays(key, 7 if turb == "sst" else 5)
    p = tmp_path / "process_00.dat"
    FI.write_tecplot(p, qp, nodes, variables=VARS[kind], turbulence=turb, extra={"Mu": mu})
    back = np.full_like(qp, -7.0)
    FI.read_tecplot(p, back, VARS[kind], turbulence=turb)
    imx, jmx, kmx = qp.shape[0] - 5, qp.shape[1] - 5, qp.shape[2] - 5
    cells = (slice(3, imx + 2), slice(3, jmx + 2), slice(3, kmx + 2))
    for l in range(5):
        assert np.array_equal(back[cells + (l,)], qp[cells + (l,)])
    ghost = np.ones(qp.shape[:3], bool)
    ghost[cells] = False
    assert np.all(back[ghost] == -7.0)
    if turb == "sst":
        assert np.all(back[..., 5:] == -7.0)  # TKE/Omega not in the file, not read


def test_tecplot_round_trip_of_an_arbitrary_state(tmp_path):
    """Any double goes through the file to within the 16 significant digits
    ES28.15E4 keeps (the reference's restarts lose the same)."""
    ext = abi.Extent(9, 7, 4, 5)
    nodes = cases.box_nodes(ext, perturb=0.05)
    qp = np.asfortranarray(cases.random_state(ext, seed=3))
    p = tmp_path / "s.dat"
    FI.write_tecplot(p, qp, nodes)
    back = np.zeros_like(qp)
    FI.read_tecplot(p, back)
    c = (slice(3, 11), slice(3, 9), slice(3, 6))
    assert np.allclose(back[c], qp[c], rtol=6e-16, atol=0)


def test_tecplot_reader_refuses_a_short_file(tmp_path):
    qp, nodes, _ = block_arrays("bump0", 5)
    p = tmp_path / "short.dat"
    txt = FI.tecplot_text(qp, nodes)
    p.write_text("\n".join(txt.split("\n")[:-100]))
    with pytest.raises(ValueError):
        FI.read_tecplot(p, np.zeros_like(qp))


@pytest.mark.parametrize("key", ["bump0", "tfp1"])
def test_restart_log_matches_the_reference_bytes(key, tmp_path):
    """write_restart_log (dump_solution.f90:120-153) of what
    read_restart_file reads back reproduces the reference's log."""
    text = str(REF[key + "_restart"])
    src = tmp_path / "in"
    src.write_text(text)
    kind, last, prev = FI.read_restart_log(src)
    assert kind == ("viscous" if key.startswith("bump") else "sst")
    dst = tmp_path / "out"
    FI.write_restart_log(dst, "none" if kind == "viscous" else kind, last, prev)
    assert dst.read_text() == text


def test_grid_file_matches_the_reference_bytes(tmp_path):
    """The SmoothBump block-0 grid file (49x49x2 nodes) written from its
    nodes is the reference's grid_00.txt, byte for byte; read back, the
    nodes are identical."""
    nodes = np.load(os.path.join(GOLD, "smoothbump_nodes.npz"))["nodes"][:49]
    p = tmp_path / "grid_00.txt"
    FI.write_grid(p, nodes)
    assert hashlib.sha256(p.read_bytes()).hexdigest() == str(REF["grid00_sha256"])
    assert np.array_equal(FI.read_grid(p), nodes)


def test_fortran_edit_descriptors():
    es = FI.fortran_es
    assert es(-1.5) == "    -1.500000000000000E+0000"
    assert es(0.0) == "     0.000000000000000E+0000"
    assert es(-0.0) == "    -0.000000000000000E+0000"
    assert es(1.0e-300) == "     1.000000000000000E-0300"
    assert es(float("nan")) == "NaN".rjust(28)
    e = FI.fortran_e
    assert e(1.234e-5, 14, 6) == "  0.123400E-04"
    assert e(-1.234e-5, 14, 6) == " -0.123400E-04"
    assert e(9.9999996e-3, 14, 6) == "  0.100000E-01"  # rounding carries into the exponent
    assert e(0.0, 14, 6) == "  0.000000E+00"
    assert e(3.0e120, 14, 6) == "*" * 14  # exponent beyond two digits
    assert e(0.1015625, 14, 6) == "  0.101562E+00"  # an exact tie rounds to even
    f0 = FI.fortran_f0
    assert f0(0.0) == ".0000000000000000"
    assert f0(1.5) == "1.5000000000000000"
    assert f0(-0.25) == "-.2500000000000000"


def test_resnorm_file():
    """write_resnorm (resnorm.f90:241-377) lines and the relative-norm
    bookkeeping: saved norms of iteration 3 (Res_itr), lines at 1, 3 and
    every interval-th iteration, continued after a restart."""
    names = ("Mass_abs", "Viscous_abs", "Continuity_abs", "TKE_abs", "Continuity_rel")
    ra = np.array([2e-3, 3.0, 4.0, 0.0, 0.0, 12.0])
    line = FI.resnorm_line(7, ra, ra / 2, names)
    assert line == ("7    " + "  0.200000E-02    " + "  0.130000E+02    " + "  0.300000E+01    "
                    + "  0.150000E+01    " + "\n")  # TKE_abs left out without SST
    assert FI.resnorm_header(names[:2]) == "Iteration  Mass_abs  Viscous_abs  \n"


def test_resnorm_log(tmp_path):
    p = tmp_path / "resnorm"
    log = FI.ResnormLog(p, ("Continuity_abs", "Continuity_rel"), interval=4)
    for it in range(1, 9):
        rr = log.record(it, [0.0, 10.0 / it, 1, 1, 1, 1])
    log.close()
    rows = p.read_text().splitlines()
    assert rows[0] == "Iteration  Continuity_abs  Continuity_rel  "
    assert [int(r.split()[0]) for r in rows[1:]] == [1, 3, 4, 8]
    assert rr[1] == pytest.approx((10.0 / 8) / (10.0 / 3))
    # a restart: relative to the log's saved norms, iterations continued
    log = FI.ResnormLog(p, ("Continuity_rel",), interval=4, previous_res=[1, 2, 1, 1, 1, 1],
                        last_iter=8)
    rr = log.record(1, [0, 1, 1, 1, 1, 1])
    log.close()
    assert rr[1] == 0.5
    assert p.read_text().splitlines()[-1].split()[0] == "9"


def test_vtk_output_format_and_round_trip(tmp_path):
    """write_file/read_file of the legacy VTK format (write_output_vtk.f90,
    read_output_vtk.f90): known answers for the records the writer's edit
    descriptors give, and the SST state (with TKE and Omega) read back to
    within 17 significant digits of rounding."""
    ext = abi.Extent(6, 5, 3, 7)
    nodes = cases.box_nodes(ext, perturb=0.05)
    qp = np.asfortranarray(cases.random_state(ext, seed=5, tk=1.5, tw=800.0))
    qp[3, 3, 3, 1:4] = (-1.5, 0.25, 0.0)
    qp[3, 3, 3, 0] = 1.225
    mu = np.full(qp.shape[:3], 1.8e-5, order="F")
    names = ("Velocity", "Density", "Pressure", "TKE", "Omega", "Mu")
    txt = FI.vtk_text(qp, nodes, variables=names, turbulence="sst", extra={"Mu": mu})
    rows = txt.split("\n")
    assert rows[:6] == ["# vtk DataFile Version 3.1", "cfd-iitm output", "ASCII",
                        "DATASET STRUCTURED_GRID", "DIMENSIONS 6 5 3", "POINTS 90 DOUBLE"]
    assert rows[6] == "%s %s %s" % tuple(FI.fortran_f0(nodes[c, 3, 3, 3]) for c in range(3))
    v = rows.index("VECTORS Velocity FLOAT")
    assert rows[v - 1] == "CELL_DATA 40" and rows[v - 2] == "" and rows[v - 3] != ""
    assert rows[v + 1] == "  -1.5000000000000000E+0000    2.5000000000000000E-0001    0.0000000000000000E+0000"
    d = rows.index("SCALARS Density FLOAT")
    assert rows[d + 1] == "LOOKUP_TABLE default"
    assert rows[d + 2] == " 1.2250000000000001E+0000"  # 17 significant digits of the double 1.225
    assert "SCALARS Mu FLOAT" in rows and txt.endswith("\n\n")
    p = tmp_path / "process_00.vtk"
    p.write_text(txt)
    back = np.zeros_like(qp)
    FI.read_vtk(p, back, ("Velocity", "Density", "Pressure", "TKE", "Omega", "Mu"), turbulence="sst")
    c = (slice(3, 8), slice(3, 7), slice(3, 5))
    assert np.array_equal(back[c], qp[c])  # 17 digits round-trip every double
    # 'do not read' skips a scalar field
    back2 = np.zeros_like(qp)
    FI.read_vtk(p, back2, ("Velocity", "do not read", "Pressure"), turbulence="sst")
    assert np.array_equal(back2[c + (4,)], qp[c + (4,)]) and np.all(back2[c + (0,)] == 0)


def test_tecplot_nodal_output():
    """'tecplot_nodal' output (write_output_tec_node.f90): header with
    k = kmx-1 node planes and nodal data, node coordinates of those planes,
    each field the four-cell mean around a node (ghost cells included, the
    reference's summation order), 35 E25.15 values per record."""
    ext = abi.Extent(5, 4, 3, 5)
    nodes = cases.box_nodes(ext, perturb=0.05)
    qp = np.asfortranarray(cases.random_state(ext, seed=7))
    txt = FI.tecplot_nodal_text(qp, nodes, block=2, solution_time=4)
    rows = txt.split("\n")
    assert rows[:9] == ["variables = x y z ", " u v w ", "Density ", "Pressure ",
                        "zone T=block0002  i=00005 j=00004 k=00002 Datapacking=Block",
                        " Varlocation=([1-3]=Nodal)", "Varlocation=([4-08]=Nodal)",
                        "STRANDID=0001", "SOLUTIONTIME=0004"]
    n = 5 * 4 * 2  # values per field: 40 -> records of 35 and 5
    body = rows[9:-1]
    assert len(body) == 8 * 2 and all(len(r) == 25 * 35 for r in body[0::2])
    assert all(len(r) == 25 * 5 for r in body[1::2])
    vals = np.array([float(r[m:m + 25]) for r in body for m in range(0, len(r), 25)]).reshape(8, n)
    x = [nodes[0, i + 2, j + 2, k + 2] for k in (1, 2) for j in range(1, 5) for i in range(1, 6)]
    assert np.allclose(vals[0], x, rtol=1e-14, atol=0)  # 15 significant digits
    expect = []
    for l in (1, 2, 3, 0, 4):
        q = qp[..., l]
        expect.append([0.25 * (q[i + 2, j + 2, k + 2] + q[i + 1, j + 2, k + 2] + q[i + 2, j + 1, k + 2]
                               + q[i + 1, j + 1, k + 2])
                       for k in (1, 2) for j in range(1, 5) for i in range(1, 6)])
    first = [FI.fortran_e(v, 25, 15, None) for v in expect[0]]
    assert body[6] == "".join(first[:35]) and body[7] == "".join(first[35:])
    assert np.allclose(vals[3:], expect, rtol=1e-14, atol=0)
    assert FI.fortran_e(-2e-120, 25, 15, None) == "   -0.200000000000000-119"


def test_tecplot_sst_state_round_trip(tmp_path):
    """An SST state written with TKE and Omega (write_output_tec.f90's tk/tw
    fields, header 'TKE ' and 'Omega ', 10 variables) reads back into
    variables 6 and 7; asking for them without a k-omega model is refused."""
    ext = abi.Extent(7, 6, 3, 7)
    nodes = cases.box_nodes(ext)
    qp = np.asfortranarray(cases.random_state(ext, seed=11, tk=2.0, tw=900.0))
    names = ("Velocity", "Density", "Pressure", "TKE", "Omega")
    p = tmp_path / "sst.dat"
    FI.write_tecplot(p, qp, nodes, variables=names, turbulence="sst")
    rows = p.read_text().split("\n")
    assert rows[4:6] == ["TKE ", "Omega "] and rows[8] == "Varlocation=([4-10]=CELLCENTERED)"
    back = np.zeros_like(qp)
    FI.read_tecplot(p, back, names, turbulence="sst")
    c = (slice(3, 9), slice(3, 8), slice(3, 5))
    assert np.allclose(back[c], qp[c], rtol=6e-16, atol=0)
    with pytest.raises(ValueError):
        FI.tecplot_text(qp, nodes, variables=names, turbulence="none")
