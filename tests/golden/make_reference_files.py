"""Make reference_files.npz: the contents and SHA-256 digests of files the
reference wrote in its own test cases, for the byte-for-byte checks of
fest3d.files:

* Tecplot block output (write_output_tec.f90): SmoothBump
  time_directories/0010/process_0{0,1}.dat (u v w, density, pressure) and
  Tfp time_directories/0002/process_0{0,1}.dat (u v w, density, pressure,
  Mu).  Stored: the interior nodes and cell fields as parsed from the
  files (16 significant digits, which format back to the same text), the
  block number, the solution time and the digest of the file's bytes.
* the restart logs next to them (dump_solution.f90), as text;
* the SmoothBump grid file system/mesh/gridfiles/grid_00.txt: its digest
  (its nodes are block 0 of smoothbump_nodes.npz).

Run in the container that holds the reference:

    python tests/golden/make_reference_files.py /root/reference/tests
"""
import argparse
import hashlib
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

TEC = {
    "bump0": ("SmoothBump/time_directories/0010/process_00.dat", 10),
    "bump1": ("SmoothBump/time_directories/0010/process_01.dat", 10),
    "tfp0": ("Tfp/time_directories/0002/process_00.dat", 2),
    "tfp1": ("Tfp/time_directories/0002/process_01.dat", 2),
}
RESTART = {
    "bump0": "SmoothBump/time_directories/0010/restart/process_00",
    "tfp1": "Tfp/time_directories/0002/restart/process_01",
}
GRID = "SmoothBump/system/mesh/gridfiles/grid_00.txt"


def parse_tecplot(path):
    """(block, imx, jmx, kmx, labels, nodes (imx,jmx,kmx,3), fields
    (imx-1,jmx-1,kmx-1,n)) of a FEST-3D Tecplot block file."""
    lines = open(path).read().split("\n")
    z = next(i for i, ln in enumerate(lines) if ln.startswith("zone T=block"))
    head = lines[z]
    block = int(head.split("block")[1][:4])
    imx, jmx, kmx = (int(head.split(t)[1][:5]) for t in ("i=", "j=", "k="))
    labels = " ".join(lines[1:z]).split()
    vals = np.array(" ".join(lines[z + 5:]).split(), dtype=np.float64)
    nn, nc = imx * jmx * kmx, (imx - 1) * (jmx - 1) * (kmx - 1)
    assert vals.size == 3 * nn + len(labels) * nc, (path, vals.size)
    nodes = np.stack([vals[c * nn:(c + 1) * nn].reshape((imx, jmx, kmx), order="F")
                      for c in range(3)], axis=-1)
    fields = np.stack([vals[3 * nn + l * nc:3 * nn + (l + 1) * nc].reshape((imx - 1, jmx - 1, kmx - 1), order="F")
                       for l in range(len(labels))], axis=-1)
    return block, labels, nodes, fields


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("tests_dir", help="the reference's tests directory")
    a = ap.parse_args()
    out = {}
    for key, (rel, t) in TEC.items():
        p = os.path.join(a.tests_dir, rel)
        block, labels, nodes, fields = parse_tecplot(p)
        out[key + "_nodes"] = nodes
        out[key + "_fields"] = fields
        out[key + "_labels"] = np.array(labels)
        out[key + "_meta"] = np.array([block, t])
        out[key + "_sha256"] = np.array(hashlib.sha256(open(p, "rb").read()).hexdigest())
    for key, rel in RESTART.items():
        out[key + "_restart"] = np.array(open(os.path.join(a.tests_dir, rel)).read())
    g = os.path.join(a.tests_dir, GRID)
    out["grid00_sha256"] = np.array(hashlib.sha256(open(g, "rb").read()).hexdigest())
    dst = os.path.join(HERE, "reference_files.npz")
    np.savez_compressed(dst, **out)
    print(dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
