"""Output files: OutputCloudTecplot's marker file (ZJS_IO_DEM.F90:82-121) and the
per-body probe lines of fluid.F90:392-397, written by the library's host
writers (no GPU needed).

Every number is written with 17 significant digits, so reading the columns
back gives the doubles exactly.  The field layout follows gfortran's
list-directed output: a record starts with a blank, REAL(8) items are G25.17E3
fields (F20.(17-k) and 5 blanks for 0.1 <= |x| < 1e17, else 1PE25.17E3),
INTEGER items take 12 columns.
"""
import numpy as np
import pytest

from ibmdem import api
from ibmdem.records import MULTISPHERE, PARCEL


@pytest.fixture(scope="module")
def lib():
    import build as b
    import os
    if not os.path.exists(b.LIB):
        b.build()
    return api.load()


def fields(line):
    """Split a list-directed record into its 25- and 12-column items: 6 reals, 1 integer, 3 reals."""
    assert line[0] == " "
    body = line[1:]
    widths = [25] * 6 + [12] + [25] * 3
    out, at = [], 0
    for w in widths:
        out.append(body[at:at + w])
        at += w
    assert at == len(body)
    return out


def test_list_directed_layout(lib, tmp_path):
    p = np.zeros(1, PARCEL)
    p["x"] = [[1.0, 0.1, 123.456]]
    p["v"] = [[1e-5, -2.5, 0.0]]
    p["MSIdx"] = 7
    p["vgap"] = [[1e20, -1e-300, 0.01]]
    path = tmp_path / "Particle_1_0.dat"
    api.write_tecplot_markers(path, p)
    lines = path.read_text().splitlines()
    assert lines[0] == " variables=x,y,z,u,v,w,index,ugap,vgap,wgap"
    assert lines[1] == " zone i=           1 j=           1"
    f = fields(lines[2])
    assert f == ["  1.0000000000000000     ", " 0.10000000000000001     ", "  123.45600000000000     ",
                 "  1.0000000000000001E-005", " -2.5000000000000000     ", "  0.0000000000000000     ",
                 "           7",
                 "  1.0000000000000000E+020", " -1.0000000000000000E-300", "  1.0000000000000000E-002"]


def test_values_read_back_exactly(lib, tmp_path):
    rng = np.random.default_rng(0)
    n = 5000
    p = np.zeros(n, PARCEL)
    mags = 10.0 ** rng.uniform(-30, 30, (n, 3))
    p["x"] = rng.standard_normal((n, 3)) * 40
    p["v"] = rng.standard_normal((n, 3)) * mags
    p["vgap"] = rng.standard_normal((n, 3)) * 1e-3
    p["MSIdx"] = rng.integers(1, 10**6, n)
    path = tmp_path / "m.dat"
    api.write_tecplot_markers(path, p)
    lines = path.read_text().splitlines()
    assert lines[1] == " zone i=%12d j=%12d" % (n, 1)
    rows = [fields(l) for l in lines[2:]]
    assert len(rows) == n
    got = np.array([[float(v) for v in r[:6] + r[7:]] for r in rows])
    want = np.concatenate([p["x"], p["v"], p["vgap"]], axis=1)
    assert np.array_equal(got, want)
    assert np.array_equal([int(r[6]) for r in rows], p["MSIdx"])


def test_empty_rank_writes_the_centre(lib, tmp_path):
    path = tmp_path / "e.dat"
    api.write_tecplot_markers(path, np.zeros(0, PARCEL), centre=(8.0, 4.0, 2.5))
    lines = path.read_text().splitlines()
    assert lines[1] == " zone i=           1 j=           1"
    f = fields(lines[2])
    assert [float(v) for v in f[:3]] == [8.0, 4.0, 2.5] and int(f[6]) == 0


def test_body_probe_lines_append(lib, tmp_path):
    b = np.zeros(2, MULTISPHERE)
    b["globalIdx"] = [3, 11]
    b["m"], b["I"] = 2.0, 0.5
    b["x"] = [[1.5, 2.5, 3.5], [4.0, 5.0, 6.0]]
    b["v"] = [[0.1, 0.2, 0.3], [0.0, 0.0, -1.0]]
    b["omega"] = [[1.0, 0.0, 0.0], [0.0, 2.0, 0.0]]
    b["fdrag"] = [[2.0, 4.0, 6.0], [1.0, 1.0, 1.0]]
    b["fmom"] = [[0.5, 0.0, 0.0], [0.0, 0.25, 0.0]]
    b["fcol"] = [[8.0, 0.0, 0.0], [0.0, 0.0, 2.0]]
    api.write_body_probes(tmp_path, 0, b, 1000.0)
    api.write_body_probes(tmp_path, 1, b, 1000.0)
    for q in range(2):
        lines = (tmp_path / ("%d.probe" % b["globalIdx"][q])).read_text().splitlines()
        assert len(lines) == 2
        for step, line in enumerate(lines):
            assert line[0] == " " and len(line) == 1 + 12 + 18 * 25
            assert int(line[1:13]) == step
            vals = [float(line[13 + 25 * i: 13 + 25 * (i + 1)]) for i in range(18)]
            B = b[q]
            want = np.concatenate([B["x"], B["v"], B["omega"], B["fdrag"] / B["m"] * 1000.0,
                                   B["fmom"] / B["I"] * 1000.0, B["fcol"] / B["m"]])
            assert np.array_equal(vals, want)
