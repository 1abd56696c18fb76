"""Independent reader of AMReX plot files and VisMF MultiFabs (test
infrastructure).  The plot-file Header is parsed field by field in the order
the reference's own reader takes it (tools/amrex_plotfile.py,
AmrexPlotFile.parse_header); FAB data follows the published AMReX layout: a
text line "FAB <real descriptor><box> <ncomp>" then the values, component by
component, x fastest."""
import pathlib
import re

import numpy as np

_BOX = re.compile(r"\(\((-?\d+),(-?\d+),(-?\d+)\) \((-?\d+),(-?\d+),(-?\d+)\) \((\d+),(\d+),(\d+)\)\)")


def parse_box(text):
    m = _BOX.search(text)
    v = [int(x) for x in m.groups()]
    return v[0:3], v[3:6], v[6:9]


def read_vismf(prefix):
    """(header dict, array (ncomp, nz, ny, nx) over the FAB's full box)."""
    prefix = pathlib.Path(prefix)
    lines = (prefix.parent / (prefix.name + "_H")).read_text().splitlines()
    hdr = {"version": int(lines[0]), "how": int(lines[1]), "ncomp": int(lines[2]), "ngrow": int(lines[3])}
    assert lines[4].startswith("(1 0")
    hdr["box"] = parse_box(lines[5])
    assert lines[6] == ")"
    assert int(lines[7]) == 1
    fod = lines[8].split()
    assert fod[0] == "FabOnDisk:" and int(fod[2]) == 0
    i = 9
    while lines[i] == "":
        i += 1
    nb, nc = (int(x) for x in lines[i].split(","))
    hdr["min"] = [float(x) for x in lines[i + 1].rstrip(",").split(",")]
    i += 2
    while lines[i] == "":
        i += 1
    hdr["max"] = [float(x) for x in lines[i + 1].rstrip(",").split(",")]
    raw = (prefix.parent / fod[1]).read_bytes()
    eol = raw.index(b"\n")
    line = raw[:eol].decode()
    assert line.startswith("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))")
    lo, hi, typ = parse_box(line[line.index(")))") + 3:])
    ncomp = int(line.rsplit(" ", 1)[1])
    shape = (ncomp, hi[2] - lo[2] + 1, hi[1] - lo[1] + 1, hi[0] - lo[0] + 1)
    data = np.frombuffer(raw[eol + 1:], dtype="<f8", count=int(np.prod(shape))).reshape(shape)
    hdr["fab_box"] = (lo, hi, typ)
    return hdr, data


def read_plotfile(path):
    path = pathlib.Path(path)
    with open(path / "Header") as f:
        h = {"version": f.readline().strip()}
        ncomp = int(f.readline())
        h["names"] = [f.readline().rstrip() for _ in range(ncomp)]
        h["spacedim"] = int(f.readline())
        h["time"] = float(f.readline())
        h["finest_level"] = int(f.readline())
        h["prob_lo"] = [float(x) for x in f.readline().split()]
        h["prob_hi"] = [float(x) for x in f.readline().split()]
        h["ref_ratio"] = [int(x) for x in f.readline().split()]
        h["domain"] = parse_box(f.readline())
        h["level_steps"] = [int(x) for x in f.readline().split()]
        h["dx"] = [float(x) for x in f.readline().split()]
        h["coord"] = int(f.readline())
        h["bwidth"] = int(f.readline())
        lev, nboxes, t = f.readline().split()
        h["level_line"] = (int(lev), int(nboxes), float(t))
        h["level_step"] = int(f.readline())
        h["box_extent"] = [[float(x) for x in f.readline().split()] for _ in range(3)]
        h["mf_path"] = f.readline().strip()
    cell_hdr, data = read_vismf(path / h["mf_path"])
    return h, cell_hdr, data
