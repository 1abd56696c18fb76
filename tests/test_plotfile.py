"""The AMReX plot-file writer on host data (no device): every Header field the
reference's reader parses, the VisMF header and the FAB layout, read back by
the independent reader in amrex_reader.py."""
import numpy as np

from amrex_reader import read_plotfile


def test_plotfile_host_roundtrip(ks_lib, tmp_path):
    rng = np.random.default_rng(5)
    nx, ny, nz = 6, 4, 8
    names = ["density", "gpx", "gpy", "gpz", "p", "velocityx", "velocityy", "velocityz"]
    data = rng.standard_normal((len(names), nz, ny, nx))
    out = tmp_path / "plt00012"
    ks_lib.write_plotfile_host(out, names, data, (0.0, -1.0, 0.5), (3.0, 1.0, 4.5), time=1.25, step=12)
    h, ch, d = read_plotfile(out)
    assert h["version"] == "HyperCLaw-V1.1" and h["names"] == names and h["spacedim"] == 3
    assert h["time"] == 1.25 and h["finest_level"] == 0 and h["ref_ratio"] == []
    assert h["prob_lo"] == [0.0, -1.0, 0.5] and h["prob_hi"] == [3.0, 1.0, 4.5]
    assert h["domain"] == ([0, 0, 0], [nx - 1, ny - 1, nz - 1], [0, 0, 0])
    assert h["level_steps"] == [12] and h["level_step"] == 12 and h["level_line"] == (0, 1, 1.25)
    assert np.allclose(h["dx"], [0.5, 0.5, 0.5]) and h["coord"] == 0 and h["bwidth"] == 0
    assert h["box_extent"] == [[0.0, 3.0], [-1.0, 1.0], [0.5, 4.5]] and h["mf_path"] == "Level_0/Cell"
    assert ch["version"] == 1 and ch["how"] == 1 and ch["ncomp"] == len(names) and ch["ngrow"] == 0
    assert ch["box"] == ([0, 0, 0], [nx - 1, ny - 1, nz - 1], [0, 0, 0])
    assert np.array_equal(d, data)
    assert np.allclose(ch["min"], data.reshape(len(names), -1).min(axis=1), rtol=1e-16, atol=0)
    assert np.allclose(ch["max"], data.reshape(len(names), -1).max(axis=1), rtol=1e-16, atol=0)
    assert (out / "kynema_sgf_info").exists()
