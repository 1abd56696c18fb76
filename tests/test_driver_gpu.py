"""The deck-compatible driver executable (ks_run) on the GPU: an input file
plus command-line overrides, the Evolve loop's console lines, and a non-zero
exit with the library status for decks outside the path."""
import subprocess

import pytest

from kynema_sgf_gb300 import build, decks

pytestmark = pytest.mark.gpu


def test_driver_runs_deck(cuda_dev, tmp_path):
    deck = tmp_path / "tgv.inp"
    deck.write_text(decks.tgv(16, steps=20))
    r = subprocess.run([build.driver_path(), str(deck), "time.max_step=2"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Step: 1 " in r.stdout and "Step: 2 " in r.stdout and "Step: 3 " not in r.stdout
    assert r.stdout.count("Nodal_projection") == 2 and "Time stepping finished." in r.stdout


def test_driver_rejects_unsupported_deck(cuda_dev, tmp_path):
    deck = tmp_path / "amr.inp"
    deck.write_text(decks.tgv(16, steps=2))
    r = subprocess.run([build.driver_path(), str(deck), "amr.max_level=1"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 2 and "single level" in r.stderr


def test_driver_writes_plot_and_checkpoint_files_and_restarts(cuda_dev, tmp_path):
    """The reference's stratified ABL configuration through the driver: plot and
    checkpoint files at the deck's intervals, then a restart from the checkpoint
    (io.restart_file) that continues the step count."""
    deck = tmp_path / "abl.inp"
    deck.write_text(decks.abl_temperature((16, 16, 16), steps=4, diffusion_type=1, fixed_dt=0.5))
    r = subprocess.run([build.driver_path(), str(deck), "time.plot_interval=2", "time.checkpoint_interval=4"], capture_output=True,
                       text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    made = sorted(p.name for p in tmp_path.iterdir() if p.is_dir())
    assert made == ["chk00000", "chk00004", "plt00000", "plt00002", "plt00004"]
    names = (tmp_path / "plt00004" / "Header").read_text().splitlines()[2:14]
    assert "temperature" in names and "temperature_mueff" in names and "mu_turb" in names
    r = subprocess.run([build.driver_path(), str(deck), "io.restart_file=chk00004", "time.max_step=6"], capture_output=True, text=True,
                       timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "Step: 5 " in r.stdout and "Step: 6 " in r.stdout and "Step: 1 " not in r.stdout
