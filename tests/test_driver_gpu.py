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
