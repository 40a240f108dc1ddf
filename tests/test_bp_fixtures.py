"""The reference's own bandpass files (tests/golden/*.bp, copied by
tests/golden/make_bp_fixtures.py from the reference's test data and pipeline
configurations) load in the library's and the oracle's BandPassAdapter
readers (lib/src/BandPassAdapter.cpp:30-108), and a broken file fails with
the reference's messages (CPU only)."""
import glob
import os

import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FILES = sorted(glob.glob(os.path.join(GOLDEN, "*.bp")))


def test_every_reference_bandpass_file_is_here():
    assert len(FILES) == 6


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_reference_bandpass_file_loads(pv, oracle, path):
    text = open(path).read()
    assert text.startswith("#")
    pv.RFI(text, history=10)
    oracle.RFI(text, history=10)


@pytest.mark.parametrize("path", FILES[:2], ids=[os.path.basename(f) for f in FILES[:2]])
def test_broken_bandpass_files_fail_with_the_reference_messages(pv, oracle, path):
    lines = open(path).read().splitlines()
    short = "\n".join(lines[:6]) + "\n"          # 5 numbers: nChan .. rms
    blank = "\n".join(lines[:3] + [""] + lines[3:]) + "\n"
    for text, msg in ((short, "data format wrong"), (blank, "syntax error on line 4")):
        with pytest.raises(pv.PvError, match=msg):
            pv.RFI(text, history=10)
        with pytest.raises(ValueError):
            oracle.RFI(text, history=10)


def test_kill_lines_are_checked_as_the_reference_reads_them(pv, oracle):
    """BandPassAdapter reads a kill line's index as its frequency too (:60-70),
    so 'K index frequency' passes its bin check only when the index names its
    own bin: with start 0 and width 1 it does, elsewhere it fails."""
    body = open(FILES[0]).read().splitlines()
    own = "\n".join(["# start 0, width 1", "64", "0", "64", "1", "2.0", "10.0", "K 5 5.0"]) + "\n"
    pv.RFI(own, history=10)
    oracle.RFI(own, history=10)
    other = "\n".join(body + ["K 5 131.25"]) + "\n"
    with pytest.raises(pv.PvError, match="Frequency kill mismatch"):
        pv.RFI(other, history=10)
    with pytest.raises(ValueError, match="Frequency kill mismatch"):
        oracle.RFI(other, history=10)
