"""Copies the reference's bandpass fixtures (BandPassAdapter format) into this
directory.  Run in a checkout that has the reference next to it:

    python tests/golden/make_bp_fixtures.py /path/to/pelican-lofar

The files are the ones the reference's own tests and pipeline configurations
load: lib/test/data/t191_BAND.bp (BandPassTest), pipelines/udpstream/test/data/
band31.bp, and the pipelines' data/*.bp.  tests/test_bp_fixtures.py parses
every copy with the library's and the oracle's readers."""
import os
import shutil
import sys

FIXTURES = [
    "src/lib/test/data/t191_BAND.bp",
    "src/pipelines/udpstream/test/data/band31.bp",
    "src/pipelines/udpstream/data/alfaburst.bp",
    "src/pipelines/udpstream/data/band220-249.bp",
    "src/pipelines/udpstream/data/band220-250.bp",
    "src/pipelines/udpstream/data/gbt.bp",
]


def main(root):
    here = os.path.dirname(os.path.abspath(__file__))
    for rel in FIXTURES:
        shutil.copyfile(os.path.join(root, rel), os.path.join(here, os.path.basename(rel)))
        print(rel)


if __name__ == "__main__":
    main(sys.argv[1])
