"""Seeded synthetic inputs shared by the tests.

``generator_pulse`` restates the reference's test fixture
DedispersionDataGenerator::generate (lib/test/src/DedispersionDataGenerator.cpp:26-81):
32 subbands x 64 channels from 150 MHz with foff = -6/2048 MHz, 327.68 us
samples, value 1.0 inside a 10-sample dispersed track and 0 elsewhere.
"""
import numpy as np

GEN_NSUB, GEN_NCHAN = 32, 64
GEN_FCH1 = 150.0
GEN_FOFF = -6.0 / (GEN_NSUB * GEN_NCHAN)
GEN_TSAMP = 0.00032768
GEN_WIDTH = 10


def generator_pulse(nsamples, dm, nblocks=1, nsub=GEN_NSUB, nchan=GEN_NCHAN, fch1=GEN_FCH1,
                    foff=None, tsamp=GEN_TSAMP, width=GEN_WIDTH, start_bin=0):
    """Blobs [t][sub][1][chan] float32, as the reference generator builds them."""
    if foff is None:
        foff = -6.0 / (nsub * nchan)
    dm = float(np.float32(dm))
    blobs = []
    for i in range(nblocks):
        I = np.zeros((nsamples, nsub, 1, nchan), np.float32)
        offset = i * nsamples
        for ac in range(nsub * nchan):
            f = fch1 + foff * ac
            index = int(dm * (4148.741601 * ((1.0 / f / f) - (1.0 / fch1 / fch1)) / tsamp)) + start_bin
            sample = index - offset
            s, c = divmod(ac, nchan)
            lo, hi = max(sample, 0), min(sample + width, nsamples)
            if hi > lo:
                I[lo:hi, s, 0, c] = 1.0
        blobs.append(I)
    return blobs


def dm_index(dm, dm_low, dm_step):
    """BinMap::binIndex with the float start/width of DedispersionSpectra::resize."""
    return int(0.5 + ((dm - float(np.float32(dm_low))) / float(np.float32(dm_step))))


def buffer_with_padding(rng, nchan, nout, max_shift, dist="normal"):
    """A [nchan][nout+max_shift+pad] float32 buffer of noise."""
    ld = nout + max_shift + 8
    if dist == "normal":
        return rng.standard_normal((nchan, ld), dtype=np.float32)
    return rng.random((nchan, ld), dtype=np.float32)


def make_bp_text(nbins, start, width, median, rms, coeffs=()):
    """A bandpass file in the BandPassAdapter format (BandPassAdapter.cpp:30-108):
    nChan, start, end, channel width, rms, then the polynomial coefficients
    starting with the median."""
    end = start + width * nbins
    lines = ["# synthetic bandpass", "%d" % nbins, repr(float(start)), repr(float(end)),
             repr(float(width)), repr(float(rms)), repr(float(median))]
    lines += [repr(float(c)) for c in coeffs]
    return "\n".join(lines) + "\n"
