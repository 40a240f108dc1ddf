"""The C++ module shim (include/pv/ampp.hpp): the reference's module classes
over the C ABI, configured from the reference's XML keys.  The test program
tests/cpp/test_ampp.cpp is compiled with g++ against libpv.so; its outputs
are compared with the Python binding (itself checked against the oracle)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from gen import GEN_FCH1, GEN_NCHAN, GEN_NSUB, GEN_TSAMP, generator_pulse, make_bp_text, voltages

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pelican-lofar_gb300")


@pytest.fixture(scope="module")
def shim_exe(pv, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("shim") / "test_ampp")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_ampp.cpp"), "-L", PKG, "-lpv",
           "-Wl,-rpath," + PKG, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "warning" not in r.stderr, r.stderr
    return out


def _run(exe, *args):
    r = subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_shim_reads_the_reference_xml_keys(shim_exe):
    assert "CONFIG OK" in _run(shim_exe, "config")


CHAIN_XML = """<?xml version="1.0"?>
<configuration>
  <PPFChanneliser>
    <outputChannelsPerSubband value="{nchan}"/>
    <filter nTaps="8" filterWindow="kaiser"/>
  </PPFChanneliser>
  <StokesGenerator><numberOfStokes value="1"/></StokesGenerator>
  <StokesIntegrator>
    <integrateTimeBins value="4"/>
    <integrateFrequencyChannels value="1"/>
  </StokesIntegrator>
  <RFI_Clipper active="true" channelRejectionRMS="5.0" spectrumRejectionRMS="4.0">
    <BandPassData file="band.bp"/>
    <Band matching="true"/>
    <History maximum="1000"/>
    <zeroDMing active="true"/>
  </RFI_Clipper>
</configuration>
"""


@pytest.mark.gpu
def test_shim_chain_equals_the_binding(pv, cuda, shim_exe, tmp_path):
    import torch
    nsub, npol, nchan, nblk = 6, 2, 16, 4 * 400
    rng = np.random.default_rng(41)
    _, x = voltages(rng, nsub, npol, nblk * nchan)
    x.tofile(tmp_path / "volt.bin")
    (tmp_path / "shape.txt").write_text("%d %d %d %d\n" % (nsub, npol, nblk, nchan))
    foff = 0.1953125 / nchan
    fch1 = 140.0 - (nchan // 2) * foff
    # the bandpass at the filterbank's own level, as a flat model
    ppf = pv.PPF(nchan, 8, window="kaiser")
    fb = pv.integrate(pv.stokes(ppf.run(torch.from_numpy(x).to(cuda)), 1), 4, 1).cpu().numpy()
    (tmp_path / "band.bp").write_text(make_bp_text(nsub * nchan, fch1, foff, float(fb.mean()),
                                                   float(fb.std())))
    (tmp_path / "config.xml").write_text(CHAIN_XML.format(nchan=nchan))
    out = _run(shim_exe, "chain", tmp_path)
    nu = nblk // 4
    assert out.split()[1:5] == [str(nu), str(nsub), "1", str(nchan)]
    assert abs(float(out.split()[5]) - 5.12e-6 * nchan * 4) < 1e-12
    want_ppf = pv.PPF(nchan, 8, window="kaiser").run(torch.from_numpy(x).to(cuda))
    got_ppf = np.fromfile(tmp_path / "ppf.bin", np.complex64).reshape(want_ppf.shape)
    assert np.array_equal(got_ppf, want_ppf.cpu().numpy())
    st = pv.stokes(want_ppf, 1)
    assert np.array_equal(np.fromfile(tmp_path / "stokes.bin", np.float32), st.cpu().numpy().ravel())
    it = pv.integrate(st, 4, 1)
    assert np.array_equal(np.fromfile(tmp_path / "integ.bin", np.float32), it.cpu().numpy().ravel())
    rfi = pv.RFI((tmp_path / "band.bp").read_text(), cr=5.0, sr=4.0, history=1000, zero_dming=True)
    rfi.run(it)
    got = np.fromfile(tmp_path / "rfi.bin", np.float32)
    assert np.array_equal(got, it.cpu().numpy().ravel())
    assert np.std(got) > 0.1  # clipped and normalised, not blanked


DD_XML = """<configuration>
  <DedispersionModule>
    <timeBinsPerBufferPow2 value="13"/>
    <dedispersionSamples value="200"/>
    <dedispersionStepSize value="0.1"/>
    <dedispersionMinimum value="0"/>
    <frequencyChannel1 MHz="{fch1}"/>
    <channelBandwidth MHz="{foff}"/>
  </DedispersionModule>
  <DedispersionAnalyser>
    <detectionThreshold in_sigma="6.0"/>
    <power2ForBinning value="6"/>
  </DedispersionAnalyser>
</configuration>
"""


@pytest.mark.gpu
def test_shim_dedispersion_module_known_answer(pv, cuda, shim_exe, tmp_path):
    """DedispersionModuleTest::test_method through the module API:
    dmAmplitude(0, 10.0) == 2048 for the generator's DM-10 pulse."""
    blob = generator_pulse(8192, 10.0)[0]
    blob.tofile(tmp_path / "blob.bin")
    (tmp_path / "shape.txt").write_text("%d %d %d %r\n" % (8192, GEN_NSUB, GEN_NCHAN, GEN_TSAMP))
    foff = -6.0 / (GEN_NSUB * GEN_NCHAN)
    (tmp_path / "config.xml").write_text(DD_XML.format(fch1=repr(GEN_FCH1), foff=repr(foff)))
    out = _run(shim_exe, "ddmod", tmp_path, 1).split()
    vals = dict(zip(out[::2], out[1::2]))
    assert float(vals["AMP"]) == 2048.0
    assert int(vals["EVENTS"]) > 200  # more events than DM bins (DedispersionAnalyserTest)
    assert vals["FIRST"] == "0" and vals["UNLOCKED"] == "1" and vals["COMPLETED"] == "1"
    o = pv.DedispersionModule(8192, 200, 0.0, 0.1, GEN_FCH1, foff)
    o.add(blob, GEN_TSAMP)
    assert int(vals["MAXSHIFT"]) == o.params()["maxshift"]


UDP_XML = """<configuration>
  <AdapterTimeSeriesDataSet>
    <fixedSizePackets value="true"/>
    <dataBitSize value="{bits}"/>
    <udpPacketsPerIteration value="{npk}"/>
    <samplesPerPacket value="16"/>
    <outputChannelsPerSubband value="16"/>
    <subbandsPerPacket value="{nsub}"/>
    <nRawPolarisations value="2"/>
    <clock value="200"/>
  </AdapterTimeSeriesDataSet>
</configuration>
"""


@pytest.mark.gpu
@pytest.mark.parametrize("bits", [8, 16])
def test_shim_udp_adapter_equals_the_oracle(pv, oracle, cuda, shim_exe, tmp_path, bits):
    from test_udp import FIXED, make_chunk
    rng = np.random.default_rng(bits)
    npk, nsub = 64, (61 if bits == 16 else 122)
    chunk, _ = make_chunk(rng, npk, nsub, 16, 2, bits, True)
    chunk.tofile(tmp_path / "chunk.bin")
    (tmp_path / "config.xml").write_text(UDP_XML.format(bits=bits, npk=npk, nsub=nsub))
    out = _run(shim_exe, "udp", tmp_path).split()
    assert out[1:5] == [str(npk * 16 // 16), str(nsub), "2", "16"]
    assert float(out[6]) == 1234567890 + 1000 / 195313 and float(out[7]) == 1.0 / 195313
    want = oracle.udp_unpack(chunk, FIXED, npk, bits, nsub, 2, 16)
    got = np.fromfile(tmp_path / "ts.bin", np.complex64).reshape(want.shape)
    assert np.array_equal(got, want)
