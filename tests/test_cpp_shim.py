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
    lines = _run(shim_exe, "ddmod", tmp_path, 1).splitlines()
    vals = {ln.split()[0]: ln.split()[1:] for ln in lines}
    assert float(vals["AMP"][0]) == 2048.0
    assert int(vals["EVENTS"][0]) > 200  # more events than DM bins (DedispersionAnalyserTest)
    assert vals["FIRST"] == ["0"] and vals["COMPLETED"] == ["1"]
    # the blob fills the buffer: locked for it and for the next buffer's overlap, so one lock
    # remains after the export and the unlock callback releases nothing yet
    assert int(vals["LOCKS_ADD0"][0]) == 2 and vals["LOCKS_END"] == ["1"] and vals["UNLOCKED"] == []
    assert vals["ASYNC"] == ["1"] and vals["THREAD"] == ["1"]
    o = pv.DedispersionModule(8192, 200, 0.0, 0.1, GEN_FCH1, foff)
    o.add(blob, GEN_TSAMP)
    assert int(vals["MAXSHIFT"][0]) == o.params()["maxshift"]


@pytest.mark.gpu
def test_shim_dedispersion_module_locks_and_returns_before_the_functors(pv, cuda, shim_exe, tmp_path):
    """DedispersionModuleTest::test_multipleBlobsPerBuffer (lib/test/src/
    DedispersionModuleTest.cpp:201-270): two blobs of half a buffer.  The
    first only buffers (no locks, no functor call); the second fills the
    buffer, dedisperse() returns before the functor runs (on another
    thread), the second blob holds more than one lock (it is also in the
    next buffer's overlap); after the chain the first blob is free and was
    passed to the unlock callback, the second keeps one lock."""
    blobs = generator_pulse(4096, 10.0, nblocks=2)
    np.concatenate(blobs).tofile(tmp_path / "blob.bin")
    (tmp_path / "shape.txt").write_text("%d %d %d %r\n" % (4096, GEN_NSUB, GEN_NCHAN, GEN_TSAMP))
    foff = -6.0 / (GEN_NSUB * GEN_NCHAN)
    (tmp_path / "config.xml").write_text(DD_XML.format(fch1=repr(GEN_FCH1), foff=repr(foff)))
    lines = _run(shim_exe, "ddmod", tmp_path, 2).splitlines()
    vals = {ln.split()[0]: ln.split()[1:] for ln in lines}
    assert vals["LOCKS_ADD0"] == ["0", "0"]
    assert int(vals["LOCKS_ADD1"][1]) > 1
    assert float(vals["AMP"][0]) == 2048.0 and vals["INPUTS"] == ["2"] and vals["COMPLETED"] == ["1"]
    assert vals["LOCKS_END"] == ["0", "1"] and vals["UNLOCKED"] == ["0"]
    assert vals["ASYNC"] == ["1"] and vals["THREAD"] == ["1"]


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
    lines = {ln.split()[0]: ln.split()[1:] for ln in _run(shim_exe, "udp", tmp_path).splitlines() if ln}
    assert lines["SHAPE"] == [str(npk * 16 // 16), str(nsub), "2", "16"]
    assert float(lines["TIME"][0]) == 1234567890 + 1000 / 195313 and float(lines["TIME"][1]) == 1.0 / 195313
    assert "Adapter:" in lines  # the first chunk follows time 0: the reference's out-of-sequence note
    want = oracle.udp_unpack(chunk, FIXED, npk, bits, nsub, 2, 16)
    got = np.fromfile(tmp_path / "ts.bin", np.complex64).reshape(want.shape)
    assert np.array_equal(got, want)


DDOUT_XML = """<configuration>
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
  <DedispersionDataAnalysisOutput>
    <file name="{path}"/>
  </DedispersionDataAnalysisOutput>
</configuration>
"""


@pytest.mark.gpu
def test_shim_event_output_file_equals_the_oracle_text(pv, oracle, cuda, shim_exe, tmp_path):
    """DedispersionModule -> DedispersionAnalyser -> DedispersionDataAnalysisOutput
    through the module API: the .dat file is the reference's header and, per
    buffer, the oracle's formatting of the events the analyser found."""
    blob = generator_pulse(8192, 10.0)[0]
    blob.tofile(tmp_path / "blob.bin")
    t0 = 1.3e9 + 0.25
    (tmp_path / "shape.txt").write_text("%d %d %d %r %r\n" % (8192, GEN_NSUB, GEN_NCHAN, GEN_TSAMP, t0))
    foff = -6.0 / (GEN_NSUB * GEN_NCHAN)
    (tmp_path / "config.xml").write_text(DDOUT_XML.format(fch1=repr(GEN_FCH1), foff=repr(foff),
                                                          path=str(tmp_path / "events")))
    out = _run(shim_exe, "ddout", tmp_path, 1)
    metas = [line.split()[1:] for line in out.splitlines() if line.startswith("META")]
    assert len(metas) == 1
    files = list(tmp_path.glob("events_D*.dat"))
    assert len(files) == 1
    ev = np.fromfile(tmp_path / "events.bin", pv.EVENT_DTYPE)
    start, rate, first, dm_low, dm_step, rms, n = metas[0]
    assert int(n) == len(ev) > 200 and float(start) == t0
    want = oracle.EVENTS_TEXT_HEADER + oracle.events_text(ev, float(start), float(rate), int(first),
                                                          float(dm_low), float(dm_step), np.float32(rms), 1)
    assert files[0].read_text() == want


TRIGGER_XML = """  <TriggerOutput>
    <Receiver host="127.0.0.1" port="{port}"/>
    <Trigger format="FRATS"/>
    <Logfile name="{log}"/>
    <Telescope stationID="CS302" beamID="7"/>
    <RADec rajd="83.633" decjd="22.014"/>
    <frequencyChannel1 MHz="150.0"/>
    <Threshold snr="{snr}" events="2"/>
  </TriggerOutput>
</configuration>
"""


OUTPUTS_XML = """<configuration>
  <DedispersionDataAnalysisOutput>
    <file name="{path}"/>
  </DedispersionDataAnalysisOutput>
""" + TRIGGER_XML


def test_shim_outputs_of_an_analysed_buffer_equal_the_oracle(pv, oracle, shim_exe, tmp_path):
    """No GPU: one analysed buffer, sent twice, through the shim's
    DedispersionDataAnalysisOutput (the .dat text) and TriggerOutput (the
    datagrams, numbered 0001 and 0002, and the log lines)."""
    import re
    import socket
    from test_outputs import _events
    ev = _events(np.random.default_rng(41), 30)
    ev.tofile(tmp_path / "events.bin")
    start, rate, first, rms = 1.31e9 + 0.5, 327.68e-6, 8192, np.float32(45.254834)
    (tmp_path / "meta.txt").write_text("%r %r %d %r %r %r %d %d\n" % (start, rate, first, 0.0, 0.25,
                                                                       float(rms), 4096, 200))
    rx = socket.socket(socket.AF_INET, socket.SOCK_DGRAM)
    rx.bind(("127.0.0.1", 0))
    rx.settimeout(5.0)
    (tmp_path / "config.xml").write_text(OUTPUTS_XML.format(path=tmp_path / "ev", port=rx.getsockname()[1],
                                                            log=tmp_path / "trig.log", snr=5.0))
    out = _run(shim_exe, "outputs", tmp_path)
    sent = [ln[len("TRIGGER "):] for ln in out.splitlines() if ln.startswith("TRIGGER ")]
    assert len(sent) == 2
    root = re.fullmatch(r"artemis:CS302##ID:(\d{12}-07)0001##.*", sent[0]).group(1)
    want = [oracle.trigger_message(ev, start, rate, first, 0.0, float(np.float32(0.25)), rms, 2, 5.0, "CS302", root,
                                   k, "150.0", "83.633", "22.014") for k in (1, 2)]
    assert sent == want
    assert [rx.recv(4096).decode() for _ in range(2)] == want
    assert (tmp_path / "trig.log").read_text() == want[0] + "\n" + want[1] + "\n"
    files = list(tmp_path.glob("ev_D*.dat"))
    assert len(files) == 1
    text = "".join(oracle.events_text(ev, start, rate, first, 0.0, float(np.float32(0.25)), rms, k) for k in (1, 2))
    assert files[0].read_text() == oracle.EVENTS_TEXT_HEADER + text
    rx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("snr", [8.0, 1e9])
def test_shim_trigger_output_sends_the_oracle_message(pv, oracle, cuda, shim_exe, tmp_path, snr):
    """DedispersionModule -> DedispersionAnalyser -> TriggerOutput through the
    module API: the datagram received on the loopback port and the log line are
    the oracle's FRATS message for the events the analyser found; a threshold
    no event reaches sends nothing."""
    import re
    import socket
    rx = socket.socket(socket.AF_INET, socket.SOCK_DGRAM)
    rx.bind(("127.0.0.1", 0))
    rx.settimeout(5.0)
    blob = generator_pulse(8192, 10.0)[0]
    blob.tofile(tmp_path / "blob.bin")
    t0 = 1.3e9 + 0.25
    (tmp_path / "shape.txt").write_text("%d %d %d %r %r\n" % (8192, GEN_NSUB, GEN_NCHAN, GEN_TSAMP, t0))
    foff = -6.0 / (GEN_NSUB * GEN_NCHAN)
    xml = DDOUT_XML.format(fch1=repr(GEN_FCH1), foff=repr(foff), path=str(tmp_path / "events"))
    xml = xml.replace("</configuration>\n", TRIGGER_XML.format(port=rx.getsockname()[1], log=tmp_path / "trig.log",
                                                                snr=snr))
    (tmp_path / "config.xml").write_text(xml)
    out = _run(shim_exe, "ddout", tmp_path, 1)
    metas = [line.split()[1:] for line in out.splitlines() if line.startswith("META")]
    sent = [line[len("TRIGGER "):] for line in out.splitlines() if line.startswith("TRIGGER ")]
    ev = np.fromfile(tmp_path / "events.bin", pv.EVENT_DTYPE)
    start, rate, first, dm_low, dm_step, rms, n = metas[0]
    if snr > 1e6:
        assert sent == []
        assert not (tmp_path / "trig.log").exists() or (tmp_path / "trig.log").read_text() == ""
        rx.close()
        return
    assert len(sent) == 1
    m = re.fullmatch(r"artemis:CS302##ID:(\d{12}-07)0001##.*", sent[0])
    assert m, sent[0]
    want = oracle.trigger_message(ev, float(start), float(rate), int(first), float(dm_low), float(dm_step),
                                  np.float32(rms), 2, snr, "CS302", m.group(1), 1, "150.0", "83.633", "22.014")
    assert sent[0] == want
    assert rx.recv(4096).decode() == want
    assert (tmp_path / "trig.log").read_text() == want + "\n"
    rx.close()


AB_XML = """<configuration>
  <ABDataAdapter>
    <spectrum packets="4"/>
    <packet channels="{nch}"/>
    <samplingTime seconds="{tsamp}"/>
  </ABDataAdapter>
  <ABPipeline>
    <history value="2048"/>
    <events min="{emin}" max="{emax}"/>
  </ABPipeline>
  <RFI_Clipper active="true" channelRejectionRMS="3.5" spectrumRejectionRMS="6.0">
    <zeroDMing active="true"/>
    <BandPassData file="band.bp"/>
    <Band matching="true"/>
    <History maximum="1000"/>
  </RFI_Clipper>
  <DedispersionModule>
    <timeBinsPerBufferPow2 value="12"/>
    <frequencyChannel1 MHz="{fch1}"/>
    <sampleTime seconds="{tsamp}"/>
    <channelBandwidth MHz="{foff}"/>
    <dedispersionSamples value="{tdms}"/>
    <dedispersionStepSize value="{dm_step}"/>
    <dedispersionMinimum value="0"/>
  </DedispersionModule>
  <DedispersionAnalyser>
    <detectionThreshold in_sigma="{thr}"/>
    <power2ForBinning value="4"/>
  </DedispersionAnalyser>
  <DedispersionDataAnalysisOutput>
    <file name="{path}"/>
  </DedispersionDataAnalysisOutput>
</configuration>
"""


@pytest.mark.gpu
@pytest.mark.parametrize("emin,emax", [(1, 0), (10 ** 6, 10 ** 7)])
def test_shim_ab_pipeline_from_spectrometer_packets_to_event_file(pv, oracle, cuda, shim_exe, tmp_path, emin,
                                                                  emax):
    """ALFABURST packets -> ABDataAdapter -> ABPipeline (StokesIntegrator with
    its defaults, RFI_Clipper, DedispersionModule, analyser) ->
    DedispersionDataAnalysisOutput, with 8 packets lost in the fourth chunk:
    the adapter's blobs equal the oracle's, and the event file equals the same
    chain composed through the Python binding."""
    import torch
    from gen import ab_emulator_packets
    nch, npk, nchunks, tdms, dm_step, thr = 64, 4096, 10, 32, 1.0, 3.0
    fch1, foff, tsamp = 1500.0, -0.1, 0.000128
    rng = np.random.default_rng(23)
    total = nchunks * npk + 8
    lost = tuple(range(3 * npk + 100, 3 * npk + 108))
    stream = ab_emulator_packets(total, nch, counter0=5000, records=rng.integers(0, 65536, (total, nch, 4)),
                                 skip=lost)
    stream.tofile(tmp_path / "chunks.bin")
    chunk_bytes = len(stream) // nchunks
    chunks = [stream[k * chunk_bytes:(k + 1) * chunk_bytes] for k in range(nchunks)]
    ad = pv.ABDataAdapter(packets=4, channels=nch, seconds=tsamp)
    spectra, times, ost = [], [], {"seen": 0, "count0": 0, "last_time": 0.0}
    for c in chunks:
        x = ad.deserialise(c)
        want, t, _, _ = oracle.ab_deserialise(c, 4, nch, 0, tsamp, ost)
        assert np.array_equal(x.cpu().numpy().reshape(want.shape), want) and ad.timestamp == t
        spectra.append(x)
        times.append(t)
    fb0 = spectra[0].cpu().numpy()
    (tmp_path / "band.bp").write_text(make_bp_text(nch, fch1 + foff * (nch - 1), -foff, float(fb0.mean()),
                                                   float(fb0.std())))
    (tmp_path / "config.xml").write_text(AB_XML.format(nch=nch, tsamp=repr(tsamp), emin=emin, emax=emax,
                                                       fch1=repr(fch1), foff=repr(foff), tdms=tdms,
                                                       dm_step=dm_step, thr=thr, path=str(tmp_path / "ev")))
    out = _run(shim_exe, "ab", tmp_path, nchunks)
    lines = out.splitlines()
    got_times = [float(ln.split()[1]) for ln in lines if ln.startswith("TIME")]
    assert got_times == times
    assert all(float(ln.split()[2]) == float(np.float32(tsamp)) for ln in lines if ln.startswith("TIME"))
    assert int(out.split("GAPS")[1].split()[0]) == 1
    got_sp = np.fromfile(tmp_path / "spectra.bin", np.float32)
    assert np.array_equal(got_sp, torch.cat([s.reshape(-1) for s in spectra]).cpu().numpy())
    nbuf = int(out.split("BUFFERS")[1].split()[0])
    # the same chain through the binding
    rfi = pv.RFI((tmp_path / "band.bp").read_text(), cr=3.5, sr=6.0, history=1000, zero_dming=True)
    dd = pv.DedispersionModule(1 << 12, tdms, 0.0, dm_step, fch1, foff)
    rate = float(np.float32(tsamp))
    rms = float(np.sqrt(np.float32(nch) * np.float32(1)))
    text, dump, nbuf_want, signal = "", 0, 0, []
    nblk = npk // 4
    for x in spectra:
        xi = pv.integrate(x, 1, 1)
        rfi.run(xi)
        for buf, first in dd.add(xi.cpu().numpy(), rate):
            nbuf_want += 1
            ev, n = pv.analyse(torch.from_numpy(buf).to(cuda), thr, rms, 4)
            if (n >= emin) if emin >= emax else (emin <= n <= emax):
                dump += 1
                text += pv.events_text(ev, times[0], rate, first, 0.0, dm_step, np.float32(rms), dump)
                # SignalFoundSpectrum: the chunks whose samples the 4096-sample buffer holds
                signal += [(dump, times[k], nblk) for k in range(nchunks)
                           if k * nblk < first + 4096 and (k + 1) * nblk > first]
    assert nbuf == nbuf_want >= 2
    got_signal = [(int(ln.split()[1]), float(ln.split()[2]), int(ln.split()[3])) for ln in lines
                  if ln.startswith("SIGNAL")]
    assert got_signal == signal and (emin > 1000) == (signal == [])
    files = list(tmp_path.glob("ev_D*.dat"))
    assert len(files) == 1
    assert files[0].read_text() == pv.EVENTS_TEXT_HEADER + text
    if emin > 1000:
        assert text == ""
    else:
        assert text.count("\n") > 2


SIGPROC_XML = """<configuration>
  <SigprocStokesWriter writeHeader="true">
    <file filepath="{path}"/>
    <subbandsPerPacket value="{nsub}"/>
    <totalComplexSubbands value="512"/>
    <clock value="200"/>
    <integrateTimeBins value="4"/>
    <outputChannelsPerSubband value="{nchan}"/>
    <topSubbandIndex value="180.5"/>
    <dataBits value="{bits}"/>
    <scale min="10.0" max="210.0"/>
    <params nPolsToWrite="{npw}"/>
    <RAJ value="053432.0"/>
    <DecJ value="220052.0"/>
  </SigprocStokesWriter>
</configuration>
"""


@pytest.mark.gpu
@pytest.mark.parametrize("bits", [8, 32])
def test_shim_sigproc_file_equals_the_oracle(pv, oracle, cuda, shim_exe, tmp_path, bits):
    from test_outputs import _stokes
    rng = np.random.default_rng(bits)
    nt, nsub, npol, nchan, npw = 64, 31, 4, 16, 2
    x = _stokes(rng, nt, nsub, npol, nchan)
    x.tofile(tmp_path / "stokes.bin")
    t0 = 1.31e9 + 0.5
    (tmp_path / "shape.txt").write_text("%d %d %d %d %r\n" % (nt, nsub, npol, nchan, t0))
    (tmp_path / "config.xml").write_text(SIGPROC_XML.format(path=str(tmp_path / "fb"), nsub=nsub, nchan=nchan,
                                                            bits=bits, npw=npw))
    out = _run(shim_exe, "sigproc", tmp_path)
    assert "NCHANS %d" % (nsub * nchan) in out
    files = list(tmp_path.glob("fb_D*.fil"))
    assert len(files) == 1
    opts = {"subbandsPerPacket": nsub, "totalComplexSubbands": 512, "clock": 200, "integrateTimeBins": 4,
            "outputChannelsPerSubband": nchan, "topSubbandIndex": 180.5, "dataBits": bits, "nPolsToWrite": npw,
            "RAJ": "053432.0", "DecJ": "220052.0"}
    head = oracle.sigproc_header(oracle.sigproc_params(opts), (t0 - 1293840000.0) / 86400 + 55562.0)
    half = nt // 2
    data = b"".join(oracle.sigproc_pack(x[k * half:(k + 1) * half], npw, bits, 10.0, 210.0).tobytes()
                    for k in range(2))
    assert files[0].read_bytes() == head + data


PIPELINE_XML = """<configuration>
  <AdapterTimeSeriesDataSet>
    <fixedSizePackets value="true"/>
    <dataBitSize value="16"/>
    <udpPacketsPerIteration value="{npk}"/>
    <samplesPerPacket value="16"/>
    <outputChannelsPerSubband value="{nchan}"/>
    <subbandsPerPacket value="{nsub}"/>
    <nRawPolarisations value="2"/>
  </AdapterTimeSeriesDataSet>
  <DedispersionPipeline>
    <history value="{history}"/>
    <events min="{emin}" max="{emax}"/>
    <fused value="{fused}"/>
  </DedispersionPipeline>
  <PPFChanneliser>
    <outputChannelsPerSubband value="{nchan}"/>
    <filter nTaps="8" filterWindow="kaiser"/>
  </PPFChanneliser>
  <StokesGenerator><numberOfStokes value="1"/></StokesGenerator>
  <RFI_Clipper active="true" channelRejectionRMS="5.0" spectrumRejectionRMS="4.0">
    <BandPassData file="band.bp"/>
    <Band matching="true"/>
    <History maximum="{rfi_history}"/>
    <zeroDMing active="true"/>
  </RFI_Clipper>
  <DedispersionModule>
    <timeBinsPerBufferPow2 value="{pow2}"/>
    <dedispersionSamples value="{tdms}"/>
    <dedispersionStepSize value="{dm_step}"/>
    <dedispersionMinimum value="0"/>
    <frequencyChannel1 MHz="{fch1}"/>
    <channelBandwidth MHz="{foff}"/>
  </DedispersionModule>
  <DedispersionAnalyser>
    <detectionThreshold in_sigma="{thr}"/>
    <power2ForBinning value="4"/>
  </DedispersionAnalyser>
  <DedispersionDataAnalysisOutput>
    <file name="{path}"/>
  </DedispersionDataAnalysisOutput>
</configuration>
"""


@pytest.mark.gpu
@pytest.mark.parametrize("emin,emax", [(1, 0), (10 ** 6, 10 ** 7)])
def test_shim_pipeline_from_packets_to_event_file(pv, oracle, cuda, shim_exe, tmp_path, emin, emax):
    """Station packets -> AdapterTimeSeriesDataSet -> DedispersionPipeline
    (PPF, Stokes, RFI_Clipper, DedispersionModule, analyser; no integrator)
    -> DedispersionDataAnalysisOutput, against the same chain composed
    through the Python binding; a window of [min, max] events that no buffer
    reaches writes no lines."""
    import torch
    from test_udp import make_chunk
    nsub, nchan, npk, nchunks, tdms, dm_step, thr = 8, 16, 2048, 4, 48, 0.5, 4.0
    rng = np.random.default_rng(17)
    chunks, ts0 = [], 1300000000
    for k in range(nchunks):
        c, _ = make_chunk(rng, npk, nsub, 16, 2, 16, True, ts0=ts0, seq0=1000 + k * npk * 16)
        chunks.append(c)
    np.concatenate(chunks).tofile(tmp_path / "chunks.bin")
    foff = -0.1953125 / nchan
    fch1 = 150.0
    ad = pv.UdpAdapter(True, 16, npk, 16, nchan, nsub, 2)
    ppf = pv.PPF(nchan, 8, window="kaiser")
    st = []
    for c in chunks:
        ts = ad.deserialise(torch.from_numpy(c).to(cuda))
        st.append(pv.stokes(ppf.run(ts.reshape(nsub, 2, -1)), 1))
    fb0 = st[0].cpu().numpy()
    (tmp_path / "band.bp").write_text(make_bp_text(nsub * nchan, fch1 + foff * (nsub * nchan - 1), -foff,
                                                   float(fb0.mean()), float(fb0.std())))
    (tmp_path / "config.xml").write_text(PIPELINE_XML.format(
        npk=npk, nchan=nchan, nsub=nsub, emin=emin, emax=emax, tdms=tdms, dm_step=dm_step, fch1=repr(fch1),
        foff=repr(foff), thr=thr, path=str(tmp_path / "ev"), history=10, fused="true", rfi_history=1000,
        pow2=12))
    out = _run(shim_exe, "pipeline", tmp_path, nchunks)
    assert "FUSED 1" in out
    nbuf = int(out.split("BUFFERS")[1].split()[0])
    # the same chain through the binding
    rfi = pv.RFI((tmp_path / "band.bp").read_text(), cr=5.0, sr=4.0, history=1000, zero_dming=True)
    dd = pv.DedispersionModule(1 << 12, tdms, 0.0, dm_step, fch1, foff)
    tsamp = ad.block_rate * nchan  # the adapter's 1/195313 s (even second) times the PPF length
    rms = float(np.sqrt(np.float32(nchan) * np.float32(nsub)))
    text, dump = "", 0
    t_start = ts0 + 1000 / 195313
    for x in st:
        rfi.run(x)
        for buf, first in dd.add(x.cpu().numpy(), tsamp):
            ev, n = pv.analyse(torch.from_numpy(buf).to(cuda), thr, rms, 4)
            assert n == len(ev)
            if (n >= emin) if emin >= emax else (emin <= n <= emax):
                dump += 1
                text += pv.events_text(ev, t_start, tsamp, first, 0.0, dm_step, np.float32(rms), dump)
    assert nbuf >= 2
    files = list(tmp_path.glob("ev_D*.dat"))
    assert len(files) == 1
    assert files[0].read_text() == pv.EVENTS_TEXT_HEADER + text
    if emin > 1000:
        assert text == ""  # no buffer has a million events


@pytest.mark.gpu
def test_shim_pipeline_plain_single_beam_full_size(pv, oracle, cuda, shim_exe, tmp_path):
    """The plain single-beam workload through the reference's pipeline
    structure (DedispersionPipeline has no integrator): 32 subbands from
    140 MHz in 16-bit station packets, 65536 samples per subband per chunk,
    16 channels per subband (81.92 us), RFI_Clipper at 5 sigma with a
    10000-spectrum history, 512 trials over DM 0-100 in buffers of 2^15
    spectra, events at 6 sigma; the DM 56.8 pulse 0.5 s into the stream.
    The fused device chain and the module chain write the same event file,
    which equals the chain composed through the Python binding, and the
    strongest event is the pulse."""
    import torch
    from gen import lofar_band, lofar_packets, lofar_stream
    nsub, nchan, per_chunk, nchunks, tdms, thr = 32, 16, 65536, 9, 512, 6.0
    dm_step = np.float32(100.0 / 511)
    fch1, foff = lofar_band(140.0, nsub, nchan)
    rng = np.random.default_rng(56)
    v = lofar_stream(rng, nsub, per_chunk * nchunks, 140.0, nchan, pulses=[(56.8, 0.5, 1e-3, 0.52)])
    npk = per_chunk // 16
    chunks = [lofar_packets(np.ascontiguousarray(v[:, :, k * per_chunk:(k + 1) * per_chunk]), seq0=1000 + k * per_chunk)
              for k in range(nchunks)]
    np.concatenate(chunks).tofile(tmp_path / "chunks.bin")
    ad = pv.UdpAdapter(True, 16, npk, 16, nchan, nsub, 2)
    ppf = pv.PPF(nchan, 8, window="kaiser")
    st = []
    for c in chunks:
        ts = ad.deserialise(torch.from_numpy(c).to(cuda))
        st.append(pv.stokes(ppf.run(ts.reshape(nsub, 2, -1)), 1))
    fb0 = st[0].cpu().numpy()
    (tmp_path / "band.bp").write_text(make_bp_text(nsub * nchan, fch1, foff, float(fb0.mean()),
                                                   float(fb0.std())))
    texts = {}
    for fused in ("true", "false"):
        d = tmp_path / fused
        d.mkdir()
        (d / "band.bp").write_text((tmp_path / "band.bp").read_text())
        os.symlink(tmp_path / "chunks.bin", d / "chunks.bin")
        (d / "config.xml").write_text(PIPELINE_XML.format(
            npk=npk, nchan=nchan, nsub=nsub, emin=1, emax=0, tdms=tdms, dm_step=repr(float(dm_step)),
            fch1=repr(fch1), foff=repr(foff), thr=thr, path=str(d / "ev"), history=32, fused=fused,
            rfi_history=10000, pow2=15))
        out = _run(shim_exe, "pipeline", d, nchunks)
        assert ("FUSED 1" in out) == (fused == "true")
        assert int(out.split("BUFFERS")[1].split()[0]) == 1
        files = list(d.glob("ev_D*.dat"))
        assert len(files) == 1
        texts[fused] = files[0].read_text()
    assert texts["true"] == texts["false"]
    # the same chain through the binding
    rfi = pv.RFI((tmp_path / "band.bp").read_text(), cr=5.0, sr=4.0, history=10000, zero_dming=True)
    dd = pv.DedispersionModule(1 << 15, tdms, 0.0, float(dm_step), fch1, foff)
    tsamp = ad.block_rate * nchan
    rms = float(np.sqrt(np.float32(nchan) * np.float32(nsub)))
    t_start = 1300000000 + 1000 / 195313
    text, dump, best = "", 0, None
    for x in st:
        rfi.run(x)
        for buf, first in dd.add(x.cpu().numpy(), tsamp):
            ev, n = pv.analyse(torch.from_numpy(buf).to(cuda), thr, rms, 4)
            dump += 1
            text += pv.events_text(ev, t_start, tsamp, first, 0.0, float(dm_step), np.float32(rms), dump)
            snr = ev["value"][1:] / (rms * np.sqrt(ev["bin_factor"][1:]))
            k = int(np.argmax(snr)) + 1
            best = (float(snr[k - 1]), int(ev["dm"][k]), first + int(ev["t"][k]))
    assert texts["true"] == pv.EVENTS_TEXT_HEADER + text
    snr, d_best, t_best = best
    assert abs(d_best - 56.8 / float(dm_step)) <= 2 and abs(t_best - 0.5 / tsamp) <= 32 and snr >= 10, best
