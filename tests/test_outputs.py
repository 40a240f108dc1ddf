"""Outputs after the path: the sigproc filterbank writer (header on the host,
reorder and 8-bit quantisation on the GPU) and the event text stream, each
against the oracle's restatement of the reference writer."""
import numpy as np
import pytest


def _events(rng, n, tdms=200):
    from pv import EVENT_DTYPE
    ev = np.zeros(n, EVENT_DTYPE)
    ev[0] = (0, 0, 1.0, 0.0)  # the analyser's first event carries the time stamp
    ev["dm"][1:] = rng.integers(0, tdms, n - 1)
    ev["t"][1:] = rng.integers(0, 8192, n - 1)
    ev["bin_factor"][1:] = 2.0 ** rng.integers(0, 7, n - 1)
    ev["value"][1:] = rng.uniform(100, 5000, n - 1).astype(np.float32)
    return ev


@pytest.mark.parametrize("n", [1, 2, 50])
def test_event_text_equals_the_oracle(pv, oracle, n):
    rng = np.random.default_rng(n)
    ev = _events(rng, n)
    args = (1.3e9 + 0.123456789, 327.68e-6, 16384, float(np.float32(0.0)), float(np.float32(0.1)),
            np.float32(45.254834), 3)
    got = pv.events_text(ev, *args)
    assert got == oracle.events_text(ev, *args)
    lines = got.splitlines()
    assert len(lines) == n  # n-1 events and the buffer summary
    assert lines[-1].startswith("# Written buffer :3 | MJDstart: ") and lines[-1].endswith("  Done")
    if n > 1:
        mjd, dm, snr, bf = lines[0].split(",")
        assert lines[0].split(",")[1].startswith("   ")
        assert int(bf) == int(ev["bin_factor"][1])
        assert abs(float(mjd) - (args[0] + (ev["t"][1] + 16384) * args[1]) / 86400) < 1e-9
    assert pv.EVENTS_TEXT_HEADER == oracle.EVENTS_TEXT_HEADER


@pytest.mark.parametrize("n,min_events,snr", [(1, 0, 0.0), (2, 2, 5.0), (50, 10, 20.0), (50, 51, 5.0),
                                             (50, 0, 1e6), (3, 0, 0.0)])
def test_trigger_message_equals_the_oracle(pv, oracle, n, min_events, snr):
    rng = np.random.default_rng(100 + n)
    ev = _events(rng, n)
    if n == 3:
        ev["value"][1:] = ev["value"][1]  # equal SNRs: the first is kept
        ev["bin_factor"][1:] = 1.0
    args = (1.3e9 + 0.123456789, 327.68e-6, 16384, float(np.float32(0.0)), float(np.float32(0.1)),
            np.float32(45.254834), min_events, snr, "CS302", "202612031200-07", 12, "150.0", "", "-22.014")
    got = pv.trigger_message(ev, *args)
    assert got == oracle.trigger_message(ev, *args)
    raises = n > 1 and n >= min_events and snr < 1e6
    assert (got is not None) == raises
    if raises:
        f = dict(kv.split(":", 1) for kv in got.split("##"))
        assert f["artemis"] == "CS302" and f["ID"] == "202612031200-070012"
        assert f["cFreqMHz"] == "00000150.0" and f["beamRA"] == "0000000000" and f["beamDec"] == "00-22.014"
        assert len(f["eTime"]) == 20 and len(f["eDM"]) == 9 and len(f["eSNR"]) == 6
        snr_all = ev["value"][1:] / (np.float32(45.254834) * np.sqrt(ev["bin_factor"][1:]))
        i = 1 + int(np.argmax(snr_all))
        assert float(f["eDM"]) == pytest.approx(0.1 * int(ev["dm"][i]), abs=1e-3)


def test_trigger_output_sends_one_datagram_and_log_line(pv, tmp_path):
    import socket
    rx = socket.socket(socket.AF_INET, socket.SOCK_DGRAM)
    rx.bind(("127.0.0.1", 0))
    rx.settimeout(5.0)
    out = pv.TriggerOutput(station="CS302", beamID="7", rajd="83.6", decjd="22.0", cfreq_mhz="150", snr=5.0,
                           events=2, receiver=("127.0.0.1", rx.getsockname()[1]), logfile=str(tmp_path / "t.log"))
    ev = _events(np.random.default_rng(5), 20)
    args = (1.3e9, 327.68e-6, 0, 0.0, 0.1, 45.254834)
    first = out.send_stream(ev, *args)
    second = out.send_stream(ev, *args)
    assert out.send_stream(ev[:1], *args) is None  # fewer events than the threshold count
    out.close()
    assert first.split("##")[1].endswith("0001") and second.split("##")[1].endswith("0002")
    assert first.split("##")[1][3:] == out.id_root + "0001"
    assert rx.recv(4096).decode() == first and rx.recv(4096).decode() == second
    assert (tmp_path / "t.log").read_text() == first + "\n" + second + "\n"
    rx.close()


OPTIONS = [
    {},  # every default
    {"subbandsPerPacket": 31, "totalComplexSubbands": 512, "clock": 200, "integrateTimeBins": 4,
     "outputChannelsPerSubband": 16, "nRawPolarisations": 2, "topSubbandIndex": 180.7, "dataBits": 8,
     "RAJ": "053432.0", "DecJ": "220052.0", "nPolsToWrite": 1},
    {"clock": 160, "totalComplexSubbands": 512, "outputChannelsPerSubband": 64, "integrateFrequencyChannels": 4,
     "LBA_0_or_HBA_1": 1, "DecJ": "-123000.5", "MachineID": 10, "TelescopeID": 11},
    {"LBA_0_or_HBA_1": 0, "totalComplexSubbands": 512, "topSubbandIndex": 300},
    {"fch1": 150.5, "foff": -0.01, "tsamp": 0.000327, "subbandsPerPacket": 61},
]


@pytest.mark.parametrize("opts", OPTIONS)
def test_sigproc_header_equals_the_oracle(pv, oracle, opts):
    p = oracle.sigproc_params(opts)
    tstart = pv.sigproc_mjd(1.3e9)
    assert pv.sigproc_header(p, tstart) == oracle.sigproc_header(p, tstart)
    assert pv.sigproc_mjd(1293840000.0) == 55562.0
    assert tstart == (1.3e9 - 1293840000.0) / 86400 + 55562.0


def _stokes(rng, nt, nsub, npol, nchan):
    x = rng.normal(120.0, 60.0, (nt, nsub, npol, nchan)).astype(np.float32)
    flat = x.reshape(-1)
    flat[::97] = np.float32(2.5)     # a rounding tie: rint to even
    flat[1::89] = np.float32(3.5)
    flat[5::211] = np.nan
    flat[7::223] = np.inf
    flat[9::227] = -np.inf
    flat[11::229] = -7.0             # below the crop minimum
    flat[13::233] = 1e6              # above the crop maximum
    return x


@pytest.mark.gpu
@pytest.mark.parametrize("nbits,npol,npw,crop,nchan", [(8, 1, 1, (0.0, 255.0), 16), (8, 4, 2, (10.0, 210.0), 16),
                                                        (32, 4, 4, (0.0, 255.0), 16), (32, 1, 1, (0.0, 255.0), 16),
                                                        (8, 2, 1, (0.0, 255.0), 6), (32, 1, 1, (0.0, 255.0), 6)])
def test_gpu_sigproc_pack_equals_the_oracle(pv, oracle, cuda, nbits, npol, npw, crop, nchan):
    """Four outputs per thread when nchan % 4 == 0, one otherwise."""
    import torch
    rng = np.random.default_rng(nbits + npol + nchan)
    x = _stokes(rng, 37, 31, npol, nchan)
    got = pv.sigproc_pack(torch.from_numpy(x).to(cuda), npw, nbits, *crop).cpu().numpy()
    want = oracle.sigproc_pack(x, npw, nbits, *crop)
    assert got.size == want.size and np.array_equal(got, want)
    if nbits == 32:  # the floats themselves, channels and subbands descending
        first = got[: 4 * nchan].view(np.float32)
        assert np.array_equal(first, x[0, -1, 0, ::-1], equal_nan=True)


@pytest.mark.gpu
def test_gpu_sigproc_pack_rejects_other_bit_widths(pv, cuda):
    import torch
    with pytest.raises(pv.PvError, match="16 bit datafiles not yet supported"):
        pv.sigproc_pack(torch.zeros((2, 1, 1, 4), device=cuda), 1, 16)
