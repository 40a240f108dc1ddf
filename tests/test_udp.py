"""LOFAR UDP ingest (AdapterTimeSeriesDataSet): the oracle against an
independent numpy reading of the packet layout and the reference test's
sizes (AdapterTimeSeriesDataSetTest.cpp); the library's checks and messages
on the CPU; the GPU unpack bit for bit against the oracle."""
import numpy as np
import pytest

HEADER = 16
FIXED = 8148  # sizeof(UDPPacket): 16-byte header + 8130 bytes, 4-byte aligned


def make_chunk(rng, npk, nsub, spp, npol, bits, fixed, ts0=1234567890, seq0=1000):
    """npk packets with counting headers and random complex samples; returns
    (chunk bytes as uint8, samples [k][s][t][p][2])."""
    dt = np.int16 if bits == 16 else np.int8
    lim = 32767 if bits == 16 else 127
    data = rng.integers(-lim - 1, lim + 1, size=(npk, nsub, spp, npol, 2)).astype(dt)
    useful = data[0].nbytes
    psize = FIXED if fixed else HEADER + useful
    chunk = np.zeros((npk, psize), np.uint8)
    hdr = np.zeros(npk, dtype=[("version", "u1"), ("source", "u1"), ("config", "<u2"), ("station", "<u2"),
                               ("beamlets", "u1"), ("blocks", "u1"), ("ts", "<u4"), ("seq", "<u4")])
    hdr["version"] = 3
    hdr["config"] = bits
    hdr["beamlets"] = nsub
    hdr["blocks"] = spp
    hdr["ts"] = ts0
    hdr["seq"] = seq0 + spp * np.arange(npk)
    chunk[:, :HEADER] = hdr.view(np.uint8).reshape(npk, HEADER)
    chunk[:, HEADER:HEADER + useful] = data.reshape(npk, -1).view(np.uint8)
    if fixed:
        chunk[:, HEADER + useful:] = 0xAB  # padding the adapter skips
    return chunk.reshape(-1), data


def numpy_unpack(data):
    """[k][s][t][p][2] -> complex [s][p][k*spp + t]."""
    npk, nsub, spp, npol, _ = data.shape
    z = data[..., 0].astype(np.float32) + 1j * data[..., 1].astype(np.float32)
    return np.ascontiguousarray(z.transpose(1, 3, 0, 2).reshape(nsub, npol, npk * spp)).astype(np.complex64)


def test_reference_test_sizes(oracle):
    """AdapterTimeSeriesDataSetTest::test_checkDataFixedPacket / VariablePacket."""
    npk, spp, nchan, nsub, npol = 16384, 16, 16, 61, 2
    rc, psize, nblocks = oracle.udp_check(1, 16, npk, spp, nchan, nsub, npol, FIXED * npk)
    assert (rc, psize, nblocks) == (0, FIXED, npk * spp // nchan)
    assert nblocks * npol * nsub == 16384 * 2 * 61  # nTimeSeries
    var = HEADER + nsub * npol * spp * 16 * 2 // 8
    rc, psize, nblocks = oracle.udp_check(0, 16, npk, spp, nchan, nsub, npol, var * npk)
    assert (rc, psize, nblocks) == (0, var, 16384)


def test_oracle_checks_fail_in_the_reference_order(oracle):
    assert oracle.udp_check(1, 12, 4, 16, 16, 61, 2, FIXED * 4)[0] == 1
    assert oracle.udp_check(1, 16, 4, 16, 16, 61, 2, FIXED * 4 + 1)[0] == 2
    assert oracle.udp_check(1, 16, 4, 16, 16, 64, 2, FIXED * 4)[0] == 3  # 8192 > 8130 bytes
    assert oracle.udp_check(1, 16, 3, 16, 32, 61, 2, FIXED * 3)[0] == 4


@pytest.mark.parametrize("bits,fixed,npol", [(16, True, 2), (16, False, 2), (8, True, 2), (8, False, 1)])
def test_oracle_unpack_equals_numpy(oracle, bits, fixed, npol):
    rng = np.random.default_rng(bits + npol)
    nsub = 61 if bits == 16 else 122
    chunk, data = make_chunk(rng, 8, nsub, 16, npol, bits, fixed)
    rc, psize, _ = oracle.udp_check(int(fixed), bits, 8, 16, 16, nsub, npol, chunk.size)
    assert rc == 0
    got = oracle.udp_unpack(chunk, psize, 8, bits, nsub, npol, 16)
    assert np.array_equal(got, numpy_unpack(data))


def test_oracle_time_stamp(oracle):
    h = np.zeros(16, np.uint8)
    h[8:12] = np.frombuffer(np.uint32(100).tobytes(), np.uint8)
    h[12:16] = np.frombuffer(np.uint32(97656).tobytes(), np.uint8)
    ts, rate = oracle.udp_time(h, 200)
    assert rate == 1.0 / 195313 and ts == 100 + 97656 / 195313
    h[8] = 101
    assert oracle.udp_time(h, 200) == (101 + 97656 / 195312, 1.0 / 195312)
    assert oracle.udp_time(h, 160)[1] == 1.0 / 156250


def test_library_checks_and_messages(pv):
    """pv_udp_check is host code: the reference's messages, no GPU needed."""
    a = pv.UdpAdapter(True, 16, 16384, 16, 16, 61, 2)
    assert a.check(FIXED * 16384) == (FIXED, 16384)
    with pytest.raises(pv.PvError, match="Chunk size '10' != '133496832' expected for 16384 UDP packets."):
        a.check(10)
    with pytest.raises(pv.PvError, match=r"Sample size \(12 bits\) not supported."):
        pv.UdpAdapter(True, 12, 4, 16, 16, 61, 2).check(FIXED * 4)
    with pytest.raises(pv.PvError, match="Dimensions decribe more data than fits into a UDP packet"):
        pv.UdpAdapter(True, 16, 4, 16, 16, 64, 2).check(FIXED * 4)
    with pytest.raises(pv.PvError, match="evenly divisible"):
        pv.UdpAdapter(True, 16, 3, 16, 32, 61, 2).check(FIXED * 3)
    with pytest.raises(pv.PvError, match="two polarisations"):
        pv.UdpAdapter(True, 16, 4, 16, 16, 61, 1).check(FIXED * 4)


@pytest.mark.gpu
@pytest.mark.parametrize("bits,fixed,npol,out", [(16, True, 2, "c32"), (16, False, 2, "i16"),
                                                 (8, True, 2, "c32"), (8, False, 1, "c32"),
                                                 (8, True, 2, "i16")])
def test_gpu_unpack_equals_oracle(pv, oracle, cuda, bits, fixed, npol, out):
    import torch
    rng = np.random.default_rng(7 * bits + npol)
    npk, nsub, spp, nchan = 203, (61 if bits == 16 else 122), 16, 16  # ragged last CTA of packets
    chunk, data = make_chunk(rng, npk, nsub, spp, npol, bits, fixed)
    a = pv.UdpAdapter(fixed, bits, npk, spp, nchan, nsub, npol)
    psize, nblocks = a.check(chunk.size)
    want = oracle.udp_unpack(chunk, psize, npk, bits, nsub, npol, spp)
    got = a.deserialise(torch.from_numpy(chunk).to(cuda), out=out)
    torch.cuda.synchronize()
    if out == "c32":
        assert tuple(got.shape) == (nsub, npol, nblocks, nchan)
        assert np.array_equal(got.cpu().numpy().reshape(nsub, npol, -1), want)
    else:
        g = got.cpu().numpy()
        assert np.array_equal(g[..., 0].astype(np.float32), want.real)
        assert np.array_equal(g[..., 1].astype(np.float32), want.imag)
    assert a.timestamp == 1234567890 + 1000 / 195313 and a.block_rate == 1.0 / 195313


@pytest.mark.gpu
def test_gpu_unpacked_packets_feed_the_beam_chain(pv, cuda):
    """Station packets -> int16 voltages -> pv_beam: the same filterbank as the
    voltages given directly."""
    import torch
    from test_gpu_batch import beam_kw
    rng = np.random.default_rng(3)
    nsub, nch, chunk_len = 6, 16, 512
    npk = chunk_len * 4 * nch // 16
    chunk, data = make_chunk(rng, npk, nsub, 16, 2, 16, True)
    a = pv.UdpAdapter(True, 16, npk, 16, nch, nsub, 2)
    v = a.deserialise(torch.from_numpy(chunk).to(cuda), out="i16")
    direct = torch.from_numpy(np.ascontiguousarray(data.transpose(1, 3, 0, 2, 4).reshape(nsub, 2, -1, 2))).to(cuda)
    cfg = pv.beam_config(**dict(beam_kw(nsub, nch, 16, 1.0, chunk=chunk_len), rfi_active=0, bp_text=None))
    outs = []
    for x in (v, direct):
        b = pv.Beam(cfg)
        b.process(x.reshape(nsub, 2, -1))
        torch.cuda.synchronize()
        outs.append(pv.device_array(b.buffers()[0], (chunk_len, nsub * nch)).cpu().numpy())
    assert np.array_equal(outs[0], outs[1])


def _beam_packets(rng, nsub, per_packet, npk, fixed):
    """One chunk of a beam as packet streams (nsub / per_packet of them, one after another) and the
    same samples as int16 voltages [sub][pol][t][2]."""
    chunks, volts = [], []
    for _ in range(nsub // per_packet):
        c, data = make_chunk(rng, npk, per_packet, 16, 2, 16, fixed)
        chunks.append(c)
        volts.append(data.transpose(1, 3, 0, 2, 4).reshape(per_packet, 2, npk * 16, 2))
    return np.concatenate(chunks), np.ascontiguousarray(np.concatenate(volts))


@pytest.mark.gpu
@pytest.mark.parametrize("nch,fixed", [(16, True), (32, False), (64, True)])
def test_gpu_packet_fed_beam_equals_voltage_fed_beam(pv, cuda, nch, fixed):
    """The channeliser reads the packets in place: filterbank, dedispersed window and events
    equal those of the same beam given the unpacked voltages, chunk after chunk."""
    import torch
    from test_gpu_batch import beam_kw
    rng = np.random.default_rng(nch)
    nsub, per_packet, chunk = 6, 3, 256
    npk = chunk * 4 * nch // 16
    psize = FIXED if fixed else HEADER + per_packet * 16 * 2 * 4
    kw = dict(beam_kw(nsub, nch, 24, 1.0, chunk=chunk), rfi_active=0, bp_text=None, prefilled=1)
    b_pkt = pv.Beam(pv.beam_config(**dict(kw, udp_packet_bytes=psize, udp_subbands=per_packet)))
    b_vol = pv.Beam(pv.beam_config(**kw))
    assert b_pkt.input_bytes() == (nsub // per_packet) * npk * psize
    for _ in range(3):
        pk, v = _beam_packets(rng, nsub, per_packet, npk, fixed)
        b_pkt.process(torch.from_numpy(pk).to(cuda))
        b_vol.process(torch.from_numpy(v.reshape(nsub, 2, -1)).to(cuda))
        torch.cuda.synchronize()
        fa, _, oa, _ = b_pkt.buffers()
        fb, _, ob, _ = b_vol.buffers()
        nbins = nsub * nch
        assert np.array_equal(pv.device_array(fa, (chunk, nbins)).cpu().numpy(),
                              pv.device_array(fb, (chunk, nbins)).cpu().numpy())
        ea, na, firsta = b_pkt.events()
        eb, nb, firstb = b_vol.events()
        assert (na, firsta) == (nb, firstb) and np.array_equal(ea, eb)
        assert np.array_equal(pv.device_array(oa, (24, chunk)).cpu().numpy(),
                              pv.device_array(ob, (24, chunk)).cpu().numpy())


@pytest.mark.gpu
def test_gpu_batch_with_packet_fed_beam_equals_beams_alone(pv, cuda):
    import torch
    from test_gpu_batch import beam_kw
    rng = np.random.default_rng(31)
    chunk = 256
    kw_a = dict(beam_kw(4, 16, 24, 1.0, chunk=chunk), rfi_active=0, bp_text=None, prefilled=1,
                udp_packet_bytes=FIXED, udp_subbands=2)
    kw_b = dict(beam_kw(3, 32, 16, 0.7, chunk=chunk), rfi_active=0, bp_text=None, prefilled=1)
    cfgs = [pv.beam_config(**kw_a), pv.beam_config(**kw_b)]
    batch = pv.Batch(cfgs, tune=False, graph=True, pipelined=True)
    alone = [pv.Beam(c) for c in cfgs]
    hist = []
    for step in range(4):
        pk, _ = _beam_packets(rng, 4, 2, chunk * 4 * 16 // 16, True)
        v = rng.normal(0.0, 16.0, (3, 2, chunk * 4 * 32 * 2))
        ins = [torch.from_numpy(pk).to(cuda), torch.from_numpy(np.rint(v).astype(np.int16)).to(cuda)]
        rec = []
        for i, x in enumerate(ins):
            batch.set_input(i, x)
            alone[i].process(x)
        batch.run()
        torch.cuda.synchronize()
        for i, b in enumerate(alone):
            rec.append(b.events())
        hist.append(rec)
        if step >= 1:  # pipelined: a window's events come one step later
            for i in range(2):
                ev, n, first = batch.events(i)
                ea, na, firsta = hist[step - 1][i]
                assert (n, first) == (na, firsta) and np.array_equal(ev, ea)
