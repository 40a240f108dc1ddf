"""DedispersionModule with the reference's buffering (pv_ddmod) against the
oracle's DedispersionModule + DedispersionBuffer restatement."""
import numpy as np
import pytest

from gen import GEN_FCH1, GEN_FOFF, GEN_NCHAN, GEN_NSUB, GEN_TSAMP, dm_index, generator_pulse

pytestmark = pytest.mark.gpu


def test_module_known_answer(pv, oracle, cuda):
    """DedispersionModuleTest::test_method: dmAmplitude(0, 10.0) == 2048."""
    blob = generator_pulse(8192, 10.0)[0]
    m = pv.DedispersionModule(8192, 200, 0.0, 0.1, GEN_FCH1, GEN_FOFF)
    outs = m.add(blob, GEN_TSAMP)
    assert len(outs) == 1
    data, first = outs[0]
    p = m.params()
    assert p["nchan"] == GEN_NSUB * GEN_NCHAN and p["inverted"] == 0
    assert data.shape == (200, 8192 - p["maxshift"] - p["remaining"])
    assert first == 0
    assert data[dm_index(10.0, 0.0, 0.1), 0] == np.float32(GEN_NSUB * GEN_NCHAN)
    o = oracle.DedispersionModule(8192, 200, 0.0, 0.1, GEN_FCH1, GEN_FOFF)
    want, wfirst = o.add(blob, GEN_TSAMP)[0]
    assert np.array_equal(data, want) and wfirst == first


@pytest.mark.parametrize("foff", [-0.05, 0.05])
def test_module_stream_of_uneven_blobs(pv, oracle, cuda, foff):
    """Blobs of uneven length cross buffer boundaries; every completed buffer
    matches the reference's buffering bit for bit (descending and ascending
    bands)."""
    rng = np.random.default_rng(17)
    nsub, nchan, npol, tdms, B = 6, 16, 2, 40, 2048
    m = pv.DedispersionModule(B, tdms, 0.0, 0.7, 150.0, foff)
    o = oracle.DedispersionModule(B, tdms, 0.0, 0.7, 150.0, foff)
    got, want = [], []
    for n in (700, 1500, 333, 2048, 4100, 17, 999):
        blob = rng.standard_normal((n, nsub, npol, nchan)).astype(np.float32)
        got += m.add(blob, 1e-3)
        want += o.add(blob, 1e-3)
    assert len(got) == len(want) >= 3
    for (g, gf), (w, wf) in zip(got, want):
        assert gf == wf and np.array_equal(g, w)


def test_module_maxshift_error(pv, cuda):
    m = pv.DedispersionModule(256, 200, 0.0, 0.1, GEN_FCH1, GEN_FOFF)
    with pytest.raises(pv.PvError, match="maxshift requirements"):
        m.add(np.zeros((10, GEN_NSUB, 1, GEN_NCHAN), np.float32), GEN_TSAMP)
