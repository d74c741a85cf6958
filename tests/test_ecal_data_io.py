"""The ROOT-format reader and the driver mirror (CPU): the reference's data
files read without ROOT, the driver's conditions, its physics check, and the
oracle's replay fits pinned by tests/golden/replay_mysample_100.npz.

Tests that read the reference's data files skip where the reference tree is
absent; the fixture carries what they read for the GPU tests."""
import math
import os
import struct

import numpy as np
import pytest

from _helpers import reference_data_dir

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "replay_mysample_100.npz")
DATA = reference_data_dir()
SAMPLE_100 = os.path.join(DATA, "mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root")
SAMPLE_1000 = os.path.join(DATA,
                           "mysample_1000_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root")
SHAPE = os.path.join(DATA, "EmptyFile.root")
needs_data = pytest.mark.skipif(not (os.path.exists(SAMPLE_100) and os.path.exists(SHAPE)),
                                reason="the reference's data files are absent")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="module")
def eio(mf):
    import multifit_gb300.ecal_data_io as m

    return m


@pytest.fixture(scope="module")
def rootio(mf):
    import multifit_gb300.rootio as m

    return m


# -- reader on the reference's files ------------------------------------------

@needs_data
def test_reader_samples_tree_matches_file_name_and_fixture(rootio, gold):
    f = rootio.RootFile(SAMPLE_100)
    assert f.closed and [k.name for k in f.keys()] == ["Samples"]
    t = f.tree("Samples")
    assert t.entries == 100  # mysample_<nEventsTotal=100>_...
    assert {"amplitudeTruth", "samples", "nSmpl", "nFreq", "pulse_tau", "sigmaNoise"} <= set(t.branch_names())
    # the file name's parameters: 10 samples, 25 ns, 10 GeV signal, CRRC tau 43
    assert (t.array("nSmpl", np.int32) == 10).all()
    assert (t.array("nFreq", np.float32) == 25).all()
    assert (t.array("pulse_tau", np.float32) == 43).all()
    assert (t.array("signalTruth", np.float64) == 10).all()
    assert (t.array("sigmaNoise", np.float32) == np.float32(0.044)).all()
    truth = t.array("amplitudeTruth", np.float64)
    vecs = t.vectors("samples")
    assert all(v.shape == (10,) for v in vecs)
    assert np.array_equal(np.stack(vecs), gold["samples"])
    assert np.array_equal(truth, gold["truth"])
    # every sample vector holds a pulse near the in-time sample
    assert (np.stack(vecs).argmax(axis=1) >= 4).all()


@needs_data
def test_reader_pulse_shape_file(rootio, eio, gold):
    f = rootio.RootFile(SHAPE)
    assert [k.name for k in f.keys()] == ["PulseShape", "PileupPDFs"]
    assert [k.name for k in f.keys("PulseShape")] == ["grPulseShape", "Tail"]
    x, y, bits = f.graph("PulseShape/grPulseShape")
    assert x.shape == (1000,) and np.array_equal(x, np.arange(1000.0))
    assert 0.99 < y.max() <= 1.0
    p = eio.Pulse(SHAPE)
    assert p.sorted_x == bool(gold["graph_sorted"]) and len(p.gx) == int(gold["graph_points"])
    assert np.array_equal([p.tmin, p.par0, p.par1], gold["tail"])
    assert p.tmin == 800.0  # the tail starts where fShape switches to it
    tpl = eio.driver_template(p)
    assert np.array_equal(tpl, gold["template"])
    assert tpl.argmax() == 2  # "intime sample is [2]"
    # the template's abscissae 13 + 25 i fall on graph points: exact values
    assert np.array_equal(tpl, y[13 + 25 * np.arange(12)])
    assert np.array_equal(eio.driver_fullpulse(p), gold["fullpulse"])


@needs_data
def test_reader_unclosed_file_raises(rootio):
    if not os.path.exists(SAMPLE_1000):
        pytest.skip("file absent")
    f = rootio.RootFile(SAMPLE_1000)
    # written without TFile::Close: the header still says fEND = 378, and the
    # tree record and keys list were never written
    assert not f.closed and f.end < len(f.data)
    with pytest.raises(rootio.RootFormatError, match="not closed"):
        f.tree("Samples")
    names = {k.name for k in f.walk() if k.class_name == "TBasket"}
    assert "samples" in names and "amplitudeTruth" not in names


@needs_data
def test_reader_rejects_unsupported_compression_and_truncation(rootio):
    data = bytearray(open(SAMPLE_100, "rb").read())
    f = rootio.RootFile(bytes(data))
    bk = [k for k in f.walk() if k.class_name == "TBasket" and k.name == "samples"][0]
    p = bk.seek_key + bk.keylen
    assert bytes(data[p:p + 2]) == b"ZL"
    data[p:p + 2] = b"L4"
    with pytest.raises(rootio.RootFormatError, match="compression"):
        rootio.RootFile(bytes(data)).tree("Samples").vectors("samples")
    cut = open(SAMPLE_100, "rb").read()[: bk.seek_key + 100]
    with pytest.raises(rootio.RootFormatError):
        rootio.RootFile(cut).tree("Samples")


@needs_data
def test_ecal_data_io_round_robin(eio, mf, gold):
    io = eio.ecal_data_io(SAMPLE_100, SHAPE, mf)
    ents = io.get_n_entries(250)
    assert len(ents) == 250
    for i in (0, 37, 99, 100, 249):
        s, P = ents[i]
        assert np.array_equal(s, gold["samples"][i % 100])
        assert np.array_equal(P, gold["P"])


def test_reader_rejects_non_root_bytes(rootio):
    with pytest.raises(rootio.RootFormatError, match="not a ROOT file"):
        rootio.RootFile(b"\x00" * 128)
    hdr = b"root" + struct.pack(">iii", 61103, 10 ** 6, 10 ** 6) + b"\x00" * 100
    with pytest.raises(rootio.RootFormatError, match="fBEGIN"):
        rootio.RootFile(hdr)


# -- driver conditions and physics check ---------------------------------------

def test_driver_noise_correlation_formula(gold):
    # Pulse::NoiseInit: mC_k = 1 - (1 - exp(-25 k / (sqrt(2) * 43)))^2
    R = gold["noisecor"]
    for i in range(10):
        for j in range(10):
            y = 1.0 - math.exp(-float(25 * abs(i - j)) / (math.sqrt(2.0) * 43.0))
            assert R[i, j] == 1.0 - y * y


def test_driver_pulse_matrix_is_the_io_rule(mf, gold):
    # io/src/ecal_data_io.cpp:27-41: column ip (bx) holds pulse_extended from
    # first_sample_t = max(0, bx+3) on, at offset 7 - 3 - bx
    fp = gold["fullpulse"]
    P = np.zeros((10, 10))
    for ip, bx in enumerate(range(-5, 5)):
        first = max(0, bx + 3)
        off = 7 - 3 - bx
        P[first:, ip] = fp[first + off:10 + off]
    assert np.array_equal(P, gold["P"])
    assert np.array_equal(mf.build_pulse_matrix(fp, gold["bxs"], 10), P)


def test_graph_eval_linear_rule(eio):
    x = np.array([0.0, 1.0, 2.0, 4.0])
    y = np.array([0.0, 0.3, 0.7, 0.1])
    for s in (False, True):
        assert eio.graph_eval(x, y, 3.0, s) == pytest.approx(0.4, abs=1e-15)
        assert eio.graph_eval(x, y, 0.5, s) == pytest.approx(0.15, abs=1e-15)
        assert eio.graph_eval(x, y, 5.0, s) == pytest.approx(-0.2, abs=1e-15)   # beyond: last two points
        assert eio.graph_eval(x, y, -1.0, s) == pytest.approx(-0.3, abs=1e-15)  # before: first two points
    # an unsorted graph returns the point's own value on an abscissa
    assert eio.graph_eval(x, y, 2.0, False) == 0.7
    xs = np.array([2.0, 0.0, 4.0, 1.0])
    ys = np.array([0.7, 0.0, 0.1, 0.3])
    assert eio.graph_eval(xs, ys, 3.0, False) == pytest.approx(0.4, abs=1e-15)


def test_h01_summary_as_the_histogram_reports(eio):
    d = np.array([0.5, -0.25, 1.0, 7.0, -5.0, 5.0])
    h = eio.h01_summary(d)
    inr = np.array([0.5, -0.25, 1.0, -5.0])  # 7 and 5 are overflow, -5 is the first bin
    assert h["entries"] == 6 and h["in_range"] == 4
    assert h["mean"] == pytest.approx(inr.mean(), rel=1e-15)
    assert h["rms"] == pytest.approx(inr.std(), rel=1e-12)


def test_oracle_replay_reproduces_fixture(oracle, eio, gold):
    """The oracle fits of the replayed file (pins the oracle on the reference's
    own data; the GPU tests compare the engine against the same arrays)."""
    n = gold["samples"].shape[0]
    for mode, kw in (("ref", dict(start=0, max_iter_nnls=10)), ("kkt", dict(start=1, max_iter_nnls=1000))):
        r = oracle.fit_batch(gold["samples"], np.ones(n), gold["P"], gold["noisecor"], gold["bxs"], **kw)
        for k in ("amplitudes", "chi2", "active_mask", "status"):
            assert np.array_equal(r[k], gold[f"{mode}_{k}"]), (mode, k)
        h = eio.h01_summary(r["amplitudes"][:, 5] - gold["truth"])
        assert np.array_equal([h["mean"], h["rms"], h["entries"], h["in_range"]], gold[f"{mode}_h01"])
    # the KKT fits are NNLS optima of the whitened problems
    L = np.linalg.cholesky(gold["noisecor"])
    A = np.linalg.solve(L, gold["P"])
    for i in range(0, n, 7):
        b = np.linalg.solve(L, gold["samples"][i])
        assert oracle.kkt_violation(A, b, gold["kkt_amplitudes"][i]) < 1e-8
    # the reference start reaches the same points on this file
    assert np.array_equal(gold["ref_active_mask"], gold["kkt_active_mask"])


@needs_data
def test_reader_mutated_files_fail_cleanly(rootio):
    """Random byte changes in the data files: every read either returns or
    raises RootFormatError / KeyError (a name no longer found)."""
    rng = np.random.default_rng(3)
    for path in (SAMPLE_100, SHAPE):
        orig = bytearray(open(path, "rb").read())
        for _ in range(300):
            d = bytearray(orig)
            for _ in range(int(rng.integers(1, 9))):
                d[int(rng.integers(len(d)))] = int(rng.integers(256))
            try:
                f = rootio.RootFile(bytes(d))
                list(f.walk())
                for k in f.keys():
                    if k.class_name == "TTree":
                        t = f.tree(k.name)
                        t.array("amplitudeTruth", np.float64)
                        t.vectors("samples")
                    elif k.class_name.startswith("TDirectory"):
                        f.graph(k.name + "/grPulseShape")
                        f.tree(k.name + "/Tail").array("timeMin", np.float32)
            except (rootio.RootFormatError, KeyError):
                pass


OUTPUT_CPU = os.path.join(os.path.dirname(DATA), "analysis", "output_cpu.root")


@pytest.mark.skipif(not os.path.exists(OUTPUT_CPU), reason="the reference's analysis output is absent")
def test_reader_reference_output_histograms(rootio):
    """The reference's own multifit_cpu output (analysis/output_cpu.root): its
    Duration histogram holds the 10 batch times of the 65,536-channel run
    whose mean, 277.7 ms, is the last entry of analysis/cpu_i7-4770K_gpu_V100/
    multifit_cpu.csv; h01 (reco - true in-time amplitude) and reco_ampl were
    filled once per channel and iteration. Its input (a -13 ns shifted sample
    file) is not in the reference tree, so the physics numbers are recorded,
    not replayed."""
    f = rootio.RootFile(OUTPUT_CPU)
    assert {k.name for k in f.keys()} == {"RecoAndSim", "h01", "reco_ampl", "Duration"}
    dur = f.th1_stats("Duration")
    assert dur["entries"] == 10 and dur["ncells"] == 102
    assert round(dur["mean"], 6) == 277.7
    h = f.th1_stats("h01")
    assert h["entries"] == 655_360 == 10 * 65_536 and h["ncells"] == 1002
    reco = f.th1_stats("reco_ampl")
    assert reco["entries"] == h["entries"]
    # reco = truth + dA with truth = 10 GeV for every channel: the moments agree
    assert abs(reco["mean"] - 10.0 - h["mean"]) < 1e-9 and abs(reco["rms"] - h["rms"]) < 1e-8
    assert abs(h["mean"]) < 0.01 and 0.02 < h["rms"] < 0.04
    assert f.tree("RecoAndSim").entries == 0  # the tree record holds no entries


def test_reader_compressed_record_blocks(rootio):
    """A record split into several compressed blocks, zlib and LZMA (each block:
    2-letter algorithm, method byte, 3-byte little-endian compressed and
    uncompressed sizes, then the stream), inflated back to its ObjLen bytes."""
    import lzma
    import zlib

    rng = np.random.default_rng(4)
    parts = [np.cumsum(rng.standard_normal(3000)).astype(">f8").tobytes(), b"multifit" * 700, bytes(5000)]

    def block(alg, raw):
        z = zlib.compress(raw, 6) if alg == b"ZL" else lzma.compress(raw, format=lzma.FORMAT_XZ)
        return alg + b"\x08" + len(z).to_bytes(3, "little") + len(raw).to_bytes(3, "little") + z

    body = block(b"ZL", parts[0]) + block(b"XZ", parts[1]) + block(b"ZL", parts[2])
    keylen = 40
    data = bytes(keylen) + body
    rf = rootio.RootFile.__new__(rootio.RootFile)
    rf.path, rf.data = "<blocks>", data
    objlen = sum(len(p) for p in parts)
    key = rootio.Key(0, len(data), 4, objlen, keylen, 1, 0, 0, "TBasket", "b", "t", keylen)
    assert rf.payload(key) == b"".join(parts)
    bad = rootio.Key(0, len(data), 4, objlen + 1, keylen, 1, 0, 0, "TBasket", "b", "t", keylen)
    with pytest.raises(rootio.RootFormatError):
        rf.payload(bad)
    rf.data = bytes(keylen) + b"L4" + body[2:]
    with pytest.raises(rootio.RootFormatError, match="not supported"):
        rf.payload(key)


def test_committed_data_files_are_the_references():
    """tests/golden/reference_data/ holds the reference's files unchanged."""
    import hashlib

    from _helpers import COMMITTED_DATA

    want = {"mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root":
            "12bd30188d1f5084b7fa0bc795fb7483823acc78846cc2e01ee5143c45cd10b8",
            "EmptyFile.root": "e771768a1b1d5b55cadaccce00aabe507a2949dac136904381ce3cf6d0cbe3a9"}
    for name, digest in want.items():
        data = open(os.path.join(COMMITTED_DATA, name), "rb").read()
        assert hashlib.sha256(data).hexdigest() == digest, name
        ref = os.path.join(DATA, name)
        if DATA != COMMITTED_DATA and os.path.exists(ref):
            assert open(ref, "rb").read() == data, name

