"""The tuning table's entries change the kernels that rawspec_initialize
picks, and the results stay those of the FP64 oracle; the tuner runs a small
configuration end to end and writes a table the library reads."""
import ctypes as C

import numpy as np
import pytest

from cases import derived_nb
from oracle import oracle as O
from rawspec_gb300 import api, serve, synth, tune
from util import REL_TOL, normalized_error

pytestmark = pytest.mark.gpu


def with_table(tmp_path, monkeypatch, text):
    p = tmp_path / "t.tune"
    p.write_text(text)
    monkeypatch.setenv("RAWSPEC_GB300_TUNE_FILE", str(p))
    monkeypatch.delenv("RAWSPEC_GB300_TENSOR_DFT", raising=False)


def run(c, blocks):
    spec = api.Spectrometer(c["Nc"], c["Np"], c["Ntpb"], 8, c["products"])
    try:
        kinds = [spec.product_kernel(i) for i in range(len(c["products"]))]
        spec.process(blocks)
        return [np.array(d) for d in spec.dumps], kinds
    finally:
        spec.close()


def oracle(c, blocks):
    cfg = O.make_cfg(c["Nc"], c["Np"], c["Ntpb"], derived_nb(c), 8, c["products"])
    return O.run_oracle(cfg, blocks)[0]


@pytest.mark.parametrize("text,nt,npol,want", [
    ("", 1024, 1, "tc"),                          # the library's own choice
    ("1024 8 1 dft=cuda\n", 1024, 1, "small"),
    ("1024 8 1 dft=cuda ctas=16\n", 1024, 1, "small"),
    ("256 8 4 dft=tc\n", 256, 4, "tc"),          # a case k_tc supports but is not the default for
    ("512 8 -4 ctas=1\n", 512, -4, "small"),
])
def test_table_selects_the_kernel(cuda_device, tmp_path, monkeypatch, text, nt, npol, want):
    with_table(tmp_path, monkeypatch, text)
    # integrations within a buffer: one dump per buffer
    c = dict(Nc=4, Np=2, Ntpb=1 << 14, products=[(nt, min(64, (1 << 14) // nt), npol)])
    blocks = synth.gaussian_blocks(2, 4, 1 << 14, 2, sigma=20.0, seed=900 + nt)
    got, kinds = run(c, blocks)
    assert kinds == [want]
    assert normalized_error(got[0], oracle(c, blocks)[0], npol, 4, nt) < REL_TOL


@pytest.mark.parametrize("npol", [1, 4])
def test_fused_lag_and_ring_do_not_change_the_result(cuda_device, tmp_path, monkeypatch, npol):
    nt, Ntpb = 1 << 16, 1 << 18
    c = dict(Nc=3, Np=2, Ntpb=Ntpb, products=[(nt, 1, npol)])
    blocks = synth.gaussian_blocks(1, 3, Ntpb, 2, sigma=20.0, seed=950 + npol)
    with_table(tmp_path, monkeypatch, "")
    base, kinds = run(c, blocks)
    assert kinds == ["large_fused"]
    for lag, ring in [(2, 3), (3, 6), (6, 12)]:
        with_table(tmp_path, monkeypatch, f"{nt} 8 {npol} lag={lag} ring={ring}\n")
        got, _ = run(c, blocks)
        assert np.array_equal(got[0], base[0]), (lag, ring)


def test_estimate_follows_the_table(cuda_device, tmp_path, monkeypatch):
    prods = [(1 << 20, 51, 1), (8, 128, 1), (1024, 3072, 1)]
    for text in ["", "1048576 8 1 lag=6 ring=12\n8 8 1 ctas=16\n1024 8 1 dft=cuda ctas=8\n"]:
        with_table(tmp_path, monkeypatch, text)
        ctx = api.make_context(64, 2, 1 << 19, 8, prods)
        est = serve.device_bytes_estimate(ctx)
        spec = api.Spectrometer(64, 2, 1 << 19, 8, prods, collect=False)
        try:
            got = spec.lib.rawspec_gb300_device_bytes(C.byref(spec.ctx))
        finally:
            spec.close()
        assert est == got, (text, est, got)


def test_tuner_end_to_end(cuda_device, tmp_path, monkeypatch):
    monkeypatch.delenv("RAWSPEC_GB300_TUNE_FILE", raising=False)
    out = tmp_path / "tuned.txt"
    rc = tune.main(["--nc", "4", "--ntpb", str(1 << 16), "--nt", str(1 << 16), "--na", "1", "--nt", "1024",
                    "--na", "16", "--steps", "3", "--reps", "1", "--out", str(out)])
    assert rc == 0
    text = out.read_text()
    assert "library defaults" in text and "tuned:" in text
    monkeypatch.setenv("RAWSPEC_GB300_TUNE_FILE", str(out))
    for line in text.splitlines():
        if line and not line.startswith("#"):
            n, b, p = (int(x) for x in line.split()[:3])
            assert api.tune_lookup(n, b, p)[0] == 1
