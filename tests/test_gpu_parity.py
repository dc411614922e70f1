"""Parity of the native CUDA path (through the C-ABI) with the FP64 oracle.

Small configurations are compared bin by bin with the committed golden
fixtures and with the oracle run on the fly; full-size configurations are
checked through size-independent properties (Parseval per integration, the
Stokes identities between modes)."""
import ctypes as C
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from cases import CASES, derived_nb
from oracle import oracle as O
from rawspec_gb300 import api, synth
from util import REL_TOL, load_golden, normalized_error

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def run_gpu(c, blocks, weights=None, fft_dir=None, Nbc=0):
    spec = api.Spectrometer(c["Nc"], c["Np"], c["Ntpb"], c["nbits"], c["products"], Nant=c.get("Nant", 1),
                            conj=c["conj"], weights=None if weights is None else list(weights), Nbc=Nbc)
    try:
        spec.process(blocks, fft_dir=c["fft_dir"] if fft_dir is None else fft_dir)
        return [np.array(d) for d in spec.dumps], [np.array(s) for s in spec.ics], spec.events, spec.kernel_launches()
    finally:
        spec.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_parity(cuda_device, name):
    c = CASES[name]
    g = load_golden(name)
    dumps, ics, _, launches = run_gpu(c, g["blocks"], g.get("weights"))
    assert launches > 0
    for i, (nt, na, npol) in enumerate(c["products"]):
        ref = g[f"out{i}"]
        assert dumps[i].shape == ref.shape, (i, dumps[i].shape, ref.shape)
        err = normalized_error(dumps[i], ref, npol, c["Nc"], nt)
        assert err < REL_TOL, (name, i, err)
        if c.get("ics"):
            eri = normalized_error(ics[i], g[f"ics{i}"], npol, c["Nc"] // c["Nant"], nt)
            assert eri < REL_TOL, (name, i, "ics", eri)


def oracle_for(c, blocks, weights=None, inverse=None):
    cfg = O.make_cfg(c["Nc"], c["Np"], c["Ntpb"], derived_nb(c), c["nbits"], c["products"], Nant=c.get("Nant", 1),
                     conj=c["conj"], inverse=(1 if c["fft_dir"] <= 0 else 0) if inverse is None else inverse,
                     weights=weights)
    return O.run_oracle(cfg, blocks)


@pytest.mark.parametrize("logn", list(range(0, 13)))
@pytest.mark.parametrize("npol", [1, 4, -4])
def test_small_lengths_all_modes(cuda_device, monkeypatch, logn, npol):
    # the CUDA-core kernel k_small at every length (the tensor-core kernel,
    # the default at 1024 points, has its own tests)
    monkeypatch.setenv("RAWSPEC_GB300_TENSOR_DFT", "0")
    nt = 1 << logn
    Ntpb = max(4096, nt)
    # Na chosen so that some integrations stay within the buffer (Nd > 1),
    # and large enough that one unit is split over several CTAs.
    na = max(1, min(64, (2 * Ntpb) // nt // 2))
    c = dict(Nc=3, Np=2, Ntpb=Ntpb, nbits=8, nblocks=2, products=[(nt, na, npol)], conj=1, fft_dir=1)
    blocks = synth.gaussian_blocks(2, 3, Ntpb, 2, sigma=18.0, seed=100 + logn)
    dumps, _, _, _ = run_gpu(c, blocks)
    ref, _ = oracle_for(c, blocks)
    err = normalized_error(dumps[0], ref[0], npol, 3, nt)
    assert err < REL_TOL, (nt, npol, err)


@pytest.mark.parametrize("logn,npol", [(13, 4), (14, 1), (16, 4), (17, -4), (18, 1), (19, 4), (20, 4), (21, 1),
                                       (22, -4)])
def test_large_lengths(cuda_device, logn, npol):
    # every four-step shape (N1 x N2 from 64 x 128 to 2048 x 2048), both the
    # two-kernel and the fused path, integrations spanning two buffers
    nt = 1 << logn
    c = dict(Nc=1, Np=2, Ntpb=nt // 2, nbits=8, nblocks=4, products=[(nt, 2, npol)], conj=0, fft_dir=1)
    blocks = synth.gaussian_blocks(4, 1, nt // 2, 2, sigma=16.0, seed=200 + logn)
    dumps, _, _, _ = run_gpu(c, blocks)
    ref, _ = oracle_for(c, blocks)
    err = normalized_error(dumps[0], ref[0], npol, 1, nt)
    assert err < REL_TOL, (nt, err)


def test_large_single_polarisation(cuda_device):
    # one input polarisation takes the two-kernel four-step path
    nt = 1 << 16
    c = dict(Nc=2, Np=1, Ntpb=nt, nbits=8, nblocks=2, products=[(nt, 1, 1)], conj=0, fft_dir=1)
    blocks = synth.gaussian_blocks(2, 2, nt, 1, sigma=16.0, seed=250)
    dumps, _, _, _ = run_gpu(c, blocks)
    ref, _ = oracle_for(c, blocks)
    assert normalized_error(dumps[0], ref[0], 1, 2, nt) < REL_TOL


@pytest.mark.parametrize("npol,conj,fft_dir", [(1, 0, 1), (1, 1, -1), (4, 1, -1), (-4, 1, 1)])
def test_fused_long_fft_many_slabs(cuda_device, npol, conj, fft_dir):
    # 2^16-point FFTs, one spectrum per integration, 4 spectra per channel
    # and 3 channels: 12 slabs, fewer than the lag the plan chooses for this
    # length, so every column tile is queued before the first row tile.
    nt, Ntpb = 1 << 16, 1 << 18
    c = dict(Nc=3, Np=2, Ntpb=Ntpb, nbits=8, nblocks=1, products=[(nt, 1, npol)], conj=conj, fft_dir=fft_dir)
    blocks = synth.gaussian_blocks(1, 3, Ntpb, 2, sigma=20.0, seed=300 + npol)
    dumps, _, _, _ = run_gpu(c, blocks)
    ref, _ = oracle_for(c, blocks)
    assert dumps[0].shape == ref[0].shape
    assert normalized_error(dumps[0], ref[0], npol, 3, nt) < REL_TOL


@pytest.mark.parametrize("npol", [1, 4, -4])
def test_fused_ring_slot_reuse(cuda_device, npol):
    # 2^20-point FFTs, one spectrum per integration, 2 spectra per channel and
    # 5 channels: the 10 slabs outnumber the intermediate ring the plan sizes
    # for this length (6 slabs on a 152-SM GPU), so slots are reused and the
    # column tiles of a slab wait for the row tiles of an earlier one.
    nt, Ntpb = 1 << 20, 1 << 21
    c = dict(Nc=5, Np=2, Ntpb=Ntpb, nbits=8, nblocks=1, products=[(nt, 1, npol)], conj=0, fft_dir=1)
    blocks = synth.gaussian_blocks(1, 5, Ntpb, 2, sigma=20.0, seed=350 - npol)
    dumps, _, _, _ = run_gpu(c, blocks)
    ref, _ = oracle_for(c, blocks)
    assert dumps[0].shape == ref[0].shape
    assert normalized_error(dumps[0], ref[0], npol, 5, nt) < REL_TOL


def test_fused_with_incoherent_sum(cuda_device):
    # two antennas of 3 channels, 2^16-point products on the fused path in
    # total power and full Stokes, integrations spanning the 2 buffers, and
    # the weighted sum over antennas of both
    nt = 1 << 16
    c = dict(Nc=6, Np=2, Ntpb=nt, nbits=8, nblocks=2, Nant=2, products=[(nt, 2, 1), (nt, 2, -4)], conj=0,
             fft_dir=1)
    blocks = synth.gaussian_blocks(2, 6, nt, 2, sigma=18.0, seed=410)
    w = synth.weights(2, seed=411)
    dumps, ics, _, _ = run_gpu(c, blocks, weights=w)
    ref, ref_ics = oracle_for(c, blocks, weights=w)
    for i, (_, _, npol) in enumerate(c["products"]):
        assert dumps[i].shape == ref[i].shape
        assert normalized_error(dumps[i], ref[i], npol, 6, nt) < REL_TOL
        assert normalized_error(ics[i], ref_ics[i], npol, 3, nt) < REL_TOL


@pytest.mark.parametrize("npol", [1, 4])
def test_long_integration_3072_spectra(cuda_device, npol):
    # Nint 3072 of 1024-point spectra spanning three 2-block buffers (the
    # production's third product): the per-chunk register sums, the
    # fixed-order chunk reduction and the compensated accumulation across
    # buffers stay within the FP32 tolerance of the FP64 oracle.
    Nc, Ntpb = 2, 524288
    c = dict(Nc=Nc, Np=2, Ntpb=Ntpb, nbits=8, nblocks=6, products=[(1024, 3072, npol), (1 << 20, 3, npol)],
             conj=0, fft_dir=1)
    blocks = synth.gaussian_blocks(6, Nc, Ntpb, 2, sigma=20.0, seed=500 + npol)
    dumps, _, _, _ = run_gpu(c, blocks)
    ref, _ = oracle_for(c, blocks)
    for i, (nt, _, _) in enumerate(c["products"]):
        assert dumps[i].shape == ref[i].shape == (1, abs(npol) * Nc * nt)
        err = normalized_error(dumps[i], ref[i], npol, Nc, nt)
        print(f"Nt {nt}, Npolout {npol}: normalized error {err:.2e}")
        assert err < REL_TOL


def test_inverse_direction_and_nis_chunks(cuda_device):
    c = dict(Nc=4, Np=2, Ntpb=8192, nbits=8, nblocks=6, products=[(1024, 24, -4), (8192, 3, 1)], conj=1, fft_dir=-1)
    blocks = synth.gaussian_blocks(6, 4, 8192, 2, sigma=20.0, seed=7)
    dumps, _, events, _ = run_gpu(c, blocks)
    ref, _ = oracle_for(c, blocks)
    for i, (nt, na, npol) in enumerate(c["products"]):
        assert dumps[i].shape == ref[i].shape
        assert normalized_error(dumps[i], ref[i], npol, 4, nt) < REL_TOL


def test_dump_callbacks_are_ordered(cuda_device):
    c = dict(Nc=2, Np=2, Ntpb=1024, nbits=8, nblocks=6, products=[(256, 8, 1), (64, 32, 4)], conj=0, fft_dir=1)
    blocks = synth.gaussian_blocks(6, 2, 1024, 2, seed=9)
    dumps, _, events, _ = run_gpu(c, blocks)
    # product 0: Nis = 2 -> 3 dumps in 6 buffers; product 1: Nis = 2 -> 3 dumps
    assert len(dumps[0]) == 3 and len(dumps[1]) == 3
    for prod in (0, 1):
        seq = [k for p, k in events if p == prod]
        # every POST is directly preceded by its PRE
        for j, k in enumerate(seq):
            if k == api.RAWSPEC_CALLBACK_POST_DUMP:
                assert j > 0 and seq[j - 1] == api.RAWSPEC_CALLBACK_PRE_DUMP
        assert seq.count(api.RAWSPEC_CALLBACK_POST_DUMP) == 3


def test_reset_zero_and_completion(cuda_device):
    lib = api.load_library()
    # Nt 256, Na 4, Ntpb 1024: one integration (one dump) per buffer
    spec = api.Spectrometer(2, 2, 1024, 8, [(256, 4, 1)])
    try:
        blocks = synth.gaussian_blocks(1, 2, 1024, 2, seed=3)
        spec.load_blocks(blocks)
        spec.copy_to_gpu()
        spec.start()
        assert spec.wait() == 0
        assert lib.rawspec_check_for_completion(C.byref(spec.ctx)) == 1
        assert len(spec.dumps[0]) == 1 and np.all(spec.dumps[0][0] > 0)
        # zeroed input gives all-zero integrations after a reset
        assert lib.rawspec_reset_integration(C.byref(spec.ctx)) == 0
        assert lib.rawspec_zero_blocks_to_gpu(C.byref(spec.ctx), 0, 1) == 0
        for _ in range(8):
            spec.start()
        assert spec.wait() == 0
        assert len(spec.dumps[0]) == 9
        assert all(np.all(d == 0) for d in spec.dumps[0][1:])
    finally:
        spec.close()


def test_reset_restarts_multi_buffer_integration(cuda_device):
    # Nt 256, Na 8, Ntpb 1024: Nis = 2 buffers per dump; a reset in the middle
    # of an integration discards the partial sum.
    c = dict(Nc=2, Np=2, Ntpb=1024, nbits=8, nblocks=2, products=[(256, 8, 1)], conj=0, fft_dir=1)
    blocks = synth.gaussian_blocks(2, 2, 1024, 2, seed=4)
    lib = api.load_library()
    spec = api.Spectrometer(2, 2, 1024, 8, [(256, 8, 1)])
    try:
        spec.load_blocks(blocks[:1])
        spec.copy_to_gpu()
        spec.start()                      # half an integration of block 0
        assert lib.rawspec_reset_integration(C.byref(spec.ctx)) == 0
        spec.process(blocks)              # blocks 0 and 1 -> one dump
        assert len(spec.dumps[0]) == 1
        ref, _ = oracle_for(c, blocks)
        assert normalized_error(np.array(spec.dumps[0]), ref[0], 1, 2, 256) < REL_TOL
    finally:
        spec.close()


def test_exit_soon_is_returned(cuda_device):
    spec = api.Spectrometer(2, 2, 1024, 8, [(256, 4, 1)])
    try:
        spec.ctx.exit_soon = 1
        assert spec.wait() == 1
    finally:
        spec.close()


def _parseval_check(nt, na, blocks, Nc, Ntpb, dumps, npol):
    """Sum over fine channels of each integrated spectrum equals Nt times the
    voltage power of the integration's samples (size-independent property)."""
    x = blocks.view(np.int8).reshape(-1, Nc, Ntpb, 2, 2).astype(np.float64)
    x = np.maximum(x, -127) / 127.0
    x = np.transpose(x, (1, 0, 2, 3, 4)).reshape(Nc, -1, 2, 2)  # [c][t][pol][ri]
    p = (x ** 2).sum(axis=(2, 3)) if npol != 4 else (x ** 2).sum(axis=3)  # [c][t] or [c][t][pol]
    nint = p.shape[1] // (nt * na)
    if npol == 4:
        want = p[:, : nint * nt * na].reshape(Nc, nint, nt * na, 2).sum(axis=2) * nt  # [c][d][pol]
        got = dumps.reshape(nint, 4, Nc, nt)[:, :2].sum(axis=-1)                    # [d][pol][c]
        got = np.transpose(got, (2, 0, 1))
    else:
        want = p[:, : nint * nt * na].reshape(Nc, nint, nt * na).sum(axis=2) * nt
        got = dumps.reshape(nint, abs(npol), Nc, nt)[:, 0].sum(axis=-1).T
    np.testing.assert_allclose(got, want, rtol=1e-5)


@pytest.mark.parametrize("npol", [1, 4])
def test_full_size_production_shape_parseval(cuda_device, npol):
    # 64 channels, Ntpb 524288 (128 MiB blocks), one 2-block buffer; the
    # products of the production configuration with integration lengths
    # that dump within the buffer.
    Nc, Ntpb = 64, 524288
    blocks = synth.gaussian_blocks(2, Nc, Ntpb, 2, sigma=20.0, seed=21)
    prods = [(1 << 20, 1, npol), (8, 128, npol), (1024, 1024, npol)]
    c = dict(Nc=Nc, Np=2, Ntpb=Ntpb, nbits=8, products=prods, conj=0, fft_dir=1)
    dumps, _, _, _ = run_gpu(c, blocks)
    for i, (nt, na, _) in enumerate(prods):
        assert len(dumps[i]) == 1
        _parseval_check(nt, na, blocks, Nc, Ntpb, dumps[i][0], npol)


def test_full_size_stokes_identities(cuda_device):
    Nc, Ntpb = 64, 524288
    blocks = synth.gaussian_blocks(2, Nc, Ntpb, 2, sigma=20.0, seed=22)
    base = dict(Nc=Nc, Np=2, Ntpb=Ntpb, nbits=8, conj=1, fft_dir=1)
    full, _, _, _ = run_gpu(dict(base, products=[(1 << 20, 1, 4), (1024, 1024, 4)]), blocks)
    stokes, _, _, _ = run_gpu(dict(base, products=[(1 << 20, 1, -4), (1024, 1024, -4)]), blocks)
    for i, nt in enumerate([1 << 20, 1024]):
        F = full[i][0].reshape(4, Nc, nt).astype(np.float64)
        S = stokes[i][0].reshape(4, Nc, nt).astype(np.float64)
        scale = S[0]
        assert np.max(np.abs(S[0] - (F[0] + F[1])) / scale) < 1e-6
        assert np.max(np.abs(S[1] - (F[0] - F[1])) / scale) < 1e-6
        assert np.max(np.abs(S[2] - F[2]) / scale) < 1e-6
        assert np.max(np.abs(S[3] - F[3]) / scale) < 1e-6


def test_full_size_multi_antenna_4bit(cuda_device):
    # The batched multi-antenna 4-bit shape: 4 antennas x 16 channels, 2 pols,
    # Ntpb 262144, 8 blocks, full Stokes products Nfft 4096 / 64 with Nint
    # 64 / 1024, weighted incoherent sum.  Checked through properties that
    # hold at any size: the incoherent sum equals the weighted sum of the
    # antennas' dumps, and Stokes I obeys Parseval per integration.
    Nant, Nc, Ntpb, nb = 4, 64, 262144, 8
    prods = [(4096, 64, -4), (64, 1024, -4)]
    blocks, _ = synth.int4_blocks(nb, Nc, Ntpb, 2, Nant=Nant, seed=31)
    w = synth.weights(Nant, seed=32)
    c = dict(Nc=Nc, Np=2, Ntpb=Ntpb, nbits=4, products=prods, Nant=Nant, conj=0, fft_dir=1)
    dumps, ics, _, _ = run_gpu(c, blocks, weights=w)
    nca = Nc // Nant
    # voltage power per channel and time sample, from the packed nibbles
    pw = np.empty((nb, Nc, Ntpb), dtype=np.int32)
    for k in range(nb):
        b = blocks[k].reshape(Nc, Ntpb, 2).astype(np.int32)
        re = ((b >> 4) ^ 8) - 8
        im = ((b & 15) ^ 8) - 8
        pw[k] = (re * re + im * im).sum(axis=2)
    for i, (nt, na, _) in enumerate(prods):
        d = np.array(dumps[i], dtype=np.float64)          # [dump][Nd*4*Nc*nt]
        n_int = d.size // (4 * Nc * nt)
        d = d.reshape(n_int, 4, Nc, nt)
        assert n_int == nb * Ntpb // (nt * na)
        # incoherent sum
        got_ics = np.array(ics[i], dtype=np.float64).reshape(n_int, 4, nca, nt)
        want_ics = sum(float(w[a]) * d[:, :, a * nca:(a + 1) * nca, :] for a in range(Nant))
        scale = np.abs(want_ics[:, 0]).max()
        assert np.max(np.abs(got_ics - want_ics)) / scale < 1e-6
        # Parseval on Stokes I
        want = pw.transpose(1, 0, 2).reshape(Nc, n_int, nt * na).sum(axis=2, dtype=np.float64) * nt / 127.0 ** 2
        got = d[:, 0].sum(axis=-1).T
        np.testing.assert_allclose(got, want, rtol=1e-5)


def test_unpack_matches_texture_unit(cuda_device, tmp_path):
    so = tmp_path / "libsnorm_probe.so"
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-shared", "-Xcompiler",
           "-fPIC", f"-I{ROOT / 'rawspec_gb300' / 'csrc'}", "-o", str(so), str(ROOT / "tests" / "probe" / "snorm_probe.cu")]
    subprocess.run(cmd, check=True)
    lib = C.CDLL(str(so))
    t8, o8 = np.zeros(256, np.float32), np.zeros(256, np.float32)
    t16, o16 = np.zeros(65536, np.float32), np.zeros(65536, np.float32)
    fp = C.POINTER(C.c_float)
    rc = lib.snorm_probe(t8.ctypes.data_as(fp), o8.ctypes.data_as(fp), t16.ctypes.data_as(fp), o16.ctypes.data_as(fp))
    assert rc == 0
    assert np.array_equal(t8.view(np.uint32), o8.view(np.uint32)), np.nonzero(t8 != o8)
    assert np.array_equal(t16.view(np.uint32), o16.view(np.uint32)), np.nonzero(t16 != o16)
    # and the oracle's unpack agrees with both
    assert all(float(o8[i]) == O.snorm(int(np.int8(np.uint8(i))), 8) for i in range(256))


@pytest.mark.parametrize("nbits,Nc", [(8, 8), (4, 8), (8, 13)])
def test_combined_call_pipelines_copy_and_processing(cuda_device, nbits, Nc):
    # rawspec_copy_blocks_to_gpu_and_start_processing on buffers of 16 MiB
    # and more copies channel groups on a second stream and processes each
    # group as it lands; results must equal the separate calls' and the
    # oracle's.  13 channels make groups of one and two channels.
    Ntpb, nblocks = 1 << 19, 3
    prods = [(1024, 16, 1), (1 << 16, 1, 4), (8, 128, -4)]
    if nbits == 4:
        blocks, _ = synth.int4_blocks(nblocks, Nc, Ntpb, 2, Nant=1, seed=41)
    else:
        blocks = synth.gaussian_blocks(nblocks, Nc, Ntpb, 2, sigma=20.0, seed=41)
    spec = api.Spectrometer(Nc, 2, Ntpb, nbits, prods, conj=1)
    try:
        spec.process(blocks, combined=True)
        got = [np.array(d) for d in spec.dumps]
    finally:
        spec.close()
    c = dict(Nc=Nc, Np=2, Ntpb=Ntpb, nbits=nbits, products=prods, conj=1, fft_dir=1)
    ref, _ = oracle_for(c, blocks)
    for i, (nt, na, npol) in enumerate(prods):
        assert got[i].shape == ref[i].shape
        assert normalized_error(got[i], ref[i], npol, Nc, nt) < REL_TOL, (nbits, nt)


def test_graph_replay_equals_direct_launches(cuda_device, monkeypatch):
    # rawspec_start_processing replays a CUDA graph per buffer pattern
    # (write/add mode and dump of every product); the results and the kernel
    # launch count equal those of launching the kernels directly
    Nc, Ntpb, nblocks = 4, 1 << 16, 7
    prods = [(1 << 17, 1, 1), (1024, 256, 4), (8, 512, -4)]
    blocks = synth.gaussian_blocks(nblocks, Nc, Ntpb, 2, sigma=20.0, seed=77)
    out = {}
    for graphs in ("1", "0"):
        monkeypatch.setenv("RAWSPEC_GB300_GRAPHS", graphs)
        spec = api.Spectrometer(Nc, 2, Ntpb, 8, prods, conj=1)
        try:
            spec.process(blocks)
            out[graphs] = ([[np.array(d) for d in p] for p in spec.dumps], spec.events, spec.kernel_launches())
        finally:
            spec.close()
    (d1, e1, n1), (d0, e0, n0) = out["1"], out["0"]
    # callbacks of one product keep their order; the products' streams interleave freely
    per_product = lambda ev: [[k for q, k in ev if q == p] for p in range(len(prods))]  # noqa: E731
    assert n1 == n0 > 0 and per_product(e1) == per_product(e0)
    for p in range(len(prods)):
        assert len(d1[p]) == len(d0[p]) > 0
        assert all(np.array_equal(a, b) for a, b in zip(d1[p], d0[p]))
