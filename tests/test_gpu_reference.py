"""Parity of the native library with the reference's own GPU library: the
reference's rawspec_gpu.cu (cuFFT plans with its load and store callbacks)
compiled unchanged into oracle/_ref/libreference_rawspec.so and run in a
child process on the same inputs (oracle/ref_gpu.py).

Both libraries are driven through the same C interface (rawspec.h) with the
reference CLI's per-buffer sequence, and their dumps are compared bin by bin
with the normalised error of tests/util.py (tolerance 1e-5).  Where the FP64
oracle's output is at hand (the golden fixtures, the small configuration),
the reference build is also compared with it, which pins the oracle to the
reference's cuFFT output.

Configurations are chosen free of the reference's out-of-range accesses
(see oracle/ref_gpu.py): incoherent sums run in the reference with channel
batches of one antenna.

4-bit input.  The reference expands packed 4-bit samples through a table
whose entries are `((char)(b & 0xf0)) >> 4` and `((char)((b & 0x0f) << 4)) >> 4`
(rawspec_gpu.cu:342-350): sign-extended nibbles where `char` is signed (x86),
but 0..15 where it is unsigned, as on the aarch64 host of the GB300, so the
reference build there reads every negative nibble as its value plus 16.  For
4-bit cases the reference is therefore given the bytes its table produces on
x86 (each nibble sign-extended to int8 on the host, high nibble real) as
8-bit input; the native library gets the packed 4-bit blocks.  The native
nibble expansion itself is bit-exact against the oracle (golden fixtures)."""
import numpy as np
import pytest

from cases import CASES, derived_nb
from oracle import oracle as O
from oracle import ref_build, ref_gpu
from rawspec_gb300 import api, synth
from util import REL_TOL, load_golden, normalized_error, rms_normalized_error

pytestmark = pytest.mark.gpu


def _req(Nc, Np, Ntpb, nbits, products, *, Nant=1, conj=0, fft_dir=1, weights=None, keep=None):
    r = dict(Nc=Nc, Np=Np, Ntpb=Ntpb, nbits=nbits, products=[list(p) for p in products], Nant=Nant, conj=conj,
             fft_dir=fft_dir, weights=None if weights is None else [float(w) for w in weights])
    if weights is not None and Nant > 1:
        r["Nbc"] = Nc // Nant  # one antenna per channel batch (the reference's safe form of the sum)
    if keep:
        r["keep"] = keep
    return r


def expand4_like_reference_x86(blocks):
    """Packed 4-bit blocks -> the int8 [re, im] bytes of the reference's
    expansion table with signed char (high nibble real, low nibble imaginary)."""
    b = blocks.astype(np.uint8)
    hi = b.view(np.int8) >> 4
    lo = (b << 4).view(np.int8) >> 4
    return np.stack([hi, lo], axis=-1).reshape(b.shape[0], -1).view(np.uint8)


def reference_job(req, blocks):
    """(request, blocks) for the reference child (4-bit input pre-expanded)."""
    if req["nbits"] == 4:
        return dict(req, nbits=8), expand4_like_reference_x86(blocks)
    return req, blocks


def run_ours(req, blocks):
    spec = api.Spectrometer(req["Nc"], req["Np"], req["Ntpb"], req["nbits"], [tuple(p) for p in req["products"]],
                            Nant=req.get("Nant", 1), conj=req.get("conj", 0), weights=req.get("weights"))
    try:
        spec.process(blocks, fft_dir=req.get("fft_dir", 1))
        return [np.array(d) for d in spec.dumps], [np.array(s) for s in spec.ics]
    finally:
        spec.close()


@pytest.fixture(scope="session")
def reference_gpu(cuda_device):
    """Builds the reference GPU library (from the reference tree or its staged
    copy) and checks that cuFFT accepts its callbacks on a tiny context."""
    lib = ref_build.build_gpu()
    if lib is None:
        pytest.skip("the reference's GPU sources are not present (neither the tree nor the staged copy)")
    blocks = synth.gaussian_blocks(1, 1, 1024, 2, sigma=16.0, seed=7)
    try:
        out = ref_gpu.run_in_child([(_req(1, 2, 1024, 8, [(256, 1, 1)]), blocks)])[0]
    except RuntimeError as e:
        msg = str(e)
        if "CUFFT" in msg:
            pytest.skip(f"cuFFT refused the reference build's callbacks: {msg[-300:]}")
        raise
    print("reference cuFFT", str(out["cufft_version"]))
    return lib


def _compare(tag, ours, ref, npol, Nc, nt):
    assert ours.shape == ref.shape, (tag, ours.shape, ref.shape)
    err = normalized_error(ours, ref, npol, Nc, nt)
    rms = rms_normalized_error(ours, ref, npol, Nc, nt)
    print(f"{tag}: max {err:.2e} rms {rms:.2e}")
    assert err < REL_TOL, (tag, err)
    return err


def test_small_configuration_matches_reference_and_oracle(reference_gpu):
    # 8 channels, 8-bit Gaussian (sigma 16) plus a tone at fine offset 0.3 in
    # channel 3, Ntpb 65536, 4 blocks; Nfft 1024, Nint 16, total power
    Nc, Ntpb, prods = 8, 65536, [(1024, 16, 1)]
    blocks = synth.gaussian_blocks(4, Nc, Ntpb, 2, sigma=16.0, seed=1, tone=(3, 0.3, 8.0))
    req = _req(Nc, 2, Ntpb, 8, prods)
    ref = ref_gpu.run_in_child([(req, blocks)])[0]
    ours, _ = run_ours(req, blocks)
    orc, _ = O.run_oracle(O.make_cfg(Nc, 2, Ntpb, 1, 8, prods), blocks)
    _compare("ours vs reference", ours[0], ref["out0"], 1, Nc, 1024)
    _compare("reference vs FP64 oracle", ref["out0"], orc[0], 1, Nc, 1024)
    _compare("ours vs FP64 oracle", ours[0], orc[0], 1, Nc, 1024)


@pytest.fixture(scope="module")
def golden_reference(reference_gpu):
    """The reference's dumps of every golden case, from one child process."""
    jobs, names = [], sorted(CASES)
    for name in names:
        c = CASES[name]
        g = load_golden(name)
        jobs.append((_req(c["Nc"], c["Np"], c["Ntpb"], c["nbits"], c["products"], Nant=c.get("Nant", 1),
                          conj=c["conj"], fft_dir=c["fft_dir"], weights=g.get("weights")), g["blocks"]))
    return dict(zip(names, ref_gpu.run_in_child([reference_job(r, b) for r, b in jobs]))), dict(zip(names, jobs))


@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_cases_match_reference(golden_reference, name):
    refs, jobs = golden_reference
    ref, (req, blocks) = refs[name], jobs[name]
    c = CASES[name]
    g = load_golden(name)
    ours, ours_ics = run_ours(req, blocks)
    for i, (nt, _na, npol) in enumerate(c["products"]):
        _compare(f"{name} product {i} ours vs reference", ours[i], ref[f"out{i}"], npol, c["Nc"], nt)
        # the FP64 oracle's golden output against the reference build
        _compare(f"{name} product {i} reference vs oracle", ref[f"out{i}"], g[f"out{i}"], npol, c["Nc"], nt)
        if c.get("ics"):
            nca = c["Nc"] // c["Nant"]
            _compare(f"{name} product {i} ICS ours vs reference", ours_ics[i], ref[f"ics{i}"], npol, nca, nt)
            _compare(f"{name} product {i} ICS reference vs oracle", ref[f"ics{i}"], g[f"ics{i}"], npol, nca, nt)


def _length_cases():
    cases = []
    for logn in range(1, 13):
        nt = 1 << logn
        npol = (1, 4, -4)[logn % 3]
        Ntpb = max(4096, nt)
        na = max(1, min(64, Ntpb // nt // 2))
        cases.append((f"nfft {nt}", _req(3, 2, Ntpb, 8, [(nt, na, npol)], conj=logn & 1, fft_dir=1 - 2 * (logn % 2)),
                      synth.gaussian_blocks(2, 3, Ntpb, 2, sigma=18.0, seed=400 + logn)))
    for logn, npol in [(13, 4), (14, 1), (16, -4), (17, 4), (18, 1), (19, 4), (20, 1), (20, 4), (21, -4), (22, 1)]:
        nt = 1 << logn
        cases.append((f"nfft 2^{logn} P{npol}", _req(1, 2, nt // 2, 8, [(nt, 2, npol)], conj=logn & 1),
                      synth.gaussian_blocks(4, 1, nt // 2, 2, sigma=16.0, seed=500 + logn)))
    return cases


def test_every_length_matches_reference(reference_gpu):
    # the k_small lengths 1..4096 (tensor-core kernels where they are the
    # default), and every four-step shape including the fused 2^16..2^22 path
    cases = _length_cases()
    refs = ref_gpu.run_in_child([(r, b) for _, r, b in cases])
    worst = 0.0
    for (tag, req, blocks), ref in zip(cases, refs):
        ours, _ = run_ours(req, blocks)
        nt, _na, npol = req["products"][0]
        worst = max(worst, _compare(tag, ours[0], ref["out0"], npol, req["Nc"], nt))
    print(f"worst over lengths: {worst:.2e}")


@pytest.mark.parametrize("npol", [1, 4])
def test_mixed_precision_products_match_reference(reference_gpu, npol):
    # the small configuration's voltages over 192 blocks, Nfft 8/256/1024/4096
    # with Nint 128/256/512/3072 (each product dumps at least once); the
    # tensor-core DFT kernels are the default for 1024/4096 total power
    Nc, Ntpb = 8, 65536
    prods = [(8, 128, npol), (256, 256, npol), (1024, 512, npol), (4096, 3072, npol)]
    blocks = synth.gaussian_blocks(192, Nc, Ntpb, 2, sigma=16.0, seed=1, tone=(3, 0.3, 8.0))
    req = _req(Nc, 2, Ntpb, 8, prods)
    ref = ref_gpu.run_in_child([(req, blocks)])[0]
    ours, _ = run_ours(req, blocks)
    for i, (nt, _na, _p) in enumerate(prods):
        assert len(ours[i]) == int(ref[f"ndumps{i}"]) > 0, (i, len(ours[i]), int(ref[f"ndumps{i}"]))
        _compare(f"Nfft {nt} Npolout {npol}", ours[i], ref[f"out{i}"], npol, Nc, nt)


def test_multi_antenna_4bit_stokes_with_incoherent_sum_matches_reference(reference_gpu):
    # 4 antennas x 16 channels, 4-bit uniform voltages with per-antenna gains,
    # Ntpb 262144, 8 blocks; Nfft 4096 / Nint 64 and Nfft 64 / Nint 1024,
    # Stokes, weighted incoherent sum
    Nant, Nc, Ntpb = 4, 64, 262144
    blocks, _gains = synth.int4_blocks(8, Nc, Ntpb, 2, Nant=Nant, seed=3)
    w = synth.weights(Nant, seed=5)
    prods = [(4096, 64, -4), (64, 1024, -4)]
    req = _req(Nc, 2, Ntpb, 4, prods, Nant=Nant, weights=w)
    ref = ref_gpu.run_in_child([reference_job(req, blocks)])[0]
    ours, ours_ics = run_ours(req, blocks)
    for i, (nt, _na, npol) in enumerate(prods):
        _compare(f"4-bit Nfft {nt}", ours[i], ref[f"out{i}"], npol, Nc, nt)
        _compare(f"4-bit Nfft {nt} ICS", ours_ics[i], ref[f"ics{i}"], npol, Nc // Nant, nt)
