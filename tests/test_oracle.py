"""The FP64 oracle against known answers (CPU only).

Pins: the impulse case of the reference's own test program rawspectest.c
(rawspectest.c:46-103: pol0 sample 8 = 127 + 0j, pol1 sample 9 = 0 + 64j,
four products, conjugated input, inverse FFT), single tones, the Stokes
identities between the +4 and -4 modes, the exact unpack rounding, 4-bit
nibble order and the committed golden fixtures."""
from fractions import Fraction

import numpy as np
import pytest

from cases import CASES, blocks_for, derived_nb
from oracle import oracle as O
from util import load_golden


def f32_exact(fr: Fraction) -> float:
    """Correct round-to-nearest-even of a rational to float32."""
    c = np.float32(float(fr))
    best = None
    for v in (c, np.nextafter(c, np.float32(np.inf)), np.nextafter(c, np.float32(-np.inf))):
        key = (abs(Fraction(float(v)) - fr), int(np.float32(v).view(np.uint32)) & 1)
        if best is None or key < best[0]:
            best = (key, v)
    return float(best[1])


@pytest.mark.parametrize("nbits,step", [(8, 1), (16, 97)])
def test_unpack_is_correctly_rounded_snorm(nbits, step):
    d = 127 if nbits == 8 else 32767
    lo = -(d + 1)
    for code in list(range(lo, d + 1, step)) + [lo, lo + 1, -1, 0, 1, d]:
        want = f32_exact(Fraction(max(code, -d), d))
        assert O.snorm(code, nbits) == want, code


def test_oracle_fft_matches_numpy():
    rng = np.random.default_rng(0)
    for n in [1, 2, 8, 64, 1024, 3, 12, 100]:
        z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        np.testing.assert_allclose(O.fft(z), np.fft.fft(z), rtol=1e-12, atol=1e-12 * n)
        np.testing.assert_allclose(O.fft(z, inverse=True), np.fft.ifft(z) * n, rtol=1e-12, atol=1e-12 * n)


def rawspectest_blocks(Nc, Ntpb, nbits=8):
    Np = 2
    bpc = nbits // 8
    blk = np.zeros((1, Nc * Ntpb * Np * 2 * bpc), np.uint8)
    blk[0, (8 * Np * 2) * bpc] = 127   # pol 0, sample 8, real
    blk[0, (9 * Np * 2 + 3) * bpc] = 64  # pol 1, sample 9, imaginary
    return blk


@pytest.mark.parametrize("inverse", [0, 1])
def test_rawspectest_impulse_known_answers(inverse):
    Nc, Ntpb = 4, 1024
    prods = [(1024, 1, 1), (8, 128, 1), (1024, 1, 4), (1024, 1, -4)]
    cfg = O.make_cfg(Nc, 2, Ntpb, 1, 8, prods, conj=1, inverse=inverse)
    outs, _ = O.run_oracle(cfg, rawspectest_blocks(Nc, Ntpb))
    # The FFT sees the SNORM values rounded to float: 127 -> 1.0, 64 -> fl(64/127).
    a = float(np.float32(64 / 127))
    p1 = 1.0
    p2 = a * a
    P = outs[0].reshape(Nc, 1024)
    np.testing.assert_allclose(P[0], p1 + p2, rtol=1e-12)
    assert np.all(P[1:] == 0)
    P8 = outs[1].reshape(1, Nc, 8)[0]
    np.testing.assert_allclose(P8[0], p1 + p2, rtol=1e-12)  # 128 spectra, one of them holds the impulses
    F = outs[2].reshape(4, Nc, 1024)
    np.testing.assert_allclose(F[0, 0], p1, rtol=1e-12)
    np.testing.assert_allclose(F[1, 0], p2, rtol=1e-12)
    np.testing.assert_allclose(np.hypot(F[2, 0], F[3, 0]), a, rtol=1e-12)
    S = outs[3].reshape(4, Nc, 1024)
    np.testing.assert_allclose(S[0, 0], p1 + p2, rtol=1e-12)
    np.testing.assert_allclose(S[1, 0], p1 - p2, rtol=1e-12)
    np.testing.assert_allclose(S[2, 0], F[2, 0], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(S[3, 0], F[3, 0], rtol=1e-12, atol=1e-15)
    # X0 = 1*W^(8k), X1 = (64/127) i W^(9k) -> X0 X1* = -(64/127) i W^(-k) (forward),
    # conjugated input negates the imaginary part.
    k = np.arange(1024)
    shift = (k + 512) % 1024
    sgn = 1 if inverse else -1
    w = np.exp(sgn * 2j * np.pi * k * (8 - 9) / 1024)
    xy = 1.0 * np.conj(1j * a) * w
    np.testing.assert_allclose(F[2, 0, shift], xy.real, atol=1e-12)
    np.testing.assert_allclose(F[3, 0, shift], -xy.imag, atol=1e-12)


def test_single_tone_lands_in_shifted_bin():
    Nc, Ntpb, Nt = 1, 4096, 256
    kbin = 37
    t = np.arange(Ntpb)
    x = np.rint(100 * np.exp(2j * np.pi * kbin * t / Nt))
    raw = np.zeros((Nc, Ntpb, 2, 2), np.int8)
    raw[0, :, 0, 0] = x.real
    raw[0, :, 0, 1] = x.imag
    blocks = raw.reshape(1, -1).view(np.uint8)
    cfg = O.make_cfg(Nc, 2, Ntpb, 1, 8, [(Nt, 16, 1)])
    outs, _ = O.run_oracle(cfg, blocks)
    P = outs[0].reshape(-1, Nt)
    peak = np.argmax(P, axis=1)
    assert np.all(peak == (kbin + Nt // 2) % Nt)
    frac = P[:, peak[0]] / P.sum(axis=1)
    assert np.all(frac > 0.999)


def test_dc_goes_to_center_and_zero_input_gives_zero():
    Nc, Ntpb, Nt = 2, 512, 64
    raw = np.zeros((Nc, Ntpb, 2, 2), np.int8)
    raw[1, :, 1, 0] = 10
    cfg = O.make_cfg(Nc, 2, Ntpb, 1, 8, [(Nt, 8, 1)])
    outs, _ = O.run_oracle(cfg, raw.reshape(1, -1).view(np.uint8))
    P = outs[0].reshape(-1, Nc, Nt)
    assert np.all(P[:, 0] == 0)
    assert np.all(np.argmax(P[:, 1], axis=-1) == Nt // 2)
    np.testing.assert_allclose(P[:, 1, Nt // 2], 8 * (Nt * float(np.float32(10 / 127))) ** 2, rtol=1e-12)


def test_stokes_identities_between_modes():
    c = dict(CASES["c1_mini"])
    blocks, _ = blocks_for("c1_mini")
    def run(npol, conj):
        cfg = O.make_cfg(c["Nc"], 2, c["Ntpb"], 1, 8, [(256, 4, npol)], conj=conj)
        return O.run_oracle(cfg, blocks)[0][0].reshape(-1, abs(npol), c["Nc"], 256)
    for conj in (0, 1):
        F, S, T = run(4, conj), run(-4, conj), run(1, conj)
        np.testing.assert_allclose(S[:, 0], F[:, 0] + F[:, 1], rtol=1e-12)
        np.testing.assert_allclose(S[:, 1], F[:, 0] - F[:, 1], rtol=1e-10, atol=1e-9)
        np.testing.assert_allclose(S[:, 2], F[:, 2], rtol=1e-12)
        np.testing.assert_allclose(S[:, 3], F[:, 3], rtol=1e-12)
        np.testing.assert_allclose(T[:, 0], S[:, 0], rtol=1e-12)
    F0, F1 = run(4, 0), run(4, 1)
    np.testing.assert_allclose(F1[:, 3], -F0[:, 3], rtol=1e-12)


def test_int4_nibble_order():
    # one byte per complex sample: high nibble real, low nibble imaginary
    Nc, Ntpb = 1, 16
    b = np.zeros((Nc, Ntpb, 2), np.uint8)
    b[0, 0, 0] = 0x7F   # re +7, im -1
    b[0, 1, 1] = 0x81   # re -8, im +1
    cfg = O.make_cfg(Nc, 2, Ntpb, 1, 4, [(1, 1, 4)])
    outs, _ = O.run_oracle(cfg, b.reshape(1, -1))
    F = outs[0].reshape(Ntpb, 4)  # Nd = 16 spectra of length 1
    np.testing.assert_allclose(F[0, 0], (7 / 127) ** 2 + (1 / 127) ** 2, rtol=1e-6)
    np.testing.assert_allclose(F[1, 1], (8 / 127) ** 2 + (1 / 127) ** 2, rtol=1e-6)


@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_fixtures_reproduce(name):
    c = CASES[name]
    g = load_golden(name)
    blocks, weights = blocks_for(name)
    assert np.array_equal(blocks, g["blocks"])
    cfg = O.make_cfg(c["Nc"], c["Np"], c["Ntpb"], derived_nb(c), c["nbits"], c["products"], Nant=c.get("Nant", 1),
                     conj=c["conj"], inverse=1 if c["fft_dir"] <= 0 else 0, weights=weights)
    outs, icss = O.run_oracle(cfg, blocks)
    for i, o in enumerate(outs):
        np.testing.assert_allclose(o, g[f"out{i}"], rtol=1e-12, atol=1e-12)
    for i, s in enumerate(icss):
        np.testing.assert_allclose(s, g[f"ics{i}"], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("name", ["c1_mini", "multi_pol_conj_inv", "int4_ics", "large_span"])
def test_cpu_fp32_chain_matches_oracle(name):
    from util import normalized_error
    c = CASES[name]
    g = load_golden(name)
    weights = g.get("weights")
    cfg = O.make_cfg(c["Nc"], c["Np"], c["Ntpb"], derived_nb(c), c["nbits"], c["products"], Nant=c.get("Nant", 1),
                     conj=c["conj"], inverse=1 if c["fft_dir"] <= 0 else 0, weights=weights)
    outs, icss = O.run_cpu(cfg, g["blocks"], nthreads=2)
    for i, (nt, na, npol) in enumerate(c["products"]):
        assert normalized_error(outs[i], g[f"out{i}"], npol, c["Nc"], nt) < 1e-4


@pytest.mark.parametrize("logn,npol,inverse", [(15, 1, 0), (17, 4, 1), (16, -4, 0), (3, 4, 1), (9, 1, 0)])
def test_cpu_fp32_chain_long_and_short_transforms(logn, npol, inverse):
    # the CPU chain's FFT: Stockham radix-4 up to 16384 points, the four-step
    # split above, against the FP64 oracle on the same seeded input
    from util import normalized_error
    from rawspec_gb300 import synth
    nt = 1 << logn
    ntpb = max(nt, 1 << 14)
    blocks = synth.gaussian_blocks(1, 2, ntpb, 2, sigma=20.0, seed=logn)
    cfg = O.make_cfg(2, 2, ntpb, 1, 8, [(nt, 1, npol)], inverse=inverse)
    ref = O.run_oracle(cfg, blocks)[0][0]
    got = O.run_cpu(cfg, blocks, nthreads=2)[0][0]
    assert normalized_error(got, ref, npol, 2, nt) < 1e-5
