"""Parity cases shared by the golden-fixture generator and the tests.

Each case is a small, seeded configuration of the spectrometer: the input
format and shape, the products (Nt, Na, Npolout) and the flags.  The products
are given after the library's coercions (Npolout 1 for Np == 1)."""

CASES = {
    # Config-0 shape reduced in channels: 8-bit Gaussian (sigma 16) plus a tone.
    "c1_mini": dict(Nc=3, Np=2, Ntpb=4096, nbits=8, nblocks=2, products=[(1024, 2, 1)], sigma=16.0,
                    tone=(1, 0.3, 8.0), conj=0, fft_dir=1),
    # Several products, full pol and Stokes, conjugated input, inverse FFT,
    # an integration spanning two buffers (Nt 2048, Na 2).
    "multi_pol_conj_inv": dict(Nc=2, Np=2, Ntpb=2048, nbits=8, nblocks=4,
                               products=[(64, 8, 4), (512, 4, -4), (2048, 2, 1)], sigma=20.0, conj=1, fft_dir=-1),
    # Single polarisation, 16-bit samples.
    "int16_np1": dict(Nc=2, Np=1, Ntpb=1024, nbits=16, nblocks=2, products=[(256, 2, 1), (16, 8, 1)],
                      sigma=3000.0, conj=0, fft_dir=1),
    # 4-bit packed input, two antennas of two channels, Stokes, incoherent sum.
    "int4_ics": dict(Nc=4, Np=2, Ntpb=1024, nbits=4, nblocks=2, Nant=2, products=[(256, 4, -4), (16, 32, 1)],
                     conj=0, fft_dir=1, ics=True),
    # Four-step long FFT within a block, and one spanning two blocks.
    "large_8192": dict(Nc=1, Np=2, Ntpb=8192, nbits=8, nblocks=2, products=[(8192, 1, 4)], sigma=16.0, conj=1,
                       fft_dir=1),
    "large_span": dict(Nc=2, Np=2, Ntpb=4096, nbits=8, nblocks=4, products=[(16384, 1, 1), (1024, 4, 1)],
                       sigma=16.0, conj=0, fft_dir=1),
    # FFTs spanning two blocks in the small kernel (Ntpb 512 < Nt 1024).
    "span_small": dict(Nc=2, Np=2, Ntpb=512, nbits=8, nblocks=4, products=[(1024, 2, 1), (32, 16, 4)],
                       sigma=16.0, conj=0, fft_dir=1),
}


def blocks_for(name: str, seed: int = 11):
    """Seeded input bytes of a case ([nblocks, block_bytes] uint8) and weights."""
    from rawspec_gb300 import synth
    c = CASES[name]
    if c["nbits"] == 4:
        blocks, _gains = synth.int4_blocks(c["nblocks"], c["Nc"], c["Ntpb"], c["Np"], Nant=c.get("Nant", 1),
                                           seed=seed)
    else:
        blocks = synth.gaussian_blocks(c["nblocks"], c["Nc"], c["Ntpb"], c["Np"], sigma=c.get("sigma", 16.0),
                                       seed=seed, nbits=c["nbits"], tone=c.get("tone"))
    weights = synth.weights(c["Nant"], seed=seed + 1) if c.get("ics") else None
    return blocks, weights


def derived_nb(c) -> int:
    ntmax = max(p[0] for p in c["products"])
    return 1 if ntmax < c["Ntpb"] else ntmax // c["Ntpb"]
