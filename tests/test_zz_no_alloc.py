"""The allocation-free entry point rawspec_gb300_product_noalloc against the
regular path (rawspec_initialize + rawspec_start_processing) on the same
input, through the C-ABI, and against the FP64 oracle.

Callers that cannot allocate device memory (a pipeline thread that must not
stall on cudaMalloc's device-wide synchronisation, or a framework that owns
all device memory) use this entry point; it keeps its scratch in a static
device array shared by all calls.  Calls in a row with different
configurations check that nothing stale in the shared scratch leaks from one
call into the next.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from rawspec_gb300 import api, synth
from util import REL_TOL, normalized_error

pytestmark = pytest.mark.gpu


def entry(lib):
    f = lib.rawspec_gb300_product_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_ulonglong, C.c_uint, C.c_uint, C.c_int, C.c_int,
                  C.c_int, C.POINTER(C.c_float), C.c_void_p]
    return f


def regular_path(blocks, c):
    spec = api.Spectrometer(c["Nc"], c["Np"], c["Ntpb"], c["nbits"], [(c["nt"], c["na"], c["npol"])], conj=c["conj"])
    try:
        assert spec.Nb == 1
        spec.process(blocks, fft_dir=c["fft_dir"])
        return np.array(spec.dumps[0])
    finally:
        spec.close()


def noalloc_path(f, blocks, c):
    import torch
    d_in = torch.from_numpy(blocks[0].copy()).cuda()
    nd = c["Ntpb"] // (c["nt"] * c["na"])
    out = torch.full((nd * abs(c["npol"]) * c["Nc"] * c["nt"],), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = f(C.c_void_p(d_in.data_ptr()), c["Nc"], c["Np"], c["nbits"], c["Ntpb"], c["nt"], c["na"], c["npol"],
           c["fft_dir"], c["conj"], C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_float)), C.c_void_p(stream))
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()[None, :]


def oracle_path(blocks, c):
    cfg = O.make_cfg(c["Nc"], c["Np"], c["Ntpb"], 1, c["nbits"], [(c["nt"], c["na"], c["npol"])], conj=c["conj"],
                     inverse=1 if c["fft_dir"] <= 0 else 0)
    return O.run_oracle(cfg, blocks)[0][0]


# Calls in a row on the shared scratch: one long integration per channel
# split over many CTAs (partial sums in the scratch); another length, mode and
# direction; single polarisation 16-bit samples; many short integrations that
# need no split (each CTA writes its units directly); and a Stokes product
# whose first-choice split would overflow the 4 MiB of partial sums, so that
# the split is reduced until it fits.
CALLS = [
    dict(Nc=2, Np=2, nbits=8, Ntpb=65536, nt=256, na=256, npol=1, conj=0, fft_dir=1, seed=31),
    dict(Nc=3, Np=2, nbits=8, Ntpb=32768, nt=1024, na=16, npol=-4, conj=1, fft_dir=-1, seed=32),
    dict(Nc=2, Np=1, nbits=16, Ntpb=32768, nt=512, na=8, npol=1, conj=0, fft_dir=1, seed=33),
    dict(Nc=64, Np=2, nbits=8, Ntpb=16384, nt=64, na=4, npol=4, conj=0, fft_dir=1, seed=34),
    dict(Nc=8, Np=2, nbits=8, Ntpb=524288, nt=4096, na=128, npol=-4, conj=0, fft_dir=1, seed=35),
]


def _blocks(c):
    sigma = 3000.0 if c["nbits"] == 16 else 20.0
    return synth.gaussian_blocks(1, c["Nc"], c["Ntpb"], c["Np"], sigma=sigma, seed=c["seed"], nbits=c["nbits"])


def test_noalloc_matches_regular_path_and_oracle_in_a_row(cuda_device):
    f = entry(api.load_library())
    for c in CALLS:
        blocks = _blocks(c)
        want = regular_path(blocks, c)
        got = noalloc_path(f, blocks, c)
        assert got.shape == want.shape, (c, got.shape, want.shape)
        assert np.all(np.isfinite(got)), c
        err = normalized_error(got, want, c["npol"], c["Nc"], c["nt"])
        assert err < REL_TOL, (c, err)
        if c["Nc"] * c["Ntpb"] <= 4 << 20:
            ref = oracle_path(blocks, c)[None, :]
            erro = normalized_error(got, ref, c["npol"], c["Nc"], c["nt"])
            print(f"Nt {c['nt']} Npolout {c['npol']}: vs regular path {err:.2e}, vs FP64 oracle {erro:.2e}")
            assert erro < REL_TOL, (c, erro)


def test_noalloc_rejects_invalid_requests(cuda_device):
    import torch
    f = entry(api.load_library())
    d_in = torch.zeros(1 << 16, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1 << 16, dtype=torch.float32, device="cuda")
    pin, pout = d_in.data_ptr(), C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_float))
    ok = (pin, 1, 2, 8, 4096, 256, 4, 1, 1, 0, pout, None)
    assert f(*ok) == 0
    torch.cuda.synchronize()
    bad = [
        (pin, 1, 2, 8, 1 << 14, 8192, 1, 1, 1, 0, pout, None),   # Nt above the 4096-entry twiddle scratch
        (pin, 1, 2, 8, 4096, 256, 4, 2, 1, 0, pout, None),       # Npolout 2
        (pin, 1, 1, 8, 4096, 256, 4, 4, 1, 0, pout, None),       # full pol of one polarisation
        (pin + 2, 1, 2, 8, 4096, 256, 4, 1, 1, 0, pout, None),   # input not aligned to a sample word
        (pin, 1, 2, 8, 4096, 256, 3, 1, 1, 0, pout, None),       # Nt * Na does not divide the samples
        (pin, 1, 2, 8, 4096, 300, 4, 1, 1, 0, pout, None),       # Nt not a power of two
    ]
    for args in bad:
        assert f(*args) == 1, args
