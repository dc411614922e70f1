"""The allocation-free entry point rawspec_gb300_product_noalloc against the
regular path (rawspec_initialize + rawspec_start_processing) on the same
input, through the C-ABI.

Callers that cannot allocate device memory (a pipeline thread that must not
stall on cudaMalloc's device-wide synchronisation, or a framework that owns
all device memory) use this entry point; it keeps its scratch in a static
device array shared by all calls.  Two calls in a row with different
configurations check that nothing stale in the shared scratch leaks from the
first call into the second.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from rawspec_gb300 import api, synth
from util import REL_TOL, normalized_error

pytestmark = pytest.mark.gpu


def regular_path(blocks, Nc, Ntpb, nt, na, npol, conj, fft_dir):
    spec = api.Spectrometer(Nc, 2, Ntpb, 8, [(nt, na, npol)], conj=conj)
    try:
        assert spec.Nb == 1
        spec.process(blocks, fft_dir=fft_dir)
        return np.array(spec.dumps[0])
    finally:
        spec.close()


def noalloc_path(lib, blocks, Nc, Ntpb, nt, na, npol, conj, fft_dir):
    import torch
    d_in = torch.from_numpy(blocks[0].copy()).cuda()
    nd = Ntpb // (nt * na)
    out = torch.full((nd * abs(npol) * Nc * nt,), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.rawspec_gb300_product_noalloc(C.c_void_p(d_in.data_ptr()), Nc, 2, 8, Ntpb, nt, na, npol, fft_dir, conj,
                                           C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_float)),
                                           C.c_void_p(stream))
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()[None, :]


def test_noalloc_matches_regular_path_twice(cuda_device):
    import torch  # noqa: F401
    lib = api.load_library()
    f = lib.rawspec_gb300_product_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_ulonglong, C.c_uint, C.c_uint, C.c_int, C.c_int,
                  C.c_int, C.POINTER(C.c_float), C.c_void_p]
    # call 1: one long integration per channel, split over many CTAs (the
    # static scratch holds the partial sums); call 2: another length, mode and
    # direction on the same scratch.
    calls = [
        dict(Nc=2, Ntpb=65536, nt=256, na=256, npol=1, conj=0, fft_dir=1, seed=31),
        dict(Nc=3, Ntpb=32768, nt=1024, na=16, npol=-4, conj=1, fft_dir=-1, seed=32),
    ]
    for c in calls:
        blocks = synth.gaussian_blocks(1, c["Nc"], c["Ntpb"], 2, sigma=20.0, seed=c["seed"])
        args = (blocks, c["Nc"], c["Ntpb"], c["nt"], c["na"], c["npol"], c["conj"], c["fft_dir"])
        want = regular_path(*args)
        got = noalloc_path(lib, *args)
        assert got.shape == want.shape
        assert np.all(np.isfinite(got))
        assert normalized_error(got, want, c["npol"], c["Nc"], c["nt"]) < REL_TOL


def test_noalloc_rejects_oversized_fft(cuda_device):
    lib = api.load_library()
    f = lib.rawspec_gb300_product_noalloc
    f.restype = C.c_int
    # Nt above the 4096-entry twiddle scratch is rejected before any launch
    rc = f(C.c_void_p(1), 1, 2, 8, C.c_ulonglong(1 << 16), 8192, 1, 1, 1, 0, C.cast(C.c_void_p(1), C.POINTER(C.c_float)),
           C.c_void_p(0))
    assert rc == 1
