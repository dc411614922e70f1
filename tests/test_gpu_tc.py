"""The tensor-core DFT kernel (k_tc: tcgen05 MMAs on FP16 hi/lo operands,
FP32 accumulation in tensor memory) against the FP64 oracle.

First the MMA building block alone: a host-built shared-memory image of two
K-major FP16 operands goes through the library's descriptors and MMA
wrappers (tests/probe/umma_probe.cu) and must give the exact integer matrix
product.  Then whole products with RAWSPEC_GB300_TENSOR_DFT=1 (the kernels
for every length they support: the one-stage k_tcs at 8, 16, 32, the
two-stage k_tc at 256, 1024, 4096), every mode, direction, integration
spanning buffers and the pipelined combined call.  The errors
against the oracle are printed (pytest -s) as well as checked."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cases import derived_nb
from oracle import oracle as O
from rawspec_gb300 import api, synth
from util import REL_TOL, normalized_error, rms_normalized_error

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
TC = api.KERNEL_CLASS_NAMES.index("tc")
SMALL = api.KERNEL_CLASS_NAMES.index("small")


def pack_kmajor(mat: np.ndarray, lbo: int, sbo: int) -> np.ndarray:
    """FP16 matrix [rows][K] -> bytes of 8-row x 16-byte core matrices:
    element (r, k) at (r//8)*sbo + (k//8)*lbo + (r%8)*16 + (k%8)*2."""
    rows, k = mat.shape
    out = np.zeros(((rows // 8 - 1) * sbo + (k // 8 - 1) * lbo + 128 + 15) // 16 * 16, np.uint8)
    h = mat.astype(np.float16).view(np.uint16)
    for r in range(rows):
        for kk in range(k):
            off = (r // 8) * sbo + (kk // 8) * lbo + (r % 8) * 16 + (kk % 8) * 2
            out[off:off + 2] = np.frombuffer(h[r, kk].tobytes(), np.uint8)
    return out


def unpack_kmajor(img: np.ndarray, off: int, rows: int, k: int, lbo: int, sbo: int) -> np.ndarray:
    h = np.zeros((rows, k), np.float32)
    for r in range(rows):
        for kk in range(k):
            o = off + (r // 8) * sbo + (kk // 8) * lbo + (r % 8) * 16 + (kk % 8) * 2
            if o + 2 <= img.size:
                h[r, kk] = np.frombuffer(img[o:o + 2].tobytes(), np.float16)[0]
    return h


@pytest.fixture(scope="module")
def probe_lib(tmp_path_factory):
    so = tmp_path_factory.mktemp("umma") / "libumma_probe.so"
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-shared", "-Xcompiler",
           "-fPIC", f"-I{ROOT / 'rawspec_gb300' / 'csrc'}", "-o", str(so), str(ROOT / "tests" / "probe" / "umma_probe.cu")]
    subprocess.run(cmd, check=True)
    return C.CDLL(str(so))


@pytest.mark.parametrize("k,n", [(32, 64), (64, 128), (128, 256)])
def test_mma_operand_layout_and_descriptors(cuda_device, probe_lib, k, n):
    rng = np.random.default_rng(k + n)
    lbo, sbo = 144, (k // 8) * 144
    A = rng.integers(-4, 5, size=(128, k)).astype(np.float32)
    B = rng.integers(-4, 5, size=(n, k)).astype(np.float32)
    ia, ib = pack_kmajor(A, lbo, sbo), pack_kmajor(B, lbo, sbo)
    img = np.concatenate([ia, ib])
    out = np.zeros((128, n), np.float32)
    rc = probe_lib.umma_probe(img.ctypes.data_as(C.c_void_p), img.size, 0, ia.size, lbo, sbo, n, k,
                              out.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == 0, rc
    want = A @ B.T
    if not np.array_equal(out, want):
        # which reading of the image would the hardware have made?
        swapped = unpack_kmajor(img, 0, 128, k, sbo, lbo) @ unpack_kmajor(img, ia.size, n, k, sbo, lbo).T
        bad = np.argwhere(out != want)
        pytest.fail(f"MMA result differs at {len(bad)} places (first {bad[:4].tolist()}); "
                    f"matches the LBO/SBO-swapped reading: {np.array_equal(out, swapped)}")


def run_tc(monkeypatch, c, blocks, combined=False, tensor=True):
    monkeypatch.setenv("RAWSPEC_GB300_TENSOR_DFT", "1" if tensor else "0")
    spec = api.Spectrometer(c["Nc"], c["Np"], c["Ntpb"], c["nbits"], c["products"], conj=c["conj"])
    try:
        spec.set_profiling(True)
        spec.process(blocks, fft_dir=c["fft_dir"], combined=combined)
        n_tc, n_small = spec.profile(TC)[1], spec.profile(SMALL)[1]
        return [np.array(d) for d in spec.dumps], n_tc, n_small
    finally:
        spec.close()


def oracle_for(c, blocks):
    cfg = O.make_cfg(c["Nc"], c["Np"], c["Ntpb"], derived_nb(c), c["nbits"], c["products"], conj=c["conj"],
                     inverse=1 if c["fft_dir"] <= 0 else 0)
    return O.run_oracle(cfg, blocks)[0]


@pytest.mark.parametrize("logn,npol,na,conj,fft_dir", [
    (3, 1, 128, 0, 1), (3, 4, 64, 1, 1), (3, -4, 256, 1, -1), (4, 1, 64, 0, -1), (4, -4, 128, 1, 1),
    (5, 1, 64, 0, 1), (5, 4, 128, 1, -1), (5, -4, 64, 0, 1),
    (8, 1, 16, 0, 1), (8, 4, 8, 1, 1), (8, -4, 64, 1, -1),
    (10, 1, 8, 0, 1), (10, 4, 2, 1, -1), (10, -4, 16, 0, 1), (10, 1, 32, 1, -1),
    (12, 1, 4, 0, 1), (12, 1, 1, 0, -1)])
def test_tensor_dft_matches_oracle(cuda_device, monkeypatch, logn, npol, na, conj, fft_dir):
    nt, Ntpb = 1 << logn, 1 << 14
    c = dict(Nc=3, Np=2, Ntpb=Ntpb, nbits=8, nblocks=2, products=[(nt, na, npol)], conj=conj, fft_dir=fft_dir)
    blocks = synth.gaussian_blocks(2, 3, Ntpb, 2, sigma=18.0, seed=700 + logn + na)
    got, n_tc, n_small = run_tc(monkeypatch, c, blocks)
    assert n_tc > 0 and n_small == 0, (n_tc, n_small)
    ref = oracle_for(c, blocks)
    assert got[0].shape == ref[0].shape
    err = normalized_error(got[0], ref[0], npol, 3, nt)
    print(f"k_tc N={nt} Npolout={npol} Na={na} conj={conj} fft_dir={fft_dir}: normalized error {err:.2e}")
    assert err < REL_TOL, (nt, npol, err)


@pytest.mark.parametrize("nt,npol", [(1024, 1), (1024, 4), (8, 1), (16, -4)])
def test_tensor_dft_integration_across_buffers(cuda_device, monkeypatch, nt, npol):
    # one block of spectra per channel per buffer, integrations of six
    # buffers (the accumulation into the dump buffer), units spread over
    # several CTAs (partial sums + k_finalize)
    Ntpb = 1 << 14
    na = 6 * Ntpb // nt
    c = dict(Nc=2, Np=2, Ntpb=Ntpb, nbits=8, nblocks=6, products=[(nt, na, npol)], conj=1, fft_dir=1)
    blocks = synth.gaussian_blocks(6, 2, Ntpb, 2, sigma=20.0, seed=811 + npol)
    got, n_tc, _ = run_tc(monkeypatch, c, blocks)
    assert n_tc > 0
    ref = oracle_for(c, blocks)
    assert got[0].shape == ref[0].shape
    err = normalized_error(got[0], ref[0], npol, 2, nt)
    print(f"k_tc N={nt} Npolout={npol} Na={na} over six buffers: normalized error {err:.2e}")
    assert err < REL_TOL


@pytest.mark.parametrize("nbits", [8, 4])
def test_tensor_dft_in_the_pipelined_call(cuda_device, monkeypatch, nbits):
    # the combined copy-and-process call launches the kernel per channel
    # group (the finer chunking); 4-bit input is expanded to 8 bits first
    Nc, Ntpb, nblocks = 8, 1 << 19, 3
    prods = [(1024, 16, 1), (256, 64, -4), (4096, 8, 1)]
    if nbits == 4:
        blocks, _ = synth.int4_blocks(nblocks, Nc, Ntpb, 2, Nant=1, seed=43)
    else:
        blocks = synth.gaussian_blocks(nblocks, Nc, Ntpb, 2, sigma=20.0, seed=43)
    c = dict(Nc=Nc, Np=2, Ntpb=Ntpb, nbits=nbits, products=prods, conj=1, fft_dir=1)
    got, n_tc, n_small = run_tc(monkeypatch, c, blocks, combined=True)
    assert n_tc >= 3 * 8 and n_small == 0, (n_tc, n_small)
    ref = oracle_for(c, blocks)
    for i, (nt, na, npol) in enumerate(prods):
        assert got[i].shape == ref[i].shape
        assert normalized_error(got[i], ref[i], npol, Nc, nt) < REL_TOL, (nbits, nt)


def test_tensor_dft_equals_plain_path_at_production_shape(cuda_device, monkeypatch):
    # 64 channels x 2^19 samples, 1024-point spectra integrated over 512:
    # the tensor-core and the CUDA-core kernels agree bin by bin
    Nc, Ntpb = 64, 1 << 19
    c = dict(Nc=Nc, Np=2, Ntpb=Ntpb, nbits=8, products=[(1024, 512, 1)], conj=0, fft_dir=1)
    blocks = synth.gaussian_blocks(1, Nc, Ntpb, 2, sigma=20.0, seed=97)
    got_tc, n_tc, _ = run_tc(monkeypatch, c, blocks)
    got_cc, n_tc2, n_small = run_tc(monkeypatch, c, blocks, tensor=False)
    assert n_tc > 0 and n_tc2 == 0 and n_small > 0
    assert normalized_error(got_tc[0], got_cc[0], 1, Nc, 1024) < 2 * REL_TOL


@pytest.mark.parametrize("npol", [1, 4])
def test_mixed_precision_products_error_report(cuda_device, monkeypatch, npol):
    # the mixed-precision configuration: Gaussian int8 voltages (sigma 16,
    # one tone), products Nfft 8/256/1024/4096 with Nint 128/256/512/3072,
    # on the tensor-core DFT where it applies (256, 1024, 4096 total power)
    # and on the CUDA-core kernels; max and RMS error per product against
    # the FP64 oracle.  Two channels and 192 blocks of 65536 samples, so
    # that the 3072 x 4096-point integration completes.
    Nc, Ntpb, nblocks = 2, 1 << 16, 192
    prods = [(8, 128, npol), (256, 256, npol), (1024, 512, npol), (4096, 3072, npol)]
    blocks = synth.gaussian_blocks(nblocks, Nc, Ntpb, 2, sigma=16.0, seed=31, tone=(1, 0.3, 8.0))
    c = dict(Nc=Nc, Np=2, Ntpb=Ntpb, nbits=8, nblocks=nblocks, products=prods, conj=0, fft_dir=1)
    ref = oracle_for(c, blocks)
    got_tc, n_tc, _ = run_tc(monkeypatch, c, blocks)
    got_cc, n_tc0, _ = run_tc(monkeypatch, c, blocks, tensor=False)
    assert n_tc > 0 and n_tc0 == 0
    for i, (nt, na, _) in enumerate(prods):
        assert got_tc[i].shape == ref[i].shape and got_tc[i].size > 0
        e = {k: (normalized_error(g[i], ref[i], npol, Nc, nt), rms_normalized_error(g[i], ref[i], npol, Nc, nt))
             for k, g in (("tensor", got_tc), ("fp32", got_cc))}
        print(f"Nfft {nt} Nint {na} Npolout {npol}: tensor-core path max {e['tensor'][0]:.2e} rms "
              f"{e['tensor'][1]:.2e}; CUDA-core path max {e['fp32'][0]:.2e} rms {e['fp32'][1]:.2e}")
        assert e["tensor"][0] < REL_TOL and e["fp32"][0] < REL_TOL, (nt, e)
