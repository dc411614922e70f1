"""The drop-in boundary, checked on the CPU: the library loads, exports every
function include/*.h declares, its context has the reference's exact layout
(fixture made from the reference header), and the host-side validation
reproduces the reference's rules (rawspec_gpu.cu:471-641, :732-760)."""
import ctypes as C
import json
import re
import subprocess
from pathlib import Path

import pytest

from rawspec_gb300 import api

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"


def declared_functions() -> set[str]:
    """Function names declared by the public headers (prototypes only)."""
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = "\n".join(l for l in text.splitlines() if not l.lstrip().startswith("#"))
        text = text.replace('extern "C" {', "")
        for stmt in text.split(";"):
            stmt = stmt.strip()
            if not stmt or stmt.startswith("typedef") or "(" not in stmt or "{" in stmt:
                continue
            m = re.search(r"([A-Za-z_]\w*)\s*\($", stmt[: stmt.index("(") + 1])
            if m:
                names.add(m.group(1))
    return names


def test_library_exports_every_declared_function():
    lib = api.load_library()
    declared = declared_functions()
    assert set(api.REFERENCE_ENTRY_POINTS) <= declared
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing


def test_exports_nothing_else():
    out = subprocess.run(["nm", "-D", "--defined-only", str(api.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if l.split()[1] == "T"}
    assert exported == declared_functions()


def test_context_layout_matches_reference(tmp_path):
    exe = tmp_path / "abi_probe"
    subprocess.run(["gcc", "-O0", f"-I{ROOT / 'include'}", "-o", str(exe), str(GOLDEN / "abi_probe.c")], check=True)
    ours = json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    ref = json.loads((GOLDEN / "abi_layout.json").read_text())
    assert ours == ref


def test_ctypes_mirror_matches_reference_layout():
    ref = json.loads((GOLDEN / "abi_layout.json").read_text())
    for name, (off, size) in ref.items():
        if name in ("sizeof",) or name.isupper() or name.startswith("RAWSPEC"):
            continue
        f = getattr(api.RawspecContext, name)
        assert (f.offset, f.size) == (off, size), name
    assert C.sizeof(api.RawspecContext) == ref["sizeof"][0]


def test_version_strings():
    lib = api.load_library()
    assert lib.get_librawspec_version().decode()
    assert "native" in lib.get_cufft_version().decode()


def validate(**kw):
    lib = api.load_library()
    products = kw.pop("products")
    ctx = api.make_context(products=products, **kw)
    rc = lib.rawspec_gb300_validate(C.byref(ctx))
    return rc, ctx


def info(ctx, i):
    lib = api.load_library()
    a, b, c = C.c_uint(), C.c_uint(), C.c_uint()
    assert lib.rawspec_gb300_product_info(C.byref(ctx), i, C.byref(a), C.byref(b), C.byref(c)) == 0
    return a.value, b.value, c.value


def test_rawspectest_configuration():
    # rawspectest.c:46-84: 88 channels, 92274688-byte blocks, four products
    rc, ctx = validate(Nc=88, Np=2, Ntpb=92274688 // (2 * 2 * 88), nbits=8,
                       products=[(1 << 20, 1, 1), (8, 1 << 17, 1), (1024, 1024, 4), (1024, 1024, -4)], Nbc=1)
    assert rc == 0
    assert ctx.Ntmax == 1 << 20 and ctx.Nb == 4 and ctx.Nb_host == 4
    assert ctx.Nbc == 88 // 8  # auto batching: largest Nc/i for i <= 10 dividing Nc
    assert [ctx.Nds[i] for i in range(4)] == [1, 1, 1, 1]
    assert ctx.h_pwrbuf_size[2] == 4 * 1024 * 88 * 4
    assert info(ctx, 0) == (1, 1, 1)
    assert info(ctx, 1) == (1 << 17, 1, 1)


def test_production_configuration_derived_quantities():
    # 64 channels, 8 bit, Ntpb 524288, Nts 2^20/8/1024, Nas 51/128/3072
    rc, ctx = validate(Nc=64, Np=2, Ntpb=524288, nbits=8, products=[(1 << 20, 51, 1), (8, 128, 1), (1024, 3072, 1)])
    assert rc == 0 and ctx.Nb == 2
    assert info(ctx, 0) == (1, 51, 1)
    assert info(ctx, 1) == (131072, 1, 1024)
    assert info(ctx, 2) == (1024, 3, 1)


def test_coercions():
    rc, ctx = validate(Nc=4, Np=1, Ntpb=1024, nbits=4, products=[(64, 4, 4), (64, 4, -4), (64, 4, 2)])
    assert rc == 0
    assert list(ctx.Npolout)[:3] == [1, 1, 1]   # Np != 2 -> total power
    assert ctx.Nbps == 8                         # 4-bit input is stored back as 8
    rc, ctx = validate(Nc=4, Np=2, Ntpb=1024, nbits=0, products=[(64, 4, 3)])
    assert rc == 0 and ctx.Nbps == 8 and ctx.Npolout[0] == 1
    rc, ctx = validate(Nc=16, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1)], Nant=4, Nbc=1)
    assert rc == 0 and ctx.Nbc == 4            # auto batching by antenna
    rc, ctx = validate(Nc=16, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1)], Nant=0)
    assert rc == 0 and ctx.Nant == 1 and ctx.Nbc == 16


@pytest.mark.parametrize("kw", [
    dict(Nc=4, Np=2, Ntpb=1024, nbits=8, products=[]),                       # No = 0
    dict(Nc=4, Np=3, Ntpb=1024, nbits=8, products=[(64, 4, 1)]),             # Np = 3
    dict(Nc=4, Np=2, Ntpb=0, nbits=8, products=[(64, 4, 1)]),                # Ntpb = 0
    dict(Nc=4, Np=2, Ntpb=1024, nbits=12, products=[(64, 4, 1)]),            # Nbps = 12
    dict(Nc=4, Np=2, Ntpb=1024, nbits=8, products=[(0, 4, 1)]),              # Nt = 0
    dict(Nc=4, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1), (48, 4, 1)]), # 48 does not divide 64
    dict(Nc=4, Np=2, Ntpb=1000, nbits=8, products=[(64, 4, 1)]),             # Ntmax does not divide Ntpb
    dict(Nc=4, Np=2, Ntpb=1024, nbits=8, products=[(64, 0, 1)]),             # Na = 0
    dict(Nc=4, Np=2, Ntpb=1024, nbits=8, products=[(64, 3, 1)]),             # 64*3 does not divide 1024
    dict(Nc=4, Np=2, Ntpb=1024, nbits=8, products=[(64, 24, 1)]),            # 1024 does not divide 64*24
    dict(Nc=6, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1)], Nbc=4),      # 6 channels in batches of 4
    dict(Nc=4, Np=2, Ntpb=960, nbits=8, products=[(96, 10, 1)]),             # not a power of two (this library)
])
def test_invalid_configurations_are_rejected(kw):
    rc, _ = validate(**kw)
    assert rc == 1


def test_caller_managed_blocks_need_nb_host():
    lib = api.load_library()
    ctx = api.make_context(Nc=4, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1)])
    bufs = (C.c_void_p * 1)()
    ctx.h_blkbufs = C.cast(bufs, C.POINTER(C.c_void_p))
    assert lib.rawspec_gb300_validate(C.byref(ctx)) == 1
    ctx.Nb_host = 1
    assert lib.rawspec_gb300_validate(C.byref(ctx)) == 0


def test_incoherent_sum_weights():
    rc, _ = validate(Nc=8, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1)], Nant=4, weights=[1.0, 2.0])
    assert rc == 1   # 2 weights for 4 antennas
    rc, _ = validate(Nc=8, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1)], Nant=4, weights=[1.0])
    assert rc == 0   # one weight broadcast
    rc, _ = validate(Nc=8, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1)], Nant=4, weights=[1, 2, 3, 4])
    assert rc == 0
    rc, _ = validate(Nc=6, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1)], Nant=4, weights=[1.0])
    assert rc == 1   # 6 channels cannot be split among 4 antennas


def test_initialize_without_gpu_fails_cleanly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = api.load_library()
    ctx = api.make_context(Nc=4, Np=2, Ntpb=1024, nbits=8, products=[(64, 4, 1)])
    assert lib.rawspec_initialize(C.byref(ctx)) == 1
    assert ctx.gpu_ctx is None
