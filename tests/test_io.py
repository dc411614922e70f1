"""The callers either side of the path, on the host: GUPPI RAW header cards,
packet-index gap handling and SIGPROC filterbank output
(include/rawspec_gb300_io.h).

Header parsing and filterbank header bytes are compared with the reference's
own rawspec_rawutils.c / rawspec_fbutils.c, compiled unchanged into
oracle/_ref (skipped where the reference sources are absent); the gap logic
and the per-product header values with restatements of the reference CLI
(rawspec.c:913-971, 800-826) written here; the dump file writer with a
context whose host buffers are filled by the test (no GPU)."""
from __future__ import annotations

import ctypes as C
import os
import struct
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

from oracle import ref_build  # noqa: E402
from rawspec_gb300 import io  # noqa: E402
from rawspec_gb300.api import RawspecContext  # noqa: E402


@pytest.fixture(scope="module")
def ref():
    path = ref_build.build()
    if path is None:
        pytest.skip("reference sources not available")
    L = C.CDLL(str(path))
    L.rawspec_raw_read_header.restype = C.c_long
    L.rawspec_raw_read_header.argtypes = [C.c_int, C.POINTER(io.RawHeader)]
    L.rawspec_raw_parse_header.restype = None
    L.rawspec_raw_parse_header.argtypes = [C.c_char_p, C.POINTER(io.RawHeader)]
    L.fb_buf_write_padded_header.restype = C.c_void_p
    L.fb_buf_write_padded_header.argtypes = [C.c_void_p, C.POINTER(io.FilHeader), C.c_int32]
    L.fb_telescope_id.restype = C.c_int
    L.fb_telescope_id.argtypes = [C.c_char_p]
    return L


def _fields(h: io.RawHeader) -> dict:
    return {name: (bytes(getattr(h, name)).rstrip(b"\0") if name in ("src_name", "telescop") else getattr(h, name))
            for name, _ in io.RawHeader._fields_}


HEADERS = {
    "plain": io.raw_block_header(64, 2, 8, 524288, 1234),
    "directio_npol4": io.raw_block_header(8, 4, 8, 8192, 77, directio=True),
    "4bit_hex_nbits": io.header_cards([("OBSFREQ", 1420.5), ("OBSBW", 100.0), ("OBSNCHAN", 16), ("NPOL", 2),
                                       ("NBITS", "0x4"), ("TBIN", "1.6D-07"), ("BLOCSIZE", 131072),
                                       ("PKTIDX", "0x10"), ("NANTS", 4), ("BEAM_ID", 3), ("NBEAM", 7),
                                       ("REFBEAM", 0), ("RA_STR", "-12:00:36"), ("DEC_STR", "-05:30"),
                                       ("SRC_NAME", "  SPACES  "), ("TELESCOP", "MeerKAT")]),
    "comments_and_case": (b"obsfreq =              1500.25 / centre frequency".ljust(80)
                          + b"OBSBW   =                -3.125 / bandwidth".ljust(80)
                          + b"NPOLS   =                     9".ljust(80)
                          + b"NPOL    =                     2".ljust(80)
                          + b"OBSNCHAN=                     4".ljust(80)
                          + b"TBIN    =                 1E-6".ljust(80)
                          + b"BLOCSIZE=                 4096".ljust(80)
                          + b"PKTIDX  =                   42".ljust(80)
                          + b"SRC_NAME= 'A/B' / quoted slash".ljust(80)
                          + b"STT_IMJD=                59000".ljust(80)
                          + b"STT_SMJD=                  100".ljust(80)
                          + b"END".ljust(80)),
    "missing_pktidx": io.header_cards([("OBSFREQ", 1.0), ("OBSBW", 1.0), ("OBSNCHAN", 1), ("NPOL", 1),
                                       ("TBIN", 1.0), ("BLOCSIZE", 512)]),
}


@pytest.mark.parametrize("name", sorted(HEADERS))
def test_raw_header_matches_reference(ref, tmp_path, name):
    text = HEADERS[name]
    data = np.arange(4096, dtype=np.uint32).astype(np.uint8).tobytes()  # data after the header
    path = tmp_path / "h.raw"
    path.write_bytes(text + data)
    got, want = io.RawHeader(), io.RawHeader()
    fd = os.open(path, os.O_RDONLY)
    try:
        pos_got = io.lib().rawspec_gb300_raw_read_header(fd, C.byref(got))
        os.lseek(fd, 0, os.SEEK_SET)
        pos_want = ref.rawspec_raw_read_header(fd, C.byref(want))
    finally:
        os.close(fd)
    assert pos_got == pos_want
    if pos_want > 0:
        assert _fields(got) == _fields(want)
    # the parse alone (every field, required or not)
    g2, w2 = io.parse_header(text), io.RawHeader()
    ref.rawspec_raw_parse_header(text + b"\0", C.byref(w2))
    for k in ("blocsize", "npol", "obsnchan", "nbits", "obsfreq", "obsbw", "tbin", "directio", "pktidx", "beam_id",
              "nbeam", "refbeam", "nants", "ra", "dec", "mjd", "src_name", "telescop"):
        assert _fields(g2)[k] == _fields(w2)[k], k


def test_raw_blocks_are_walked_like_the_reference(ref, tmp_path):
    # three blocks, the second with DIRECTIO padding: the readers agree on
    # every header offset
    path = tmp_path / "s.0000.raw"
    rng = np.random.default_rng(0)
    blocks = [rng.integers(0, 256, 2 * 2 * 4 * 256, dtype=np.uint8) for _ in range(3)]
    with open(path, "wb") as f:
        for i, b in enumerate(blocks):
            f.write(io.raw_block_header(4, 2, 8, 256, 10 * i, directio=(i == 1)))
            f.write(b.tobytes())
    seen = []
    for L, fn in ((io.lib(), "rawspec_gb300_raw_read_header"), (ref, "rawspec_raw_read_header")):
        fd = os.open(path, os.O_RDONLY)
        offs = []
        h = io.RawHeader()
        while True:
            pos = getattr(L, fn)(fd, C.byref(h))
            if pos <= 0:
                break
            offs.append((pos, h.pktidx, h.hdr_pos, h.hdr_size))
            os.lseek(fd, h.blocsize, os.SEEK_CUR)
        os.close(fd)
        seen.append(offs)
    assert seen[0] == seen[1] and len(seen[0]) == 3


def test_dms_conversion():
    f = io.lib().rawspec_gb300_raw_dms_to_decimal
    assert f(b"03:30:00") == pytest.approx(3.5)
    assert f(b"-05:30") == pytest.approx(-5.5)
    assert f(b"+10") == 10.0
    assert f(b"12::30") == pytest.approx(12.5)


def _reference_gap_walk(pktidx):
    """rawspec.c:600-605, 913-971 restated: per block, ('take', nfill),
    ('end_file',) or ('stop', reason)."""
    out = []
    prev, step = pktidx[0], 0
    for p in pktidx:
        if step == 0 and p > prev:
            step = p - prev
        if p - prev != step:
            if p < prev:
                out.append(("stop", io.PKT_BACKWARD))
                break
            if (p - prev) % step != 0:
                out.append(("stop", io.PKT_MISALIGNED))
                break
            if p == prev:
                out.append(("end_file",))
                break
            nfill = 0
            while p - prev != step:
                prev += step
                nfill += 1
            out.append(("take", nfill))
        else:
            out.append(("take", 0))
        prev = p
    return out


@pytest.mark.parametrize("seq", [
    [0, 10, 20, 30], [5, 5, 5], [0, 10, 40, 50], [0, 10, 25], [0, 10, 5], [0, 10, 20, 20, 30],
    [100, 300, 500, 1100], [7], [0, 0, 10, 20, 50],
])
def test_pktidx_gaps_follow_the_reference(seq):
    st = io.PktidxState()
    got = []
    for p in seq:
        n = C.c_int64(0)
        a = io.lib().rawspec_gb300_pktidx_step(C.byref(st), p, C.byref(n))
        if a == io.PKT_TAKE:
            got.append(("take", n.value))
        elif a == io.PKT_END_FILE:
            got.append(("end_file",))
            break
        else:
            got.append(("stop", a))
            break
    assert got == _reference_gap_walk(seq)


def _fil_hdr(**kw) -> io.FilHeader:
    h = io.FilHeader()
    defaults = dict(machine_id=20, telescope_id=6, data_type=1, src_raj=3.54982, src_dej=54.5788, fch1=1687.5,
                    foff=-2.86102294921875e-06, nchans=64 << 20, nbeams=1, ibeam=-1, nbits=32, tstart=58000.5,
                    tsamp=18.253611008, nifs=1, source_name=b"B0329+54", rawdatafile=b"guppi_58000.0000.raw")
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(h, k, v)
    return h


@pytest.mark.parametrize("kw", [{}, dict(barycentric=1, pulsarcentric=1, nifs=4),
                                dict(src_raj=-0.5, src_dej=-89.99999, source_name=b"x" * 80),
                                dict(telescope_id=-1, rawdatafile=b"", az_start=12.5, za_start=80.25)])
def test_filterbank_header_matches_reference(ref, kw):
    h = _fil_hdr(**kw)
    got = io.fil_header_bytes(h)
    buf = C.create_string_buffer(4096)
    end = ref.fb_buf_write_padded_header(buf, C.byref(h), 0)
    want = buf.raw[:end - C.addressof(buf)]
    assert got == want


def test_telescope_ids_match_reference(ref):
    for name in [b"GBT", b"gbt", b"MeerKAT", b"ATA", b"140FT", b"Parkes", b"SRT", b"FAKE", b"nowhere", b""]:
        assert io.lib().rawspec_gb300_telescope_id(name) == ref.fb_telescope_id(name), name


def _context(Nc, Nant, prods, ics=False):
    ctx = RawspecContext()
    ctx.Nc, ctx.Np, ctx.Nant = Nc, 2, Nant
    ctx.No = len(prods)
    for i, (nt, na, npol, nds) in enumerate(prods):
        ctx.Nts[i], ctx.Nas[i], ctx.Npolout[i], ctx.Nds[i] = nt, na, npol, nds
    ctx.incoherently_sum = 1 if ics else 0
    return ctx


def test_product_header_values_follow_the_reference_cli():
    raw = io.parse_header(io.raw_block_header(64, 2, 8, 524288, 0, obsfreq=1501.46484375, obsbw=-187.5, nants=1))
    ctx = _context(16, 1, [(1 << 20, 51, 1, 1), (8, 128, 4, 1)])
    ctx.Nc = 16
    for i, (nt, na, npol, _) in enumerate([(1 << 20, 51, 1, 1), (8, 128, 4, 1)]):
        h = io.FilHeader()
        assert io.lib().rawspec_gb300_fil_header_for_product(C.byref(raw), C.byref(ctx), i, 8, b"f.0000.raw",
                                                             C.byref(h)) == 0
        ncpa = raw.obsnchan // raw.nants
        foff = raw.obsbw / ncpa / nt
        fch1 = (raw.obsfreq - raw.obsbw * (ncpa - 1) / (2 * ncpa) - (nt // 2) * foff
                + (8 % ncpa) * raw.obsbw / ncpa)
        assert h.foff == foff and h.fch1 == fch1
        assert h.nchans == 16 * nt and h.nfpc == nt and h.nifs == abs(npol)
        assert h.tsamp == raw.tbin * nt * na
        assert (h.machine_id, h.data_type, h.nbits, h.nbeams, h.telescope_id) == (20, 1, 32, 1, 6)
        assert h.tstart == 58000.5 and bytes(h.source_name).rstrip(b"\0") == b"B0329+54"


def _read_fil(path, hdr_len):
    b = Path(path).read_bytes()
    return b[:hdr_len], np.frombuffer(b[hdr_len:], dtype=np.float32)


@pytest.mark.parametrize("per_antenna,ics", [(False, False), (True, False), (True, True), (False, True)])
def test_dump_writer_layout(tmp_path, per_antenna, ics):
    # [Nds][nifs][Nant][Nc/Nant][Nt] dumps: one file, one file per antenna,
    # and the incoherent sum's file, written in the reference's order
    Nant = 1 if (not per_antenna and not ics) else 2
    Nc, nt, nds, npol = 4, 8, 3, 4
    ctx = _context(Nc, Nant, [(nt, 2, npol, nds)], ics=ics)
    pwr = np.arange(nds * npol * Nc * nt, dtype=np.float32) * 0.5
    icsb = np.arange(nds * npol * (Nc // Nant) * nt, dtype=np.float32) + 1000.0
    ctx.h_pwrbuf[0] = pwr.ctypes.data_as(C.POINTER(C.c_float))
    ctx.h_pwrbuf_size[0] = pwr.nbytes
    if ics:
        ctx.h_icsbuf[0] = icsb.ctypes.data_as(C.POINTER(C.c_float))
    h = _fil_hdr(nifs=npol)
    L = io.lib()
    w = L.rawspec_gb300_fil_writer_open(C.byref(ctx), 0, C.byref(h), str(tmp_path).encode(), b"/x/stem", 0,
                                        1 if per_antenna else 0, b"/x/stem-ics")
    assert w
    arr = (C.c_void_p * 1)(w)
    ctx.user_data = C.cast(arr, C.c_void_p)
    for _ in range(2):  # two dumps of the same buffers
        L.rawspec_gb300_fil_dump_callback(C.byref(ctx), 0, 0)  # PRE
        L.rawspec_gb300_fil_dump_callback(C.byref(ctx), 0, 1)  # POST
    assert L.rawspec_gb300_fil_writer_close(w) == 0
    hdr = io.fil_header_bytes(h)
    split = Nant > 1 and (per_antenna or not ics)
    if Nant == 1:
        head, data = _read_fil(tmp_path / "stem.rawspec.0000.fil", len(hdr))
        assert head == hdr
        np.testing.assert_array_equal(data, np.concatenate([pwr, pwr]))
    elif split:
        v = pwr.reshape(nds, npol, Nant, Nc // Nant, nt)
        for a in range(Nant):
            head, data = _read_fil(tmp_path / f"stem-ant{a:03d}.rawspec.0000.fil", len(hdr))
            assert head == hdr
            one = v[:, :, a].reshape(-1)
            np.testing.assert_array_equal(data, np.concatenate([one, one]))
    else:
        assert not (tmp_path / "stem.rawspec.0000.fil").exists()
    if ics:
        head, data = _read_fil(tmp_path / "stem-ics.rawspec.0000.fil", len(hdr))
        assert head == hdr
        np.testing.assert_array_equal(data, np.concatenate([icsb, icsb]))
