"""UDP output of the dumps (rawspec_gb300_net_*, the behaviour of the
reference's rawspec_socket.c), on the host over the loopback interface: a
context whose dump buffer the test fills stands in for the GPU.

The padded SIGPROC header is compared byte for byte with the reference's own
fb_buf_write_padded_header (rawspec_fbutils.c, compiled unchanged) where the
reference sources exist."""
import ctypes as C
import os
import socket
import sys
import time
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

from oracle import ref_build  # noqa: E402
from rawspec_gb300 import io  # noqa: E402
from rawspec_gb300.api import RAWSPEC_CALLBACK_POST_DUMP, RAWSPEC_CALLBACK_PRE_DUMP, RawspecContext  # noqa: E402

FRAME = 0x6C


@pytest.fixture(scope="module")
def ref():
    path = ref_build.build()
    if path is None:
        pytest.skip("reference sources not available")
    L = C.CDLL(str(path))
    L.fb_buf_write_padded_header.restype = C.c_void_p
    L.fb_buf_write_padded_header.argtypes = [C.c_void_p, C.POINTER(io.FilHeader), C.c_int32]
    return L


def fil_hdr(nchans=64, **kw) -> io.FilHeader:
    h = io.FilHeader()
    vals = dict(machine_id=20, telescope_id=6, data_type=1, src_raj=3.54982, src_dej=54.5788, fch1=1687.5,
                foff=-0.125, nchans=nchans, nbeams=1, ibeam=-1, nbits=32, tstart=58000.5, tsamp=0.5, nifs=1,
                source_name=b"B0329+54", rawdatafile=b"guppi_58000.0000.raw")
    vals.update(kw)
    for k, v in vals.items():
        setattr(h, k, v)
    return h


@pytest.mark.parametrize("minlen", [0, 100, 353, 354, 373, 374, 433, 452, 512, 700, 1024, 2049])
def test_padded_header_matches_reference(ref, minlen):
    h = fil_hdr(barycentric=minlen % 2)
    got = io.fil_header_bytes(h, minlen)
    buf = C.create_string_buffer(8192)
    end = ref.fb_buf_write_padded_header(buf, C.byref(h), minlen)
    assert got == buf.raw[:end - C.addressof(buf)]


def test_rates_follow_data_volume():
    ctx = RawspecContext()
    ctx.No = 3
    for i, na in enumerate((51, 128, 3072)):
        ctx.Nas[i] = na
    r = (C.c_double * 3)()
    io.lib().rawspec_gb300_net_rates(C.byref(ctx), 6.0, r)
    inv = np.array([1 / 51, 1 / 128, 1 / 3072])
    np.testing.assert_allclose(list(r), 6.0 * inv / inv.sum(), rtol=1e-12)


def one_dump(nds, nchans, rate, fch1=1500.0, foff=-0.25, tstart=58000.25, tsamp=0.75, dumps=1):
    """Sends `dumps` dumps of a filled buffer to a loopback receiver; returns
    (packets as bytes, the buffer, stats, elapsed seconds)."""
    rx = socket.socket(socket.AF_INET, socket.SOCK_DGRAM)
    rx.setsockopt(socket.SOL_SOCKET, socket.SO_RCVBUF, 32 << 20)
    rx.bind(("127.0.0.1", 0))
    port = rx.getsockname()[1]
    L = io.lib()
    fd = L.rawspec_gb300_net_open(b"127.0.0.1", str(port).encode())
    assert fd >= 0
    buf = np.arange(nds * nchans, dtype=np.float32) * 0.5 + 1.0
    ctx = RawspecContext()
    ctx.No = 1
    ctx.Nds[0] = nds
    ctx.Nts[0] = nchans
    ctx.Nc = 1
    ctx.h_pwrbuf[0] = buf.ctypes.data_as(C.POINTER(C.c_float))
    ctx.h_pwrbuf_size[0] = buf.nbytes
    h = fil_hdr(nchans=nchans, fch1=fch1, foff=foff, tstart=tstart, tsamp=tsamp)
    w = L.rawspec_gb300_net_writer_open(C.byref(ctx), 0, C.byref(h), fd, rate)
    assert w
    ws = (C.c_void_p * 1)(w)
    ctx.user_data = C.cast(ws, C.c_void_p)
    t0 = time.perf_counter()
    for _ in range(dumps):
        L.rawspec_gb300_net_dump_callback(C.byref(ctx), 0, RAWSPEC_CALLBACK_PRE_DUMP)
        L.rawspec_gb300_net_dump_callback(C.byref(ctx), 0, RAWSPEC_CALLBACK_POST_DUMP)
    L.rawspec_gb300_net_dump_callback(C.byref(ctx), 0, RAWSPEC_CALLBACK_PRE_DUMP)
    elapsed = time.perf_counter() - t0
    st = io.NetStats()
    L.rawspec_gb300_net_writer_stats(w, C.byref(st))
    assert L.rawspec_gb300_net_writer_close(w) == 0
    rx.setblocking(False)
    pkts = []
    while True:
        try:
            pkts.append(rx.recv(1 << 17))
        except BlockingIOError:
            break
    rx.close()
    os.close(fd)
    return pkts, buf, st, elapsed


@pytest.mark.parametrize("nds,nchans", [(40, 64), (3, 2048), (2, 5000), (5, 3)])
def test_dump_packets(nds, nchans):
    pkts, buf, st, _ = one_dump(nds, nchans, rate=1000.0)
    # packet plan of the reference: up to 2048 floats, whole spectra when they fit
    if nchans >= 2048:
        cpp, spp = 2048, 1
    else:
        cpp, spp = nchans, min(2048 // nchans, nds)
    want_pkts = -(-nds // spp) * -(-nchans // cpp)
    assert st.packets == len(pkts) == want_pkts and st.error_packets == 0 and st.dumps == 1
    assert st.bytes == sum(len(p) for p in pkts)
    data = buf.reshape(nds, nchans)
    k = 0
    for s0 in range(0, nds, spp):
        ns = min(spp, nds - s0)
        for c0 in range(0, nchans, cpp):
            nc = min(cpp, nchans - c0)
            hdr, hl = io.parse_fil_header(pkts[k])
            assert (FRAME + hl) % 512 == 0            # data on a 512-byte boundary of the frame
            assert hdr["nchans"] == nc
            assert hdr["fch1"] == pytest.approx(1500.0 - 0.25 * c0)
            assert hdr["tstart"] == pytest.approx(58000.25 + s0 * 0.75 / 86400.0, abs=1e-10)  # summed per packet
            assert hdr["rawdatafile"] == "guppi_58000.0000.raw"
            got = np.frombuffer(pkts[k][hl:], dtype=np.float32).reshape(ns, nc)
            np.testing.assert_array_equal(got, data[s0:s0 + ns, c0:c0 + nc])
            k += 1


def test_start_time_advances_across_dumps():
    pkts, _, st, _ = one_dump(4, 1024, rate=1000.0, dumps=3)
    assert st.dumps == 3 and st.packets == len(pkts) == 6
    t = [io.parse_fil_header(p)[0]["tstart"] for p in pkts]
    step = 2 * 0.75 / 86400.0
    np.testing.assert_allclose(np.diff(t), step, rtol=1e-6)


def test_sender_paces_to_the_rate():
    rate = 0.02  # Gbit/s
    pkts, _, st, elapsed = one_dump(24, 2048, rate=rate)
    assert st.packets == len(pkts) == 24
    want = 8.0 * st.bytes / (rate * 1e9)
    assert st.seconds >= 0.95 * want and elapsed >= 0.95 * want
    assert st.seconds < want + 0.5
