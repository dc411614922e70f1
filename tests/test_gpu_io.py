"""GUPPI RAW in, SIGPROC filterbank out, through the GPU path: the ingest
(include/rawspec_gb300_io.h) reads a two-file stem with a missing packet
index and DIRECTIO padding, selects a channel range, puts in a zero block
for the gap and hands full buffers to the library; the filterbank writer,
installed as the dump callback, writes the dumps.  The files must hold
exactly the dumps the library produces when fed the same block sequence
directly."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from rawspec_gb300 import api, io

pytestmark = pytest.mark.gpu

OBSNCHAN, NP, NBITS, NTPB = 8, 2, 8, 8192
SCHAN, NCHAN = 2, 4
PRODUCTS = [(16384, 1, 1), (1024, 8, 4)]
PKTIDX = [0, 64, 128, 256, 320]   # 192 is missing
FILES = [(0, 3, False), (3, 5, True)]  # blocks of each file, DIRECTIO


def _blocks():
    rng = np.random.default_rng(17)
    v = np.clip(np.rint(rng.standard_normal((len(PKTIDX), OBSNCHAN, NTPB, NP, 2)) * 20), -128, 127)
    return v.astype(np.int8)


def test_raw_stem_to_filterbank_files(cuda_device, tmp_path):
    blocks = _blocks()
    paths = []
    for k, (a, b, dio) in enumerate(FILES):
        p = tmp_path / f"stem.{k:04d}.raw"
        io.write_raw_file(p, [blocks[i].view(np.uint8).reshape(-1) for i in range(a, b)], PKTIDX[a:b], OBSNCHAN, NP,
                          NBITS, NTPB, directio=dio)
        paths.append(p)

    L = io.lib()
    first = io.RawHeader()
    fd = os.open(paths[0], os.O_RDONLY)
    assert L.rawspec_gb300_raw_read_header(fd, C.byref(first)) > 0
    os.close(fd)

    ctx = api.RawspecContext()
    expand4 = C.c_int(0)
    assert L.rawspec_gb300_ingest_geometry(C.byref(first), SCHAN, NCHAN, C.byref(ctx), C.byref(expand4)) == 0
    assert (ctx.Nc, ctx.Np, ctx.Ntpb, ctx.Nbps, ctx.input_conjugated, expand4.value) == (NCHAN, NP, NTPB, 8, 1, 0)
    ctx.No = len(PRODUCTS)
    for i, (nt, na, npol) in enumerate(PRODUCTS):
        ctx.Nts[i], ctx.Nas[i], ctx.Npolout[i] = nt, na, npol
    assert L.rawspec_initialize(C.byref(ctx)) == 0
    writers = []
    try:
        for i in range(ctx.No):
            h = io.FilHeader()
            assert L.rawspec_gb300_fil_header_for_product(C.byref(first), C.byref(ctx), i, SCHAN, b"stem.0000.raw",
                                                          C.byref(h)) == 0
            w = L.rawspec_gb300_fil_writer_open(C.byref(ctx), i, C.byref(h), str(tmp_path).encode(), b"out", i, 0,
                                                None)
            assert w
            writers.append((w, io.fil_header_bytes(h)))
        arr = (C.c_void_p * len(writers))(*[w for w, _ in writers])
        ctx.user_data = C.cast(arr, C.c_void_p)
        ctx.dump_callback = C.cast(L.rawspec_gb300_fil_dump_callback, api.DUMP_CALLBACK)
        plist = (C.c_char_p * len(paths))(*[str(p).encode() for p in paths])
        st = io.IngestStats()
        assert L.rawspec_gb300_ingest_files(C.byref(ctx), plist, len(paths), SCHAN, expand4.value, C.byref(st)) == 0
        assert (st.blocks_read, st.blocks_zero, st.buffers, st.stop) == (5, 1, 3, 0)
    finally:
        for w, _ in writers:
            assert L.rawspec_gb300_fil_writer_close(w) == 0
        L.rawspec_cleanup(C.byref(ctx))

    # the same block sequence, fed directly: data blocks and one zero block
    seq = [blocks[0], blocks[1], blocks[2], np.zeros_like(blocks[0]), blocks[3], blocks[4]]
    host = np.stack([b[SCHAN:SCHAN + NCHAN] for b in seq]).view(np.uint8).reshape(len(seq), -1)
    spec = api.Spectrometer(NCHAN, NP, NTPB, 8, PRODUCTS, conj=1)
    try:
        spec.process(host, combined=True)
        want = [np.concatenate([np.asarray(d, dtype=np.float32).reshape(-1) for d in spec.dumps[i]])
                for i in range(len(PRODUCTS))]
    finally:
        spec.close()
    for i, (_, hdr) in enumerate(writers):
        raw = (tmp_path / f"out.rawspec.{i:04d}.fil").read_bytes()
        assert raw[:len(hdr)] == hdr
        got = np.frombuffer(raw[len(hdr):], dtype=np.float32)
        assert got.size == want[i].size
        np.testing.assert_array_equal(got, want[i])


def test_ingest_handle_streams_several_stems(cuda_device, tmp_path):
    # one handle, the same stem twice with the integration reset between:
    # the second pass's dumps repeat the first's (both host-block sets are
    # used, the context's own blocks are restored after each stem)
    blocks = _blocks()
    paths = []
    for k, (a, b, dio) in enumerate(FILES):
        p = tmp_path / f"stem.{k:04d}.raw"
        io.write_raw_file(p, [blocks[i].view(np.uint8).reshape(-1) for i in range(a, b)], PKTIDX[a:b], OBSNCHAN, NP,
                          NBITS, NTPB, directio=dio)
        paths.append(p)
    L = io.lib()
    first = io.RawHeader()
    fd = os.open(paths[0], os.O_RDONLY)
    assert L.rawspec_gb300_raw_read_header(fd, C.byref(first)) > 0
    os.close(fd)
    spec = api.Spectrometer(NCHAN, NP, NTPB, 8, PRODUCTS, conj=1)  # collects the dumps
    try:
        own = [spec.ctx.h_blkbufs[b] for b in range(spec.ctx.Nb)]
        ing = L.rawspec_gb300_ingest_open(C.byref(spec.ctx), 0)
        assert ing
        plist = (C.c_char_p * len(paths))(*[str(p).encode() for p in paths])
        st = io.IngestStats()
        try:
            assert L.rawspec_gb300_ingest_stem(ing, plist, len(paths), SCHAN, C.byref(st)) == 0
            n1 = [len(d) for d in spec.dumps]
            assert L.rawspec_reset_integration(C.byref(spec.ctx)) == 0
            assert L.rawspec_gb300_ingest_stem(ing, plist, len(paths), SCHAN, C.byref(st)) == 0
        finally:
            L.rawspec_gb300_ingest_close(ing)
        assert [spec.ctx.h_blkbufs[b] for b in range(spec.ctx.Nb)] == own
        assert (st.blocks_read, st.blocks_zero, st.buffers) == (5, 1, 3)
        for i in range(len(PRODUCTS)):
            d = [np.asarray(x) for x in spec.dumps[i]]
            assert len(d) == 2 * n1[i]
            for a, b in zip(d[:n1[i]], d[n1[i]:]):
                np.testing.assert_array_equal(a, b)
    finally:
        spec.close()


def test_dumps_over_udp_equal_the_direct_dumps(cuda_device):
    # the UDP sender as the dump callback of a GPU context: the packets of
    # every dump, reassembled, equal the dumps of the same buffers collected
    # directly
    import socket

    Nc, Ntpb, nbuf = 4, 1 << 15, 4
    prods = [(1024, 8, 1), (64, 256, 1)]
    rng = np.random.default_rng(23)
    blocks = np.clip(np.rint(rng.standard_normal((nbuf, Nc, Ntpb, NP, 2)) * 20), -128, 127).astype(np.int8)
    host = blocks.view(np.uint8).reshape(nbuf, -1)
    spec = api.Spectrometer(Nc, NP, Ntpb, 8, prods)
    try:
        spec.process(host)
        want = [[np.array(d) for d in p] for p in spec.dumps]
    finally:
        spec.close()

    rx = socket.socket(socket.AF_INET, socket.SOCK_DGRAM)
    rx.setsockopt(socket.SOL_SOCKET, socket.SO_RCVBUF, 32 << 20)
    rx.bind(("127.0.0.1", 0))
    L = io.lib()
    fd = L.rawspec_gb300_net_open(b"127.0.0.1", str(rx.getsockname()[1]).encode())
    assert fd >= 0
    ctx = api.make_context(Nc, NP, Ntpb, 8, prods)
    assert L.rawspec_initialize(C.byref(ctx)) == 0
    rates = (C.c_double * len(prods))()
    L.rawspec_gb300_net_rates(C.byref(ctx), 50.0, rates)
    writers = []
    try:
        for i, (nt, na, npol) in enumerate(prods):
            h = io.FilHeader()
            h.nchans, h.nbits, h.nifs, h.fch1, h.foff, h.tsamp = Nc * nt, 32, 1, 1500.0, -0.001, 1e-3 * i + 1e-3
            h.rawdatafile = f"product{i}".encode()
            w = L.rawspec_gb300_net_writer_open(C.byref(ctx), i, C.byref(h), fd, rates[i])
            assert w
            writers.append(w)
        arr = (C.c_void_p * len(writers))(*writers)
        ctx.user_data = C.cast(arr, C.c_void_p)
        ctx.dump_callback = C.cast(L.rawspec_gb300_net_dump_callback, api.DUMP_CALLBACK)
        nbytes = Nc * Ntpb * NP * 2
        for b in range(nbuf):
            assert L.rawspec_wait_for_completion(C.byref(ctx)) == 0
            C.memmove(ctx.h_blkbufs[0], host[b].ctypes.data, nbytes)
            assert L.rawspec_copy_blocks_to_gpu_and_start_processing(C.byref(ctx), 1, 0, 1) == 0
        assert L.rawspec_wait_for_completion(C.byref(ctx)) == 0
    finally:
        for w in writers:
            assert L.rawspec_gb300_net_writer_close(w) == 0
        L.rawspec_cleanup(C.byref(ctx))
        os.close(fd)
    rx.setblocking(False)
    got = {i: [] for i in range(len(prods))}
    while True:
        try:
            p = rx.recv(1 << 17)
        except BlockingIOError:
            break
        hdr, hl = io.parse_fil_header(p)
        got[int(hdr["rawdatafile"][-1])].append(np.frombuffer(p[hl:], dtype=np.float32))
    rx.close()
    for i in range(len(prods)):
        stream = np.concatenate(got[i])
        assert stream.size == sum(d.size for d in want[i]) > 0
        np.testing.assert_array_equal(stream, np.concatenate(want[i]))
