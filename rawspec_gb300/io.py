"""ctypes mirror of include/rawspec_gb300_io.h: GUPPI RAW ingest and SIGPROC
filterbank output around the spectrometer (host-side C in librawspec.so).

Also writes synthetic GUPPI RAW files (header cards + block data), the input
format the ingest reads, for tests and examples.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Sequence

import numpy as np

from .api import RawspecContext, load_library

PKT_TAKE, PKT_END_FILE, PKT_BACKWARD, PKT_MISALIGNED = 0, 1, 2, 3
RAW_MAX_HDR = 25600


class RawHeader(C.Structure):
    """rawspec_gb300_raw_hdr (field order and types as in the C header)."""
    _fields_ = [
        ("directio", C.c_int),
        ("blocsize", C.c_size_t),
        ("npol", C.c_uint),
        ("obsnchan", C.c_uint),
        ("nbits", C.c_uint),
        ("pktidx", C.c_int64),
        ("obsfreq", C.c_double),
        ("obsbw", C.c_double),
        ("tbin", C.c_double),
        ("ra", C.c_double),
        ("dec", C.c_double),
        ("mjd", C.c_double),
        ("beam_id", C.c_int),
        ("nbeam", C.c_int),
        ("refbeam", C.c_int),
        ("nants", C.c_uint),
        ("src_name", C.c_char * 81),
        ("telescop", C.c_char * 81),
        ("hdr_pos", C.c_long),
        ("hdr_size", C.c_size_t),
    ]


class PktidxState(C.Structure):
    _fields_ = [("started", C.c_int), ("prev", C.c_int64), ("step", C.c_int64)]


class IngestStats(C.Structure):
    _fields_ = [("blocks_read", C.c_longlong), ("blocks_zero", C.c_longlong), ("buffers", C.c_longlong),
                ("stop", C.c_int)]


class FilHeader(C.Structure):
    """rawspec_gb300_fil_hdr (field order and types as in the C header)."""
    _fields_ = [
        ("machine_id", C.c_int), ("telescope_id", C.c_int), ("data_type", C.c_int), ("barycentric", C.c_int),
        ("pulsarcentric", C.c_int),
        ("src_raj", C.c_double), ("src_dej", C.c_double), ("az_start", C.c_double), ("za_start", C.c_double),
        ("fch1", C.c_double), ("foff", C.c_double),
        ("nchans", C.c_int), ("nbeams", C.c_int), ("ibeam", C.c_int), ("nbits", C.c_int),
        ("tstart", C.c_double), ("tsamp", C.c_double),
        ("nifs", C.c_int),
        ("source_name", C.c_char * 81), ("rawdatafile", C.c_char * 81),
        ("nfpc", C.c_int), ("refbeam", C.c_int),
    ]


class NetStats(C.Structure):
    _fields_ = [("dumps", C.c_longlong), ("spectra", C.c_longlong), ("packets", C.c_longlong),
                ("bytes", C.c_longlong), ("error_packets", C.c_longlong), ("seconds", C.c_double)]


_declared = False


def lib() -> C.CDLL:
    """librawspec.so with the I/O entry points declared."""
    global _declared
    L = load_library()
    if not _declared:
        P = C.POINTER(RawspecContext)
        sig = {
            "rawspec_gb300_raw_parse_header": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(RawHeader)]),
            "rawspec_gb300_raw_header_size": (C.c_size_t, [C.c_char_p, C.c_size_t, C.c_int]),
            "rawspec_gb300_raw_read_header": (C.c_long, [C.c_int, C.POINTER(RawHeader)]),
            "rawspec_gb300_raw_dms_to_decimal": (C.c_double, [C.c_char_p]),
            "rawspec_gb300_pktidx_step": (C.c_int, [C.POINTER(PktidxState), C.c_int64, C.POINTER(C.c_int64)]),
            "rawspec_gb300_ingest_geometry": (C.c_int, [C.POINTER(RawHeader), C.c_uint, C.c_uint, P,
                                                        C.POINTER(C.c_int)]),
            "rawspec_gb300_ingest_files": (C.c_int, [P, C.POINTER(C.c_char_p), C.c_int, C.c_uint, C.c_int,
                                                     C.POINTER(IngestStats)]),
            "rawspec_gb300_ingest_open": (C.c_void_p, [P, C.c_int]),
            "rawspec_gb300_ingest_stem": (C.c_int, [C.c_void_p, C.POINTER(C.c_char_p), C.c_int, C.c_uint,
                                                    C.POINTER(IngestStats)]),
            "rawspec_gb300_ingest_close": (None, [C.c_void_p]),
            "rawspec_gb300_fil_header": (C.c_long, [C.POINTER(FilHeader), C.c_void_p, C.c_size_t]),
            "rawspec_gb300_telescope_id": (C.c_int, [C.c_char_p]),
            "rawspec_gb300_fil_header_for_product": (C.c_int, [C.POINTER(RawHeader), P, C.c_int, C.c_uint,
                                                               C.c_char_p, C.POINTER(FilHeader)]),
            "rawspec_gb300_fil_writer_open": (C.c_void_p, [P, C.c_int, C.POINTER(FilHeader), C.c_char_p,
                                                           C.c_char_p, C.c_int, C.c_int, C.c_char_p]),
            "rawspec_gb300_fil_writer_close": (C.c_int, [C.c_void_p]),
            "rawspec_gb300_fil_dump_callback": (None, [P, C.c_int, C.c_int]),
            "rawspec_gb300_fil_header_padded": (C.c_long, [C.POINTER(FilHeader), C.c_void_p, C.c_size_t, C.c_int]),
            "rawspec_gb300_net_open": (C.c_int, [C.c_char_p, C.c_char_p]),
            "rawspec_gb300_net_rates": (None, [P, C.c_double, C.POINTER(C.c_double)]),
            "rawspec_gb300_net_writer_open": (C.c_void_p, [P, C.c_int, C.POINTER(FilHeader), C.c_int, C.c_double]),
            "rawspec_gb300_net_writer_stats": (C.c_int, [C.c_void_p, C.POINTER(NetStats)]),
            "rawspec_gb300_net_writer_close": (C.c_int, [C.c_void_p]),
            "rawspec_gb300_net_dump_callback": (None, [P, C.c_int, C.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _declared = True
    return L


def parse_header(text: bytes) -> RawHeader:
    h = RawHeader()
    lib().rawspec_gb300_raw_parse_header(text, len(text), C.byref(h))
    return h


def fil_header_bytes(h: FilHeader, minlen: int = 0) -> bytes:
    buf = C.create_string_buffer(4096)
    n = lib().rawspec_gb300_fil_header_padded(C.byref(h), buf, len(buf), minlen)
    if n < 0:
        raise ValueError("header larger than 4096 bytes")
    return buf.raw[:n]


# ---------------------------------------------------------------------------
# Synthetic GUPPI RAW files
# ---------------------------------------------------------------------------

def header_cards(cards: Sequence[tuple[str, object]], directio: bool = False) -> bytes:
    """80-byte header cards "KEYWORD = value" (strings quoted, numbers right
    justified), an END card, and with directio the padding to 512 bytes."""
    out = []
    for key, val in cards:
        if isinstance(val, str):
            v = f"'{val:<8}'"
            card = f"{key:<8}= {v:<20}"
        else:
            card = f"{key:<8}= {val!s:>20}"
        out.append(card.ljust(80)[:80])
    out.append("END".ljust(80))
    raw = "".join(out).encode("ascii")
    if directio:
        raw += b" " * ((-len(raw)) % 512)
    return raw


def raw_block_header(obsnchan: int, npol: int, nbits: int, ntpb: int, pktidx: int, *, directio: bool = False,
                     obsfreq: float = 1500.0, obsbw: float = -187.5, tbin: float = 5.33333333333333e-06,
                     nants: int = 1, extra: Sequence[tuple[str, object]] = ()) -> bytes:
    blocsize = 2 * npol * obsnchan * nbits // 8 * ntpb
    cards = [("BACKEND", "GUPPI"), ("TELESCOP", "GBT"), ("OBSFREQ", obsfreq), ("OBSBW", obsbw),
             ("OBSNCHAN", obsnchan), ("NPOL", npol), ("NBITS", nbits), ("TBIN", tbin), ("BLOCSIZE", blocsize),
             ("PKTIDX", pktidx), ("DIRECTIO", 1 if directio else 0), ("NANTS", nants), ("SRC_NAME", "B0329+54"),
             ("RA_STR", "03:32:59.3680"), ("DEC_STR", "+54:34:43.5700"), ("STT_IMJD", 58000),
             ("STT_SMJD", 43200), *extra]
    return header_cards(cards, directio)


def write_raw_file(path: str | Path, blocks: Sequence[np.ndarray], pktidx: Sequence[int], obsnchan: int, npol: int,
                   nbits: int, ntpb: int, directio: bool = False, **kw) -> None:
    """Writes blocks (uint8 arrays of BLOCSIZE bytes, [chan][time][pol][re,im])
    with their headers."""
    with open(path, "wb") as f:
        for b, p in zip(blocks, pktidx):
            f.write(raw_block_header(obsnchan, npol, nbits, ntpb, p, directio=directio, **kw))
            f.write(np.ascontiguousarray(b, dtype=np.uint8).tobytes())  # data follow the header directly


# ---------------------------------------------------------------------------
# SIGPROC header parsing (for checking output)
# ---------------------------------------------------------------------------

_INT_KEYS = {"machine_id", "telescope_id", "data_type", "nchans", "nbeams", "ibeam", "nbits", "nifs",
             "barycentric", "pulsarcentric"}
_STR_KEYS = {"source_name", "rawdatafile"}


def parse_fil_header(buf: bytes) -> tuple[dict, int]:
    """(keyword values, header length) of a SIGPROC header at the start of buf;
    a repeated keyword keeps its last value."""
    import struct

    def string(o):
        n = struct.unpack_from("<i", buf, o)[0]
        return buf[o + 4:o + 4 + n].decode("latin-1"), o + 4 + n

    kw, o = string(0)
    if kw != "HEADER_START":
        raise ValueError("not a SIGPROC header")
    out = {}
    while True:
        kw, o = string(o)
        if kw == "HEADER_END":
            return out, o
        if kw in _INT_KEYS:
            out[kw] = struct.unpack_from("<i", buf, o)[0]
            o += 4
        elif kw in _STR_KEYS:
            out[kw], o = string(o)
        else:
            out[kw] = struct.unpack_from("<d", buf, o)[0]
            o += 8
