"""Test infrastructure: a Python restatement of the message bytes a u-FedNL distributed client
(dopt/bin_fednl_distr_client) sends to its master in one round, the oracle for the engine's
encoder (fednl_gpu_encode_client_round).  Not part of the product.

Framing (dopt/bin_fednl_distr_client/include/UsedTypes.h:1022-1125, WorkerContextForFedNL::
prepareUpdate): one byte signal, the payload length as an unsigned LEB128 integer
(dopt/copylocal/include/MutableData.h:488-536, putUnsignedVaryingInteger), the payload bytes.
Signals (UsedTypes.h:1005-1020): 41 gradient, 42/43 Hessian indices (chunk / last chunk), 44/45
Hessian items (chunk / last chunk), 47 Lk, 48 f_i, 49 round finished.

Chunks (LocalWorkerForFedNL_TopK.h:20-35): (MTU 1500 - IP header 40 - TCP header 20 - 1 - 2) / 4 =
359 entries.
"""
from __future__ import annotations

import struct

import numpy as np

SIG_GRAD, SIG_IDX, SIG_IDX_LAST, SIG_ITEMS, SIG_ITEMS_LAST = 41, 42, 43, 44, 45
SIG_LK, SIG_FI, SIG_FINISH = 47, 48, 49
CHUNK = (1500 - 40 - 20 - 1 - 2) // 4            # 359
WIRE_LK, WIRE_FI, WIRE_FINISH, WIRE_RANDK_INDICES = 1, 2, 4, 8


def varint(n: int) -> bytes:
    """MutableData::putUnsignedVaryingInteger (MutableData.h:488-536): 7 bits per byte, low first,
    high bit set on every byte but the last."""
    out = bytearray()
    while True:
        b = n & 0x7F
        n >>= 7
        if n == 0:
            out.append(b)
            return bytes(out)
        out.append(b | 0x80)


def frame(sig: int, payload: bytes) -> bytes:
    return bytes([sig]) + varint(len(payload)) + payload


def pack2_natural(a: float, b: float) -> bytes:
    """pack2FP64NoMantissa (dopt/system/include/FloatUtils.h:193-221) as the 3 low bytes sent
    (LocalWorkerForFedNL_Natural.h:173-174)."""
    ba = struct.unpack("<Q", struct.pack("<d", a))[0]
    bb = struct.unpack("<Q", struct.pack("<d", b))[0]
    sa, ea = ba >> 63, (ba >> 52) & 0x7FF
    sb, eb = bb >> 63, (bb >> 52) & 0x7FF
    w = (sa << 23) | (ea << 12) | (sb << 11) | eb
    return struct.pack("<I", w)[:3]


def _chunked(idx, items, send_idx: bool):
    """TopK / TopLEK / RandK / RandSeqK chunk loop (LocalWorkerForFedNL_TopK.h:147-189,
    RandK.h:171-219, RandSeqK.h:172-236): indices then items per chunk of 359, the last chunk
    flagged (an empty selection still sends one empty pair)."""
    out = bytearray()
    n = len(idx)
    k = 0
    while True:
        last = not (k + CHUNK < n)
        end = n if last else k + CHUNK
        ib = np.asarray(idx[k:end], dtype="<u4").tobytes() if send_idx else b""
        out += frame(SIG_IDX_LAST if last else SIG_IDX, ib)
        out += frame(SIG_ITEMS_LAST if last else SIG_ITEMS, np.asarray(items[k:end], dtype="<f8").tobytes())
        k = end
        if last:
            return bytes(out)


def encode_client_round(compressor: str, grad, lk: float, fi: float, idx, diff_at_idx, diff_upper,
                        prescale: float, U: int, k: int, flags: int) -> bytes:
    """One client's round (LocalWorkerForFedNL_*.h of the distributed client, the FedNL body):
    gradient, Lk (Option B), the Hessian message, f_i (tracking / line search), the finished flag.

    idx: the selected flat indices in sending order; diff_at_idx: H_i - shift_i at them;
    diff_upper: the whole upper triangle in scan order (Natural / Identity)."""
    out = bytearray()
    out += frame(SIG_GRAD, np.asarray(grad, dtype="<f8").tobytes())
    if flags & WIRE_LK:
        out += frame(SIG_LK, struct.pack("<d", lk))
    if compressor in ("topk", "toplek"):
        items = np.asarray(diff_at_idx, dtype=np.float64) * prescale
        out += _chunked(idx, items, True)
    elif compressor in ("randk", "randseqk"):
        mult = float(U) / float(k)                                   # RandK.h:139
        items = np.asarray(diff_at_idx, dtype=np.float64) * (prescale * mult)
        out += _chunked(idx, items, bool(flags & WIRE_RANDK_INDICES))
    elif compressor == "natural":                                    # Natural.h:143-201
        vals = list(np.asarray(diff_upper, dtype=np.float64))
        packs = [0.0, 0.0]
        filled = 0
        count = 0
        chunk = bytearray()
        for v in vals:
            packs[filled] = v
            filled += 1
            if filled == 2:
                chunk += pack2_natural(packs[0], packs[1])
                count += 2
                filled = 0
            if count == CHUNK or count == CHUNK - 1:
                out += frame(SIG_IDX, b"") + frame(SIG_ITEMS, bytes(chunk))
                chunk = bytearray()
                count = 0
        chunk += pack2_natural(packs[0], packs[1])                   # the trailing pair
        out += frame(SIG_IDX_LAST, b"") + frame(SIG_ITEMS_LAST, bytes(chunk))
    elif compressor == "identity":                                   # Identical.h:138-167
        chunk = bytearray()
        count = 0
        for v in np.asarray(diff_upper, dtype=np.float64):
            count += 1
            chunk += struct.pack("<d", float(v) * prescale)
            if count == CHUNK:
                out += frame(SIG_IDX, b"") + frame(SIG_ITEMS, bytes(chunk))
                chunk = bytearray()
                count = 0
        out += frame(SIG_IDX_LAST, b"") + frame(SIG_ITEMS_LAST, bytes(chunk))
    else:
        raise ValueError(compressor)
    if flags & WIRE_FI:
        out += frame(SIG_FI, struct.pack("<d", fi))
    if flags & WIRE_FINISH:
        out += frame(SIG_FINISH, b"")
    return bytes(out)


def decode(buf: bytes):
    """[(signal, payload bytes)] of a framed stream."""
    out = []
    p = 0
    while p < len(buf):
        sig = buf[p]
        p += 1
        n, sh = 0, 0
        while True:
            b = buf[p]
            p += 1
            n |= (b & 0x7F) << sh
            sh += 7
            if not b & 0x80:
                break
        out.append((sig, bytes(buf[p:p + n])))
        p += n
    return out
