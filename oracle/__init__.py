"""ORACLE (test infrastructure only).

ctypes wrapper of ``oracle/fzoracle.c``, the CPU restatement of FZ-GPU's compression
path.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker: the product library never
calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libfzoracle.so")
_lock = threading.Lock()
_lib = None

HEADER_BYTES = 64
BLOCK_CODES = 2048


def build(force: bool = False) -> str:
    """Compile the oracle (gcc, OpenMP) into oracle/_build/."""
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("fzoracle.c", "fzoracle.h")
    ):
        os.makedirs(os.path.dirname(_SO), exist_ok=True)
        subprocess.check_call(
            ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-std=c11", "-shared",
             os.path.join(_HERE, "fzoracle.c"), "-o", _SO, "-lm"])
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_SO)
            u64, u32, p = C.c_uint64, C.c_uint32, C.c_void_p
            L.fzo_ndim.restype = C.c_int
            L.fzo_ndim.argtypes = [u32, u32, u32]
            L.fzo_value_range.argtypes = [p, u64, p, p]
            L.fzo_ebx2_r.restype = C.c_float
            L.fzo_ebx2_r.argtypes = [C.c_double]
            L.fzo_ebx2.restype = C.c_float
            L.fzo_ebx2.argtypes = [C.c_double]
            L.fzo_f2u16.restype = C.c_uint16
            L.fzo_f2u16.argtypes = [C.c_float]
            L.fzo_lorenzo_construct.restype = u32
            L.fzo_lorenzo_construct.argtypes = [p, u64, u32, u32, u32, C.c_float, p, p]
            L.fzo_bitshuffle_flag.argtypes = [p, u64, p, p, p]
            L.fzo_scan_encode.restype = u64
            L.fzo_scan_encode.argtypes = [p, p, u64, p, p]
            L.fzo_layout.argtypes = [u64, C.c_int, C.c_int, p, p, p, p]
            L.fzo_compress.restype = u64
            L.fzo_compress.argtypes = [p, u64, u32, u32, u32, C.c_double, C.c_int, C.c_int, p]
            L.fzo_lorenzo_reconstruct.argtypes = [p, p, u64, u32, u32, u32, C.c_float, p]
            L.fzo_decompress.restype = C.c_int
            L.fzo_decompress.argtypes = [p, u64, p, u64]
            L.fzo_metrics.argtypes = [p, p, u64, p, p, p, p]
            L.fzo_threads.restype = C.c_int
            L.fzo_set_threads.restype = None
            L.fzo_set_threads.argtypes = [C.c_int]
            _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def cdiv(a, b):
    return (a + b - 1) // b


def ndim(x, y, z):
    return lib().fzo_ndim(x, y, z)


def threads():
    return lib().fzo_threads()


def set_threads(n: int):
    """Threads of the oracle's parallel loops from now on (calling thread)."""
    lib().fzo_set_threads(int(n))


def value_range(data):
    data = np.ascontiguousarray(data, dtype=np.float32)
    mn, mx = C.c_float(), C.c_float()
    lib().fzo_value_range(_ptr(data), data.size, C.byref(mn), C.byref(mx))
    return np.float32(mn.value), np.float32(mx.value)


def ebx2_r(eb_abs):
    return np.float32(lib().fzo_ebx2_r(eb_abs))


def ebx2(eb_abs):
    return np.float32(lib().fzo_ebx2(eb_abs))


def eb_abs_of(data, eb, rel=True):
    """fz.cu:137,149: eb * (max - min), with max-min in float."""
    if not rel:
        return float(eb), np.float32(0)
    mn, mx = value_range(data)
    rng = np.float32(mx - mn)
    return float(eb) * float(rng), rng


def lorenzo_construct(data, dims, ebx2_r_f, signum=False):
    """Codes u16[n] (and optionally the 1D signum u8[n]); returns (codes, signum, ovf)."""
    data = np.ascontiguousarray(data, dtype=np.float32).ravel()
    n = data.size
    codes = np.empty(n, np.uint16)
    sg = np.empty(n, np.uint8) if signum else None
    x, y, z = dims
    ovf = lib().fzo_lorenzo_construct(_ptr(data), n, x, y, z, float(ebx2_r_f), _ptr(codes), _ptr(sg))
    return codes, sg, int(ovf)


def bitshuffle_flag(codes):
    """Returns (S as u32[ceil(n/2)], F u32[32*ceil(n/256)], B u32[ceil(n/256)])."""
    codes = np.ascontiguousarray(codes, dtype=np.uint16)
    n = codes.size
    S = np.empty(cdiv(n, 2), np.uint32)
    nw = cdiv(n, 256)
    F = np.empty(32 * nw, np.uint32)
    B = np.empty(nw, np.uint32)
    lib().fzo_bitshuffle_flag(_ptr(codes), n, _ptr(S), _ptr(F), _ptr(B))
    return S, F, B


def scan_encode(S, F, n):
    """Returns (P u32[M+1], out u8[16*nnz], nnz)."""
    S = np.ascontiguousarray(S, dtype=np.uint32)
    F = np.ascontiguousarray(F, dtype=np.uint32)
    m = 32 * cdiv(n, 256)
    P = np.empty(m + 1, np.uint32)
    nnz = lib().fzo_scan_encode(_ptr(S), _ptr(F), n, _ptr(P), None)
    out = np.empty(16 * nnz, np.uint8)
    lib().fzo_scan_encode(_ptr(S), _ptr(F), n, None, _ptr(out))
    return P, out, int(nnz)


def layout(n, nd, mode):
    a, c, b, sc = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint32()
    lib().fzo_layout(n, nd, mode, C.byref(a), C.byref(c), C.byref(b), C.byref(sc))
    return a.value, c.value, b.value, sc.value


def max_stream_bytes(n, nd, mode):
    _, _, b, _ = layout(n, nd, mode)
    return b + 16 * 256 * (n // BLOCK_CODES)


def compress(data, dims, eb, rel=True, mode=1):
    """Full compression into the stream format; returns a u8 array."""
    data = np.ascontiguousarray(data, dtype=np.float32).ravel()
    n = data.size
    x, y, z = dims
    out = np.zeros(max_stream_bytes(n, ndim(x, y, z), mode), np.uint8)
    size = lib().fzo_compress(_ptr(data), n, x, y, z, float(eb), 1 if rel else 0, mode, _ptr(out))
    if size == 0:
        raise ValueError("oracle compress rejected the input")
    return out[:size].copy()


def lorenzo_reconstruct(codes, dims, ebx2_f, signbits=None):
    codes = np.ascontiguousarray(codes, dtype=np.uint16)
    out = np.empty(codes.size, np.float32)
    x, y, z = dims
    sb = None if signbits is None else np.ascontiguousarray(signbits, dtype=np.uint8)
    lib().fzo_lorenzo_reconstruct(_ptr(codes), _ptr(sb), codes.size, x, y, z, float(ebx2_f), _ptr(out))
    return out


def decompress(stream, n=None):
    stream = np.ascontiguousarray(stream, dtype=np.uint8)
    hdr_n = int(stream[24:32].view(np.uint64)[0])
    out = np.empty(hdr_n, np.float32)
    rc = lib().fzo_decompress(_ptr(stream), stream.size, _ptr(out), hdr_n)
    if rc != 0:
        raise ValueError(f"oracle decompress: malformed stream ({rc})")
    return out


def metrics(orig, recon):
    orig = np.ascontiguousarray(orig, dtype=np.float32).ravel()
    recon = np.ascontiguousarray(recon, dtype=np.float32).ravel()
    me, ps, nr, rg = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    lib().fzo_metrics(_ptr(orig), _ptr(recon), orig.size, C.byref(me), C.byref(ps), C.byref(nr), C.byref(rg))
    return {"max_abs_err": me.value, "psnr": ps.value, "nrmse": nr.value, "range": rg.value}


def parse_header(stream):
    s = np.ascontiguousarray(stream[:HEADER_BYTES], dtype=np.uint8)
    u32 = s.view(np.uint32)
    return {
        "magic": int(u32[0]), "version": int(s[4]) | (int(s[5]) << 8), "mode": int(s[6]),
        "ndim": int(s[7]), "x": int(u32[2]), "y": int(u32[3]), "z": int(u32[4]),
        "flags": int(u32[5]), "n": int(s[24:32].view(np.uint64)[0]),
        "eb_abs": float(s[32:40].view(np.float64)[0]),
        "ebx2_r": np.float32(s[40:44].view(np.float32)[0]),
        "ebx2": np.float32(s[44:48].view(np.float32)[0]),
        "nnz": int(s[48:56].view(np.uint64)[0]), "range": np.float32(s[56:60].view(np.float32)[0]),
        "sidecar_bytes": int(u32[15]),
    }
