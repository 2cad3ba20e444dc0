"""fz_gpu_gb300 -- Python host mirror of the GB300-native FZ pipeline.

Every call goes through the C ABI of ``libfzgb300.so`` (``include/fz.h``); torch is
used only for device memory and streams.  There is no CPU fallback: if the library is
missing or no CUDA device is present the calls raise ``FzError``.

The operator surface mirrors the reference's:
  * ``compress`` / ``decompress``      -- runSzs (fz.cu:113-224) and its inverse
  * ``lorenzo_construct`` / ``_reconstruct`` -- launch_{construct,reconstruct}_LorenzoI_var
                                           (lorenzo_var.cuh:520-673)
  * ``bitshuffle_flag``                -- bitshuffleAndBitflag (fz.cu:61-111)
  * ``scan_encode``                    -- cub ExclusiveSum + encodeDebug (fz.cu:49-59,187-205)
  * ``reference_sizes``                -- the three lines fz-gpu prints (fz.cu:207-209)
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfzgb300.so")
CLI_PATH = os.path.join(HERE, "fz-gpu")

# fz_status (include/fz.h)
SUCCESS = 0x00
INVALID_ARG = 0x0200
CORRUPT_STREAM = 0x0201
OUT_OF_SPACE = 0x0202
TIMEOUT = 0x0203
NONFINITE_INPUT = 0x0205
MODE_COMPAT, MODE_SIDECAR = 0, 1
FLAG_CODE_OVERFLOW, FLAG_FAILED = 0x1, 0x2  # fz_header.flags
EB_ABS, EB_REL = 0, 1
HEADER_BYTES = 64
BLOCK_CODES = 2048


class FzError(RuntimeError):
    def __init__(self, what, status):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} (0x{status:x})")


class Dims(C.Structure):
    _fields_ = [("x", C.c_uint32), ("y", C.c_uint32), ("z", C.c_uint32)]


class Header(C.Structure):
    _fields_ = [("magic", C.c_uint32), ("version", C.c_uint16), ("mode", C.c_uint8),
                ("ndim", C.c_uint8), ("x", C.c_uint32), ("y", C.c_uint32), ("z", C.c_uint32),
                ("flags", C.c_uint32), ("n", C.c_uint64), ("eb_abs", C.c_double),
                ("ebx2_r", C.c_float), ("ebx2", C.c_float), ("nnz", C.c_uint64),
                ("range", C.c_float), ("sidecar_bytes", C.c_uint32)]


assert C.sizeof(Header) == HEADER_BYTES


class Field(C.Structure):
    _fields_ = [("src", C.c_void_p), ("dst", C.c_void_p), ("n", C.c_uint64), ("dims", Dims),
                ("eb", C.c_double), ("dst_capacity", C.c_uint64), ("src_bytes", C.c_uint64),
                ("header", Header)]


COMPRESS, DECOMPRESS = 0, 1


class Request(C.Structure):
    _fields_ = [("id", C.c_uint64), ("dir", C.c_int), ("src", C.c_void_p), ("dst", C.c_void_p),
                ("n", C.c_uint64), ("dims", Dims), ("eb", C.c_double), ("eb_mode", C.c_int),
                ("mode", C.c_int), ("dst_capacity", C.c_uint64), ("src_bytes", C.c_uint64),
                ("flags", C.c_uint32), ("header", C.POINTER(Header))]


REQUEST_DEVICE = 1  # FZ_REQUEST_DEVICE: src and dst are device pointers


class Completion(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int), ("bytes", C.c_uint64)]

_lock = threading.Lock()
_lib = None

# every symbol include/fz.h declares, with its ctypes signature
_P, _U64, _U32, _I, _D = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int, C.c_double
_PU64 = C.POINTER(C.c_uint64)
SIGNATURES = {
    "fz_status_string": (C.c_char_p, [_I]),
    "fz_version": (C.c_char_p, []),
    "fz_ndim": (_I, [Dims]),
    "fz_stream_layout": (_I, [_U64, Dims, _I, _PU64, _PU64, _PU64, C.POINTER(C.c_uint32)]),
    "fz_max_compressed_bytes": (_I, [_U64, Dims, _I, _PU64]),
    "fz_stream_bytes": (_I, [C.POINTER(Header), _PU64]),
    "fz_reference_sizes": (_I, [_U64, _U64, _PU64, _PU64, C.POINTER(C.c_double)]),
    "fz_workspace_create": (_I, [_U64, C.POINTER(_P)]),
    "fz_workspace_destroy": (_I, [_P]),
    "fz_workspace_bytes": (_I, [_U64, _PU64]),
    "fz_workspace_status": (_I, [_P, _P]),
    "fz_selftest_wait_timeout": (_I, [_P, _P]),
    "fz_workspace_enable_timing": (_I, [_P, _U32]),
    "fz_workspace_kernel_time": (_I, [_P, _I, C.POINTER(C.c_uint32), C.POINTER(C.c_double)]),
    "fz_compress": (_I, [_P, _P, _U64, Dims, _D, _I, _I, _P, _U64, _PU64, _P]),
    "fz_decompress": (_I, [_P, _P, _U64, C.POINTER(Header), _P, _U64, _P]),
    "fz_compress_noalloc": (_I, [_P, _U64, Dims, _D, _I, _I, _P, _U64, _PU64, _P]),
    "fz_compress_host": (_I, [_P, _P, _U64, Dims, _D, _I, _I, _P, _U64, _PU64, _P]),
    "fz_decompress_host": (_I, [_P, _P, _U64, _P, _U64, _P]),
    "fz_lorenzo_construct": (_I, [_P, _P, _P, Dims, _D, _P]),
    "fz_lorenzo_reconstruct": (_I, [_P, _P, _P, Dims, _D, _P]),
    "fz_bitshuffle_flag": (_I, [_P, _P, _U64, _P, _P, _P]),
    "fz_scan_encode": (_I, [_P, _P, _P, _U64, _P, _P, _PU64, _P]),
    "fz_compress_batch": (_I, [_P, _P, _U32, _I, _I, _P]),
    "fz_decompress_batch": (_I, [_P, _P, _U32, _P]),
    "fz_batch_create": (_I, [_P, _P, _U32, _I, _I, _I, C.POINTER(_P)]),
    "fz_batch_launch": (_I, [_P, _P]),
    "fz_batch_destroy": (_I, [_P]),
    "fz_batch_create_ex": (_I, [_P, _P, _U32, _I, _I, _I, _U32, C.POINTER(_P)]),
    "fz_batch_create_pair": (_I, [_P, _P, _P, _U32, _I, _I, _U32, C.POINTER(_P)]),
    "fz_batch_autotune": (_I, [_P, _P, _U32, _I, _I, _I, _U32, _P, C.POINTER(_U32), C.POINTER(C.c_double)]),
    "fz_batch_create_sched": (_I, [_P, _P, _P, _U32, _I, _I, C.c_void_p, C.POINTER(_P)]),
    "fz_batch_autotune_sched": (_I, [_P, _P, _P, _U32, _I, _I, _U32, _P, C.c_void_p, C.POINTER(C.c_double)]),
    "fz_server_create": (_I, [_U64, _U32, _U64, C.POINTER(_P)]),
    "fz_server_submit": (_I, [_P, C.POINTER(Request)]),
    "fz_server_poll": (_I, [_P, C.POINTER(Completion), _U32, C.POINTER(C.c_uint32)]),
    "fz_server_pending": (_I, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), _PU64]),
    "fz_server_destroy": (_I, [_P]),
}


def lib():
    """Load libfzgb300.so (fails loudly when it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise FzError("libfzgb300.so is not built (run __graft_entry__.build())", 0x0204)
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype, f.argtypes = res, args
            _lib = L
    return _lib


def status_string(st):
    try:
        return lib().fz_status_string(st).decode()
    except FzError:
        return f"status {st}"


def _check(what, st):
    if st != SUCCESS:
        raise FzError(what, st)


def _dims(dims):
    x, y, z = (tuple(dims) + (1, 1))[:3]
    return Dims(int(x), int(y), int(z))


def ndim(dims):
    return lib().fz_ndim(_dims(dims))


def _stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def stream_layout(n, dims, mode=MODE_SIDECAR):
    a, c, b, sc = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint32()
    _check("fz_stream_layout", lib().fz_stream_layout(n, _dims(dims), mode, C.byref(a), C.byref(c), C.byref(b), C.byref(sc)))
    return a.value, c.value, b.value, sc.value


def max_compressed_bytes(n, dims, mode=MODE_SIDECAR):
    v = C.c_uint64()
    _check("fz_max_compressed_bytes", lib().fz_max_compressed_bytes(n, _dims(dims), mode, C.byref(v)))
    return v.value


def reference_sizes(file_bytes, nnz):
    """(original, compressed, ratio) exactly as fz-gpu prints them (fz.cu:207-209)."""
    o, c, r = C.c_uint64(), C.c_uint64(), C.c_double()
    _check("fz_reference_sizes", lib().fz_reference_sizes(file_bytes, nnz, C.byref(o), C.byref(c), C.byref(r)))
    return o.value, c.value, r.value


def parse_header(buf) -> Header:
    """Header of a stream held in a host buffer (bytes / numpy / CPU tensor)."""
    import numpy as np
    b = bytes(np.asarray(buf[:HEADER_BYTES]).astype(np.uint8).tobytes()) if not isinstance(buf, (bytes, bytearray)) else bytes(buf[:HEADER_BYTES])
    return Header.from_buffer_copy(b)


def stream_bytes(h: Header):
    v = C.c_uint64()
    _check("fz_stream_bytes", lib().fz_stream_bytes(C.byref(h), C.byref(v)))
    return v.value


class Workspace:
    """Device scan state + decode scratch for fields of up to ``max_n`` elements.
    One workspace per stream; calls on one workspace are stream-ordered."""

    def __init__(self, max_n):
        self.max_n = int(max_n)
        h = C.c_void_p()
        _check("fz_workspace_create", lib().fz_workspace_create(self.max_n, C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().fz_workspace_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def status(self, stream=None):
        return lib().fz_workspace_status(self.handle, _stream_handle(stream))

    def selftest_wait_timeout(self, stream=None):
        """Status of a look-back that waits on a tile nothing publishes (FZ_TIMEOUT)."""
        return lib().fz_selftest_wait_timeout(self.handle, _stream_handle(stream))

    # timing kinds of fz_workspace_kernel_time, by the kernels they time:
    # k_encode_fields<ND> and k_decompress{1,2,3}d are templated / specialised per
    # dimensionality
    KERNELS = ("k_range_fields", "k_encode_fields", "k_offsets", "k_decompress", "k_recon", "k_compact_fields")

    def enable_timing(self, capacity):
        _check("fz_workspace_enable_timing", lib().fz_workspace_enable_timing(self.handle, int(capacity)))

    def kernel_time(self, kind):
        """(launches, total ms) recorded for one kernel kind since the last query."""
        k = self.KERNELS.index(kind) if isinstance(kind, str) else int(kind)
        n, ms = C.c_uint32(), C.c_double()
        _check("fz_workspace_kernel_time", lib().fz_workspace_kernel_time(self.handle, k, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    @staticmethod
    def bytes_for(max_n):
        v = C.c_uint64()
        _check("fz_workspace_bytes", lib().fz_workspace_bytes(int(max_n), C.byref(v)))
        return v.value


def _ws_for(ws, n):
    return ws if ws is not None else Workspace(n)


def compress(x, dims, eb, rel=True, mode=MODE_SIDECAR, ws=None, out=None, stream=None, readback=True):
    """Compress a CUDA float32 tensor ``x`` (n elements, x-fastest ``dims``).

    Returns the stream as a CUDA uint8 tensor trimmed to its size (``readback=True``,
    one sync), or the untrimmed output buffer (``readback=False``, no sync)."""
    import torch
    x = x.contiguous().view(-1)
    if x.dtype != torch.float32 or not x.is_cuda:
        raise FzError("compress wants a CUDA float32 tensor", INVALID_ARG)
    n = x.numel()
    cap = max_compressed_bytes(n, dims, mode)
    if out is None:
        out = torch.empty(cap, dtype=torch.uint8, device=x.device)
    ws = _ws_for(ws, n)
    nbytes = C.c_uint64(0)
    st = lib().fz_compress(ws.handle, C.c_void_p(x.data_ptr()), n, _dims(dims), float(eb),
                           EB_REL if rel else EB_ABS, mode, C.c_void_p(out.data_ptr()), out.numel(),
                           C.byref(nbytes) if readback else None, _stream_handle(stream))
    _check("fz_compress", st)
    return out[: nbytes.value] if readback else out


def decompress(stream_t, header=None, out=None, ws=None, stream=None):
    """Decompress a stream held in a CUDA uint8 tensor; returns a CUDA float32 tensor."""
    import torch
    if header is None:
        header = parse_header(stream_t[:HEADER_BYTES].cpu().numpy())
    n = header.n
    if out is None:
        out = torch.empty(n, dtype=torch.float32, device=stream_t.device)
    ws = _ws_for(ws, n)
    st = lib().fz_decompress(ws.handle, C.c_void_p(stream_t.data_ptr()), stream_t.numel(), C.byref(header),
                             C.c_void_p(out.data_ptr()), out.numel(), _stream_handle(stream))
    _check("fz_decompress", st)
    return out


def compress_host(x_np, dims, eb, rel=True, mode=MODE_SIDECAR, ws=None, out_np=None):
    """Host-buffer compression (H2D + compress + D2H); returns a uint8 numpy array."""
    import numpy as np
    x_np = np.ascontiguousarray(x_np, dtype=np.float32).ravel()
    n = x_np.size
    cap = max_compressed_bytes(n, dims, mode)
    if out_np is None:
        out_np = np.empty(cap, np.uint8)
    ws = _ws_for(ws, n)
    nbytes = C.c_uint64(0)
    st = lib().fz_compress_host(ws.handle, x_np.ctypes.data_as(C.c_void_p), n, _dims(dims), float(eb),
                                EB_REL if rel else EB_ABS, mode, out_np.ctypes.data_as(C.c_void_p),
                                out_np.size, C.byref(nbytes), None)
    _check("fz_compress_host", st)
    return out_np[: nbytes.value]


def decompress_host(stream_np, ws=None, out_np=None):
    import numpy as np
    stream_np = np.ascontiguousarray(stream_np, dtype=np.uint8)
    h = parse_header(stream_np)
    if out_np is None:
        out_np = np.empty(h.n, np.float32)
    ws = _ws_for(ws, h.n)
    st = lib().fz_decompress_host(ws.handle, stream_np.ctypes.data_as(C.c_void_p), stream_np.size,
                                  out_np.ctypes.data_as(C.c_void_p), out_np.size, None)
    _check("fz_decompress_host", st)
    return out_np


# ------------------------------------------------------------ stage drop-ins
def lorenzo_construct(data, dims, eb_abs, signum=False, quant=None, stream=None):
    """u16 sign-magnitude codes of ``data`` (launch_construct_LorenzoI_var).  Codes at
    i >= x*y*z are left as given in ``quant`` (zeros when allocated here)."""
    import torch
    data = data.contiguous().view(-1)
    if quant is None:
        quant = torch.zeros(data.numel(), dtype=torch.int16, device=data.device)
    sg = torch.zeros(data.numel(), dtype=torch.uint8, device=data.device) if signum else None
    st = lib().fz_lorenzo_construct(C.c_void_p(data.data_ptr()), C.c_void_p(quant.data_ptr()),
                                    C.c_void_p(sg.data_ptr()) if sg is not None else None,
                                    _dims(dims), float(eb_abs), _stream_handle(stream))
    _check("fz_lorenzo_construct", st)
    return (quant, sg) if signum else quant


def lorenzo_reconstruct(quant, dims, eb_abs, signum=None, out=None, stream=None):
    import torch
    nl = int(dims[0]) * int(dims[1]) * int(dims[2])
    if out is None:
        out = torch.empty(nl, dtype=torch.float32, device=quant.device)
    st = lib().fz_lorenzo_reconstruct(C.c_void_p(quant.data_ptr()),
                                      C.c_void_p(signum.data_ptr()) if signum is not None else None,
                                      C.c_void_p(out.data_ptr()), _dims(dims), float(eb_abs), _stream_handle(stream))
    _check("fz_lorenzo_reconstruct", st)
    return out


def bitshuffle_flag(codes, stream=None):
    """(shuffled, bitflag u32[ceil(n/256)], byteflag u32[32 ceil(n/256)]) of u16 codes."""
    import torch
    n = codes.numel()
    nw = (n + 255) // 256
    words = (n + 1) // 2
    src = codes
    if n % 2:
        src = torch.zeros(n + 1, dtype=codes.dtype, device=codes.device)
        src[:n] = codes
    out = torch.zeros(2 * words, dtype=codes.dtype, device=codes.device)
    bit = torch.empty(nw, dtype=torch.int32, device=codes.device)
    byte = torch.empty(32 * nw, dtype=torch.int32, device=codes.device)
    st = lib().fz_bitshuffle_flag(C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()), n,
                                  C.c_void_p(bit.data_ptr()), C.c_void_p(byte.data_ptr()), _stream_handle(stream))
    _check("fz_bitshuffle_flag", st)
    return out[:n], bit, byte


def scan_encode(shuffled, byteflag, n_codes, ws=None, stream=None):
    """(presum u32[M+1], compacted chunks u8[16 nnz], nnz)."""
    import torch
    m = 32 * ((n_codes + 255) // 256)
    pre = torch.empty(m + 1, dtype=torch.int32, device=shuffled.device)
    out = torch.empty(16 * m, dtype=torch.uint8, device=shuffled.device)  # d_out's size, fz.cu:165
    ws = _ws_for(ws, max(n_codes, 1))
    nnz = C.c_uint64()
    st = lib().fz_scan_encode(ws.handle, C.c_void_p(shuffled.data_ptr()), C.c_void_p(byteflag.data_ptr()),
                              n_codes, C.c_void_p(pre.data_ptr()), C.c_void_p(out.data_ptr()),
                              C.byref(nnz), _stream_handle(stream))
    _check("fz_scan_encode", st)
    return pre, out[: 16 * nnz.value], nnz.value


# ------------------------------------------------------------------ batches
def fields_array(items):
    """ctypes array of Field from dicts with the struct's keys."""
    arr = (Field * len(items))()
    for i, it in enumerate(items):
        f = arr[i]
        f.src = it.get("src")
        f.dst = it.get("dst")
        f.n = int(it.get("n", 0))
        f.dims = _dims(it.get("dims", (1, 1, 1)))
        f.eb = float(it.get("eb", 0.0))
        f.dst_capacity = int(it.get("dst_capacity", 0))
        f.src_bytes = int(it.get("src_bytes", 0))
        if it.get("header") is not None:
            f.header = it["header"]
    return arr


def compress_batch(ws, fields, rel=True, mode=MODE_SIDECAR, stream=None):
    _check("fz_compress_batch", lib().fz_compress_batch(ws.handle, fields, len(fields), EB_REL if rel else EB_ABS,
                                                        mode, _stream_handle(stream)))


def decompress_batch(ws, fields, stream=None):
    _check("fz_decompress_batch", lib().fz_decompress_batch(ws.handle, fields, len(fields), _stream_handle(stream)))


def batch_autotune(ws, fields, direction, rel=True, mode=MODE_SIDECAR, reps=3, stream=None):
    """fz_batch_autotune: (best branch count, {branches: mean replay ms}) for these fields."""
    best, ms = C.c_uint32(), (C.c_double * 5)()
    _check("fz_batch_autotune", lib().fz_batch_autotune(ws.handle, fields, len(fields), direction,
                                                        EB_REL if rel else EB_ABS, mode, int(reps),
                                                        _stream_handle(stream), C.byref(best), ms))
    return best.value, {b: ms[i] for i, b in enumerate((1, 2, 4, 8, 16)) if ms[i] > 0}


class Schedule(C.Structure):
    """fz_batch_schedule: parallel branches, and whether the compression runs as list
    launches over all fields."""
    _fields_ = [("branches", C.c_uint32), ("list", C.c_uint32)]


def batch_autotune_schedule(ws, comp=None, dec=None, rel=True, mode=MODE_SIDECAR, reps=3, stream=None):
    """fz_batch_autotune_sched: (best Schedule, {(branches, list): mean replay ms})."""
    best, ms = Schedule(), (C.c_double * 10)()
    n = len(comp) if comp is not None else len(dec)
    _check("fz_batch_autotune_sched", lib().fz_batch_autotune_sched(ws.handle, comp, dec, n, EB_REL if rel else EB_ABS,
                                                                    mode, int(reps), _stream_handle(stream),
                                                                    C.byref(best), ms))
    return best, {((1, 2, 4, 8, 16)[i % 5], i // 5): ms[i] for i in range(10) if ms[i] > 0}


class Batch:
    """A batch recorded once into a CUDA graph (fz_batch_create / fz_batch_create_ex with
    `branches` parallel branches, 0 = default) and replayed."""

    def __init__(self, ws, fields, direction, rel=True, mode=MODE_SIDECAR, branches=0):
        self.ws, self.fields = ws, fields  # keep the buffers' owners alive
        h = C.c_void_p()
        _check("fz_batch_create_ex", lib().fz_batch_create_ex(ws.handle, fields, len(fields), direction,
                                                              EB_REL if rel else EB_ABS, mode, int(branches),
                                                              C.byref(h)))
        self.handle = h

    @classmethod
    def pair(cls, ws, comp, dec, rel=True, mode=MODE_SIDECAR, branches=0):
        """Round-trip batch (fz_batch_create_pair): comp[i] compressed, then dec[i]
        decompressed, per field on one branch."""
        self = cls.__new__(cls)
        self.ws, self.fields = ws, (comp, dec)
        h = C.c_void_p()
        _check("fz_batch_create_pair", lib().fz_batch_create_pair(ws.handle, comp, dec, len(comp),
                                                                  EB_REL if rel else EB_ABS, mode, int(branches),
                                                                  C.byref(h)))
        self.handle = h
        return self

    @classmethod
    def scheduled(cls, ws, comp=None, dec=None, schedule=None, rel=True, mode=MODE_SIDECAR):
        """fz_batch_create_sched: compression of comp and/or decompression of dec under a
        Schedule (default: 8 branches, per-field compression)."""
        self = cls.__new__(cls)
        self.ws, self.fields = ws, (comp, dec)
        sch = schedule if schedule is not None else Schedule(0, 0)
        n = len(comp) if comp is not None else len(dec)
        h = C.c_void_p()
        _check("fz_batch_create_sched", lib().fz_batch_create_sched(ws.handle, comp, dec, n, EB_REL if rel else EB_ABS,
                                                                    mode, C.byref(sch), C.byref(h)))
        self.handle = h
        return self

    def launch(self, stream=None):
        _check("fz_batch_launch", lib().fz_batch_launch(self.handle, _stream_handle(stream)))

    def close(self):
        if self.handle:
            lib().fz_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ serving
class Server:
    """Request loop with continuous batching under an HBM budget (fz_server_*).
    Requests use host buffers, or device buffers with device=True (FZ_REQUEST_DEVICE);
    keep them alive until their completion is polled.  submit and poll may be called
    from several threads; a completion goes to whichever thread polls it."""

    def __init__(self, hbm_budget, slots, max_n):
        import threading
        h = C.c_void_p()
        _check("fz_server_create", lib().fz_server_create(int(hbm_budget), int(slots), int(max_n), C.byref(h)))
        self.handle = h
        self._tls = threading.local()  # completion buffer per polling thread

    def submit(self, rid, direction, src, dst, dst_capacity, n=0, dims=(1, 1, 1), eb=0.0, rel=True,
               mode=MODE_SIDECAR, src_bytes=0, device=False, header=None):
        """``header``: the Header of a device-resident stream to decompress (saves the
        server a header fetch); fz_server_submit copies the request and the header."""
        r = Request(int(rid), int(direction), src, dst, int(n), _dims(dims), float(eb),
                    EB_REL if rel else EB_ABS, int(mode), int(dst_capacity), int(src_bytes),
                    REQUEST_DEVICE if device else 0, C.pointer(header) if header is not None else None)
        _check("fz_server_submit", lib().fz_server_submit(self.handle, C.byref(r)))

    def poll(self):
        """Retire finished requests and admit queued ones; returns [(id, status, bytes)]."""
        out = getattr(self._tls, "out", None)
        if out is None:
            out = self._tls.out = (Completion * 256)()
        cnt = C.c_uint32()
        _check("fz_server_poll", lib().fz_server_poll(self.handle, out, 256, C.byref(cnt)))
        return [(out[i].id, out[i].status, out[i].bytes) for i in range(cnt.value)]

    def pending(self):
        q, r, u = C.c_uint32(), C.c_uint32(), C.c_uint64()
        _check("fz_server_pending", lib().fz_server_pending(self.handle, C.byref(q), C.byref(r), C.byref(u)))
        return q.value, r.value, u.value

    def close(self):
        if self.handle:
            lib().fz_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
