"""fz_compress_noalloc: compression for callers that cannot allocate device memory (for
example a framework that owns all device memory through its own pool).  Its scratch is a
fixed static array inside
the library.  This file is collected last so that a failure here comes after every other
test has run; it also passes alone in a fresh process (the first call does the per-device
set-up)."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(fz, x, dims, eb, rel, mode, out):
    nbytes = C.c_uint64(0)
    st = fz.lib().fz_compress_noalloc(C.c_void_p(x.data_ptr()), x.numel(), fz._dims(dims), float(eb),
                                      fz.EB_REL if rel else fz.EB_ABS, mode, C.c_void_p(out.data_ptr()),
                                      out.numel(), C.byref(nbytes), fz._stream_handle(None))
    return st, nbytes.value


def test_noalloc_matches_workspace_path_on_consecutive_calls(fz, synth):
    """Two calls in a row (different shapes, the second reusing the shared scratch) give
    streams byte-identical to fz_compress with a workspace."""
    cases = [(synth.peaks2d(2000, 333, seed=31, npeaks=40), (2000, 333, 1), 1e-3, True, fz.MODE_SIDECAR),
             (synth.smooth3d(60, 50, 41, seed=32), (60, 50, 41), 1e-2, True, fz.MODE_SIDECAR),
             (synth.smooth1d(30001, seed=33), (30001, 1, 1), 0.004, False, fz.MODE_COMPAT)]
    ws = fz.Workspace(max(d.size for d, *_ in cases))
    for data, dims, eb, rel, mode in cases:
        x = torch.from_numpy(data).cuda()
        cap = fz.max_compressed_bytes(x.numel(), dims, mode)
        out = torch.full((cap,), 0xCD, dtype=torch.uint8, device="cuda")
        st, nbytes = _noalloc(fz, x, dims, eb, rel, mode, out)
        assert st == fz.SUCCESS, fz.status_string(st)
        want = fz.compress(x, dims, eb, rel=rel, mode=mode, ws=ws).cpu().numpy()
        assert nbytes == want.size
        got = out[:nbytes].cpu().numpy()
        assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} bytes differ"


def test_noalloc_rejects_fields_beyond_its_scratch(fz):
    big = (1 << 26) + 2048  # past FZ_NOALLOC_MAX_ELEMS: rejected before any launch
    x = torch.zeros(16, device="cuda")
    out = torch.zeros(16, dtype=torch.uint8, device="cuda")
    st = fz.lib().fz_compress_noalloc(C.c_void_p(x.data_ptr()), big, fz._dims((big, 1, 1)), 1e-3, fz.EB_REL,
                                      fz.MODE_SIDECAR, C.c_void_p(out.data_ptr()), 1 << 40, None,
                                      fz._stream_handle(None))
    assert st == fz.INVALID_ARG


def test_noalloc_failure_without_readback_marks_the_stream(fz, synth):
    """With out_bytes NULL the call returns without waiting, so a failure found on the
    device (here NaN in a relative-eb input) is recorded in the stream: its header gets
    FZ_FLAG_FAILED and readers reject it.  The next call on the shared scratch is clean."""
    good = synth.smooth2d(700, 300, seed=34)
    bad = good.copy()
    bad[4321] = np.nan
    dims = (700, 300, 1)
    cap = fz.max_compressed_bytes(good.size, dims, fz.MODE_SIDECAR)
    for data, failed in ((bad, True), (good, False)):
        x = torch.from_numpy(data).cuda()
        out = torch.zeros(cap, dtype=torch.uint8, device="cuda")
        st = fz.lib().fz_compress_noalloc(C.c_void_p(x.data_ptr()), x.numel(), fz._dims(dims), 1e-3, fz.EB_REL,
                                          fz.MODE_SIDECAR, C.c_void_p(out.data_ptr()), cap, None,
                                          fz._stream_handle(None))
        assert st == fz.SUCCESS
        torch.cuda.synchronize()
        h = fz.parse_header(out[:64].cpu().numpy())
        assert bool(h.flags & fz.FLAG_FAILED) == failed
        if failed:
            with pytest.raises(fz.FzError) as e:
                fz.stream_bytes(h)
            assert e.value.status == fz.CORRUPT_STREAM
        else:
            want = fz.compress(x, dims, 1e-3).cpu().numpy()
            assert np.array_equal(out[: want.size].cpu().numpy(), want)
