"""The C ABI without a GPU: the library loads, exports every function include/fz.h
declares, and its host-side logic (layout, sizes, header validation, status strings)
agrees with the oracle.  No call here launches a kernel."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fz.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fz_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib(fz):
    if not os.path.exists(fz.LIB_PATH):
        import __graft_entry__ as g
        g._load_build_module().build()
    return fz.lib()


def test_exports_every_declared_symbol(fz, lib):
    names = declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
        assert name in fz.SIGNATURES, f"{name} has no Python binding"
    assert set(fz.SIGNATURES) == set(names)


def test_status_strings_and_version(fz, lib):
    assert lib.fz_status_string(0) == b"success"
    assert lib.fz_status_string(0x0201) == b"corrupt stream"
    assert b"sm_103a" in lib.fz_version()


@pytest.mark.parametrize("dims,nd", [((100, 1, 1), 1), ((10, 10, 1), 2), ((4, 5, 6), 3), ((9, 1, 3), 3)])
def test_ndim_dispatch(fz, dims, nd):
    assert fz.ndim(dims) == nd


@pytest.mark.parametrize("n,dims", [(1, (1, 1, 1)), (2047, (2047, 1, 1)), (2048, (64, 32, 1)),
                                    (6480000, (3600, 1800, 1)), (15209600, (39200, 388, 1)),
                                    (25000000, (500, 500, 100)), (5000, (70, 70, 1))])
@pytest.mark.parametrize("mode", [0, 1])
def test_layout_matches_oracle(fz, oracle, n, dims, mode):
    got = fz.stream_layout(n, dims, mode)
    want = oracle.layout(n, fz.ndim(dims), mode)
    assert got == want
    assert fz.max_compressed_bytes(n, dims, mode) == oracle.max_stream_bytes(n, fz.ndim(dims), mode)


def test_reference_sizes_readme_pin(fz):
    # README.md:33-38: CESM CLDHGH 3600x1800 at 1e-3 -> 25920000 / 3105556 / 8.346332
    orig, comp, ratio = fz.reference_sizes(25920000, 187769)
    assert orig == 25920000 and comp == 3105556
    assert f"{ratio:f}" == "8.346332"
    # dataChunkSize uses ceil(2 len / 512) (fz.cu:177-178)
    assert fz.reference_sizes(4 * 257, 0)[1] == 4 * 2
    assert fz.reference_sizes(4 * 257 + 3, 1)[1] == 4 * 2 + 16  # len = fileSize/4 (fz.cu:118)


def test_invalid_arguments_rejected_on_host(fz, lib):
    h = C.c_uint64()
    assert lib.fz_max_compressed_bytes(0, fz.Dims(1, 1, 1), 1, C.byref(h)) == fz.INVALID_ARG
    assert lib.fz_max_compressed_bytes(10, fz.Dims(4, 4, 1), 1, C.byref(h)) == fz.INVALID_ARG  # x*y*z > n
    assert lib.fz_max_compressed_bytes(10, fz.Dims(0, 1, 1), 1, C.byref(h)) == fz.INVALID_ARG
    assert lib.fz_max_compressed_bytes(1 << 32, fz.Dims(1, 1, 1), 1, C.byref(h)) == fz.INVALID_ARG
    assert lib.fz_workspace_bytes(0, C.byref(h)) == fz.INVALID_ARG
    assert lib.fz_compress(None, None, 10, fz.Dims(10, 1, 1), 1e-3, 1, 1, None, 0, None, None) == fz.INVALID_ARG


def test_header_validation_against_oracle_stream(fz, oracle, synth):
    data = synth.smooth2d(300, 40, seed=3)
    st = oracle.compress(data, (300, 40, 1), 1e-3)
    h = fz.parse_header(st)
    assert (h.n, h.nnz, h.ndim) == (data.size, oracle.parse_header(st)["nnz"], 2)
    assert fz.stream_bytes(h) == st.size
    bad = fz.parse_header(st)
    bad.magic = 0
    with pytest.raises(fz.FzError):
        fz.stream_bytes(bad)
    bad = fz.parse_header(st)
    bad.sidecar_bytes += 16
    with pytest.raises(fz.FzError):
        fz.stream_bytes(bad)
    bad = fz.parse_header(st)
    bad.nnz = 256 * (data.size // 2048) + 1
    with pytest.raises(fz.FzError):
        fz.stream_bytes(bad)


def test_cli_usage_without_arguments(fz, lib):
    r = subprocess.run([fz.CLI_PATH], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def test_header_with_wrapping_dims_rejected(fz, oracle, synth):
    """Dims whose product wraps 64 bits (8 * 2^30 * 2^31 = 2^64) must not pass as a small
    field: header validation -- the check every decompression makes before it launches
    anything -- reports a corrupt stream."""
    st = oracle.compress(synth.smooth3d(20, 10, 8, seed=4), (20, 10, 8), 1e-3)
    h = fz.parse_header(st)
    h.x, h.y, h.z = 8, 1 << 30, 1 << 31
    with pytest.raises(fz.FzError) as e:
        fz.stream_bytes(h)
    assert e.value.status == fz.CORRUPT_STREAM
    h.x, h.y, h.z = 1 << 31, 1 << 31, 4  # x*y alone exceeds n
    with pytest.raises(fz.FzError):
        fz.stream_bytes(h)
    v = C.c_uint64()
    assert fz.lib().fz_max_compressed_bytes(1 << 20, fz.Dims(8, 1 << 30, 1 << 31), 1, C.byref(v)) == fz.INVALID_ARG


def test_header_marked_failed_rejected(fz, oracle, synth):
    """A stream whose compressing kernels reported a failure carries FZ_FLAG_FAILED in its
    header; readers reject it."""
    st = oracle.compress(synth.smooth2d(64, 64, seed=5), (64, 64, 1), 1e-3)
    h = fz.parse_header(st)
    assert fz.stream_bytes(h) == st.size
    h.flags |= fz.FLAG_FAILED
    with pytest.raises(fz.FzError) as e:
        fz.stream_bytes(h)
    assert e.value.status == fz.CORRUPT_STREAM
