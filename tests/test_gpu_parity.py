"""GPU parity: the sm_103a kernels, called through the C ABI, against the oracle.

Streams must be byte-identical, codes/flags/offsets bit-exact and reconstructions
bit-identical to the oracle's; reconstructions must also meet the error bound
|x - x'| <= eb (1 + 2^-21) + 2^-21 |x| at every point."""
import zlib

import numpy as np
import pytest
import torch

from conftest import error_tolerance

pytestmark = pytest.mark.gpu

BIG = 1 << 25  # workspace capacity: covers the 25M-element 3D workload


@pytest.fixture(scope="module")
def ws(fz):
    torch.cuda.set_device(0)
    return fz.Workspace(BIG)


def run_both(fz, oracle, ws, data, dims, eb, rel=True, mode=1):
    xt = torch.from_numpy(np.ascontiguousarray(data)).cuda()
    st = fz.compress(xt, dims, eb, rel=rel, mode=mode, ws=ws)
    got = st.cpu().numpy()
    want = oracle.compress(data, dims, eb, rel=rel, mode=mode)
    return st, got, want


def assert_same_stream(got, want):
    assert got.size == want.size, f"stream size {got.size} != oracle {want.size}"
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, f"{bad.size} bytes differ, first at {bad[:8]}"


SMALL = [
    ("smooth2d", (300, 70, 1), 1e-3), ("peaks2d", (400, 90, 1), 1e-4), ("smooth2d", (101, 37, 1), 1e-3),
    ("smooth2d", (1, 3000, 1), 1e-3), ("smooth2d", (17, 2049, 1), 1e-2), ("smooth3d", (40, 33, 20), 1e-3),
    ("smooth3d", (37, 19, 11), 1e-2), ("smooth3d", (33, 1, 70), 1e-3), ("smooth3d", (9, 9, 9), 1e-3),
    ("smooth3d", (7, 300, 2), 1e-3), ("smooth3d", (63, 130, 3), 1e-3), ("smooth3d", (961, 20, 9), 1e-3),
    ("smooth1d", (100000, 1, 1), 1e-3), ("smooth1d", (1500, 1, 1), 1e-3), ("smooth1d", (2048, 1, 1), 1e-3),
    ("smooth1d", (4097, 1, 1), 1e-4), ("smooth2d", (64, 32, 1), 1e-3), ("smooth1d", (7, 1, 1), 1e-3),
]


def _seed(kind, dims):
    """A seed fixed by the case (Python's str hash changes from process to process)."""
    return zlib.crc32(f"{kind}{dims}".encode()) % 1000


@pytest.mark.parametrize("kind,dims,eb", SMALL, ids=[f"{k}-{'x'.join(map(str, d))}-{e}" for k, d, e in SMALL])
@pytest.mark.parametrize("mode", [0, 1])
def test_compress_decompress_small(fz, oracle, synth, ws, kind, dims, eb, mode):
    data = synth.field(kind, dims, seed=_seed(kind, dims))
    st, got, want = run_both(fz, oracle, ws, data, dims, eb, mode=mode)
    assert_same_stream(got, want)
    rec = fz.decompress(st, ws=ws).cpu().numpy()
    rec_o = oracle.decompress(want)
    assert np.array_equal(rec.view(np.uint32), rec_o.view(np.uint32))
    if mode == 1:
        h = oracle.parse_header(want)
        assert (np.abs(rec.astype(np.float64) - data) <= error_tolerance(data, h["eb_abs"])).all()


# Row widths around the switches of the whole-block encode paths: x < 128 (positions by
# division) against x >= 128 (incremental), x a multiple of 4 or not (16-byte halo rows or
# scalar ones), rows shorter and longer than a 2048-code block, 1D lengths around whole
# blocks, and 3D rows and planes of few elements.
WIDTHS = [((x, y, 1), 1e-3) for x, y in ((4, 1500), (8, 900), (12, 700), (124, 70), (128, 64), (132, 70),
                                        (127, 66), (129, 65), (130, 66), (2044, 9), (2048, 8), (2049, 9),
                                        (2050, 9), (2051, 9), (2052, 9), (4100, 5), (5, 900), (6, 800), (7, 700))]
WIDTHS += [((n, 1, 1), 1e-3) for n in (2047, 2049, 4096, 6143, 10240 + 17)]
WIDTHS += [((x, y, z), 1e-3) for x, y, z in ((4, 4, 300), (8, 9, 40), (128, 3, 12), (132, 5, 9), (127, 8, 8),
                                             (4, 513, 2))]


@pytest.mark.parametrize("dims,eb", WIDTHS, ids=["x".join(map(str, d)) for d, _ in WIDTHS])
def test_row_width_edges(fz, oracle, synth, ws, dims, eb):
    """Streams byte-identical and reconstructions bit-identical to the oracle's at the row
    widths where the whole-block paths change method."""
    kind = {1: "smooth1d", 2: "peaks2d", 3: "smooth3d"}[fz.ndim(dims)]
    data = synth.field(kind, dims, seed=_seed(kind, dims))
    for mode in (0, 1):
        st, got, want = run_both(fz, oracle, ws, data, dims, eb, mode=mode)
        assert_same_stream(got, want)
        rec = fz.decompress(st, ws=ws).cpu().numpy()
        assert np.array_equal(rec.view(np.uint32), oracle.decompress(want).view(np.uint32))


TALL = [((4, 1 << 21, 1), 1e-3), ((6, 1 << 20, 1), 1e-3), ((8, 1 << 21, 2), 1e-3), ((5, 1 << 19, 3), 1e-2)]


@pytest.mark.parametrize("dims,eb", TALL, ids=["x".join(map(str, d)) for d, _ in TALL])
def test_tall_fields(fz, oracle, ws, dims, eb):
    """Fields with more than 65535 tile bands along y: the decompression kernels index
    their CTAs with a flat block index, so these launch and match the oracle."""
    n = dims[0] * dims[1] * dims[2]
    rng = np.random.default_rng(n)
    data = np.cumsum(rng.normal(0, 1, n)).astype(np.float32)
    st, got, want = run_both(fz, oracle, ws, data, dims, eb, mode=1)
    assert_same_stream(got, want)
    rec = fz.decompress(st, ws=ws).cpu().numpy()
    assert np.array_equal(rec.view(np.uint32), oracle.decompress(want).view(np.uint32))
    # the two-pass reconstruction kernels behind the stage API
    eb_abs = oracle.parse_header(want)["eb_abs"]
    codes, _, _ = oracle.lorenzo_construct(data, dims, oracle.ebx2_r(eb_abs))
    q = torch.from_numpy(codes.view(np.int16)).cuda()
    rec2 = fz.lorenzo_reconstruct(q, dims, eb_abs).cpu().numpy()
    rec2_o = oracle.lorenzo_reconstruct(codes, dims, oracle.ebx2(eb_abs))
    assert np.array_equal(rec2.view(np.uint32), rec2_o.view(np.uint32))


FULL = [
    ("cesm-like 3600x1800", "smooth2d", (3600, 1800, 1), 0, 1e-3),
    ("exafel-like 39200x388", "peaks2d", (39200, 388, 1), 1, 1e-3),
    ("exafel-like 39200x388", "peaks2d", (39200, 388, 1), 1, 1e-4),
    ("hurricane-like 500x500x100", "smooth3d", (500, 500, 100), 2, 1e-2),
    ("hurricane-like 500x500x100", "smooth3d", (500, 500, 100), 2, 1e-3),
    ("hurricane-like 500x500x100", "smooth3d", (500, 500, 100), 2, 1e-4),
    # rows that are not a multiple of 4 elements: the whole-block paths with per-element
    # positions and scalar halo loads, at full size
    ("cesm-like 3601x1800", "smooth2d", (3601, 1800, 1), 0, 1e-3),
    ("exafel-like 39201x388", "peaks2d", (39201, 388, 1), 1, 1e-3),
    ("hurricane-like 501x500x100", "smooth3d", (501, 500, 100), 2, 1e-3),
]


@pytest.mark.parametrize("name,kind,dims,seed,eb", FULL, ids=[f"{f[0].split()[1]}-{f[4]}" for f in FULL])
def test_full_size_workloads(fz, oracle, synth, ws, name, kind, dims, seed, eb):
    data = synth.field(kind, dims, seed)
    st, got, want = run_both(fz, oracle, ws, data, dims, eb, mode=1)
    assert_same_stream(got, want)
    rec = fz.decompress(st, ws=ws).cpu().numpy()
    rec_o = oracle.decompress(want)
    assert np.array_equal(rec.view(np.uint32), rec_o.view(np.uint32))
    h = oracle.parse_header(want)
    assert (np.abs(rec.astype(np.float64) - data) <= error_tolerance(data, h["eb_abs"])).all()
    m = oracle.metrics(data, rec)
    assert m["max_abs_err"] <= h["eb_abs"] * (1 + 2 ** -10)
    print(f"{name} eb={eb}: nnz={h['nnz']} ratio(ref)={fz.reference_sizes(4 * data.size, h['nnz'])[2]:.3f} "
          f"psnr={m['psnr']:.2f} max_err/eb={m['max_abs_err'] / h['eb_abs']:.6f}")


def test_absolute_eb_and_len_longer_than_dims(fz, oracle, synth, ws):
    d = np.concatenate([synth.smooth2d(64, 64, seed=18), np.linspace(-1, 1, 777, dtype=np.float32)])
    for rel, eb in [(False, 0.004), (True, 1e-3)]:
        st, got, want = run_both(fz, oracle, ws, d, (64, 64, 1), eb, rel=rel)
        assert_same_stream(got, want)
        rec = fz.decompress(st, ws=ws).cpu().numpy()
        assert np.array_equal(rec.view(np.uint32), oracle.decompress(want).view(np.uint32))
        assert not rec[64 * 64:].any()


def crafted(vals, nd):
    if nd == 2:
        g = np.zeros((16, 16 * vals.size), np.float32)
        g[0, ::16] = vals
        g[5, 3::16] = vals[::-1]
        return g.ravel(), (16 * vals.size, 16, 1)
    if nd == 1:
        g = np.zeros(256 * vals.size, np.float32)
        g[::256] = vals
        g[131::256] = vals[::-1]
        return g, (g.size, 1, 1)
    g = np.zeros((8, 8, 8 * vals.size), np.float32)
    g[0, 0, ::8] = vals
    g[3, 2, 5::8] = vals[::-1]
    return g.ravel(), (8 * vals.size, 8, 8)


LIMITS = np.array([0, 1, -1, 2.5, -2.5, 0.5, -0.5, 1.5, 30000, 32767, 32768, -32768, 40000, 65535,
                   65536, -65536, 70000, -70000, 1e6, -1e9, 3e38, np.inf, -np.inf, np.nan, -np.nan,
                   12345.5, -0.0, 7, 100000, 32767.5, 65535.5, 65534.7], np.float32)


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_code_field_limits_and_nonfinite(fz, oracle, ws, nd):
    """Deltas at and beyond the 15/16-bit code fields, Inf and NaN (absolute eb 0.5,
    ebx2_r = 1): codes and the overflow flag match the oracle bit for bit."""
    data, dims = crafted(LIMITS, nd)
    st, got, want = run_both(fz, oracle, ws, data, dims, 0.5, rel=False)
    assert_same_stream(got, want)
    assert oracle.parse_header(want)["flags"] & 1
    rec = fz.decompress(st, ws=ws).cpu().numpy()
    assert np.array_equal(rec.view(np.uint32), oracle.decompress(want).view(np.uint32))


def test_stage_lorenzo_construct_reconstruct(fz, oracle, synth, ws):
    for kind, dims, eb in [("smooth2d", (300, 70, 1), 1e-3), ("smooth3d", (37, 19, 11), 1e-2),
                           ("smooth1d", (5000, 1, 1), 1e-3), ("peaks2d", (513, 33, 1), 1e-4)]:
        data = synth.field(kind, dims, seed=3)
        eb_abs = eb * float(np.float32(data.max() - data.min()))
        xt = torch.from_numpy(data).cuda()
        q, sg = fz.lorenzo_construct(xt, dims, eb_abs, signum=True)
        codes, sgo, _ = oracle.lorenzo_construct(data, dims, oracle.ebx2_r(eb_abs), signum=True)
        assert np.array_equal(q.cpu().numpy().view(np.uint16), codes)
        if dims[1] == 1 and dims[2] == 1:
            assert np.array_equal(sg.cpu().numpy(), sgo)
        rec = fz.lorenzo_reconstruct(q, dims, eb_abs, signum=sg).cpu().numpy()
        sb = np.packbits(sgo, bitorder="little") if dims[1] == 1 and dims[2] == 1 else None
        rec_o = oracle.lorenzo_reconstruct(codes, dims, oracle.ebx2(eb_abs), sb)
        assert np.array_equal(rec.view(np.uint32), rec_o.view(np.uint32))


@pytest.mark.parametrize("n", [100, 2048, 5000, 3 * 2048 + 17, 40000])
def test_stage_bitshuffle_scan_encode(fz, oracle, ws, n):
    rng = np.random.default_rng(n)
    codes = (rng.random(n) < 0.05).astype(np.uint16) * rng.integers(1, 60000, n).astype(np.uint16)
    ct = torch.from_numpy(codes.view(np.int16)).cuda()
    sh, bit, byte = fz.bitshuffle_flag(ct)
    S, F, B = oracle.bitshuffle_flag(codes)
    assert np.array_equal(sh.cpu().numpy().view(np.uint16), S.view(np.uint16)[:n])
    assert np.array_equal(byte.cpu().numpy().view(np.uint32), F)
    assert np.array_equal(bit.cpu().numpy().view(np.uint32), B)
    pad = torch.zeros(2 * ((n + 1) // 2) + 16, dtype=torch.int16, device="cuda")
    pad[:n] = sh
    pre, out, nnz = fz.scan_encode(pad, byte, n, ws=ws)
    P, outo, nnzo = oracle.scan_encode(S, F, n)
    assert nnz == nnzo
    assert np.array_equal(pre.cpu().numpy().view(np.uint32), P)
    assert np.array_equal(out.cpu().numpy(), outo)


def test_host_buffer_path_matches_device_path(fz, oracle, synth, ws):
    data = synth.smooth3d(60, 50, 40, seed=4)
    st_h = fz.compress_host(data, (60, 50, 40), 1e-3, ws=ws)
    want = oracle.compress(data, (60, 50, 40), 1e-3)
    assert_same_stream(st_h, want)
    rec = fz.decompress_host(st_h, ws=ws)
    assert np.array_equal(rec.view(np.uint32), oracle.decompress(want).view(np.uint32))


def test_workspace_reuse_across_calls(fz, oracle, synth, ws):
    """Epoch-tagged scan state: back-to-back calls of different sizes on one workspace."""
    fields = [(synth.smooth2d(500, 300, seed=i), (500, 300, 1)) for i in range(2)]
    fields += [(synth.smooth1d(30000, seed=9), (30000, 1, 1)), (synth.smooth3d(30, 30, 30, seed=2), (30, 30, 30))]
    for rep in range(3):
        for data, dims in fields:
            st, got, want = run_both(fz, oracle, ws, data, dims, 1e-3)
            assert_same_stream(got, want)


@pytest.mark.parametrize("n", [5001, (1 << 22) + 3])
def test_nonfinite_input_relative_bound(fz, oracle, synth, ws, n):
    """NaN, +Inf or -Inf anywhere in a field (first element, middle, the last elements past
    the 16-byte loads) makes a relative-bound compression return FZ_NONFINITE_INPUT; the
    workspace then compresses a finite field exactly as the oracle does."""
    base = synth.smooth1d(n, seed=5)
    for bad in (np.nan, np.inf, -np.inf):
        for pos in (0, n // 2 + 1, n - 1, n - 4):
            x = base.copy()
            x[pos] = bad
            with pytest.raises(fz.FzError) as e:
                fz.compress(torch.from_numpy(x).cuda(), (n, 1, 1), 1e-3, rel=True, ws=ws)
            assert e.value.status == fz.NONFINITE_INPUT, (bad, pos)
        st, got, want = run_both(fz, oracle, ws, base, (n, 1, 1), 1e-3)
        assert_same_stream(got, want)


def test_failure_without_readback_marks_the_stream(fz, ws):
    """fz_compress without out_bytes does not wait: NaN in a relative-eb input then marks
    the header FZ_FLAG_FAILED (readers reject the stream) and the workspace status reports
    FZ_NONFINITE_INPUT; the next call's header is clean."""
    y = torch.linspace(0, 1, 9000, device="cuda")
    y[4000] = float("nan")
    out = fz.compress(y, (9000, 1, 1), 1e-3, rel=True, ws=ws, readback=False)
    torch.cuda.synchronize()
    h = fz.parse_header(out[:64].cpu().numpy())
    assert h.flags & fz.FLAG_FAILED
    with pytest.raises(fz.FzError) as e:
        fz.stream_bytes(h)
    assert e.value.status == fz.CORRUPT_STREAM
    assert ws.status() == fz.NONFINITE_INPUT
    y[4000] = 0.5
    out = fz.compress(y, (9000, 1, 1), 1e-3, rel=True, ws=ws, readback=False)
    torch.cuda.synchronize()
    assert not fz.parse_header(out[:64].cpu().numpy()).flags & fz.FLAG_FAILED
    assert ws.status() == fz.SUCCESS


def test_errors_are_statuses(fz, ws):
    x = torch.zeros(4096 + 4, device="cuda")
    out = torch.empty(1 << 16, dtype=torch.uint8, device="cuda")
    with pytest.raises(fz.FzError) as e:
        fz.compress(x[1:4097], (4096, 1, 1), 1e-3, ws=ws, out=out)  # misaligned input
    assert e.value.status == fz.INVALID_ARG
    with pytest.raises(fz.FzError) as e:
        fz.compress(x[:4096], (4096, 1, 1), 1e-3, ws=ws, out=out[:100])
    assert e.value.status == fz.OUT_OF_SPACE
    with pytest.raises(fz.FzError) as e:
        fz.compress(x[:4096], (64, 65, 1), 1e-3, ws=ws)  # x*y*z > n
    assert e.value.status == fz.INVALID_ARG
    with pytest.raises(fz.FzError) as e:
        fz.compress(x[:4096], (4096, 1, 1), -1.0, ws=ws)
    assert e.value.status == fz.INVALID_ARG
    y = torch.ones(5000, device="cuda")
    y[77] = float("nan")
    with pytest.raises(fz.FzError) as e:
        fz.compress(y, (5000, 1, 1), 1e-3, rel=True, ws=ws)
    assert e.value.status == fz.NONFINITE_INPUT
    # the workspace stays usable after an error status
    st = fz.compress(torch.linspace(0, 1, 5000, device="cuda"), (5000, 1, 1), 1e-3, ws=ws)
    assert st.numel() > 64


def test_corrupt_stream_is_detected(fz, oracle, synth, ws):
    data = synth.smooth2d(300, 70, seed=1)
    want = oracle.compress(data, (300, 70, 1), 1e-3)
    st = torch.from_numpy(want.copy()).cuda()
    bad = st.clone()
    bad[64:64 + 32] = 255  # bitmap of block 0 claims 256 chunks
    h = fz.parse_header(want)
    fz.decompress(bad, header=h, ws=ws)       # stream-ordered: the kernel flags it
    assert ws.status() == fz.CORRUPT_STREAM   # sticky until read
    assert ws.status() == fz.SUCCESS
    short = st[: want.size - 16]
    with pytest.raises(fz.FzError) as e:
        fz.decompress(short, header=h, ws=ws)
    assert e.value.status == fz.CORRUPT_STREAM


def test_bounded_wait_times_out_without_fault(fz, ws):
    """A look-back on a tile that never publishes gives up and reports FZ_TIMEOUT; the
    context stays usable."""
    assert ws.selftest_wait_timeout() == fz.TIMEOUT
    st = fz.compress(torch.linspace(0, 1, 9000, device="cuda"), (9000, 1, 1), 1e-3, ws=ws)
    assert st.numel() > 64


def _mixed_fields(synth):
    return [
        (synth.smooth2d(700, 300, seed=21), (700, 300, 1), 1e-3),
        (synth.smooth3d(40, 30, 20, seed=22), (40, 30, 20), 1e-2),
        (synth.smooth1d(50000, seed=23), (50000, 1, 1), 1e-3),
        (synth.peaks2d(1001, 77, seed=24, npeaks=20), (1001, 77, 1), 1e-4),
        (synth.smooth2d(64, 64, seed=25), (64, 64, 1), 1e-3),
    ]


def _batch_buffers(fz, items):
    xs = [torch.from_numpy(d).cuda() for d, _, _ in items]
    caps = [fz.max_compressed_bytes(d.size, dims) for d, dims, _ in items]
    ss = [torch.empty(c, dtype=torch.uint8, device="cuda") for c in caps]
    ys = [torch.empty(d.size, dtype=torch.float32, device="cuda") for d, _, _ in items]
    comp = fz.fields_array([{"src": x.data_ptr(), "dst": s.data_ptr(), "n": x.numel(), "dims": dims, "eb": eb,
                             "dst_capacity": s.numel()} for x, s, (_, dims, eb) in zip(xs, ss, items)])
    return xs, ss, ys, comp


def test_batch_calls_match_oracle(fz, oracle, synth):
    items = _mixed_fields(synth)
    ws = fz.Workspace(max(d.size for d, _, _ in items))
    xs, ss, ys, comp = _batch_buffers(fz, items)
    fz.compress_batch(ws, comp)
    wants = [oracle.compress(d, dims, eb) for d, dims, eb in items]
    for s, want in zip(ss, wants):
        assert_same_stream(s[: want.size].cpu().numpy(), want)
    dec = fz.fields_array([{"src": s.data_ptr(), "dst": y.data_ptr(), "src_bytes": w.size, "dst_capacity": y.numel(),
                            "header": fz.parse_header(w)} for s, y, w in zip(ss, ys, wants)])
    fz.decompress_batch(ws, dec)
    for y, w in zip(ys, wants):
        assert np.array_equal(y.cpu().numpy().view(np.uint32), oracle.decompress(w).view(np.uint32))
    assert ws.status() == fz.SUCCESS


def test_graph_batch_replays_are_exact(fz, oracle, synth):
    """A batch captured in a CUDA graph replays with frozen kernel parameters; the
    device-side epoch keeps every replay's scan state fresh."""
    items = _mixed_fields(synth)
    ws = fz.Workspace(max(d.size for d, _, _ in items))
    xs, ss, ys, comp = _batch_buffers(fz, items)
    wants = [oracle.compress(d, dims, eb) for d, dims, eb in items]
    g = fz.Batch(ws, comp, fz.COMPRESS)
    dec = fz.fields_array([{"src": s.data_ptr(), "dst": y.data_ptr(), "src_bytes": w.size, "dst_capacity": y.numel(),
                            "header": fz.parse_header(w)} for s, y, w in zip(ss, ys, wants)])
    gd = fz.Batch(ws, dec, fz.DECOMPRESS)
    for rep in range(4):
        for s in ss:
            s.fill_(0xAB)
        for y in ys:
            y.fill_(7.0)
        g.launch()
        gd.launch()
        torch.cuda.synchronize()
        for s, y, w in zip(ss, ys, wants):
            assert_same_stream(s[: w.size].cpu().numpy(), w)
            assert np.array_equal(y.cpu().numpy().view(np.uint32), oracle.decompress(w).view(np.uint32))
    assert ws.status() == fz.SUCCESS


def test_batch_range_ahead_edges(fz, oracle, synth):
    """Range ahead (each compression's encode launch takes the range of the next field on
    its stream): a field without full shuffle blocks (no compaction launch, so the field
    after it runs its own range launch), a 1D field with a tail, and a NaN field between
    clean ones -- the NaN marks only its own header FZ_FLAG_FAILED and reaches the workspace
    status; every other stream matches the oracle.  On one stream (fz_compress_batch) and
    on 1 and 2 graph branches (the NaN field on a branch with its own workspace), replayed
    twice."""
    nanf = synth.smooth3d(40, 30, 20, seed=32).copy()
    nanf[5000] = np.nan
    items = [
        (synth.smooth2d(700, 300, seed=31), (700, 300, 1), 1e-3),
        (synth.smooth1d(1000, seed=33), (1000, 1, 1), 1e-3),
        (synth.smooth1d(50000, seed=34), (50000, 1, 1), 1e-2),
        (nanf, (40, 30, 20), 1e-3),
        (synth.smooth2d(64, 64, seed=35), (64, 64, 1), 1e-4),
        (synth.smooth1d(2053, seed=36), (2053, 1, 1), 1e-3),
        (synth.peaks2d(1001, 77, seed=37, npeaks=20), (1001, 77, 1), 1e-3),
    ]
    bad = 3
    ws = fz.Workspace(max(d.size for d, _, _ in items))
    xs, ss, ys, comp = _batch_buffers(fz, items)
    wants = {i: oracle.compress(d, dims, eb) for i, (d, dims, eb) in enumerate(items) if i != bad}

    def check(what, status=True):
        for i, s in enumerate(ss):
            h = fz.parse_header(s[:64].cpu().numpy())
            if i == bad:
                assert h.flags & fz.FLAG_FAILED, what
            else:
                assert not h.flags & fz.FLAG_FAILED, (what, i)
                assert_same_stream(s[: wants[i].size].cpu().numpy(), wants[i])
        if status:  # the NaN field ran on the caller's workspace
            assert ws.status() == fz.NONFINITE_INPUT, what
        assert ws.status() == fz.SUCCESS, what  # reading the status clears it

    for s in ss:
        s.fill_(0x5A)
    fz.compress_batch(ws, comp)
    torch.cuda.synchronize()
    check("one stream")
    for branches in (1, 2):
        g = fz.Batch(ws, comp, fz.COMPRESS, branches=branches)
        for rep in range(2):
            for s in ss:
                s.fill_(0x3C + rep)
            g.launch()
            torch.cuda.synchronize()
            check(f"{branches} branches, replay {rep}", status=bad % branches == 0)
        g.close()
    # the workspace is clean for a single call afterwards
    d, dims, eb = items[0]
    assert_same_stream(fz.compress(xs[0], dims, eb, ws=ws).cpu().numpy(), wants[0])


def test_batch_range_ahead_stops_at_an_invalid_field(fz, oracle, synth):
    """A field whose arguments are invalid (input not 16-byte aligned) is not read ahead:
    fz_compress_batch compresses the fields before it exactly, then returns
    FZ_INVALID_ARG for it, and the workspace serves the next call normally."""
    d0 = synth.smooth2d(700, 300, seed=41)
    d1 = synth.smooth1d(50000, seed=42)
    ws = fz.Workspace(d0.size)
    x0 = torch.from_numpy(d0).cuda()
    x1 = torch.zeros(d1.size + 1, device="cuda")
    x1[1:] = torch.from_numpy(d1).cuda()
    caps = [fz.max_compressed_bytes(d0.size, (700, 300, 1)), fz.max_compressed_bytes(d1.size, (d1.size, 1, 1))]
    ss = [torch.full((c,), 0x11, dtype=torch.uint8, device="cuda") for c in caps]
    comp = fz.fields_array([
        {"src": x0.data_ptr(), "dst": ss[0].data_ptr(), "n": d0.size, "dims": (700, 300, 1), "eb": 1e-3,
         "dst_capacity": caps[0]},
        {"src": x1[1:].data_ptr(), "dst": ss[1].data_ptr(), "n": d1.size, "dims": (d1.size, 1, 1), "eb": 1e-3,
         "dst_capacity": caps[1]}])
    with pytest.raises(fz.FzError) as e:
        fz.compress_batch(ws, comp)
    assert e.value.status == fz.INVALID_ARG
    want = oracle.compress(d0, (700, 300, 1), 1e-3)
    assert_same_stream(ss[0][: want.size].cpu().numpy(), want)
    assert ws.status() == fz.SUCCESS
    want1 = oracle.compress(d1, (d1.size, 1, 1), 1e-3)
    assert_same_stream(fz.compress(x1[1:].clone(), (d1.size, 1, 1), 1e-3, ws=ws).cpu().numpy(), want1)


def test_batch_branch_counts_and_autotune(fz, oracle, synth):
    """Every branch count gives the same streams and reconstructions; the autotuner
    times the candidates on these fields and returns one of them."""
    items = _mixed_fields(synth)
    ws = fz.Workspace(max(d.size for d, _, _ in items))
    xs, ss, ys, comp = _batch_buffers(fz, items)
    wants = [oracle.compress(d, dims, eb) for d, dims, eb in items]
    dec = fz.fields_array([{"src": s.data_ptr(), "dst": y.data_ptr(), "src_bytes": w.size, "dst_capacity": y.numel(),
                            "header": fz.parse_header(w)} for s, y, w in zip(ss, ys, wants)])
    for branches in (1, 3, 16):
        g, gd = fz.Batch(ws, comp, fz.COMPRESS, branches=branches), fz.Batch(ws, dec, fz.DECOMPRESS, branches=branches)
        for s in ss:
            s.fill_(0xCD)
        g.launch()
        gd.launch()
        torch.cuda.synchronize()
        for s, y, w in zip(ss, ys, wants):
            assert_same_stream(s[: w.size].cpu().numpy(), w)
            assert np.array_equal(y.cpu().numpy().view(np.uint32), oracle.decompress(w).view(np.uint32))
        g.close(), gd.close()
    best, ms = fz.batch_autotune(ws, comp, fz.COMPRESS, reps=2)
    assert best in ms and all(t > 0 for t in ms.values())
    assert set(ms) <= {1, 2, 4, 8, 16} and 1 in ms
    torch.cuda.synchronize()
    for s, w in zip(ss, wants):  # the tuning replays wrote the same streams
        assert_same_stream(s[: w.size].cpu().numpy(), w)
    with pytest.raises(fz.FzError):
        fz.Batch(ws, comp, fz.COMPRESS, branches=17)
    assert ws.status() == fz.SUCCESS


@pytest.mark.parametrize("nblocks,extra", [(512, 0), (1024, 0), (1025, 5), (31, 2047), (32, 0), (33, 1), (544, 100),
                                           (64, 0), (65, 3), (127, 0), (128, 1), (4, 0), (5, 7),
                                           (4095, 9), (4096, 0), (4097, 1), (8192, 2047), (8257, 0)])
def test_compaction_group_boundaries(fz, oracle, ws, nblocks, extra):
    """Fields ending exactly on or just past a 64-block and a 4096-block count group, a
    32-block compaction item and a 4-block compaction warp: offsets, offset table and
    header match the oracle."""
    n = nblocks * 2048 + extra
    rng = np.random.default_rng(n)
    data = np.cumsum(rng.normal(0, 1, n)).astype(np.float32)
    data[rng.random(n) < 0.3] = 0  # uneven chunk counts per block
    for mode in (0, 1):
        st, got, want = run_both(fz, oracle, ws, data, (n, 1, 1), 1e-3, mode=mode)
        assert_same_stream(got, want)
        rec = fz.decompress(st, ws=ws).cpu().numpy()
        assert np.array_equal(rec.view(np.uint32), oracle.decompress(want).view(np.uint32))


def test_list_schedule_batches_and_autotune(fz, oracle, synth):
    """Compression as list launches over all fields (fz_batch_create_sched, list = 1):
    compress-only and round-trip batches, replayed three times (the per-field control words
    and group sums are restored by each replay's last compaction item), equal the oracle;
    the schedule autotuner times both kinds of schedule and returns one of them."""
    items = _mixed_fields(synth) + [(synth.smooth2d(130, 9, seed=26), (130, 9, 1), 1e-3),
                                    (synth.smooth1d(1500, seed=27), (1500, 1, 1), 1e-2)]
    ws = fz.Workspace(max(d.size for d, _, _ in items))
    xs, ss, ys, comp = _batch_buffers(fz, items)
    wants = [oracle.compress(d, dims, eb) for d, dims, eb in items]
    dec = fz.fields_array([{"src": s.data_ptr(), "dst": y.data_ptr(), "src_bytes": w.size, "dst_capacity": y.numel(),
                            "header": fz.parse_header(w)} for s, y, w in zip(ss, ys, wants)])
    for pair in (False, True):
        g = fz.Batch.scheduled(ws, comp, dec if pair else None, fz.Schedule(4, 1))
        for _ in range(3):
            for s in ss:
                s.fill_(0x3C)
            for y in ys:
                y.fill_(9.0)
            g.launch()
            torch.cuda.synchronize()
            for s, y, w in zip(ss, ys, wants):
                assert_same_stream(s[: w.size].cpu().numpy(), w)
                if pair:
                    assert np.array_equal(y.cpu().numpy().view(np.uint32), oracle.decompress(w).view(np.uint32))
        g.close()
    best, ms = fz.batch_autotune_schedule(ws, comp, dec, reps=2)
    assert (best.branches, best.list) in ms and (1, 1) in ms and (1, 0) in ms
    torch.cuda.synchronize()
    for s, w in zip(ss, wants):
        assert_same_stream(s[: w.size].cpu().numpy(), w)
    assert ws.status() == fz.SUCCESS


def test_round_trip_pair_batch(fz, oracle, synth):
    """fz_batch_create_pair: each field compressed then decompressed on one branch of one
    graph; every replay reproduces the oracle's streams and reconstructions."""
    items = _mixed_fields(synth)
    ws = fz.Workspace(max(d.size for d, _, _ in items))
    xs, ss, ys, comp = _batch_buffers(fz, items)
    wants = [oracle.compress(d, dims, eb) for d, dims, eb in items]
    dec = fz.fields_array([{"src": s.data_ptr(), "dst": y.data_ptr(), "src_bytes": w.size, "dst_capacity": y.numel(),
                            "header": fz.parse_header(w)} for s, y, w in zip(ss, ys, wants)])
    for branches in (1, 2, 16):
        g = fz.Batch.pair(ws, comp, dec, branches=branches)
        for _ in range(2):
            for s in ss:
                s.fill_(0x5A)
            for y in ys:
                y.fill_(3.0)
            g.launch()
            torch.cuda.synchronize()
            for s, y, w in zip(ss, ys, wants):
                assert_same_stream(s[: w.size].cpu().numpy(), w)
                assert np.array_equal(y.cpu().numpy().view(np.uint32), oracle.decompress(w).view(np.uint32))
        g.close()
    assert ws.status() == fz.SUCCESS
