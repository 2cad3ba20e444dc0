"""The oracle against independent restatements (numpy bit-level definitions and a
per-element Python restatement) and hand-made known answers.  CPU only."""
import numpy as np
import pytest

from conftest import error_tolerance


def np_shuffle(codes):
    """fz.cu:61-111 by the bit-level definition: S[b*1024+p*32+g] bit j = bit p of
    W[b*1024+g*32+j]; flags per 4 words; bitmap bit j of word 8b+k = flag 256b+32k+j."""
    n = codes.size
    nb = n // 2048
    nw = (n + 255) // 256
    S = np.zeros((n + 1) // 2, np.uint32)
    S.view(np.uint16)[:n] = codes
    W = codes[: nb * 2048].view(np.uint32).reshape(nb, 32, 32)
    bits = (W[..., None] >> np.arange(32, dtype=np.uint32)) & 1          # [b][g][j][p]
    Sb = (bits.transpose(0, 3, 1, 2).astype(np.uint64) << np.arange(32, dtype=np.uint64)).sum(-1)
    S[: nb * 1024] = Sb.astype(np.uint32).reshape(-1)
    F = np.zeros(32 * nw, np.uint32)
    F[: nb * 256] = (S[: nb * 1024].reshape(-1, 4) != 0).any(1)
    B = np.zeros(nw, np.uint32)
    for k in range(nb * 8):
        B[k] = sum(int(F[32 * k + j]) << j for j in range(32))
    return S, F, B


@pytest.mark.parametrize("n", [1, 100, 2047, 2048, 2049, 4096 + 511, 3 * 2048, 5 * 2048 + 1])
def test_shuffle_flags_match_bit_definition(oracle, n):
    rng = np.random.default_rng(n)
    codes = rng.integers(0, 65536, n, dtype=np.uint16)
    codes[: min(n, 2048) // 2] = 0                     # zero chunks
    seg = codes[n // 3: n // 3 + 300]
    seg[:] = rng.integers(0, 2, seg.size).astype(np.uint16)
    S, F, B = oracle.bitshuffle_flag(codes)
    S2, F2, B2 = np_shuffle(codes)
    assert np.array_equal(S, S2) and np.array_equal(F, F2) and np.array_equal(B, B2)


def test_scan_encode_matches_numpy(oracle):
    rng = np.random.default_rng(3)
    n = 7 * 2048 + 300
    codes = (rng.random(n) < 0.02).astype(np.uint16) * rng.integers(1, 9, n).astype(np.uint16)
    S, F, B = oracle.bitshuffle_flag(codes)
    P, out, nnz = oracle.scan_encode(S, F, n)
    m = 32 * ((n + 255) // 256)
    assert np.array_equal(P[:m], np.concatenate([[0], np.cumsum(F[: m - 1])]).astype(np.uint32))
    assert P[m] == F.sum() == nnz
    chunks = S.view(np.uint8)[: 16 * (n * 2 // 16)].reshape(-1, 16)
    want = chunks[np.nonzero(F[: chunks.shape[0]])[0]].reshape(-1)
    assert np.array_equal(out, want)


def py_codes(data, dims, r):
    """Per-element restatement of lorenzo_var.cuh:47-295 in numpy float32 scalars."""
    x, y, z = dims
    f32 = np.float32
    r = f32(r)

    def pq(i):
        v = f32(data[i]) * r
        return f32(np.sign(v) * np.floor(np.abs(v) + f32(0.5))) if np.isfinite(v) else v

    def pack(d, signed=True):
        a = abs(float(d))
        m = 0 if not a > 0 else (0xFFFF if a >= 2.0 ** 32 else int(a) & 0xFFFF)
        return (m | ((d < 0) << 15)) & 0xFFFF if signed else m

    out = np.zeros(data.size, np.uint16)
    nd = 1 if (y == 1 and z == 1) else (2 if z == 1 else 3)
    for i in range(x * y * z):
        if nd == 1:
            k = i % 256
            d = f32(pq(i) - (pq(i - 1) if k else f32(0)))
            out[i] = pack(d, k % 4 == 0)
        elif nd == 2:
            rr, cc = divmod(i, x)
            ri, ci = rr % 16 != 0, cc % 16 != 0
            n_ = pq(i - x) if ri else f32(0)
            w = pq(i - 1) if ci else f32(0)
            nw = pq(i - x - 1) if (ri and ci) else f32(0)
            out[i] = pack(f32(f32(pq(i) - n_) - f32(w - nw)))
        else:
            zz, rem = divmod(i, x * y)
            yy, xx = divmod(rem, x)
            zi, yi, xi = zz % 8 != 0, yy % 8 != 0, xx % 8 != 0
            xy = x * y
            g = lambda cond, j: pq(j) if cond else f32(0)
            s = f32(g(zi and yi and xi, i - xy - x - 1) - g(yi and xi, i - x - 1))
            s = f32(s - g(zi and xi, i - xy - 1))
            s = f32(s - g(zi and yi, i - xy - x))
            s = f32(s + g(xi, i - 1))
            s = f32(s + g(yi, i - x))
            s = f32(s + g(zi, i - xy))
            out[i] = pack(f32(pq(i) - s))
    return out


@pytest.mark.parametrize("dims", [(700, 1, 1), (37, 21, 1), (33, 17, 1), (19, 11, 9), (9, 1, 10)])
def test_lorenzo_matches_per_element_restatement(oracle, dims):
    rng = np.random.default_rng(sum(dims))
    n = dims[0] * dims[1] * dims[2] + 5
    data = (rng.normal(0, 1, n) * 50).astype(np.float32)
    data[rng.random(n) < 0.02] = np.float32(1e6)   # deltas past the 16-bit field
    data[rng.random(n) < 0.2] = 0
    r = oracle.ebx2_r(0.01)
    codes, _, _ = oracle.lorenzo_construct(data, dims, r)
    assert np.array_equal(codes, py_codes(data, dims, r))
    assert not codes[dims[0] * dims[1] * dims[2]:].any()


def test_lorenzo_known_answers(oracle):
    # 2D, one 16x16 tile + one column of the next; ebx2_r = 1 (eb_abs = 0.5)
    r = oracle.ebx2_r(0.5)
    assert r == np.float32(1.0)
    x, y = 17, 2
    d = np.zeros(x * y, np.float32)
    d[0] = 3.0            # origin: d = c
    d[1] = 1.0            # (0,1): d = c - w = 1 - 3 = -2
    d[x] = -4.0           # (1,0): d = c - n = -4 - 3 = -7
    d[x + 1] = 0.0        # (1,1): (0 - 1) - (-4 - 3) = 6
    d[16] = 2.5           # next tile origin: round(2.5) = 3 (ties away)
    d[16 + x] = -2.5      # (1,16): -3 - 3 = -6
    codes, _, _ = oracle.lorenzo_construct(d, (x, y, 1), r)
    assert codes[0] == 3 and codes[1] == 0x8002 and codes[x] == 0x8007 and codes[x + 1] == 6
    assert codes[16] == 3 and codes[16 + x] == 0x8006
    # 1D: sign only at i % 4 == 0 (lorenzo_var.cuh:51-63)
    d1 = np.array([1, 0, 5, 2, 0, 3, 3, -1], np.float32)
    c1, sg, _ = oracle.lorenzo_construct(d1, (8, 1, 1), r, signum=True)
    assert list(c1) == [1, 1, 5, 3, 0x8002, 3, 0, 4]
    assert list(sg) == [0, 1, 0, 1, 1, 0, 0, 1]
    # code field limits: |d| = 32767 signed fits, 32768 sets the overflow flag
    for v, ovf in [(32767.0, 0), (32768.0, 1), (-32767.0, 0)]:
        c, _, o = oracle.lorenzo_construct(np.array([v, 0], np.float32), (1, 2, 1), r)
        assert o == ovf
    # the device conversion (pinned by tests/golden/*crafted*): saturating f32 -> u32,
    # then the low 16 bits
    f2u16 = oracle.lib().fzo_f2u16
    assert f2u16(np.float32(70000)) == 4464 and f2u16(np.float32(1e9)) == 51712
    assert f2u16(np.float32(65536)) == 0 and f2u16(np.float32(65535.9)) == 65535
    assert f2u16(np.float32(np.inf)) == 0xFFFF and f2u16(np.float32(1e10)) == 0xFFFF
    assert f2u16(np.float32(np.nan)) == 0 and f2u16(np.float32(65534.9)) == 65534


@pytest.mark.parametrize("kind,dims,eb", [
    ("smooth2d", (250, 90, 1), 1e-3), ("peaks2d", (300, 77, 1), 1e-4),
    ("smooth3d", (40, 30, 20), 1e-3), ("smooth1d", (20000, 1, 1), 1e-3), ("smooth1d", (1000, 1, 1), 1e-2)])
@pytest.mark.parametrize("mode", [0, 1])
def test_round_trip_error_bound(oracle, synth, kind, dims, eb, mode):
    data = synth.field(kind, dims, seed=7)
    st = oracle.compress(data, dims, eb, rel=True, mode=mode)
    h = oracle.parse_header(st)
    rec = oracle.decompress(st)
    tol = error_tolerance(data, h["eb_abs"])
    err = np.abs(rec.astype(np.float64) - data)
    n = data.size
    if mode == 1:
        assert (err <= tol).all()
        m = oracle.metrics(data, rec)
        assert m["psnr"] > 0
    else:
        # COMPAT is the reference's lossy content: the tail (n mod 2048) is not stored
        # (fz.cu:173) and 1D loses signs at i%4 != 0 (lorenzo_var.cuh:58-63)
        nb = n // 2048
        if dims[1] > 1:
            ok = err[: nb * 2048] <= tol[: nb * 2048]
            # 2D/3D tiles cut by the block boundary inherit the missing tail deltas
            assert ok.mean() > 0.9
    assert st.size == oracle.layout(n, h["ndim"], mode)[2] + 16 * h["nnz"]


def test_stream_header_and_sections(oracle, synth):
    data = synth.smooth2d(200, 50, seed=1)
    st = oracle.compress(data, (200, 50, 1), 1e-3)
    h = oracle.parse_header(st)
    assert h["magic"] == 0x31475A46 and h["version"] == 1 and h["ndim"] == 2 and h["n"] == data.size
    mn, mx = oracle.value_range(data)
    assert h["range"] == np.float32(mx - mn)
    assert h["eb_abs"] == 1e-3 * float(np.float32(mx - mn))
    a, c, b, sc = oracle.layout(data.size, 2, 1)
    pad = lambda v: 16 * ((v + 15) // 16)
    nb = data.size // 2048
    assert sc == h["sidecar_bytes"] == pad(2 * (data.size % 2048)) + pad(4 * (nb + 1))
    codes, _, _ = oracle.lorenzo_construct(data, (200, 50, 1), h["ebx2_r"])
    S, F, B = oracle.bitshuffle_flag(codes)
    assert np.array_equal(st[a: a + 4 * B.size].view(np.uint32), B)
    _, out, nnz = oracle.scan_encode(S, F, data.size)
    assert nnz == h["nnz"] and np.array_equal(st[b:], out)
    tail = data.size % 2048
    assert np.array_equal(st[c: c + 2 * tail].view(np.uint16), codes[data.size - tail:])
    # chunk offset of every shuffle block, then the total
    q = c + pad(2 * tail)
    boff = st[q: q + 4 * (nb + 1)].view(np.uint32)
    counts = np.array([sum(bin(int(w)).count("1") for w in B[8 * i: 8 * i + 8]) for i in range(nb)])
    assert np.array_equal(boff, np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32))


def test_nonfinite_relative_eb_rejected(oracle):
    d = np.ones(5000, np.float32)
    d[17] = np.nan
    with pytest.raises(ValueError):
        oracle.compress(d, (5000, 1, 1), 1e-3, rel=True)


def test_round_half_away_identity():
    """The kernels round with trunc(v + copysign(pred(1/2), v)) in float; it equals
    round-half-away-from-zero (roundf, lorenzo_var.cuh:81) for every float.  Checked
    here on the neighbourhoods of all k + 1/2 below 2^24 and on random floats (the
    exhaustive check over all 2^31 non-negative floats passes too)."""
    h = np.float32(np.nextafter(np.float32(0.5), np.float32(0)))

    def fast(x):
        return np.trunc(x + np.copysign(h, x))

    def exact(x):
        a = np.abs(x.astype(np.float64))
        r = np.where(a >= 2.0 ** 23, a, np.floor(a + 0.5))
        return (np.sign(x) * r).astype(np.float32)

    k = np.arange(0, 1 << 24, 7, dtype=np.float64)
    base = (k + 0.5).astype(np.float32)
    xs = [base]
    for _ in range(3):
        xs.append(np.nextafter(xs[-1], np.float32(np.inf)))
    lo = base
    for _ in range(3):
        lo = np.nextafter(lo, np.float32(0))
        xs.append(lo)
    rng = np.random.default_rng(0)
    xs.append(rng.integers(0, 0x7F800000, 1 << 22, dtype=np.uint32).view(np.float32))
    x = np.concatenate(xs)
    x = np.concatenate([x, -x])
    assert np.array_equal(fast(x), exact(x))
