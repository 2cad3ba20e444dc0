"""The oracle against the reference's own kernels.

tests/golden/*.npz hold the inputs and every intermediate buffer of the reference's
c_lorenzo_{1d,2d,3d}, bitshuffleAndBitflag and encodeDebug, compiled for sm_103a from
the FZ-GPU sources and run on a GB300 by tests/golden/make_golden.py.  Each fixture is
re-derived here by the oracle on the CPU and must match bit for bit."""
import glob
import os

import numpy as np
import pytest

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def test_fixtures_present():
    assert GOLDEN, "no golden fixtures: run tests/golden/make_golden.py on a GPU machine"


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_kernels(oracle, path):
    g = np.load(path)
    data, dims = g["data"], tuple(int(v) for v in g["dims"])
    n = data.size
    if bool(g["rel"]):
        mn, mx = oracle.value_range(data)
        assert np.float32(mx - mn) == g["range"]
        eb_abs = float(g["eb"]) * float(np.float32(mx - mn))
    else:
        eb_abs = float(g["eb"])
    assert eb_abs == float(g["eb_abs"])
    r = oracle.ebx2_r(eb_abs)
    assert r == g["ebx2_r"]
    codes, _, _ = oracle.lorenzo_construct(data, dims, r)
    # quantisation codes: every element, including the code-field limits and NaN/Inf
    bad = np.nonzero(codes != g["quant"])[0]
    assert bad.size == 0, f"codes differ at {bad[:8]}: oracle {codes[bad[:8]]} ref {g['quant'][bad[:8]]}"
    S, F, B = oracle.bitshuffle_flag(codes)
    assert np.array_equal(S.view(np.uint16)[:n], g["shuffled"])
    assert np.array_equal(F, g["byteflag"])
    assert np.array_equal(B, g["bitflag"])
    P, out, nnz = oracle.scan_encode(S, F, n)
    assert np.array_equal(P, g["presum"]) and nnz == int(g["nnz"])
    # encodeDebug's shared sumArr[0] is written by every lane (fz.cu:53); the
    # fixtures record what the reference actually produced on the GPU.
    assert np.array_equal(out, g["d_out"])
