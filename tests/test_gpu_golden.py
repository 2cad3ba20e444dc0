"""The product kernels against the reference's own kernel outputs (tests/golden):
codes, shuffled words, chunk flags, bitmap, prefix sums and compacted chunks, and the
stream's Sections A and B, all bit-exact."""
import glob
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_kernels_match_reference_outputs(fz, path):
    g = np.load(path)
    data, dims = g["data"], tuple(int(v) for v in g["dims"])
    n = data.size
    nl = dims[0] * dims[1] * dims[2]
    xt = torch.from_numpy(data).cuda()
    q = fz.lorenzo_construct(xt, dims, float(g["eb_abs"]))
    assert np.array_equal(q.cpu().numpy().view(np.uint16), g["quant"])
    sh, bit, byte = fz.bitshuffle_flag(q)
    assert np.array_equal(sh.cpu().numpy().view(np.uint16), g["shuffled"])
    assert np.array_equal(byte.cpu().numpy().view(np.uint32), g["byteflag"])
    assert np.array_equal(bit.cpu().numpy().view(np.uint32), g["bitflag"])
    pad = torch.zeros(2 * ((n + 1) // 2) + 16, dtype=torch.int16, device="cuda")
    pad[:n] = sh
    pre, out, nnz = fz.scan_encode(pad, byte, n)
    assert nnz == int(g["nnz"])
    assert np.array_equal(pre.cpu().numpy().view(np.uint32), g["presum"])
    assert np.array_equal(out.cpu().numpy(), g["d_out"])
    # the fused path: Sections A and B of the stream are the reference's buffers
    st = fz.compress(xt, dims, float(g["eb"]), rel=bool(g["rel"]), mode=fz.MODE_COMPAT).cpu().numpy()
    a, _, b, _ = fz.stream_layout(n, dims, fz.MODE_COMPAT)
    assert np.array_equal(st[a: a + 4 * g["bitflag"].size].view(np.uint32), g["bitflag"])
    assert np.array_equal(st[b:], g["d_out"])
    assert nl <= n
