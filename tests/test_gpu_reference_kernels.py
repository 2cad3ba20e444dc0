"""Full-size parity against the reference's own kernels, run on this GPU.

The reference's c_lorenzo_{1d,2d,3d}, bitshuffleAndBitflag, CUB ExclusiveSum and
encodeDebug (runSzs's device sequence, fz.cu:139-205; tests/golden/refpipe.py) compress
the full-size workloads, and the product's stream must hold exactly their output:
Section A = d_bitFlagArray[0..ceil(n/256)), Section B = d_out[0..16 nnz), the header's
nnz = the reference's total, and fz_lorenzo_construct's codes = the reference's quant.
Needs oracle/_ref/ref_kernels.fatbin, compiled from the FZ-GPU sources by
`make -C oracle ref REF=<dir>`; without it the module is skipped."""
import os
import sys

import numpy as np
import pytest
import torch

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import refpipe  # noqa: E402

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refpipe.available(), reason="reference-kernel fatbin not built")]

CASES = [
    ("exafel-like 39200x388", "peaks2d", (39200, 388, 1), 1, 1e-3),
    ("cesm-like 3600x1800", "smooth2d", (3600, 1800, 1), 0, 1e-3),
    ("hurricane-like 500x500x100", "smooth3d", (500, 500, 100), 2, 1e-3),
    ("cesm-like 3601x1800", "smooth2d", (3601, 1800, 1), 0, 1e-3),
    ("1D 2^24+77", "smooth1d", ((1 << 24) + 77, 1, 1), 6, 1e-3),
]


@pytest.fixture(scope="module")
def ref():
    return refpipe.RefPipeline()


@pytest.mark.parametrize("name,kind,dims,seed,eb", CASES, ids=[c[0].split()[1] for c in CASES])
@pytest.mark.parametrize("mode", [0, 1])
def test_stream_sections_equal_reference_output(fz, synth, ref, name, kind, dims, seed, eb, mode):
    data = synth.field(kind, dims, seed)
    x = torch.from_numpy(data).cuda()
    rng = np.float32(data.max() - data.min())          # fz.cu:137
    eb_abs = float(eb) * float(rng)                     # fz.cu:149
    r = ref.run(x, dims, eb_abs)
    st = fz.compress(x, dims, eb, rel=True, mode=mode).cpu().numpy()
    h = fz.parse_header(st)
    off_a, _, off_b, _ = fz.stream_layout(data.size, dims, mode)
    assert h.nnz == r["nnz"], (h.nnz, r["nnz"])
    bitmap = st[off_a: off_a + 4 * r["dcs2"]].view(np.uint32)
    assert np.array_equal(bitmap, r["bitflag"].cpu().numpy().view(np.uint32))
    assert np.array_equal(st[off_b: off_b + 16 * h.nnz], r["d_out"].cpu().numpy())
    if mode == 1:
        q = fz.lorenzo_construct(x, dims, eb_abs)
        assert torch.equal(q, r["quant"])
