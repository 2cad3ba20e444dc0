"""A slice of the 512-field mixed batch at its real sizes, through the round-trip batch
graph (fz_batch_create_pair), against the oracle field by field.

The slice is the first 33 fields of synth.mixed_specs(512, seed=3) without the 210 MB 2D
field (whose generation alone takes minutes): 32 fields, 1D/2D/3D, 84 KB to 199 MB
(field 21 is a 368x368x368 3D field), rows that are and are not a multiple of 4
elements, and every eb of {1e-2, 1e-3, 1e-4}.  Every stream must be byte-identical and
every reconstruction bit-identical to the oracle's."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SLICE = [i for i in range(33) if i != 22]


@pytest.fixture(scope="module")
def batch_slice(fz, oracle, synth):
    specs = synth.mixed_specs(512, seed=3)
    items = []
    for i in SLICE:
        kind, dims, eb, seed = specs[i]
        data = synth.field(kind, dims, seed)
        items.append((i, data, dims, eb))
    wants = [oracle.compress(d, dims, eb) for _, d, dims, eb in items]
    return items, wants


def test_slice_covers_the_mix(fz, batch_slice):
    items, _ = batch_slice
    nds = {fz.ndim(dims) for _, _, dims, _ in items}
    assert nds == {1, 2, 3}
    assert {eb for *_, eb in items} == {1e-2, 1e-3, 1e-4}
    assert max(d.nbytes for _, d, _, _ in items) >= 128 << 20
    assert any(fz.ndim(dims) > 1 and dims[0] % 4 for _, _, dims, _ in items)


@pytest.mark.parametrize("branches,listed", [(0, 0), (16, 0), (8, 1)])
def test_pair_batch_matches_oracle_at_scale(fz, oracle, batch_slice, branches, listed):
    """Round trips of the slice under each schedule: per-field launches on 8 or 16 graph
    branches, or the compression of all 32 fields as list launches (one range launch, one
    encode launch per dimensionality, one compaction launch over a device work list), each
    replayed twice."""
    items, wants = batch_slice
    ws = fz.Workspace(max(d.size for _, d, _, _ in items))
    xs = [torch.from_numpy(d).cuda() for _, d, _, _ in items]
    caps = [fz.max_compressed_bytes(d.size, dims) for _, d, dims, _ in items]
    ss = [torch.full((c,), 0xA5, dtype=torch.uint8, device="cuda") for c in caps]
    ys = [torch.full((d.size,), 5.0, dtype=torch.float32, device="cuda") for _, d, _, _ in items]
    comp = fz.fields_array([{"src": x.data_ptr(), "dst": s.data_ptr(), "n": x.numel(), "dims": dims, "eb": eb,
                             "dst_capacity": s.numel()} for x, s, (_, _, dims, eb) in zip(xs, ss, items)])
    dec = fz.fields_array([{"src": s.data_ptr(), "dst": y.data_ptr(), "src_bytes": w.size, "dst_capacity": y.numel(),
                            "header": fz.parse_header(w)} for s, y, w in zip(ss, ys, wants)])
    g = fz.Batch.scheduled(ws, comp, dec, fz.Schedule(branches, listed))
    for rep in range(2):
        for s in ss:
            s.fill_(0xA5 + rep)
        g.launch()
        torch.cuda.synchronize()
        for (i, d, dims, eb), s, y, w in zip(items, ss, ys, wants):
            got = s[: w.size].cpu().numpy()
            bad = np.nonzero(got != w)[0]
            assert bad.size == 0, f"field {i} {dims} eb={eb}: {bad.size} stream bytes differ, first at {bad[:4]}"
            rec = y.cpu().numpy()
            assert np.array_equal(rec.view(np.uint32), oracle.decompress(w).view(np.uint32)), f"field {i} {dims}"
    g.close()
    assert ws.status() == fz.SUCCESS
