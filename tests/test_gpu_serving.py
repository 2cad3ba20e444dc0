"""The request loop (fz_server_*): every result is the same alone and in the mix, with
requests overlapping on the device and waiting for HBM budget."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _fields(synth):
    return [(synth.smooth2d(900, 400, seed=41), (900, 400, 1), 1e-3),
            (synth.peaks2d(3000, 257, seed=42, npeaks=50), (3000, 257, 1), 1e-4),
            (synth.smooth3d(70, 60, 50, seed=43), (70, 60, 50), 1e-3),
            (synth.smooth1d(333333, seed=44), (333333, 1, 1), 1e-2),
            (synth.smooth2d(64, 64, seed=45), (64, 64, 1), 1e-3),
            (synth.smooth3d(33, 17, 9, seed=46), (33, 17, 9), 1e-4)]


def _run(fz, server, reqs):
    """Submit all, poll until every request has completed; returns {id: (status, bytes)}."""
    for r in reqs:
        server.submit(**r)
    done = {}
    while len(done) < len(reqs):
        for rid, st, nb in server.poll():
            done[rid] = (st, nb)
    return done


def _oracle_results(oracle, items):
    """The oracle's stream and reconstruction of every field: what each served result must
    equal, alone and in the mix."""
    streams = [oracle.compress(d, dims, eb) for d, dims, eb in items]
    return streams, [oracle.decompress(s) for s in streams]


@pytest.mark.parametrize("budget_mb,slots", [(512, 4), (24, 2)])
def test_results_identical_alone_and_in_the_mix(fz, oracle, synth, budget_mb, slots):
    """Served streams are byte-identical, and served reconstructions bit-identical, to the
    oracle's, both for requests served alone and for the same requests interleaved under a
    budget that forces queueing."""
    items = _fields(synth)
    ws = fz.Workspace(max(d.size for d, _, _ in items))
    alone = [fz.compress_host(d, dims, eb, ws=ws) for d, dims, eb in items]
    alone_rec = [fz.decompress_host(s, ws=ws) for s in alone]
    want, want_rec = _oracle_results(oracle, items)
    for a, ar, w, wr in zip(alone, alone_rec, want, want_rec):
        assert np.array_equal(a, w)
        assert np.array_equal(ar.view(np.uint32), wr.view(np.uint32))
    hin = [torch.from_numpy(d).pin_memory() for d, _, _ in items]
    caps = [fz.max_compressed_bytes(d.size, dims) for d, dims, _ in items]
    hout = [torch.empty(c, dtype=torch.uint8).pin_memory() for c in caps]
    hst = [torch.from_numpy(s.copy()).pin_memory() for s in alone]
    hrec = [torch.empty(d.size, dtype=torch.float32).pin_memory() for d, _, _ in items]
    reqs = []
    for i, (d, dims, eb) in enumerate(items):  # interleave compress and decompress requests
        reqs.append(dict(rid=2 * i, direction=fz.COMPRESS, src=hin[i].data_ptr(), dst=hout[i].data_ptr(),
                         dst_capacity=caps[i], n=d.size, dims=dims, eb=eb))
        reqs.append(dict(rid=2 * i + 1, direction=fz.DECOMPRESS, src=hst[i].data_ptr(), dst=hrec[i].data_ptr(),
                         dst_capacity=4 * d.size, src_bytes=alone[i].size))
    server = fz.Server(budget_mb << 20, slots, max(d.size for d, _, _ in items))
    done = _run(fz, server, reqs)
    for i, (d, _, _) in enumerate(items):
        st, nb = done[2 * i]
        assert st == fz.SUCCESS and nb == want[i].size
        assert np.array_equal(hout[i][:nb].numpy(), want[i])
        st, nb = done[2 * i + 1]
        assert st == fz.SUCCESS and nb == d.size
        assert np.array_equal(hrec[i].numpy().view(np.uint32), want_rec[i].view(np.uint32))
    q, r, used = server.pending()
    assert (q, r, used) == (0, 0, 0)
    server.close()


def test_request_larger_than_the_budget_is_rejected(fz, synth):
    d = synth.smooth2d(600, 600, seed=47)
    h = torch.from_numpy(d).pin_memory()
    out = torch.empty(fz.max_compressed_bytes(d.size, (600, 600, 1)), dtype=torch.uint8).pin_memory()
    server = fz.Server(1 << 20, 2, d.size)  # 1 MiB cannot hold a 1.44 MB field
    done = _run(fz, server, [dict(rid=7, direction=fz.COMPRESS, src=h.data_ptr(), dst=out.data_ptr(),
                                  dst_capacity=out.numel(), n=d.size, dims=(600, 600, 1), eb=1e-3)])
    assert done[7][0] == fz.OUT_OF_SPACE
    server.close()


@pytest.mark.parametrize("budget_mb,slots", [(512, 4), (12, 3)])
def test_device_resident_requests_match_and_mix_with_host_ones(fz, oracle, synth, budget_mb, slots):
    """FZ_REQUEST_DEVICE: fields already in HBM compress into device streams and decompress
    back in place; the streams equal the oracle's and the reconstructions equal the
    oracle's, alone and interleaved with host-buffer requests."""
    items = _fields(synth)
    ws = fz.Workspace(max(d.size for d, _, _ in items))
    xd = [torch.from_numpy(d).cuda() for d, _, _ in items]
    alone = [fz.compress(x, dims, eb, ws=ws) for x, (_, dims, eb) in zip(xd, items)]
    alone_rec = [fz.decompress(s, ws=ws) for s in alone]
    want, want_rec = _oracle_results(oracle, items)
    for a, ar, w, wr in zip(alone, alone_rec, want, want_rec):
        assert np.array_equal(a.cpu().numpy(), w)
        assert np.array_equal(ar.cpu().numpy().view(np.uint32), wr.view(np.uint32))
    caps = [fz.max_compressed_bytes(d.size, dims) for d, dims, _ in items]
    sd = [torch.zeros(c, dtype=torch.uint8, device="cuda") for c in caps]
    rd = [torch.zeros(d.size, dtype=torch.float32, device="cuda") for d, _, _ in items]
    hst = [torch.from_numpy(s.cpu().numpy()).pin_memory() for s in alone]
    hrec = [torch.empty(d.size, dtype=torch.float32).pin_memory() for d, _, _ in items]
    rd2 = [torch.zeros(d.size, dtype=torch.float32, device="cuda") for d, _, _ in items]
    reqs = []
    for i, (d, dims, eb) in enumerate(items):
        # compress in HBM; decompress in HBM with the header fetched by the server or given
        # on the host (a copy made at submit: the Header object is dropped right away);
        # decompress from host buffers
        reqs.append(dict(rid=4 * i, direction=fz.COMPRESS, src=xd[i].data_ptr(), dst=sd[i].data_ptr(),
                         dst_capacity=caps[i], n=d.size, dims=dims, eb=eb, device=True))
        reqs.append(dict(rid=4 * i + 1, direction=fz.DECOMPRESS, src=alone[i].data_ptr(), dst=rd[i].data_ptr(),
                         dst_capacity=4 * d.size, src_bytes=alone[i].numel(), device=True))
        reqs.append(dict(rid=4 * i + 2, direction=fz.DECOMPRESS, src=hst[i].data_ptr(), dst=hrec[i].data_ptr(),
                         dst_capacity=4 * d.size, src_bytes=alone[i].numel()))
        reqs.append(dict(rid=4 * i + 3, direction=fz.DECOMPRESS, src=alone[i].data_ptr(), dst=rd2[i].data_ptr(),
                         dst_capacity=4 * d.size, src_bytes=alone[i].numel(), device=True,
                         header=fz.parse_header(alone[i][:64].cpu().numpy())))
    server = fz.Server(budget_mb << 20, slots, max(d.size for d, _, _ in items))
    done = _run(fz, server, reqs)
    torch.cuda.synchronize()
    for i, (d, _, _) in enumerate(items):
        st, nb = done[4 * i]
        assert st == fz.SUCCESS and nb == want[i].size
        assert np.array_equal(sd[i][:nb].cpu().numpy(), want[i])
        for k, rec in ((1, rd[i].cpu()), (2, hrec[i]), (3, rd2[i].cpu())):
            st, nb = done[4 * i + k]
            assert st == fz.SUCCESS and nb == d.size
            assert np.array_equal(rec.numpy().view(np.uint32), want_rec[i].view(np.uint32))
    assert server.pending() == (0, 0, 0)
    server.close()


def test_device_request_with_short_output_fails_cleanly(fz, synth):
    d = synth.smooth2d(300, 200, seed=48)
    x = torch.from_numpy(d).cuda()
    st_t = fz.compress(x, (300, 200, 1), 1e-3)
    out = torch.zeros(d.size - 1, dtype=torch.float32, device="cuda")  # one element short
    server = fz.Server(64 << 20, 2, d.size)
    done = _run(fz, server, [dict(rid=1, direction=fz.DECOMPRESS, src=st_t.data_ptr(), dst=out.data_ptr(),
                                  dst_capacity=4 * out.numel(), src_bytes=st_t.numel(), device=True)])
    assert done[1][0] == fz.OUT_OF_SPACE
    assert server.pending() == (0, 0, 0)
    server.close()


def test_failed_request_does_not_poison_its_slot(fz, synth):
    """A request that fails on the device (non-finite input with a relative eb) reports
    FZ_NONFINITE_INPUT; the same slot then serves the next request normally."""
    good = synth.smooth2d(300, 200, seed=49)
    bad = good.copy()
    bad[123] = np.nan
    ws = fz.Workspace(good.size)
    alone = fz.compress(torch.from_numpy(good).cuda(), (300, 200, 1), 1e-3, ws=ws).cpu().numpy()
    xb, xg = torch.from_numpy(bad).cuda(), torch.from_numpy(good).cuda()
    cap = fz.max_compressed_bytes(good.size, (300, 200, 1))
    outs = [torch.zeros(cap, dtype=torch.uint8, device="cuda") for _ in range(2)]
    server = fz.Server(64 << 20, 1, good.size)
    for rid, (x, o) in enumerate(((xb, outs[0]), (xg, outs[1]))):
        done = _run(fz, server, [dict(rid=rid, direction=fz.COMPRESS, src=x.data_ptr(), dst=o.data_ptr(),
                                      dst_capacity=cap, n=good.size, dims=(300, 200, 1), eb=1e-3, device=True)])
        if rid == 0:
            assert done[0][0] == fz.NONFINITE_INPUT
        else:
            assert done[1][0] == fz.SUCCESS and done[1][1] == alone.size
            assert np.array_equal(outs[1][: alone.size].cpu().numpy(), alone)
    server.close()


def test_submit_and_poll_from_several_threads(fz, synth):
    """Four host threads submit compress and decompress requests and poll at the same time
    (fz_server_* may be called from any thread): every request completes exactly once and
    every result equals the one computed alone."""
    import threading
    import time
    items = _fields(synth)
    ws = fz.Workspace(max(d.size for d, _, _ in items))
    alone = [fz.compress_host(d, dims, eb, ws=ws) for d, dims, eb in items]
    alone_rec = [fz.decompress_host(s, ws=ws) for s in alone]
    caps = [fz.max_compressed_bytes(d.size, dims) for d, dims, _ in items]
    hin = [torch.from_numpy(d).pin_memory() for d, _, _ in items]
    hst = [torch.from_numpy(s.copy()).pin_memory() for s in alone]
    nthreads = 4
    outs, reqs = {}, [[] for _ in range(nthreads)]
    for t in range(nthreads):
        for i, (d, dims, eb) in enumerate(items):
            rc, rd = 1000 * t + 2 * i, 1000 * t + 2 * i + 1
            outs[rc] = torch.empty(caps[i], dtype=torch.uint8).pin_memory()
            outs[rd] = torch.empty(d.size, dtype=torch.float32).pin_memory()
            reqs[t].append(dict(rid=rc, direction=fz.COMPRESS, src=hin[i].data_ptr(), dst=outs[rc].data_ptr(),
                                dst_capacity=caps[i], n=d.size, dims=dims, eb=eb))
            reqs[t].append(dict(rid=rd, direction=fz.DECOMPRESS, src=hst[i].data_ptr(), dst=outs[rd].data_ptr(),
                                dst_capacity=4 * d.size, src_bytes=alone[i].size))
    total = sum(len(r) for r in reqs)
    server = fz.Server(256 << 20, 4, max(d.size for d, _, _ in items))
    lock, done, errors = threading.Lock(), [], []

    def worker(t):
        try:
            torch.cuda.set_device(0)
            for r in reqs[t]:
                server.submit(**r)
                got = server.poll()
                with lock:
                    done.extend(got)
            deadline = time.monotonic() + 120
            while True:
                got = server.poll()
                with lock:
                    done.extend(got)
                    if len(done) >= total:
                        return
                if time.monotonic() > deadline:
                    raise TimeoutError(f"{len(done)} of {total} requests completed")
        except Exception as ex:  # surfaced below
            errors.append(ex)

    th = [threading.Thread(target=worker, args=(t,), daemon=True) for t in range(nthreads)]
    for x in th:
        x.start()
    for x in th:
        x.join(timeout=300)
    assert not errors, errors
    assert not any(x.is_alive() for x in th)
    ids = [rid for rid, _, _ in done]
    assert len(ids) == total and len(set(ids)) == total
    for rid, st, nb in done:
        i = (rid % 1000) // 2
        assert st == fz.SUCCESS, (rid, st)
        if rid % 2 == 0:
            assert nb == alone[i].size and np.array_equal(outs[rid][:nb].numpy(), alone[i])
        else:
            assert np.array_equal(outs[rid].numpy().view(np.uint32), alone_rec[i].view(np.uint32))
    assert server.pending() == (0, 0, 0)
    server.close()

