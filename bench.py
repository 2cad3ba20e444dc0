#!/usr/bin/env python
"""Benchmark of the FZ compression hot path on GB300.

A step is one pass of the path over one batch of synthetic input: `--fields` (128)
exafel-like 39200x388 float32 fields (the single-field workload the metric is quoted on,
relative eb 1e-3; `--distinct` seeded fields, each held in several device buffers), each
compressed (range pass, encode, compaction) and then decompressed (fused decode + inverse
Lorenzo), issued as one CUDA-graph replay of a round-trip batch under the schedule the
autotuner picks.  A step holds 128 x 60.8 MB = 7.8 GB of input, far larger than the
129 MB L2, and every buffer is visited once per step.

  value      uncompressed GB/s through the codec, both directions:
             steps * fields * 2 * 4n bytes / device time (CUDA events), summed over ranks
  e2e        the same metric through the host-buffer C-ABI calls fz_compress_host /
             fz_decompress_host (pinned host memory, H2D and D2H copies inside the region):
             compressing host threads hand their streams to decompressing ones, so input
             copies and output copies share the host link at all times
  value_without_graphs  the same steps as one fz_compress_batch / fz_decompress_batch
             call per direction on one stream (each field's encode launch also takes the
             range of the next field), no graph
  roofline   the dominant kernel's algorithmic bytes per launch / its mean event-timed
             launch duration (per-field calls: the kernels of the graph's branches),
             against the measured HBM copy bandwidth
  per_dimensionality  compress / decompress GB/s and kernel fractions of the other
             single-field workloads (cesm-like 2D, hurricane-like 3D, unaligned rows, 1D)
  batch      the 512-field mixed batch: every schedule the autotuner tries against the
             plain per-field path
  serving    a Poisson request trace over the same mix through the request loop
  cpu_baseline  the oracle (C, OpenMP) on this host's cores, round trips of one field

`--impl reference` times the reference path's CPU restatement (the oracle port; the
reference has no CPU implementation and its GPU code is not a CPU baseline) on the
same metric and workload, with the same `config`.  Under torchrun each rank runs its own
batch (weak scaling); only rank 0 prints.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# single-field workloads (--field): dims, relative eb, generator, description.  The
# headline is exafel (the workload the metric is quoted on); the others profile the
# other dimensionalities on the same harness.
FIELDS = {
    "exafel": ((39200, 388, 1), 1e-3, "peaks2d", "exafel-like 39200x388 f32 (peaks on N(0,0.5) background), relative eb 1e-3"),
    "cesm": ((3600, 1800, 1), 1e-3, "smooth2d", "cesm-like 3600x1800 f32 (smooth, ~30% zeros), relative eb 1e-3"),
    "hurricane": ((500, 500, 100), 1e-3, "smooth3d", "hurricane-like 500x500x100 f32 (smooth 3D, ~40% zeros), relative eb 1e-3"),
    "exafel_u": ((39201, 388, 1), 1e-3, "peaks2d", "exafel-like 39201x388 f32 (rows not a multiple of 4), relative eb 1e-3"),
    "hurricane_u": ((501, 500, 100), 1e-3, "smooth3d",
                    "hurricane-like 501x500x100 f32 (rows not a multiple of 4), relative eb 1e-3"),
    "oned": ((1 << 25, 1, 1), 1e-3, "smooth1d", "1D 2^25 f32 (smooth series with zero runs), relative eb 1e-3"),
}
DIMS, EB, KIND, WORKLOAD = FIELDS["exafel"]
METRIC = "compress/decompress GB/s + %HBM peak"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--fields", type=int, default=128, help="field buffers per step")
    p.add_argument("--distinct", type=int, default=8, help="distinct seeded fields among them")
    p.add_argument("--impl", choices=["fz", "reference"], default="fz")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--quick", action="store_true", help="headline only: no per-dimensionality, batch or serving keys")
    p.add_argument("--workload", choices=["exafel", "batch", "serving", "kernels", "listkernels"], default="exafel",
                   help="exafel: the headline line (single-field workload, see --field); batch: 512 mixed "
                        "1D/2D/3D fields batched vs per field; serving: a Poisson request trace; kernels: "
                        "every kernel kind on the --field workload, --steps times (for a profiler); "
                        "listkernels: the batch schedule's list launches on --list-fields fields of the mix, "
                        "--steps times (for a profiler)")
    p.add_argument("--list-fields", type=int, default=32,
                   help="listkernels: the first fields of the 512-field mix of at most 32 MB")
    p.add_argument("--field", choices=sorted(FIELDS), default="exafel",
                   help="the single-field workload of the headline line (default exafel)")
    p.add_argument("--batch-fields", type=int, default=512)
    p.add_argument("--serve-seconds", type=float, default=2.0)
    p.add_argument("--serve-rate", type=float, default=2000.0)
    p.add_argument("--serve-host-fields", type=int, default=128,
                   help="fields of the mix (the first ones) that the host-buffer trace draws from")
    return p.parse_args()


def config_dict(n):
    """The `config` both arms print: the workload the metric is quoted on."""
    return {"workload": WORKLOAD, "field_elems": n, "eb": EB, "eb_mode": "relative", "stream_mode": "sidecar"}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x, dist, device=None):
    """Max of a float over all ranks of the process group (the value itself without one):
    the timing rule of the multi-GPU run, so the slowest rank sets the step time."""
    if not dist:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_seed0(rank, fields):
    """First field seed of a rank: every rank compresses its own fields (weak scaling)."""
    return 1 + rank * fields


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """Samples SM clock and clock-event reasons through NVML (read-only) every ~2 ms."""
    REASONS = {0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap",
               0x8: "hw_slowdown", 0x10: "sync_boost", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown",
               0x100: "display_clock_setting"}

    def __init__(self, device_index):
        self.samples, self.reasons, self.max_mhz = [], 0, None
        self.ok = False
        try:
            self.nv = C.CDLL("libnvidia-ml.so.1")
            if self.nv.nvmlInit_v2() != 0:
                return
            self.h = C.c_void_p()
            bus = self._bus_id(device_index)
            rc = self.nv.nvmlDeviceGetHandleByPciBusId_v2(bus, C.byref(self.h)) if bus else 1
            if rc != 0 and self.nv.nvmlDeviceGetHandleByIndex_v2(device_index, C.byref(self.h)) != 0:
                return
            m = C.c_uint()
            if self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(m)) == 0:
                self.max_mhz = m.value
            self.fn_reasons = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(self.nv, "nvmlDeviceGetCurrentClocksThrottleReasons")
            self.ok = True
        except OSError:
            pass

    @staticmethod
    def _bus_id(dev):
        try:
            rt = C.CDLL("libcudart.so")
        except OSError:
            try:
                import torch  # noqa: F401  (torch's cudart is already loaded)
                rt = C.CDLL(None)
            except OSError:
                return None
        buf = C.create_string_buffer(64)
        try:
            if rt.cudaDeviceGetPCIBusId(buf, 64, dev) == 0:
                return buf.value
        except AttributeError:
            return None
        return None

    def _run(self):
        mhz, r = C.c_uint(), C.c_ulonglong()
        while not self._stop.is_set():
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0:
                self.samples.append(mhz.value)
            if self.fn_reasons(self.h, C.byref(r)) == 0:
                self.reasons |= r.value
            time.sleep(0.002)

    def __enter__(self):
        if self.ok:
            self._stop = threading.Event()
            self._t = threading.Thread(target=self._run, daemon=True)
            self._t.start()
        return self

    def __exit__(self, *a):
        if self.ok:
            self._stop.set()
            self._t.join()

    def summary(self):
        if not self.ok:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvml unavailable"], "samples": 0}
        names = [v for k, v in self.REASONS.items() if self.reasons & k and k != 0x1]
        return {"sm_mhz": statistics.median(self.samples) if self.samples else None,
                "sm_max_mhz": self.max_mhz, "reasons": names, "samples": len(self.samples)}


# --------------------------------------------------------------- workload --
def make_fields(count, seed0):
    import importlib
    import __graft_entry__ as g
    g.load_package()
    synth = importlib.import_module("fz_gpu_gb300.synth")
    return [synth.field(KIND, DIMS, seed0 + i) for i in range(count)]


def cpu_round_trips(field, seconds, min_reps=2):
    """Oracle round trips of one field until `seconds` of CPU work; returns (GB/s, reps, s)."""
    import oracle
    n = field.size
    reps, t0 = 0, time.perf_counter()
    while True:
        st = oracle.compress(field, DIMS, EB, rel=True, mode=1)
        oracle.decompress(st)
        reps += 1
        el = time.perf_counter() - t0
        if (el >= seconds and reps >= min_reps) or el > 3 * seconds:
            break
    return 2 * 4 * n * reps / el / 1e9, reps, el


def run_reference(args, rank, world):
    """The reference path's CPU restatement on this host (rank 0 only)."""
    if rank != 0:
        return
    import oracle
    oracle.build()
    field = make_fields(1, 1)[0]
    n = field.size
    for _ in range(args.warmup):
        oracle.decompress(oracle.compress(field, DIMS, EB, rel=True, mode=1))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = oracle.compress(field, DIMS, EB, rel=True, mode=1)
        oracle.decompress(st)
    el = time.perf_counter() - t0
    gbs = 2 * 4 * n * args.steps / el / 1e9
    line = {
        "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * el / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
        "config": config_dict(n),
        "run": {"step": "one round trip (compress + decompress) of one field on the host cores"},
        "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": oracle.threads(), "kind": "port",
                         "sample": f"{args.steps} round trips of one {'x'.join(map(str, DIMS))} field"},
        "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_fz(args, rank, world, local_rank):
    import numpy as np
    import torch
    import __graft_entry__ as g

    fz = g.load_package()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = fz.lib()
    nd_ = min(args.distinct, args.fields)
    fields = make_fields(nd_, rank_seed0(rank, nd_))
    n = fields[0].size
    nf = args.fields
    cap = fz.max_compressed_bytes(n, DIMS, fz.MODE_SIDECAR)
    # field buffer i holds distinct field i % distinct: every buffer is its own memory
    X = [torch.from_numpy(fields[i % nd_]).to(dev) for i in range(nf)]
    S = [torch.empty(cap, dtype=torch.uint8, device=dev) for _ in range(nf)]
    Y = [torch.empty(n, dtype=torch.float32, device=dev) for _ in range(nf)]
    ws = fz.Workspace(n)
    stream = torch.cuda.current_stream(dev)
    sh = C.c_void_p(stream.cuda_stream)
    dims = fz._dims(DIMS)

    # first pass: validate and keep each field's header (decompression takes it from the
    # host, as a caller that just compressed would)
    headers, sizes = [], []
    for i in range(nf):
        nb = C.c_uint64()
        fz._check("compress", L.fz_compress(ws.handle, C.c_void_p(X[i].data_ptr()), n, dims, EB, fz.EB_REL,
                                            fz.MODE_SIDECAR, C.c_void_p(S[i].data_ptr()), cap, C.byref(nb), sh))
        h = fz.parse_header(S[i][:64].cpu().numpy())
        headers.append(h)
        sizes.append(nb.value)
    comp = fz.fields_array([{"src": X[i].data_ptr(), "dst": S[i].data_ptr(), "n": n, "dims": DIMS, "eb": EB,
                             "dst_capacity": cap} for i in range(nf)])
    dec = fz.fields_array([{"src": S[i].data_ptr(), "dst": Y[i].data_ptr(), "src_bytes": sizes[i],
                            "dst_capacity": n, "header": headers[i]} for i in range(nf)])

    def step():
        # one ABI call per direction: the batch's kernels go out back to back
        st = L.fz_compress_batch(ws.handle, comp, nf, fz.EB_REL, fz.MODE_SIDECAR, sh)
        st |= L.fz_decompress_batch(ws.handle, dec, nf, sh)
        if st:
            raise fz.FzError("bench step", st)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    check_recon(X, Y, headers)

    # Timed region 1 (value): the step replayed from one CUDA graph of the round-trip batch,
    # under the schedule fz_batch_autotune_sched picks on these fields before the region.
    best, tuned = fz.batch_autotune_schedule(ws, comp, dec, reps=2, stream=stream)
    gp = fz.Batch.scheduled(ws, comp, dec, best)
    for _ in range(args.warmup):
        gp.launch(stream)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local_rank)
    with clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            gp.launch(stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, dev)
    gp.close()
    check_recon(X, Y, headers)

    # Timed region 2 (kernel durations): the kernels of region 1's branches -- per field a
    # range, an encode, a compaction and a decompression launch -- issued by per-field
    # calls without graphs (every compression, then every decompression), every launch
    # bracketed by a pair of CUDA events on the launching stream (workspace timing).
    def step_fields():
        st = 0
        for i in range(nf):
            st |= L.fz_compress(ws.handle, C.c_void_p(X[i].data_ptr()), n, dims, EB, fz.EB_REL, fz.MODE_SIDECAR,
                                C.c_void_p(S[i].data_ptr()), cap, None, sh)
        for i in range(nf):
            st |= L.fz_decompress(ws.handle, C.c_void_p(S[i].data_ptr()), sizes[i], C.byref(headers[i]),
                                  C.c_void_p(Y[i].data_ptr()), n, sh)
        if st:
            raise fz.FzError("bench step", st)

    ksteps = max(1, min(args.steps, 2))
    ws.enable_timing(ksteps * nf * 5 + 16)
    torch.cuda.synchronize()
    for _ in range(ksteps):
        step_fields()
    torch.cuda.synchronize()
    kern = {k: ws.kernel_time(k) for k in fz.Workspace.KERNELS}
    ws.enable_timing(0)
    launches = args.steps * sum(c for c, _ in kern.values()) // ksteps  # region 1 launches the same kernels
    # Timed region 3 (value_without_graphs): the same steps as one batch call per direction
    # on one stream, without graphs (each field's encode launch also takes the next field's
    # range there), CUDA events around the whole region only.
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s0.record(stream)
    for _ in range(ksteps):
        step()
    s1.record(stream)
    torch.cuda.synchronize()
    calls_ms = s0.elapsed_time(s1)
    check_recon(X, Y, headers)

    bytes_step = nf * 2 * 4 * n
    value = bytes_step * args.steps * world / (ms / 1e3) / 1e9
    hbm, src = peaks()
    stream_b = float(np.mean(sizes))
    kernels, t_c, t_d = kernel_table(kern, n, stream_b, DIMS, hbm)
    dom = max(kernels, key=lambda k: kernels[k]["launches"] * kernels[k]["mean_us"])
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get(dom, {}).get("dram_bytes_per_launch")
        except Exception:
            traffic = None
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator standing in for the EXAFEL field, no dataset)",
        "config": config_dict(n),
        "run": {"fields_per_step": nf, "distinct_fields": nd_,
                "schedule": {"branches": best.branches, "list": best.list,
                             "tuned_ms": {f"{'list+' if l else ''}{b} branches": round(t, 3)
                                          for (b, l), t in tuned.items()}},
                "stream_bytes_mean": int(stream_b),
                "ratio_reference_formula": round(fz.reference_sizes(4 * n, headers[0].nnz)[2], 4),
                "timed_region_ms": round(ms, 2),
                "l2": f"inputs {nf * 4 * n / 1e9:.1f} GB per step > 129 MB L2; each buffer visited once per step"},
        "value_without_graphs": round(bytes_step * ksteps * world / (calls_ms / 1e3) / 1e9, 2),
        "compress_gbs": round(4 * n / (t_c * 1e-3) / 1e9, 1),
        "decompress_gbs": round(4 * n / (t_d * 1e-3) / 1e9, 1),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": kernels[dom]["achieved_gbs"], "peak": hbm,
                     "peak_source": src, "unit": "GB/s", "frac": kernels[dom]["frac"],
                     "traffic": traffic, "algo_bytes": kernels[dom]["algo_bytes"]},
        "kernels": kernels,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if not args.no_e2e:
        line["e2e"] = e2e(fz, L, fields, n, cap, sizes, args, dev, world, dist)
    del X, S, Y
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and not args.quick:
        line["per_dimensionality"] = per_dimensionality(fz, dev, hbm)
        torch.cuda.empty_cache()
        line["batch"] = run_batch(args, local_rank)
        torch.cuda.empty_cache()
        line["serving"] = run_serving(args, local_rank)
    if rank == 0 and world == 1:
        import oracle
        oracle.build()
        cores = oracle.threads()
        gbs, reps, el = cpu_round_trips(fields[0], args.cpu_seconds)
        # the same round trips on one thread (a short sample)
        oracle.set_threads(1)
        gbs1, reps1, el1 = cpu_round_trips(fields[0], max(0.2, args.cpu_seconds / 4), min_reps=1)
        oracle.set_threads(cores)
        line["cpu_baseline"] = {"value": round(gbs, 3), "unit": "GB/s", "cores": cores,
                                "kind": "port", "sample": f"{reps} round trips of one {'x'.join(map(str, DIMS))} field ({el:.1f} s)",
                                "one_thread": {"value": round(gbs1, 3), "sample": f"{reps1} round trips ({el1:.1f} s)"}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def check_recon(X, Y, headers):
    """Spot check: the reconstructions of the first and last buffers meet the error bound."""
    for i in (0, len(X) - 1):
        err = (Y[i] - X[i]).abs().max().item()
        assert err <= headers[i].eb_abs * (1 + 2 ** -10) + 1e-6 * X[i].abs().max().item(), err


def decompress_kernel(dims):
    """The fused decompression kernel the library runs for these dims (the name ncu shows):
    2D rows a multiple of 16 elements take k_decompress2d_x16 when its grid of 960-column x
    16-row windows fits one resident wave (3 CTAs per SM)."""
    import torch
    nd = 3 if dims[2] > 1 else (2 if dims[1] > 1 else 1)
    if nd == 2 and dims[0] % 16 == 0:
        ctas = -(-dims[0] // 960) * -(-dims[1] // 16)
        if ctas <= 3 * torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count:
            return "k_decompress2d_x16"
    return f"k_decompress{nd}d"


def kernel_table(kern, n, stream_b, dims, hbm):
    """Per kernel (by the name ncu shows): launches, mean event-timed duration, algorithmic
    bytes per launch, achieved GB/s and fraction of the HBM peak, share of kernel time;
    plus the compression and decompression time per field (ms)."""
    nb = n // 2048
    # algorithmic bytes per launch: k_range_fields 4n read; k_encode_fields (codes,
    # bitshuffle, flags, per-block compaction into slots) 4n read + the chunks written;
    # k_compact_fields the chunks moved from the slots to Section B (read + write) + the
    # counts and offsets; k_decompress (decode fused with the inverse Lorenzo) the stream
    # read + 4n written
    algo = {"k_range_fields": 4 * n, "k_encode_fields": 4 * n + stream_b,
            "k_compact_fields": 2 * stream_b + 8 * (nb + 1), "k_offsets": 4 * ((n + 255) // 256) + 4 * (nb + 1),
            "k_decompress": stream_b + 4 * n, "k_recon": 2 * n + 4 * n}
    nd = 3 if dims[2] > 1 else (2 if dims[1] > 1 else 1)
    # the names ncu shows: the encode kernel is templated on the dimensionality, the fused
    # decompression kernel has one variant per dimensionality and a second 2D one
    shown = {"k_encode_fields": f"k_encode_fields<{nd}>", "k_decompress": decompress_kernel(dims)}
    total = sum(v[1] for v in kern.values()) or 1.0
    kernels = {}
    for k, (cnt, tot) in kern.items():
        if cnt:
            us = 1e3 * tot / cnt
            gbs = algo[k] / (us * 1e-6) / 1e9
            kernels[shown.get(k, k)] = {"launches": cnt, "mean_us": round(us, 3), "algo_bytes": int(algo[k]),
                                        "achieved_gbs": round(gbs, 1), "frac": round(gbs / hbm, 4),
                                        "share": round(tot / total, 4)}
    per = max(1, kern["k_encode_fields"][0])
    t_c = sum(kern[k][1] for k in ("k_range_fields", "k_encode_fields", "k_compact_fields")) / per
    t_d = sum(kern[k][1] for k in ("k_offsets", "k_decompress", "k_recon")) / max(1, kern["k_decompress"][0])
    return kernels, t_c, t_d


# single-field workloads of the other dimensionalities and row widths: (name, kind, dims,
# relative eb, device buffers per step); every step's input exceeds the L2
OTHERS = [("cesm-like 3600x1800", "smooth2d", (3600, 1800, 1), 1e-3, 16),
          ("hurricane-like 500x500x100", "smooth3d", (500, 500, 100), 1e-3, 6),
          ("hurricane-like 500x500x100 eb 1e-2", "smooth3d", (500, 500, 100), 1e-2, 6),
          ("exafel-like 39201x388 (rows not a multiple of 4)", "peaks2d", (39201, 388, 1), 1e-3, 8),
          ("hurricane-like 501x500x100 (rows not a multiple of 4)", "smooth3d", (501, 500, 100), 1e-3, 6),
          ("1D 2^25", "smooth1d", (1 << 25, 1, 1), 1e-3, 4)]


def per_dimensionality(fz, dev, hbm):
    """For each workload of OTHERS: compress-only and decompress-only batch graphs over its
    buffers (8 branches), replayed (GB/s of uncompressed bytes per direction), and the
    kernels' event times from a pass of plain calls."""
    import importlib
    import torch
    synth = importlib.import_module("fz_gpu_gb300.synth")
    out = {}
    for name, kind, dims, eb, copies in OTHERS:
        f = synth.field(kind, dims, 7)
        n = f.size
        x0 = torch.from_numpy(f).to(dev)
        X = [x0.clone() for _ in range(copies)]
        del x0
        cap = fz.max_compressed_bytes(n, dims)
        S = [torch.empty(cap, dtype=torch.uint8, device=dev) for _ in range(copies)]
        Y = [torch.empty(n, dtype=torch.float32, device=dev) for _ in range(copies)]
        ws = fz.Workspace(n)
        heads, sizes = [], []
        for i in range(copies):
            st = fz.compress(X[i], dims, eb, ws=ws, out=S[i])
            heads.append(fz.parse_header(st[:64].cpu().numpy()))
            sizes.append(st.numel())
        comp = fz.fields_array([{"src": X[i].data_ptr(), "dst": S[i].data_ptr(), "n": n, "dims": dims, "eb": eb,
                                 "dst_capacity": cap} for i in range(copies)])
        dec = fz.fields_array([{"src": S[i].data_ptr(), "dst": Y[i].data_ptr(), "src_bytes": sizes[i],
                                "dst_capacity": n, "header": heads[i]} for i in range(copies)])
        res = {"field_elems": n, "buffers": copies, "ratio_reference_formula":
               round(fz.reference_sizes(4 * n, heads[0].nnz)[2], 3)}
        for what, g in (("compress", fz.Batch.scheduled(ws, comp, None, fz.Schedule(8, 0))),
                        ("decompress", fz.Batch.scheduled(ws, None, dec, fz.Schedule(8, 0)))):
            for _ in range(3):
                g.launch()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(5):
                g.launch()
            e1.record()
            torch.cuda.synchronize()
            res[what + "_gbs"] = round(copies * 4 * n * 5 / (e0.elapsed_time(e1) * 1e-3) / 1e9, 1)
            g.close()
        ws.enable_timing(copies * 5 + 8)
        for i in range(copies):
            fz.compress(X[i], dims, eb, ws=ws, out=S[i], readback=False)
            fz.decompress(S[i], header=heads[i], ws=ws, out=Y[i])
        torch.cuda.synchronize()
        kern = {k: ws.kernel_time(k) for k in fz.Workspace.KERNELS}
        kt, _, _ = kernel_table(kern, n, float(sum(sizes)) / copies, dims, hbm)
        res["kernels"] = {k: {"mean_us": v["mean_us"], "frac": v["frac"]} for k, v in kt.items()}
        out[name] = res
        del X, S, Y, ws
        torch.cuda.empty_cache()
    return out


# host threads on each side of the e2e pipeline: compressing threads hand their streams
# to decompressing threads, so input copies (H2D) and output copies (D2H) run at once on
# the host link (measured 210 + 193 GB/s one-way, 339 both)
E2E_THREADS = int(os.environ.get("FZ_E2E_THREADS", "8"))


def e2e(fz, L, fields, n, cap, sizes, args, dev, world, dist):
    """Host-buffer round trips through fz_compress_host / fz_decompress_host.

    E2E_THREADS compressing threads (a workspace and stream each) take the step's fields
    in turn from pinned host memory and compress each into a pinned stream buffer of a
    shared pool; E2E_THREADS decompressing threads take the finished streams in order
    and decompress each back into pinned host memory.  The calls release the GIL.  Every
    field is compressed and decompressed once per step; the region ends when the last
    decompression has returned."""
    import queue
    import numpy as np
    import torch
    steps = min(args.steps, 5)
    nf = args.fields  # round trips per step, as in the device-timed step (field i % distinct)
    nd_ = len(fields)
    items = steps * nf
    T = E2E_THREADS
    hin = [torch.from_numpy(f).pin_memory() for f in fields]
    dims = fz._dims(DIMS)
    free, ready = queue.Queue(), queue.Queue()
    for _ in range(2 * T):
        free.put(torch.empty(cap, dtype=torch.uint8).pin_memory())
    cw = [{"ws": fz.Workspace(n), "st": torch.cuda.Stream(dev), "bytes": 0, "err": None} for _ in range(T)]
    dw = [{"ws": fz.Workspace(n), "st": torch.cuda.Stream(dev), "last": None, "err": None,
           "hout": torch.empty(n, dtype=torch.float32).pin_memory()} for _ in range(T)]

    def compress(w, i, buf):
        nb = C.c_uint64()
        st = L.fz_compress_host(w["ws"].handle, C.c_void_p(hin[i].data_ptr()), n, dims, EB, fz.EB_REL,
                                fz.MODE_SIDECAR, C.c_void_p(buf.data_ptr()), cap, C.byref(nb),
                                C.c_void_p(w["st"].cuda_stream))
        if st:
            raise fz.FzError("e2e compress", st)
        return nb.value

    def decompress(w, buf, nbytes):
        st = L.fz_decompress_host(w["ws"].handle, C.c_void_p(buf.data_ptr()), nbytes,
                                  C.c_void_p(w["hout"].data_ptr()), n, C.c_void_p(w["st"].cuda_stream))
        if st:
            raise fz.FzError("e2e decompress", st)

    def run_compress(k):
        w = cw[k]
        torch.cuda.set_device(dev)
        try:
            for j in range(k, items, T):
                buf = free.get(timeout=120)  # raises if the decompressing side has stopped
                nb = compress(w, (j % nf) % nd_, buf)
                w["bytes"] += nb
                ready.put((buf, nb, (j % nf) % nd_))
        except Exception as ex:  # surfaced after join
            w["err"] = ex
            ready.put(None)

    def run_decompress(k):
        w = dw[k]
        torch.cuda.set_device(dev)
        try:
            while True:
                it = ready.get(timeout=120)
                if it is None:
                    return
                buf, nb, i = it
                decompress(w, buf, nb)
                w["last"] = i
                free.put(buf)
        except Exception as ex:
            w["err"] = ex

    # warm-up: every workspace allocates its staging buffers
    buf = free.get()
    for w in cw:
        nb = compress(w, 0, buf)
    for w in dw:
        decompress(w, buf, nb)
    free.put(buf)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tc = [threading.Thread(target=run_compress, args=(k,)) for k in range(T)]
    td = [threading.Thread(target=run_decompress, args=(k,)) for k in range(T)]
    for t in tc + td:
        t.start()
    for t in tc:
        t.join()
    for _ in td:
        ready.put(None)
    for t in td:
        t.join()
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    for w in cw + dw:
        if w["err"] is not None:
            raise w["err"]
    el = max_over_ranks(el, dist, dev)
    for w in dw:
        last = fields[w["last"]]
        err = float(np.max(np.abs(w["hout"].numpy().astype(np.float64) - last)))
        assert err <= 1e-3 * float(np.float32(last.max() - last.min())) * 1.001, err
    per_step_stream = sum(w["bytes"] for w in cw) / steps
    return {"value": round(nf * 2 * 4 * n * steps * world / el / 1e9, 2), "unit": "GB/s",
            "steps": steps, "host_threads": {"compress": T, "decompress": T},
            "h2d_bytes_per_step": int(nf * 4 * n + per_step_stream),
            "d2h_bytes_per_step": int(per_step_stream + nf * 4 * n)}


def _torch_fields(specs, dev):
    import importlib
    import __graft_entry__ as g
    g.load_package()
    synth = importlib.import_module("fz_gpu_gb300.synth")
    return [synth.field_torch(kind, dims, seed, device=dev) for kind, dims, _, seed in specs]


def run_batch(args, local_rank):
    """The 512-field mixed batch (log-uniform 64 KB-256 MB, 1D/2D/3D, eb from
    {1e-2,1e-3,1e-4}) compressed and decompressed as one round-trip CUDA-graph replay under
    every schedule fz_batch_autotune_sched tries (per-field launches on 1-16 parallel
    branches, or the compression as list launches over a device work list of all fields),
    against the plain per-field path (fz_compress with its size readback, then
    fz_decompress, one field at a time).  Returns the figures as a dict."""
    import importlib
    import torch
    import __graft_entry__ as g
    fz = g.load_package()
    synth = importlib.import_module("fz_gpu_gb300.synth")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    specs = synth.mixed_specs(args.batch_fields, seed=3)
    X = _torch_fields(specs, dev)
    ns = [x.numel() for x in X]
    caps = [fz.max_compressed_bytes(n, d) for n, (_, d, _, _) in zip(ns, specs)]
    S = [torch.empty(c, dtype=torch.uint8, device=dev) for c in caps]
    Y = [torch.empty(n, dtype=torch.float32, device=dev) for n in ns]
    ws = fz.Workspace(max(ns))
    total = 4 * sum(ns)
    stream = torch.cuda.current_stream(dev)

    def plain():
        for x, s_, y, (_, d, eb, _) in zip(X, S, Y, specs):
            st = fz.compress(x, d, eb, ws=ws, out=s_)
            fz.decompress(st, ws=ws, out=y)
    plain()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain()
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    heads = [fz.parse_header(s_[:64].cpu().numpy()) for s_ in S]
    sizes = [fz.stream_bytes(h) for h in heads]
    ref = [s_[:b].clone() for s_, b in zip(S[:16], sizes[:16])]
    comp = fz.fields_array([{"src": x.data_ptr(), "dst": s_.data_ptr(), "n": n, "dims": d, "eb": eb,
                             "dst_capacity": s_.numel()} for x, s_, n, (_, d, eb, _) in zip(X, S, ns, specs)])
    dec = fz.fields_array([{"src": s_.data_ptr(), "dst": y.data_ptr(), "src_bytes": b, "dst_capacity": y.numel(),
                            "header": h} for s_, y, b, h in zip(S, Y, sizes, heads)])
    best, tuned = fz.batch_autotune_schedule(ws, comp, dec, reps=2, stream=stream)
    gb = fz.Batch.scheduled(ws, comp, dec, best)
    for _ in range(2):
        gb.launch(stream)
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 5))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        gb.launch(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    t_batch = e0.elapsed_time(e1) / 1e3 / steps
    gb.close()
    # the replays wrote the plain path's streams (which tests check bit for bit)
    assert all(torch.equal(s_[: r.numel()], r) for s_, r in zip(S, ref))
    ratio = sum(4 * n for n in ns) / sum(sizes)
    gbs = lambda t: round(2 * total / t / 1e9, 2)
    out = {"metric": "512 mixed fields: batched vs per-field aggregate GB/s (compress + decompress)",
           "value": gbs(t_batch), "unit": "GB/s", "per_field_plain": gbs(t_plain),
           "speedup_vs_per_field": round(t_plain / t_batch, 2),
           "schedule": {"branches": best.branches, "list": best.list},
           "schedules_gbs": {f"{'list+' if l else ''}{b} branches": gbs(t / 1e3) for (b, l), t in tuned.items()},
           "fields": len(specs), "total_gb": round(total / 1e9, 3), "steps": steps,
           "aggregate_ratio": round(ratio, 3), "higher_is_better": True,
           "data": "synthetic (seeded device-side generators)",
           "config": {"workload": "mixed 1D/2D/3D, sizes log-uniform 64 KB-256 MB, eb in {1e-2,1e-3,1e-4}",
                      "batched": "one round-trip CUDA-graph replay (fz_batch_launch) per step, schedule from "
                                 "fz_batch_autotune_sched",
                      "per_field": "fz_compress with size readback + fz_decompress, one field at a time"}}
    del X, S, Y, ref
    return out


def run_serving(args, local_rank):
    """Poisson arrivals (mean --serve-rate req/s) of fields drawn from the 512-field mix,
    60/40 compress/decompress, served by the request loop (8 slots, HBM budget) against
    the same trace served one request at a time (1 slot).  Two request kinds:
    device-resident fields (FZ_REQUEST_DEVICE, the fields and results live in HBM; drawn
    from all 512 fields) and host buffers (pinned; H2D/D2H copies per request; drawn from
    the first --serve-host-fields fields).  Returns the figures as a dict."""
    import importlib
    import numpy as np
    import torch
    import __graft_entry__ as g
    fz = g.load_package()
    synth = importlib.import_module("fz_gpu_gb300.synth")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    specs = synth.mixed_specs(args.batch_fields, seed=3)
    Xd = _torch_fields(specs, dev)
    ns = [x.numel() for x in Xd]
    ws = fz.Workspace(max(ns))
    caps = [fz.max_compressed_bytes(x.numel(), d) for x, (_, d, _, _) in zip(Xd, specs)]
    Sd = [fz.compress(x, d, eb, ws=ws) for x, (_, d, eb, _) in zip(Xd, specs)]  # streams to decompress
    sbytes = [s_.numel() for s_ in Sd]
    heads = [fz.parse_header(s_[:64].cpu().numpy()) for s_ in Sd]
    out_c = [torch.empty(c, dtype=torch.uint8, device=dev) for c in caps]
    out_d = [torch.empty(n, dtype=torch.float32, device=dev) for n in ns]
    nh = min(args.serve_host_fields, len(specs))
    hin = [x.cpu().pin_memory() for x in Xd[:nh]]
    hst = [s_.cpu().pin_memory() for s_ in Sd[:nh]]
    hout_c = [torch.empty(c, dtype=torch.uint8).pin_memory() for c in caps[:nh]]
    hout_d = [torch.empty(n, dtype=torch.float32).pin_memory() for n in ns[:nh]]
    torch.cuda.synchronize()
    rng = np.random.default_rng(4)
    nreq = int(args.serve_rate * args.serve_seconds)
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, nreq))
    draw = rng.random(nreq)
    comp = rng.random(nreq) < 0.6
    free = torch.cuda.mem_get_info(dev)[0]
    budget = int(min(120 << 30, free - (16 << 30)))

    def serve(slots, device, trace=True):
        nf = len(specs) if device else nh
        fields = (draw * nf).astype(np.int64)
        server = fz.Server(budget, slots, max(ns))
        lat = np.zeros(nreq)

        def submit(i):
            f = int(fields[i])
            _, d, eb, _ = specs[f]
            if comp[i]:
                src, dst = (Xd[f], out_c[f]) if device else (hin[f], hout_c[f])
                server.submit(i, fz.COMPRESS, src.data_ptr(), dst.data_ptr(), caps[f], n=ns[f], dims=d, eb=eb,
                              device=device)
            else:
                src, dst = (Sd[f], out_d[f]) if device else (hst[f], hout_d[f])
                server.submit(i, fz.DECOMPRESS, src.data_ptr(), dst.data_ptr(), 4 * ns[f], src_bytes=sbytes[f],
                              device=device, header=heads[f] if device else None)

        i = 0
        if not trace:  # saturated: the whole trace is queued before the clock starts (no work runs until poll)
            for i in range(nreq):
                submit(i)
            i = nreq
        t0 = time.perf_counter()
        done, last = 0, 0.0
        while done < nreq:
            now = time.perf_counter() - t0
            while i < nreq and arrivals[i] <= now:
                submit(i)
                i += 1
            for rid, st, _ in server.poll():
                if st != fz.SUCCESS:
                    raise fz.FzError("serving", st)
                now = time.perf_counter() - t0
                lat[rid] = now - (arrivals[rid] if trace else 0.0)
                last = max(last, now)
                done += 1
        server.close()
        moved = float(sum(4 * ns[int(f)] for f in fields))
        return lat, moved / last / 1e9

    pct = lambda a: {"p50_ms": round(1e3 * float(np.percentile(a, 50)), 3),
                     "p99_ms": round(1e3 * float(np.percentile(a, 99)), 3),
                     "p99.9_ms": round(1e3 * float(np.percentile(a, 99.9)), 3)}

    def mode(device):
        lat8, gbs8 = serve(8, device)
        lat1, gbs1 = serve(1, device)
        sat8 = serve(8, device, trace=False)[1]
        sat1 = serve(1, device, trace=False)[1]
        return {"served": dict(slots=8, gbs=round(gbs8, 2), **pct(lat8)),
                "one_at_a_time": dict(slots=1, gbs=round(gbs1, 2), **pct(lat1)),
                "saturated_gbs": {"slots8": round(sat8, 2), "slots1": round(sat1, 2),
                                  "speedup": round(sat8 / sat1, 2)}}

    def plain():
        """The plain per-field path on the same trace, device-resident: fz_compress with
        its size readback, fz_decompress, one request at a time."""
        fields = (draw * len(specs)).astype(np.int64)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(nreq):
            f = int(fields[i])
            _, d, eb, _ = specs[f]
            if comp[i]:
                fz.compress(Xd[f], d, eb, ws=ws, out=out_c[f])
            else:
                fz.decompress(Sd[f], header=heads[f], ws=ws, out=out_d[f])
        torch.cuda.synchronize()
        return float(sum(4 * ns[int(f)] for f in fields)) / (time.perf_counter() - t0) / 1e9

    serve(8, True, trace=False)  # warm-up: workspaces, module load
    dev_mode = mode(True)
    plain_gbs = plain()
    dev_mode["saturated_gbs"]["plain_per_field"] = round(plain_gbs, 2)
    dev_mode["saturated_gbs"]["speedup_vs_plain"] = round(dev_mode["saturated_gbs"]["slots8"] / plain_gbs, 2)
    serve(8, False, trace=False)  # warm-up of the host-buffer path (staging pool, first copies)
    host_mode = mode(False)
    out = {"metric": "Poisson request trace: served latency and aggregate GB/s (uncompressed bytes)",
           "requests": nreq, "rate_req_s": args.serve_rate, "hbm_budget_gb": round(budget / 2 ** 30, 1),
           "device_resident": dev_mode, "host_buffers": host_mode,
           "data": f"synthetic (seeded device-side generators; {len(specs)}-field mix, host buffers: its first {nh})",
           "config": {"workload": "Poisson arrivals, 60/40 compress/decompress, fields drawn from the 512-field mix",
                      "requests": "device-resident fields and results (FZ_REQUEST_DEVICE); "
                                  "host_buffers: the same kind of trace with pinned host buffers"}}
    del Xd, Sd, out_c, out_d, hin, hst, hout_c, hout_d
    return out


def run_list_kernels(args, local_rank):
    """The list launches of a batch compression -- one range launch over every field, one
    encode launch per dimensionality present, one compaction launch -- on the first
    --list-fields fields of the 512-field mix of at most 32 MB (1D/2D/3D, rows that are and
    are not a multiple of 4, every eb), --steps times, every stream checked against the
    per-field calls' after the last step.  Prints one line naming a step's launches."""
    import importlib
    import numpy as np
    import torch
    import __graft_entry__ as g
    fz = g.load_package()
    synth = importlib.import_module("fz_gpu_gb300.synth")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    specs = [sp for sp in synth.mixed_specs(512, seed=3) if 4 * int(np.prod(sp[1])) <= 32 << 20][:args.list_fields]
    X = _torch_fields(specs, dev)
    ns = [x.numel() for x in X]
    caps = [fz.max_compressed_bytes(n, d) for n, (_, d, _, _) in zip(ns, specs)]
    S = [torch.empty(c, dtype=torch.uint8, device=dev) for c in caps]
    ws = fz.Workspace(max(ns))
    ref = [fz.compress(x, d, eb, ws=ws).clone() for x, (_, d, eb, _) in zip(X, specs)]
    comp = fz.fields_array([{"src": x.data_ptr(), "dst": s_.data_ptr(), "n": n, "dims": d, "eb": eb,
                             "dst_capacity": s_.numel()} for x, s_, n, (_, d, eb, _) in zip(X, S, ns, specs)])
    gb = fz.Batch.scheduled(ws, comp, None, fz.Schedule(1, 1))
    for _ in range(args.steps):
        gb.launch()
    torch.cuda.synchronize()
    gb.close()
    assert all(torch.equal(s_[: r.numel()], r) for s_, r in zip(S, ref))
    nds = sorted({fz.ndim(d) for _, d, _, _ in specs})
    by_nd = {d: {"fields": 0, "elems": 0, "stream_bytes": 0} for d in nds}
    for (_, d, _, _), n, r in zip(specs, ns, ref):
        k = by_nd[fz.ndim(d)]
        k["fields"] += 1
        k["elems"] += n
        k["stream_bytes"] += r.numel()
    print(json.dumps({"workload": f"the first {len(specs)} fields of the 512-field mix of at most 32 MB "
                                  f"({4 * sum(ns) / 1e6:.0f} MB, dimensionalities {nds})", "steps": args.steps,
                      "per_step": ["k_range_fields<list>"] + [f"k_encode_fields<{d}, list>" for d in nds] +
                                  ["k_compact_fields<list>"],
                      "by_dimensionality": by_nd}))


def run_kernels(args, local_rank):
    """Every kernel kind once per step on one --field field: compression (range, encode,
    compaction), decompression of the sidecar stream, decompression of a COMPAT stream
    (block offsets first), and the no-allocation compression (the look-back kernel), each
    checked against the workspace path's bytes.  Prints one line of launches per kind."""
    import torch
    import __graft_entry__ as g
    fz = g.load_package()
    torch.cuda.set_device(local_rank)
    f = make_fields(1, 1)[0]
    x = torch.from_numpy(f).cuda()
    n = x.numel()
    ws = fz.Workspace(n)
    caps = {m: fz.max_compressed_bytes(n, DIMS, m) for m in (fz.MODE_SIDECAR, fz.MODE_COMPAT)}
    out = {m: torch.empty(caps[m], dtype=torch.uint8, device="cuda") for m in caps}
    y = torch.empty(n, dtype=torch.float32, device="cuda")
    na = torch.empty(caps[fz.MODE_SIDECAR], dtype=torch.uint8, device="cuda")
    noalloc = n <= (1 << 26)
    for _ in range(args.steps):
        for m in (fz.MODE_SIDECAR, fz.MODE_COMPAT):
            st = fz.compress(x, DIMS, EB, mode=m, ws=ws, out=out[m])
            fz.decompress(st, ws=ws, out=y)
        if noalloc:
            nb = C.c_uint64()
            fz._check("fz_compress_noalloc", fz.lib().fz_compress_noalloc(
                C.c_void_p(x.data_ptr()), n, fz._dims(DIMS), EB, fz.EB_REL, fz.MODE_SIDECAR,
                C.c_void_p(na.data_ptr()), na.numel(), C.byref(nb), fz._stream_handle(None)))
            assert torch.equal(na[: nb.value], out[fz.MODE_SIDECAR][: nb.value])
    torch.cuda.synchronize()
    print(json.dumps({"workload": WORKLOAD, "steps": args.steps,
                      "per_step": ["k_range_fields", "k_encode_fields", "k_compact_fields", "k_decompress (sidecar)",
                                   "k_range_fields", "k_encode_fields", "k_compact_fields", "k_offsets",
                                   "k_decompress (COMPAT)"] + (["k_range", "k_compress"] if noalloc else [])}),
          flush=True)


def main():
    global DIMS, EB, KIND, WORKLOAD
    args = parse_args()
    DIMS, EB, KIND, WORKLOAD = FIELDS[args.field]
    rank, world, local_rank = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "batch":
        if rank == 0:
            print(json.dumps(run_batch(args, local_rank)), flush=True)
    elif args.workload == "serving":
        if rank == 0:
            print(json.dumps(run_serving(args, local_rank)), flush=True)
    elif args.workload == "kernels":
        if rank == 0:
            run_kernels(args, local_rank)
    elif args.workload == "listkernels":
        if rank == 0:
            run_list_kernels(args, local_rank)
    else:
        run_fz(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
