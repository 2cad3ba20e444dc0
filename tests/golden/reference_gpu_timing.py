"""Per-stage device time of the reference's own GPU pipeline on this GPU (test
infrastructure; needs oracle/_ref/ref_kernels.fatbin).

For each single-field workload: runSzs's device sequence (tests/golden/refpipe.py) is
run `--warmup` times, then `--reps` times with CUDA events around every stage; the
median of each stage is printed as one JSON line per workload, next to the product's
compression of the same field (fz_compress with a workspace, relative eb, no readback;
CUDA events around the call).  The fields (26-100 MB) fit in the 129 MB L2, so every
repetition first writes a 256 MB buffer to flush it.

    python tests/golden/reference_gpu_timing.py [--reps 20] [--warmup 3]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

WORKLOADS = [
    ("exafel-like 39200x388", "peaks2d", (39200, 388, 1), 1, 1e-3),
    ("cesm-like 3600x1800", "smooth2d", (3600, 1800, 1), 0, 1e-3),
    ("hurricane-like 500x500x100", "smooth3d", (500, 500, 100), 2, 1e-3),
]


def main():
    import numpy as np
    import torch
    import __graft_entry__ as g
    import refpipe
    from importlib import import_module

    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    args = ap.parse_args()
    fz = g.load_package()
    synth = import_module("fz_gpu_gb300.synth")
    ref = refpipe.RefPipeline()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for name, kind, dims, seed, eb in WORKLOADS:
        data = synth.field(kind, dims, seed)
        n = data.size
        x = torch.from_numpy(data).cuda()
        eb_abs = float(eb) * float(np.float32(data.max() - data.min()))
        stages = {k: [] for k in refpipe.RefPipeline.STAGES}
        for i in range(args.warmup + args.reps):
            flush.fill_(i & 0xFF)
            r = ref.run(x, dims, eb_abs, timed=True)
            if i >= args.warmup:
                for k, v in r["ms"].items():
                    stages[k].append(v)
        med = {k: statistics.median(v) for k, v in stages.items()}
        device = sum(v for k, v in med.items() if k != "scalar_copies")
        kernels = med["c_lorenzo"] + med["bitshuffleAndBitflag"] + med["cub_exclusive_sum"] + med["encodeDebug"]
        # the product on the same field
        ws = fz.Workspace(n)
        cap = fz.max_compressed_bytes(n, dims)
        out = torch.empty(cap, dtype=torch.uint8, device="cuda")
        times = []
        for i in range(args.warmup + args.reps):
            flush.fill_(i & 0xFF)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fz.compress(x, dims, eb, ws=ws, out=out, readback=False)
            e1.record()
            torch.cuda.synchronize()
            if i >= args.warmup:
                times.append(e0.elapsed_time(e1))
        ours = statistics.median(times)
        line = {"workload": name, "n": n, "eb": eb, "nnz": r["nnz"], "reps": args.reps,
                "reference_stage_ms": {k: round(v, 5) for k, v in med.items()},
                "reference_device_ms": round(device, 5),
                "reference_kernels_ms": round(kernels, 5),
                "reference_device_gbs": round(4 * n / (device * 1e-3) / 1e9, 1),
                "reference_kernels_gbs": round(4 * n / (kernels * 1e-3) / 1e9, 1),
                "fz_compress_ms": round(ours, 5),
                "fz_compress_gbs": round(4 * n / (ours * 1e-3) / 1e9, 1),
                "speedup_vs_reference_device": round(device / ours, 2),
                "note": "scalar_copies is runSzs's three blocking one-word copies around the scan, "
                        "host round trip included; excluded from reference_device_ms"}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
