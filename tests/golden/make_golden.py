"""Generate the golden fixtures that pin the oracle to the reference's own kernels.

Runs on a CUDA machine.  It launches the reference's c_lorenzo_{1d,2d,3d},
bitshuffleAndBitflag and encodeDebug -- compiled from the FZ-GPU sources into
oracle/_ref/ref_kernels.fatbin by `make -C oracle ref` -- through
oracle/ref_harness/ref_loader.cpp, repeating runSzs's buffer set-up and launch
sequence (fz.cu:136-205), and stores inputs and every intermediate buffer as
tests/golden/<case>.npz.  The exclusive scan between bitshuffle and encode is an exact
integer prefix sum (cub::DeviceScan::ExclusiveSum, fz.cu:187-192); it is computed here
with torch.cumsum on the device.

    python tests/golden/make_golden.py <outdir>

The fixtures are written to <outdir> (then copied into tests/golden/ where the machine that
ran them is not this one).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")
FATBIN = os.path.join(REF_DIR, "ref_kernels.fatbin")
LOADER_SRC = os.path.join(ROOT, "oracle", "ref_harness", "ref_loader.cpp")
LOADER_SO = os.path.join(REF_DIR, "libfzref.so")


def build_loader():
    cuda = "/usr/local/cuda"
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-I" + cuda + "/include", LOADER_SRC,
                           "-o", LOADER_SO, "-L" + cuda + "/lib64/stubs", "-lcuda"])


def cases():
    """(name, data float32[n], dims, eb, rel)"""
    sys.path.insert(0, ROOT)
    import importlib.util
    spec = importlib.util.spec_from_file_location("synth", os.path.join(ROOT, "fz-gpu_gb300", "synth.py"))
    S = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(S)
    out = []
    out.append(("2d_smooth_300x70", S.smooth2d(300, 70, seed=11), (300, 70, 1), 1e-3, True))
    out.append(("2d_peaks_400x90", S.peaks2d(400, 90, seed=12, npeaks=12), (400, 90, 1), 1e-4, True))
    out.append(("2d_odd_101x37", S.smooth2d(101, 37, seed=14), (101, 37, 1), 1e-3, True))
    out.append(("3d_smooth_40x33x20", S.smooth3d(40, 33, 20, seed=13), (40, 33, 20), 1e-3, True))
    out.append(("3d_odd_37x19x11", S.smooth3d(37, 19, 11, seed=15), (37, 19, 11), 1e-2, True))
    out.append(("1d_smooth_10000", S.smooth1d(10000, seed=16), (10000, 1, 1), 1e-3, True))
    out.append(("1d_short_1500", S.smooth1d(1500, seed=17), (1500, 1, 1), 1e-3, True))
    # file longer than the dims (fz.cu:117-118): codes past x*y stay 0
    d = np.concatenate([S.smooth2d(64, 64, seed=18), np.linspace(-1, 1, 777, dtype=np.float32)])
    out.append(("2d_len_gt_dims_64x64p777", d, (64, 64, 1), 1e-3, True))
    # crafted deltas around the 15/16-bit limits, non-finite values; ebx2_r = 1
    vals = np.array([0, 1, -1, 2.5, -2.5, 0.5, -0.5, 1.5, 30000, 32767, 32768, -32768, 40000, 65535,
                     65536, -65536, 70000, -70000, 1e6, -1e9, 3e38, np.inf, -np.inf, np.nan,
                     -np.nan, 12345.5, -0.0, 7, 100000, 32767.5, 65535.5, 65534.7], np.float32)
    g2 = np.zeros((16, 16 * vals.size), np.float32)
    g2[0, ::16] = vals
    g2[5, 3::16] = vals[::-1]
    out.append(("2d_crafted_limits", g2.ravel(), (16 * vals.size, 16, 1), 0.5, False))
    g1 = np.zeros(256 * vals.size, np.float32)
    g1[::256] = vals
    g1[131::256] = vals[::-1]
    out.append(("1d_crafted_limits", g1, (g1.size, 1, 1), 0.5, False))
    g3 = np.zeros((8, 8, 8 * vals.size), np.float32)
    g3[0, 0, ::8] = vals
    g3[3, 2, 5::8] = vals[::-1]
    out.append(("3d_crafted_limits", g3.ravel(), (8 * vals.size, 8, 8), 0.5, False))
    return out


def run(outdir):
    import torch
    if not os.path.exists(FATBIN):
        raise SystemExit(f"missing {FATBIN}: build it with `make -C oracle ref` where the FZ-GPU sources are")
    build_loader()
    torch.zeros(1, device="cuda")  # create the primary context
    L = C.CDLL(LOADER_SO)
    rc = L.ref_load(FATBIN.encode())
    if rc != 0:
        raise SystemExit(f"ref_load failed: {rc}")
    vp, u32, f32 = C.c_void_p, C.c_uint, C.c_float
    L.ref_c_lorenzo.argtypes = [C.c_int, vp, vp, vp, u32, u32, u32, f32, vp]
    L.ref_bitshuffle.argtypes = [vp, vp, u32, vp, vp, vp]
    L.ref_encode.argtypes = [vp, vp, vp, u32, vp]
    os.makedirs(outdir, exist_ok=True)
    stream = torch.cuda.current_stream().cuda_stream
    for name, data, dims, eb, rel in cases():
        data = np.ascontiguousarray(data, np.float32)
        n = data.size
        x, y, z = dims
        nd = 1 if (z == 1 and y == 1) else (2 if z == 1 else 3)
        if rel:
            rng = np.float32(np.max(data) - np.min(data))  # fz.cu:137
            eb_abs = float(eb) * float(rng)                 # fz.cu:149
        else:
            rng = np.float32(0)
            eb_abs = float(eb)
        ebx2_r = np.float32(1.0 / (eb_abs * 2))             # lorenzo_var.cuh:562-563
        d_data = torch.from_numpy(data).cuda()
        quant = torch.zeros(n + 2, dtype=torch.int16, device="cuda")  # fz.cu:140,145 (+pad)
        signum = torch.zeros(n, dtype=torch.uint8, device="cuda")
        assert L.ref_c_lorenzo(nd, d_data.data_ptr(), quant.data_ptr(), signum.data_ptr(), x, y, z,
                               float(ebx2_r), stream) == 0
        shuf = quant.clone()                                             # fz.cu:154-155
        nl = 2 * n
        nl = nl if nl % 8192 == 0 else nl - nl % 8192 + 8192              # fz.cu:158-159
        dcs1 = nl // 512 if nl % 512 == 0 else nl // 512 + 1              # fz.cu:160-161
        bitflag = torch.zeros(dcs1, dtype=torch.int32, device="cuda")
        byteflag = torch.zeros(32 * dcs1, dtype=torch.int32, device="cuda")
        d_out = torch.zeros(16 * 32 * dcs1, dtype=torch.uint8, device="cuda")
        assert L.ref_bitshuffle(quant.data_ptr(), shuf.data_ptr(), n, bitflag.data_ptr(),
                                byteflag.data_ptr(), stream) == 0
        dcs2 = (2 * n + 511) // 512                                       # fz.cu:177-178
        m = 32 * dcs2
        f = byteflag[:m].to(torch.int64)
        presum = torch.zeros(m + 1, dtype=torch.int64, device="cuda")
        presum[1:] = torch.cumsum(f, 0)
        presum32 = presum.to(torch.int32).contiguous()
        assert L.ref_encode(shuf.data_ptr(), d_out.data_ptr(), presum32.data_ptr(), n, stream) == 0
        torch.cuda.synchronize()
        nnz = int(presum[m].item())
        np.savez_compressed(
            os.path.join(outdir, name + ".npz"),
            data=data, dims=np.array(dims, np.uint32), eb=np.float64(eb), rel=np.bool_(rel),
            eb_abs=np.float64(eb_abs), ebx2_r=ebx2_r, range=rng,
            quant=quant[:n].cpu().numpy().view(np.uint16),
            signum=signum.cpu().numpy(),
            shuffled=shuf[:n].cpu().numpy().view(np.uint16),
            byteflag=byteflag[:m].cpu().numpy().view(np.uint32),
            bitflag=bitflag[:dcs2].cpu().numpy().view(np.uint32),
            presum=presum32.cpu().numpy().view(np.uint32),
            d_out=d_out[: 16 * nnz].cpu().numpy(), nnz=np.int64(nnz))
        print(f"{name}: n={n} nd={nd} nnz={nnz}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <outdir>")
    run(sys.argv[1])
