"""The reference's own compression kernels on a GPU (test infrastructure only).

Runs runSzs's device sequence (fz.cu:139-205) with the reference's kernels --
c_lorenzo_{1d,2d,3d} and bitshuffleAndBitflag and encodeDebug from
oracle/_ref/ref_kernels.fatbin (built by `make -C oracle ref REF=<FZ-GPU sources>`), the
CUB ExclusiveSum of fz.cu:187-192 (oracle/ref_harness/ref_scan.cu) -- with runSzs's
buffer sizes, memsets and device-to-device copies, minus file I/O and the per-run
cudaMalloc/cudaFree.  Used by tests/test_gpu_reference_kernels.py (full-size parity
against the reference itself) and by reference_gpu_timing.py (the reference pipeline's
per-stage times on this GPU).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")
FATBIN = os.path.join(REF_DIR, "ref_kernels.fatbin")


def available():
    return os.path.exists(FATBIN)


class RefPipeline:
    """Loads the reference kernels into the current CUDA context (device 0)."""

    STAGES = ("memset_quant", "c_lorenzo", "copy_quant", "memset_flags", "bitshuffleAndBitflag",
              "copy_byteflags", "cub_exclusive_sum", "scalar_copies", "encodeDebug")

    def __init__(self):
        import torch
        if not available():
            raise FileNotFoundError(FATBIN)
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "harness"])
        torch.zeros(1, device="cuda")  # the primary context, shared with the loader
        self.L = C.CDLL(os.path.join(REF_DIR, "libfzref.so"))
        rc = self.L.ref_load(FATBIN.encode())
        if rc != 0:
            raise RuntimeError(f"ref_load failed: {rc}")
        vp, u32, f32 = C.c_void_p, C.c_uint, C.c_float
        self.L.ref_c_lorenzo.argtypes = [C.c_int, vp, vp, vp, u32, u32, u32, f32, vp]
        self.L.ref_bitshuffle.argtypes = [vp, vp, u32, vp, vp, vp]
        self.L.ref_encode.argtypes = [vp, vp, vp, u32, vp]
        self.S = C.CDLL(os.path.join(REF_DIR, "libfzrefscan.so"))
        self.S.ref_scan_temp_bytes.argtypes = [C.c_int, C.POINTER(C.c_size_t)]
        self.S.ref_scan.argtypes = [vp, C.c_size_t, vp, vp, C.c_int, vp]

    def run(self, x, dims, eb_abs, timed=False):
        """x: CUDA float32 tensor of n elements.  Returns the reference's buffers (CUDA
        tensors) and, with timed=True, each stage's device time in ms (CUDA events on the
        launching stream)."""
        import numpy as np
        import torch
        n = x.numel()
        nx, ny, nz = dims
        nd = 1 if (nz == 1 and ny == 1) else (2 if nz == 1 else 3)
        ebx2_r = float(np.float32(1.0 / (eb_abs * 2)))             # lorenzo_var.cuh:562-563
        stream = torch.cuda.current_stream()
        sh = stream.cuda_stream
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(self.STAGES) + 1)] if timed else None
        mark = (lambda k: ev[k].record(stream)) if timed else (lambda k: None)

        quant = torch.empty(n + 2, dtype=torch.int16, device="cuda")  # (+pad: the u32 view of odd n)
        signum = torch.empty(n, dtype=torch.uint8, device="cuda")
        nl = 2 * n
        nl = nl if nl % 8192 == 0 else nl - nl % 8192 + 8192              # fz.cu:158-159
        dcs1 = nl // 512 if nl % 512 == 0 else nl // 512 + 1              # fz.cu:160-161
        dcs2 = (2 * n + 511) // 512                                       # fz.cu:177-178
        m = 32 * dcs2
        bitflag = torch.empty(dcs1, dtype=torch.int32, device="cuda")
        byteflag = torch.empty(32 * dcs1, dtype=torch.int32, device="cuda")
        d_out = torch.empty(16 * 32 * dcs1, dtype=torch.uint8, device="cuda")
        presum = torch.zeros(m + 1, dtype=torch.int32, device="cuda")
        flags_copy = torch.empty(m, dtype=torch.int32, device="cuda")
        tb = C.c_size_t()
        assert self.S.ref_scan_temp_bytes(m, C.byref(tb)) == 0
        temp = torch.empty(max(1, tb.value), dtype=torch.uint8, device="cuda")
        h3 = torch.empty(3, dtype=torch.int32).pin_memory()

        mark(0)
        quant.zero_()                                                     # fz.cu:145
        mark(1)
        assert self.L.ref_c_lorenzo(nd, x.data_ptr(), quant.data_ptr(), signum.data_ptr(), nx, ny, nz,
                                    ebx2_r, sh) == 0                      # fz.cu:149
        mark(2)
        shuf = quant.clone()                                              # fz.cu:154-155
        mark(3)
        bitflag.zero_(), byteflag.zero_(), d_out.zero_()                   # fz.cu:167-169
        mark(4)
        assert self.L.ref_bitshuffle(quant.data_ptr(), shuf.data_ptr(), n, bitflag.data_ptr(),
                                     byteflag.data_ptr(), sh) == 0        # fz.cu:172-174
        mark(5)
        flags_copy.copy_(byteflag[:m])                                    # fz.cu:183-184
        mark(6)
        assert self.S.ref_scan(temp.data_ptr(), tb.value, flags_copy.data_ptr(), presum.data_ptr(), m, sh) == 0
        mark(7)
        # the total: last prefix + last flag read back, then written to presum[m] (fz.cu:194-201)
        h3[0:1].copy_(presum[m - 1:m], non_blocking=True)
        h3[1:2].copy_(flags_copy[m - 1:m], non_blocking=True)
        stream.synchronize()
        h3[2] = h3[0] + h3[1]
        presum[m:m + 1].copy_(h3[2:3], non_blocking=True)
        mark(8)
        assert self.L.ref_encode(shuf.data_ptr(), d_out.data_ptr(), presum.data_ptr(), n, sh) == 0  # fz.cu:205
        mark(9)
        torch.cuda.synchronize()
        nnz = int(h3[2])
        out = dict(quant=quant[:n], shuffled=shuf[:n], byteflag=flags_copy, bitflag=bitflag[:dcs2],
                   presum=presum, d_out=d_out[: 16 * nnz], nnz=nnz, dcs2=dcs2)
        if timed:
            out["ms"] = {name: ev[k].elapsed_time(ev[k + 1]) for k, name in enumerate(self.STAGES)}
        return out
