// fz_noalloc.cu -- compression for callers that cannot allocate device memory.
//
// fz_compress needs a workspace, and creating one calls cudaMalloc.  Some callers cannot
// do that: host frameworks that own every byte of device memory through their own pool
// and forbid raw cudaMalloc, and latency-critical loops where cudaMalloc's implicit
// synchronisation is unacceptable.  fz_compress_noalloc
// serves them: the little scratch the scan needs lives in a fixed static device array in
// this file, which every GPU that loads the library holds until the process exits.
//
// The array is shared by every call on a device and keeps the previous call's contents:
// each call clears the words that must start from a known value (range accumulators,
// status, ticket counter); the tile states need no clearing because they are tagged
// with the device epoch, which only moves forward.  Calls whose GPU work overlaps (two
// streams, or two host threads) race on the array; serialise them.
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/fz.h"
#include "fz_internal.h"

using namespace fz;

namespace {

// Scan tiles of the largest field: ceil((n/2048 + 1) / 8), plus slack.
constexpr uint32_t kNoallocTiles = (uint32_t)((FZ_NOALLOC_MAX_ELEMS / kBlockCodes + 1) / 8 + 2);
// u64 words: tile states, then 2 words of control: [mm_min, mm_max, status, ticket],
// then 1 word [epoch, CTA exit counter].
constexpr uint32_t kNoallocWords = kNoallocTiles + 3;
static_assert(kNoallocWords * 8 <= FZ_NOALLOC_SCRATCH_BYTES, "scratch size");

// Zero-initialised when the module loads: state epoch 0 with flag 0 reads as "not
// ready", ticket 0, epoch 0.
static __device__ __align__(256) uint64_t g_noalloc_scratch[FZ_NOALLOC_SCRATCH_BYTES / 8];

constexpr int kMaxDevices = 64;
std::mutex    g_lock;
void*         g_addr[kMaxDevices];  // device address of g_noalloc_scratch, per device

// Set-up, once per device, with that device current: the host-side name of the array is
// only a stand-in, so the kernels get the device address from cudaGetSymbolAddress.
fz_status scratch_for_current_device(uint64_t** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FZ_NO_DEVICE;
    if (dev < 0 || dev >= kMaxDevices) return FZ_NO_DEVICE;
    std::lock_guard<std::mutex> g(g_lock);
    if (!g_addr[dev]) {
        void*       p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return e != cudaSuccess ? map_err(e) : FZ_FAIL_GPU_ILLEGAL_ACCESS;
        g_addr[dev] = p;
    }
    *out = static_cast<uint64_t*>(g_addr[dev]);
    return FZ_SUCCESS;
}

}  // namespace

extern "C" fz_status fz_compress_noalloc(const float* d_in, uint64_t n, fz_dims dims, double eb,
                                         fz_eb_mode eb_mode, fz_mode mode, void* d_out,
                                         uint64_t out_capacity, uint64_t* out_bytes, fz_stream_t stream)
{
    // sizes first: nothing is touched for a field beyond the fixed scratch
    if (n == 0 || n > FZ_NOALLOC_MAX_ELEMS) return FZ_INVALID_ARG;
    if (!d_in || !d_out || (reinterpret_cast<uintptr_t>(d_in) & 15u) || (reinterpret_cast<uintptr_t>(d_out) & 15u))
        return FZ_INVALID_ARG;
    if (!dims_fit(n, dims.x, dims.y, dims.z)) return FZ_INVALID_ARG;
    if (!(eb > 0) || !std::isfinite(eb)) return FZ_INVALID_ARG;
    if ((eb_mode != FZ_EB_ABS && eb_mode != FZ_EB_REL) || (mode != FZ_MODE_COMPAT && mode != FZ_MODE_SIDECAR))
        return FZ_INVALID_ARG;
    const Layout L = make_layout(n, dims.x, dims.y, dims.z, mode);
    if (out_capacity < L.off_b + 16ull * kChunks * L.nb) return FZ_OUT_OF_SPACE;

    uint64_t* scratch = nullptr;
    fz_status st      = scratch_for_current_device(&scratch);
    if (st != FZ_SUCCESS) return st;
    uint32_t* ctl   = reinterpret_cast<uint32_t*>(scratch + kNoallocTiles);  // mm_min, mm_max, status, ticket
    uint32_t* epoch = reinterpret_cast<uint32_t*>(scratch + kNoallocTiles + 2);
    uint32_t* fin   = epoch + 1;

    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // the previous call's contents: reset the range to "empty", the status, ticket and exit
    // counter to 0 (the epoch only moves forward and is kept)
    cudaError_t e = cudaMemsetAsync(ctl, 0xFF, 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctl + 1, 0, 12, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(fin, 0, 4, s);
    if (e != cudaSuccess) return map_err(e);

    CompressArgs a{};
    a.in = d_in, a.out = static_cast<uint8_t*>(d_out);
    a.n = L.n, a.nl = L.nl, a.x = L.x, a.y = L.y, a.z = L.z, a.xy = L.xy;
    a.dx = make_fastdiv(L.x), a.dxy = make_fastdiv(L.xy);
    a.al_x = (L.x % 4) == 0, a.al_xy = (L.xy % 4) == 0, a.al_xyx = ((L.xy + L.x) % 4) == 0;
    a.nb = L.nb, a.ntiles = L.nb + (L.tail ? 1 : 0), a.nwords = L.nwords;
    a.mode = mode, a.ndim = L.ndim, a.sidecar_bytes = L.sidecar_bytes;
    a.off_a = L.off_a, a.off_c = L.off_c, a.off_b = L.off_b, a.off_sign = L.off_sign, a.off_boff = L.off_boff;
    a.state = scratch, a.ticket = ctl + 3, a.status = ctl + 2, a.epoch = epoch;
    a.boff  = mode == FZ_MODE_SIDECAR ? reinterpret_cast<uint32_t*>(a.out + L.off_boff) : nullptr;
    a.fin   = fin;
    if (eb_mode == FZ_EB_REL) {
        e        = launch_range(d_in, L.n, ctl, ctl + 2, nullptr, s);
        a.mm     = ctl;
        a.eb_rel = eb;
    } else {
        a.mm            = nullptr;
        a.ebh.eb_abs    = eb;
        const double e2 = eb * 2;
        a.ebh.ebx2_r    = (float)(1 / e2);
        a.ebh.ebx2      = (float)e2;
        a.ebh.range = a.ebh.vmin = a.ebh.vmax = 0.0f;
    }
    if (e == cudaSuccess) e = launch_compress(a, s);
    if (e != cudaSuccess) return map_err(e);
    // Without the readback the call returns at once; a failure found on the device
    // (non-finite input with a relative bound, a wait that gave up) is then carried by the
    // stream itself: its header gets FZ_FLAG_FAILED, which every reader rejects.
    if (!out_bytes) return FZ_SUCCESS;
    // optional size readback into pageable host memory (synchronous)
    fz_header h;
    uint32_t  status = 0;
    e = cudaMemcpyAsync(&h, d_out, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, ctl + 2, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MEMCPY);
    *out_bytes = L.off_b + 16ull * h.nnz;
    if (status & kStatusTimeout) return FZ_TIMEOUT;
    if (status & kStatusNonfinite) return FZ_NONFINITE_INPUT;
    return FZ_SUCCESS;
}
