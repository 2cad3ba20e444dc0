// fz_api.cu -- the C ABI (include/fz.h): argument checks, stream layout, workspace,
// and the launch sequences of the full pipeline and of the stage-level drop-ins.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/fz.h"
#include "fz_internal.h"
#include "fz_workspace.h"

using namespace fz;

namespace fz {

Layout make_layout(uint64_t n, uint32_t x, uint32_t y, uint32_t z, uint32_t mode)
{
    Layout L{};
    L.n      = (uint32_t)n;
    L.x      = x, L.y = y, L.z = z;
    L.xy     = x * y;
    L.nl     = x * y * z;
    L.ndim   = (z == 1 && y == 1) ? 1 : (z == 1 ? 2 : 3);
    L.nb     = (uint32_t)(n / kBlockCodes);
    L.tail   = (uint32_t)(n - (uint64_t)L.nb * kBlockCodes);
    L.nwords = (uint32_t)cdiv(n, 256);
    L.mode   = mode;
    L.off_a  = kHeaderBytes;
    L.off_c  = L.off_a + pad16(4ull * L.nwords);
    uint64_t sc = 0;
    if (mode == FZ_MODE_SIDECAR) {
        // Section C: raw tail codes | 1D sign bits | chunk offset of every shuffle block
        sc += pad16(2ull * L.tail);
        L.off_sign = L.off_c + sc;
        if (L.ndim == 1) sc += pad16(4 * cdiv(n, 32));
        L.off_boff = L.off_c + sc;
        sc += pad16(4ull * (L.nb + 1));
    } else {
        L.off_sign = L.off_boff = L.off_c;
    }
    L.sidecar_bytes = (uint32_t)sc;
    L.off_b         = L.off_c + sc;
    return L;
}

}  // namespace fz

namespace {
constexpr uint64_t kMaxN = 1ull << 31;
}  // namespace

namespace fz {

fz_status map_err(cudaError_t e, fz_status dflt)
{
    if (e == cudaSuccess) return FZ_SUCCESS;
    if (e == cudaErrorMemoryAllocation) return FZ_FAIL_GPU_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FZ_NO_DEVICE;
    return dflt;
}

bool dims_fit(uint64_t n, uint32_t x, uint32_t y, uint32_t z)
{
    if (n == 0 || n > kMaxN || x == 0 || y == 0 || z == 0) return false;
    const uint64_t xy = (uint64_t)x * y;  // < 2^64: both factors < 2^32
    if (xy > n) return false;
    return (uint64_t)z <= n / xy;         // xy * z <= n, without forming the product
}

}  // namespace fz

namespace {

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int ndim_of(fz_dims d) { return (d.z == 1 && d.y == 1) ? 1 : (d.z == 1 ? 2 : 3); }

fz_status check_dims(uint64_t n, fz_dims d) { return dims_fit(n, d.x, d.y, d.z) ? FZ_SUCCESS : FZ_INVALID_ARG; }

uint64_t max_stream(const Layout& L) { return L.off_b + 16ull * kChunks * L.nb; }

// Brackets one kernel launch with a pair of events when timing is enabled.
struct KernelTimer {
    fz_workspace* ws;
    cudaStream_t  s;
    int           kind;
    bool          on;
    KernelTimer(fz_workspace* w, cudaStream_t st, int k) : ws(w), s(st), kind(k)
    {
        on = ws->tcap && ws->tused < ws->tcap;
        if (on) cudaEventRecord(ws->tev[2 * ws->tused], s);
    }
    ~KernelTimer()
    {
        if (!on) return;
        cudaEventRecord(ws->tev[2 * ws->tused + 1], s);
        ws->tkind[ws->tused++] = kind;
    }
};

fz_status check_device(const fz_workspace* ws)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return FZ_NO_DEVICE;
    return dev == ws->device ? FZ_SUCCESS : FZ_INVALID_ARG;
}

// Reads back the header and the sticky status word (syncs), clears the status.
fz_status readback(fz_workspace* ws, const void* d_stream, cudaStream_t s, fz_header* h)
{
    cudaError_t e = cudaMemcpyAsync(ws->h_pinned, d_stream, 64, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ws->h_pinned + 64, ws->status, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MEMCPY);
    std::memcpy(h, ws->h_pinned, 64);
    uint32_t st;
    std::memcpy(&st, ws->h_pinned + 64, 4);
    if (st) cudaMemsetAsync(ws->status, 0, 4, s);
    if (st & kStatusTimeout) return FZ_TIMEOUT;
    if (st & kStatusNonfinite) return FZ_NONFINITE_INPUT;
    if (st & kStatusCorrupt) return FZ_CORRUPT_STREAM;
    return FZ_SUCCESS;
}

fz_status validate_header(const fz_header* h, uint64_t stream_bytes, Layout* out)
{
    if (h->magic != FZ_MAGIC || h->version != FZ_FORMAT_VERSION) return FZ_CORRUPT_STREAM;
    if (h->mode > 1 || (h->flags & FZ_FLAG_FAILED)) return FZ_CORRUPT_STREAM;
    fz_dims d{h->x, h->y, h->z};
    if (check_dims(h->n, d) != FZ_SUCCESS || ndim_of(d) != h->ndim) return FZ_CORRUPT_STREAM;
    Layout L = make_layout(h->n, h->x, h->y, h->z, h->mode);
    if (L.sidecar_bytes != h->sidecar_bytes) return FZ_CORRUPT_STREAM;
    if (h->nnz > (uint64_t)L.nb * kChunks) return FZ_CORRUPT_STREAM;
    if (L.off_b + 16ull * h->nnz > stream_bytes) return FZ_CORRUPT_STREAM;
    *out = L;
    return FZ_SUCCESS;
}

}  // namespace

extern "C" {

const char* fz_status_string(fz_status s)
{
    switch (s) {
    case FZ_SUCCESS: return "success";
    case FZ_FAIL_ONDISK_FILE_ERROR: return "file error";
    case FZ_FAIL_DATA_NOT_READY: return "data not ready";
    case FZ_FAIL_GPU_MALLOC: return "device allocation failed";
    case FZ_FAIL_GPU_MEMCPY: return "device copy failed";
    case FZ_FAIL_GPU_ILLEGAL_ACCESS: return "device launch or execution failed";
    case FZ_FAIL_GPU_OUT_OF_MEMORY: return "device out of memory";
    case FZ_FAIL_INCOMPRESSIABLE: return "incompressible";
    case FZ_FAIL_UNSUPPORTED_DATATYPE: return "unsupported data type";
    case FZ_NOT_IMPLEMENTED: return "not implemented";
    case FZ_INVALID_ARG: return "invalid argument";
    case FZ_CORRUPT_STREAM: return "corrupt stream";
    case FZ_OUT_OF_SPACE: return "output buffer too small";
    case FZ_TIMEOUT: return "device-side wait timed out";
    case FZ_NO_DEVICE: return "no CUDA device";
    case FZ_NONFINITE_INPUT: return "non-finite input with a relative error bound";
    }
    return "unknown status";
}

const char* fz_version(void) { return "fz-gb300 1.0 (sm_103a)"; }

int fz_ndim(fz_dims dims) { return ndim_of(dims); }

fz_status fz_stream_layout(uint64_t n, fz_dims dims, fz_mode mode, uint64_t* off_a,
                           uint64_t* off_c, uint64_t* off_b, uint32_t* sidecar_bytes)
{
    if (check_dims(n, dims) != FZ_SUCCESS || (mode != FZ_MODE_COMPAT && mode != FZ_MODE_SIDECAR))
        return FZ_INVALID_ARG;
    Layout L = make_layout(n, dims.x, dims.y, dims.z, mode);
    if (off_a) *off_a = L.off_a;
    if (off_c) *off_c = L.off_c;
    if (off_b) *off_b = L.off_b;
    if (sidecar_bytes) *sidecar_bytes = L.sidecar_bytes;
    return FZ_SUCCESS;
}

fz_status fz_max_compressed_bytes(uint64_t n, fz_dims dims, fz_mode mode, uint64_t* bytes)
{
    if (!bytes || check_dims(n, dims) != FZ_SUCCESS || (mode != FZ_MODE_COMPAT && mode != FZ_MODE_SIDECAR))
        return FZ_INVALID_ARG;
    *bytes = max_stream(make_layout(n, dims.x, dims.y, dims.z, mode));
    return FZ_SUCCESS;
}

fz_status fz_stream_bytes(const fz_header* h, uint64_t* bytes)
{
    if (!h || !bytes) return FZ_INVALID_ARG;
    Layout    L;
    fz_status st = validate_header(h, ~0ull, &L);
    if (st != FZ_SUCCESS) return st;
    *bytes = L.off_b + 16ull * h->nnz;
    return FZ_SUCCESS;
}

fz_status fz_reference_sizes(uint64_t file_bytes, uint64_t nnz, uint64_t* original,
                             uint64_t* compressed, double* ratio)
{
    // fz.cu:118 len = fileSize/4; :178 dataChunkSize = ceil(2 len / 512); :208-209
    const uint64_t len = file_bytes / 4;
    const uint64_t dcs = cdiv(2 * len, 512);
    const uint64_t c   = 4 * dcs + 16 * nnz;
    if (original) *original = file_bytes;
    if (compressed) *compressed = c;
    if (ratio) *ratio = c ? (double)((float)file_bytes / (float)c) : 0.0;
    return FZ_SUCCESS;
}

fz_status fz_workspace_bytes(uint64_t max_n, uint64_t* bytes)
{
    if (!bytes || max_n == 0 || max_n > kMaxN) return FZ_INVALID_ARG;
    const uint64_t tiles = max_n / kBlockCodes + 2;
    uint64_t       b     = 0;
    b += pad16(8 * tiles);          // state
    b += 128;                       // tickets, status, total, field control words
    b += 16;                        // range accumulators
    b += pad16(2 * max_n + 16);     // per-block slots (k_encode_fields)
    b += pad16(4 * tiles + 4);      // block offsets
    b += pad16(4 * 2 * (uint64_t)group_sum_words((uint32_t)tiles));  // two sets of group sums
    *bytes = b;
    return FZ_SUCCESS;
}

fz_status fz_workspace_create(uint64_t max_n, fz_workspace** out)
{
    if (!out) return FZ_INVALID_ARG;
    *out = nullptr;
    uint64_t bytes;
    if (fz_workspace_bytes(max_n, &bytes) != FZ_SUCCESS) return FZ_INVALID_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FZ_NO_DEVICE;
    fz_workspace* ws = new (std::nothrow) fz_workspace();
    if (!ws) return FZ_FAIL_GPU_MALLOC;
    ws->device    = dev;
    ws->max_n     = max_n;
    ws->max_tiles = (uint32_t)(max_n / kBlockCodes + 2);
    cudaError_t e = cudaMalloc(&ws->d_base, bytes);
    if (e != cudaSuccess) {
        delete ws;
        return map_err(e, FZ_FAIL_GPU_MALLOC);
    }
    ws->d_bytes = bytes;
    uint8_t* p  = static_cast<uint8_t*>(ws->d_base);
    ws->state   = reinterpret_cast<uint64_t*>(p), p += pad16(8ull * ws->max_tiles);
    ws->tickets = reinterpret_cast<uint32_t*>(p);
    ws->status  = ws->tickets + 4;
    ws->total   = ws->tickets + 5;
    ws->epoch   = ws->tickets + 6;
    ws->fctl    = reinterpret_cast<FieldCtl*>(ws->tickets + 16);
    p += 128;
    ws->mm       = reinterpret_cast<uint32_t*>(p), p += 16;
    ws->codes    = reinterpret_cast<uint16_t*>(p), p += pad16(2 * max_n + 16);
    ws->boff     = reinterpret_cast<uint32_t*>(p), p += pad16(4ull * ws->max_tiles + 4);
    ws->supers   = reinterpret_cast<uint32_t*>(p);
    e            = cudaMemset(ws->d_base, 0, bytes);
    if (e == cudaSuccess) {
        const uint32_t init[2] = {0xFFFFFFFFu, 0u};  // empty min/max
        e                      = cudaMemcpy(ws->mm, init, sizeof(init), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(ws->fctl->mm, init, sizeof(init), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(ws->fctl->pre, init, sizeof(init), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMallocHost((void**)&ws->h_pinned, 128);
    if (e != cudaSuccess) {
        cudaFree(ws->d_base);
        delete ws;
        return map_err(e, FZ_FAIL_GPU_MALLOC);
    }
    *out = ws;
    return FZ_SUCCESS;
}

fz_status fz_workspace_enable_timing(fz_workspace* ws, uint32_t capacity)
{
    if (!ws) return FZ_INVALID_ARG;
    for (cudaEvent_t e : ws->tev) cudaEventDestroy(e);
    ws->tev.assign(2 * (size_t)capacity, nullptr);
    ws->tkind.assign(capacity, -1);
    ws->tused = 0;
    ws->tcap  = 0;
    for (auto& e : ws->tev) {
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return map_err(r);
    }
    ws->tcap = capacity;
    return FZ_SUCCESS;
}

fz_status fz_workspace_kernel_time(fz_workspace* ws, int kind, uint32_t* launches, double* total_ms)
{
    if (!ws || !launches || !total_ms) return FZ_INVALID_ARG;
    *launches = 0;
    *total_ms = 0;
    if (ws->tused) {
        cudaError_t r = cudaEventSynchronize(ws->tev[2 * ws->tused - 1]);
        if (r != cudaSuccess) return map_err(r);
    }
    uint32_t keep = 0;
    for (uint32_t i = 0; i < ws->tused; ++i) {
        if (ws->tkind[i] == kind) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ws->tev[2 * i], ws->tev[2 * i + 1]);
            *total_ms += ms;
            ++*launches;
        } else {
            // keep the other kinds' records, compacted to the front
            std::swap(ws->tev[2 * keep], ws->tev[2 * i]);
            std::swap(ws->tev[2 * keep + 1], ws->tev[2 * i + 1]);
            ws->tkind[keep++] = ws->tkind[i];
        }
    }
    ws->tused = keep;
    return FZ_SUCCESS;
}

fz_status fz_workspace_destroy(fz_workspace* ws)
{
    if (!ws) return FZ_INVALID_ARG;
    for (cudaEvent_t e : ws->tev) cudaEventDestroy(e);
    cudaFree(ws->d_base);
    cudaFreeHost(ws->h_pinned);
    cudaFree(ws->d_field);
    cudaFree(ws->d_stream);
    delete ws;
    return FZ_SUCCESS;
}

fz_status fz_workspace_status(fz_workspace* ws, fz_stream_t stream)
{
    if (!ws) return FZ_INVALID_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t  e = cudaMemcpyAsync(ws->h_pinned + 64, ws->status, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MEMCPY);
    uint32_t st;
    std::memcpy(&st, ws->h_pinned + 64, 4);
    if (st) cudaMemsetAsync(ws->status, 0, 4, s);
    if (st & kStatusTimeout) return FZ_TIMEOUT;
    if (st & kStatusNonfinite) return FZ_NONFINITE_INPUT;
    if (st & kStatusCorrupt) return FZ_CORRUPT_STREAM;
    return FZ_SUCCESS;
}

fz_status fz_compress(fz_workspace* ws, const float* d_in, uint64_t n, fz_dims dims, double eb,
                      fz_eb_mode eb_mode, fz_mode mode, void* d_out, uint64_t out_capacity,
                      uint64_t* out_bytes, fz_stream_t stream)
{
    return fz::compress_impl(ws, d_in, n, dims, eb, eb_mode, mode, d_out, out_capacity, out_bytes, stream, nullptr);
}

}  // extern "C"

// Checks the arguments of one field's compression and fills its layout and kernel
// arguments (without the scan state and mirror, which depend on the caller).
static fz_status compress_args(const float* d_in, uint64_t n, fz_dims dims, double eb, fz_eb_mode eb_mode,
                               fz_mode mode, void* d_out, uint64_t out_capacity, uint32_t* status, Layout& L,
                               CompressArgs& a)
{
    if (!d_in || !d_out || !aligned16(d_in) || !aligned16(d_out)) return FZ_INVALID_ARG;
    if (check_dims(n, dims) != FZ_SUCCESS) return FZ_INVALID_ARG;
    if (!(eb > 0) || !std::isfinite(eb)) return FZ_INVALID_ARG;
    if ((eb_mode != FZ_EB_ABS && eb_mode != FZ_EB_REL) || (mode != FZ_MODE_COMPAT && mode != FZ_MODE_SIDECAR))
        return FZ_INVALID_ARG;
    L = make_layout(n, dims.x, dims.y, dims.z, mode);
    if (out_capacity < max_stream(L)) return FZ_OUT_OF_SPACE;
    a    = CompressArgs{};
    a.in = d_in, a.out = static_cast<uint8_t*>(d_out);
    a.n = L.n, a.nl = L.nl, a.x = L.x, a.y = L.y, a.z = L.z, a.xy = L.xy;
    a.dx = make_fastdiv(L.x), a.dxy = make_fastdiv(L.xy);
    a.al_x = (L.x % 4) == 0, a.al_xy = (L.xy % 4) == 0, a.al_xyx = ((L.xy + L.x) % 4) == 0;
    a.nb = L.nb, a.ntiles = L.nb + (L.tail ? 1 : 0), a.nwords = L.nwords;
    a.mode = mode, a.ndim = L.ndim, a.sidecar_bytes = L.sidecar_bytes;
    a.off_a = L.off_a, a.off_c = L.off_c, a.off_b = L.off_b, a.off_sign = L.off_sign, a.off_boff = L.off_boff;
    a.status = status;
    a.boff   = mode == FZ_MODE_SIDECAR ? reinterpret_cast<uint32_t*>(a.out + L.off_boff) : nullptr;
    a.mm     = nullptr;
    if (eb_mode == FZ_EB_REL) {
        a.eb_rel = eb;
    } else {
        a.ebh.eb_abs    = eb;
        const double e2 = eb * 2;  // lorenzo_var.cuh:562-563
        a.ebh.ebx2_r    = (float)(1 / e2);
        a.ebh.ebx2      = (float)e2;
        a.ebh.range = a.ebh.vmin = a.ebh.vmax = 0.0f;
    }
    return FZ_SUCCESS;
}

// fz_compress with an optional device mirror of the header and status word (128 bytes,
// written by the last kernel; the request loop reads both with one copy).
fz_status fz::compress_impl(fz_workspace* ws, const float* d_in, uint64_t n, fz_dims dims, double eb,
                            fz_eb_mode eb_mode, fz_mode mode, void* d_out, uint64_t out_capacity,
                            uint64_t* out_bytes, fz_stream_t stream, uint32_t* mirror, RangeAhead* ra)
{
    if (ra) ra->done = false;
    if (!ws) return FZ_INVALID_ARG;
    if (n > ws->max_n) return FZ_INVALID_ARG;
    fz_status st = check_device(ws);
    if (st != FZ_SUCCESS) return st;
    Layout       L;
    CompressArgs a;
    st = compress_args(d_in, n, dims, eb, eb_mode, mode, d_out, out_capacity, ws->status, L, a);
    if (st != FZ_SUCCESS) return st;
    a.state = ws->state, a.ticket = ws->tickets + 0, a.epoch = ws->epoch;
    a.mirror = mirror;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // the field as a list of one: range launch (relative eb), encode launch (per-block
    // slots in the workspace scratch, one 4 KiB slot per shuffle block; chunk counts in the
    // block-offset array), compaction launch
    FieldJob J{};
    J.a      = a;
    J.ctl    = ws->fctl;
    J.slots  = reinterpret_cast<uint4*>(ws->codes);
    J.counts = ws->boff;
    J.supers = ws->supers;
    J.sstride = group_sum_words(ws->max_tiles);
    J.s2off   = group_sum_l2(ws->max_tiles);
    J.rel    = eb_mode == FZ_EB_REL;
    field_items(L.n, L.nb, a.ntiles, J.rel != 0, J.nr, J.ne, J.nc);
    if (ra && ra->have && J.rel) J.nr = 0;  // the previous call's encode launch took the range
    // range ahead: only when a compaction launch follows the encode launch (it moves the
    // accumulated range into place once every encode CTA has finished)
    if (ra && ra->next && J.rel && J.nc) {
        const fz_field& f = *ra->next;
        Layout          Ln;
        CompressArgs    an;
        if (f.n <= ws->max_n && compress_args(static_cast<const float*>(f.src), f.n, f.dims, f.eb, eb_mode, mode, f.dst,
                                              f.dst_capacity, ws->status, Ln, an) == FZ_SUCCESS) {
            uint32_t ne, nc;
            field_items(Ln.n, Ln.nb, an.ntiles, true, J.ahead_nr, ne, nc);
            J.ahead_in = an.in, J.ahead_n = an.n;
        }
    }
    cudaError_t e = cudaSuccess;
    if (J.nr) {
        KernelTimer t(ws, s, 0);
        e = launch_fields(FieldPhase::Range, (int)L.ndim, nullptr, nullptr, 0, J.nr, J, s);
    }
    if (e == cudaSuccess) {
        KernelTimer t(ws, s, 1);
        e = launch_fields(FieldPhase::Encode, (int)L.ndim, nullptr, nullptr, 0, J.ne, J, s, J.ahead_nr);
    }
    if (e == cudaSuccess) {
        KernelTimer t(ws, s, 5);
        e = launch_fields(FieldPhase::Compact, (int)L.ndim, nullptr, nullptr, 0, J.nc, J, s);
    }
    if (e != cudaSuccess) return map_err(e);
    if (ra) ra->done = J.ahead_nr != 0;
    if (out_bytes) {
        fz_header h;
        st = readback(ws, d_out, s, &h);
        *out_bytes = L.off_b + 16ull * h.nnz;
        return st;
    }
    return FZ_SUCCESS;
}

extern "C" {

fz_status fz_decompress(fz_workspace* ws, const void* d_stream, uint64_t stream_bytes,
                        const fz_header* h_header, float* d_out, uint64_t out_capacity_elems,
                        fz_stream_t stream)
{
    if (!ws || !d_stream || !d_out || !aligned16(d_stream) || !aligned16(d_out)) return FZ_INVALID_ARG;
    if (stream_bytes < FZ_HEADER_BYTES) return FZ_CORRUPT_STREAM;
    fz_status st = check_device(ws);
    if (st != FZ_SUCCESS) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    fz_header    h;
    if (h_header) {
        h = *h_header;
    } else {
        cudaError_t e = cudaMemcpyAsync(ws->h_pinned, d_stream, 64, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MEMCPY);
        std::memcpy(&h, ws->h_pinned, 64);
    }
    Layout L;
    st = validate_header(&h, stream_bytes, &L);
    if (st != FZ_SUCCESS) return st;
    if (h.n > out_capacity_elems || h.n > ws->max_n) return FZ_OUT_OF_SPACE;

    DecodeArgs d{};
    d.st    = static_cast<const uint8_t*>(d_stream);
    d.boff  = ws->boff;
    d.out   = d_out;
    d.n = L.n, d.nl = L.nl, d.x = L.x, d.y = L.y, d.z = L.z;
    d.nb = L.nb, d.tail = L.tail, d.mode = L.mode, d.nwords = L.nwords;
    d.off_a = L.off_a, d.off_c = L.off_c, d.off_b = L.off_b, d.off_sign = L.off_sign, d.nnz = h.nnz;
    d.off_boff = L.off_boff;
    d.ebx2     = h.ebx2;
    d.status   = ws->status;
    cudaError_t e = cudaSuccess;
    if (L.mode == FZ_MODE_SIDECAR) {
        d.boff = reinterpret_cast<const uint32_t*>(d.st + L.off_boff);  // written by the compressor
    } else {
        KernelTimer t(ws, s, 2);
        e = launch_offsets(d.st, L.off_a, L.nb, L.nwords, h.nnz, ws->boff, ws->state, ws->tickets + 1,
                           ws->status, ws->epoch, s);
    }
    if (e != cudaSuccess) return map_err(e);
    {
        KernelTimer t(ws, s, 3);
        e = launch_decompress_fused(d, s);
    }
    if (e == cudaSuccess && L.n > L.nl) e = launch_zero_tail(d_out, L.nl, L.n, s);
    return map_err(e);
}

static fz_status ensure_staging(fz_workspace* ws, uint64_t n, uint64_t stream_bytes)
{
    if (!ws->d_field) {
        cudaError_t e = cudaMalloc((void**)&ws->d_field, 4 * ws->max_n + 16);
        if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MALLOC);
    }
    if (ws->stream_cap < stream_bytes) {
        cudaFree(ws->d_stream);
        ws->d_stream   = nullptr;
        ws->stream_cap = 0;
        // room for the largest stream of a max_n field (1D sidecar is the largest)
        uint64_t cap = 0;
        fz_dims  d1{(uint32_t)ws->max_n, 1, 1};
        fz_max_compressed_bytes(ws->max_n, d1, FZ_MODE_SIDECAR, &cap);
        if (cap < stream_bytes) cap = stream_bytes;
        cudaError_t e = cudaMalloc((void**)&ws->d_stream, cap);
        if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MALLOC);
        ws->stream_cap = cap;
    }
    (void)n;
    return FZ_SUCCESS;
}

fz_status fz_compress_host(fz_workspace* ws, const float* h_in, uint64_t n, fz_dims dims,
                           double eb, fz_eb_mode eb_mode, fz_mode mode, void* h_out,
                           uint64_t out_capacity, uint64_t* out_bytes, fz_stream_t stream)
{
    if (!ws || !h_in || !h_out) return FZ_INVALID_ARG;
    if (check_dims(n, dims) != FZ_SUCCESS || n > ws->max_n) return FZ_INVALID_ARG;
    if (mode != FZ_MODE_COMPAT && mode != FZ_MODE_SIDECAR) return FZ_INVALID_ARG;
    const Layout L = make_layout(n, dims.x, dims.y, dims.z, mode);
    fz_status    st = ensure_staging(ws, n, max_stream(L));
    if (st != FZ_SUCCESS) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t  e = cudaMemcpyAsync(ws->d_field, h_in, 4 * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MEMCPY);
    uint64_t bytes = 0;
    st = fz_compress(ws, ws->d_field, n, dims, eb, eb_mode, mode, ws->d_stream, ws->stream_cap, &bytes, stream);
    if (st != FZ_SUCCESS) return st;
    if (bytes > out_capacity) return FZ_OUT_OF_SPACE;
    e = cudaMemcpyAsync(h_out, ws->d_stream, bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MEMCPY);
    if (out_bytes) *out_bytes = bytes;
    return FZ_SUCCESS;
}

fz_status fz_decompress_host(fz_workspace* ws, const void* h_stream, uint64_t stream_bytes,
                             float* h_out, uint64_t out_capacity_elems, fz_stream_t stream)
{
    if (!ws || !h_stream || !h_out || stream_bytes < FZ_HEADER_BYTES) return FZ_INVALID_ARG;
    fz_header h;
    std::memcpy(&h, h_stream, sizeof(h));
    Layout    L;
    fz_status st = validate_header(&h, stream_bytes, &L);
    if (st != FZ_SUCCESS) return st;
    if (h.n > out_capacity_elems || h.n > ws->max_n) return FZ_OUT_OF_SPACE;
    st = ensure_staging(ws, h.n, stream_bytes);
    if (st != FZ_SUCCESS) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t  e = cudaMemcpyAsync(ws->d_stream, h_stream, stream_bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MEMCPY);
    st = fz_decompress(ws, ws->d_stream, stream_bytes, &h, ws->d_field, ws->max_n, stream);
    if (st != FZ_SUCCESS) return st;
    e = cudaMemcpyAsync(h_out, ws->d_field, 4 * h.n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MEMCPY);
    return fz_workspace_status(ws, stream);
}

fz_status fz_selftest_wait_timeout(fz_workspace* ws, fz_stream_t stream)
{
    if (!ws) return FZ_INVALID_ARG;
    fz_status st = check_device(ws);
    if (st != FZ_SUCCESS) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // the device epoch is one no launch has used yet: tile 0 never reads as ready
    cudaError_t r = launch_wait_selftest(ws->state, ws->epoch, ws->status, s);
    if (r != cudaSuccess) return map_err(r);
    return fz_workspace_status(ws, stream);
}

// ------------------------------------------------------------------ stages --
fz_status fz_lorenzo_construct(const float* d_data, uint16_t* d_quant, uint8_t* d_signum,
                               fz_dims len3, double eb_abs, fz_stream_t stream)
{
    if (!d_data || !d_quant || !aligned16(d_data) || !aligned16(d_quant)) return FZ_INVALID_ARG;
    const uint64_t nl = (uint64_t)len3.x * len3.y * len3.z;
    if (check_dims(nl, len3) != FZ_SUCCESS || !(eb_abs > 0) || !std::isfinite(eb_abs)) return FZ_INVALID_ARG;
    const double e2 = eb_abs * 2;
    cudaError_t  e  = launch_lorenzo_construct(d_data, d_quant, d_signum, len3.x, len3.y, len3.z,
                                               (float)(1 / e2), reinterpret_cast<cudaStream_t>(stream));
    return map_err(e);
}

fz_status fz_lorenzo_reconstruct(const uint16_t* d_quant, const uint8_t* d_signum, float* d_xdata,
                                 fz_dims len3, double eb_abs, fz_stream_t stream)
{
    if (!d_quant || !d_xdata || !aligned16(d_quant) || !aligned16(d_xdata)) return FZ_INVALID_ARG;
    const uint64_t nl = (uint64_t)len3.x * len3.y * len3.z;
    if (check_dims(nl, len3) != FZ_SUCCESS || !(eb_abs > 0) || !std::isfinite(eb_abs)) return FZ_INVALID_ARG;
    ReconArgs r{};
    r.codes = d_quant, r.signbits = nullptr, r.signum = d_signum, r.out = d_xdata;
    r.n = (uint32_t)nl, r.nl = (uint32_t)nl, r.x = len3.x, r.y = len3.y, r.z = len3.z;
    r.ebx2 = (float)(eb_abs * 2);
    return map_err(launch_reconstruct(r, reinterpret_cast<cudaStream_t>(stream)));
}

fz_status fz_bitshuffle_flag(const uint32_t* d_in, uint32_t* d_out, uint64_t n_codes,
                             uint32_t* d_bitflag, uint32_t* d_byteflag, fz_stream_t stream)
{
    if (!d_in || !d_out || !d_bitflag || !d_byteflag || n_codes == 0 || n_codes > kMaxN) return FZ_INVALID_ARG;
    if (!aligned16(d_in) || !aligned16(d_out)) return FZ_INVALID_ARG;
    return map_err(launch_bitshuffle_flag(d_in, d_out, (uint32_t)n_codes, d_bitflag, d_byteflag,
                                          reinterpret_cast<cudaStream_t>(stream)));
}

fz_status fz_scan_encode(fz_workspace* ws, const uint8_t* d_shuffled, const uint32_t* d_byteflag,
                         uint64_t n_codes, uint32_t* d_presum, uint8_t* d_out, uint64_t* nnz,
                         fz_stream_t stream)
{
    if (!ws || !d_shuffled || !d_byteflag || n_codes == 0 || n_codes > ws->max_n) return FZ_INVALID_ARG;
    if (!aligned16(d_shuffled) || (d_out && !aligned16(d_out))) return FZ_INVALID_ARG;
    fz_status st = check_device(ws);
    if (st != FZ_SUCCESS) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t  e = launch_scan_encode(d_shuffled, d_byteflag, (uint32_t)n_codes, d_presum, d_out,
                                        ws->state, ws->tickets + 2, ws->status, ws->total,
                                        ws->epoch, s);
    if (e != cudaSuccess) return map_err(e);
    if (nnz) {
        e = cudaMemcpyAsync(ws->h_pinned, ws->total, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MEMCPY);
        uint32_t t;
        std::memcpy(&t, ws->h_pinned, 4);
        *nnz = t;
        return fz_workspace_status(ws, stream);
    }
    return FZ_SUCCESS;
}

// ----------------------------------------------------------------- batching --
fz_status fz_compress_batch(fz_workspace* ws, const fz_field* fields, uint32_t count, fz_eb_mode eb_mode,
                            fz_mode mode, fz_stream_t stream)
{
    if (!ws || (!fields && count)) return FZ_INVALID_ARG;
    fz::RangeAhead ra;  // each field's encode launch takes the next field's range
    for (uint32_t i = 0; i < count; ++i) {
        const fz_field& f = fields[i];
        ra.next           = i + 1 < count ? fields + i + 1 : nullptr;
        fz_status st = fz::compress_impl(ws, static_cast<const float*>(f.src), f.n, f.dims, f.eb, eb_mode, mode, f.dst,
                                         f.dst_capacity, nullptr, stream, nullptr, &ra);
        if (st != FZ_SUCCESS) return st;
        ra.have = ra.done;
    }
    return FZ_SUCCESS;
}

fz_status fz_decompress_batch(fz_workspace* ws, const fz_field* fields, uint32_t count, fz_stream_t stream)
{
    if (!ws || (!fields && count)) return FZ_INVALID_ARG;
    for (uint32_t i = 0; i < count; ++i) {
        const fz_field& f = fields[i];
        fz_status st = fz_decompress(ws, f.src, f.src_bytes, &f.header, static_cast<float*>(f.dst),
                                     f.dst_capacity, stream);
        if (st != FZ_SUCCESS) return st;
    }
    return FZ_SUCCESS;
}

}  // extern "C"

namespace {

// Device work list of a batch compression, in one allocation: every field's job and
// control words, its slots (4 KiB per shuffle block), block counts and group
// sums, and the segment tables of the range launch, of the encode launch of each
// dimensionality and of the compaction launch.
struct ListPlan {
    void*    d_mem = nullptr;
    Segment* seg[5]   = {};  // [0] range, [1..3] encode 1D..3D, [4] compaction
    uint32_t nseg[5]  = {};
    uint32_t total[5] = {};
    FieldJob* jobs    = nullptr;
};

fz_status plan_list_compress(fz_workspace* ws, const fz_field* f, uint32_t count, fz_eb_mode eb_mode, fz_mode mode,
                             ListPlan& P)
{
    std::vector<FieldJob> jobs(count);
    std::vector<Layout>   lay(count);
    for (uint32_t i = 0; i < count; ++i) {
        const fz_status st = compress_args(static_cast<const float*>(f[i].src), f[i].n, f[i].dims, f[i].eb, eb_mode,
                                           mode, f[i].dst, f[i].dst_capacity, ws->status, lay[i], jobs[i].a);
        if (st != FZ_SUCCESS) return st;
        jobs[i].rel = eb_mode == FZ_EB_REL;
        field_items(lay[i].n, lay[i].nb, jobs[i].a.ntiles, jobs[i].rel != 0, jobs[i].nr, jobs[i].ne, jobs[i].nc);
    }
    // sizes: jobs | control words | segments | per field: slots, counts, group sums
    const uint64_t b_jobs = (sizeof(FieldJob) * (uint64_t)count + 255) & ~255ull;
    const uint64_t b_ctl  = (sizeof(FieldCtl) * (uint64_t)count + 255) & ~255ull;
    const uint64_t b_seg  = (sizeof(Segment) * 5ull * count + 255) & ~255ull;
    uint64_t       b_scr  = 0;
    std::vector<uint64_t> off(count);
    for (uint32_t i = 0; i < count; ++i) {
        off[i] = b_scr;
        b_scr += 4096ull * lay[i].nb + pad16(4ull * (lay[i].nb + 2)) + pad16(8ull * group_sum_words(lay[i].nb));
        b_scr = (b_scr + 255) & ~255ull;
    }
    uint8_t*    base = nullptr;
    cudaError_t e    = cudaMalloc(reinterpret_cast<void**>(&base), b_jobs + b_ctl + b_seg + std::max<uint64_t>(b_scr, 16));
    if (e != cudaSuccess) return map_err(e, FZ_FAIL_GPU_MALLOC);
    P.d_mem        = base;
    P.jobs         = reinterpret_cast<FieldJob*>(base);
    FieldCtl* ctl  = reinterpret_cast<FieldCtl*>(base + b_jobs);
    Segment*  segd = reinterpret_cast<Segment*>(base + b_jobs + b_ctl);
    uint8_t*  scr  = base + b_jobs + b_ctl + b_seg;
    std::vector<FieldCtl> hctl(count);
    std::vector<Segment>  hseg;
    for (uint32_t i = 0; i < count; ++i) {
        hctl[i].mm[0] = hctl[i].pre[0] = 0xFFFFFFFFu;  // empty ranges
        FieldJob& J   = jobs[i];
        J.ctl         = ctl + i;
        J.slots       = reinterpret_cast<uint4*>(scr + off[i]);
        J.counts      = reinterpret_cast<uint32_t*>(scr + off[i] + 4096ull * lay[i].nb);
        J.supers      = reinterpret_cast<uint32_t*>(scr + off[i] + 4096ull * lay[i].nb + pad16(4ull * (lay[i].nb + 2)));
        J.sstride     = group_sum_words(lay[i].nb);
        J.s2off       = group_sum_l2(lay[i].nb);
    }
    for (int k = 0; k < 5; ++k) {
        P.seg[k] = segd + hseg.size();
        for (uint32_t i = 0; i < count; ++i) {
            const uint32_t items = k == 0 ? jobs[i].nr : k == 4 ? jobs[i].nc : ((int)lay[i].ndim == k ? jobs[i].ne : 0u);
            if (!items) continue;
            hseg.push_back(Segment{P.total[k], i, items, 0u});
            P.total[k] += items;
            ++P.nseg[k];
        }
    }
    e = cudaMemset(base, 0, b_jobs + b_ctl + b_seg + std::max<uint64_t>(b_scr, 16));  // both group-sum sets at 0
    if (e == cudaSuccess) e = cudaMemcpy(P.jobs, jobs.data(), sizeof(FieldJob) * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ctl, hctl.data(), sizeof(FieldCtl) * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !hseg.empty())
        e = cudaMemcpy(segd, hseg.data(), sizeof(Segment) * hseg.size(), cudaMemcpyHostToDevice);
    return map_err(e);
}

// The batch's compression: one range launch over every field (relative eb), one encode
// launch per dimensionality present, one compaction launch over every field.
cudaError_t launch_list_compress(const ListPlan& P, cudaStream_t s)
{
    const FieldJob none{};
    cudaError_t    e = cudaSuccess;
    for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
        if (!P.total[k]) continue;
        const FieldPhase ph = k == 0 ? FieldPhase::Range : k == 4 ? FieldPhase::Compact : FieldPhase::Encode;
        e = launch_fields(ph, k >= 1 && k <= 3 ? k : 2, P.jobs, P.seg[k], P.nseg[k], P.total[k], none, s);
    }
    return e;
}

}  // namespace

struct fz_batch {
    cudaGraph_t                graph = nullptr;
    cudaGraphExec_t            exec  = nullptr;
    std::vector<fz_workspace*> own_ws;  // the extra branches' workspaces (decompression)
    void*                      d_list = nullptr;  // work list of the batch's compression
};

extern "C" {

// The batch is captured with parallel branches: fields go round-robin to up to
// `branches` forked streams, each with its own workspace (scan state, range
// accumulators), so the kernels of small fields run side by side.
static constexpr uint32_t kBatchBranches = 8;

fz_status fz_batch_create(fz_workspace* ws, const fz_field* fields, uint32_t count, fz_direction dir,
                          fz_eb_mode eb_mode, fz_mode mode, fz_batch** out)
{
    return fz_batch_create_ex(ws, fields, count, dir, eb_mode, mode, 0, out);
}

// Captures count fields into one graph: comp[i] (compression, if comp) followed by
// dec[i] (decompression, if dec) on branch i % branches, each branch with its own
// workspace; the fork and the join make the graph one unit on the launching stream.
// list: the compression as list launches over every field (then decompressions, if any,
// on the branches once all streams are written); otherwise each field's compression and
// decompression on its branch.
static fz_status capture_batch(fz_workspace* ws, const fz_field* comp, const fz_field* dec, uint32_t count,
                               fz_eb_mode eb_mode, fz_mode mode, uint32_t nbranch, bool list, fz_batch* b)
{
    const uint32_t branches = std::max(1u, std::min(nbranch ? nbranch : kBatchBranches, count));
    uint64_t       max_n    = 1;
    for (uint32_t i = 0; i < count; ++i) {
        if (comp) max_n = std::max<uint64_t>(max_n, comp[i].n);
        if (dec) max_n = std::max<uint64_t>(max_n, dec[i].header.n);
    }
    fz_status st = check_device(ws);
    if (st != FZ_SUCCESS) return st;
    ListPlan plan;
    if (list && comp && count) {
        st        = plan_list_compress(ws, comp, count, eb_mode, mode, plan);
        b->d_list = plan.d_mem;
        if (st != FZ_SUCCESS) return st;
    }
    std::vector<fz_workspace*> wss{ws};
    for (uint32_t i = 1; i < branches && st == FZ_SUCCESS; ++i) {
        fz_workspace* w = nullptr;
        st              = fz_workspace_create(std::max(max_n, (uint64_t)1), &w);
        if (st == FZ_SUCCESS) b->own_ws.push_back(w), wss.push_back(w);
    }
    std::vector<cudaStream_t> cs(branches, nullptr);
    std::vector<cudaEvent_t>  ev(branches, nullptr);
    for (uint32_t i = 0; i < branches && st == FZ_SUCCESS; ++i) {
        if (cudaStreamCreateWithFlags(&cs[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess)
            st = FZ_FAIL_GPU_ILLEGAL_ACCESS;
    }
    // no timing events inside a graph (event-record nodes would serialise the replay)
    std::vector<uint32_t> tcap(wss.size());
    for (size_t i = 0; i < wss.size(); ++i) tcap[i] = wss[i]->tcap, wss[i]->tcap = 0;
    if (st == FZ_SUCCESS) {
        cudaError_t e = cudaStreamBeginCapture(cs[0], cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) st = map_err(e);
        else {
            // list schedule: the whole compression in a handful of list launches
            if (plan.d_mem) {
                e = launch_list_compress(plan, cs[0]);
                if (e != cudaSuccess) st = map_err(e);
            }
            // fork: per-field work on parallel branches
            cudaEventRecord(ev[0], cs[0]);
            for (uint32_t i = 1; i < branches; ++i) cudaStreamWaitEvent(cs[i], ev[0], 0);
            // one branch: each field's encode launch takes the range of the next field (on
            // parallel branches the range launches already overlap other branches' kernels,
            // and taking them into the encode launches measured slower)
            std::vector<fz::RangeAhead> ra(branches);
            for (uint32_t i = 0; i < count && st == FZ_SUCCESS; ++i) {
                const uint32_t k = i % branches;
                fz_stream_t    h = reinterpret_cast<fz_stream_t>(cs[k]);
                if (comp && !plan.d_mem) {
                    const fz_field& f = comp[i];
                    ra[k].next        = branches == 1 && i + 1 < count ? comp + i + 1 : nullptr;
                    st = fz::compress_impl(wss[k], static_cast<const float*>(f.src), f.n, f.dims, f.eb, eb_mode, mode,
                                           f.dst, f.dst_capacity, nullptr, h, nullptr, &ra[k]);
                    ra[k].have = ra[k].done;
                }
                if (dec && st == FZ_SUCCESS) st = fz_decompress_batch(wss[k], dec + i, 1, h);
            }
            // join
            for (uint32_t i = 1; i < branches; ++i) {
                cudaEventRecord(ev[i], cs[i]);
                cudaStreamWaitEvent(cs[0], ev[i], 0);
            }
            cudaGraph_t g = nullptr;
            e             = cudaStreamEndCapture(cs[0], &g);
            if (st == FZ_SUCCESS && e != cudaSuccess) st = map_err(e);
            b->graph = g;
            if (st == FZ_SUCCESS) {
                e = cudaGraphInstantiate(&b->exec, g, 0);
                if (e != cudaSuccess) st = map_err(e);
            }
        }
    }
    for (size_t i = 0; i < wss.size(); ++i) wss[i]->tcap = tcap[i];
    for (uint32_t i = 0; i < branches; ++i) {
        if (cs[i]) cudaStreamDestroy(cs[i]);
        if (ev[i]) cudaEventDestroy(ev[i]);
    }
    return st;
}

fz_status fz_batch_create_ex(fz_workspace* ws, const fz_field* fields, uint32_t count, fz_direction dir,
                             fz_eb_mode eb_mode, fz_mode mode, uint32_t nbranch, fz_batch** out)
{
    if (!ws || !out || (!fields && count) || (dir != FZ_COMPRESS && dir != FZ_DECOMPRESS)) return FZ_INVALID_ARG;
    if (nbranch > FZ_BATCH_MAX_BRANCHES) return FZ_INVALID_ARG;
    *out = nullptr;
    fz_batch* b = new (std::nothrow) fz_batch();
    if (!b) return FZ_FAIL_GPU_MALLOC;
    const fz_status st = capture_batch(ws, dir == FZ_COMPRESS ? fields : nullptr, dir == FZ_DECOMPRESS ? fields : nullptr,
                                       count, eb_mode, mode, nbranch, false, b);
    if (st != FZ_SUCCESS) {
        fz_batch_destroy(b);
        return st;
    }
    *out = b;
    return FZ_SUCCESS;
}

fz_status fz_batch_create_pair(fz_workspace* ws, const fz_field* comp, const fz_field* dec, uint32_t count,
                               fz_eb_mode eb_mode, fz_mode mode, uint32_t nbranch, fz_batch** out)
{
    if (!ws || !out || ((!comp || !dec) && count)) return FZ_INVALID_ARG;
    if (nbranch > FZ_BATCH_MAX_BRANCHES) return FZ_INVALID_ARG;
    *out = nullptr;
    fz_batch* b = new (std::nothrow) fz_batch();
    if (!b) return FZ_FAIL_GPU_MALLOC;
    const fz_status st = capture_batch(ws, comp, dec, count, eb_mode, mode, nbranch, false, b);
    if (st != FZ_SUCCESS) {
        fz_batch_destroy(b);
        return st;
    }
    *out = b;
    return FZ_SUCCESS;
}

fz_status fz_batch_create_sched(fz_workspace* ws, const fz_field* comp, const fz_field* dec, uint32_t count,
                                fz_eb_mode eb_mode, fz_mode mode, const fz_batch_schedule* sched, fz_batch** out)
{
    if (!ws || !out || !sched || (!comp && !dec)) return FZ_INVALID_ARG;
    if (sched->branches > FZ_BATCH_MAX_BRANCHES || sched->list > 1) return FZ_INVALID_ARG;
    *out = nullptr;
    fz_batch* b = new (std::nothrow) fz_batch();
    if (!b) return FZ_FAIL_GPU_MALLOC;
    const fz_status st = capture_batch(ws, comp, dec, count, eb_mode, mode, sched->branches, sched->list != 0, b);
    if (st != FZ_SUCCESS) {
        fz_batch_destroy(b);
        return st;
    }
    *out = b;
    return FZ_SUCCESS;
}

fz_status fz_batch_autotune_sched(fz_workspace* ws, const fz_field* comp, const fz_field* dec, uint32_t count,
                                  fz_eb_mode eb_mode, fz_mode mode, uint32_t reps, fz_stream_t stream,
                                  fz_batch_schedule* best, double* ms)
{
    if (!ws || !best || !count || (!comp && !dec) || !reps) return FZ_INVALID_ARG;
    static constexpr uint32_t kCand[5] = {1, 2, 4, 8, 16};
    cudaStream_t s  = reinterpret_cast<cudaStream_t>(stream);
    cudaEvent_t  e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return FZ_FAIL_GPU_ILLEGAL_ACCESS;
    }
    fz_status st     = FZ_SUCCESS;
    float     best_t = 0;
    *best            = fz_batch_schedule{0, 0};
    for (int c = 0; c < 10 && st == FZ_SUCCESS; ++c) {
        if (ms) ms[c] = 0;
        const fz_batch_schedule cand{kCand[c % 5], (uint32_t)(c / 5)};
        if (cand.branches > count && c % 5 > 0) continue;  // the same graph as a smaller candidate
        if (cand.list && !comp) continue;                   // nothing to list without compression
        fz_batch* b = nullptr;
        st          = fz_batch_create_sched(ws, comp, dec, count, eb_mode, mode, &cand, &b);
        if (st != FZ_SUCCESS) break;
        st = fz_batch_launch(b, stream);  // warm-up
        cudaError_t e = st == FZ_SUCCESS ? cudaEventRecord(e0, s) : cudaSuccess;
        for (uint32_t r = 0; r < reps && st == FZ_SUCCESS && e == cudaSuccess; ++r) st = fz_batch_launch(b, stream);
        if (st == FZ_SUCCESS && e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (st == FZ_SUCCESS && e == cudaSuccess) e = cudaEventSynchronize(e1);
        float t = 0;
        if (st == FZ_SUCCESS && e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        if (st == FZ_SUCCESS && e != cudaSuccess) st = map_err(e);
        if (st == FZ_SUCCESS) {
            t /= (float)reps;
            if (ms) ms[c] = t;
            if (best->branches == 0 || t < best_t) *best = cand, best_t = t;
        }
        fz_batch_destroy(b);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

fz_status fz_batch_launch(fz_batch* b, fz_stream_t stream)
{
    if (!b || !b->exec) return FZ_INVALID_ARG;
    return map_err(cudaGraphLaunch(b->exec, reinterpret_cast<cudaStream_t>(stream)));
}

fz_status fz_batch_destroy(fz_batch* b)
{
    if (!b) return FZ_INVALID_ARG;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (fz_workspace* w : b->own_ws) fz_workspace_destroy(w);
    if (b->d_list) cudaFree(b->d_list);
    delete b;
    return FZ_SUCCESS;
}

fz_status fz_batch_autotune(fz_workspace* ws, const fz_field* fields, uint32_t count, fz_direction dir,
                            fz_eb_mode eb_mode, fz_mode mode, uint32_t reps, fz_stream_t stream,
                            uint32_t* best, double* ms)
{
    if (!ws || !best || !count || !fields || !reps) return FZ_INVALID_ARG;
    static constexpr uint32_t kCand[5] = {1, 2, 4, 8, 16};
    cudaStream_t s  = reinterpret_cast<cudaStream_t>(stream);
    cudaEvent_t  e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return FZ_FAIL_GPU_ILLEGAL_ACCESS;
    }
    fz_status st     = FZ_SUCCESS;
    float     best_t = 0;
    *best            = 0;
    for (int c = 0; c < 5 && st == FZ_SUCCESS; ++c) {
        if (ms) ms[c] = 0;
        if (kCand[c] > count && c > 0) continue;  // the same graph as a smaller candidate
        fz_batch* b = nullptr;
        st          = fz_batch_create_ex(ws, fields, count, dir, eb_mode, mode, kCand[c], &b);
        if (st != FZ_SUCCESS) break;
        st = fz_batch_launch(b, stream);  // warm-up
        cudaError_t e = st == FZ_SUCCESS ? cudaEventRecord(e0, s) : cudaSuccess;
        for (uint32_t r = 0; r < reps && st == FZ_SUCCESS && e == cudaSuccess; ++r) st = fz_batch_launch(b, stream);
        if (st == FZ_SUCCESS && e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (st == FZ_SUCCESS && e == cudaSuccess) e = cudaEventSynchronize(e1);
        float t = 0;
        if (st == FZ_SUCCESS && e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        if (st == FZ_SUCCESS && e != cudaSuccess) st = map_err(e);
        if (st == FZ_SUCCESS) {
            t /= (float)reps;
            if (ms) ms[c] = t;
            if (*best == 0 || t < best_t) *best = kCand[c], best_t = t;
        }
        fz_batch_destroy(b);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

}  // extern "C"
