// fz_workspace.h -- the workspace behind the opaque fz_workspace handle (internal).
#pragma once

#include <vector>

#include "../../include/fz.h"
#include "fz_internal.h"

struct fz_workspace {
    int       device;
    uint64_t  max_n;
    uint32_t  max_tiles;
    void*     d_base;
    size_t    d_bytes;
    uint64_t* state;
    uint32_t* tickets;  // [0] look-back compress, [1] offsets, [2] scan-encode, [3] unused
    uint32_t* status;
    uint32_t* total;
    uint32_t* epoch;    // device epoch of the scan state
    uint32_t* supers;   // two sets of group sums of chunk counts (FieldJob::supers)
    fz::FieldCtl* fctl; // control words of the list compression
    uint32_t* mm;       // range accumulators (min, max as ordered u32)
    uint16_t* codes;
    uint32_t* boff;     // chunk offset of each shuffle block (decompression)
    uint8_t*  h_pinned;  // 64-byte header + status word
    // host-buffer path staging, allocated on first use
    float*    d_field;
    uint8_t*  d_stream;
    uint64_t  stream_cap;
    // per-kernel timing ring (fz_workspace_enable_timing)
    std::vector<cudaEvent_t> tev;   // 2 per record
    std::vector<int>         tkind;
    uint32_t                 tcap  = 0;
    uint32_t                 tused = 0;
};

namespace fz {
// Range ahead between consecutive compressions on one workspace and stream (relative eb):
// the call's encode launch also accumulates the range of `next`, which that field's call
// then takes instead of running its own range launch.
struct RangeAhead {
    const fz_field* next = nullptr;  // in: the field compressed next on this workspace, or null
    bool            have = false;    // in: this call's range was accumulated by the previous call
    bool            done = false;    // out: the range of `next` was accumulated
};
// fz_compress with an optional device mirror (128 bytes, 16-byte aligned) that receives
// the 64-byte header and, at word 16, the status word once the stream is complete.
fz_status compress_impl(fz_workspace* ws, const float* d_in, uint64_t n, fz_dims dims, double eb,
                        fz_eb_mode eb_mode, fz_mode mode, void* d_out, uint64_t out_capacity,
                        uint64_t* out_bytes, fz_stream_t stream, uint32_t* mirror, RangeAhead* ra = nullptr);
}  // namespace fz
