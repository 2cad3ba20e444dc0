// fz_internal.h -- host-side declarations shared by the .cu files of the library.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/fz.h"
#include "fz_device.cuh"

namespace fz {

__host__ __device__ inline uint64_t cdiv(uint64_t a, uint64_t b) { return (a + b - 1) / b; }
__host__ __device__ inline uint64_t pad16(uint64_t a) { return (a + 15) & ~uint64_t(15); }

// A CUDA error as the status the C ABI reports (allocation and device-presence errors
// keep their own codes; everything else becomes `dflt`).
fz_status map_err(cudaError_t e, fz_status dflt = FZ_FAIL_GPU_ILLEGAL_ACCESS);
// x*y*z <= n without wrapping (each product is checked against n before the next one),
// every dimension at least 1 and 0 < n <= 2^31.  Every path that sizes a launch or a
// stream from dims (arguments or a stream header) goes through this check.
bool dims_fit(uint64_t n, uint32_t x, uint32_t y, uint32_t z);

// Geometry of one field and its stream.
struct Layout {
    uint32_t n, nl, x, y, z, xy, ndim;
    uint32_t nb;       // full shuffle blocks
    uint32_t tail;     // n - 2048 nb
    uint32_t nwords;   // bitmap words ceil(n/256)
    uint32_t mode;
    uint64_t off_a, off_c, off_b, off_sign, off_boff;  // byte offsets in the stream
    uint32_t sidecar_bytes;
};
Layout make_layout(uint64_t n, uint32_t x, uint32_t y, uint32_t z, uint32_t mode);

// Arguments of the fused compression kernel.
struct CompressArgs {
    const float* in;
    uint8_t*     out;
    uint32_t     n, nl, x, y, z, xy;
    FastDiv      dx, dxy;
    uint32_t     al_x, al_xy, al_xyx;  // 1 when the halo row offsets are multiples of 4
    uint32_t     nb, ntiles, nwords, mode, ndim, sidecar_bytes;
    uint64_t     off_a, off_c, off_b, off_sign, off_boff;
    uint32_t*    mm;  // range-pass accumulators (relative eb), or null
    double       eb_rel; // relative error bound (with mm)
    EbInfo       ebh;    // constants computed on the host (absolute eb)
    uint64_t*    state;
    uint32_t*    ticket;
    uint32_t*    status;
    uint32_t*    epoch;  // device epoch word (advanced by the kernel's last ticket fetch)
    uint32_t*    boff;   // block offset table in the stream's sidecar, or null
    uint32_t*    mirror; // list compression: 64-byte header + status word copied here, or null
    uint32_t*    fin;    // k_compress: CTA exit counter (zero on entry, left zero), or null
};

// ------------------------------------------------------ list compression --
// Compression of a list of fields in three launches (range, encode per dimensionality,
// compaction), each a persistent grid over the list's items: range items (max/min of 1024
// elements, relative eb only; a CTA takes a contiguous run), encode items (8 shuffle blocks:
// codes, bitshuffle, flags, chunks into per-block slots) and compaction items (32 blocks:
// offsets, chunks to their final place; the warp holding the last block writes the
// header).  One field is a list of one, passed as a kernel parameter.

// Per-field control words (device, 32 bytes).  Between calls: mm = pre = {0xFFFFFFFF, 0},
// flags = pre_flags = 0, and epoch = the number of calls that had full shuffle blocks.
// Whoever writes a call's header moves pre/pre_flags into mm/flags and resets pre: a
// call's encode launch may accumulate the range of the next field compressed with the
// same control words into pre (range ahead), which that field's encode then reads from mm.
struct FieldCtl {
    uint32_t mm[2];      // range accumulators (order-preserving u32)
    uint32_t flags;      // this call: kStatusNonfinite, bit 8 code overflow
    uint32_t epoch;      // a call uses group-sum set (epoch & 1) and clears the other
    uint32_t pre[2];     // the next call's range accumulators (range ahead)
    uint32_t pre_flags;  // the next call's kStatusNonfinite
    uint32_t pad;
};

struct FieldJob {
    CompressArgs a;       // geometry, stream offsets, eb (a.mm unused), status, boff, mirror
    FieldCtl*    ctl;
    uint4*       slots;   // 4 KiB per shuffle block
    uint32_t*    counts;  // chunks per block
    uint32_t*    supers;  // two sets of `sstride` words of chunk counts: per group of
                          // kSuperBlocks blocks, then (from word s2off) per group of
                          // kSuper2Blocks; a call adds into one set and clears the other
    uint32_t     sstride;     // words per set (group_sum_words)
    uint32_t     s2off;       // first word of the second-level sums in a set
    uint32_t     nr, ne, nc;  // range, encode, compaction items
    uint32_t     rel;         // relative eb: the eb follows from the range items
    // range ahead (single-field encode launches only): the range of ahead_n elements at
    // ahead_in, ahead_nr range items, into ctl->pre by the CTAs that took the fewest
    // encode items; ahead_nr == 0: none
    const float* ahead_in;
    uint32_t     ahead_n, ahead_nr;
};

// Items [start, start + count) of a list launch belong to field `field` (its items 0 ..
// count-1 of that launch's kind); segments sorted by start, no gaps.
struct Segment {
    uint32_t start, field, count, pad;
};

enum class FieldPhase { Range, Encode, Compact };

// Shuffle blocks per group sum of chunk counts, on two levels: a compaction warp's offset is
// the second-level sums before its second-level group, plus at most 63 first-level sums
// inside it, plus at most 63 counts inside its first-level group -- one round of loads
// whose length grows with nb / 4096, not with nb.
constexpr uint32_t kSuperBlocks  = 64;
constexpr uint32_t kSuper2Blocks = kSuperBlocks * 64;
// Words of one set of group sums for up to nb blocks, and where its second level starts.
__host__ __device__ inline uint32_t group_sum_l2(uint32_t nb) { return nb / kSuperBlocks + 2; }
__host__ __device__ inline uint32_t group_sum_words(uint32_t nb) { return group_sum_l2(nb) + nb / kSuper2Blocks + 2; }

// A launch of a kernel that starts with pdl_wait(): with programmatic stream serialization
// when the stream is not being captured.  Measured on GB300 (128 exafel-like round trips):
// eager launches on one stream 2043 -> 2210 GB/s; in graphs, which already have no launch
// gaps, 1 branch unchanged, 16 branches -1.2% and list launches -3% (the early CTAs wait on
// SMs that other branches' kernels would use), so captured launches go without it.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              const Args&... args)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
        (void)cudaGetLastError();  // a query that failed leaves no error behind
        cs = cudaStreamCaptureStatusActive;
    }
    cudaLaunchAttribute at{};
    at.id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    at.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid, cfg.blockDim = block, cfg.dynamicSmemBytes = smem, cfg.stream = s;
    cfg.attrs = &at, cfg.numAttrs = cs == cudaStreamCaptureStatusNone ? 1u : 0u;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Items of each kind for a field of n elements (ntiles scan tiles of shuffle blocks, nb full
// blocks).
void field_items(uint32_t n, uint32_t nb, uint32_t ntiles, bool rel, uint32_t& nr, uint32_t& ne, uint32_t& nc);
// One list launch of `phase` (encode: of dimensionality nd) over `total` items: jobs/segs
// device arrays of a batch, or jobs == nullptr and `one` the only field.  The grid is
// max(total, min_ctas) CTAs, at most one resident wave (min_ctas: an encode launch with
// range ahead spreads the ahead field's range items over CTAs without encode items).
cudaError_t launch_fields(FieldPhase phase, int nd, const FieldJob* jobs, const Segment* segs, uint32_t nseg,
                          uint32_t total, const FieldJob& one, cudaStream_t s, uint32_t min_ctas = 0);

struct DecodeArgs {
    const uint8_t*  st;
    const uint32_t* boff;     // chunk offset of each shuffle block (k_offsets)
    float*          out;      // fused paths
    uint32_t        n, nl, x, y, z, nb, tail, mode, nwords;
    uint64_t        off_a, off_c, off_b, off_sign, off_boff, nnz;
    float           ebx2;
    uint32_t*       status;
};

struct ReconArgs {
    const uint16_t* codes;
    const uint32_t* signbits;  // 1D sign bits (nullable)
    const uint8_t*  signum;    // 1D per-element signs (nullable; stage API)
    float*          out;
    uint32_t        n, nl, x, y, z;
    float           ebx2;
};

// launchers (return the launch error)
// callw: nullable per-call word that also receives kStatusNonfinite
cudaError_t launch_range(const float* in, uint32_t n, uint32_t* mm, uint32_t* status, uint32_t* callw,
                         cudaStream_t s);
cudaError_t launch_compress(const CompressArgs& a, cudaStream_t s);  // fused, single launch
cudaError_t launch_offsets(const uint8_t* st, uint64_t off_a, uint32_t nb, uint32_t nwords, uint64_t nnz,
                           uint32_t* boff, uint64_t* state, uint32_t* ticket, uint32_t* status,
                           uint32_t* epoch, cudaStream_t s);
// fused decode + inverse Lorenzo (every shape)
cudaError_t launch_decompress_fused(const DecodeArgs& a, cudaStream_t s);
cudaError_t launch_reconstruct(const ReconArgs& a, cudaStream_t s);
cudaError_t launch_zero_tail(float* out, uint32_t from, uint32_t n, cudaStream_t s);

cudaError_t launch_wait_selftest(const uint64_t* state, const uint32_t* epoch, uint32_t* status, cudaStream_t s);

// stage-level launchers
cudaError_t launch_lorenzo_construct(const float* in, uint16_t* q, uint8_t* signum, uint32_t x,
                                     uint32_t y, uint32_t z, float ebx2_r, cudaStream_t s);
cudaError_t launch_bitshuffle_flag(const uint32_t* in, uint32_t* out, uint32_t n_codes,
                                   uint32_t* bitflag, uint32_t* byteflag, cudaStream_t s);
cudaError_t launch_scan_encode(const uint8_t* shuffled, const uint32_t* byteflag,
                               uint32_t n_codes, uint32_t* presum, uint8_t* out,
                               uint64_t* state, uint32_t* ticket, uint32_t* status,
                               uint32_t* total, uint32_t* epoch, cudaStream_t s);


}  // namespace fz
