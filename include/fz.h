/*
 * fz.h -- C ABI of the GB300-native FZ compression pipeline.
 *
 * The reference (FZ-GPU) exposes its hot path at three boundaries; each entry point
 * below names the reference interface it replaces:
 *   - the CLI / host orchestration  runSzs() ................. fz.cu:113-224
 *   - the C++ launchers  launch_{construct,reconstruct}_LorenzoI_var
 *                                                  include/kernel/lorenzo_var.cuh:520-673
 *   - the raw kernels  bitshuffleAndBitflag / cub::DeviceScan::ExclusiveSum / encodeDebug
 *                                                  fz.cu:49-111, fz.cu:187-205
 * The status enum keeps the values of the reference's C-ABI error enum
 * (include/cusz/type.h:25-44) and adds codes for stream and launch failures.
 *
 * Conventions
 *   - Every device-buffer entry point is stream-ordered: it enqueues work on `stream`
 *     and returns without synchronising, unless an optional host output (marked
 *     "host, nullable, syncs") is requested.
 *   - Buffers are caller-owned. Device pointers must be 16-byte aligned.
 *   - Nothing here calls exit(); every failure is a returned fz_status.
 *   - A workspace holds the scan state of one in-flight call. Use one workspace per
 *     stream (or per host thread); concurrent calls on one workspace race.
 *   - Sizes are 64-bit. Dimensions are (x, y, z) with x fastest, as the reference's
 *     dim3 len3 (fz.cu:116, 231-233).  One field holds at most 2^31 elements (the
 *     reference's int sizes cap it at 2^29, fz.cu:117-118).
 */
#ifndef FZ_GB300_FZ_H
#define FZ_GB300_FZ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without pulling in CUDA headers (same underlying type). */
typedef struct CUstream_st* fz_stream_t;

/* ---------------------------------------------------------------- status -- */
typedef enum fz_status {
    FZ_SUCCESS                  = 0x00, /* CUSZ_SUCCESS */
    FZ_FAIL_ONDISK_FILE_ERROR   = 0x01, /* CUSZ_FAIL_ONDISK_FILE_ERROR */
    FZ_FAIL_DATA_NOT_READY      = 0x02, /* CUSZ_FAIL_DATA_NOT_READY */
    FZ_FAIL_GPU_MALLOC          = 0x03, /* CUSZ_FAIL_GPU_MALLOC */
    FZ_FAIL_GPU_MEMCPY          = 0x04, /* CUSZ_FAIL_GPU_MEMCPY */
    FZ_FAIL_GPU_ILLEGAL_ACCESS  = 0x05, /* CUSZ_FAIL_GPU_ILLEGAL_ACCESS: any launch/runtime error */
    FZ_FAIL_GPU_OUT_OF_MEMORY   = 0x06, /* CUSZ_FAIL_GPU_OUT_OF_MEMORY */
    FZ_FAIL_INCOMPRESSIABLE     = 0x07, /* CUSZ_FAIL_INCOMPRESSIABLE */
    FZ_FAIL_UNSUPPORTED_DATATYPE = 0x08,
    FZ_NOT_IMPLEMENTED          = 0x0100, /* CUSZ_NOT_IMPLEMENTED */
    /* codes without a reference counterpart */
    FZ_INVALID_ARG              = 0x0200, /* bad pointer/size/dims/eb */
    FZ_CORRUPT_STREAM           = 0x0201, /* header or section sizes inconsistent */
    FZ_OUT_OF_SPACE             = 0x0202, /* output capacity too small */
    FZ_TIMEOUT                  = 0x0203, /* a bounded device-side wait gave up */
    FZ_NO_DEVICE                = 0x0204, /* no CUDA device / driver */
    FZ_NONFINITE_INPUT          = 0x0205  /* NaN/Inf in a relative-eb input */
} fz_status;

/* ------------------------------------------------------------- constants -- */
#define FZ_MAGIC            0x31475A46u /* "FZG1" little-endian */
#define FZ_FORMAT_VERSION   1u
#define FZ_HEADER_BYTES     64u
#define FZ_BLOCK_CODES      2048u /* codes per shuffle block: grid floor(N/2048), fz.cu:173 */
#define FZ_BLOCK_WORDS      1024u /* u32 words per shuffle block, fz.cu:73 */
#define FZ_CHUNK_BYTES      16u   /* blockSize, fz.cu:157 */
#define FZ_CHUNKS_PER_BLOCK 256u  /* 4 KiB / 16 B */
#define FZ_CODES_PER_WORD   256u  /* codes covered by one bitmap word (32 chunks x 8 codes) */

/* header flags */
/* some delta did not fit its code field (|d| >= 32768 signed, >= 65536 for 1D unsigned
   positions, or non-finite): the stream does not meet the error bound there */
#define FZ_FLAG_CODE_OVERFLOW 0x1u
/* the compressing kernels reported a failure (NaN/Inf in a relative-eb input, or a
   bounded device-side wait that gave up): the stream is not valid, and every entry point
   that reads a header rejects it with FZ_CORRUPT_STREAM.  Lets a caller that skips the
   size readback (out_bytes NULL) still see the failure in the stream itself. */
#define FZ_FLAG_FAILED        0x2u

typedef enum fz_mode {
    /* Sections A+B only: the reference's exact compressed content. Not invertible
       for the tail codes (N mod 2048) or for 1D signs at i%4!=0. */
    FZ_MODE_COMPAT = 0,
    /* Sections A+B unchanged, plus a fixed-size Section C holding the raw tail codes
       and (1D only) every delta's sign bit, so decompression meets the error bound. */
    FZ_MODE_SIDECAR = 1
} fz_mode;

typedef enum fz_eb_mode {
    FZ_EB_ABS = 0, /* eb is absolute (launch_construct_LorenzoI_var's eb, lorenzo_var.cuh:526) */
    FZ_EB_REL = 1  /* eb is relative to max-min of the input (fz.cu:137,149) */
} fz_eb_mode;

typedef struct fz_dims {
    uint32_t x, y, z; /* x fastest; ndim = 1 if y==z==1, 2 if z==1, else 3 */
} fz_dims;

/* 64-byte little-endian stream header.  Stream layout:
 *   [header 64 B][Section A: u32 bitmap[ceil(n/256)], padded to 16 B]
 *   [Section C: sidecar_bytes][Section B: nnz x 16 B chunks]
 * Sections A and B hold exactly the reference's d_bitFlagArray[0..ceil(n/256)) and
 * d_out[0..16*nnz) (fz.cu:109, fz.cu:57). */
typedef struct fz_header {
    uint32_t magic;
    uint16_t version;
    uint8_t  mode;     /* fz_mode */
    uint8_t  ndim;
    uint32_t x, y, z;
    uint32_t flags;    /* FZ_FLAG_* */
    uint64_t n;        /* element count = file bytes / 4 (fz.cu:118) */
    double   eb_abs;   /* absolute error bound */
    float    ebx2_r;   /* (float)(1 / (2 eb_abs)), lorenzo_var.cuh:562-563 */
    float    ebx2;     /* (float)(2 eb_abs), lorenzo_var.cuh:641 */
    uint64_t nnz;      /* non-zero 16-byte chunks in Section B */
    float    range;    /* max - min of the input (0 in FZ_EB_ABS mode) */
    uint32_t sidecar_bytes;
} fz_header;

typedef struct fz_workspace fz_workspace;

/* ------------------------------------------------------------ utilities -- */
const char* fz_status_string(fz_status s);
const char* fz_version(void);
/* Number of dimensions the reference's launcher dispatches on (lorenzo_var.cuh:537-544). */
int fz_ndim(fz_dims dims);

/* Byte offsets of the sections of a stream for `n` elements. */
fz_status fz_stream_layout(uint64_t n, fz_dims dims, fz_mode mode, uint64_t* off_a,
                           uint64_t* off_c, uint64_t* off_b, uint32_t* sidecar_bytes);
/* Worst-case stream size (every chunk non-zero). */
fz_status fz_max_compressed_bytes(uint64_t n, fz_dims dims, fz_mode mode, uint64_t* bytes);
/* Total stream bytes implied by a header (validates it). */
fz_status fz_stream_bytes(const fz_header* h, uint64_t* bytes);
/* The three numbers runSzs prints (fz.cu:207-209): file size, 4*ceil(n/256) + 16*nnz,
   and their ratio. */
fz_status fz_reference_sizes(uint64_t file_bytes, uint64_t nnz, uint64_t* original,
                             uint64_t* compressed, double* ratio);

/* ------------------------------------------------------------ workspace -- */
/* Device scratch for fields of up to max_n elements (scan state, range reduction, one
   4 KiB slot per 2048-code block for compression, block counts and offsets; about 2.5
   bytes per element) plus a pinned host word for optional readbacks. */
fz_status fz_workspace_create(uint64_t max_n, fz_workspace** ws);
fz_status fz_workspace_destroy(fz_workspace* ws);
/* Device bytes a workspace for max_n elements allocates. */
fz_status fz_workspace_bytes(uint64_t max_n, uint64_t* bytes);
/* Device-side status of the last call on this workspace (syncs `stream`):
   FZ_SUCCESS, FZ_TIMEOUT or FZ_NONFINITE_INPUT. Clears it. */
fz_status fz_workspace_status(fz_workspace* ws, fz_stream_t stream);

/* Per-kernel timing, the counterpart of the reference launcher's time_elapsed
   out-parameter (lorenzo_var.cuh:527,568-596).  Once enabled, each kernel launch made
   by a call on this workspace (up to `capacity` launches in total) is bracketed by a
   pair of CUDA events on the call's stream.  capacity 0 disables it. */
fz_status fz_workspace_enable_timing(fz_workspace* ws, uint32_t capacity);
/* Number of recorded launches of one kernel kind (0 range pass, 1 encode -- codes,
   bitshuffle, flags and per-block compaction into slots --, 2 block offsets, 3 decode --
   fused with the inverse Lorenzo --, 4 separate inverse Lorenzo, 5 compaction -- offsets
   and the move into the stream) and their summed duration; syncs on the last recorded
   event and frees those records. */
fz_status fz_workspace_kernel_time(fz_workspace* ws, int kind, uint32_t* launches,
                                   double* total_ms);

/* Diagnostic: launches one warp whose look-back waits on a tile that nothing
   publishes.  The bounded wait gives up after its poll limit (about a second) and the
   call returns FZ_TIMEOUT; any other result means the wait bound is broken.  No
   reference counterpart (the reference's only device-wide step is a CUB scan). */
fz_status fz_selftest_wait_timeout(fz_workspace* ws, fz_stream_t stream);

/* ------------------------------------------------ full pipeline, device -- */
/* Compress d_in[0..n) (dims describe the first x*y*z elements; n may exceed it as
   in fz.cu:117-118) into d_out.  Replaces runSzs (fz.cu:113-224) minus file I/O.
   out_bytes: host, nullable, syncs -- the stream's total size.  Without it, a failure
   found on the device (NaN/Inf in a relative-eb input) marks the header with
   FZ_FLAG_FAILED and stays readable through fz_workspace_status. */
fz_status fz_compress(fz_workspace* ws, const float* d_in, uint64_t n, fz_dims dims,
                      double eb, fz_eb_mode eb_mode, fz_mode mode, void* d_out,
                      uint64_t out_capacity, uint64_t* out_bytes, fz_stream_t stream);

/* Decompress a stream produced by fz_compress into d_out[0..n).  h_header is the
   stream's header copied to host memory (the caller usually has it already; pass
   NULL to have it read back, which syncs).  No reference counterpart: the
   reference has no working FZ decompressor; this is the inverse of fz_compress. */
fz_status fz_decompress(fz_workspace* ws, const void* d_stream, uint64_t stream_bytes,
                        const fz_header* h_header, float* d_out, uint64_t out_capacity_elems,
                        fz_stream_t stream);

/* Compression that allocates nothing, for callers that cannot call cudaMalloc:
   frameworks that own all device memory through their own pool, and loops that cannot
   afford cudaMalloc's implicit synchronisation.  Same arguments and result as
   fz_compress, without a workspace.  Its scratch is a fixed static device array of
   FZ_NOALLOC_SCRATCH_BYTES inside the library, held by every GPU that loads it until the
   process exits; fields larger than FZ_NOALLOC_MAX_ELEMS elements are rejected with
   FZ_INVALID_ARG before anything is launched.  The first call on a device looks up the
   array's device address (cudaGetSymbolAddress).  All calls share the array: calls whose GPU work overlaps race, so
   serialise them (one stream).  out_bytes (host, nullable) reads the size back and
   synchronises the stream; with it NULL the call returns without waiting, and a failure
   found on the device (NaN/Inf in a relative-eb input, a wait that gave up) marks the
   stream's header with FZ_FLAG_FAILED, so fz_stream_bytes and fz_decompress reject it
   with FZ_CORRUPT_STREAM.  No counterpart in the reference. */
#define FZ_NOALLOC_MAX_ELEMS     (1ull << 26)
#define FZ_NOALLOC_SCRATCH_BYTES 33280u
fz_status fz_compress_noalloc(const float* d_in, uint64_t n, fz_dims dims, double eb,
                              fz_eb_mode eb_mode, fz_mode mode, void* d_out,
                              uint64_t out_capacity, uint64_t* out_bytes, fz_stream_t stream);

/* ------------------------------------------------- full pipeline, host -- */
/* Same as above with host buffers: H2D of the input, compress, D2H of the stream;
   synchronous.  The device staging buffers live in the workspace (allocated on the
   first call, sized for its max_n).  h_in/h_out should be pinned for full bandwidth.
   This is what the fz-gpu CLI calls (fz.cu:136-209). */
fz_status fz_compress_host(fz_workspace* ws, const float* h_in, uint64_t n, fz_dims dims,
                           double eb, fz_eb_mode eb_mode, fz_mode mode, void* h_out,
                           uint64_t out_capacity, uint64_t* out_bytes, fz_stream_t stream);
fz_status fz_decompress_host(fz_workspace* ws, const void* h_stream, uint64_t stream_bytes,
                             float* h_out, uint64_t out_capacity_elems, fz_stream_t stream);

/* ------------------------------------------------ stage-level drop-ins -- */
/* Lorenzo dual-quantisation into 16-bit sign-magnitude codes; replaces
   launch_construct_LorenzoI_var<float,uint16_t,float> (lorenzo_var.cuh:520-597).
   Writes d_quant[i] for i < x*y*z only (fz.cu:145 pre-zeroes the rest).  The 1D
   sign of every delta is written to d_signum[i] (0/1) when d_signum is non-NULL; the
   reference leaves signum unused (fz.cu:152). */
fz_status fz_lorenzo_construct(const float* d_data, uint16_t* d_quant, uint8_t* d_signum,
                               fz_dims len3, double eb_abs, fz_stream_t stream);

/* Inverse of the above for sign-magnitude codes; replaces
   launch_reconstruct_LorenzoI_var (lorenzo_var.cuh:599-673), whose input format
   (separate signum + magnitude) the compressor never produces.  1D: d_signum (0/1
   per element, nullable) supplies the signs that the codes at i%4!=0 lack. */
fz_status fz_lorenzo_reconstruct(const uint16_t* d_quant, const uint8_t* d_signum,
                                 float* d_xdata, fz_dims len3, double eb_abs,
                                 fz_stream_t stream);

/* Bitshuffle of n_codes 16-bit codes (viewed as u32 words) in 4 KiB blocks with
   16-byte chunk flags and a 1-bit-per-chunk bitmap; replaces bitshuffleAndBitflag
   (fz.cu:61-111) and its grid floor(N/2048) (fz.cu:172-174).  Words past the last
   full block are copied unchanged (fz.cu:155).  d_byteflag: u32[32*ceil(n/256)],
   d_bitflag: u32[ceil(n/256)], both fully written (zero past the last full block). */
fz_status fz_bitshuffle_flag(const uint32_t* d_in, uint32_t* d_out, uint64_t n_codes,
                             uint32_t* d_bitflag, uint32_t* d_byteflag, fz_stream_t stream);

/* Exclusive prefix sum of the chunk flags plus compaction of the flagged 16-byte
   chunks; replaces cub::DeviceScan::ExclusiveSum + the total fix-up + encodeDebug
   (fz.cu:187-205).  d_presum (nullable) receives P[0..M] with M = 32*ceil(n/256)
   (fz.cu:180); d_out must hold 16*M bytes, as the reference's d_out does (fz.cu:165);
   nnz: host, nullable, syncs. */
fz_status fz_scan_encode(fz_workspace* ws, const uint8_t* d_shuffled,
                         const uint32_t* d_byteflag, uint64_t n_codes, uint32_t* d_presum,
                         uint8_t* d_out, uint64_t* nnz, fz_stream_t stream);

/* ------------------------------------------------------------- batching -- */
/* One field of a batch.  Compression reads src (float[n], dims, eb) and writes the
   stream to dst (dst_capacity bytes, at least fz_max_compressed_bytes); decompression
   reads the stream src (src_bytes, with its header copied to `header`) and writes
   dst (dst_capacity elements). */
typedef struct fz_field {
    const void* src;
    void*       dst;
    uint64_t    n;
    fz_dims     dims;
    double      eb;
    uint64_t    dst_capacity;
    uint64_t    src_bytes;
    fz_header   header;
} fz_field;

typedef enum fz_direction { FZ_COMPRESS = 0, FZ_DECOMPRESS = 1 } fz_direction;

/* Enqueues the whole batch on `stream` in one call (fields in order, one workspace:
   its capacity must cover the largest field).  With a relative bound, each field's
   encode launch also reads the next field's input for its value range (that field
   then runs no range launch of its own), so every input of the batch must be ready
   when the call is enqueued.  No counterpart in the reference, which handles one file
   per process (fz.cu:226-238). */
fz_status fz_compress_batch(fz_workspace* ws, const fz_field* fields, uint32_t count,
                            fz_eb_mode eb_mode, fz_mode mode, fz_stream_t stream);
fz_status fz_decompress_batch(fz_workspace* ws, const fz_field* fields, uint32_t count,
                              fz_stream_t stream);

/* A batch recorded once into a CUDA graph and replayed with fz_batch_launch; the
   buffers of `fields` must stay valid while the batch exists.  The graph runs the
   fields on up to 8 parallel branches (round-robin), each with its own workspace (`ws`
   serves the first; the batch allocates the others), so small fields overlap.  The
   scan state's epoch is kept in device memory, so replays with frozen kernel
   parameters stay correct. */
typedef struct fz_batch fz_batch;
fz_status fz_batch_create(fz_workspace* ws, const fz_field* fields, uint32_t count,
                          fz_direction dir, fz_eb_mode eb_mode, fz_mode mode, fz_batch** out);
fz_status fz_batch_launch(fz_batch* batch, fz_stream_t stream);
fz_status fz_batch_destroy(fz_batch* batch);

/* The same with an explicit number of parallel branches (1..FZ_BATCH_MAX_BRANCHES; 0 =
   the default of fz_batch_create, 8).  No counterpart in the reference. */
#define FZ_BATCH_MAX_BRANCHES 16u
fz_status fz_batch_create_ex(fz_workspace* ws, const fz_field* fields, uint32_t count,
                             fz_direction dir, fz_eb_mode eb_mode, fz_mode mode, uint32_t branches,
                             fz_batch** out);

/* A round-trip batch (no counterpart in the reference): field i is compressed from
   comp[i] and then decompressed from dec[i] (dec[i].src is normally comp[i].dst, with
   dec[i].header taken from a compression of the same data), the pairs on up to
   `branches` parallel branches (0 = 8) of one graph, so one field's decompression
   overlaps other fields' compression.  Replays with the same inputs reproduce the same
   streams, so the captured headers stay valid. */
fz_status fz_batch_create_pair(fz_workspace* ws, const fz_field* comp, const fz_field* dec, uint32_t count,
                               fz_eb_mode eb_mode, fz_mode mode, uint32_t branches, fz_batch** out);

/* Batch schedules (no counterpart in the reference).  branches: parallel graph branches
   for per-field work (1..FZ_BATCH_MAX_BRANCHES, 0 = 8).  list = 1: the compression of every
   field as list launches -- one range launch, one encode launch per dimensionality present
   and one compaction launch, persistent grids striding over a device work list of all the
   batch's fields (per-field jobs, control words and slots allocated with the batch, 2
   bytes per element) -- and decompressions, if any, on the branches after it; list = 0:
   each field's compression (and decompression) on its branch.  comp and dec may each be
   NULL (not both); with both, dec[i] decompresses what comp[i] compresses. */
typedef struct fz_batch_schedule {
    uint32_t branches;
    uint32_t list;
} fz_batch_schedule;
fz_status fz_batch_create_sched(fz_workspace* ws, const fz_field* comp, const fz_field* dec, uint32_t count,
                                fz_eb_mode eb_mode, fz_mode mode, const fz_batch_schedule* sched, fz_batch** out);
/* Times every schedule (branches 1, 2, 4, 8, 16 capped at count, each with list 0 and 1)
   on these fields, `reps` replays each on `stream`, and returns the fastest in *best; ms
   (nullable) receives the mean replay times, ms[0..4] list 0 and ms[5..9] list 1 (0 for
   candidates not run). */
fz_status fz_batch_autotune_sched(fz_workspace* ws, const fz_field* comp, const fz_field* dec, uint32_t count,
                                  fz_eb_mode eb_mode, fz_mode mode, uint32_t reps, fz_stream_t stream,
                                  fz_batch_schedule* best, double* ms);

/* Autotuner for batch scheduling (no counterpart in the reference).  The stream format
   fixes the shuffle block and the Lorenzo tiles, so what is tuned is how many fields run
   side by side: captures the batch with 1, 2, 4, 8 and 16 branches (capped at `count`),
   replays each `reps` times on `stream` (timed with CUDA events; the replays do the
   batch's work, so its outputs are written) and returns the fastest branch count in
   *best and, if ms is not null, each candidate's mean replay time in ms[0..4] (0 for
   candidates above `count`). */
fz_status fz_batch_autotune(fz_workspace* ws, const fz_field* fields, uint32_t count, fz_direction dir,
                            fz_eb_mode eb_mode, fz_mode mode, uint32_t reps, fz_stream_t stream,
                            uint32_t* best, double* ms);

/* -------------------------------------------------------------- serving -- */
/* A request on host buffers (pinned buffers let copies overlap with other requests).
   Compression: src float[n] with dims, eb, eb_mode, mode -> dst (dst_capacity bytes).
   Decompression: src the stream (src_bytes; its header is read from src) -> dst float[n]
   (dst_capacity bytes, at least 4n).  A request that can never run (larger than the
   budget or than max_n, or dst too small) completes with FZ_OUT_OF_SPACE/FZ_INVALID_ARG. */
/* fz_request.flags: src and dst are device pointers (the field already lives in HBM and
   the result stays there); without it both are host pointers (pinned ones let the
   copies overlap) and the server stages them through its pool. */
#define FZ_REQUEST_DEVICE 1u

typedef struct fz_request {
    uint64_t     id;           /* the caller's tag, echoed in the completion */
    fz_direction dir;
    const void*  src;
    void*        dst;
    uint64_t     n;
    fz_dims      dims;
    double       eb;
    fz_eb_mode   eb_mode;
    fz_mode      mode;
    uint64_t     dst_capacity; /* bytes */
    uint64_t     src_bytes;
    uint32_t     flags;        /* FZ_REQUEST_DEVICE or 0 */
    const fz_header* header;   /* decompression of a device-resident stream: its header on
                                  the host, or null to have the server fetch it first */
} fz_request;

typedef struct fz_completion {
    uint64_t  id;
    fz_status status;
    uint64_t  bytes; /* compression: stream bytes written to dst; decompression: elements */
} fz_completion;

/* A request loop with continuous batching under an HBM budget: `slots` streams, each with
   its own workspace, share one device pool of hbm_budget bytes from which every admitted
   host-buffer request takes its input and output buffers (a device-resident request
   counts its input and output bytes against the same budget).  Requests queue in arrival
   order; the server's worker threads (up to 8, each owning some slots) retire finished
   requests and admit queued ones as slots and pool memory free up, so requests that arrive
   while others run overlap on the device; fz_server_poll (non-blocking) hands out the
   completions.  Admission looks at the first 64 queued requests: one may start ahead of
   earlier ones that wait for pool memory.  The functions may be called from any thread.  No counterpart in the
   reference (one field per process, fz.cu:226-238). */
typedef struct fz_server fz_server;
fz_status fz_server_create(uint64_t hbm_budget, uint32_t slots, uint64_t max_n, fz_server** out);
fz_status fz_server_submit(fz_server* server, const fz_request* request);
fz_status fz_server_poll(fz_server* server, fz_completion* out, uint32_t max, uint32_t* count);
fz_status fz_server_pending(fz_server* server, uint32_t* queued, uint32_t* running,
                            uint64_t* pool_used);
fz_status fz_server_destroy(fz_server* server);

#ifdef __cplusplus
}
#endif
#endif /* FZ_GB300_FZ_H */
