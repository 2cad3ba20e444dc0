// fz_device.cuh -- device building blocks shared by the compression kernels.
//
// Everything here is written for sm_103a: 32-lane warps, redux.sync reductions,
// ld.acquire/st.release for the scan state, byte-permute for the bit transpose.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fz {

constexpr uint32_t kFull        = 0xFFFFFFFFu;
constexpr uint32_t kBlockCodes  = 2048;  // codes per shuffle block (fz.cu:173)
constexpr uint32_t kBlockWords  = 1024;  // u32 words per shuffle block (fz.cu:73)
constexpr uint32_t kChunks      = 256;   // 16-byte chunks per shuffle block
constexpr uint32_t kHeaderBytes = 64;

// ------------------------------------------------- dependent launches --
// Outside graph capture the path's kernels are launched with programmatic stream
// serialization (launch_pdl): a kernel's CTAs may be scheduled while the previous kernel on
// the stream finishes, so
// each calls pdl_wait() before its first memory access -- it returns once the grids it
// depends on have completed and their writes are visible (at once for a launch without
// the attribute) -- and pdl_trigger() to let the next launch's CTAs take SMs as its own
// retire.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// ---------------------------------------------------------------- eb info --
// Written by the range pass (relative eb) or by the host (absolute eb).
struct EbInfo {
    double   eb_abs;
    float    ebx2_r;   // (float)(1 / (2 eb)), lorenzo_var.cuh:562-563
    float    ebx2;     // (float)(2 eb), lorenzo_var.cuh:641
    float    range;    // max - min (float), fz.cu:137
    float    vmin, vmax;
    uint32_t nonfinite;
};

// Order-preserving u32 encoding of a (non-NaN) float, for atomicMin/atomicMax.
__device__ __forceinline__ uint32_t f2ord(float f)
{
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t o)
{
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

// ------------------------------------------------------------ status bits --
constexpr uint32_t kStatusTimeout   = 1u;
constexpr uint32_t kStatusNonfinite = 2u;
constexpr uint32_t kStatusCorrupt   = 4u;

// ----------------------------------------------------------- fast divide --
// floor(n / d) for n, d < 2^32 via one 64-bit high multiply: with M = floor(2^64/d)+1
// the error n*(M - 2^64/d)/2^64 < 2^-32 <= 1/d never crosses an integer.
struct FastDiv {
    uint64_t m;
    uint32_t d;
};
inline FastDiv make_fastdiv(uint32_t d)
{
    FastDiv f;
    f.d = d;
    // floor((2^64-1)/d) + 1 is floor(2^64/d) + 1, or exactly 2^64/d for powers of two
    f.m = d <= 1 ? 0 : (~0ull / d) + 1;
    return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f)
{
    return f.d == 1 ? n : (uint32_t)__umul64hi((uint64_t)n, f.m);
}

// ------------------------------------------------------------ prequant --
// Round half away from zero as trunc(v + copysign(pred(1/2), v)), pred(1/2) the float
// just below 1/2: with round-to-nearest addition this equals round(v) for every float
// (checked exhaustively over all finite floats; +-Inf and NaN pass through).
__device__ __forceinline__ float round_half_away(float v)
{
    const float h = __uint_as_float((__float_as_uint(v) & 0x80000000u) | 0x3EFFFFFFu);
    return truncf(__fadd_rn(v, h));
}
// Prequantisation round(x * ebx2_r) in float (lorenzo_var.cuh:81,125,265).
__device__ __forceinline__ float pq(float v, float r) { return round_half_away(__fmul_rn(v, r)); }

// (u16)fabs(d) | (d < 0) << 15 -- the expression of lorenzo_var.cuh:169-171.
__device__ __forceinline__ uint32_t pack_signed(float d)
{
    uint16_t tmp = static_cast<uint16_t>(fabsf(d));
    tmp |= ((d < 0) << 15);
    return tmp;
}
// Two sign-magnitude codes in one word: pack_signed(d0) | pack_signed(d1) << 16.  The
// (uint16_t) conversion of lorenzo_var.cuh:169-171 is a saturating f32 -> u32 conversion
// whose low 16 bits are kept; one byte permute takes both low halves, then both signs
// (d < 0: false for -0 and NaN) are OR-ed in.
__device__ __forceinline__ uint32_t pack_signed_pair(float d0, float d1)
{
    const uint32_t m0 = static_cast<uint32_t>(fabsf(d0)), m1 = static_cast<uint32_t>(fabsf(d1));
    return __byte_perm(m0, m1, 0x5410) | (d0 < 0.0f ? 0x8000u : 0u) | (d1 < 0.0f ? 0x80000000u : 0u);
}
// max(a, b) that returns NaN when either is NaN (max.NaN.f32): a running max of |d|
// answers "some delta does not fit 15 bits, or is NaN" with one compare at the end.
__device__ __forceinline__ float fmax_nan(float a, float b)
{
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
// max(a, b, c) with NaN propagation (the three-input max.NaN.f32 of sm_100 and later).
__device__ __forceinline__ float fmax3_nan(float a, float b, float c)
{
    float r;
    asm("max.NaN.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmin_nan(float a, float b)
{
    float r;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
// 1D positions i%4 != 0 store the magnitude only (lorenzo_var.cuh:62).
__device__ __forceinline__ uint32_t pack_unsigned(float d)
{
    return static_cast<uint16_t>(fabsf(d));
}

// ------------------------------------------------------------- transpose --
// x << J and x >> J as integer multiplies (the low and the high word of x * 2^J and of
// x * 2^(32-J)), which run on the multiply-add pipe instead of the integer/logic one.
template <int J>
__device__ __forceinline__ uint32_t shl_mul(uint32_t x)
{
    uint32_t r;
    asm("mul.lo.u32 %0, %1, %2;" : "=r"(r) : "r"(x), "n"(1u << J));
    return r;
}
template <int J>
__device__ __forceinline__ uint32_t shr_mul(uint32_t x)
{
    uint32_t r;
    asm("mul.hi.u32 %0, %1, %2;" : "=r"(r) : "r"(x), "n"(1u << (32 - J)));
    return r;
}

// One off-diagonal swap stage of width J (mask M keeps the low J bits of every 2J).
// kMul: the shifts as multiplies -- measured on GB300 (exafel-like field): decompression
// 21.8 -> 21.3 us, whose integer/logic pipe is its bound; the encode kernel, bound by
// instruction issue, 27.1 -> 27.7 us, so it keeps the shifts.
template <bool kMul, int J, uint32_t M>
__device__ __forceinline__ void swap_stage(uint32_t (&a)[32])
{
#pragma unroll
    for (int r = 0; r < 32; ++r) {
        if (r & J) continue;
        const uint32_t lo = a[r], hi = a[r + J];
        const uint32_t hs = kMul ? shl_mul<J>(hi) : hi << J;
        const uint32_t ls = kMul ? shr_mul<J>(lo) : lo >> J;
        a[r]     = (lo & M) | (hs & ~M);
        a[r + J] = (hi & ~M) | (ls & M);
    }
}

// 32x32 bit-matrix transpose in registers: bit c of a[r] becomes bit r of a[c].
// Recursive off-diagonal block swap; the 16- and 8-bit stages are byte permutes.
template <bool kMul = false>
__device__ __forceinline__ void transpose32(uint32_t (&a)[32])
{
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        uint32_t lo = a[r], hi = a[r + 16];
        a[r]        = __byte_perm(lo, hi, 0x5410);
        a[r + 16]   = __byte_perm(lo, hi, 0x7632);
    }
#pragma unroll
    for (int r = 0; r < 32; ++r) {
        if (r & 8) continue;
        uint32_t lo = a[r], hi = a[r + 8];
        a[r]        = __byte_perm(lo, hi, 0x6240);
        a[r + 8]    = __byte_perm(lo, hi, 0x7351);
    }
    swap_stage<kMul, 4, 0x0F0F0F0Fu>(a);
    swap_stage<kMul, 2, 0x33333333u>(a);
    swap_stage<kMul, 1, 0x55555555u>(a);
}

// ------------------------------------------------------ scan tile state --
// One u64 per tile: [epoch:32][flag:2][ovf:1][value:29].  flag 1 = aggregate (this
// tile only), 2 = inclusive prefix.  A word from another epoch reads as "not ready", so
// the array needs no clearing between calls.  The epoch lives in device memory and is
// advanced by each scanning kernel's last ticket fetch, so a kernel replayed from a
// CUDA graph with frozen parameters still scans in a fresh epoch.  Values (chunk
// counts) stay below 2^29 because a field holds at most 2^31 elements.
constexpr uint64_t kFlagAgg  = 1;
constexpr uint64_t kFlagIncl = 2;

__device__ __forceinline__ uint64_t state_pack(uint32_t epoch, uint64_t flag, uint32_t ovf,
                                               uint32_t value)
{
    return ((uint64_t)epoch << 32) | (flag << 30) | ((uint64_t)(ovf & 1u) << 29) | (value & 0x1FFFFFFFu);
}
__device__ __forceinline__ uint32_t state_flag(uint64_t s) { return (uint32_t)(s >> 30) & 3u; }
__device__ __forceinline__ uint32_t state_ovf(uint64_t s) { return (uint32_t)(s >> 29) & 1u; }
__device__ __forceinline__ uint32_t state_value(uint64_t s) { return (uint32_t)s & 0x1FFFFFFFu; }
// The value and its flag share one 64-bit word, so relaxed GPU-scope accesses suffice:
// no other memory is published through it.
__device__ __forceinline__ void st_state(uint64_t* p, uint64_t v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_state(const uint64_t* p)
{
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

constexpr uint32_t kSpinLimit = 1u << 22;  // polls before a wait gives up (~0.3 s)

// Warp-cooperative decoupled look-back (single pass, Merrill & Garland 2016).
// Tile `t` has published its aggregate already (unless t == 0).  Each round the warp
// inspects a window of 32 W predecessors -- lane l loads tiles t-1-Wl .. t-W-Wl -- and
// proceeds as soon as every tile nearer than the first inclusive prefix in the window
// has published (tiles beyond it may still be running).  Returns the exclusive prefix
// (value) and the OR of the predecessors' ovf bits in every lane.  A wait longer than
// kSpinLimit polls raises kStatusTimeout and counts the missing tiles as 0, so no warp
// ever waits forever.
template <int W = 4>
__device__ __forceinline__ void lookback(const uint64_t* state, uint32_t t, uint32_t epoch,
                                         uint32_t* status, uint32_t& excl, uint32_t& ovf)
{
    static_assert(W >= 1 && W <= 32, "window per lane");
    constexpr uint32_t kAllW = W == 32 ? 0xFFFFFFFFu : (1u << W) - 1u;
    const uint32_t     lane  = threadIdx.x & 31;
    uint32_t           acc = 0, acc_ovf = 0;
    int64_t            base  = (int64_t)t - 1 - W * (int64_t)lane;
    uint32_t           spins = 0;
    while (true) {
        uint64_t s[W];
        uint32_t rdy, inc;  // bit j: tile base-j has published / holds an inclusive prefix
        int      first;     // first lane holding an inclusive prefix (32: none)
        bool     gave_up = false;
        while (true) {
            rdy = 0, inc = 0;
#pragma unroll
            for (int j = 0; j < W; ++j) {
                const int64_t pos = base - j;
                s[j]         = pos >= 0 ? ld_state(state + pos) : state_pack(epoch, kFlagIncl, 0, 0);
                const bool r = (uint32_t)(s[j] >> 32) == epoch && state_flag(s[j]) != 0;
                rdy |= r ? (1u << j) : 0u;
                inc |= (r && state_flag(s[j]) == kFlagIncl) ? (1u << j) : 0u;
            }
            const uint32_t any = __ballot_sync(kFull, inc != 0);
            first              = any ? __ffs(any) - 1 : 32;
            // the tiles before the first inclusive prefix must all have published
            const uint32_t need = (int)lane < first ? kAllW : ((int)lane == first ? (inc & (0u - inc)) - 1u : 0u);
            if (__all_sync(kFull, (rdy & need) == need)) break;
            if (++spins > kSpinLimit) {
                gave_up = true;
                break;
            }
            if (spins > 64) __nanosleep(64);
        }
        if (gave_up) {
            if (lane == 0) atomicOr(status, kStatusTimeout);
            // not-ready tiles end the walk as an inclusive 0
#pragma unroll
            for (int j = 0; j < W; ++j)
                if (!((rdy >> j) & 1u)) s[j] = state_pack(epoch, kFlagIncl, 0, 0), inc |= 1u << j;
            const uint32_t any = __ballot_sync(kFull, inc != 0);
            first              = any ? __ffs(any) - 1 : 32;
        }
        // lanes before the first lane holding a prefix take all W tiles; that lane takes
        // its tiles up to its first prefix; later lanes take none
        const int jmax = (int)lane < first ? W - 1 : ((int)lane == first ? __ffs(inc) - 1 : -1);
        uint32_t  v = 0, o = 0;
#pragma unroll
        for (int j = 0; j < W; ++j)
            if (j <= jmax) v += state_value(s[j]), o |= state_ovf(s[j]);
        acc += __reduce_add_sync(kFull, v);
        acc_ovf |= __reduce_or_sync(kFull, o);
        if (first < 32) break;
        base -= 32 * W;
    }
    excl = acc;
    ovf  = acc_ovf;
}

// Publish helpers (lane 0 only).
__device__ __forceinline__ void publish(uint64_t* state, uint32_t t, uint32_t epoch,
                                        uint64_t flag, uint32_t ovf, uint32_t value)
{
    st_state(state + t, state_pack(epoch, flag, ovf, value));
}

// Ticket fetch of a scanning kernel: tiles are handed out in launch order (so every
// predecessor of a tile has started and the look-back makes progress).  The last of the
// `fetches` fetches of the launch resets the counter and advances the device epoch for
// the next launch; every CTA reads the epoch before its first fetch.
struct Ticket {
    uint32_t tile;
    bool     last;
};
__device__ __forceinline__ Ticket take_ticket(uint32_t* ticket, uint32_t* epoch_word, uint32_t fetches)
{
    Ticket         t;
    const uint32_t c = atomicAdd(ticket, 1u);
    t.tile           = c;
    t.last           = (c == fetches - 1);
    if (t.last) {
        atomicExch(ticket, 0u);
        atomicAdd(epoch_word, 1u);
    }
    return t;
}

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace fz
