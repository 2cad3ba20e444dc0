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
// round(x * ebx2_r) in float, ties away from zero (lorenzo_var.cuh:81,125,265).
__device__ __forceinline__ float pq(float v, float r) { return roundf(__fmul_rn(v, r)); }

// (u16)fabs(d) | (d < 0) << 15 -- the expression of lorenzo_var.cuh:169-171.
__device__ __forceinline__ uint32_t pack_signed(float d)
{
    uint16_t tmp = static_cast<uint16_t>(fabsf(d));
    tmp |= ((d < 0) << 15);
    return tmp;
}
// 1D positions i%4 != 0 store the magnitude only (lorenzo_var.cuh:62).
__device__ __forceinline__ uint32_t pack_unsigned(float d)
{
    return static_cast<uint16_t>(fabsf(d));
}

// ------------------------------------------------------------- transpose --
// 32x32 bit-matrix transpose in registers: bit c of a[r] becomes bit r of a[c].
// Recursive off-diagonal block swap; the 16- and 8-bit stages are byte permutes.
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
#define FZ_SWAP_STAGE(J, M)                                        \
    _Pragma("unroll") for (int r = 0; r < 32; ++r)                 \
    {                                                              \
        if (r & (J)) continue;                                     \
        uint32_t lo = a[r], hi = a[r + (J)];                       \
        a[r]        = (lo & (M)) | ((hi << (J)) & ~(M));           \
        a[r + (J)]  = (hi & ~(M)) | ((lo >> (J)) & (M));           \
    }
    FZ_SWAP_STAGE(4, 0x0F0F0F0Fu)
    FZ_SWAP_STAGE(2, 0x33333333u)
    FZ_SWAP_STAGE(1, 0x55555555u)
#undef FZ_SWAP_STAGE
}

// ------------------------------------------------------ scan tile state --
// One u64 per tile: [epoch:28][flag:2][ovf:1][0:1][value:32].  flag 1 = aggregate
// (this tile only), 2 = inclusive prefix.  A word from another epoch reads as "not
// ready", so the array needs no clearing between calls.
constexpr uint64_t kFlagAgg  = 1;
constexpr uint64_t kFlagIncl = 2;

__device__ __forceinline__ uint64_t state_pack(uint32_t epoch, uint64_t flag, uint32_t ovf,
                                               uint32_t value)
{
    return ((uint64_t)epoch << 36) | (flag << 34) | ((uint64_t)(ovf & 1u) << 32) | value;
}
__device__ __forceinline__ void st_release(uint64_t* p, uint64_t v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire(const uint64_t* p)
{
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

constexpr uint32_t kSpinLimit = 1u << 22;  // polls before a wait gives up (~0.3 s)

// Warp-cooperative decoupled look-back (single pass, Merrill & Garland 2016).
// Tile `t` has published its aggregate already (unless t == 0).  Lane l inspects tile
// t-1-l-32k.  Returns the exclusive prefix (value) and OR of the ovf bits of all
// predecessors; every lane gets the result.  On a wait that exceeds kSpinLimit polls
// the status word gets kStatusTimeout and the missing tiles count as 0, so no warp
// ever waits forever.
__device__ __forceinline__ void lookback(const uint64_t* state, uint32_t t, uint32_t epoch,
                                         uint32_t* status, uint32_t& excl, uint32_t& ovf)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t       acc = 0, acc_ovf = 0;
    int64_t        pos   = (int64_t)t - 1 - lane;
    uint32_t       spins = 0;
    bool           gave_up = false;
    while (true) {
        uint64_t s;
        bool     ready;
        while (true) {
            s     = pos >= 0 ? ld_acquire(state + pos) : state_pack(epoch, kFlagIncl, 0, 0);
            ready = (uint32_t)(s >> 36) == epoch && ((s >> 34) & 3u) != 0;
            if (__all_sync(kFull, ready)) break;
            if (++spins > kSpinLimit) {
                gave_up = true;
                break;
            }
            if (spins > 64) __nanosleep(64);
        }
        if (gave_up) {
            if (lane == 0) atomicOr(status, kStatusTimeout);
            // not-ready tiles count as an inclusive 0 so the chain terminates here
            if (!ready) s = state_pack(epoch, kFlagIncl, 0, 0);
        }
        const uint32_t flag  = (uint32_t)(s >> 34) & 3u;
        const uint32_t incl  = __ballot_sync(kFull, flag == kFlagIncl);
        const uint32_t val   = (uint32_t)s;
        const uint32_t ovbit = (uint32_t)(s >> 32) & 1u;
        if (incl) {
            const uint32_t k = __ffs(incl) - 1;  // nearest predecessor holding a prefix
            acc += __reduce_add_sync(kFull, lane <= k ? val : 0u);
            acc_ovf |= __reduce_or_sync(kFull, lane <= k ? ovbit : 0u);
            break;
        }
        acc += __reduce_add_sync(kFull, val);
        acc_ovf |= __reduce_or_sync(kFull, ovbit);
        pos -= 32;
    }
    excl = acc;
    ovf  = acc_ovf;
}

// Publish helpers (lane 0 only).
__device__ __forceinline__ void publish(uint64_t* state, uint32_t t, uint32_t epoch,
                                        uint64_t flag, uint32_t ovf, uint32_t value)
{
    st_release(state + t, state_pack(epoch, flag, ovf, value));
}

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace fz
