// fz_decompress.cu -- decompression kernels (the inverse of fz_compress.cu).
//
//   k_decompress1d/2d/3d  fused decode + inverse bitshuffle + inverse Lorenzo, from the
//              stream straight into the field: each CTA decodes the 64-code groups its
//              rows (or 256-element blocks) need -- rank of every flagged chunk from the
//              bitmap and the block offset table, inverse 32x32 bit transposes -- then
//              runs the per-tile inclusive prefix sums in 32-bit integers (1D 256, 2D
//              16x16, 3D 8x8x8 -- the tiling of x_lorenzo_{1d,2d,3d},
//              lorenzo_var.cuh:297-518) and writes (float)p * ebx2.
//   k_offsets  block offset table from the bitmap (COMPAT streams, which carry none).
//   k_recon{1,2,3}d  inverse Lorenzo of a code array (the stage-level API,
//              fz_lorenzo_reconstruct).
//
// The reference has no working FZ decompressor (its x_lorenzo kernels read a separate
// signum array that its compressor never writes), so this path is the exact inverse of
// the compressed format rather than a restatement.
#include <algorithm>
#include <atomic>

#include "fz_internal.h"

namespace fz {

// ------------------------------------------------------------- offsets --
// boff[b] = chunks of blocks 0..b-1 (the exclusive scan fz.cu:187-192 restricted to
// block granularity), boff[nb] = the total, checked against the header's nnz.  One
// thread per block (two 16-byte bitmap loads), CTAs of 256 chained by look-back.
constexpr uint32_t kOffThreads = 256;

__global__ void __launch_bounds__(kOffThreads) k_offsets(const uint8_t* __restrict__ st, uint64_t off_a,
                                                        uint32_t nb, uint64_t nnz, uint32_t* boff,
                                                        uint64_t* state, uint32_t* ticket,
                                                        uint32_t* status, uint32_t* epoch_word)
{
    __shared__ uint32_t s_w[kOffThreads / 32];
    __shared__ uint32_t cta_tile, s_excl, s_epoch;
    if (threadIdx.x == 0) {
        s_epoch = __ldcg(epoch_word);
        __threadfence();
        cta_tile = take_ticket(ticket, epoch_word, gridDim.x).tile;
    }
    __syncthreads();
    const uint32_t ct = cta_tile, lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t epoch = s_epoch;
    const uint32_t b  = ct * kOffThreads + threadIdx.x;
    uint32_t       c  = 0;
    if (b < nb) {
        const uint4* A = reinterpret_cast<const uint4*>(st + off_a) + 2 * (size_t)b;
        const uint4  u = __ldg(A), v = __ldg(A + 1);
        c = __popc(u.x) + __popc(u.y) + __popc(u.z) + __popc(u.w) + __popc(v.x) + __popc(v.y) +
            __popc(v.z) + __popc(v.w);
    }
    uint32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(kFull, inc, o);
        if (lane >= (uint32_t)o) inc += u;
    }
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const uint32_t v = lane < kOffThreads / 32 ? s_w[lane] : 0u;
        uint32_t       vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(kFull, vi, o);
            if (lane >= (uint32_t)o) vi += u;
        }
        if (lane < kOffThreads / 32) s_w[lane] = vi - v;  // exclusive warp offsets
        const uint32_t tot  = __shfl_sync(kFull, vi, 31);
        uint32_t       excl = 0, povf = 0;
        if (ct == 0) {
            if (lane == 0) publish(state, 0, epoch, kFlagIncl, 0, tot);
        } else {
            if (lane == 0) publish(state, ct, epoch, kFlagAgg, 0, tot);
            lookback(state, ct, epoch, status, excl, povf);
            if (lane == 0) publish(state, ct, epoch, kFlagIncl, 0, excl + tot);
        }
        if (lane == 0) {
            s_excl = excl;
            if (ct == gridDim.x - 1) {
                boff[nb] = excl + tot;
                if (excl + tot != nnz) atomicOr(status, kStatusCorrupt);
            }
        }
    }
    __syncthreads();
    if (b < nb) boff[b] = s_excl + s_w[wid] + inc - c;
}

cudaError_t launch_offsets(const uint8_t* st, uint64_t off_a, uint32_t nb, uint32_t nwords, uint64_t nnz,
                           uint32_t* boff, uint64_t* state, uint32_t* ticket, uint32_t* status,
                           uint32_t* epoch, cudaStream_t s)
{
    (void)nwords;
    const uint32_t ctas = (uint32_t)std::max<uint64_t>(1, cdiv(nb, kOffThreads));
    k_offsets<<<ctas, kOffThreads, 0, s>>>(st, off_a, nb, nnz, boff, state, ticket, status, epoch);
    return cudaGetLastError();
}

// Gathers the shuffled image S of block t (words 4c..4c+3 of chunk c = lane + 32 i) into
// shared memory; flagged chunks come from Section B in order, the others are zero.
__device__ __forceinline__ void gather_block(const DecodeArgs& a, uint32_t t, uint32_t lane, uint32_t* sm)
{
    const uint4*   A4 = reinterpret_cast<const uint4*>(a.st + a.off_a) + 2 * (size_t)t;
    const uint4    b0 = __ldg(A4), b1 = __ldg(A4 + 1);
    const uint32_t bm[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
    const uint4*   B   = reinterpret_cast<const uint4*>(a.st + a.off_b);
    const uint32_t lt  = lanemask_lt();
    uint32_t       pre = __ldg(a.boff + t);
    const uint32_t end = __ldg(a.boff + t + 1);
    bool           bad = false;
#pragma unroll
    for (uint32_t i = 0; i < 8; ++i) {
        uint4          v    = make_uint4(0, 0, 0, 0);
        const uint32_t rank = pre + __popc(bm[i] & lt);
        if ((bm[i] >> lane) & 1u) {
            if (rank < a.nnz) v = __ldg(B + rank);
            else bad = true;  // the bitmap claims more chunks than the stream holds
        }
        *reinterpret_cast<uint4*>(sm + (lane + 32 * i) * 4) = v;
        pre += __popc(bm[i]);
    }
    bad |= pre != end;  // bitmap and offset table disagree
    if (bad) atomicOr(a.status, kStatusCorrupt);
}

__device__ __forceinline__ uint32_t sm_decode(uint32_t c)
{
    const uint32_t mag = c & 0x7FFFu;
    return (c & 0x8000u) ? 0u - mag : mag;
}

// Both sign-magnitude codes of a word w = c0 | c1 << 16 as two's-complement deltas: the
// sign bit 15 (31) spread into an all-ones mask m, (mag ^ m) - m is -mag exactly when the
// sign is set -- sm_decode for both halves.
__device__ __forceinline__ void sm_decode2(uint32_t w, uint32_t& d0, uint32_t& d1)
{
    // m0, m1: byte permutes whose selectors replicate the sign bit of byte 1 (bit 15) and of
    // byte 3 (bit 31) into every byte (prmt's default mode, selector nibble 8 + byte)
    uint32_t m0, m1;
    asm("prmt.b32 %0, %1, 0, 0x9999;" : "=r"(m0) : "r"(w));
    asm("prmt.b32 %0, %1, 0, 0xBBBB;" : "=r"(m1) : "r"(w));
    d0 = ((w & 0x7FFFu) ^ m0) - m0;
    d1 = ((__byte_perm(w, 0u, 0x4432) & 0x7FFFu) ^ m1) - m1;
}

// Decodes the 64 codes of group g (codes g*64 .. g*64+63) into 32 words w[j] =
// code[2j] | code[2j+1] << 16.  Group gg of block b is word r4 = gg % 4 of the 32
// chunks (p, k = gg / 4): its rank among the flagged chunks follows from the block's
// bitmap and its offset boff[b].  Groups past the last full block read the sidecar.
__device__ __forceinline__ void decode_group(const DecodeArgs& a, uint32_t g, uint32_t (&w)[32])
{
    const uint32_t b = g >> 5;
    if (b < a.nb) {
        const uint32_t gg = g & 31u, k = gg >> 2, r4 = gg & 3u;
        const uint4*   A4 = reinterpret_cast<const uint4*>(a.st + a.off_a) + 2 * (size_t)b;
        const uint4    b0 = __ldg(A4), b1 = __ldg(A4 + 1);
        const uint32_t bm[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
        const uint32_t base  = __ldg(a.boff + b);
        const uint32_t* W4   = reinterpret_cast<const uint32_t*>(a.st + a.off_b) + r4;
        // chunk c = 8p + k sits in bitmap word p/4 at bit 8(p%4) + k
        uint32_t lowm[4], bit[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            bit[q]  = 1u << (8 * q + k);
            lowm[q] = bit[q] - 1u;
        }
        uint32_t       pw  = base;
        const uint32_t end = __ldg(a.boff + b + 1);
        // the table agrees with the bitmap and the block's chunks lie inside the stream:
        // then every rank below is < nnz; otherwise nothing is read
        const bool bad = end - base != (uint32_t)(__popc(b0.x) + __popc(b0.y) + __popc(b0.z) + __popc(b0.w) +
                                                  __popc(b1.x) + __popc(b1.y) + __popc(b1.z) + __popc(b1.w)) ||
                         end < base || end > a.nnz;
        const uint32_t live = bad ? 0u : kFull;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const uint32_t bmi = bm[i] & live;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int      p    = 4 * i + q;
                const uint32_t rank = pw + __popc(bmi & lowm[q]);
                w[p]                = (bmi & bit[q]) ? __ldg(W4 + 4 * (size_t)rank) : 0u;
            }
            pw += __popc(bmi);
        }
        if (bad) atomicOr(a.status, kStatusCorrupt);
        transpose32<true>(w);  // w[p] = S[p*32 + gg]  ->  w[j] = W[gg*32 + j]
    } else {
        const uint16_t* tc  = a.mode == 1 ? reinterpret_cast<const uint16_t*>(a.st + a.off_c) : nullptr;
        const uint32_t  e0  = g * 64;
        const uint32_t  tb  = a.nb * kBlockCodes;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const uint32_t e  = e0 + 2 * j;
            const uint32_t lo = (tc && e < a.n) ? tc[e - tb] : 0u;
            const uint32_t hi = (tc && e + 1 < a.n) ? tc[e + 1 - tb] : 0u;
            w[j] = lo | (hi << 16);
        }
    }
}

// Decoded row buffers (fused 2D/3D paths): a row of the field's window is held as 64-code
// slots (one decode group each) of eight 16-byte chunks, in one of two layouts:
//   padded (2D): code e at word (e / 64) * kSlotWords + (e % 64) / 2.  The 16-byte pad
//     per slot puts neighbouring slots 4 banks apart, so the 16-byte stores of 8 threads
//     writing chunk tt of consecutive groups hit distinct banks, and a read address is a
//     shift, a mask and a multiply-add.
//   swizzled (3D, whose kernel runs at its register limit): 32 words per slot, chunk c of
//     slot G at chunk position c ^ (G & 7).
constexpr uint32_t kSlotWords = 36;

// word of chunk c of slot G
template <bool kPad>
__device__ __forceinline__ uint32_t rb_chunk(uint32_t G, uint32_t c)
{
    return kPad ? G * kSlotWords + 4 * c : (G * 8 + (c ^ (G & 7u))) << 2;
}
// word holding code e
template <bool kPad>
__device__ __forceinline__ uint32_t rb_word(uint32_t e)
{
    return kPad ? (e >> 6) * kSlotWords + ((e & 63u) >> 1) : rb_chunk<false>(e >> 6, (e >> 3) & 7u) + ((e >> 1) & 3u);
}

template <bool kPad>
__device__ __forceinline__ void rb_put_group(uint32_t* rb, uint32_t j, const uint32_t (&w)[32])
{
#pragma unroll
    for (uint32_t tt = 0; tt < 8; ++tt)
        *reinterpret_cast<uint4*>(rb + rb_chunk<kPad>(j, tt)) =
            make_uint4(w[4 * tt], w[4 * tt + 1], w[4 * tt + 2], w[4 * tt + 3]);
}

// Integer deltas of codes i..i+3 of a row buffer.  i % 4 is the same for every thread of
// a row, so the branch is uniform.
template <bool kPad>
__device__ __forceinline__ void rb_read4(const uint32_t* rb, uint32_t i, uint32_t (&d)[4])
{
    if ((i & 3u) == 0) {
        const uint2 v = *reinterpret_cast<const uint2*>(rb + rb_word<kPad>(i));
        sm_decode2(v.x, d[0], d[1]);
        sm_decode2(v.y, d[2], d[3]);
    } else {
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) {
            const uint32_t e  = i + k;
            const uint32_t wv = rb[rb_word<kPad>(e)];
            d[k]              = sm_decode((e & 1u) ? wv >> 16 : wv & 0xFFFFu);
        }
    }
}

// Stores min(live, 4) reconstructed values at element lin (16-byte store when aligned).
__device__ __forceinline__ void store4(float* out, uint32_t lin, uint32_t live, const uint32_t (&acc)[4], float ebx2)
{
    const float f0 = (float)(int32_t)acc[0] * ebx2, f1 = (float)(int32_t)acc[1] * ebx2;
    const float f2 = (float)(int32_t)acc[2] * ebx2, f3 = (float)(int32_t)acc[3] * ebx2;
    if (live >= 4 && (lin & 3u) == 0) {
        *reinterpret_cast<float4*>(out + lin) = make_float4(f0, f1, f2, f3);
    } else {
        out[lin] = f0;
        if (live > 1) out[lin + 1] = f1;
        if (live > 2) out[lin + 2] = f2;
        if (live > 3) out[lin + 3] = f3;
    }
}

// ------------------------------------------------------ fused 2D decode --
// A CTA owns a 16-row tile band and a 960-column window (60 tile columns); the flat
// block index runs over windows fastest.  Phase 1: thread (row rr, j) decodes group
// glo(rr) + j of that row's span into the row buffer.  Phase 2: thread t owns columns
// 4t..4t+3; prefix along x (serial + quad shuffles), running sum along y, (float)p *
// ebx2, coalesced stores.  Traffic: the chunks once (plus the at most two groups a row
// shares with the next window) and the output once.
constexpr uint32_t kW2 = 960;

// kAl: x % 4 == 0.  Windows start at multiples of 960 columns, so every row's window then
// starts on a 4-code boundary: a thread's 4 codes are one 8-byte pair of row-buffer words,
// its 4 outputs one 16-byte store (c1 - c0 is a multiple of 4, so a live thread has all
// 4 columns), and nothing about alignment or width is decided per row.
template <bool kAl>
__global__ void __launch_bounds__(256, 5) k_decompress2d(const DecodeArgs a, uint32_t nwin)
{
    pdl_wait();
    pdl_trigger();
    __shared__ __align__(16) uint32_t rows[16][16 * kSlotWords];  // 16 rows x 16 slots of 64 codes
    const uint32_t tid = threadIdx.x;
    const uint32_t bx = blockIdx.x % nwin, by = blockIdx.x / nwin;
    const uint32_t c0 = bx * kW2, c1 = min(c0 + kW2, a.x);
    const uint32_t r0 = by * 16;
    {
        const uint32_t rr = tid >> 4, j = tid & 15u, row = r0 + rr;
        if (row < a.y) {
            const uint32_t lin0 = row * a.x + c0, lin1 = row * a.x + c1;
            const uint32_t g = (lin0 >> 6) + j;
            if (g <= ((lin1 - 1) >> 6)) {
                uint32_t w[32];
                decode_group(a, g, w);
                rb_put_group<true>(rows[rr], j, w);
            }
        }
    }
    __syncthreads();
    const uint32_t col  = c0 + 4 * tid;
    const bool     live = col < c1;
    const uint32_t q    = tid & 3u;
    uint32_t       acc[4] = {0, 0, 0, 0};
    if (kAl) {
        const uint32_t nrows = min(16u, a.y - r0);
        uint32_t       lin0  = r0 * a.x + c0;  // first code of the window in row r0 + rr
        // threads past the window's end read the row's first word (in bounds; their values
        // only reach higher quad positions, which are past the end too, and are not stored)
        const uint32_t t4 = live ? 4 * tid : 0u;
#pragma unroll 4
        for (uint32_t rr = 0; rr < 16; ++rr) {
            if (rr >= nrows) break;  // uniform across the CTA
            uint32_t d[4];
            {
                // code i of the row at word 36 (i >> 6) + (i & 63) / 2 = i / 2 + 4 (i >> 6)
                const uint32_t i = (lin0 & 63u) + t4;
                const uint2    v = *reinterpret_cast<const uint2*>(rows[rr] + (i >> 1) + 4 * (i >> 6));
                sm_decode2(v.x, d[0], d[1]);
                sm_decode2(v.y, d[2], d[3]);
            }
            d[1] += d[0], d[2] += d[1], d[3] += d[2];
            uint32_t v = d[3];
            uint32_t u = __shfl_up_sync(kFull, v, 1);
            if (q >= 1) v += u;
            u = __shfl_up_sync(kFull, v, 2);
            if (q >= 2) v += u;
            const uint32_t ex = v - d[3];
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[j] += d[j] + ex;
            if (live)
                *reinterpret_cast<float4*>(a.out + lin0 + 4 * tid) =
                    make_float4((float)(int32_t)acc[0] * a.ebx2, (float)(int32_t)acc[1] * a.ebx2,
                                (float)(int32_t)acc[2] * a.ebx2, (float)(int32_t)acc[3] * a.ebx2);
            lin0 += a.x;
        }
        return;
    }
#pragma unroll 4
    for (uint32_t rr = 0; rr < 16; ++rr) {
        const uint32_t row = r0 + rr;
        if (row >= a.y) break;  // uniform across the CTA
        const uint32_t lin0 = row * a.x + c0;
        uint32_t       d[4];
        // threads past the window's end read the row's first codes (same alignment, in bounds,
        // never stored; their values reach only higher quad positions, past the end too)
        rb_read4<true>(rows[rr], (lin0 & 63u) + (live ? 4 * tid : 0u), d);
        d[1] += d[0], d[2] += d[1], d[3] += d[2];
        uint32_t v = d[3];
        uint32_t u = __shfl_up_sync(kFull, v, 1);
        if (q >= 1) v += u;
        u = __shfl_up_sync(kFull, v, 2);
        if (q >= 2) v += u;
        const uint32_t ex = v - d[3];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] += d[j] + ex;
        if (live) store4(a.out, lin0 + 4 * tid, c1 - col, acc, a.ebx2);
    }
}

// ------------------------------------------- fused 2D decode, x % 16 == 0 --
// Rows a multiple of 16 elements long: every 16-column tile row lies inside one 64-code
// group (group and tile boundaries are both multiples of 16 in the linear index), so
// phase 1 does the whole x direction.  Thread (row rr, j) decodes group glo(rr) + j, and for
// each of its four tiles inside the window decodes the 16 codes, prefix-sums them serially
// and writes the 16 partial sums as 32-bit words into the window's row (chunk c of 4 words
// at c ^ ((c >> 4) & 7): the lanes' stores, 64 words apart, and phase 2's loads spread over
// all banks).  Phase 2: thread t owns columns 4t..4t+3 -- a running sum over the band's
// rows, (float)p * ebx2, coalesced stores; no shuffles, so threads past the window leave.
constexpr uint32_t kW16 = 960;
constexpr uint32_t kX16Smem = 16 * kW16 * 4;  // 16 rows x 960 partial sums

__device__ __forceinline__ uint32_t x16_chunk(uint32_t c) { return c ^ ((c >> 4) & 7u); }

__global__ void __launch_bounds__(256, 3) k_decompress2d_x16(const DecodeArgs a, uint32_t nwin)
{
    pdl_wait();
    pdl_trigger();
    extern __shared__ __align__(16) uint32_t xs[];  // [16][kW16] partial sums along x
    const uint32_t tid = threadIdx.x;
    const uint32_t bx = blockIdx.x % nwin, by = blockIdx.x / nwin;
    const uint32_t c0 = bx * kW16, c1 = min(c0 + kW16, a.x);
    const uint32_t r0 = by * 16;
    {
        const uint32_t rr = tid >> 4, j = tid & 15u, row = r0 + rr;
        if (row < a.y) {
            const uint32_t lin0 = row * a.x + c0, lin1 = row * a.x + c1;
            const uint32_t g = (lin0 >> 6) + j;
            if (g <= ((lin1 - 1) >> 6)) {
                uint32_t w[32];
                decode_group(a, g, w);
                uint32_t* xr = xs + rr * kW16;
#pragma unroll
                for (uint32_t q = 0; q < 4; ++q) {
                    const uint32_t e = g * 64 + q * 16;  // the tile row's first code
                    if (e < lin0 || e >= lin1) continue;
                    uint32_t v[16], acc = 0;
#pragma unroll
                    for (uint32_t k = 0; k < 8; ++k) {
                        uint32_t d0, d1;
                        sm_decode2(w[8 * q + k], d0, d1);
                        acc += d0, v[2 * k] = acc;
                        acc += d1, v[2 * k + 1] = acc;
                    }
                    const uint32_t c = (e - lin0) >> 2;  // first chunk of the tile row in the window row
#pragma unroll
                    for (uint32_t s = 0; s < 4; ++s)
                        *reinterpret_cast<uint4*>(xr + 4 * x16_chunk(c + s)) =
                            make_uint4(v[4 * s], v[4 * s + 1], v[4 * s + 2], v[4 * s + 3]);
                }
            }
        }
    }
    __syncthreads();
    const uint32_t col = c0 + 4 * tid;
    if (col >= c1) return;  // phase 2 has no shuffles or barriers
    const uint32_t nrows = min(16u, a.y - r0);
    const uint32_t* xp   = xs + 4 * x16_chunk(tid);
    float*          out  = a.out + (size_t)r0 * a.x + col;
    uint32_t        acc[4] = {0, 0, 0, 0};
#pragma unroll 4
    for (uint32_t rr = 0; rr < 16; ++rr) {
        if (rr >= nrows) break;  // uniform across the CTA
        const uint4 p = *reinterpret_cast<const uint4*>(xp + rr * kW16);
        acc[0] += p.x, acc[1] += p.y, acc[2] += p.z, acc[3] += p.w;
        *reinterpret_cast<float4*>(out) = make_float4((float)(int32_t)acc[0] * a.ebx2, (float)(int32_t)acc[1] * a.ebx2,
                                                      (float)(int32_t)acc[2] * a.ebx2, (float)(int32_t)acc[3] * a.ebx2);
        out += a.x;
    }
}

// Resident CTAs of k_decompress2d_x16 on the current device (0 on error), cached per device;
// the first call also opts the kernel in to its dynamic shared memory (above 48 KB).
static uint32_t x16_wave()
{
    static std::atomic<uint32_t> cache[64];
    int                          dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::atomic<uint32_t>* slot = (dev >= 0 && dev < 64) ? &cache[dev] : nullptr;
    uint32_t               w    = slot ? slot->load(std::memory_order_acquire) : 0u;
    if (w) return w;
    int sms = 0, per_sm = 0;
    if (cudaFuncSetAttribute(k_decompress2d_x16, cudaFuncAttributeMaxDynamicSharedMemorySize, kX16Smem) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_decompress2d_x16, 256, kX16Smem) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    w = (uint32_t)std::max(0, sms * per_sm);
    if (slot && w) slot->store(w, std::memory_order_release);
    return w;
}

// ------------------------------------------------------ fused 3D decode --
// A CTA owns `bands` 8-row tile bands x one 8-plane tile slab x a window of w columns
// (w a multiple of 8, at most 960); the flat block index runs over windows, then band
// groups, then slabs.  The slab is walked two planes at a time.  Phase 1 decodes the
// pass's codes into row buffers: when the window spans whole rows (x <= 960) a plane's
// rows are one contiguous range of codes, decoded group by group into one buffer of pg
// slots ("span" mode, no group decoded twice inside the CTA); otherwise each of the
// bands x 8 rows of a plane gets its own buffer of g slots.  Phase 2: thread (band, cq)
// owns columns 4cq..4cq+3 of its band; prefix along x within the 8-column tile row (pair
// shuffle), running sum along y within the plane, running sum along z in shared memory
// (one 16-byte slot per thread and row: in registers they would spill), then the
// stores.
struct Brick3 {
    uint32_t w, q2, bands, g;  // window columns, column quads, bands per CTA, slots per row
    uint32_t nwin, nbgrp;      // windows along x, band groups along y
    uint32_t span, pg;         // span mode; slots per plane buffer
};
constexpr uint32_t kW3 = 960;

__global__ void __launch_bounds__(256, 4) k_decompress3d(const DecodeArgs a, const Brick3 k)
{
    pdl_wait();
    pdl_trigger();
    extern __shared__ __align__(16) uint32_t rb3[];
    const uint32_t tid = threadIdx.x;
    const uint32_t bx = blockIdx.x % k.nwin, rest = blockIdx.x / k.nwin;
    const uint32_t by = rest % k.nbgrp, bz = rest / k.nbgrp;
    const uint32_t c0 = bx * k.w, c1 = min(c0 + k.w, a.x);
    const uint32_t yb0 = by * k.bands, z0 = bz * 8;
    const uint32_t ys = yb0 * 8, ye = min(ys + 8 * k.bands, a.y);  // the CTA's rows
    const uint32_t band = tid / k.q2, cq = tid - band * k.q2;
    const uint32_t col = c0 + 4 * cq, ybase = ys + band * 8;
    const bool     bandlive = band < k.bands && ybase < a.y;
    // buffer words per plane (span) or per row
    const uint32_t rowwords = (k.span ? k.pg : k.g) * 32;
    const uint32_t ntask    = k.span ? 2 * k.pg : k.bands * 16 * k.g;
    // running sums along z, one 16-byte slot per thread and row of its band (after the row buffers)
    uint4* zs = reinterpret_cast<uint4*>(rb3 + (k.span ? 2 * k.pg : k.bands * 16 * k.g) * 32) + tid;
#pragma unroll
    for (int yy = 0; yy < 8; ++yy) zs[yy * 256] = make_uint4(0, 0, 0, 0);
    for (uint32_t pz = 0; pz < 8; pz += 2) {
        if (z0 + pz >= a.z) break;  // uniform across the CTA
        for (uint32_t task = tid; task < ntask; task += 256) {
            uint32_t r, j, lin0, lin1;
            if (k.span) {
                r = task / k.pg, j = task - r * k.pg;
                const uint32_t zz = z0 + pz + r;
                if (zz >= a.z) continue;
                lin0 = (zz * a.y + ys) * a.x, lin1 = (zz * a.y + ye) * a.x;
            } else {
                r = task / k.g, j = task - r * k.g;
                const uint32_t zz = z0 + pz + ((r >> 3) & 1u), yv = ys + (r >> 4) * 8 + (r & 7u);
                if (zz >= a.z || yv >= a.y) continue;
                lin0 = (zz * a.y + yv) * a.x + c0, lin1 = lin0 + (c1 - c0);
            }
            const uint32_t g = (lin0 >> 6) + j;
            if (g > ((lin1 - 1) >> 6)) continue;
            uint32_t w[32];
            decode_group(a, g, w);
            rb_put_group<false>(rb3 + r * rowwords, j, w);
        }
        __syncthreads();
        for (uint32_t p = 0; p < 2; ++p) {
            const uint32_t zz = z0 + pz + p;
            if (zz >= a.z) break;  // uniform across the CTA
            const uint32_t pbase = ((zz * a.y + ys) * a.x) & ~63u;  // span mode: first slot's code
            uint32_t       colacc[4] = {0, 0, 0, 0};
#pragma unroll
            for (uint32_t yy = 0; yy < 8; ++yy) {
                const uint32_t yv   = ybase + yy;
                const bool     live = bandlive && yv < a.y && col < c1;
                const uint32_t lin0 = (zz * a.y + yv) * a.x + c0;
                uint32_t       d[4] = {0, 0, 0, 0};
                if (live) {
                    if (k.span) rb_read4<false>(rb3 + p * rowwords, lin0 + 4 * cq - pbase, d);
                    else rb_read4<false>(rb3 + (band * 16 + p * 8 + yy) * rowwords, (lin0 & 63u) + 4 * cq, d);
                }
                d[1] += d[0], d[2] += d[1], d[3] += d[2];
                const uint32_t u  = __shfl_up_sync(kFull, d[3], 1);
                const uint32_t ex = (cq & 1u) ? u : 0u;
                const uint4    z4 = zs[yy * 256];
                uint32_t       zv[4] = {z4.x, z4.y, z4.z, z4.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    colacc[j] += d[j] + ex;
                    zv[j] += colacc[j];
                }
                zs[yy * 256] = make_uint4(zv[0], zv[1], zv[2], zv[3]);
                if (live) store4(a.out, lin0 + 4 * cq, c1 - col, zv, a.ebx2);
            }
        }
        __syncthreads();
    }
}

// Brick shape of the fused 3D path for a field of width x and height y.  Span mode
// (whole rows) takes as many bands as keep both the compute threads (bands x q2) and the
// pass's decode tasks (2 pg) within the CTA's 256 threads.
static Brick3 brick3(uint32_t x, uint32_t y)
{
    Brick3 k{};
    k.w  = std::min<uint32_t>(kW3, (x + 7) & ~7u);
    k.q2 = k.w / 4;
    k.g  = (k.w + 62) / 64 + 1;
    k.nwin = (uint32_t)cdiv(x, k.w);
    const uint32_t nbands = (uint32_t)cdiv(y, 8);
    k.span = k.nwin == 1;
    if (k.span) {
        k.bands = std::max(1u, std::min(256u / k.q2, nbands));
        for (;;) {
            // a plane's span is at most 8 bands x rows of x codes, starting anywhere in a group;
            // rows' last quads read up to 3 codes past it
            k.pg = (8 * k.bands * x + 66) / 64 + 1;
            if (k.bands == 1 || 2 * k.pg <= 256) break;
            --k.bands;
        }
    } else {
        k.bands = std::max(1u, std::min({8u, 256u / k.q2, nbands}));
        while (k.bands > 1 && k.bands * 16 * k.g * 128 > 48 * 1024) --k.bands;
    }
    k.nbgrp = (uint32_t)cdiv(nbands, k.bands);
    return k;
}

// Dynamic shared memory of a k_decompress3d CTA: the row buffers (span mode at most 2 x 122
// slots, otherwise at most 48 KB) and the z sums (8 rows x 256 threads x 16 bytes).
constexpr uint32_t kDecompress3dSmemMax = 48 * 1024 + 8 * 256 * 16;

static uint32_t brick3_smem(const Brick3& k)
{
    return (k.span ? 2 * k.pg * 128 : k.bands * 16 * k.g * 128) + 8 * 256 * 16;
}

// Above 48 KB a kernel's dynamic shared memory needs an opt-in, which is per device.
static cudaError_t allow_decompress3d_smem()
{
    static std::atomic<uint64_t> done{0};  // bit d: opted in on device d
    int         dev = 0;
    cudaError_t e   = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev < 64 ? 1ull << dev : 0ull;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(k_decompress3d, cudaFuncAttributeMaxDynamicSharedMemorySize, kDecompress3dSmemMax);
    if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
    return e;
}

// ------------------------------------------------------ fused 1D decode --
// One warp per shuffle block: lane g decodes its 64 codes (a quarter of one 256-element
// x_lorenzo block), prefix-sums them serially, adds the quad's carry, and writes 64
// floats through shared memory as coalesced 16-byte stores.  Codes at i%4 == 0 carry
// their sign; the others take it from the sidecar sign bits (or are non-negative).
constexpr int kDecode1dWarps = 4;

// Word of prefix value j of lane l in a warp's shared buffer: the lane's 64 values as sixteen
// 16-byte chunks, chunk c at position c ^ (l & 7), so that both the lanes' chunk stores here
// and the output loop's chunk loads (16 lanes on one owner's 16 chunks) spread over all 32
// banks.
__device__ __forceinline__ uint32_t run1d_word(uint32_t l, uint32_t j) { return 64 * l + 4 * ((j >> 2) ^ (l & 7u)); }

// Lane-local inclusive prefix of the lane's 64 deltas into shared memory, four values per
// 16-byte store; codes at i%4 == 0 carry their sign, the others take it from the sidecar
// words s0, s1.  kCheck: only the first lim deltas count (the run ends past x*y*z).
template <bool kCheck>
__device__ __forceinline__ uint32_t run1d(const uint32_t (&w)[32], uint32_t s0, uint32_t s1, uint32_t lim,
                                          uint32_t lane, uint32_t* sm)
{
    uint32_t acc = 0, q[4];
#pragma unroll
    for (int j = 0; j < 64; ++j) {
        const uint32_t c   = (j & 1) ? (w[j >> 1] >> 16) : (w[j >> 1] & 0xFFFFu);
        const uint32_t sgn = ((j < 32 ? s0 >> j : s1 >> (j - 32)) & 1u);
        const uint32_t d   = (j & 3) == 0 ? sm_decode(c) : (sgn ? 0u - c : c);
        acc += (!kCheck || (uint32_t)j < lim) ? d : 0u;
        q[j & 3] = acc;
        if ((j & 3) == 3) *reinterpret_cast<uint4*>(sm + run1d_word(lane, j)) = make_uint4(q[0], q[1], q[2], q[3]);
    }
    return acc;
}

__global__ void __launch_bounds__(kDecode1dWarps * 32) k_decompress1d(const DecodeArgs a)
{
    pdl_wait();
    pdl_trigger();
    __shared__ __align__(16) uint32_t smem[kDecode1dWarps][2048];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t t    = blockIdx.x * kDecode1dWarps + wid;
    const uint32_t ntiles = a.nb + (a.tail ? 1u : 0u);
    if (t >= ntiles) return;  // warp-uniform
    uint32_t* sm = smem[wid];
    uint32_t  w[32];
    if (t < a.nb) {
        gather_block(a, t, lane, sm);
        __syncwarp();
#pragma unroll
        for (uint32_t p = 0; p < 32; ++p) w[p] = sm[p * 32 + lane];
        transpose32<true>(w);
        __syncwarp();
    } else {
        decode_group(a, t * 32 + lane, w);  // tail: sidecar codes
    }
    const uint32_t  e0 = t * kBlockCodes + lane * 64;
    const uint32_t* sb = (a.mode == 1) ? reinterpret_cast<const uint32_t*>(a.st + a.off_sign) : nullptr;
    uint32_t        s0 = 0, s1 = 0;
    if (sb && e0 < a.n) {
        s0 = __ldg(sb + (e0 >> 5));
        s1 = (e0 + 32 < a.n) ? __ldg(sb + (e0 >> 5) + 1) : 0u;
    }
    // elements of this lane's run inside x*y*z (all 64 except in the last block)
    const uint32_t lim = a.nl > e0 ? a.nl - e0 : 0u;
    const uint32_t acc = lim >= 64 ? run1d<false>(w, s0, s1, lim, lane, sm) : run1d<true>(w, s0, s1, lim, lane, sm);
    // carry across the 4 lanes of each 256-element block
    uint32_t v = acc, u = __shfl_up_sync(kFull, v, 1);
    if (lane & 3u) v += u;
    u = __shfl_up_sync(kFull, v, 2);
    if ((lane & 3u) >= 2) v += u;
    const uint32_t ex = v - acc;
    __syncwarp();
    // write: pass i covers elements i*128 .. i*128+127 of the block; lane owns 4
    float* out = a.out + (size_t)t * kBlockCodes;
    for (uint32_t i = 0; i < 16; ++i) {
        const uint32_t el = i * 128 + lane * 4;   // element within the block
        const uint32_t ow = el >> 6, j0 = el & 63u;  // owning lane, index in its run
        const uint32_t exo = __shfl_sync(kFull, ex, ow);
        const uint4    pv  = *reinterpret_cast<const uint4*>(sm + run1d_word(ow, j0));  // j0 % 4 == 0
        const float    f[4] = {(float)(int32_t)(pv.x + exo) * a.ebx2, (float)(int32_t)(pv.y + exo) * a.ebx2,
                               (float)(int32_t)(pv.z + exo) * a.ebx2, (float)(int32_t)(pv.w + exo) * a.ebx2};
        const uint32_t e = t * kBlockCodes + el;
        if (e + 3 < a.nl) {
            *reinterpret_cast<float4*>(out + el) = make_float4(f[0], f[1], f[2], f[3]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (e + k < a.nl) out[el + k] = f[k];
        }
    }
}

cudaError_t launch_decompress_fused(const DecodeArgs& a, cudaStream_t s)
{
    const int nd = (a.z == 1 && a.y == 1) ? 1 : (a.z == 1 ? 2 : 3);
    if (nd == 2 && a.x % 16 == 0) {
        // the x-in-phase-1 kernel (3 CTAs/SM) when its grid is one resident wave: measured on
        // GB300, cesm-like 3600x1800 (452 CTAs) 14.0 -> 12.2 us a launch (in 8-branch graphs,
        // where it leaves less room to other branches' kernels, the same throughput);
        // exafel-like 39200x388 (1025 CTAs: 2.25 waves against 1.35 for k_decompress2d at 5
        // CTAs/SM) 20.4 us either way
        const uint32_t nwin = (uint32_t)cdiv(a.x, kW16);
        const uint32_t ctas = (uint32_t)(nwin * cdiv(a.y, 16));
        if (ctas <= x16_wave()) return launch_pdl(k_decompress2d_x16, dim3(ctas), dim3(256), kX16Smem, s, a, nwin);
    }
    if (nd == 2) {
        const uint32_t nwin = (uint32_t)cdiv(a.x, kW2);
        const uint32_t ctas = (uint32_t)(nwin * cdiv(a.y, 16));
        if (a.x % 4 == 0) return launch_pdl(k_decompress2d<true>, dim3(ctas), dim3(256), 0, s, a, nwin);
        return launch_pdl(k_decompress2d<false>, dim3(ctas), dim3(256), 0, s, a, nwin);
    }
    if (nd == 3) {
        const cudaError_t e = allow_decompress3d_smem();
        if (e != cudaSuccess) return e;
        const Brick3   k    = brick3(a.x, a.y);
        if (brick3_smem(k) > kDecompress3dSmemMax) return cudaErrorInvalidConfiguration;
        const uint64_t ctas = (uint64_t)k.nwin * k.nbgrp * cdiv(a.z, 8);
        return launch_pdl(k_decompress3d, dim3((uint32_t)ctas), dim3(256), brick3_smem(k), s, a, k);
    }
    const uint32_t ntiles = a.nb + (a.tail ? 1u : 0u);
    return launch_pdl(k_decompress1d, dim3((uint32_t)cdiv(ntiles, kDecode1dWarps)), dim3(kDecode1dWarps * 32), 0, s,
                      a);
}

// ------------------------------------------------------------- recon --
// 2D: a CTA covers 16 rows x 512 columns; lane owns 4 consecutive columns, lanes 4k..4k+3
// one 16-column tile row.  Row prefix: serial over 4 + quad shuffle scan; column prefix:
// running sum over the 16 rows.
__global__ void __launch_bounds__(128) k_recon2d(const ReconArgs a, uint32_t nwin)
{
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t c0   = (blockIdx.x % nwin) * 512 + wid * 128 + lane * 4;
    const uint32_t r0   = (blockIdx.x / nwin) * 16;
    const uint32_t q    = lane & 3u;
    const bool     vec  = (a.x % 4 == 0) && (c0 + 3 < a.x);
    uint32_t       acc[4] = {0, 0, 0, 0};
    for (uint32_t rr = 0; rr < 16; ++rr) {
        const uint32_t row = r0 + rr;
        if (row >= a.y) break;  // uniform across the CTA
        const size_t base = (size_t)row * a.x + c0;
        uint32_t     d[4] = {0, 0, 0, 0};
        if (vec) {
            const uint2 v = __ldg(reinterpret_cast<const uint2*>(a.codes + base));
            sm_decode2(v.x, d[0], d[1]);
            sm_decode2(v.y, d[2], d[3]);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (c0 + j < a.x) d[j] = sm_decode(a.codes[base + j]);
        }
        d[1] += d[0], d[2] += d[1], d[3] += d[2];
        uint32_t v = d[3];
        uint32_t u = __shfl_up_sync(kFull, v, 1);
        if (q >= 1) v += u;
        u = __shfl_up_sync(kFull, v, 2);
        if (q >= 2) v += u;
        const uint32_t ex = v - d[3];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] += d[j] + ex;
        if (vec) {
            *reinterpret_cast<float4*>(a.out + base) =
                make_float4((float)(int32_t)acc[0] * a.ebx2, (float)(int32_t)acc[1] * a.ebx2,
                            (float)(int32_t)acc[2] * a.ebx2, (float)(int32_t)acc[3] * a.ebx2);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (c0 + j < a.x) a.out[base + j] = (float)(int32_t)acc[j] * a.ebx2;
        }
    }
}

// 3D: a warp covers 128 columns of one 8x8 (y, z) tile column; lane owns 4 columns, lane
// pairs one 8-column tile row.  zacc[y] keeps the running z-sum of each of the 8 rows.
// The flat block index runs over x windows, then groups of 4 bands, then z slabs.
__global__ void __launch_bounds__(128) k_recon3d(const ReconArgs a, uint32_t nwin, uint32_t nyg)
{
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t rest = blockIdx.x / nwin;
    const uint32_t c0   = (blockIdx.x % nwin) * 128 + lane * 4;
    const uint32_t y0   = ((rest % nyg) * 4 + wid) * 8;
    const uint32_t z0   = (rest / nyg) * 8;
    if (y0 >= a.y) return;  // warp-uniform
    const bool     vec = (a.x % 4 == 0) && (c0 + 3 < a.x);
    const size_t   xy  = (size_t)a.x * a.y;
    uint32_t       zacc[8][4];
#pragma unroll
    for (int yy = 0; yy < 8; ++yy) zacc[yy][0] = zacc[yy][1] = zacc[yy][2] = zacc[yy][3] = 0;
    for (uint32_t zz = 0; zz < 8; ++zz) {
        if (z0 + zz >= a.z) break;
        uint32_t colacc[4] = {0, 0, 0, 0};
#pragma unroll
        for (uint32_t yy = 0; yy < 8; ++yy) {
            const bool   live = y0 + yy < a.y;
            const size_t base = (size_t)(z0 + zz) * xy + (size_t)(y0 + yy) * a.x + c0;
            uint32_t     d[4] = {0, 0, 0, 0};
            if (live) {
                if (vec) {
                    const uint2 v = __ldg(reinterpret_cast<const uint2*>(a.codes + base));
                    sm_decode2(v.x, d[0], d[1]);
                    sm_decode2(v.y, d[2], d[3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (c0 + j < a.x) d[j] = sm_decode(a.codes[base + j]);
                }
            }
            d[1] += d[0], d[2] += d[1], d[3] += d[2];
            const uint32_t u = __shfl_up_sync(kFull, d[3], 1);
            const uint32_t ex = (lane & 1u) ? u : 0u;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                colacc[j] += d[j] + ex;
                zacc[yy][j] += colacc[j];
            }
            if (!live) continue;
            if (vec) {
                *reinterpret_cast<float4*>(a.out + base) = make_float4(
                    (float)(int32_t)zacc[yy][0] * a.ebx2, (float)(int32_t)zacc[yy][1] * a.ebx2,
                    (float)(int32_t)zacc[yy][2] * a.ebx2, (float)(int32_t)zacc[yy][3] * a.ebx2);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (c0 + j < a.x) a.out[base + j] = (float)(int32_t)zacc[yy][j] * a.ebx2;
            }
        }
    }
}

// 1D: one warp per 256-element block; lane owns 8 consecutive elements.  Codes at
// i%4 == 0 carry their sign in bit 15; the others take it from the sidecar sign bits
// (or the stage API's signum bytes), and are non-negative without either.
__global__ void __launch_bounds__(256) k_recon1d(const ReconArgs a)
{
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t blk  = blockIdx.x * 8 + wid;
    const uint32_t e0   = blk * 256 + lane * 8;
    if (blk * 256 >= a.nl) return;  // warp-uniform
    uint32_t c[8];
    if (e0 + 7 < a.nl) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(a.codes + e0));
        c[0] = v.x & 0xFFFFu, c[1] = v.x >> 16, c[2] = v.y & 0xFFFFu, c[3] = v.y >> 16;
        c[4] = v.z & 0xFFFFu, c[5] = v.z >> 16, c[6] = v.w & 0xFFFFu, c[7] = v.w >> 16;
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) c[j] = e0 + j < a.nl ? a.codes[e0 + j] : 0u;
    }
    uint32_t sb = 0;  // sign bits of the 8 elements
    if (a.signbits) {
        sb = (__ldg(a.signbits + (e0 >> 5)) >> (e0 & 31u)) & 0xFFu;
    } else if (a.signum) {
#pragma unroll
        for (int j = 0; j < 8; ++j) sb |= (e0 + j < a.nl && a.signum[e0 + j]) ? (1u << j) : 0u;
    }
    uint32_t d[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if ((j & 3) == 0) {
            d[j] = sm_decode(c[j]);
        } else {
            d[j] = ((sb >> j) & 1u) ? 0u - c[j] : c[j];
        }
        if (j) d[j] += d[j - 1];
    }
    uint32_t v = d[7];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(kFull, v, o);
        if (lane >= (uint32_t)o) v += u;
    }
    const uint32_t ex = v - d[7];
    float          f[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) f[j] = (float)(int32_t)(d[j] + ex) * a.ebx2;
    if (e0 + 7 < a.nl) {
        float4* o = reinterpret_cast<float4*>(a.out + e0);
        o[0]      = make_float4(f[0], f[1], f[2], f[3]);
        o[1]      = make_float4(f[4], f[5], f[6], f[7]);
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (e0 + j < a.nl) a.out[e0 + j] = f[j];
    }
}

// elements past x*y*z (fz.cu:117-118 lets the file be longer than the dims) decode to 0
__global__ void k_zero_tail(float* out, uint32_t from, uint32_t n)
{
    for (uint32_t i = from + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = 0.0f;
}

cudaError_t launch_zero_tail(float* out, uint32_t from, uint32_t n, cudaStream_t s)
{
    k_zero_tail<<<(uint32_t)std::min<uint64_t>(cdiv(n - from, 256), 1024), 256, 0, s>>>(out, from, n);
    return cudaGetLastError();
}

cudaError_t launch_reconstruct(const ReconArgs& a, cudaStream_t s)
{
    const int nd = (a.z == 1 && a.y == 1) ? 1 : (a.z == 1 ? 2 : 3);
    if (nd == 1) {
        k_recon1d<<<(uint32_t)cdiv(cdiv(a.nl, 256), 8), 256, 0, s>>>(a);
    } else if (nd == 2) {
        const uint32_t nwin = (uint32_t)cdiv(a.x, 512);
        k_recon2d<<<(uint32_t)(nwin * cdiv(a.y, 16)), 128, 0, s>>>(a, nwin);
    } else {
        const uint32_t nwin = (uint32_t)cdiv(a.x, 128), nyg = (uint32_t)cdiv(cdiv(a.y, 8), 4);
        k_recon3d<<<(uint32_t)((uint64_t)nwin * nyg * cdiv(a.z, 8)), 128, 0, s>>>(a, nwin, nyg);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && a.n > a.nl) {
        k_zero_tail<<<(uint32_t)std::min<uint64_t>(cdiv(a.n - a.nl, 256), 1024), 256, 0, s>>>(a.out, a.nl, a.n);
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace fz
