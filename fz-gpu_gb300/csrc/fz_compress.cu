// fz_compress.cu -- compression kernels.
//
//   k_range_fields    max/min of 1024-element items of a list of fields (fz.cu:137),
//                     the error-bound constants following from them (lorenzo_var.cuh:
//                     562-563).
//   k_encode_fields   Lorenzo dual-quantisation (lorenzo_var.cuh:47-295), bitshuffle +
//                     chunk flags + bitmap (fz.cu:61-111) and each block's non-zero chunks
//                     compacted into its own slot (encodeDebug, fz.cu:49-59); independent
//                     CTAs, one 2048-code shuffle block per warp.
//   k_compact_fields  the prefix sum over the blocks' chunk counts (replacing
//                     cub::DeviceScan, fz.cu:187-201) from per-group sums, the move of the
//                     chunks to their final offsets, the offset table and the header.
//   k_range, k_compress  the same forward path with a decoupled look-back over scan
//                     tiles in a single persistent launch after a range pass; used where no
//                     scratch for the slots exists (fz_compress_noalloc).
//
// Work decomposition: one warp owns one 2048-code shuffle block.  The warp computes its
// codes from the floats (halo rows come from L2), stages them in 4 KiB of shared memory,
// transposes 32x32 bit tiles in registers, derives the chunk flags with 8 ballots (which
// are exactly the 8 bitmap words of the block) and writes its non-zero chunks with
// 128-bit stores.
#include <algorithm>
#include <atomic>

#include "fz_internal.h"

#ifndef FZ_ENCODE_RING
#define FZ_ENCODE_RING 4
#endif
#ifndef FZ_RANGE_VEC
#define FZ_RANGE_VEC 8
#endif
#ifndef FZ_ENCODE_CTAS
#define FZ_ENCODE_CTAS 3
#endif
#ifndef FZ_BLOCK3D_UNROLL
#define FZ_BLOCK3D_UNROLL 2
#endif
#ifndef FZ_ENCODE_CTAS_2D
#define FZ_ENCODE_CTAS_2D 5
#endif
#ifndef FZ_RANGE_CTAS
#define FZ_RANGE_CTAS 5
#endif

namespace fz {

// Group rows per iteration of block3d's loop: unrolled by 2 the rotation of the next row's
// loads needs no register moves (hurricane-like 500x500x100 on GB300: 59.6 -> 57.8 us).
constexpr int kBlock3dUnroll = FZ_BLOCK3D_UNROLL;
#ifndef FZ_BLOCK3D_U_UNROLL
#define FZ_BLOCK3D_U_UNROLL 2
#endif
constexpr int kBlock3dUUnroll = FZ_BLOCK3D_U_UNROLL;  // the same for block3d_u (501x500x100: 84.0 -> 81.2 us)

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// Prequantised values of in[e0+j-off], j=0..3 (0 where e0+j < off or e0+j-off >= lim).
__device__ __forceinline__ void row4(const float* __restrict__ in, uint32_t e0, uint32_t off,
                                     uint32_t aligned, uint32_t lim, float r, float (&q)[4])
{
    if (aligned && e0 >= off && e0 - off + 3 < lim) {
        const float4 v = ldg4(in + (e0 - off));
        q[0] = pq(v.x, r), q[1] = pq(v.y, r), q[2] = pq(v.z, r), q[3] = pq(v.w, r);
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t e = e0 + j;
            q[j] = (e >= off && e - off < lim) ? pq(__ldg(in + (e - off)), r) : 0.0f;
        }
    }
}

__device__ __forceinline__ float west_of(const float* __restrict__ in, uint32_t e0, uint32_t off,
                                         float r)
{
    return e0 >= off + 1 ? pq(__ldg(in + (e0 - 1 - off)), r) : 0.0f;
}

// Codes of the 4 consecutive elements e0..e0+3 (e0 % 4 == 0).  All 32 lanes of the warp
// must call this together (the west neighbours come from lane-1 by shuffle).  `lim` is
// the number of readable input elements; codes at e >= nl are 0.  `ovf` collects
// "delta does not fit its field"; `sgn` (1D) gets bit j = (delta_j < 0).
struct Geo {
    uint32_t nl, x, y, xy, lim;
    FastDiv  dx, dxy;
    uint32_t al_x, al_xy, al_xyx;
};

// Fast variants for the common case, chosen warp-uniformly: all four elements live and
// rows a multiple of 4 elements long (so no row starts inside a group and halo rows are
// 16-byte aligned).  Same float expressions as the generic code below.
__device__ __forceinline__ void fast2d(const float* __restrict__ in, const Geo& g, uint32_t e0, float r,
                                       uint32_t lane, uint32_t (&code)[4], uint32_t& ovf)
{
    const float4   v   = ldg4(in + e0);
    const uint32_t row = fdiv(e0, g.dx), col = e0 - row * g.x;
    const bool     rin = (row & 15u) != 0, cin = (col & 15u) != 0;
    float4         u   = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (rin) u = ldg4(in + (e0 - g.x));
    // t = c - n per element: pred2d's first step (lorenzo_var.cuh:140); the west
    // neighbour's t is what pred2d shuffles in (lorenzo_var.cuh:141)
    float t[4];
    t[0] = __fsub_rn(pq(v.x, r), rin ? pq(u.x, r) : 0.0f);
    t[1] = __fsub_rn(pq(v.y, r), rin ? pq(u.y, r) : 0.0f);
    t[2] = __fsub_rn(pq(v.z, r), rin ? pq(u.z, r) : 0.0f);
    t[3] = __fsub_rn(pq(v.w, r), rin ? pq(u.w, r) : 0.0f);
    float tw = __shfl_up_sync(kFull, t[3], 1);
    if (lane == 0 && cin)
        tw = __fsub_rn(pq(__ldg(in + e0 - 1), r), rin ? pq(__ldg(in + e0 - 1 - g.x), r) : 0.0f);
    tw = cin ? tw : 0.0f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float d = __fsub_rn(t[j], j ? t[j - 1] : tw);
        code[j]       = pack_signed(d);
        ovf |= !(fabsf(d) < 32768.0f) ? 1u : 0u;
    }
}

__device__ __forceinline__ void fast3d(const float* __restrict__ in, const Geo& g, uint32_t e0, float r,
                                       uint32_t lane, uint32_t (&code)[4], uint32_t& ovf)
{
    const float4   v  = ldg4(in + e0);
    const uint32_t zz = fdiv(e0, g.dxy), rem = e0 - zz * g.xy;
    const uint32_t yy = fdiv(rem, g.dx), xx = rem - yy * g.x;
    const bool     zi = (zz & 7u) != 0, yi = (yy & 7u) != 0, xi = (xx & 7u) != 0;
    const float4   z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    // halo rows, zero where the tile has no such neighbour
    const float4 un = yi ? ldg4(in + (e0 - g.x)) : z4;
    const float4 ub = zi ? ldg4(in + (e0 - g.xy)) : z4;
    const float4 uc = (zi && yi) ? ldg4(in + (e0 - g.xy - g.x)) : z4;
    float        p[4]  = {pq(v.x, r), pq(v.y, r), pq(v.z, r), pq(v.w, r)};
    float        nq[4] = {pq(un.x, r), pq(un.y, r), pq(un.z, r), pq(un.w, r)};
    float        bq[4] = {pq(ub.x, r), pq(ub.y, r), pq(ub.z, r), pq(ub.w, r)};
    float        bn[4] = {pq(uc.x, r), pq(uc.y, r), pq(uc.z, r), pq(uc.w, r)};
    float        wp = __shfl_up_sync(kFull, p[3], 1), wn = __shfl_up_sync(kFull, nq[3], 1);
    float        wb = __shfl_up_sync(kFull, bq[3], 1), wbn = __shfl_up_sync(kFull, bn[3], 1);
    if (lane == 0 && xi) {
        wp  = pq(__ldg(in + e0 - 1), r);
        wn  = yi ? pq(__ldg(in + e0 - 1 - g.x), r) : 0.0f;
        wb  = zi ? pq(__ldg(in + e0 - 1 - g.xy), r) : 0.0f;
        wbn = (zi && yi) ? pq(__ldg(in + e0 - 1 - g.xy - g.x), r) : 0.0f;
    }
    if (!xi) wp = wn = wb = wbn = 0.0f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        // c - (A - B - C - D + E + F + G), lorenzo_var.cuh:277-283
        float s = __fsub_rn(j ? bn[j - 1] : wbn, j ? nq[j - 1] : wn);
        s       = __fsub_rn(s, j ? bq[j - 1] : wb);
        s       = __fsub_rn(s, bn[j]);
        s       = __fadd_rn(s, j ? p[j - 1] : wp);
        s       = __fadd_rn(s, nq[j]);
        s       = __fadd_rn(s, bq[j]);
        const float d = __fsub_rn(p[j], s);
        code[j]       = pack_signed(d);
        ovf |= !(fabsf(d) < 32768.0f) ? 1u : 0u;
    }
}

// Swizzled position (in u32 words) of 16-byte chunk q of a block's code image: chunk
// (g, t) of group g lives at g*8 + (t ^ (g & 7)) so that both the row-major writes of
// the Lorenzo phase and the per-group reads of the transpose are conflict-free.
__device__ __forceinline__ uint32_t swz(uint32_t q)
{
    const uint32_t g = q >> 3, t = q & 7u;
    return ((g << 3) | (t ^ (g & 7u))) << 2;
}

// Store offsets of the whole-block paths.  Group row it of a lane writes its 4 codes (one
// half of chunk q = 16 it + lane/2) at word swz(q) + 2 (lane & 1) = 64 it + x(it % 4), with
// x(k) = 32 h + 2 (lane & 1) + 4 (tq ^ (2k + h)), h = lane / 16, tq = (lane / 2) % 8.  The
// four values rotate by one per group row: a loop unrolled by 4 keeps them in registers
// and adds 64 it as an immediate offset.
struct SwzRot {
    uint32_t x0, x1, x2, x3;
    __device__ __forceinline__ explicit SwzRot(uint32_t lane)
    {
        const uint32_t h = lane >> 4, tq = (lane >> 1) & 7u, lo = (h << 5) + (lane & 1u) * 2;
        x0 = lo + ((tq ^ h) << 2), x1 = lo + ((tq ^ (2u + h)) << 2);
        x2 = lo + ((tq ^ (4u + h)) << 2), x3 = lo + ((tq ^ (6u + h)) << 2);
    }
    __device__ __forceinline__ void next()
    {
        const uint32_t t = x0;
        x0 = x1, x1 = x2, x2 = x3, x3 = t;
    }
};

// Position (row, col) of element e0 + 128 given that of e0 (x a multiple of 4).
__device__ __forceinline__ void advance128(const Geo& g, uint32_t e0, uint32_t& row, uint32_t& col)
{
    if (g.x >= 128) {
        col += 128;
        if (col >= g.x) col -= g.x, ++row;
    } else {
        row = fdiv(e0 + 128, g.dx), col = e0 + 128 - row * g.x;
    }
}

// A whole 2D shuffle block [base, base+2048) when every element lies inside x*y and rows
// are a multiple of 4 elements long (so a group of 4 never straddles a row and halo rows
// are 16-byte aligned).  Same float expressions as fast2d; the west neighbour's t of lane
// 0 is carried from lane 31 of the previous group row, row/column advance incrementally,
// and the next group row's loads are issued before the current one is processed (a
// two-stage rotation, so unrolling by 4 leaves no register moves and folds the swizzled
// store offsets).  The north row is zero outside the tile, so its prequantised values
// need no select.
__device__ __forceinline__ void block2d(const float* __restrict__ in, const Geo& g, uint32_t base, float r,
                                        uint32_t lane, uint32_t* sm, uint32_t& ovf)
{
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t     e0 = base + lane * 4;
    uint32_t     row0 = fdiv(e0, g.dx), col0 = e0 - row0 * g.x;
    float4       v0 = ldg4(in + e0), u0 = (row0 & 15u) ? ldg4(in + (e0 - g.x)) : z4;
    // t = c - n of element base-1, the west neighbour of lane 0's first group
    float carry = 0.0f;
    if (lane == 0 && (col0 & 15u))
        carry = __fsub_rn(pq(__ldg(in + e0 - 1), r), (row0 & 15u) ? pq(__ldg(in + e0 - 1 - g.x), r) : 0.0f);
    SwzRot         so(lane);
    const uint32_t prev = (lane + 31u) & 31u;
    float          amax = 0.0f;  // max |d| (NaN if any d is NaN)
#pragma unroll 4
    for (uint32_t it = 0; it < 16; ++it) {
        // group row it+1 of this lane: 128 elements on
        uint32_t row1 = row0, col1 = col0;
        float4   v1 = z4, u1 = z4;
        if (it < 15) {
            advance128(g, e0, row1, col1);
            v1 = ldg4(in + e0 + 128);
            if (row1 & 15u) u1 = ldg4(in + (e0 + 128 - g.x));
        }
        const bool cin = (col0 & 15u) != 0;
        float      t[4];
        t[0] = __fsub_rn(pq(v0.x, r), pq(u0.x, r));
        t[1] = __fsub_rn(pq(v0.y, r), pq(u0.y, r));
        t[2] = __fsub_rn(pq(v0.z, r), pq(u0.z, r));
        t[3] = __fsub_rn(pq(v0.w, r), pq(u0.w, r));
        // lane l - 1's t[3]; lane 0 gets lane 31's, its west neighbour one group row on
        const float rot = __shfl_sync(kFull, t[3], prev);
        const float tw  = cin ? (lane ? rot : carry) : 0.0f;
        carry           = rot;
        float d[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) d[j] = __fsub_rn(t[j], j ? t[j - 1] : tw);
        amax = fmax3_nan(amax, fabsf(d[0]), fabsf(d[1]));
        amax = fmax3_nan(amax, fabsf(d[2]), fabsf(d[3]));
        *reinterpret_cast<uint2*>(sm + it * 64 + so.x0) =
            make_uint2(pack_signed_pair(d[0], d[1]), pack_signed_pair(d[2], d[3]));
        so.next();
        v0 = v1, u0 = u1, row0 = row1, col0 = col1;
        e0 += 128;
    }
    ovf |= !(amax < 32768.0f) ? 1u : 0u;
}

// A whole 1D shuffle block [base, base+2048) inside the field (c_lorenzo_1d1l,
// lorenzo_var.cuh:176-214): 256-element Lorenzo blocks with p[-1] = 0 at their start;
// the code at i%4 == 0 carries its sign, the others the magnitude only (Q2), and the
// signs of all deltas go to the sidecar words when signw is set.  Lane 0's west
// neighbour is carried from lane 31 of the previous group row (group rows at odd
// multiples of 128 continue a 256-element block), and the next row's load is issued
// before the current one is processed.
__device__ __forceinline__ void block1d(const float* __restrict__ in, uint32_t base, float r, uint32_t lane,
                                        uint32_t* sm, uint32_t* signw, uint32_t& ovf)
{
    uint32_t e0    = base + lane * 4;
    float4   v     = ldg4(in + e0);
    float    carry = 0.0f;
    float    amax0 = 0.0f, amax1 = 0.0f;  // max |d| of the signed / magnitude-only positions
    SwzRot         so(lane);
    const uint32_t prev = (lane + 31u) & 31u;
#pragma unroll 4
    for (uint32_t it = 0; it < 16; ++it) {
        const float4 vn = it < 15 ? ldg4(in + e0 + 128) : v;
        const float  p0 = pq(v.x, r), p1 = pq(v.y, r), p2 = pq(v.z, r), p3 = pq(v.w, r);
        const float  rot = __shfl_sync(kFull, p3, prev);  // lane 0: lane 31's, for the next group row
        const float  w   = (e0 & 255u) ? (lane ? rot : carry) : 0.0f;
        carry            = rot;
        const float d0 = __fsub_rn(p0, w), d1 = __fsub_rn(p1, p0), d2 = __fsub_rn(p2, p1), d3 = __fsub_rn(p3, p2);
        amax0          = fmax_nan(amax0, fabsf(d0));
        amax1          = fmax_nan(amax1, fmax3_nan(fabsf(d1), fabsf(d2), fabsf(d3)));
        const uint32_t m0 = static_cast<uint32_t>(fabsf(d0)), m1 = static_cast<uint32_t>(fabsf(d1));
        const uint32_t m2 = static_cast<uint32_t>(fabsf(d2)), m3 = static_cast<uint32_t>(fabsf(d3));
        *reinterpret_cast<uint2*>(sm + it * 64 + so.x0) =
            make_uint2(__byte_perm(m0, m1, 0x5410) | (d0 < 0.0f ? 0x8000u : 0u), __byte_perm(m2, m3, 0x5410));
        so.next();
        if (signw) {
            // 4 sign bits per lane -> one u32 per 8 lanes (32 consecutive elements)
            const uint32_t sgn = (d0 < 0.0f ? 1u : 0u) | (d1 < 0.0f ? 2u : 0u) | (d2 < 0.0f ? 4u : 0u) |
                                 (d3 < 0.0f ? 8u : 0u);
            uint32_t sv = sgn << ((lane & 7u) * 4);
            sv |= __shfl_xor_sync(kFull, sv, 1);
            sv |= __shfl_xor_sync(kFull, sv, 2);
            sv |= __shfl_xor_sync(kFull, sv, 4);
            if ((lane & 7u) == 0) signw[(base >> 5) + it * 4 + (lane >> 3)] = sv;
        }
        v = vn;
        e0 += 128;
    }
    ovf |= (!(amax0 < 32768.0f) || !(amax1 < 65536.0f)) ? 1u : 0u;
}

// ------------------------------------------------- asynchronous row ring --
// The whole-block paths below keep kRing group rows of input in flight per warp without
// holding them in registers: every lane copies its own 16-byte pieces (its 4 elements of
// the centre row and of the north row) into a per-warp ring in shared memory with
// cp.async, kRing group rows ahead, and waits only for its own copies (cp.async.wait_group),
// so no lane waits for another.  A north row outside the element's tile is zero-filled
// (source size 0) instead of read.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// block2d with the ring: the same float expressions, positions and carried west values;
// group row it's inputs come from ring slot it % kRing, refilled with group row it + kRing
// once they have been used.
template <int kRing>
__device__ __forceinline__ void block2d_ring(const float* __restrict__ in, const Geo& g, uint32_t base, float r,
                                             uint32_t lane, uint32_t* sm, float4* ring, uint32_t& ovf)
{
    static_assert(kRing >= 2 && 4 % kRing == 0, "slot of an unrolled row is a constant");
    uint32_t       e0 = base + lane * 4;
    uint32_t       row0 = fdiv(e0, g.dx), col0 = e0 - row0 * g.x;  // group row being computed
    uint32_t       ei = e0, rowi = row0, coli = col0;              // group row being fetched
    const uint32_t rs = (uint32_t)__cvta_generic_to_shared(ring) + lane * 16;
#pragma unroll
    for (int k = 0; k < kRing; ++k) {
        const bool nin = (rowi & 15u) != 0;
        cp_async16(rs + k * 1024, in + ei, 16);
        cp_async16(rs + k * 1024 + 512, nin ? in + (ei - g.x) : in + ei, nin ? 16u : 0u);
        cp_async_commit();
        advance128(g, ei, rowi, coli);
        ei += 128;
    }
    // t = c - n of element base-1, the west neighbour of lane 0's first group
    float carry = 0.0f;
    if (lane == 0 && (col0 & 15u))
        carry = __fsub_rn(pq(__ldg(in + e0 - 1), r), (row0 & 15u) ? pq(__ldg(in + e0 - 1 - g.x), r) : 0.0f);
    SwzRot         so(lane);
    const uint32_t prev = (lane + 31u) & 31u;
    float          amax = 0.0f;
#pragma unroll 4
    for (uint32_t it = 0; it < 16; ++it) {
        cp_async_wait<kRing - 1>();  // this lane's copies of group row it have landed
        const float4* slot = ring + (it % kRing) * 64 + lane;
        const float4  v0 = slot[0], u0 = slot[32];
        const bool    cin = (col0 & 15u) != 0;
        float         t[4];
        t[0] = __fsub_rn(pq(v0.x, r), pq(u0.x, r));
        t[1] = __fsub_rn(pq(v0.y, r), pq(u0.y, r));
        t[2] = __fsub_rn(pq(v0.z, r), pq(u0.z, r));
        t[3] = __fsub_rn(pq(v0.w, r), pq(u0.w, r));
        const float rot = __shfl_sync(kFull, t[3], prev);
        const float tw  = cin ? (lane ? rot : carry) : 0.0f;
        carry           = rot;
        float d[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) d[j] = __fsub_rn(t[j], j ? t[j - 1] : tw);
        amax = fmax3_nan(amax, fabsf(d[0]), fabsf(d[1]));
        amax = fmax3_nan(amax, fabsf(d[2]), fabsf(d[3]));
        *reinterpret_cast<uint2*>(sm + it * 64 + so.x0) =
            make_uint2(pack_signed_pair(d[0], d[1]), pack_signed_pair(d[2], d[3]));
        so.next();
        if (it + kRing < 16) {  // the slot's values are in registers and used: refill it
            const bool     nin = (rowi & 15u) != 0;
            const uint32_t dst = rs + (it % kRing) * 1024;
            cp_async16(dst, in + ei, 16);
            cp_async16(dst + 512, nin ? in + (ei - g.x) : in + ei, nin ? 16u : 0u);
            advance128(g, ei, rowi, coli);
            ei += 128;
        }
        cp_async_commit();  // (empty in the last rows: keeps the group count per row)
        advance128(g, e0, row0, col0);
        e0 += 128;
    }
    ovf |= !(amax < 32768.0f) ? 1u : 0u;
}

// block1d with the ring (centre rows only).
template <int kRing>
__device__ __forceinline__ void block1d_ring(const float* __restrict__ in, uint32_t base, float r, uint32_t lane,
                                             uint32_t* sm, uint32_t* signw, float4* ring, uint32_t& ovf)
{
    static_assert(kRing >= 2 && 4 % kRing == 0, "slot of an unrolled row is a constant");
    uint32_t       e0 = base + lane * 4;
    const uint32_t rs = (uint32_t)__cvta_generic_to_shared(ring) + lane * 16;
#pragma unroll
    for (int k = 0; k < kRing; ++k) {
        cp_async16(rs + k * 1024, in + e0 + 128 * k, 16);
        cp_async_commit();
    }
    float          carry = 0.0f;
    float          amax0 = 0.0f, amax1 = 0.0f;
    SwzRot         so(lane);
    const uint32_t prev = (lane + 31u) & 31u;
#pragma unroll 4
    for (uint32_t it = 0; it < 16; ++it) {
        cp_async_wait<kRing - 1>();
        const float4 v  = ring[(it % kRing) * 64 + lane];
        const float  p0 = pq(v.x, r), p1 = pq(v.y, r), p2 = pq(v.z, r), p3 = pq(v.w, r);
        const float  rot = __shfl_sync(kFull, p3, prev);
        const float  w   = (e0 & 255u) ? (lane ? rot : carry) : 0.0f;
        carry            = rot;
        const float d0 = __fsub_rn(p0, w), d1 = __fsub_rn(p1, p0), d2 = __fsub_rn(p2, p1), d3 = __fsub_rn(p3, p2);
        amax0          = fmax_nan(amax0, fabsf(d0));
        amax1          = fmax_nan(amax1, fmax3_nan(fabsf(d1), fabsf(d2), fabsf(d3)));
        const uint32_t m0 = static_cast<uint32_t>(fabsf(d0)), m1 = static_cast<uint32_t>(fabsf(d1));
        const uint32_t m2 = static_cast<uint32_t>(fabsf(d2)), m3 = static_cast<uint32_t>(fabsf(d3));
        *reinterpret_cast<uint2*>(sm + it * 64 + so.x0) =
            make_uint2(__byte_perm(m0, m1, 0x5410) | (d0 < 0.0f ? 0x8000u : 0u), __byte_perm(m2, m3, 0x5410));
        so.next();
        if (signw) {
            const uint32_t sgn = (d0 < 0.0f ? 1u : 0u) | (d1 < 0.0f ? 2u : 0u) | (d2 < 0.0f ? 4u : 0u) |
                                 (d3 < 0.0f ? 8u : 0u);
            uint32_t sv = sgn << ((lane & 7u) * 4);
            sv |= __shfl_xor_sync(kFull, sv, 1);
            sv |= __shfl_xor_sync(kFull, sv, 2);
            sv |= __shfl_xor_sync(kFull, sv, 4);
            if ((lane & 7u) == 0) signw[(base >> 5) + it * 4 + (lane >> 3)] = sv;
        }
        if (it + kRing < 16) cp_async16(rs + (it % kRing) * 1024, in + e0 + 128 * kRing, 16);
        cp_async_commit();
        e0 += 128;
    }
    ovf |= (!(amax0 < 32768.0f) || !(amax1 < 65536.0f)) ? 1u : 0u;
}

// The 4 elements e0..e0+3 of a lane when rows are not a multiple of 4 elements long
// (x >= 4: a group wraps a row at most once).  Position of each, from the first's.
struct Pos4 {
    uint32_t row[4], col[4];
};
__device__ __forceinline__ Pos4 pos4(const Geo& g, uint32_t row0, uint32_t col0)
{
    Pos4 P;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t c = col0 + j;
        const bool     w = c >= g.x;
        P.col[j]         = w ? c - g.x : c;
        P.row[j]         = w ? row0 + 1 : row0;
    }
    return P;
}

// A whole 2D shuffle block inside x*y whose rows are not a multiple of 4 elements long
// (x >= 4).  Same float expressions as the per-group path; the north row comes in four
// coalesced scalar loads per group, the west neighbour of lane 0 is carried from lane 31
// of the previous group row, and positions advance incrementally.
__device__ __forceinline__ void block2d_u(const float* __restrict__ in, const Geo& g, uint32_t base, float r,
                                          uint32_t lane, uint32_t* sm, uint32_t& ovf)
{
    uint32_t e0   = base + lane * 4;
    uint32_t row0 = fdiv(e0, g.dx), col0 = e0 - row0 * g.x;
    float    carry = 0.0f;  // t = c - n of element e0-1 (lane 0: the previous group row's last)
    if (lane == 0 && (col0 & 15u))
        carry = __fsub_rn(pq(__ldg(in + e0 - 1), r), (row0 & 15u) ? pq(__ldg(in + e0 - 1 - g.x), r) : 0.0f);
    float4 v    = ldg4(in + e0);
    float          amax = 0.0f;
    SwzRot         so(lane);
    const uint32_t prev = (lane + 31u) & 31u;
#pragma unroll 4
    for (uint32_t it = 0; it < 16; ++it) {
        const float4 vn = it < 15 ? ldg4(in + e0 + 128) : v;
        const float  c[4] = {v.x, v.y, v.z, v.w};
        // the lane's 4 elements cross a row end only where a row boundary falls inside its
        // group (rare): otherwise they share one row and the tile tests are made once
        const bool wrap = col0 + 3 >= g.x;
        float      t[4];
        if (!wrap) {
            const bool nz = (row0 & 15u) != 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float nq = nz ? pq(__ldg(in + (e0 + j - g.x)), r) : 0.0f;
                t[j]           = __fsub_rn(pq(c[j], r), nq);
            }
        } else {
            const Pos4 P = pos4(g, row0, col0);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float nq = (P.row[j] & 15u) ? pq(__ldg(in + (e0 + j - g.x)), r) : 0.0f;
                t[j]           = __fsub_rn(pq(c[j], r), nq);
            }
        }
        const float rot = __shfl_sync(kFull, t[3], prev);  // lane 0: lane 31's, for the next group row
        const float tw  = lane ? rot : carry;
        carry           = rot;
        float d[4];
        if (!wrap) {
            const uint32_t k = (0u - col0) & 15u;  // element k starts a tile row (when k < 4)
#pragma unroll
            for (int j = 0; j < 4; ++j) d[j] = __fsub_rn(t[j], (uint32_t)j == k ? 0.0f : (j ? t[j - 1] : tw));
        } else {
            const Pos4 P = pos4(g, row0, col0);
#pragma unroll
            for (int j = 0; j < 4; ++j) d[j] = __fsub_rn(t[j], (P.col[j] & 15u) ? (j ? t[j - 1] : tw) : 0.0f);
        }
        amax = fmax3_nan(amax, fabsf(d[0]), fabsf(d[1]));
        amax = fmax3_nan(amax, fabsf(d[2]), fabsf(d[3]));
        *reinterpret_cast<uint2*>(sm + it * 64 + so.x0) =
            make_uint2(pack_signed_pair(d[0], d[1]), pack_signed_pair(d[2], d[3]));
        so.next();
        advance128(g, e0, row0, col0);
        v = vn;
        e0 += 128;
    }
    ovf |= !(amax < 32768.0f) ? 1u : 0u;
}

// Plane/row/column of element e0 + 128 given that of e0 (x a multiple of 4).
__device__ __forceinline__ void advance128_3d(const Geo& g, uint32_t e0, uint32_t& zz, uint32_t& yy,
                                              uint32_t& xx)
{
    if (g.x >= 128) {
        xx += 128;
        if (xx >= g.x) {
            xx -= g.x;
            if (++yy == g.y) yy = 0, ++zz;
        }
    } else {
        const uint32_t e = e0 + 128;
        zz               = fdiv(e, g.dxy);
        const uint32_t rem = e - zz * g.xy;
        yy               = fdiv(rem, g.dx), xx = rem - yy * g.x;
    }
}

// A whole 3D shuffle block inside x*y*z whose rows are not a multiple of 4 elements long
// (x >= 4: a lane's group wraps a row at most once).  Same float expressions as the
// per-group path: halo values are zero where the element's tile has no such neighbour,
// and the west terms of an element are its left neighbour's (same row whenever they are
// used) -- for lane 0's first element carried from lane 31 of the previous group row.
__device__ __forceinline__ void block3d_u(const float* __restrict__ in, const Geo& g, uint32_t base, float r,
                                          uint32_t lane, uint32_t* sm, uint32_t& ovf)
{
    uint32_t e0 = base + lane * 4;
    uint32_t zz = fdiv(e0, g.dxy);
    uint32_t yy = fdiv(e0 - zz * g.xy, g.dx), xx = e0 - zz * g.xy - yy * g.x;
    // prequantised c, n, b, bn of element e0-1 (lane 0's west neighbour, same row)
    float cw = 0.0f, nw = 0.0f, bw = 0.0f, bnw = 0.0f;
    if (lane == 0 && (xx & 7u)) {
        const bool zi = (zz & 7u) != 0, yi = (yy & 7u) != 0;
        cw  = pq(__ldg(in + e0 - 1), r);
        nw  = yi ? pq(__ldg(in + e0 - 1 - g.x), r) : 0.0f;
        bw  = zi ? pq(__ldg(in + e0 - 1 - g.xy), r) : 0.0f;
        bnw = (zi && yi) ? pq(__ldg(in + e0 - 1 - g.xy - g.x), r) : 0.0f;
    }
    float4         v    = ldg4(in + e0);
    float          amax = 0.0f;
    const uint32_t prev = (lane + 31u) & 31u;
#pragma unroll kBlock3dUUnroll
    for (uint32_t it = 0; it < 16; ++it) {
        const float4 vn   = it < 15 ? ldg4(in + e0 + 128) : v;
        const float  c[4] = {v.x, v.y, v.z, v.w};
        float        p[4], nq[4], bq[4], bn[4];
        bool         xi[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            uint32_t xj = xx + j, yj = yy, zj = zz;
            if (xj >= g.x) {
                xj -= g.x;
                if (++yj == g.y) yj = 0, ++zj;
            }
            const bool     zi = (zj & 7u) != 0, yi = (yj & 7u) != 0;
            const uint32_t e  = e0 + j;
            xi[j]             = (xj & 7u) != 0;
            p[j]              = pq(c[j], r);
            nq[j]             = yi ? pq(__ldg(in + (e - g.x)), r) : 0.0f;
            bq[j]             = zi ? pq(__ldg(in + (e - g.xy)), r) : 0.0f;
            bn[j]             = (zi && yi) ? pq(__ldg(in + (e - g.xy - g.x)), r) : 0.0f;
        }
        // lane l - 1's values; lane 0 gets lane 31's, its west neighbours one group row on
        const float rp = __shfl_sync(kFull, p[3], prev), rn = __shfl_sync(kFull, nq[3], prev);
        const float rb = __shfl_sync(kFull, bq[3], prev), rbn = __shfl_sync(kFull, bn[3], prev);
        float       wp = lane ? rp : cw, wn = lane ? rn : nw, wb = lane ? rb : bw, wbn = lane ? rbn : bnw;
        cw = rp, nw = rn, bw = rb, bnw = rbn;
        float d[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            // c - (A - B - C - D + E + F + G), lorenzo_var.cuh:277-283; absent terms are 0
            const float A = xi[j] ? (j ? bn[j - 1] : wbn) : 0.0f;
            const float B = xi[j] ? (j ? nq[j - 1] : wn) : 0.0f;
            const float C = xi[j] ? (j ? bq[j - 1] : wb) : 0.0f;
            const float E = xi[j] ? (j ? p[j - 1] : wp) : 0.0f;
            float       s = __fsub_rn(A, B);
            s             = __fsub_rn(s, C);
            s             = __fsub_rn(s, bn[j]);
            s             = __fadd_rn(s, E);
            s             = __fadd_rn(s, nq[j]);
            s             = __fadd_rn(s, bq[j]);
            d[j]          = __fsub_rn(p[j], s);
        }
        amax = fmax3_nan(amax, fabsf(d[0]), fabsf(d[1]));
        amax = fmax3_nan(amax, fabsf(d[2]), fabsf(d[3]));
        const uint32_t q = it * 16 + (lane >> 1);
        *reinterpret_cast<uint2*>(sm + swz(q) + (lane & 1u) * 2) =
            make_uint2(pack_signed_pair(d[0], d[1]), pack_signed_pair(d[2], d[3]));
        advance128_3d(g, e0, zz, yy, xx);
        v = vn;
        e0 += 128;
    }
    ovf |= !(amax < 32768.0f) ? 1u : 0u;
}

// A whole 3D shuffle block [base, base+2048) inside x*y*z with rows a multiple of 4
// elements long (so a lane's 4 elements share one row, and the halo rows -- north,
// below, below-north -- are 16-byte aligned).  Same float expressions as fast3d; the
// west neighbours of lane 0 (prequantised c, n, b, bn of element e0-1) are carried from
// lane 31 of the previous group row, coordinates advance incrementally, and the loads of
// group row it+1 are issued before group row it is processed.
__device__ __forceinline__ void block3d(const float* __restrict__ in, const Geo& g, uint32_t base, float r,
                                        uint32_t lane, uint32_t* sm, uint32_t& ovf)
{
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t     e0 = base + lane * 4;
    uint32_t     zz = fdiv(e0, g.dxy);
    uint32_t     yy = fdiv(e0 - zz * g.xy, g.dx), xx = e0 - zz * g.xy - yy * g.x;
    bool         zi = (zz & 7u) != 0, yi = (yy & 7u) != 0;
    float4       v = ldg4(in + e0);
    float4       un = yi ? ldg4(in + (e0 - g.x)) : z4;
    float4       ub = zi ? ldg4(in + (e0 - g.xy)) : z4;
    float4       uc = (zi && yi) ? ldg4(in + (e0 - g.xy - g.x)) : z4;
    // prequantised c, n, b, bn of element base-1 (lane 0's west neighbour)
    float cw = 0.0f, nw = 0.0f, bw = 0.0f, bnw = 0.0f;
    if (lane == 0 && (xx & 7u)) {
        cw  = pq(__ldg(in + e0 - 1), r);
        nw  = yi ? pq(__ldg(in + e0 - 1 - g.x), r) : 0.0f;
        bw  = zi ? pq(__ldg(in + e0 - 1 - g.xy), r) : 0.0f;
        bnw = (zi && yi) ? pq(__ldg(in + e0 - 1 - g.xy - g.x), r) : 0.0f;
    }
    float          amax = 0.0f;  // max |d| (NaN if any d is NaN)
    const uint32_t prev = (lane + 31u) & 31u;
#pragma unroll kBlock3dUnroll
    for (uint32_t it = 0; it < 16; ++it) {
        uint32_t zn = zz, yn = yy, xn = xx;
        float4   vn = z4, unn = z4, ubn = z4, ucn = z4;
        if (it < 15) {
            advance128_3d(g, e0, zn, yn, xn);
            const bool zin = (zn & 7u) != 0, yin = (yn & 7u) != 0;
            const uint32_t e1 = e0 + 128;
            vn = ldg4(in + e1);
            if (yin) unn = ldg4(in + (e1 - g.x));
            if (zin) ubn = ldg4(in + (e1 - g.xy));
            if (zin && yin) ucn = ldg4(in + (e1 - g.xy - g.x));
        }
        const float p[4]  = {pq(v.x, r), pq(v.y, r), pq(v.z, r), pq(v.w, r)};
        const float nq[4] = {pq(un.x, r), pq(un.y, r), pq(un.z, r), pq(un.w, r)};
        const float bq[4] = {pq(ub.x, r), pq(ub.y, r), pq(ub.z, r), pq(ub.w, r)};
        const float bn[4] = {pq(uc.x, r), pq(uc.y, r), pq(uc.z, r), pq(uc.w, r)};
        // lane l - 1's values; lane 0 gets lane 31's, its west neighbours one group row on
        const float rp = __shfl_sync(kFull, p[3], prev), rn = __shfl_sync(kFull, nq[3], prev);
        const float rb = __shfl_sync(kFull, bq[3], prev), rbn = __shfl_sync(kFull, bn[3], prev);
        float       wp = lane ? rp : cw, wn = lane ? rn : nw, wb = lane ? rb : bw, wbn = lane ? rbn : bnw;
        cw = rp, nw = rn, bw = rb, bnw = rbn;
        if ((xx & 7u) == 0) wp = wn = wb = wbn = 0.0f;  // the group starts a tile row
        float d[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            // c - (A - B - C - D + E + F + G), lorenzo_var.cuh:277-283; absent terms are 0
            float s = __fsub_rn(j ? bn[j - 1] : wbn, j ? nq[j - 1] : wn);
            s       = __fsub_rn(s, j ? bq[j - 1] : wb);
            s       = __fsub_rn(s, bn[j]);
            s       = __fadd_rn(s, j ? p[j - 1] : wp);
            s       = __fadd_rn(s, nq[j]);
            s       = __fadd_rn(s, bq[j]);
            d[j]    = __fsub_rn(p[j], s);
        }
        amax = fmax3_nan(amax, fabsf(d[0]), fabsf(d[1]));
        amax = fmax3_nan(amax, fabsf(d[2]), fabsf(d[3]));
        const uint32_t q = it * 16 + (lane >> 1);
        *reinterpret_cast<uint2*>(sm + swz(q) + (lane & 1u) * 2) =
            make_uint2(pack_signed_pair(d[0], d[1]), pack_signed_pair(d[2], d[3]));
        v = vn, un = unn, ub = ubn, uc = ucn, zz = zn, yy = yn, xx = xn;
        e0 += 128;
    }
    ovf |= !(amax < 32768.0f) ? 1u : 0u;
}

template <int ND>
__device__ __forceinline__ void codes4(const float* __restrict__ in, const Geo& g, uint32_t e0,
                                       float r, uint32_t lane, uint32_t (&code)[4],
                                       uint32_t& ovf, uint32_t& sgn)
{
    // warp-uniform choice of the fast variant (the shuffles need all 32 lanes)
    const bool fast = __all_sync(kFull, e0 + 3 < g.nl) && (ND == 1 || g.al_x);
    if constexpr (ND == 2) {
        if (fast) {
            fast2d(in, g, e0, r, lane, code, ovf);
            return;
        }
    }
    if constexpr (ND == 3) {
        if (fast) {
            fast3d(in, g, e0, r, lane, code, ovf);
            return;
        }
    }
    float p[4];
    row4(in, e0, 0, 1, g.lim, r, p);
    float wp = __shfl_up_sync(kFull, p[3], 1);
    if (lane == 0) wp = west_of(in, e0, 0, r);

    if constexpr (ND == 1) {
        // c_lorenzo_1d1l (lorenzo_var.cuh:176-214): 256-element blocks, p[-1] = 0.
        const uint32_t k = e0 & 255u;
        float          d[4];
        d[0] = __fsub_rn(p[0], k ? wp : 0.0f);
        d[1] = __fsub_rn(p[1], p[0]);
        d[2] = __fsub_rn(p[2], p[1]);
        d[3] = __fsub_rn(p[3], p[2]);
        sgn  = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const bool live = e0 + j < g.nl;
            code[j]         = live ? (j == 0 ? pack_signed(d[j]) : pack_unsigned(d[j])) : 0u;
            ovf |= (live && !(fabsf(d[j]) < (j == 0 ? 32768.0f : 65536.0f))) ? 1u : 0u;
            sgn |= (live && d[j] < 0) ? (1u << j) : 0u;
        }
        return;
    }

    if constexpr (ND == 2) {
        // c_lorenzo_2d1l_16x16data_mapto16x2 (lorenzo_var.cuh:216-238): 16x16 tiles,
        // d = (c - n) - (w - nw), zero outside the tile.
        float nq[4];
        row4(in, e0, g.x, g.al_x, g.lim, r, nq);
        float wn = __shfl_up_sync(kFull, nq[3], 1);
        if (lane == 0) wn = west_of(in, e0, g.x, r);
        uint32_t row = fdiv(e0, g.dx), col = e0 - row * g.x;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j) {
                if (++col == g.x) col = 0, ++row;
            }
            const bool  rin = (row & 15u) != 0, cin = (col & 15u) != 0;
            const float N   = rin ? nq[j] : 0.0f;
            const float W   = cin ? (j ? p[j - 1] : wp) : 0.0f;
            const float NW  = (rin && cin) ? (j ? nq[j - 1] : wn) : 0.0f;
            const float d   = __fsub_rn(__fsub_rn(p[j], N), __fsub_rn(W, NW));
            const bool  live = e0 + j < g.nl;
            code[j]          = live ? pack_signed(d) : 0u;
            ovf |= (live && !(fabsf(d) < 32768.0f)) ? 1u : 0u;
        }
        return;
    }

    if constexpr (ND == 3) {
        // c_lorenzo_3d1l_32x8x8data_mapto32x1x8 (lorenzo_var.cuh:240-295): 8x8x8 tiles,
        // the 7-term expression of :277-283 evaluated left to right.
        float nq[4], bq[4], bn[4];
        row4(in, e0, g.x, g.al_x, g.lim, r, nq);
        row4(in, e0, g.xy, g.al_xy, g.lim, r, bq);
        row4(in, e0, g.xy + g.x, g.al_xyx, g.lim, r, bn);
        float wn  = __shfl_up_sync(kFull, nq[3], 1);
        float wb  = __shfl_up_sync(kFull, bq[3], 1);
        float wbn = __shfl_up_sync(kFull, bn[3], 1);
        if (lane == 0) {
            wn  = west_of(in, e0, g.x, r);
            wb  = west_of(in, e0, g.xy, r);
            wbn = west_of(in, e0, g.xy + g.x, r);
        }
        uint32_t zz = fdiv(e0, g.dxy), rem = e0 - zz * g.xy;
        uint32_t yy = fdiv(rem, g.dx), xx = rem - yy * g.x;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j) {
                if (++xx == g.x) {
                    xx = 0;
                    if (++yy == g.y) yy = 0, ++zz;
                }
            }
            const bool  zi = (zz & 7u) != 0, yi = (yy & 7u) != 0, xi = (xx & 7u) != 0;
            const float A  = (zi && yi && xi) ? (j ? bn[j - 1] : wbn) : 0.0f;
            const float B  = (yi && xi) ? (j ? nq[j - 1] : wn) : 0.0f;
            const float Cc = (zi && xi) ? (j ? bq[j - 1] : wb) : 0.0f;
            const float D  = (zi && yi) ? bn[j] : 0.0f;
            const float E  = xi ? (j ? p[j - 1] : wp) : 0.0f;
            const float F  = yi ? nq[j] : 0.0f;
            const float G  = zi ? bq[j] : 0.0f;
            float       s  = __fsub_rn(A, B);
            s              = __fsub_rn(s, Cc);
            s              = __fsub_rn(s, D);
            s              = __fadd_rn(s, E);
            s              = __fadd_rn(s, F);
            s              = __fadd_rn(s, G);
            const float d  = __fsub_rn(p[j], s);
            const bool  live = e0 + j < g.nl;
            code[j]          = live ? pack_signed(d) : 0u;
            ovf |= (live && !(fabsf(d) < 32768.0f)) ? 1u : 0u;
        }
    }
}

// --------------------------------------------------------------- range --
constexpr int kRangeUnroll = 8;
// max and min of the field (fz.cu:137) as order-preserving integers folded with one
// atomicMin/atomicMax per CTA into mm[0..1], which the consuming compress kernel resets
// to "empty" for the next call.  Each thread issues kRangeUnroll 16-byte loads at once
// (coalesced across the CTA); the grid covers the field in one batch per thread, so the
// block scheduler keeps every SM streaming until the last CTAs.  NaN/Inf raise
// kStatusNonfinite: the running min and max propagate NaN (min.NaN / max.NaN), so one
// test of each thread's final pair finds any NaN, -Inf or +Inf it has seen; the bit also
// goes to `callw` (a per-call word the header writer reads and resets), when given.
__global__ void __launch_bounds__(256) k_range(const float* __restrict__ in, uint32_t n, uint32_t* mm,
                                               uint32_t* status, uint32_t* callw)
{
    __shared__ uint32_t smn[8], smx[8], snf[8];
    float          mn = INFINITY, mx = -INFINITY;
    uint32_t       nonfinite = 0;
    const uint32_t n4        = n / 4;
    const uint32_t per       = blockDim.x * kRangeUnroll;
    for (uint32_t b = blockIdx.x * per + threadIdx.x; b < n4; b += gridDim.x * per) {
        float4 v[kRangeUnroll];
#pragma unroll
        for (int k = 0; k < kRangeUnroll; ++k)
            if (b + k * blockDim.x < n4) v[k] = ldg4(in + 4 * (size_t)(b + k * blockDim.x));
#pragma unroll
        for (int k = 0; k < kRangeUnroll; ++k) {
            if (b + k * blockDim.x >= n4) continue;
            mn = fmin_nan(fmin_nan(mn, v[k].x), fmin_nan(v[k].y, fmin_nan(v[k].z, v[k].w)));
            mx = fmax_nan(fmax_nan(mx, v[k].x), fmax_nan(v[k].y, fmax_nan(v[k].z, v[k].w)));
        }
    }
    // NaN leaves both NaN; -Inf shows in the min, +Inf in the max (the start values
    // +Inf / -Inf of a thread without elements stay on the other side)
    nonfinite = (mn != mn) | (mn == -INFINITY) | (mx == INFINITY);
    if (blockIdx.x == 0 && threadIdx.x < n - 4 * n4) {
        const float v = in[4 * n4 + threadIdx.x];
        mn = fminf(mn, v), mx = fmaxf(mx, v);
        nonfinite |= !isfinite(v);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(kFull, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    }
    nonfinite = __reduce_or_sync(kFull, nonfinite);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) smn[w] = f2ord(mn), smx[w] = f2ord(mx), snf[w] = nonfinite;
    __syncthreads();
    if (threadIdx.x < 32) {
        const uint32_t nw = blockDim.x >> 5;
        const uint32_t a  = __reduce_min_sync(kFull, lane < nw ? smn[lane] : 0xFFFFFFFFu);
        const uint32_t c  = __reduce_max_sync(kFull, lane < nw ? smx[lane] : 0u);
        const uint32_t f  = __reduce_or_sync(kFull, lane < nw ? snf[lane] : 0u);
        if (lane == 0) {
            atomicMin(mm, a);
            atomicMax(mm + 1, c);
            if (f) {
                atomicOr(status, kStatusNonfinite);
                if (callw) atomicOr(callw, kStatusNonfinite);
            }
        }
    }
}

// Error-bound constants from the range, as runSzs and the launcher derive them:
// eb = rel * range in double (fz.cu:149), ebx2_r = (float)(1/(2 eb))
// (lorenzo_var.cuh:562-563), ebx2 = (float)(2 eb) (lorenzo_var.cuh:641).
__device__ EbInfo eb_from_range(float vmin, float vmax, double rel)
{
    EbInfo e;
    e.vmin            = vmin;
    e.vmax            = vmax;
    e.range           = __fsub_rn(vmax, vmin);
    e.eb_abs          = rel * (double)e.range;
    const double ebx2 = e.eb_abs * 2;
    e.ebx2_r          = (float)(1 / ebx2);
    e.ebx2            = (float)ebx2;
    e.nonfinite       = 0;
    return e;
}

// ------------------------------------------------------------ compress --
constexpr int kCompressWarps = 8;

// Stream header (struct fz_header, include/fz.h), written once the stream's chunk count is
// known.  flags: FZ_FLAG_CODE_OVERFLOW (1) and FZ_FLAG_FAILED (2).
__device__ void write_header(const CompressArgs& a, const EbInfo& e, uint32_t flags, uint32_t nnz,
                             uint4* mirror = nullptr)
{
    const unsigned long long eb = __double_as_longlong(e.eb_abs);
    const uint4 w[4] = {make_uint4(0x31475A46u, 1u | (a.mode << 16) | (a.ndim << 24), a.x, a.y),
                        make_uint4(a.z, flags, a.n, 0u),
                        make_uint4((uint32_t)eb, (uint32_t)(eb >> 32), __float_as_uint(e.ebx2_r), __float_as_uint(e.ebx2)),
                        make_uint4(nnz, 0u, __float_as_uint(e.range), a.sidecar_bytes)};
    uint4* h = reinterpret_cast<uint4*>(a.out);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        h[k] = w[k];
        if (mirror) mirror[k] = w[k];
    }
}


// Phases A-C for shuffle block t of the field: its codes into the warp's shared buffer
// `sm` (swizzled), the bit transpose, the shuffled image back into `sm`, the chunk flags
// as 8 ballots (= bitmap words 8t..8t+7, stored), the chunk count and the overflow bit.
// Block t == nb (the n mod 2048 tail, never shuffled, fz.cu:173) writes its codes to the
// sidecar and zero-fills the 16-byte pads of Sections A and C.
// kRing > 0: the aligned 1D/2D whole-block paths take their inputs through a cp.async ring
// of kRing group rows at `ring` (1 KiB per group row and warp).
template <int ND, int kRing = 0>
__device__ __forceinline__ void compute_block(const CompressArgs& a, const Geo& g, uint32_t t, float r,
                                              uint32_t lane, uint32_t* sm, uint32_t* signw,
                                              uint32_t (&bm)[8], uint32_t& cnt, uint32_t& ovf,
                                              float4* ring = nullptr)
{
    const uint32_t base = t * kBlockCodes;
    if (t < a.nb) {
        // ---- phase A: codes of the block into shared memory (swizzled) ----
        if (ND == 1 && base + kBlockCodes <= g.nl) {
            if constexpr (kRing > 0) block1d_ring<kRing>(a.in, base, r, lane, sm, signw, ring, ovf);
            else block1d(a.in, base, r, lane, sm, signw, ovf);
        } else if (ND == 2 && g.al_x && base + kBlockCodes <= g.nl) {
            if constexpr (kRing > 0) block2d_ring<kRing>(a.in, g, base, r, lane, sm, ring, ovf);
            else block2d(a.in, g, base, r, lane, sm, ovf);
        } else if (ND == 2 && g.x >= 4 && base + kBlockCodes <= g.nl) {
            block2d_u(a.in, g, base, r, lane, sm, ovf);
        } else if (ND == 3 && g.al_x && base + kBlockCodes <= g.nl) {
            block3d(a.in, g, base, r, lane, sm, ovf);
        } else if (ND == 3 && g.x >= 4 && base + kBlockCodes <= g.nl) {
            block3d_u(a.in, g, base, r, lane, sm, ovf);
        } else {
#pragma unroll 4
            for (uint32_t it = 0; it < 16u; ++it) {
                const uint32_t e0 = base + it * 128 + lane * 4;
                uint32_t       c[4], sgn = 0;
                codes4<ND>(a.in, g, e0, r, lane, c, ovf, sgn);
                const uint32_t q = it * 16 + (lane >> 1);
                *reinterpret_cast<uint2*>(sm + swz(q) + (lane & 1u) * 2) =
                    make_uint2(c[0] | (c[1] << 16), c[2] | (c[3] << 16));
                if (ND == 1 && signw) {
                    // 4 sign bits per lane -> one u32 per 8 lanes (32 consecutive elements)
                    uint32_t v = sgn << ((lane & 7u) * 4);
                    v |= __shfl_xor_sync(kFull, v, 1);
                    v |= __shfl_xor_sync(kFull, v, 2);
                    v |= __shfl_xor_sync(kFull, v, 4);
                    if ((lane & 7u) == 0) signw[(base >> 5) + it * 4 + (lane >> 3)] = v;
                }
            }
        }
        __syncwarp();
        // ---- phase B: lane g transposes group g (words g*32 .. g*32+31) ----
        uint32_t w[32];
#pragma unroll
        for (uint32_t tt = 0; tt < 8; ++tt) {
            const uint4 v = *reinterpret_cast<const uint4*>(sm + swz(lane * 8 + tt));
            w[4 * tt] = v.x, w[4 * tt + 1] = v.y, w[4 * tt + 2] = v.z, w[4 * tt + 3] = v.w;
        }
        transpose32(w);
        __syncwarp();
        // shuffled image S[p*32 + g] = w[p] (bitshuffleAndBitflag's out, fz.cu:82)
#pragma unroll
        for (uint32_t p = 0; p < 32; ++p) sm[p * 32 + lane] = w[p];
        __syncwarp();
        // ---- phase C: chunk c = lane + 32 i; ballot i is bitmap word 8t+i ----
#pragma unroll
        for (uint32_t i = 0; i < 8; ++i) {
            const uint4 v = *reinterpret_cast<const uint4*>(sm + (lane + 32 * i) * 4);
            bm[i] = __ballot_sync(kFull, (v.x | v.y | v.z | v.w) != 0);
            cnt += __popc(bm[i]);
        }
        if (lane == 0) {
            uint4* A = reinterpret_cast<uint4*>(a.out + a.off_a) + 2 * (size_t)t;
            A[0]     = make_uint4(bm[0], bm[1], bm[2], bm[3]);
            A[1]     = make_uint4(bm[4], bm[5], bm[6], bm[7]);
        }
    } else if (t == a.nb && a.n > base) {
        // ---- tail block: n mod 2048 codes, never shuffled (fz.cu:173) ----
        const uint32_t tail = a.n - base;
        uint16_t*      tc   = (a.mode == 1) ? reinterpret_cast<uint16_t*>(a.out + a.off_c) : nullptr;
        for (uint32_t it = 0; it * 128 < tail; ++it) {
            const uint32_t e0 = base + it * 128 + lane * 4;
            uint32_t       c[4], sgn = 0;
            codes4<ND>(a.in, g, e0, r, lane, c, ovf, sgn);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (tc && e0 + j < a.n) tc[e0 + j - base] = (uint16_t)c[j];
            if (ND == 1 && signw) {
                uint32_t v = sgn << ((lane & 7u) * 4);
                v |= __shfl_xor_sync(kFull, v, 1);
                v |= __shfl_xor_sync(kFull, v, 2);
                v |= __shfl_xor_sync(kFull, v, 4);
                const uint32_t wi = (base >> 5) + it * 4 + (lane >> 3);
                if ((lane & 7u) == 0 && wi * 32 < a.n) signw[wi] = v;
            }
        }
        // zero padding of the tail code array and of the sign array
        if (tc)
            for (uint32_t i = tail + lane; i < (uint32_t)(pad16(2 * (uint64_t)tail) / 2); i += 32) tc[i] = 0;
        if (ND == 1 && signw) {
            const uint32_t nsw = (uint32_t)cdiv(a.n, 32);
            const uint32_t pw  = (uint32_t)(pad16(4 * (uint64_t)nsw) / 4);
            for (uint32_t i = nsw + lane; i < pw; i += 32) signw[i] = 0;
        }
        // bitmap words of the partial block are zero (fz.cu:167), then the 16-byte pad
        uint32_t*      A  = reinterpret_cast<uint32_t*>(a.out + a.off_a);
        const uint32_t pa = (uint32_t)(pad16(4 * (uint64_t)a.nwords) / 4);
        for (uint32_t i = a.nb * 8 + lane; i < pa; i += 32) A[i] = 0;
    }
    ovf = __reduce_or_sync(kFull, ovf);
}

// Persistent: one resident wave of CTAs; each CTA repeatedly takes the next scan tile
// (8 shuffle blocks, one per warp) from the ticket counter.  Tickets are handed out in
// order, so every predecessor of a tile has been taken by a running CTA and the
// look-back always makes progress, whatever else runs on the GPU.  The last of the
// nct + gridDim.x fetches resets the counter, the range accumulators and advances the
// epoch.
//
// Software pipeline over a CTA's tiles, shared memory double-buffered, two CTA barriers
// per tile: iteration k computes tile k (codes, transposes, flags) -- thread 0 takes the
// CTA's next ticket as soon as its own block is done -- then warp 0 publishes tile k's
// aggregate and resolves tile k-1 (look-back, inclusive prefix, per-block offsets), and
// every warp writes its block of tile k-1.  By then tile k-1's predecessors have long
// published, so its look-back is about one round trip.
template <int ND>
__global__ void __launch_bounds__(kCompressWarps * 32, 3) k_compress(const CompressArgs a)
{
    extern __shared__ __align__(16) uint32_t dsm[];  // [2][kCompressWarps][kBlockWords]
    __shared__ uint32_t s_cnt[2][kCompressWarps], s_ovf[2][kCompressWarps], s_tile[2], s_tot[2];
    __shared__ uint32_t s_pre[kCompressWarps], s_epoch;
    __shared__ EbInfo   s_eb;
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t nct  = (uint32_t)cdiv(a.ntiles, kCompressWarps);
    const uint32_t nfetch = nct + gridDim.x;

    if (threadIdx.x == 0) {
        s_eb    = a.mm ? eb_from_range(ord2f(__ldcg(a.mm)), ord2f(__ldcg(a.mm + 1)), a.eb_rel) : a.ebh;
        s_epoch = __ldcg(a.epoch);
        __threadfence();  // both reads complete before the first ticket (the last one resets them)
        const Ticket tk = take_ticket(a.ticket, a.epoch, nfetch);
        if (tk.last && a.mm) a.mm[0] = 0xFFFFFFFFu, a.mm[1] = 0u;  // empty range for the next call
        s_tile[0] = tk.tile;
    }
    __syncthreads();
    const EbInfo   eb    = s_eb;
    const uint32_t epoch = s_epoch;
    Geo g;
    g.nl = a.nl, g.x = a.x, g.y = a.y, g.xy = a.xy, g.lim = a.n;
    g.dx = a.dx, g.dxy = a.dxy, g.al_x = a.al_x, g.al_xy = a.al_xy, g.al_xyx = a.al_xyx;
    uint32_t* signw = (ND == 1 && a.mode == 1) ? reinterpret_cast<uint32_t*>(a.out + a.off_sign) : nullptr;
    uint32_t  bm_prev[8];  // bitmap words of this warp's block of the previous tile
    uint32_t  prev_ct = 0;

    for (uint32_t k = 0;; ++k) {
        const uint32_t buf   = k & 1u;
        uint32_t*      sm    = dsm + (buf * kCompressWarps + wid) * kBlockWords;
        const uint32_t ct    = s_tile[buf];
        const bool     have  = ct < nct;  // uniform
        uint32_t       bm[8] = {0, 0, 0, 0, 0, 0, 0, 0};

        if (have) {
            uint32_t ovf = 0, cnt = 0;
            compute_block<ND>(a, g, ct * kCompressWarps + wid, eb.ebx2_r, lane, sm, signw, bm, cnt, ovf);
            if (lane == 0) s_cnt[buf][wid] = cnt, s_ovf[buf][wid] = ovf;
            if (threadIdx.x == 0) {  // the CTA's next tile; slot buf^1 (tile k-1) is read only via prev_ct now
                const Ticket tk = take_ticket(a.ticket, a.epoch, nfetch);
                if (tk.last && a.mm) a.mm[0] = 0xFFFFFFFFu, a.mm[1] = 0u;
                s_tile[buf ^ 1u] = tk.tile;
            }
        }
        __syncthreads();
        // ---- tile k: CTA aggregate published; tile k-1: look-back and block offsets ----
        if (wid == 0) {
            if (have) {
                const uint32_t tot = __reduce_add_sync(kFull, lane < kCompressWarps ? s_cnt[buf][lane] : 0u);
                const uint32_t tov = __reduce_or_sync(kFull, lane < kCompressWarps ? s_ovf[buf][lane] : 0u);
                if (lane == 0) {
                    s_tot[buf] = tot;
                    publish(a.state, ct, epoch, ct == 0 ? kFlagIncl : kFlagAgg, tov, tot);
                }
            }
            if (k > 0) {
                const uint32_t pb   = buf ^ 1u;
                const uint32_t tot  = s_tot[pb];
                const uint32_t c    = lane < kCompressWarps ? s_cnt[pb][lane] : 0u;
                const uint32_t tov  = __reduce_or_sync(kFull, lane < kCompressWarps ? s_ovf[pb][lane] : 0u);
                uint32_t       excl = 0, povf = 0;
                if (prev_ct != 0) {
                    lookback(a.state, prev_ct, epoch, a.status, excl, povf);
                    if (lane == 0) publish(a.state, prev_ct, epoch, kFlagIncl, tov | povf, excl + tot);
                }
                uint32_t inc = c;  // exclusive offsets of tile k-1's blocks
#pragma unroll
                for (uint32_t o = 1; o < kCompressWarps; o <<= 1) {
                    const uint32_t v = __shfl_up_sync(kFull, inc, o);
                    if (lane >= o) inc += v;
                }
                if (lane < kCompressWarps) s_pre[lane] = excl + inc - c;
                if (lane == 0 && prev_ct == nct - 1) {
                    write_header(a, eb, (tov | povf) ? 1u : 0u, excl + tot);
                    if (a.boff) {
                        // the total closes the offset table; zero its 16-byte pad
                        a.boff[a.nb] = excl + tot;
                        for (uint32_t i = a.nb + 1; i < (uint32_t)(pad16(4ull * (a.nb + 1)) / 4); ++i) a.boff[i] = 0;
                    }
                }
            }
        }
        __syncthreads();
        // ---- tile k-1: block offset table and compacted 128-bit stores ----
        if (k > 0) {
            const uint32_t t = prev_ct * kCompressWarps + wid;
            if (t < a.nb) {
                uint32_t pre = s_pre[wid];
                if (a.boff && lane == 0) a.boff[t] = pre;
                const uint32_t* smp = dsm + ((buf ^ 1u) * kCompressWarps + wid) * kBlockWords;
                uint4*          B   = reinterpret_cast<uint4*>(a.out + a.off_b);
                const uint32_t  lt  = lanemask_lt();
#pragma unroll
                for (uint32_t i = 0; i < 8; ++i) {
                    if ((bm_prev[i] >> lane) & 1u)
                        B[pre + __popc(bm_prev[i] & lt)] = *reinterpret_cast<const uint4*>(smp + (lane + 32 * i) * 4);
                    pre += __popc(bm_prev[i]);
                }
            }
        }
        if (!have) break;  // uniform; tile k-1 (if any) has been resolved above
#pragma unroll
        for (int i = 0; i < 8; ++i) bm_prev[i] = bm[i];
        prev_ct = ct;
    }
    // The last CTA to leave marks the header when this call raised a status bit (non-finite
    // input, a wait that gave up), so a caller that reads no status still sees the failure
    // in the stream; it also resets the exit counter for the next call.
    if (a.fin) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();  // this CTA's stream writes (the header, if it wrote it) come first
            if (atomicAdd(a.fin, 1u) == gridDim.x - 1) {
                __threadfence();
                if (__ldcg(a.status) & (kStatusTimeout | kStatusNonfinite))
                    atomicOr(reinterpret_cast<uint32_t*>(a.out + 20), FZ_FLAG_FAILED);
                *a.fin = 0;
            }
        }
    }
}

// ================================================ list compression ==
// Compression of a list of fields in three launches, each a persistent grid striding over
// a device work list (FieldJob / Segment, fz_internal.h):
//   k_range_fields     range items: max/min of 1024 elements (relative eb); each CTA a
//                      contiguous run of items, one reduction per field it touches
//   k_encode_fields    encode items: 8 shuffle blocks, one per warp -- codes, bitshuffle,
//                      chunk flags, bitmap words, sidecar, the block's non-zero chunks
//                      compacted into its own 4 KiB slot, its count into counts[] and the
//                      sum of its group of 64 blocks; no CTA waits for another
//   k_compact_fields   compaction items: 32 blocks -- every block's chunk offset (all
//                      counts are known: the group sums before it plus the counts in its
//                      group), the offset table, the chunks moved from the slots to
//                      Section B; the field's last item writes the header
// A single field is a list of one whose job is a kernel parameter.  The stream bytes equal
// the single-pass look-back kernel's.
constexpr uint32_t kCompactBlocks = 32;   // shuffle blocks per compaction item
constexpr int      kEncodeRing    = FZ_ENCODE_RING;  // group rows in flight per warp (1D/2D)
constexpr int      kEncodeCtas    = FZ_ENCODE_CTAS;  // CTAs per SM the 1D/2D encode kernels are built for


// ---------------------------------------------------------------- items --
constexpr uint32_t kCtlOverflow    = 1u << 8;                    // FieldCtl::flags: some code overflowed
constexpr uint32_t kRangeBatch     = FZ_RANGE_VEC;  // range items (16-byte loads) in flight per thread
constexpr uint32_t kRangeItemElems = 256 * 4;       // one 16-byte load per thread

void field_items(uint32_t n, uint32_t nb, uint32_t ntiles, bool rel, uint32_t& nr, uint32_t& ne, uint32_t& nc)
{
    nr = rel ? (uint32_t)std::max<uint64_t>(1, cdiv(n, kRangeItemElems)) : 0u;
    ne = (uint32_t)cdiv(ntiles, kCompressWarps);
    nc = (uint32_t)cdiv(nb, kCompactBlocks);  // none without full blocks (the encode launch writes the header)
}

// Item k of a list launch: field f owns items [segs[f].start, segs[f].start + segs[f].count)
// of the launch (segments sorted by start).  Binary search; the result is CTA-uniform.
__device__ __forceinline__ void locate(const Segment* __restrict__ segs, uint32_t nseg, uint32_t k, uint32_t& f,
                                       uint32_t& i)
{
    uint32_t lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(&segs[mid].start) <= k) lo = mid;
        else hi = mid - 1;
    }
    f = __ldg(&segs[lo].field);
    i = k - __ldg(&segs[lo].start);
}

// Range items: 1024 elements each (one 16-byte load per thread).  A CTA takes a contiguous
// run of items -- CTA c of G the items [c T / G, (c + 1) T / G) of a launch over T items --
// so runs differ by at most one item, and keeps kRangeBatch loads per thread in flight.  The
// running max/min of a thread is carried across its items and folded into the field's
// accumulators once per field the run touches.
// The CTA's running max/min go into mm[0..1] (and a non-finite element into *flags and
// *status) of the field they belong to.
__device__ __forceinline__ void range_flush(uint32_t* mm, uint32_t* flags, uint32_t* status, float mn, float mx,
                                            uint32_t nonfinite, uint32_t (*sred)[kCompressWarps])
{
    // NaN leaves both NaN; -Inf shows in the min, +Inf in the max (the start values +Inf /
    // -Inf of a thread without elements stay on the other side)
    nonfinite |= (mn != mn) | (mn == -INFINITY) | (mx == INFINITY);
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(kFull, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    }
    nonfinite = __reduce_or_sync(kFull, nonfinite);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, wid = tid >> 5;
    if (lane == 0) sred[0][wid] = f2ord(mn), sred[1][wid] = f2ord(mx), sred[2][wid] = nonfinite;
    __syncthreads();
    if (tid < 32) {
        const uint32_t a = __reduce_min_sync(kFull, lane < kCompressWarps ? sred[0][lane] : 0xFFFFFFFFu);
        const uint32_t c = __reduce_max_sync(kFull, lane < kCompressWarps ? sred[1][lane] : 0u);
        const uint32_t f = __reduce_or_sync(kFull, lane < kCompressWarps ? sred[2][lane] : 0u);
        if (lane == 0) {
            atomicMin(mm, a);
            atomicMax(mm + 1, c);
            if (f) atomicOr(status, kStatusNonfinite), atomicOr(flags, kStatusNonfinite);
        }
    }
    __syncthreads();  // sred before the next flush
}

// Items [i, i + cnt) of the n-element field at in (cnt <= kRangeBatch) into the thread's
// running max/min; the field's last item also takes the n mod 4 elements past its 16-byte
// loads.
__device__ __forceinline__ void range_items(const float* __restrict__ in, uint32_t n, uint32_t i, uint32_t cnt,
                                            float& mn, float& mx, uint32_t& nonfinite)
{
    const uint32_t n4 = n / 4, tid = threadIdx.x;
    const uint32_t q0 = i * (kRangeItemElems / 4) + tid;
    float4         v[kRangeBatch];
#pragma unroll
    for (uint32_t k = 0; k < kRangeBatch; ++k)
        if (k < cnt && q0 + k * 256 < n4) v[k] = ldg4(in + 4 * (size_t)(q0 + k * 256));
#pragma unroll
    for (uint32_t k = 0; k < kRangeBatch; ++k) {
        if (k >= cnt || q0 + k * 256 >= n4) continue;
        mn = fmin_nan(fmin_nan(mn, v[k].x), fmin_nan(v[k].y, fmin_nan(v[k].z, v[k].w)));
        mx = fmax_nan(fmax_nan(mx, v[k].x), fmax_nan(v[k].y, fmax_nan(v[k].z, v[k].w)));
    }
    if ((uint64_t)(i + cnt) * kRangeItemElems >= n && tid < n - 4 * n4) {
        const float x = in[4 * n4 + tid];
        mn = fminf(mn, x), mx = fmaxf(mx, x);
        nonfinite |= !isfinite(x);
    }
}

// Encode item i of field J: scan tile ne-1-i (the last tile first: the range launch read
// the field front to back, so its end is the part most likely still in L2), one shuffle
// block per warp; r = ebx2_r; par = this call's group-sum set, also kept in bit 31 of each
// block's count for the compaction launch.
constexpr uint32_t kCountPar = 1u << 31;

template <int ND, int kRing>
__device__ __forceinline__ void encode_item(const FieldJob& J, uint32_t i, float r, uint32_t par, uint32_t* sm,
                                            float4* ring)
{
    const uint32_t      lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const CompressArgs& a    = J.a;
    Geo                 g;
    g.nl = a.nl, g.x = a.x, g.y = a.y, g.xy = a.xy, g.lim = a.n;
    g.dx = a.dx, g.dxy = a.dxy, g.al_x = a.al_x, g.al_xy = a.al_xy, g.al_xyx = a.al_xyx;
    uint32_t* signw = (ND == 1 && a.mode == 1) ? reinterpret_cast<uint32_t*>(a.out + a.off_sign) : nullptr;
    const uint32_t t  = (J.ne - 1 - i) * kCompressWarps + wid;
    uint32_t       bm[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cnt = 0, ovf = 0;
    compute_block<ND, kRing>(a, g, t, r, lane, sm, signw, bm, cnt, ovf, ring);  // warp-uniform t
    if (t < a.nb) {
        uint4*         S   = J.slots + (size_t)t * kChunks;
        const uint32_t lt  = lanemask_lt();
        uint32_t       pre = 0;
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) {
            if ((bm[k] >> lane) & 1u) S[pre + __popc(bm[k] & lt)] = *reinterpret_cast<const uint4*>(sm + (lane + 32 * k) * 4);
            pre += __popc(bm[k]);
        }
        if (lane == 0) {
            J.counts[t] = cnt | (par ? kCountPar : 0u);
            if (cnt) {  // into the block's group sum of each level
                uint32_t* set = J.supers + par * J.sstride;
                atomicAdd(set + t / kSuperBlocks, cnt);
                atomicAdd(set + J.s2off + t / kSuper2Blocks, cnt);
            }
        }
    }
    if (ovf && lane == 0) atomicOr(&J.ctl->flags, kCtlOverflow);
}

// The words the header of field J follows from, loaded by the thread that will write it as
// early as they are final (the range and encode launches have finished), so that they
// travel with its other loads.
struct FieldFinal {
    uint32_t mm0, mm1, flags, status, epoch, pre0, pre1, pre_flags;
};
__device__ __forceinline__ FieldFinal final_loads(const FieldJob& J)
{
    FieldFinal v;
    v.mm0    = __ldcg(J.ctl->mm);
    v.mm1    = __ldcg(J.ctl->mm + 1);
    v.flags  = __ldcg(&J.ctl->flags);
    v.epoch  = __ldcg(&J.ctl->epoch);
    v.status = J.a.mirror ? __ldcg(J.a.status) : 0u;
    v.pre0      = __ldcg(J.ctl->pre);
    v.pre1      = __ldcg(J.ctl->pre + 1);
    v.pre_flags = __ldcg(&J.ctl->pre_flags);
    return v;
}

// The header of field J with `total` chunks (and its copy in the mirror, with the status
// word), the offset table's total, and the control words set for the next call: its range
// and non-finite flag from pre (the range ahead this call's encode launch accumulated, or
// the empty range), pre reset (one thread; after every encode item of the call).
__device__ void finish_field(const FieldJob& J, uint32_t total, const FieldFinal& v)
{
    const CompressArgs& a  = J.a;
    FieldCtl*           C  = J.ctl;
    const EbInfo        eb = J.rel ? eb_from_range(ord2f(v.mm0), ord2f(v.mm1), a.eb_rel) : a.ebh;
    // header and status in the mirror too, so a caller reads both with one copy
    write_header(a, eb, ((v.flags & kCtlOverflow) ? 1u : 0u) | ((v.flags & kStatusNonfinite) ? 2u : 0u), total,
                 reinterpret_cast<uint4*>(a.mirror));
    if (a.mirror) a.mirror[16] = v.status;
    if (a.boff) {
        a.boff[a.nb] = total;  // the total closes the offset table; zero its 16-byte pad
        for (uint32_t k = a.nb + 1; k < (uint32_t)(pad16(4ull * (a.nb + 1)) / 4); ++k) a.boff[k] = 0;
    }
    C->mm[0] = v.pre0, C->mm[1] = v.pre1;
    C->flags = v.pre_flags;
    C->pre[0] = 0xFFFFFFFFu, C->pre[1] = 0u;
    C->pre_flags = 0;
}

// Compaction item i of field J: blocks [32 i, 32 i + 32), four per warp, each warp on its
// own.  A warp's first chunk offset is the sum of this call's group sums before its group
// (second-level sums of kSuper2Blocks blocks, then first-level sums of kSuperBlocks) plus
// the counts of the blocks of its group before its own; then it writes the offset table
// entries of its 4 blocks and moves their chunks from the slots to Section B (output chunk
// q of the warp comes from the last of its blocks whose prefix is <= q; 16-byte loads,
// four in flight per lane).  The call's group-sum set is
// the parity bit of the counts; the warps clear the other set for the next call.  The warp
// holding the last block knows the total: it writes the header and advances the call
// counter.  No CTA uses what another compaction CTA writes: no barrier, fence or atomic.
constexpr uint32_t kCompactWarpBlocks = kCompactBlocks / kCompressWarps;  // 4

__device__ __forceinline__ void compact_item(const FieldJob& J, uint32_t i)
{
    const uint32_t      lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const CompressArgs& a    = J.a;
    const uint32_t      gw = i * kCompressWarps + wid;  // warp of the launch's items of this field
    const uint32_t      b0 = gw * kCompactWarpBlocks, sup = b0 / kSuperBlocks, sup2 = b0 / kSuper2Blocks;
    const bool          live = b0 < a.nb, last = live && b0 + kCompactWarpBlocks >= a.nb;
    // Every load the warp's offsets need is issued before any is used: the call's parity (the
    // top bit of block 0's count); in both sets (the parity picks one) the second-level sums
    // before the warp's second-level group and the first-level sums before its first-level
    // group inside it; the counts before its blocks in its first-level group and its own 4
    // counts.  The last block's warp also loads the words its header follows from.
    static_assert(kSuperBlocks <= 64 && kSuper2Blocks / kSuperBlocks <= 64, "inside a group: two loads per lane");
    FieldFinal fin{};
    if (last && lane == 0) fin = final_loads(J);
    const uint32_t c0 = __ldcg(J.counts);
    uint32_t       s0 = 0, s1 = 0, acc = 0, c = 0;
    if (live) {
        const uint32_t* L2 = J.supers + J.s2off;
        for (uint32_t k = lane; k < sup2; k += 32) s0 += __ldcg(L2 + k), s1 += __ldcg(L2 + J.sstride + k);
        const uint32_t h0 = sup2 * (kSuper2Blocks / kSuperBlocks);  // first-level groups before
#pragma unroll
        for (uint32_t k = lane; k < 64; k += 32)
            if (h0 + k < sup) s0 += __ldcg(J.supers + h0 + k), s1 += __ldcg(J.supers + J.sstride + h0 + k);
        const uint32_t g0 = sup * kSuperBlocks;
        if (g0 + lane < b0) acc += __ldcg(J.counts + g0 + lane) & ~kCountPar;
        if (g0 + 32 + lane < b0) acc += __ldcg(J.counts + g0 + 32 + lane) & ~kCountPar;
        if (lane < kCompactWarpBlocks && b0 + lane < a.nb) c = __ldcg(J.counts + b0 + lane) & ~kCountPar;
    }
    // every warp of the field's items, past the last block too, clears its share of the set
    // this call did not use (another warp may still read it above: that sum is discarded)
    const uint32_t par = c0 >> 31;
    uint32_t*      old = J.supers + (par ^ 1u) * J.sstride;
    for (uint32_t k = gw * 32 + lane; k < J.sstride; k += J.nc * kCompressWarps * 32) old[k] = 0;
    if (!live) return;
    const uint32_t exc = __reduce_add_sync(kFull, acc + (par ? s1 : s0));
    // inclusive prefix of the 4 counts in lanes 0..3
    uint32_t v = c;
#pragma unroll
    for (uint32_t o = 1; o < kCompactWarpBlocks; o <<= 1) {
        const uint32_t u = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v += u;
    }
    if (a.boff && lane < kCompactWarpBlocks && b0 + lane < a.nb) a.boff[b0 + lane] = exc + v - c;
    const uint32_t p1 = __shfl_sync(kFull, v - c, 1), p2 = __shfl_sync(kFull, v - c, 2);
    const uint32_t p3 = __shfl_sync(kFull, v - c, 3), tot = __shfl_sync(kFull, v, 3);
    if (last && lane == 0) {
        // the last block's warp: every count is in, so the total is exc + tot; the header
        // needs none of the chunk moves below
        finish_field(J, exc + tot, fin);
        J.ctl->epoch = fin.epoch + 1u;  // the next call uses the set cleared here
    }
    uint4* B = reinterpret_cast<uint4*>(a.out + a.off_b) + exc;
    for (uint32_t q0 = lane; q0 < tot; q0 += 4 * 32) {
        uint4 val[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t q = q0 + u * 32;
            if (q < tot) {
                const uint32_t j  = (q >= p1) + (q >= p2) + (q >= p3);  // blocks with no chunks never match last
                const uint32_t pj = j == 0 ? 0u : j == 1 ? p1 : j == 2 ? p2 : p3;
                val[u]            = __ldcg(J.slots + (size_t)(b0 + j) * kChunks + (q - pj));
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (q0 + u * 32 < tot) B[q0 + u * 32] = val[u];
    }
}

// -------------------------------------------------------------- kernels --
// kList false: one field, `one` (a kernel parameter: its fields are constant-bank operands
// and take no registers); true: the fields jobs[] of a batch, located through segs[].
template <bool kList>
__global__ void __launch_bounds__(256, FZ_RANGE_CTAS) k_range_fields(const FieldJob* __restrict__ jobs, const Segment* __restrict__ segs,
                                                      uint32_t nseg, uint32_t total, const __grid_constant__ FieldJob one)
{
    pdl_wait();
    pdl_trigger();
    __shared__ uint32_t s_red[3][kCompressWarps];
    uint32_t       k  = (uint32_t)((uint64_t)blockIdx.x * total / gridDim.x);
    const uint32_t k1 = (uint32_t)((uint64_t)(blockIdx.x + 1) * total / gridDim.x);
    if (k >= k1) return;  // (CTA-uniform)
    // segment s (field f, items [fs, fend) of the launch) holds the run's first item
    uint32_t s = 0, f = 0, fs = 0, fend = total;
    if (kList) {
        uint32_t hi = nseg - 1;
        while (s < hi) {
            const uint32_t mid = (s + hi + 1) >> 1;
            if (__ldg(&segs[mid].start) <= k) s = mid;
            else hi = mid - 1;
        }
        f    = __ldg(&segs[s].field);
        fs   = __ldg(&segs[s].start);
        fend = fs + __ldg(&segs[s].count);
    }
    for (;;) {
        const FieldJob& J = kList ? jobs[f] : one;
        const uint32_t  e = min(k1, fend);
        float           mn = INFINITY, mx = -INFINITY;
        uint32_t        nonfinite = 0;
#pragma unroll 1
        while (k < e) {  // ends with k == e: the next field's items start there
            const uint32_t cnt = min(kRangeBatch, e - k);
            range_items(J.a.in, J.a.n, k - fs, cnt, mn, mx, nonfinite);
            k += cnt;
        }
        range_flush(J.ctl->mm, &J.ctl->flags, J.a.status, mn, mx, nonfinite, s_red);
        if (!kList || k >= k1) break;
        ++s;  // the run goes on in the next field
        f    = __ldg(&segs[s].field);
        fs   = __ldg(&segs[s].start);
        fend = fs + __ldg(&segs[s].count);
    }
}

// Ring depth (group rows in flight per warp) of the encode kernels: 1D only.  Measured on
// GB300 (encode launch, relative eb 1e-3): 1D 2^25 elements 49.2 -> 45.3 us with 4 rows at
// 3 CTAs/SM; 2D exafel-like 27.1 -> 29.2 us and cesm-like 16.6 -> 17.4 us, so 2D keeps its
// one row of register lookahead at 5 CTAs/SM (the extra warps hide more than the ring).
template <int ND>
__host__ __device__ constexpr int encode_ring() { return ND == 1 ? kEncodeRing : 0; }
template <int ND>
__host__ __device__ constexpr int encode_ctas() { return ND == 3 ? 4 : (ND == 1 && kEncodeRing ? kEncodeCtas : FZ_ENCODE_CTAS_2D); }
// Dynamic shared memory of an encode CTA: per warp the code image and the ring.
template <int ND>
__host__ __device__ constexpr uint32_t encode_smem() { return kCompressWarps * (kBlockWords * 4 + 1024u * encode_ring<ND>()); }

// Range ahead of a single-field encode launch over `total` items: the CTAs that took one
// item fewer than the others (all CTAs when the items divide evenly; the CTAs without an
// item when the grid, sized for the ahead field, is larger than `total`) split the ahead
// field's range items into contiguous runs, as the range launch would, while the others
// still encode -- the memory-bound pass fills the launch's last, partial wave.
__device__ __forceinline__ void range_ahead(const FieldJob& J, uint32_t total)
{
    __shared__ uint32_t s_red[3][kCompressWarps];
    const uint32_t      G = gridDim.x, rem = total % G;
    uint32_t            c = blockIdx.x, m = G;
    if (rem) {
        if (c < rem) return;  // CTA-uniform
        c -= rem, m = G - rem;
    }
    const uint32_t T = J.ahead_nr;
    uint32_t       k = (uint32_t)((uint64_t)c * T / m);
    const uint32_t k1 = (uint32_t)((uint64_t)(c + 1) * T / m);
    if (k >= k1) return;
    float    mn = INFINITY, mx = -INFINITY;
    uint32_t nonfinite = 0;
#pragma unroll 1
    while (k < k1) {
        const uint32_t cnt = min(kRangeBatch, k1 - k);
        range_items(J.ahead_in, J.ahead_n, k, cnt, mn, mx, nonfinite);
        k += cnt;
    }
    range_flush(J.ctl->pre, &J.ctl->pre_flags, J.a.status, mn, mx, nonfinite, s_red);
}

template <int ND, bool kList>
__global__ void __launch_bounds__(kCompressWarps * 32, encode_ctas<ND>())
    k_encode_fields(const FieldJob* __restrict__ jobs, const Segment* __restrict__ segs, uint32_t nseg, uint32_t total,
                    const __grid_constant__ FieldJob one)
{
    pdl_wait();
    pdl_trigger();
    // per warp: the block's 4 KiB code image, then (1D/2D) its ring of input rows
    extern __shared__ __align__(16) uint32_t esm[];
    constexpr int kR = encode_ring<ND>();
    uint32_t*     smem = esm + (threadIdx.x >> 5) * kBlockWords;
    float4*       ring = kR ? reinterpret_cast<float4*>(esm + kCompressWarps * kBlockWords) + (threadIdx.x >> 5) * kR * 64
                            : nullptr;
    __shared__ float    s_r;
    __shared__ uint32_t s_rf, s_par;
    if (threadIdx.x == 0) s_rf = 0xFFFFFFFFu;
    for (uint32_t k = blockIdx.x; k < total; k += gridDim.x) {
        uint32_t f = 0, i = k;
        if (kList) locate(segs, nseg, k, f, i);
        const FieldJob& J = kList ? jobs[f] : one;
        if (threadIdx.x == 0 && s_rf != f) {
            // ebx2_r of the field: from its range (relative eb; complete once the range launch,
            // or the previous call's encode launch for a range ahead, has finished);
            // the call's group-sum set (the compaction launch moves the counter on)
            s_r   = J.rel ? eb_from_range(ord2f(__ldcg(J.ctl->mm)), ord2f(__ldcg(J.ctl->mm + 1)), J.a.eb_rel).ebx2_r
                          : J.a.ebh.ebx2_r;
            s_par = __ldcg(&J.ctl->epoch) & 1u;
            s_rf  = f;
        }
        __syncthreads();
        encode_item<ND, kR>(J, i, s_r, s_par, smem, ring);
        __syncthreads();  // the blocks' shared images before the next item
        // a field without full shuffle blocks has one encode item and no compaction: the
        // header is written here (its counter stays, no group sums were used)
        if (J.a.nb == 0 && threadIdx.x == 0) finish_field(J, 0u, final_loads(J));
    }
    if constexpr (!kList) {
        if (one.ahead_nr) range_ahead(one, total);
    }
}

template <bool kList>
__global__ void __launch_bounds__(256) k_compact_fields(const FieldJob* __restrict__ jobs, const Segment* __restrict__ segs,
                                                        uint32_t nseg, uint32_t total, const __grid_constant__ FieldJob one)
{
    pdl_wait();
    pdl_trigger();
    for (uint32_t k = blockIdx.x; k < total; k += gridDim.x) {
        uint32_t f = 0, i = k;
        if (kList) locate(segs, nseg, k, f, i);
        compact_item(kList ? jobs[f] : one, i);
    }
}

// One warp looks back from tile 1 at tile 0, which nothing publishes in this epoch: the
// bounded wait must give up and raise kStatusTimeout (fz_selftest_wait_timeout).
__global__ void k_wait_selftest(const uint64_t* state, const uint32_t* epoch, uint32_t* status)
{
    // the current device epoch has not been used by any launch yet
    const uint32_t e    = __ldcg(epoch);
    uint32_t       excl = 0, ovf = 0;
    lookback(state, 1, e, status, excl, ovf);
}

cudaError_t launch_wait_selftest(const uint64_t* state, const uint32_t* epoch, uint32_t* status, cudaStream_t s)
{
    k_wait_selftest<<<1, 32, 0, s>>>(state, epoch, status);
    return cudaGetLastError();
}

// Resident CTAs of a kernel on the current device (SM count x CTAs per SM), after the
// device's opt-in to more than 48 KiB of dynamic shared memory where the kernel needs it;
// 0 when a query fails.
template <typename K>
static uint32_t resident_ctas(K kernel, int threads, int dyn_smem = 0)
{
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    // the opt-in is needed once static + dynamic shared memory passes 48 KiB; made for any
    // dynamic size (it only raises the kernel's limit)
    if (dyn_smem > 0 &&
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, dyn_smem) != cudaSuccess) return 0;
    return (uint32_t)std::max(1, sms * std::max(per_sm, 1));
}

cudaError_t launch_range(const float* in, uint32_t n, uint32_t* mm, uint32_t* status, uint32_t* callw,
                         cudaStream_t s)
{
    const uint64_t want = cdiv(n / 4, 256ull * kRangeUnroll);  // n < 2^31: at most 2^18 CTAs
    const uint32_t ctas = (uint32_t)std::max<uint64_t>(1, want);
    k_range<<<ctas, 256, 0, s>>>(in, n, mm, status, callw);
    return cudaGetLastError();
}






// Resident CTAs of each list-compression kernel on the current device, cached per device
// (ordinals below 64): [0] range, [1..3] encode<1..3>, [4] compaction.
static uint32_t list_wave(int which, bool list)
{
    static std::atomic<uint32_t> cache[64][2][5];
    int                          dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::atomic<uint32_t>* slot = (dev >= 0 && dev < 64) ? &cache[dev][list ? 1 : 0][which] : nullptr;
    uint32_t               w    = slot ? slot->load(std::memory_order_acquire) : 0u;
    if (w) return w;
    constexpr int T = kCompressWarps * 32;
    // resident_ctas also opts the encode kernels in to their dynamic shared memory
    if (list) {
        w = which == 0 ? resident_ctas(k_range_fields<true>, T)
            : which == 1 ? resident_ctas(k_encode_fields<1, true>, T, encode_smem<1>())
            : which == 2 ? resident_ctas(k_encode_fields<2, true>, T, encode_smem<2>())
            : which == 3 ? resident_ctas(k_encode_fields<3, true>, T, encode_smem<3>())
                         : resident_ctas(k_compact_fields<true>, T);
    } else {
        w = which == 0 ? resident_ctas(k_range_fields<false>, T)
            : which == 1 ? resident_ctas(k_encode_fields<1, false>, T, encode_smem<1>())
            : which == 2 ? resident_ctas(k_encode_fields<2, false>, T, encode_smem<2>())
            : which == 3 ? resident_ctas(k_encode_fields<3, false>, T, encode_smem<3>())
                         : resident_ctas(k_compact_fields<false>, T);
    }
    if (slot) slot->store(w, std::memory_order_release);
    return w;
}

cudaError_t launch_fields(FieldPhase phase, int nd, const FieldJob* jobs, const Segment* segs, uint32_t nseg,
                          uint32_t total, const FieldJob& one, cudaStream_t s, uint32_t min_ctas)
{
    if (!total) return cudaSuccess;
    const bool list = jobs != nullptr;
    if (list && (!segs || !nseg)) return cudaErrorInvalidValue;
    const int      which = phase == FieldPhase::Range ? 0 : phase == FieldPhase::Encode ? nd : 4;
    const uint32_t wave  = list_wave(which, list);
    if (!wave) return cudaErrorInvalidDevice;
    const dim3 grid(std::min(std::max(total, min_ctas), wave)), block(kCompressWarps * 32);
    // eager launches with programmatic stream serialization: each kernel's CTAs may start
    // as the previous kernel of the call (or of the previous call on the stream) retires
    if (phase == FieldPhase::Range) {
        if (list) return launch_pdl(k_range_fields<true>, grid, block, 0, s, jobs, segs, nseg, total, one);
        return launch_pdl(k_range_fields<false>, grid, block, 0, s, jobs, segs, nseg, total, one);
    }
    if (phase == FieldPhase::Compact) {
        if (list) return launch_pdl(k_compact_fields<true>, grid, block, 0, s, jobs, segs, nseg, total, one);
        return launch_pdl(k_compact_fields<false>, grid, block, 0, s, jobs, segs, nseg, total, one);
    }
    if (list) {
        switch (nd) {
        case 1: return launch_pdl(k_encode_fields<1, true>, grid, block, encode_smem<1>(), s, jobs, segs, nseg, total, one);
        case 2: return launch_pdl(k_encode_fields<2, true>, grid, block, encode_smem<2>(), s, jobs, segs, nseg, total, one);
        default: return launch_pdl(k_encode_fields<3, true>, grid, block, encode_smem<3>(), s, jobs, segs, nseg, total, one);
        }
    }
    switch (nd) {
    case 1: return launch_pdl(k_encode_fields<1, false>, grid, block, encode_smem<1>(), s, jobs, segs, nseg, total, one);
    case 2: return launch_pdl(k_encode_fields<2, false>, grid, block, encode_smem<2>(), s, jobs, segs, nseg, total, one);
    default: return launch_pdl(k_encode_fields<3, false>, grid, block, encode_smem<3>(), s, jobs, segs, nseg, total, one);
    }
}

// One resident wave of k_compress<ND> on the current device.  The 64 KiB of dynamic shared
// memory needs a per-device opt-in, and the wave depends on the device's SM count, so
// both are done and cached per device (device ordinals below 64; others are computed on
// every call).
static uint32_t compress_wave(int nd)
{
    constexpr int                       kSmem = 2 * kCompressWarps * kBlockWords * 4;  // two tile buffers
    static std::atomic<uint32_t>        cache[64][3];
    int                                 dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::atomic<uint32_t>* slot = (dev >= 0 && dev < 64) ? &cache[dev][nd - 1] : nullptr;
    uint32_t               w    = slot ? slot->load(std::memory_order_acquire) : 0u;
    if (w) return w;
    w = nd == 1 ? resident_ctas(k_compress<1>, kCompressWarps * 32, kSmem)
        : nd == 2 ? resident_ctas(k_compress<2>, kCompressWarps * 32, kSmem)
                  : resident_ctas(k_compress<3>, kCompressWarps * 32, kSmem);
    if (slot) slot->store(w, std::memory_order_release);
    return w;
}

cudaError_t launch_compress(const CompressArgs& a, cudaStream_t s)
{
    // persistent: min(tiles, one resident wave) CTAs; a tile is 8 shuffle blocks
    constexpr int  kSmem = 2 * kCompressWarps * kBlockWords * 4;  // two tile buffers
    const uint32_t wave  = compress_wave((int)a.ndim);
    if (!wave) return cudaErrorInvalidDevice;
    const uint32_t nct  = (uint32_t)cdiv(a.ntiles, kCompressWarps);
    const uint32_t ctas = std::min(nct, wave);
    switch (a.ndim) {
    case 1: k_compress<1><<<ctas, kCompressWarps * 32, kSmem, s>>>(a); break;
    case 2: k_compress<2><<<ctas, kCompressWarps * 32, kSmem, s>>>(a); break;
    default: k_compress<3><<<ctas, kCompressWarps * 32, kSmem, s>>>(a); break;
    }
    return cudaGetLastError();
}

// =================================================== stage-level kernels ==
// fz_lorenzo_construct: codes of [0, x*y*z) into a u16 array (launch_construct_
// LorenzoI_var, lorenzo_var.cuh:520-597).  One warp per 128 consecutive elements.
template <int ND>
__global__ void __launch_bounds__(256) k_lorenzo_codes(const float* __restrict__ in, uint16_t* q,
                                                       uint8_t* signum, Geo g, float r)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t e0   = warp * 128 + lane * 4;
    if (warp * 128 >= g.nl) return;  // warp-uniform
    uint32_t c[4], ovf = 0, sgn = 0;
    codes4<ND>(in, g, e0, r, lane, c, ovf, sgn);
    if (e0 + 3 < g.nl) {
        *reinterpret_cast<uint2*>(q + e0) = make_uint2(c[0] | (c[1] << 16), c[2] | (c[3] << 16));
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (e0 + j < g.nl) q[e0 + j] = (uint16_t)c[j];
    }
    if (ND == 1 && signum) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (e0 + j < g.nl) signum[e0 + j] = (sgn >> j) & 1u;
    }
}

cudaError_t launch_lorenzo_construct(const float* in, uint16_t* q, uint8_t* signum, uint32_t x,
                                     uint32_t y, uint32_t z, float ebx2_r, cudaStream_t s)
{
    Geo g;
    g.x = x, g.y = y, g.xy = x * y, g.nl = x * y * z, g.lim = g.nl;
    g.dx = make_fastdiv(x), g.dxy = make_fastdiv(g.xy);
    g.al_x = (x % 4) == 0, g.al_xy = (g.xy % 4) == 0, g.al_xyx = ((g.xy + x) % 4) == 0;
    const int      nd    = (z == 1 && y == 1) ? 1 : (z == 1 ? 2 : 3);
    const uint32_t warps = (uint32_t)cdiv(g.nl, 128);
    const uint32_t ctas  = (uint32_t)cdiv(warps, 8);
    if (nd == 1) k_lorenzo_codes<1><<<ctas, 256, 0, s>>>(in, q, signum, g, ebx2_r);
    else if (nd == 2) k_lorenzo_codes<2><<<ctas, 256, 0, s>>>(in, q, signum, g, ebx2_r);
    else k_lorenzo_codes<3><<<ctas, 256, 0, s>>>(in, q, signum, g, ebx2_r);
    return cudaGetLastError();
}

// fz_bitshuffle_flag: bitshuffleAndBitflag over floor(n/2048) blocks (fz.cu:61-111)
// plus the raw tail copy (fz.cu:155) and zeroed flags past the last full block.
__global__ void __launch_bounds__(256) k_bitshuffle(const uint32_t* __restrict__ in, uint32_t* out,
                                                    uint32_t n_codes, uint32_t* bitflag,
                                                    uint32_t* byteflag)
{
    __shared__ __align__(16) uint32_t smem[8][kBlockWords];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t t    = blockIdx.x * 8 + wid;
    const uint32_t nb   = n_codes / kBlockCodes;
    const uint32_t nw   = (uint32_t)cdiv(n_codes, 256);
    uint32_t*      sm   = smem[wid];
    if (t < nb) {
        const uint4* src = reinterpret_cast<const uint4*>(in + (size_t)t * kBlockWords);
#pragma unroll
        for (uint32_t i = 0; i < 8; ++i) {
            const uint32_t q = lane + 32 * i;
            *reinterpret_cast<uint4*>(sm + swz(q)) = src[q];
        }
        __syncwarp();
        uint32_t w[32];
#pragma unroll
        for (uint32_t tt = 0; tt < 8; ++tt) {
            const uint4 v = *reinterpret_cast<const uint4*>(sm + swz(lane * 8 + tt));
            w[4 * tt] = v.x, w[4 * tt + 1] = v.y, w[4 * tt + 2] = v.z, w[4 * tt + 3] = v.w;
        }
        transpose32(w);
        __syncwarp();
#pragma unroll
        for (uint32_t p = 0; p < 32; ++p) sm[p * 32 + lane] = w[p];
        __syncwarp();
        uint4* dst = reinterpret_cast<uint4*>(out + (size_t)t * kBlockWords);
#pragma unroll
        for (uint32_t i = 0; i < 8; ++i) {
            const uint4 v = *reinterpret_cast<const uint4*>(sm + (lane + 32 * i) * 4);
            dst[lane + 32 * i] = v;
            const bool f = (v.x | v.y | v.z | v.w) != 0;
            byteflag[(size_t)t * kChunks + lane + 32 * i] = f;
            const uint32_t b = __ballot_sync(kFull, f);
            if (lane == 0) bitflag[(size_t)t * 8 + i] = b;
        }
        return;
    }
    if (t == nb) {
        // tail: raw copy of the remaining bytes (2n total) and zero flags
        const uint8_t* s8 = reinterpret_cast<const uint8_t*>(in);
        uint8_t*       d8 = reinterpret_cast<uint8_t*>(out);
        for (uint64_t b = (uint64_t)nb * 4096 + lane; b < 2ull * n_codes; b += 32) d8[b] = s8[b];
        for (uint32_t i = nb * 8 + lane; i < nw; i += 32) bitflag[i] = 0;
        for (uint32_t i = nb * kChunks + lane; i < 32 * nw; i += 32) byteflag[i] = 0;
    }
}

cudaError_t launch_bitshuffle_flag(const uint32_t* in, uint32_t* out, uint32_t n_codes,
                                   uint32_t* bitflag, uint32_t* byteflag, cudaStream_t s)
{
    const uint32_t tiles = n_codes / kBlockCodes + 1;
    k_bitshuffle<<<(uint32_t)cdiv(tiles, 8), 256, 0, s>>>(in, out, n_codes, bitflag, byteflag);
    return cudaGetLastError();
}

// fz_scan_encode: exclusive scan of M u32 flags (cub::DeviceScan::ExclusiveSum,
// fz.cu:187-192) + total (fz.cu:194-201) + compaction (encodeDebug, fz.cu:49-59).
// One warp per 256 flags, decoupled look-back across warps.
__global__ void __launch_bounds__(256) k_scan_encode(const uint8_t* __restrict__ shuffled,
                                                     const uint32_t* __restrict__ flags,
                                                     uint32_t n_codes, uint32_t m,
                                                     uint32_t* presum, uint8_t* out,
                                                     uint64_t* state, uint32_t* ticket,
                                                     uint32_t* status, uint32_t* total,
                                                     uint32_t* epoch_word)
{
    __shared__ uint32_t cta_tile, s_epoch;
    const uint32_t      lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        s_epoch = __ldcg(epoch_word);
        __threadfence();
        cta_tile = take_ticket(ticket, epoch_word, gridDim.x).tile;
    }
    __syncthreads();
    const uint32_t epoch = s_epoch;
    const uint32_t t      = cta_tile * 8 + wid;
    const uint32_t ntiles = m / 256;  // m = 32 * ceil(n/256), a multiple of 32; tiles of 256
    const uint32_t ntl    = (m + 255) / 256;
    if (t >= ntl) return;
    (void)ntiles;
    uint32_t bm[8], cnt = 0;
#pragma unroll
    for (uint32_t i = 0; i < 8; ++i) {
        const uint32_t idx = t * 256 + 32 * i + lane;
        bm[i] = __ballot_sync(kFull, idx < m && flags[idx] != 0);
        cnt += __popc(bm[i]);
    }
    uint32_t excl = 0, povf = 0;
    if (t == 0) {
        if (lane == 0) publish(state, 0, epoch, kFlagIncl, 0, cnt);
    } else {
        if (lane == 0) publish(state, t, epoch, kFlagAgg, 0, cnt);
        lookback(state, t, epoch, status, excl, povf);
        if (lane == 0) publish(state, t, epoch, kFlagIncl, 0, excl + cnt);
    }
    const uint32_t lt       = lanemask_lt();
    uint32_t       pre      = excl;
    const uint64_t srcbytes = 2ull * n_codes;
#pragma unroll
    for (uint32_t i = 0; i < 8; ++i) {
        const uint32_t idx  = t * 256 + 32 * i + lane;
        const uint32_t rank = pre + __popc(bm[i] & lt);
        if (presum && idx < m) presum[idx] = rank;
        if ((bm[i] >> lane) & 1u && out) {
            const uint64_t b0 = 16ull * idx;
            if (b0 + 16 <= srcbytes) {
                reinterpret_cast<uint4*>(out)[rank] = reinterpret_cast<const uint4*>(shuffled)[idx];
            } else {
                for (int k = 0; k < 16; ++k) out[16ull * rank + k] = b0 + k < srcbytes ? shuffled[b0 + k] : 0;
            }
        }
        pre += __popc(bm[i]);
    }
    if (t == ntl - 1 && lane == 0) {
        if (presum) presum[m] = pre;
        *total = pre;
    }
}

cudaError_t launch_scan_encode(const uint8_t* shuffled, const uint32_t* byteflag,
                               uint32_t n_codes, uint32_t* presum, uint8_t* out,
                               uint64_t* state, uint32_t* ticket, uint32_t* status,
                               uint32_t* total, uint32_t* epoch, cudaStream_t s)
{
    const uint32_t m     = 32u * (uint32_t)cdiv(n_codes, 256);
    const uint32_t tiles = (uint32_t)cdiv(m, 256);
    k_scan_encode<<<(uint32_t)cdiv(tiles, 8), 256, 0, s>>>(shuffled, byteflag, n_codes, m, presum,
                                                           out, state, ticket, status, total, epoch);
    return cudaGetLastError();
}

}  // namespace fz
