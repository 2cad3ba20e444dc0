// fz_decompress.cu -- decompression kernels (the inverse of fz_compress.cu).
//
//   k_decode   one warp per 2048-code shuffle block: popcounts of its 8 bitmap words,
//              decoupled look-back for its first chunk, gather of the flagged 16-byte
//              chunks (unflagged ones are zero), inverse 32x32 bit transposes, and a
//              coalesced write of the 2048 codes.  The tail block copies the sidecar.
//   k_recon    inverse Lorenzo on the codes: per-tile inclusive prefix sums in 32-bit
//              integers (1D 256, 2D 16x16, 3D 8x8x8 -- the tiling of x_lorenzo_{1d,2d,
//              3d}, lorenzo_var.cuh:297-518), then (float)p * ebx2.
//
// The reference has no working FZ decompressor (its x_lorenzo kernels read a separate
// signum array that its compressor never writes), so this path is the exact inverse of
// the compressed format rather than a restatement.
#include <algorithm>

#include "fz_internal.h"

namespace fz {

constexpr int kDecodeWarps = 8;

__device__ __forceinline__ uint32_t swz_d(uint32_t q)
{
    const uint32_t g = q >> 3, t = q & 7u;
    return ((g << 3) | (t ^ (g & 7u))) << 2;
}

__global__ void __launch_bounds__(kDecodeWarps * 32) k_decode(const DecodeArgs a)
{
    __shared__ __align__(16) uint32_t smem[kDecodeWarps][kBlockWords];
    __shared__ uint32_t               s_cnt[kDecodeWarps];
    __shared__ uint32_t               cta_tile, s_excl;
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    uint32_t*      sm   = smem[wid];
    if (threadIdx.x == 0) {
        const uint32_t c = atomicAdd(a.ticket, 1u);
        if (c == gridDim.x - 1) atomicExch(a.ticket, 0u);
        cta_tile = c;
    }
    __syncthreads();
    const uint32_t ct = cta_tile;
    const uint32_t t  = ct * kDecodeWarps + wid;

    uint32_t bm[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cnt = 0;
    if (t < a.nb) {
        const uint4* A4 = reinterpret_cast<const uint4*>(a.st + a.off_a) + 2 * (size_t)t;
        const uint4  b0 = __ldg(A4), b1 = __ldg(A4 + 1);
        bm[0] = b0.x, bm[1] = b0.y, bm[2] = b0.z, bm[3] = b0.w;
        bm[4] = b1.x, bm[5] = b1.y, bm[6] = b1.z, bm[7] = b1.w;
#pragma unroll
        for (int i = 0; i < 8; ++i) cnt += __popc(bm[i]);
    }
    // CTA total, then the CTA's first chunk by decoupled look-back
    if (lane == 0) s_cnt[wid] = cnt;
    __syncthreads();
    if (wid == 0) {
        const uint32_t tot  = __reduce_add_sync(kFull, lane < kDecodeWarps ? s_cnt[lane] : 0u);
        uint32_t       excl = 0, povf = 0;
        if (ct == 0) {
            if (lane == 0) publish(a.state, 0, a.epoch, kFlagIncl, 0, tot);
        } else {
            if (lane == 0) publish(a.state, ct, a.epoch, kFlagAgg, 0, tot);
            lookback(a.state, ct, a.epoch, a.status, excl, povf);
            if (lane == 0) publish(a.state, ct, a.epoch, kFlagIncl, 0, excl + tot);
        }
        if (lane == 0) {
            s_excl = excl;
            if (ct == gridDim.x - 1 && excl + tot != a.nnz) atomicOr(a.status, kStatusCorrupt);
        }
    }
    __syncthreads();

    if (t < a.nb) {
        uint32_t pre = s_excl;
        for (uint32_t w2 = 0; w2 < wid; ++w2) pre += s_cnt[w2];
        // gather: chunk c = lane + 32 i into the shuffled image S (words 4c..4c+3)
        const uint4*   B   = reinterpret_cast<const uint4*>(a.st + a.off_b);
        const uint32_t lt  = lanemask_lt();
        bool           bad = false;
#pragma unroll
        for (uint32_t i = 0; i < 8; ++i) {
            uint4          v    = make_uint4(0, 0, 0, 0);
            const uint32_t rank = pre + __popc(bm[i] & lt);
            if ((bm[i] >> lane) & 1u) {
                if (rank < a.nnz) v = __ldg(B + rank);
                else bad = true;  // bitmap claims more chunks than the stream holds
            }
            *reinterpret_cast<uint4*>(sm + (lane + 32 * i) * 4) = v;
            pre += __popc(bm[i]);
        }
        if (bad) atomicOr(a.status, kStatusCorrupt);
        __syncwarp();
        // un-shuffle: W[g*32 + j] bit p = S[p*32 + g] bit j (the transpose is an involution)
        uint32_t w[32];
#pragma unroll
        for (uint32_t p = 0; p < 32; ++p) w[p] = sm[p * 32 + lane];
        transpose32(w);
        __syncwarp();
#pragma unroll
        for (uint32_t tt = 0; tt < 8; ++tt)
            *reinterpret_cast<uint4*>(sm + swz_d(lane * 8 + tt)) =
                make_uint4(w[4 * tt], w[4 * tt + 1], w[4 * tt + 2], w[4 * tt + 3]);
        __syncwarp();
        uint4* dst = reinterpret_cast<uint4*>(a.codes) + (size_t)t * 256;
#pragma unroll
        for (uint32_t i = 0; i < 8; ++i) dst[lane + 32 * i] = *reinterpret_cast<const uint4*>(sm + swz_d(lane + 32 * i));
    } else if (t == a.nb && a.tail) {
        // tail block: raw codes from the sidecar, or zeros without one
        const uint16_t* src  = a.mode == 1 ? reinterpret_cast<const uint16_t*>(a.st + a.off_c) : nullptr;
        uint16_t*       dstc = a.codes + (size_t)a.nb * kBlockCodes;
        for (uint32_t i = lane; i < a.tail; i += 32) dstc[i] = src ? src[i] : (uint16_t)0;
    }
}

cudaError_t launch_decode(const DecodeArgs& a, cudaStream_t s)
{
    const uint32_t ntiles = a.nb + (a.tail ? 1u : 0u);
    k_decode<<<(uint32_t)cdiv(ntiles, kDecodeWarps), kDecodeWarps * 32, 0, s>>>(a);
    return cudaGetLastError();
}

// ------------------------------------------------------------- recon --
__device__ __forceinline__ uint32_t sm_decode(uint32_t c)
{
    const uint32_t mag = c & 0x7FFFu;
    return (c & 0x8000u) ? 0u - mag : mag;
}

// 2D: a CTA covers 16 rows x 512 columns; lane owns 4 consecutive columns, lanes 4k..4k+3
// one 16-column tile row.  Row prefix: serial over 4 + quad shuffle scan; column prefix:
// running sum over the 16 rows.
__global__ void __launch_bounds__(128) k_recon2d(const ReconArgs a)
{
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t c0   = blockIdx.x * 512 + wid * 128 + lane * 4;
    const uint32_t r0   = blockIdx.y * 16;
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
            d[0] = sm_decode(v.x & 0xFFFFu), d[1] = sm_decode(v.x >> 16);
            d[2] = sm_decode(v.y & 0xFFFFu), d[3] = sm_decode(v.y >> 16);
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
__global__ void __launch_bounds__(128) k_recon3d(const ReconArgs a)
{
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t c0   = blockIdx.x * 128 + lane * 4;
    const uint32_t y0   = (blockIdx.y * 4 + wid) * 8;
    const uint32_t z0   = blockIdx.z * 8;
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
                    d[0] = sm_decode(v.x & 0xFFFFu), d[1] = sm_decode(v.x >> 16);
                    d[2] = sm_decode(v.y & 0xFFFFu), d[3] = sm_decode(v.y >> 16);
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

cudaError_t launch_reconstruct(const ReconArgs& a, cudaStream_t s)
{
    const int nd = (a.z == 1 && a.y == 1) ? 1 : (a.z == 1 ? 2 : 3);
    if (nd == 1) {
        k_recon1d<<<(uint32_t)cdiv(cdiv(a.nl, 256), 8), 256, 0, s>>>(a);
    } else if (nd == 2) {
        dim3 grid((uint32_t)cdiv(a.x, 512), (uint32_t)cdiv(a.y, 16));
        k_recon2d<<<grid, 128, 0, s>>>(a);
    } else {
        dim3 grid((uint32_t)cdiv(a.x, 128), (uint32_t)cdiv(cdiv(a.y, 8), 4), (uint32_t)cdiv(a.z, 8));
        k_recon3d<<<grid, 128, 0, s>>>(a);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && a.n > a.nl) {
        k_zero_tail<<<(uint32_t)std::min<uint64_t>(cdiv(a.n - a.nl, 256), 1024), 256, 0, s>>>(a.out, a.nl, a.n);
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace fz
