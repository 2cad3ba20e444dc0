/*
 * fzoracle.c -- ORACLE (test infrastructure only; never linked into the product).
 *
 * A plain-C (C11 + OpenMP) restatement of FZ-GPU's compression path and of the
 * inverse the product defines.  Used by tests/ as the bit-exact checker, by the smoke
 * check, and as the timed CPU baseline of bench.py.  References are to the FZ-GPU
 * source tree: fz.cu and include/kernel/lorenzo_var.cuh.
 *
 * Build: -O3 -fopenmp -ffp-contract=off (no FMA contraction; float evaluation order
 * below is the reference's).
 */
#include "fzoracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define BLOCK_CODES 2048u
#define BLOCK_WORDS 1024u
#define CHUNKS_PER_BLOCK 256u
#define HDR 64u

static inline uint64_t cdiv(uint64_t a, uint64_t b) { return (a + b - 1) / b; }
static inline uint64_t pad16(uint64_t a) { return (a + 15) & ~(uint64_t)15; }

int fzo_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void fzo_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* lorenzo_var.cuh:537-544: 1D iff z==1 and y==1, 2D iff z==1, else 3D. */
int fzo_ndim(uint32_t x, uint32_t y, uint32_t z)
{
    (void)x;
    if (z == 1 && y == 1) return 1;
    if (z == 1) return 2;
    return 3;
}

/* fz.cu:137: *max_element - *min_element over the whole file, in float.  For NaN-free
   input the order of the scan does not matter. */
void fzo_value_range(const float* data, uint64_t n, float* mn, float* mx)
{
    float lo = data[0], hi = data[0];
#pragma omp parallel for reduction(max : hi) reduction(min : lo) schedule(static)
    for (uint64_t i = 0; i < n; i++) {
        float v = data[i];
        if (v > hi) hi = v;
        if (v < lo) lo = v;
    }
    *mn = lo;
    *mx = hi;
}

/* lorenzo_var.cuh:562-563: ebx2 = eb*2 (double), ebx2_r = 1/ebx2 (double), passed as FP=float. */
float fzo_ebx2_r(double eb_abs)
{
    double ebx2 = eb_abs * 2;
    double r    = 1 / ebx2;
    return (float)r;
}
/* lorenzo_var.cuh:641: the inverse scales by ebx2, passed as FP=float. */
float fzo_ebx2(double eb_abs) { return (float)(eb_abs * 2); }

/* static_cast<uint16_t>(fabs(delta)) as the device evaluates it (lorenzo_var.cuh:53,169,
   289): a float-to-u32 conversion rounding toward zero that clamps to [0, 2^32-1] and
   maps NaN to 0, then the low 16 bits.  So |d| = 70000 gives 4464 and Inf gives 0xFFFF.
   Pinned by the reference kernels' own output on a GB300 (the crafted-limits
   fixtures in tests/golden). */
uint16_t fzo_f2u16(float v)
{
    if (!(v > 0.0f)) return 0;                  /* +-0 and NaN */
    if (v >= 4294967296.0f) return 0xFFFFu;     /* clamps to 2^32 - 1 */
    return (uint16_t)((uint32_t)v & 0xFFFFu);
}

/* Prequantisation, lorenzo_var.cuh:81,125,265: round(data * ebx2_r) in float, ties away
   from zero. */
static inline float pq(const float* d, uint64_t i, float r) { return roundf(d[i] * r); }

static inline uint16_t pack_signed(float d)
{
    /* lorenzo_var.cuh:169-171 (and :53-54, :289-290): (u16)|d| | (d<0)<<15, OR in int. */
    uint16_t t = fzo_f2u16(fabsf(d));
    t          = (uint16_t)(t | ((d < 0) << 15));
    return t;
}

uint32_t fzo_lorenzo_construct(const float* data, uint64_t n, uint32_t x, uint32_t y, uint32_t z,
                               float r, uint16_t* codes, uint8_t* signum)
{
    int      nd  = fzo_ndim(x, y, z);
    uint32_t ovf = 0;
    uint64_t nl = (uint64_t)x * y * z;
    /* elements outside len3 keep the memset 0 (fz.cu:145) */
#pragma omp parallel for schedule(static)
    for (uint64_t i = nl; i < n; i++) {
        codes[i] = 0;
        if (signum) signum[i] = 0;
    }

    if (nd == 1) {
        /* c_lorenzo_1d1l<.., 256, 4> (lorenzo_var.cuh:176-214): 256-element blocks;
           delta = p[i] - p[i-1], p[-1] = 0 at each block start; pred1d<..,true> stores
           the sign bit only for each thread's first element (i%4 == 0, :51-56), the
           other three store the magnitude alone (:58-63). */
        uint64_t nblk = cdiv(nl, 256);
#pragma omp parallel for reduction(| : ovf) schedule(static)
        for (uint64_t b = 0; b < nblk; b++) {
            float prev = 0.0f;
            for (uint32_t k = 0; k < 256; k++) {
                uint64_t i = b * 256 + k;
                if (i >= nl) break;
                float    p = pq(data, i, r);
                float    d = p - prev;
                uint16_t c = fzo_f2u16(fabsf(d));
                if ((k & 3) == 0) c = (uint16_t)(c | ((d < 0) << 15));
                ovf |= !(fabsf(d) < ((k & 3) == 0 ? 32768.0f : 65536.0f));
                codes[i] = c;
                if (signum) signum[i] = d < 0;
                prev = p;
            }
        }
        return ovf;
    }

    if (nd == 2) {
        /* c_lorenzo_2d1l_16x16data_mapto16x2 (lorenzo_var.cuh:110-174,216-238): 16x16
           tiles, zero outside the tile; delta = (c - n) - (w - nw) in that float order
           (pred2d :139-143). */
#pragma omp parallel for reduction(| : ovf) schedule(static)
        for (uint64_t row = 0; row < y; row++) {
            int rin = (row % 16) != 0;
            for (uint64_t col = 0; col < x; col++) {
                uint64_t i   = row * x + col;
                int      cin = (col % 16) != 0;
                float    c   = pq(data, i, r);
                float    nn  = rin ? pq(data, i - x, r) : 0.0f;
                float    w   = cin ? pq(data, i - 1, r) : 0.0f;
                float    nw  = (rin && cin) ? pq(data, i - x - 1, r) : 0.0f;
                float    d   = (c - nn) - (w - nw);
                codes[i]     = pack_signed(d);
                ovf |= !(fabsf(d) < 32768.0f);
            }
        }
        return ovf;
    }

    /* c_lorenzo_3d1l_32x8x8data_mapto32x1x8 (lorenzo_var.cuh:240-295): effective 8x8x8
       tiles (x = TIX % 8, :271); the 7-term expression of :277-283, left to right. */
    uint64_t xy = (uint64_t)x * y;
#pragma omp parallel for collapse(2) reduction(| : ovf) schedule(static)
    for (uint64_t zz = 0; zz < z; zz++) {
        for (uint64_t yy = 0; yy < y; yy++) {
            int zi = (zz % 8) != 0, yi = (yy % 8) != 0;
            for (uint64_t xx = 0; xx < x; xx++) {
                int      xi  = (xx % 8) != 0;
                uint64_t i   = zz * xy + yy * x + xx;
                float    c   = pq(data, i, r);
                float    a   = (zi && yi && xi) ? pq(data, i - xy - x - 1, r) : 0.0f;
                float    b   = (yi && xi) ? pq(data, i - x - 1, r) : 0.0f;
                float    cc  = (zi && xi) ? pq(data, i - xy - 1, r) : 0.0f;
                float    dd  = (zi && yi) ? pq(data, i - xy - x, r) : 0.0f;
                float    e   = xi ? pq(data, i - 1, r) : 0.0f;
                float    f   = yi ? pq(data, i - x, r) : 0.0f;
                float    g   = zi ? pq(data, i - xy, r) : 0.0f;
                float    d   = c - (a - b - cc - dd + e + f + g);
                codes[i]     = pack_signed(d);
                ovf |= !(fabsf(d) < 32768.0f);
            }
        }
    }
    return ovf;
}

/* Transpose a 32x32 bit matrix held as 32 words (bit c of a[r] = M[r][c]) so that bit c
   of a[r] becomes M[c][r]: recursive swap of the off-diagonal blocks, sizes 16..1. */
static void transpose32(uint32_t a[32])
{
    static const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u,
                                      0x55555555u};
    for (int s = 0, j = 16; s < 5; s++, j >>= 1) {
        uint32_t m = masks[s];
        for (int r = 0; r < 32; r++) {
            if (r & j) continue;
            uint32_t lo = a[r], hi = a[r + j];
            a[r]        = (lo & m) | ((hi << j) & ~m);
            a[r + j]    = (hi & ~m) | ((lo >> j) & m);
        }
    }
}

/* bitshuffleAndBitflag (fz.cu:61-111): block b of 1024 words; warp g (threadIdx.y)
   ballots bit p of its 32 words (:75-79), giving S[b*1024 + p*32 + g] bit j =
   bit p of W[b*1024 + g*32 + j] (:82).  Chunk flag = OR of 4 words != 0 (:84-91);
   bitmap word 8b+k bit j = flag 256b+32k+j (:95-99,109). */
void fzo_bitshuffle_flag(const uint16_t* codes, uint64_t n, uint32_t* S, uint32_t* F,
                         uint32_t* B)
{
    uint64_t nb = n / BLOCK_CODES;
    uint64_t nw = cdiv(n, 256);
    /* raw copy of the codes (fz.cu:155): the tail keeps it */
    memset(S, 0, cdiv(n, 2) * 4);
    memcpy(S, codes, n * 2);
    memset(F, 0, nw * 32 * 4);
    memset(B, 0, nw * 4);
#pragma omp parallel for schedule(static)
    for (uint64_t b = 0; b < nb; b++) {
        uint32_t*       s = S + b * BLOCK_WORDS;
        const uint16_t* c = codes + b * BLOCK_CODES;
        uint32_t        blk[BLOCK_WORDS];
        for (uint32_t g = 0; g < 32; g++) {
            uint32_t a[32];
            for (uint32_t j = 0; j < 32; j++) {
                uint32_t k = g * 32 + j;
                a[j]       = (uint32_t)c[2 * k] | ((uint32_t)c[2 * k + 1] << 16);
            }
            transpose32(a);
            for (uint32_t p = 0; p < 32; p++) blk[p * 32 + g] = a[p];
        }
        memcpy(s, blk, sizeof(blk));
        for (uint32_t k = 0; k < 8; k++) {
            uint32_t word = 0;
            for (uint32_t j = 0; j < 32; j++) {
                uint32_t ch = k * 32 + j;
                uint32_t f  = (blk[4 * ch] | blk[4 * ch + 1] | blk[4 * ch + 2] | blk[4 * ch + 3]) != 0;
                F[b * CHUNKS_PER_BLOCK + ch] = f;
                word |= f << j;
            }
            B[b * 8 + k] = word;
        }
    }
}

/* cub::DeviceScan::ExclusiveSum over M = 32*ceil(n/256) flags, total = P[M-1] + F[M-1]
   written to P[M] (fz.cu:187-201), then encodeDebug's intended compaction: chunk t with
   P[t+1] != P[t] is copied to out[16*P[t]] (fz.cu:49-59). */
/* Block-wise parallel form: every thread counts the flags of its contiguous range, one
   thread turns the counts into exclusive range offsets, then every thread writes its
   prefix sums and copies its flagged chunks from its range's offset on.  The result is
   the serial scan's, whatever the thread count. */
uint64_t fzo_scan_encode(const uint32_t* S, const uint32_t* F, uint64_t n, uint32_t* P,
                         uint8_t* out)
{
    uint64_t  m     = 32 * cdiv(n, 256);
    int       nt    = fzo_threads();
    uint64_t* part  = (uint64_t*)calloc((size_t)nt + 1, sizeof(uint64_t));
    uint64_t  total = 0;
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num(), th = omp_get_num_threads();
#else
        int tid = 0, th = 1;
#endif
        uint64_t lo = m * (uint64_t)tid / (uint64_t)th, hi = m * (uint64_t)(tid + 1) / (uint64_t)th;
        uint64_t c  = 0;
        for (uint64_t t = lo; t < hi; t++) c += F[t] != 0;
        part[tid + 1] = c;
#pragma omp barrier
#pragma omp single
        {
            for (int k = 1; k <= th; k++) part[k] += part[k - 1];
            total = part[th];
        }
        uint64_t acc = part[tid];
        for (uint64_t t = lo; t < hi; t++) {
            if (P) P[t] = (uint32_t)acc;
            if (F[t] && out) memcpy(out + 16 * acc, (const uint8_t*)S + 16 * t, 16);
            acc += F[t] != 0;
        }
    }
    free(part);
    if (P) P[m] = (uint32_t)total;
    return total;
}

/* Chunk offset of every shuffle block (boff[b] = flagged chunks of blocks 0..b-1, the
   exclusive scan of fz.cu:187-192 at block granularity) from the bitmap: per-block counts
   in parallel, then their prefix.  Returns the total. */
static uint64_t block_offsets(const uint32_t* B, uint64_t nb, uint64_t* boff)
{
#pragma omp parallel for schedule(static)
    for (uint64_t b = 0; b < nb; b++) {
        uint64_t c = 0;
        for (int k = 0; k < 8; k++) c += (uint64_t)__builtin_popcount(B[b * 8 + k]);
        boff[b] = c;
    }
    uint64_t acc = 0;
    for (uint64_t b = 0; b < nb; b++) {
        uint64_t c = boff[b];
        boff[b]    = acc;
        acc += c;
    }
    boff[nb] = acc;
    return acc;
}

void fzo_layout(uint64_t n, int ndim, int mode, uint64_t* off_a, uint64_t* off_c,
                uint64_t* off_b, uint32_t* sidecar_bytes)
{
    uint64_t nw = cdiv(n, 256);
    uint64_t a  = HDR;
    uint64_t c  = a + pad16(4 * nw);
    uint64_t sc = 0;
    if (mode == 1) {
        sc += pad16(2 * (n % BLOCK_CODES));          /* raw tail codes */
        if (ndim == 1) sc += pad16(4 * cdiv(n, 32)); /* 1D sign bits */
        sc += pad16(4 * (n / BLOCK_CODES + 1));      /* chunk offset of each shuffle block */
    }
    *off_a         = a;
    *off_c         = c;
    *off_b         = c + sc;
    *sidecar_bytes = (uint32_t)sc;
}

static void put32(uint8_t* p, uint32_t v) { memcpy(p, &v, 4); }
static void put64(uint8_t* p, uint64_t v) { memcpy(p, &v, 8); }

uint64_t fzo_compress(const float* data, uint64_t n, uint32_t x, uint32_t y, uint32_t z,
                      double eb, int eb_mode, int mode, uint8_t* out)
{
    uint64_t nl = (uint64_t)x * y * z;
    if (n == 0 || x == 0 || y == 0 || z == 0 || nl > n || !(eb > 0)) return 0;
    int   nd    = fzo_ndim(x, y, z);
    float range = 0.0f;
    double eb_abs = eb;
    if (eb_mode == 1) {
        float mn, mx;
        int   bad = 0;
#pragma omp parallel for reduction(| : bad) schedule(static)
        for (uint64_t i = 0; i < n; i++) bad |= !isfinite(data[i]);
        if (bad) return 0; /* relative eb of a non-finite field */
        fzo_value_range(data, n, &mn, &mx);
        range  = mx - mn;
        eb_abs = eb * range; /* fz.cu:149: eb * range, double * float */
    }
    float r  = fzo_ebx2_r(eb_abs);
    float e2 = fzo_ebx2(eb_abs);

    uint16_t* codes = (uint16_t*)malloc(n * 2);
    uint8_t*  sg    = (nd == 1 && mode == 1) ? (uint8_t*)malloc(n) : NULL;
    uint64_t  nw    = cdiv(n, 256);
    uint32_t* S     = (uint32_t*)malloc(cdiv(n, 2) * 4);
    uint32_t* F     = (uint32_t*)malloc(nw * 32 * 4);
    uint32_t* B     = (uint32_t*)malloc(nw * 4);
    /* header flag bit 0: some delta did not fit its field (a signed code needs
       |d| < 32768, an unsigned 1D code |d| < 65536; NaN/Inf count as not fitting) */
    uint32_t flags = fzo_lorenzo_construct(data, n, x, y, z, r, codes, sg) ? 1u : 0u;

    fzo_bitshuffle_flag(codes, n, S, F, B);
    uint64_t off_a, off_c, off_b;
    uint32_t sc;
    fzo_layout(n, nd, mode, &off_a, &off_c, &off_b, &sc);
    memset(out, 0, off_b);
    uint64_t nnz = fzo_scan_encode(S, F, n, NULL, out + off_b);
    memcpy(out + off_a, B, nw * 4);
    if (mode == 1) {
        uint64_t nb   = n / BLOCK_CODES;
        uint64_t tail = n - nb * BLOCK_CODES;
        memcpy(out + off_c, codes + nb * BLOCK_CODES, tail * 2);
        uint64_t q = off_c + pad16(2 * tail);
        if (nd == 1) {
            /* one sign bit per element, bit i%8 of byte i/8 */
            uint8_t* sb = out + q;
            uint64_t nbytes = cdiv(n, 8);
#pragma omp parallel for schedule(static)
            for (uint64_t k = 0; k < nbytes; k++) {
                uint8_t v = 0;
                for (uint64_t i = 8 * k; i < 8 * k + 8 && i < n; i++) v |= (uint8_t)((sg[i] ? 1u : 0u) << (i & 7));
                sb[k] = v;
            }
            q += pad16(4 * cdiv(n, 32));
        }
        /* boff[b] = chunks of blocks 0..b-1, boff[nb] = nnz */
        uint64_t* boff = (uint64_t*)malloc((nb + 1) * 8);
        block_offsets(B, nb, boff);
        for (uint64_t b = 0; b <= nb; b++) put32(out + q + 4 * b, (uint32_t)boff[b]);
        free(boff);
    }
    /* header (include/fz.h, struct fz_header) */
    put32(out + 0, 0x31475A46u);
    out[4] = 1;
    out[5] = 0;
    out[6] = (uint8_t)mode;
    out[7] = (uint8_t)nd;
    put32(out + 8, x);
    put32(out + 12, y);
    put32(out + 16, z);
    put32(out + 20, flags);
    put64(out + 24, n);
    memcpy(out + 32, &eb_abs, 8);
    memcpy(out + 40, &r, 4);
    memcpy(out + 44, &e2, 4);
    put64(out + 48, nnz);
    memcpy(out + 56, &range, 4);
    put32(out + 60, sc);

    free(codes);
    free(sg);
    free(S);
    free(F);
    free(B);
    return off_b + 16 * nnz;
}

/* Inverse Lorenzo: per-tile inclusive prefix sums of the signed deltas (1D 256, 2D 16x16,
   3D 8x8x8 -- the tiling of x_lorenzo_{1d,2d,3d}, lorenzo_var.cuh:297-518) in wrapping
   32-bit integers, then (float)p * ebx2.  Elements at i >= x*y*z are 0. */
void fzo_lorenzo_reconstruct(const uint16_t* codes, const uint8_t* signbits, uint64_t n,
                             uint32_t x, uint32_t y, uint32_t z, float ebx2, float* out)
{
    int      nd = fzo_ndim(x, y, z);
    uint64_t nl = (uint64_t)x * y * z;
    for (uint64_t i = nl; i < n; i++) out[i] = 0.0f;

    if (nd == 1) {
        uint64_t nblk = cdiv(nl, 256);
#pragma omp parallel for schedule(static)
        for (uint64_t b = 0; b < nblk; b++) {
            uint32_t acc = 0;
            for (uint32_t k = 0; k < 256; k++) {
                uint64_t i = b * 256 + k;
                if (i >= nl) break;
                uint32_t c = codes[i], mag, neg;
                if ((k & 3) == 0) {
                    mag = c & 0x7FFFu;
                    neg = c >> 15;
                } else {
                    mag = c;
                    neg = signbits ? (signbits[i >> 3] >> (i & 7)) & 1u : 0u;
                }
                acc += neg ? (0u - mag) : mag;
                out[i] = (float)(int32_t)acc * ebx2;
            }
        }
        return;
    }

    if (nd == 2) {
        uint64_t tr = cdiv(y, 16), tc = cdiv(x, 16);
#pragma omp parallel for collapse(2) schedule(static)
        for (uint64_t a = 0; a < tr; a++) {
            for (uint64_t b = 0; b < tc; b++) {
                uint32_t colacc[16] = {0};
                for (uint64_t rr = a * 16; rr < a * 16 + 16 && rr < y; rr++) {
                    uint32_t rowacc = 0;
                    for (uint64_t cc = b * 16; cc < b * 16 + 16 && cc < x; cc++) {
                        uint64_t i   = rr * x + cc;
                        uint32_t c   = codes[i];
                        uint32_t mag = c & 0x7FFFu;
                        rowacc += (c >> 15) ? (0u - mag) : mag;
                        colacc[cc - b * 16] += rowacc;
                        out[i] = (float)(int32_t)colacc[cc - b * 16] * ebx2;
                    }
                }
            }
        }
        return;
    }

    uint64_t xy = (uint64_t)x * y;
    uint64_t tz = cdiv(z, 8), ty = cdiv(y, 8), tx = cdiv(x, 8);
#pragma omp parallel for collapse(3) schedule(static)
    for (uint64_t a = 0; a < tz; a++) {
        for (uint64_t b = 0; b < ty; b++) {
            for (uint64_t cidx = 0; cidx < tx; cidx++) {
                uint32_t plane[8][8];
                memset(plane, 0, sizeof(plane));
                for (uint64_t zz = a * 8; zz < a * 8 + 8 && zz < z; zz++) {
                    uint32_t colacc[8] = {0};
                    for (uint64_t yy = b * 8; yy < b * 8 + 8 && yy < y; yy++) {
                        uint32_t rowacc = 0;
                        for (uint64_t xx = cidx * 8; xx < cidx * 8 + 8 && xx < x; xx++) {
                            uint64_t i   = zz * xy + yy * x + xx;
                            uint32_t c   = codes[i];
                            uint32_t mag = c & 0x7FFFu;
                            rowacc += (c >> 15) ? (0u - mag) : mag;
                            colacc[xx - cidx * 8] += rowacc;
                            plane[yy - b * 8][xx - cidx * 8] += colacc[xx - cidx * 8];
                            out[i] = (float)(int32_t)plane[yy - b * 8][xx - cidx * 8] * ebx2;
                        }
                    }
                }
            }
        }
    }
}

static uint32_t get32(const uint8_t* p)
{
    uint32_t v;
    memcpy(&v, p, 4);
    return v;
}
static uint64_t get64(const uint8_t* p)
{
    uint64_t v;
    memcpy(&v, p, 8);
    return v;
}

int fzo_decompress(const uint8_t* st, uint64_t bytes, float* out, uint64_t n_capacity)
{
    if (bytes < HDR || get32(st) != 0x31475A46u) return -1;
    int      mode = st[6], nd = st[7];
    uint32_t x = get32(st + 8), y = get32(st + 12), z = get32(st + 16);
    uint64_t n   = get64(st + 24);
    uint64_t nnz = get64(st + 48);
    float    e2;
    memcpy(&e2, st + 44, 4);
    if (n > n_capacity || (uint64_t)x * y * z > n || nd != fzo_ndim(x, y, z)) return -2;
    uint64_t off_a, off_c, off_b;
    uint32_t sc;
    fzo_layout(n, nd, mode, &off_a, &off_c, &off_b, &sc);
    if (sc != get32(st + 60) || off_b + 16 * nnz > bytes) return -3;

    uint64_t        nb    = n / BLOCK_CODES;
    uint64_t        nw    = cdiv(n, 256);
    const uint32_t* B     = (const uint32_t*)(st + off_a);
    const uint8_t*  ch    = st + off_b;
    uint16_t*       codes = (uint16_t*)calloc(n ? n : 1, 2);
    /* block offsets into Section B */
    uint64_t* boff = (uint64_t*)malloc((nb + 1) * 8);
    uint64_t  acc  = block_offsets(B, nb, boff);
    if (acc != nnz) {
        free(codes);
        free(boff);
        return -4;
    }
    for (uint64_t k = nb * 8; k < nw; k++)
        if (B[k]) {
            free(codes);
            free(boff);
            return -5;
        }
    if (mode == 1) {
        /* the sidecar's block offsets must agree with the bitmap */
        uint64_t tail = n - nb * BLOCK_CODES;
        uint64_t q    = off_c + pad16(2 * tail) + (nd == 1 ? pad16(4 * cdiv(n, 32)) : 0);
        for (uint64_t b = 0; b <= nb; b++)
            if (get32(st + q + 4 * b) != (b < nb ? boff[b] : nnz)) {
                free(codes);
                free(boff);
                return -6;
            }
    }
#pragma omp parallel for schedule(static)
    for (uint64_t b = 0; b < nb; b++) {
        uint32_t s[BLOCK_WORDS];
        memset(s, 0, sizeof(s));
        uint64_t slot = boff[b];
        for (uint32_t c = 0; c < CHUNKS_PER_BLOCK; c++) {
            if ((B[b * 8 + c / 32] >> (c % 32)) & 1u) {
                memcpy(&s[4 * c], ch + 16 * slot, 16);
                slot++;
            }
        }
        /* un-shuffle: W[g*32 + j] bit p = S[p*32 + g] bit j (the 32x32 transpose is an
           involution) */
        for (uint32_t g = 0; g < 32; g++) {
            uint32_t a[32];
            for (uint32_t p = 0; p < 32; p++) a[p] = s[p * 32 + g];
            transpose32(a);
            for (uint32_t j = 0; j < 32; j++) {
                uint64_t k              = b * BLOCK_CODES + 2 * (g * 32 + j);
                codes[k]                = (uint16_t)(a[j] & 0xFFFFu);
                codes[k + 1]            = (uint16_t)(a[j] >> 16);
            }
        }
    }
    const uint8_t* signbits = NULL;
    if (mode == 1) {
        uint64_t tail = n - nb * BLOCK_CODES;
        memcpy(codes + nb * BLOCK_CODES, st + off_c, tail * 2);
        if (nd == 1) signbits = st + off_c + pad16(2 * tail);
    }
    fzo_lorenzo_reconstruct(codes, signbits, n, x, y, z, e2, out);
    free(codes);
    free(boff);
    return 0;
}

/* verify.hh:24-83: max |x - x'|, MSE, NRMSE = sqrt(MSE)/range, PSNR = 20 log10(range) -
   10 log10(MSE), all in double. */
void fzo_metrics(const float* orig, const float* recon, uint64_t n, double* max_abs_err,
                 double* psnr, double* nrmse, double* range)
{
    double mx = orig[0], mn = orig[0], me = 0, se = 0;
#pragma omp parallel for reduction(max : mx, me) reduction(min : mn) reduction(+ : se) schedule(static)
    for (uint64_t i = 0; i < n; i++) {
        double o = orig[i], e = fabs((double)recon[i] - o);
        if (o > mx) mx = o;
        if (o < mn) mn = o;
        if (e > me) me = e;
        se += e * e;
    }
    double rng = mx - mn, mse = se / (double)n;
    *max_abs_err = me;
    *range       = rng;
    *nrmse       = sqrt(mse) / rng;
    *psnr        = 20 * log10(rng) - 10 * log10(mse);
}
