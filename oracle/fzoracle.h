/*
 * fzoracle.h -- ORACLE (test infrastructure only).
 *
 * CPU restatement of the FZ-GPU compression path, used by tests/, by the smoke check
 * and by the CPU-baseline leg of bench.py as the checker.  Nothing in the product
 * library links or calls this code.  Every function cites the reference lines it
 * restates (paths relative to the FZ-GPU source tree).
 */
#ifndef FZ_ORACLE_H
#define FZ_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* lorenzo_var.cuh:537-544 */
int fzo_ndim(uint32_t x, uint32_t y, uint32_t z);

/* fz.cu:137  range = max - min over all n values, in float. */
void fzo_value_range(const float* data, uint64_t n, float* mn, float* mx);

/* lorenzo_var.cuh:562-563 ebx2_r = (float)(1 / (2 eb)), lorenzo_var.cuh:641 ebx2 = (float)(2 eb) */
float fzo_ebx2_r(double eb_abs);
float fzo_ebx2(double eb_abs);

/* Device conversion (uint16_t)fabsf(d) (lorenzo_var.cuh:53,169,289) for d >= 0 or NaN:
   saturating float->u32, then the low 16 bits. */
uint16_t fzo_f2u16(float v);

/* Dual-quant Lorenzo codes, lorenzo_var.cuh:47-295.  codes[0..n) fully written;
   codes at i >= x*y*z are 0 (fz.cu:145).  signum (nullable): 1D delta<0 per element.
   Returns 1 if some delta did not fit its code field (|d| >= 32768 for a signed code,
   >= 65536 for a 1D unsigned one, or non-finite), else 0. */
uint32_t fzo_lorenzo_construct(const float* data, uint64_t n, uint32_t x, uint32_t y, uint32_t z,
                           float ebx2_r, uint16_t* codes, uint8_t* signum);

/* bitshuffleAndBitflag over floor(n/2048) blocks (fz.cu:61-111,172-174), with the raw
   copy of the tail (fz.cu:155).  S: u32[ceil(n/2)], F: u32[32*ceil(n/256)],
   B: u32[ceil(n/256)]; F and B are zero past the last full block (fz.cu:167-168). */
void fzo_bitshuffle_flag(const uint16_t* codes, uint64_t n, uint32_t* S, uint32_t* F,
                         uint32_t* B);

/* Exclusive scan of F over M = 32*ceil(n/256) entries plus total (fz.cu:187-201) and
   the intended encodeDebug compaction (fz.cu:49-59).  P: u32[M+1] (nullable),
   out: 16*nnz bytes (nullable).  Returns nnz. */
uint64_t fzo_scan_encode(const uint32_t* S, const uint32_t* F, uint64_t n, uint32_t* P,
                         uint8_t* out);

/* Stream layout (the format the product defines; see include/fz.h). */
void fzo_layout(uint64_t n, int ndim, int mode, uint64_t* off_a, uint64_t* off_c,
                uint64_t* off_b, uint32_t* sidecar_bytes);

/* Full compression into the stream format.  eb_mode 0 = absolute, 1 = relative.
   Returns the stream size, or 0 on error.  out must hold the worst case. */
uint64_t fzo_compress(const float* data, uint64_t n, uint32_t x, uint32_t y, uint32_t z,
                      double eb, int eb_mode, int mode, uint8_t* out);

/* Inverse Lorenzo for sign-magnitude codes (integer prefix sums per tile, then
   *ebx2 in float; the semantics of lorenzo_var.cuh:297-518).  signs (nullable): 1D
   sign bits, bit i of byte i/8. */
void fzo_lorenzo_reconstruct(const uint16_t* codes, const uint8_t* signbits, uint64_t n,
                             uint32_t x, uint32_t y, uint32_t z, float ebx2, float* out);

/* Decompress a stream; returns 0 on success, negative on a malformed stream. */
int fzo_decompress(const uint8_t* stream, uint64_t bytes, float* out, uint64_t n_capacity);

/* Quality metrics of verify.hh:24-83, in FP64. */
void fzo_metrics(const float* orig, const float* recon, uint64_t n, double* max_abs_err,
                 double* psnr, double* nrmse, double* range);

/* OpenMP thread count used (1 when built without OpenMP). */
int fzo_threads(void);
/* Threads of the following parallel regions of the calling thread (OpenMP). */
void fzo_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
