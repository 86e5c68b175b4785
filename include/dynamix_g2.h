/*
 * dynamix_g2.h -- C ABI of the GB300 (sm_103a) g2 correlator kernels.
 *
 * All pointers named *_dev are device pointers owned by the caller; the
 * library allocates no device memory at run time.  The one device buffer it
 * holds itself is the file-scope array of g2_normalize_static
 * (G2_STATIC_DENOM_MAX int64, 4 MiB), which every GPU that loads the library
 * keeps until the process exits.  Every entry point is asynchronous on
 * the given CUDA stream (a cudaStream_t passed as void*; NULL = legacy default
 * stream), returns a status code (G2_OK = 0) and never throws.  Argument
 * errors are detected on the host before anything is launched.
 *
 * Quantities (per q-bin b with P_b pixels, frames I(t,p), t = 0..T-1):
 *   N_b(tau) = sum_t sum_{p in b} I(t,p) I(t+tau,p)      numerator   (int64)
 *   S_b(t)   = sum_{p in b} I(t,p)                        bin sums    (int64)
 *   D_b(tau) = sum_t S_b(t) S_b(t+tau)                    denominator (int64)
 *   g2_b(tau)= scale_b * N_b(tau) / D_b(tau)              (float64 -> float32)
 *
 * Citations are paths inside the dynamix project (silx-kit/dynamix).
 */
#ifndef DYNAMIX_G2_H
#define DYNAMIX_G2_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define G2_OK               0
#define G2_ERR_ARG          1  /* bad argument (null pointer, size, alignment) */
#define G2_ERR_CUDA         2  /* a CUDA runtime call failed */
#define G2_ERR_UNSUPPORTED  3  /* device is not sm_103 or feature missing */
#define G2_ERR_TOO_LARGE    4  /* a size exceeds a kernel limit */

/* bits a kernel may set in its device error word (int32) */
#define G2_DEVERR_TIMEOUT   1  /* a bounded wait expired; the kernel bailed out */
#define G2_DEVERR_BOUNDS    2  /* an index was out of range and was skipped */
#define G2_DEVERR_RANGE     4  /* a count does not fit the requested packing */
#define G2_DEVERR_RANGE_CHECK 8 /* a count may not fit the packing: check the exact maximum */

#define G2_ABI_VERSION      1

/* Tile sizes of the tensor-core Gram: an item covers a 128 x 256 block of
 * the (t, t') Gram, the plain kernel a 128 x 128 block.  A pipeline stage
 * holds 128 bytes of K per row: 64 fp16 or 128 e4m3 elements; an item's k
 * offsets and k_len are multiples of that. */
#define G2_TC_BM      128
#define G2_TC_BN      256
#define G2_PLAIN_BM   128
#define G2_PLAIN_BN   128
#define G2_PAD        128  /* packed_cols and bin segments are multiples of this */
#define G2_PACK_CHUNK 2048 /* source pixels per pack chunk */
#define G2_PACK_MAX_SLOTS  128  /* distinct bins per chunk */
#define G2_PACK_MAX_PIECES 512  /* (64-column segment x chunk) pieces per chunk */
#define G2_PACK_WORDS_PER_CHUNK 768 /* 4-column words per chunk: 2048/4 + partial words at bin edges */
#define G2_MAX_JOBS   32

/* element kinds of a packed operand matrix */
#define G2_KIND_FP16  0    /* 16-bit raw counts <= 2048, MMA kind::f16 */
#define G2_KIND_E4M3  1    /* 8-bit raw counts <= 16, MMA kind::f8f6f4 (e4m3) */

/* One unit of Gram work: rows [i0, i0+BM) of the A operand against rows
 * [j0, j0+BN) of the B operand over packed columns [a_k0, a_k0+k_len) and
 * [b_k0, b_k0+k_len).  The lag-diagonal sums of the t' >= t part are added,
 * multiplied by 2^shift, to numer[out_off + tau] for 0 <= tau < nframes; rows
 * and columns >= nframes never enter them.  When the job's packed matrix has a
 * row of ones at row nframes (g2_job.ones_row) and s_off >= 0, the column of
 * that row holds the bin sums: G(t, nframes) = sum_k A(t, k) = S(t), added to
 * sums[s_off + t] for t < nframes.
 * The persistent Gram kernels give worker w (a CTA, or a CTA pair for
 * g2_gram_tc_pair) the items w, w + W, w + 2W, ... of the list (W workers, see
 * g2_gram_workers); a caller that balances the work per worker fills the
 * unused slots of that pattern with G2_ITEM_EMPTY. */
#define G2_ITEM_EMPTY (-1)  /* g2_gram_item.job of an empty slot: skipped by every role */

typedef struct g2_gram_item {
    int32_t job;       /* index into the jobs array of the launch, or G2_ITEM_EMPTY */
    int32_t i0;        /* first frame of the A rows */
    int32_t j0;        /* first frame of the B rows */
    int32_t a_k0;      /* first packed column of A (multiple of the stage width) */
    int32_t b_k0;      /* first packed column of B (multiple of the stage width) */
    int32_t k_len;     /* packed columns, multiple of the stage width, > 0 */
    int32_t shift;     /* weight 2^shift (0, 8 or 16 for byte-split planes) */
    int32_t nframes;   /* T of the job */
    int64_t out_off;   /* element offset of N_b(0) in numer */
    int64_t s_off;     /* element offset of S_b(0) in sums, or -1 */
} g2_gram_item;

/* A dense job: its packed operand matrix, row-major [nframes][packed_cols]
 * of raw integer counts, 16-bit (G2_KIND_FP16, counts <= 2048, read as fp16 =
 * count * 2^-24) or 8-bit (G2_KIND_E4M3, counts <= 16, read as e4m3 =
 * count * 2^-9); both represent the counts exactly. */
typedef struct g2_job {
    const void* packed_dev;
    int64_t nframes;
    int64_t packed_cols;   /* multiple of G2_PAD */
    int32_t elem_kind;     /* G2_KIND_FP16 or G2_KIND_E4M3 */
    int32_t ones_row;      /* 1: row nframes of the packed matrix holds 1 in every
                              binned column and 0 in the padding (bin sums) */
} g2_job;

/* ---- host utilities ---------------------------------------------------- */
int         g2_abi_version(void);
const char* g2_status_string(int status);
/* SM count and compute capability of a device. */
int g2_device_info(int device, int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor);
/* Host-only: longest-processing-time schedule of n items (cost[i] >= 0) over
 * `workers` persistent workers of a Gram launch.  Item i goes to slot
 * slot_out[i] of a list of *n_slots slots read by worker w at w, w + workers,
 * ...; slots left over hold G2_ITEM_EMPTY items (the caller fills them).  No
 * reference counterpart (the reference launches one thread per output). */
int g2_balance_lpt(const double* cost, int64_t n, int32_t workers, int64_t* slot_out, int64_t* n_slots);
/* Host-to-device copy of the byte columns [col0, col0 + width) of `rows`
 * rows of pitch src_pitch (a stack of frames seen as T*H rows) into rows of
 * pitch `width` at dst_dev, on `stream` (one cudaMemcpy2DAsync): frames in
 * host memory cropped to the q-mask's bounding columns on their way in, so
 * that only the bytes the pack reads cross the host link.  The reference
 * reads whole frames from host memory (dense.py:49, `frames[:, ind]`). */
int g2_copy_cols_h2d(void* dst_dev, const void* src_host, int64_t src_pitch, int64_t col0, int64_t width,
                     int64_t rows, void* stream);

/* ---- G1: pack + bin sums ------------------------------------------------
 * Replaces compute_sums_dense (dynamix/resources/opencl/densecorrelator.cl:65-150)
 * and the per-bin gather + float32 cast of py_dense_correlator
 * (dynamix/correlator/dense.py:48-50).
 *
 * frames_dev: [nframes][npix] counts, elem_bytes 1 (u8) or 2 (u16), 16-byte
 * aligned (the chunks are read with aligned 16-byte loads).  The
 * pixels are cut into n_chunks = ceil(npix / G2_PACK_CHUNK) chunks.  The
 * binned pixels of chunk c are entries [chunk_entry_off[c], chunk_entry_off[c+1])
 * (in pixel order); entry e goes to packed column entry_dst[e] (plane 0) and
 * entry_meta[e] = offset in the chunk | local bin slot << 11 | local piece << 18.
 * chunk_slot_bin[c * G2_PACK_MAX_SLOTS + slot] is the 0-based bin of a slot (-1
 * unused).  A piece is one 64-column output segment within one chunk; chunk c
 * owns pieces [chunk_piece_off[c], chunk_piece_off[c+1]).
 * The packed values are the raw integers: read as fp16, the 16-bit values
 * 0..2048 are exactly count * 2^-24; read as e4m3, the bytes 0..16 are exactly
 * count * 2^-9 (g2_gram_tc rescales by the power of two).
 * mode 0: the count as a 16-bit value at entry_dst (counts <= 2048).
 * mode 1 (u16 only): high byte (16-bit) at entry_dst, low byte at entry_dst +
 *   bin_kpad[bin] (the low-byte plane of the bin).
 * mode 2: the count as a byte at entry_dst (counts <= 16).
 * A count that does not fit the mode sets G2_DEVERR_RANGE in err_dev.
 * Adds S_b(t) into sums_dev[b * nframes + t] (caller zeroes it; null: no bin
 * sums, for operands whose Gram takes them from a row of ones) and raises
 * piece_emax_dev[plane * n_pieces + piece] (2 * n_pieces words; caller zeroes
 * them): plane 0 (and, in mode 1, plane 1 for the low bytes) bounds the sum of
 * squared packed values of the piece in every frame (the max over groups of 4
 * frames of the sum over entries of each entry's largest square in the
 * group); in modes 0 and 2 plane 1 holds, at each chunk's first piece, the
 * largest squared value of the chunk (0 elsewhere).
 * Packed columns that no entry maps to (bin padding) are not written.
 */
int g2_pack_frames(const void* frames_dev, int32_t elem_bytes, int64_t nframes, int64_t npix,
                   const int32_t* chunk_entry_off_dev, const int32_t* entry_dst_dev,
                   const uint32_t* entry_meta_dev, const int32_t* chunk_slot_bin_dev,
                   const int32_t* chunk_piece_off_dev, const int32_t* bin_kpad_dev, int64_t n_chunks,
                   int32_t mode, void* packed_dev, int64_t packed_cols, int64_t* sums_dev,
                   int32_t n_bins, uint32_t* piece_emax_dev, int64_t n_pieces, int32_t* err_dev,
                   void* stream);

/* G1 for e4m3 operands (every count <= 16): a pure byte permutation.  The
 * raw count bytes are the operand (bytes 0..16 read as e4m3 are exactly
 * count * 2^-9; g2_gram_tc rescales).  Chunks as for g2_pack_frames; chunk c
 * owns words [chunk_word_off[c], chunk_word_off[c+1]) of at most
 * G2_PACK_WORDS_PER_CHUNK; word w covers packed columns word_dst[w] ..
 * word_dst[w]+3 of one bin, word_src[2w], word_src[2w+1] hold the 4 chunk-local
 * source offsets (12 bits each, 0xFFF = column owned by another chunk) and the
 * bin slot (bits 16-20 of word_src[2w+1], unused here).  Bit 0 of
 * word_src[2w+1] >> 21 set means the 4 sources are consecutive pixels.  A
 * count above 16 sets G2_DEVERR_RANGE.  The bin sums are not computed here:
 * g2_gram_tc takes them from the row of ones (g2_job.ones_row).  Same packed
 * result as g2_pack_frames mode 2. */
int g2_pack_e4m3(const void* frames_dev, int32_t elem_bytes, int64_t nframes, int64_t npix,
                 const int32_t* chunk_word_off_dev, const int32_t* word_dst_dev,
                 const uint32_t* word_src_dev, int64_t n_chunks, void* packed_dev, int64_t packed_cols,
                 int32_t* err_dev, void* stream);

/* The same packed result as g2_pack_e4m3 for u8 frames, by work units: the
 * destination bytes of chunk c are the units of blocks [unit_block_off[c],
 * unit_block_off[c+1]), 32 units per block (units_dev: 4 uint32 per unit,
 * 16-byte aligned): {destination, source, source, class} with class 1 = 16
 * bytes from 16 consecutive source bytes at source (destination in 16-byte
 * units), 2 = 4 bytes from 4 consecutive (destination in 4-byte units), 3 = 4
 * bytes from sources src0 | src1 << 16, src2 | src3 << 16 (4-byte units),
 * 4 = one byte (destination in bytes), 0 = none; sources are offsets in the
 * chunk.  A block holds one class.  Instead of checking every count, the
 * kernel sets G2_DEVERR_RANGE_CHECK when a count above 15 may be present (an
 * OR of the moved bytes exceeds 16); the caller then checks the exact maximum
 * (g2_binned_max) before using the e4m3 operand. */
int g2_pack_e4m3_units(const void* frames_dev, int64_t nframes, int64_t npix,
                       const int32_t* unit_block_off_dev, const uint32_t* units_dev, int64_t n_chunks,
                       void* packed_dev, int64_t packed_cols, int32_t* err_dev, void* stream);

/* Largest count over the binned pixels (col_src >= 0): picks split 0/1.
 * No reference counterpart (the reference never checks its dtype range). */
int g2_binned_max(const void* frames_dev, int32_t elem_bytes, int64_t nframes, int64_t npix,
                  const int32_t* col_src_dev, int64_t n_cols, uint32_t* max_dev, void* stream);

/* ---- G2: tensor-core Gram with fused lag-diagonal sums ------------------
 * Replaces the numerator of py_dense_correlator (dynamix/correlator/dense.py:54,
 * :61-64), CublasMatMulCorrelator._correlate_matmul_cublas + extract_upper_diags
 * (dynamix/correlator/cuda.py:67-74, :101-116) and correlator_multiQ_dense
 * (dynamix/resources/opencl/densecorrelator.cl:6-56).
 * tcgen05.mma kind::f16 (fp16 x fp16 -> fp32 in TMEM) on TMA-staged tiles;
 * every FP32 partial sum is an integer below 2^24 when the caller's K split
 * honours the segment energy bound, and is promoted to int64 per item.
 * numer_dev is accumulated into (uint64 two's complement of int64).
 * items_dev: n_items g2_gram_item (BM=128, BN=256).  grid <= 0: one CTA per SM.
 */
int g2_gram_tc(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
               uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev, int64_t sums_len,
               int32_t* err_dev, int32_t grid, void* stream);

/* The same Gram on CTA pairs (replaces the same reference code as
 * g2_gram_tc): an item covers a 256 x n block, rows [i0, i0+256) against rows
 * [j0, j0+n), n = min(256, frames (and row of ones) left from j0, rounded up
 * to 32).  Two CTAs on two SMs share one tcgen05.mma.cta_group::2 M256: each
 * loads its own 128 rows of A and n/2 rows of B per stage (32 KB), so each SM
 * streams a third less from L2 per MMA cycle than g2_gram_tc.  Same item
 * fields, exactness contract and outputs.  grid <= 0: as many CTA pairs as
 * can be resident; otherwise about grid CTAs (rounded up to pairs). */
int g2_gram_tc_pair(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                    uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev, int64_t sums_len,
                    int32_t* err_dev, int32_t grid, void* stream);

/* The same Gram on CTA pairs with wide items: rows [i0, i0+256) against
 * rows [j0, j0+512) as two pair MMAs (N <= 256 each) that share each stage's
 * A rows, so each SM streams 48 instead of 64 bytes per MMA cycle.  The left
 * half is skipped when it lies below the diagonal (j0 + 256 <= i0); each
 * half's width is the frames (and row of ones) it holds, rounded up to 32.
 * The accumulator fills the whole TMEM, so an item's epilogue does not
 * overlap the next item's MMAs: meant for long K.  Same item fields,
 * exactness contract and outputs as g2_gram_tc. */
int g2_gram_tc_wide(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                    uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev, int64_t sums_len,
                    int32_t* err_dev, int32_t grid, void* stream);

/* Number of persistent workers W a Gram launch with grid <= 0 uses on the
 * current device: CTAs for g2_gram_tc (pair = 0), CTA pairs resident at once
 * for g2_gram_tc_pair (pair = 1) or g2_gram_tc_wide (pair = 2).  No reference counterpart (the reference's
 * work-group shapes are fixed, dense.py:184-188). */
int g2_gram_workers(int32_t pair, int32_t* workers);

/* ---- G5: plain direct kernel (CUDA cores, integer) ----------------------
 * The same-GPU non-tensor-core comparator: the direct integer numerator of
 * correlator_multiQ_dense (dynamix/resources/opencl/densecorrelator.cl:6-56),
 * register-tiled on CUDA cores (uint32 IMAD) over 128 x 128 items. */
int g2_plain_direct(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev,
                    int64_t n_items, uint64_t* numer_dev, int64_t numer_len, int32_t* err_dev,
                    void* stream);

/* The same direct integer sums on the raw u8 counts, four byte products per
 * __dp4a (the fastest CUDA-core form of correlator_multiQ_dense,
 * dynamix/resources/opencl/densecorrelator.cl:6-56, for 8-bit frames).
 * Packed operand: the e4m3 packing of g2_pack_e4m3, read as raw u8 bytes
 * (elem_kind G2_KIND_E4M3, any count 0..255).  Items: 128 x 128 blocks with
 * k_len a multiple of 64 and <= 65,536 (uint32 entries exact for any u8);
 * with the job's row of ones and s_off >= 0 the bin sums are added to
 * sums_dev as in g2_gram_tc. */
int g2_plain_dp4a(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev,
                  int64_t n_items, uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev,
                  int64_t sums_len, int32_t* err_dev, void* stream);

/* ---- tensor-core rate probe ---------------------------------------------
 * No counterpart in the reference: a measurement utility.  One CTA per SM
 * (grid <= 0) or `grid` CTAs each issue `iters` x 4 tcgen05.mma M128 N256
 * (K = 32 for kind G2_KIND_E4M3, 16 for G2_KIND_FP16) on shared-memory
 * resident count-like operands, no global memory traffic: the dense rate of
 * the MMA kind the Gram uses, for its roofline.  MACs per launch =
 * grid * iters * 4 * 128 * 256 * K. */
int g2_tc_rate_probe(int32_t kind, int64_t iters, int32_t grid, int32_t* err_dev, void* stream);

/* ---- G6: event-list pair sums -------------------------------------------
 * Replaces event_correlator (dynamix/resources/opencl/evtcorrelator.cl:3-47)
 * behind EventCorrelator.correlate (dynamix/correlator/event.py:162-204).
 * Events of pixel p: [offsets[p], offsets[p+1]) of times_dev (frame, int32) and
 * data_dev (count, elem_bytes 1 or 2), the layout of FramesCompressor
 * (event.py:267-284); their order within a pixel does not matter.  pix_list
 * holds binned pixels grouped by bin; range r covers pix_list[range_off[r] ..
 * range_off[r+1]) of bin range_bin[r] (0-based); CTA c of the n_ctas launched
 * processes ranges [cta_range_off[c], cta_range_off[c+1]).  For every pair i <= j of a
 * pixel's events adds v_i v_j to numer[bin * nframes + |t_j - t_i|] and v_i to
 * sums[bin * nframes + t_i] (int64 as uint64, caller zeroes them).  max_count
 * is an upper bound of the counts (selects the shared-memory kernel). */
int g2_event_pairsum(const int32_t* times_dev, const void* data_dev, int32_t elem_bytes,
                     int64_t n_events, const uint32_t* offsets_dev, int64_t npix,
                     const int32_t* pix_list_dev, const int32_t* range_off_dev,
                     const int32_t* range_bin_dev, int32_t n_ranges, const int32_t* cta_range_off_dev,
                     int32_t n_ctas, int32_t nframes, int32_t n_bins,
                     int32_t max_count, uint64_t* numer_dev, uint64_t* sums_dev, int32_t* err_dev,
                     void* stream);

/* g2_event_pairsum on packed event words (t << 16) | v (as written by
 * g2_csr_scatter_packed), nframes <= 65536; same plan arguments and sums. */
int g2_event_pairsum_packed(const uint32_t* words_dev, int64_t n_events, const uint32_t* offsets_dev,
                            int64_t npix, const int32_t* pix_list_dev, const int32_t* range_off_dev,
                            const int32_t* range_bin_dev, int32_t n_ranges, const int32_t* cta_range_off_dev,
                            int32_t n_ctas, int32_t nframes, int32_t n_bins, int32_t max_count,
                            uint64_t* numer_dev, uint64_t* sums_dev, int32_t* err_dev, void* stream);

/* ---- G7: CSR frames -> per-pixel event lists ----------------------------
 * Replaces the CSR path of SparseCorrelator (dynamix/correlator/intensity.py:
 * 70-128: compute_sums and correlator_oneQ_Nt, correlator.cl:19-217): the CSR
 * stack is transposed to the event layout and correlated by g2_event_pairsum.
 * CSR of frame t: elements [offsets[t], offsets[t+1]) of data (count,
 * elem_bytes 1 or 2) and indices (column); indptr[t*(height+1) + r] ..
 * indptr[t*(height+1) + r + 1] are the elements of row r relative to
 * offsets[t].  indices, indptr and offsets share one integer type of
 * index_bytes (4 = uint32, 8 = int64).
 * g2_csr_count adds 1 to counts[r*width + col] per element (caller zeroes).
 * g2_exclusive_scan_u32 writes out[i] = sum(in[0..i)) for i <= n (out has n+1
 * entries; totals below 2^32); scratch holds ceil(n / 8192) entries.
 * g2_csr_scatter writes element (t, v) of pixel p to slot ev_offsets[p] +
 * (cursor[p]++) of ev_times / ev_data (cursor zeroed by the caller). */
int g2_csr_count(const void* indices_dev, const void* indptr_dev, const void* offsets_dev,
                 int32_t index_bytes, int64_t n_elem, int32_t nframes, int32_t height, int32_t width,
                 uint32_t* counts_dev, int32_t* err_dev, void* stream);
int g2_exclusive_scan_u32(const uint32_t* in_dev, int64_t n, uint32_t* out_dev, uint32_t* scratch_dev,
                          int64_t scratch_len, void* stream);
/* values_dev[0 .. n] += *carry_dev, then *carry_dev = values_dev[n]: continues
 * an exclusive scan (g2_exclusive_scan_u32 writes n + 1 values) across pieces
 * scanned one after another on the same stream. */
int g2_add_carry_u32(uint32_t* values_dev, int64_t n, uint32_t* carry_dev, void* stream);
int g2_csr_scatter(const void* data_dev, int32_t elem_bytes, const void* indices_dev,
                   const void* indptr_dev, const void* offsets_dev, int32_t index_bytes, int64_t n_elem,
                   int32_t nframes, int32_t height, int32_t width, const uint32_t* ev_offsets_dev,
                   uint32_t* cursor_dev, int32_t* ev_times_dev, void* ev_data_dev, int32_t* err_dev,
                   void* stream);

/* Sub-blocked variants with packed event words (frames < 2^16, image rows up
 * to 29,000 pixels, fewer than 2^32 elements): the frames are cut into
 * sub-blocks of 1024, n_sb = ceil(nframes / 1024).
 * g2_csr_count_blocked writes row_bounds_dev[r * nframes + t] (uint32, the
 * absolute index of row r's first element in frame t, r = 0..H; (H+1) *
 * nframes entries), sb_counts_dev[sb * H*W + p] (uint16, the elements of
 * pixel p in sub-block sb; n_sb * H*W entries), row_totals_dev[sb * H + r]
 * (uint32, the elements of row r in sub-block sb; n_sb * H entries) and adds
 * each pixel's total to counts_dev (caller zeroes).  Column indices must
 * increase strictly within a row (sorted CSR), else G2_DEVERR_BOUNDS.
 * g2_csr_stage_blocked takes row_base_dev (the exclusive scan of row_totals,
 * n_sb * H + 1 entries) and writes every element as one word (t << 16) | v
 * into stage_dev (n_elem words), grouped by sub-block, row and pixel, and the
 * start of every 64-pixel tile's run of each sub-block into tile_pos_dev
 * (n_sb * ceil(H*W / 64) entries).
 * g2_csr_gather_blocked copies the runs into ev_words_dev[ev_offsets[p] ..)
 * (ev_offsets: exclusive scan of the pixel totals, H*W + 1 entries; stage_dev
 * and ev_words_dev hold n_elem words), in sub-block order, and with sort != 0
 * in frame order inside each run -- then every pixel's list is in
 * frame order.  g2_events_unpack splits words into ev_times (int32) and
 * ev_data (elem_bytes 1 or 2): with the sort, the FramesCompressor layout
 * (event.py:267-284).  G2_ERR_UNSUPPORTED when nframes > 65536 (stage,
 * gather), height > 65535 or width > 29,000. */
int g2_csr_count_blocked(const void* indices_dev, const void* indptr_dev, const void* offsets_dev,
                         int32_t index_bytes, int64_t n_elem, int32_t nframes, int32_t height, int32_t width,
                         uint32_t* row_bounds_dev, uint32_t* counts_dev, uint16_t* sb_counts_dev,
                         uint32_t* row_totals_dev, int32_t* err_dev, void* stream);
int g2_csr_stage_blocked(const void* data_dev, int32_t elem_bytes, const void* indices_dev,
                         const uint32_t* row_bounds_dev, int32_t index_bytes, int64_t n_elem, int32_t nframes,
                         int32_t height, int32_t width, const uint16_t* sb_counts_dev, const uint32_t* row_base_dev,
                         uint32_t* tile_pos_dev, uint32_t* stage_dev, int32_t* err_dev, void* stream);
/* g2_csr_stage_blocked for the frames frame0 .. frame0 + nframes - 1 only
 * (frame0 a multiple of 1024; row_bounds_dev as written by
 * g2_csr_count_blocked for those frames, sb_counts_dev, row_base_dev and
 * tile_pos_dev pointing at their first sub-block; frame_elems, the elements of
 * those frames, sizes the shared-memory buffer): a stack arriving frame group
 * by frame group is staged while the next group is copied. */
int g2_csr_stage_frames(const void* data_dev, int32_t elem_bytes, const void* indices_dev,
                        const uint32_t* row_bounds_dev, int32_t index_bytes, int64_t n_elem, int32_t frame0,
                        int32_t nframes, int64_t frame_elems, int32_t height, int32_t width,
                        const uint16_t* sb_counts_dev, const uint32_t* row_base_dev, uint32_t* tile_pos_dev,
                        uint32_t* stage_dev, int32_t* err_dev, void* stream);
int g2_csr_gather_blocked(const uint32_t* stage_dev, const uint32_t* tile_pos_dev, const uint16_t* sb_counts_dev,
                          int32_t nframes, int64_t npix, int64_t n_elem, const uint32_t* ev_offsets_dev,
                          int32_t sort, uint32_t* ev_words_dev, int32_t* err_dev, void* stream);
int g2_events_unpack(const uint32_t* ev_words_dev, int64_t n_events, int32_t elem_bytes, int32_t* ev_times_dev,
                     void* ev_data_dev, void* stream);

/* ---- frame compression: dense frames -> event lists ----------------------
 * Device counterpart of FramesCompressor (event.py:207-321) with the
 * hot-pixel threshold, sticky mask and sum frame of neigercompress
 * (io/readdata.py:441-468).  frames_dev: (nframes, npix) values of kind
 * elem_kind (1 u8, 2 u16, -1 i8, -2 i16); a value > 0 is an event, as in the
 * reference's `frames > 0`.  n_sb = ceil(nframes / 1024), n_blk =
 * ceil(npix / 1024) (at most 65535), n_tiles = ceil(npix / 64).
 * g2_compress_count writes sb_counts_dev[sb * npix + p] (uint16, positives of
 * pixel p in sub-block sb) and blk_totals_dev[sb * n_blk + b] (their sums over
 * 1024-pixel blocks); threshold >= 0 also writes sb_first_dev (the first frame
 * of the sub-block, counted from its start, with a value above the threshold;
 * 0xFFFF for none) and sb_before_dev (positives before that frame);
 * sum_frame_dev (int64 per pixel, nullable, caller zeroes) gets every raw
 * value added.
 * g2_compress_finish applies the sticky mask: mask_dev (uint8 per pixel,
 * nullable, updated in place) drops every event of a masked pixel, and a
 * value above the threshold masks its pixel from that frame on.  It corrects
 * sb_counts and blk_totals and writes counts_dev (uint32 events per pixel)
 * and t_cut_dev (int32 per pixel, nullable: the first dropped frame, nframes
 * for none; needed by the stage pass when a threshold or a mask is used).
 * Scan counts -> ev_offsets (npix + 1) and blk_totals -> blk_base
 * (n_sb * n_blk + 1) with g2_exclusive_scan_u32; g2_compress_stage then
 * writes stage_dev (n_stage words, at least the events) and tile_pos_dev
 * (n_sb * n_tiles), and g2_events_gather_rel the event lists: packed words
 * (t << 16) | v into ev_words_dev (nframes <= 65536; the input of
 * g2_event_pairsum_packed), or ev_times_dev (int32) and ev_data_dev
 * (elem_bytes 1 or 2) with ev_words_dev NULL (nframes up to 409,600).  Within
 * a pixel the events come in frame order: exactly the compress_all_stack
 * layout (event.py:267-284). */
int g2_compress_count(const void* frames_dev, int32_t elem_kind, int32_t nframes, int64_t npix, int32_t threshold,
                      uint16_t* sb_counts_dev, uint16_t* sb_first_dev, uint16_t* sb_before_dev,
                      uint32_t* blk_totals_dev, int64_t* sum_frame_dev, void* stream);
int g2_compress_finish(uint16_t* sb_counts_dev, const uint16_t* sb_first_dev, const uint16_t* sb_before_dev,
                       int32_t nframes, int64_t npix, uint8_t* mask_dev, uint32_t* blk_totals_dev,
                       uint32_t* counts_dev, int32_t* t_cut_dev, void* stream);
int g2_compress_stage(const void* frames_dev, int32_t elem_kind, int32_t nframes, int64_t npix,
                      const uint16_t* sb_counts_dev, const int32_t* t_cut_dev, const uint32_t* blk_base_dev,
                      uint32_t* tile_pos_dev, uint32_t* stage_dev, int64_t n_stage, int32_t* err_dev, void* stream);
int g2_events_gather_rel(const uint32_t* stage_dev, const uint32_t* tile_pos_dev, const uint16_t* sb_counts_dev,
                         int32_t nframes, int64_t npix, int64_t n_elem, const uint32_t* ev_offsets_dev,
                         int32_t elem_bytes, uint32_t* ev_words_dev, int32_t* ev_times_dev, void* ev_data_dev,
                         int32_t* err_dev, void* stream);

/* Streaming (process_frame and get_compacted_events, event.py:286-321): one
 * call appends n_batch frames (frame numbers frame0, frame0 + 1, ...) to the
 * per-pixel rows of events_dev (npix x max_nnz, the frames' type) and
 * times_dev (int32); counter_dev (int32 per pixel) holds each row's length and
 * stops at max_nnz, setting G2_DEVERR_RANGE; threshold >= 0 and mask_dev act
 * as in g2_compress_finish (the mask persists across calls); sum_frame_dev
 * (nullable) adds the raw values.  g2_stream_compact copies the rows to
 * out_data_dev / out_times_dev at offsets_dev (the exclusive scan of
 * counter_dev, npix + 1 entries); capacity is the outputs' length. */
int g2_stream_compress(const void* frames_dev, int32_t elem_kind, int32_t n_batch, int64_t frame0, int64_t npix,
                       int32_t max_nnz, int32_t threshold, uint8_t* mask_dev, int64_t* sum_frame_dev,
                       void* events_dev, int32_t* times_dev, int32_t* counter_dev, int32_t* err_dev, void* stream);
int g2_stream_compact(const void* events_dev, const int32_t* times_dev, const int32_t* counter_dev,
                      int32_t elem_bytes, int64_t npix, int32_t max_nnz, const uint32_t* offsets_dev,
                      int64_t capacity, void* out_data_dev, int32_t* out_times_dev, int32_t* err_dev, void* stream);

/* ---- calc_std deviation (dense.py:58-66) ---------------------------------
 * g2_gram_std runs the Gram tiles of the items again (full K per item, fp32
 * accumulation: a float statistic, not an exact sum) and, for every pair
 * t' >= t of a bin, r = P * G(t,t') / (S(t) S(t')) with P = item.shift (the
 * bin's pixel count) and S read at item.s_off + t from sums_dev; it adds
 * d = r - centre[item.out_off + tau] and d^2 to sum_d / sum_d2 (double) and
 * counts pairs with S(t) S(t') = 0 in zeros (caller zeroes the three).  The
 * centre (the bin's g2, say) keeps the variance free of cancellation.
 * g2_std_finalize gives dev = std_t(r) / sqrt(T - tau), NaN where a zero
 * denominator occurred (the reference divides by zero there). */
int g2_gram_std(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                const int64_t* sums_dev, int64_t sums_len, const float* centre_dev, double* sum_d_dev,
                double* sum_d2_dev, uint32_t* zeros_dev, int64_t out_len, int32_t* err_dev, int32_t grid,
                void* stream);
int g2_std_finalize(const double* sum_d_dev, const double* sum_d2_dev, const uint32_t* zeros_dev, int32_t n_rows,
                    int64_t nframes, float* dev_f32, double* dev_f64, void* stream);

/* calc_std for stacks whose counts need byte planes (above 2048), where the
 * per-pair ratio needs the four plane Grams of a pair together:
 * g2_gram_matrix runs one bin's items of ONE plane combination (whole K;
 * item.shift = the combination's weight exponent 0, 8 or 16) and writes
 * 2^shift * G(t,t') for every pair t' >= t into matrix_dev[t * ld + t']
 * (float32), or adds it with accumulate != 0 -- one launch per combination,
 * so no element is written twice in a launch.  g2_matrix_deviation then
 * reduces the bin's matrix as g2_gram_std does (r = npix * G / (S(t) S(t')),
 * d = r - centre[tau]; sums of d and d^2 in double, zero denominators counted)
 * into sum_d / sum_d2 / zeros (caller zeroes them); g2_std_finalize follows. */
int g2_gram_matrix(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                   float* matrix_dev, int64_t nframes, int64_t ld, int32_t accumulate, int32_t* err_dev,
                   int32_t grid, void* stream);
int g2_matrix_deviation(const float* matrix_dev, int64_t nframes, int64_t ld, const int64_t* bin_sums_dev,
                        double npix, const float* centre_dev, double* sum_d_dev, double* sum_d2_dev,
                        uint32_t* zeros_dev, void* stream);

/* ---- two-time correlation (the TTCF of event_y.py:141-157) ---------------
 * g2_gram_ttcf runs the Gram tiles of one bin's items (built as for
 * g2_gram_std: whole K, shift = the bin's pixel count P, s_off = the offset of
 * its sums) and writes r = P G(t,t') / (S(t) S(t')) for every pair t' > t as
 * float32 into ttcf_dev[t * ld + t'] and, with mirror != 0, into
 * ttcf_dev[t' * ld + t] (0/0 gives NaN, as in the reference); items with more
 * frames than nframes are skipped (G2_DEVERR_BOUNDS).  g2_ttcf_finish
 * completes the matrix as the reference does: without mirror, 0 below the
 * diagonal (NaN where S(t) S(t') = 0); on the diagonal the mean of the
 * positive elements of the first upper diagonal (NaN when there are none),
 * except the last element: 0, or NaN when S(T-1) = 0.  The reference mirrors
 * when its diagonal k = -5 sums below 1: when no S(t) S(t+5) is 0, or T <= 5. */
int g2_gram_ttcf(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                 const int64_t* sums_dev, int64_t sums_len, float* ttcf_dev, int64_t nframes, int64_t ld,
                 int32_t mirror, int32_t* err_dev, int32_t grid, void* stream);
int g2_ttcf_finish(float* ttcf_dev, int64_t nframes, int64_t ld, const int64_t* bin_sums_dev, int32_t mirror,
                   void* stream);

/* ---- G3: denominator ----------------------------------------------------
 * Replaces correlate_1D (dynamix/resources/opencl/densecorrelator.cl:156-176),
 * the denominator loop of normalize_correlation (evtcorrelator.cl:70-73) and
 * the mean outer product of py_dense_correlator (dense.py:50, :55, :63).
 * D[r][tau] = sum_t S[r][t] S[r][t+tau] in int64 for n_rows rows. */
int g2_denominator(const int64_t* sums_dev, int32_t n_rows, int64_t nframes,
                   int64_t* denom_dev, void* stream);

/* ---- G4: finalize -------------------------------------------------------
 * Replaces the division of dense.py:64, densecorrelator.cl:54 and
 * normalize_correlation (evtcorrelator.cl:58-77): g2 = scale[r] * N / D in
 * float64; written as float32 (g2_f32_dev) and/or float64 (either may be NULL). */
int g2_finalize(const int64_t* numer_dev, const int64_t* denom_dev, const double* scale_dev,
                int32_t n_rows, int64_t nframes, float* g2_f32_dev, double* g2_f64_dev,
                void* stream);

/* ---- G3+G4 without allocation -------------------------------------------
 * No counterpart in the reference.  Same result as g2_denominator followed by
 * g2_finalize, for callers that cannot allocate device memory: hosts that hand
 * this library a device-memory budget that is already fully reserved (the
 * frame buffers of a detector acquisition pipeline, for instance), and loops
 * that must not call cudaMalloc/cudaFree because cudaFree waits for the whole
 * device.  The denominator lives in a file-scope device array of
 * G2_STATIC_DENOM_MAX elements (int64, 4 MiB) that every GPU which loads this
 * library holds until the process exits; n_rows * nframes above that maximum
 * returns G2_ERR_TOO_LARGE.  The caller passes N, S, scale and the outputs.
 * The first call on a device looks up that array's device address (with the
 * device current) -- make that first call before any stream capture.  The
 * address is cached per device ordinal for the life of the process: after a
 * cudaDeviceReset (or any teardown of the device's primary context) the
 * cached address is stale, so do not call this entry point again in that
 * process after such a reset.  All
 * calls share the one array and it keeps the last call's contents (every
 * element a call reads is written by the same call first, so nothing needs
 * clearing); calls whose work overlaps on the GPU race on it.  This entry
 * point allocates nothing: no cudaMalloc, no cudaFree. */
#define G2_STATIC_DENOM_MAX (1 << 19)

int g2_normalize_static(const int64_t* numer_dev, const int64_t* sums_dev, const double* scale_dev,
                        int32_t n_rows, int64_t nframes, float* g2_f32_dev, double* g2_f64_dev,
                        void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DYNAMIX_G2_H */
