// G1: gather each q-bin's pixels of every frame into the packed operand matrix
// of the Gram, and compute the per-frame bin sums S_b(t) on the way.
//
// Input-oriented: a block owns a chunk of G2_PACK_CHUNK consecutive pixels of
// the frame and walks a group of frames.  Per step it loads F frames' chunks
// with aligned 16-byte loads into shared memory (the frames are read exactly
// once, coalesced), then every thread moves its binned pixels -- up to 8 per
// thread, their destinations kept in registers for the whole kernel -- to the
// packed matrix.  Within a chunk the pixels of one bin are consecutive packed
// columns, so the stores of a warp are contiguous.  Bin sums (when asked for:
// a Gram with a row of ones gives them otherwise) and the squared-count
// energies used for the Gram's exact K split are reduced per warp (match_any +
// reduce_add), then per block in shared memory; S gets one int64 atomic per
// (chunk, bin, frame).  Energies are kept per "piece" = (64-column output
// segment) x (chunk): per step of F frames each entry takes its largest
// square, and piece_emax[p] = max over steps of the piece's sum of those,
// which bounds the piece's sum of squares in every frame; the host sums the
// pieces of a segment, which bounds the segment's energy in every frame.
// Replaces compute_sums_dense (densecorrelator.cl:65-150) and the gather /
// float32 cast of py_dense_correlator (dense.py:48-50).
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace pack {

constexpr int THREADS = 256;
constexpr int CH = G2_PACK_CHUNK;        // pixels per chunk
constexpr int EPT = CH / THREADS;        // binned pixels per thread (max)
constexpr int MAX_SLOTS = G2_PACK_MAX_SLOTS;
constexpr int MAX_PIECES = G2_PACK_MAX_PIECES;
constexpr int PPT = MAX_PIECES / THREADS;  // pieces per thread for the running maxima


// Frames per step and bytes of one frame's chunk in shared memory (+16 B for
// the unaligned start).
template <typename Tin>
struct Cfg {
  static constexpr int F = 4;
  static constexpr int CHUNK_BYTES = CH * static_cast<int>(sizeof(Tin));
  static constexpr int BUF = CHUNK_BYTES + 16;
  static constexpr int WORDS = CHUNK_BYTES / 16 + 1;  // 16-byte words covering one unaligned chunk
  static_assert(BUF % 16 == 0, "staging rows must keep 16-byte cp.async destinations aligned");
};

template <typename Tin, int MODE, bool SUMS>
__global__ void __launch_bounds__(THREADS, 3)
    pack_kernel(const Tin* __restrict__ frames, int64_t T, int64_t npix, const int32_t* __restrict__ chunk_entry_off,
                const int32_t* __restrict__ entry_dst, const uint32_t* __restrict__ entry_meta,
                const int32_t* __restrict__ chunk_slot_bin, const int32_t* __restrict__ chunk_piece_off,
                const int32_t* __restrict__ bin_kpad, uint8_t* __restrict__ packed, int64_t packed_cols,
                unsigned long long* __restrict__ sums, int n_bins, uint32_t* __restrict__ piece_emax,
                int64_t n_pieces, int32_t* __restrict__ err) {
  using C = Cfg<Tin>;
  constexpr int F = C::F;
  constexpr int PL = MODE == 1 ? 2 : 1;  // energy planes (mode 1: high and low bytes)
  __shared__ __align__(16) uint8_t s_buf[2][F][C::BUF];  // double buffer: cp.async fills one while
                                                          // the other is consumed
  __shared__ uint32_t s_sum[F][MAX_SLOTS];
  __shared__ uint32_t s_e[PL][MAX_PIECES];
  __shared__ int s_bin[MAX_SLOTS];
  __shared__ int s_kpad[MAX_SLOTS];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int64_t c = blockIdx.x;
  const int64_t p0 = c * CH;
  const int e0 = chunk_entry_off[c];
  const int ne = min(chunk_entry_off[c + 1] - e0, CH);
  const int64_t g0 = chunk_piece_off[c];
  const int64_t np64 = chunk_piece_off[c + 1] - g0;
  const int np = static_cast<int>(np64 < MAX_PIECES ? np64 : MAX_PIECES);

  int32_t dst[EPT];
  uint32_t meta[EPT];
  bool bad = false;
#pragma unroll
  for (int k = 0; k < EPT; ++k) {
    const int e = tid + k * THREADS;
    dst[k] = -1;
    meta[k] = 0;
    if (e < ne) {
      const int32_t d = entry_dst[e0 + e];
      const uint32_t m = entry_meta[e0 + e];
      const int so = static_cast<int>(m & 2047u);
      const int pc = static_cast<int>(m >> 18);
      if (d < 0 || d >= packed_cols || p0 + so >= npix || pc >= np) {
        bad = true;
      } else {
        dst[k] = d;
        meta[k] = m;
      }
    }
  }
  if (tid < MAX_SLOTS) {
    int b = chunk_slot_bin[c * MAX_SLOTS + tid];
    if (b >= n_bins) {
      bad = true;
      b = -1;
    }
    s_bin[tid] = b;
    s_kpad[tid] = (b >= 0 && MODE == 1) ? bin_kpad[b] : 0;
  }
  for (int i = tid; i < F * MAX_SLOTS; i += THREADS) (&s_sum[0][0])[i] = 0;
  for (int i = tid; i < PL * MAX_PIECES; i += THREADS) (&s_e[0][0])[i] = 0;
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
  uint32_t run_max[PL][PPT];
#pragma unroll
  for (int q = 0; q < PL; ++q)
#pragma unroll
    for (int j = 0; j < PPT; ++j) run_max[q][j] = 0;
  uint32_t range_bad = 0;
  uint32_t sq_max = 0;  // largest squared count this thread moved (modes 0 and 2)
  const int64_t total_bytes = T * npix * static_cast<int64_t>(sizeof(Tin));
  const uint8_t* fbytes = reinterpret_cast<const uint8_t*>(frames);
  const int64_t row_bytes = packed_cols * (MODE == 2 ? 1 : 2);
  __syncthreads();

  // Warp groups of equal bin slot / piece among the valid entries: fixed for
  // the whole kernel, so computed once.
  unsigned gslot[EPT], gpiece[EPT];
#pragma unroll
  for (int k = 0; k < EPT; ++k) {
    const bool valid = dst[k] >= 0;
    const unsigned amask = __ballot_sync(0xffffffffu, valid);
    gslot[k] = gpiece[k] = 0;
    if (valid) {
      gslot[k] = __match_any_sync(amask, static_cast<int>((meta[k] >> 11) & 127u));
      gpiece[k] = __match_any_sync(amask, static_cast<int>(meta[k] >> 18));
    }
  }

  // Issue the asynchronous copies of one step's F chunks into buffer `buf`:
  // aligned 16-byte words, zero-filled past the end of the frames.
  auto issue = [&](int64_t t0, int buf) {
    for (int w = tid; w < F * C::WORDS; w += THREADS) {
      const int f = w / C::WORDS;
      const int wi = w - f * C::WORDS;
      const int64_t t = t0 + f;
      const int64_t start = (t * npix + p0) * static_cast<int64_t>(sizeof(Tin));
      const int64_t a = (start & ~int64_t(15)) + static_cast<int64_t>(wi) * 16;
      int64_t avail = t < T ? total_bytes - a : 0;
      const int nbytes = avail <= 0 ? 0 : (avail >= 16 ? 16 : static_cast<int>(avail));
      const uint8_t* src = nbytes ? fbytes + a : fbytes;
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(&s_buf[buf][f][wi * 16])),
                   "l"(src), "r"(nbytes)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  const int64_t stride = static_cast<int64_t>(gridDim.y) * F;
  int64_t t0 = static_cast<int64_t>(blockIdx.y) * F;
  if (t0 < T) issue(t0, 0);
  for (int step = 0; t0 < T; ++step, t0 += stride) {
    const int buf = step & 1;
    // prefetch the next step into the other buffer (always commit a group so
    // that "wait for all but the newest group" means this step's data)
    if (t0 + stride < T) {
      issue(t0 + stride, buf ^ 1);
    } else {
      asm volatile("cp.async.commit_group;" ::: "memory");
    }
    asm volatile("cp.async.wait_group 1;" ::: "memory");
    __syncthreads();
    int delta[F];
#pragma unroll
    for (int f = 0; f < F; ++f) {
      const int64_t start = ((t0 + f) * npix + p0) * static_cast<int64_t>(sizeof(Tin));
      delta[f] = static_cast<int>(start & 15);
    }

    // ---- move binned pixels to the packed matrix, reduce sums and energies
#pragma unroll
    for (int k = 0; k < EPT; ++k) {
      if (dst[k] < 0) continue;
      const int so = static_cast<int>(meta[k] & 2047u);
      const int sl = static_cast<int>((meta[k] >> 11) & 127u);
      const int pc = static_cast<int>(meta[k] >> 18);
      const bool lead_s = (__ffs(gslot[k]) - 1) == lane;
      const bool lead_p = (__ffs(gpiece[k]) - 1) == lane;
      uint32_t e0 = 0, e1 = 0;  // the entry's largest squared value(s) over the step's frames
#pragma unroll
      for (int f = 0; f < F; ++f) {
        const int64_t t = t0 + f;
        uint32_t v = 0;
        if (t < T) {
          const int off = delta[f] + so * static_cast<int>(sizeof(Tin));
          v = sizeof(Tin) == 1 ? static_cast<uint32_t>(s_buf[buf][f][off])
                               : static_cast<uint32_t>(*reinterpret_cast<const uint16_t*>(&s_buf[buf][f][off]));
          uint8_t* row = packed + t * row_bytes;
          if (MODE == 2) {
            range_bad |= v > 16u ? 1u : 0u;
            row[dst[k]] = static_cast<uint8_t>(v);
          } else if (MODE == 0) {
            range_bad |= v > 2048u ? 1u : 0u;
            reinterpret_cast<uint16_t*>(row)[dst[k]] = static_cast<uint16_t>(v);
          } else {
            reinterpret_cast<uint16_t*>(row)[dst[k]] = static_cast<uint16_t>(v >> 8);
            const int64_t d1 = static_cast<int64_t>(dst[k]) + s_kpad[sl];
            if (d1 < packed_cols)
              reinterpret_cast<uint16_t*>(row)[d1] = static_cast<uint16_t>(v & 255u);
            else
              range_bad |= 2u;
          }
        }
        if (SUMS) {
          const uint32_t vs = __reduce_add_sync(gslot[k], v);
          if (lead_s && vs) atomicAdd(&s_sum[f][sl], vs);
        }
        if (MODE == 1) {
          const uint32_t h = v >> 8, l = v & 255u;
          e0 = max(e0, h * h);
          e1 = max(e1, l * l);
        } else {
          // counts above the mode's range are flagged; keep the energy finite
          e0 = max(e0, v <= 2048u ? v * v : 4194304u);
        }
      }
      // The piece's sum over its entries of each entry's largest square over
      // the step's frames bounds the piece's sum of squares in each of them:
      // one reduction per step instead of one per frame.
      const uint32_t ea = __reduce_add_sync(gpiece[k], e0);
      if (lead_p && ea) atomicAdd(&s_e[0][pc], ea);
      if (MODE == 1) {
        const uint32_t eb = __reduce_add_sync(gpiece[k], e1);
        if (lead_p && eb) atomicAdd(&s_e[1][pc], eb);
      } else {
        sq_max = max(sq_max, e0);
      }
    }
    __syncthreads();

    // ---- flush bin sums, fold piece energies into running maxima
    for (int i = tid; SUMS && i < F * MAX_SLOTS; i += THREADS) {
      const int f = i / MAX_SLOTS, sl = i - f * MAX_SLOTS;
      const uint32_t s = s_sum[f][sl];
      if (s) {
        const int b = s_bin[sl];
        if (b >= 0 && t0 + f < T)
          atomicAdd(&sums[static_cast<int64_t>(b) * T + t0 + f], static_cast<unsigned long long>(s));
        s_sum[f][sl] = 0;
      }
    }
#pragma unroll
    for (int q = 0; q < PL; ++q)
#pragma unroll
      for (int j = 0; j < PPT; ++j) {
        const int pc = tid + j * THREADS;
        if (pc < np) {
          run_max[q][j] = max(run_max[q][j], s_e[q][pc]);
          s_e[q][pc] = 0;
        }
      }
    // the accumulators are reused and the buffer just read is refilled by the
    // copies issued at the top of the next step: wait for every thread here
    __syncthreads();
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
#pragma unroll
  for (int q = 0; q < PL; ++q)
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
      const int pc = tid + j * THREADS;
      if (pc < np && g0 + pc < n_pieces && run_max[q][j])
        atomicMax(&piece_emax[q * n_pieces + g0 + pc], run_max[q][j]);
    }
  if (MODE != 1) {
    // the chunk's largest squared count, in plane 1 at its first piece
    const uint32_t m = __reduce_max_sync(0xffffffffu, sq_max);
    if (lane == 0 && m && np > 0 && g0 < n_pieces) atomicMax(&piece_emax[n_pieces + g0], m);
  }
  if (range_bad & 1u) atomicOr(err, G2_DEVERR_RANGE);
  if (range_bad & 2u) atomicOr(err, G2_DEVERR_BOUNDS);
}

// ---- e4m3 (counts <= 16): a pure byte permutation --------------------------
// The raw count bytes are the e4m3 operand (bytes 0..16 read as e4m3 are
// count * 2^-9), so no conversion is needed; counts <= 16 bound every Gram sum
// by themselves, so no energies are needed; and the bin sums come from the
// Gram (row of ones), so this kernel only moves bytes.  A thread owns up to WPT
// "words" = 4 consecutive packed columns of one bin; per frame it reads the 4
// source bytes from the staged chunk -- one funnel shift of two aligned 32-bit
// shared loads when the sources are consecutive pixels (inside a run of the
// annulus), four byte loads otherwise -- and stores one 32-bit word (byte
// stores only for the partial words at the ends of a bin's run in the chunk,
// whose other bytes belong to the neighbouring chunk).
constexpr int WPT = G2_PACK_WORDS_PER_CHUNK / THREADS;
constexpr uint32_t NO_SRC = 0xFFFu;

template <typename Tin>
__global__ void __launch_bounds__(THREADS, 4)
    pack_e4m3_kernel(const Tin* __restrict__ frames, int64_t T, int64_t npix,
                     const int32_t* __restrict__ chunk_word_off, const int32_t* __restrict__ word_dst,
                     const uint2* __restrict__ word_src, uint8_t* __restrict__ packed, int64_t packed_cols,
                     int32_t* __restrict__ err) {
  using C = Cfg<Tin>;
  constexpr int F = C::F;
  // rows stay multiples of 16 bytes (cp.async destinations); the 16 spare bytes
  // cover the second word of the funnel-shift read at the end of a chunk
  __shared__ __align__(16) uint8_t s_buf[2][F][C::BUF + 16];

  const int tid = threadIdx.x;
  const int64_t c = blockIdx.x;
  const int64_t p0 = c * CH;
  const int w0 = chunk_word_off[c];
  const int nw = min(chunk_word_off[c + 1] - w0, WPT * THREADS);

  int32_t dst[WPT];
  uint32_t src[WPT][4];
  bool full[WPT], run4[WPT];
  bool bad = false;
#pragma unroll
  for (int k = 0; k < WPT; ++k) {
    const int w = tid + k * THREADS;
    dst[k] = -1;
    full[k] = run4[k] = false;
#pragma unroll
    for (int i = 0; i < 4; ++i) src[k][i] = NO_SRC;
    if (w < nw) {
      const int32_t d = word_dst[w0 + w];
      const uint2 m = word_src[w0 + w];
      if (d >= 0) {
        uint32_t sv[4] = {m.x & 0xFFFu, (m.x >> 12) & 0xFFFu, (m.x >> 24) | ((m.y & 0xFu) << 8),
                          (m.y >> 4) & 0xFFFu};
        bool ok = (d & 3) == 0 && d + 4 <= packed_cols;
        bool all = true;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          if (sv[i] == NO_SRC) {
            all = false;
          } else if (sv[i] >= static_cast<uint32_t>(CH) || p0 + sv[i] >= npix) {
            ok = false;
          }
        }
        const bool consec = all && sv[1] == sv[0] + 1 && sv[2] == sv[0] + 2 && sv[3] == sv[0] + 3;
        if (!ok) {
          bad = true;
        } else {
          dst[k] = d;
          full[k] = all;
          run4[k] = consec && sizeof(Tin) == 1;
#pragma unroll
          for (int i = 0; i < 4; ++i) src[k][i] = sv[i];
        }
      }
    }
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
  uint32_t range_bad = 0;
  const int64_t total_bytes = T * npix * static_cast<int64_t>(sizeof(Tin));
  const uint8_t* fbytes = reinterpret_cast<const uint8_t*>(frames);

  auto issue = [&](int64_t t0, int buf) {
    for (int w = tid; w < F * C::WORDS; w += THREADS) {
      const int f = w / C::WORDS;
      const int wi = w - f * C::WORDS;
      const int64_t t = t0 + f;
      const int64_t start = (t * npix + p0) * static_cast<int64_t>(sizeof(Tin));
      const int64_t a = (start & ~int64_t(15)) + static_cast<int64_t>(wi) * 16;
      const int64_t avail = t < T ? total_bytes - a : 0;
      const int nbytes = avail <= 0 ? 0 : (avail >= 16 ? 16 : static_cast<int>(avail));
      const uint8_t* srcp = nbytes ? fbytes + a : fbytes;
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(&s_buf[buf][f][wi * 16])),
                   "l"(srcp), "r"(nbytes)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  const int64_t stride = static_cast<int64_t>(gridDim.y) * F;
  int64_t t0 = static_cast<int64_t>(blockIdx.y) * F;
  if (t0 < T) issue(t0, 0);
  for (int step = 0; t0 < T; ++step, t0 += stride) {
    const int buf = step & 1;
    if (t0 + stride < T) {
      issue(t0 + stride, buf ^ 1);
    } else {
      asm volatile("cp.async.commit_group;" ::: "memory");
    }
    asm volatile("cp.async.wait_group 1;" ::: "memory");
    __syncthreads();
#pragma unroll
    for (int f = 0; f < F; ++f) {
      const int64_t t = t0 + f;
      if (t >= T) break;
      const int delta = static_cast<int>(((t * npix + p0) * static_cast<int64_t>(sizeof(Tin))) & 15);
      const uint8_t* base = &s_buf[buf][f][0];
      uint8_t* row = packed + t * packed_cols;
#pragma unroll
      for (int k = 0; k < WPT; ++k) {
        if (dst[k] < 0) continue;
        uint32_t word = 0;
        if (run4[k]) {
          // 4 consecutive source bytes at byte offset o: two aligned words and a funnel shift
          const uint32_t o = static_cast<uint32_t>(delta) + src[k][0];
          const uint32_t* wp = reinterpret_cast<const uint32_t*>(base + (o & ~3u));
          word = __funnelshift_r(wp[0], wp[1], 8 * (o & 3u));
          // a byte > 16: ((b + 0x6F) | b) has bit 7 set (bytes are < 256, no carry between them)
          range_bad |= ((word & 0x7F7F7F7Fu) + 0x6F6F6F6Fu | word) & 0x80808080u;
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            if (src[k][i] != NO_SRC) {
              const uint32_t v = sizeof(Tin) == 1
                                     ? static_cast<uint32_t>(base[delta + src[k][i]])
                                     : static_cast<uint32_t>(
                                           *reinterpret_cast<const uint16_t*>(base + delta + 2 * src[k][i]));
              range_bad |= v > 16u ? 1u : 0u;
              word |= (v & 0xFFu) << (8 * i);
            }
          }
        }
        if (full[k]) {
          *reinterpret_cast<uint32_t*>(row + dst[k]) = word;
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if (src[k][i] != NO_SRC) row[dst[k] + i] = static_cast<uint8_t>(word >> (8 * i));
        }
      }
    }
    // the buffer just read is refilled by the copies issued at the next step
    __syncthreads();
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  if (range_bad) atomicOr(err, G2_DEVERR_RANGE);
}

// ---- e4m3 from u8 counts, by work units -----------------------------------
// The same byte permutation as pack_e4m3_kernel, organised so that a warp
// never diverges: the host cuts each chunk's destination bytes into units
// of four classes -- 16 bytes from 16 consecutive source bytes (one 16-byte
// store), 4 from 4 consecutive (one 32-bit funnel shift), 4 gathered from 4
// arbitrary source bytes, single bytes (words shared with a neighbouring
// chunk or bin padding) -- and groups them in blocks of 32 units of one
// class, each run by one warp over a step's F frames.  Units are uint4
// {destination (in units of the class's size), source(s), source(s), class}.
// The range check ORs every moved byte into one word per thread: with counts
// <= 15 every byte of it stays <= 15, and only a count of 16 or more can make
// one exceed 16, in which case G2_DEVERR_RANGE_CHECK asks the caller for the
// exact maximum (g2_binned_max) -- one instruction per word instead of four.
constexpr uint32_t UNIT_VEC = 1, UNIT_WORD = 2, UNIT_GATHER = 3, UNIT_BYTE = 4;

// One unit over the step's nf frames: source rows at base + delta[f], packed
// rows at row[f].
template <int F>
__device__ __forceinline__ void move_unit(const uint4& u, const uint8_t* base, const uint32_t (&delta)[F],
                                          uint8_t* const (&row)[F], int nf, int64_t n_vec, int64_t n_word,
                                          int64_t packed_cols, uint32_t& seen, bool& bad) {
  if (u.w == UNIT_VEC) {
    if (u.x >= n_vec || u.y > CH - 16) {
      bad = true;
      return;
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
      if (f >= nf) break;
      // the 16 bytes at o from the two aligned 16-byte words around them:
      // two 16-byte shared loads (a warp's consecutive units read one
      // contiguous span, 4 wavefronts each) instead of five 4-byte loads
      // that a 16-byte lane stride puts four lanes on one bank
      const uint32_t o = delta[f] + u.y;
      const uint4 q0 = *reinterpret_cast<const uint4*>(base + (o & ~15u));
      const uint4 q1 = *reinterpret_cast<const uint4*>(base + (o & ~15u) + 16);
      const uint32_t w[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
      const uint32_t k = (o >> 2) & 3u, sh = 8 * (o & 3u);
      uint32_t x[5];
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        const uint32_t lo = (k & 1u) ? w[i + 1] : w[i];
        const uint32_t hi = (k & 1u) ? w[i + 3] : w[i + 2];
        x[i] = (k & 2u) ? hi : lo;
      }
      uint4 v;
      v.x = __funnelshift_r(x[0], x[1], sh);
      v.y = __funnelshift_r(x[1], x[2], sh);
      v.z = __funnelshift_r(x[2], x[3], sh);
      v.w = __funnelshift_r(x[3], x[4], sh);
      seen |= v.x | v.y | v.z | v.w;
      *reinterpret_cast<uint4*>(row[f] + 16 * static_cast<int64_t>(u.x)) = v;
    }
  } else if (u.w == UNIT_WORD) {
    if (u.x >= n_word || u.y > CH - 4) {
      bad = true;
      return;
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
      if (f >= nf) break;
      const uint32_t o = delta[f] + u.y;
      const uint32_t* p = reinterpret_cast<const uint32_t*>(base + (o & ~3u));
      const uint32_t v = __funnelshift_r(p[0], p[1], 8 * (o & 3u));
      seen |= v;
      *reinterpret_cast<uint32_t*>(row[f] + 4 * static_cast<int64_t>(u.x)) = v;
    }
  } else if (u.w == UNIT_GATHER) {
    const uint32_t s0 = u.y & 0xFFFFu, s1 = u.y >> 16, s2 = u.z & 0xFFFFu, s3 = u.z >> 16;
    if (u.x >= n_word || s0 >= CH || s1 >= CH || s2 >= CH || s3 >= CH) {
      bad = true;
      return;
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
      if (f >= nf) break;
      const uint8_t* q = base + delta[f];
      const uint32_t v = static_cast<uint32_t>(q[s0]) | (static_cast<uint32_t>(q[s1]) << 8) |
                         (static_cast<uint32_t>(q[s2]) << 16) | (static_cast<uint32_t>(q[s3]) << 24);
      seen |= v;
      *reinterpret_cast<uint32_t*>(row[f] + 4 * static_cast<int64_t>(u.x)) = v;
    }
  } else if (u.w == UNIT_BYTE) {
    if (u.x >= packed_cols || u.y >= CH) {
      bad = true;
      return;
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
      if (f >= nf) break;
      const uint8_t v = base[delta[f] + u.y];
      seen |= v;
      row[f][u.x] = v;
    }
  }
}

// The kernel: a CTA owns one 2048-pixel chunk over every gridDim.y-th step of
// F frames.  The frames stream through a ring of RING_STAGES steps of staged
// rows: warp 0 lane 0 copies each step's F frame rows of the chunk with 1-D
// bulk copies (one per frame, completing on the stage's full barrier); warps
// 1..RING_MOVERS each keep one block of units in registers for the whole
// launch, move it at every step and arrive on the stage's empty barrier.  No
// block-wide barrier per step, no per-thread copy instructions, and warps
// without a block leave at once (a chunk of the 514 x 1030 detector holds 9
// blocks on average, 13 at most): fewer instructions per moved byte than a
// ring of per-thread cp.async copies and __syncthreads, which counts most
// when the pack runs beside the Gram on the same SMs.  The ring (16.6 KB)
// leaves room for a pack CTA beside a Gram CTA on one SM.
constexpr int RING_THREADS = 512;
constexpr int RING_MOVERS = RING_THREADS / 32 - 1;  // chunks rarely hold more than 13 blocks
constexpr int RING_STAGES = 2;

__global__ void __launch_bounds__(RING_THREADS, 2)
    pack_e4m3_ring_kernel(const uint8_t* __restrict__ frames, int64_t T, int64_t npix,
                          const int32_t* __restrict__ block_off, const uint4* __restrict__ units,
                          uint8_t* __restrict__ packed, int64_t packed_cols, int32_t* __restrict__ err) {
  using C = Cfg<uint8_t>;
  constexpr int F = C::F;
  constexpr int ROW = C::BUF + 16;                        // staging row: the chunk, its unaligned start, spare words
  constexpr uint32_t SPAN = C::WORDS * 16;                // bytes per frame: the chunk from its aligned start
  static_assert(ROW % 16 == 0 && SPAN <= ROW, "bulk copy rows");
  __shared__ __align__(128) uint8_t s_buf[RING_STAGES][F][ROW];
  __shared__ __align__(8) uint64_t full[RING_STAGES];
  __shared__ __align__(8) uint64_t empty[RING_STAGES];
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t c = blockIdx.x;
  const int64_t p0 = c * CH;  // < npix: the launch has ceil(npix / CH) chunks
  const int b0 = block_off[c];
  const int nb = block_off[c + 1] - b0;
  const int movers = nb < RING_MOVERS ? nb : RING_MOVERS;
  if (movers <= 0) return;  // no packed byte comes from this chunk
  if (threadIdx.x == 0) {
    for (int s = 0; s < RING_STAGES; ++s) {
      mbar_init(&full[s], 1);        // the copier's arrive.expect_tx, then the bytes
      mbar_init(&empty[s], movers);  // one arrival per mover warp
    }
    s_abort = 0;
    fence_mbar_init();
  }
  __syncthreads();
  volatile int* abort_flag = &s_abort;
  const int64_t total_bytes = T * npix;
  const int64_t stride = static_cast<int64_t>(gridDim.y) * F;
  const int64_t first = static_cast<int64_t>(blockIdx.y) * F;

  if (warp == 0) {
    // ------------------------------------------------------------ copier
    if (lane == 0) {
      int64_t k = 0;
      for (int64_t t0 = first; t0 < T; t0 += stride, ++k) {
        const int s = static_cast<int>(k % RING_STAGES);
        const uint32_t ph = static_cast<uint32_t>((k / RING_STAGES) & 1);
        if (k >= RING_STAGES && !mbar_wait(&empty[s], ph ^ 1u, abort_flag, err)) break;
        const int nf = static_cast<int>(T - t0 < F ? T - t0 : F);
        uint32_t bytes = 0;
#pragma unroll
        for (int f = 0; f < F; ++f) {
          if (f >= nf) break;
          const int64_t a = ((t0 + f) * npix + p0) & ~int64_t(15);
          const int64_t avail = total_bytes - a;  // > 0
          const uint32_t n = avail >= SPAN ? SPAN : static_cast<uint32_t>(avail);
          // the stack's last bytes short of a multiple of 16: plain copies,
          // made visible by the arrive below (only the last frame has them)
          for (uint32_t i = n & ~15u; i < n; ++i) s_buf[s][f][i] = frames[a + i];
          bytes += n & ~15u;
        }
        mbar_arrive_expect_tx(&full[s], bytes);
#pragma unroll
        for (int f = 0; f < F; ++f) {
          if (f >= nf) break;
          const int64_t a = ((t0 + f) * npix + p0) & ~int64_t(15);
          const int64_t avail = total_bytes - a;
          const uint32_t n = (avail >= SPAN ? SPAN : static_cast<uint32_t>(avail)) & ~15u;
          if (n) bulk_load_1d(&s_buf[s][f][0], frames + a, n, &full[s]);
        }
      }
      // after a timed-out wait a copy of this CTA may still be landing
      if (*abort_flag) {
        const uint64_t w0 = global_timer_ns();
        while (global_timer_ns() - w0 < 100000ull) {
        }
      }
    }
    return;
  }

  // -------------------------------------------------------------- movers
  const int mw = warp - 1;
  if (mw >= movers) return;
  const uint4 u0 = units[static_cast<int64_t>(b0 + mw) * 32 + lane];
  const int64_t n_vec = packed_cols / 16, n_word = packed_cols / 4;
  uint32_t seen = 0;  // OR of every moved byte
  bool bad = false;
  int64_t k = 0;
  for (int64_t t0 = first; t0 < T; t0 += stride, ++k) {
    const int s = static_cast<int>(k % RING_STAGES);
    const uint32_t ph = static_cast<uint32_t>((k / RING_STAGES) & 1);
    if (!mbar_wait(&full[s], ph, abort_flag, err)) break;
    const int nf = static_cast<int>(T - t0 < F ? T - t0 : F);
    uint32_t delta[F];
    uint8_t* row[F];
#pragma unroll
    for (int f = 0; f < F; ++f) {
      delta[f] = static_cast<uint32_t>(((t0 + f) * npix + p0) & 15) + f * ROW;
      row[f] = packed + (t0 + f) * packed_cols;
    }
    const uint8_t* base = &s_buf[s][0][0];
    move_unit<F>(u0, base, delta, row, nf, n_vec, n_word, packed_cols, seen, bad);
    for (int blk = mw + RING_MOVERS; blk < nb; blk += RING_MOVERS) {
      const uint4 u = units[static_cast<int64_t>(b0 + blk) * 32 + lane];
      move_unit<F>(u, base, delta, row, nf, n_vec, n_word, packed_cols, seen, bad);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
  if (((seen & 0x7F7F7F7Fu) + 0x6F6F6F6Fu | seen) & 0x80808080u) atomicOr(err, G2_DEVERR_RANGE_CHECK);
}

template <typename Tin>
__global__ void binned_max_kernel(const Tin* __restrict__ frames, int64_t T, int64_t npix,
                                  const int32_t* __restrict__ col_src, int64_t n_cols, uint32_t* __restrict__ out) {
  uint32_t m = 0;
  const int64_t total = T * n_cols;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t t = i / n_cols;
    const int32_t s = col_src[i - t * n_cols];
    if (s >= 0 && s < npix) m = max(m, static_cast<uint32_t>(frames[t * npix + s]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

template <typename Tin, int MODE>
void launch(dim3 grid, cudaStream_t st, const void* frames, int64_t T, int64_t npix, const int32_t* ceo,
            const int32_t* ed, const uint32_t* em, const int32_t* csb, const int32_t* cpo, const int32_t* bk,
            void* packed, int64_t cols, int64_t* sums, int n_bins, uint32_t* pe, int64_t n_pieces, int32_t* err) {
  auto* s = reinterpret_cast<unsigned long long*>(sums);
  if (sums)
    pack_kernel<Tin, MODE, true><<<grid, THREADS, 0, st>>>(reinterpret_cast<const Tin*>(frames), T, npix, ceo, ed,
                                                           em, csb, cpo, bk, reinterpret_cast<uint8_t*>(packed),
                                                           cols, s, n_bins, pe, n_pieces, err);
  else
    pack_kernel<Tin, MODE, false><<<grid, THREADS, 0, st>>>(reinterpret_cast<const Tin*>(frames), T, npix, ceo, ed,
                                                            em, csb, cpo, bk, reinterpret_cast<uint8_t*>(packed),
                                                            cols, s, n_bins, pe, n_pieces, err);
}

}  // namespace pack
}  // namespace g2

extern "C" int g2_pack_frames(const void* frames_dev, int32_t elem_bytes, int64_t nframes, int64_t npix,
                              const int32_t* chunk_entry_off_dev, const int32_t* entry_dst_dev,
                              const uint32_t* entry_meta_dev, const int32_t* chunk_slot_bin_dev,
                              const int32_t* chunk_piece_off_dev, const int32_t* bin_kpad_dev, int64_t n_chunks,
                              int32_t mode, void* packed_dev, int64_t packed_cols, int64_t* sums_dev, int32_t n_bins,
                              uint32_t* piece_emax_dev, int64_t n_pieces, int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!frames_dev || !chunk_entry_off_dev || !entry_dst_dev || !entry_meta_dev || !chunk_slot_bin_dev ||
      !chunk_piece_off_dev || !packed_dev || !piece_emax_dev || !err_dev)
    return G2_ERR_ARG;
  if ((elem_bytes != 1 && elem_bytes != 2) || nframes <= 0 || npix <= 0 || n_chunks < 0 ||
      n_chunks != (npix + G2_PACK_CHUNK - 1) / G2_PACK_CHUNK || mode < 0 || mode > 2 ||
      (mode == 1 && (!bin_kpad_dev || elem_bytes != 2)) || packed_cols <= 0 || packed_cols % G2_PAD != 0 ||
      n_bins <= 0 || n_pieces < 0)
    return G2_ERR_ARG;
  if (!aligned(packed_dev, 16) || !aligned(frames_dev, 16)) return G2_ERR_ARG;
  if (n_chunks == 0) return G2_OK;
  if (n_chunks > 0x7fffffff) return G2_ERR_TOO_LARGE;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int F = elem_bytes == 1 ? pack::Cfg<uint8_t>::F : pack::Cfg<uint16_t>::F;
  int64_t gy = (static_cast<int64_t>(sms) * 16 + n_chunks - 1) / n_chunks;
  const int64_t max_gy = (nframes + F - 1) / F;
  if (gy > max_gy) gy = max_gy;
  if (gy > 65535) gy = 65535;
  if (gy < 1) gy = 1;
  dim3 grid(static_cast<unsigned>(n_chunks), static_cast<unsigned>(gy));
  cudaStream_t st = as_stream(stream);
#define G2_PACK_ARGS                                                                                                 \
  grid, st, frames_dev, nframes, npix, chunk_entry_off_dev, entry_dst_dev, entry_meta_dev, chunk_slot_bin_dev,       \
      chunk_piece_off_dev, bin_kpad_dev, packed_dev, packed_cols, sums_dev, n_bins, piece_emax_dev, n_pieces, err_dev
  if (elem_bytes == 1) {
    if (mode == 0) pack::launch<uint8_t, 0>(G2_PACK_ARGS);
    else pack::launch<uint8_t, 2>(G2_PACK_ARGS);
  } else {
    if (mode == 0) pack::launch<uint16_t, 0>(G2_PACK_ARGS);
    else if (mode == 1) pack::launch<uint16_t, 1>(G2_PACK_ARGS);
    else pack::launch<uint16_t, 2>(G2_PACK_ARGS);
  }
#undef G2_PACK_ARGS
  return launch_status();
}

extern "C" int g2_pack_e4m3(const void* frames_dev, int32_t elem_bytes, int64_t nframes, int64_t npix,
                            const int32_t* chunk_word_off_dev, const int32_t* word_dst_dev,
                            const uint32_t* word_src_dev, int64_t n_chunks, void* packed_dev, int64_t packed_cols,
                            int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!frames_dev || !chunk_word_off_dev || !word_dst_dev || !word_src_dev || !packed_dev || !err_dev)
    return G2_ERR_ARG;
  if ((elem_bytes != 1 && elem_bytes != 2) || nframes <= 0 || npix <= 0 ||
      n_chunks != (npix + G2_PACK_CHUNK - 1) / G2_PACK_CHUNK || packed_cols <= 0 || packed_cols % G2_PAD != 0)
    return G2_ERR_ARG;
  if (!aligned(packed_dev, 16) || !aligned(frames_dev, 16) || !aligned(word_src_dev, 8)) return G2_ERR_ARG;
  if (n_chunks == 0) return G2_OK;
  if (n_chunks > 0x7fffffff) return G2_ERR_TOO_LARGE;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int F = elem_bytes == 1 ? pack::Cfg<uint8_t>::F : pack::Cfg<uint16_t>::F;
  int64_t gy = (static_cast<int64_t>(sms) * 16 + n_chunks - 1) / n_chunks;
  const int64_t max_gy = (nframes + F - 1) / F;
  if (gy > max_gy) gy = max_gy;
  if (gy > 65535) gy = 65535;
  if (gy < 1) gy = 1;
  dim3 grid(static_cast<unsigned>(n_chunks), static_cast<unsigned>(gy));
  auto* ws = reinterpret_cast<const uint2*>(word_src_dev);
  auto* out = reinterpret_cast<uint8_t*>(packed_dev);
  if (elem_bytes == 1)
    pack::pack_e4m3_kernel<uint8_t><<<grid, pack::THREADS, 0, as_stream(stream)>>>(
        reinterpret_cast<const uint8_t*>(frames_dev), nframes, npix, chunk_word_off_dev, word_dst_dev, ws, out,
        packed_cols, err_dev);
  else
    pack::pack_e4m3_kernel<uint16_t><<<grid, pack::THREADS, 0, as_stream(stream)>>>(
        reinterpret_cast<const uint16_t*>(frames_dev), nframes, npix, chunk_word_off_dev, word_dst_dev, ws, out,
        packed_cols, err_dev);
  return launch_status();
}

extern "C" int g2_pack_e4m3_units(const void* frames_dev, int64_t nframes, int64_t npix,
                                  const int32_t* unit_block_off_dev, const uint32_t* units_dev, int64_t n_chunks,
                                  void* packed_dev, int64_t packed_cols, int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!frames_dev || !unit_block_off_dev || !units_dev || !packed_dev || !err_dev) return G2_ERR_ARG;
  if (nframes <= 0 || npix <= 0 || n_chunks != (npix + G2_PACK_CHUNK - 1) / G2_PACK_CHUNK || packed_cols <= 0 ||
      packed_cols % G2_PAD != 0)
    return G2_ERR_ARG;
  if (!aligned(packed_dev, 16) || !aligned(frames_dev, 16) || !aligned(units_dev, 16)) return G2_ERR_ARG;
  if (n_chunks == 0) return G2_OK;
  if (n_chunks > 0x7fffffff) return G2_ERR_TOO_LARGE;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int F = pack::Cfg<uint8_t>::F;
  int64_t gy = (static_cast<int64_t>(sms) * 16 + n_chunks - 1) / n_chunks;
  const int64_t max_gy = (nframes + F - 1) / F;
  if (gy > max_gy) gy = max_gy;
  if (gy > 65535) gy = 65535;
  if (gy < 1) gy = 1;
  dim3 grid(static_cast<unsigned>(n_chunks), static_cast<unsigned>(gy));
  pack::pack_e4m3_ring_kernel<<<grid, pack::RING_THREADS, 0, as_stream(stream)>>>(
      reinterpret_cast<const uint8_t*>(frames_dev), nframes, npix, unit_block_off_dev,
      reinterpret_cast<const uint4*>(units_dev), reinterpret_cast<uint8_t*>(packed_dev), packed_cols, err_dev);
  return launch_status();
}

extern "C" int g2_binned_max(const void* frames_dev, int32_t elem_bytes, int64_t nframes, int64_t npix,
                             const int32_t* col_src_dev, int64_t n_cols, uint32_t* max_dev, void* stream) {
  using namespace g2;
  if (!frames_dev || !col_src_dev || !max_dev || (elem_bytes != 1 && elem_bytes != 2) || nframes <= 0 ||
      npix <= 0 || n_cols < 0)
    return G2_ERR_ARG;
  if (n_cols == 0) return G2_OK;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const unsigned grid = static_cast<unsigned>(sms * 8);
  if (elem_bytes == 1)
    pack::binned_max_kernel<uint8_t><<<grid, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const uint8_t*>(frames_dev), nframes, npix, col_src_dev, n_cols, max_dev);
  else
    pack::binned_max_kernel<uint16_t><<<grid, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const uint16_t*>(frames_dev), nframes, npix, col_src_dev, n_cols, max_dev);
  return launch_status();
}
