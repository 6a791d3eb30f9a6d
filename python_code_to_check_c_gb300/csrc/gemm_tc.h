// Tensor-core (tcgen05) slice-product backend: tile constants.  The argument
// blocks PackArgs / TcArgs live in engine.h; see gemm_tc.cu for the method.
#pragma once

#include <cuda_runtime.h>

#include "engine.h"

namespace tdcc {

constexpr int TC_BM = 128;                   // UMMA M (rows of A per CTA)
constexpr int TC_BN = 64;                    // packed B rows are padded to this (both variants)
constexpr int TC_BK = 64;                    // K per TMA box (128 B of BF16)
constexpr int TC_CHUNK_KB = 8;               // 512-wide K chunks (exact FP32 level sums)
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;
constexpr int TC_MAX_SLICES = 6;

// Kernel variants: tile width BN (UMMA N), ring depth, TMEM-drain warps and
// CTAs per SM.  The ring must hold the S slices of one K block (STAGES >= S).
template <int BN_, int STAGES_, int EPI_, int MINB_>
struct TcCfg {
  static constexpr int BN = BN_, STAGES = STAGES_, EPI = EPI_, MINB = MINB_;
  static constexpr int B_BYTES = BN * TC_BK * 2;
  static constexpr int THREADS = 64 + 32 * EPI;  // + TMA producer warp + MMA warp
  static constexpr int SMEM = 1024 + STAGES * (TC_A_BYTES + B_BYTES) + 2048;
};
// one CTA per SM: 64-wide tile, 8 stages, 16 drain warps (four per lane quarter)
using TcWide = TcCfg<64, 8, 16, 1>;
// two CTAs per SM (one's drain overlaps the other's MMAs): 32-wide tile, 5
// stages, 8 drain warps; TMEM (S + 2) x 32 <= 256 columns, so S <= 5
using TcNarrow = TcCfg<32, 5, 8, 2>;
// 128-wide tile, one K chunk per CTA (no int64 partial sums): S x 128 <= 512
// TMEM columns, so S <= 4.  Its ring holds single slices (one 128 x 64 tile
// of A or of B, 16 KB, SWIZZLE_128B) in 12 slots, each with its own
// barriers, so that a slice is released after its last product rather than
// with the whole K block; 16 drain warps; one CTA per SM.
struct TcTile128 {
  static constexpr int BN = 128, STAGES = 12, EPI = 16, MINB = 1;
  static constexpr int SLOT_BYTES = TC_BM * TC_BK * 2;  // 16 KB (A: 128 rows, B: BN = 128 rows)
  static constexpr int THREADS = 64 + 32 * EPI;
  // + 1 KB alignment and the barrier block
  static constexpr int SMEM = 1024 + STAGES * SLOT_BYTES + 2048;
};
constexpr int TC_TILE128_MAX_S = 4;

// Persistent 64-column form for S <= 4 slices: one CTA per SM walks a list
// of output tiles; S level accumulators of 64 columns make one TMEM buffer
// (S x 64 <= 256 columns), two buffers fill TMEM, so that the drain warps
// empty tile i's buffer while the MMAs of tile i + 1 fill the other.  Slices
// of A (128 x 64, 16 KB) and of B (64 x 64, 8 KB) have rings of their own;
// the drain stages 16 columns per warp in an area of its own (the rings keep
// loading the next tile meanwhile).
struct TcPersist {
  static constexpr int BN = 64, EPI = 16, MINB = 1;
  static constexpr int RA = 5, RB = 6;               // ring slots of A and B slices
  static constexpr int A_SLOT = TC_BM * TC_BK * 2;   // 16 KB
  static constexpr int B_SLOT = BN * TC_BK * 2;      // 8 KB
  static constexpr int STAGE_WARP = 4608;            // staging bytes per drain warp
  static constexpr int THREADS = 64 + 32 * EPI;
  static constexpr int SMEM = 1024 + RA * A_SLOT + RB * B_SLOT + EPI * STAGE_WARP + 2048;
};

// K blocks one CTA of the 128-wide tile may accumulate exactly: the FP32
// level sums grow by at most sum_{s+t=L} |q_s| |q_t| per K index (|q_1| <=
// 128, |q_s| <= 64 for s >= 2) and must stay within 2^24.
constexpr int tc_chunk_kblocks(int S) {
  return S <= 2 ? 16 : S == 3 ? (1 << 24) / (20480 * 64) : (1 << 24) / (24576 * 64);
}

}  // namespace tdcc
