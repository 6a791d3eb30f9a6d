// Tensor-core (tcgen05) slice-product backend: tile constants.  The argument
// blocks PackArgs / TcArgs live in engine.h; see gemm_tc.cu for the method.
#pragma once

#include <cuda_runtime.h>

#include "engine.h"

namespace tdcc {

constexpr int TC_BM = 128;                   // UMMA M (rows of A per CTA)
constexpr int TC_BN = 64;                    // UMMA N (rows of B per CTA)
constexpr int TC_BK = 64;                    // K per TMA box (128 B of BF16)
constexpr int TC_STAGES = 8;                 // shared-memory ring depth
constexpr int TC_CHUNK_KB = 16;              // 1024-wide K chunks (exact FP32 sums)
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;
constexpr int TC_B_BYTES = TC_BN * TC_BK * 2;
constexpr int TC_SMEM_BYTES = 1024 + TC_STAGES * (TC_A_BYTES + TC_B_BYTES) + 2048;
constexpr int TC_MAX_SLICES = 6;
constexpr int TC_EPI_WARPS = 16;             // TMEM drain warps (four per lane quarter)
constexpr int TC_THREADS = 64 + 32 * TC_EPI_WARPS;  // + TMA producer warp + MMA warp

}  // namespace tdcc
