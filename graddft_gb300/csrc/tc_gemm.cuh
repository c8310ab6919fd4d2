// tc_gemm.cuh - tensor-core GEMMs on packed operand blocks (TF32x3 and block-scaled three-slice), and the packers.
#pragma once

#include "common.cuh"

namespace gdft {

// D = A B^T over K, operands as [tile of 128 rows][K chunk of 32][slices] blocks
// (hi|lo for launch_tcg, hi|lo|lo2 of umma::store_row3 for launch_tcg3).
struct TcgArgs {
  const float *a, *b;
  int m_tiles, n_tiles;       // 128-row tiles of A and of B
  int64_t a_chunks, b_chunks;  // K chunks stored per tile (tile stride)
  int64_t k_chunks;            // K chunks contracted (<= both)
  int64_t chunks_per_split;    // K chunks per blockIdx.y
  float *out32;                // single split: FP32 row-major output, ld ldo
  int ldo;
  double *out64;               // split-K: FP64 partials [split][m_valid][n_valid]
  int m_valid, n_valid;        // output rows / columns written
  int *err;                    // device error word (bounded waits)
};
cudaError_t launch_tcg(const TcgArgs &a, int nsplit, cudaStream_t st);
// Block-scaled three-slice form (six products, exact hi*hi chunk sums); FP64
// split-K partials only.
cudaError_t launch_tcg3(const TcgArgs &a, int nsplit, cudaStream_t st);

// Row-tile packing: X (rows x cols, row-major, leading dimension ld) into
// blocks [rows/128][kchunks][hi|lo] with block(row, k) = X[t*128 + row][kc*32 + k]
// (zero outside X).
template <class T>
cudaError_t launch_pack_rt(const T *X, int64_t rows, int cols, int ld, int64_t tiles, int kchunks, float *out,
                           cudaStream_t st);
// Row-tile packing into three-slice blocks [rows/128][kchunks][hi|lo|lo2]
// (umma::store_row3, quantised per row and K chunk).
cudaError_t launch_pack_rt3(const double *X, int64_t rows, int cols, int ld, int64_t tiles, int kchunks, float *out,
                            cudaStream_t st);
// Column-tile packing (K = rows): blocks [ftiles][rchunks][hi|lo] with
// block(m, k) = X[rc*32 + k][ft*128 + m] (zero outside X).
template <class T>
cudaError_t launch_pack_ct(const T *X, int64_t rows, int cols, int ld, int ftiles, int64_t rchunks, float *out,
                           cudaStream_t st);

}  // namespace gdft
