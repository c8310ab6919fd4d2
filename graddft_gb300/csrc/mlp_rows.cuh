// mlp_rows.cuh - shared pieces of the fused network row kernels (mlp_tc.cu,
// mlp_hvp_tc.cu): the 32-row activation tile written straight into both packed
// TF32 hi|lo operand layouts, and the Kahan step of their parameter sums.
#pragma once

#include "umma.cuh"

namespace gdft {
namespace {

constexpr size_t kRowPackBlk = 2 * (umma::kBlockBytes / 4);  // floats in one packed hi|lo block pair

// The fused row kernels of the network passes take 32 grid points at a time: each warp handles
// 4 of them (one row per warp at a time), the 32 x W activation tile is staged in
// shared memory (row stride W + 4) and then written in both packed operand
// layouts of the next GEMMs, so neither packing pass re-reads it from memory:
//   rt (row tiles, A of z = h W and dh = dz W^T): block (r / 128, c / 32)
//   ct (column tiles, A / B of dW = h^T dz):      block (c / 128, r / 32)
// A warp's 16-byte stores cover 512 contiguous bytes of a block in both.
constexpr int kRowTile = 32;

// hi = tf32(x), lo = tf32(x - hi) of four values.
__device__ __forceinline__ void split_f4(const float (&v)[4], float4 &h, float4 &l) {
  umma::split_tf32f(v[0], h.x, l.x);
  umma::split_tf32f(v[1], h.y, l.y);
  umma::split_tf32f(v[2], h.z, l.z);
  umma::split_tf32f(v[3], h.w, l.w);
}

template <int PL>
__device__ __forceinline__ void store_tile_packs(const float *tile, int64_t r0, float *__restrict__ rt_out,
                                                 float *__restrict__ ct_out, int64_t rchunks) {
  constexpr int W = 32 * PL, LD = W + 4, KC = W / 32, FT = W / 128;
  const int u = threadIdx.x;
  if (rt_out) {
    const int64_t t = r0 / 128;
    const int rb = (int)(r0 % 128);
    const int row = (u >> 6) * 8 + (u & 7), kg = (u >> 3) & 7;
    const uint32_t off = umma::kblock_off(rb + row, kg * 4) / 4;
#pragma unroll
    for (int kc = 0; kc < KC; ++kc) {
      const float4 v = *(const float4 *)(tile + row * LD + kc * 32 + kg * 4);
      const float a[4] = {v.x, v.y, v.z, v.w};
      float4 h, l;
      split_f4(a, h, l);
      float *blk = rt_out + ((size_t)t * KC + kc) * kRowPackBlk;
      *(float4 *)(blk + off) = h;
      *(float4 *)(blk + umma::kBlockBytes / 4 + off) = l;
    }
  }
  if (ct_out) {
    const int64_t rc = r0 / 32;
#pragma unroll
    for (int ft = 0; ft < FT; ++ft) {
      float *blk = ct_out + ((size_t)ft * rchunks + rc) * kRowPackBlk;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int v = u + 256 * i;
        const int f = (v >> 6) * 8 + (v & 7), pg = (v >> 3) & 7;
        const float *col = tile + ft * 128 + f;
        const float a[4] = {col[(pg * 4 + 0) * LD], col[(pg * 4 + 1) * LD], col[(pg * 4 + 2) * LD],
                            col[(pg * 4 + 3) * LD]};
        float4 h, l;
        split_f4(a, h, l);
        const uint32_t off = umma::kblock_off(f, pg * 4) / 4;
        *(float4 *)(blk + off) = h;
        *(float4 *)(blk + umma::kBlockBytes / 4 + off) = l;
      }
    }
  }
}

// Dynamic shared memory of the reverse row kernels: per-warp Kahan sums of
// three parameter gradients ([8][3][W] float2) and the row tile.
template <int PL>
constexpr size_t bwd_pack_smem() {
  return sizeof(float2) * 8 * 3 * (32 * PL) + sizeof(float) * kRowTile * (32 * PL + 4);
}

// Kahan step on a (total, compensation) pair: total + (v - compensation).
__device__ __forceinline__ void kahan_add(float2 &a, float v) {
  const float y = v - a.y;
  const float t = a.x + y;
  a.y = (t - a.x) - y;
  a.x = t;
}

}  // namespace
}  // namespace gdft
