// Learned Widom proposal: test-particle insertions whose points come from a
// mixture of a learned sub-cell proposal and the uniform proposal of
// compute_mu (src/compute_widom_chem_pot.c:32-182), each weighted by
// 1 / (V q(x)) so that the mean of w * [no overlap] estimates the insertion
// probability <exp(-beta dU)> without bias.  The overlap test of every point
// is the reference's FP64 test (point_overlaps, as for plain Widom).
//
//   k_sub_count, k_sub_pattern  particles per sub-cell (edge ~0.5 sigma, so at
//                               most one per sub-cell in a valid configuration)
//                               and the 27-bit occupancy pattern of each
//                               sub-cell's 3x3x3 neighbourhood
//   k_mlp_logits                MLP 27 -> 64 -> 64 -> 1 on the tensor cores:
//                               tcgen05.mma with BF16 operands in shared memory
//                               and FP32 accumulators in TMEM; output layer in
//                               FP32 on the CUDA cores
//   k_mlp_grad                  forward and backward of weighted binary
//                               cross-entropy; the weight gradients come from
//                               one M=128 product per tile, [dh2^T; dh1^T] x
//                               [h1^T; x^T; 1], accumulated in TMEM over tiles
//   k_grad_reduce, k_adam, k_pack_ops   FP32 master weights, Adam, BF16 copies
//                               in the tensor-core operand layout
//   k_pi, k_scan_*              proposal weights sqrt(sigmoid(z)) per sub-cell
//                               and their FP64 inclusive prefix sum
//   k_widom_is                  mixture draws, overlap test, weights, optional
//                               training outcomes (pattern | success << 31)
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/hsmc_gpu.h"
#include "cellview.cuh"
#include "tcgen05.cuh"

namespace hsmc {

// ------------------------------------------------------------- parameters
constexpr int HID = 64;                     // hidden width
constexpr int KIN = 32;                     // 27 inputs, constant 1, 4 zeros
constexpr int BIAS_COL = 27;                // input column holding the constant 1
constexpr int P_W1 = 0;                     // W1 [64][32] (column 27 = bias of layer 1)
constexpr int P_W2 = P_W1 + HID * KIN;      // W2 [64][64]
constexpr int P_B2 = P_W2 + HID * HID;      // b2 [64]
constexpr int P_W3 = P_B2 + HID;            // w3 [64]
constexpr int P_B3 = P_W3 + HID;            // b3
constexpr int NPARAM = P_B3 + 1;            // 6273
static_assert(NPARAM == HSMC_LWIDOM_NPARAMS, "parameter count");
// BF16 operand copies (K-major core-matrix layout), in one buffer
constexpr int OP_W1 = 0;                    // 64 x 32
constexpr int OP_W2 = OP_W1 + HID * KIN;    // 64 x 64
constexpr int OP_W2T = OP_W2 + HID * HID;   // 64 x 64, W2 transposed
constexpr int NOPS = OP_W2T + HID * HID;    // 10240 elements

constexpr uint32_t TAG_LWIDOM = 6u;
constexpr int ST_TC_TIMEOUT = 1 << 8;
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s bound on any tensor-core wait

__device__ __forceinline__ uint16_t bf16_bits(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf16_val(uint16_t b) { return __bfloat162float(__ushort_as_bfloat16(b)); }

__device__ __forceinline__ uint32_t pack2(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }

// Row r of the input operand X (K = 32): the 27 pattern bits as 0/1, the
// constant 1 in column 27, zeros after it.
__device__ __forceinline__ void write_x_row(uint16_t *sX, int r, uint32_t pat) {
  const uint32_t bits = (pat & 0x07FFFFFFu) | (1u << BIAS_COL);
#pragma unroll
  for (int kc = 0; kc < 4; kc++) {
    uint32_t w[4];
#pragma unroll
    for (int h = 0; h < 4; h++) {
      const uint16_t lo = ((bits >> (8 * kc + 2 * h)) & 1u) ? 0x3F80 : 0;
      const uint16_t hi = ((bits >> (8 * kc + 2 * h + 1)) & 1u) ? 0x3F80 : 0;
      w[h] = pack2(lo, hi);
    }
    *reinterpret_cast<uint4 *>(sX + tc::kmajor(r, 8 * kc, KIN)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Row r of a 64-column K-major operand from 64 BF16 values.
__device__ __forceinline__ void write_row64(uint16_t *s, int r, const uint16_t *v) {
#pragma unroll
  for (int kc = 0; kc < 8; kc++) {
    const uint16_t *q = v + 8 * kc;
    *reinterpret_cast<uint4 *>(s + tc::kmajor(r, 8 * kc, HID)) =
        make_uint4(pack2(q[0], q[1]), pack2(q[2], q[3]), pack2(q[4], q[5]), pack2(q[6], q[7]));
  }
}

// ---------------------------------------------------------- sub-cells
struct SubGrid {
  int ns[3];
  int nsub;
  double inv[3];  // ns / L
  double e[3];    // L / ns
  double len[3];
};

__global__ void k_sub_count(const double *pos, int n, SubGrid g, unsigned *occ) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[3];
  load_xyz(pos, i, x[0], x[1], x[2]);
  int c[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    int v = (int)__dmul_rn(x[d], g.inv[d]);
    c[d] = v < 0 ? 0 : (v >= g.ns[d] ? g.ns[d] - 1 : v);
  }
  atomicAdd(&occ[c[0] + g.ns[0] * (c[1] + g.ns[1] * c[2])], 1u);
}

__global__ void k_sub_pattern(const unsigned *occ, SubGrid g, uint32_t *pat) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nsub) return;
  const int cx = c % g.ns[0], cyz = c / g.ns[0], cy = cyz % g.ns[1], cz = cyz / g.ns[1];
  uint32_t bits = 0;
#pragma unroll
  for (int dz = -1; dz <= 1; dz++) {
    const int z = cz + dz < 0 ? cz + dz + g.ns[2] : (cz + dz >= g.ns[2] ? cz + dz - g.ns[2] : cz + dz);
#pragma unroll
    for (int dy = -1; dy <= 1; dy++) {
      const int y = cy + dy < 0 ? cy + dy + g.ns[1] : (cy + dy >= g.ns[1] ? cy + dy - g.ns[1] : cy + dy);
#pragma unroll
      for (int dx = -1; dx <= 1; dx++) {
        const int x = cx + dx < 0 ? cx + dx + g.ns[0] : (cx + dx >= g.ns[0] ? cx + dx - g.ns[0] : cx + dx);
        if (occ[x + g.ns[0] * (y + g.ns[1] * z)] > 0u) bits |= 1u << ((dx + 1) + 3 * (dy + 1) + 9 * (dz + 1));
      }
    }
  }
  pat[c] = bits;
}

// ------------------------------------------------------ weight packing
__global__ void k_pack_ops(const float *prm, uint16_t *ops) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < HID * KIN) {
    const int r = i / KIN, k = i % KIN;
    ops[OP_W1 + tc::kmajor(r, k, KIN)] = bf16_bits(prm[P_W1 + i]);
  }
  if (i < HID * HID) {
    const int r = i / HID, k = i % HID;
    ops[OP_W2 + tc::kmajor(r, k, HID)] = bf16_bits(prm[P_W2 + i]);
    ops[OP_W2T + tc::kmajor(k, r, HID)] = bf16_bits(prm[P_W2 + i]);
  }
}

// ------------------------------------------------------------- forward
// Shared memory of k_mlp_logits (bytes); 48 KB are requested so that at most
// four blocks (4 x 128 TMEM columns) share an SM.
constexpr int FL_X = 0, FL_W1 = 8192, FL_W2 = 12288, FL_H1 = 20480, FL_B2 = 36864, FL_W3 = 37120, FL_B3 = 37376,
              FL_BAR = 37392, FL_TSLOT = 37400;
constexpr int FL_SMEM = 49152;

__global__ void __launch_bounds__(128) k_mlp_logits(const uint32_t *pat, long long n, const uint16_t *ops,
                                                    const float *prm, float *z_out, int *status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  uint16_t *sX = reinterpret_cast<uint16_t *>(sm + FL_X);
  uint16_t *sW1 = reinterpret_cast<uint16_t *>(sm + FL_W1);
  uint16_t *sW2 = reinterpret_cast<uint16_t *>(sm + FL_W2);
  uint16_t *sH1 = reinterpret_cast<uint16_t *>(sm + FL_H1);
  float *sB2 = reinterpret_cast<float *>(sm + FL_B2);
  float *sW3 = reinterpret_cast<float *>(sm + FL_W3);
  float *sB3 = reinterpret_cast<float *>(sm + FL_B3);
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + FL_BAR);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + FL_TSLOT);
  const int tid = threadIdx.x, warp = tid >> 5;

  // W1 and W2 are adjacent in `ops` and in shared memory
  for (int i = tid; i < (HID * KIN + HID * HID) / 8; i += 128)
    reinterpret_cast<uint4 *>(sW1)[i] = reinterpret_cast<const uint4 *>(ops + OP_W1)[i];
  if (tid < HID) {
    sB2[tid] = prm[P_B2 + tid];
    sW3[tid] = prm[P_W3 + tid];
  }
  if (tid == 0) {
    sB3[0] = prm[P_B3];
    tc::mbar_init(bar, 1);
  }
  if (warp == 0) {
    tc::alloc(tslot, 128);
    tc::relinquish();
  }
  tc::fence_proxy_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  constexpr uint32_t IDESC = tc::idesc_bf16(128, 64);
  uint32_t phase = 0;
  bool failed = false;

  for (long long t0 = (long long)blockIdx.x * 128; t0 < n && !failed; t0 += (long long)gridDim.x * 128) {
    const long long row = t0 + tid;
    write_x_row(sX, tid, row < n ? pat[row] : 0u);
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < KIN / 16; s++)
        tc::mma_bf16(tmem, tc::sdesc(sX + s * 16 * 8, 128, KIN * 16), tc::sdesc(sW1 + s * 16 * 8, 128, KIN * 16),
                     IDESC, s > 0);
      tc::commit(bar);
    }
    bool ok = tc::mbar_wait(bar, phase, kWaitNs);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    tc::fence_after();
    float a[HID];
    tc::ld32(tmem + lane_base, a);
    tc::ld32(tmem + lane_base + 32, a + 32);
    uint16_t h[HID];
#pragma unroll
    for (int j = 0; j < HID; j++) h[j] = bf16_bits(fmaxf(a[j], 0.0f));
    write_row64(sH1, tid, h);
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < HID / 16; s++)
        tc::mma_bf16(tmem + 64, tc::sdesc(sH1 + s * 16 * 8, 128, HID * 16),
                     tc::sdesc(sW2 + s * 16 * 8, 128, HID * 16), IDESC, s > 0);
      tc::commit(bar);
    }
    ok = tc::mbar_wait(bar, phase, kWaitNs);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    tc::fence_after();
    tc::ld32(tmem + lane_base + 64, a);
    tc::ld32(tmem + lane_base + 96, a + 32);
    float z = 0.0f;
#pragma unroll
    for (int j = 0; j < HID; j++) z = fmaf(sW3[j], fmaxf(a[j] + sB2[j], 0.0f), z);
    z += sB3[0];
    if (row < n) z_out[row] = z;
    tc::fence_before();
    __syncthreads();  // the next tile rewrites X, H1 and the accumulators
  }
  if (failed) {
    if (tid == 0) atomicOr(status, ST_TC_TIMEOUT);
    tc::mbar_wait(bar, phase, kWaitNs);  // let an MMA still in flight finish before TMEM is released
  }
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    tc::dealloc(tmem, 128);
  }
}

// ------------------------------------------------------------ training
// Shared memory of k_mlp_grad (bytes): one block per SM, 256 TMEM columns.
constexpr int TG_X = 0, TG_W1 = 8192, TG_W2 = 12288, TG_W2T = 20480, TG_H1 = 28672, TG_D2 = 45056, TG_BG = 61440,
              TG_AG = 90112, TG_B2 = 122880, TG_W3 = 123136, TG_B3 = 123392, TG_RED = 123408, TG_BAR = 124464,
              TG_TSLOT = 124472;
constexpr int TG_SMEM = 124480;
constexpr int NG = 112;  // columns of the gradient product: h1 (64), x (32), ones, zero padding

__global__ void __launch_bounds__(128, 1) k_mlp_grad(const uint32_t *samples, long long n, float w_pos, float w_neg,
                                                     float inv_n, const uint16_t *ops, const float *prm,
                                                     float *part, int *status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  uint16_t *sX = reinterpret_cast<uint16_t *>(sm + TG_X);
  uint16_t *sW1 = reinterpret_cast<uint16_t *>(sm + TG_W1);
  uint16_t *sW2 = reinterpret_cast<uint16_t *>(sm + TG_W2);
  uint16_t *sW2T = reinterpret_cast<uint16_t *>(sm + TG_W2T);
  uint16_t *sH1 = reinterpret_cast<uint16_t *>(sm + TG_H1);
  uint16_t *sD2 = reinterpret_cast<uint16_t *>(sm + TG_D2);
  uint16_t *sBg = reinterpret_cast<uint16_t *>(sm + TG_BG);  // [112][128]: h1^T, x^T, ones, zeros
  uint16_t *sAg = reinterpret_cast<uint16_t *>(sm + TG_AG);  // [128][128]: dh2^T, dh1^T
  float *sB2 = reinterpret_cast<float *>(sm + TG_B2);
  float *sW3 = reinterpret_cast<float *>(sm + TG_W3);
  float *sB3 = reinterpret_cast<float *>(sm + TG_B3);
  float *red = reinterpret_cast<float *>(sm + TG_RED);  // [4][66]
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + TG_BAR);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + TG_TSLOT);
  const int tid = threadIdx.x, warp = tid >> 5;

  for (int i = tid; i < NOPS / 8; i += 128) reinterpret_cast<uint4 *>(sW1)[i] = reinterpret_cast<const uint4 *>(ops)[i];
  if (tid < HID) {
    sB2[tid] = prm[P_B2 + tid];
    sW3[tid] = prm[P_W3 + tid];
  }
  // rows 96..111 of the gradient B operand: ones, then zeros (fixed)
  for (int f = 96; f < NG; f++) sBg[tc::kmajor(f, tid, 128)] = f == 96 ? (uint16_t)0x3F80 : (uint16_t)0;
  if (tid == 0) {
    sB3[0] = prm[P_B3];
    tc::mbar_init(bar, 1);
  }
  if (warp == 0) {
    tc::alloc(tslot, 256);
    tc::relinquish();
  }
  tc::fence_proxy_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  constexpr uint32_t ID64 = tc::idesc_bf16(128, 64);
  constexpr uint32_t IDG = tc::idesc_bf16(128, NG);
  uint32_t phase = 0;
  bool failed = false;
  int tiles = 0;
  float acc3[HID];
#pragma unroll
  for (int j = 0; j < HID; j++) acc3[j] = 0.0f;
  float accb3 = 0.0f, loss = 0.0f;

  auto wait_all = [&]() -> bool {
    const bool ok = tc::mbar_wait(bar, phase, kWaitNs);
    phase ^= 1u;
    return !__syncthreads_or(!ok);
  };

  for (long long t0 = (long long)blockIdx.x * 128; t0 < n && !failed; t0 += (long long)gridDim.x * 128) {
    const long long row = t0 + tid;
    const uint32_t smp = row < n ? samples[row] : 0u;
    const float y = (smp >> 31) ? 1.0f : 0.0f;
    const float wt = row < n ? ((smp >> 31) ? w_pos : w_neg) : 0.0f;
    write_x_row(sX, tid, smp);
    {
      const uint32_t bits = (smp & 0x07FFFFFFu) | (1u << BIAS_COL);
#pragma unroll
      for (int f = 0; f < KIN; f++) sBg[tc::kmajor(64 + f, tid, 128)] = ((bits >> f) & 1u) ? (uint16_t)0x3F80 : 0;
    }
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < KIN / 16; s++)
        tc::mma_bf16(tmem, tc::sdesc(sX + s * 128, 128, KIN * 16), tc::sdesc(sW1 + s * 128, 128, KIN * 16), ID64,
                     s > 0);
      tc::commit(bar);
    }
    if (!wait_all()) {
      failed = true;
      break;
    }
    tc::fence_after();
    float a[HID];
    tc::ld32(tmem + lane_base, a);
    tc::ld32(tmem + lane_base + 32, a + 32);
    uint16_t h[HID];
#pragma unroll
    for (int j = 0; j < HID; j++) {
      h[j] = bf16_bits(fmaxf(a[j], 0.0f));
      sBg[tc::kmajor(j, tid, 128)] = h[j];
    }
    write_row64(sH1, tid, h);
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < HID / 16; s++)
        tc::mma_bf16(tmem + 64, tc::sdesc(sH1 + s * 128, 128, HID * 16), tc::sdesc(sW2 + s * 128, 128, HID * 16),
                     ID64, s > 0);
      tc::commit(bar);
    }
    if (!wait_all()) {
      failed = true;
      break;
    }
    tc::fence_after();
    tc::ld32(tmem + lane_base + 64, a);
    tc::ld32(tmem + lane_base + 96, a + 32);
    float z = 0.0f;
#pragma unroll
    for (int j = 0; j < HID; j++) {
      a[j] = fmaxf(a[j] + sB2[j], 0.0f);  // h2
      z = fmaf(sW3[j], a[j], z);
    }
    z += sB3[0];
    const float sg = 1.0f / (1.0f + expf(-z));
    loss += wt * (fmaxf(z, 0.0f) - z * y + log1pf(expf(-fabsf(z))));
    const float dz = wt * (sg - y) * inv_n;
    accb3 += dz;
    uint16_t d2[HID];
#pragma unroll
    for (int j = 0; j < HID; j++) {
      acc3[j] = fmaf(dz, a[j], acc3[j]);
      d2[j] = bf16_bits(a[j] > 0.0f ? dz * sW3[j] : 0.0f);
      sAg[tc::kmajor(j, tid, 128)] = d2[j];
    }
    write_row64(sD2, tid, d2);
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < HID / 16; s++)
        tc::mma_bf16(tmem, tc::sdesc(sD2 + s * 128, 128, HID * 16), tc::sdesc(sW2T + s * 128, 128, HID * 16), ID64,
                     s > 0);
      tc::commit(bar);
    }
    if (!wait_all()) {
      failed = true;
      break;
    }
    tc::fence_after();
    tc::ld32(tmem + lane_base, a);
    tc::ld32(tmem + lane_base + 32, a + 32);
#pragma unroll
    for (int j = 0; j < HID; j++) {
      const bool live = h[j] != 0 && !(h[j] & 0x8000u);  // h1 > 0
      sAg[tc::kmajor(64 + j, tid, 128)] = bf16_bits(live ? a[j] : 0.0f);
    }
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < 128 / 16; s++)
        tc::mma_bf16(tmem + 128, tc::sdesc(sAg + s * 128, 128, 128 * 16), tc::sdesc(sBg + s * 128, 128, 128 * 16),
                     IDG, (tiles > 0 || s > 0) ? 1u : 0u);
      tc::commit(bar);
    }
    if (!wait_all()) {  // the next tile rewrites A and B of this product
      failed = true;
      break;
    }
    tiles++;
  }

  float *out = part + (size_t)blockIdx.x * (NPARAM + 1);
  if (failed) {
    if (tid == 0) atomicOr(status, ST_TC_TIMEOUT);
    tc::mbar_wait(bar, phase, kWaitNs);
  } else {
    // weight gradients from the accumulator: lanes 0-63 hold dW2 rows and
    // db2, lanes 64-127 hold dW1 rows (bias of layer 1 in column 27)
    tc::fence_after();
    float g[96], g2[16];
    if (tiles > 0) {
      tc::ld32(tmem + lane_base + 128, g);
      tc::ld32(tmem + lane_base + 160, g + 32);
      tc::ld32(tmem + lane_base + 192, g + 64);
      tc::ld16(tmem + lane_base + 224, g2);
    } else {
#pragma unroll
      for (int j = 0; j < 96; j++) g[j] = 0.0f;
#pragma unroll
      for (int j = 0; j < 16; j++) g2[j] = 0.0f;
    }
    if (tid < HID) {
#pragma unroll
      for (int j = 0; j < HID; j++) out[P_W2 + tid * HID + j] = g[j];
      out[P_B2 + tid] = g2[0];
    } else {
#pragma unroll
      for (int j = 0; j < KIN; j++) out[P_W1 + (tid - HID) * KIN + j] = j < 28 ? g[64 + j] : 0.0f;
    }
    // w3, b3 and the loss: warp sums, then across the four warps
#pragma unroll
    for (int j = 0; j < HID + 2; j++) {
      float v = j < HID ? acc3[j] : (j == HID ? accb3 : loss);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if ((tid & 31) == 0) red[warp * 66 + j] = v;
    }
    __syncthreads();
    if (tid < HID + 2) {
      const float v = red[tid] + red[66 + tid] + red[132 + tid] + red[198 + tid];
      if (tid < HID) out[P_W3 + tid] = v;
      else if (tid == HID) out[P_B3] = v;
      else out[NPARAM] = v;  // loss sum of this block
    }
  }
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    tc::dealloc(tmem, 256);
  }
}

__global__ void k_grad_reduce(const float *part, int nblk, float *grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > NPARAM) return;
  double s = 0.0;
  for (int b = 0; b < nblk; b++) s += (double)part[(size_t)b * (NPARAM + 1) + i];
  grad[i] = (float)s;  // grad[NPARAM] = summed loss
}

// Adam (Kingma & Ba 2015) in FP32, operation by operation without contraction:
//   m = b1 m + (1 - b1) g;  v = b2 v + ((1 - b2) g) g;
//   p = p - (lr (m / c1)) / (sqrt(v / c2) + eps),
// with 1 - b and c = 1 - b^t rounded from double on the host.
__global__ void k_adam(float *prm, float *m, float *v, const float *grad, float lr, float b1, float omb1, float b2,
                       float omb2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  const float g = grad[i];
  const float mi = __fadd_rn(__fmul_rn(b1, m[i]), __fmul_rn(omb1, g));
  const float vi = __fadd_rn(__fmul_rn(b2, v[i]), __fmul_rn(__fmul_rn(omb2, g), g));
  m[i] = mi;
  v[i] = vi;
  const float step = __fdiv_rn(__fmul_rn(lr, __fdiv_rn(mi, c1)), __fadd_rn(__fsqrt_rn(__fdiv_rn(vi, c2)), eps));
  prm[i] = __fsub_rn(prm[i], step);
}

// ------------------------------------------------------------- proposal
// pi_c = sqrt(sigmoid(z_c)) in FP32 (the FP64 pipe of this GPU is narrow);
// the proposal and the weights both use this same value, so the estimate
// stays unbiased.
__global__ void k_pi(const float *z, double *pi, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pi[i] = (double)sqrtf(1.0f / (1.0f + expf(-z[i])));
}

// Inclusive FP64 prefix sum: 4096 values per block (4 per thread), block
// totals scanned by one block, then added back.  Fixed order: deterministic.
constexpr int SCAN_T = 1024, SCAN_PER = 4, SCAN_BLK = SCAN_T * SCAN_PER;

__global__ void __launch_bounds__(SCAN_T) k_scan_block(const double *in, double *out, double *totals, int n) {
  __shared__ double warp_tot[SCAN_T / 32];
  const int base = blockIdx.x * SCAN_BLK + threadIdx.x * SCAN_PER;
  double v[SCAN_PER];
  double run = 0.0;
#pragma unroll
  for (int k = 0; k < SCAN_PER; k++) {
    run += (base + k < n) ? in[base + k] : 0.0;
    v[k] = run;
  }
  double x = run;  // inclusive scan of thread totals within the warp
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    double t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  const double before = (x - run) + (w > 0 ? warp_tot[w - 1] : 0.0);
#pragma unroll
  for (int k = 0; k < SCAN_PER; k++)
    if (base + k < n) out[base + k] = before + v[k];
  if (threadIdx.x == SCAN_T - 1 && totals) totals[blockIdx.x] = before + run;
}

__global__ void k_scan_add(double *out, const double *block_incl, int n) {
  if (blockIdx.x == 0) return;
  const double add = block_incl[blockIdx.x - 1];
  const int base = blockIdx.x * SCAN_BLK + threadIdx.x * SCAN_PER;
#pragma unroll
  for (int k = 0; k < SCAN_PER; k++)
    if (base + k < n) out[base + k] += add;
}

// ------------------------------------------------------------ insertions
struct IsOut {
  double *sums;               // per block: sum w, sum w^2 over successes
  unsigned long long *cnts;   // per block: successes, learned draws, collected successes
  uint32_t *collect;          // training outcomes (pattern | success << 31), or null
  long long collect_cap;      // room left in `collect`
  unsigned long long *collect_n;  // outcomes claimed (may exceed the room)
  unsigned long long keep_thr;    // a failure is kept when its keep draw < keep_thr (2^32 keeps all)
  double *t_pts;              // optional trace: points, sub-cell, branch, weight, success
  int *t_cell;
  uint8_t *t_uni;
  double *t_w;
  uint8_t *t_ok;
};

constexpr int IS_BLOCKS = 1216, IS_THREADS = 256;
// Coarse index of the CDF in shared memory: the last value of each of
// CDF_TAB equal chunks, so a learned draw searches the table, then one chunk
// in global memory (about 10 dependent L2 loads fewer than a search of the
// whole CDF, which bounded the insertion's latency).
constexpr int CDF_TAB = 1024;

__global__ void __launch_bounds__(IS_THREADS) k_widom_is(SysPtrs p, SubGrid g, const double *cdf, const double *pi,
                                                         const uint32_t *pat, long long n, unsigned long long seq,
                                                         unsigned long long seed, unsigned long long thr,
                                                         double alpha, IsOut o) {
  const CellView v = current_view(p);
  const Box *bx = p.box;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const Stencil s{{1, 1, 1}};
  const double total = cdf[g.nsub - 1];
  const double inv_span = __ddiv_rn(1.0, 4294967296.0 - (double)thr);
  // chunk j covers [j nsub / T, (j + 1) nsub / T); tab[j] holds the bits of
  // its last value
  __shared__ long long tab[CDF_TAB];
  const bool coarse = g.nsub >= CDF_TAB;
  if (coarse)
    for (int j = threadIdx.x; j < CDF_TAB; j += blockDim.x)
      tab[j] = __ldg(reinterpret_cast<const long long *>(cdf) + ((long long)(j + 1) * g.nsub) / CDF_TAB - 1);
  __syncthreads();
  const double kmix = __ddiv_rn(__dmul_rn(1.0 - alpha, (double)g.nsub), total);
  double sw = 0.0, sw2 = 0.0;
  unsigned long long nok = 0, nlearn = 0, ncol = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const U32x4 r = draw4(seed, (uint32_t)k, (uint32_t)(k >> 32), seq, TAG_LWIDOM);
    const bool uni = (unsigned long long)r.x < thr;
    double x[3];
    int cell = 0;
    if (uni) {
      x[0] = __dmul_rn(open_unit(r.y), len[0]);
      x[1] = __dmul_rn(open_unit(r.z), len[1]);
      x[2] = __dmul_rn(open_unit(r.w), len[2]);
    } else {
      const double t = __dmul_rn(__dmul_rn(__dadd_rn((double)((unsigned long long)r.x - thr), 0.5), inv_span), total);
      // first index with cdf > t; positive doubles order as their bit
      // patterns, so the comparisons stay off the FP64 pipe
      const long long tb = __double_as_longlong(t);
      const long long *cdf_bits = reinterpret_cast<const long long *>(cdf);
      int lo = 0, hi = g.nsub - 1;
      if (coarse) {  // the first chunk whose last value exceeds t holds the index
        int a = 0, b = CDF_TAB - 1;
        while (a < b) {
          const int mid = (a + b) >> 1;
          if (tab[mid] > tb) b = mid;
          else a = mid + 1;
        }
        lo = (int)(((long long)a * g.nsub) / CDF_TAB);
        hi = (int)(((long long)(a + 1) * g.nsub) / CDF_TAB) - 1;
      }
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cdf_bits + mid) > tb) hi = mid;
        else lo = mid + 1;
      }
      cell = lo;
      const int cx = cell % g.ns[0], cyz = cell / g.ns[0], cy = cyz % g.ns[1], cz = cyz / g.ns[1];
      x[0] = __dmul_rn(__dadd_rn((double)cx, open_unit(r.y)), g.e[0]);
      x[1] = __dmul_rn(__dadd_rn((double)cy, open_unit(r.z)), g.e[1]);
      x[2] = __dmul_rn(__dadd_rn((double)cz, open_unit(r.w)), g.e[2]);
    }
    int c3[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const int q = (int)__dmul_rn(x[d], g.inv[d]);
      c3[d] = q < 0 ? 0 : (q >= g.ns[d] ? g.ns[d] - 1 : q);
    }
    const int sub = c3[0] + g.ns[0] * (c3[1] + g.ns[1] * c3[2]);
    const double w = __ddiv_rn(1.0, __dadd_rn(alpha, __dmul_rn(kmix, pi[sub])));  // no contraction
    const bool ok = !point_overlaps(v, p, s, x[0], x[1], x[2], -1, len, half);
    if (ok) {
      sw += w;
      sw2 += w * w;
      nok++;
    }
    nlearn += uni ? 0 : 1;
    if (o.collect) {
      // every success is kept; a failure with probability keep_thr / 2^32,
      // from a draw of its own (counter word b with the top bit set)
      bool keep = ok;
      if (!keep && o.keep_thr) {
        const U32x4 rk = draw4(seed, (uint32_t)k, (uint32_t)(k >> 32) | 0x80000000u, seq, TAG_LWIDOM);
        keep = (unsigned long long)rk.x < o.keep_thr;
      }
      if (keep) {
        const unsigned long long at = atomicAdd(o.collect_n, 1ull);
        if ((long long)at < o.collect_cap) {
          o.collect[at] = pat[sub] | (ok ? 0x80000000u : 0u);
          ncol += ok ? 1 : 0;
        }
      }
    }
    if (o.t_pts) {
      o.t_pts[3 * k] = x[0];
      o.t_pts[3 * k + 1] = x[1];
      o.t_pts[3 * k + 2] = x[2];
      o.t_cell[k] = uni ? -1 : cell;
      o.t_uni[k] = uni ? 1 : 0;
      o.t_w[k] = w;
      o.t_ok[k] = ok ? 1 : 0;
    }
  }
  __shared__ double s_sum[2][IS_THREADS / 32];
  __shared__ unsigned long long s_cnt[3][IS_THREADS / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    sw += __shfl_down_sync(0xffffffffu, sw, off);
    sw2 += __shfl_down_sync(0xffffffffu, sw2, off);
    nok += __shfl_down_sync(0xffffffffu, nok, off);
    nlearn += __shfl_down_sync(0xffffffffu, nlearn, off);
    ncol += __shfl_down_sync(0xffffffffu, ncol, off);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_sum[0][w] = sw;
    s_sum[1][w] = sw2;
    s_cnt[0][w] = nok;
    s_cnt[1][w] = nlearn;
    s_cnt[2][w] = ncol;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    unsigned long long c0 = 0, c1 = 0, c2 = 0;
    for (int i = 0; i < IS_THREADS / 32; i++) {
      a += s_sum[0][i];
      b += s_sum[1][i];
      c0 += s_cnt[0][i];
      c1 += s_cnt[1][i];
      c2 += s_cnt[2][i];
    }
    o.sums[2 * blockIdx.x] = a;
    o.sums[2 * blockIdx.x + 1] = b;
    o.cnts[3 * blockIdx.x] = c0;
    o.cnts[3 * blockIdx.x + 1] = c1;
    o.cnts[3 * blockIdx.x + 2] = c2;
  }
}

// Plain uniform Widom with the same overlap test (the reference estimator),
// timed on the same stream for comparisons.
__global__ void __launch_bounds__(IS_THREADS) k_widom_plain(SysPtrs p, long long n, unsigned long long seq,
                                                            unsigned long long seed, unsigned long long *cnts) {
  const CellView v = current_view(p);
  const Box *bx = p.box;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const Stencil s{{1, 1, 1}};
  unsigned long long nok = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const U32x4 r = draw4(seed, (uint32_t)k, (uint32_t)(k >> 32), seq, TAG_WIDOM);
    const double x = __dmul_rn(open_unit(r.x), len[0]);
    const double y = __dmul_rn(open_unit(r.y), len[1]);
    const double z = __dmul_rn(open_unit(r.z), len[2]);
    nok += point_overlaps(v, p, s, x, y, z, -1, len, half) ? 0 : 1;
  }
  nok = warp_sum_u64(nok);
  __shared__ unsigned long long s_cnt[IS_THREADS / 32];
  if ((threadIdx.x & 31) == 0) s_cnt[threadIdx.x >> 5] = nok;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int i = 0; i < IS_THREADS / 32; i++) t += s_cnt[i];
    cnts[blockIdx.x] = t;
  }
}

}  // namespace hsmc

// =================================================================== C ABI
using namespace hsmc;

namespace {

template <class T>
struct DevBuf {
  T *ptr = nullptr;
  size_t count = 0;
  cudaError_t ensure(size_t want) {
    if (want <= count) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    count = 0;
    cudaError_t e = cudaMalloc(&ptr, sizeof(T) * want);
    if (e == cudaSuccess) count = want;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    count = 0;
  }
};

int cuda_fail(cudaError_t e) {
  fprintf(stderr, "hsmc_lwidom: CUDA error %s\n", cudaGetErrorString(e));
  return HSMC_ERR_CUDA;
}

#define LW_CUDA(call)                          \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess) return cuda_fail(e_); \
  } while (0)

}  // namespace

struct hsmc_lwidom {
  hsmc_ctx *ctx = nullptr;
  CtxView view{};
  double target_edge = 0.5;
  unsigned long long seed = 0, seq = 0, plain_seq = 0;
  SubGrid g{};
  int num_sms = 0;
  int grad_blocks = 0;
  long long adam_step = 0;
  DevBuf<float> prm, mom1, mom2, grad, part, logits;
  DevBuf<uint16_t> ops;
  DevBuf<unsigned> occ;
  DevBuf<uint32_t> pat, samples, qpat;
  DevBuf<double> pi, cdf, totals, sums;
  DevBuf<unsigned long long> cnts;
  DevBuf<int> status;
  DevBuf<unsigned long long> counter;
  DevBuf<double> t_pts, t_w;
  DevBuf<int> t_cell;
  DevBuf<uint8_t> t_uni, t_ok;
  long long n_samples = 0, n_pos = 0, capacity = 0;
  bool refreshed = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double last_ms = 0.0;
};

namespace {

int sync_status(hsmc_lwidom *lw) {
  cudaError_t e = cudaStreamSynchronize(lw->view.stream);
  if (e != cudaSuccess) return cuda_fail(e);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e);
  int st = 0;
  LW_CUDA(cudaMemcpy(&st, lw->status.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  if (st & ST_TC_TIMEOUT) return HSMC_ERR_TIMEOUT;
  if (st) return HSMC_ERR_CELL_OVERFLOW;
  return HSMC_OK;
}

int set_grid(hsmc_lwidom *lw) {
  int e = ctx_view(lw->ctx, &lw->view);
  if (e) return e;
  SubGrid g{};
  long long nsub = 1;
  for (int d = 0; d < 3; d++) {
    const double L = lw->view.box.len[d];
    int ns = (int)std::floor(L / lw->target_edge);
    if (ns < 3) ns = 3;
    g.ns[d] = ns;
    g.inv[d] = (double)ns / L;
    g.e[d] = L / (double)ns;
    g.len[d] = L;
    nsub *= ns;
  }
  if (nsub > (long long)SCAN_BLK * SCAN_BLK) return HSMC_ERR_INVALID_ARG;
  g.nsub = (int)nsub;
  lw->g = g;
  LW_CUDA(lw->occ.ensure(g.nsub));
  LW_CUDA(lw->pat.ensure(g.nsub));
  LW_CUDA(lw->logits.ensure(g.nsub));
  LW_CUDA(lw->pi.ensure(g.nsub));
  LW_CUDA(lw->cdf.ensure(g.nsub));
  LW_CUDA(lw->totals.ensure((g.nsub + SCAN_BLK - 1) / SCAN_BLK + 1));
  return HSMC_OK;
}

void launch_logits(hsmc_lwidom *lw, const uint32_t *pat, long long n, float *z) {
  long long tiles = (n + 127) / 128;
  long long grid = 4ll * lw->num_sms;
  if (tiles < grid) grid = tiles;
  if (grid < 1) grid = 1;
  k_mlp_logits<<<(int)grid, 128, FL_SMEM, lw->view.stream>>>(pat, n, lw->ops.ptr, lw->prm.ptr, z, lw->status.ptr);
}

// Gradient of the mean weighted loss over samples[0, n) into lw->grad
// (NPARAM entries, then the summed loss).
int run_grad(hsmc_lwidom *lw, const uint32_t *samples, long long n, float w_pos, float w_neg) {
  const cudaStream_t s = lw->view.stream;
  k_mlp_grad<<<lw->grad_blocks, 128, TG_SMEM, s>>>(samples, n, w_pos, w_neg, (float)(1.0 / (double)n), lw->ops.ptr,
                                                   lw->prm.ptr, lw->part.ptr, lw->status.ptr);
  k_grad_reduce<<<(NPARAM + 1 + 255) / 256, 256, 0, s>>>(lw->part.ptr, lw->grad_blocks, lw->grad.ptr);
  return HSMC_OK;
}

void adam_and_pack(hsmc_lwidom *lw, float lr) {
  const cudaStream_t s = lw->view.stream;
  lw->adam_step++;
  const float c1 = (float)(1.0 - std::pow(0.9, (double)lw->adam_step));
  const float c2 = (float)(1.0 - std::pow(0.999, (double)lw->adam_step));
  k_adam<<<(NPARAM + 255) / 256, 256, 0, s>>>(lw->prm.ptr, lw->mom1.ptr, lw->mom2.ptr, lw->grad.ptr, lr, 0.9f,
                                              (float)(1.0 - 0.9), 0.999f, (float)(1.0 - 0.999), 1e-8f, c1, c2);
  k_pack_ops<<<(HID * HID + 255) / 256, 256, 0, s>>>(lw->prm.ptr, lw->ops.ptr);
}

}  // namespace

extern "C" {

int hsmc_lwidom_create(hsmc_ctx *ctx, double subcell_edge, uint64_t seed, int64_t train_capacity,
                       hsmc_lwidom **out) {
  if (!ctx || !out || !(subcell_edge > 0.0) || subcell_edge > 1.0 / std::sqrt(3.0) || train_capacity < 0)
    return HSMC_ERR_INVALID_ARG;
  hsmc_lwidom *lw = new hsmc_lwidom();
  lw->ctx = ctx;
  lw->target_edge = subcell_edge;
  lw->seed = seed;
  lw->capacity = train_capacity;
  auto fail = [&](int e) {
    hsmc_lwidom_destroy(lw);
    return e;
  };
  int e = set_grid(lw);
  if (e) return fail(e);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&lw->num_sms, cudaDevAttrMultiProcessorCount, dev);
  lw->grad_blocks = lw->num_sms;
  cudaError_t ce;
  if ((ce = cudaFuncSetAttribute(k_mlp_logits, cudaFuncAttributeMaxDynamicSharedMemorySize, FL_SMEM)) ||
      (ce = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, TG_SMEM)))
    return fail(cuda_fail(ce));
  if ((ce = lw->prm.ensure(NPARAM)) || (ce = lw->mom1.ensure(NPARAM)) || (ce = lw->mom2.ensure(NPARAM)) ||
      (ce = lw->grad.ensure(NPARAM + 1)) || (ce = lw->part.ensure((size_t)lw->grad_blocks * (NPARAM + 1))) ||
      (ce = lw->ops.ensure(NOPS)) || (ce = lw->status.ensure(1)) || (ce = lw->sums.ensure(2 * IS_BLOCKS)) ||
      (ce = lw->cnts.ensure(3 * IS_BLOCKS)) || (ce = lw->counter.ensure(1)) ||
      (ce = lw->samples.ensure(train_capacity > 0 ? (size_t)train_capacity : 1)))
    return fail(cuda_fail(ce));
  if ((ce = cudaEventCreate(&lw->e0)) || (ce = cudaEventCreate(&lw->e1))) return fail(cuda_fail(ce));
  // default initialisation: He-normal weights from the seed, zero biases
  std::vector<float> p(NPARAM, 0.0f);
  unsigned long long st = seed * 0x9E3779B97F4A7C15ull + 1ull;
  auto normal = [&]() {  // Box-Muller on a 64-bit LCG (initial values only)
    auto u01 = [&]() {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      return ((double)(st >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    const double a = u01(), b = u01();
    return std::sqrt(-2.0 * std::log(a)) * std::cos(6.283185307179586 * b);
  };
  for (int r = 0; r < HID; r++)
    for (int k = 0; k < 27; k++) p[P_W1 + r * KIN + k] = (float)(normal() * std::sqrt(2.0 / 28.0));
  for (int i = 0; i < HID * HID; i++) p[P_W2 + i] = (float)(normal() * std::sqrt(2.0 / HID));
  for (int i = 0; i < HID; i++) p[P_W3 + i] = (float)(normal() * std::sqrt(1.0 / HID));
  e = hsmc_lwidom_set_params(lw, p.data());
  if (e) return fail(e);
  *out = lw;
  return HSMC_OK;
}

void hsmc_lwidom_destroy(hsmc_lwidom *lw) {
  if (!lw) return;
  if (lw->view.stream) cudaStreamSynchronize(lw->view.stream);
  lw->prm.release();
  lw->mom1.release();
  lw->mom2.release();
  lw->grad.release();
  lw->part.release();
  lw->logits.release();
  lw->ops.release();
  lw->occ.release();
  lw->pat.release();
  lw->samples.release();
  lw->qpat.release();
  lw->pi.release();
  lw->cdf.release();
  lw->totals.release();
  lw->sums.release();
  lw->cnts.release();
  lw->status.release();
  lw->counter.release();
  lw->t_pts.release();
  lw->t_w.release();
  lw->t_cell.release();
  lw->t_uni.release();
  lw->t_ok.release();
  if (lw->e0) cudaEventDestroy(lw->e0);
  if (lw->e1) cudaEventDestroy(lw->e1);
  delete lw;
}

int hsmc_lwidom_set_params(hsmc_lwidom *lw, const float *params) {
  if (!lw || !params) return HSMC_ERR_INVALID_ARG;
  const cudaStream_t s = lw->view.stream;
  LW_CUDA(cudaMemcpyAsync(lw->prm.ptr, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, s));
  LW_CUDA(cudaMemsetAsync(lw->mom1.ptr, 0, sizeof(float) * NPARAM, s));
  LW_CUDA(cudaMemsetAsync(lw->mom2.ptr, 0, sizeof(float) * NPARAM, s));
  LW_CUDA(cudaMemsetAsync(lw->ops.ptr, 0, sizeof(uint16_t) * NOPS, s));
  LW_CUDA(cudaMemsetAsync(lw->status.ptr, 0, sizeof(int), s));
  k_pack_ops<<<(HID * HID + 255) / 256, 256, 0, s>>>(lw->prm.ptr, lw->ops.ptr);
  lw->adam_step = 0;
  lw->refreshed = false;
  return sync_status(lw);
}

int hsmc_lwidom_get_params(hsmc_lwidom *lw, float *params) {
  if (!lw || !params) return HSMC_ERR_INVALID_ARG;
  LW_CUDA(cudaStreamSynchronize(lw->view.stream));
  LW_CUDA(cudaMemcpy(params, lw->prm.ptr, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return HSMC_OK;
}

int hsmc_lwidom_subgrid(hsmc_lwidom *lw, int ns[3]) {
  if (!lw || !ns) return HSMC_ERR_INVALID_ARG;
  for (int d = 0; d < 3; d++) ns[d] = lw->g.ns[d];
  return HSMC_OK;
}

int hsmc_lwidom_refresh(hsmc_lwidom *lw) {
  if (!lw) return HSMC_ERR_INVALID_ARG;
  int e = set_grid(lw);  // the box may have changed (NpT)
  if (e) return e;
  if (!lw->view.uploaded) return HSMC_ERR_INVALID_ARG;
  const cudaStream_t s = lw->view.stream;
  const SubGrid &g = lw->g;
  LW_CUDA(cudaEventRecord(lw->e0, s));
  LW_CUDA(cudaMemsetAsync(lw->status.ptr, 0, sizeof(int), s));
  LW_CUDA(cudaMemsetAsync(lw->occ.ptr, 0, sizeof(unsigned) * g.nsub, s));
  const int n = lw->view.sp.n;
  k_sub_count<<<(n + 255) / 256, 256, 0, s>>>(lw->view.sp.pos, n, g, lw->occ.ptr);
  k_sub_pattern<<<(g.nsub + 255) / 256, 256, 0, s>>>(lw->occ.ptr, g, lw->pat.ptr);
  launch_logits(lw, lw->pat.ptr, g.nsub, lw->logits.ptr);
  k_pi<<<(g.nsub + 255) / 256, 256, 0, s>>>(lw->logits.ptr, lw->pi.ptr, g.nsub);
  const int nb = (g.nsub + SCAN_BLK - 1) / SCAN_BLK;
  k_scan_block<<<nb, SCAN_T, 0, s>>>(lw->pi.ptr, lw->cdf.ptr, lw->totals.ptr, g.nsub);
  k_scan_block<<<1, SCAN_T, 0, s>>>(lw->totals.ptr, lw->totals.ptr, nullptr, nb);
  k_scan_add<<<nb, SCAN_T, 0, s>>>(lw->cdf.ptr, lw->totals.ptr, g.nsub);
  LW_CUDA(cudaEventRecord(lw->e1, s));
  e = sync_status(lw);
  if (e) return e;
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, lw->e0, lw->e1);
  lw->last_ms = ms;
  lw->refreshed = true;
  return HSMC_OK;
}

int hsmc_lwidom_patterns(hsmc_lwidom *lw, uint32_t *out, int64_t n) {
  if (!lw || !out || n != lw->g.nsub || !lw->refreshed) return HSMC_ERR_INVALID_ARG;
  LW_CUDA(cudaMemcpy(out, lw->pat.ptr, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToHost));
  return HSMC_OK;
}

int hsmc_lwidom_proposal(hsmc_lwidom *lw, double *pi, double *cdf, int64_t n) {
  if (!lw || n != lw->g.nsub || !lw->refreshed) return HSMC_ERR_INVALID_ARG;
  if (pi) LW_CUDA(cudaMemcpy(pi, lw->pi.ptr, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
  if (cdf) LW_CUDA(cudaMemcpy(cdf, lw->cdf.ptr, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
  return HSMC_OK;
}

int hsmc_lwidom_logits(hsmc_lwidom *lw, const uint32_t *patterns, int64_t n, float *logits) {
  if (!lw || !patterns || !logits || n <= 0) return HSMC_ERR_INVALID_ARG;
  const cudaStream_t s = lw->view.stream;
  LW_CUDA(lw->qpat.ensure((size_t)n));
  LW_CUDA(lw->logits.ensure((size_t)n > (size_t)lw->g.nsub ? (size_t)n : (size_t)lw->g.nsub));
  LW_CUDA(cudaMemcpyAsync(lw->qpat.ptr, patterns, sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, s));
  LW_CUDA(cudaMemsetAsync(lw->status.ptr, 0, sizeof(int), s));
  launch_logits(lw, lw->qpat.ptr, n, lw->logits.ptr);
  int e = sync_status(lw);
  if (e) return e;
  lw->refreshed = false;  // the logits buffer now holds these rows
  LW_CUDA(cudaMemcpy(logits, lw->logits.ptr, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost));
  return HSMC_OK;
}

int hsmc_lwidom_grad(hsmc_lwidom *lw, const uint32_t *samples, int64_t n, float w_pos, float w_neg, float *grad,
                     double *loss) {
  if (!lw || !samples || !grad || n <= 0) return HSMC_ERR_INVALID_ARG;
  const cudaStream_t s = lw->view.stream;
  LW_CUDA(lw->qpat.ensure((size_t)n));
  LW_CUDA(cudaMemcpyAsync(lw->qpat.ptr, samples, sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, s));
  LW_CUDA(cudaMemsetAsync(lw->status.ptr, 0, sizeof(int), s));
  run_grad(lw, lw->qpat.ptr, n, w_pos, w_neg);
  int e = sync_status(lw);
  if (e) return e;
  std::vector<float> g(NPARAM + 1);
  LW_CUDA(cudaMemcpy(g.data(), lw->grad.ptr, sizeof(float) * (NPARAM + 1), cudaMemcpyDeviceToHost));
  std::memcpy(grad, g.data(), sizeof(float) * NPARAM);
  if (loss) *loss = (double)g[NPARAM] / (double)n;
  return HSMC_OK;
}

int hsmc_lwidom_adam_step(hsmc_lwidom *lw, const float *grad, float lr) {
  if (!lw || !grad) return HSMC_ERR_INVALID_ARG;
  LW_CUDA(cudaMemcpyAsync(lw->grad.ptr, grad, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, lw->view.stream));
  adam_and_pack(lw, lr);
  lw->refreshed = false;
  return sync_status(lw);
}

static int insert_impl(hsmc_lwidom *lw, int64_t n, double alpha, double keep, hsmc_lwidom_stats *st, bool trace) {
  if (!lw || n < 0 || !st || !(alpha >= 0.0 && alpha <= 1.0) || !lw->refreshed) return HSMC_ERR_INVALID_ARG;
  if (!(keep <= 1.0)) return HSMC_ERR_INVALID_ARG;
  if (!(alpha > 0.0)) return HSMC_ERR_INVALID_ARG;  // the uniform component keeps every weight finite
  const cudaStream_t s = lw->view.stream;
  IsOut o{};
  o.sums = lw->sums.ptr;
  o.cnts = lw->cnts.ptr;
  const long long room = lw->capacity - lw->n_samples;
  if (keep >= 0.0 && room > 0) {
    o.collect = lw->samples.ptr + lw->n_samples;
    o.collect_cap = room;
    o.collect_n = lw->counter.ptr;
    o.keep_thr = keep >= 1.0 ? 4294967296ull : (unsigned long long)(keep * 4294967296.0);
    LW_CUDA(cudaMemsetAsync(lw->counter.ptr, 0, sizeof(unsigned long long), lw->view.stream));
  }
  if (trace) {
    LW_CUDA(lw->t_pts.ensure(3 * (size_t)n));
    LW_CUDA(lw->t_w.ensure((size_t)n));
    LW_CUDA(lw->t_cell.ensure((size_t)n));
    LW_CUDA(lw->t_uni.ensure((size_t)n));
    LW_CUDA(lw->t_ok.ensure((size_t)n));
    o.t_pts = lw->t_pts.ptr;
    o.t_w = lw->t_w.ptr;
    o.t_cell = lw->t_cell.ptr;
    o.t_uni = lw->t_uni.ptr;
    o.t_ok = lw->t_ok.ptr;
  }
  const unsigned long long thr =
      alpha >= 1.0 ? 4294967296ull : (unsigned long long)(alpha * 4294967296.0);
  LW_CUDA(cudaMemsetAsync(lw->status.ptr, 0, sizeof(int), s));
  LW_CUDA(cudaEventRecord(lw->e0, s));
  k_widom_is<<<IS_BLOCKS, IS_THREADS, 0, s>>>(lw->view.sp, lw->g, lw->cdf.ptr, lw->pi.ptr, lw->pat.ptr, n, lw->seq,
                                              lw->seed, thr, alpha, o);
  LW_CUDA(cudaEventRecord(lw->e1, s));
  int e = sync_status(lw);
  if (e) return e;
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, lw->e0, lw->e1);
  lw->last_ms = ms;
  lw->seq++;
  std::vector<double> sums(2 * IS_BLOCKS);
  std::vector<unsigned long long> cnts(3 * IS_BLOCKS);
  LW_CUDA(cudaMemcpy(sums.data(), lw->sums.ptr, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost));
  LW_CUDA(cudaMemcpy(cnts.data(), lw->cnts.ptr, sizeof(unsigned long long) * cnts.size(), cudaMemcpyDeviceToHost));
  hsmc_lwidom_stats r{};
  r.n = (uint64_t)n;
  unsigned long long col_pos = 0;
  for (int b = 0; b < IS_BLOCKS; b++) {
    r.sum_w += sums[2 * b];
    r.sum_w2 += sums[2 * b + 1];
    r.n_ok += cnts[3 * b];
    r.n_learned += cnts[3 * b + 1];
    col_pos += cnts[3 * b + 2];
  }
  *st = r;
  if (o.collect) {
    unsigned long long claimed = 0;
    LW_CUDA(cudaMemcpy(&claimed, lw->counter.ptr, sizeof(claimed), cudaMemcpyDeviceToHost));
    lw->n_samples += (long long)claimed < room ? (long long)claimed : room;
    lw->n_pos += (long long)col_pos;
  }
  return HSMC_OK;
}

int hsmc_lwidom_insert(hsmc_lwidom *lw, int64_t n, double alpha, double keep_failures, hsmc_lwidom_stats *st) {
  return insert_impl(lw, n, alpha, keep_failures, st, false);
}

int hsmc_lwidom_insert_traced(hsmc_lwidom *lw, int64_t n, double alpha, double *points, int32_t *subcell,
                              uint8_t *uniform, double *weight, uint8_t *ok, hsmc_lwidom_stats *st) {
  if (!points || !subcell || !uniform || !weight || !ok) return HSMC_ERR_INVALID_ARG;
  int e = insert_impl(lw, n, alpha, -1.0, st, true);
  if (e || n == 0) return e;
  LW_CUDA(cudaMemcpy(points, lw->t_pts.ptr, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost));
  LW_CUDA(cudaMemcpy(subcell, lw->t_cell.ptr, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
  LW_CUDA(cudaMemcpy(uniform, lw->t_uni.ptr, (size_t)n, cudaMemcpyDeviceToHost));
  LW_CUDA(cudaMemcpy(weight, lw->t_w.ptr, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
  LW_CUDA(cudaMemcpy(ok, lw->t_ok.ptr, (size_t)n, cudaMemcpyDeviceToHost));
  return HSMC_OK;
}

int hsmc_lwidom_uniform(hsmc_lwidom *lw, int64_t n, uint64_t *accepted) {
  if (!lw || n < 0 || !accepted) return HSMC_ERR_INVALID_ARG;
  int e = ctx_view(lw->ctx, &lw->view);
  if (e) return e;
  if (!lw->view.uploaded) return HSMC_ERR_INVALID_ARG;
  const cudaStream_t s = lw->view.stream;
  LW_CUDA(cudaMemsetAsync(lw->status.ptr, 0, sizeof(int), s));
  LW_CUDA(cudaEventRecord(lw->e0, s));
  k_widom_plain<<<IS_BLOCKS, IS_THREADS, 0, s>>>(lw->view.sp, n, lw->plain_seq, lw->seed, lw->cnts.ptr);
  LW_CUDA(cudaEventRecord(lw->e1, s));
  e = sync_status(lw);
  if (e) return e;
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, lw->e0, lw->e1);
  lw->last_ms = ms;
  lw->plain_seq++;
  std::vector<unsigned long long> cnts(IS_BLOCKS);
  LW_CUDA(cudaMemcpy(cnts.data(), lw->cnts.ptr, sizeof(unsigned long long) * IS_BLOCKS, cudaMemcpyDeviceToHost));
  unsigned long long t = 0;
  for (int b = 0; b < IS_BLOCKS; b++) t += cnts[b];
  *accepted = t;
  return HSMC_OK;
}

int hsmc_lwidom_train(hsmc_lwidom *lw, int epochs, int64_t batch, float lr, float w_pos, float w_neg,
                      double *last_loss) {
  if (!lw || epochs < 0 || batch <= 0 || !(lr > 0.0f) || !(w_pos > 0.0f) || !(w_neg > 0.0f))
    return HSMC_ERR_INVALID_ARG;
  if (lw->n_samples == 0) return HSMC_ERR_INVALID_ARG;
  const cudaStream_t s = lw->view.stream;
  LW_CUDA(cudaMemsetAsync(lw->status.ptr, 0, sizeof(int), s));
  LW_CUDA(cudaEventRecord(lw->e0, s));
  for (int ep = 0; ep < epochs; ep++) {
    for (long long b0 = 0; b0 < lw->n_samples; b0 += batch) {
      const long long nb = (lw->n_samples - b0) < batch ? (lw->n_samples - b0) : batch;
      run_grad(lw, lw->samples.ptr + b0, nb, w_pos, w_neg);
      adam_and_pack(lw, lr);
    }
  }
  LW_CUDA(cudaEventRecord(lw->e1, s));
  int e = sync_status(lw);
  if (e) return e;
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, lw->e0, lw->e1);
  lw->last_ms = ms;
  if (last_loss) {
    float l = 0.0f;
    LW_CUDA(cudaMemcpy(&l, lw->grad.ptr + NPARAM, sizeof(float), cudaMemcpyDeviceToHost));
    const long long nb_last = lw->n_samples - ((lw->n_samples - 1) / batch) * batch;
    *last_loss = (double)l / (double)nb_last;  // mean weighted loss of the last minibatch
  }
  lw->refreshed = false;
  return HSMC_OK;
}

int hsmc_lwidom_samples(hsmc_lwidom *lw, int64_t *n, int64_t *n_pos) {
  if (!lw) return HSMC_ERR_INVALID_ARG;
  if (n) *n = lw->n_samples;
  if (n_pos) *n_pos = lw->n_pos;
  return HSMC_OK;
}

int hsmc_lwidom_clear_samples(hsmc_lwidom *lw) {
  if (!lw) return HSMC_ERR_INVALID_ARG;
  lw->n_samples = 0;
  lw->n_pos = 0;
  return HSMC_OK;
}

int hsmc_lwidom_last_timing(hsmc_lwidom *lw, double *ms) {
  if (!lw || !ms) return HSMC_ERR_INVALID_ARG;
  *ms = lw->last_ms;
  return HSMC_OK;
}

}  // extern "C"
