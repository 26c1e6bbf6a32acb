// Neural martingale control variate for the Heston arithmetic-Asian option
// (no reference counterpart; the path it wraps is the reference Euler sampler
// with full-truncation Heston coefficients, tff/models/euler_sampling.py:513-537).
//
// Network g(t, log S, v): 3 -> 64 -> 64 -> 1, SiLU, BF16 weights and
// activations, FP32 accumulation.  Layer 2 (64 x 64, the GEMM-shaped part)
// runs on the tcgen05 tensor cores: a warpgroup's 128 rows (one per thread)
// form an M = 128 tile with the accumulator in TMEM.  Layer 1 (K = 3) is 192
// FMAs per row on the CUDA cores with the same BF16-rounded operands the
// tensor cores would use; W1 column 3 holds its bias (input feature 1).
// SiLU runs in packed BF16 (one SFU tanh per pair); layer 3 is a 64-term
// FP32 dot product.  The backward GEMMs (d1 = d2 W2, dW2 = d2^T H1,
// db2 = d2^T 1, dW1 = d1^T X) are tcgen05 MMAs.
//
// heston_asian_kernel<MODE>: full-truncation Euler paths (Philox in-kernel),
//   num_dates monitoring dates marked in the step table's slot column.
//   MODE 0: plain estimator sums of Y = e^{-rT} max(mean_k S_k - K, 0).
//   MODE 1: pilot data — per path and interval k the start features
//           (t_k, log S_k, v_k), the discounted-spot increment
//           dS~_k = e^{-r t_{k+1}} S_{k+1} - e^{-r t_k} S_k, and Y.
//   MODE 2: fused control variate C = sum_k g(t_k, X_k, V_k) dS~_k with the
//           network evaluated per warpgroup tile at every interval start.
//   Modes 0/2 accumulate (Y, Y^2, C, C^2, Y C) in FP64 (fixed order).
//   Under the log-Euler step E[S~_{i+1} | F_i] = S~_i, so E[C] = 0 exactly.
// mlp_train_step_kernel: one Adam step's gradient for a minibatch of paths,
//   loss = mean_p (Y_p - c - sum_k g_pk dS~_pk)^2: per CTA one 128-row tile
//   of whole paths — forward on tensor cores, per-path residuals, backward
//   with d1 = d2 W2, dW2 = d2^T H1, db2, dw3 and dW1 = d1^T X as tcgen05 MMAs.
// mlp_adam_kernel: fixed-order parallel reduction of the per-CTA gradients
//   and the Adam update of the FP32 master parameters and their BF16 copies.
#include <cuda_bf16.h>
#include <string.h>

#include "tqf_tc.cuh"

namespace tqf {
namespace {

constexpr int kH = 64;            // hidden width
constexpr int kIn = 16;           // padded input width (K of layer 1)
constexpr int kMaxDates = 64;
constexpr int kPathThreads = 256;  // two warpgroups
constexpr int kTrainThreads = 128;
// parameter vector layout (FP32 master copy)
constexpr int kOffW1 = 0;
constexpr int kOffW2 = kOffW1 + kH * kIn;   // 1024
constexpr int kOffB2 = kOffW2 + kH * kH;    // 5120
constexpr int kOffW3 = kOffB2 + kH;         // 5184
constexpr int kOffB3 = kOffW3 + kH;         // 5248
constexpr int kOffC = kOffB3 + 1;           // 5249
constexpr int kNumParams = kOffC + 1;       // 5250
constexpr int kGradWidth = kNumParams + 2;  // + loss sum + one zero pad (16-byte rows)

// Canonical no-swizzle K-major tiles with the 8-row groups contiguous
// (SBO = 128 B) and the 8-column groups R/8 x 128 B apart (LBO): a K-slice of
// the operand is one contiguous block, which the tensor core reads without
// shared-memory bank conflicts.
constexpr uint32_t kXLbo = 2048, kXSbo = 128;   // [128 x 16]
constexpr uint32_t kHLbo = 2048, kHSbo = 128;   // [128 x 64]
constexpr uint32_t kW2Lbo = 1024, kW2Sbo = 128; // [64 x 64]
constexpr uint32_t kOnesLbo = 128, kOnesSbo = 2048;  // [16 x 128] read MN-major
constexpr int kXBytes = 128 * kIn * 2;
constexpr int kHBytes = 128 * kH * 2;
constexpr int kW2Bytes = kH * kH * 2;

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t p) { return __uint_as_float(p << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t p) { return __uint_as_float(p & 0xFFFF0000u); }
__device__ __forceinline__ float round_bf16(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// SiLU of two values in packed BF16 (one SFU op for the pair):
// x -> h = bf16(x)/2, s = h + h tanh(h) = x sigmoid(x), returned as bf16x2.
__device__ __forceinline__ uint32_t silu_bf16x2(float a, float b) {
  const uint32_t x2 = pack_bf16x2(a, b);
  uint32_t h2, t2, s2;
  asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(h2) : "r"(x2), "r"(0x3F003F00u));
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t2) : "r"(h2));
  asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(s2) : "r"(h2), "r"(t2), "r"(h2));
  return s2;
}

__device__ __forceinline__ uint32_t bf2_mul(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t bf2_fma(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
constexpr uint32_t kBf2Half = 0x3F003F00u, kBf2One = 0x3F803F80u, kBf2MinusOne = 0xBF80BF80u;

// SiLU'(x) = s (1 + x (1 - s)), s = sigmoid(x) = (1 + tanh(x/2)) / 2, for a
// packed BF16 pair (one SFU op for the pair).
__device__ __forceinline__ uint32_t dsilu_bf16x2(uint32_t x2) {
  uint32_t h2, t2;
  asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(h2) : "r"(x2), "r"(kBf2Half));
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t2) : "r"(h2));
  const uint32_t sg = bf2_fma(t2, kBf2Half, kBf2Half);
  const uint32_t om = bf2_fma(sg, kBf2MinusOne, kBf2One);  // 1 - s
  return bf2_mul(sg, bf2_fma(x2, om, kBf2One));
}

// Layer 1 on the CUDA cores (K = 3 is not GEMM-shaped): a1_j = w1_j . (f0,
// f1, f2) + b1_j with BF16-rounded operands (exact products, FP32 sums, as
// the tensor cores would form them), SiLU in packed BF16, written as row r of
// the K-major H tile.  s_l1[j] = (w_j0, w_j1, w_j2, b1_j).  If a1 is given,
// the FP32 pre-activations are also returned.
__device__ __forceinline__ void layer1_row(const float4* __restrict__ s_l1, float f0, float f1, float f2,
                                           unsigned char* sH, int r, float* a1 = nullptr) {
#pragma unroll
  for (int jc = 0; jc < 8; ++jc) {
    uint32_t pk[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 wa = s_l1[8 * jc + 2 * q];
      const float4 wb = s_l1[8 * jc + 2 * q + 1];
      const float aa = fmaf(wa.x, f0, fmaf(wa.y, f1, fmaf(wa.z, f2, wa.w)));
      const float ab = fmaf(wb.x, f0, fmaf(wb.y, f1, fmaf(wb.z, f2, wb.w)));
      if (a1) {
        a1[8 * jc + 2 * q] = aa;
        a1[8 * jc + 2 * q + 1] = ab;
      }
      pk[q] = silu_bf16x2(aa, ab);
    }
    *reinterpret_cast<uint4*>(sH + tc::kmajor_off(r, 8 * jc, kHLbo, kHSbo)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
  }
}

// Warpgroup barrier (named barrier 1 or 2, 128 threads).  Immediate barrier
// ids keep the kernel's barrier count at 3; a register id would reserve all
// 16 and make the occupancy calculator allow one CTA per SM.
__device__ __forceinline__ void wg_sync(int wg) {
  if (wg == 0)
    asm volatile("bar.sync 1, 128;" ::: "memory");
  else
    asm volatile("bar.sync 2, 128;" ::: "memory");
}

// Bounded wait on an MMA-completion mbarrier; on time-out records the status
// and waits once more (bounded) so that no MMA is in flight afterwards.
__device__ __forceinline__ bool mma_wait(uint64_t* bar, uint32_t& phase, int32_t* status) {
  bool ok = mbar_wait_bounded(bar, phase);
  if (!ok) {
    if (status) atomicExch(status, TQF_E_TIMEOUT);
    ok = mbar_wait_bounded(bar, phase);
  }
  phase ^= 1u;
  tc::fence_after_sync();
  return ok;
}

struct MlpScalars {
  float4 l1[kH];  // (w_j0, w_j1, w_j2, b1_j), BF16-rounded
  float b2[kH];
  float w3[kH];
  float b3;
  float fscale[3], fshift[3];
};

// The same network weights in kernel parameters (constant bank): inference
// reads them as direct FMA operands, with no shared-memory load instructions.
struct MlpConst {
  float4 l1[kH];
  float b2[kH];
  float w3[kH];
  float b3;
  float fscale[3], fshift[3];
};

// Normalised, BF16-rounded input features.
template <class W>
__device__ __forceinline__ void features(const W& ms, float t, float x, float v, float& f0, float& f1,
                                         float& f2) {
  f0 = round_bf16((t - ms.fshift[0]) * ms.fscale[0]);
  f1 = round_bf16((x - ms.fshift[1]) * ms.fscale[1]);
  f2 = round_bf16((v - ms.fshift[2]) * ms.fscale[2]);
}

// Issue half of one network evaluation for the warpgroup's 128 rows: layer 1
// on the CUDA cores into the H tile, then (one thread) layer 2 as four
// tcgen05 MMAs into the warpgroup's 64 TMEM columns, committed to `bar`.
template <class W>
__device__ __forceinline__ void mlp_issue(int wg, int tid, const W& ms, unsigned char* sH,
                                          const unsigned char* sW2, uint32_t tmem_d, uint64_t* bar, float t,
                                          float x, float v) {
  float f0, f1, f2;
  features(ms, t, x, v, f0, f1, f2);
  layer1_row(ms.l1, f0, f1, f2, sH, tid);
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  wg_sync(wg);
  tc::fence_after_sync();
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, kH, false, false);
#pragma unroll
    for (int s = 0; s < kH / 16; ++s)
      tc::mma_bf16(tmem_d, tc::smem_desc(smem_addr(sH) + 2u * s * kHLbo, kHLbo, kHSbo),
                   tc::smem_desc(smem_addr(sW2) + 2u * s * kW2Lbo, kW2Lbo, kW2Sbo), idesc, s > 0 ? 1u : 0u);
    tc::commit(bar);
  }
}

// Completes an evaluation: waits for the MMAs, reads this row's 64 layer-2
// accumulators, applies bias and SiLU (packed BF16) and the FP32 layer-3 dot
// product.  Optionally returns the FP32 pre-activations a2 and the BF16
// activations h2 (as floats).
template <class W>
__device__ __forceinline__ float mlp_collect(int tid, const W& ms, uint32_t tmem_d, uint64_t* bar,
                                             uint32_t& phase, int32_t* status, float* a2 = nullptr,
                                             float* h2 = nullptr) {
  mma_wait(bar, phase, status);
  const uint32_t lane_base = (uint32_t)(32 * ((tid >> 5) & 3)) << 16;
  float g = ms.b3;
#pragma unroll
  for (int c = 0; c < kH; c += 16) {
    float acc[16];
    tc::tmem_ld16(tmem_d + lane_base + (uint32_t)c, acc);
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
      const float aa = acc[j] + ms.b2[c + j], ab = acc[j + 1] + ms.b2[c + j + 1];
      const uint32_t sp = silu_bf16x2(aa, ab);
      const float ha = bf16_lo(sp), hb = bf16_hi(sp);
      if (a2) {
        a2[c + j] = aa;
        a2[c + j + 1] = ab;
      }
      if (h2) {
        h2[c + j] = ha;
        h2[c + j + 1] = hb;
      }
      g = fmaf(ms.w3[c + j], ha, fmaf(ms.w3[c + j + 1], hb, g));
    }
  }
  tc::fence_before_sync();  // orders these TMEM reads before the next MMA into tmem_d
  return g;
}

// ---- path kernel -----------------------------------------------------------------
struct AsianSmem {
  uint64_t bar[2];
  uint32_t tmem_slot;
  uint32_t pad;
  double acc[kPathThreads / 32][5];
  float date_t[kMaxDates], date_disc[kMaxDates];
};

// Mode 2 pipelines the network with the simulation: the evaluation for
// interval k is issued at its start date (layer 1 + the layer-2 MMAs) and
// collected at its end date, so the tensor-core work overlaps the ~T/D of
// path stepping in between.  Each warpgroup owns 64 TMEM columns.
template <int MODE>
__global__ void __launch_bounds__(kPathThreads, MODE == 2 ? 4 : 1)
    heston_asian_kernel(tqf_heston_asian_args a, const __grid_constant__ MlpConst wc) {
  extern __shared__ __align__(1024) unsigned char smem[];
  AsianSmem* S = reinterpret_cast<AsianSmem*>(smem);
  unsigned char* tiles = smem + ((sizeof(AsianSmem) + 1023) & ~(size_t)1023);
  unsigned char* sW2 = tiles;
  unsigned char* sHw = sW2 + kW2Bytes;  // 2 x [128 x 64]
  float* table = reinterpret_cast<float*>(MODE == 2 ? sHw + 2 * kHBytes : tiles);  // [steps][8]
  const int tid = threadIdx.x & 127, wg = threadIdx.x >> 7;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int D = a.num_dates;
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    S->date_t[i] = a.date_table[4 * i];
    S->date_disc[i] = a.date_table[4 * i + 1];
  }
  for (int i = threadIdx.x; i < (kPathThreads / 32) * 5; i += blockDim.x) (&S->acc[0][0])[i] = 0.0;
  for (int i = threadIdx.x; i < a.num_steps * 8; i += blockDim.x) table[i] = a.step_table[i];
  if (MODE == 2) {
    const uint4* w2 = static_cast<const uint4*>(a.mlp.w2_bf16);
    for (int i = threadIdx.x; i < kH * kH / 8; i += blockDim.x)
      *reinterpret_cast<uint4*>(sW2 + tc::kmajor_off(i >> 3, 8 * (i & 7), kW2Lbo, kW2Sbo)) = w2[i];
    if (threadIdx.x == 0) {
      mbar_init(&S->bar[0], 1);
      mbar_init(&S->bar[1], 1);
    }
    if (warp == 0) tc::tmem_alloc(&S->tmem_slot, 128);
  }
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem_d = MODE == 2 ? S->tmem_slot + (uint32_t)(wg * kH) : 0u;
  unsigned char* sH = sHw + wg * kHBytes;
  uint64_t* bar = &S->bar[wg];
  uint32_t phase = 0;
  const float K = (float)a.strike, discT = (float)a.discount_T, x0 = (float)a.x0, v0 = (float)a.v0;
  const float S0 = __expf(x0);
  const float inv_D = 1.f / (float)D;
  const int64_t N = a.num_paths;
  const int64_t per_round = (int64_t)gridDim.x * kPathThreads;
  for (int64_t base = 0; base < N; base += per_round) {
    const int64_t path = base + (int64_t)blockIdx.x * kPathThreads + threadIdx.x;
    const bool valid = path < N;
    const int64_t p = (valid ? path : 0) + a.draws.path_offset;
    const uint32_t plo = (uint32_t)p, phi = (uint32_t)((uint64_t)p >> 32);
    float x = x0, v = v0, avg = 0.f, cv = 0.f, prev = S0;
    if (MODE == 2) mlp_issue(wg, tid, wc, sH, sW2, tmem_d, bar, 0.f, x0, v0);
    if (MODE == 1 && valid) reinterpret_cast<float4*>(a.pilot_feats)[path * D] = make_float4(0.f, x0, v0, 0.f);
    float zbuf[4];
    for (int i = 0; i < a.num_steps; ++i) {
      if ((i & 1) == 0) {
        const uint4 r = philox4x32_10(make_uint4((uint32_t)(i >> 1), plo, phi, 0u), a.draws.key0, a.draws.key1);
        box_muller_f32(r.x, r.y, zbuf[0], zbuf[1]);
        box_muller_f32(r.z, r.w, zbuf[2], zbuf[3]);
      }
      const float za = (i & 1) ? zbuf[2] : zbuf[0];
      const float zb = (i & 1) ? zbuf[3] : zbuf[1];
      const float4 c0 = reinterpret_cast<const float4*>(table)[2 * i];
      const float4 c1 = reinterpret_cast<const float4*>(table)[2 * i + 1];
      {
        const float vp = fmaxf(v, 0.f);
        const float sq = sqrt_approx(vp);
        const float dw0 = za * c0.y, dw1 = zb * c0.y;
        const float xn = x + fmaf(-c0.x, vp, c0.z) + sq * dw0;
        const float vn = v + fmaf(-c0.w, vp, c1.x) + sq * fmaf(c1.z, dw1, c1.y * dw0);
        x = xn;
        v = vn;
      }
      const int k = (int)c1.w;  // date index or -1 (uniform across the CTA)
      if (k >= 0) {
        const float Sk = __expf(x);
        const float dsk = S->date_disc[k] * Sk - prev;
        avg += Sk;
        if (MODE == 2) {
          const float g = mlp_collect(tid, wc, tmem_d, bar, phase, a.dev_status);
          cv = fmaf(g, dsk, cv);
        }
        if (MODE == 1 && valid) {
          a.pilot_dS[path * D + k] = dsk;
          if (k + 1 < D)
            reinterpret_cast<float4*>(a.pilot_feats)[path * D + k + 1] = make_float4(S->date_t[k], x, v, 0.f);
        }
        prev = S->date_disc[k] * Sk;
        if (MODE == 2 && k + 1 < D) mlp_issue(wg, tid, wc, sH, sW2, tmem_d, bar, S->date_t[k], x, v);
      }
    }
    const float Y = discT * fmaxf(avg * inv_D - K, 0.f);
    if (MODE == 1) {
      if (valid) a.pilot_Y[path] = Y;
    } else {
      float q[5];
      q[0] = valid ? Y : 0.f;
      q[1] = q[0] * q[0];
      q[2] = valid ? cv : 0.f;
      q[3] = q[2] * q[2];
      q[4] = q[0] * q[2];
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        float s = q[j];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) S->acc[warp][j] += (double)s;
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (MODE != 1 && threadIdx.x < 5) {
    double s = 0.0;
    for (int w = 0; w < kPathThreads / 32; ++w) s += S->acc[w][threadIdx.x];
    static_cast<double*>(a.workspace)[(size_t)blockIdx.x * 5 + threadIdx.x] = s;
  }
  if (MODE == 2 && warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(S->tmem_slot, 128);
  }
}

// Mode 2 holds W2 and two H tiles; its 45..56 KB of shared memory lets at most
// 4 CTAs (4 x 128 TMEM columns = the SM's 512) share an SM, so no TMEM
// allocation ever has to wait.
size_t asian_smem_bytes(int mode, int steps) {
  const size_t head = (sizeof(AsianSmem) + 1023) & ~(size_t)1023;
  const size_t tiles = mode == 2 ? (size_t)kW2Bytes + 2 * kHBytes : 0;
  size_t total = head + tiles + (size_t)steps * 8 * sizeof(float);
  if (mode == 2 && total < 46 * 1024) total = 46 * 1024;
  return total;
}

template <int MODE>
int asian_grid(int64_t n, size_t smem) {
  auto k = heston_asian_kernel<MODE>;
  set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kPathThreads, smem) != cudaSuccess || occ < 1) occ = 1;
  // The runtime reports one resident CTA for this tcgen05 kernel although its
  // registers (64), shared memory and barriers allow four (ncu: all limits 4);
  // size the persistent grid for four, the most whose 128 TMEM columns fit
  // the SM's 512.
  if (MODE == 2) occ = 4;
  int64_t g = (n + kPathThreads - 1) / kPathThreads;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

// ---- training step ---------------------------------------------------------------------
// One CTA = one warpgroup = one 128-row tile holding all num_dates rows of
// paths_per_cta paths (paths_per_cta x num_dates <= 128), so the forward pass
// runs once and the per-path residual never crosses CTAs.  With
// q2 = w3 (.) SiLU'(a2) (known after the forward pass) and the per-row output
// gradient d3 = -2 r_p dS_pk / B (known after the residual):
//   d2 = d3 q2,  d1 = d3 (Q2 W2) (.) SiLU'(a1),
//   dW2 = Q2^T (d3 H1),  db2 = Q2^T d3,  dw3 = H2^T d3,  dW1 = D1^T X,
// so the Q2 W2 product is issued before the residual is known and overlaps
// it.  Layer 1 runs on the tensor cores here (X [128 x 16] x W1^T, bias in
// input column 3) and its pre-activations stay in TMEM for the backward
// pass.  The backward elementwise work (SiLU', the d3 scaling) runs in
// packed BF16, two values per instruction; its operands are BF16 anyway.
// TMEM (128 columns): [64, 128) a1, then dW2; [0, 64) the layer-2
// accumulator, then Q2 W2, then db2 | dw3 | dW1 (16 columns each).
constexpr uint32_t kW1Lbo = 1024, kW1Sbo = 128;  // W1 [64 x 16] K-major
constexpr int kW1Bytes = kH * kIn * 2;

struct TrainSmem {
  uint64_t bar;
  uint32_t tmem_slot;
  uint32_t pad;
  float b2[kH];
  float w3[kH];
  uint32_t w3p[kH / 2];  // w3 as BF16 pairs
  float4 fs;             // feature scale (x, y, z)
  float4 fo;             // feature shift
  float b3, c;
  float gds[128];     // g x dS~ per row
  float resid[128];   // per path
  float wloss[4], wsum[4], wb3[4];
};

__global__ void __launch_bounds__(kTrainThreads) mlp_train_step_kernel(tqf_mlp_train_args a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  TrainSmem* S = reinterpret_cast<TrainSmem*>(smem);
  unsigned char* t0 = smem + ((sizeof(TrainSmem) + 1023) & ~(size_t)1023);
  unsigned char* sW2 = t0;
  unsigned char* sW1 = sW2 + kW2Bytes;
  unsigned char* sX = sW1 + kW1Bytes;
  unsigned char* sH = sX + kXBytes;   // H1, scaled by d3 in place before dW2
  unsigned char* sH2 = sH + kHBytes;
  unsigned char* sQ2 = sH2 + kHBytes;
  unsigned char* sD1 = sQ2 + kHBytes;
  unsigned char* sT3 = sD1 + kHBytes;  // [16 x 128] MN-major, column 0 = d3
  const int D = a.num_dates;
  const int P = a.paths_per_cta;
  const int rows = P * D;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t p0 = a.path_begin + (int64_t)blockIdx.x * P;
  const float inv_B = 1.f / (float)a.batch_paths;
  {
    // W2 (BF16 [64][64] row-major) and W1 (BF16 [64][16]) into K-major tiles
    const uint4* w2 = static_cast<const uint4*>(a.w2_bf16);
    for (int i = tid; i < kH * kH / 8; i += kTrainThreads)
      *reinterpret_cast<uint4*>(sW2 + tc::kmajor_off(i >> 3, 8 * (i & 7), kW2Lbo, kW2Sbo)) = w2[i];
    const uint4* w1 = static_cast<const uint4*>(a.w1_bf16);
    for (int i = tid; i < kH * kIn / 8; i += kTrainThreads)
      *reinterpret_cast<uint4*>(sW1 + tc::kmajor_off(i >> 1, 8 * (i & 1), kW1Lbo, kW1Sbo)) = w1[i];
  }
  const float* Pm = a.params;
  for (int i = tid; i < kH; i += kTrainThreads) {
    S->b2[i] = Pm[kOffB2 + i];
    S->w3[i] = Pm[kOffW3 + i];
  }
  for (int i = tid; i < kH / 2; i += kTrainThreads) S->w3p[i] = pack_bf16x2(Pm[kOffW3 + 2 * i], Pm[kOffW3 + 2 * i + 1]);
  for (int i = tid; i < 16 * 128 * 2 / 16; i += kTrainThreads)
    reinterpret_cast<uint4*>(sT3)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    S->b3 = Pm[kOffB3];
    S->c = Pm[kOffC];
    S->fs = make_float4(a.feat_scale[0], a.feat_scale[1], a.feat_scale[2], 0.f);
    S->fo = make_float4(a.feat_shift[0], a.feat_shift[1], a.feat_shift[2], 0.f);
    mbar_init(&S->bar, 1);
  }
  if (warp == 0) tc::tmem_alloc(&S->tmem_slot, 128);
  // this row's inputs
  const int r = tid;
  const bool in = r < rows;
  const int pl = in ? r / D : 0, dd = in ? r % D : 0;
  const int64_t gi = (p0 + pl) * D + dd;
  const float4 f = in ? reinterpret_cast<const float4*>(a.feats)[gi] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float dsv = in ? a.dS[gi] : 0.f;
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = S->tmem_slot;
  const uint32_t t_fwd = tm, t_a1 = tm + 64, t_db2 = tm, t_dw3 = tm + 16, t_dw1 = tm + 32, t_dw2 = tm + 64;
  const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
  uint32_t phase = 0;
  // ---- forward.  Layer 1: X row = (BF16 features, 1, 0...) -> a1 in TMEM
  {
    const float4 fs = S->fs, fo = S->fo;
    const float f0 = round_bf16((f.x - fo.x) * fs.x), f1 = round_bf16((f.y - fo.y) * fs.y),
                f2 = round_bf16((f.z - fo.z) * fs.z);
    *reinterpret_cast<uint4*>(sX + tc::kmajor_off(r, 0, kXLbo, kXSbo)) =
        make_uint4(pack_bf16x2(f0, f1), pack_bf16x2(f2, 1.f), 0u, 0u);
    *reinterpret_cast<uint4*>(sX + tc::kmajor_off(r, 8, kXLbo, kXSbo)) = make_uint4(0u, 0u, 0u, 0u);
  }
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (tid == 0) {
    tc::mma_bf16(t_a1, tc::smem_desc(smem_addr(sX), kXLbo, kXSbo), tc::smem_desc(smem_addr(sW1), kW1Lbo, kW1Sbo),
                 tc::idesc_bf16(128, kH, false, false), 0u);
    tc::commit(&S->bar);
  }
  mma_wait(&S->bar, phase, a.dev_status);
#pragma unroll
  for (int c = 0; c < kH; c += 16) {
    float acc[16];
    tc::tmem_ld16(t_a1 + lane_base + (uint32_t)c, acc);
#pragma unroll
    for (int h = 0; h < 16; h += 8)
      *reinterpret_cast<uint4*>(sH + tc::kmajor_off(r, c + h, kHLbo, kHSbo)) =
          make_uint4(silu_bf16x2(acc[h], acc[h + 1]), silu_bf16x2(acc[h + 2], acc[h + 3]),
                     silu_bf16x2(acc[h + 4], acc[h + 5]), silu_bf16x2(acc[h + 6], acc[h + 7]));
  }
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  // Layer 2 on the tensor cores
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, kH, false, false);
#pragma unroll
    for (int s = 0; s < kH / 16; ++s)
      tc::mma_bf16(t_fwd, tc::smem_desc(smem_addr(sH) + 2u * s * kHLbo, kHLbo, kHSbo),
                   tc::smem_desc(smem_addr(sW2) + 2u * s * kW2Lbo, kW2Lbo, kW2Sbo), idesc, s > 0 ? 1u : 0u);
    tc::commit(&S->bar);
  }
  mma_wait(&S->bar, phase, a.dev_status);
  // bias, SiLU (H2), layer 3 (g, FP32) and q2 = w3 SiLU'(a2) (Q2)
  float g = S->b3;
  const uint32_t keep = in ? 0xFFFFFFFFu : 0u;
#pragma unroll
  for (int c = 0; c < kH; c += 16) {
    float acc[16];
    tc::tmem_ld16(t_fwd + lane_base + (uint32_t)c, acc);
#pragma unroll
    for (int h = 0; h < 16; h += 8) {
      const float4 ba = *reinterpret_cast<const float4*>(&S->b2[c + h]);
      const float4 bb = *reinterpret_cast<const float4*>(&S->b2[c + h + 4]);
      const float4 wa = *reinterpret_cast<const float4*>(&S->w3[c + h]);
      const float4 wb = *reinterpret_cast<const float4*>(&S->w3[c + h + 4]);
      const uint4 wp = *reinterpret_cast<const uint4*>(&S->w3p[(c + h) / 2]);
      const float bias[8] = {ba.x, ba.y, ba.z, ba.w, bb.x, bb.y, bb.z, bb.w};
      const float w3v[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
      const uint32_t w3pv[4] = {wp.x, wp.y, wp.z, wp.w};
      uint32_t hp[4], qp[4];
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        const float aa = acc[h + j] + bias[j], ab = acc[h + j + 1] + bias[j + 1];
        const uint32_t sp = silu_bf16x2(aa, ab);
        g = fmaf(w3v[j], bf16_lo(sp), fmaf(w3v[j + 1], bf16_hi(sp), g));
        hp[j >> 1] = sp;
        qp[j >> 1] = bf2_mul(w3pv[j >> 1], dsilu_bf16x2(pack_bf16x2(aa, ab))) & keep;
      }
      *reinterpret_cast<uint4*>(sH2 + tc::kmajor_off(r, c + h, kHLbo, kHSbo)) = make_uint4(hp[0], hp[1], hp[2], hp[3]);
      *reinterpret_cast<uint4*>(sQ2 + tc::kmajor_off(r, c + h, kHLbo, kHSbo)) = make_uint4(qp[0], qp[1], qp[2], qp[3]);
    }
  }
  S->gds[r] = in ? g * dsv : 0.f;
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (tid == 0) {
    // Q2 W2: A = Q2 [128 x 64] K-major, B = W2 read MN-major (N = in, K = out)
    const uint32_t id_b1 = tc::idesc_bf16(128, kH, false, true);
#pragma unroll
    for (int s = 0; s < 4; ++s)
      tc::mma_bf16(t_fwd, tc::smem_desc(smem_addr(sQ2) + 2u * s * kHLbo, kHLbo, kHSbo),
                   tc::smem_desc(smem_addr(sW2) + 2u * s * kW2Sbo, kW2Sbo, kW2Lbo), id_b1, s > 0 ? 1u : 0u);
    tc::commit(&S->bar);
  }
  // ---- per-path residuals r_p = Y_p - c - sum_k g_pk dS~_pk (one warp per path)
  {
    float wl = 0.f, ws = 0.f;
    for (int p = warp; p < P; p += 4) {
      float sum = 0.f;
      for (int k = lane; k < D; k += 32) sum += S->gds[p * D + k];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
      const float rr = a.Y[p0 + p] - S->c - sum;
      if (lane == 0) S->resid[p] = rr;
      wl = fmaf(rr, rr, wl);
      ws += rr;
    }
    if (lane == 0) {
      S->wloss[warp] = wl;
      S->wsum[warp] = ws;
    }
  }
  __syncthreads();
  const float d3 = in ? -2.f * S->resid[pl] * dsv * inv_B : 0.f;
  {
    float b3p = d3;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) b3p += __shfl_xor_sync(0xffffffffu, b3p, off);
    if (lane == 0) S->wb3[warp] = b3p;
  }
  *reinterpret_cast<uint4*>(sT3 + tc::mnmajor_off(0, r, kOnesLbo, kOnesSbo)) =
      make_uint4(pack_bf16x2(d3, 0.f), 0u, 0u, 0u);
  // H1 row scaled by d3 (the B operand of dW2)
  {
    const uint32_t d3p = pack_bf16x2(d3, d3);
#pragma unroll
    for (int jc = 0; jc < 8; ++jc) {
      uint4* line = reinterpret_cast<uint4*>(sH + tc::kmajor_off(r, 8 * jc, kHLbo, kHSbo));
      uint4 w = *line;
      w.x = bf2_mul(w.x, d3p);
      w.y = bf2_mul(w.y, d3p);
      w.z = bf2_mul(w.z, d3p);
      w.w = bf2_mul(w.w, d3p);
      *line = w;
    }
  }
  // d1 = d3 (Q2 W2) (.) SiLU'(a1)
  mma_wait(&S->bar, phase, a.dev_status);
#pragma unroll
  for (int c = 0; c < kH; c += 16) {
    float p2[16], a1[16];
    tc::tmem_ld16(t_fwd + lane_base + (uint32_t)c, p2);
    tc::tmem_ld16(t_a1 + lane_base + (uint32_t)c, a1);
#pragma unroll
    for (int h = 0; h < 16; h += 8) {
      uint32_t dp[4];
#pragma unroll
      for (int j = 0; j < 8; j += 2)
        dp[j >> 1] = bf2_mul(pack_bf16x2(d3 * p2[h + j], d3 * p2[h + j + 1]),
                             dsilu_bf16x2(pack_bf16x2(a1[h + j], a1[h + j + 1])));
      *reinterpret_cast<uint4*>(sD1 + tc::kmajor_off(r, c + h, kHLbo, kHSbo)) = make_uint4(dp[0], dp[1], dp[2], dp[3]);
    }
  }
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (tid == 0) {
    // weight gradients, K = rows: A read MN-major with M = 64 (hidden)
    const uint32_t id_w2 = tc::idesc_bf16(64, kH, true, true);
    const uint32_t id_n16 = tc::idesc_bf16(64, 16, true, true);
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const uint32_t acc = s > 0 ? 1u : 0u;
      const uint64_t dq2 = tc::smem_desc(smem_addr(sQ2) + 2u * s * kHSbo, kHSbo, kHLbo);
      const uint64_t dt3 = tc::smem_desc(smem_addr(sT3) + 2u * s * kOnesLbo, kOnesLbo, kOnesSbo);
      tc::mma_bf16(t_dw2, dq2, tc::smem_desc(smem_addr(sH) + 2u * s * kHSbo, kHSbo, kHLbo), id_w2, acc);
      tc::mma_bf16(t_db2, dq2, dt3, id_n16, acc);
      tc::mma_bf16(t_dw3, tc::smem_desc(smem_addr(sH2) + 2u * s * kHSbo, kHSbo, kHLbo), dt3, id_n16, acc);
      tc::mma_bf16(t_dw1, tc::smem_desc(smem_addr(sD1) + 2u * s * kHSbo, kHSbo, kHLbo),
                   tc::smem_desc(smem_addr(sX) + 2u * s * kXSbo, kXSbo, kXLbo), id_n16, acc);
    }
    tc::commit(&S->bar);
  }
  mma_wait(&S->bar, phase, a.dev_status);
  // ---- this CTA's gradient partials.  M = 64 accumulators: row m lives in
  // lane 32 (m / 16) + m % 16.
  float* G = a.grad_partials + (size_t)blockIdx.x * kGradWidth;
  {
    float v[kH];
#pragma unroll
    for (int c = 0; c < kH; c += 16) tc::tmem_ld16(t_dw2 + lane_base + (uint32_t)c, v + c);
    float vb[16], vw1[16], vw3[16];
    tc::tmem_ld16(t_db2 + lane_base, vb);
    tc::tmem_ld16(t_dw1 + lane_base, vw1);
    tc::tmem_ld16(t_dw3 + lane_base, vw3);
    if (lane < 16) {
      const int m = 16 * warp + lane;
      float4* gw2 = reinterpret_cast<float4*>(G + kOffW2 + m * kH);
#pragma unroll
      for (int j = 0; j < kH / 4; ++j) gw2[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
      G[kOffB2 + m] = vb[0];
      G[kOffW3 + m] = vw3[0];
      float4* gw1 = reinterpret_cast<float4*>(G + kOffW1 + m * kIn);
      gw1[0] = make_float4(vw1[0], vw1[1], vw1[2], vw1[3]);
#pragma unroll
      for (int j = 1; j < kIn / 4; ++j) gw1[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  if (tid == 0) {
    float l = 0.f, cs = 0.f, b3 = 0.f;
    for (int w = 0; w < 4; ++w) {
      l += S->wloss[w];
      cs += S->wsum[w];
      b3 += S->wb3[w];
    }
    G[kOffB3] = b3;
    G[kOffC] = -2.f * cs * inv_B;
    G[kNumParams] = l * inv_B;
    G[kNumParams + 1] = 0.f;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tm, 128);
  }
}

// 128 TMEM columns and ~86 KB of shared memory per training CTA: two CTAs
// share an SM.
size_t train_smem_bytes() {
  return ((sizeof(TrainSmem) + 1023) & ~(size_t)1023) + kW2Bytes + kW1Bytes + kXBytes + 4 * kHBytes + 16 * 128 * 2;
}

// ---- Adam ------------------------------------------------------------------------------
// Block b owns parameters [32 b, 32 b + 32): thread (slice, lane) sums the
// partials slice, slice + 32, ... of parameter 32 b + lane in order, then the
// 32 slice sums are added in slice order (a fixed order for any launch).
constexpr int kAdamSlices = 32;
__global__ void __launch_bounds__(32 * kAdamSlices) mlp_adam_kernel(tqf_mlp_adam_args a) {
  __shared__ float part[kAdamSlices][33];
  const int lane = threadIdx.x & 31, slice = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  float g = 0.f;
  if (i <= kNumParams) {
    const float* src = a.grad_partials + i;
#pragma unroll 8
    for (int b = slice; b < a.num_partials; b += kAdamSlices) g += src[(size_t)b * kGradWidth];
  }
  part[slice][lane] = g;
  __syncthreads();
  if (slice != 0 || i > kNumParams) return;
  g = 0.f;
#pragma unroll
  for (int s2 = 0; s2 < kAdamSlices; ++s2) g += part[s2][lane];
  if (i == kNumParams) {
    if (a.loss_out) a.loss_out[0] = g;
    return;
  }
  if (i >= kOffW1 && i < kOffW2 && (i - kOffW1) % kIn >= 4) return;  // padded input columns stay zero
  float m = a.m[i] = a.beta1 * a.m[i] + (1.f - a.beta1) * g;
  float v = a.v[i] = a.beta2 * a.v[i] + (1.f - a.beta2) * g * g;
  const float mh = m / a.bias1, vh = v / a.bias2;
  const float p = a.params[i] - a.lr * mh / (sqrtf(vh) + a.eps);
  a.params[i] = p;
  uint16_t* w1b = static_cast<uint16_t*>(a.w1_bf16);
  uint16_t* w2b = static_cast<uint16_t*>(a.w2_bf16);
  __nv_bfloat16 pb = __float2bfloat16_rn(p);
  if (i < kOffW2) w1b[i - kOffW1] = *reinterpret_cast<uint16_t*>(&pb);
  else if (i < kOffB2) w2b[i - kOffW2] = *reinterpret_cast<uint16_t*>(&pb);
}

}  // namespace
}  // namespace tqf

using namespace tqf;

// Host-side round-to-nearest-even to BF16 (the device's __float2bfloat16_rn).
static float bf16_round_host(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7F800000u) != 0x7F800000u) u += 0x7FFFu + ((u >> 16) & 1u);
  u &= 0xFFFF0000u;
  float r;
  memcpy(&r, &u, 4);
  return r;
}

extern "C" size_t tqf_heston_asian_workspace_bytes(int32_t mode, int64_t num_paths, int32_t num_steps) {
  const size_t smem = asian_smem_bytes(mode, num_steps);
  int grid = mode == 2 ? asian_grid<2>(num_paths, smem) : asian_grid<0>(num_paths, smem);
  return (size_t)grid * 5 * sizeof(double);
}

extern "C" int tqf_heston_asian(const tqf_heston_asian_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_heston_asian: null args");
  TQF_REQUIRE(a->mode >= 0 && a->mode <= 2, "tqf_heston_asian: mode must be 0, 1 or 2");
  TQF_REQUIRE(a->num_paths >= 1 && a->num_steps >= 1 && a->num_steps <= 4096, "tqf_heston_asian: bad sizes");
  TQF_REQUIRE(a->num_dates >= 1 && a->num_dates <= kMaxDates, "tqf_heston_asian: num_dates must be in [1, %d]",
              kMaxDates);
  TQF_REQUIRE(a->step_table && a->date_table, "tqf_heston_asian: null table");
  TQF_REQUIRE((reinterpret_cast<uintptr_t>(a->step_table) & 15u) == 0, "tqf_heston_asian: step_table must be 16-byte aligned");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX && !a->draws.antithetic,
              "tqf_heston_asian: draws must be (non-antithetic) Philox");
  if (a->mode == 1)
    TQF_REQUIRE(a->pilot_feats && a->pilot_dS && a->pilot_Y, "tqf_heston_asian: pilot outputs required");
  if (a->mode == 2)
    TQF_REQUIRE(a->mlp.w2_bf16 && a->mlp.host, "tqf_heston_asian: network weights required (w2_bf16, host)");
  if (a->mode == 2)
    TQF_REQUIRE((reinterpret_cast<uintptr_t>(a->mlp.w2_bf16) & 15u) == 0, "tqf_heston_asian: w2_bf16 must be 16-byte aligned");
  const size_t smem = asian_smem_bytes(a->mode, a->num_steps);
  TQF_REQUIRE(smem <= 227 * 1024, "tqf_heston_asian: step table too large for shared memory");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int grid;
  if (a->mode == 0) grid = asian_grid<0>(a->num_paths, smem);
  else if (a->mode == 1) grid = asian_grid<1>(a->num_paths, smem);
  else grid = asian_grid<2>(a->num_paths, smem);
  if (a->mode != 1) {
    const size_t need = (size_t)grid * 5 * sizeof(double);
    TQF_REQUIRE(a->out && a->workspace && a->workspace_bytes >= need, "tqf_heston_asian: workspace %zu < %zu",
                a->workspace_bytes, need);
  }
  MlpConst wc;
  memset(&wc, 0, sizeof(wc));
  if (a->mode == 2) {
    const tqf_mlp_host_weights* h = a->mlp.host;
    for (int j = 0; j < kH; ++j) {
      // layer-1 weights and bias as the BF16 values the training kernels use
      wc.l1[j] = make_float4(bf16_round_host(h->w1[j][0]), bf16_round_host(h->w1[j][1]),
                             bf16_round_host(h->w1[j][2]), bf16_round_host(h->w1[j][3]));
      wc.b2[j] = h->b2[j];
      wc.w3[j] = h->w3[j];
    }
    wc.b3 = h->b3;
    for (int j = 0; j < 3; ++j) {
      wc.fscale[j] = a->mlp.feat_scale[j];
      wc.fshift[j] = a->mlp.feat_shift[j];
    }
  }
  if (a->mode == 0) heston_asian_kernel<0><<<grid, kPathThreads, smem, s>>>(*a, wc);
  else if (a->mode == 1) heston_asian_kernel<1><<<grid, kPathThreads, smem, s>>>(*a, wc);
  else heston_asian_kernel<2><<<grid, kPathThreads, smem, s>>>(*a, wc);
  int rc = check_launch("heston_asian_kernel");
  if (rc || a->mode == 1) return rc;
  return reduce_partials(static_cast<const double*>(a->workspace), grid, 5, a->out, s);
}

extern "C" int tqf_heston_asian_occupancy(int32_t mode, int32_t num_steps) {
  clear_error();
  const size_t smem = asian_smem_bytes(mode, num_steps);
  int occ = -1;
  cudaError_t e;
  if (mode == 2) {
    set_smem_config(heston_asian_kernel<2>, smem);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, heston_asian_kernel<2>, kPathThreads, smem);
  } else {
    set_smem_config(heston_asian_kernel<0>, smem);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, heston_asian_kernel<0>, kPathThreads, smem);
  }
  if (e != cudaSuccess) return check_cuda(e, "tqf_heston_asian_occupancy");
  return occ;
}

extern "C" int tqf_mlp_num_params(void) { return kNumParams; }

extern "C" int tqf_mlp_train_step(const tqf_mlp_train_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_mlp_train_step: null args");
  TQF_REQUIRE(a->num_dates >= 1 && a->num_dates <= kMaxDates, "tqf_mlp_train_step: bad num_dates");
  TQF_REQUIRE(a->paths_per_cta >= 1 && a->paths_per_cta * a->num_dates <= 128,
              "tqf_mlp_train_step: paths_per_cta x num_dates must be in [1, 128]");
  TQF_REQUIRE(a->batch_paths >= a->paths_per_cta && a->batch_paths % a->paths_per_cta == 0,
              "tqf_mlp_train_step: batch_paths must be a positive multiple of paths_per_cta");
  TQF_REQUIRE(a->feats && a->dS && a->Y && a->params && a->w1_bf16 && a->w2_bf16 && a->grad_partials,
              "tqf_mlp_train_step: null pointer");
  TQF_REQUIRE((reinterpret_cast<uintptr_t>(a->feats) & 15u) == 0 && (reinterpret_cast<uintptr_t>(a->w2_bf16) & 15u) == 0 &&
                  (reinterpret_cast<uintptr_t>(a->grad_partials) & 15u) == 0 &&
                  (reinterpret_cast<uintptr_t>(a->w1_bf16) & 7u) == 0,
              "tqf_mlp_train_step: feats, w2_bf16 and grad_partials must be 16-byte aligned, w1_bf16 8-byte aligned");
  const int grid = a->batch_paths / a->paths_per_cta;
  const size_t smem = train_smem_bytes();
  set_smem_config(mlp_train_step_kernel, smem);
  mlp_train_step_kernel<<<grid, kTrainThreads, smem, static_cast<cudaStream_t>(stream)>>>(*a);
  return check_launch("mlp_train_step_kernel");
}

extern "C" int tqf_mlp_adam(const tqf_mlp_adam_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a && a->params && a->m && a->v && a->grad_partials && a->w1_bf16 && a->w2_bf16,
              "tqf_mlp_adam: null pointer");
  TQF_REQUIRE(a->num_partials >= 1, "tqf_mlp_adam: num_partials must be >= 1");
  const int blocks = (kNumParams + 1 + 31) / 32;
  mlp_adam_kernel<<<blocks, 32 * kAdamSlices, 0, static_cast<cudaStream_t>(stream)>>>(*a);
  return check_launch("mlp_adam_kernel");
}
