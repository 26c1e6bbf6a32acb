// Neural martingale control variate for the Heston arithmetic-Asian option
// (no reference counterpart; the path it wraps is the reference Euler sampler
// with full-truncation Heston coefficients, tff/models/euler_sampling.py:513-537).
//
// Network g(t, log S, v): 3 -> 64 -> 64 -> 1, SiLU, BF16 weights and
// activations, FP32 accumulation.  Every layer runs on the tcgen05 tensor
// cores: a warpgroup's 128 rows (one per thread) form an M = 128 tile with
// the accumulator in TMEM.  Layer 1 is K = 16 (three features, a 1 for the
// bias in W1 column 3, zero padding); layer 3 has N = 16 (w3 split into BF16
// high and low rows).  SiLU runs in packed BF16 (one SFU tanh per pair).
// The backward GEMMs (Q2 W2, dW2, db2, dw3, dW1) are tcgen05 MMAs as well.
//
// heston_asian_kernel<MODE>: full-truncation Euler paths (Philox in-kernel),
//   num_dates monitoring dates marked in the step table's slot column; the
//   control dates are the monitoring dates the date table does not mark
//   "hold", and the last date.
//   MODE 0: plain estimator sums of Y = e^{-rT} max(mean_k S_k - K, 0).
//   MODE 1: pilot data — per path and control interval j the start features
//           (t_j, log S_j, v_j), the discounted-spot increment
//           dS~_j = e^{-r t_{j+1}} S_{j+1} - e^{-r t_j} S_j, and Y.
//   MODE 2: fused control variate C = sum_j g(t_j, X_j, V_j) dS~_j with the
//           network evaluated per warpgroup tile at every control interval
//           start (held over the monitoring dates in between).
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
constexpr int kCvCtasPerSm = 4;    // fused-inference CTAs per SM (4 x 128 TMEM columns = 512)
// Plain and pilot path kernels: register bound for 5 CTAs per SM (48
// registers; 4 and 6 measured within 1% of it).
constexpr int kPlainCtasPerSm = 5;
constexpr int kTrainThreads = 256;  // two threads per tile row
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

// The same SiLU from the halved pre-activations h = x/2 (the inference tiles
// hold W1, W2 and b2 scaled by 1/2, which is exact in BF16 and in the FP32
// accumulation, so bf16(x/2) = bf16(x)/2 bit for bit): one multiply fewer.
__device__ __forceinline__ uint32_t silu_half_bf16x2(float ha, float hb) {
  const uint32_t h2 = pack_bf16x2(ha, hb);
  uint32_t t2, s2;
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
  bool ok = mbar_wait_suspend(bar, phase);
  if (!ok) {
    if (status) atomicExch(status, TQF_E_TIMEOUT);
    ok = mbar_wait_suspend(bar, phase);
  }
  phase ^= 1u;
  tc::fence_after_sync();
  return ok;
}

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

// ---- fused inference: a three-stage tensor-core pipeline per warpgroup ---------
// One evaluation of g for the warpgroup's 128 paths (one row each) is
//   L1: a1 = X W1^T (X row = BF16 features, 1, 1; W1 column 3 = b1)
//   S1: H = SiLU(a1); a2 = H W2^T + X B2^T (B2 columns 3, 4 = b2 split into
//       BF16 high and low parts, so the bias is exact to ~2^-16)
//   S2: H = SiLU(a2); (g_hi, g_lo) = H W3^T (W3 rows 0, 1 = w3 high / low)
//   g = g_hi + g_lo + b3,
// each stage a wait on the previous MMAs, a TMEM read, packed-BF16 SiLU into
// the warpgroup's H tile and the next MMAs.  The path kernel runs S1 and S2
// at marked steps between two monitoring dates, so the tensor-core latency
// hides behind path stepping; at the date any stage still pending runs
// there.  TMEM: the warpgroup's 64 columns hold a1, then a2, then g.
constexpr uint32_t kW1Lbo = 1024, kW1Sbo = 128;  // W1, B2 [64 x 16] K-major
constexpr int kW1Bytes = kH * kIn * 2;
constexpr uint32_t kW3Lbo = 256, kW3Sbo = 128;   // W3 [16 x 64] K-major
constexpr int kW3Bytes = 16 * kH * 2;

struct EvalPipe {
  unsigned char* sX;  // [128 x 16] this warpgroup's inputs
  unsigned char* sH;  // [128 x 64] its hidden activations
  uint32_t tmem;      // its 64 TMEM columns
  uint64_t* bar;
  uint32_t phase;
  int stage;          // 0 idle, 1 L1 in flight, 2 layer 2 in flight, 3 layer 3 in flight
};

// Makes this warpgroup's shared-memory tile writes and TMEM reads visible to
// the MMAs that its thread 0 issues next.  (A variant in which warps 1-3
// only arrive on the named barrier measured ~1% slower.)
__device__ __forceinline__ void wg_publish(int wg, int tid) {
  (void)tid;
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  wg_sync(wg);
  tc::fence_after_sync();
}

// 16 FP32 TMEM columns of this thread's lane, without the wait.
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// SiLU of this row's 64 TMEM accumulators (halved pre-activations, packed
// BF16) into row r of sH, 16 columns per TMEM round trip (fewer live
// registers than 32 at a time, which measured faster at this kernel's
// 64-register budget).
__device__ __forceinline__ void silu_row_from_tmem(uint32_t taddr, unsigned char* sH, int r) {
#pragma unroll
  for (int c = 0; c < kH; c += 16) {
    uint32_t u[16];
    tmem_ld16_nowait(taddr + (uint32_t)c, u);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    float acc[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j] = __uint_as_float(u[j]);
#pragma unroll
    for (int h = 0; h < 16; h += 8)
      *reinterpret_cast<uint4*>(sH + tc::kmajor_off(r, c + h, kHLbo, kHSbo)) =
          make_uint4(silu_half_bf16x2(acc[h], acc[h + 1]), silu_half_bf16x2(acc[h + 2], acc[h + 3]),
                     silu_half_bf16x2(acc[h + 4], acc[h + 5]), silu_half_bf16x2(acc[h + 6], acc[h + 7]));
  }
}

__device__ __forceinline__ void eval_issue_l1(int wg, int tid, const MlpConst& wc, EvalPipe& P,
                                              const unsigned char* sW1, float t, float x, float v) {
  float f0, f1, f2;
  features(wc, t, x, v, f0, f1, f2);
  *reinterpret_cast<uint4*>(P.sX + tc::kmajor_off(tid, 0, kXLbo, kXSbo)) =
      make_uint4(pack_bf16x2(f0, f1), pack_bf16x2(f2, 1.f), pack_bf16x2(1.f, 0.f), 0u);
  wg_publish(wg, tid);
  if (tid == 0) {
    tc::mma_bf16(P.tmem, tc::smem_desc(smem_addr(P.sX), kXLbo, kXSbo), tc::smem_desc(smem_addr(sW1), kW1Lbo, kW1Sbo),
                 tc::idesc_bf16(128, kH, false, false), 0u);
    tc::commit(P.bar);
  }
  P.stage = 1;
}

__device__ __forceinline__ void eval_stage1(int wg, int tid, EvalPipe& P, const unsigned char* sW2,
                                            const unsigned char* sB2, int32_t* status) {
  mma_wait(P.bar, P.phase, status);
  silu_row_from_tmem(P.tmem + ((uint32_t)(32 * (tid >> 5)) << 16), P.sH, tid);
  wg_publish(wg, tid);
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, kH, false, false);
#pragma unroll
    for (int s = 0; s < kH / 16; ++s)
      tc::mma_bf16(P.tmem, tc::smem_desc(smem_addr(P.sH) + 2u * s * kHLbo, kHLbo, kHSbo),
                   tc::smem_desc(smem_addr(sW2) + 2u * s * kW2Lbo, kW2Lbo, kW2Sbo), idesc, s > 0 ? 1u : 0u);
    tc::mma_bf16(P.tmem, tc::smem_desc(smem_addr(P.sX), kXLbo, kXSbo), tc::smem_desc(smem_addr(sB2), kW1Lbo, kW1Sbo),
                 idesc, 1u);
    tc::commit(P.bar);
  }
  P.stage = 2;
}

__device__ __forceinline__ void eval_stage2(int wg, int tid, EvalPipe& P, const unsigned char* sW3, int32_t* status) {
  mma_wait(P.bar, P.phase, status);
  silu_row_from_tmem(P.tmem + ((uint32_t)(32 * (tid >> 5)) << 16), P.sH, tid);
  wg_publish(wg, tid);
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, 16, false, false);
#pragma unroll
    for (int s = 0; s < kH / 16; ++s)
      tc::mma_bf16(P.tmem, tc::smem_desc(smem_addr(P.sH) + 2u * s * kHLbo, kHLbo, kHSbo),
                   tc::smem_desc(smem_addr(sW3) + 2u * s * kW3Lbo, kW3Lbo, kW3Sbo), idesc, s > 0 ? 1u : 0u);
    tc::commit(P.bar);
  }
  P.stage = 3;
}

__device__ __forceinline__ float eval_finish(int wg, int tid, const MlpConst& wc, EvalPipe& P,
                                             const unsigned char* sW2, const unsigned char* sB2,
                                             const unsigned char* sW3, int32_t* status) {
  if (P.stage == 1) eval_stage1(wg, tid, P, sW2, sB2, status);
  if (P.stage == 2) eval_stage2(wg, tid, P, sW3, status);
  mma_wait(P.bar, P.phase, status);
  uint32_t r0, r1;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];"
               : "=r"(r0), "=r"(r1)
               : "r"(P.tmem + ((uint32_t)(32 * (tid >> 5)) << 16)));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  P.stage = 0;
  return __uint_as_float(r0) + __uint_as_float(r1) + wc.b3;
}

// Weight tiles of the inference pipeline from the constant-bank copy; W1
// (with b1) and b2 halved, so that layers 1 and 2 produce x/2 for the SiLU.
__device__ __forceinline__ void build_eval_tiles(const MlpConst& wc, unsigned char* sW1, unsigned char* sB2,
                                                 unsigned char* sW3) {
  for (int i = threadIdx.x; i < kH * kIn; i += blockDim.x) {
    const int n = i >> 4, k = i & 15;
    const float4 l = wc.l1[n];
    const float w = 0.5f * (k == 0 ? l.x : k == 1 ? l.y : k == 2 ? l.z : k == 3 ? l.w : 0.f);
    const float hi = round_bf16(wc.b2[n]);
    const float b = 0.5f * (k == 3 ? hi : k == 4 ? wc.b2[n] - hi : 0.f);
    __nv_bfloat16 wb = __float2bfloat16_rn(w), bb = __float2bfloat16_rn(b);
    *reinterpret_cast<__nv_bfloat16*>(sW1 + tc::kmajor_off(n, k, kW1Lbo, kW1Sbo)) = wb;
    *reinterpret_cast<__nv_bfloat16*>(sB2 + tc::kmajor_off(n, k, kW1Lbo, kW1Sbo)) = bb;
  }
  for (int i = threadIdx.x; i < 16 * kH; i += blockDim.x) {
    const int n = i / kH, k = i % kH;
    const float hi = round_bf16(wc.w3[k]);
    const float w = n == 0 ? hi : n == 1 ? wc.w3[k] - hi : 0.f;
    *reinterpret_cast<__nv_bfloat16*>(sW3 + tc::kmajor_off(n, k, kW3Lbo, kW3Sbo)) = __float2bfloat16_rn(w);
  }
}

// ---- path kernel -----------------------------------------------------------------
struct AsianSmem {
  uint64_t bar[2];
  uint32_t tmem_slot;
  uint32_t pad;
  double acc[kPathThreads / 32][5];
  float date_t[kMaxDates], date_disc[kMaxDates];
  int date_cv[kMaxDates];  // control interval ending at date k, or -1 (held)
  int num_cv;              // control dates
};

// Mode 2 pipelines the network with the simulation: the evaluation for
// interval k starts (layer 1) at its start date, advances one stage at each
// step the table marks with slot -2, and completes at its end date.  Mode 2
// reads the step table from global memory (L1-resident) so that its shared
// memory stays under a quarter of the SM's.
template <int MODE>
__global__ void __launch_bounds__(kPathThreads, MODE == 2 ? kCvCtasPerSm : kPlainCtasPerSm)
    heston_asian_kernel(tqf_heston_asian_args a, const __grid_constant__ MlpConst wc,
                        const float4* __restrict__ pair_table) {
  extern __shared__ __align__(1024) unsigned char smem[];
  AsianSmem* S = reinterpret_cast<AsianSmem*>(smem);
  unsigned char* tiles = smem + ((sizeof(AsianSmem) + 1023) & ~(size_t)1023);
  unsigned char* sW2 = tiles;
  unsigned char* sW1 = sW2 + kW2Bytes;
  unsigned char* sB2 = sW1 + kW1Bytes;
  unsigned char* sW3 = sB2 + kW1Bytes;
  unsigned char* sWg = sW3 + kW3Bytes;  // per warpgroup: X [128 x 16], H [128 x 64]
  float* table = reinterpret_cast<float*>(tiles);  // modes 0, 1: two-step blocks (ft_pair_block)
  const int tid = threadIdx.x & 127, wg = threadIdx.x >> 7;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int D = a.num_dates;
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    S->date_t[i] = a.date_table[4 * i];
    S->date_disc[i] = a.date_table[4 * i + 1];
  }
  if (threadIdx.x == 0) {
    int j = 0;
    for (int k = 0; k < D; ++k) S->date_cv[k] = (k + 1 < D && a.date_table[4 * k + 2] != 0.f) ? -1 : j++;
    S->num_cv = j;
  }
  for (int i = threadIdx.x; i < (kPathThreads / 32) * 5; i += blockDim.x) (&S->acc[0][0])[i] = 0.0;
  if (MODE != 2)
    for (int p = threadIdx.x; p < (a.num_steps + 1) / 2; p += blockDim.x)
      ft_pair_block(a.step_table, a.num_steps, p, reinterpret_cast<float4*>(table) + 4 * p);
  EvalPipe P;
  if (MODE == 2) {
    const uint4* w2 = static_cast<const uint4*>(a.mlp.w2_bf16);
    for (int i = threadIdx.x; i < kH * kH / 8; i += blockDim.x) {
      const uint4 q = w2[i];  // halved (exact in BF16)
      *reinterpret_cast<uint4*>(sW2 + tc::kmajor_off(i >> 3, 8 * (i & 7), kW2Lbo, kW2Sbo)) =
          make_uint4(bf2_mul(q.x, kBf2Half), bf2_mul(q.y, kBf2Half), bf2_mul(q.z, kBf2Half), bf2_mul(q.w, kBf2Half));
    }
    build_eval_tiles(wc, sW1, sB2, sW3);
    for (int i = threadIdx.x; i < 2 * (kXBytes + kHBytes) / 16; i += blockDim.x)
      reinterpret_cast<uint4*>(sWg)[i] = make_uint4(0u, 0u, 0u, 0u);
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
  if (MODE == 2) {
    P.sX = sWg + wg * (kXBytes + kHBytes);
    P.sH = P.sX + kXBytes;
    P.tmem = S->tmem_slot + (uint32_t)(wg * kH);
    P.bar = &S->bar[wg];
    P.phase = 0;
    P.stage = 0;
  }
  // two-step blocks: mode 2 from global memory (L1-resident), modes 0, 1 from shared memory
  const float4* tp = MODE == 2 ? pair_table : reinterpret_cast<const float4*>(table);
  const float K = (float)a.strike, discT = (float)a.discount_T, x0 = (float)a.x0, v0 = (float)a.v0;
  const float S0 = __expf(x0);
  const float inv_D = 1.f / (float)D;
  const int Dc = S->num_cv;
  const int64_t N = a.num_paths;
  const int64_t per_round = (int64_t)gridDim.x * kPathThreads;
  for (int64_t base = 0; base < N; base += per_round) {
    const int64_t path = base + (int64_t)blockIdx.x * kPathThreads + threadIdx.x;
    const bool valid = path < N;
    const int64_t p = (valid ? path : 0) + a.draws.path_offset;
    const uint32_t plo = (uint32_t)p, phi = (uint32_t)((uint64_t)p >> 32);
    float x = x0, v = v0, avg = 0.f, cv = 0.f, prev = S0;
    if (MODE == 2) eval_issue_l1(wg, tid, wc, P, sW1, 0.f, x0, v0);
    if (MODE == 1 && valid) reinterpret_cast<float4*>(a.pilot_feats)[path] = make_float4(0.f, x0, v0, 0.f);
    // after each step: k = its slot (date index, -1, or -2 for a pipeline
    // stage; uniform across the CTA)
    auto after_step = [&](int k) {
      if (MODE == 2 && k == -2) {
        if (P.stage == 1) eval_stage1(wg, tid, P, sW2, sB2, a.dev_status);
        else if (P.stage == 2) eval_stage2(wg, tid, P, sW3, a.dev_status);
      }
      if (k >= 0) {
        const float Sk = __expf(x);
        avg += Sk;
        const int j = MODE == 0 ? -1 : S->date_cv[k];
        if (j >= 0) {
          const float dsk = S->date_disc[k] * Sk - prev;
          if (MODE == 2) {
            const float g = eval_finish(wg, tid, wc, P, sW2, sB2, sW3, a.dev_status);
            cv = fmaf(g, dsk, cv);
          }
          if (MODE == 1 && valid) {
            a.pilot_dS[j * N + path] = dsk;
            if (j + 1 < Dc)
              reinterpret_cast<float4*>(a.pilot_feats)[(j + 1) * N + path] = make_float4(S->date_t[k], x, v, 0.f);
          }
          prev = S->date_disc[k] * Sk;
          if (MODE == 2 && j + 1 < Dc) eval_issue_l1(wg, tid, wc, P, sW1, S->date_t[k], x, v);
        }
      }
    };
    // steps 2 pb and 2 pb + 1 from Philox block pb, in f32x2 pairs
    auto two_steps = [&](int pb, bool both) {
      const uint4 r = philox4x32_10(make_uint4((uint32_t)pb, plo, phi, 0u), a.draws.key0, a.draws.key1);
      float2 ze, zo;
      box_muller_pair_f32(r, ze, zo);
      const float4 qa = MODE == 2 ? __ldg(tp + 4 * pb) : tp[4 * pb];
      const float4 qs = MODE == 2 ? __ldg(tp + 4 * pb + 2) : tp[4 * pb + 2];
      const float4 qx = MODE == 2 ? __ldg(tp + 4 * pb + 3) : tp[4 * pb + 3];
      float2 dw0, e;
      ft_pair_increments(ze, zo, qs, qx, dw0, e);
      ft_half_step(qa, dw0.x, e.x, x, v);
      after_step((int)qx.z);
      if (both) {
        const float4 qb = MODE == 2 ? __ldg(tp + 4 * pb + 1) : tp[4 * pb + 1];
        ft_half_step(qb, dw0.y, e.y, x, v);
        after_step((int)qx.w);
      }
    };
    if constexpr (MODE != 2) {
      const int full = a.num_steps >> 1;
#pragma unroll 1
      for (int pb = 0; pb < full; ++pb) two_steps(pb, true);
      if (a.num_steps & 1) two_steps(full, false);
    } else {
      // one step per iteration (a single copy of the network stages in the
      // loop body), the block's normals and increments taken at even steps
      float2 dw0 = make_float2(0.f, 0.f), e = make_float2(0.f, 0.f);
      float2 slots = make_float2(-1.f, -1.f);
      for (int i = 0; i < a.num_steps; ++i) {
        const int pb = i >> 1;
        const bool odd = (i & 1) != 0;
        if (!odd) {
          const uint4 r = philox4x32_10(make_uint4((uint32_t)pb, plo, phi, 0u), a.draws.key0, a.draws.key1);
          float2 ze, zo;
          box_muller_pair_f32(r, ze, zo);
          const float4 qx = __ldg(tp + 4 * pb + 3);
          ft_pair_increments(ze, zo, __ldg(tp + 4 * pb + 2), qx, dw0, e);
          slots = make_float2(qx.z, qx.w);
        }
        ft_half_step(__ldg(tp + 4 * pb + (odd ? 1 : 0)), odd ? dw0.y : dw0.x, odd ? e.y : e.x, x, v);
        after_step((int)(odd ? slots.y : slots.x));
      }
    }
    const float Y = discT * fmaxf(avg * inv_D - K, 0.f);
    if (MODE == 1) {
      if (valid) a.pilot_Y[path] = Y;
    } else {
      if (a.path_values != nullptr && valid) reinterpret_cast<float2*>(a.path_values)[path] = make_float2(Y, cv);
      float q[5];
      q[0] = valid ? Y : 0.f;
      q[1] = q[0] * q[0];
      q[2] = valid ? cv : 0.f;
      q[3] = q[2] * q[2];
      q[4] = q[0] * q[2];
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        float sum = q[j];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
        if (lane == 0) S->acc[warp][j] += (double)sum;
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (MODE != 1 && threadIdx.x < 5) {
    double sum = 0.0;
    for (int w = 0; w < kPathThreads / 32; ++w) sum += S->acc[w][threadIdx.x];
    static_cast<double*>(a.workspace)[(size_t)blockIdx.x * 5 + threadIdx.x] = sum;
  }
  if (MODE == 2 && warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(S->tmem_slot, 128);
  }
}

// Mode 2 holds the weight tiles (14 KB) and per warpgroup an X and an H tile
// (20 KB): with 128 TMEM columns per CTA, four CTAs share an SM.
size_t asian_smem_bytes(int mode, int steps) {
  const size_t head = (sizeof(AsianSmem) + 1023) & ~(size_t)1023;
  if (mode == 2) return head + kW2Bytes + 2 * kW1Bytes + kW3Bytes + 2 * (kXBytes + kHBytes);
  return head + (size_t)((steps + 1) & ~1) * 8 * sizeof(float);
}

// Mode 2 reads the step table as two-step blocks from global memory: this
// kernel writes them into the caller's workspace, after the partial sums.
__global__ void ft_pair_table_kernel(const float* __restrict__ rows, int steps, float4* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < (steps + 1) / 2) ft_pair_block(rows, steps, p, out + 4 * p);
}

size_t asian_partials_bytes(int grid) { return ((size_t)grid * 5 * sizeof(double) + 15) & ~(size_t)15; }
size_t asian_pair_table_bytes(int steps) { return (size_t)((steps + 1) / 2) * 16 * sizeof(float); }

template <int MODE>
int asian_grid(int64_t n, size_t smem) {
  auto k = heston_asian_kernel<MODE>;
  set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kPathThreads, smem) != cudaSuccess || occ < 1) occ = 1;
  // The runtime's occupancy calculation admits one CTA per SM for any kernel
  // that allocates TMEM (a query-only probe shows it for a trivial kernel),
  // although this one's registers (64), shared memory and barriers allow
  // four (ncu: all limits 4, four resident); size the persistent grid for
  // four, the most whose 128 TMEM columns fit the SM's 512.
  if (MODE == 2) occ = kCvCtasPerSm;
  int64_t g = (n + kPathThreads - 1) / kPathThreads;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

// ---- training step ---------------------------------------------------------------------
// One CTA = one 128-row tile holding all num_dates rows of paths_per_cta
// paths (paths_per_cta x num_dates <= 128), so the forward pass runs once and
// the per-path residual never crosses CTAs.  Two threads share a row: warp w
// reads TMEM lanes 32 (w % 4) .. + 31 and owns hidden columns
// 32 (w / 4) .. + 31.  With q2 = w3 (.) SiLU'(a2) (known after the forward
// pass) and the per-row output gradient d3 = -2 r_p dS_pk / B (known after
// the residual):
//   d2 = d3 q2,  d1 = d3 (Q2 W2) (.) SiLU'(a1),
//   dW2 = Q2^T (d3 H1),  db2 = Q2^T d3,  dw3 = H2^T d3,  dW1 = D1^T X,
// so the Q2 W2 product is issued before the residual is known and overlaps
// it.  Layer 1 runs on the tensor cores here (X [128 x 16] x W1^T, bias in
// input column 3) and its pre-activations stay in TMEM for the backward
// pass.  The backward elementwise work (SiLU', the d3 scaling) runs in
// packed BF16, two values per instruction; its operands are BF16 anyway.
// TMEM (128 columns): [64, 128) a1, then dW2; [0, 64) the layer-2
// accumulator, then Q2 W2, then db2 | dw3 | dW1 (16 columns each).
struct TrainSmem {
  uint64_t bar;
  uint32_t tmem_slot;
  uint32_t pad;
  float b2[kH];
  float w3[kH];
  uint32_t w3p[kH / 2];  // w3 as BF16 pairs
  float b3, c;
  float gpart[2][128];  // layer-3 partial sums of the two column halves
  float ds[128];        // dS~ per row
  float resid[128];     // per path
  float Y[128];         // per path
  float wloss[8], wsum[8], wb3[4];
};

// One training step's gradient for this CTA's tile: loads the pilot rows
// and the current parameters, runs the forward and backward passes and
// writes the CTA's gradient partials.  TMEM (128 columns), the MMA barrier
// and the zeroed d3 tile are set up by the caller; `phase` is the MMA
// barrier's parity, carried across calls.
__device__ __forceinline__ void train_tile(const tqf_mlp_train_args& a, unsigned char* smem, uint32_t tm,
                                           uint32_t& phase, bool dependent_launch, int tile, int tid) {
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
  const int warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3, half = warp >> 2;
  const int64_t p0 = a.path_begin + (int64_t)tile * P;
  const float inv_B = 1.f / (float)a.batch_paths;
  // independent of the previous step: the pilot rows
  if (tid < P) S->Y[tid] = a.Y[p0 + tid];
  const int r = 32 * quarter + lane;
  const int c0 = 32 * half;  // first hidden column of this thread
  const bool in = r < rows;
  const int pl = in ? r / D : 0, dd = in ? r % D : 0;
  const int64_t gi = (int64_t)dd * a.pilot_paths + p0 + pl;
  const float dsv = in ? a.dS[gi] : 0.f;
  const float4 f = (in && half == 0) ? reinterpret_cast<const float4*>(a.feats)[gi] : make_float4(0.f, 0.f, 0.f, 0.f);
  // the parameters (and the gradient buffer) belong to the previous step until it completes
  if (dependent_launch) grid_dependency_wait();
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
  if (tid == 0) {
    S->b3 = Pm[kOffB3];
    S->c = Pm[kOffC];
  }
  if (half == 0) {
    // X row = (BF16 features, 1, 0, ...)
    S->ds[r] = dsv;
    const float f0 = round_bf16((f.x - a.feat_shift[0]) * a.feat_scale[0]);
    const float f1 = round_bf16((f.y - a.feat_shift[1]) * a.feat_scale[1]);
    const float f2 = round_bf16((f.z - a.feat_shift[2]) * a.feat_scale[2]);
    *reinterpret_cast<uint4*>(sX + tc::kmajor_off(r, 0, kXLbo, kXSbo)) =
        make_uint4(pack_bf16x2(f0, f1), pack_bf16x2(f2, 1.f), 0u, 0u);
    *reinterpret_cast<uint4*>(sX + tc::kmajor_off(r, 8, kXLbo, kXSbo)) = make_uint4(0u, 0u, 0u, 0u);
  }
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t t_fwd = tm, t_a1 = tm + 64, t_db2 = tm, t_dw3 = tm + 16, t_dw1 = tm + 32, t_dw2 = tm + 64;
  const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
  // ---- forward.  Layer 1 -> a1 in TMEM
  if (tid == 0) {
    tc::mma_bf16(t_a1, tc::smem_desc(smem_addr(sX), kXLbo, kXSbo), tc::smem_desc(smem_addr(sW1), kW1Lbo, kW1Sbo),
                 tc::idesc_bf16(128, kH, false, false), 0u);
    tc::commit(&S->bar);
  }
  mma_wait(&S->bar, phase, a.dev_status);
  {
    uint32_t u[32];
    tmem_ld16_nowait(t_a1 + lane_base + (uint32_t)c0, u);
    tmem_ld16_nowait(t_a1 + lane_base + (uint32_t)c0 + 16u, u + 16);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int h = 0; h < 32; h += 8)
      *reinterpret_cast<uint4*>(sH + tc::kmajor_off(r, c0 + h, kHLbo, kHSbo)) =
          make_uint4(silu_bf16x2(__uint_as_float(u[h]), __uint_as_float(u[h + 1])),
                     silu_bf16x2(__uint_as_float(u[h + 2]), __uint_as_float(u[h + 3])),
                     silu_bf16x2(__uint_as_float(u[h + 4]), __uint_as_float(u[h + 5])),
                     silu_bf16x2(__uint_as_float(u[h + 6]), __uint_as_float(u[h + 7])));
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
  // bias, SiLU (H2), this half's layer-3 partial sum and q2 = w3 SiLU'(a2) (Q2)
  {
    const uint32_t keep = in ? 0xFFFFFFFFu : 0u;
    uint32_t u[32];
    tmem_ld16_nowait(t_fwd + lane_base + (uint32_t)c0, u);
    tmem_ld16_nowait(t_fwd + lane_base + (uint32_t)c0 + 16u, u + 16);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    float g = 0.f;
#pragma unroll
    for (int h = 0; h < 32; h += 8) {
      const int col = c0 + h;
      const float4 ba = *reinterpret_cast<const float4*>(&S->b2[col]);
      const float4 bb = *reinterpret_cast<const float4*>(&S->b2[col + 4]);
      const float4 wa = *reinterpret_cast<const float4*>(&S->w3[col]);
      const float4 wb = *reinterpret_cast<const float4*>(&S->w3[col + 4]);
      const uint4 wp = *reinterpret_cast<const uint4*>(&S->w3p[col / 2]);
      const float bias[8] = {ba.x, ba.y, ba.z, ba.w, bb.x, bb.y, bb.z, bb.w};
      const float w3v[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
      const uint32_t w3pv[4] = {wp.x, wp.y, wp.z, wp.w};
      uint32_t hp[4], qp[4];
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        const float aa = __uint_as_float(u[h + j]) + bias[j], ab = __uint_as_float(u[h + j + 1]) + bias[j + 1];
        const uint32_t sp = silu_bf16x2(aa, ab);
        g = fmaf(w3v[j], bf16_lo(sp), fmaf(w3v[j + 1], bf16_hi(sp), g));
        hp[j >> 1] = sp;
        qp[j >> 1] = bf2_mul(w3pv[j >> 1], dsilu_bf16x2(pack_bf16x2(aa, ab))) & keep;
      }
      *reinterpret_cast<uint4*>(sH2 + tc::kmajor_off(r, col, kHLbo, kHSbo)) = make_uint4(hp[0], hp[1], hp[2], hp[3]);
      *reinterpret_cast<uint4*>(sQ2 + tc::kmajor_off(r, col, kHLbo, kHSbo)) = make_uint4(qp[0], qp[1], qp[2], qp[3]);
    }
    S->gpart[half][r] = g;
  }
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
    const float b3 = S->b3;
    float wl = 0.f, ws = 0.f;
    for (int p = warp; p < P; p += kTrainThreads / 32) {
      float sum = 0.f;
      for (int k = lane; k < D; k += 32) {
        const int row = p * D + k;
        sum = fmaf((S->gpart[0][row] + S->gpart[1][row]) + b3, S->ds[row], sum);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
      const float rr = S->Y[p] - S->c - sum;
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
  if (half == 0) {
    float b3p = d3;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) b3p += __shfl_xor_sync(0xffffffffu, b3p, off);
    if (lane == 0) S->wb3[quarter] = b3p;
    *reinterpret_cast<uint4*>(sT3 + tc::mnmajor_off(0, r, kOnesLbo, kOnesSbo)) =
        make_uint4(pack_bf16x2(d3, 0.f), 0u, 0u, 0u);
  }
  // this half of the H1 row scaled by d3 (the B operand of dW2)
  {
    const uint32_t d3p = pack_bf16x2(d3, d3);
#pragma unroll
    for (int jc = 0; jc < 4; ++jc) {
      uint4* line = reinterpret_cast<uint4*>(sH + tc::kmajor_off(r, c0 + 8 * jc, kHLbo, kHSbo));
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
  {
    uint32_t p2[32], a1[32];
    tmem_ld16_nowait(t_fwd + lane_base + (uint32_t)c0, p2);
    tmem_ld16_nowait(t_fwd + lane_base + (uint32_t)c0 + 16u, p2 + 16);
    tmem_ld16_nowait(t_a1 + lane_base + (uint32_t)c0, a1);
    tmem_ld16_nowait(t_a1 + lane_base + (uint32_t)c0 + 16u, a1 + 16);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int h = 0; h < 32; h += 8) {
      uint32_t dp[4];
#pragma unroll
      for (int j = 0; j < 8; j += 2)
        dp[j >> 1] = bf2_mul(pack_bf16x2(d3 * __uint_as_float(p2[h + j]), d3 * __uint_as_float(p2[h + j + 1])),
                             dsilu_bf16x2(pack_bf16x2(__uint_as_float(a1[h + j]), __uint_as_float(a1[h + j + 1]))));
      *reinterpret_cast<uint4*>(sD1 + tc::kmajor_off(r, c0 + h, kHLbo, kHSbo)) = make_uint4(dp[0], dp[1], dp[2], dp[3]);
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
  // lane 32 (m / 16) + m % 16; each half of the warps writes 32 columns of dW2.
  float* G = a.grad_partials + (size_t)tile * kGradWidth;
  {
    uint32_t v[32];
    tmem_ld16_nowait(t_dw2 + lane_base + (uint32_t)c0, v);
    tmem_ld16_nowait(t_dw2 + lane_base + (uint32_t)c0 + 16u, v + 16);
    uint32_t vb[16];
    tmem_ld16_nowait((half == 0 ? t_db2 : t_dw3) + lane_base, vb);
    uint32_t vw1[16];
    tmem_ld16_nowait(t_dw1 + lane_base, vw1);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (lane < 16) {
      const int m = 16 * quarter + lane;
      float4* gw2 = reinterpret_cast<float4*>(G + kOffW2 + m * kH + c0);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        gw2[j] = make_float4(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1]), __uint_as_float(v[4 * j + 2]),
                             __uint_as_float(v[4 * j + 3]));
      if (half == 0) {
        G[kOffB2 + m] = __uint_as_float(vb[0]);
        float4* gw1 = reinterpret_cast<float4*>(G + kOffW1 + m * kIn);
        gw1[0] = make_float4(__uint_as_float(vw1[0]), __uint_as_float(vw1[1]), __uint_as_float(vw1[2]),
                             __uint_as_float(vw1[3]));
#pragma unroll
        for (int j = 1; j < kIn / 4; ++j) gw1[j] = make_float4(0.f, 0.f, 0.f, 0.f);
      } else {
        G[kOffW3 + m] = __uint_as_float(vb[0]);
      }
    }
  }
  if (tid == 0) {
    float l = 0.f, cs = 0.f, b3 = 0.f;
    for (int w = 0; w < kTrainThreads / 32; ++w) {
      l += S->wloss[w];
      cs += S->wsum[w];
    }
    for (int w = 0; w < 4; ++w) b3 += S->wb3[w];
    G[kOffB3] = b3;
    G[kOffC] = -2.f * cs * inv_B;
    G[kNumParams] = l * inv_B;
    G[kNumParams + 1] = 0.f;
  }
}

// Shared memory of one tile's working set (train_tile): 128 TMEM columns and
// ~88 KB per training CTA, so two CTAs share an SM.
size_t __host__ __device__ train_smem_bytes() {
  return ((sizeof(TrainSmem) + 1023) & ~(size_t)1023) + kW2Bytes + kW1Bytes + kXBytes + 4 * kHBytes + 16 * 128 * 2;
}

// Sets up what train_tile expects for each of the CTA's `tiles` tiles: the
// MMA barrier and the zeroed d3 tile; TMEM (128 columns per tile) is
// allocated once, its base left in the first tile's slot.
__device__ __forceinline__ void train_setup(unsigned char* smem, int tiles) {
  const size_t stride = train_smem_bytes();
  for (int t = 0; t < tiles; ++t) {
    unsigned char* base = smem + t * stride;
    unsigned char* sT3 = base + ((sizeof(TrainSmem) + 1023) & ~(size_t)1023) + kW2Bytes + kW1Bytes + kXBytes + 4 * kHBytes;
    for (int i = threadIdx.x; i < 16 * 128 * 2 / 16; i += blockDim.x)
      reinterpret_cast<uint4*>(sT3)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x == 0) mbar_init(&reinterpret_cast<TrainSmem*>(base)->bar, 1);
  }
  if (threadIdx.x < 32) tc::tmem_alloc(&reinterpret_cast<TrainSmem*>(smem)->tmem_slot, 128u * (uint32_t)tiles);
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

__device__ __forceinline__ void train_teardown(unsigned char* smem, int tiles) {
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(reinterpret_cast<TrainSmem*>(smem)->tmem_slot, 128u * (uint32_t)tiles);
  }
}

__global__ void __launch_bounds__(kTrainThreads) mlp_train_step_kernel(tqf_mlp_train_args a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  allow_dependent_launch();
  train_setup(smem, 1);
  uint32_t phase = 0;
  train_tile(a, smem, reinterpret_cast<TrainSmem*>(smem)->tmem_slot, phase, true, (int)blockIdx.x, (int)threadIdx.x);
  train_teardown(smem, 1);
}

// ---- Adam ------------------------------------------------------------------------------
// Block b owns parameters [32 b, 32 b + 32): thread (slice, lane) sums the
// partials slice, slice + 32, ... of parameter 32 b + lane in order, then the
// 32 slice sums are added in slice order (a fixed order for any launch).
constexpr int kAdamSlices = 32;
__global__ void __launch_bounds__(32 * kAdamSlices) mlp_adam_kernel(tqf_mlp_adam_args a) {
  __shared__ float part[kAdamSlices][33];
  allow_dependent_launch();
  const int lane = threadIdx.x & 31, slice = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  // the moments and parameters are not written by the training step: read them early
  float m0 = 0.f, v0 = 0.f, p0 = 0.f;
  if (slice == 0 && i < kNumParams) {
    m0 = a.m[i];
    v0 = a.v[i];
    p0 = a.params[i];
  }
  grid_dependency_wait();  // the gradient partials of the training step
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
  float m = a.m[i] = a.beta1 * m0 + (1.f - a.beta1) * g;
  float v = a.v[i] = a.beta2 * v0 + (1.f - a.beta2) * g * g;
  const float mh = m / a.bias1, vh = v / a.bias2;
  const float p = p0 - a.lr * mh / (sqrtf(vh) + a.eps);
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
  return asian_partials_bytes(grid) + (mode == 2 ? asian_pair_table_bytes(num_steps) : 0);
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
  TQF_REQUIRE((reinterpret_cast<uintptr_t>(a->path_values) & 7u) == 0, "tqf_heston_asian: path_values must be 8-byte aligned");
  const size_t smem = asian_smem_bytes(a->mode, a->num_steps);
  TQF_REQUIRE(smem <= 227 * 1024, "tqf_heston_asian: step table too large for shared memory");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int grid;
  if (a->mode == 0) grid = asian_grid<0>(a->num_paths, smem);
  else if (a->mode == 1) grid = asian_grid<1>(a->num_paths, smem);
  else grid = asian_grid<2>(a->num_paths, smem);
  if (a->mode != 1) {
    const size_t need = asian_partials_bytes(grid) + (a->mode == 2 ? asian_pair_table_bytes(a->num_steps) : 0);
    TQF_REQUIRE(a->out && a->workspace && a->workspace_bytes >= need, "tqf_heston_asian: workspace %zu < %zu",
                a->workspace_bytes, need);
    TQF_REQUIRE((reinterpret_cast<uintptr_t>(a->workspace) & 15u) == 0, "tqf_heston_asian: workspace must be 16-byte aligned");
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
  if (a->mode == 0) {
    heston_asian_kernel<0><<<grid, kPathThreads, smem, s>>>(*a, wc, nullptr);
  } else if (a->mode == 1) {
    heston_asian_kernel<1><<<grid, kPathThreads, smem, s>>>(*a, wc, nullptr);
  } else {
    float4* pairs = reinterpret_cast<float4*>(static_cast<unsigned char*>(a->workspace) + asian_partials_bytes(grid));
    const int np = (a->num_steps + 1) / 2;
    ft_pair_table_kernel<<<(np + 127) / 128, 128, 0, s>>>(a->step_table, a->num_steps, pairs);
    int rc = check_launch("ft_pair_table_kernel");
    if (rc) return rc;
    heston_asian_kernel<2><<<grid, kPathThreads, smem, s>>>(*a, wc, pairs);
  }
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
  TQF_REQUIRE(a->path_begin >= 0 && a->path_begin + a->batch_paths <= a->pilot_paths,
              "tqf_mlp_train_step: minibatch [%lld, %lld) outside the %lld pilot paths", (long long)a->path_begin,
              (long long)(a->path_begin + a->batch_paths), (long long)a->pilot_paths);
  TQF_REQUIRE((reinterpret_cast<uintptr_t>(a->feats) & 15u) == 0 && (reinterpret_cast<uintptr_t>(a->w2_bf16) & 15u) == 0 &&
                  (reinterpret_cast<uintptr_t>(a->grad_partials) & 15u) == 0 &&
                  (reinterpret_cast<uintptr_t>(a->w1_bf16) & 7u) == 0,
              "tqf_mlp_train_step: feats, w2_bf16 and grad_partials must be 16-byte aligned, w1_bf16 8-byte aligned");
  const int grid = a->batch_paths / a->paths_per_cta;
  const size_t smem = train_smem_bytes();
  set_smem_config(mlp_train_step_kernel, smem);
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = pdl_config(dim3(grid), dim3(kTrainThreads), smem, static_cast<cudaStream_t>(stream), attr);
  cudaError_t e = cudaLaunchKernelEx(&cfg, mlp_train_step_kernel, *a);
  if (e != cudaSuccess) return check_cuda(e, "mlp_train_step_kernel");
  return check_launch("mlp_train_step_kernel");
}

extern "C" int tqf_mlp_adam(const tqf_mlp_adam_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a && a->params && a->m && a->v && a->grad_partials && a->w1_bf16 && a->w2_bf16,
              "tqf_mlp_adam: null pointer");
  TQF_REQUIRE(a->num_partials >= 1, "tqf_mlp_adam: num_partials must be >= 1");
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = pdl_config(dim3((kNumParams + 1 + 31) / 32), dim3(32 * kAdamSlices), 0,
                                      static_cast<cudaStream_t>(stream), attr);
  cudaError_t e = cudaLaunchKernelEx(&cfg, mlp_adam_kernel, *a);
  if (e != cudaSuccess) return check_cuda(e, "mlp_adam_kernel");
  return check_launch("mlp_adam_kernel");
}
