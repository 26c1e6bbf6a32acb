// Neural martingale control variate for the Heston arithmetic-Asian option
// (no reference counterpart; the path it wraps is the reference Euler sampler
// with full-truncation Heston coefficients, tff/models/euler_sampling.py:513-537).
//
// Network g(t, log S, v): 3 -> 64 -> 64 -> 1, SiLU, BF16 weights and
// activations, FP32 accumulation.  Layers 1 and 2 run on the tcgen05 tensor
// cores: a warpgroup's 128 rows (one per thread) form an M = 128 tile; the
// input row is [f0, f1, f2, 1, 0 ... 0] (K = 16, the 1 carries layer 1's
// bias in column 3 of W1); layer 3 is a 64-term FP32 dot product.
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
//   loss = mean_p (Y_p - c - sum_k g_pk dS~_pk)^2: per CTA 32 paths x
//   num_dates rows in 128-row tiles — forward on tensor cores, per-path
//   residuals, backward with dW2 = d2^T H1, db2 = d2^T 1, dW1 = d1^T X and
//   d1 = d2 W2 as tcgen05 MMAs accumulated in TMEM across tiles.
// mlp_adam_kernel: fixed-order reduction of the per-CTA gradients and the
//   Adam update of the FP32 master parameters and their BF16 copies.
#include <cuda_bf16.h>

#include "tqf_tc.cuh"

namespace tqf {
namespace {

constexpr int kH = 64;            // hidden width
constexpr int kIn = 16;           // padded input width (K of layer 1)
constexpr int kMaxDates = 64;
constexpr int kPathThreads = 256;  // two warpgroups
constexpr int kTrainThreads = 128;
constexpr int kTrainPaths = 32;    // paths per training CTA
// parameter vector layout (FP32 master copy)
constexpr int kOffW1 = 0;
constexpr int kOffW2 = kOffW1 + kH * kIn;   // 1024
constexpr int kOffB2 = kOffW2 + kH * kH;    // 5120
constexpr int kOffW3 = kOffB2 + kH;         // 5184
constexpr int kOffB3 = kOffW3 + kH;         // 5248
constexpr int kOffC = kOffB3 + 1;           // 5249
constexpr int kNumParams = kOffC + 1;       // 5250
constexpr int kGradWidth = kNumParams + 1;  // + loss sum

// canonical no-swizzle K-major tiles (byte strides)
constexpr uint32_t kXLbo = 128, kXSbo = 256;    // [128 x 16]
constexpr uint32_t kHLbo = 128, kHSbo = 1024;   // [128 x 64]
constexpr uint32_t kW1Lbo = 128, kW1Sbo = 256;  // [64 x 16]
constexpr uint32_t kW2Lbo = 128, kW2Sbo = 1024; // [64 x 64]
constexpr int kXBytes = 128 * kIn * 2;
constexpr int kHBytes = 128 * kH * 2;
constexpr int kW1Bytes = kH * kIn * 2;
constexpr int kW2Bytes = kH * kH * 2;

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// x * sigmoid(x) = h (1 + tanh h), h = x / 2
__device__ __forceinline__ float silu_fast(float x) {
  const float h = 0.5f * x;
  return fmaf(h, tanh_approx(h), h);
}
// d/dx [x sigmoid(x)] = s + x s (1 - s), s = (1 + tanh(x/2)) / 2
__device__ __forceinline__ float dsilu_fast(float x) {
  const float s = fmaf(0.5f, tanh_approx(0.5f * x), 0.5f);
  return fmaf(x * s, 1.f - s, s);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

// Writes 8*nlines values of row r of a K-major BF16 tile (16-byte lines).
__device__ __forceinline__ void write_row_kmajor(unsigned char* tile, int r, const float* v, int nlines,
                                                 uint32_t lbo, uint32_t sbo) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    if (j >= nlines) break;
    uint4 w;
    w.x = pack_bf16x2(v[8 * j + 0], v[8 * j + 1]);
    w.y = pack_bf16x2(v[8 * j + 2], v[8 * j + 3]);
    w.z = pack_bf16x2(v[8 * j + 4], v[8 * j + 5]);
    w.w = pack_bf16x2(v[8 * j + 6], v[8 * j + 7]);
    *reinterpret_cast<uint4*>(tile + tc::kmajor_off(r, 8 * j, lbo, sbo)) = w;
  }
}

__device__ __forceinline__ void wg_sync(int wg) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + wg), "r"(128) : "memory");
}

// Loads the BF16 weights (row-major [out][in] in global) into K-major tiles.
__device__ __forceinline__ void load_weight_tiles(unsigned char* sW1, unsigned char* sW2, const uint16_t* w1,
                                                  const uint16_t* w2) {
  for (int i = threadIdx.x; i < kH * kIn; i += blockDim.x)
    *reinterpret_cast<uint16_t*>(sW1 + tc::kmajor_off(i / kIn, i % kIn, kW1Lbo, kW1Sbo)) = w1[i];
  for (int i = threadIdx.x; i < kH * kH; i += blockDim.x)
    *reinterpret_cast<uint16_t*>(sW2 + tc::kmajor_off(i / kH, i % kH, kW2Lbo, kW2Sbo)) = w2[i];
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
  float b2[kH];
  float w3[kH];
  float b3;
  float fscale[3], fshift[3];
};

// One warpgroup evaluates g for its 128 rows (this thread: row `tid`).
// tmem_d: 64 FP32 columns owned by the warpgroup (layer 1 then layer 2).
__device__ __forceinline__ float mlp_forward_tile(int wg, int tid, unsigned char* sX, unsigned char* sH,
                                                  const unsigned char* sW1, const unsigned char* sW2,
                                                  const MlpScalars& ms, uint32_t tmem_d, uint64_t* bar,
                                                  uint32_t& phase, float f0, float f1, float f2,
                                                  int32_t* status, float* a1_out = nullptr,
                                                  float* a2_out = nullptr) {
  float xin[16];
  xin[0] = (f0 - ms.fshift[0]) * ms.fscale[0];
  xin[1] = (f1 - ms.fshift[1]) * ms.fscale[1];
  xin[2] = (f2 - ms.fshift[2]) * ms.fscale[2];
  xin[3] = 1.f;
#pragma unroll
  for (int j = 4; j < 16; ++j) xin[j] = 0.f;
  write_row_kmajor(sX, tid, xin, 2, kXLbo, kXSbo);
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  wg_sync(wg);
  tc::fence_after_sync();
  if (tid == 0) {
    tc::mma_bf16(tmem_d, tc::smem_desc(smem_addr(sX), kXLbo, kXSbo), tc::smem_desc(smem_addr(sW1), kW1Lbo, kW1Sbo),
                 tc::idesc_bf16(128, kH, false, false), 0u);
    tc::commit(bar);
  }
  mma_wait(bar, phase, status);
  const uint32_t lane_base = (uint32_t)(32 * ((tid >> 5) & 3)) << 16;
  float h[kH];
#pragma unroll
  for (int c = 0; c < kH; c += 16) tc::tmem_ld16(tmem_d + lane_base + (uint32_t)c, h + c);
#pragma unroll
  for (int j = 0; j < kH; ++j) {
    if (a1_out) a1_out[j] = h[j];
    h[j] = silu_fast(h[j]);
  }
  write_row_kmajor(sH, tid, h, 8, kHLbo, kHSbo);
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
  mma_wait(bar, phase, status);
#pragma unroll
  for (int c = 0; c < kH; c += 16) tc::tmem_ld16(tmem_d + lane_base + (uint32_t)c, h + c);
  float g = ms.b3;
#pragma unroll
  for (int j = 0; j < kH; ++j) {
    const float a2 = h[j] + ms.b2[j];
    if (a2_out) a2_out[j] = a2;
    g = fmaf(ms.w3[j], silu_fast(a2), g);
  }
  tc::fence_before_sync();  // the next MMA into tmem_d is ordered after these loads
  return g;
}

// ---- path kernel -----------------------------------------------------------------
struct AsianSmem {
  uint64_t bar[2];
  uint32_t tmem_slot;
  uint32_t pad;
  double acc[kPathThreads / 32][5];
  float date_t[kMaxDates], date_disc[kMaxDates];
  MlpScalars ms;
};

template <int MODE>
__global__ void __launch_bounds__(kPathThreads) heston_asian_kernel(tqf_heston_asian_args a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  AsianSmem* S = reinterpret_cast<AsianSmem*>(smem);
  unsigned char* tiles = smem + ((sizeof(AsianSmem) + 1023) & ~(size_t)1023);
  unsigned char* sW1 = tiles;
  unsigned char* sW2 = sW1 + kW1Bytes;
  unsigned char* sXw = sW2 + kW2Bytes;                 // 2 x [128 x 16]
  unsigned char* sHw = sXw + 2 * kXBytes;              // 2 x [128 x 64]
  // step table [steps][8] after the network tiles (mode 2) or right away
  float* table = reinterpret_cast<float*>(MODE == 2 ? sHw + 2 * kHBytes : tiles);
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
    load_weight_tiles(sW1, sW2, static_cast<const uint16_t*>(a.mlp.w1_bf16),
                      static_cast<const uint16_t*>(a.mlp.w2_bf16));
    for (int i = threadIdx.x; i < kH; i += blockDim.x) {
      S->ms.b2[i] = a.mlp.b2[i];
      S->ms.w3[i] = a.mlp.w3[i];
    }
    if (threadIdx.x == 0) {
      S->ms.b3 = a.mlp.b3[0];
      for (int j = 0; j < 3; ++j) {
        S->ms.fscale[j] = a.mlp.feat_scale[j];
        S->ms.fshift[j] = a.mlp.feat_shift[j];
      }
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
  unsigned char* sX = sXw + wg * kXBytes;
  unsigned char* sH = sHw + wg * kHBytes;
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
    float g = 0.f;
    if (MODE == 2) g = mlp_forward_tile(wg, tid, sX, sH, sW1, sW2, S->ms, tmem_d, &S->bar[wg], phase, 0.f, x0, v0,
                                        a.dev_status);
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
        if (MODE == 2) cv = fmaf(g, dsk, cv);
        if (MODE == 1 && valid) {
          a.pilot_dS[path * D + k] = dsk;
          if (k + 1 < D)
            reinterpret_cast<float4*>(a.pilot_feats)[path * D + k + 1] = make_float4(S->date_t[k], x, v, 0.f);
        }
        prev = S->date_disc[k] * Sk;
        if (MODE == 2 && k + 1 < D)
          g = mlp_forward_tile(wg, tid, sX, sH, sW1, sW2, S->ms, tmem_d, &S->bar[wg], phase, S->date_t[k], x, v,
                               a.dev_status);
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

// Mode 2 also holds the network tiles; its ~60 KB keeps at most 3 CTAs (3 x 128
// TMEM columns <= 512) on an SM, so no TMEM allocation ever has to wait.
size_t asian_smem_bytes(int mode, int steps) {
  const size_t head = (sizeof(AsianSmem) + 1023) & ~(size_t)1023;
  const size_t tiles = mode == 2 ? (size_t)kW1Bytes + kW2Bytes + 2 * kXBytes + 2 * kHBytes : 0;
  size_t total = head + tiles + (size_t)steps * 8 * sizeof(float);
  if (mode == 2 && total < 58 * 1024) total = 58 * 1024;
  return total;
}

template <int MODE>
int asian_grid(int64_t n, size_t smem) {
  auto k = heston_asian_kernel<MODE>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kPathThreads, smem) != cudaSuccess || occ < 1) occ = 1;
  if (MODE == 2 && occ > 4) occ = 4;  // 4 CTAs x 128 TMEM columns = the SM's 512
  int64_t g = (n + kPathThreads - 1) / kPathThreads;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

// ---- training step ---------------------------------------------------------------------
struct TrainSmem {
  uint64_t bar;
  uint32_t tmem_slot;
  uint32_t pad;
  MlpScalars ms;
  float c;
  float resid[kTrainPaths];
  float Y[kTrainPaths];
  float w3acc[4][kH];
  float b3acc[4];
  float lossacc;
  float cacc;
};

__global__ void __launch_bounds__(kTrainThreads) mlp_train_step_kernel(tqf_mlp_train_args a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  TrainSmem* S = reinterpret_cast<TrainSmem*>(smem);
  unsigned char* t0 = smem + ((sizeof(TrainSmem) + 1023) & ~(size_t)1023);
  unsigned char* sW1 = t0;
  unsigned char* sW2 = sW1 + kW1Bytes;
  unsigned char* sX = sW2 + kW2Bytes;
  unsigned char* sH = sX + kXBytes;
  unsigned char* sD2 = sH + kHBytes;
  unsigned char* sD1 = sD2 + kHBytes;
  unsigned char* sOnes = sD1 + kHBytes;              // [16 x 128] MN-major, all ones
  float* g_rows = reinterpret_cast<float*>(sOnes + 16 * 128 * 2);
  const int D = a.num_dates;
  const int rows = kTrainPaths * D;
  float* ds_rows = g_rows + rows;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t p0 = a.path_begin + (int64_t)blockIdx.x * kTrainPaths;
  const float inv_B = 1.f / (float)a.batch_paths;
  // weights (BF16 tiles) and scalars
  load_weight_tiles(sW1, sW2, static_cast<const uint16_t*>(a.w1_bf16), static_cast<const uint16_t*>(a.w2_bf16));
  const float* P = a.params;
  for (int i = tid; i < kH; i += kTrainThreads) {
    S->ms.b2[i] = P[kOffB2 + i];
    S->ms.w3[i] = P[kOffW3 + i];
    for (int w = 0; w < 4; ++w) S->w3acc[w][i] = 0.f;
  }
  for (int i = tid; i < 16 * 128; i += kTrainThreads)
    *reinterpret_cast<uint16_t*>(sOnes + 2 * i) = (uint16_t)0x3F80u;  // bf16 1.0 everywhere
  if (tid < kTrainPaths) S->Y[tid] = a.Y[p0 + tid];
  if (tid == 0) {
    S->ms.b3 = P[kOffB3];
    S->c = P[kOffC];
    for (int j = 0; j < 3; ++j) {
      S->ms.fscale[j] = a.feat_scale[j];
      S->ms.fshift[j] = a.feat_shift[j];
    }
    for (int w = 0; w < 4; ++w) S->b3acc[w] = 0.f;
    S->lossacc = 0.f;
    S->cacc = 0.f;
    mbar_init(&S->bar, 1);
  }
  if (warp == 0) tc::tmem_alloc(&S->tmem_slot, 512);
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = S->tmem_slot;
  const uint32_t t_d1 = tm, t_d2 = tm + 64, t_d3 = tm + 128, t_dw2 = tm + 192, t_db2 = tm + 256, t_dw1 = tm + 272;
  uint32_t phase = 0;
  const int tiles = (rows + 127) / 128;
  const float4* feats = reinterpret_cast<const float4*>(a.feats);
  // ---- phase A: forward over every row, keep g
  for (int t = 0; t < tiles; ++t) {
    const int r = t * 128 + tid;
    const bool in = r < rows;
    const int pl = in ? r / D : 0, d = in ? r % D : 0;
    const float4 f = in ? feats[(p0 + pl) * D + d] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float gg = mlp_forward_tile(0, tid, sX, sH, sW1, sW2, S->ms, t_d1, &S->bar, phase, f.x, f.y, f.z,
                                      a.dev_status);
    if (in) {
      g_rows[r] = gg;
      ds_rows[r] = a.dS[(p0 + pl) * D + d];
    }
  }
  __syncthreads();
  // ---- phase B: per-path residuals r_p = Y_p - c - sum_k g_pk dS_pk
  if (tid < kTrainPaths) {
    float s = 0.f;
    for (int d = 0; d < D; ++d) s = fmaf(g_rows[tid * D + d], ds_rows[tid * D + d], s);
    S->resid[tid] = S->Y[tid] - S->c - s;
  }
  __syncthreads();
  if (warp == 0) {
    float rr = S->resid[lane];
    float l = rr * rr, cc = rr;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      l += __shfl_xor_sync(0xffffffffu, l, off);
      cc += __shfl_xor_sync(0xffffffffu, cc, off);
    }
    if (lane == 0) {
      S->lossacc = l * inv_B;
      S->cacc = -2.f * cc * inv_B;
    }
  }
  // ---- phase C: backward, weight gradients accumulated in TMEM across tiles
  const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
  for (int t = 0; t < tiles; ++t) {
    const int r = t * 128 + tid;
    const bool in = r < rows;
    const int pl = in ? r / D : 0, d = in ? r % D : 0;
    const float4 f = in ? feats[(p0 + pl) * D + d] : make_float4(0.f, 0.f, 0.f, 0.f);
    float a1[kH], a2[kH];
    mlp_forward_tile(0, tid, sX, sH, sW1, sW2, S->ms, t_d1, &S->bar, phase, f.x, f.y, f.z, a.dev_status, a1, a2);
    const float d3 = in ? -2.f * S->resid[pl] * ds_rows[r] * inv_B : 0.f;
    float d2[kH];
    float b3p = d3;
#pragma unroll
    for (int j = 0; j < kH; ++j) {
      const float h2 = silu_fast(a2[j]);
      float w = d3 * h2;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) w += __shfl_xor_sync(0xffffffffu, w, off);
      if (lane == 0) S->w3acc[warp][j] += w;
      d2[j] = d3 * S->ms.w3[j] * dsilu_fast(a2[j]);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) b3p += __shfl_xor_sync(0xffffffffu, b3p, off);
    if (lane == 0) S->b3acc[warp] += b3p;
    write_row_kmajor(sD2, tid, d2, 8, kHLbo, kHSbo);
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      // d1pre = d2 W2: A = d2 [128 x 64] K-major, B = W2 read MN-major (N = in, K = out)
      const uint32_t id_b1 = tc::idesc_bf16(128, kH, false, true);
#pragma unroll
      for (int s = 0; s < 4; ++s)
        tc::mma_bf16(t_d3, tc::smem_desc(smem_addr(sD2) + 2u * s * kHLbo, kHLbo, kHSbo),
                     tc::smem_desc(smem_addr(sW2) + 2u * s * kW2Sbo, kW2Sbo, kW2Lbo), id_b1, s > 0 ? 1u : 0u);
      // dW2 += d2^T H1: A = d2 read MN-major (M = out), B = H1 read MN-major (N = in), K = rows
      const uint32_t id_w2 = tc::idesc_bf16(64, kH, true, true);
      const uint32_t id_b2 = tc::idesc_bf16(64, 16, true, true);
#pragma unroll
      for (int s = 0; s < 8; ++s) {
        const uint32_t acc = (t > 0 || s > 0) ? 1u : 0u;
        tc::mma_bf16(t_dw2, tc::smem_desc(smem_addr(sD2) + 2u * s * kHSbo, kHSbo, kHLbo),
                     tc::smem_desc(smem_addr(sH) + 2u * s * kHSbo, kHSbo, kHLbo), id_w2, acc);
        tc::mma_bf16(t_db2, tc::smem_desc(smem_addr(sD2) + 2u * s * kHSbo, kHSbo, kHLbo),
                     tc::smem_desc(smem_addr(sOnes) + 2u * s * 256u, 256u, 128u), id_b2, acc);
      }
      tc::commit(&S->bar);
    }
    mma_wait(&S->bar, phase, a.dev_status);
    float d1[kH];
#pragma unroll
    for (int c = 0; c < kH; c += 16) tc::tmem_ld16(t_d3 + lane_base + (uint32_t)c, d1 + c);
#pragma unroll
    for (int j = 0; j < kH; ++j) d1[j] = in ? d1[j] * dsilu_fast(a1[j]) : 0.f;
    write_row_kmajor(sD1, tid, d1, 8, kHLbo, kHSbo);
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      // dW1 += d1^T X: A = d1 read MN-major (M = hidden), B = X read MN-major (N = feature), K = rows
      const uint32_t id_w1 = tc::idesc_bf16(64, 16, true, true);
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(t_dw1, tc::smem_desc(smem_addr(sD1) + 2u * s * kHSbo, kHSbo, kHLbo),
                     tc::smem_desc(smem_addr(sX) + 2u * s * kXSbo, kXSbo, kXLbo), id_w1,
                     (t > 0 || s > 0) ? 1u : 0u);
      tc::commit(&S->bar);
    }
    mma_wait(&S->bar, phase, a.dev_status);
  }
  // ---- write this CTA's gradient partials
  float* G = a.grad_partials + (size_t)blockIdx.x * kGradWidth;
  {
    // M = 64 accumulators: row m lives in lane 32 (m / 16) + m % 16.
    float v[kH];
#pragma unroll
    for (int c = 0; c < kH; c += 16) tc::tmem_ld16(t_dw2 + lane_base + (uint32_t)c, v + c);
    float vb[16], vw1[16];
    tc::tmem_ld16(t_db2 + lane_base, vb);
    tc::tmem_ld16(t_dw1 + lane_base, vw1);
    if (lane < 16) {
      const int m = 16 * warp + lane;
#pragma unroll
      for (int j = 0; j < kH; ++j) G[kOffW2 + m * kH + j] = v[j];
      G[kOffB2 + m] = vb[0];
#pragma unroll
      for (int j = 0; j < kIn; ++j) G[kOffW1 + m * kIn + j] = j < 4 ? vw1[j] : 0.f;
    }
  }
  __syncthreads();
  if (tid < kH) {
    float s = 0.f;
    for (int w = 0; w < 4; ++w) s += S->w3acc[w][tid];
    G[kOffW3 + tid] = s;
  }
  if (tid == 0) {
    float s = 0.f;
    for (int w = 0; w < 4; ++w) s += S->b3acc[w];
    G[kOffB3] = s;
    G[kOffC] = S->cacc;
    G[kNumParams] = S->lossacc;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tm, 512);
  }
}

// The training CTA holds all 512 TMEM columns; >= 116 KB of shared memory keeps
// it alone on its SM so that no allocation has to wait.
size_t train_smem_bytes(int dates) {
  size_t total = ((sizeof(TrainSmem) + 1023) & ~(size_t)1023) + kW1Bytes + kW2Bytes + kXBytes + 3 * kHBytes +
                 16 * 128 * 2 + (size_t)2 * kTrainPaths * dates * sizeof(float);
  if (total < 116 * 1024) total = 116 * 1024;
  return total;
}

// ---- Adam ------------------------------------------------------------------------------
__global__ void mlp_adam_kernel(tqf_mlp_adam_args a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > kNumParams) return;
  float g = 0.f;
  for (int b = 0; b < a.num_partials; ++b) g += a.grad_partials[(size_t)b * kGradWidth + i];
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
    TQF_REQUIRE(a->mlp.w1_bf16 && a->mlp.w2_bf16 && a->mlp.b2 && a->mlp.w3 && a->mlp.b3,
                "tqf_heston_asian: network weights required");
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
  if (a->mode == 0) heston_asian_kernel<0><<<grid, kPathThreads, smem, s>>>(*a);
  else if (a->mode == 1) heston_asian_kernel<1><<<grid, kPathThreads, smem, s>>>(*a);
  else heston_asian_kernel<2><<<grid, kPathThreads, smem, s>>>(*a);
  int rc = check_launch("heston_asian_kernel");
  if (rc || a->mode == 1) return rc;
  return reduce_partials(static_cast<const double*>(a->workspace), grid, 5, a->out, s);
}

extern "C" int tqf_mlp_num_params(void) { return kNumParams; }

extern "C" int tqf_mlp_train_step(const tqf_mlp_train_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_mlp_train_step: null args");
  TQF_REQUIRE(a->num_dates >= 1 && a->num_dates <= kMaxDates, "tqf_mlp_train_step: bad num_dates");
  TQF_REQUIRE(a->batch_paths >= kTrainPaths && a->batch_paths % kTrainPaths == 0,
              "tqf_mlp_train_step: batch_paths must be a positive multiple of %d", kTrainPaths);
  TQF_REQUIRE(a->feats && a->dS && a->Y && a->params && a->w1_bf16 && a->w2_bf16 && a->grad_partials,
              "tqf_mlp_train_step: null pointer");
  const int grid = a->batch_paths / kTrainPaths;
  const size_t smem = train_smem_bytes(a->num_dates);
  TQF_REQUIRE(smem <= 227 * 1024, "tqf_mlp_train_step: too many dates");
  cudaFuncSetAttribute(mlp_train_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  mlp_train_step_kernel<<<grid, kTrainThreads, smem, static_cast<cudaStream_t>(stream)>>>(*a);
  return check_launch("mlp_train_step_kernel");
}

extern "C" int tqf_mlp_adam(const tqf_mlp_adam_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a && a->params && a->m && a->v && a->grad_partials && a->w1_bf16 && a->w2_bf16,
              "tqf_mlp_adam: null pointer");
  TQF_REQUIRE(a->num_partials >= 1, "tqf_mlp_adam: num_partials must be >= 1");
  const int threads = 256;
  const int blocks = (kNumParams + 1 + threads - 1) / threads;
  mlp_adam_kernel<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(*a);
  return check_launch("mlp_adam_kernel");
}
