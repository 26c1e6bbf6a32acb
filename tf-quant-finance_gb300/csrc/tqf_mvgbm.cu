// Correlated geometric Brownian motion (the exact log scheme of
// MultivariateGeometricBrownianMotion._sample_paths,
// tff/models/geometric_brownian_motion/multivariate_geometric_brownian_motion.py:229-281)
// and a fused arithmetic-basket pricer with pathwise Greeks.
//
// mvgbm_paths_kernel: one thread per path, log-state (the running cumsum of
//   (mu - sigma^2/2) dt + sqrt(dt) sigma (L z)) in registers; L staged in
//   shared memory; states x0 * exp(cumsum) stored at their slots as
//   contiguous [dim] rows (float: the cumsum kept in base 2, one ex2 per
//   state).
// basket_price_kernel: the terminal log-state is linear in the draws,
//   log S_T,i = log S0_i + (mu_i - sigma_i^2/2) T + sigma_i (L w)_i with
//   w = sum_k sqrt(dt_k) z_k, so the kernel accumulates w (dim FMAs per
//   step) and applies L once per path.  Per path it forms the basket
//   B = sum_i a_i S_T,i, the payoff and g_i = 1{B > K} a_i S_T,i, from which
//   dP/dS0_i = g_i / S0_i, dP/dsigma_i = g_i (y_i - sigma_i T), dP/dmu_i =
//   g_i T.  Warp-level FP32 partial sums feed per-warp FP64 accumulators
//   (fixed order, deterministic).
#include <cuda_bf16.h>

#include "tqf_tc.cuh"

namespace tqf {
namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;

template <typename T, int DM>
struct GbmCoef {
  T L[DM * DM];
  T drift[DM];  // mu - sigma^2 / 2
  T sigma[DM];
};

template <typename T, int DM>
__device__ __forceinline__ void load_coef(GbmCoef<T, DM>* c, int dim, const void* chol,
                                          const void* drift, const void* sigma) {
  for (int i = threadIdx.x; i < DM * DM; i += blockDim.x) {
    const int r = i / DM, q = i % DM;
    T v = T(0);
    if (r < dim && q < dim) {
      v = chol ? static_cast<const T*>(chol)[r * dim + q] : (r == q ? T(1) : T(0));
    }
    c->L[i] = v;
  }
  for (int i = threadIdx.x; i < DM; i += blockDim.x) {
    c->drift[i] = i < dim ? static_cast<const T*>(drift)[i] : T(0);
    c->sigma[i] = i < dim ? static_cast<const T*>(sigma)[i] : T(0);
  }
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// A recorded state from its log-state: float log-states are kept in base 2
// (drift and volatility scaled by log2(e) when the coefficients are loaded),
// so a state is x0 2^cs, one SFU ex2; double ones in base e.
__device__ __forceinline__ float gbm_level(float x0, float cs) { return x0 * ex2_approx(cs); }
__device__ __forceinline__ double gbm_level(double x0, double cs) { return x0 * exp(cs); }

// cs += (mu - sigma^2/2) dt + sqrt(dt) sigma (L z), L lower triangular.
template <typename T, int DM>
__device__ __forceinline__ void gbm_advance(const GbmCoef<T, DM>& cf, T (&cs)[DM], const T* z, T dt, T sdt) {
#pragma unroll
  for (int r = 0; r < DM; ++r) {
    T y = T(0);
#pragma unroll
    for (int c = 0; c <= r; ++c) y += cf.L[r * DM + c] * z[c];
    cs[r] += cf.drift[r] * dt + sdt * cf.sigma[r] * y;
  }
}

// STAGE: 1 = recorded states go through the coalescing RowStager (dynamic
// shared memory), chosen when a path's output row is at least 64 bytes; then
// every thread runs every round and a thread past the last path simulates
// that path again with its output dropped.  2 = WarpRowStager (every date
// declared recorded in order; every lane of a warp that has a path runs every
// round).  0 = direct stores.
template <typename T, int DM, int STAGE>
__global__ void __launch_bounds__(kBlock) mvgbm_paths_kernel(tqf_mvgbm_args a) {
  __shared__ GbmCoef<T, DM> coef;
  extern __shared__ __align__(16) unsigned char stage_smem[];
  const int dim = a.dim;
  load_coef<T, DM>(&coef, dim, a.chol, a.drift, a.vol);
  if constexpr (sizeof(T) == 4) {
    // base-2 log-states (gbm_level); the threads that loaded the values scale them
    for (int i = threadIdx.x; i < DM; i += blockDim.x) {
      coef.drift[i] *= 1.4426950408889634f;
      coef.sigma[i] *= 1.4426950408889634f;
    }
  }
  __syncthreads();
  const T* table = static_cast<const T*>(a.step_table);
  T* out = static_cast<T*>(a.output.ptr);
  const int ns = a.output.num_slots;
  const int64_t N = a.num_paths;
  if constexpr (STAGE == 2) {
    // verify the every-step declaration on the table (see tqf_path_output)
    const int base = a.output.init_slot >= 0 ? 1 : 0;
    int ok = (a.output.init_slot < 0 || a.output.init_slot == 0) && base + a.num_steps == ns;
    for (int i = threadIdx.x; i < a.num_steps; i += kBlock) ok &= (int)table[i * 4 + 2] == base + i;
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0 && a.dev_status) atomicExch(a.dev_status, TQF_E_INVALID);
      return;
    }
  }
  // In-kernel Philox draws of exactly DM <= 4 components per step (table
  // rows aligned for pair loads): the loop walks whole Philox blocks.
  using PG = PhiloxGroup<T, DM>;
  constexpr bool kWhole = DM <= 4;
  const bool whole_blocks = kWhole && dim == DM && a.draws.source == TQF_DRAWS_PHILOX &&
                            (reinterpret_cast<uintptr_t>(table) & (2 * sizeof(T) - 1)) == 0;
  // one-factor coefficients live in registers
  GbmCoef<T, DM> creg;
  if constexpr (DM == 1) creg = coef;
  const GbmCoef<T, DM>* cf = DM == 1 ? &creg : &coef;
  RowStager<T, DM, kBlock> stg(stage_smem, dim);
  WarpRowStager wst(stage_smem);
  uint32_t* out_words = reinterpret_cast<uint32_t*>(out);
  const int64_t row_words = (int64_t)ns * dim * (int64_t)(sizeof(T) / 4);
  const int64_t per_round = (int64_t)gridDim.x * kBlock;
  for (int64_t base = 0; base < N; base += per_round) {
    const int64_t row0 = base + (int64_t)blockIdx.x * kBlock;
    const int64_t path = row0 + threadIdx.x;
    const int64_t warp0 = row0 + (threadIdx.x & ~31);
    if (STAGE == 2 ? warp0 >= N : (STAGE == 0 && path >= N)) break;
    const int64_t pc = path < N ? path : N - 1;
    const T* x0p = static_cast<const T*>(a.x0) + (a.x0_per_path ? pc * dim : 0);
    T x0[DM], cs[DM];
#pragma unroll
    for (int j = 0; j < DM; ++j) {
      x0[j] = j < dim ? x0p[j] : T(0);
      cs[j] = T(0);
    }
    if constexpr (STAGE == 2) wst.begin();
    if (a.output.init_slot >= 0) {
      if constexpr (STAGE == 2) {
        wst.put<T, DM>(x0, dim, out_words, row_words, warp0, N);
      } else if constexpr (STAGE == 1) {
        stg.put(out, ns, row0, N, a.output.init_slot, x0);
      } else {
        T* o = out + (path * ns + a.output.init_slot) * dim;
#pragma unroll
        for (int j = 0; j < DM; ++j)
          if (j < dim) o[j] = x0[j];
      }
    }
    // records x0 e^cs (float: 2^cs) after step i at its slot (STAGE 2: every date, in order)
    auto record = [&](int i) {
      if constexpr (STAGE == 2) {
        T xs[DM];
#pragma unroll
        for (int j = 0; j < DM; ++j) xs[j] = gbm_level(x0[j], cs[j]);
        wst.put<T, DM>(xs, dim, out_words, row_words, warp0, N);
      } else {
        const int slot = (int)table[i * 4 + 2];
        if (slot >= 0) {
          if constexpr (STAGE == 1) {
            T xs[DM];
#pragma unroll
            for (int j = 0; j < DM; ++j) xs[j] = gbm_level(x0[j], cs[j]);
            stg.put(out, ns, row0, N, slot, xs);
          } else {
            T* o = out + (path * ns + slot) * dim;
#pragma unroll
            for (int j = 0; j < DM; ++j)
              if (j < dim) o[j] = gbm_level(x0[j], cs[j]);
          }
        }
      }
    };
    DrawSource<T> src(a.draws, pc, dim);
    if (kWhole && whole_blocks) {
      // sqrt(dt) carries the antithetic sign: L (sign z) = sign (L z) exactly;
      // the warp stager makes room for a whole group's words at once
      constexpr int kGroupWords = PG::kNormals * (int)(sizeof(T) / 4);
      static_assert(kGroupWords <= 32, "a group's words fit one piece");
      for (int i = 0; i < a.num_steps; i += PG::kSteps) {
        if constexpr (STAGE == 2) wst.make_room(kGroupWords, out_words, row_words, warp0, N);
        T z[PG::kNormals];
#pragma unroll
        for (int s = 0; s < PG::kSteps; ++s) {
          if (PG::kSteps > 1 && i + s >= a.num_steps) break;
          PG::fill_step(i / PG::kSteps, s, src.rng.path, src.rng.k0, src.rng.k1, z);
          T dt, sdt;
          step_pair<true>(table + (size_t)(i + s) * 4, dt, sdt);
          gbm_advance<T, DM>(*cf, cs, z + s * DM, dt, sdt * src.sign);
          if constexpr (STAGE == 2) {
            T xs[DM];
#pragma unroll
            for (int j = 0; j < DM; ++j) xs[j] = gbm_level(x0[j], cs[j]);
            wst.append<T, DM>(xs);
          } else {
            record(i + s);
          }
        }
      }
    } else {
      for (int i = 0; i < a.num_steps; ++i) {
        const T dt = table[i * 4], sdt = table[i * 4 + 1];
        T z[DM];
#pragma unroll
        for (int c = 0; c < DM; ++c) z[c] = c < dim ? src.get(i, c) : T(0);
        gbm_advance<T, DM>(*cf, cs, z, dt, sdt);
        record(i);
      }
    }
    if (STAGE == 1 && stg.cnt > 0) stg.flush(out, ns, row0, N);
    if (STAGE == 2 && wst.nw > 0) wst.flush(out_words, row_words, warp0, N);
  }
}

// ---- tensor-core L z (split BF16, three products) ------------------------------
// Float32 factors 16 <= dim <= 64, padded with zeros to KP = 16 KB.  One
// warpgroup = 128 paths = one M = 128 tile.  Per step each thread writes its
// normals split as z = hi + lo (BF16 each) into A_hi / A_lo [128 x KP];
// D = A_hi L_hi^T + A_hi L_lo^T + A_lo L_hi^T (M = 128, N = KP, K = KP in KB
// instructions of K = 16 each) accumulates y = L z in FP32 in TMEM.  The
// step's MMAs are issued one step ahead (double-buffered tiles and TMEM
// columns), so the tensor core works while the threads consume the previous
// step's y.  Layouts (K-major, no swizzle): A has its 8-column k-blocks
// 2 KiB apart (128 rows x 16 bytes each), B [KP x KP] its k-blocks KP x 16
// bytes apart; instruction j of a product starts 2 k-blocks further in both.
constexpr int kLzThreads = 128;
constexpr int kLzMaxKB = 4;  // up to 64 factors
constexpr uint32_t kLzALbo = 2048, kLzASbo = 128;

template <int KB>
struct LzShape {
  static constexpr int KP = 16 * KB;
  static constexpr uint32_t kBLbo = (uint32_t)KP * 16, kBSbo = 128;
  static constexpr int kATile = 128 * KP * 2;
  static constexpr int kBTile = KP * KP * 2;
  // TMEM columns: two buffers of KP, rounded up to a power of two >= 32
  static constexpr uint32_t kTmemCols = KB == 1 ? 32u : (KB == 2 ? 64u : 128u);
  // From 48 factors on, one A buffer: the next step's normals are staged
  // once this step's MMAs have read the tile (its TMEM result stays double
  // buffered), which halves the A tiles and lets more CTAs share an SM.
  static constexpr bool kSingleA = KB >= 3;
  static constexpr int kATiles = kSingleA ? 2 : 4;
  static constexpr size_t kSmem = 1024 + kATiles * (size_t)kATile + 2 * (size_t)kBTile;
};

__device__ __forceinline__ uint32_t pack2_bf16(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

struct LzSmem {
  uint64_t bar[2];
  uint32_t tmem_slot;
  uint32_t pad;
  float drift[16 * kLzMaxKB], sigma[16 * kLzMaxKB], x0[16 * kLzMaxKB];  // drift, sigma pre-scaled by log2(e)
};

// FULL: dim == KP (no padded factors), so every normal is drawn and every
// row is whole float4 stores without per-factor checks.
template <int KB, bool FULL>
__global__ void __launch_bounds__(kLzThreads) mvgbm_paths_tc_kernel(tqf_mvgbm_args a) {
  using Sh = LzShape<KB>;
  constexpr int KP = Sh::KP;
  extern __shared__ __align__(1024) unsigned char smem[];
  LzSmem* S = reinterpret_cast<LzSmem*>(smem);
  unsigned char* sA = smem + 1024;                 // [1 or 2 buffers][hi, lo] x kATile
  unsigned char* sB = sA + Sh::kATiles * Sh::kATile;  // L_hi, L_lo
  const int tid = threadIdx.x, warp = tid >> 5;
  const int dim = FULL ? KP : a.dim;
  // split L (row-major [dim][dim], lower; zero-padded to KP) into BF16 hi/lo
  // B tiles: B[n][k] = L[n][k]
  for (int i = tid; i < KP * KP; i += kLzThreads) {
    const int n = i / KP, k = i % KP;
    const float l = (n < dim && k < dim) ? static_cast<const float*>(a.chol)[n * dim + k] : 0.f;
    const __nv_bfloat16 hi = __float2bfloat16_rn(l);
    const __nv_bfloat16 lo = __float2bfloat16_rn(l - __bfloat162float(hi));
    *reinterpret_cast<__nv_bfloat16*>(sB + tc::kmajor_off(n, k, Sh::kBLbo, Sh::kBSbo)) = hi;
    *reinterpret_cast<__nv_bfloat16*>(sB + Sh::kBTile + tc::kmajor_off(n, k, Sh::kBLbo, Sh::kBSbo)) = lo;
  }
  if (tid < KP) {
    // the log-state is carried in base 2: x0 * 2^(cumsum / ln 2)
    const bool in = tid < dim;
    S->drift[tid] = in ? static_cast<const float*>(a.drift)[tid] * 1.4426950408889634f : 0.f;
    S->sigma[tid] = in ? static_cast<const float*>(a.vol)[tid] * 1.4426950408889634f : 0.f;
    S->x0[tid] = (in && !a.x0_per_path) ? static_cast<const float*>(a.x0)[tid] : 0.f;
  }
  if (tid == 0) {
    mbar_init(&S->bar[0], 1);
    mbar_init(&S->bar[1], 1);
  }
  if (warp == 0) tc::tmem_alloc(&S->tmem_slot, Sh::kTmemCols);
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S->tmem_slot;
  const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
  const uint32_t idesc = tc::idesc_bf16(128, KP, false, false);
  const float* table = static_cast<const float*>(a.step_table);
  float* out = static_cast<float*>(a.output.ptr);
  const int ns = a.output.num_slots;
  const int steps = a.num_steps;
  // whole float4 rows: dim a multiple of 4 (the dispatcher checks the base
  // pointer's 16-byte alignment)
  const bool vec = FULL || (dim & 3) == 0;
  const bool philox = a.draws.source == TQF_DRAWS_PHILOX;
  uint32_t phase[2] = {0u, 0u};
  const int64_t per_round = (int64_t)gridDim.x * kLzThreads;
  for (int64_t base = 0; base < a.num_paths; base += per_round) {
    const int64_t path = base + (int64_t)blockIdx.x * kLzThreads + tid;
    const bool valid = path < a.num_paths;
    const int64_t pp = valid ? path : 0;
    DrawSource<float> src(a.draws, pp, dim);
    const float* x0p = a.x0_per_path ? static_cast<const float*>(a.x0) + pp * dim : S->x0;
    float cs[KP];
#pragma unroll
    for (int j = 0; j < KP; ++j) cs[j] = 0.f;
    auto record = [&](int slot, bool initial) {
      float* o = out + (pp * ns + slot) * dim;
#pragma unroll
      for (int q = 0; q < KP / 4; ++q) {
        const int c = 4 * q;
        if (!FULL && c >= dim) break;
        float v[4];
#pragma unroll
        for (int e = 0; e < 4; ++e)
          v[e] = (FULL || c + e < dim) ? (initial ? x0p[c + e] : x0p[c + e] * ex2_approx(cs[c + e])) : 0.f;
        if (vec) {
          reinterpret_cast<float4*>(o)[q] = make_float4(v[0], v[1], v[2], v[3]);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (c + e < dim) o[c + e] = v[e];
        }
      }
    };
    if (valid && a.output.init_slot >= 0) record(a.output.init_slot, true);
    // write the split normals of `step` into buffer b
    auto stage = [&](int step, int b) {
      unsigned char* th = sA + (Sh::kSingleA ? 0 : 2 * b) * Sh::kATile;
      unsigned char* tl = th + Sh::kATile;
#pragma unroll
      for (int kb = 0; kb < KB; ++kb) {
        float z[16];
        if (FULL && philox) {
          // the 16 draws of this column block are 4 whole Philox blocks
          const int64_t b0 = ((int64_t)step * KP + 16 * kb) >> 2;
#pragma unroll
          for (int q = 0; q < 4; ++q) philox_normals(b0 + q, src.rng.path, src.rng.k0, src.rng.k1, z + 4 * q);
#pragma unroll
          for (int c = 0; c < 16; ++c) z[c] *= src.sign;
        } else {
#pragma unroll
          for (int c = 0; c < 16; ++c) z[c] = (FULL || 16 * kb + c < dim) ? src.get(step, 16 * kb + c) : 0.f;
        }
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          hi[q] = pack2_bf16(z[2 * q], z[2 * q + 1]);
          const float h0 = __uint_as_float(hi[q] << 16), h1 = __uint_as_float(hi[q] & 0xFFFF0000u);
          lo[q] = pack2_bf16(z[2 * q] - h0, z[2 * q + 1] - h1);
        }
        const uint32_t o0 = tc::kmajor_off(tid, 16 * kb, kLzALbo, kLzASbo);
        const uint32_t o1 = tc::kmajor_off(tid, 16 * kb + 8, kLzALbo, kLzASbo);
        *reinterpret_cast<uint4*>(th + o0) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4*>(th + o1) = make_uint4(hi[4], hi[5], hi[6], hi[7]);
        *reinterpret_cast<uint4*>(tl + o0) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
        *reinterpret_cast<uint4*>(tl + o1) = make_uint4(lo[4], lo[5], lo[6], lo[7]);
      }
    };
    auto issue = [&](int b) {
      tc::fence_smem_to_async();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      if (tid == 0) {
        const uint32_t ah = smem_addr(sA + (Sh::kSingleA ? 0 : 2 * b) * Sh::kATile), al = ah + Sh::kATile;
        const uint32_t bh = smem_addr(sB), bl = bh + Sh::kBTile;
        const uint32_t d = tmem + (uint32_t)(KP * b);
#pragma unroll
        for (int j = 0; j < KB; ++j) {
          const uint32_t ao = 2u * (uint32_t)j * kLzALbo, bo = 2u * (uint32_t)j * Sh::kBLbo;
          tc::mma_bf16(d, tc::smem_desc(ah + ao, kLzALbo, kLzASbo), tc::smem_desc(bh + bo, Sh::kBLbo, Sh::kBSbo),
                       idesc, j > 0 ? 1u : 0u);
          tc::mma_bf16(d, tc::smem_desc(ah + ao, kLzALbo, kLzASbo), tc::smem_desc(bl + bo, Sh::kBLbo, Sh::kBSbo),
                       idesc, 1u);
          tc::mma_bf16(d, tc::smem_desc(al + ao, kLzALbo, kLzASbo), tc::smem_desc(bh + bo, Sh::kBLbo, Sh::kBSbo),
                       idesc, 1u);
        }
        tc::commit(&S->bar[b]);
      }
    };
    float dt = 0.f, sdt = 0.f;
    int slot = -1;
    if (steps > 0) {
      dt = table[0];
      sdt = table[1];
      slot = (int)table[2];
      stage(0, 0);
      issue(0);
    }
    for (int i = 0; i < steps; ++i) {
      const int b = i & 1;
      if (!Sh::kSingleA && i + 1 < steps) {
        stage(i + 1, b ^ 1);
        issue(b ^ 1);
      }
      bool ok = mbar_wait_bounded(&S->bar[b], phase[b]);
      if (!ok) {
        if (a.dev_status) atomicExch(a.dev_status, TQF_E_TIMEOUT);
        mbar_wait_bounded(&S->bar[b], phase[b]);
      }
      phase[b] ^= 1u;
      tc::fence_after_sync();
      if (Sh::kSingleA && i + 1 < steps) {
        // step i's MMAs have read the single A tile: stage and issue step
        // i + 1 (into the other TMEM buffer) before consuming step i
        stage(i + 1, b ^ 1);
        issue(b ^ 1);
      }
#pragma unroll
      for (int kb = 0; kb < KB; ++kb) {
        float y[16];
        tc::tmem_ld16(tmem + lane_base + (uint32_t)(KP * b + 16 * kb), y);
#pragma unroll
        for (int j = 0; j < 16; ++j)
          cs[16 * kb + j] += S->drift[16 * kb + j] * dt + sdt * S->sigma[16 * kb + j] * y[j];
      }
      tc::fence_before_sync();
      if (valid && slot >= 0) record(slot, false);
      if (i + 1 < steps) {
        dt = table[(i + 1) * 4];
        sdt = table[(i + 1) * 4 + 1];
        slot = (int)table[(i + 1) * 4 + 2];
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, Sh::kTmemCols);
  }
}

// ---- any dimension on CUDA cores: one warp per path ---------------------------
// Lane l owns factors r = l, l + 32, ...; each step the warp writes its
// normals into a per-warp shared buffer, every lane forms y_r = sum_{c<=r}
// L_rc z_c (L stored transposed in shared memory when it fits, so the lanes
// read consecutive words; else row-major from global memory) and updates
// its log-states, kept in a second per-warp buffer.  Recorded rows are
// written by consecutive lanes (coalesced).
constexpr int kWideWarps = kBlock / 32;
constexpr size_t kWideLSmem = 96 * 1024;

template <typename T, bool LS>
__global__ void __launch_bounds__(kBlock) mvgbm_paths_wide_kernel(tqf_mvgbm_args a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int dim = a.dim;
  const size_t dd = (size_t)dim * dim;
  const T* gL = static_cast<const T*>(a.chol);
  T* Ls = reinterpret_cast<T*>(smem);
  size_t off = 0;
  if (LS) {
    for (size_t i = threadIdx.x; i < dd; i += kBlock) {
      const size_t r = i / dim, c = i - r * dim;
      Ls[c * dim + r] = gL ? gL[i] : (r == c ? T(1) : T(0));
    }
    off = (dd * sizeof(T) + 15) & ~(size_t)15;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* zs = reinterpret_cast<T*>(smem + off) + (size_t)warp * 2 * dim;
  T* cs = zs + dim;
  __syncthreads();
  const T* drift = static_cast<const T*>(a.drift);
  const T* sigma = static_cast<const T*>(a.vol);
  const T* table = static_cast<const T*>(a.step_table);
  T* out = static_cast<T*>(a.output.ptr);
  const int ns = a.output.num_slots;
  const int64_t N = a.num_paths;
  const int64_t nwarps = (int64_t)gridDim.x * kWideWarps;
  for (int64_t path = (int64_t)blockIdx.x * kWideWarps + warp; path < N; path += nwarps) {
    const T* x0 = static_cast<const T*>(a.x0) + (a.x0_per_path ? path * dim : 0);
    for (int r = lane; r < dim; r += 32) cs[r] = T(0);
    if (a.output.init_slot >= 0) {
      T* o = out + (path * ns + a.output.init_slot) * dim;
      for (int r = lane; r < dim; r += 32) o[r] = x0[r];
    }
    DrawSource<T> src(a.draws, path, dim);
    for (int i = 0; i < a.num_steps; ++i) {
      const T dt = table[i * 4], sdt = table[i * 4 + 1];
      const int slot = (int)table[i * 4 + 2];
      __syncwarp();
      for (int c = lane; c < dim; c += 32) zs[c] = src.get(i, c);
      __syncwarp();
      for (int r = lane; r < dim; r += 32) {
        T y = T(0);
        for (int c = 0; c <= r; ++c) {
          const T l = LS ? Ls[(size_t)c * dim + r] : (gL ? gL[(size_t)r * dim + c] : (r == c ? T(1) : T(0)));
          y += l * zs[c];
        }
        cs[r] += drift[r] * dt + sdt * sigma[r] * y;
      }
      if (slot >= 0) {
        T* o = out + (path * ns + slot) * dim;
        for (int r = lane; r < dim; r += 32) o[r] = x0[r] * exp(cs[r]);
      }
    }
    __syncwarp();
  }
}

// Arithmetic basket, any dimension: one warp per path.  Lane-owned assets
// accumulate w_c = sum_k sqrt(dt_k) z_kc, then y = L w, S_T, the basket
// (warp sum), the payoff and the per-asset pathwise terms; per-warp FP64
// accumulators in shared memory hold [P, P^2, g_i, g_i (y_i - sigma_i T)].
template <typename T, bool LS>
__global__ void __launch_bounds__(kBlock) basket_price_wide_kernel(tqf_basket_args a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int dim = a.dim;
  const size_t dd = (size_t)dim * dim;
  const T* gL = static_cast<const T*>(a.chol);
  T* Ls = reinterpret_cast<T*>(smem);
  size_t off = 0;
  if (LS) {
    for (size_t i = threadIdx.x; i < dd; i += kBlock) {
      const size_t r = i / dim, c = i - r * dim;
      Ls[c * dim + r] = gL ? gL[i] : (r == c ? T(1) : T(0));
    }
    off = (dd * sizeof(T) + 15) & ~(size_t)15;
  }
  const int width = 2 + 2 * dim;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* acc = reinterpret_cast<double*>(smem + off) + (size_t)warp * width;
  T* ws = reinterpret_cast<T*>(smem + off + (size_t)kWideWarps * width * sizeof(double)) + (size_t)warp * 2 * dim;
  T* ys = ws + dim;
  for (int j = lane; j < width; j += 32) acc[j] = 0.0;
  __syncthreads();
  const T* spot = static_cast<const T*>(a.spot);
  const T* drift = static_cast<const T*>(a.drift);
  const T* sigma = static_cast<const T*>(a.vol);
  const T* wts = static_cast<const T*>(a.weights);
  const T* sdt_tab = static_cast<const T*>(a.sqrt_dt);
  const T T_total = (T)a.total_time;
  const T K = (T)a.strike;
  const T sign = a.is_call ? T(1) : T(-1);
  const int64_t N = a.num_paths;
  const int64_t nwarps = (int64_t)gridDim.x * kWideWarps;
  for (int64_t path = (int64_t)blockIdx.x * kWideWarps + warp; path < N; path += nwarps) {
    DrawSource<T> src(a.draws, path, dim);
    __syncwarp();
    for (int c = lane; c < dim; c += 32) {
      T w = T(0);
      for (int i = 0; i < a.num_steps; ++i) w += sdt_tab[i] * src.get(i, c);
      ws[c] = w;
    }
    __syncwarp();
    T part = T(0);
    for (int r = lane; r < dim; r += 32) {
      T y = T(0);
      for (int c = 0; c <= r; ++c) {
        const T l = LS ? Ls[(size_t)c * dim + r] : (gL ? gL[(size_t)r * dim + c] : (r == c ? T(1) : T(0)));
        y += l * ws[c];
      }
      ys[r] = y;
      part += wts[r] * spot[r] * exp(drift[r] * T_total + sigma[r] * y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    const T pay = sign * (part - K);
    const bool itm = pay > T(0);
    if (lane == 0 && itm) {
      acc[0] += (double)pay;
      acc[1] += (double)pay * (double)pay;
    }
    if (itm) {
      for (int r = lane; r < dim; r += 32) {
        const T S = spot[r] * exp(drift[r] * T_total + sigma[r] * ys[r]);
        const T g = sign * wts[r] * S;
        acc[2 + r] += (double)g;
        acc[2 + dim + r] += (double)(g * (ys[r] - sigma[r] * T_total));
      }
    }
  }
  __syncthreads();
  double* wsp = static_cast<double*>(a.workspace);
  for (int j = threadIdx.x; j < width; j += blockDim.x) {
    double s2 = 0.0;
    for (int wi = 0; wi < kWideWarps; ++wi)
      s2 += reinterpret_cast<const double*>(smem + off)[(size_t)wi * width + j];
    wsp[(size_t)blockIdx.x * width + j] = s2;
  }
}

// ---- fused basket pricing --------------------------------------------------
// Per-path quantities reduced: [0] payoff, [1] payoff^2, [2 + i] g_i,
// [2 + dim + i] g_i (y_i - sigma_i T).
template <typename T, int DM>
__global__ void __launch_bounds__(kBlock) basket_price_kernel(tqf_basket_args a) {
  __shared__ GbmCoef<T, DM> coef;
  __shared__ T s_spot[DM], s_w[DM];
  __shared__ double acc[kWarps][2 + 2 * DM];
  const int dim = a.dim;
  load_coef<T, DM>(&coef, dim, a.chol, a.drift, a.vol);
  for (int i = threadIdx.x; i < DM; i += blockDim.x) {
    s_spot[i] = i < dim ? static_cast<const T*>(a.spot)[i] : T(0);
    s_w[i] = i < dim ? static_cast<const T*>(a.weights)[i] : T(0);
  }
  for (int i = threadIdx.x; i < kWarps * (2 + 2 * DM); i += blockDim.x) (&acc[0][0])[i] = 0.0;
  __syncthreads();
  const T* sdt_tab = static_cast<const T*>(a.sqrt_dt);
  const T T_total = (T)a.total_time;
  const T K = (T)a.strike;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t per_round = (int64_t)gridDim.x * kBlock;
  for (int64_t base = 0; base < a.num_paths; base += per_round) {
    const int64_t path = base + (int64_t)blockIdx.x * kBlock + threadIdx.x;
    const bool valid = path < a.num_paths;
    T q[2 + 2 * DM];
#pragma unroll
    for (int j = 0; j < 2 + 2 * DM; ++j) q[j] = T(0);
    if (valid) {
      T w[DM];
#pragma unroll
      for (int j = 0; j < DM; ++j) w[j] = T(0);
      DrawSource<T> src(a.draws, path, dim);
      using PG = PhiloxGroup<T, DM>;
      if (dim == DM && a.draws.source == TQF_DRAWS_PHILOX) {
        // whole Philox blocks per group of steps; sqrt(dt) carries the
        // antithetic sign (sdt (sign z) = (sign sdt) z exactly)
        for (int i = 0; i < a.num_steps; i += PG::kSteps) {
          T z[PG::kNormals];
#pragma unroll
          for (int s = 0; s < PG::kSteps; ++s) {
            if (PG::kSteps > 1 && i + s >= a.num_steps) break;
            PG::fill_step(i / PG::kSteps, s, src.rng.path, src.rng.k0, src.rng.k1, z);
            const T sdt = sdt_tab[i + s] * src.sign;
#pragma unroll
            for (int c = 0; c < DM; ++c) w[c] += sdt * z[s * DM + c];
          }
        }
      } else {
        for (int i = 0; i < a.num_steps; ++i) {
          const T sdt = sdt_tab[i];
#pragma unroll
          for (int c = 0; c < DM; ++c)
            if (c < dim) w[c] += sdt * src.get(i, c);
        }
      }
      T S[DM], y[DM];
      T B = T(0);
#pragma unroll
      for (int r = 0; r < DM; ++r) {
        T acc_y = T(0);
#pragma unroll
        for (int c = 0; c <= r; ++c) acc_y += coef.L[r * DM + c] * w[c];
        y[r] = acc_y;
        S[r] = r < dim ? s_spot[r] * exp(coef.drift[r] * T_total + coef.sigma[r] * acc_y) : T(0);
        B += s_w[r] * S[r];
      }
      const T pay = a.is_call ? (B - K) : (K - B);
      const bool itm = pay > T(0);
      q[0] = itm ? pay : T(0);
      q[1] = q[0] * q[0];
      const T sign = a.is_call ? T(1) : T(-1);
#pragma unroll
      for (int r = 0; r < DM; ++r) {
        const T g = itm ? sign * s_w[r] * S[r] : T(0);
        q[2 + r] = g;
        q[2 + DM + r] = g * (y[r] - coef.sigma[r] * T_total);
      }
    }
    // warp sums in the path dtype, then FP64 per warp (lane 0), fixed order
#pragma unroll
    for (int j = 0; j < 2 + 2 * DM; ++j) {
      T v = q[j];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0) acc[warp][j] += (double)v;
    }
  }
  __syncthreads();
  double* ws = static_cast<double*>(a.workspace);
  const int width = 2 + 2 * dim;
  for (int j = threadIdx.x; j < width; j += blockDim.x) {
    const int src_j = j < 2 ? j : (j < 2 + dim ? j : j - dim + DM);  // compact [2 + 2*dim]
    double s = 0.0;
    for (int wi = 0; wi < kWarps; ++wi) s += acc[wi][src_j];
    ws[(size_t)blockIdx.x * width + j] = s;
  }
}

// FP64 Cholesky of an n x n SPD matrix (n <= 64) in one CTA: right-looking,
// column by column in shared memory.  info = 0, or k + 1 if the k-th pivot is
// not positive (the matrix is not positive definite).
constexpr int kCholMax = 64;
__global__ void __launch_bounds__(256) cholesky_f64_kernel(const double* __restrict__ A, int n,
                                                          double* __restrict__ L, int* info) {
  __shared__ double s[kCholMax * kCholMax];
  __shared__ int bad;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) s[i] = A[i];
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      const double d = s[k * n + k];
      if (!(d > 0.0) && bad == 0) bad = k + 1;
      s[k * n + k] = d > 0.0 ? sqrt(d) : 0.0;
    }
    __syncthreads();
    const double piv = s[k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) s[i * n + k] = piv > 0.0 ? s[i * n + k] / piv : 0.0;
    __syncthreads();
    const int m = n - k - 1;
    for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
      const int i = k + 1 + t / m, j = k + 1 + t % m;
      if (j <= i) s[i * n + j] -= s[i * n + k] * s[j * n + k];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    const int i = t / n, j = t % n;
    L[t] = j <= i ? s[t] : 0.0;
  }
  if (threadIdx.x == 0) *info = bad;
}

// The same factorisation for n > 64, working in place in L (global memory,
// L2-resident) instead of shared memory.
__global__ void __launch_bounds__(256) cholesky_f64_global_kernel(const double* __restrict__ A, int n,
                                                                 double* __restrict__ L, int* info) {
  __shared__ int bad;
  const size_t nn = (size_t)n * n;
  for (size_t i = threadIdx.x; i < nn; i += blockDim.x) L[i] = A[i];
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      const double d = L[(size_t)k * n + k];
      if (!(d > 0.0) && bad == 0) bad = k + 1;
      L[(size_t)k * n + k] = d > 0.0 ? sqrt(d) : 0.0;
    }
    __syncthreads();
    const double piv = L[(size_t)k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x)
      L[(size_t)i * n + k] = piv > 0.0 ? L[(size_t)i * n + k] / piv : 0.0;
    __syncthreads();
    const int m = n - k - 1;
    for (int64_t t = threadIdx.x; t < (int64_t)m * m; t += blockDim.x) {
      const int i = k + 1 + (int)(t / m), j = k + 1 + (int)(t % m);
      if (j <= i) L[(size_t)i * n + j] -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
    }
    __syncthreads();
  }
  for (size_t t = threadIdx.x; t < nn; t += blockDim.x) {
    const size_t i = t / n, j = t % n;
    if (j > i) L[t] = 0.0;
  }
  if (threadIdx.x == 0) *info = bad;
}

template <typename T, int DM>
int launch_paths(const tqf_mvgbm_args& a, cudaStream_t s) {
  // the warp stager for every-date outputs; else stage the output when a
  // path's row is at least 64 bytes
  const size_t row = (size_t)a.output.num_slots * a.dim * sizeof(T);
  const bool warp_rows = a.output.every_step && (reinterpret_cast<uintptr_t>(a.output.ptr) & (sizeof(T) - 1)) == 0;
  const bool stage = !warp_rows && row >= 64;
  auto k = stage ? mvgbm_paths_kernel<T, DM, 1> : mvgbm_paths_kernel<T, DM, 0>;
  if (warp_rows) k = mvgbm_paths_kernel<T, DM, 2>;
  const size_t smem =
      warp_rows ? WarpRowStager::bytes(kBlock / 32) : (stage ? RowStager<T, DM, kBlock>::kBytes : 0);
  if (smem > 48 * 1024) set_smem_config(k, smem);
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBlock, smem);
  if (occ < 1) occ = 1;
  int64_t grid = (a.num_paths + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  k<<<(unsigned)grid, kBlock, smem, s>>>(a);
  return check_launch("mvgbm_paths_kernel");
}

template <typename T, int DM>
int basket_grid(int64_t n) {
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, basket_price_kernel<T, DM>, kBlock, 0);
  if (occ < 1) occ = 1;
  int64_t grid = (n + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  return (int)grid;
}

template <typename T, int DM>
int launch_basket(const tqf_basket_args& a, cudaStream_t s) {
  const int grid = basket_grid<T, DM>(a.num_paths);
  const int width = 2 + 2 * a.dim;
  const size_t need = (size_t)grid * width * sizeof(double);
  TQF_REQUIRE(a.workspace && a.workspace_bytes >= need, "tqf_basket_price: workspace %zu < required %zu",
              a.workspace_bytes, need);
  basket_price_kernel<T, DM><<<grid, kBlock, 0, s>>>(a);
  int rc = check_launch("basket_price_kernel");
  if (rc || a.out == nullptr) return rc;
  return reduce_partials(static_cast<const double*>(a.workspace), grid, width, a.out, s);
}

template <int KB, bool FULL>
int launch_paths_tc_kb(const tqf_mvgbm_args& a, cudaStream_t s) {
  using Sh = LzShape<KB>;
  // at least 16 KB keeps <= 13 CTAs of 32 TMEM columns on an SM; larger
  // tiles bound the resident CTAs (by shared memory) below 512 / columns
  const size_t smem_alloc = Sh::kSmem < 16 * 1024 ? 16 * 1024 : Sh::kSmem;
  auto k = mvgbm_paths_tc_kernel<KB, FULL>;
  set_smem_config(k, smem_alloc);
  // Resident CTAs per SM from the register file (256-register warp
  // granularity), shared memory and the 512 TMEM columns.
  cudaFuncAttributes fa{};
  int occ = 4;
  if (cudaFuncGetAttributes(&fa, k) == cudaSuccess && fa.numRegs > 0) {
    const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;
    occ = 65536 / (warp_regs * (kLzThreads / 32));
    const int by_smem = (int)((227 * 1024) / (smem_alloc + 1024));
    if (by_smem < occ) occ = by_smem;
  }
  const int by_tmem = (int)(512 / Sh::kTmemCols);
  if (by_tmem < occ) occ = by_tmem;
  if (occ > 12) occ = 12;
  if (occ < 1) occ = 1;
  int64_t grid = (a.num_paths + kLzThreads - 1) / kLzThreads;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  k<<<(unsigned)grid, kLzThreads, smem_alloc, s>>>(a);
  return check_launch("mvgbm_paths_tc_kernel");
}

int launch_paths_tc(const tqf_mvgbm_args& a, cudaStream_t s) {
  const bool full = (a.dim & 15) == 0;
  switch ((a.dim + 15) / 16) {
    case 1: return full ? launch_paths_tc_kb<1, true>(a, s) : launch_paths_tc_kb<1, false>(a, s);
    case 2: return full ? launch_paths_tc_kb<2, true>(a, s) : launch_paths_tc_kb<2, false>(a, s);
    case 3: return full ? launch_paths_tc_kb<3, true>(a, s) : launch_paths_tc_kb<3, false>(a, s);
    default: return full ? launch_paths_tc_kb<4, true>(a, s) : launch_paths_tc_kb<4, false>(a, s);
  }
}

template <typename T>
size_t wide_l_bytes(int dim) {
  return ((size_t)dim * dim * sizeof(T) + 15) & ~(size_t)15;
}

template <typename T>
int launch_paths_wide(const tqf_mvgbm_args& a, cudaStream_t s) {
  const bool ls = wide_l_bytes<T>(a.dim) <= kWideLSmem;
  const size_t smem = (ls ? wide_l_bytes<T>(a.dim) : 0) + (size_t)kWideWarps * 2 * a.dim * sizeof(T);
  TQF_REQUIRE(smem <= 200 * 1024, "tqf_mvgbm_paths: dim %d needs %zu bytes of shared memory (max 200 KiB)",
              a.dim, smem);
  auto k = ls ? mvgbm_paths_wide_kernel<T, true> : mvgbm_paths_wide_kernel<T, false>;
  set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBlock, smem) != cudaSuccess || occ < 1) occ = 1;
  int64_t grid = (a.num_paths + kWideWarps - 1) / kWideWarps;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  k<<<(unsigned)grid, kBlock, smem, s>>>(a);
  return check_launch("mvgbm_paths_wide_kernel");
}

template <typename T>
size_t basket_wide_smem(int dim, bool* ls_out) {
  const bool ls = wide_l_bytes<T>(dim) <= kWideLSmem;
  if (ls_out) *ls_out = ls;
  return (ls ? wide_l_bytes<T>(dim) : 0) + (size_t)kWideWarps * (2 + 2 * (size_t)dim) * sizeof(double) +
         (size_t)kWideWarps * 2 * dim * sizeof(T);
}

template <typename T>
int basket_wide_grid(int dim, int64_t n) {
  bool ls = true;
  const size_t smem = basket_wide_smem<T>(dim, &ls);
  auto k = ls ? basket_price_wide_kernel<T, true> : basket_price_wide_kernel<T, false>;
  set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBlock, smem) != cudaSuccess || occ < 1) occ = 1;
  int64_t grid = (n + kWideWarps - 1) / kWideWarps;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  return (int)grid;
}

template <typename T>
int launch_basket_wide(const tqf_basket_args& a, cudaStream_t s) {
  bool ls = true;
  const size_t smem = basket_wide_smem<T>(a.dim, &ls);
  TQF_REQUIRE(smem <= 200 * 1024, "tqf_basket_price: dim %d needs %zu bytes of shared memory (max 200 KiB)",
              a.dim, smem);
  const int grid = basket_wide_grid<T>(a.dim, a.num_paths);
  const int width = 2 + 2 * a.dim;
  const size_t need = (size_t)grid * width * sizeof(double);
  TQF_REQUIRE(a.workspace && a.workspace_bytes >= need, "tqf_basket_price: workspace %zu < required %zu",
              a.workspace_bytes, need);
  auto k = ls ? basket_price_wide_kernel<T, true> : basket_price_wide_kernel<T, false>;
  k<<<grid, kBlock, smem, s>>>(a);
  int rc = check_launch("basket_price_wide_kernel");
  if (rc || a.out == nullptr) return rc;
  return reduce_partials(static_cast<const double*>(a.workspace), grid, width, a.out, s);
}

template <typename T>
int dispatch_paths(const tqf_mvgbm_args& a, cudaStream_t s) {
  // Tensor-core L z (split BF16) for 16 to 64 correlated float32 factors.
  if (sizeof(T) == 4 && a.dim >= 16 && a.dim <= 16 * kLzMaxKB && a.chol != nullptr && a.lz_mode != 1 &&
      (reinterpret_cast<uintptr_t>(a.output.ptr) & 15u) == 0)
    return launch_paths_tc(a, s);
  if (a.dim <= 1) return launch_paths<T, 1>(a, s);
  if (a.dim <= 2) return launch_paths<T, 2>(a, s);
  if (a.dim == 3) return launch_paths<T, 3>(a, s);
  if (a.dim <= 4) return launch_paths<T, 4>(a, s);
  if (a.dim <= 8) return launch_paths<T, 8>(a, s);
  if (a.dim <= 16) return launch_paths<T, 16>(a, s);
  return launch_paths_wide<T>(a, s);
}

template <typename T>
int dispatch_basket(const tqf_basket_args& a, cudaStream_t s) {
  if (a.dim <= 4) return launch_basket<T, 4>(a, s);
  if (a.dim <= 8) return launch_basket<T, 8>(a, s);
  if (a.dim <= 16) return launch_basket<T, 16>(a, s);
  return launch_basket_wide<T>(a, s);
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_cholesky_f64(const double* a, int32_t n, double* l, int32_t* info, void* stream) {
  clear_error();
  TQF_REQUIRE(a && l && info, "tqf_cholesky_f64: null pointer");
  TQF_REQUIRE(n >= 1, "tqf_cholesky_f64: n must be >= 1, got %d", n);
  if (n <= kCholMax) {
    cholesky_f64_kernel<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, n, l, info);
    return check_launch("cholesky_f64_kernel");
  }
  cholesky_f64_global_kernel<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, n, l, info);
  return check_launch("cholesky_f64_global_kernel");
}

extern "C" int tqf_mvgbm_paths(const tqf_mvgbm_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_mvgbm_paths: null args");
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "tqf_mvgbm_paths: bad dtype");
  TQF_REQUIRE(a->dim >= 1, "tqf_mvgbm_paths: dim must be >= 1, got %d", a->dim);
  TQF_REQUIRE(a->num_paths >= 1 && a->num_steps >= 0, "tqf_mvgbm_paths: bad sizes");
  TQF_REQUIRE(a->x0 && a->drift && a->vol && (a->num_steps == 0 || a->step_table),
              "tqf_mvgbm_paths: null pointer");
  TQF_REQUIRE(a->output.ptr && a->output.num_slots >= 1 && a->output.init_slot < a->output.num_slots,
              "tqf_mvgbm_paths: output required");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr || a->num_steps == 0,
              "tqf_mvgbm_paths: memory draws need draws.ptr");
  TQF_REQUIRE(!a->draws.antithetic || 2 * a->draws.antithetic_half == a->num_paths,
              "tqf_mvgbm_paths: antithetic needs num_paths == 2 * antithetic_half");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? dispatch_paths<float>(*a, s) : dispatch_paths<double>(*a, s);
}

extern "C" int tqf_basket_price(const tqf_basket_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_basket_price: null args");
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "tqf_basket_price: bad dtype");
  TQF_REQUIRE(a->dim >= 1, "tqf_basket_price: dim must be >= 1, got %d", a->dim);
  TQF_REQUIRE(a->num_paths >= 1 && a->num_steps >= 1, "tqf_basket_price: bad sizes");
  TQF_REQUIRE(a->sqrt_dt && a->spot && a->drift && a->vol && a->weights, "tqf_basket_price: null pointer");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr, "tqf_basket_price: memory draws need ptr");
  TQF_REQUIRE(!a->draws.antithetic || 2 * a->draws.antithetic_half == a->num_paths,
              "tqf_basket_price: antithetic needs num_paths == 2 * antithetic_half");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? dispatch_basket<float>(*a, s) : dispatch_basket<double>(*a, s);
}

extern "C" size_t tqf_basket_workspace_bytes(int32_t dtype, int32_t dim, int64_t num_paths) {
  int grid;
  if (dim > 16) {
    grid = dtype == TQF_F32 ? basket_wide_grid<float>(dim, num_paths) : basket_wide_grid<double>(dim, num_paths);
    return (size_t)grid * (2 + 2 * (size_t)dim) * sizeof(double);
  }
  if (dim <= 4) grid = dtype == TQF_F32 ? basket_grid<float, 4>(num_paths) : basket_grid<double, 4>(num_paths);
  else if (dim <= 8) grid = dtype == TQF_F32 ? basket_grid<float, 8>(num_paths) : basket_grid<double, 8>(num_paths);
  else grid = dtype == TQF_F32 ? basket_grid<float, 16>(num_paths) : basket_grid<double, 16>(num_paths);
  return (size_t)grid * (2 + 2 * dim) * sizeof(double);
}
