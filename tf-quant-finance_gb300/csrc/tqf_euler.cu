// Euler–Maruyama kernels (tff/models/euler_sampling.py:335-537).
//
// euler_affine_kernel: the whole while-loop of the reference fused into one
// pass for structured coefficients a(x) = m + M x, B(x)_ij = (s0_i + s1_i x_i)
// C_ij — state in registers, the step table (dt, sqrt dt, output slot)
// staged by TMA into shared memory, draws read with strides or generated
// in-kernel, recorded states stored at their slots.
//
// euler_update_kernel: one step x + dt a + B (z sqrt dt) for coefficients the
// caller evaluated itself (arbitrary drift_fn / volatility_fn).
#include "tqf_internal.cuh"

namespace tqf {
namespace {

constexpr int kBlock = 256;
constexpr int kCols = 4;

template <typename T, int DM>
struct AffineCoef {
  T m[DM], M[DM * DM], s0[DM], s1[DM], C[DM * DM];
};

// Shared memory: mbarrier, coefficients, the staged step table, then (STAGE)
// the output staging buffer.
template <typename T, int DM>
__host__ __device__ inline size_t affine_stage_offset(int steps, bool staged) {
  const size_t head = (16 + sizeof(AffineCoef<T, DM>) + 15) & ~(size_t)15;
  return (head + (staged ? (size_t)steps * kCols * sizeof(T) : 0) + 15) & ~(size_t)15;
}

// x <- x + dt (m + M x) + (s0 + s1 x) (C dw): rows in order, columns summed
// in order (padding rows and columns are zero).
template <typename T, int DM>
__device__ __forceinline__ void affine_advance(const AffineCoef<T, DM>& cf, T (&x)[DM], const T (&dw)[DM], T dt) {
  T xn[DM];
#pragma unroll
  for (int r = 0; r < DM; ++r) {
    T drift = cf.m[r];
    T y = T(0);
#pragma unroll
    for (int c = 0; c < DM; ++c) {
      drift += cf.M[r * DM + c] * x[c];
      y += cf.C[r * DM + c] * dw[c];
    }
    const T vol = cf.s0[r] + cf.s1[r] * x[r];
    xn[r] = x[r] + dt * drift + vol * y;
  }
#pragma unroll
  for (int r = 0; r < DM; ++r) x[r] = xn[r];
}

// STAGE: 0 = each thread stores its own recorded states; 1 = through the
// coalescing RowStager (chosen when a path's output row is long enough for
// scattered stores to cost more than the stager's registers and shared
// memory); 2 = WarpRowStager (every step declared recorded in order: no
// per-step slot lookup, 128-byte row pieces per store instruction, no CTA
// barrier).
template <typename T, int DM, int SRC, int STAGE>
__global__ void __launch_bounds__(kBlock)
    euler_affine_kernel(tqf_euler_affine_args a, int staged) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  AffineCoef<T, DM>* coef = reinterpret_cast<AffineCoef<T, DM>*>(smem + 16);
  unsigned char* tab_raw = smem + ((16 + sizeof(AffineCoef<T, DM>) + 15) & ~(size_t)15);
  const int dim = a.dim;
  for (int i = threadIdx.x; i < DM; i += kBlock) {
    const bool in = i < dim;
    coef->m[i] = in ? static_cast<const T*>(a.drift_m)[i] : T(0);
    coef->s0[i] = in ? static_cast<const T*>(a.vol_s0)[i] : T(0);
    coef->s1[i] = in ? static_cast<const T*>(a.vol_s1)[i] : T(0);
  }
  for (int i = threadIdx.x; i < DM * DM; i += kBlock) {
    const int r = i / DM, c = i % DM;
    const bool in = r < dim && c < dim;
    coef->M[i] = in ? static_cast<const T*>(a.drift_M)[r * dim + c] : T(0);
    coef->C[i] = in ? static_cast<const T*>(a.vol_C)[r * dim + c] : T(0);
  }
  const int steps = a.num_steps;
  const T* table = static_cast<const T*>(a.step_table);
  if (staged) {
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    uint32_t phase = 0;
    if (!stage_to_smem(tab_raw, a.step_table, (uint32_t)(steps * kCols * sizeof(T)), bar, phase,
                       a.dev_status))
      return;
    table = reinterpret_cast<const T*>(tab_raw);
  } else {
    __syncthreads();
  }
  const int64_t N = a.num_paths;
  T* out = static_cast<T*>(a.output.ptr);
  const int ns = a.output.num_slots;
  if constexpr (STAGE == 2) {
    // verify the every-step declaration on the table (see tqf_path_output)
    const int base = a.output.init_slot >= 0 ? 1 : 0;
    int ok = (a.output.init_slot < 0 || a.output.init_slot == 0) && base + steps == ns;
    for (int i = threadIdx.x; i < steps; i += kBlock) ok &= (int)table[(size_t)i * kCols + 2] == base + i;
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0 && a.dev_status) atomicExch(a.dev_status, TQF_E_INVALID);
      return;
    }
  }
  // In-kernel Philox draws of exactly DM <= 4 components per step with the
  // table in shared memory: the loop walks whole Philox blocks (PhiloxGroup).
  // (From 8 factors on the step's matrix products outweigh the per-draw
  // block test, and the unrolled group would cost registers.)
  using PG = PhiloxGroup<T, DM>;
  constexpr bool kWhole = SRC == TQF_DRAWS_PHILOX && DM <= 4;
  const bool whole_blocks = kWhole && dim == DM && staged;
  // one-factor coefficients live in registers
  AffineCoef<T, DM> creg;
  if constexpr (DM == 1) creg = *coef;
  const AffineCoef<T, DM>* cf = DM == 1 ? &creg : coef;
  // with the RowStager every thread runs every round, with the warp stager
  // every lane of a warp that has a path (a thread past the last path
  // simulates that path again and its output is dropped)
  const bool stage_out = STAGE == 1 && out != nullptr;
  RowStager<T, DM, kBlock> stg(smem + affine_stage_offset<T, DM>(steps, staged != 0), dim);
  WarpRowStager wst(smem + affine_stage_offset<T, DM>(steps, staged != 0));
  uint32_t* out_words = reinterpret_cast<uint32_t*>(out);
  const int64_t row_words = (int64_t)ns * dim * (int64_t)(sizeof(T) / 4);
  const int64_t per_round = (int64_t)gridDim.x * kBlock;
  for (int64_t base = 0; base < N; base += per_round) {
    const int64_t row0 = base + (int64_t)blockIdx.x * kBlock;
    const int64_t path = row0 + threadIdx.x;
    const int64_t warp0 = row0 + (threadIdx.x & ~31);
    if (STAGE == 2 ? warp0 >= N : (path >= N && !stage_out)) break;
    const int64_t pc = path < N ? path : N - 1;
    T x[DM];
    const T* x0 = static_cast<const T*>(a.x0) + (a.x0_per_path ? pc * dim : 0);
#pragma unroll
    for (int j = 0; j < DM; ++j) x[j] = j < dim ? x0[j] : T(0);
    if constexpr (STAGE == 2) wst.begin();
    if (out && a.output.init_slot >= 0) {
      if constexpr (STAGE == 2) {
        wst.put<T, DM>(x, dim, out_words, row_words, warp0, N);
      } else if (stage_out) {
        stg.put(out, ns, row0, N, a.output.init_slot, x);
      } else {
        T* o = out + (path * ns + a.output.init_slot) * dim;
#pragma unroll
        for (int j = 0; j < DM; ++j)
          if (j < dim) o[j] = x[j];
      }
    }
    // records the state after step i at its slot (STAGE 2: every step, in order)
    auto record = [&](int i) {
      if constexpr (STAGE == 2) {
        wst.put<T, DM>(x, dim, out_words, row_words, warp0, N);
      } else {
        const int slot = (int)table[(size_t)i * kCols + 2];
        if (out && slot >= 0) {
          if (stage_out) {
            stg.put(out, ns, row0, N, slot, x);
          } else {
            T* o = out + (path * ns + slot) * dim;
#pragma unroll
            for (int j = 0; j < DM; ++j)
              if (j < dim) o[j] = x[j];
          }
        }
      }
    };
    DrawSource<T> src(a.draws, pc, dim);
    if (kWhole && whole_blocks) {
      // dw = z (sign sqrt dt) equals (sign z) sqrt dt exactly (sign = +-1);
      // the warp stager makes room for a whole group's words at once
      constexpr int kGroupWords = PG::kNormals * (int)(sizeof(T) / 4);
      static_assert(kGroupWords <= 32, "a group's words fit one piece");
      for (int i = 0; i < steps; i += PG::kSteps) {
        if constexpr (STAGE == 2) wst.make_room(kGroupWords, out_words, row_words, warp0, N);
        T z[PG::kNormals];
#pragma unroll
        for (int s = 0; s < PG::kSteps; ++s) {
          if (PG::kSteps > 1 && i + s >= steps) break;
          PG::fill_step(i / PG::kSteps, s, src.rng.path, src.rng.k0, src.rng.k1, z);
          T dt, sdt;
          step_pair<false>(table + (size_t)(i + s) * kCols, dt, sdt);
          sdt *= src.sign;
          T dw[DM];
#pragma unroll
          for (int c = 0; c < DM; ++c) dw[c] = z[s * DM + c] * sdt;
          affine_advance<T, DM>(*cf, x, dw, dt);
          if constexpr (STAGE == 2) {
            wst.append<T, DM>(x);
          } else {
            record(i + s);
          }
        }
      }
    } else {
      for (int i = 0; i < steps; ++i) {
        const T* row = table + (size_t)i * kCols;
        const T dt = row[0], sdt = row[1];
        T dw[DM];
#pragma unroll
        for (int c = 0; c < DM; ++c) dw[c] = c < dim ? src.get(i, c) * sdt : T(0);
        affine_advance<T, DM>(*cf, x, dw, dt);
        record(i);
      }
    }
    if (stage_out && stg.cnt > 0) stg.flush(out, ns, row0, N);
    if (STAGE == 2 && wst.nw > 0) wst.flush(out_words, row_words, warp0, N);
  }
}

template <typename T, int DM>
__global__ void __launch_bounds__(kBlock) euler_update_kernel(tqf_euler_update_args a) {
  const int64_t path = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (path >= a.num_paths) return;
  const int dim = a.dim;
  const T* x = static_cast<const T*>(a.x) + path * dim;
  const T* drift = static_cast<const T*>(a.drift) + path * dim;
  const T* vol = static_cast<const T*>(a.vol) + path * dim * dim;
  DrawSource<T> src(a.draws, path, dim);
  const T dt = (T)a.dt, sdt = (T)a.sqrt_dt;
  T dw[DM];
#pragma unroll
  for (int c = 0; c < DM; ++c) dw[c] = c < dim ? src.get(a.step, c) * sdt : T(0);
  T* xn = static_cast<T*>(a.x_next) + path * dim;
  T* po = a.paths_out && a.out_slot >= 0
              ? static_cast<T*>(a.paths_out) + (path * a.num_slots + a.out_slot) * dim
              : nullptr;
#pragma unroll
  for (int r = 0; r < DM; ++r) {
    if (r < dim) {
      T y = T(0);
#pragma unroll
      for (int c = 0; c < DM; ++c)
        if (c < dim) y += vol[r * dim + c] * dw[c];
      const T v = x[r] + dt * drift[r] + y;
      xn[r] = v;
      if (po) po[r] = v;
    }
  }
}

// ---- any dimension: one warp per path ---------------------------------------
// For dim > 16 the state no longer fits a thread's registers.  A warp carries
// one path: lane l owns state rows r = l, l + 32, ...; each step the warp
// writes its scaled draws dw = z sqrt(dt) and its state into per-warp shared
// buffers, every lane forms its rows' drift m_r + sum_c M_rc x_c and
// y_r = sum_c C_rc dw_c (M and C stored transposed, so the lanes of a warp
// read consecutive words; summed in column order as the register kernel
// does), and writes x'_r = x_r + dt drift + (s0_r + s1_r x_r) y_r into the
// second state buffer.  Recorded rows are stored by consecutive lanes, i.e.
// coalesced.  Coefficients sit in shared memory when they fit
// (kWideCoefSmem), else they are read from global memory (L2-resident).
constexpr int kWideWarps = kBlock / 32;
constexpr size_t kWideCoefSmem = 96 * 1024;

template <typename T>
size_t wide_coef_bytes(int dim) {
  return ((size_t)2 * dim * dim + 3 * (size_t)dim) * sizeof(T);
}
template <typename T>
size_t wide_warp_bytes(int dim) {
  return (size_t)3 * dim * sizeof(T);
}

// CS: coefficients copied (M and C transposed) into shared memory; else read
// row-major from global memory.
template <typename T, int SRC, bool CS>
__global__ void __launch_bounds__(kBlock) euler_affine_wide_kernel(tqf_euler_affine_args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int dim = a.dim;
  const size_t dd = (size_t)dim * dim;
  const T* gM = static_cast<const T*>(a.drift_M);
  const T* gC = static_cast<const T*>(a.vol_C);
  const T* m = static_cast<const T*>(a.drift_m);
  const T* s0 = static_cast<const T*>(a.vol_s0);
  const T* s1 = static_cast<const T*>(a.vol_s1);
  T* cs = reinterpret_cast<T*>(smem);
  size_t off = 0;
  if (CS) {
    // cs = Mt [dim][dim] (Mt[c][r] = M[r][c]), Ct, m, s0, s1
    for (size_t i = threadIdx.x; i < dd; i += kBlock) {
      const size_t r = i / dim, c = i - r * dim;
      cs[c * dim + r] = gM[i];
      cs[dd + c * dim + r] = gC[i];
    }
    for (int i = threadIdx.x; i < dim; i += kBlock) {
      cs[2 * dd + i] = m[i];
      cs[2 * dd + dim + i] = s0[i];
      cs[2 * dd + 2 * dim + i] = s1[i];
    }
    m = cs + 2 * dd;
    s0 = m + dim;
    s1 = s0 + dim;
    off = ((2 * dd + 3 * (size_t)dim) * sizeof(T) + 15) & ~(size_t)15;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* xs = reinterpret_cast<T*>(smem + off) + (size_t)warp * 3 * dim;
  T* xn = xs + dim;
  T* dws = xn + dim;
  __syncthreads();
  const T* table = static_cast<const T*>(a.step_table);
  T* out = static_cast<T*>(a.output.ptr);
  const int ns = a.output.num_slots;
  const int64_t N = a.num_paths;
  const int64_t nwarps = (int64_t)gridDim.x * kWideWarps;
  for (int64_t path = (int64_t)blockIdx.x * kWideWarps + warp; path < N; path += nwarps) {
    const T* x0 = static_cast<const T*>(a.x0) + (a.x0_per_path ? path * dim : 0);
    for (int r = lane; r < dim; r += 32) xs[r] = x0[r];
    if (out && a.output.init_slot >= 0) {
      T* o = out + (path * ns + a.output.init_slot) * dim;
      for (int r = lane; r < dim; r += 32) o[r] = xs[r];
    }
    DrawSource<T> src(a.draws, path, dim);
    for (int i = 0; i < a.num_steps; ++i) {
      const T* row = table + (size_t)i * kCols;
      const T dt = row[0], sdt = row[1];
      const int slot = (int)row[2];
      for (int c = lane; c < dim; c += 32) dws[c] = src.get(i, c) * sdt;
      __syncwarp();
      for (int r = lane; r < dim; r += 32) {
        T drift = m[r];
        T y = T(0);
        for (int c = 0; c < dim; ++c) {
          const T mv = CS ? cs[(size_t)c * dim + r] : gM[(size_t)r * dim + c];
          const T cv = CS ? cs[dd + (size_t)c * dim + r] : gC[(size_t)r * dim + c];
          drift += mv * xs[c];
          y += cv * dws[c];
        }
        const T vol = s0[r] + s1[r] * xs[r];
        xn[r] = xs[r] + dt * drift + vol * y;
      }
      __syncwarp();
      T* t = xs;
      xs = xn;
      xn = t;
      if (out && slot >= 0) {
        T* o = out + (path * ns + slot) * dim;
        for (int r = lane; r < dim; r += 32) o[r] = xs[r];
      }
    }
    __syncwarp();
  }
}

// One Euler step, any dimension: one warp per path; the scaled draws go to a
// per-warp shared buffer, then for each row r the warp reads B[r][:]
// coalesced, reduces y_r = sum_c B_rc dw_c across its lanes and lane r % 32
// writes x + dt a + y.
template <typename T>
__global__ void __launch_bounds__(kBlock) euler_update_wide_kernel(tqf_euler_update_args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int dim = a.dim;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* dws = reinterpret_cast<T*>(smem) + (size_t)warp * dim;
  const int64_t path = (int64_t)blockIdx.x * kWideWarps + warp;
  if (path >= a.num_paths) return;
  const T* x = static_cast<const T*>(a.x) + path * dim;
  const T* drift = static_cast<const T*>(a.drift) + path * dim;
  const T* vol = static_cast<const T*>(a.vol) + path * (int64_t)dim * dim;
  const T dt = (T)a.dt, sdt = (T)a.sqrt_dt;
  DrawSource<T> src(a.draws, path, dim);
  for (int c = lane; c < dim; c += 32) dws[c] = src.get(a.step, c) * sdt;
  __syncwarp();
  T* xn = static_cast<T*>(a.x_next) + path * dim;
  T* po = a.paths_out && a.out_slot >= 0
              ? static_cast<T*>(a.paths_out) + (path * a.num_slots + a.out_slot) * dim
              : nullptr;
  for (int r = 0; r < dim; ++r) {
    T y = T(0);
    for (int c = lane; c < dim; c += 32) y += vol[(size_t)r * dim + c] * dws[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
    if (lane == (r & 31)) {
      const T v = x[r] + dt * drift[r] + y;
      xn[r] = v;
      if (po) po[r] = v;
    }
  }
}

template <typename T>
int launch_affine_wide(const tqf_euler_affine_args& a, cudaStream_t s) {
  const int dim = a.dim;
  const size_t cbytes = (wide_coef_bytes<T>(dim) + 15) & ~(size_t)15;
  const bool cs = cbytes <= kWideCoefSmem;
  const size_t smem = (cs ? cbytes : 0) + kWideWarps * wide_warp_bytes<T>(dim);
  TQF_REQUIRE(smem <= 200 * 1024, "tqf_euler_affine: dim %d needs %zu bytes of shared memory (max 200 KiB)", dim,
              smem);
  const bool philox = a.draws.source == TQF_DRAWS_PHILOX;
  void (*k)(tqf_euler_affine_args) =
      cs ? (philox ? euler_affine_wide_kernel<T, TQF_DRAWS_PHILOX, true> : euler_affine_wide_kernel<T, TQF_DRAWS_MEMORY, true>)
         : (philox ? euler_affine_wide_kernel<T, TQF_DRAWS_PHILOX, false> : euler_affine_wide_kernel<T, TQF_DRAWS_MEMORY, false>);
  set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBlock, smem) != cudaSuccess || occ < 1) occ = 1;
  int64_t grid = (a.num_paths + kWideWarps - 1) / kWideWarps;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  k<<<(unsigned)grid, kBlock, smem, s>>>(a);
  return check_launch("euler_affine_wide_kernel");
}

template <typename T, int DM>
int launch_affine(const tqf_euler_affine_args& a, cudaStream_t s) {
  const size_t tab_bytes = (size_t)a.num_steps * kCols * sizeof(T);
  const bool staged = tab_bytes > 0 && tab_bytes <= 96 * 1024 &&
                      (reinterpret_cast<uintptr_t>(a.step_table) & 15u) == 0;
  // the warp stager for every-step outputs; else stage the output when a
  // path's row is at least 64 bytes
  const size_t row = (size_t)a.output.num_slots * a.dim * sizeof(T);
  const bool warp_rows = a.output.ptr != nullptr && a.output.every_step &&
                         (reinterpret_cast<uintptr_t>(a.output.ptr) & (sizeof(T) - 1)) == 0;
  const bool stage_out = !warp_rows && a.output.ptr != nullptr && row >= 64;
  const size_t smem = affine_stage_offset<T, DM>(a.num_steps, staged) +
                      (warp_rows ? WarpRowStager::bytes(kBlock / 32)
                                 : (stage_out ? RowStager<T, DM, kBlock>::kBytes : 0));
  const bool philox = a.draws.source == TQF_DRAWS_PHILOX;
  void (*k)(tqf_euler_affine_args, int) =
      stage_out ? (philox ? euler_affine_kernel<T, DM, TQF_DRAWS_PHILOX, 1>
                          : euler_affine_kernel<T, DM, TQF_DRAWS_MEMORY, 1>)
                : (philox ? euler_affine_kernel<T, DM, TQF_DRAWS_PHILOX, 0>
                          : euler_affine_kernel<T, DM, TQF_DRAWS_MEMORY, 0>);
  if (warp_rows)
    k = philox ? euler_affine_kernel<T, DM, TQF_DRAWS_PHILOX, 2> : euler_affine_kernel<T, DM, TQF_DRAWS_MEMORY, 2>;
  if (smem > 48 * 1024) set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBlock, smem) != cudaSuccess || occ < 1)
    occ = 1;
  int64_t grid = (a.num_paths + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  k<<<(unsigned)grid, kBlock, smem, s>>>(a, staged ? 1 : 0);
  return check_launch("euler_affine_kernel");
}

template <typename T>
int dispatch_affine(const tqf_euler_affine_args& a, cudaStream_t s) {
  if (a.dim <= 1) return launch_affine<T, 1>(a, s);
  if (a.dim <= 2) return launch_affine<T, 2>(a, s);
  if (a.dim == 3) return launch_affine<T, 3>(a, s);
  if (a.dim <= 4) return launch_affine<T, 4>(a, s);
  if (a.dim <= 8) return launch_affine<T, 8>(a, s);
  if (a.dim <= 16) return launch_affine<T, 16>(a, s);
  return launch_affine_wide<T>(a, s);
}

template <typename T>
int dispatch_update(const tqf_euler_update_args& a, cudaStream_t s) {
  if (a.dim > 16) {
    const int64_t grid = (a.num_paths + kWideWarps - 1) / kWideWarps;
    TQF_REQUIRE(grid <= 2147483647LL, "tqf_euler_update: too many paths");
    const size_t smem = (size_t)kWideWarps * a.dim * sizeof(T);
    TQF_REQUIRE(smem <= 200 * 1024, "tqf_euler_update: dim %d too large (max %d)", a.dim,
                (int)(200 * 1024 / (kWideWarps * sizeof(T))));
    set_smem_config(euler_update_wide_kernel<T>, smem);
    euler_update_wide_kernel<T><<<(unsigned)grid, kBlock, smem, s>>>(a);
    return check_launch("euler_update_wide_kernel");
  }
  const int64_t grid = (a.num_paths + kBlock - 1) / kBlock;
  TQF_REQUIRE(grid <= 2147483647LL, "tqf_euler_update: too many paths");
  if (a.dim <= 1) euler_update_kernel<T, 1><<<(unsigned)grid, kBlock, 0, s>>>(a);
  else if (a.dim <= 2) euler_update_kernel<T, 2><<<(unsigned)grid, kBlock, 0, s>>>(a);
  else if (a.dim <= 4) euler_update_kernel<T, 4><<<(unsigned)grid, kBlock, 0, s>>>(a);
  else if (a.dim <= 8) euler_update_kernel<T, 8><<<(unsigned)grid, kBlock, 0, s>>>(a);
  else euler_update_kernel<T, 16><<<(unsigned)grid, kBlock, 0, s>>>(a);
  return check_launch("euler_update_kernel");
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_euler_affine(const tqf_euler_affine_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_euler_affine: null args");
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "tqf_euler_affine: bad dtype %d", a->dtype);
  TQF_REQUIRE(a->dim >= 1, "tqf_euler_affine: dim must be >= 1, got %d", a->dim);
  TQF_REQUIRE(a->num_paths >= 1 && a->num_steps >= 0, "tqf_euler_affine: bad sizes");
  TQF_REQUIRE(a->x0 && a->drift_m && a->drift_M && a->vol_s0 && a->vol_s1 && a->vol_C,
              "tqf_euler_affine: null coefficient pointer");
  TQF_REQUIRE(a->num_steps == 0 || a->step_table, "tqf_euler_affine: null step_table");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr || a->num_steps == 0,
              "tqf_euler_affine: memory draws need draws.ptr");
  TQF_REQUIRE(!a->draws.antithetic || 2 * a->draws.antithetic_half == a->num_paths,
              "tqf_euler_affine: antithetic needs num_paths == 2 * antithetic_half");
  TQF_REQUIRE(!a->output.ptr || (a->output.num_slots >= 1 && a->output.init_slot < a->output.num_slots),
              "tqf_euler_affine: bad output slots");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? dispatch_affine<float>(*a, s) : dispatch_affine<double>(*a, s);
}

extern "C" int tqf_euler_update(const tqf_euler_update_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_euler_update: null args");
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "tqf_euler_update: bad dtype %d", a->dtype);
  TQF_REQUIRE(a->dim >= 1, "tqf_euler_update: dim must be >= 1, got %d", a->dim);
  TQF_REQUIRE(a->num_paths >= 1, "tqf_euler_update: num_paths must be >= 1");
  TQF_REQUIRE(a->x && a->drift && a->vol && a->x_next, "tqf_euler_update: null pointer");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr,
              "tqf_euler_update: memory draws need draws.ptr");
  TQF_REQUIRE(!a->paths_out || a->out_slot < a->num_slots, "tqf_euler_update: out_slot out of range");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? dispatch_update<float>(*a, s) : dispatch_update<double>(*a, s);
}
