// Short-rate model path kernels — the GB300 replacement of the loops in
// tff/models/hull_white/vector_hull_white.py:641-781 (exact Hull-White
// transition) and tff/models/hjm/gaussian_hjm.py:404-457 (Gaussian HJM Euler).
//
// The reference evaluates the exact one-step transition with a tf.while_loop
// of whole-tensor ops per time step.  Here the per-step transition constants
// (decay, conditional mean increment, conditional standard deviation, forward
// rate, correlation factor) are tabulated once on the host and every thread
// carries one path's state vector in registers through all steps.
#include "tqf_internal.cuh"

namespace tqf {
namespace {

constexpr int kBlock = 256;

// STAGE: recorded rates go through the coalescing RowStager (dynamic shared
// memory), chosen when a path's output row is at least 64 bytes; then every
// thread runs every round and a thread past the last path simulates that path
// again with its output dropped.
// Per-step tables in shared memory (when they fit): transition constants
// [steps][d][3], forward rates [steps + 1][d], Cholesky factors [steps][d][d]
// (optional) and output slots [steps], each 16-byte aligned.
template <typename T>
struct HwTables {
  size_t tab, f0, chol, slots, total;
};
template <typename T>
__host__ __device__ inline HwTables<T> hw_tables(int steps, int d, bool chol) {
  HwTables<T> t;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = (off + bytes + 15) & ~(size_t)15;
    return at;
  };
  t.tab = take((size_t)steps * d * 3 * sizeof(T));
  t.f0 = take((size_t)(steps + 1) * d * sizeof(T));
  t.chol = take(chol ? (size_t)steps * d * d * sizeof(T) : 0);
  t.slots = take((size_t)steps * sizeof(int32_t));
  t.total = off;
  return t;
}
constexpr size_t kHwMaxSmemTables = 64 * 1024;

template <typename T, int DM, bool STAGE>
__global__ void __launch_bounds__(kBlock) hull_white_kernel(tqf_hull_white_args a, int tables_in_smem) {
  extern __shared__ __align__(16) unsigned char stage_smem[];
  const int d = a.dim;
  const T* tab = static_cast<const T*>(a.table);
  const T* f0 = static_cast<const T*>(a.f0);
  const T* L = static_cast<const T*>(a.chol);
  const int32_t* slots = a.slots;
  size_t stage_off = 0;
  if (tables_in_smem) {
    const HwTables<T> lay = hw_tables<T>(a.num_steps, d, L != nullptr);
    T* s_tab = reinterpret_cast<T*>(stage_smem + lay.tab);
    T* s_f0 = reinterpret_cast<T*>(stage_smem + lay.f0);
    T* s_chol = reinterpret_cast<T*>(stage_smem + lay.chol);
    int32_t* s_slots = reinterpret_cast<int32_t*>(stage_smem + lay.slots);
    for (int i = threadIdx.x; i < a.num_steps * d * 3; i += kBlock) s_tab[i] = tab[i];
    for (int i = threadIdx.x; i < (a.num_steps + 1) * d; i += kBlock) s_f0[i] = f0[i];
    if (L)
      for (int i = threadIdx.x; i < a.num_steps * d * d; i += kBlock) s_chol[i] = L[i];
    for (int i = threadIdx.x; i < a.num_steps; i += kBlock) s_slots[i] = slots[i];
    __syncthreads();
    tab = s_tab;
    f0 = s_f0;
    if (L) L = s_chol;
    slots = s_slots;
    stage_off = lay.total;
  }
  T* out = static_cast<T*>(a.output.ptr);
  const int ns = a.output.num_slots;
  const int64_t N = a.num_paths;
  RowStager<T, DM, kBlock> stg(stage_smem + stage_off, d);
  const int64_t per_round = (int64_t)gridDim.x * kBlock;
  for (int64_t base = 0; base < N; base += per_round) {
    const int64_t row0 = base + (int64_t)blockIdx.x * kBlock;
    const int64_t path = row0 + threadIdx.x;
    if (!STAGE && path >= N) break;
    const int64_t pc = path < N ? path : N - 1;
    T x[DM];
#pragma unroll
    for (int k = 0; k < DM; ++k) x[k] = T(0);
    if (a.output.init_slot >= 0) {
      if constexpr (STAGE) {
        T r0[DM];
#pragma unroll
        for (int k = 0; k < DM; ++k) r0[k] = k < d ? f0[k] : T(0);
        stg.put(out, ns, row0, N, a.output.init_slot, r0);
      } else {
        T* o = out + (path * ns + a.output.init_slot) * d;
        for (int k = 0; k < d; ++k) o[k] = f0[k];
      }
    }
    DrawSource<T> src(a.draws, pc, d);
    for (int i = 0; i < a.num_steps; ++i) {
      T z[DM], y[DM];
#pragma unroll
      for (int c = 0; c < DM; ++c) z[c] = c < d ? src.get(i, c) : T(0);
      if (L) {
        const T* Li = L + (size_t)i * d * d;
#pragma unroll
        for (int r = 0; r < DM; ++r) {
          T s = T(0);
#pragma unroll
          for (int c = 0; c < DM; ++c)
            if (r < d && c <= r) s += Li[r * d + c] * z[c];
          y[r] = s;
        }
      } else {
#pragma unroll
        for (int r = 0; r < DM; ++r) y[r] = z[r];
      }
      const T* row = tab + (size_t)i * d * 3;
#pragma unroll
      for (int k = 0; k < DM; ++k)
        if (k < d) x[k] = row[3 * k] * x[k] + row[3 * k + 1] + row[3 * k + 2] * y[k];
      const int slot = slots[i];
      if (slot >= 0) {
        const T* f = f0 + (size_t)(i + 1) * d;
        if constexpr (STAGE) {
          T r[DM];
#pragma unroll
          for (int k = 0; k < DM; ++k) r[k] = k < d ? x[k] + f[k] : T(0);
          stg.put(out, ns, row0, N, slot, r);
        } else {
          T* o = out + (path * ns + slot) * d;
#pragma unroll
          for (int k = 0; k < DM; ++k)
            if (k < d) o[k] = x[k] + f[k];
        }
      }
    }
    if (STAGE && stg.cnt > 0) stg.flush(out, ns, row0, N);
  }
}

template <typename T, int DM>
int launch(const tqf_hull_white_args& a, cudaStream_t s) {
  // stage the output when a path's row is at least 64 bytes
  const bool stage = (size_t)a.output.num_slots * a.dim * sizeof(T) >= 64;
  auto k = stage ? hull_white_kernel<T, DM, true> : hull_white_kernel<T, DM, false>;
  const size_t tables = hw_tables<T>(a.num_steps, a.dim, a.chol != nullptr).total;
  const bool tables_in_smem = tables <= kHwMaxSmemTables;
  const size_t smem = (tables_in_smem ? tables : 0) + (stage ? RowStager<T, DM, kBlock>::kBytes : 0);
  if (smem > 48 * 1024) set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBlock, smem) != cudaSuccess || occ < 1) occ = 1;
  int64_t grid = (a.num_paths + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  k<<<(unsigned)grid, kBlock, smem, s>>>(a, tables_in_smem ? 1 : 0);
  return check_launch("hull_white_kernel");
}

template <typename T>
int dispatch(const tqf_hull_white_args& a, cudaStream_t s) {
  if (a.dim == 1) return launch<T, 1>(a, s);
  if (a.dim <= 2) return launch<T, 2>(a, s);
  if (a.dim <= 4) return launch<T, 4>(a, s);
  return launch<T, 16>(a, s);
}

// Gaussian HJM: Euler for the factors with the short rate and discount factor
// accumulated in registers (the reference stores every grid point and takes a
// cumulative product afterwards).
// STAGE: the recorded rates, discount factors and (when requested) factors go
// through coalescing RowStagers (dynamic shared memory), chosen when a path's
// rate row is at least 64 bytes; the three flush at the same slots.  Then
// every thread runs every round and a thread past the last path simulates
// that path again with its output dropped.
template <typename T, int DM, bool STAGE>
__global__ void __launch_bounds__(kBlock) hjm_kernel(tqf_hjm_args a) {
  extern __shared__ __align__(16) unsigned char stage_smem[];
  const int d = a.dim;
  const int W = 2 + d + d * d;
  const T* tab = static_cast<const T*>(a.table);
  const T* f0 = static_cast<const T*>(a.f0);
  const T* kk = static_cast<const T*>(a.mean_reversion);
  T* rate_out = static_cast<T*>(a.rate_out);
  T* df_out = static_cast<T*>(a.df_out);
  T* x_out = static_cast<T*>(a.x_out);
  const int ns = a.num_slots;
  const int64_t N = a.num_paths;
  RowStager<T, 1, kBlock> st_rate(stage_smem, 1);
  RowStager<T, 1, kBlock> st_df(stage_smem + RowStager<T, 1, kBlock>::kBytes, 1);
  RowStager<T, DM, kBlock> st_x(stage_smem + 2 * RowStager<T, 1, kBlock>::kBytes, d);
  T k[DM];
#pragma unroll
  for (int c = 0; c < DM; ++c) k[c] = c < d ? kk[c] : T(0);
  const int64_t per_round = (int64_t)gridDim.x * kBlock;
  for (int64_t base = 0; base < N; base += per_round) {
    const int64_t row0 = base + (int64_t)blockIdx.x * kBlock;
    const int64_t path = row0 + threadIdx.x;
    if (!STAGE && path >= N) break;
    const int64_t pc = path < N ? path : N - 1;
    T x[DM];
#pragma unroll
    for (int c = 0; c < DM; ++c) x[c] = T(0);
    T df = T(1);
    T rate = f0[0];  // sum of zero factors + f0(t_0)
    auto record = [&](int slot) {
      if constexpr (STAGE) {
        st_rate.put(rate_out, ns, row0, N, slot, &rate);
        st_df.put(df_out, ns, row0, N, slot, &df);
        if (x_out) st_x.put(x_out, ns, row0, N, slot, x);
      } else {
        rate_out[path * ns + slot] = rate;
        df_out[path * ns + slot] = df;
        if (x_out) {
#pragma unroll
          for (int c = 0; c < DM; ++c)
            if (c < d) x_out[(path * ns + slot) * d + c] = x[c];
        }
      }
    };
    int slot = a.grid_slot[0];
    if (slot >= 0) record(slot);
    DrawSource<T> src(a.draws, pc, d);
    for (int i = 0; i < a.num_steps; ++i) {
      const T* row = tab + (size_t)i * W;
      const T dt = row[0], sdt = row[1];
      df = df * exp(-rate * dt);
      T dw[DM], xn[DM];
#pragma unroll
      for (int c = 0; c < DM; ++c) dw[c] = c < d ? src.get(i, c) * sdt : T(0);
#pragma unroll
      for (int r = 0; r < DM; ++r) {
        if (r >= d) {
          xn[r] = T(0);
          continue;
        }
        T bw = T(0);
#pragma unroll
        for (int c = 0; c < DM; ++c)
          if (c < d) bw += row[2 + d + r * d + c] * dw[c];
        xn[r] = x[r] + dt * (row[2 + r] - k[r] * x[r]) + bw;
      }
      T s = T(0);
#pragma unroll
      for (int c = 0; c < DM; ++c) {
        x[c] = xn[c];
        s += x[c];
      }
      rate = s + f0[i + 1];
      slot = a.grid_slot[i + 1];
      if (slot >= 0) record(slot);
    }
    if (STAGE && st_rate.cnt > 0) {
      st_rate.flush(rate_out, ns, row0, N);
      st_df.flush(df_out, ns, row0, N);
      if (x_out) st_x.flush(x_out, ns, row0, N);
    }
  }
}

template <typename T, int DM>
int launch_hjm(const tqf_hjm_args& a, cudaStream_t s) {
  // stage the outputs when a path's rate row is at least 64 bytes
  const bool stage = (size_t)a.num_slots * sizeof(T) >= 64;
  auto k = stage ? hjm_kernel<T, DM, true> : hjm_kernel<T, DM, false>;
  const size_t smem = stage ? 2 * RowStager<T, 1, kBlock>::kBytes + (a.x_out ? RowStager<T, DM, kBlock>::kBytes : 0)
                            : 0;
  if (smem > 48 * 1024) set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBlock, smem) != cudaSuccess || occ < 1) occ = 1;
  int64_t grid = (a.num_paths + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  k<<<(unsigned)grid, kBlock, smem, s>>>(a);
  return check_launch("hjm_kernel");
}

template <typename T>
int dispatch_hjm(const tqf_hjm_args& a, cudaStream_t s) {
  if (a.dim == 1) return launch_hjm<T, 1>(a, s);
  if (a.dim <= 2) return launch_hjm<T, 2>(a, s);
  if (a.dim <= 4) return launch_hjm<T, 4>(a, s);
  return launch_hjm<T, 16>(a, s);
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_hjm_paths(const tqf_hjm_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_hjm_paths: null args");
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "tqf_hjm_paths: bad dtype %d", a->dtype);
  TQF_REQUIRE(a->dim >= 1 && a->dim <= 16, "tqf_hjm_paths: dim must be in [1, 16], got %d", a->dim);
  TQF_REQUIRE(a->num_paths >= 1 && a->num_steps >= 0 && a->num_slots >= 1, "tqf_hjm_paths: bad sizes");
  TQF_REQUIRE(a->table && a->mean_reversion && a->f0 && a->grid_slot && a->rate_out && a->df_out,
              "tqf_hjm_paths: null pointer");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr || a->num_steps == 0,
              "tqf_hjm_paths: memory draws need draws.ptr");
  TQF_REQUIRE(!a->draws.antithetic || 2 * a->draws.antithetic_half == a->num_paths,
              "tqf_hjm_paths: antithetic needs num_paths == 2 * antithetic_half");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? dispatch_hjm<float>(*a, s) : dispatch_hjm<double>(*a, s);
}

extern "C" int tqf_hull_white_paths(const tqf_hull_white_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_hull_white_paths: null args");
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "tqf_hull_white_paths: bad dtype %d", a->dtype);
  TQF_REQUIRE(a->dim >= 1 && a->dim <= 16, "tqf_hull_white_paths: dim must be in [1, 16], got %d", a->dim);
  TQF_REQUIRE(a->num_paths >= 1 && a->num_steps >= 0, "tqf_hull_white_paths: bad sizes");
  TQF_REQUIRE(a->f0 && (a->num_steps == 0 || (a->table && a->slots)), "tqf_hull_white_paths: null table");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr || a->num_steps == 0,
              "tqf_hull_white_paths: memory draws need draws.ptr");
  TQF_REQUIRE(!a->draws.antithetic || 2 * a->draws.antithetic_half == a->num_paths,
              "tqf_hull_white_paths: antithetic needs num_paths == 2 * antithetic_half");
  TQF_REQUIRE(a->output.ptr && a->output.num_slots >= 1 && a->output.init_slot < a->output.num_slots,
              "tqf_hull_white_paths: bad output");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? dispatch<float>(*a, s) : dispatch<double>(*a, s);
}
