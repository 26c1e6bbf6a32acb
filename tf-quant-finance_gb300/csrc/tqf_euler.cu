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

// STAGE: recorded states go through the coalescing RowStager (chosen when a
// path's output row is long enough for scattered stores to cost more than
// the stager's registers and shared memory).
template <typename T, int DM, int SRC, bool STAGE>
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
  // with the stager every thread runs every round (a thread past the last
  // path simulates that path again and its output is dropped)
  const bool stage_out = STAGE && out != nullptr;
  RowStager<T, DM, kBlock> stg(smem + affine_stage_offset<T, DM>(steps, staged != 0), dim);
  const int64_t per_round = (int64_t)gridDim.x * kBlock;
  for (int64_t base = 0; base < N; base += per_round) {
    const int64_t row0 = base + (int64_t)blockIdx.x * kBlock;
    const int64_t path = row0 + threadIdx.x;
    if (path >= N && !stage_out) break;
    const int64_t pc = path < N ? path : N - 1;
    T x[DM];
    const T* x0 = static_cast<const T*>(a.x0) + (a.x0_per_path ? pc * dim : 0);
#pragma unroll
    for (int j = 0; j < DM; ++j) x[j] = j < dim ? x0[j] : T(0);
    if (out && a.output.init_slot >= 0) {
      if (stage_out) {
        stg.put(out, ns, row0, N, a.output.init_slot, x);
      } else {
        T* o = out + (path * ns + a.output.init_slot) * dim;
#pragma unroll
        for (int j = 0; j < DM; ++j)
          if (j < dim) o[j] = x[j];
      }
    }
    DrawSource<T> src(a.draws, pc, dim);
    for (int i = 0; i < steps; ++i) {
      const T* row = table + (size_t)i * kCols;
      const T dt = row[0], sdt = row[1];
      T dw[DM];
#pragma unroll
      for (int c = 0; c < DM; ++c) dw[c] = c < dim ? src.get(i, c) * sdt : T(0);
      T xn[DM];
#pragma unroll
      for (int r = 0; r < DM; ++r) {
        T drift = coef->m[r];
        T y = T(0);
#pragma unroll
        for (int c = 0; c < DM; ++c) {
          drift += coef->M[r * DM + c] * x[c];
          y += coef->C[r * DM + c] * dw[c];
        }
        const T vol = coef->s0[r] + coef->s1[r] * x[r];
        xn[r] = x[r] + dt * drift + vol * y;
      }
#pragma unroll
      for (int r = 0; r < DM; ++r) x[r] = xn[r];
      const int slot = (int)row[2];
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
    if (stage_out && stg.cnt > 0) stg.flush(out, ns, row0, N);
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

template <typename T, int DM>
int launch_affine(const tqf_euler_affine_args& a, cudaStream_t s) {
  const size_t tab_bytes = (size_t)a.num_steps * kCols * sizeof(T);
  const bool staged = tab_bytes > 0 && tab_bytes <= 96 * 1024 &&
                      (reinterpret_cast<uintptr_t>(a.step_table) & 15u) == 0;
  // stage the output when a path's row is at least 64 bytes
  const bool stage_out =
      a.output.ptr != nullptr && (size_t)a.output.num_slots * a.dim * sizeof(T) >= 64;
  const size_t smem =
      affine_stage_offset<T, DM>(a.num_steps, staged) + (stage_out ? RowStager<T, DM, kBlock>::kBytes : 0);
  const bool philox = a.draws.source == TQF_DRAWS_PHILOX;
  void (*k)(tqf_euler_affine_args, int) =
      stage_out ? (philox ? euler_affine_kernel<T, DM, TQF_DRAWS_PHILOX, true>
                          : euler_affine_kernel<T, DM, TQF_DRAWS_MEMORY, true>)
                : (philox ? euler_affine_kernel<T, DM, TQF_DRAWS_PHILOX, false>
                          : euler_affine_kernel<T, DM, TQF_DRAWS_MEMORY, false>);
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
  if (a.dim <= 4) return launch_affine<T, 4>(a, s);
  if (a.dim <= 8) return launch_affine<T, 8>(a, s);
  return launch_affine<T, 16>(a, s);
}

template <typename T>
int dispatch_update(const tqf_euler_update_args& a, cudaStream_t s) {
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
  TQF_REQUIRE(a->dim >= 1 && a->dim <= 16, "tqf_euler_affine: dim must be in [1, 16], got %d", a->dim);
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
  TQF_REQUIRE(a->dim >= 1 && a->dim <= 16, "tqf_euler_update: dim must be in [1, 16], got %d", a->dim);
  TQF_REQUIRE(a->num_paths >= 1, "tqf_euler_update: num_paths must be >= 1");
  TQF_REQUIRE(a->x && a->drift && a->vol && a->x_next, "tqf_euler_update: null pointer");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr,
              "tqf_euler_update: memory draws need draws.ptr");
  TQF_REQUIRE(!a->paths_out || a->out_slot < a->num_slots, "tqf_euler_update: out_slot out of range");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? dispatch_update<float>(*a, s) : dispatch_update<double>(*a, s);
}
