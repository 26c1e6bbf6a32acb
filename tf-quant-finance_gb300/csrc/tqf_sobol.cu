// Sobol sequence kernels (natural order, index skip+1+n, nd-digit scaling) —
// the GB300 replacement of tff/math/random_ops/sobol/sobol_impl.py:39-167.
//
// The reference materialises an [nd, n, dim] product tensor and XOR-reduces
// it (O(nd·n·dim) memory).  Here every thread owns a few dimensions and walks
// points with a power-of-two stride 2^m: adding 2^m to the index i flips bits
// m..m+c of i, c = number of trailing ones of (i >> m), so
//     x(i + 2^m) = x(i) XOR G_m[c],   G_m[c] = v_m ^ v_{m+1} ^ ... ^ v_{m+c}.
// One table lookup and one XOR per element; only the first point of each
// thread is built directly (<= nd XORs).  The kernels are HBM-write bound.
#include "tqf_internal.cuh"

namespace tqf {
namespace {

constexpr int kThreads = 256;

template <int KIND>
struct SobolOut;
template <>
struct SobolOut<TQF_SOBOL_U32> {
  using T = uint32_t;
  __device__ static T conv(uint32_t x, float, double) { return x; }
};
template <>
struct SobolOut<TQF_SOBOL_F32> {
  using T = float;
  __device__ static T conv(uint32_t x, float sc, double) { return __fmul_rn(__uint2float_rn(x), sc); }
};
template <>
struct SobolOut<TQF_SOBOL_F64> {
  using T = double;
  __device__ static T conv(uint32_t x, float, double sc) { return (double)x * sc; }
};
template <>
struct SobolOut<TQF_SOBOL_NORMAL_F32> {
  using T = float;
  __device__ static T conv(uint32_t x, float sc, double) { return sobol_normal_f32(x, 2.0f * sc); }
};
template <>
struct SobolOut<TQF_SOBOL_NORMAL_F64> {
  using T = double;
  __device__ static T conv(uint32_t x, float, double sc) { return sobol_normal_f64(x, sc); }
};
template <>
struct SobolOut<TQF_SOBOL_F32_CENTERED> {
  using T = float;
  __device__ static T conv(uint32_t x, float sc, double) {
    // (x + 0.5) 2^-nd rounded to float32, kept below 1.0 (largest float < 1)
    return fminf(__fmul_rn(__fadd_rn(__uint2float_rn(x), 0.5f), sc), 0.99999994039535522461f);
  }
};

__device__ __forceinline__ uint32_t bits32(uint32_t x) { return x; }
__device__ __forceinline__ uint32_t bits32(float x) { return __float_as_uint(x); }
__device__ __forceinline__ uint32_t bits32(double) { return 0u; }  // never used (8-byte types take the scalar path)

__device__ __forceinline__ uint32_t sobol_direct(const uint32_t* __restrict__ v_row, uint32_t i,
                                                 int nd, int sh) {
  uint32_t x = 0;
  for (int j = 0; j < nd; ++j)
    if ((i >> j) & 1u) x ^= v_row[j];
  return x >> sh;
}

// ---- [n, dim] row-major output (sobol.sample) ---------------------------------
// Block = DX dim-threads x PT point-threads (PT = 2^mt); each thread owns VEC
// consecutive dims.  The grid's CTAs interleave row by row: CTA b takes rows
// PT (b + gridDim.x s) .. + PT - 1, so a thread's rows are 2^m = PT gridDim.x
// apart (gridDim.x a power of two) and at any time the whole grid writes one
// contiguous window of rows, as a fill does, which keeps the HBM writes
// sequential.  The walk table G_m holds the `levels` prefixes that the
// indices can reach (c <= bit length of (last index >> m)).
// Shape by output kind (measured on dim 1024): the store-bound outputs take
// whole rows per CTA (up to 1024 dims, ~2 CTAs per SM as the walk table
// allows), which keeps each row's 4 KB a single CTA's contiguous write; the
// inverse-normal outputs, bound by erfinv's arithmetic, take half-rows (512
// dims, half the table) and ~4 CTAs per SM for more resident warps.
__host__ __device__ constexpr bool arithmetic_bound(int kind) {
  return kind == TQF_SOBOL_NORMAL_F32 || kind == TQF_SOBOL_NORMAL_F64;
}
template <int KIND, int VEC>
__global__ void __launch_bounds__(kThreads)
    sobol_rowmajor_kernel(const uint32_t* __restrict__ v, int dim, int64_t n, uint32_t first_index,
                          int nd, int dx, int mt, int m, int levels, void* __restrict__ out_raw) {
  using T = typename SobolOut<KIND>::T;
  T* out = static_cast<T*>(out_raw);
  extern __shared__ uint32_t g_tab[];  // [levels][dx * VEC]
  const int sh = 32 - nd;
  const int width = dx * VEC;
  const int dim0 = blockIdx.y * width;
  for (int idx = threadIdx.x; idx < width; idx += blockDim.x) {
    const int d = dim0 + idx;
    uint32_t run = 0;
    for (int c = 0; c < levels; ++c) {
      if (d < dim) run ^= v[(size_t)d * 32 + m + c];
      g_tab[c * width + idx] = run >> sh;
    }
  }
  __syncthreads();
  const int tx = threadIdx.x % dx;
  const int py = threadIdx.x / dx;
  const int dl = tx * VEC;  // local dim
  const int d = dim0 + dl;
  const int64_t stride = (int64_t)1 << m;
  int64_t row = ((int64_t)blockIdx.x << mt) + py;
  uint32_t i = first_index + (uint32_t)row;
  uint32_t x[VEC];
#pragma unroll
  for (int e = 0; e < VEC; ++e) x[e] = (d + e < dim) ? sobol_direct(v + (size_t)(d + e) * 32, i, nd, sh) : 0u;
  const float scf = __uint_as_float((uint32_t)(127 - nd) << 23);  // 2^-nd
  const double scd = ldexp(1.0, -nd);
  const bool full = (VEC == 4) && (d + 3 < dim);
  for (; row < n; row += stride) {
    T* dst = out + row * (int64_t)dim + d;
    if (VEC == 4 && full && sizeof(T) == 4) {
      uint4 w;
      w.x = bits32(SobolOut<KIND>::conv(x[0], scf, scd));
      w.y = bits32(SobolOut<KIND>::conv(x[VEC > 1 ? 1 : 0], scf, scd));
      w.z = bits32(SobolOut<KIND>::conv(x[VEC > 2 ? 2 : 0], scf, scd));
      w.w = bits32(SobolOut<KIND>::conv(x[VEC > 3 ? 3 : 0], scf, scd));
      __stcs(reinterpret_cast<uint4*>(dst), w);  // streamed: written once, not re-read by this kernel
    } else {
#pragma unroll
      for (int e = 0; e < VEC; ++e)
        if (d + e < dim) dst[e] = SobolOut<KIND>::conv(x[e], scf, scd);
    }
    const int c = __ffs(~(i >> m)) - 1;
    const uint32_t* g = g_tab + c * width + dl;
#pragma unroll
    for (int e = 0; e < VEC; ++e) x[e] ^= g[e];
    i += (uint32_t)stride;
  }
}

// ---- [steps, N, d] draw layout (generate_mc_normal_draws, SOBOL) --------------
// Thread t owns paths n0 + t + s*256 (s < P) and the KB draw dimensions of
// blockIdx.y; stride 256 = 2^8.
constexpr int kDrawKB = 8;
template <int KIND>
__global__ void __launch_bounds__(kThreads)
    sobol_draws_kernel(const uint32_t* __restrict__ v, int d_per_step, int num_steps, int64_t N,
                       uint32_t first_index, int nd, int P, void* __restrict__ out_raw) {
  using T = typename SobolOut<KIND>::T;
  T* out = static_cast<T*>(out_raw);
  constexpr int m = 8;
  constexpr int levels = 32 - m;
  __shared__ uint32_t g_tab[kDrawKB][levels];
  const int K = d_per_step * num_steps;
  const int k0 = blockIdx.y * kDrawKB;
  const int sh = 32 - nd;
  for (int idx = threadIdx.x; idx < kDrawKB; idx += blockDim.x) {
    const int k = k0 + idx;
    uint32_t run = 0;
    for (int c = 0; c < levels; ++c) {
      if (k < K) run ^= v[(size_t)k * 32 + m + c];
      g_tab[idx][c] = run >> sh;
    }
  }
  __syncthreads();
  const float scf = __uint_as_float((uint32_t)(127 - nd) << 23);
  const double scd = ldexp(1.0, -nd);
  const int64_t n_first = (int64_t)blockIdx.x * kThreads * P + threadIdx.x;
  for (int kk = 0; kk < kDrawKB; ++kk) {
    const int k = k0 + kk;
    if (k >= K) break;
    const int step = k / d_per_step;
    const int comp = k - step * d_per_step;
    int64_t n = n_first;
    uint32_t i = first_index + (uint32_t)n;
    uint32_t x = sobol_direct(v + (size_t)k * 32, i, nd, sh);
    T* base = out + (int64_t)step * N * d_per_step + comp;
    for (int s = 0; s < P && n < N; ++s) {
      base[n * d_per_step] = SobolOut<KIND>::conv(x, scf, scd);
      const int c = __ffs(~(i >> m)) - 1;
      x ^= g_tab[kk][c];
      i += 256u;
      n += 256;
    }
  }
}

template <int KIND>
int launch_rowmajor(const uint32_t* v, int dim, int64_t n, uint32_t first, int nd, void* out,
                    cudaStream_t s) {
  const bool vec4 = (dim % 4 == 0) && ((reinterpret_cast<uintptr_t>(out) & 15u) == 0);
  const int vec = vec4 ? 4 : 1;
  // a CTA spans up to dx_cap * vec dims with dx dim-threads
  int need = (dim + vec - 1) / vec;
  int dx = 1;
  const int dx_cap = arithmetic_bound(KIND) ? 128 : 256;
  while (dx < need && dx < dx_cap) dx <<= 1;
  const int pt = kThreads / dx;
  int mt = 0;
  while ((1 << mt) < pt) ++mt;
  const int gy = (dim + dx * vec - 1) / (dx * vec);
  // a power of two along the rows, and no more CTAs than rows / pt
  int64_t want = (int64_t)(arithmetic_bound(KIND) ? 4 : 2) * num_sms() / gy;
  if (want < 1) want = 1;
  int64_t gx = 1;
  while (gx * 2 <= want && gx * 2 * pt <= n) gx *= 2;
  int q = 0;
  while ((1LL << q) < gx) ++q;
  const int m = mt + q;
  TQF_REQUIRE(m <= 31 && gy <= 65535, "tqf_sobol_sample: request too large for one launch");
  // c = trailing ones of (i >> m) <= bit length of (last index >> m)
  const uint32_t last = (uint32_t)(first + (uint32_t)(n - 1)) >> m;
  int levels = 1;
  while (levels < 32 - m && (last >> (levels - 1)) != 0u) ++levels;
  const size_t smem = (size_t)levels * dx * vec * sizeof(uint32_t);
  dim3 grid((unsigned)gx, (unsigned)gy);
  if (vec4) {
    set_smem_config(sobol_rowmajor_kernel<KIND, 4>, smem);
    sobol_rowmajor_kernel<KIND, 4><<<grid, kThreads, smem, s>>>(v, dim, n, first, nd, dx, mt, m, levels, out);
  } else {
    set_smem_config(sobol_rowmajor_kernel<KIND, 1>, smem);
    sobol_rowmajor_kernel<KIND, 1><<<grid, kThreads, smem, s>>>(v, dim, n, first, nd, dx, mt, m, levels, out);
  }
  return check_launch("sobol_rowmajor_kernel");
}

template <int KIND>
int launch_draws(const uint32_t* v, int d, int steps, int64_t N, uint32_t first, int nd, void* out,
                 cudaStream_t s) {
  const int P = 16;
  const int64_t gx = (N + (int64_t)kThreads * P - 1) / ((int64_t)kThreads * P);
  const int K = d * steps;
  const int gy = (K + kDrawKB - 1) / kDrawKB;
  TQF_REQUIRE(gx <= 2147483647LL && gy <= 65535, "tqf_sobol_normal_draws: request too large");
  dim3 grid((unsigned)gx, (unsigned)gy);
  sobol_draws_kernel<KIND><<<grid, kThreads, 0, s>>>(v, d, steps, N, first, nd, P, out);
  return check_launch("sobol_draws_kernel");
}

int check_sobol_common(const char* who, const uint32_t* v, int64_t n, int64_t skip, int nd, void* out) {
  TQF_REQUIRE(v != nullptr && out != nullptr, "%s: null pointer", who);
  TQF_REQUIRE(n >= 1, "%s: num_results must be >= 1, got %lld", who, (long long)n);
  TQF_REQUIRE(skip >= 0, "%s: skip must be >= 0, got %lld", who, (long long)skip);
  TQF_REQUIRE(skip + n <= 2147483647LL, "%s: skip + num_results must be < 2^31", who);
  TQF_REQUIRE(nd >= 1 && nd <= 32, "%s: nd must be in [1, 32], got %d", who, nd);
  return TQF_OK;
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_sobol_sample(const uint32_t* v_dev, int32_t dim, int64_t num_results,
                                int64_t skip, int32_t nd, int32_t out_kind, void* out,
                                void* stream) {
  clear_error();
  int rc = check_sobol_common("tqf_sobol_sample", v_dev, num_results, skip, nd, out);
  if (rc) return rc;
  TQF_REQUIRE(dim >= 1, "tqf_sobol_sample: dim must be >= 1, got %d", dim);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint32_t first = (uint32_t)(skip + 1);
  switch (out_kind) {
    case TQF_SOBOL_U32: return launch_rowmajor<TQF_SOBOL_U32>(v_dev, dim, num_results, first, nd, out, s);
    case TQF_SOBOL_F32: return launch_rowmajor<TQF_SOBOL_F32>(v_dev, dim, num_results, first, nd, out, s);
    case TQF_SOBOL_F64: return launch_rowmajor<TQF_SOBOL_F64>(v_dev, dim, num_results, first, nd, out, s);
    case TQF_SOBOL_NORMAL_F32:
      return launch_rowmajor<TQF_SOBOL_NORMAL_F32>(v_dev, dim, num_results, first, nd, out, s);
    case TQF_SOBOL_NORMAL_F64:
      return launch_rowmajor<TQF_SOBOL_NORMAL_F64>(v_dev, dim, num_results, first, nd, out, s);
    case TQF_SOBOL_F32_CENTERED:
      return launch_rowmajor<TQF_SOBOL_F32_CENTERED>(v_dev, dim, num_results, first, nd, out, s);
    default:
      set_error("tqf_sobol_sample: unknown out_kind %d", out_kind);
      return TQF_E_INVALID;
  }
}

extern "C" int tqf_sobol_normal_draws(const uint32_t* v_dev, int32_t num_normal_draws,
                                      int32_t num_steps, int64_t num_paths, int64_t skip,
                                      int32_t nd, int32_t out_kind, void* out, void* stream) {
  clear_error();
  int rc = check_sobol_common("tqf_sobol_normal_draws", v_dev, num_paths, skip, nd, out);
  if (rc) return rc;
  TQF_REQUIRE(num_normal_draws >= 1 && num_steps >= 1,
              "tqf_sobol_normal_draws: num_normal_draws and num_steps must be >= 1");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint32_t first = (uint32_t)(skip + 1);
  if (out_kind == TQF_SOBOL_NORMAL_F32)
    return launch_draws<TQF_SOBOL_NORMAL_F32>(v_dev, num_normal_draws, num_steps, num_paths, first,
                                              nd, out, s);
  if (out_kind == TQF_SOBOL_NORMAL_F64)
    return launch_draws<TQF_SOBOL_NORMAL_F64>(v_dev, num_normal_draws, num_steps, num_paths, first,
                                              nd, out, s);
  if (out_kind == TQF_SOBOL_U32)
    return launch_draws<TQF_SOBOL_U32>(v_dev, num_normal_draws, num_steps, num_paths, first, nd,
                                       out, s);
  set_error("tqf_sobol_normal_draws: out_kind must be NORMAL_F32, NORMAL_F64 or U32");
  return TQF_E_INVALID;
}
