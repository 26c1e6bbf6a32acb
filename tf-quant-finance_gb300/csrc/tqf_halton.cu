// Halton sequence — the GB300 replacement of
// tff/math/random_ops/halton/halton_impl.py:59-375.
//
// The reference builds a [n, dim, max_size] tensor of digits with float floor
// division and mod, scales by radix powers and reduces over the digit axis.
// Here one thread produces one (point, axis) element: the base-p digits of the
// index come from integer division in registers, the (optionally permuted)
// digits are folded into the radical inverse sum_k digit_k p^-(k+1) by Horner's
// rule from the most significant position (FP64, then rounded to the output
// type), and the point is written in row-major [n, dim] order.
#include <math.h>

#include "tqf_internal.cuh"

namespace tqf {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxDigits = 64;

template <int KIND>
__global__ void __launch_bounds__(kThreads) halton_kernel(tqf_halton_args a) {
  const int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const int64_t total = a.num_results * a.dim;
  if (e >= total) return;
  const int64_t i = e / a.dim;
  const int d = (int)(e - i * a.dim);
  uint64_t idx = (uint64_t)(a.sequence_indices ? a.sequence_indices[i] : a.first_index + i) + 1;
  const uint32_t p = (uint32_t)a.primes[d];
  const int ms = a.max_sizes[d];
  uint32_t dig[kMaxDigits];
#pragma unroll 1
  for (int k = 0; k < ms; ++k) {
    const uint64_t q = idx / p;
    dig[k] = (uint32_t)(idx - q * p);
    idx = q;
  }
  if (a.perms) {
    const int32_t* pm = a.perms + a.perm_offsets[d];
#pragma unroll 1
    for (int k = 0; k < ms; ++k) dig[k] = (uint32_t)pm[(int64_t)k * a.radix_sum + dig[k]];
  }
  const double inv_p = 1.0 / (double)p;
  double v = 0.0;
#pragma unroll 1
  for (int k = ms - 1; k >= 0; --k) v = ((double)dig[k] + v) * inv_p;
  if (KIND == TQF_SOBOL_F32 || KIND == TQF_SOBOL_NORMAL_F32) {
    float u = (float)v;
    if (a.zero_correction) u = u + static_cast<const float*>(a.zero_correction)[d];
    float* out = static_cast<float*>(a.out);
    if (KIND == TQF_SOBOL_F32)
      out[e] = u;
    else
      out[e] = __fmul_rn(erfinvf(__fmul_rn(__fsub_rn(u, 0.5f), 2.0f)), 1.41421353816986083984375f);
  } else {
    double u = v;
    if (a.zero_correction) u = u + static_cast<const double*>(a.zero_correction)[d];
    double* out = static_cast<double*>(a.out);
    out[e] = KIND == TQF_SOBOL_F64 ? u : erfinv((u - 0.5) * 2.0) * 1.4142135623730951;
  }
}

// One thread per (digit position k, axis d): Fisher-Yates shuffle of 0..p-1.
__global__ void __launch_bounds__(kThreads)
    halton_perm_kernel(int dim, int num_coeffs, const int32_t* __restrict__ primes,
                       const int32_t* __restrict__ offsets, int radix_sum, uint32_t k0, uint32_t k1,
                       int32_t* __restrict__ perms, double* __restrict__ uniforms) {
  const int s = blockIdx.x * kThreads + threadIdx.x;
  if (s < dim && uniforms) {
    // zero-correction uniforms: counter (s, 0xFFFFFFFF, 0, 0)
    const uint4 r = philox4x32_10(make_uint4((uint32_t)s, 0xFFFFFFFFu, 0u, 0u), k0, k1);
    uniforms[s] = u01_co_f64(r.x, r.y);
  }
  if (s >= dim * num_coeffs) return;
  const int k = s / dim, d = s - k * dim;
  const int p = primes[d];
  int32_t* pm = perms + (int64_t)k * radix_sum + offsets[d];
  for (int j = 0; j < p; ++j) pm[j] = j;
  uint4 r = make_uint4(0, 0, 0, 0);
  for (int i = p - 1, c = 0; i >= 1; --i, ++c) {
    if ((c & 3) == 0) r = philox4x32_10(make_uint4((uint32_t)s, (uint32_t)(c >> 2), 1u, 0u), k0, k1);
    const uint32_t u = (c & 3) == 0 ? r.x : (c & 3) == 1 ? r.y : (c & 3) == 2 ? r.z : r.w;
    const int j = (int)(((uint64_t)u * (uint64_t)(i + 1)) >> 32);  // uniform in [0, i]
    const int32_t t = pm[i];
    pm[i] = pm[j];
    pm[j] = t;
  }
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_halton_sample(const tqf_halton_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_halton_sample: null args");
  TQF_REQUIRE(a->dim >= 1 && a->dim <= 1000, "tqf_halton_sample: dim must be in [1, 1000], got %d", a->dim);
  TQF_REQUIRE(a->num_results >= 0, "tqf_halton_sample: num_results must be >= 0");
  TQF_REQUIRE(a->primes && a->max_sizes && a->out, "tqf_halton_sample: null pointer");
  TQF_REQUIRE(!a->perms || (a->perm_offsets && a->radix_sum > 0), "tqf_halton_sample: perms need offsets");
  if (a->num_results == 0) return TQF_OK;
  const int64_t total = a->num_results * a->dim;
  const int64_t grid = (total + kThreads - 1) / kThreads;
  TQF_REQUIRE(grid <= 2147483647LL, "tqf_halton_sample: request too large");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (a->out_kind) {
    case TQF_SOBOL_F32: halton_kernel<TQF_SOBOL_F32><<<(unsigned)grid, kThreads, 0, s>>>(*a); break;
    case TQF_SOBOL_F64: halton_kernel<TQF_SOBOL_F64><<<(unsigned)grid, kThreads, 0, s>>>(*a); break;
    case TQF_SOBOL_NORMAL_F32: halton_kernel<TQF_SOBOL_NORMAL_F32><<<(unsigned)grid, kThreads, 0, s>>>(*a); break;
    case TQF_SOBOL_NORMAL_F64: halton_kernel<TQF_SOBOL_NORMAL_F64><<<(unsigned)grid, kThreads, 0, s>>>(*a); break;
    default:
      set_error("tqf_halton_sample: out_kind must be F32, F64, NORMAL_F32 or NORMAL_F64");
      return TQF_E_INVALID;
  }
  return check_launch("halton_kernel");
}

extern "C" int tqf_halton_permutations(int32_t dim, int32_t num_coeffs, const int32_t* primes,
                                       const int32_t* perm_offsets, int32_t radix_sum, uint64_t seed,
                                       int32_t* perms, double* uniforms, void* stream) {
  clear_error();
  TQF_REQUIRE(dim >= 1 && dim <= 1000 && num_coeffs >= 1 && num_coeffs <= kMaxDigits,
              "tqf_halton_permutations: bad sizes");
  TQF_REQUIRE(primes && perm_offsets && perms && radix_sum > 0, "tqf_halton_permutations: null pointer");
  const int n = dim * num_coeffs;
  const int grid = (n + kThreads - 1) / kThreads;
  halton_perm_kernel<<<grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      dim, num_coeffs, primes, perm_offsets, radix_sum, (uint32_t)seed, (uint32_t)(seed >> 32), perms, uniforms);
  return check_launch("halton_perm_kernel");
}
