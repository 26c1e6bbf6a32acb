// tff.math.qmc point sets — the GB300 replacement of
// tff/math/qmc/digital_net.py:205-419 (digital_net_sample) and
// tff/math/qmc/lattice_rule.py:99-229 (lattice_rule_sample).
//
// The reference loops over the index bits with whole-tensor XORs (one
// [n, dim] tensor per bit) or forms the [n, dim] product tensor; here one
// thread computes one (point, axis) value from the generating matrix column
// in registers and writes it once in row-major [n, dim] order.
#include "tqf_internal.cuh"

namespace tqf {
namespace {

constexpr int kThreads = 256;

template <typename I, typename T>
__global__ void __launch_bounds__(kThreads) digital_net_kernel(tqf_digital_net_args a) {
  const int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (e >= a.count * a.dim) return;
  const int64_t i = e / a.dim;
  const int d = (int)(e - i * a.dim);
  const uint64_t idx = (uint64_t)(a.sequence_indices ? a.sequence_indices[i] : i);
  const I* M = static_cast<const I*>(a.matrices) + (int64_t)d * a.log_num_results;
  I x = a.digital_shift ? static_cast<const I*>(a.digital_shift)[d] : I(0);
  for (int b = 0; b < a.log_num_results; ++b)
    if ((idx >> b) & 1u) x ^= M[b];
  const T v = (T)x / (T)((uint64_t)1 << a.num_digits);
  static_cast<T*>(a.out)[e] = a.tent ? (v < T(0.5) ? T(2) * v : T(2) * (T(1) - v)) : v;
}

template <typename I, typename T>
__global__ void __launch_bounds__(kThreads) lattice_kernel(tqf_lattice_args a) {
  const int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (e >= a.count * a.dim) return;
  const int64_t i = e / a.dim;
  const int d = (int)(e - i * a.dim);
  const int64_t idx = a.sequence_indices ? a.sequence_indices[i] : i;
  const T scaled = (T)static_cast<const I*>(a.generating_vectors)[d] / (T)a.num_results;
  const T frac = scaled - floor(scaled);
  T p = (T)idx * frac;
  if (a.additive_shift) p = p + static_cast<const T*>(a.additive_shift)[d];
  p = p - floor(p);
  static_cast<T*>(a.out)[e] = a.tent ? (p < T(0.5) ? T(2) * p : T(2) * (T(1) - p)) : p;
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_digital_net_sample(const tqf_digital_net_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_digital_net_sample: null args");
  TQF_REQUIRE(a->dim >= 1 && a->log_num_results >= 0 && a->log_num_results < 64 && a->num_digits >= 1 &&
                  a->num_digits < 64 && a->count >= 0,
              "tqf_digital_net_sample: bad sizes");
  TQF_REQUIRE(a->int_bits == 32 || a->int_bits == 64, "tqf_digital_net_sample: int_bits must be 32 or 64");
  TQF_REQUIRE(a->matrices && a->out, "tqf_digital_net_sample: null pointer");
  TQF_REQUIRE(a->out_kind == TQF_SOBOL_F32 || a->out_kind == TQF_SOBOL_F64, "tqf_digital_net_sample: bad out_kind");
  if (a->count == 0) return TQF_OK;
  const int64_t grid = (a->count * a->dim + kThreads - 1) / kThreads;
  TQF_REQUIRE(grid <= 2147483647LL, "tqf_digital_net_sample: request too large");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool f32 = a->out_kind == TQF_SOBOL_F32;
  if (a->int_bits == 32)
    f32 ? digital_net_kernel<uint32_t, float><<<(unsigned)grid, kThreads, 0, s>>>(*a)
        : digital_net_kernel<uint32_t, double><<<(unsigned)grid, kThreads, 0, s>>>(*a);
  else
    f32 ? digital_net_kernel<uint64_t, float><<<(unsigned)grid, kThreads, 0, s>>>(*a)
        : digital_net_kernel<uint64_t, double><<<(unsigned)grid, kThreads, 0, s>>>(*a);
  return check_launch("digital_net_kernel");
}

extern "C" int tqf_lattice_rule_sample(const tqf_lattice_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_lattice_rule_sample: null args");
  TQF_REQUIRE(a->dim >= 1 && a->num_results >= 1 && a->count >= 0, "tqf_lattice_rule_sample: bad sizes");
  TQF_REQUIRE(a->int_bits == 32 || a->int_bits == 64, "tqf_lattice_rule_sample: int_bits must be 32 or 64");
  TQF_REQUIRE(a->generating_vectors && a->out, "tqf_lattice_rule_sample: null pointer");
  TQF_REQUIRE(a->out_kind == TQF_SOBOL_F32 || a->out_kind == TQF_SOBOL_F64, "tqf_lattice_rule_sample: bad out_kind");
  if (a->count == 0) return TQF_OK;
  const int64_t grid = (a->count * a->dim + kThreads - 1) / kThreads;
  TQF_REQUIRE(grid <= 2147483647LL, "tqf_lattice_rule_sample: request too large");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool f32 = a->out_kind == TQF_SOBOL_F32;
  if (a->int_bits == 32)
    f32 ? lattice_kernel<int32_t, float><<<(unsigned)grid, kThreads, 0, s>>>(*a)
        : lattice_kernel<int32_t, double><<<(unsigned)grid, kThreads, 0, s>>>(*a);
  else
    f32 ? lattice_kernel<int64_t, float><<<(unsigned)grid, kThreads, 0, s>>>(*a)
        : lattice_kernel<int64_t, double><<<(unsigned)grid, kThreads, 0, s>>>(*a);
  return check_launch("lattice_kernel");
}
