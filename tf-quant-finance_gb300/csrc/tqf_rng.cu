// Philox4x32-10 raw blocks and materialised normal draws in the reference's
// [steps, N, d] layout (the PSEUDO / STATELESS / *_ANTITHETIC branches of
// tff/models/utils.py:20-128 and multivariate_normal.py:248-311).  The draw
// for (path n, dimension k) comes from the same device functions the fused
// path kernels call, so both routes give identical numbers.
#include "tqf_internal.cuh"

namespace tqf {
namespace {

__global__ void philox_raw_kernel(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                  uint32_t k1, int64_t nblocks, uint4* __restrict__ out) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  out[b] = philox4x32_10(make_uint4(c0 + (uint32_t)b, c1, c2, c3), k0, k1);
}

// One thread per (path, Philox block); writes that block's normals.
template <typename T>
__global__ void __launch_bounds__(256)
    philox_draws_kernel(tqf_draws dr, int d, int steps, int64_t N, T* __restrict__ out) {
  constexpr int NPB = NormalsPerBlock<T>::value;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int64_t K = (int64_t)d * steps;
  int64_t p = n;
  T sign = T(1);
  if (dr.antithetic && p >= dr.antithetic_half) {
    p -= dr.antithetic_half;
    sign = T(-1);
  }
  p += dr.path_offset;
  for (int64_t b = blockIdx.y; b * NPB < K; b += gridDim.y) {
    T z[NPB];
    if constexpr (NPB == 4) {
      philox_normals4_f32(b, p, dr.key0, dr.key1, z);
    } else {
      philox_normals2_f64(b, p, dr.key0, dr.key1, z);
    }
#pragma unroll
    for (int l = 0; l < NPB; ++l) {
      const int64_t k = b * NPB + l;
      if (k < K) {
        const int64_t step = k / d;
        const int64_t comp = k - step * d;
        out[(step * N + n) * d + comp] = sign * z[l];
      }
    }
  }
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_philox4x32_10(uint32_t ctr0, uint32_t c1, uint32_t c2, uint32_t c3,
                                 uint32_t key0, uint32_t key1, int64_t num_blocks, uint32_t* out,
                                 void* stream) {
  clear_error();
  TQF_REQUIRE(out != nullptr, "tqf_philox4x32_10: null output");
  TQF_REQUIRE(num_blocks >= 0 && num_blocks < (1LL << 32), "tqf_philox4x32_10: bad num_blocks");
  TQF_REQUIRE((reinterpret_cast<uintptr_t>(out) & 15u) == 0, "tqf_philox4x32_10: out must be 16-byte aligned");
  if (num_blocks == 0) return TQF_OK;
  const int threads = 256;
  const int64_t grid = (num_blocks + threads - 1) / threads;
  philox_raw_kernel<<<(unsigned)grid, threads, 0, static_cast<cudaStream_t>(stream)>>>(
      ctr0, c1, c2, c3, key0, key1, num_blocks, reinterpret_cast<uint4*>(out));
  return check_launch("philox_raw_kernel");
}

extern "C" int tqf_philox_normal_draws(const tqf_draws* draws, int32_t num_normal_draws,
                                       int32_t num_steps, int64_t num_paths, int32_t dtype,
                                       void* out, void* stream) {
  clear_error();
  TQF_REQUIRE(draws != nullptr && out != nullptr, "tqf_philox_normal_draws: null pointer");
  TQF_REQUIRE(draws->source == TQF_DRAWS_PHILOX, "tqf_philox_normal_draws: draws.source must be PHILOX");
  TQF_REQUIRE(num_normal_draws >= 1 && num_steps >= 1 && num_paths >= 1,
              "tqf_philox_normal_draws: sizes must be >= 1");
  TQF_REQUIRE(!draws->antithetic || 2 * draws->antithetic_half == num_paths,
              "tqf_philox_normal_draws: antithetic needs num_paths == 2 * antithetic_half");
  const int threads = 256;
  const int64_t gx = (num_paths + threads - 1) / threads;
  TQF_REQUIRE(gx <= 2147483647LL, "tqf_philox_normal_draws: too many paths");
  const int64_t K = (int64_t)num_normal_draws * num_steps;
  const int npb = dtype == TQF_F32 ? 4 : 2;
  int64_t gy = (K + npb - 1) / npb;
  if (gy > 65535) gy = 65535;
  dim3 grid((unsigned)gx, (unsigned)gy);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == TQF_F32) {
    philox_draws_kernel<float><<<grid, threads, 0, s>>>(*draws, num_normal_draws, num_steps,
                                                        num_paths, static_cast<float*>(out));
  } else if (dtype == TQF_F64) {
    philox_draws_kernel<double><<<grid, threads, 0, s>>>(*draws, num_normal_draws, num_steps,
                                                         num_paths, static_cast<double*>(out));
  } else {
    set_error("tqf_philox_normal_draws: bad dtype %d", dtype);
    return TQF_E_INVALID;
  }
  return check_launch("philox_draws_kernel");
}
