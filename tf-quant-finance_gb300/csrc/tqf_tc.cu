// Self-check of the tcgen05 encodings (no reference counterpart): stages
// A [M x K] and B [N x K] (row-major BF16 in global memory) into shared
// memory in the K-major or MN-major canonical no-swizzle layout, runs
// D = A B^T as K/16 tcgen05.mma instructions into TMEM and dumps TMEM lanes
// 0..127 x N columns to out [128 x N] (FP32).  Used by the tests to pin the
// descriptor formats the MLP kernels rely on.
#include "tqf_tc.cuh"

namespace tqf {
namespace {

constexpr int kTcThreads = 128;
constexpr int kTcOperandBytes = 32768;  // up to 128 x 128 BF16

__global__ void __launch_bounds__(kTcThreads)
    tc_selftest_kernel(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B, int M, int N, int K,
                       int a_mn, int b_mn, float* __restrict__ out, int32_t* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + 16);
  unsigned char* sA = smem + 1024;
  unsigned char* sB = sA + kTcOperandBytes;
  const int t = threadIdx.x;
  const uint32_t a_lbo = a_mn ? (uint32_t)(M / 8) * 128u : 128u;
  const uint32_t a_sbo = a_mn ? 128u : (uint32_t)(K / 8) * 128u;
  const uint32_t b_lbo = b_mn ? (uint32_t)(N / 8) * 128u : 128u;
  const uint32_t b_sbo = b_mn ? 128u : (uint32_t)(K / 8) * 128u;
  for (int i = t; i < M * K; i += kTcThreads) {
    const int r = i / K, k = i % K;
    const uint32_t off = a_mn ? tc::mnmajor_off(r, k, a_lbo, a_sbo) : tc::kmajor_off(r, k, a_lbo, a_sbo);
    *reinterpret_cast<uint16_t*>(sA + off) = A[i];
  }
  for (int i = t; i < N * K; i += kTcThreads) {
    const int r = i / K, k = i % K;
    const uint32_t off = b_mn ? tc::mnmajor_off(r, k, b_lbo, b_sbo) : tc::kmajor_off(r, k, b_lbo, b_sbo);
    *reinterpret_cast<uint16_t*>(sB + off) = B[i];
  }
  if (t == 0) mbar_init(bar, 1);
  if (t < 32) tc::tmem_alloc(slot, 256);
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;
  if (t == 0) {
    const uint32_t idesc = tc::idesc_bf16(M, N, a_mn != 0, b_mn != 0);
    for (int s = 0; s < K / 16; ++s) {
      const uint32_t a_addr = smem_addr(sA) + 2u * (uint32_t)s * a_lbo;
      const uint32_t b_addr = smem_addr(sB) + 2u * (uint32_t)s * b_lbo;
      tc::mma_bf16(tmem, tc::smem_desc(a_addr, a_lbo, a_sbo), tc::smem_desc(b_addr, b_lbo, b_sbo), idesc,
                   s > 0 ? 1u : 0u);
    }
    tc::commit(bar);
  }
  bool ok = mbar_wait_bounded(bar, 0);
  ok = __syncthreads_and(ok) != 0;
  if (!ok) {
    if (t == 0 && status) atomicExch(status, TQF_E_TIMEOUT);
    mbar_wait_bounded(bar, 0);  // let an in-flight MMA finish before the TMEM is released
  }
  tc::fence_after_sync();
  if (ok) {
    const uint32_t lane_base = (uint32_t)(32 * (t / 32)) << 16;
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + (uint32_t)c, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) out[t * N + c + j] = v[j];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (t < 32) tc::tmem_dealloc(tmem, 256);
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_tc_selftest(const uint16_t* a, const uint16_t* b, int32_t m, int32_t n, int32_t k,
                               int32_t a_mn, int32_t b_mn, float* out, int32_t* status, void* stream) {
  clear_error();
  TQF_REQUIRE(a && b && out, "tqf_tc_selftest: null pointer");
  TQF_REQUIRE(m == 64 || m == 128, "tqf_tc_selftest: m must be 64 or 128");
  TQF_REQUIRE(n >= 16 && n <= 128 && n % 16 == 0, "tqf_tc_selftest: n must be a multiple of 16 in [16, 128]");
  TQF_REQUIRE(k >= 16 && k <= 128 && k % 16 == 0, "tqf_tc_selftest: k must be a multiple of 16 in [16, 128]");
  const size_t smem = 1024 + 2 * (size_t)kTcOperandBytes;
  set_smem_config(tc_selftest_kernel, smem);
  tc_selftest_kernel<<<1, kTcThreads, smem, static_cast<cudaStream_t>(stream)>>>(a, b, m, n, k, a_mn, b_mn,
                                                                                 out, status);
  return check_launch("tc_selftest_kernel");
}
