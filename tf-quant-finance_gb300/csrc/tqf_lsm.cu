// Longstaff–Schwartz regression Monte Carlo — the GB300 replacement of
// tff/models/longstaff_schwartz/lsm.py:128-436 and payoff_utils.py:27-98.
//
// The reference loops backwards over exercise dates; each iteration builds a
// [batch, N, G] design, masks it by "in the money", forms X'X and X'y with two
// matmuls, takes tf.linalg.pinv (SVD) and re-projects every path.  Here:
//   lsm_gather_kernel  one coalesced pass over the paths: copies the states at
//                      the exercise times into [Bp][E][N][d] (so every later
//                      pass reads contiguous rows) and sums their columns in
//                      FP64 (the basis centring means, lsm.py:106-108);
//   lsm_pass_kernel    per date: applies the previous date's regression
//                      (continuation value, exercise decision, cashflow and
//                      value update, discounting) and accumulates this date's
//                      masked normal equations — the design is built per path
//                      in shared memory, never stored.  Products are summed in
//                      the paths' dtype over at most 16 paths, then in FP64;
//   reduce_partials    fixed-order sum of the per-CTA partials;
//   lsm_solve_kernel   one CTA per batch member: Jacobi eigen-decomposition of
//                      X'X in FP64 (serial for <= 16 basis functions, parallel
//                      round-robin rotations above), pinv with tf.linalg.pinv's
//                      cutoff, beta.
//   lsm_loop_kernel    the structured single-payoff case (d <= 2, <= 5 basis
//                      functions) in one cooperative launch: every date's
//                      masked Gram matrix (which does not depend on the
//                      coefficients) and its pseudo-inverse first, in
//                      parallel; then per date one pass (exercise update +
//                      the G sums of X'y), a fixed-order reduction and
//                      beta = P X'y, between bounded grid barriers.
// tqf_lsm_price runs the whole backward loop for the structured basis and
// payoff without returning to the caller.
#include <math.h>

#include "tqf_internal.cuh"

namespace tqf {
namespace {

constexpr int kMaxBasis = 128;
constexpr int kMaxDimLsm = 16;
constexpr int kSolveThreads = 256;
constexpr int kMaxJacobiSweeps = 40;
constexpr int kGatherThreads = 256;
constexpr size_t kGatherTileBytes = 96 * 1024;
constexpr int kSubSum = 16;  // products summed in the paths' dtype before FP64

__host__ __device__ inline int lsm_entries(int G) { return G * (G + 1) / 2 + G; }

// Design-tile row stride (elements): odd, so that threads reading one column
// of consecutive rows hit distinct banks.
__host__ __device__ inline int lsm_row_stride(int G) { return (G + 1) | 1; }

// Shared memory of the pass kernel: design tile [C][W] (dtype), accumulators
// [max(En, C)] (FP64), entry -> (j, k) table [max(En, C)], beta [G] and the
// two centring means [2][16] in the dtype, block-sum scratch, exponents [G][16].
template <typename T>
__host__ __device__ inline size_t lsm_pass_smem(int G, int C) {
  const int En = lsm_entries(G);
  const size_t items = (size_t)(En > C ? En : C);
  const size_t tile = ((size_t)C * lsm_row_stride(G) * sizeof(T) + 15) & ~(size_t)15;
  return tile + items * 8 + items * 4 + ((G + 2 * kMaxDimLsm) * sizeof(T) + 15) / 16 * 16 + 64 * 8 +
         (size_t)G * kMaxDimLsm;
}

// Paths per CTA iteration (= threads per CTA): the largest of 256/128/64
// whose tiles fit in 200 KB.
template <typename T>
__host__ inline int lsm_chunk(int G) {
  for (int C = 256; C >= 64; C >>= 1)
    if (lsm_pass_smem<T>(G, C) <= 200 * 1024) return C;
  return 64;
}

template <typename T, int DM, int GR>
__global__ void lsm_pass_kernel(tqf_lsm_args a, const T* __restrict__ xt, void* __restrict__ partials_raw,
                                const double* __restrict__ beta, const double* __restrict__ means, int C);

// The instantiation for a call: path-state registers for the dimension bucket
// (1, 2, 4, 16); GR = number of basis functions when it is 2..5 and d <= 2
// (per-thread register accumulation), else 0 (shared-memory design tile).
template <typename T>
__host__ inline void* pass_kernel_for(int d, int G);

template <typename T>
__host__ inline int lsm_pass_grid(const tqf_lsm_args& a, int* chunk_out, size_t* smem_out) {
  const int G = a.num_basis;
  const int C = lsm_chunk<T>(G);
  const size_t smem = lsm_pass_smem<T>(G, C);
  const void* k = pass_kernel_for<T>(a.degree >= 0 ? a.dim : 1, G);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, C, smem) != cudaSuccess || occ < 1) occ = 1;
  if (occ > 8) occ = 8;
  const int64_t chunks = (a.num_paths + C - 1) / C;
  int64_t g = (int64_t)num_sms() * occ;
  if (g > chunks) g = chunks;
  if (chunk_out) *chunk_out = C;
  if (smem_out) *smem_out = smem;
  return (int)(g < 1 ? 1 : g);
}

// Gather tile: whole path rows [Cn][T*d] when at least 8 fit in 96 KB
// (full = 1, Cn a multiple of 4 so chunk starts stay 16-byte aligned), else
// the exercise columns [Cn][E*d].  Returns Cn (0: does not fit, rejected).
__host__ inline int lsm_gather_chunk(const tqf_lsm_args& a, int* full_out = nullptr) {
  const size_t es = a.dtype == TQF_F32 ? 4 : 8;
  const size_t Ed = (size_t)a.num_exercise * a.dim;
  const size_t R = Ed >= kGatherThreads ? 1 : kGatherThreads / Ed;
  const size_t fixed = ((Ed * R + 1) & ~(size_t)1) * 8 + 2 * ((Ed + 3) & ~(size_t)3) * 4;
  if (fixed >= 200 * 1024) return 0;
  size_t room = 200 * 1024 - fixed;
  if (room > kGatherTileBytes) room = kGatherTileBytes;
  const size_t full_row = (size_t)a.num_times * a.dim * es;
  size_t c = room / full_row;
  int full = 1;
  if (c >= 8) {
    c &= ~(size_t)3;
  } else {
    full = 0;
    c = room / ((Ed | 1) * es);
  }
  if (c > 256) c = 256;
  if (full_out) *full_out = full;
  return (int)c;
}

__host__ inline size_t lsm_gather_smem(const tqf_lsm_args& a, int Cn, int full) {
  const size_t es = a.dtype == TQF_F32 ? 4 : 8;
  const size_t Ed = (size_t)a.num_exercise * a.dim;
  const size_t R = Ed >= kGatherThreads ? 1 : kGatherThreads / Ed;
  const size_t row = full ? (size_t)a.num_times * a.dim : (Ed | 1);
  return ((Ed * R + 1) & ~(size_t)1) * 8 + 2 * ((Ed + 3) & ~(size_t)3) * 4 + (size_t)Cn * row * es;
}

__host__ inline int lsm_gather_grid(const tqf_lsm_args& a) {
  const int Cn = lsm_gather_chunk(a);
  if (Cn < 1) return 1;
  int64_t g = (a.num_paths + Cn - 1) / Cn;
  if (g > num_sms() * 2) g = num_sms() * 2;
  return (int)(g < 1 ? 1 : g);
}

struct WsLayout {
  size_t partials, sums, beta, means, mean_partials, eig_v, xt, sync, gram, pinv, total;
};

// Grid of the one-launch date loop (0 when the call does not qualify).
__host__ int lsm_loop_grid(const tqf_lsm_args& a);

__host__ inline WsLayout lsm_layout(const tqf_lsm_args& a) {
  const int G = a.num_basis, B = a.batch, E = a.num_exercise;
  const int En = lsm_entries(G);
  const int gx = a.dtype == TQF_F32 ? lsm_pass_grid<float>(a, nullptr, nullptr)
                                    : lsm_pass_grid<double>(a, nullptr, nullptr);
  const int gg = lsm_gather_grid(a);
  const int gl = lsm_loop_grid(a);
  const size_t es = a.dtype == TQF_F32 ? 4 : 8;
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  WsLayout w{};
  size_t off = 0;
  w.partials = off;
  off += up((size_t)(gx > gl ? gx : gl) * B * (En > 1 ? En : 1) * 8);
  w.sums = off;
  off += up((size_t)B * En * 8);
  w.beta = off;
  off += up((size_t)B * G * 8);
  w.means = off;
  off += up((size_t)E * a.paths_batch * kMaxDimLsm * 8);
  w.mean_partials = off;
  off += up((size_t)gg * E * a.paths_batch * kMaxDimLsm * 8);
  w.eig_v = off;
  off += up((size_t)B * G * G * 8);
  w.xt = off;
  if (a.degree >= 0) off += up((size_t)a.paths_batch * E * a.num_paths * a.dim * es);
  w.sync = off;
  off += 256;
  // one-launch loop: per-CTA Gram partials of every date, then each date's
  // pseudo-inverse (FP64 [G][G])
  w.gram = off;
  if (gl >= 1) off += up((size_t)E * gl * (size_t)(G * (G + 1) / 2) * 8);
  w.pinv = off;
  if (gl >= 1) off += up((size_t)E * G * G * 8);
  w.total = off;
  return w;
}

template <typename T>
__device__ __forceinline__ T ipow(T x, int e) {
  T r = T(1);
  for (int i = 0; i < e; ++i) r *= x;
  return r;
}

// ---- cross-path accumulators --------------------------------------------------
// FP64 is a narrow pipe on this GPU, so float paths accumulate in compensated
// double-float (an unevaluated float pair hi + lo, Knuth TwoSum additions:
// ~2^-48 relative, FP32 pipe) and convert to double once per entry at the end;
// double paths accumulate in FP64.
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  const float s = a.x + b.x;
  const float bb = s - a.x;
  const float err = (a.x - (s - bb)) + (b.x - bb);
  const float lo = err + a.y + b.y;
  const float hi = s + lo;
  return make_float2(hi, lo - (hi - s));
}

template <typename T>
struct Acc;
template <>
struct Acc<double> {
  using S = double;
  __device__ static S zero() { return 0.0; }
  __device__ static S add(S a, double v) { return a + v; }
  __device__ static S sum(S a, S b) { return a + b; }
  __device__ static double value(S a) { return a; }
  __device__ static S shfl_down(S a, int o) { return __shfl_down_sync(0xffffffffu, a, o); }
};
template <>
struct Acc<float> {
  using S = float2;
  __device__ static S zero() { return make_float2(0.f, 0.f); }
  __device__ static S add(S a, float v) { return df_add(a, make_float2(v, 0.f)); }
  __device__ static S sum(S a, S b) { return df_add(a, b); }
  __device__ static double value(S a) { return (double)a.x + (double)a.y; }
  __device__ static S shfl_down(S a, int o) {
    return make_float2(__shfl_down_sync(0xffffffffu, a.x, o), __shfl_down_sync(0xffffffffu, a.y, o));
  }
};
static_assert(sizeof(Acc<float>::S) == 8 && sizeof(Acc<double>::S) == 8, "8-byte accumulators");

// Fixed-order reduction of per-CTA accumulator rows [rows][width] -> double out[width].
template <typename T>
__global__ void __launch_bounds__(1024)
    lsm_reduce_kernel(const typename Acc<T>::S* __restrict__ part, int rows, int width, double* __restrict__ out) {
  grid_dependency_wait();  // a programmatic dependent launch in the exercise-date chain
  allow_dependent_launch();
  using A = Acc<T>;
  __shared__ typename A::S s[32][33];
  const int c = threadIdx.x % 32, r = threadIdx.x / 32;
  const int w = blockIdx.x * 32 + c;
  typename A::S acc = A::zero();
  if (w < width)
    for (int i = r; i < rows; i += 32) acc = A::sum(acc, part[(size_t)i * width + w]);
  s[r][c] = acc;
  __syncthreads();
  for (int st = 16; st > 0; st >>= 1) {
    if (r < st) s[r][c] = A::sum(s[r][c], s[r + st][c]);
    __syncthreads();
  }
  if (r == 0 && w < width) out[w] = A::value(s[0][c]);
}


// ---- gather the exercise-time states, column sums -------------------------------
// CTA (x, pb): chunks of Cn consecutive paths.  When whole path rows fit
// (full = 1) the chunk [Cn][T*d] is one contiguous range, copied with 16-byte
// loads; otherwise only the exercise columns are loaded.  Column sums use R
// replicas per column, combined in a fixed order at the end.
template <typename T>
__global__ void __launch_bounds__(kGatherThreads)
    lsm_gather_kernel(tqf_lsm_args a, T* __restrict__ xt, typename Acc<T>::S* __restrict__ partials, int Cn,
                      int full) {
  using A = Acc<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int d = a.dim, E = a.num_exercise;
  const int Ed = E * d;
  const int64_t Td = (int64_t)a.num_times * d;
  const int Wt = full ? (int)Td : (Ed | 1);
  const int R = Ed >= kGatherThreads ? 1 : kGatherThreads / Ed;
  const int nacc = Ed * R;
  typename A::S* acc = reinterpret_cast<typename A::S*>(smem);  // [nacc]
  int* col = reinterpret_cast<int*>(acc + ((nacc + 1) & ~1));   // [Ed] column of each exercise state in a tile row
  int* src = col + ((Ed + 3) & ~3);                              // [Ed] column within a path row
  T* tile = reinterpret_cast<T*>(src + ((Ed + 3) & ~3));         // [Cn][Wt]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int pb = blockIdx.y;
  const int64_t N = a.num_paths;
  const T* P = static_cast<const T*>(a.paths) + (int64_t)pb * N * Td;
  T* X = xt + (int64_t)pb * E * N * d;
  for (int j = tid; j < nacc; j += kGatherThreads) acc[j] = A::zero();
  for (int j = tid; j < Ed; j += kGatherThreads) {
    src[j] = a.exercise_times[j / d] * d + j % d;
    col[j] = full ? src[j] : j;
  }
  const int64_t nchunks = (N + Cn - 1) / Cn;
  for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int64_t n0 = ch * Cn;
    const int cn = (int)((N - n0) < Cn ? (N - n0) : Cn);
    __syncthreads();
    if (full) {
      const T* base = P + n0 * Td;
      const int64_t count = (int64_t)cn * Td;
      constexpr int V = 16 / sizeof(T);
      if ((reinterpret_cast<uintptr_t>(base) & 15u) == 0 && count % V == 0) {
        const uint4* b4 = reinterpret_cast<const uint4*>(base);
        uint4* t4 = reinterpret_cast<uint4*>(tile);
        const int64_t n4 = count / V;
#pragma unroll 4
        for (int64_t q = tid; q < n4; q += kGatherThreads) t4[q] = __ldg(b4 + q);
      } else {
        for (int64_t q = tid; q < count; q += kGatherThreads) tile[q] = base[q];
      }
    } else {
      // one warp per path row, lanes over the exercise columns
      for (int nl = warp; nl < cn; nl += kGatherThreads / 32) {
        const T* row = P + (n0 + nl) * Td;
        for (int r = lane; r < Ed; r += 32) tile[nl * Wt + r] = row[src[r]];
      }
    }
    __syncthreads();
    // store [E][N][d]: one warp per exercise date, lanes over (path, component)
    for (int e = warp; e < E; e += kGatherThreads / 32) {
      T* dst = X + ((int64_t)e * N + n0) * d;
      if (d == 1) {
        const int ce = col[e];
        for (int q = lane; q < cn; q += 32) dst[q] = tile[q * Wt + ce];
      } else {
        for (int q = lane; q < cn * d; q += 32) {
          const int nl = q / d, c = q - nl * d;
          dst[q] = tile[nl * Wt + col[e * d + c]];
        }
      }
    }
    // column sums: replica r sums paths r, r + R, ... in the dtype
    for (int it = tid; it < nacc; it += kGatherThreads) {
      const int j = it % Ed, r = it / Ed;
      const int cj = col[j];
      T sum = T(0);
      for (int nl = r; nl < cn; nl += R) sum += tile[(int64_t)nl * Wt + cj];
      acc[it] = A::add(acc[it], sum);
    }
  }
  __syncthreads();
  typename A::S* out = partials + ((size_t)blockIdx.x * gridDim.y + pb) * E * kMaxDimLsm;
  for (int j = tid; j < E * kMaxDimLsm; j += kGatherThreads) {
    const int e = j / kMaxDimLsm, c = j % kMaxDimLsm;
    typename A::S v = A::zero();
    if (c < d)
      for (int r = 0; r < R; ++r) v = A::sum(v, acc[r * Ed + e * d + c]);
    out[j] = v;
  }
}

template <typename T, int DM>
struct LsmCtx {
  const tqf_lsm_args& a;
  const T* xt;
  int b, pb, G, d;
  const int8_t* exps;  // [G][16] in shared memory (structured)
  __device__ T ratio(int i, int64_t n) const {
    const T* D = static_cast<const T*>(a.discount);
    const int64_t o = n * a.disc_stride_n + (int64_t)b * a.disc_stride_b;
    return D[(int64_t)(i + 1) * a.disc_stride_e + o] / D[(int64_t)i * a.disc_stride_e + o];
  }
  // D[i+1]/D[i] for this path: hoisted value when the discounts do not vary by path.
  __device__ __forceinline__ T ratio_at(int i, int64_t n, T hoisted) const {
    return a.disc_stride_n == 0 ? hoisted : ratio(i, n);
  }
  // Exercise value at exercise index e (basket put on the gathered states) or
  // from the caller's [N][B] array; x receives the states.
  __device__ T payoff(const void* expl, int e, int64_t n, T* x) const {
    if (a.degree < 0) return static_cast<const T*>(expl)[n * a.batch + b];
    const T* S = xt + (((int64_t)pb * a.num_exercise + e) * a.num_paths + n) * d;
    T s = T(0);
#pragma unroll
    for (int c = 0; c < DM; ++c)
      if (c < d) {
        x[c] = S[c];
        s += x[c];
      }
    const T K = static_cast<const T*>(a.strikes)[b];
    const T v = K - (d == 1 ? s : s / (T)d);
    return v > T(0) ? v : T(0);
  }
  // Basis function g at the path (structured: centred powers of x).
  __device__ T basis(const void* expl, int g, int64_t n, const T* xc) const {
    if (a.degree < 0) return static_cast<const T*>(expl)[((int64_t)pb * G + g) * a.num_paths + n];
    T p = T(1);
#pragma unroll
    for (int c = 0; c < DM; ++c)
      if (c < d) p *= ipow(xc[c], (int)exps[g * kMaxDimLsm + c]);
    return p;
  }
  // All NG basis functions (compile-time count).  One dimension: the powers
  // 1, x, x^2, ... by repeated multiplication (the same products as ipow).
  template <int NG>
  __device__ __forceinline__ void basis_all(const void* expl, int64_t n, const T* xc, T* phi) const {
    if (DM == 1 && a.degree >= 0) {
      phi[0] = T(1);
#pragma unroll
      for (int g = 1; g < NG; ++g) phi[g] = phi[g - 1] * xc[0];
    } else {
#pragma unroll
      for (int g = 0; g < NG; ++g) phi[g] = basis(expl, g, n, xc);
    }
  }
};

template <typename T, int DM, int GR>
__global__ void lsm_pass_kernel(tqf_lsm_args a, const T* __restrict__ xt, void* __restrict__ partials_raw,
                                const double* __restrict__ beta, const double* __restrict__ means, int C) {
  grid_dependency_wait();  // a programmatic dependent launch in the exercise-date chain
  allow_dependent_launch();
  using A = Acc<T>;
  using S = typename A::S;
  constexpr int GN = GR > 0 ? GR : 1;                    // compile-time basis size (register mode)
  constexpr int EN = GN * (GN + 1) / 2 + GN;              // its accumulator entries
  S* partials = static_cast<S*>(partials_raw);
  extern __shared__ __align__(16) unsigned char smem[];
  const int G = GR > 0 ? GR : a.num_basis, d = a.dim, B = a.batch;
  const int En = lsm_entries(G);
  const int W = lsm_row_stride(G);
  const int nitems = En > C ? En : C;
  T* phi_s = reinterpret_cast<T*>(smem);  // [C][W]
  S* acc_s = reinterpret_cast<S*>(smem + (((size_t)C * W * sizeof(T) + 15) & ~(size_t)15));  // [nitems]
  uint32_t* pair_s = reinterpret_cast<uint32_t*>(acc_s + nitems);                          // [nitems]
  T* beta_s = reinterpret_cast<T*>(pair_s + nitems);                                       // [G]
  T* mu_s = beta_s + G;                                                                    // [2][16]
  double* red_s = reinterpret_cast<double*>(
      reinterpret_cast<unsigned char*>(beta_s) + ((G + 2 * kMaxDimLsm) * sizeof(T) + 15) / 16 * 16);  // [64]
  int8_t* exps_s = reinterpret_cast<int8_t*>(red_s + 64);  // [G][16]
  const int tid = threadIdx.x;
  const int b = blockIdx.y;
  const int pb = a.paths_batch > 1 ? b : 0;
  const int R = En >= C ? 1 : C / En;  // replicas of each accumulator entry
  const int items = En * R;
  const int tri = G * (G + 1) / 2;
  for (int i = tid; i < items; i += C) {
    acc_s[i] = A::zero();
    // entry -> (j, k): packed upper triangle row-major, then the X'y column (k = G)
    const int e = i % En;
    int j = 0, k = G;
    if (e < tri) {
      int rem = e;
      while (rem >= G - j) {
        rem -= G - j;
        ++j;
      }
      k = j + rem;
    } else {
      j = e - tri;
    }
    pair_s[i] = (uint32_t)j | ((uint32_t)k << 16);
  }
  if (a.upd_index >= 1)
    for (int g = tid; g < G; g += C) beta_s[g] = (T)beta[(size_t)b * G + g];
  if (a.degree >= 0) {
    for (int i = tid; i < G * kMaxDimLsm; i += C) {
      const int g = i / kMaxDimLsm, c = i % kMaxDimLsm;
      exps_s[i] = c < d ? (int8_t)a.exponents[g * d + c] : (int8_t)0;
    }
    const int E0 = a.num_exercise;
    for (int i = tid; i < 2 * kMaxDimLsm; i += C) {
      const int which = i / kMaxDimLsm, c = i % kMaxDimLsm;
      const int idx = which == 0 ? a.upd_index : a.acc_index;
      mu_s[i] = idx >= 1 ? (T)means[((size_t)pb * E0 + (idx - 1)) * kMaxDimLsm + c] : T(0);
    }
  }
  __syncthreads();
  LsmCtx<T, DM> ctx{a, xt, b, pb, G, d, exps_s};
  // discount ratios that do not depend on the path
  const T r_upd = a.upd_index >= 1 && a.disc_stride_n == 0 ? ctx.ratio(a.upd_index, 0) : T(0);
  const T r_acc = a.acc_index >= 1 && a.disc_stride_n == 0 ? ctx.ratio(a.acc_index, 0) : T(0);
  const T r_fin = a.final_pass && a.disc_stride_n == 0 ? ctx.ratio(0, 0) : T(0);
  // register mode: per-thread products summed in the dtype over <= kSubSum paths
  T part[EN];
  S acc2[EN];
  int cnt = 0;
#pragma unroll
  for (int e = 0; e < EN; ++e) {
    part[e] = T(0);
    acc2[e] = A::zero();
  }
  const int E = a.num_exercise;
  T* state = static_cast<T*>(a.state);
  T* cash = state + (size_t)b * a.num_paths;
  T* vals = state + ((size_t)B + b) * a.num_paths;
  const int64_t n_cal = a.num_calibration > 0 ? a.num_calibration : a.num_paths;
  const int64_t price_from = a.num_calibration > 0 ? a.num_calibration : 0;
  S final_acc = A::zero();
  const int64_t nchunks = (a.num_paths + C - 1) / C;
  for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int64_t n = ch * C + tid;
    const bool valid = n < a.num_paths;
    T x[DM], xc[DM];
    T c = T(0), v = T(0);
    if (valid) {
      if (a.init) {
        c = ctx.payoff(a.init_payoff, E - 1, n, x);
        v = T(0);
      } else {
        c = cash[n];
        v = vals[n];
      }
      if (a.upd_index >= 1) {
        // continuation = relu(design . beta), exercise where payoff > continuation (lsm.py:380-400)
        const int iu = a.upd_index;
        const T evu = ctx.payoff(a.upd_payoff, iu - 1, n, x);
        if (a.degree >= 0) {
#pragma unroll
          for (int q = 0; q < DM; ++q) xc[q] = q < d ? x[q] - mu_s[q] : T(0);
        }
        T cont = T(0);
        if (GR > 0) {
          T phi[GN];
          ctx.template basis_all<GN>(a.upd_design, n, xc, phi);
#pragma unroll
          for (int g = 0; g < GN; ++g) cont += phi[g] * beta_s[g];
        } else {
          for (int g = 0; g < G; ++g) cont += ctx.basis(a.upd_design, g, n, xc) * beta_s[g];
        }
        cont = cont > T(0) ? cont : T(0);
        const bool ex_now = evu > cont;
        const T vn = ex_now ? T(0) : c + v;
        c = ex_now ? evu : T(0);
        v = ctx.ratio_at(iu, n, r_upd) * vn;
      }
      if (a.final_pass) {
        if (n >= price_from) final_acc = A::add(final_acc, ctx.ratio_at(0, n, r_fin) * (c + v));
      } else {
        cash[n] = c;
        vals[n] = v;
      }
    }
    if (GR > 0 && a.acc_index >= 1) {
      // masked normal equations of exercise index ia (lsm.py:355-379), in registers
      const int ia = a.acc_index;
      if (valid && n < n_cal) {
        const T cv = ctx.ratio_at(ia, n, r_acc) * (v + c);
        const T eva = ctx.payoff(a.acc_payoff, ia - 1, n, x);
        if (a.degree >= 0) {
#pragma unroll
          for (int q = 0; q < DM; ++q) xc[q] = q < d ? x[q] - mu_s[kMaxDimLsm + q] : T(0);
        }
        T phi[GN];
        ctx.template basis_all<GN>(a.acc_design, n, xc, phi);
        const bool use = eva > T(0);
#pragma unroll
        for (int g = 0; g < GN; ++g) phi[g] = use ? phi[g] : T(0);
        int e = 0;
#pragma unroll
        for (int j = 0; j < GN; ++j)
#pragma unroll
          for (int k = j; k < GN; ++k) part[e++] += phi[j] * phi[k];
#pragma unroll
        for (int j = 0; j < GN; ++j) part[e++] += phi[j] * cv;
        if (++cnt == kSubSum) {
#pragma unroll
          for (int q = 0; q < EN; ++q) {
            acc2[q] = A::add(acc2[q], part[q]);
            part[q] = T(0);
          }
          cnt = 0;
        }
      }
    } else if (a.acc_index >= 1) {
      // masked normal equations of exercise index ia (lsm.py:355-379)
      const int ia = a.acc_index;
      T* row = phi_s + (size_t)tid * W;
      if (valid) {
        const T cv = ctx.ratio_at(ia, n, r_acc) * (v + c);
        const T eva = ctx.payoff(a.acc_payoff, ia - 1, n, x);
        const bool use = eva > T(0) && n < n_cal;
        if (a.degree >= 0) {
#pragma unroll
          for (int q = 0; q < DM; ++q) xc[q] = q < d ? x[q] - mu_s[kMaxDimLsm + q] : T(0);
        }
        for (int g = 0; g < G; ++g) row[g] = use ? ctx.basis(a.acc_design, g, n, xc) : T(0);
        row[G] = n < n_cal ? cv : T(0);
      } else {
        for (int g = 0; g <= G; ++g) row[g] = T(0);
      }
      __syncthreads();
      for (int it = tid; it < items; it += C) {
        const int r = it / En;
        const int j = (int)(pair_s[it] & 0xFFFFu), k = (int)(pair_s[it] >> 16);
        S s = A::zero();
        int p = r;
        while (p < C) {
          T part = T(0);
          for (int q = 0; q < kSubSum && p < C; ++q, p += R) part += phi_s[(size_t)p * W + j] * phi_s[(size_t)p * W + k];
          s = A::add(s, part);
        }
        acc_s[it] = A::sum(acc_s[it], s);
      }
      __syncthreads();
    }
  }
  if (GR > 0 && a.acc_index >= 1) {
    // flush, then a fixed-order block reduction (warp shuffles, then warps in order)
    // Each thread's value (at most kSubSum products unless it was flushed) is
    // rounded to the dtype for a pairwise warp tree (32 values); warps and CTAs
    // are then combined in the compensated / FP64 accumulator.
    S* red = acc_s;  // [C/32][EN]
#pragma unroll
    for (int q = 0; q < EN; ++q) {
      T t = (T)A::value(A::add(acc2[q], part[q]));
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if ((tid & 31) == 0) red[(tid >> 5) * EN + q] = A::add(A::zero(), t);
    }
    __syncthreads();
    S* out = partials + ((size_t)blockIdx.x * B + b) * EN;
    for (int q = tid; q < EN; q += C) {
      S t = A::zero();
      for (int w = 0; w < C / 32; ++w) t = A::sum(t, red[w * EN + q]);
      out[q] = t;
    }
  } else if (a.acc_index >= 1) {
    S* out = partials + ((size_t)blockIdx.x * B + b) * En;
    for (int e = tid; e < En; e += C) {
      S s = A::zero();
      for (int r = 0; r < R; ++r) s = A::sum(s, acc_s[r * En + e]);
      out[e] = s;
    }
  }
  if (a.final_pass) {
    // fixed-order block sum
    for (int o = 16; o > 0; o >>= 1) final_acc = A::sum(final_acc, A::shfl_down(final_acc, o));
    S* red = reinterpret_cast<S*>(red_s);
    if ((tid & 31) == 0) red[tid >> 5] = final_acc;
    __syncthreads();
    if (tid == 0) {
      S s = A::zero();
      for (int w = 0; w < C / 32; ++w) s = A::sum(s, red[w]);
      partials[(size_t)blockIdx.x * B + b] = s;
    }
  }
}

template <typename T, int DM>
__host__ inline void* pass_kernel_dm(int G) {
  if constexpr (DM <= 2) {
    switch (G) {
      case 2: return reinterpret_cast<void*>(&lsm_pass_kernel<T, DM, 2>);
      case 3: return reinterpret_cast<void*>(&lsm_pass_kernel<T, DM, 3>);
      case 4: return reinterpret_cast<void*>(&lsm_pass_kernel<T, DM, 4>);
      case 5: return reinterpret_cast<void*>(&lsm_pass_kernel<T, DM, 5>);
      default: break;
    }
  }
  return reinterpret_cast<void*>(&lsm_pass_kernel<T, DM, 0>);
}

template <typename T>
__host__ inline void* pass_kernel_for(int d, int G) {
  if (d <= 1) return pass_kernel_dm<T, 1>(G);
  if (d <= 2) return pass_kernel_dm<T, 2>(G);
  if (d <= 4) return pass_kernel_dm<T, 4>(G);
  return pass_kernel_dm<T, 16>(G);
}

__global__ void lsm_scale_kernel(double* __restrict__ v, int n, double s) {
  grid_dependency_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] *= s;
}

// Jacobi rotation (c, s) for the symmetric 2x2 block (app, apq; apq, aqq)
// (Golub & Van Loan, sym.schur2).  The angle only has to shrink apq, so it is
// computed in FP32 from the entries scaled by sc (a power of two); (c, s) are
// then renormalised in FP64 to c^2 + s^2 = 1 with a second-order correction
// (|c^2 + s^2 - 1| ~ 1e-7 before, ~1e-21 after), keeping the rotation
// orthogonal to FP64 precision without FP64 division or square root.  The
// residual apq (~1e-7 of its old value) is removed by the following sweeps.
__device__ __forceinline__ void jacobi_cs(double app, double aqq, double apq, double sc, double& c, double& s) {
  c = 1.0;
  s = 0.0;
  const float fp = (float)(apq * sc);
  if (fp == 0.f) return;
  const float fd = (float)((aqq - app) * sc);
  const float th = fd / (2.f * fp);
  const float ath = fabsf(th);
  float t;
  if (ath > 1e18f)
    t = 0.5f / th;
  else
    t = copysignf(1.f, th) / (ath + sqrtf(fmaf(th, th, 1.f)));
  const float cf = rsqrtf(fmaf(t, t, 1.f));
  c = (double)cf;
  s = (double)(t * cf);
  const double dl = fma(c, c, s * s) - 1.0;
  const double f = 1.0 - dl * (0.5 - 0.375 * dl);
  c *= f;
  s *= f;
}

// One CTA per batch member: A = X'X (packed) -> Jacobi eigen-decomposition
// A = V diag(l) V^T; beta = V diag(l+) V^T (X'y), l+ = 1/l where |l| > cutoff.
// Parallel cyclic Jacobi: each round applies G/2 disjoint rotations (round-
// robin pairing), columns then rows.  One warp for <= 16 basis functions
// (V in shared memory), 256 threads above (V in the workspace).
template <int GC>
__global__ void __launch_bounds__(kSolveThreads)
    lsm_solve_kernel(const double* __restrict__ sums, int Gr, double rcond, double* __restrict__ beta,
                     double* __restrict__ Vg, int warm) {
  grid_dependency_wait();  // a programmatic dependent launch in the exercise-date chain
  allow_dependent_launch();
  extern __shared__ __align__(16) unsigned char smem[];
  const int G = GC > 0 ? GC : Gr;  // compile-time size for small systems (constant index arithmetic)
  const int P = G + 1;  // row stride of A
  const int nt = blockDim.x;
  double* A = reinterpret_cast<double*>(smem);  // [G][G+1]
  double* rhs = A + (size_t)G * P;               // [G]
  double* w = rhs + G;                           // [G]
  double* cs = w + G;                            // [2][kMaxBasis/2]
  int* pq = reinterpret_cast<int*>(cs + kMaxBasis);  // [2][kMaxBasis/2]
  double* red = reinterpret_cast<double*>(pq + kMaxBasis);  // [kSolveThreads/32][2]
  double* Vs = red + kSolveThreads / 32 * 2;                // [G][G] when G <= 16
  double* Tm = Vs + (G <= 16 ? G * G : 0);                  // [G][G+1] when warm
  const int b = blockIdx.x, tid = threadIdx.x;
  const int En = lsm_entries(G);
  const double* s = sums + (size_t)b * En;
  double* Vb = Vg + (size_t)b * G * G;  // eigenvectors kept between exercise dates
  double* V = G <= 16 ? Vs : Vb;
  const int tri = G * (G + 1) / 2;
  for (int e = tid; e < tri; e += nt) {
    int j = 0, rem = e;
    while (rem >= G - j) {
      rem -= G - j;
      ++j;
    }
    const int k = j + rem;
    A[j * P + k] = s[e];
    A[k * P + j] = s[e];
  }
  for (int j = tid; j < G; j += nt) rhs[j] = s[tri + j];
  if (warm) {
    // warm start from the previous exercise date's eigenvectors: A <- V^T A V
    if (G <= 16)
      for (int i = tid; i < G * G; i += nt) V[i] = Vb[i];
    __syncthreads();
    for (int it = tid; it < G * G; it += nt) {
      const int i = it / G, j = it % G;
      double x = 0.0;
      for (int k = 0; k < G; ++k) x = fma(A[i * P + k], V[k * G + j], x);
      Tm[i * P + j] = x;
    }
    __syncthreads();
    for (int it = tid; it < G * G; it += nt) {
      const int i = it / G, j = it % G;
      double x = 0.0;
      for (int k = 0; k < G; ++k) x = fma(V[k * G + i], Tm[k * P + j], x);
      A[i * P + j] = x;
    }
    __syncthreads();
    // exact symmetry
    for (int it = tid; it < G * G; it += nt) {
      const int i = it / G, j = it % G;
      if (i < j) {
        const double m = 0.5 * (A[i * P + j] + A[j * P + i]);
        A[i * P + j] = m;
        A[j * P + i] = m;
      }
    }
  } else {
    for (int i = tid; i < G * G; i += nt) V[i] = (i / G == i % G) ? 1.0 : 0.0;
  }
  __syncthreads();
  const int Pe = G + (G & 1);
  const int half = Pe / 2;
  for (int sweep = 0; sweep < kMaxJacobiSweeps && G > 1; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = tid; i < G * G; i += nt) {
      const double x = A[(i / G) * P + i % G];
      tot += x * x;
      if (i / G != i % G) off += x * x;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_down_sync(0xffffffffu, off, o);
      tot += __shfl_down_sync(0xffffffffu, tot, o);
    }
    if ((tid & 31) == 0) {
      red[(tid >> 5) * 2] = off;
      red[(tid >> 5) * 2 + 1] = tot;
    }
    __syncthreads();
    double OFF = 0.0, TOT = 0.0;
    for (int q = 0; q < nt / 32; ++q) {
      OFF += red[q * 2];
      TOT += red[q * 2 + 1];
    }
    __syncthreads();
    if (OFF <= 1e-30 * TOT || OFF == 0.0) break;
    int ex2;
    frexp(TOT, &ex2);
    const double sc = ldexp(1.0, -(ex2 / 2));  // power of two: entries * sc = O(1)
    for (int r = 0; r < Pe - 1; ++r) {
      // round-robin pairing: round r pairs (r + k, r - k) mod (Pe - 1), k = 0 with the last index
      if (tid < half) {
        const int k = tid;
        const int i1 = (r + k) % (Pe - 1);
        const int i2 = k == 0 ? Pe - 1 : (Pe - 1 - k + r) % (Pe - 1);
        const int p = i1 < i2 ? i1 : i2, q = i1 < i2 ? i2 : i1;
        double c = 1.0, sn = 0.0;
        if (q < G) jacobi_cs(A[p * P + p], A[q * P + q], A[p * P + q], sc, c, sn);
        cs[2 * k] = c;
        cs[2 * k + 1] = sn;
        pq[2 * k] = p;
        pq[2 * k + 1] = q < G ? q : -1;
      }
      __syncthreads();
      // A <- A J (columns p, q)
      for (int it = tid; it < G * half; it += nt) {
        const int i = it / half, k = it % half;
        const int p = pq[2 * k], q = pq[2 * k + 1];
        if (q < 0) continue;
        const double c = cs[2 * k], sn = cs[2 * k + 1];
        const double aip = A[i * P + p], aiq = A[i * P + q];
        A[i * P + p] = c * aip - sn * aiq;
        A[i * P + q] = sn * aip + c * aiq;
      }
      __syncthreads();
      // A <- J^T A (rows p, q)
      for (int it = tid; it < G * half; it += nt) {
        const int k = it / G, j = it % G;
        const int p = pq[2 * k], q = pq[2 * k + 1];
        if (q < 0) continue;
        const double c = cs[2 * k], sn = cs[2 * k + 1];
        const double apj = A[p * P + j], aqj = A[q * P + j];
        A[p * P + j] = c * apj - sn * aqj;
        A[q * P + j] = sn * apj + c * aqj;
      }
      // V <- V J
      for (int it = tid; it < G * half; it += nt) {
        const int i = it / half, k = it % half;
        const int p = pq[2 * k], q = pq[2 * k + 1];
        if (q < 0) continue;
        const double c = cs[2 * k], sn = cs[2 * k + 1];
        const double vip = V[i * G + p], viq = V[i * G + q];
        V[i * G + p] = c * vip - sn * viq;
        V[i * G + q] = sn * vip + c * viq;
      }
      __syncthreads();
    }
  }
  __syncthreads();
  // cutoff = rcond * max |l|  (tf.linalg.pinv keeps singular values > cutoff)
  double lmax = 0.0;
  for (int j = 0; j < G; ++j) lmax = fmax(lmax, fabs(A[j * P + j]));
  const double cutoff = rcond * lmax;
  for (int j = tid; j < G; j += nt) {
    double u = 0.0;
    for (int i = 0; i < G; ++i) u += V[i * G + j] * rhs[i];
    const double l = A[j * P + j];
    w[j] = fabs(l) > cutoff && l != 0.0 ? u / l : 0.0;
  }
  __syncthreads();
  for (int i = tid; i < G; i += nt) {
    double x = 0.0;
    for (int j = 0; j < G; ++j) x += V[i * G + j] * w[j];
    beta[(size_t)b * G + i] = x;
  }
  if (G <= 16)
    for (int i = tid; i < G * G; i += nt) Vb[i] = V[i];
}

// ---- the whole backward loop in one cooperative kernel --------------------------
// For the common structured case (one payoff, one path set, d <= 2 and 2..5
// basis functions) tqf_lsm_price runs every exercise date in one cooperative
// launch instead of three launches per date.  Per date all CTAs run the pass
// (the register-mode arithmetic of lsm_pass_kernel) and store their partial
// sums; a grid barrier; CTA 0 reduces the partials in a fixed order and its
// first warp solves the 2..5-function system (below); a second barrier
// releases the next date.  Both barriers are bounded waits: after
// kLoopSpinLimit polls the CTA sets the abort word and TQF_E_TIMEOUT in
// dev_status and every CTA leaves.  Data crossing CTAs (partials, beta) is
// written and read with L2-only accesses (__stcg / __ldcg).
constexpr int kLoopThreads = 256;
constexpr unsigned kLoopSpinLimit = 1u << 24;
constexpr int kLoopMaxG = 5;
constexpr int kLoopMaxEn = kLoopMaxG * (kLoopMaxG + 1) / 2 + kLoopMaxG;

struct LoopSync {
  unsigned int count;
  unsigned int abort;
};

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) {
  return *reinterpret_cast<const volatile unsigned*>(p);
}

// Grid barrier number `gen` (1, 2, ...): returns false when it was aborted.
__device__ bool loop_barrier(LoopSync* sy, unsigned gen, int32_t* status) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(&sy->count, 1u);
    const unsigned target = gen * gridDim.x;
    int ok = 1;
    for (unsigned it = 0;; ++it) {
      if (ld_volatile(&sy->count) >= target) break;
      if (ld_volatile(&sy->abort)) {
        ok = 0;
        break;
      }
      if (it > kLoopSpinLimit) {
        ok = 0;
        atomicExch(&sy->abort, 1u);
        if (status) atomicExch(status, TQF_E_TIMEOUT);
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// The rotation (c, s) of the pair (x, xp) of the current round, from the
// lanes holding A_pp, A_qq and A_pq (Golub & Van Loan, sym.schur2); identity
// when x has no partner.  Kept out of line: the pseudo-inverse runs in one
// warp per date, so its code is cold in the instruction cache and small code
// is what makes it fast.
template <int G>
__device__ __noinline__ float2 jacobi_rot_f32(float af, int x, int xp) {
  const int p = xp < 0 ? x : (x < xp ? x : xp), q = xp < 0 ? x : (x < xp ? xp : x);
  const float app = __shfl_sync(0xffffffffu, af, p * G + p);
  const float aqq = __shfl_sync(0xffffffffu, af, q * G + q);
  const float apq = __shfl_sync(0xffffffffu, af, p * G + q);
  float c = 1.f, sn = 0.f;
  // |apq| below 2^-100 of the diagonal gap needs no rotation (and keeps the
  // fast approximate division away from overflow); the angle only has to be
  // FP32-accurate, so the SFU division and square root serve
  const float gap = aqq - app;
  if (xp >= 0 && fabsf(apq) > 7.9e-31f * fabsf(gap) && apq != 0.f) {
    const float th = __fdividef(gap, 2.f * apq);
    const float ath = fabsf(th);
    const float t = ath > 1e18f ? __fdividef(0.5f, th)
                                : __fdividef(copysignf(1.f, th), ath + sqrt_approx(fmaf(th, th, 1.f)));
    c = rsqrtf(fmaf(t, t, 1.f));
    sn = t * c;
  }
  return make_float2(c, sn);
}

// The pseudo-inverse of one date's masked Gram matrix A (G x G, G <= 5;
// packed upper triangle in `gram`, FP64, shared memory) as an explicit FP64
// matrix P = V_K B_KK^-1 V_K^T, formed by one warp.  FP64 is a narrow pipe on
// this GPU (a warp-wide FP64 instruction occupies it for ~64 cycles,
// measured, whatever the active lanes), so the eigenvectors come from cyclic
// Jacobi in FP32 and only a short FP64 stage follows:
//   1. lane i*G + j holds A_ij (and V_ij); A scaled by a power of two to
//      O(1); FP32 Jacobi sweeps from the identity (round-robin pairing over G
//      rounded up to even, partner of x in round r = 2r - x mod (Pe - 1), the
//      last index with r; the rotation of Golub & Van Loan's sym.schur2)
//      until the off-diagonal is below 1e-12 of the total or stops shrinking;
//   2. FP64: B = V^T A V with the FP32 V (any invertible V gives
//      A^-1 = V B^-1 V^T exactly, and B is diagonal to ~1e-7, so its diagonal
//      holds the eigenvalues to FP64 accuracy);
//   3. tf.linalg.pinv's cutoff (rcond x max |B_kk|) drops directions; the
//      kept block B_KK X = I_K is solved by Gaussian elimination in FP64 (one
//      row per lane, pivots on the diagonal, reciprocals from the FP32
//      reciprocal refined by two Newton steps; back substitution one column
//      per lane), and P = V X V^T.
// The Gram matrices do not depend on the regression coefficients, so the
// one-launch loop forms every date's P before its date loop, dates spread
// over CTAs; a date's coefficients are then P X'y.  Vs: [G G] FP32, Ws:
// [2 G G] and Bs: [G G + G] FP64 shared scratch.
template <int G>
__device__ __noinline__ void warp_pinv_matrix(const double* gram, double rcond, float* Vs, double* Ws, double* Bs,
                                              double* P_out) {
  const int lane = threadIdx.x & 31;
  const bool in = lane < G * G;
  const int i = in ? lane / G : 0, j = in ? lane % G : 0;
  auto packed = [](int r, int c) {
    const int p = r < c ? r : c, q = r < c ? c : r;
    return p * G - p * (p - 1) / 2 + (q - p);
  };
  const double a = in ? gram[packed(i, j)] : 0.0;
  // 1. FP32 Jacobi on A scaled by 2^-e (e from the largest diagonal entry)
  float af = (float)a;
  float dm = in && i == j ? fabsf(af) : 0.f;
  for (int o = 16; o > 0; o >>= 1) dm = fmaxf(dm, __shfl_xor_sync(0xffffffffu, dm, o));
  int e2 = 0;
  frexpf(dm > 0.f ? dm : 1.f, &e2);
  af *= ldexpf(1.f, -e2);
  float vf = in && i == j ? 1.f : 0.f;
  constexpr int Pe = G + (G & 1);
  auto partner = [](int x, int r) {
    constexpr int m = Pe - 1;
    int p;
    if (x == m) p = r;
    else if (x == r) p = m;
    else p = ((2 * r - x) % m + m) % m;
    return p < G ? p : -1;
  };
  float prev = 0.f;
#pragma unroll 1
  for (int sweep = 0; sweep < 30 && G > 1; ++sweep) {
    float off = in && i != j ? af * af : 0.f, tot = in ? af * af : 0.f;
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if (off <= 1e-12f * tot || off == 0.f) break;
    if (sweep > 0 && off > 0.25f * prev) break;  // at the FP32 rounding floor
    prev = off;
#pragma unroll 1
    for (int r = 0; r < Pe - 1; ++r) {
      const int ip = partner(i, r), jp = partner(j, r);
      const float2 rr = jacobi_rot_f32<G>(af, i, ip);
      const float2 rc = jacobi_rot_f32<G>(af, j, jp);
      const float cr = rr.x, sr = rr.y, cc = rc.x, sc2 = rc.y;
      const int jj = jp < 0 ? j : jp, ii = ip < 0 ? i : ip;
      const float a_ijp = __shfl_sync(0xffffffffu, af, i * G + jj);
      const float a_ipj = __shfl_sync(0xffffffffu, af, ii * G + j);
      const float a_ipjp = __shfl_sync(0xffffffffu, af, ii * G + jj);
      const float v_ijp = __shfl_sync(0xffffffffu, vf, i * G + jj);
      auto colr = [&](float self, float other) {
        if (jp < 0) return self;
        return j < jp ? cc * self - sc2 * other : sc2 * other + cc * self;
      };
      const float b_ij = colr(af, a_ijp), b_ipj = colr(a_ipj, a_ipjp);
      float an = b_ij;
      if (ip >= 0) an = i < ip ? cr * b_ij - sr * b_ipj : sr * b_ipj + cr * b_ij;
      const float vn = colr(vf, v_ijp);
      af = in ? an : 0.f;
      vf = in ? vn : 0.f;
    }
  }
  // 2. FP64: B = V^T A V (W = A V first)
  double* As = Ws + G * G;
  if (in) {
    Vs[lane] = vf;
    As[lane] = a;
  }
  __syncwarp();
  {
    double w = 0.0;
    if (in)
      for (int l = 0; l < G; ++l) w = fma(As[i * G + l], (double)Vs[l * G + j], w);
    __syncwarp();
    if (in) Ws[lane] = w;
    __syncwarp();
    double b = 0.0;
    if (in)
      for (int k = 0; k < G; ++k) b = fma((double)Vs[k * G + i], Ws[k * G + j], b);
    if (in) Bs[lane] = b;
    __syncwarp();
  }
  // 3. cutoff on the diagonal; B_KK X = I_K by elimination, row i in lane i
  double lmax = 0.0;
  for (int k = 0; k < G; ++k) lmax = fmax(lmax, fabs(Bs[k * G + k]));
  const double cutoff = rcond * lmax;
  auto kept = [&](int k) { const double l = Bs[k * G + k]; return fabs(l) > cutoff && l != 0.0; };
  double row[2 * G];
  const int ri = lane < G ? lane : 0;
  const bool kr = kept(ri);
#pragma unroll
  for (int c = 0; c < G; ++c) {
    row[c] = kr && kept(c) ? Bs[ri * G + c] : (c == ri ? 1.0 : 0.0);
    row[G + c] = kr && c == ri ? 1.0 : 0.0;
  }
  __syncwarp();
  double rcp[G];
#pragma unroll
  for (int p = 0; p < G; ++p) {
    const double dd = __shfl_sync(0xffffffffu, row[p], p);
    double r0 = (double)__frcp_rn((float)dd);
    r0 = r0 * fma(-dd, r0, 2.0);
    r0 = r0 * fma(-dd, r0, 2.0);
    rcp[p] = r0;
    const double f = row[p] * r0;
#pragma unroll
    for (int c = p + 1; c < 2 * G; ++c) {
      const double pc = __shfl_sync(0xffffffffu, row[c], p);
      if (lane > p) row[c] = fma(-f, pc, row[c]);
    }
  }
  // U | Y rows to shared memory; lane m solves column m of X
  if (lane < G)
#pragma unroll
    for (int c = 0; c < 2 * G; ++c) Ws[lane * 2 * G + c] = row[c];
  __syncwarp();
  double x[G];
  const int m = lane < G ? lane : 0;
#pragma unroll
  for (int p = G - 1; p >= 0; --p) {
    double t = Ws[p * 2 * G + G + m];
#pragma unroll
    for (int c = p + 1; c < G; ++c) t = fma(-Ws[p * 2 * G + c], x[c], t);
    x[p] = t * rcp[p];
  }
  __syncwarp();
  if (lane < G)
#pragma unroll
    for (int p = 0; p < G; ++p) Bs[p * G + m] = x[p];  // X[p][m]
  __syncwarp();
  // 4. P = V X V^T, lane (j, k) = (i, j)
  if (in) {
    double pv = 0.0;
    for (int r = 0; r < G; ++r) {
      double w = 0.0;
      for (int c = 0; c < G; ++c) w = fma(Bs[r * G + c], (double)Vs[j * G + c], w);
      pv = fma((double)Vs[i * G + r], w, pv);
    }
    __stcg(P_out + lane, pv);
  }
  __syncwarp();
}

// Per-thread path state of the loop kernel lives in shared memory for the
// whole loop: the K paths n = (blockIdx.x + k gridDim.x) C + tid of thread
// tid keep cashflow, value and the states at the last accumulated date
// (which the next date's update reads), [K][C] each, so a date reads only
// its new exercise date from the gathered states.
template <typename T, int DM>
__host__ __device__ inline size_t lsm_loop_smem(int K) {
  return (size_t)K * kLoopThreads * (2 + DM) * sizeof(T);
}

// Two CTAs per SM (three, with 85 registers, measured 1.44 against 1.29 ms
// per call for 2^20 float paths x 50 dates: more CTAs at every barrier and
// more partial rows per reduction).
template <typename T, int DM, int GN>
__global__ void __launch_bounds__(kLoopThreads, 2)
    lsm_loop_kernel(tqf_lsm_args a, const T* __restrict__ xt, typename Acc<T>::S* __restrict__ partials,
                    double* __restrict__ beta, const double* __restrict__ means, LoopSync* sy, int K,
                    double* __restrict__ gram, double* __restrict__ pinv) {
  using A = Acc<T>;
  using S = typename A::S;
  constexpr int EA = GN * (GN + 1) / 2;  // Gram entries (packed upper triangle)
  constexpr int C = kLoopThreads;
  constexpr int KB = 8;  // paths per batch of loads
  extern __shared__ __align__(16) unsigned char dsm[];
  T* cs_ = reinterpret_cast<T*>(dsm);  // [K][C] cashflow
  T* vs_ = cs_ + (size_t)K * C;        // [K][C] value
  T* xs_ = vs_ + (size_t)K * C;        // [K][DM][C] states at the last accumulated date
  __shared__ T beta_s[GN];
  __shared__ T mu_s[2][kMaxDimLsm];
  __shared__ S red[C / 32][EA];
  __shared__ double sums_s[kLoopMaxEn];
  __shared__ float Vs[kLoopMaxG * kLoopMaxG];
  __shared__ double Ws[2 * kLoopMaxG * kLoopMaxG], Bs[kLoopMaxG * kLoopMaxG + kLoopMaxG];
  __shared__ S rsum[16][16];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int d = a.dim, E = a.num_exercise;
  const int64_t N = a.num_paths;
  const T K_strike = static_cast<const T*>(a.strikes)[0];
  const int64_t n_cal = a.num_calibration > 0 ? a.num_calibration : N;
  const int64_t price_from = a.num_calibration > 0 ? a.num_calibration : 0;
  const double eps = sizeof(T) == 4 ? 1.1920928955078125e-07 : 2.220446049250313e-16;
  const double rcond = 10.0 * GN * eps;
  LsmCtx<T, DM> ctx{a, xt, 0, 0, GN, d, nullptr};
  // basket put on the states (make_basket_put_payoff: relu(K - mean_d S))
  auto pay = [&](const T* x) {
    T sm = T(0);
#pragma unroll
    for (int c = 0; c < DM; ++c) sm += x[c];
    const T v = K_strike - (DM == 1 ? sm : sm / (T)d);
    return v > T(0) ? v : T(0);
  };
  auto load_x = [&](int date, int64_t n, T* x) {
    const T* p = xt + ((int64_t)date * N + n) * d;
#pragma unroll
    for (int c = 0; c < DM; ++c) x[c] = p[c];
  };
  // centred basis: DM = 1 the powers of x; DM = 2 the exponent grid
  // (g / (degree + 1), g % (degree + 1)) of make_polynomial_basis
  const int deg = a.degree;
  auto basis = [&](const T* xc, T* phi) {
    if constexpr (DM == 1) {
      phi[0] = T(1);
#pragma unroll
      for (int g = 1; g < GN; ++g) phi[g] = phi[g - 1] * xc[0];
    } else {
#pragma unroll
      for (int g = 0; g < GN; ++g)
        phi[g] = ipow(xc[0], (int)a.exponents[g * 2]) * ipow(xc[1], (int)a.exponents[g * 2 + 1]);
    }
  };
  (void)deg;
  // Block reduction of per-thread accumulators (the register mode of
  // lsm_pass_kernel) into this CTA's row of `dst` ([rows][width], 8-byte S).
  auto block_store = [&](const S* accv, const T* partv, int width, double* dst) {
    for (int q = 0; q < width; ++q) {
      T t = (T)A::value(A::add(accv[q], partv[q]));
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0) red[warp][q] = A::add(A::zero(), t);
    }
    __syncthreads();
    for (int q = tid; q < width; q += C) {
      S t = A::zero();
      for (int w = 0; w < C / 32; ++w) t = A::sum(t, red[w][q]);
      __stcg(dst + (size_t)blockIdx.x * width + q, *reinterpret_cast<double*>(&t));
    }
    __syncthreads();
  };
  // Fixed-order reduction of rows [gridDim.x][width] of `src` into sums_s:
  // thread (r, e), r < 16, sums rows r, r + 16, ... of entry e (eight loads
  // in flight), then the 16 groups in order.
  auto grid_reduce = [&](const double* src, int width) {
    const int e = tid & 15, r = tid >> 4;
    S t = A::zero();
    if (e < width) {
      const int rows = (int)gridDim.x;
      for (int row0 = r; row0 < rows; row0 += 128) {
        double raw[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int row = row0 + 16 * q;
          raw[q] = row < rows ? __ldcg(src + (size_t)row * width + e) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (row0 + 16 * q < rows) t = A::sum(t, *reinterpret_cast<const S*>(&raw[q]));
      }
    }
    rsum[r][e] = t;
    __syncthreads();
    if (tid < width) {
      S u = A::zero();
      for (int q = 0; q < 16; ++q) u = A::sum(u, rsum[q][tid]);
      sums_s[tid] = A::value(u);
    }
    __syncthreads();
  };
  unsigned gen = 0;
  // Phase 1: the masked Gram matrix of every regression date (lsm.py:355-372)
  // depends only on that date's states, not on the coefficients of later
  // dates, so all of them are summed here, before the date loop, and each
  // date's pseudo-inverse is formed once (dates spread over CTAs).
  for (int acc = 1; acc <= E - 1; ++acc) {
    __syncthreads();
    for (int c = tid; c < DM; c += C) mu_s[1][c] = (T)means[(size_t)(acc - 1) * kMaxDimLsm + c];
    __syncthreads();
    T part[EA];
    S acc2[EA];
    int cnt = 0;
#pragma unroll
    for (int e = 0; e < EA; ++e) {
      part[e] = T(0);
      acc2[e] = A::zero();
    }
    for (int kb = 0; kb < K; kb += KB) {
      T xa[KB][DM];
#pragma unroll
      for (int q = 0; q < KB; ++q) {
        const int64_t n = ((int64_t)blockIdx.x + (int64_t)(kb + q) * gridDim.x) * C + tid;
#pragma unroll
        for (int c = 0; c < DM; ++c) xa[q][c] = T(0);
        if (kb + q < K && n < n_cal) load_x(acc - 1, n, xa[q]);
      }
#pragma unroll
      for (int q = 0; q < KB; ++q) {
        const int64_t n = ((int64_t)blockIdx.x + (int64_t)(kb + q) * gridDim.x) * C + tid;
        if (kb + q >= K || n >= n_cal) continue;
        T xc[DM], phi[GN];
#pragma unroll
        for (int cc = 0; cc < DM; ++cc) xc[cc] = xa[q][cc] - mu_s[1][cc];
        basis(xc, phi);
        const bool use = pay(xa[q]) > T(0);
#pragma unroll
        for (int g = 0; g < GN; ++g) phi[g] = use ? phi[g] : T(0);
        int e = 0;
#pragma unroll
        for (int jj = 0; jj < GN; ++jj)
#pragma unroll
          for (int kk = jj; kk < GN; ++kk) part[e++] += phi[jj] * phi[kk];
        if (++cnt == kSubSum) {
#pragma unroll
          for (int qq = 0; qq < EA; ++qq) {
            acc2[qq] = A::add(acc2[qq], part[qq]);
            part[qq] = T(0);
          }
          cnt = 0;
        }
      }
    }
    block_store(acc2, part, EA, gram + (size_t)acc * gridDim.x * EA);
  }
  if (!loop_barrier(sy, ++gen, a.dev_status)) return;
  for (int acc = 1 + (int)blockIdx.x; acc <= E - 1; acc += (int)gridDim.x) {
    grid_reduce(gram + (size_t)acc * gridDim.x * EA, EA);
    if (warp == 0) warp_pinv_matrix<GN>(sums_s, rcond, Vs, Ws, Bs, pinv + (size_t)acc * GN * GN);
    __syncthreads();
  }
  if (!loop_barrier(sy, ++gen, a.dev_status)) return;
  // Phase 2: the backward date loop.  Per date one pass (the exercise update
  // of the previous date with its coefficients, fused with this date's
  // masked right-hand side X'y), one grid barrier, then every CTA reduces the
  // GN sums in the same fixed order and forms beta = P X'y in FP64 itself
  // (identical in every CTA), so no second barrier broadcasts it.  The
  // partial rows alternate between two buffers by date: a CTA can run at
  // most one date ahead of the slowest reader (it cannot pass the next
  // barrier before every CTA has reduced), so it never overwrites rows that
  // are still being read.
  for (int step = 0;; ++step) {
    double* pout = reinterpret_cast<double*>(partials) + (size_t)(step & 1) * gridDim.x * GN;
    const int init = step == 0;
    const int upd = step == 0 ? 0 : E - step;
    const int acc = E - 1 - step;
    const int fin = acc < 1;
    __syncthreads();
    for (int i = tid; i < 2 * kMaxDimLsm; i += C) {
      const int which = i / kMaxDimLsm, c = i % kMaxDimLsm;
      const int idx = which == 0 ? upd : acc;
      mu_s[which][c] = idx >= 1 ? (T)means[(size_t)(idx - 1) * kMaxDimLsm + c] : T(0);
    }
    __syncthreads();
    const T r_upd = upd >= 1 && a.disc_stride_n == 0 ? ctx.ratio(upd, 0) : T(0);
    const T r_acc = acc >= 1 && a.disc_stride_n == 0 ? ctx.ratio(acc, 0) : T(0);
    const T r_fin = fin && a.disc_stride_n == 0 ? ctx.ratio(0, 0) : T(0);
    T part[GN];
    S acc2[GN];
    int cnt = 0;
#pragma unroll
    for (int e = 0; e < GN; ++e) {
      part[e] = T(0);
      acc2[e] = A::zero();
    }
    S final_acc = A::zero();
    for (int kb = 0; kb < K; kb += KB) {
      // the batch's loads first (the new accumulation date, and at the start
      // the last exercise date), so that they are in flight together
      T xa[KB][DM], xi[KB][DM];
#pragma unroll
      for (int q = 0; q < KB; ++q) {
        const int64_t n = ((int64_t)blockIdx.x + (int64_t)(kb + q) * gridDim.x) * C + tid;
        const bool ok = kb + q < K && n < N;
#pragma unroll
        for (int c = 0; c < DM; ++c) xa[q][c] = xi[q][c] = T(0);
        if (ok && acc >= 1) load_x(acc - 1, n, xa[q]);
        if (ok && init) load_x(E - 1, n, xi[q]);
      }
#pragma unroll
      for (int q = 0; q < KB; ++q) {
        const int k = kb + q;
        const int64_t n = ((int64_t)blockIdx.x + (int64_t)k * gridDim.x) * C + tid;
        if (k >= K || n >= N) continue;
        const size_t o = (size_t)k * C + tid;
        T c, v;
        if (init) {
          c = pay(xi[q]);
          v = T(0);
        } else {
          c = cs_[o];
          v = vs_[o];
        }
        if (upd >= 1) {
          // continuation = relu(design . beta), exercise where payoff > continuation (lsm.py:380-400)
          T xu[DM], xc[DM], phi[GN];
#pragma unroll
          for (int cc = 0; cc < DM; ++cc) {
            xu[cc] = xs_[((size_t)k * DM + cc) * C + tid];
            xc[cc] = xu[cc] - mu_s[0][cc];
          }
          const T evu = pay(xu);
          basis(xc, phi);
          T cont = T(0);
#pragma unroll
          for (int g = 0; g < GN; ++g) cont += phi[g] * beta_s[g];
          cont = cont > T(0) ? cont : T(0);
          const bool ex_now = evu > cont;
          const T vn = ex_now ? T(0) : c + v;
          c = ex_now ? evu : T(0);
          v = ctx.ratio_at(upd, n, r_upd) * vn;
        }
        if (fin) {
          if (n >= price_from) final_acc = A::add(final_acc, ctx.ratio_at(0, n, r_fin) * (c + v));
          continue;
        }
        cs_[o] = c;
        vs_[o] = v;
#pragma unroll
        for (int cc = 0; cc < DM; ++cc) xs_[((size_t)k * DM + cc) * C + tid] = xa[q][cc];
        if (n < n_cal) {
          // masked right-hand side of exercise index acc (lsm.py:373-379)
          const T eva = pay(xa[q]);
          if (eva > T(0)) {
            const T cv = ctx.ratio_at(acc, n, r_acc) * (v + c);
            T xc[DM], phi[GN];
#pragma unroll
            for (int cc = 0; cc < DM; ++cc) xc[cc] = xa[q][cc] - mu_s[1][cc];
            basis(xc, phi);
#pragma unroll
            for (int jj = 0; jj < GN; ++jj) part[jj] += phi[jj] * cv;
          }
          if (++cnt == kSubSum) {
#pragma unroll
            for (int qq = 0; qq < GN; ++qq) {
              acc2[qq] = A::add(acc2[qq], part[qq]);
              part[qq] = T(0);
            }
            cnt = 0;
          }
        }
      }
    }
    const int width = fin ? 1 : GN;
    if (!fin) {
      block_store(acc2, part, GN, pout);
    } else {
      for (int o = 16; o > 0; o >>= 1) final_acc = A::sum(final_acc, A::shfl_down(final_acc, o));
      if (lane == 0) red[warp][0] = final_acc;
      __syncthreads();
      if (tid == 0) {
        S t = A::zero();
        for (int w = 0; w < C / 32; ++w) t = A::sum(t, red[w][0]);
        __stcg(pout + blockIdx.x, *reinterpret_cast<double*>(&t));
      }
    }
    if (!loop_barrier(sy, ++gen, a.dev_status)) return;
    if (fin) {
      if (blockIdx.x == 0) {
        grid_reduce(pout, width);
        if (tid == 0) {
          const int64_t count = a.num_calibration > 0 ? N - a.num_calibration : N;
          a.out[0] = sums_s[0] * (1.0 / (double)count);
        }
      }
      return;
    }
    grid_reduce(pout, width);
    if (tid < GN) {
      // beta = P X'y (FP64), P this date's pseudo-inverse from phase 1
      const double* P = pinv + (size_t)acc * GN * GN + (size_t)tid * GN;
      double b = 0.0;
#pragma unroll
      for (int k = 0; k < GN; ++k) b = fma(__ldcg(P + k), sums_s[k], b);
      beta_s[tid] = (T)b;
    }
  }
}

// The one-launch loop applies to structured calls with one payoff, one path
// set, d <= 2 and 2..5 basis functions.
__host__ inline bool lsm_loop_eligible(const tqf_lsm_args& a) {
  return a.degree >= 0 && a.batch == 1 && a.paths_batch == 1 && a.dim >= 1 && a.dim <= 2 && a.num_basis >= 2 &&
         a.num_basis <= kLoopMaxG && a.num_exercise >= 1;
}

template <typename T>
__host__ void* loop_kernel_for(int d, int G) {
  if (d == 1) {
    switch (G) {
      case 2: return reinterpret_cast<void*>(&lsm_loop_kernel<T, 1, 2>);
      case 3: return reinterpret_cast<void*>(&lsm_loop_kernel<T, 1, 3>);
      case 4: return reinterpret_cast<void*>(&lsm_loop_kernel<T, 1, 4>);
      default: return reinterpret_cast<void*>(&lsm_loop_kernel<T, 1, 5>);
    }
  }
  switch (G) {
    case 2: return reinterpret_cast<void*>(&lsm_loop_kernel<T, 2, 2>);
    case 3: return reinterpret_cast<void*>(&lsm_loop_kernel<T, 2, 3>);
    case 4: return reinterpret_cast<void*>(&lsm_loop_kernel<T, 2, 4>);
    default: return reinterpret_cast<void*>(&lsm_loop_kernel<T, 2, 5>);
  }
}

// Grid and paths per thread (K) of the loop kernel: the largest resident
// grid (2 or 1 CTAs per SM) whose per-thread path state fits
// kLoopStateSmem of shared memory; 0 when none does (the per-date kernels
// run instead).
constexpr size_t kLoopStateSmem = 64 * 1024;

__host__ int lsm_loop_config(const tqf_lsm_args& a, int* K_out, size_t* smem_out) {
  if (!lsm_loop_eligible(a)) return 0;
  const bool f32 = a.dtype == TQF_F32;
  const void* k = f32 ? loop_kernel_for<float>(a.dim, a.num_basis) : loop_kernel_for<double>(a.dim, a.num_basis);
  const int64_t chunks = (a.num_paths + kLoopThreads - 1) / kLoopThreads;
  const size_t per_k = f32 ? (a.dim == 1 ? lsm_loop_smem<float, 1>(1) : lsm_loop_smem<float, 2>(1))
                           : (a.dim == 1 ? lsm_loop_smem<double, 1>(1) : lsm_loop_smem<double, 2>(1));
  for (int occ_try = 2; occ_try >= 1; --occ_try) {
    int64_t g = (int64_t)num_sms() * occ_try;
    if (g > chunks) g = chunks;
    if (g < 1) g = 1;
    const int64_t K = (chunks + g - 1) / g;
    const size_t smem = (size_t)K * per_k;
    if (smem > kLoopStateSmem) continue;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLoopStateSmem) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kLoopThreads, smem) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    if ((int64_t)occ * num_sms() < g) continue;  // cooperative launch needs every CTA resident
    if (K_out) *K_out = (int)K;
    if (smem_out) *smem_out = smem;
    return (int)g;
  }
  return 0;
}

__host__ int lsm_loop_grid(const tqf_lsm_args& a) { return lsm_loop_config(a, nullptr, nullptr); }

// Cooperative launch of the whole date loop (all CTAs resident).
int launch_loop(const tqf_lsm_args& a, cudaStream_t s) {
  const WsLayout L = lsm_layout(a);
  unsigned char* ws = static_cast<unsigned char*>(a.workspace);
  int K = 0;
  size_t smem = 0;
  const int grid = lsm_loop_config(a, &K, &smem);
  TQF_REQUIRE(grid >= 1, "tqf_lsm_price: the one-launch loop does not apply");
  LoopSync* sy = reinterpret_cast<LoopSync*>(ws + L.sync);
  int rc = check_cuda(cudaMemsetAsync(sy, 0, sizeof(LoopSync), s), "tqf_lsm_price: cudaMemsetAsync");
  if (rc) return rc;
  const bool f32 = a.dtype == TQF_F32;
  void* k = f32 ? loop_kernel_for<float>(a.dim, a.num_basis) : loop_kernel_for<double>(a.dim, a.num_basis);
  tqf_lsm_args args = a;
  const void* xt = ws + L.xt;
  void* partials = ws + L.partials;
  double* beta = reinterpret_cast<double*>(ws + L.beta);
  const double* means = reinterpret_cast<const double*>(ws + L.means);
  double* gram = reinterpret_cast<double*>(ws + L.gram);
  double* pinv = reinterpret_cast<double*>(ws + L.pinv);
  void* params[] = {&args, const_cast<void**>(&xt), &partials, &beta, const_cast<double**>(&means), &sy, &K,
                    &gram, &pinv};
  rc = check_cuda(cudaLaunchCooperativeKernel(k, dim3((unsigned)grid), dim3(kLoopThreads), params, smem, s),
                  "lsm_loop_kernel cooperative launch");
  if (rc) return rc;
  note_launch();
  return TQF_OK;
}

constexpr int kMaxWarmBasis = 64;  // warm start needs a second [G][G+1] buffer

size_t solve_smem(int G) {
  const size_t base =
      (size_t)G * (G + 1) * 8 + 2 * (size_t)G * 8 + kMaxBasis * 8 + kMaxBasis * 4 + kSolveThreads / 32 * 16;
  return base + (G <= 16 ? (size_t)G * G * 8 : 0) + (G <= kMaxWarmBasis ? (size_t)G * (G + 1) * 8 : 0);
}

int check_args(const tqf_lsm_args* a, const char* who) {
  TQF_REQUIRE(a != nullptr, "%s: null args", who);
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "%s: bad dtype %d", who, a->dtype);
  TQF_REQUIRE(a->num_paths >= 1 && a->batch >= 1 && a->num_exercise >= 1, "%s: bad sizes", who);
  TQF_REQUIRE(a->num_basis >= 1 && a->num_basis <= kMaxBasis, "%s: num_basis must be in [1, %d], got %d", who,
              kMaxBasis, a->num_basis);
  TQF_REQUIRE(a->paths_batch == 1 || a->paths_batch == a->batch, "%s: paths_batch must be 1 or batch", who);
  TQF_REQUIRE(a->num_calibration >= 0 && a->num_calibration <= a->num_paths, "%s: bad num_calibration", who);
  TQF_REQUIRE(a->exercise_times && a->discount && a->state, "%s: null pointer", who);
  if (a->degree >= 0) {
    TQF_REQUIRE(a->dim >= 1 && a->dim <= kMaxDimLsm, "%s: dim must be in [1, 16], got %d", who, a->dim);
    TQF_REQUIRE(a->paths && a->strikes && a->exponents, "%s: structured mode needs paths, strikes, exponents",
                who);
    TQF_REQUIRE(a->degree <= 127, "%s: degree too large", who);
    TQF_REQUIRE(lsm_gather_chunk(*a) >= 1, "%s: num_exercise * dim too large for one gather tile", who);
    TQF_REQUIRE(a->paths_batch <= 65535, "%s: paths batch too large", who);
  }
  TQF_REQUIRE(a->batch <= 65535, "%s: batch too large", who);
  TQF_REQUIRE(a->workspace && a->workspace_bytes >= lsm_layout(*a).total, "%s: workspace too small", who);
  return TQF_OK;
}

template <typename T>
int launch_pass(const tqf_lsm_args& a, cudaStream_t s) {
  const WsLayout L = lsm_layout(a);
  unsigned char* ws = static_cast<unsigned char*>(a.workspace);
  const int G = a.num_basis;
  int C = 256;
  size_t smem = 0;
  const int gx = lsm_pass_grid<T>(a, &C, &smem);
  dim3 grid((unsigned)gx, (unsigned)a.batch);
  using S = typename Acc<T>::S;
  S* partials = reinterpret_cast<S*>(ws + L.partials);
  const T* xt = reinterpret_cast<const T*>(ws + L.xt);
  const double* beta = reinterpret_cast<const double*>(ws + L.beta);
  const double* means = reinterpret_cast<const double*>(ws + L.means);
  const int d = a.degree >= 0 ? a.dim : 1;
  void* k = pass_kernel_for<T>(d, G);
  void* params[] = {const_cast<tqf_lsm_args*>(&a), const_cast<T**>(&xt), &partials, const_cast<double**>(&beta),
                    const_cast<double**>(&means), &C};
  // The date loop's kernels are programmatic dependent launches: each starts
  // launching while its predecessor finishes and waits (griddepcontrol.wait,
  // at its top) before it reads anything.
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = pdl_config(grid, dim3((unsigned)C), smem, s, attr);
  int rc = check_cuda(cudaLaunchKernelExC(&cfg, k, params), "lsm_pass_kernel launch");
  if (rc) return rc;
  rc = check_launch("lsm_pass_kernel");
  if (rc) return rc;
  const int width = a.final_pass ? a.batch : a.batch * lsm_entries(G);
  if (a.final_pass || a.acc_index >= 1) {
    double* out = a.final_pass ? a.out : reinterpret_cast<double*>(ws + L.sums);
    cudaLaunchConfig_t rcfg = pdl_config(dim3((unsigned)((width + 31) / 32)), dim3(1024), 0, s, attr);
    rc = check_cuda(cudaLaunchKernelEx(&rcfg, lsm_reduce_kernel<T>, static_cast<const S*>(partials), gx, width, out),
                    "lsm_reduce_kernel launch");
    if (rc) return rc;
    return check_launch("lsm_reduce_kernel");
  }
  return TQF_OK;
}

template <typename T>
int launch_gather(const tqf_lsm_args& a, cudaStream_t s) {
  const WsLayout L = lsm_layout(a);
  unsigned char* ws = static_cast<unsigned char*>(a.workspace);
  int full = 0;
  const int Cn = lsm_gather_chunk(a, &full);
  const int gx = lsm_gather_grid(a);
  const size_t smem = lsm_gather_smem(a, Cn, full);
  set_smem_config(lsm_gather_kernel<T>, smem);
  using S = typename Acc<T>::S;
  S* part = reinterpret_cast<S*>(ws + L.mean_partials);
  double* means = reinterpret_cast<double*>(ws + L.means);
  lsm_gather_kernel<T><<<dim3((unsigned)gx, (unsigned)a.paths_batch), kGatherThreads, smem, s>>>(
      a, reinterpret_cast<T*>(ws + L.xt), part, Cn, full);
  int rc = check_launch("lsm_gather_kernel");
  if (rc) return rc;
  const int width = a.paths_batch * a.num_exercise * kMaxDimLsm;
  lsm_reduce_kernel<T><<<(width + 31) / 32, 1024, 0, s>>>(part, gx, width, means);
  rc = check_launch("lsm_reduce_kernel");
  if (rc) return rc;
  lsm_scale_kernel<<<(width + 255) / 256, 256, 0, s>>>(means, width, 1.0 / (double)a.num_paths);
  return check_launch("lsm_scale_kernel");
}

int launch_solve(const tqf_lsm_args& a, cudaStream_t s) {
  const WsLayout L = lsm_layout(a);
  unsigned char* ws = static_cast<unsigned char*>(a.workspace);
  const int G = a.num_basis;
  const double eps = a.dtype == TQF_F32 ? 1.1920928955078125e-07 : 2.220446049250313e-16;
  const double rcond = 10.0 * G * eps;
  const size_t smem = solve_smem(G);
  // warm start from the previous date's eigenvectors (every solve after the first)
  const int warm = (G <= kMaxWarmBasis && a.acc_index >= 1 && a.acc_index < a.num_exercise - 1) ? 1 : 0;
  void (*k)(const double*, int, double, double*, double*, int) = lsm_solve_kernel<0>;
  switch (G) {
    case 2: k = lsm_solve_kernel<2>; break;
    case 3: k = lsm_solve_kernel<3>; break;
    case 4: k = lsm_solve_kernel<4>; break;
    case 5: k = lsm_solve_kernel<5>; break;
    case 6: k = lsm_solve_kernel<6>; break;
    case 8: k = lsm_solve_kernel<8>; break;
    case 9: k = lsm_solve_kernel<9>; break;
    default: break;
  }
  set_smem_config(k, smem);
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = pdl_config(dim3((unsigned)a.batch), dim3(G <= 16 ? 32 : kSolveThreads), smem, s, attr);
  const int rc = check_cuda(cudaLaunchKernelEx(&cfg, k, reinterpret_cast<const double*>(ws + L.sums), G, rcond,
                                               reinterpret_cast<double*>(ws + L.beta),
                                               reinterpret_cast<double*>(ws + L.eig_v), warm),
                            "lsm_solve_kernel launch");
  if (rc) return rc;
  return check_launch("lsm_solve_kernel");
}

int check_pass(const tqf_lsm_args* a) {
  TQF_REQUIRE(a->upd_index < a->num_exercise && a->acc_index < a->num_exercise,
              "tqf_lsm_pass: exercise index out of range");
  TQF_REQUIRE(!a->final_pass || a->out, "tqf_lsm_pass: final pass needs out");
  TQF_REQUIRE(!(a->final_pass && a->acc_index >= 1), "tqf_lsm_pass: final pass cannot accumulate");
  if (a->degree < 0) {
    TQF_REQUIRE(!a->init || a->init_payoff, "tqf_lsm_pass: explicit mode needs init_payoff");
    TQF_REQUIRE(a->upd_index < 1 || (a->upd_payoff && a->upd_design), "tqf_lsm_pass: explicit update needs data");
    TQF_REQUIRE(a->acc_index < 1 || (a->acc_payoff && a->acc_design), "tqf_lsm_pass: explicit accumulate needs data");
  }
  return TQF_OK;
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" size_t tqf_lsm_workspace_bytes(const tqf_lsm_args* a) {
  if (!a || a->num_basis < 1 || a->num_basis > kMaxBasis) return 0;
  return lsm_layout(*a).total;
}

extern "C" int tqf_lsm_gather(const tqf_lsm_args* a, void* stream) {
  clear_error();
  int rc = check_args(a, "tqf_lsm_gather");
  if (rc) return rc;
  TQF_REQUIRE(a->degree >= 0, "tqf_lsm_gather: structured basis only");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? launch_gather<float>(*a, s) : launch_gather<double>(*a, s);
}

extern "C" int tqf_lsm_pass(const tqf_lsm_args* a, void* stream) {
  clear_error();
  int rc = check_args(a, "tqf_lsm_pass");
  if (rc) return rc;
  rc = check_pass(a);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? launch_pass<float>(*a, s) : launch_pass<double>(*a, s);
}

extern "C" int tqf_lsm_solve(const tqf_lsm_args* a, void* stream) {
  clear_error();
  int rc = check_args(a, "tqf_lsm_solve");
  if (rc) return rc;
  return launch_solve(*a, static_cast<cudaStream_t>(stream));
}

extern "C" int tqf_lsm_price(const tqf_lsm_args* args, void* stream) {
  clear_error();
  int rc = check_args(args, "tqf_lsm_price");
  if (rc) return rc;
  TQF_REQUIRE(args->degree >= 0, "tqf_lsm_price: structured basis and payoff only (explicit mode runs per pass)");
  TQF_REQUIRE(args->out, "tqf_lsm_price: null out");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tqf_lsm_args a = *args;
  const bool f32 = a.dtype == TQF_F32;
  {
    const int64_t count = a.num_calibration > 0 ? a.num_paths - a.num_calibration : a.num_paths;
    TQF_REQUIRE(count >= 1, "tqf_lsm_price: no paths left to price after calibration");
  }
  rc = f32 ? launch_gather<float>(a, s) : launch_gather<double>(a, s);
  if (rc) return rc;
  if (lsm_loop_grid(a) >= 1) return launch_loop(a, s);
  auto pass = [&](int init, int upd, int acc, int fin) {
    a.init = init;
    a.upd_index = upd;
    a.acc_index = acc;
    a.final_pass = fin;
    return f32 ? launch_pass<float>(a, s) : launch_pass<double>(a, s);
  };
  const int E = a.num_exercise;
  if (E == 1) {
    rc = pass(1, 0, 0, 1);
  } else {
    rc = pass(1, 0, E - 1, 0);
    if (!rc) rc = launch_solve(a, s);
    for (int i = E - 1; i > 1 && !rc; --i) {
      rc = pass(0, i, i - 1, 0);
      if (!rc) rc = launch_solve(a, s);
    }
    if (!rc) rc = pass(0, 1, 0, 1);
  }
  if (rc) return rc;
  const int64_t count = a.num_calibration > 0 ? a.num_paths - a.num_calibration : a.num_paths;
  TQF_REQUIRE(count >= 1, "tqf_lsm_price: no paths left to price after calibration");
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = pdl_config(dim3((unsigned)((a.batch + 255) / 256)), dim3(256), 0, s, attr);
  rc = check_cuda(cudaLaunchKernelEx(&cfg, lsm_scale_kernel, a.out, a.batch, 1.0 / (double)count),
                  "lsm_scale_kernel launch");
  if (rc) return rc;
  return check_launch("lsm_scale_kernel");
}
