// Longstaff–Schwartz regression Monte Carlo — the GB300 replacement of
// tff/models/longstaff_schwartz/lsm.py:128-436 and payoff_utils.py:27-98.
//
// The reference loops backwards over exercise dates; each iteration builds a
// [batch, N, G] design, masks it by "in the money", forms X'X and X'y with two
// matmuls, takes tf.linalg.pinv (SVD) and re-projects every path.  Here each
// iteration is:
//   lsm_pass_kernel   one pass over the paths: applies the previous date's
//                     regression (continuation value, exercise decision,
//                     cashflow/value update, discounting) and accumulates this
//                     date's masked normal equations in FP64 — the design is
//                     built per path in registers/shared memory, never stored;
//   reduce_partials   fixed-order sum of the per-CTA partials;
//   lsm_solve_kernel  one CTA per batch member: cyclic Jacobi eigen-
//                     decomposition of X'X in FP64 (parallel round-robin
//                     rotations), pinv with tf.linalg.pinv's cutoff, beta.
// Per-path arithmetic runs in the dtype of the paths, as in the reference.
#include <math.h>

#include "tqf_internal.cuh"

namespace tqf {
namespace {

constexpr int kMaxBasis = 128;
constexpr int kMaxDimLsm = 16;
constexpr int kSolveThreads = 256;
constexpr int kMaxJacobiSweeps = 40;

__host__ __device__ inline int lsm_entries(int G) { return G * (G + 1) / 2 + G; }

// Chunk of paths per CTA iteration (= threads per CTA), chosen so that the
// design tile [C][G+1], the accumulators and the beta row fit in 200 KB.
__host__ inline int lsm_chunk(int G) {
  const int En = lsm_entries(G);
  for (int C = 256; C >= 64; C >>= 1) {
    const int W = (G + 1) | 1;
    const size_t bytes = (size_t)C * W * 8 + (size_t)(En > C ? En : C) * 8 + (size_t)G * 8 + 64 * 8 +
                         (size_t)G * kMaxDimLsm;
    if (bytes <= 200 * 1024) return C;
  }
  return 64;
}

__host__ inline size_t lsm_pass_smem(int G, int C) {
  const int En = lsm_entries(G);
  const int W = (G + 1) | 1;
  return (size_t)C * W * 8 + (size_t)(En > C ? En : C) * 8 + (size_t)G * 8 + 64 * 8 + (size_t)G * kMaxDimLsm;
}

__host__ inline int lsm_grid_x(const tqf_lsm_args& a, int C) {
  const int64_t chunks = (a.num_paths + C - 1) / C;
  int64_t g = (int64_t)num_sms() * (C >= 256 ? 2 : 1);
  if (g > chunks) g = chunks;
  return (int)(g < 1 ? 1 : g);
}

struct WsLayout {
  size_t partials, sums, beta, means, mean_partials, eig_v, total;
};

__host__ inline WsLayout lsm_layout(const tqf_lsm_args& a) {
  const int G = a.num_basis, B = a.batch, E = a.num_exercise;
  const int En = lsm_entries(G);
  const int gx = num_sms() * 2;
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  WsLayout w{};
  size_t off = 0;
  w.partials = off;
  off += up((size_t)gx * B * (En > 1 ? En : 1) * 8);
  w.sums = off;
  off += up((size_t)B * En * 8);
  w.beta = off;
  off += up((size_t)B * G * 8);
  w.means = off;
  off += up((size_t)E * a.paths_batch * kMaxDimLsm * 8);
  w.mean_partials = off;
  off += up((size_t)gx * E * a.paths_batch * kMaxDimLsm * 8);
  w.eig_v = off;
  off += up((size_t)B * G * G * 8);
  w.total = off;
  return w;
}

template <typename T>
__device__ __forceinline__ T ipow(T x, int e) {
  T r = T(1);
  for (int i = 0; i < e; ++i) r *= x;
  return r;
}

// Packed upper triangle, row-major: entry e <-> (j, k), j <= k < G.
__device__ __forceinline__ void sym_pair(int e, int G, int& j, int& k) {
  const double g2 = 2.0 * G + 1.0;
  int jj = (int)((g2 - sqrt(g2 * g2 - 8.0 * e)) * 0.5);
  if (jj < 0) jj = 0;
  while (jj > 0 && jj * G - jj * (jj - 1) / 2 > e) --jj;
  while (jj + 1 < G && (jj + 1) * G - (jj + 1) * jj / 2 <= e) ++jj;
  j = jj;
  k = jj + (e - (jj * G - jj * (jj - 1) / 2));
}

template <typename T>
struct LsmCtx {
  const tqf_lsm_args& a;
  int b, pb, G, d;
  const int8_t* exps;  // [G][16] in shared memory (structured)
  __device__ T ratio(int i, int64_t n) const {
    const T* D = static_cast<const T*>(a.discount);
    const int64_t o = n * a.disc_stride_n + (int64_t)b * a.disc_stride_b;
    return D[(int64_t)(i + 1) * a.disc_stride_e + o] / D[(int64_t)i * a.disc_stride_e + o];
  }
  // Exercise value at path time t (basket put) or from the caller's [N][B] array.
  __device__ T payoff(const void* expl, int t, int64_t n, T* x) const {
    if (a.degree < 0) return static_cast<const T*>(expl)[n * a.batch + b];
    const T* S = static_cast<const T*>(a.paths) + (((int64_t)pb * a.num_paths + n) * a.num_times + t) * d;
    T s = T(0);
    for (int c = 0; c < d; ++c) {
      x[c] = S[c];
      s += x[c];
    }
    const T K = static_cast<const T*>(a.strikes)[b];
    const T v = K - s / (T)d;
    return v > T(0) ? v : T(0);
  }
  // Basis function g at the path (structured: centred powers of x).
  __device__ T basis(const void* expl, int g, int64_t n, const T* xc) const {
    if (a.degree < 0) return static_cast<const T*>(expl)[((int64_t)pb * G + g) * a.num_paths + n];
    T p = T(1);
    for (int c = 0; c < d; ++c) p *= ipow(xc[c], (int)exps[g * kMaxDimLsm + c]);
    return p;
  }
};

template <typename T>
__global__ void lsm_pass_kernel(tqf_lsm_args a, double* __restrict__ partials, const double* __restrict__ beta,
                                const double* __restrict__ means, int C, double* __restrict__ final_partials) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int G = a.num_basis, d = a.dim, B = a.batch;
  const int En = lsm_entries(G);
  const int W = (G + 1) | 1;
  double* phi_s = reinterpret_cast<double*>(smem);                 // [C][W]
  double* acc_s = phi_s + (size_t)C * W;                            // [max(En, C)]
  double* beta_s = acc_s + (En > C ? En : C);                       // [G]
  double* red_s = beta_s + G;                                       // [64]
  int8_t* exps_s = reinterpret_cast<int8_t*>(red_s + 64);           // [G][16]
  const int tid = threadIdx.x;
  const int b = blockIdx.y;
  const int pb = a.paths_batch > 1 ? b : 0;
  const int R = En >= C ? 1 : C / En;  // replicas of each accumulator entry
  const int items = En * R;
  for (int i = tid; i < items; i += C) acc_s[i] = 0.0;
  if (a.upd_index >= 1)
    for (int g = tid; g < G; g += C) beta_s[g] = beta[(size_t)b * G + g];
  if (a.degree >= 0)
    for (int i = tid; i < G * kMaxDimLsm; i += C) {
      const int g = i / kMaxDimLsm, c = i % kMaxDimLsm;
      exps_s[i] = c < d ? (int8_t)a.exponents[g * d + c] : (int8_t)0;
    }
  __syncthreads();
  LsmCtx<T> ctx{a, b, pb, G, d, exps_s};
  const int E = a.num_exercise;
  const int* ex = a.exercise_times;
  T* state = static_cast<T*>(a.state);
  T* cash = state + (size_t)b * a.num_paths;
  T* vals = state + ((size_t)B + b) * a.num_paths;
  const int64_t n_cal = a.num_calibration > 0 ? a.num_calibration : a.num_paths;
  const int64_t price_from = a.num_calibration > 0 ? a.num_calibration : 0;
  double final_acc = 0.0;
  const int64_t nchunks = (a.num_paths + C - 1) / C;
  for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int64_t n = ch * C + tid;
    const bool valid = n < a.num_paths;
    T x[kMaxDimLsm], xc[kMaxDimLsm];
    T c = T(0), v = T(0);
    if (valid) {
      if (a.init) {
        c = ctx.payoff(a.init_payoff, ex[E - 1], n, x);
        v = T(0);
      } else {
        c = cash[n];
        v = vals[n];
      }
      if (a.upd_index >= 1) {
        // continuation = relu(design . beta), exercise where payoff > continuation (lsm.py:380-400)
        const int iu = a.upd_index;
        const int t = ex[iu - 1];
        const T evu = ctx.payoff(a.upd_payoff, t, n, x);
        if (a.degree >= 0) {
          const double* mu = means + ((size_t)pb * E + (iu - 1)) * kMaxDimLsm;
          for (int q = 0; q < d; ++q) xc[q] = x[q] - (T)mu[q];
        }
        T cont = T(0);
        for (int g = 0; g < G; ++g) cont += ctx.basis(a.upd_design, g, n, xc) * (T)beta_s[g];
        cont = cont > T(0) ? cont : T(0);
        const bool ex_now = evu > cont;
        const T vn = ex_now ? T(0) : c + v;
        c = ex_now ? evu : T(0);
        v = ctx.ratio(iu, n) * vn;
      }
      if (a.final_pass) {
        if (n >= price_from) final_acc += (double)(ctx.ratio(0, n) * (c + v));
      } else {
        cash[n] = c;
        vals[n] = v;
      }
    }
    if (a.acc_index >= 1) {
      // masked normal equations of exercise index ia (lsm.py:355-379)
      const int ia = a.acc_index;
      double* row = phi_s + (size_t)tid * W;
      if (valid) {
        const int t = ex[ia - 1];
        const T cv = ctx.ratio(ia, n) * (v + c);
        const T eva = ctx.payoff(a.acc_payoff, t, n, x);
        const bool use = eva > T(0) && n < n_cal;
        if (a.degree >= 0) {
          const double* mu = means + ((size_t)pb * E + (ia - 1)) * kMaxDimLsm;
          for (int q = 0; q < d; ++q) xc[q] = x[q] - (T)mu[q];
        }
        for (int g = 0; g < G; ++g) row[g] = use ? (double)ctx.basis(a.acc_design, g, n, xc) : 0.0;
        row[G] = n < n_cal ? (double)cv : 0.0;
      } else {
        for (int g = 0; g <= G; ++g) row[g] = 0.0;
      }
      __syncthreads();
      for (int it = tid; it < items; it += C) {
        const int e = it % En, r = it / En;
        int j, k;
        if (e < G * (G + 1) / 2) {
          sym_pair(e, G, j, k);
        } else {
          j = e - G * (G + 1) / 2;
          k = G;
        }
        double s = 0.0;
        for (int p = r; p < C; p += R) s += phi_s[(size_t)p * W + j] * phi_s[(size_t)p * W + k];
        acc_s[it] += s;
      }
      __syncthreads();
    }
  }
  if (a.acc_index >= 1) {
    double* out = partials + ((size_t)blockIdx.x * B + b) * En;
    for (int e = tid; e < En; e += C) {
      double s = 0.0;
      for (int r = 0; r < R; ++r) s += acc_s[r * En + e];
      out[e] = s;
    }
  }
  if (a.final_pass) {
    // fixed-order block sum
    for (int o = 16; o > 0; o >>= 1) final_acc += __shfl_down_sync(0xffffffffu, final_acc, o);
    if ((tid & 31) == 0) red_s[tid >> 5] = final_acc;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < C / 32; ++w) s += red_s[w];
      final_partials[(size_t)blockIdx.x * B + b] = s;
    }
  }
}

// Column sums of the paths at every exercise time: partial [gx][Bp][E][16].
template <typename T>
__global__ void __launch_bounds__(256) lsm_means_kernel(tqf_lsm_args a, double* __restrict__ partials) {
  const int e = blockIdx.y % a.num_exercise;
  const int pb = blockIdx.y / a.num_exercise;
  const int d = a.dim;
  const int t = a.exercise_times[e];
  __shared__ double red[8][kMaxDimLsm];
  double s[kMaxDimLsm];
#pragma unroll
  for (int c = 0; c < kMaxDimLsm; ++c) s[c] = 0.0;
  const T* P = static_cast<const T*>(a.paths);
  for (int64_t n = (int64_t)blockIdx.x * 256 + threadIdx.x; n < a.num_paths; n += (int64_t)gridDim.x * 256) {
    const T* S = P + (((int64_t)pb * a.num_paths + n) * a.num_times + t) * d;
#pragma unroll
    for (int c = 0; c < kMaxDimLsm; ++c)
      if (c < d) s[c] += (double)S[c];
  }
#pragma unroll
  for (int c = 0; c < kMaxDimLsm; ++c) {
    double v = s[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < kMaxDimLsm) {
    double v = 0.0;
    for (int w = 0; w < 8; ++w) v += red[w][threadIdx.x];
    partials[((size_t)blockIdx.x * gridDim.y + blockIdx.y) * kMaxDimLsm + threadIdx.x] = v;
  }
}

__global__ void lsm_scale_kernel(double* __restrict__ v, int n, double s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] *= s;
}

// One CTA per batch member: A = X'X (packed) -> Jacobi eigen-decomposition
// A = V diag(l) V^T; beta = V diag(l+) V^T (X'y), l+ = 1/l where |l| > cutoff.
__global__ void __launch_bounds__(kSolveThreads)
    lsm_solve_kernel(const double* __restrict__ sums, int G, double rcond, double* __restrict__ beta,
                     double* __restrict__ Vg) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int P = G + 1;  // row stride of A
  double* A = reinterpret_cast<double*>(smem);  // [G][G+1]
  double* rhs = A + (size_t)G * P;               // [G]
  double* w = rhs + G;                           // [G]
  double* cs = w + G;                            // [2][kMaxBasis/2]
  int* pq = reinterpret_cast<int*>(cs + kMaxBasis);  // [2][kMaxBasis/2]
  double* red = reinterpret_cast<double*>(pq + kMaxBasis);  // [kSolveThreads/32][2]
  const int b = blockIdx.x, tid = threadIdx.x;
  const int En = lsm_entries(G);
  const double* s = sums + (size_t)b * En;
  double* V = Vg + (size_t)b * G * G;
  const int tri = G * (G + 1) / 2;
  for (int e = tid; e < tri; e += kSolveThreads) {
    int j, k;
    sym_pair(e, G, j, k);
    A[j * P + k] = s[e];
    A[k * P + j] = s[e];
  }
  for (int j = tid; j < G; j += kSolveThreads) rhs[j] = s[tri + j];
  for (int i = tid; i < G * G; i += kSolveThreads) V[i] = (i / G == i % G) ? 1.0 : 0.0;
  __syncthreads();
  const int Pe = G + (G & 1);
  const int half = Pe / 2;
  for (int sweep = 0; sweep < kMaxJacobiSweeps && G > 1; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = tid; i < G * G; i += kSolveThreads) {
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
    for (int q = 0; q < kSolveThreads / 32; ++q) {
      OFF += red[q * 2];
      TOT += red[q * 2 + 1];
    }
    __syncthreads();
    if (OFF <= 1e-30 * TOT || OFF == 0.0) break;
    for (int r = 0; r < Pe - 1; ++r) {
      if (tid < half) {
        const int k = tid;
        int i1 = (r + k) % (Pe - 1);
        int i2 = k == 0 ? Pe - 1 : (Pe - 1 - k + r) % (Pe - 1);
        const int p = i1 < i2 ? i1 : i2, q = i1 < i2 ? i2 : i1;
        double c = 1.0, sn = 0.0;
        if (q < G) {
          const double apq = A[p * P + q];
          if (apq != 0.0) {
            const double theta = (A[q * P + q] - A[p * P + p]) / (2.0 * apq);
            double t;
            if (fabs(theta) > 1e150)
              t = 0.5 / theta;
            else
              t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(1.0 + theta * theta));
            c = 1.0 / sqrt(1.0 + t * t);
            sn = t * c;
          }
        }
        cs[2 * k] = c;
        cs[2 * k + 1] = sn;
        pq[2 * k] = p;
        pq[2 * k + 1] = q < G ? q : -1;
      }
      __syncthreads();
      // A <- A J (columns p, q)
      for (int it = tid; it < G * half; it += kSolveThreads) {
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
      for (int it = tid; it < G * half; it += kSolveThreads) {
        const int k = it / G, j = it % G;
        const int p = pq[2 * k], q = pq[2 * k + 1];
        if (q < 0) continue;
        const double c = cs[2 * k], sn = cs[2 * k + 1];
        const double apj = A[p * P + j], aqj = A[q * P + j];
        A[p * P + j] = c * apj - sn * aqj;
        A[q * P + j] = sn * apj + c * aqj;
      }
      // V <- V J
      for (int it = tid; it < G * half; it += kSolveThreads) {
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
  for (int j = tid; j < G; j += kSolveThreads) {
    double u = 0.0;
    for (int i = 0; i < G; ++i) u += V[i * G + j] * rhs[i];
    const double l = A[j * P + j];
    w[j] = fabs(l) > cutoff && l != 0.0 ? u / l : 0.0;
  }
  __syncthreads();
  for (int i = tid; i < G; i += kSolveThreads) {
    double x = 0.0;
    for (int j = 0; j < G; ++j) x += V[i * G + j] * w[j];
    beta[(size_t)b * G + i] = x;
  }
}

size_t solve_smem(int G) {
  return (size_t)G * (G + 1) * 8 + 2 * (size_t)G * 8 + kMaxBasis * 8 + kMaxBasis * 4 + kSolveThreads / 32 * 16;
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
  }
  TQF_REQUIRE(a->workspace && a->workspace_bytes >= lsm_layout(*a).total, "%s: workspace too small", who);
  return TQF_OK;
}

template <typename T>
int launch_pass(const tqf_lsm_args& a, cudaStream_t s) {
  const WsLayout L = lsm_layout(a);
  unsigned char* ws = static_cast<unsigned char*>(a.workspace);
  const int G = a.num_basis;
  const int C = lsm_chunk(G);
  const size_t smem = lsm_pass_smem(G, C);
  set_smem_config(lsm_pass_kernel<T>, smem);
  const int gx = lsm_grid_x(a, C);
  dim3 grid((unsigned)gx, (unsigned)a.batch);
  double* partials = reinterpret_cast<double*>(ws + L.partials);
  lsm_pass_kernel<T><<<grid, C, smem, s>>>(a, partials, reinterpret_cast<const double*>(ws + L.beta),
                                           reinterpret_cast<const double*>(ws + L.means), C, partials);
  int rc = check_launch("lsm_pass_kernel");
  if (rc) return rc;
  if (a.final_pass) return reduce_partials(partials, gx, a.batch, a.out, s);
  if (a.acc_index >= 1)
    return reduce_partials(partials, gx, a.batch * lsm_entries(G), reinterpret_cast<double*>(ws + L.sums), s);
  return TQF_OK;
}

template <typename T>
int launch_means(const tqf_lsm_args& a, cudaStream_t s) {
  const WsLayout L = lsm_layout(a);
  unsigned char* ws = static_cast<unsigned char*>(a.workspace);
  const int rows = a.num_exercise * a.paths_batch;
  int64_t gx = (a.num_paths + 255) / 256;
  if (gx > num_sms() * 2) gx = num_sms() * 2;
  TQF_REQUIRE(rows <= 65535, "tqf_lsm_means: too many exercise times");
  double* part = reinterpret_cast<double*>(ws + L.mean_partials);
  double* means = reinterpret_cast<double*>(ws + L.means);
  lsm_means_kernel<T><<<dim3((unsigned)gx, (unsigned)rows), 256, 0, s>>>(a, part);
  int rc = check_launch("lsm_means_kernel");
  if (rc) return rc;
  rc = reduce_partials(part, (int)gx, rows * kMaxDimLsm, means, s);
  if (rc) return rc;
  const int n = rows * kMaxDimLsm;
  lsm_scale_kernel<<<(n + 255) / 256, 256, 0, s>>>(means, n, 1.0 / (double)a.num_paths);
  return check_launch("lsm_scale_kernel");
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" size_t tqf_lsm_workspace_bytes(const tqf_lsm_args* a) {
  if (!a) return 0;
  return lsm_layout(*a).total;
}

extern "C" int tqf_lsm_means(const tqf_lsm_args* a, void* stream) {
  clear_error();
  int rc = check_args(a, "tqf_lsm_means");
  if (rc) return rc;
  TQF_REQUIRE(a->degree >= 0, "tqf_lsm_means: structured basis only");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? launch_means<float>(*a, s) : launch_means<double>(*a, s);
}

extern "C" int tqf_lsm_pass(const tqf_lsm_args* a, void* stream) {
  clear_error();
  int rc = check_args(a, "tqf_lsm_pass");
  if (rc) return rc;
  TQF_REQUIRE(a->upd_index < a->num_exercise && a->acc_index < a->num_exercise,
              "tqf_lsm_pass: exercise index out of range");
  TQF_REQUIRE(!a->final_pass || a->out, "tqf_lsm_pass: final pass needs out");
  TQF_REQUIRE(!(a->final_pass && a->acc_index >= 1), "tqf_lsm_pass: final pass cannot accumulate");
  if (a->degree < 0) {
    TQF_REQUIRE(!a->init || a->init_payoff, "tqf_lsm_pass: explicit mode needs init_payoff");
    TQF_REQUIRE(a->upd_index < 1 || (a->upd_payoff && a->upd_design), "tqf_lsm_pass: explicit update needs data");
    TQF_REQUIRE(a->acc_index < 1 || (a->acc_payoff && a->acc_design), "tqf_lsm_pass: explicit accumulate needs data");
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? launch_pass<float>(*a, s) : launch_pass<double>(*a, s);
}

extern "C" int tqf_lsm_solve(const tqf_lsm_args* a, void* stream) {
  clear_error();
  int rc = check_args(a, "tqf_lsm_solve");
  if (rc) return rc;
  const WsLayout L = lsm_layout(*a);
  unsigned char* ws = static_cast<unsigned char*>(a->workspace);
  const int G = a->num_basis;
  const double eps = a->dtype == TQF_F32 ? 1.1920928955078125e-07 : 2.220446049250313e-16;
  const double rcond = 10.0 * G * eps;
  const size_t smem = solve_smem(G);
  set_smem_config(lsm_solve_kernel, smem);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  lsm_solve_kernel<<<a->batch, kSolveThreads, smem, s>>>(reinterpret_cast<const double*>(ws + L.sums), G, rcond,
                                                         reinterpret_cast<double*>(ws + L.beta),
                                                         reinterpret_cast<double*>(ws + L.eig_v));
  return check_launch("lsm_solve_kernel");
}
