// Milstein scheme kernels — the GB300 replacement of
// tff/models/milstein_sampling.py:258-671.
//
// milstein_affine_kernel: the whole time loop for structured coefficients
//   a(x) = m + M x, B(x)_kj = (s0_k + s1_k x_k) C_kj, whose volatility gradient
//   is exact (dB_kj/dx_i = delta_ik s1_k C_kj); path state, B and the
//   Stratonovich integrals J live in registers, the step table is staged in
//   shared memory by a bulk copy, draws come from memory or in-kernel Philox.
// milstein_update_kernel: one step for coefficients (drift, B, dB/dx) that the
//   caller evaluated at t_{i+1}.
//
// The update is the reference's, term for term (milstein_sampling.py:565-593):
//   d = 1: x + dt a + b dW + b b' (dW^2 - dt) / 2
//   d > 1: x + dt (a - u) + B dW + h, with
//     u_k = sum_{i,j} dB_kj/dx_i B_ij                 (_stratonovich_drift_update)
//     h_s = sum_{i,m} (sum_j dB_sj/dx_i B_jm) J_im     (_milstein_hot)
//     J_ij = dt (dW_i dW_j / 2 + sqrt(rho_p) (mu_i xi_j - xi_i mu_j))
//          + dt / (2 pi) sum_r (1/r) (zeta_ir (sqrt2 xi_j + eta_jr) - (sqrt2 xi_i + eta_ir) zeta_jr),
//     J_ii = dW_i^2 / 2, xi = dW / sqrt(dt)             (_stratonovich_integral)
#include "tqf_internal.cuh"

// Full unrolling for the small dimension buckets only; the 8-wide bucket keeps
// runtime loops (register arrays there would spill anyway).

namespace tqf {
namespace {

constexpr int kBlock = 128;
constexpr int kMaxDimMil = 8;

template <typename T, int DM>
struct AffineMil {
  T m[DM], M[DM * DM], s0[DM], s1[DM], C[DM * DM];
};

// Off-diagonal Stratonovich integrals J (diagonal set to dW^2 / 2).
template <typename T, int DM>
__device__ __forceinline__ void stratonovich_J(int d, int order, T dt, T sqrt_dt, T sqrt_rho, const T* dw,
                                               DrawSource<T>& src, int step, T (&J)[DM][DM]) {
  T xi[DM], mup[DM];
  const int p = order - 1;
#pragma unroll(DM <= 4 ? DM : 1)
  for (int c = 0; c < DM; ++c) {
    xi[c] = c < d ? dw[c] / sqrt_dt : T(0);
    mup[c] = c < d ? src.get(step, d + c * order + p) : T(0);
  }
  T acc[DM][DM];
#pragma unroll(DM <= 4 ? DM : 1)
  for (int i = 0; i < DM; ++i)
#pragma unroll(DM <= 4 ? DM : 1)
    for (int j = 0; j < DM; ++j) {
      J[i][j] = dt * (dw[i] * dw[j] / T(2) + sqrt_rho * (mup[i] * xi[j] - xi[i] * mup[j]));
      acc[i][j] = T(0);
    }
  const T s2 = (T)1.4142135623730951;
  for (int r = 0; r < order; ++r) {
    T z[DM], w[DM];
#pragma unroll(DM <= 4 ? DM : 1)
    for (int c = 0; c < DM; ++c) {
      z[c] = c < d ? src.get(step, d + d * order + c * order + r) : T(0);
      const T e = c < d ? src.get(step, d + 2 * d * order + c * order + r) : T(0);
      w[c] = s2 * xi[c] + e;
    }
    const T inv = T(1) / T(r + 1);
#pragma unroll(DM <= 4 ? DM : 1)
    for (int i = 0; i < DM; ++i)
#pragma unroll(DM <= 4 ? DM : 1)
      for (int j = 0; j < DM; ++j) acc[i][j] += (z[i] * w[j] - w[i] * z[j]) * inv;
  }
  const T two_pi = (T)6.283185307179586;
#pragma unroll(DM <= 4 ? DM : 1)
  for (int i = 0; i < DM; ++i)
#pragma unroll(DM <= 4 ? DM : 1)
    for (int j = 0; j < DM; ++j) J[i][j] = i == j ? dw[i] * dw[i] / T(2) : J[i][j] + dt * acc[i][j] / two_pi;
}

// Shared memory: mbarrier, coefficients, staged step table, then (STAGE)
// the output staging buffer.
template <typename T, int DM>
__host__ __device__ inline size_t milstein_stage_offset(int steps, bool staged) {
  const size_t head = (16 + sizeof(AffineMil<T, DM>) + 15) & ~(size_t)15;
  return (head + (staged ? (size_t)steps * 4 * sizeof(T) : 0) + 15) & ~(size_t)15;
}

// STAGE: recorded states go through the coalescing RowStager, chosen when a
// path's output row is at least 64 bytes; then every thread runs every round
// and a thread past the last path simulates that path again with its output
// dropped.
template <typename T, int DM, int SRC, bool STAGE>
__global__ void __launch_bounds__(kBlock) milstein_affine_kernel(tqf_milstein_affine_args a, double rho_c,
                                                                 int staged) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  AffineMil<T, DM>* cf = reinterpret_cast<AffineMil<T, DM>*>(smem + 16);
  unsigned char* tab_raw = smem + ((16 + sizeof(AffineMil<T, DM>) + 15) & ~(size_t)15);
  const int d = a.dim, order = a.order;
  for (int i = threadIdx.x; i < DM; i += kBlock) {
    const bool in = i < d;
    cf->m[i] = in ? static_cast<const T*>(a.drift_m)[i] : T(0);
    cf->s0[i] = in ? static_cast<const T*>(a.vol_s0)[i] : T(0);
    cf->s1[i] = in ? static_cast<const T*>(a.vol_s1)[i] : T(0);
  }
  for (int i = threadIdx.x; i < DM * DM; i += kBlock) {
    const int r = i / DM, c = i % DM;
    const bool in = r < d && c < d;
    cf->M[i] = in ? static_cast<const T*>(a.drift_M)[r * d + c] : T(0);
    cf->C[i] = in ? static_cast<const T*>(a.vol_C)[r * d + c] : T(0);
  }
  const T* table = static_cast<const T*>(a.step_table);
  if (staged) {
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    uint32_t phase = 0;
    if (!stage_to_smem(tab_raw, a.step_table, (uint32_t)(a.num_steps * 4 * sizeof(T)), bar, phase, a.dev_status))
      return;
    table = reinterpret_cast<const T*>(tab_raw);
  } else {
    __syncthreads();
  }
  const T sqrt_rho = sqrt((T)rho_c);
  const int K = d + 3 * d * order;  // normals per step
  T* out = static_cast<T*>(a.output.ptr);
  const int ns = a.output.num_slots;
  const int64_t N = a.num_paths;
  RowStager<T, DM, kBlock> stg(smem + milstein_stage_offset<T, DM>(a.num_steps, staged != 0), d);
  const int64_t per_round = (int64_t)gridDim.x * kBlock;
  for (int64_t base = 0; base < N; base += per_round) {
    const int64_t row0 = base + (int64_t)blockIdx.x * kBlock;
    const int64_t path = row0 + threadIdx.x;
    if (!STAGE && path >= N) break;
    const int64_t pc = path < N ? path : N - 1;
    T x[DM];
    const T* x0 = static_cast<const T*>(a.x0) + (a.x0_per_path ? pc * d : 0);
#pragma unroll(DM <= 4 ? DM : 1)
    for (int j = 0; j < DM; ++j) x[j] = j < d ? x0[j] : T(0);
    if (a.output.init_slot >= 0) {
      if (STAGE) {
        stg.put(out, ns, row0, N, a.output.init_slot, x);
      } else {
        T* o = out + (path * ns + a.output.init_slot) * d;
#pragma unroll(DM <= 4 ? DM : 1)
        for (int j = 0; j < DM; ++j)
          if (j < d) o[j] = x[j];
      }
    }
    DrawSource<T> src(a.draws, pc, K);
    for (int i = 0; i < a.num_steps; ++i) {
      const T dt = table[i * 4], sdt = table[i * 4 + 1];
      const int slot = (int)table[i * 4 + 2];
      T dw[DM], xn[DM];
#pragma unroll(DM <= 4 ? DM : 1)
      for (int c = 0; c < DM; ++c) dw[c] = c < d ? src.get(i, c) * sdt : T(0);
      T lev[DM];  // s0_k + s1_k x_k
#pragma unroll(DM <= 4 ? DM : 1)
      for (int k = 0; k < DM; ++k) lev[k] = cf->s0[k] + cf->s1[k] * x[k];
      if (DM == 1) {
        const T b = lev[0] * cf->C[0], g = cf->s1[0] * cf->C[0];
        const T drift = cf->m[0] + cf->M[0] * x[0];
        xn[0] = x[0] + dt * drift + b * dw[0] + (b * g) * (dw[0] * dw[0] - dt) / T(2);
      } else {
        T J[DM][DM];
        stratonovich_J<T, DM>(d, order, dt, sdt, sqrt_rho, dw, src, i, J);
#pragma unroll(DM <= 4 ? DM : 1)
        for (int k = 0; k < DM; ++k) {
          if (k >= d) {
            xn[k] = T(0);
            continue;
          }
          T drift = cf->m[k];
#pragma unroll(DM <= 4 ? DM : 1)
          for (int c = 0; c < DM; ++c) drift += cf->M[k * DM + c] * x[c];
          T u = T(0), dwi = T(0), h = T(0);
#pragma unroll(DM <= 4 ? DM : 1)
          for (int j = 0; j < DM; ++j) {
            const T Bkj = lev[k] * cf->C[k * DM + j];
            u += cf->s1[k] * cf->C[k * DM + j] * Bkj;
            dwi += Bkj * dw[j];
          }
#pragma unroll(DM <= 4 ? DM : 1)
          for (int m = 0; m < DM; ++m) {
            T l = T(0);  // sum_j dB_kj/dx_k B_jm
#pragma unroll(DM <= 4 ? DM : 1)
            for (int j = 0; j < DM; ++j) l += cf->s1[k] * cf->C[k * DM + j] * (lev[j] * cf->C[j * DM + m]);
            h += l * J[k][m];
          }
          xn[k] = x[k] + dt * (drift - u) + dwi + h;
        }
      }
#pragma unroll(DM <= 4 ? DM : 1)
      for (int k = 0; k < DM; ++k) x[k] = xn[k];
      if (slot >= 0) {
        if (STAGE) {
          stg.put(out, ns, row0, N, slot, x);
        } else {
          T* o = out + (path * ns + slot) * d;
#pragma unroll(DM <= 4 ? DM : 1)
          for (int j = 0; j < DM; ++j)
            if (j < d) o[j] = x[j];
        }
      }
    }
    if (STAGE && stg.cnt > 0) stg.flush(out, ns, row0, N);
  }
}

template <typename T, int DM>
__global__ void __launch_bounds__(kBlock) milstein_update_kernel(tqf_milstein_update_args a, double rho_c) {
  const int64_t path = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (path >= a.num_paths) return;
  const int d = a.dim, order = a.order;
  const int K = d + 3 * d * order;
  const T* x = static_cast<const T*>(a.x) + path * d;
  const T* A = static_cast<const T*>(a.drift) + path * d;
  const T* B = static_cast<const T*>(a.vol) + path * d * d;
  const T* G = static_cast<const T*>(a.grad) + path * d * d * d;  // [i][k][j]
  DrawSource<T> src(a.draws, path, K);
  const T dt = (T)a.dt, sdt = (T)a.sqrt_dt;
  T dw[DM], xn[DM];
#pragma unroll(DM <= 4 ? DM : 1)
  for (int c = 0; c < DM; ++c) dw[c] = c < d ? src.get(a.step, c) * sdt : T(0);
  T* io = a.increments_out ? static_cast<T*>(a.increments_out) + path * (int64_t)(d + d * d) : nullptr;
  if (DM == 1) {
    xn[0] = x[0] + dt * A[0] + B[0] * dw[0] + (B[0] * G[0]) * (dw[0] * dw[0] - dt) / T(2);
    if (io) {
      io[0] = dw[0];
      io[1] = dw[0] * dw[0] / T(2);
    }
  } else {
    T J[DM][DM];
    stratonovich_J<T, DM>(d, order, dt, sdt, sqrt((T)rho_c), dw, src, a.step, J);
    if (io) {
#pragma unroll(DM <= 4 ? DM : 1)
      for (int i = 0; i < DM; ++i) {
        if (i >= d) continue;
        io[i] = dw[i];
#pragma unroll(DM <= 4 ? DM : 1)
        for (int m = 0; m < DM; ++m)
          if (m < d) io[d + i * d + m] = J[i][m];
      }
    }
#pragma unroll(DM <= 4 ? DM : 1)
    for (int k = 0; k < DM; ++k) {
      if (k >= d) {
        xn[k] = T(0);
        continue;
      }
      T u = T(0), dwi = T(0), h = T(0);
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) u += G[(i * d + k) * d + j] * B[i * d + j];
      for (int j = 0; j < d; ++j) dwi += B[k * d + j] * dw[j];
#pragma unroll(DM <= 4 ? DM : 1)
      for (int i = 0; i < DM; ++i) {
        if (i >= d) continue;
#pragma unroll(DM <= 4 ? DM : 1)
        for (int m = 0; m < DM; ++m) {
          if (m >= d) continue;
          T l = T(0);
          for (int j = 0; j < d; ++j) l += G[(i * d + k) * d + j] * B[j * d + m];
          h += l * J[i][m];
        }
      }
      xn[k] = x[k] + dt * (A[k] - u) + dwi + h;
    }
  }
  T* xo = static_cast<T*>(a.x_next) + path * d;
  T* po = a.paths_out && a.out_slot >= 0 ? static_cast<T*>(a.paths_out) + (path * a.num_slots + a.out_slot) * d
                                          : nullptr;
#pragma unroll(DM <= 4 ? DM : 1)
  for (int k = 0; k < DM; ++k)
    if (k < d) {
      xo[k] = xn[k];
      if (po) po[k] = xn[k];
    }
}

// ---- any dimension: one warp per path -----------------------------------------
// For dim > 8 a warp carries one path.  Per step the warp writes the step's
// normals into per-warp shared buffers (dW, xi = dW / sqrt(dt), the last mu
// term, zeta, w = sqrt2 xi + eta), builds the Stratonovich integrals J (lane
// l owns rows i = l, l + 32, ...; stored transposed, Jt[m][i] = J_im, so the
// lanes of a warp touch consecutive words) with the arithmetic of
// stratonovich_J, then each lane updates its state rows.  Coefficients are
// read from global memory (L1/L2-resident).  Per-warp shared memory:
// 6 d + 2 d order + 2 d^2 values.
template <typename T>
__host__ __device__ inline size_t mil_wide_warp_elems(int d, int order) {
  return (size_t)6 * d + (size_t)2 * d * order + (size_t)2 * d * d;
}

template <typename T>
struct MilWarpBufs {
  T *x, *xn, *lev, *dw, *xi, *mu, *zeta, *w, *Jt, *Rt;
  __device__ MilWarpBufs(T* base, int d, int order) {
    x = base;
    xn = x + d;
    lev = xn + d;
    dw = lev + d;
    xi = dw + d;
    mu = xi + d;
    zeta = mu + d;
    w = zeta + (size_t)d * order;
    Jt = w + (size_t)d * order;
    Rt = Jt + (size_t)d * d;
  }
};

// Normals of `step` and the transposed J for this warp's path.
template <typename T>
__device__ __forceinline__ void mil_wide_draws_and_J(MilWarpBufs<T>& b, DrawSource<T>& src, int step, int d,
                                                     int order, T dt, T sdt, T sqrt_rho, int lane) {
  const T s2 = (T)1.4142135623730951;
  const int p = order - 1;
  for (int c = lane; c < d; c += 32) {
    const T dwc = src.get(step, c) * sdt;
    b.dw[c] = dwc;
    b.xi[c] = dwc / sdt;
    b.mu[c] = src.get(step, d + c * order + p);
    for (int r = 0; r < order; ++r) {
      b.zeta[c * order + r] = src.get(step, d + d * order + c * order + r);
      b.w[c * order + r] = s2 * b.xi[c] + src.get(step, d + 2 * d * order + c * order + r);
    }
  }
  __syncwarp();
  const T two_pi = (T)6.283185307179586;
  for (int i = lane; i < d; i += 32) {
    for (int m = 0; m < d; ++m) {
      T v;
      if (m == i) {
        v = b.dw[i] * b.dw[i] / T(2);
      } else {
        v = dt * (b.dw[i] * b.dw[m] / T(2) + sqrt_rho * (b.mu[i] * b.xi[m] - b.xi[i] * b.mu[m]));
        T acc = T(0);
        for (int r = 0; r < order; ++r) {
          const T inv = T(1) / T(r + 1);
          acc += (b.zeta[i * order + r] * b.w[m * order + r] - b.w[i * order + r] * b.zeta[m * order + r]) * inv;
        }
        v = v + dt * acc / two_pi;
      }
      b.Jt[(size_t)m * d + i] = v;
    }
  }
  __syncwarp();
}

template <typename T, int SRC>
__global__ void milstein_affine_wide_kernel(tqf_milstein_affine_args a, double rho_c) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int d = a.dim, order = a.order;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  MilWarpBufs<T> b(reinterpret_cast<T*>(smem) + (size_t)warp * mil_wide_warp_elems<T>(d, order), d, order);
  const T* m = static_cast<const T*>(a.drift_m);
  const T* M = static_cast<const T*>(a.drift_M);
  const T* s0 = static_cast<const T*>(a.vol_s0);
  const T* s1 = static_cast<const T*>(a.vol_s1);
  const T* C = static_cast<const T*>(a.vol_C);
  const T* table = static_cast<const T*>(a.step_table);
  const T sqrt_rho = sqrt((T)rho_c);
  const int K = d + 3 * d * order;
  T* out = static_cast<T*>(a.output.ptr);
  const int ns = a.output.num_slots;
  const int64_t N = a.num_paths;
  const int64_t nwarps = (int64_t)gridDim.x * wpb;
  for (int64_t path = (int64_t)blockIdx.x * wpb + warp; path < N; path += nwarps) {
    const T* x0 = static_cast<const T*>(a.x0) + (a.x0_per_path ? path * d : 0);
    for (int k = lane; k < d; k += 32) b.x[k] = x0[k];
    if (a.output.init_slot >= 0) {
      T* o = out + (path * ns + a.output.init_slot) * d;
      for (int k = lane; k < d; k += 32) o[k] = x0[k];
    }
    DrawSource<T> src(a.draws, path, K);
    for (int i = 0; i < a.num_steps; ++i) {
      const T dt = table[i * 4], sdt = table[i * 4 + 1];
      const int slot = (int)table[i * 4 + 2];
      __syncwarp();
      for (int k = lane; k < d; k += 32) b.lev[k] = s0[k] + s1[k] * b.x[k];
      mil_wide_draws_and_J<T>(b, src, i, d, order, dt, sdt, sqrt_rho, lane);
      for (int k = lane; k < d; k += 32) {
        T drift = m[k];
        for (int c = 0; c < d; ++c) drift += M[(size_t)k * d + c] * b.x[c];
        T u = T(0), dwi = T(0), h = T(0);
        for (int j = 0; j < d; ++j) {
          const T ckj = C[(size_t)k * d + j];
          const T Bkj = b.lev[k] * ckj;
          u += s1[k] * ckj * Bkj;
          dwi += Bkj * b.dw[j];
        }
        for (int mm = 0; mm < d; ++mm) {
          T l = T(0);  // sum_j dB_kj/dx_k B_jm
          for (int j = 0; j < d; ++j) l += s1[k] * C[(size_t)k * d + j] * (b.lev[j] * C[(size_t)j * d + mm]);
          h += l * b.Jt[(size_t)mm * d + k];
        }
        b.xn[k] = b.x[k] + dt * (drift - u) + dwi + h;
      }
      __syncwarp();
      for (int k = lane; k < d; k += 32) b.x[k] = b.xn[k];
      if (slot >= 0) {
        T* o = out + (path * ns + slot) * d;
        for (int k = lane; k < d; k += 32) o[k] = b.x[k];
      }
    }
    __syncwarp();
  }
}

// One step for caller-evaluated drift, B and dB/dx (any dimension):
// u_k = sum_{i,j} G_ikj B_ij and h_k = sum_{i,j} G_ikj R_ji with
// R_ji = sum_m B_jm J_im (the reference's sums, regrouped so that R is formed
// once per path-step).
template <typename T>
__global__ void milstein_update_wide_kernel(tqf_milstein_update_args a, double rho_c) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int d = a.dim, order = a.order;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  const int64_t path = (int64_t)blockIdx.x * wpb + warp;
  if (path >= a.num_paths) return;
  MilWarpBufs<T> b(reinterpret_cast<T*>(smem) + (size_t)warp * mil_wide_warp_elems<T>(d, order), d, order);
  const int K = d + 3 * d * order;
  const T* x = static_cast<const T*>(a.x) + path * d;
  const T* A = static_cast<const T*>(a.drift) + path * d;
  const T* B = static_cast<const T*>(a.vol) + path * (int64_t)d * d;
  const T* G = static_cast<const T*>(a.grad) + path * (int64_t)d * d * d;  // [i][k][j]
  DrawSource<T> src(a.draws, path, K);
  const T dt = (T)a.dt, sdt = (T)a.sqrt_dt;
  mil_wide_draws_and_J<T>(b, src, a.step, d, order, dt, sdt, sqrt((T)rho_c), lane);
  // Rt[i][j] = R_ji = sum_m B_jm J_im, lane-owned rows i
  for (int i = lane; i < d; i += 32)
    for (int j = 0; j < d; ++j) {
      T r = T(0);
      for (int mm = 0; mm < d; ++mm) r += B[(size_t)j * d + mm] * b.Jt[(size_t)mm * d + i];
      b.Rt[(size_t)i * d + j] = r;
    }
  __syncwarp();
  if (a.increments_out) {
    T* io = static_cast<T*>(a.increments_out) + path * ((int64_t)d + (int64_t)d * d);
    for (int c = lane; c < d; c += 32) io[c] = b.dw[c];
    for (int e = lane; e < d * d; e += 32) io[d + e] = b.Jt[(size_t)(e % d) * d + e / d];  // J_im, row-major
  }
  T* xo = static_cast<T*>(a.x_next) + path * d;
  T* po = a.paths_out && a.out_slot >= 0 ? static_cast<T*>(a.paths_out) + (path * a.num_slots + a.out_slot) * d
                                          : nullptr;
  for (int k = lane; k < d; k += 32) {
    T u = T(0), dwi = T(0), h = T(0);
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j) {
        const T g = G[((size_t)i * d + k) * d + j];
        u += g * B[(size_t)i * d + j];
        h += g * b.Rt[(size_t)i * d + j];
      }
    for (int j = 0; j < d; ++j) dwi += B[(size_t)k * d + j] * b.dw[j];
    const T v = x[k] + dt * (A[k] - u) + dwi + h;
    xo[k] = v;
    if (po) po[k] = v;
  }
}

// Warps per CTA for the wide kernels: up to 4, as shared memory allows.
template <typename T>
int mil_wide_warps(int d, int order) {
  const size_t per = mil_wide_warp_elems<T>(d, order) * sizeof(T);
  int w = (int)((200 * 1024) / (per > 0 ? per : 1));
  return w > 4 ? 4 : w;
}

// 1/12 - sum_{r=1}^{order} r^-2 / (2 pi^2), the variance factor rho_p of the
// truncated Fourier expansion (milstein_sampling.py:500-503).
double rho_constant(int order) {
  double s = 0.0;
  for (int r = 1; r <= order; ++r) s += 1.0 / ((double)r * r);
  const double pi = 3.14159265358979323846;
  return 1.0 / 12.0 - s / 2.0 / (pi * pi);
}

template <typename T, int DM>
int launch_affine(const tqf_milstein_affine_args& a, cudaStream_t s) {
  const size_t tab_bytes = (size_t)a.num_steps * 4 * sizeof(T);
  const bool staged = tab_bytes > 0 && tab_bytes <= 96 * 1024 && (reinterpret_cast<uintptr_t>(a.step_table) & 15u) == 0;
  // stage the output when a path's row is at least 64 bytes
  const bool stage = (size_t)a.output.num_slots * a.dim * sizeof(T) >= 64;
  const size_t smem =
      milstein_stage_offset<T, DM>(a.num_steps, staged) + (stage ? RowStager<T, DM, kBlock>::kBytes : 0);
  const bool philox = a.draws.source == TQF_DRAWS_PHILOX;
  void (*k)(tqf_milstein_affine_args, double, int) =
      stage ? (philox ? milstein_affine_kernel<T, DM, TQF_DRAWS_PHILOX, true>
                      : milstein_affine_kernel<T, DM, TQF_DRAWS_MEMORY, true>)
            : (philox ? milstein_affine_kernel<T, DM, TQF_DRAWS_PHILOX, false>
                      : milstein_affine_kernel<T, DM, TQF_DRAWS_MEMORY, false>);
  if (smem > 48 * 1024) set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBlock, smem) != cudaSuccess || occ < 1) occ = 1;
  int64_t grid = (a.num_paths + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  k<<<(unsigned)grid, kBlock, smem, s>>>(a, rho_constant(a.order), staged ? 1 : 0);
  return check_launch("milstein_affine_kernel");
}

template <typename T>
int launch_affine_wide(const tqf_milstein_affine_args& a, cudaStream_t s) {
  const int wpb = mil_wide_warps<T>(a.dim, a.order);
  TQF_REQUIRE(wpb >= 1, "tqf_milstein_affine: dim %d with order %d needs more than 200 KiB of shared memory", a.dim,
              a.order);
  const size_t smem = (size_t)wpb * mil_wide_warp_elems<T>(a.dim, a.order) * sizeof(T);
  auto k = a.draws.source == TQF_DRAWS_PHILOX ? milstein_affine_wide_kernel<T, TQF_DRAWS_PHILOX>
                                              : milstein_affine_wide_kernel<T, TQF_DRAWS_MEMORY>;
  set_smem_config(k, smem);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 32 * wpb, smem) != cudaSuccess || occ < 1) occ = 1;
  int64_t grid = (a.num_paths + wpb - 1) / wpb;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (grid > cap) grid = cap;
  k<<<(unsigned)grid, 32 * wpb, smem, s>>>(a, rho_constant(a.order));
  return check_launch("milstein_affine_wide_kernel");
}

template <typename T>
int dispatch_affine(const tqf_milstein_affine_args& a, cudaStream_t s) {
  if (a.dim == 1) return launch_affine<T, 1>(a, s);
  if (a.dim <= 2) return launch_affine<T, 2>(a, s);
  if (a.dim <= 4) return launch_affine<T, 4>(a, s);
  if (a.dim <= 8) return launch_affine<T, 8>(a, s);
  return launch_affine_wide<T>(a, s);
}

template <typename T>
int dispatch_update(const tqf_milstein_update_args& a, cudaStream_t s) {
  if (a.dim > kMaxDimMil) {
    const int wpb = mil_wide_warps<T>(a.dim, a.order);
    TQF_REQUIRE(wpb >= 1, "tqf_milstein_update: dim %d with order %d needs more than 200 KiB of shared memory",
                a.dim, a.order);
    const size_t smem = (size_t)wpb * mil_wide_warp_elems<T>(a.dim, a.order) * sizeof(T);
    const int64_t grid = (a.num_paths + wpb - 1) / wpb;
    TQF_REQUIRE(grid <= 2147483647LL, "tqf_milstein_update: too many paths");
    set_smem_config(milstein_update_wide_kernel<T>, smem);
    milstein_update_wide_kernel<T><<<(unsigned)grid, 32 * wpb, smem, s>>>(a, rho_constant(a.order));
    return check_launch("milstein_update_wide_kernel");
  }
  const int64_t grid = (a.num_paths + kBlock - 1) / kBlock;
  TQF_REQUIRE(grid <= 2147483647LL, "tqf_milstein_update: too many paths");
  const double rc = rho_constant(a.order);
  if (a.dim == 1) milstein_update_kernel<T, 1><<<(unsigned)grid, kBlock, 0, s>>>(a, rc);
  else if (a.dim <= 2) milstein_update_kernel<T, 2><<<(unsigned)grid, kBlock, 0, s>>>(a, rc);
  else if (a.dim <= 4) milstein_update_kernel<T, 4><<<(unsigned)grid, kBlock, 0, s>>>(a, rc);
  else milstein_update_kernel<T, 8><<<(unsigned)grid, kBlock, 0, s>>>(a, rc);
  return check_launch("milstein_update_kernel");
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_milstein_affine(const tqf_milstein_affine_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_milstein_affine: null args");
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "tqf_milstein_affine: bad dtype %d", a->dtype);
  TQF_REQUIRE(a->dim >= 1, "tqf_milstein_affine: dim must be >= 1, got %d", a->dim);
  TQF_REQUIRE(a->order >= 1 && a->order <= 64, "tqf_milstein_affine: order must be in [1, 64], got %d", a->order);
  TQF_REQUIRE(a->num_paths >= 1 && a->num_steps >= 0, "tqf_milstein_affine: bad sizes");
  TQF_REQUIRE(a->x0 && a->drift_m && a->drift_M && a->vol_s0 && a->vol_s1 && a->vol_C,
              "tqf_milstein_affine: null coefficient pointer");
  TQF_REQUIRE(a->num_steps == 0 || a->step_table, "tqf_milstein_affine: null step_table");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr || a->num_steps == 0,
              "tqf_milstein_affine: memory draws need draws.ptr");
  TQF_REQUIRE(!a->draws.antithetic || 2 * a->draws.antithetic_half == a->num_paths,
              "tqf_milstein_affine: antithetic needs num_paths == 2 * antithetic_half");
  TQF_REQUIRE(a->output.ptr && a->output.num_slots >= 1 && a->output.init_slot < a->output.num_slots,
              "tqf_milstein_affine: bad output");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? dispatch_affine<float>(*a, s) : dispatch_affine<double>(*a, s);
}

extern "C" int tqf_milstein_update(const tqf_milstein_update_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_milstein_update: null args");
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "tqf_milstein_update: bad dtype %d", a->dtype);
  TQF_REQUIRE(a->dim >= 1, "tqf_milstein_update: dim must be >= 1, got %d", a->dim);
  TQF_REQUIRE(a->order >= 1 && a->order <= 64, "tqf_milstein_update: bad order %d", a->order);
  TQF_REQUIRE(a->num_paths >= 1, "tqf_milstein_update: num_paths must be >= 1");
  TQF_REQUIRE(a->x && a->drift && a->vol && a->grad && a->x_next, "tqf_milstein_update: null pointer");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr, "tqf_milstein_update: memory draws need ptr");
  TQF_REQUIRE(!a->paths_out || a->out_slot < a->num_slots, "tqf_milstein_update: out_slot out of range");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? dispatch_update<float>(*a, s) : dispatch_update<double>(*a, s);
}
