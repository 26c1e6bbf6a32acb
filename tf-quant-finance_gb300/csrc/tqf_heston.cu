// Heston path kernels: full-truncation Euler (the reference Euler sampler run
// with Heston coefficients, tff/models/euler_sampling.py:513-537) and the
// Andersen QE scheme of HestonModel.sample_paths
// (tff/models/heston/heston_model.py:322-460, 522-572).
//
// One thread per path, state (log-spot, variance) in registers, the per-step
// table staged once per CTA into shared memory by a TMA bulk copy, draws
// generated in-kernel (Philox4x32-10, one block = two steps of two normals)
// or read from memory.  Optional coalescing-friendly stores of the recorded
// states and a fused European payoff over up to 1024 strikes with FP64
// cross-path accumulation in a fixed order (deterministic).  The CTA loop is
// persistent: grid = SMs x resident CTAs, each CTA walks path tiles.
#include <mutex>
#include <vector>

#include "tqf_internal.cuh"

namespace tqf {
namespace {

constexpr int kBlock = 256;
constexpr int kFtCols = 8;
constexpr int kQeCols = 12;
constexpr size_t kMaxStagedTable = 96 * 1024;

struct SmemLayout {
  size_t bar, table, acc, spot, strike, call, stage, sobol, total;
};

// In-kernel Sobol draws: tables for this many steps (two dimensions each)
// are built per window (SobolTables).
constexpr int kSobolWindow = 64;

// Recorded states are staged in shared memory, kStage<T> consecutive slots
// (128 bytes of a path's output row) per flush; see SlotStager.
template <typename T>
constexpr int kStage = 128 / (2 * (int)sizeof(T));

template <typename T>
SmemLayout smem_layout(int steps, int cols, int ns, bool staged, bool store, bool sobol = false) {
  SmemLayout L;
  size_t off = 0;
  L.bar = off;
  off += 16;
  L.table = off;
  // an even number of rows: the paired full-truncation loop rewrites the
  // table as two-step blocks (pair_ft_table)
  if (staged) off += (size_t)((steps + 1) & ~1) * cols * sizeof(T);
  off = (off + 15) & ~(size_t)15;
  L.acc = off;
  off += (size_t)ns * 4 * 2 * sizeof(double);
  L.spot = off;
  off += (ns > 0 ? kBlock : 0) * sizeof(T);
  L.strike = off;
  off += (size_t)ns * sizeof(T);
  L.call = off;
  off += (size_t)ns;
  off = (off + 15) & ~(size_t)15;
  L.stage = off;
  if (store) off += (size_t)kStage<T> * (kBlock + 1) * 2 * sizeof(T);
  off = (off + 15) & ~(size_t)15;
  L.sobol = off;
  if (sobol) off += (size_t)2 * kSobolWindow * SobolTables::kRow * sizeof(uint32_t);
  L.total = (off + 15) & ~(size_t)15;
  return L;
}

// ---- one step of each scheme ---------------------------------------------
// Full-truncation Euler in the Euler sampler's form with pre-scaled step
// constants: row = (dt/2, sqrt dt, r dt, kappa dt, kappa theta dt, xi rho,
// xi sqrt(1 - rho^2), slot):
//   x' = x + (r dt - dt/2 v+) + sqrt(v+) dw0
//   v' = v + (kappa theta dt - kappa dt v+) + sqrt(v+) (xi rho dw0 + xi sqrt(1-rho^2) dw1)
template <typename T>
struct FtRow {
  T hdt, sdt, rdt, kdt, kthdt, xirho, xisq, slot;
};

template <typename T>
__device__ __forceinline__ FtRow<T> load_ft_row(const T* __restrict__ row) {
  FtRow<T> r;
  if constexpr (sizeof(T) == 4) {
    const float4 a = reinterpret_cast<const float4*>(row)[0];
    const float4 b = reinterpret_cast<const float4*>(row)[1];
    r.hdt = a.x; r.sdt = a.y; r.rdt = a.z; r.kdt = a.w;
    r.kthdt = b.x; r.xirho = b.y; r.xisq = b.z; r.slot = b.w;
  } else {
    r.hdt = row[0]; r.sdt = row[1]; r.rdt = row[2]; r.kdt = row[3];
    r.kthdt = row[4]; r.xirho = row[5]; r.xisq = row[6]; r.slot = row[7];
  }
  return r;
}

template <typename T>
__device__ __forceinline__ void ft_step(const FtRow<T>& c, T z0, T z1, T& x, T& v) {
  const T vp = v > T(0) ? v : T(0);
  const T sq = sqrt_approx(vp);
  const T dw0 = z0 * c.sdt;
  const T dw1 = z1 * c.sdt;
  const T x_next = x + fma(-c.hdt, vp, c.rdt) + sq * dw0;
  const T v_next = v + fma(-c.kdt, vp, c.kthdt) + sq * fma(c.xisq, dw1, c.xirho * dw0);
  x = x_next;
  v = v_next;
}

template <typename T>
__device__ __forceinline__ void ft_step(const T* __restrict__ row, T z0, T z1, T& x, T& v) {
  ft_step<T>(load_ft_row<T>(row), z0, z1, x, v);
}

// Rewrites a staged float FT table [steps][8] in place as two-step blocks
// (ft_pair_block).  Each thread rewrites whole blocks of its own; the caller
// synchronises.
__device__ __forceinline__ void pair_ft_table(float* tb, int steps) {
  const int pairs = (steps + 1) >> 1;
  for (int p = threadIdx.x; p < pairs; p += blockDim.x) {
    float4 q[4];
    ft_pair_block(tb, steps, p, q);
    float4* blk = reinterpret_cast<float4*>(tb + 16 * p);
    blk[0] = q[0];
    blk[1] = q[1];
    blk[2] = q[2];
    blk[3] = q[3];
  }
}

template <typename T>
__device__ __forceinline__ T qe_erf(T x);
template <>
__device__ __forceinline__ float qe_erf<float>(float x) { return erff(x); }
template <>
__device__ __forceinline__ double qe_erf<double>(double x) { return erf(x); }

// Division and square root of the QE step: in float32 the SFU square root
// and the fast division (both within 2 ulp; the operands are moderate
// positive numbers: m >= theta (1 - E) > 0, psi > 0, b2 >= 1), in float64
// the IEEE operations.  log and erf stay the library functions (log(1 - p)
// near 1 needs their accuracy).
__device__ __forceinline__ float qe_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double qe_div(double a, double b) { return a / b; }
__device__ __forceinline__ float qe_sqrt(float a) { return sqrt_approx(a); }
__device__ __forceinline__ double qe_sqrt(double a) { return sqrt(a); }

template <typename T>
__device__ __forceinline__ void qe_step(const T* __restrict__ row, T zv, T zx, T& x, T& v) {
  // float rows [skip, theta, E, A | B, k0, k1, k2 | k3, k4, -, slot] are
  // 16-byte aligned (the table base is, and a row is 48 bytes): three vector
  // loads; double rows are read value by value, the log-spot constants after
  // the variance update (loading them up front costs the double kernels up
  // to 15 registers)
  T theta, E, A, B, k0, k1, k2, k3, k4;
  if constexpr (sizeof(T) == 4) {
    const float4 q0 = reinterpret_cast<const float4*>(row)[0];
    if (q0.x != 0.f) return;  // dt <= tolerance: state kept, draws consumed
    const float4 q1 = reinterpret_cast<const float4*>(row)[1];
    const float4 q2 = reinterpret_cast<const float4*>(row)[2];
    theta = q0.y; E = q0.z; A = q0.w;
    B = q1.x; k0 = q1.y; k1 = q1.z; k2 = q1.w;
    k3 = q2.x; k4 = q2.y;
  } else {
    if (row[0] != T(0)) return;
    theta = row[1]; E = row[2]; A = row[3]; B = row[4];
  }
  const T m = theta + (v - theta) * E;
  const T s2 = v * A + B;
  const T psi = qe_div(s2, m * m);
  T v_next;
  if (psi < T(1.5)) {
    const T psi_inv = qe_div(T(2), psi);
    const T b2 = psi_inv - T(1) + qe_sqrt(psi_inv * (psi_inv - T(1)));
    const T a = qe_div(m, T(1) + b2);
    const T t = qe_sqrt(b2) + zv;
    v_next = a * (t * t);
  } else {
    const T p = qe_div(psi - T(1), psi + T(1));
    const T beta = qe_div(T(1) - p, m);
    const T u = T(0.5) * (T(1) + qe_erf<T>(qe_div(zv, T(1.41421356237309504880))));
    v_next = u > p ? qe_div(log(T(1) - p) - log(T(1) - u), beta) : T(0);
  }
  if constexpr (sizeof(T) == 8) {
    k0 = row[5]; k1 = row[6]; k2 = row[7]; k3 = row[8]; k4 = row[9];
  }
  x = x + k0 + k1 * v + k2 * v_next + qe_sqrt(k3 * v + k4 * v_next) * zx;
  v = v_next;
}

template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
  using type = float2;
};
template <>
struct Vec2<double> {
  using type = double2;
};

// Coalesced output of the recorded states.  Each recorded step a thread puts
// its (x, v) into row `cnt` of a [kStage][kBlock + 1] shared-memory buffer;
// when the buffer is full, or the next slot does not continue the buffered
// run, the CTA writes the run out: consecutive threads take consecutive slots
// of one path, so a warp stores whole 128-byte pieces of two output rows
// instead of 32 scattered 8-byte pieces (the padded row stride keeps the
// shared-memory reads conflict-free).  Slots come from the step table, so
// every thread of the CTA puts and flushes at the same steps.
template <typename T>
struct SlotStager {
  using V2 = typename Vec2<T>::type;
  static constexpr int S = kStage<T>;
  V2* buf;
  int cnt, slot0;
  __device__ explicit SlotStager(unsigned char* smem) : buf(reinterpret_cast<V2*>(smem)), cnt(0), slot0(0) {}
  __device__ __forceinline__ void put(const tqf_path_output& o, int64_t row0, int64_t N, int slot, T x, T v) {
    if (cnt > 0 && (cnt == S || slot != slot0 + cnt)) flush(o, row0, N);
    if (cnt == 0) slot0 = slot;
    V2 w;
    w.x = x;
    w.y = v;
    buf[cnt * (kBlock + 1) + threadIdx.x] = w;
    ++cnt;
  }
  __device__ __forceinline__ void flush(const tqf_path_output& o, int64_t row0, int64_t N) {
    __syncthreads();
    V2* out = reinterpret_cast<V2*>(o.ptr);
    if (cnt == S) {
#pragma unroll 4
      for (int idx = threadIdx.x; idx < S * kBlock; idx += kBlock) {
        const int p = idx / S, j = idx % S;
        if (row0 + p < N) out[(row0 + p) * o.num_slots + slot0 + j] = buf[j * (kBlock + 1) + p];
      }
    } else {
      for (int idx = threadIdx.x; idx < cnt * kBlock; idx += kBlock) {
        const int p = idx / cnt, j = idx - p * cnt;
        if (row0 + p < N) out[(row0 + p) * o.num_slots + slot0 + j] = buf[j * (kBlock + 1) + p];
      }
    }
    __syncthreads();
    cnt = 0;
  }
};

// SCHEME 0 = full-truncation Euler, 1 = QE.  SRC = TQF_DRAWS_* (compile-time);
// ANTI: antithetic Philox pairing.
template <typename T, int SCHEME, int SRC, bool STORE, bool PRICE, bool ANTI>
__global__ void __launch_bounds__(kBlock)
    heston_kernel(tqf_heston_args a, int staged, SmemLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int COLS = SCHEME == 0 ? kFtCols : kQeCols;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L.bar);
  const T* table = staged ? reinterpret_cast<const T*>(smem + L.table)
                          : static_cast<const T*>(a.step_table);
  const int steps = a.num_steps;
  if (staged) {
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    uint32_t phase = 0;
    if (!stage_to_smem(smem + L.table, a.step_table, (uint32_t)(steps * COLS * sizeof(T)), bar,
                       phase, a.dev_status))
      return;
  }
  // Full-truncation float paths with in-kernel draws take two steps per
  // Philox block in f32x2 arithmetic from the staged table's pair blocks.
  constexpr bool kPairable = SCHEME == 0 && SRC == TQF_DRAWS_PHILOX && sizeof(T) == 4;
  const bool paired = kPairable && staged;
  // With in-kernel Sobol draws, a staged full-truncation table whose rows
  // are all equal (a uniform grid with constant parameters and no recorded
  // steps: the pricing calls) is read once into registers instead of once
  // per step; rows are compared bit for bit, so the arithmetic is unchanged.
  bool uniform = false;
  if (SCHEME == 0 && SRC == TQF_DRAWS_SOBOL && staged && !STORE) {
    int same = 1;
    const uint32_t* tw = reinterpret_cast<const uint32_t*>(table);
    constexpr int W = COLS * (int)sizeof(T) / 4;
    for (int idx = threadIdx.x; idx < steps * W; idx += kBlock) same &= tw[idx] == tw[idx % W];
    uniform = __syncthreads_and(same) != 0;
  }
  if (kPairable && paired) {
    pair_ft_table(reinterpret_cast<float*>(smem + L.table), steps);
    __syncthreads();
  }
  double* acc = reinterpret_cast<double*>(smem + L.acc);
  T* s_spot = reinterpret_cast<T*>(smem + L.spot);
  T* s_strike = reinterpret_cast<T*>(smem + L.strike);
  uint8_t* s_call = smem + L.call;
  const int ns = a.payoff.num_strikes;
  if (PRICE) {
    for (int i = threadIdx.x; i < 8 * ns; i += kBlock) acc[i] = 0.0;
    for (int i = threadIdx.x; i < ns; i += kBlock) {
      s_strike[i] = static_cast<const T*>(a.payoff.strikes)[i];
      s_call[i] = a.payoff.is_call ? a.payoff.is_call[i] : (uint8_t)1;
    }
    __syncthreads();
  }
  const T x0 = (T)a.x0, v0 = (T)a.v0;
  const T spot_scale = (T)a.payoff.spot_scale;
  const int64_t N = a.num_paths;
  const int64_t per_round = (int64_t)gridDim.x * kBlock;
  SlotStager<T> stg(smem + L.stage);
  for (int64_t base = 0; base < N; base += per_round) {
    const int64_t row0 = base + (int64_t)blockIdx.x * kBlock;
    const int64_t path = row0 + threadIdx.x;
    const bool valid = path < N;
    // with stores every thread runs the steps (the stager's flushes are CTA
    // barriers); a thread past the last path simulates that path again and
    // its output is dropped
    const int64_t pc = valid ? path : N - 1;
    T x = x0, v = v0;
    // In-kernel Sobol draws build shared tables per window (CTA barriers),
    // so every thread runs the steps; a thread past the last path takes the
    // next point index and its result is dropped.
    if (valid || STORE || SRC == TQF_DRAWS_SOBOL) {
      if (STORE && a.output.init_slot >= 0) stg.put(a.output, row0, N, a.output.init_slot, x, v);
      if (SRC == TQF_DRAWS_PHILOX && sizeof(T) == 4) {
        // Canonical stream, 2 normals per step: block b = steps 2b, 2b+1.
        int64_t p = pc;
        float sign = 1.f;
        if (ANTI && p >= a.draws.antithetic_half) {
          p -= a.draws.antithetic_half;
          sign = -1.f;
        }
        p += a.draws.path_offset;
        const uint32_t k0 = a.draws.key0, k1 = a.draws.key1;
        const uint32_t plo = (uint32_t)p, phi = (uint32_t)((uint64_t)p >> 32);
        auto one_step = [&](int i, float za, float zb) {
          const T* r0 = table + (size_t)i * COLS;
          if (ANTI) {
            za *= sign;
            zb *= sign;
          }
          if constexpr (SCHEME == 0) {
            const FtRow<T> row = load_ft_row<T>(r0);
            ft_step<T>(row, (T)za, (T)zb, x, v);
            if (STORE) {
              const int slot = (int)row.slot;
              if (slot >= 0) stg.put(a.output, row0, N, slot, x, v);
            }
          } else {
            qe_step<T>(r0, (T)za, (T)zb, x, v);
            if (STORE) {
              const int slot = (int)r0[COLS - 1];
              if (slot >= 0) stg.put(a.output, row0, N, slot, x, v);
            }
          }
        };
        if constexpr (kPairable) {
          if (paired) {
            const float4* tp = reinterpret_cast<const float4*>(table);
            // steps 2p and 2p + 1 from Philox block p
            auto pair_steps = [&](int pb, bool both) {
              const uint4 r = philox4x32_10(make_uint4((uint32_t)pb, plo, phi, 0u), k0, k1);
              float2 ze, zo;
              box_muller_pair_f32(r, ze, zo);
              if (ANTI) {
                ze = mul2(ze, make_float2(sign, sign));
                zo = mul2(zo, make_float2(sign, sign));
              }
              const float4 qa = tp[4 * pb], qx = tp[4 * pb + 3];
              float2 dw0, e;
              ft_pair_increments(ze, zo, tp[4 * pb + 2], qx, dw0, e);
              ft_half_step(qa, dw0.x, e.x, x, v);
              if (STORE) {
                const int slot = (int)qx.z;
                if (slot >= 0) stg.put(a.output, row0, N, slot, x, v);
              }
              if (both) {
                ft_half_step(tp[4 * pb + 1], dw0.y, e.y, x, v);
                if (STORE) {
                  const int slot = (int)qx.w;
                  if (slot >= 0) stg.put(a.output, row0, N, slot, x, v);
                }
              }
            };
            // (the constants stay shared-memory operands even for a uniform
            // table: holding them in registers costs this loop ~18 registers
            // and two resident CTAs per SM, measured 15 % slower)
            const int full = steps >> 1;
#pragma unroll 1
            for (int pb = 0; pb < full; ++pb) pair_steps(pb, true);
            if (steps & 1) pair_steps(full, false);
          }
        }
        int i = paired ? steps : 0;
#pragma unroll 2
        for (; i + 1 < steps; i += 2) {
          const uint4 r = philox4x32_10(make_uint4((uint32_t)(i >> 1), plo, phi, 0u), k0, k1);
          float2 ze, zo;  // (z0, z2), (z1, z3): box_muller_f32 of (x, y) and (z, w)
          box_muller_pair_f32(r, ze, zo);
          one_step(i, ze.x, zo.x);
          one_step(i + 1, ze.y, zo.y);
        }
        if (i < steps) {
          const uint4 r = philox4x32_10(make_uint4((uint32_t)(i >> 1), plo, phi, 0u), k0, k1);
          float z0, z1;
          box_muller_f32(r.x, r.y, z0, z1);
          one_step(i, z0, z1);
        }
      } else if constexpr (SRC == TQF_DRAWS_SOBOL) {
        const uint32_t* sv = static_cast<const uint32_t*>(a.draws.ptr);
        const int nd = (int)a.draws.key0;
        const uint32_t i0 = (uint32_t)(a.draws.path_offset + 1 + row0);
        const uint32_t ip = i0 + threadIdx.x;
        const int lo = (int)(ip & 15u), mid = 16 + (int)((ip >> 4) & 15u);
        const int hi = 32 + (int)((ip >> 8) - (i0 >> 8));
        uint32_t* tabs = reinterpret_cast<uint32_t*>(smem + L.sobol);
        T sc;  // float32: 2^(1-nd) (sobol_normal_f32), float64: 2^-nd
        if constexpr (sizeof(T) == 4) sc = __uint_as_float((uint32_t)(128 - nd) << 23);
        else sc = ldexp(1.0, -nd);
        for (int s0 = 0; s0 < steps; s0 += kSobolWindow) {
          const int nw = steps - s0 < kSobolWindow ? steps - s0 : kSobolWindow;
          __syncthreads();
          SobolTables::build(tabs, sv, 2 * s0, 2 * nw, i0, nd);
          __syncthreads();
          if (SCHEME == 0 && uniform) {
            const FtRow<T> row = load_ft_row<T>(table);
#pragma unroll 2
            for (int s = 0; s < nw; ++s) {
              const uint32_t* t0 = tabs + 2 * s * SobolTables::kRow;
              const uint32_t* t1 = t0 + SobolTables::kRow;
              const T z0 = sobol_normal(t0[lo] ^ t0[mid] ^ t0[hi], sc);
              const T z1 = sobol_normal(t1[lo] ^ t1[mid] ^ t1[hi], sc);
              ft_step<T>(row, z0, z1, x, v);
            }
            continue;
          }
#pragma unroll 2
          for (int s = 0; s < nw; ++s) {
            const uint32_t* t0 = tabs + 2 * s * SobolTables::kRow;
            const uint32_t* t1 = t0 + SobolTables::kRow;
            const T z0 = sobol_normal(t0[lo] ^ t0[mid] ^ t0[hi], sc);
            const T z1 = sobol_normal(t1[lo] ^ t1[mid] ^ t1[hi], sc);
            const T* r0 = table + (size_t)(s0 + s) * COLS;
            if (SCHEME == 0) ft_step<T>(r0, z0, z1, x, v);
            else qe_step<T>(r0, z0, z1, x, v);
            if (STORE) {
              const int slot = (int)r0[COLS - 1];
              if (slot >= 0) stg.put(a.output, row0, N, slot, x, v);
            }
          }
        }
      } else {
        DrawSource<T> src(a.draws, pc, 2);
        for (int i = 0; i < steps; ++i) {
          const T z0 = src.get(i, 0);
          const T z1 = src.get(i, 1);
          const T* r0 = table + (size_t)i * COLS;
          if (SCHEME == 0) ft_step<T>(r0, z0, z1, x, v);
          else qe_step<T>(r0, z0, z1, x, v);
          if (STORE) {
            const int slot = (int)r0[COLS - 1];
            if (slot >= 0) stg.put(a.output, row0, N, slot, x, v);
          }
        }
      }
    }
    if (STORE && stg.cnt > 0) stg.flush(a.output, row0, N);
    if (PRICE) {
      __syncthreads();
      s_spot[threadIdx.x] = valid ? spot_scale * exp(x) : T(NAN);
      __syncthreads();
      payoff_round<kBlock, T>(s_spot, s_strike, s_call, ns, acc);
    }
  }
  if (PRICE) {
    __syncthreads();
    payoff_flush(acc, ns, 4, static_cast<double*>(a.payoff.workspace));
  }
}

// ---- pathwise adjoint of the full-truncation Euler pricer ------------------
// Replays each path from its counter-based draws carrying forward tangents
// of (x, v) with respect to P = (log S0, v0, kappa, theta, xi, rho, r), then
// contracts with the upstream weights: per path
//   c = sum_j w_j dPayoff_j/dS_T (call: 1{S > K_j}, put: -1{S < K_j}),
//   out_p += c * S_T * dx_T/dP_p.
// Parameters are constant in time here (the pricing API's grid).
constexpr int kAdjParams = 7;

template <int P, typename T>
__device__ __forceinline__ void adj_param_step(T dt, T dw0, T dw1, T vp, T sq, T dsq, T kappa, T theta,
                                               T A, T B, T rho, T xi, T sr, T& xd, T& vd) {
  // explicit derivatives of the step coefficients w.r.t. parameter P
  constexpr bool is_k = P == 2, is_th = P == 3, is_xi = P == 4, is_rho = P == 5, is_r = P == 6;
  const T vpd = vp > T(0) ? vd : T(0);
  const T sqd = dsq * vpd;
  T xdn = xd + dt * (-T(0.5) * vpd) + sqd * dw0;
  if (is_r) xdn += dt;
  T vdn = vd + dt * (-kappa * vpd);
  if (is_k) vdn += dt * (theta - vp);
  if (is_th) vdn += dt * kappa;
  T Ad = T(0), Bd = T(0);
  if (is_xi) {
    Ad = rho;
    Bd = sr;
  }
  if (is_rho) {
    Ad = xi;
    Bd = -xi * rho / sr;
  }
  vdn += (Ad * sq + A * sqd) * dw0 + (Bd * sq + B * sqd) * dw1;
  xd = xdn;
  vd = vdn;
}

// The same tangent step for parameters P and Q at once, as the two lanes of
// f32x2 pairs (float32 replay: tangents carried as pairs (0, 1), (2, 3),
// (4, 5)).  The broadcast pairs hold one step's values in both lanes; the
// parameter-specific terms enter as lane constants (0 in a lane without one).
template <int P>
__device__ __forceinline__ void adj_vol_terms(float rho, float xi, float sr, float& Ad, float& Bd) {
  Ad = P == 4 ? rho : (P == 5 ? xi : 0.f);
  Bd = P == 4 ? sr : (P == 5 ? -xi * rho / sr : 0.f);
}
template <int P, int Q>
__device__ __forceinline__ void adj_pair_step(float2 dtb, float2 dw0b, float2 dw1b, float vp, float sq, float2 dsqb,
                                              float2 nkb, float kappa, float theta, float2 Ab, float2 Bb,
                                              float rho, float xi, float sr, float2& xd, float2& vd) {
  const float m = vp > 0.f ? 1.f : 0.f;
  const float2 vpd = mul2(vd, make_float2(m, m));
  const float2 sqd = mul2(dsqb, vpd);
  float2 xdn = fma2(dtb, mul2(make_float2(-0.5f, -0.5f), vpd), xd);
  xdn = fma2(sqd, dw0b, xdn);
  if (P == 6 || Q == 6) xdn = add2(xdn, make_float2(P == 6 ? dtb.x : 0.f, Q == 6 ? dtb.x : 0.f));
  float2 vdn = fma2(dtb, mul2(nkb, vpd), vd);
  if (P == 2 || Q == 2 || P == 3 || Q == 3) {
    auto c = [&](int r) { return r == 2 ? dtb.x * (theta - vp) : (r == 3 ? dtb.x * kappa : 0.f); };
    vdn = add2(vdn, make_float2(c(P), c(Q)));
  }
  float AdP, BdP, AdQ, BdQ;
  adj_vol_terms<P>(rho, xi, sr, AdP, BdP);
  adj_vol_terms<Q>(rho, xi, sr, AdQ, BdQ);
  const float2 e0 = fma2(Ab, sqd, make_float2(AdP * sq, AdQ * sq));
  const float2 e1 = fma2(Bb, sqd, make_float2(BdP * sq, BdQ * sq));
  vdn = fma2(e0, dw0b, vdn);
  vdn = fma2(e1, dw1b, vdn);
  xd = xdn;
  vd = vdn;
}

template <typename T, int SRC>
__global__ void __launch_bounds__(kBlock) heston_adjoint_kernel(tqf_heston_adjoint_args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  T* s_strike = reinterpret_cast<T*>(smem);
  T* s_w = s_strike + a.num_strikes;
  uint8_t* s_call = reinterpret_cast<uint8_t*>(s_w + a.num_strikes);
  __shared__ double acc[kBlock / 32][kAdjParams];
  for (int i = threadIdx.x; i < a.num_strikes; i += kBlock) {
    s_strike[i] = static_cast<const T*>(a.strikes)[i];
    s_w[i] = static_cast<const T*>(a.weights)[i];
    s_call[i] = a.is_call ? a.is_call[i] : (uint8_t)1;
  }
  for (int i = threadIdx.x; i < (kBlock / 32) * kAdjParams; i += kBlock) (&acc[0][0])[i] = 0.0;
  __syncthreads();
  const T* table = static_cast<const T*>(a.step_table);
  const T xi = (T)a.xi, rho = (T)a.rho, sr = sqrt(T(1) - rho * rho);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t per_round = (int64_t)gridDim.x * kBlock;
  for (int64_t base = 0; base < a.num_paths; base += per_round) {
    const int64_t path = base + (int64_t)blockIdx.x * kBlock + threadIdx.x;
    T q[kAdjParams];
#pragma unroll
    for (int p = 0; p < kAdjParams; ++p) q[p] = T(0);
    if (path < a.num_paths && sizeof(T) == 4) {
      if constexpr (sizeof(T) == 4) {
        // float32: tangents of (log S0, v0), (kappa, theta), (xi, rho) in
        // f32x2 pairs, the rate's alone
        float x = (float)a.x0, v = (float)a.v0;
        float2 xd01 = make_float2(1.f, 0.f), vd01 = make_float2(0.f, 1.f);
        float2 xd23 = make_float2(0.f, 0.f), vd23 = xd23, xd45 = xd23, vd45 = xd23;
        float xd6 = 0.f, vd6 = 0.f;
        DrawSource<float> src(a.draws, path, 2);
        const float kappa = (float)a.kappa, theta = (float)a.theta;
        const float2 nkb = make_float2(-kappa, -kappa);
        for (int i = 0; i < a.num_steps; ++i) {
          const FtRow<float> row = load_ft_row<float>(table + (size_t)i * kFtCols);
          const float dt = 2.f * row.hdt, sdt = row.sdt, A = row.xirho, B = row.xisq;
          const float z0 = src.get(i, 0), z1 = src.get(i, 1);
          const float vp = v > 0.f ? v : 0.f;
          const float sq = sqrt_approx(vp);  // shared with ft_step below
          const float dsq = sq > 0.f ? qe_div(0.5f, sq) : 0.f;
          const float dw0 = z0 * sdt, dw1 = z1 * sdt;
          const float2 dtb = make_float2(dt, dt), dw0b = make_float2(dw0, dw0), dw1b = make_float2(dw1, dw1);
          const float2 dsqb = make_float2(dsq, dsq), Ab = make_float2(A, A), Bb = make_float2(B, B);
          adj_pair_step<0, 1>(dtb, dw0b, dw1b, vp, sq, dsqb, nkb, kappa, theta, Ab, Bb, rho, xi, sr, xd01, vd01);
          adj_pair_step<2, 3>(dtb, dw0b, dw1b, vp, sq, dsqb, nkb, kappa, theta, Ab, Bb, rho, xi, sr, xd23, vd23);
          adj_pair_step<4, 5>(dtb, dw0b, dw1b, vp, sq, dsqb, nkb, kappa, theta, Ab, Bb, rho, xi, sr, xd45, vd45);
          adj_param_step<6, float>(dt, dw0, dw1, vp, sq, dsq, kappa, theta, A, B, rho, xi, sr, xd6, vd6);
          ft_step<float>(row, z0, z1, x, v);
        }
        const float S = exp(x);
        float c = 0.f;
        for (int j = 0; j < a.num_strikes; ++j) {
          const bool call = s_call[j] != 0;
          if (call ? (S > s_strike[j]) : (S < s_strike[j])) c += call ? s_w[j] : -s_w[j];
        }
        const float xdv[kAdjParams] = {xd01.x, xd01.y, xd23.x, xd23.y, xd45.x, xd45.y, xd6};
#pragma unroll
        for (int p = 0; p < kAdjParams; ++p) q[p] = c * S * xdv[p];
      }
    } else if (path < a.num_paths) {
      T x = (T)a.x0, v = (T)a.v0;
      T xd[kAdjParams], vd[kAdjParams];
#pragma unroll
      for (int p = 0; p < kAdjParams; ++p) {
        xd[p] = p == 0 ? T(1) : T(0);
        vd[p] = p == 1 ? T(1) : T(0);
      }
      DrawSource<T> src(a.draws, path, 2);
      for (int i = 0; i < a.num_steps; ++i) {
        const FtRow<T> row = load_ft_row<T>(table + (size_t)i * kFtCols);
        const T dt = T(2) * row.hdt, sdt = row.sdt, kappa = (T)a.kappa;
        const T theta = (T)a.theta, A = row.xirho, B = row.xisq;
        const T z0 = src.get(i, 0), z1 = src.get(i, 1);
        const T vp = v > T(0) ? v : T(0);
        // the forward step's square root (sqrt_approx, shared with ft_step
        // below) and its derivative 1 / (2 sqrt(v+))
        const T sq = sqrt_approx(vp);
        const T dsq = sq > T(0) ? qe_div(T(0.5), sq) : T(0);
        const T dw0 = z0 * sdt, dw1 = z1 * sdt;
        adj_param_step<0, T>(dt, dw0, dw1, vp, sq, dsq, kappa, theta, A, B, rho, xi, sr, xd[0], vd[0]);
        adj_param_step<1, T>(dt, dw0, dw1, vp, sq, dsq, kappa, theta, A, B, rho, xi, sr, xd[1], vd[1]);
        adj_param_step<2, T>(dt, dw0, dw1, vp, sq, dsq, kappa, theta, A, B, rho, xi, sr, xd[2], vd[2]);
        adj_param_step<3, T>(dt, dw0, dw1, vp, sq, dsq, kappa, theta, A, B, rho, xi, sr, xd[3], vd[3]);
        adj_param_step<4, T>(dt, dw0, dw1, vp, sq, dsq, kappa, theta, A, B, rho, xi, sr, xd[4], vd[4]);
        adj_param_step<5, T>(dt, dw0, dw1, vp, sq, dsq, kappa, theta, A, B, rho, xi, sr, xd[5], vd[5]);
        adj_param_step<6, T>(dt, dw0, dw1, vp, sq, dsq, kappa, theta, A, B, rho, xi, sr, xd[6], vd[6]);
        ft_step<T>(row, z0, z1, x, v);
      }
      const T S = exp(x);
      T c = T(0);
      for (int j = 0; j < a.num_strikes; ++j) {
        const bool call = s_call[j] != 0;
        if (call ? (S > s_strike[j]) : (S < s_strike[j])) c += call ? s_w[j] : -s_w[j];
      }
#pragma unroll
      for (int p = 0; p < kAdjParams; ++p) q[p] = c * S * xd[p];
    }
#pragma unroll
    for (int p = 0; p < kAdjParams; ++p) {
      T v = q[p];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0) acc[warp][p] += (double)v;
    }
  }
  __syncthreads();
  double* ws = static_cast<double*>(a.workspace);
  for (int p = threadIdx.x; p < kAdjParams; p += kBlock) {
    double s = 0.0;
    for (int w = 0; w < kBlock / 32; ++w) s += acc[w][p];
    ws[(size_t)blockIdx.x * kAdjParams + p] = s;
  }
}

template <typename T, int SRC>
int adjoint_grid(int64_t n, size_t smem) {
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, heston_adjoint_kernel<T, SRC>, kBlock, smem);
  if (occ < 1) occ = 1;
  int64_t g = (n + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

template <typename T>
int run_adjoint(const tqf_heston_adjoint_args& a, cudaStream_t s) {
  const size_t smem = (size_t)a.num_strikes * (2 * sizeof(T) + 1) + 16;
  const bool philox = a.draws.source == TQF_DRAWS_PHILOX;
  const int grid = philox ? adjoint_grid<T, TQF_DRAWS_PHILOX>(a.num_paths, smem)
                          : adjoint_grid<T, TQF_DRAWS_MEMORY>(a.num_paths, smem);
  const size_t need = (size_t)grid * kAdjParams * sizeof(double);
  TQF_REQUIRE(a.workspace && a.workspace_bytes >= need, "tqf_heston_euler_adjoint: workspace %zu < %zu",
              a.workspace_bytes, need);
  if (philox)
    heston_adjoint_kernel<T, TQF_DRAWS_PHILOX><<<grid, kBlock, smem, s>>>(a);
  else
    heston_adjoint_kernel<T, TQF_DRAWS_MEMORY><<<grid, kBlock, smem, s>>>(a);
  int rc = check_launch("heston_adjoint_kernel");
  if (rc) return rc;
  return reduce_partials(static_cast<const double*>(a.workspace), grid, kAdjParams, a.out, s);
}

template <typename T, int SCHEME>
using KernelFn = void (*)(tqf_heston_args, int, SmemLayout);

template <typename T, int SCHEME, int SRC, bool ANTI>
KernelFn<T, SCHEME> pick(bool store, bool price) {
  if (store && price) return heston_kernel<T, SCHEME, SRC, true, true, ANTI>;
  if (store) return heston_kernel<T, SCHEME, SRC, true, false, ANTI>;
  if (price) return heston_kernel<T, SCHEME, SRC, false, true, ANTI>;
  return heston_kernel<T, SCHEME, SRC, false, false, ANTI>;
}

template <typename T, int SCHEME>
KernelFn<T, SCHEME> pick_kernel(int src, bool store, bool price, bool anti = false) {
  if (src == TQF_DRAWS_SOBOL) return pick<T, SCHEME, TQF_DRAWS_SOBOL, false>(store, price);
  if (src != TQF_DRAWS_PHILOX) return pick<T, SCHEME, TQF_DRAWS_MEMORY, false>(store, price);
  return anti ? pick<T, SCHEME, TQF_DRAWS_PHILOX, true>(store, price)
              : pick<T, SCHEME, TQF_DRAWS_PHILOX, false>(store, price);
}

// cuCtxGetId through the runtime's driver entry-point query, so the library
// needs no link against libcuda.  nullptr when the driver lacks it.
using CtxGetIdFn = int (*)(void* ctx, unsigned long long* id);
CtxGetIdFn ctx_get_id_fn() {
  static CtxGetIdFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    cudaGetLastError();
    return reinterpret_cast<CtxGetIdFn>(p);
  }();
  return fn;
}

template <typename T, int SCHEME>
int grid_for(int64_t N, int ns, int steps, bool staged, int src, bool store, bool price,
             SmemLayout* out_layout, bool anti = false) {
  const int cols = SCHEME == 0 ? kFtCols : kQeCols;
  SmemLayout L = smem_layout<T>(steps, cols, price ? ns : 0, staged, store, src == TQF_DRAWS_SOBOL);
  if (out_layout) *out_layout = L;
  // The kernel attributes and the occupancy query are driver calls that a
  // pricing call would otherwise repeat (twice: workspace size, launch); the
  // result is kept per context (a reset context needs the attributes again).
  struct Key {
    unsigned long long ctx;
    int64_t N;
    int ns, steps, src;
    bool staged, store, price, anti;
  };
  static std::mutex mu;
  static std::vector<std::pair<Key, int>> cache;
  unsigned long long ctx = 0;
  const CtxGetIdFn get_id = ctx_get_id_fn();
  const bool have_ctx = get_id != nullptr && get_id(nullptr, &ctx) == 0;
  const Key key{ctx, N, ns, steps, src, staged, store, price, anti};
  auto same = [&](const Key& k) {
    return k.ctx == key.ctx && k.N == key.N && k.ns == key.ns && k.steps == key.steps && k.src == key.src &&
           k.staged == key.staged && k.store == key.store && k.price == key.price && k.anti == key.anti;
  };
  if (have_ctx) {
    std::lock_guard<std::mutex> lock(mu);
    for (const auto& e : cache)
      if (same(e.first)) return e.second;
  }
  auto k = pick_kernel<T, SCHEME>(src, store, price, anti);
  set_smem_config(k, L.total);
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kBlock, L.total) != cudaSuccess ||
      occ < 1)
    occ = 1;
  int64_t blocks = (N + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * occ;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (have_ctx) {
    std::lock_guard<std::mutex> lock(mu);
    if (cache.size() >= 256) cache.erase(cache.begin());
    cache.push_back({key, (int)blocks});
  }
  return (int)blocks;
}

bool table_staged(const void* table, int steps, int cols, size_t elt) {
  const size_t bytes = (size_t)steps * cols * elt;
  return bytes > 0 && bytes <= kMaxStagedTable && (reinterpret_cast<uintptr_t>(table) & 15u) == 0;
}

template <typename T, int SCHEME>
int run(const tqf_heston_args& a, cudaStream_t s) {
  const int cols = SCHEME == 0 ? kFtCols : kQeCols;
  const bool store = a.output.ptr != nullptr;
  const bool price = a.payoff.num_strikes > 0;
  const bool staged = table_staged(a.step_table, a.num_steps, cols, sizeof(T));
  SmemLayout L;
  const int grid = grid_for<T, SCHEME>(a.num_paths, a.payoff.num_strikes, a.num_steps, staged,
                                       a.draws.source, store, price, &L, a.draws.antithetic != 0);
  if (price) {
    const size_t need = (size_t)grid * a.payoff.num_strikes * 2 * sizeof(double);
    TQF_REQUIRE(a.payoff.workspace && a.payoff.workspace_bytes >= need,
                "heston: payoff workspace %zu bytes < required %zu", a.payoff.workspace_bytes, need);
  }
  auto k = pick_kernel<T, SCHEME>(a.draws.source, store, price, a.draws.antithetic != 0);
  k<<<grid, kBlock, L.total, s>>>(a, staged ? 1 : 0, L);
  int rc = check_launch(SCHEME == 0 ? "heston_kernel<FT>" : "heston_kernel<QE>");
  if (rc || !price || a.payoff.out == nullptr) return rc;
  return reduce_partials(static_cast<const double*>(a.payoff.workspace), grid,
                         2 * a.payoff.num_strikes, a.payoff.out, s);
}

int validate(const tqf_heston_args* a, const char* who) {
  TQF_REQUIRE(a != nullptr, "%s: null args", who);
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "%s: bad dtype %d", who, a->dtype);
  TQF_REQUIRE(a->num_paths >= 1, "%s: num_paths must be >= 1", who);
  TQF_REQUIRE(a->num_steps >= 0, "%s: num_steps must be >= 0", who);
  TQF_REQUIRE(a->num_steps == 0 || a->step_table != nullptr, "%s: null step_table", who);
  TQF_REQUIRE((reinterpret_cast<uintptr_t>(a->step_table) & 15u) == 0, "%s: step_table must be 16-byte aligned", who);
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.source == TQF_DRAWS_MEMORY ||
                  a->draws.source == TQF_DRAWS_SOBOL,
              "%s: bad draws.source %d", who, a->draws.source);
  if (a->draws.source == TQF_DRAWS_SOBOL) {
    TQF_REQUIRE(a->draws.ptr != nullptr, "%s: Sobol draws need the direction numbers in draws.ptr", who);
    TQF_REQUIRE(a->draws.key1 == 2, "%s: Sobol draws need key1 = 2 normals per step, got %u", who, a->draws.key1);
    TQF_REQUIRE(a->draws.key0 >= 1 && a->draws.key0 <= 32, "%s: Sobol nd (key0) must be in [1, 32]", who);
    TQF_REQUIRE(!a->draws.antithetic, "%s: Sobol draws have no antithetic form", who);
    TQF_REQUIRE(a->draws.path_offset >= 0 && a->draws.path_offset + a->num_paths <= 2147483647LL,
                "%s: Sobol point indices must stay below 2^31", who);
    TQF_REQUIRE(a->draws.path_offset + a->num_paths < (1LL << a->draws.key0),
                "%s: Sobol point indices must fit in nd = %u digits", who, a->draws.key0);
  }
  TQF_REQUIRE(a->draws.source != TQF_DRAWS_MEMORY || a->num_steps == 0 || a->draws.ptr != nullptr,
              "%s: memory draws need draws.ptr", who);
  TQF_REQUIRE(!a->draws.antithetic || 2 * a->draws.antithetic_half == a->num_paths,
              "%s: antithetic needs num_paths == 2 * antithetic_half", who);
  if (a->output.ptr) {
    TQF_REQUIRE(a->output.num_slots >= 1, "%s: output.num_slots must be >= 1", who);
    TQF_REQUIRE(a->output.init_slot < a->output.num_slots, "%s: init_slot out of range", who);
  }
  TQF_REQUIRE(a->payoff.num_strikes >= 0 && a->payoff.num_strikes <= 1024,
              "%s: num_strikes must be in [0, 1024]", who);
  TQF_REQUIRE(a->payoff.num_strikes == 0 || a->payoff.strikes, "%s: payoff needs strikes", who);
  return TQF_OK;
}

// ---- allocation-free pricing variant ------------------------------------------
// For callers that cannot call cudaMalloc (see tqf_heston_euler_price_noalloc
// in tqf.h): the per-CTA partial sums live in this file-scope device array
// instead of a caller workspace.  2 MiB = 2048 CTAs x 64 strikes x (sum, sum
// of squares); every GPU that loads the library holds it until exit.
constexpr int kNoAllocMaxStrikes = 64;
constexpr size_t kNoAllocDoubles = (size_t)2048 * kNoAllocMaxStrikes * 2;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocDoubles];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
struct NoAllocSlot {
  unsigned long long ctx_id;  // id of the context the address belongs to
  double* ptr;
};
NoAllocSlot g_noalloc_slot[kNoAllocMaxDevices] = {};


// Device address of g_noalloc_partials in the current device's context (the
// host-side symbol is only a stand-in, never a device pointer).  The address
// is looked up on the first call in each context and kept with that
// context's unique id: after a cudaDeviceReset the runtime makes a new
// primary context, the module loads again at another address, and the next
// call sees a new id and looks the address up again.  Without cuCtxGetId
// (drivers older than CUDA 12) it is looked up on every call.
int noalloc_scratch(double** out) {
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "tqf_heston_euler_price_noalloc: cudaGetDevice");
  if (rc) return rc;
  TQF_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "tqf_heston_euler_price_noalloc: device %d out of range", dev);
  // cudaSetDevice initialises the device's primary context (again, after a
  // reset), so the id read next is the context the kernels will run in.
  rc = check_cuda(cudaSetDevice(dev), "tqf_heston_euler_price_noalloc: cudaSetDevice");
  if (rc) return rc;
  unsigned long long id = 0;
  const CtxGetIdFn get_id = ctx_get_id_fn();
  const bool have_id = get_id != nullptr && get_id(nullptr, &id) == 0;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocSlot& slot = g_noalloc_slot[dev];
  if (!have_id || slot.ptr == nullptr || slot.ctx_id != id) {
    void* p = nullptr;
    rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_partials),
                    "tqf_heston_euler_price_noalloc: cudaGetSymbolAddress");
    if (rc) return rc;
    slot.ptr = static_cast<double*>(p);
    slot.ctx_id = id;
  }
  *out = slot.ptr;
  return TQF_OK;
}

template <typename T>
int run_noalloc(const tqf_heston_args& a, double* scratch, cudaStream_t s) {
  const bool store = a.output.ptr != nullptr;
  const bool staged = table_staged(a.step_table, a.num_steps, kFtCols, sizeof(T));
  SmemLayout L;
  int grid = grid_for<T, 0>(a.num_paths, a.payoff.num_strikes, a.num_steps, staged, a.draws.source, store,
                            true, &L, a.draws.antithetic != 0);
  // The CTA loop is persistent, so a smaller grid still covers every path.
  const int cap = (int)(kNoAllocDoubles / (2 * (size_t)a.payoff.num_strikes));
  if (grid > cap) grid = cap;
  tqf_heston_args b = a;
  b.payoff.workspace = scratch;
  b.payoff.workspace_bytes = kNoAllocDoubles * sizeof(double);
  auto k = pick_kernel<T, 0>(b.draws.source, store, true, b.draws.antithetic != 0);
  k<<<grid, kBlock, L.total, s>>>(b, staged ? 1 : 0, L);
  int rc = check_launch("heston_kernel<FT> (no-alloc)");
  if (rc) return rc;
  return reduce_partials(scratch, grid, 2 * b.payoff.num_strikes, b.payoff.out, s);
}

}  // namespace
}  // namespace tqf

using namespace tqf;

extern "C" int tqf_heston_euler(const tqf_heston_args* a, void* stream) {
  clear_error();
  int rc = validate(a, "tqf_heston_euler");
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? run<float, 0>(*a, s) : run<double, 0>(*a, s);
}

extern "C" int tqf_heston_euler_price_noalloc(const tqf_heston_args* a, void* stream) {
  clear_error();
  int rc = validate(a, "tqf_heston_euler_price_noalloc");
  if (rc) return rc;
  TQF_REQUIRE(a->payoff.num_strikes >= 1 && a->payoff.num_strikes <= kNoAllocMaxStrikes,
              "tqf_heston_euler_price_noalloc: num_strikes must be in [1, %d], got %d", kNoAllocMaxStrikes,
              a->payoff.num_strikes);
  TQF_REQUIRE(a->payoff.out != nullptr, "tqf_heston_euler_price_noalloc: payoff.out is required");
  double* scratch = nullptr;
  rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? run_noalloc<float>(*a, scratch, s) : run_noalloc<double>(*a, scratch, s);
}

extern "C" int tqf_heston_qe(const tqf_heston_args* a, void* stream) {
  clear_error();
  int rc = validate(a, "tqf_heston_qe");
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? run<float, 1>(*a, s) : run<double, 1>(*a, s);
}

extern "C" int tqf_heston_euler_adjoint(const tqf_heston_adjoint_args* a, void* stream) {
  clear_error();
  TQF_REQUIRE(a != nullptr, "tqf_heston_euler_adjoint: null args");
  TQF_REQUIRE(a->dtype == TQF_F32 || a->dtype == TQF_F64, "tqf_heston_euler_adjoint: bad dtype");
  TQF_REQUIRE(a->num_paths >= 1 && a->num_steps >= 1, "tqf_heston_euler_adjoint: bad sizes");
  TQF_REQUIRE(a->step_table && a->strikes && a->weights && a->out, "tqf_heston_euler_adjoint: null pointer");
  TQF_REQUIRE(a->num_strikes >= 1 && a->num_strikes <= 4096, "tqf_heston_euler_adjoint: bad num_strikes");
  TQF_REQUIRE(a->rho > -1.0 && a->rho < 1.0, "tqf_heston_euler_adjoint: rho must be in (-1, 1)");
  TQF_REQUIRE(a->draws.source == TQF_DRAWS_PHILOX || a->draws.ptr, "tqf_heston_euler_adjoint: memory draws need ptr");
  TQF_REQUIRE(!a->draws.antithetic || 2 * a->draws.antithetic_half == a->num_paths,
              "tqf_heston_euler_adjoint: antithetic needs num_paths == 2 * antithetic_half");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a->dtype == TQF_F32 ? run_adjoint<float>(*a, s) : run_adjoint<double>(*a, s);
}

extern "C" size_t tqf_heston_adjoint_workspace_bytes(int64_t num_paths) {
  int64_t g = (num_paths + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)num_sms() * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (size_t)g * kAdjParams * sizeof(double);
}

extern "C" size_t tqf_heston_workspace_bytes(int32_t dtype, int32_t qe, int64_t num_paths,
                                             int32_t num_strikes) {
  if (num_strikes <= 0) return 0;
  // The grid does not depend on the step count or staging beyond smem size;
  // use the largest layout (unstaged table is smaller, so occupancy >=).
  int grid;
  if (dtype == TQF_F32)
    grid = qe ? grid_for<float, 1>(num_paths, num_strikes, 0, false, TQF_DRAWS_PHILOX, false, true, nullptr)
              : grid_for<float, 0>(num_paths, num_strikes, 0, false, TQF_DRAWS_PHILOX, false, true, nullptr);
  else
    grid = qe ? grid_for<double, 1>(num_paths, num_strikes, 0, false, TQF_DRAWS_PHILOX, false, true, nullptr)
              : grid_for<double, 0>(num_paths, num_strikes, 0, false, TQF_DRAWS_PHILOX, false, true, nullptr);
  // Occupancy may differ between kernel variants; size for the largest
  // possible grid (all SMs x the maximum resident CTAs of 256 threads).
  int64_t cap = (int64_t)num_sms() * 8;
  int64_t blocks = (num_paths + kBlock - 1) / kBlock;
  if (blocks > cap) blocks = cap;
  if (blocks < grid) blocks = grid;
  return (size_t)blocks * num_strikes * 2 * sizeof(double);
}
