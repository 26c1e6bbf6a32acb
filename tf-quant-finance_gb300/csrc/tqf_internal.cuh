// Internal helpers shared by the tqf CUDA translation units: error state,
// launch accounting, Philox4x32-10, Box–Muller, TMA bulk staging with bounded
// mbarrier waits, and the FP64 payoff accumulator used by the path kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tqf.h"

namespace tqf {

// ---- host-side error state ----------------------------------------------
void set_error(const char* fmt, ...);
void clear_error();
int check_cuda(cudaError_t e, const char* where);
void note_launch(uint64_t n = 1);
int num_sms();
// Checks the launch just issued; returns TQF_OK or TQF_E_CUDA.
int check_launch(const char* kernel_name);

#define TQF_REQUIRE(cond, ...)        \
  do {                                \
    if (!(cond)) {                    \
      ::tqf::set_error(__VA_ARGS__);  \
      return TQF_E_INVALID;           \
    }                                 \
  } while (0)

// Opts a kernel into `smem` bytes of dynamic shared memory and the maximum
// shared-memory carveout, so that occupancy queries (and launches) see the
// full shared-memory configuration.
template <typename K>
inline void set_smem_config(K kernel, size_t smem) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start before the previous kernel in the stream has
// finished; grid_dependency_wait() blocks until that kernel has completed and
// its memory is visible (a no-op for an ordinary launch), and
// allow_dependent_launch() lets the next such kernel start launching.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_dependent_launch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch configuration of a programmatic dependent launch on `stream`
// (attr is filled in and must outlive the launch call).
inline cudaLaunchConfig_t pdl_config(dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                                     cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  attr->id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr->val.programmaticStreamSerializationAllowed = 1;
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -------------------
// Ten rounds of the published round function; the key is bumped by the
// Weyl constants between rounds.
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

__host__ __device__ __forceinline__ void mulhilo32(uint32_t a, uint32_t b,
                                                   uint32_t& hi, uint32_t& lo) {
#ifdef __CUDA_ARCH__
  const uint64_t p = (uint64_t)a * (uint64_t)b;  // one 32x32->64 wide multiply
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
#else
  uint64_t p = (uint64_t)a * (uint64_t)b;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
#endif
}

__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0,
                                                        uint32_t k1) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(kPhiloxM0, c.x, hi0, lo0);
    mulhilo32(kPhiloxM1, c.z, hi1, lo1);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += kPhiloxW0;
    k1 += kPhiloxW1;
  }
  return c;
}

// Counter of the canonical normal stream: block b of path n.
__device__ __forceinline__ uint4 philox_counter(int64_t block, int64_t path) {
  return make_uint4((uint32_t)block, (uint32_t)path,
                    (uint32_t)((uint64_t)path >> 32), (uint32_t)((uint64_t)block >> 32));
}

// ---- uniform -> normal (Box–Muller) ---------------------------------------
// float32: u1 in (0, 1] with 2^-32 resolution assembled from the 32 random
// bits through two exponent-trick conversions (no integer->float convert),
// u2 in [0, 1) with 2^-23 resolution for the angle.
__device__ __forceinline__ float u01_oc_f32(uint32_t r) {
  float hi = __uint_as_float(0x3f800000u | (r >> 9));          // [1, 2)
  float lo = __uint_as_float(0x3f800000u | (r << 23 >> 9)) - 1.0f; // [0, 1), low 9 bits
  // (2 - hi) in {2^-23, ..., 1}; subtract lo * 2^-23 for the low bits.
  return __fmaf_rn(lo, -1.1920928955078125e-07f, 2.0f - hi);
}
__device__ __forceinline__ float u01_co_f32(uint32_t r) {
  return __uint_as_float(0x3f800000u | (r >> 9)) - 1.0f;
}

// Single-instruction SFU square root (relative error ~2^-23; no IEEE rounding).
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ double sqrt_approx(double x) { return sqrt(x); }

// Flush-to-zero SFU forms: the same approximations as __log2f / __sincosf
// on normal inputs, without the subnormal handling around them.
__device__ __forceinline__ float lg2_ftz(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ void sincos_ftz(float x, float& s, float& c) {
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"(x));
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(c) : "f"(x));
}

// Two N(0,1) from two 32-bit words (radius from a, angle from b).  Uses the
// SFU approximations (lg2, sqrt, sin, cos); the angle is taken in [-pi, pi)
// where the hardware sin/cos are accurate.  All SFU inputs are normal numbers
// (u1 >= 2^-32; the angle is 0 or at least 2 pi 2^-23 in magnitude), so the
// flush-to-zero forms change nothing.
__device__ __forceinline__ void box_muller_f32(uint32_t a, uint32_t b, float& z0,
                                               float& z1) {
  const float u1 = u01_oc_f32(a);
  const float u2 = u01_co_f32(b);
  const float rad = sqrt_approx(__fmul_rn(-1.3862943611198906f, lg2_ftz(u1)));  // sqrt(-2 ln u1)
  const float ang = __fmul_rn(__fsub_rn(u2, 0.5f), 6.283185307179586f);
  float s, c;
  sincos_ftz(ang, s, c);
  z0 = __fmul_rn(rad, c);
  z1 = __fmul_rn(rad, s);
}

// float64: 53-bit uniforms from word pairs.
__device__ __forceinline__ double u01_oc_f64(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);  // 53 bits
  return ((double)m + 1.0) * 1.1102230246251565e-16;       // (m+1) * 2^-53
}
__device__ __forceinline__ double u01_co_f64(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
  return (double)m * 1.1102230246251565e-16;
}
__device__ __forceinline__ void box_muller_f64(uint4 r, double& z0, double& z1) {
  const double u1 = u01_oc_f64(r.x, r.y);
  const double u2 = u01_co_f64(r.z, r.w);
  const double rad = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  z0 = rad * c;
  z1 = rad * s;
}

// ---- packed FP32 pairs ------------------------------------------------------
// sm_100-family f32x2 arithmetic: one issued instruction does the two lanes'
// work, each lane rounded exactly as the scalar .rn operation would be.
__device__ __forceinline__ uint64_t f2_bits(float2 a) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 f2_from_bits(uint64_t r) {
  float2 v;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
  return v;
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from_bits(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  uint64_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from_bits(d);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)), "l"(f2_bits(c)));
  return f2_from_bits(d);
}
// The four normals of one Philox block as two pairs, even = (z0, z2) and
// odd = (z1, z3), with (z0, z1) from words (x, y) and (z2, z3) from (z, w):
// the arithmetic of box_muller_f32 run on both halves at once in f32x2
// instructions.  Every input of the flush-to-zero SFU forms is a normal
// number (u1 >= 2^-32; the angle is 0 or at least 2 pi 2^-23 in magnitude),
// so the results equal box_muller_f32's bit for bit.
__device__ __forceinline__ void box_muller_pair_f32(uint4 r, float2& even, float2& odd) {
  const float2 hi = make_float2(__uint_as_float(0x3f800000u | (r.x >> 9)), __uint_as_float(0x3f800000u | (r.z >> 9)));
  const float2 lo = make_float2(__uint_as_float(0x3f800000u | (r.x << 23 >> 9)),
                                __uint_as_float(0x3f800000u | (r.z << 23 >> 9)));
  const float2 two_minus_hi = fma2(hi, make_float2(-1.f, -1.f), make_float2(2.f, 2.f));  // 2 - hi, exact product
  const float2 u1 = fma2(add2(lo, make_float2(-1.f, -1.f)), make_float2(-1.1920928955078125e-07f, -1.1920928955078125e-07f),
                         two_minus_hi);
  const float2 m = mul2(make_float2(-1.3862943611198906f, -1.3862943611198906f), make_float2(lg2_ftz(u1.x), lg2_ftz(u1.y)));
  const float2 rad = make_float2(sqrt_approx(m.x), sqrt_approx(m.y));
  const float2 u2 = add2(make_float2(__uint_as_float(0x3f800000u | (r.y >> 9)), __uint_as_float(0x3f800000u | (r.w >> 9))),
                         make_float2(-1.f, -1.f));
  const float2 ang = mul2(add2(u2, make_float2(-0.5f, -0.5f)), make_float2(6.283185307179586f, 6.283185307179586f));
  float2 s, c;
  sincos_ftz(ang.x, s.x, c.x);
  sincos_ftz(ang.y, s.y, c.y);
  even = mul2(rad, c);
  odd = mul2(rad, s);
}

// ---- full-truncation Heston steps in pairs ---------------------------------
// Block p of the two-step layout of a float FT table [steps][8] with rows
// (dt/2, sqrt dt, r dt, kappa dt, kappa theta dt, xi rho, xi sqrt(1-rho^2),
// slot): for steps a = 2p, b = 2p + 1 the 16 floats
//   (-hdt_a, -kdt_a, rdt_a, kthdt_a), (-hdt_b, -kdt_b, rdt_b, kthdt_b),
//   (sdt_a, sdt_b, xirho_a, xirho_b), (xisq_a, xisq_b, slot_a, slot_b),
// so that a loop taking both steps of a Philox block reads its constants as
// f32x2 operands with four 16-byte loads.  An odd last step pairs with a
// zero step whose slot is -1.  All reads happen before the caller writes.
__device__ __forceinline__ void ft_pair_block(const float* rows, int steps, int p, float4 q[4]) {
  const float4* r = reinterpret_cast<const float4*>(rows + 16 * p);
  const float4 a0 = r[0], a1 = r[1];
  float4 b0 = make_float4(0.f, 0.f, 0.f, 0.f), b1 = make_float4(0.f, 0.f, 0.f, -1.f);
  if (2 * p + 1 < steps) {
    b0 = r[2];
    b1 = r[3];
  }
  q[0] = make_float4(-a0.x, -a0.w, a0.z, a1.x);
  q[1] = make_float4(-b0.x, -b0.w, b0.z, b1.x);
  q[2] = make_float4(a0.y, b0.y, a1.y, b1.y);
  q[3] = make_float4(a1.z, b1.z, a1.w, b1.w);
}

// Increments of both steps of a block: dw0 = z_even sqrt dt, dw1 = z_odd
// sqrt dt and e = xi rho dw0 + xi sqrt(1 - rho^2) dw1, each as a pair
// (step a, step b); qs, qx are the block's third and fourth float4.
__device__ __forceinline__ void ft_pair_increments(float2 ze, float2 zo, float4 qs, float4 qx, float2& dw0,
                                                   float2& e) {
  const float2 sdt = make_float2(qs.x, qs.y);
  dw0 = mul2(ze, sdt);
  const float2 dw1 = mul2(zo, sdt);
  e = fma2(make_float2(qx.x, qx.y), dw1, mul2(make_float2(qs.z, qs.w), dw0));
}

// One full-truncation step from a block's half q = (-hdt, -kdt, rdt, kthdt),
// the step's dw0 and e: the scalar step's arithmetic, with the two drift
// sums in one f32x2 add.
__device__ __forceinline__ void ft_half_step(const float4 q, float dw0, float e, float& x, float& v) {
  const float vp = fmaxf(v, 0.f);
  const float sq = sqrt_approx(vp);
  const float2 u = add2(make_float2(x, v), make_float2(fmaf(q.x, vp, q.z), fmaf(q.y, vp, q.w)));
  x = fmaf(sq, dw0, u.x);
  v = fmaf(sq, e, u.y);
}

// ---- coalesced output of recorded path states ---------------------------------
// A CTA of THREADS paths records w <= W values per recorded slot into output
// rows out[path][slot][w].  Each recorded step a thread puts its w values
// into the next w rows of a [S w][THREADS + 1] shared-memory buffer (S slots
// ~ 128 bytes of a path's row); when the buffer is full, or the next slot
// does not continue the buffered run, the CTA writes the run out with
// consecutive threads on consecutive values of one path, so each warp stores
// whole pieces of output rows instead of 32 scattered ones (the padded row
// stride keeps the shared-memory reads conflict-free; the value -> (path,
// offset) walk is incremental, one division per flush).  put() and flush()
// are CTA barriers: every thread of the CTA calls them at the same steps (the
// slots come from a table shared by the CTA), including threads whose path
// is past the end (their values are dropped).
template <typename T, int W, int THREADS>
struct RowStager {
  static constexpr int kRowValues = 128 / (int)sizeof(T);
  static constexpr int kMaxPerPath = W > kRowValues ? W : kRowValues;
  static constexpr size_t kBytes = (size_t)kMaxPerPath * (THREADS + 1) * sizeof(T);
  T* buf;
  int w, S, cnt, slot0;
  __device__ RowStager(void* smem, int width)
      : buf(static_cast<T*>(smem)), w(width), S(kRowValues / width > 0 ? kRowValues / width : 1), cnt(0),
        slot0(0) {}
  __device__ __forceinline__ void put(T* out, int num_slots, int64_t row0, int64_t N, int slot, const T* x) {
    if (cnt > 0 && (cnt == S || slot != slot0 + cnt)) flush(out, num_slots, row0, N);
    if (cnt == 0) slot0 = slot;
#pragma unroll
    for (int c = 0; c < W; ++c)
      if (c < w) buf[(cnt * w + c) * (THREADS + 1) + threadIdx.x] = x[c];
    ++cnt;
  }
  __device__ __forceinline__ void flush(T* out, int num_slots, int64_t row0, int64_t N) {
    __syncthreads();
    const int per = cnt * w;  // values of one path in this run
    const int dq = THREADS / per, dr = THREADS - dq * per;
    int p = threadIdx.x / per, e = threadIdx.x - p * per;
    for (int idx = threadIdx.x; idx < per * THREADS; idx += THREADS) {
      if (row0 + p < N) out[((row0 + p) * num_slots + slot0) * w + e] = buf[e * (THREADS + 1) + p];
      p += dq;
      e += dr;
      if (e >= per) {
        e -= per;
        ++p;
      }
    }
    __syncthreads();
    cnt = 0;
  }
};

// Four float normals of block b for path n: draw dims 4b..4b+3 (the two
// Box–Muller pairs in f32x2 form, equal to box_muller_f32 on each pair).
__device__ __forceinline__ void philox_normals4_f32(int64_t block, int64_t path,
                                                    uint32_t k0, uint32_t k1,
                                                    float z[4]) {
  uint4 r = philox4x32_10(philox_counter(block, path), k0, k1);
  float2 ze, zo;
  box_muller_pair_f32(r, ze, zo);
  z[0] = ze.x;
  z[1] = zo.x;
  z[2] = ze.y;
  z[3] = zo.y;
}
// Two double normals of block b: draw dims 2b, 2b+1.
__device__ __forceinline__ void philox_normals2_f64(int64_t block, int64_t path,
                                                    uint32_t k0, uint32_t k1,
                                                    double z[2]) {
  uint4 r = philox4x32_10(philox_counter(block, path), k0, k1);
  box_muller_f64(r, z[0], z[1]);
}

template <typename T>
struct NormalsPerBlock;
template <>
struct NormalsPerBlock<float> {
  static constexpr int value = 4;
};
template <>
struct NormalsPerBlock<double> {
  static constexpr int value = 2;
};

// Sequential reader of the canonical stream for one path: get(k) for
// non-decreasing k regenerates a block only when k leaves it.  Register-only
// (selects instead of a dynamically indexed array).
template <typename T>
struct PhiloxReader;

template <>
struct PhiloxReader<float> {
  int64_t path;
  uint32_t k0, k1;
  int64_t blk;
  float z0, z1, z2, z3;
  __device__ __forceinline__ PhiloxReader(int64_t p, uint32_t a, uint32_t b)
      : path(p), k0(a), k1(b), blk(-1), z0(0), z1(0), z2(0), z3(0) {}
  __device__ __forceinline__ float get(int64_t k) {
    const int64_t b = k >> 2;
    if (b != blk) {
      float z[4];
      philox_normals4_f32(b, path, k0, k1, z);
      z0 = z[0]; z1 = z[1]; z2 = z[2]; z3 = z[3];
      blk = b;
    }
    const int l = (int)(k & 3);
    return l == 0 ? z0 : (l == 1 ? z1 : (l == 2 ? z2 : z3));
  }
};

template <>
struct PhiloxReader<double> {
  int64_t path;
  uint32_t k0, k1;
  int64_t blk;
  double z0, z1;
  __device__ __forceinline__ PhiloxReader(int64_t p, uint32_t a, uint32_t b)
      : path(p), k0(a), k1(b), blk(-1), z0(0), z1(0) {}
  __device__ __forceinline__ double get(int64_t k) {
    const int64_t b = k >> 1;
    if (b != blk) {
      double z[2];
      philox_normals2_f64(b, path, k0, k1, z);
      z0 = z[0]; z1 = z[1];
      blk = b;
    }
    return (k & 1) ? z1 : z0;
  }
};

__device__ __forceinline__ void philox_normals(int64_t block, int64_t path, uint32_t k0, uint32_t k1, float* z) {
  philox_normals4_f32(block, path, k0, k1, z);
}
__device__ __forceinline__ void philox_normals(int64_t block, int64_t path, uint32_t k0, uint32_t k1, double* z) {
  philox_normals2_f64(block, path, k0, k1, z);
}

constexpr int gcd_int(int a, int b) { return b == 0 ? a : gcd_int(b, a % b); }

// Whole-block walk of the canonical stream for steps of exactly DM draws
// each (draw k = step DM + c): a group of kSteps steps takes kNormals =
// lcm(DM, normals per block) draws, i.e. exactly kBlocks whole Philox
// blocks, so a loop over groups needs no per-draw block test or lane select.
// Group g holds steps g kSteps .. g kSteps + kSteps - 1 and blocks g kBlocks
// .. g kBlocks + kBlocks - 1; a last partial group is generated whole and
// its tail dropped, as the stream is the same either way.
template <typename T, int DM>
struct PhiloxGroup {
  static constexpr int kNpb = NormalsPerBlock<T>::value;
  static constexpr int kNormals = DM / gcd_int(DM, kNpb) * kNpb;
  static constexpr int kSteps = kNormals / DM;
  static constexpr int kBlocks = kNormals / kNpb;
  // Generates the blocks that begin within step s of the group (z holds the
  // group's kNormals draws), so that each block is made just before its
  // first use.
  __device__ __forceinline__ static void fill_step(int64_t group, int s, int64_t path, uint32_t k0, uint32_t k1,
                                                   T* z) {
#pragma unroll
    for (int c = 0; c < DM; ++c) {
      const int q = s * DM + c;
      if (q % kNpb == 0) philox_normals(group * kBlocks + q / kNpb, path, k0, k1, z + q);
    }
  }
};

// dt and sqrt(dt) of a step-table row [dt, sqrt dt, slot, -] with one
// vector load (the row aligned to two values); GLOBAL reads through the
// read-only path.
template <bool GLOBAL>
__device__ __forceinline__ void step_pair(const float* row, float& dt, float& sdt) {
  const float2 v = GLOBAL ? __ldg(reinterpret_cast<const float2*>(row)) : *reinterpret_cast<const float2*>(row);
  dt = v.x;
  sdt = v.y;
}
template <bool GLOBAL>
__device__ __forceinline__ void step_pair(const double* row, double& dt, double& sdt) {
  const double2 v = GLOBAL ? __ldg(reinterpret_cast<const double2*>(row)) : *reinterpret_cast<const double2*>(row);
  dt = v.x;
  sdt = v.y;
}

// ---- Sobol normals ------------------------------------------------------------
// Inverse-normal conversion of a Sobol integer x at nd digits:
// u = float(x) 2^-nd, z = sqrt(2) erfinv((u - 1/2) 2)
// (tff/math/random_ops/multivariate_normal.py:420).  In float32,
// (u - 1/2) 2 = fma(float(x), 2^(1-nd), -1) exactly: the product is a power-
// of-two scaling (exact) and scaling by 2 commutes with rounding, so the one
// rounding of the fma equals the reference's rounding of u - 1/2, doubled.
// sc2 = 2^(1-nd) (float32), sc = 2^-nd (float64).  The Sobol kernels and the
// fused Sobol draws of the path kernels share these, so materialised and
// fused draws agree bit for bit.
__device__ __forceinline__ float sobol_normal_f32(uint32_t x, float sc2) {
  return __fmul_rn(erfinvf(fmaf(__uint2float_rn(x), sc2, -1.0f)), 1.41421353816986083984375f);
}
__device__ __forceinline__ double sobol_normal_f64(uint32_t x, double sc) {
  const double u = __dmul_rn((double)x, sc);
  return __dmul_rn(erfinv(__dmul_rn(__dsub_rn(u, 0.5), 2.0)), 1.4142135623730951);
}
__device__ __forceinline__ float sobol_normal(uint32_t x, float sc) { return sobol_normal_f32(x, sc); }
__device__ __forceinline__ double sobol_normal(uint32_t x, double sc) { return sobol_normal_f64(x, sc); }

// Sobol integers of a CTA's tile of 256 consecutive point indices, for a
// window of draw dimensions, from shared-memory tables.  Point i's integer in
// dimension k is XOR_j bit_j(i) v_kj >> (32 - nd) (sobol_impl.py:128-157);
// split i into bits 0-3, 4-7 and the rest: row k of the tables holds
//   [0, 16):  XOR of v_kj, j in 0..3, over the set bits of each 4-bit value,
//   [16, 32): the same for j in 4..7,
//   32, 33:   the XOR over bits >= 8 of the two 256-blocks the tile touches
// (its indices i0 .. i0 + 255 span at most two), so a thread reads three
// words per draw: T[lo4] ^ T[16 + mid4] ^ T[32 + block].  Within a warp
// the lo4 reads hit 16 consecutive words and the other two at most three
// distinct words, so the reads are conflict-free.  The tables of a window
// are rebuilt per tile (the high part depends on it); the build is ~2 jobs
// per thread per window, against ~100 instructions per path-step.
struct SobolTables {
  static constexpr int kRow = 34;
  // cooperative build of dimensions k0 .. k0 + nk - 1; the caller brackets it
  // with __syncthreads (tables of the previous window may still be in use)
  static __device__ __forceinline__ void build(uint32_t* tabs, const uint32_t* __restrict__ v, int k0, int nk,
                                               uint32_t i0, int nd) {
    const int sh = 32 - nd;
    const uint32_t hA = i0 & ~255u, hB = hA + 256u;
    for (int job = threadIdx.x; job < 3 * nk; job += blockDim.x) {
      const int kk = job / 3, t = job - 3 * kk;
      const uint32_t* vk = v + (size_t)(k0 + kk) * 32;
      uint32_t* row = tabs + kk * kRow;
      if (t < 2) {
        const uint32_t b0 = vk[4 * t] >> sh, b1 = vk[4 * t + 1] >> sh;
        const uint32_t b2 = vk[4 * t + 2] >> sh, b3 = vk[4 * t + 3] >> sh;
        uint32_t* o = row + 16 * t;
#pragma unroll
        for (int e = 0; e < 16; ++e)
          o[e] = ((e & 1) ? b0 : 0u) ^ ((e & 2) ? b1 : 0u) ^ ((e & 4) ? b2 : 0u) ^ ((e & 8) ? b3 : 0u);
      } else {
        uint32_t xa = 0u, xb = 0u;
#pragma unroll
        for (int j = 8; j < 32; ++j) {  // independent loads, predicated on j < nd
          if (j < nd) {
            const uint32_t vj = vk[j] >> sh;
            xa ^= ((hA >> j) & 1u) ? vj : 0u;
            xb ^= ((hB >> j) & 1u) ? vj : 0u;
          }
        }
        row[32] = xa;
        row[33] = xb;
      }
    }
  }
};

// Per-path view of a tqf_draws block: resolves antithetic pairing and the
// global path index once, then serves draws by (step, component).
template <typename T>
struct DrawSource {
  const T* base;
  int64_t s_step, s_comp;
  T sign;
  PhiloxReader<T> rng;
  int d;
  bool mem;
  __device__ __forceinline__ DrawSource(const tqf_draws& dr, int64_t path, int dim)
      : base(nullptr), s_step(0), s_comp(0), sign(T(1)), rng(0, dr.key0, dr.key1),
        d(dim), mem(dr.source == TQF_DRAWS_MEMORY) {
    if (mem) {
      base = static_cast<const T*>(dr.ptr) + path * dr.stride_path;
      s_step = dr.stride_step;
      s_comp = dr.stride_comp;
    } else {
      int64_t p = path;
      if (dr.antithetic && p >= dr.antithetic_half) {
        p -= dr.antithetic_half;
        sign = T(-1);
      }
      rng.path = p + dr.path_offset;
    }
  }
  __device__ __forceinline__ T get(int step, int comp) {
    if (mem) return base[step * s_step + comp * s_comp];
    return sign * rng.get((int64_t)step * d + comp);
  }
};

// ---- shared-memory staging by TMA bulk copy -------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> this CTA's shared memory; src, dst 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after ~`limit` polls (tens of ms), never hangs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  int limit = 1 << 20) {
  for (int it = 0; it < limit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    __nanosleep(64);
  }
  return false;
}

// Bounded wait that lets the hardware suspend the thread until the phase
// completes (or ~64 us pass) on each try instead of polling: waiting warps
// take no issue slots.  Gives up after `limit` tries (about a second).
__device__ __forceinline__ bool mbar_wait_suspend(uint64_t* bar, uint32_t parity, int limit = 1 << 14) {
  for (int it = 0; it < limit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(65536u)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Stages `nbytes` (multiple of 16) from global `src` into shared `dst` with
// one elected thread issuing bulk copies of <= 64 KiB; every thread of the
// CTA returns true once the data is visible, or false (uniformly) after a
// timed-out wait, having recorded TQF_E_TIMEOUT in *status.
__device__ __forceinline__ bool stage_to_smem(void* dst, const void* src, uint32_t nbytes,
                                              uint64_t* bar, uint32_t& phase, int32_t* status) {
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(bar, nbytes);
    uint32_t off = 0;
    while (off < nbytes) {
      uint32_t chunk = nbytes - off;
      if (chunk > 65536u) chunk = 65536u;
      bulk_copy_g2s(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off, chunk,
                    bar);
      off += chunk;
    }
  }
  bool ok = mbar_wait_bounded(bar, phase);
  ok = __syncthreads_and(ok) != 0;
  if (!ok) {
    if (threadIdx.x == 0 && status) atomicExch(status, TQF_E_TIMEOUT);
    mbar_wait_bounded(bar, phase);  // let in-flight copies land before exit
    __syncthreads();
    return false;
  }
  phase ^= 1u;
  return true;
}

// ---- every-step output rows ------------------------------------------------------
// Every-step output rows through a per-warp transposition buffer.  Each step
// a lane appends its path's values (as 32-bit words) to its own row of the
// warp's [32][33] word buffer in shared memory; when 32 words per path have
// gathered, the warp writes them path by path: one store instruction puts 32
// consecutive words (128 bytes) of one path's output row.  Only __syncwarp,
// no CTA barrier, no per-step slot lookup: the launch has checked that every
// step is recorded in order (tqf_path_output.every_step), so each path's row
// fills front to back.  Every lane of the warp takes part in every put and
// flush (a lane past the last path works on a duplicate path and its stores
// are dropped).  Row padding of 33 words keeps both the appends and the
// column reads free of bank conflicts.
struct WarpRowStager {
  static constexpr int kStride = 33;
  static constexpr int kWarpWords = 32 * kStride;
  static constexpr size_t bytes(int warps) { return (size_t)warps * kWarpWords * 4; }
  uint32_t* wbuf;  // this warp's buffer
  int nw;          // words per lane gathered in the current piece (warp-uniform)
  int64_t w0;      // row word offset of the current piece
  __device__ explicit WarpRowStager(void* smem)
      : wbuf(static_cast<uint32_t*>(smem) + (threadIdx.x >> 5) * kWarpWords), nw(0), w0(0) {}
  __device__ __forceinline__ void begin() {
    nw = 0;
    w0 = 0;
  }
  // Writes the gathered words of the warp's 32 paths path0 .. path0 + 31
  // (rows of row_words words) and starts the next piece.
  __device__ __forceinline__ void flush(uint32_t* out, int64_t row_words, int64_t path0, int64_t N) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    const int rmax = N - path0 < 32 ? (int)(N - path0) : 32;
    const bool on = lane < nw;
    const uint32_t* src = wbuf + lane;
    uint32_t* dst = out + path0 * row_words + w0 + lane;
#pragma unroll 8
    for (int r = 0; r < 32; ++r) {
      const uint32_t v = src[r * kStride];
      if (on && r < rmax) *dst = v;
      dst += row_words;
    }
    __syncwarp();
    w0 += nw;
    nw = 0;
  }
  __device__ __forceinline__ void push(uint32_t w, uint32_t* out, int64_t row_words, int64_t path0, int64_t N) {
    wbuf[(threadIdx.x & 31) * kStride + nw] = w;
    if (++nw == 32) flush(out, row_words, path0, N);
  }
  // Appends all DM values of this step without the full-piece test: the
  // caller runs make_room before the piece could pass 32 words.
  template <typename T, int DM>
  __device__ __forceinline__ void append(const T* x) {
    uint32_t* row = wbuf + (threadIdx.x & 31) * kStride;
#pragma unroll
    for (int c = 0; c < DM; ++c) {
      if constexpr (sizeof(T) == 4) {
        row[nw++] = __float_as_uint(x[c]);
      } else {
        const unsigned long long u = __double_as_longlong(x[c]);
        row[nw++] = (uint32_t)u;
        row[nw++] = (uint32_t)(u >> 32);
      }
    }
  }
  // Flushes the piece unless `words` more still fit in it.
  __device__ __forceinline__ void make_room(int words, uint32_t* out, int64_t row_words, int64_t path0, int64_t N) {
    if (nw > 32 - words) flush(out, row_words, path0, N);
  }
  // Appends the first `dim` of the DM values of this step.
  template <typename T, int DM>
  __device__ __forceinline__ void put(const T* x, int dim, uint32_t* out, int64_t row_words, int64_t path0,
                                      int64_t N) {
#pragma unroll
    for (int c = 0; c < DM; ++c) {
      if (c < dim) {
        if constexpr (sizeof(T) == 4) {
          push(__float_as_uint(x[c]), out, row_words, path0, N);
        } else {
          const unsigned long long u = __double_as_longlong(x[c]);
          push((uint32_t)u, out, row_words, path0, N);
          push((uint32_t)(u >> 32), out, row_words, path0, N);
        }
      }
    }
  }
};

// ---- FP64 European payoff accumulation --------------------------------------
// Each round, the CTA's BLOCK threads have one terminal spot each in
// s_spot[] (NaN for no path).  Work item w = (strike j, quarter q) sums
// payoffs of the paths of quarter q in FP32 and folds them into its own FP64
// accumulators acc[w] — fixed order, no atomics.
template <int BLOCK>
struct PayoffAccum {
  static constexpr int kQuarters = 4;
  static constexpr int kPathsPerQuarter = BLOCK / kQuarters;
};

template <int BLOCK, typename T>
__device__ __forceinline__ void payoff_round(const T* s_spot, const T* s_strike,
                                             const uint8_t* s_call, int num_strikes,
                                             double* acc /* smem [num_strikes*4][2] */) {
  constexpr int Q = PayoffAccum<BLOCK>::kQuarters;
  constexpr int PPQ = PayoffAccum<BLOCK>::kPathsPerQuarter;
  const int items = num_strikes * Q;
  for (int w = threadIdx.x; w < items; w += BLOCK) {
    const int j = w % num_strikes;
    const int q = w / num_strikes;
    const T K = s_strike[j];
    const bool call = s_call[j] != 0;
    T s1 = T(0), s2 = T(0);
#pragma unroll 8
    for (int p = 0; p < PPQ; ++p) {
      const T S = s_spot[q * PPQ + p];
      T f = call ? (S - K) : (K - S);
      f = f > T(0) ? f : T(0);  // NaN spot (no path) -> 0
      s1 += f;
      s2 = fma(f, f, s2);
    }
    acc[2 * w] += (double)s1;
    acc[2 * w + 1] += (double)s2;
  }
}

// Writes the CTA's partial sums (quarters folded in order) to
// workspace[blockIdx.x][num_strikes][2].
__device__ __forceinline__ void payoff_flush(const double* acc, int num_strikes, int quarters,
                                             double* workspace) {
  for (int j = threadIdx.x; j < num_strikes; j += blockDim.x) {
    double a = 0.0, b = 0.0;
    for (int q = 0; q < quarters; ++q) {
      a += acc[2 * (q * num_strikes + j)];
      b += acc[2 * (q * num_strikes + j) + 1];
    }
    workspace[((size_t)blockIdx.x * num_strikes + j) * 2] = a;
    workspace[((size_t)blockIdx.x * num_strikes + j) * 2 + 1] = b;
  }
}

// Host: launches the fixed-order reduction of `num_partials` partial rows of
// width `width` doubles into out[width].
int reduce_partials(const double* partials, int num_partials, int width, double* out,
                    cudaStream_t stream);

}  // namespace tqf
