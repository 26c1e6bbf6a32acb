/*
 * tqf.h — C ABI of the GB300 (sm_103a) Monte Carlo engine for the SDE
 * path-simulation hot path of tf-quant-finance.
 *
 * Every entry point is asynchronous on the caller's CUDA stream (`stream`, a
 * cudaStream_t passed as void*), allocates no device memory, never throws and
 * returns an int status: TQF_OK (0) or a negative TQF_E_* code, with a
 * message readable through tqf_last_error() on the calling thread.  All
 * buffers are caller-owned device pointers unless a parameter says "host".
 *
 * Random draws follow one canonical layout, shared by every kernel: the draw
 * for path n and draw dimension k (k = step * num_normal_draws + component,
 * the dimension order of tff/models/utils.py:95-127) is a pure function of
 * (key, n, k), so fused in-kernel generation and materialised draws agree and
 * a path range can be resumed or sharded by `path_offset`.
 */
#ifndef TQF_H_
#define TQF_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define TQF_API __attribute__((visibility("default")))
#else
#define TQF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TQF_OK 0
#define TQF_E_INVALID (-1)     /* bad argument (shape, size, null pointer) */
#define TQF_E_CUDA (-2)        /* a CUDA runtime call failed */
#define TQF_E_UNSUPPORTED (-3) /* valid request outside what is built */
#define TQF_E_TIMEOUT (-4)     /* a bounded device-side wait ran out */
#define TQF_E_IO (-5)          /* host file could not be read/parsed */

/* ---- dtypes / enums ------------------------------------------------------ */
#define TQF_F32 0
#define TQF_F64 1

#define TQF_DRAWS_MEMORY 0 /* read normals from `tqf_draws.ptr` with strides */
#define TQF_DRAWS_PHILOX 1 /* generate them in-kernel (Philox4x32-10) */
#define TQF_DRAWS_SOBOL 2  /* Sobol normals generated in-kernel (Heston kernels only) */

/* Sobol output kinds (tqf_sobol_sample / tqf_sobol_normal_draws). */
#define TQF_SOBOL_U32 0        /* integer at the reference's nd-digit scaling */
#define TQF_SOBOL_F32 1        /* float32(int) * 2^-nd (reference float) */
#define TQF_SOBOL_F64 2        /* float64(int) * 2^-nd */
#define TQF_SOBOL_NORMAL_F32 3 /* erfinv((u-0.5)*2)*sqrt(2) on the f32 value */
#define TQF_SOBOL_NORMAL_F64 4 /* same on the f64 value */
#define TQF_SOBOL_F32_CENTERED 5 /* (int + 0.5) * 2^-nd: strictly inside (0,1) */

/* ---- shared argument blocks --------------------------------------------- */

/* Source of the N(0,1) draws consumed by a path kernel.  Memory draws are
 * addressed as ptr[step*stride_step + path*stride_path + comp*stride_comp]
 * (elements of the kernel's dtype), so both the reference's [steps, N, d]
 * layout and the caller-facing [N, steps, d] layout are read without a
 * transpose copy.  Philox draws use key (key0, key1) and the canonical
 * counter layout; `antithetic` makes paths [half, 2*half) the negation of
 * paths [0, half) (tff/math/random_ops/multivariate_normal.py:276-311).
 * Sobol draws (TQF_DRAWS_SOBOL) are the SOBOL branch of
 * generate_mc_normal_draws (tff/models/utils.py:95-127) computed inside the
 * path kernel: ptr = the device direction numbers [dims][32] of
 * tqf_sobol_direction_numbers (dims >= key1 * num_steps), key0 = nd (the
 * digit count of the whole request), key1 = normals per step, and path n
 * takes point path_offset + 1 + n, step i component c dimension i*key1 + c;
 * the values equal tqf_sobol_normal_draws's bit for bit. */
typedef struct tqf_draws {
  int32_t source;
  int32_t antithetic;
  const void* ptr;
  int64_t stride_step;
  int64_t stride_path;
  int64_t stride_comp;
  uint32_t key0;
  uint32_t key1;
  int64_t path_offset;
  int64_t antithetic_half;
} tqf_draws;

/* Recorded output: paths[N, num_slots, dim] in the kernel's dtype.  The
 * state after step i is stored to the slot held (as an exact integer value,
 * -1 = none) in the last column of row i of the kernel's step table, and the
 * initial state to init_slot (-1 = none).  The host derives the slots from
 * the reference's written_count/keep_mask recursion
 * (tff/models/euler_sampling.py:424-455).  every_step = 1 declares that step
 * i records slot base + i for every step (base = 1 after an initial state at
 * slot 0, else 0) and num_slots = base + num_steps: path rows then fill front
 * to back, and the Euler (tqf_euler_affine) and GBM (tqf_mvgbm_paths) kernels
 * gather 32 words of 32 paths' rows per warp in shared memory and write each
 * path's 128 bytes with one store instruction.  Such a kernel that finds the
 * declaration false writes no states and sets *dev_status to TQF_E_INVALID;
 * the other kernels ignore the field. */
typedef struct tqf_path_output {
  void* ptr;
  int32_t num_slots;
  int32_t init_slot;
  int32_t every_step;
  int32_t pad0;
} tqf_path_output;

/* Fused European payoff over the final state: for each strike j the kernel
 * accumulates, in FP64 across paths, sum_p f_j(S_p) and sum_p f_j(S_p)^2 with
 * f_j = max(S - K_j, 0) (call) or max(K_j - S, 0) (put) and
 * S = spot_scale * exp(state[0]) (log-spot models) or state[0] (level models,
 * see each entry point).  out[2*j] = sum, out[2*j+1] = sum of squares.
 * `workspace` holds per-CTA partial sums; its size is given by the matching
 * *_workspace_bytes query.  With out == NULL the path kernels leave the
 * partial sums in the workspace and skip the reduction launch.  Results are deterministic (fixed summation order)
 * for a given device and launch shape. */
typedef struct tqf_payoff {
  int32_t num_strikes; /* 0 disables the payoff */
  int32_t pad0;
  const void* strikes;    /* device, [num_strikes], kernel dtype */
  const uint8_t* is_call; /* device, [num_strikes] or NULL (all calls) */
  double spot_scale;
  double* out;            /* device, [num_strikes * 2] */
  void* workspace;
  size_t workspace_bytes;
} tqf_payoff;

/* ---- library ------------------------------------------------------------- */

/* ABI version (major*100 + minor). */
TQF_API int tqf_abi_version(void);

/* Message of the last failing call on this thread ("" if none). */
TQF_API const char* tqf_last_error(void);

/* Number of kernels this library has launched in the process (all threads);
 * used to count kernel launches inside a timed region. */
TQF_API uint64_t tqf_launch_count(void);

/* FP32-pipe peak probe (no reference counterpart; roofline denominator):
 * launches SMs x blocks_per_sm CTAs of 256 threads running independent FMA
 * chains and stores the number of FMA lane operations issued in *lane_ops
 * (host).  Time it with events on `stream`. */
TQF_API int tqf_fma_peak_probe(int32_t iters, int32_t blocks_per_sm, float* out, double* lane_ops,
                               void* stream);

/* tcgen05 self-check (no reference counterpart): D = A B^T with A [m x k]
 * and B [n x k] row-major BF16 (device), staged in the K-major (a_mn/b_mn = 0)
 * or MN-major (1) canonical no-swizzle layout and multiplied by tcgen05.mma;
 * out (device, [128 x n] FP32) receives TMEM lanes 0..127.  m in {64, 128},
 * n and k multiples of 16 up to 128.  *status (device, may be NULL) is set to
 * TQF_E_TIMEOUT if the MMA completion wait runs out. */
TQF_API int tqf_tc_selftest(const uint16_t* a, const uint16_t* b, int32_t m, int32_t n, int32_t k,
                            int32_t a_mn, int32_t b_mn, float* out, int32_t* status, void* stream);

/* ---- Sobol (tff/math/random_ops/sobol/sobol_impl.py) --------------------- */

/* Host-only.  Parses the Joe–Kuo file (new-joe-kuo-6.21201) and writes the
 * 32-bit direction numbers v[d*32 + j] = m_dj << (31 - j) for dimensions
 * 0..dim-1 (dimension 0: all m = 1).  Replaces _compute_direction_numbers
 * and load_data (sobol_impl.py:171-197, 237-261). */
TQF_API int tqf_sobol_direction_numbers(const char* joe_kuo_path, int32_t dim,
                                uint32_t* v_host);

/* Number of binary digits the reference uses for a request:
 * ceil(log(skip + num_results + 1) / log 2) (sobol_impl.py:118-123). */
TQF_API int32_t tqf_sobol_num_digits(int64_t num_results, int64_t skip);

/* out[n, d] for n in [0, num_results), d in [0, dim): Sobol point with
 * sequence index skip + 1 + n (natural order), scaled to nd digits, written
 * as `out_kind`.  v_dev is the device copy of tqf_sobol_direction_numbers.
 * Replaces sobol.sample (sobol_impl.py:39-167). */
TQF_API int tqf_sobol_sample(const uint32_t* v_dev, int32_t dim, int64_t num_results,
                     int64_t skip, int32_t nd, int32_t out_kind, void* out,
                     void* stream);

/* Normal draws in the reference's path-simulation layout
 * out[i, n, c] = normal(point skip+1+n, dimension i*num_normal_draws + c),
 * shape [num_steps, num_paths, num_normal_draws]; out_kind is
 * TQF_SOBOL_NORMAL_F32 or TQF_SOBOL_NORMAL_F64.  Replaces the SOBOL branch
 * of generate_mc_normal_draws (tff/models/utils.py:20-128,
 * multivariate_normal.py:356-424). */
TQF_API int tqf_sobol_normal_draws(const uint32_t* v_dev, int32_t num_normal_draws,
                           int32_t num_steps, int64_t num_paths, int64_t skip,
                           int32_t nd, int32_t out_kind, void* out,
                           void* stream);

/* ---- Philox draws (PSEUDO / STATELESS / *_ANTITHETIC) -------------------- */

/* Raw Philox4x32-10 blocks: out[4*b + l] = philox(ctr=(ctr0+b, c1, c2, c3),
 * key)[l] for b in [0, num_blocks).  Known-answer testing of the generator. */
TQF_API int tqf_philox4x32_10(uint32_t ctr0, uint32_t c1, uint32_t c2, uint32_t c3,
                      uint32_t key0, uint32_t key1, int64_t num_blocks,
                      uint32_t* out, void* stream);

/* Materialised normal draws out[i, n, c] (shape [num_steps, num_paths,
 * num_normal_draws], dtype TQF_F32/TQF_F64) from the canonical stream of
 * `draws` (source must be TQF_DRAWS_PHILOX).  Replaces the PSEUDO/STATELESS
 * branches of generate_mc_normal_draws (tff/models/utils.py:20-128,
 * multivariate_normal.py:248-311). */
TQF_API int tqf_philox_normal_draws(const tqf_draws* draws, int32_t num_normal_draws,
                            int32_t num_steps, int64_t num_paths, int32_t dtype,
                            void* out, void* stream);

/* ---- Euler–Maruyama (tff/models/euler_sampling.py) ----------------------- */

/* Structured coefficients of dX = a(X) dt + B(X) dW, dim <= 16:
 *   a(x)   = drift_m + drift_M x                       ([dim], [dim, dim])
 *   B(x)ij = (vol_s0_i + vol_s1_i x_i) vol_C_ij        ([dim], [dim], [dim, dim])
 * (GBM, arithmetic BM, OU, correlated GBM in levels).  step_table is
 * [num_steps][4] = (dt_i, sqrt(dt_i), slot_i, 0).  x0 is [dim] or [num_paths, dim]
 * (x0_per_path = 1).  One kernel pass, state in registers; replaces the
 * while-loop body _euler_step (euler_sampling.py:513-537). */
typedef struct tqf_euler_affine_args {
  int32_t dtype;
  int32_t dim;
  int64_t num_paths;
  int32_t num_steps;
  int32_t x0_per_path;
  const void* step_table;
  const void* x0;
  const void* drift_m;
  const void* drift_M;
  const void* vol_s0;
  const void* vol_s1;
  const void* vol_C;
  tqf_draws draws;
  tqf_path_output output;
  int32_t* dev_status; /* device int or NULL: set to TQF_E_TIMEOUT on a timed-out wait */
} tqf_euler_affine_args;

TQF_API int tqf_euler_affine(const tqf_euler_affine_args* args, void* stream);

/* One Euler step for arbitrary coefficients evaluated by the caller:
 * x_next = x + dt * a + B · (z * sqrt_dt), x/a [num_paths, dim], B
 * [num_paths, dim, dim] row-major, z from `draws` at `step`.  If
 * out_slot >= 0 the new state is also stored to output.ptr[:, out_slot, :].
 * (euler_sampling.py:519-530). */
typedef struct tqf_euler_update_args {
  int32_t dtype;
  int32_t dim;
  int64_t num_paths;
  int32_t step;
  int32_t out_slot;
  double dt;
  double sqrt_dt;
  const void* x;
  const void* drift;
  const void* vol;
  void* x_next;
  tqf_draws draws;
  void* paths_out;
  int32_t num_slots;
  int32_t pad0;
} tqf_euler_update_args;

TQF_API int tqf_euler_update(const tqf_euler_update_args* args, void* stream);

/* ---- Halton sequence (tff/math/random_ops/halton/halton_impl.py) ----------
 * tqf_halton_sample: out[i][d] (row-major [num_results][dim]) = radical inverse
 * of index_i + 1 in the d-th prime base over max_sizes[d] digit positions
 * (halton_impl.py:250-299), index_i = sequence_indices[i] (device int64) or
 * first_index + i.  With perms (device int32 [num_coeffs * radix_sum]) the
 * digit at position k is replaced by perms[k * radix_sum + perm_offsets[d] +
 * digit] and zero_correction[d] (device, out dtype) is added (Owen
 * scrambling, :282-299).  out_kind: TQF_SOBOL_F32 / _F64 (uniform) or
 * TQF_SOBOL_NORMAL_F32 / _F64 (sqrt2 erfinv(2u - 1)). */
typedef struct tqf_halton_args {
  int32_t dim;
  int32_t out_kind;
  int64_t num_results;
  int64_t first_index;
  const int64_t* sequence_indices; /* device [num_results] or NULL */
  const int32_t* primes;           /* device [dim] */
  const int32_t* max_sizes;        /* device [dim] digit positions per axis */
  const int32_t* perms;            /* device or NULL (unscrambled) */
  const int32_t* perm_offsets;     /* device [dim]: sum of the primes before axis d */
  int32_t radix_sum;               /* sum of the dim primes */
  int32_t pad0;
  const void* zero_correction;     /* device [dim] (out dtype) or NULL */
  void* out;
} tqf_halton_args;

TQF_API int tqf_halton_sample(const tqf_halton_args* args, void* stream);

/* Independent uniform permutations for the Owen scrambling: for every digit
 * position k < num_coeffs and axis d a Fisher-Yates shuffle of 0..p_d-1
 * written at perms[k * radix_sum + perm_offsets[d]], and uniforms[d] in [0, 1)
 * for the zero correction.  Counter-based (Philox4x32-10, key = seed), so a
 * seed reproduces the same permutations on any device.  Replaces
 * _get_permutations (halton_impl.py:321-343) with this engine's own stream. */
TQF_API int tqf_halton_permutations(int32_t dim, int32_t num_coeffs, const int32_t* primes,
                                    const int32_t* perm_offsets, int32_t radix_sum, uint64_t seed,
                                    int32_t* perms, double* uniforms, void* stream);

/* ---- tff.math.qmc: digital nets and rank-1 lattice rules ------------------
 * tqf_digital_net_sample: out[i][d] = (shift_d XOR (XOR over set bits b of
 * index_i of M[d][b])) / 2^num_digits in the output dtype, optionally tent
 * transformed (digital_net.py:205-419; index_i = sequence_indices[i] or i,
 * starting at 0).  M: device [dim][log_num_results], int32 or int64 (int_bits).
 * tqf_lattice_rule_sample: out[i][d] = frac(index_i * frac(g_d / n) + shift_d)
 * in the output dtype (lattice_rule.py:99-229).  out_kind TQF_SOBOL_F32/_F64. */
typedef struct tqf_digital_net_args {
  int32_t dim;
  int32_t log_num_results;
  int32_t num_digits;
  int32_t out_kind;
  int32_t tent;
  int32_t int_bits;              /* 32 or 64: element type of matrices / digital_shift */
  int64_t count;                 /* points produced */
  const int64_t* sequence_indices; /* device [count] or NULL (0 .. count-1) */
  const void* matrices;
  const void* digital_shift;     /* device [dim] or NULL */
  void* out;
} tqf_digital_net_args;

TQF_API int tqf_digital_net_sample(const tqf_digital_net_args* args, void* stream);

typedef struct tqf_lattice_args {
  int32_t dim;
  int32_t out_kind;
  int32_t tent;
  int32_t int_bits;              /* element type of generating_vectors */
  int64_t num_results;           /* n of the rule */
  int64_t count;                 /* points produced */
  const int64_t* sequence_indices; /* device [count] or NULL */
  const void* generating_vectors;  /* device [>= dim] */
  const void* additive_shift;      /* device [>= dim] (out dtype) or NULL */
  void* out;
} tqf_lattice_args;

TQF_API int tqf_lattice_rule_sample(const tqf_lattice_args* args, void* stream);

/* ---- Hull-White short-rate paths (tff/models/hull_white/vector_hull_white.py) ----
 * Exact discretisation of the vector Hull-White model with piecewise-constant
 * parameters (_sample_paths, vector_hull_white.py:641-781): per step i and
 * axis d, x_d <- decay[i][d] x_d + mean[i][d] + vol[i][d] (L_i z)_d, and the
 * rate x_d + f0[i+1][d] is stored at slot[i] (f0[0][d] at output.init_slot).
 * table [num_steps][dim][3] = (exp(-a_{i+1} dt_i), conditional mean increment,
 * sqrt of the conditional variance); f0 [num_steps + 1][dim] (instantaneous
 * forward rates on the grid); chol [num_steps][dim][dim] lower Cholesky
 * factors of the correlation or NULL; slots [num_steps] int32.  dim <= 16. */
typedef struct tqf_hull_white_args {
  int32_t dtype;
  int32_t dim;
  int64_t num_paths;
  int32_t num_steps;
  int32_t pad0;
  const void* table;
  const void* f0;
  const void* chol;
  const int32_t* slots;
  tqf_draws draws;
  tqf_path_output output;
} tqf_hull_white_args;

TQF_API int tqf_hull_white_paths(const tqf_hull_white_args* args, void* stream);

/* ---- Gaussian HJM factor paths (tff/models/hjm/gaussian_hjm.py) -----------
 * Euler on the grid for the factors x (gaussian_hjm.py:209-227, 404-457):
 * x <- x + dt_i (c_i - k x) + B_i (z sqrt(dt_i)), c_i = sum_j y_.j(t_{i+1}),
 * B_i = chol(rho) scaled by row by sigma(t_{i+1}); along the way the short
 * rate r_g = sum_k x_k + f0[g] and the discount factor D_{g+1} = D_g exp(-r_g dt_g)
 * (D_0 = 1).  table [num_steps][2 + dim + dim*dim] = (dt, sqrt dt, c, B);
 * grid_slot [num_steps + 1]: output slot of each grid point or -1.
 * rate_out, df_out [N][num_slots]; x_out [N][num_slots][dim] or NULL. */
typedef struct tqf_hjm_args {
  int32_t dtype;
  int32_t dim;
  int64_t num_paths;
  int32_t num_steps;
  int32_t num_slots;
  const void* table;
  const void* mean_reversion;  /* [dim] */
  const void* f0;              /* [num_steps + 1] */
  const int32_t* grid_slot;    /* [num_steps + 1] */
  tqf_draws draws;
  void* rate_out;
  void* df_out;
  void* x_out;
} tqf_hjm_args;

TQF_API int tqf_hjm_paths(const tqf_hjm_args* args, void* stream);

/* ---- Milstein scheme (tff/models/milstein_sampling.py) ---------------------
 * Step of _milstein_1d / _milstein_nd (milstein_sampling.py:565-593) with the
 * Stratonovich integral approximation of _stratonovich_integral (:481-525) and
 * the drift correction of _stratonovich_drift_update (:555-562), the grid and
 * recording of _while_loop (:356-424).  Every step consumes
 * dim + 3 * dim * order normals (draw dimension k = step * K + c, K that count):
 * [0, dim) the Wiener increments, then the mu, zeta, eta blocks of dim * order
 * each, element (component c, term r) at c * order + r.
 *
 * tqf_milstein_affine: the whole loop for structured coefficients
 * a(x) = m + M x, B(x)_kj = (s0_k + s1_k x_k) C_kj (exact dB_kj/dx_i =
 * delta_ik s1_k C_kj), step table [num_steps][4] = (dt, sqrt dt, slot, 0),
 * any dim (above 8, one warp per path). */
typedef struct tqf_milstein_affine_args {
  int32_t dtype;
  int32_t dim;
  int64_t num_paths;
  int32_t num_steps;
  int32_t x0_per_path;
  int32_t order;             /* stratonovich_order >= 1 */
  int32_t pad0;
  const void* step_table;
  const void* x0;
  const void* drift_m;
  const void* drift_M;
  const void* vol_s0;
  const void* vol_s1;
  const void* vol_C;
  tqf_draws draws;
  tqf_path_output output;
  int32_t* dev_status;
} tqf_milstein_affine_args;

TQF_API int tqf_milstein_affine(const tqf_milstein_affine_args* args, void* stream);

/* One Milstein step for coefficients the caller evaluated at t_{i+1}:
 * drift [N][d], vol [N][d][d] = B, grad [N][d(i)][d(k)][d(j)] = dB_kj/dx_i.
 * increments_out (optional, [N][d + d*d] in the dtype) receives the step's
 * dW and Stratonovich integrals J (row-major J_im; J_00 = dW^2/2 for d = 1),
 * which a backward pass through the step needs. */
typedef struct tqf_milstein_update_args {
  int32_t dtype;
  int32_t dim;
  int64_t num_paths;
  int32_t step;
  int32_t out_slot;
  int32_t order;
  int32_t num_slots;
  double dt;
  double sqrt_dt;
  const void* x;
  const void* drift;
  const void* vol;
  const void* grad;
  void* x_next;
  tqf_draws draws;
  void* paths_out;           /* [N][num_slots][d] or NULL */
  void* increments_out;      /* [N][d + d*d] or NULL */
} tqf_milstein_update_args;

TQF_API int tqf_milstein_update(const tqf_milstein_update_args* args, void* stream);

/* Full-truncation Euler for the Heston model in log-spot form, as the
 * reference Euler sampler runs it with drift [r - v+/2, kappa (theta - v+)]
 * and volatility [[sqrt v+, 0], [xi rho sqrt v+, xi sqrt(1-rho^2) sqrt v+]],
 * v+ = max(v, 0), coefficients evaluated at t_{i+1}.  step_table (16-byte
 * aligned) is [num_steps][8] = (dt/2, sqrt_dt, r*dt, kappa*dt,
 * kappa*theta*dt, xi*rho, xi*sqrt(1-rho^2), slot).  Component 0 of the draws drives the log-spot.
 * Optional path store and fused European payoff (S = spot_scale*exp(x_T)). */
typedef struct tqf_heston_args {
  int32_t dtype;
  int32_t num_steps;
  int64_t num_paths;
  const void* step_table;
  double x0;
  double v0;
  tqf_draws draws;
  tqf_path_output output;
  tqf_payoff payoff;
  int32_t* dev_status;
} tqf_heston_args;

TQF_API int tqf_heston_euler(const tqf_heston_args* args, void* stream);

/* Allocation-free variant of tqf_heston_euler's fused pricing (no
 * counterpart in the reference).  Some callers cannot call cudaMalloc: hosts
 * with a custom or fixed-budget device allocator that forbids stray
 * allocations, and plugins whose host application owns all device memory and
 * hands the library only its input and output buffers.  They still pass
 * inputs and outputs (step table, strikes, payoff.out); the per-CTA partial
 * sums go to a 2 MiB array compiled into the library instead of
 * payoff.workspace (ignored).  Limit: payoff.num_strikes <= 64; more is
 * rejected with TQF_E_INVALID.  The first call on each device (and the first
 * after a cudaDeviceReset) looks up that array's device address
 * (cudaGetSymbolAddress), so make it before any stream capture.  All calls
 * share the array: two calls that overlap on the GPU (different streams, or
 * concurrent host threads) race; serialise them.  Nothing needs clearing
 * between calls — every partial row the final reduction reads is written by
 * the same call. */
TQF_API int tqf_heston_euler_price_noalloc(const tqf_heston_args* args, void* stream);

/* Andersen QE scheme exactly as HestonModel.sample_paths runs it
 * (tff/models/heston/heston_model.py:322-460, 522-572): step_table is
 * [num_steps][12] = (skip, theta, E=exp(-kappa dt), A, B, k0, k1, k2, k3,
 * k4, 0, slot) with s^2 = v A + B; skip != 0 marks dt <= tolerance steps that
 * consume draws but leave the state unchanged.  Component 0 of the draws
 * drives the variance, component 1 the log-spot; output slots hold
 * (log-spot, variance). */
TQF_API int tqf_heston_qe(const tqf_heston_args* args, void* stream);

/* Pathwise adjoint of the full-truncation Euler European pricer (no
 * reference counterpart beyond the GradientTape of the Euler sampler with
 * watch_params, tff/models/euler_sampling.py:467-510): replays the paths of
 * tqf_heston_euler from the same draws with forward tangents of (x, v) with
 * respect to (log S0, v0, kappa, theta, xi, rho, r) and writes
 * out[7] (device, FP64) = sum_paths c_p S_T,p dx_T,p/dparam with
 * c_p = sum_j weights_j dPayoff_j/dS_T.  step_table as tqf_heston_euler
 * with constant parameters, also passed explicitly (kappa, theta, xi, rho). */
typedef struct tqf_heston_adjoint_args {
  int32_t dtype;
  int32_t num_steps;
  int64_t num_paths;
  const void* step_table;
  double x0;
  double v0;
  double kappa;
  double theta;
  double xi;
  double rho;
  tqf_draws draws;
  int32_t num_strikes;
  int32_t pad0;
  const void* strikes;    /* [num_strikes] dtype */
  const uint8_t* is_call; /* [num_strikes] or NULL */
  const void* weights;    /* [num_strikes] dtype */
  double* out;            /* [7] */
  void* workspace;
  size_t workspace_bytes;
  int32_t* dev_status;
} tqf_heston_adjoint_args;

TQF_API int tqf_heston_euler_adjoint(const tqf_heston_adjoint_args* args, void* stream);
TQF_API size_t tqf_heston_adjoint_workspace_bytes(int64_t num_paths);

/* Workspace bytes that tqf_heston_euler / tqf_heston_qe need in
 * payoff.workspace for a given dtype, path count and strike count. */
TQF_API size_t tqf_heston_workspace_bytes(int32_t dtype, int32_t qe, int64_t num_paths,
                                  int32_t num_strikes);

/* ---- correlated GBM (multivariate_geometric_brownian_motion.py) ------------ */

/* Exact log scheme of MultivariateGeometricBrownianMotion.sample_paths
 * (tff/models/geometric_brownian_motion/multivariate_geometric_brownian_motion.py:229-281):
 * cumsum_i += drift_i dt + sqrt(dt) vol_i (L z)_i, state x0_i exp(cumsum_i)
 * stored at the slots of step_table [num_steps][4] = (dt, sqrt_dt, slot, 0).
 * drift = mu - vol^2/2 ([dim]), vol [dim], chol = L [dim, dim] row-major
 * lower-triangular or NULL (independent components), dim <= 16. */
typedef struct tqf_mvgbm_args {
  int32_t dtype;
  int32_t dim;
  int64_t num_paths;
  int32_t num_steps;
  int32_t x0_per_path;
  const void* step_table;
  const void* x0;
  const void* drift;
  const void* vol;
  const void* chol;
  tqf_draws draws;
  tqf_path_output output;
  int32_t* dev_status;
  int32_t lz_mode; /* 0: tensor-core split-BF16 L z for 16 <= dim <= 64 (float32), else CUDA cores; 1: CUDA cores */
  int32_t pad0;
} tqf_mvgbm_args;

/* FP64 Cholesky factor L (row-major, lower) of an n x n symmetric positive
 * definite matrix (any n; shared memory up to n = 64, global memory beyond),
 * on the GPU in one CTA (replaces
 * tf.linalg.cholesky at multivariate_geometric_brownian_motion.py:264 and
 * multivariate_normal.py:436).  *info (device int) = 0 on success, k + 1
 * when the k-th pivot is not positive. */
TQF_API int tqf_cholesky_f64(const double* a, int32_t n, double* l, int32_t* info, void* stream);

TQF_API int tqf_mvgbm_paths(const tqf_mvgbm_args* args, void* stream);

/* Arithmetic-basket European option on correlated GBM at the last step, with
 * pathwise sensitivities, FP64 accumulation.  out[2 + 2*dim] (device) =
 * (sum P, sum P^2, sum_p g_i (i < dim), sum_p g_i (y_i - vol_i T) (i < dim))
 * with P the undiscounted payoff on B = sum_i weights_i S_T,i,
 * g_i = dP/dB * weights_i * S_T,i and y = L sum_k sqrt(dt_k) z_k, so that
 * dP/dS0_i = g_i / S0_i, dP/dvol_i = g_i (y_i - vol_i T), dP/dmu_i = g_i T.
 * With out == NULL the per-CTA partials stay in the workspace. */
typedef struct tqf_basket_args {
  int32_t dtype;
  int32_t dim;
  int64_t num_paths;
  int32_t num_steps;
  int32_t is_call;
  const void* sqrt_dt; /* [num_steps] */
  double total_time;
  double strike;
  const void* spot;    /* [dim] */
  const void* drift;   /* [dim] mu - vol^2/2 */
  const void* vol;     /* [dim] */
  const void* chol;    /* [dim, dim] or NULL */
  const void* weights; /* [dim] */
  tqf_draws draws;
  double* out;
  void* workspace;
  size_t workspace_bytes;
  int32_t* dev_status;
} tqf_basket_args;

TQF_API int tqf_basket_price(const tqf_basket_args* args, void* stream);
TQF_API size_t tqf_basket_workspace_bytes(int32_t dtype, int32_t dim, int64_t num_paths);

/* ---- neural control variate (no reference counterpart) --------------------- */

/* Network g(t, log S, v) = b3 + w3 . silu(W2 silu(W1 x) + b2), x = (f0, f1, f2,
 * 1, 0 ... 0) with f_i = (raw_i - feat_shift_i) * feat_scale_i; W1 [64][16]
 * (column 3 is layer 1's bias, columns 4-15 zero) and W2 [64][64] are BF16
 * row-major (out, in); silu uses the SFU tanh. */
typedef struct tqf_mlp_host_weights {
  float w1[64][4]; /* (w_j0, w_j1, w_j2, b1_j) — columns 0-3 of W1 */
  float b2[64];
  float w3[64];
  float b3;
} tqf_mlp_host_weights;

/* Inference weights: W2 as a device BF16 [64][64] array (tensor-core operand)
 * and the small layers from host memory, passed to the kernel by value so
 * that they are read from the constant bank. */
typedef struct tqf_mlp_weights {
  const void* w2_bf16;
  const tqf_mlp_host_weights* host;
  float feat_scale[3];
  float feat_shift[3];
} tqf_mlp_weights;

/* Full-truncation Euler Heston paths (Philox in-kernel, FP32) with an
 * arithmetic-Asian payoff Y = discount_T max(mean_k S(t_k) - strike, 0) over
 * num_dates monitoring dates marked in the step table's slot column (date
 * index, -1 otherwise; table layout of tqf_heston_euler).  Mode 2 also reads
 * slot -2 as "advance the network pipeline one stage here"; two such steps
 * between consecutive dates let the tensor-core work overlap the stepping
 * (without them every stage runs at the date).  date_table
 * [num_dates][4] = (t_k, exp(-r t_k), hold_k, 0).  The control's intervals
 * run between the control dates: the monitoring dates with hold_k = 0, and
 * always the last date.  At a date with hold_k != 0 the network's position
 * carries over (no evaluation ends or starts there); with every hold_k = 0
 * the network is evaluated at every monitoring interval.  D_c below is the
 * number of control dates.
 *  mode 0: out[5] (device, FP64) = sums of (Y, Y^2, 0, 0, 0);
 *  mode 1: pilot data, date-major so that the stores coalesce:
 *          pilot_feats [D_c][N][4] = (t, log S, v, 0) at each control
 *          interval start, pilot_dS [D_c][N] discounted-spot increments over
 *          the control intervals, pilot_Y [N];
 *  mode 2: out[5] = sums of (Y, Y^2, C, C^2, Y C), C = sum_j g_j dS~_j the
 *          martingale control variate with the network evaluated on the
 *          tensor cores at every control interval start.
 * Modes 0 and 2 also write, when path_values is non-null (8-byte aligned),
 * each path's (Y, C) as float pairs [N][2] (C = 0 in mode 0).
 * Estimator of the price: mean(Y - C). */
typedef struct tqf_heston_asian_args {
  int32_t mode;
  int32_t num_steps;
  int64_t num_paths;
  const float* step_table;
  int32_t num_dates;
  int32_t pad0;
  const float* date_table;
  double x0;
  double v0;
  double strike;
  double discount_T;
  tqf_draws draws;
  tqf_mlp_weights mlp;
  float* pilot_feats;
  float* pilot_dS;
  float* pilot_Y;
  double* out;
  void* workspace;
  size_t workspace_bytes;
  int32_t* dev_status;
  float* path_values; /* optional [N][2] per-path (Y, C), modes 0 and 2 */
} tqf_heston_asian_args;

TQF_API int tqf_heston_asian(const tqf_heston_asian_args* args, void* stream);
/* Device workspace (16-byte aligned) that modes 0 and 2 need: the per-CTA
 * FP64 partial sums and, for mode 2, a two-step-block copy of the step table
 * that the call writes before its path kernel reads it. */
TQF_API size_t tqf_heston_asian_workspace_bytes(int32_t mode, int64_t num_paths, int32_t num_steps);
/* Resident CTAs per SM of the tqf_heston_asian kernel for `mode`, or a
 * negative TQF_E_* code. */
TQF_API int tqf_heston_asian_occupancy(int32_t mode, int32_t num_steps);

/* Number of FP32 parameters of the network plus the loss offset c:
 * [W1 64x16 | W2 64x64 | b2 64 | w3 64 | b3 | c]. */
TQF_API int tqf_mlp_num_params(void);

/* Gradient of loss = mean_p (Y_p - c - sum_k g(feats_pk) dS_pk)^2 over the
 * paths [path_begin, path_begin + batch_paths) of the pilot data, one CTA per
 * paths_per_cta paths; grad_partials [batch_paths/paths_per_cta][num_params + 2]
 * (16-byte aligned) receives each CTA's gradient, in column num_params its
 * share of the loss, and a zero in the last column.  Forward and backward
 * GEMMs run on tcgen05 tensor cores (BF16 operands, FP32 accumulation). */
typedef struct tqf_mlp_train_args {
  int32_t num_dates;
  int32_t batch_paths;
  int32_t paths_per_cta; /* paths_per_cta x num_dates <= 128: one CTA = one 128-row tile */
  int32_t pad0;
  int64_t path_begin;
  int64_t pilot_paths; /* N: the pilot data's path count (its date stride) */
  const float* feats;  /* [num_dates][N][4] (tqf_heston_asian mode 1), 16-byte aligned */
  const float* dS;     /* [num_dates][N] */
  const float* Y;     /* [N] */
  const float* params;
  const void* w1_bf16;
  const void* w2_bf16;
  float feat_scale[3];
  float feat_shift[3];
  float* grad_partials;
  int32_t* dev_status;
} tqf_mlp_train_args;

TQF_API int tqf_mlp_train_step(const tqf_mlp_train_args* args, void* stream);

/* Adam update: sums the gradient partials in a fixed order, updates the FP32
 * master parameters and moments and refreshes the BF16 weight copies;
 * loss_out[0] (device, may be NULL) receives the minibatch loss.
 * bias1 = 1 - beta1^t, bias2 = 1 - beta2^t. */
typedef struct tqf_mlp_adam_args {
  float* params;
  float* m;
  float* v;
  const float* grad_partials;
  int32_t num_partials;
  int32_t pad0;
  void* w1_bf16;
  void* w2_bf16;
  float lr, beta1, beta2, eps, bias1, bias2;
  float* loss_out;
} tqf_mlp_adam_args;

TQF_API int tqf_mlp_adam(const tqf_mlp_adam_args* args, void* stream);

/* ---- payoff reduction over stored values ----------------------------------- */

/* ---- Longstaff–Schwartz regression Monte Carlo ------------------------------
 * Replaces least_square_mc (tff/models/longstaff_schwartz/lsm.py:128-295)
 * with its loop body (lsm.py:403-436), _expected_exercise_fn (lsm.py:328-383),
 * make_polynomial_basis (lsm.py:50-125) and make_basket_put_payoff
 * (payoff_utils.py:27-98).  The caller runs the backward loop over exercise
 * indices i = E-1 .. 1 as one tqf_lsm_pass (update with the regression of
 * i+1, accumulate the normal equations of i) and one tqf_lsm_solve per index,
 * then a final pass; tqf_lsm_gather first when the basis is structured.
 * tqf_lsm_price runs that whole sequence (structured mode) in one call.
 *
 * Structured mode (degree >= 0, strikes != NULL): exercise values are basket
 * puts relu(K_b - mean_d S) and the design is the centred tensor-product
 * polynomial basis of the given degree, both computed in the kernels from the
 * paths.  Explicit mode (degree < 0): the caller supplies exercise values
 * [N][B] and the design [Bp][G][N] for the two exercise dates of each pass.
 * Sums of the masked normal equations X'X, X'y are FP64; the pseudo-inverse
 * is an FP64 Jacobi eigen-decomposition with tf.linalg.pinv's cutoff
 * (10 G eps(dtype) x the largest eigenvalue). */
typedef struct tqf_lsm_args {
  int32_t dtype;             /* TQF_F32 / TQF_F64: paths, strikes, discounts, payoffs, design, state */
  int32_t dim;               /* d <= 16 (structured mode) */
  int64_t num_paths;         /* N */
  int32_t num_times;         /* T: time axis of the paths */
  int32_t paths_batch;       /* Bp: 1 for paths [N][T][d], B for [B][N][T][d] */
  int32_t batch;             /* B: payoff batch (strikes) */
  int32_t num_basis;         /* G <= 128 basis functions ((degree + 1)^d when structured) */
  int32_t degree;            /* >= 0: structured polynomial basis; < 0: explicit design */
  int32_t num_exercise;      /* E */
  int64_t num_calibration;   /* > 0: regress on paths [0, n), price on [n, N); 0: all paths */
  const void* paths;         /* [Bp][N][T][d] contiguous (structured mode) */
  const void* strikes;       /* [B] (structured mode) */
  const int32_t* exponents;  /* device [G][d] exponent grid (structured mode) */
  const int32_t* exercise_times; /* device [E] time indices into the paths */
  const void* discount;      /* D[E+1][Nd][Bd] with D[0] = 1 (lsm.py:258-272) */
  int64_t disc_stride_e, disc_stride_n, disc_stride_b; /* elements; 0 broadcasts */
  void* state;               /* [2][B][N]: cashflow, option values (dtype) */
  int32_t init;              /* 1: cashflow = payoff at exercise E-1, values = 0 */
  int32_t upd_index;         /* >= 1: apply the regression of this exercise index first */
  int32_t acc_index;         /* >= 1: accumulate the normal equations of this exercise index */
  int32_t final_pass;        /* 1: out[b] = sum over priced paths of D[1]/D[0] (cashflow + values) */
  const void* init_payoff;   /* explicit mode: [N][B] at exercise E-1 */
  const void* upd_payoff;    /* explicit mode: [N][B] at exercise upd_index - 1 */
  const void* upd_design;    /* explicit mode: [Bp][G][N] */
  const void* acc_payoff;
  const void* acc_design;
  double* out;               /* [B] (final pass) */
  void* workspace;
  size_t workspace_bytes;
  int32_t* dev_status;
} tqf_lsm_args;

/* Workspace for a given argument block (needs the CUDA device: sized by occupancy). */
TQF_API size_t tqf_lsm_workspace_bytes(const tqf_lsm_args* args);
/* Structured mode: copies the states at the exercise times into the workspace
 * ([Bp][E][N][d], one coalesced pass) and their column means (basis centring,
 * lsm.py:106-108). */
TQF_API int tqf_lsm_gather(const tqf_lsm_args* args, void* stream);
TQF_API int tqf_lsm_pass(const tqf_lsm_args* args, void* stream);
/* Solves beta = pinv(X'X) X'y per batch member from the last pass's sums. */
TQF_API int tqf_lsm_solve(const tqf_lsm_args* args, void* stream);
/* Structured mode, whole algorithm: out[b] = least_square_mc price of payoff b
 * (lsm.py:128-295).  The per-pass fields of args are ignored. */
TQF_API int tqf_lsm_price(const tqf_lsm_args* args, void* stream);

/* FP64 sums of European payoffs over values[p * stride] for p < num_values
 * (level model: S = spot_scale * values, or log model: S = spot_scale *
 * exp(values) when log_values != 0).  Same output layout as tqf_payoff. */
TQF_API int tqf_european_payoff_sums(int32_t dtype, const void* values, int64_t stride,
                             int64_t num_values, int32_t log_values,
                             const tqf_payoff* payoff, void* stream);

TQF_API size_t tqf_european_workspace_bytes(int64_t num_values, int32_t num_strikes);

/* Monte Carlo estimate from payoff sums (the [num_strikes][2] (sum, sum of
 * squares) output of the pricing calls): price_se[j] = discount * mean_j and
 * price_se[num_strikes + j] = discount * sqrt(var_j / n) with the unbiased
 * variance, all in FP64 on the device.  The reference's callers take the
 * discounted mean of payoff tensors themselves (e.g.
 * tff/models/heston/heston_model_test.py:349-352); this is that step as one
 * kernel. */
TQF_API int tqf_mc_price_stats(const double* sums, int32_t num_strikes, int64_t num_paths, double discount,
                               double* price_se, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TQF_H_ */
