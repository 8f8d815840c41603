// Internal declarations shared by the libcpals translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "cpals.h"

namespace cpals {

constexpr int kMaxOrder = CPALS_MAX_ORDER;
#define CPALS_MAX_RANK_SOLVE 512

// Device-resident state of a FitCheck / NoCheck (fit_check.jl:5-20, no_check.jl:1-9).
// The fit kernel updates it once per sweep, so sweeps can be replayed from a CUDA
// graph without a host round trip.  `done` makes the kernels of later sweeps return
// at once: the factors stay as they were at the converged sweep.
struct DevCheck {
  int kind;
  int iter;
  int counter;
  int max_counter;
  double tol;
  double ref_norm;
  double lastfit;
  double final_fit;
  int total_iter;
  int done;
  int nan_flag;
  int sweeps;  // sweeps whose check ran (index into the trajectory)
  long long fallbacks;  // pivoted-QR fallbacks taken by the normal-equation solve
  // CPDiffCheck / CPAngleCheck: norm_prev_iter, PrevCP !== nothing, and which of the two
  // previous-iterate buffers holds PrevCP (the other receives the current iterate)
  double norm_prev;
  int has_prev;
  int psel;
  // ||T||^2 of the handle's tensor as an unevaluated sum t2_hi + t2_lo, computed on the
  // device whenever the tensor is set (t2_valid = 0: not available, e.g. a non-finite entry)
  double t2_hi, t2_lo;
  int t2_valid;
  // The fit's terms from the last mode's update, as exact 128-bit fixed-point sums (lo, hi
  // words and the base, see Fx below): <T, X> (the saved MTTKRP against the new factor,
  // fit_check.jl:22-28) and ||X||^2 (converge_checks.jl:5-11).  terms_ready says they are
  // newer than the last check that read them.
  int terms_ready;
  int inner_base, fsq_base;
  unsigned long long inner_lo, fsq_lo;
  long long inner_hi, fsq_hi;
};

// ---- exact sums of doubles in 128-bit fixed point (integer pipe) ----
// GB300 issues FP64 at 2 operations per clock per SM with a dependent latency of some 128
// cycles, so compensated FP64 sums (chains of a dozen dependent operations per add) cost tens
// of microseconds on one SM.  Integer adds cost a few cycles.  A finite double
// v = +-m 2^(e - 1075) (m < 2^53, e = max(biased exponent, 1)) is added exactly as the integer
// m 2^(e - base) into a signed 128-bit accumulator whose unit is 2^(base - 1075); with
// base = e_max - 40 (e_max over the summed terms) the largest term stays below 2^93, so 2^34
// terms fit, and a term far below the largest drops its bits under 2^-92 of it.  The sums
// are exact otherwise, and independent of the order of the adds.
constexpr int kFxHead = 40;
constexpr int kFxBad = 4096;  // base marking a non-finite term: the sum is NaN
__device__ __forceinline__ int fx_exp(double v) {
  const int e = (int)((__double_as_longlong(v) >> 52) & 0x7ff);
  return e == 0 ? 1 : e;  // 0x7ff: non-finite
}
__device__ __forceinline__ __int128 fx_term(double v, int base) {
  const long long b = __double_as_longlong(v);
  const int eb = (int)((b >> 52) & 0x7ff);
  const unsigned long long m = (unsigned long long)(b & 0xFFFFFFFFFFFFFll) | (eb ? (1ull << 52) : 0ull);
  const int sh = (eb ? eb : 1) - base;
  __int128 t = 0;
  if (sh >= 0)
    t = (__int128)m << (sh < 80 ? sh : 80);
  else if (sh > -64)
    t = (__int128)(m >> (-sh));
  return (b < 0) ? -t : t;
}
__device__ __forceinline__ __int128 fx_shfl_xor(__int128 q, int off) {
  const unsigned long long lo = __shfl_xor_sync(0xffffffffu, (unsigned long long)q, off);
  const long long hi = __shfl_xor_sync(0xffffffffu, (long long)(q >> 64), off);
  return (__int128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}
__device__ __forceinline__ __int128 fx_warp_sum(__int128 q) {
  for (int off = 16; off > 0; off >>= 1) q += fx_shfl_xor(q, off);
  return q;
}
// q 2^(from - 1075) re-expressed in units of 2^(to - 1075), to >= from (low bits dropped)
__device__ __forceinline__ __int128 fx_align(__int128 q, int from, int to) {
  const int d = to - from;
  return d >= 127 ? (__int128)0 : (q >> d);
}
// q 2^(base - 1075) rounded to a double (two conversions and one add: within 2 ulps)
__device__ __forceinline__ double fx_to_double(__int128 q, int base) {
  const bool neg = q < 0;
  const unsigned __int128 a = neg ? (unsigned __int128)(-q) : (unsigned __int128)q;
  const double d = fma((double)(unsigned long long)(a >> 64), 18446744073709551616.0,
                       (double)(unsigned long long)a);
  return ldexp(neg ? -d : d, base - 1075);
}

// An unevaluated sum hi + lo (a double-double), as ||T||^2 is kept.
struct DD {
  double hi, lo;
};

struct FactorSet {
  const double* F[kMaxOrder];  // FP64 factors, row-major [I_n][R]
};
struct GramSet {
  const double* G[kMaxOrder];  // FP64 Grams, R x R
};

// Geometry of the MTTKRP of one mode.  The reduction index space (every mode but
// `mode`) is cut into chunks of `chunk` consecutive values of the fastest
// reduction mode `fmode` at fixed values of the other ("outer") reduction modes.
struct ModeGeom {
  int order, mode, fmode, n_outer;
  int outer_modes[kMaxOrder];
  int64_t dims[kMaxOrder];
  int64_t strides[kMaxOrder];  // element strides of the column-major tensor
  int64_t In, If, nfb, nchunks;
};

inline ModeGeom make_geom(int order, const int64_t* dims, int mode, int64_t chunk, const int64_t* fdims = nullptr) {
  ModeGeom g{};
  g.order = order;
  g.mode = mode;
  int64_t s = 1;
  for (int m = 0; m < order; ++m) {
    g.dims[m] = dims[m];
    g.strides[m] = s;
    s *= dims[m];
  }
  g.fmode = (mode == 0) ? 1 : 0;
  g.In = dims[mode];
  g.If = fdims ? fdims[g.fmode] : dims[g.fmode];
  g.nfb = (g.If + chunk - 1) / chunk;
  g.n_outer = 0;
  int64_t outer = 1;
  for (int m = 0; m < order; ++m) {
    if (m == mode || m == g.fmode) continue;
    g.outer_modes[g.n_outer++] = m;
    outer *= dims[m];
  }
  g.nchunks = g.nfb * outer;
  return g;
}

// A grid-wide barrier for cooperative launches (sense-reversing: `count` is back at zero
// after every barrier, `gen` counts them).  Zero-initialised once.
struct GridBar {
  unsigned count;
  unsigned gen;
};

// Status of one normal-equation factorisation (written by the factorize kernel).
struct SolveInfo {
  int rank;      // rank reached by the pivoted Cholesky
  int fallback;  // 1 if the pivoted-QR path produced the solve operator
  int qr_rank;   // numerical rank found by the QR path
  int refine;    // 1: the FP32 sweep's inverse W and V = V_hi + V_lo (FP32) are in the
                 // workspace; the solve refines X once with the residual M - X V
  int swept;     // 1: the cluster sweep factorised V at full rank (W, U, dinv, piv written)
};

// ---- launchers (defined in the kernel translation units) ----

// FP64 MTTKRP partials: part[split][In][R] (FP64).
int mttkrp_f64_splits(const ModeGeom& g, int64_t R, int num_sms, int64_t* chunks_per_split);
cudaError_t launch_mttkrp_f64(const void* T, int tdtype, const FactorSet& fs, const ModeGeom& g, int64_t R,
                              int splits, int64_t chunks_per_split, double* part, const DevCheck* chk,
                              cudaStream_t st);

// V = Hadamard of the Grams of every mode but `skip`; pivoted Cholesky (upper,
// tol 1e-6) with a column-pivoted QR fallback.  Single CTA.
// mixed = 1 (split-BF16 path, R <= 128): the sweep runs in FP32 first, and the FP64 sweep
// only if the FP32 pivots signal ill-conditioning (info->refine tells the solve which).
cudaError_t launch_factorize(const GramSet& gs, int order, int skip, int R, double* work, double* U, int* piv,
                             double* W, SolveInfo* info, DevCheck* chk, cudaStream_t st, int mixed = 0);
size_t factorize_work_doubles(int R);
// kernels one launch_factorize issues; the cluster size of the FP64 sweep at rank R (0: one
// CTA); the smallest rank given to the cluster sweep (process-wide, returns the previous)
int factorize_launches(int R, int mixed);
int cluster_sweep_size(int R);
int cluster_sweep_device_size();  // the current device's cluster size, whatever the rank
int set_cluster_sweep_min_rank(int r);

// Reduce the MTTKRP partials, solve X = M V^{-1} one warp per row, write X and
// (optionally) per-row sums of M .* X for the fit, exact in fixed point (three words per row).  `work` is the factorize workspace.
// With gram_part, every block also writes its rows' share of G = X^T X (upper triangle,
// R(R+1)/2 doubles per block, solve_blocks(In, R) blocks) for launch_gram_rows.
cudaError_t launch_solve_rows(const void* part, int part_is_f32, int splits, int64_t In, int R, const double* work,
                              const double* U, const int* piv, const double* W, const SolveInfo* info, double* X,
                              double* inner_rows, const DevCheck* chk, cudaStream_t st, double* gram_part = nullptr);
int solve_blocks(int64_t In, int R);
// G (Graw) from the solve blocks' partial Grams, then launch_finalize's work in the last
// block (without G_n, which launch_normalize writes); gram_part needs room for
// nblk * R(R+1)/2 + (R(R+1)/2 + 31)/32 doubles; counter: one zeroed unsigned.
// run_check = 0 leaves the check's update to launch_check_step (a caller-driven sweep).
cudaError_t launch_gram_rows(const double* gram_part, int nblk, int R, unsigned* counter, double* Graw, double* lam,
                             double* lam_inv, double* Gn, const GramSet& gs, int order, int last,
                             const double* inner_rows, int64_t In, DevCheck* chk, double* traj, int64_t traj_cap,
                             cudaStream_t st, int run_check = 1);
// Room in gram_part: nblk * R(R+1)/2 doubles of partial Grams, then three words per block of
// launch_gram_rows for the ||X||^2 shares (exact fixed-point sums).
size_t gram_rows_part_doubles(int nblk, int R);

// G = X^T X (row-major X, In x R) over S2 row splits; part: gram_tiles(R)*S2*256 doubles,
// counters: gram_tiles(R)+1 zero-initialised unsigneds (left zeroed after each launch).
int gram_tiles(int R);
int gram_splits(int64_t In, int R, int num_sms);
cudaError_t launch_gram(const double* X, int64_t In, int R, int S2, double* part, unsigned* counters, double* G,
                        const DevCheck* chk, cudaStream_t st);

// launch_gram followed, in the last block to finish, by launch_finalize's work on Graw
// (without G_n, which launch_normalize then writes).  part needs gram_tiles(R)*(S2*256+1)
// doubles.
cudaError_t launch_gram_finalize(const double* X, int64_t In, int R, int S2, double* part, unsigned* counters,
                                 double* Graw, double* lam, double* lam_inv, double* Gn, const GramSet& gs, int order,
                                 int last, const double* inner_rows, DevCheck* chk, double* traj, int64_t traj_cap,
                                 cudaStream_t st, int run_check = 1);
// Room in part for launch_gram_finalize: the tile partials and three words per tile.
size_t gram_finalize_part_doubles(int S2, int R);

// The check's update (FitCheck / NoCheck) from the terms the last mode's update saved in
// chk, as the fused finalize runs it; one thread.
cudaError_t launch_check_step(DevCheck* chk, double* traj, int64_t traj_cap, cudaStream_t st);

// ||T||^2 as a double-double into chk->t2_hi / t2_lo (t2_valid = 1), for the fit.  Two
// passes: the largest |entry|, then the squares summed exactly in 128-bit fixed point
// anchored at it (FP32 entries: m^2 is an exact 48-bit integer; FP64 entries: each square
// split exactly by TwoProduct, both parts added).  scratch: norm2_scratch_doubles() doubles.
size_t norm2_scratch_doubles();
cudaError_t launch_tensor_norm2(const void* T, int tdtype, int64_t n, double* scratch, DevCheck* chk, int num_sms,
                                cudaStream_t st);

// lambda = sqrt(diag Graw), G_n = Graw ./ (lambda lambda^T); on the last mode also the fit
// and the device check update (trajectory entry per sweep).  inner_rows holds two doubles
// per row: an exact fixed-point row sum (lo, hi words and its base).
cudaError_t launch_finalize(const double* Graw, int R, double* lam, double* lam_inv, double* Gn, const GramSet& gs,
                            int order, int last, const double* inner_rows, int64_t In, DevCheck* chk, double* traj,
                            int64_t traj_cap, cudaStream_t st);

// Where the tensor-core MTTKRP keeps the BF16 hi/lo tiles of a factor that is its fastest
// reduction mode: tiles of nb columns x 64 rows, hi plane then lo plane, 128-byte rows
// swizzled in 16-byte chunks (chunk c of row r at (c ^ (r & 7)) * 16).
struct BtileDesc {
  uint8_t* bt;   // null: no tiles
  int nb;        // columns per tile
  int n_blocks;  // column tiles
};

// F = X .* (1 ./ lambda) (lam_inv may be null: plain copy), (when F32r is non-null) an
// FP32 row-major copy [In][rpad], (when Gn is non-null) the normalised Gram
// Gn = Graw ./ (lambda lambda^T), (when bt.bt is non-null) the BF16 factor tiles and (when
// F32lo is non-null) the FP32 remainder F - (float)F in the F32r layout.
cudaError_t launch_normalize(const double* X, const double* lam_inv, int64_t In, int R, double* F, float* F32r,
                             int64_t rpad, const double* Graw, double* Gn, const DevCheck* chk, cudaStream_t st,
                             BtileDesc bt = BtileDesc{nullptr, 0, 0}, float* F32lo = nullptr);

// The mode's tail in one cooperative launch: the solve, the Gram, lambda, the new factor (and
// its FP32 / BF16 copies), G_n, and on the last mode the fit (and the check when run_check).
// gram_part: mode_tail_part_doubles(solve_blocks(In, R), R) doubles; bar: a zeroed GridBar;
// err: set when a grid barrier's bounded wait expired.  cudaErrorNotSupported when the
// blocks cannot all be resident: the caller runs launch_solve_rows, launch_gram_rows and
// launch_normalize instead.
cudaError_t launch_mode_tail(const void* part, int part_is_f32, int splits, int64_t In, int R, const double* work,
                             const double* W, const SolveInfo* info, double* X, double* gram_part, double* F,
                             float* F32r, float* F32lo, int64_t rpad, BtileDesc btd, double* Graw, double* lam,
                             double* lam_inv, double* Gn, const GramSet& gs, int order, int last,
                             const double* inner_rows, DevCheck* chk, double* traj, int64_t traj_cap, GridBar* bar,
                             int* err, int num_sms, int run_check, cudaStream_t st);
size_t mode_tail_part_doubles(int nblk, int R);

// Row-major rows x cols -> row-major cols x rows (FP64).
cudaError_t launch_transpose_f64(const double* src, int64_t rows, int64_t cols, double* dst, cudaStream_t st);

// Reduce MTTKRP partials to a row-major FP64 M (for cpals_mttkrp).
cudaError_t launch_reduce_partials(const void* part, int part_is_f32, int splits, int64_t In, int R, double* M,
                                   cudaStream_t st);

// ---- gathers (k_gather.cu) ----
cudaError_t launch_pivot_hadamard(const FactorSet& fs, int order, int mode, const int64_t* dims,
                                  const int64_t* piv, int64_t nsamps, int R, double* out, int* err, cudaStream_t st);
cudaError_t launch_fibers(const void* T, int tdtype, int order, int mode, const int64_t* dims, const int64_t* piv,
                          int64_t nsamps, void* out, int* err, cudaStream_t st);
cudaError_t launch_colmajor_to_rowmajor(const double* src, int64_t rows, int R, double* dst, cudaStream_t st);
// The sampled system's products as compensated FP32 (Dot2) sums: G = S^T S from the column-major
// nsamps x R S (split into pairs Spair), and the split-K partials part[splits][In][R] of T_s S
// (T_s column-major In x nsamps, FP32 or FP64; Tpair: In x nsamps pairs for FP64 T_s).  part:
// sampled_splits(nsamps) x max(R, In) x R doubles.
int sampled_splits(int64_t nsamps);
cudaError_t launch_sampled_gram(const double* Scol, int64_t nsamps, int R, float2* Spair, double* part, double* G,
                                cudaStream_t st);
cudaError_t launch_sampled_rhs(const void* Ts, int tdtype, int64_t In, int64_t nsamps, int R, const float2* Spair,
                               float2* Tpair, double* part, int* splits_out, cudaStream_t st);
cudaError_t launch_leverage_rows(const double* F, int64_t In, int R, const double* work, const double* U,
                                 const int* piv, const SolveInfo* info, double scale, double* probs, cudaStream_t st);

// CPDiffCheck / CPAngleCheck on the current iterate (k_cpcheck.cu).  The previous iterate
// lives in prevF[psel] / prevLam[psel] (DevCheck::psel); the current one is copied into the
// other buffer by the same launches.
struct CrossArgs {
  const double* F[kMaxOrder];  // current factors, row-major [I_m][R]
  const double* G[kMaxOrder];  // their Grams F_m^T F_m
  const double* lam;
  double* prevF[2];            // modes concatenated, row-major, mode m at off[m]
  double* prevLam[2];
  int64_t dims[kMaxOrder];
  int64_t off[kMaxOrder];
  int order, R;
  int64_t rows;                // rows of one split
  int S[kMaxOrder];            // splits of mode m: ceil(I_m / rows)
  int Smax;
  double* xpart;               // [order][Smax][R][R] partial cross Grams P_m^T F_m
  double* red;                 // two doubles per block of the check kernel
  unsigned* counter;           // zero between launches
  DevCheck* chk;
  double* traj;
  int64_t traj_cap;
};
// Rows of one cross-Gram split (a multiple of 8) for about six blocks per SM.
int64_t cross_rows(int order, const int64_t* dims, int R, int num_sms);
// Two launches: the split cross Grams (and the copy of the iterate), then the check.
cudaError_t launch_cp_check(const CrossArgs& a, cudaStream_t st);

// Sparse sign embedding (k_sketch.cu): n columns of zeta (row, +-1/sqrt(zeta)) entries.
cudaError_t launch_sparse_sign(int64_t l, int64_t n, int zeta, int injective, uint64_t seed, int32_t* rows,
                               double* vals, cudaStream_t st);
// out (In x l, column-major) = sum over each output column's entries p (seg[j] .. seg[j+1])
// of v[p] times the fibre starting at T[pos[p]] with element stride `stride`.
cudaError_t launch_sketch_gather(const void* T, int tdtype, int64_t In, int64_t stride, const int64_t* seg,
                                 const int64_t* pos, const double* v, int64_t l, double* out, cudaStream_t st);

// Column-pivoted QR (k_qrcp.cu).  A (m x n, column-major FP64) is factored in place; pivots
// are chosen among columns [0, ncand); at most kmax steps, fewer when a step's |r_jj| is at
// most stop_ratio |r_00| (stop_ratio < 0: never).  part holds qrcp_parts(n) entries.
struct QrcpArg {
  double v;
  int64_t i;
};
struct QrcpState {
  double r00, tau;
  int64_t steps;   // steps run
  int64_t active;  // j + 1 for the step whose reflector is current
  int done, pad;
};
struct KrpDims {
  int64_t dims[kMaxOrder];
};
struct QrcpJob {
  double* A;
  int64_t m, n, ncand, kmax;
  double stop_ratio;
  double *vn1, *vn2, *vbuf, *taus, *rdiag;
  int64_t* perm;  // 0-based original column of each position
  QrcpArg* part;
  QrcpState* st;
  int num_sms;
};
int qrcp_parts(int64_t n, int num_sms);
cudaError_t launch_qrcp_init(const QrcpJob& q, cudaStream_t st);
cudaError_t launch_qrcp_step(const QrcpJob& q, int64_t j, cudaStream_t st);
// Q (m x k) = H_0 ... H_{k-1} [I; 0] from the factored A and its taus.
cudaError_t launch_qr_form_q(const double* A, int64_t m, int64_t k, const double* taus, double* Q, int num_sms,
                             cudaStream_t st);
// out (In x ncols) = the columns cols (0-based, identity when null) of the mode unfolding whose
// fibres start at (col / stride) stride In + col % stride with element stride `stride`.
cudaError_t launch_unfold_cols(const void* T, int tdtype, int64_t In, int64_t stride, const int64_t* cols,
                               int64_t ncols, double* out, cudaStream_t st);
// out (R x ncols) = rows cols of the Khatri-Rao product of the factors other than `mode`, transposed.
cudaError_t launch_krp_cols(const FactorSet& fs, int order, int mode, const int64_t* dims, const int64_t* cols,
                            int64_t ncols, int R, double* out, cudaStream_t st);
// out[r sr + j sj] = sum over Omega's row j (entries seg[j] .. seg[j+1]) of v[p] KRP(cols[p], r).
cudaError_t launch_omega_hadamard(const FactorSet& fs, int order, int mode, const int64_t* dims, const int64_t* seg,
                                  const int64_t* cols, const double* v, int64_t l, int R, double* out, int64_t sr,
                                  int64_t sj, cudaStream_t st);

// Makes `dev` the current device for the scope of an entry point and restores the
// caller's device on exit, so a call never leaves another device current.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// Raises a kernel's dynamic shared-memory limit on the current device, once per (device,
// kernel) per process (thread-safe).  The attribute is per device, so a process that drives
// several GPUs sets it on each.
cudaError_t set_smem_limit_once(const void* kernel, int bytes);

}  // namespace cpals

#define CPALS_CUDA_TRY(expr)                                                            \
  do {                                                                                   \
    cudaError_t _e = (expr);                                                             \
    if (_e != cudaSuccess) {                                                             \
      fprintf(stderr, "libcpals: %s failed: %s (%s:%d)\n", #expr, cudaGetErrorString(_e), \
              __FILE__, __LINE__);                                                       \
      return CPALS_E_CUDA;                                                               \
    }                                                                                    \
  } while (0)
