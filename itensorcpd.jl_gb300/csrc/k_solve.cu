// FP64 normal-equation kernels of one ALS mode update:
//   factorize  : V = Hadamard of the other modes' Grams (compute_krp,
//                MttkrpAlgorithm.jl:18-31); pivoted Cholesky P^T V P = U^T U with
//                LAPACK dpstrf's stopping rule (pivot <= 1e-6 or NaN -> rank deficient,
//                ldiv_solve.jl:17-18); on rank deficiency a column-pivoted Householder QR
//                gives the least-squares operator instead (ldiv_solve.jl:19-21).
//   solve_rows : reduce the MTTKRP split-K partials, X = M V^{-1} one warp per row
//                (solve_ls_problem, MttkrpAlgorithm.jl:34-41), partial sums of M .* X
//                for the fit.
//   gram       : X^T X by 16x16 tiles of the upper triangle over row splits, each tile
//                reduced by its last block in split order (deterministic).
//   finalize   : lambda = column norms (row_norm.jl:4-24), G_n = F_n^T F_n (post_solve,
//                standard/tensor.jl:22-25, 46-49); after the last mode the fit and the
//                FitCheck / NoCheck update (fit_check.jl:24-66, no_check.jl:11-19).
//   normalize  : F_n = X ./ lambda, plus the FP32 column-major copy the tensor-core
//                MTTKRP reads.
// FP64 runs at under 2 FMA/clk/SM on GB300, so every O(I_n R^2) piece is spread over many
// CTAs; the O(R^3) factorisation is a single CTA below rank 40 and a 16-CTA cluster from 40
// to 256, and it runs on a side stream concurrently with the MTTKRP of the same mode.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <map>
#include <mutex>

#include "cpals_internal.cuh"

namespace cpals {
namespace {

constexpr double kCholTol = 1e-6;  // src/ITensorCPD.jl:2 cholesky_epsilon
// Factorize threads.  FP64 on this part issues at a low rate per warp (2 DFMA/clk/SM at
// best, 128-cycle latency): the single-CTA factorisation needs many warps per scheduler
// to keep the FP64 pipes busy (a 2016-FMA sweep step: ~3200 cycles at 256 threads,
// ~1400 at 1024).
constexpr int FT = 1024;

__device__ __forceinline__ bool done_flag(const DevCheck* chk) { return chk != nullptr && chk->done; }

// block-wide argmax with first-index tie break; NaN is treated as +inf so it is picked
// (and then rejected by the stopping test, like DISNAN in dpstf2).
__device__ void block_argmax(double v, int idx, double* sv, int* si, double* out_v, int* out_i) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double key = isnan(v) ? INFINITY : v;
  for (int off = 16; off > 0; off >>= 1) {
    double ok = __shfl_down_sync(0xffffffffu, key, off);
    int oi = __shfl_down_sync(0xffffffffu, idx, off);
    double ov = __shfl_down_sync(0xffffffffu, v, off);
    if (ok > key || (ok == key && oi < idx)) {
      key = ok;
      idx = oi;
      v = ov;
    }
  }
  if (lane == 0) {
    sv[w] = v;
    si[w] = idx;
  }
  __syncthreads();
  if (w == 0) {
    v = lane < nw ? sv[lane] : -INFINITY;
    idx = lane < nw ? si[lane] : 0x7fffffff;
    key = isnan(v) ? INFINITY : v;
    for (int off = 16; off > 0; off >>= 1) {
      double ok = __shfl_down_sync(0xffffffffu, key, off);
      int oi = __shfl_down_sync(0xffffffffu, idx, off);
      double ov = __shfl_down_sync(0xffffffffu, v, off);
      if (ok > key || (ok == key && oi < idx)) {
        key = ok;
        idx = oi;
        v = ov;
      }
    }
    if (lane == 0) {
      *out_v = v;
      *out_i = idx;
    }
  }
  __syncthreads();
}

__device__ double block_sum(double v, double* sv) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  __syncthreads();
  if (lane == 0) sv[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < nw; ++i) t += sv[i];
  __syncthreads();
  if (threadIdx.x == 0) sv[0] = t;
  __syncthreads();
  t = sv[0];
  __syncthreads();
  return t;
}

// Column-pivoted Householder QR of V (R x R) and the least-squares operator W with
// X^T = W M^T.  Rank is cut where |R_kk| <= R * eps * |R_00| (Julia's QRPivoted ldiv!
// uses rcond = min(m,n) * eps); a rank-deficient system gets the minimum-norm solution.
__device__ void qr_fallback(const GramSet& gs, int order, int skip, int R, double* __restrict__ B,
                            double* __restrict__ Z, double* __restrict__ Y, double* __restrict__ tau,
                            int* __restrict__ perm, double* __restrict__ W, SolveInfo* info, double* sv, int* si,
                            double* cn) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int e = tid; e < R * R; e += blockDim.x) {
    double v = 1.0;
    for (int m = 0; m < order; ++m)
      if (m != skip) v *= gs.G[m][e];
    B[e] = v;
  }
  for (int k = tid; k < R; k += blockDim.x) perm[k] = k;
  __syncthreads();
  __shared__ double s_bv, s_tau, s_beta;
  __shared__ int s_p;
  for (int j = 0; j < R; ++j) {
    // column norms of the trailing block
    for (int k = j + warp; k < R; k += nw) {
      double s = 0.0;
      for (int i = j + lane; i < R; i += 32) s += B[i * R + k] * B[i * R + k];
      for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
      if (lane == 0) cn[k] = s;
    }
    __syncthreads();
    double bv = -INFINITY;
    int bi = 0x7fffffff;
    for (int k = j + tid; k < R; k += blockDim.x) {
      double c = cn[k];
      double key = isnan(c) ? INFINITY : c, bkey = isnan(bv) ? INFINITY : bv;
      if (key > bkey || (key == bkey && k < bi)) {
        bv = c;
        bi = k;
      }
    }
    double outv;
    int outi;
    block_argmax(bv, bi, sv, si, &outv, &outi);
    if (tid == 0) s_p = outi;
    __syncthreads();
    const int p = s_p;
    if (p != j) {
      for (int i = tid; i < R; i += blockDim.x) {
        double t = B[i * R + j];
        B[i * R + j] = B[i * R + p];
        B[i * R + p] = t;
      }
      if (tid == 0) {
        int t = perm[j];
        perm[j] = perm[p];
        perm[p] = t;
      }
    }
    __syncthreads();
    // Householder reflector for x = B[j:, j] (dlarfg convention)
    double sg = 0.0;
    for (int i = j + 1 + tid; i < R; i += blockDim.x) sg += B[i * R + j] * B[i * R + j];
    sg = block_sum(sg, sv);
    if (tid == 0) {
      const double alpha = B[j * R + j];
      double t = 0.0, beta = alpha, vs = 0.0;
      if (sg > 0.0 || isnan(sg)) {
        beta = -copysign(sqrt(alpha * alpha + sg), alpha);
        t = (beta - alpha) / beta;
        vs = 1.0 / (alpha - beta);
      }
      s_tau = t;
      s_beta = beta;
      s_bv = vs;
      tau[j] = t;
    }
    __syncthreads();
    const double tj = s_tau, scale = s_bv;
    for (int i = j + 1 + tid; i < R; i += blockDim.x) B[i * R + j] *= scale;
    __syncthreads();
    if (tid == 0) B[j * R + j] = s_beta;
    // apply H = I - tau v v^T (v_j = 1) to the trailing columns
    if (tj != 0.0) {
      for (int k = j + 1 + warp; k < R; k += nw) {
        double w = (lane == 0) ? B[j * R + k] : 0.0;
        for (int i = j + 1 + lane; i < R; i += 32) w += B[i * R + j] * B[i * R + k];
        for (int off = 16; off > 0; off >>= 1) w += __shfl_down_sync(0xffffffffu, w, off);
        w = __shfl_sync(0xffffffffu, w, 0) * tj;
        if (lane == 0) B[j * R + k] -= w;
        for (int i = j + 1 + lane; i < R; i += 32) B[i * R + k] -= w * B[i * R + j];
      }
    }
    __syncthreads();
  }
  // numerical rank
  __shared__ int s_rnk;
  if (tid == 0) {
    const double r00 = fabs(B[0]), rcond = (double)R * 2.220446049250313e-16;
    int rnk = 1;
    while (rnk < R && fabs(B[rnk * R + rnk]) > rcond * r00) ++rnk;
    if (!(r00 > 0.0)) rnk = 0;
    s_rnk = rnk;
    info->qr_rank = rnk;
  }
  __syncthreads();
  const int rnk = s_rnk;
  // Z = Q^T = H_{R-1} ... H_0 I
  for (int e = tid; e < R * R; e += blockDim.x) Z[e] = ((e / R) == (e % R)) ? 1.0 : 0.0;
  __syncthreads();
  for (int j = 0; j < R; ++j) {
    const double tj = tau[j];
    if (tj != 0.0) {
      for (int k = warp; k < R; k += nw) {
        double w = (lane == 0) ? Z[j * R + k] : 0.0;
        for (int i = j + 1 + lane; i < R; i += 32) w += B[i * R + j] * Z[i * R + k];
        for (int off = 16; off > 0; off >>= 1) w += __shfl_down_sync(0xffffffffu, w, off);
        w = __shfl_sync(0xffffffffu, w, 0) * tj;
        if (lane == 0) Z[j * R + k] -= w;
        for (int i = j + 1 + lane; i < R; i += 32) Z[i * R + k] -= w * B[i * R + j];
      }
    }
    __syncthreads();
  }
  if (rnk == R) {
    // Y = R^{-1} Z, back substitution column by column (columns in parallel)
    for (int c = tid; c < R; c += blockDim.x) {
      for (int k = R - 1; k >= 0; --k) {
        double s = Z[k * R + c];
        for (int l = k + 1; l < R; ++l) s -= B[k * R + l] * Y[l * R + c];
        Y[k * R + c] = s / B[k * R + k];
      }
    }
  } else if (rnk > 0) {
    // minimum-norm: Y = Rt^T (Rt Rt^T)^{-1} Z[0:rnk, :], Rt = upper rows 0..rnk-1 of R.
    double* S = tau + R;  // rnk x rnk scratch after tau (sized R*R in the workspace)
    for (int e = tid; e < rnk * rnk; e += blockDim.x) {
      const int a = e / rnk, b = e % rnk;
      double s = 0.0;
      for (int l = max(a, b); l < R; ++l) s += B[a * R + l] * B[b * R + l];
      S[e] = s;
    }
    __syncthreads();
    // Cholesky S = L L^T (lower, in place), serial over columns
    for (int j = 0; j < rnk; ++j) {
      if (tid == 0) {
        double d = S[j * rnk + j];
        for (int l = 0; l < j; ++l) d -= S[j * rnk + l] * S[j * rnk + l];
        S[j * rnk + j] = sqrt(fmax(d, 0.0));
      }
      __syncthreads();
      for (int i = j + 1 + tid; i < rnk; i += blockDim.x) {
        double s = S[i * rnk + j];
        for (int l = 0; l < j; ++l) s -= S[i * rnk + l] * S[j * rnk + l];
        S[i * rnk + j] = s / S[j * rnk + j];
      }
      __syncthreads();
    }
    // Z1 = S^{-1} Z[0:rnk,:] (columns in parallel), stored in Z rows 0..rnk-1
    for (int c = tid; c < R; c += blockDim.x) {
      for (int k = 0; k < rnk; ++k) {
        double s = Z[k * R + c];
        for (int l = 0; l < k; ++l) s -= S[k * rnk + l] * Z[l * R + c];
        Z[k * R + c] = s / S[k * rnk + k];
      }
      for (int k = rnk - 1; k >= 0; --k) {
        double s = Z[k * R + c];
        for (int l = k + 1; l < rnk; ++l) s -= S[l * rnk + k] * Z[l * R + c];
        Z[k * R + c] = s / S[k * rnk + k];
      }
    }
    __syncthreads();
    for (int e = tid; e < R * R; e += blockDim.x) {
      const int k = e / R, c = e % R;
      double s = 0.0;
      for (int a = 0; a < rnk && a <= k; ++a) s += B[a * R + k] * Z[a * R + c];
      Y[e] = s;
    }
  } else {
    for (int e = tid; e < R * R; e += blockDim.x) Y[e] = NAN;
  }
  __syncthreads();
  // operator (P Y), stored transposed: X = M W^T reads W^T[c][perm[k]] = Y[k][c]
  for (int e = tid; e < R * R; e += blockDim.x) {
    const int k = e / R, c = e % R;
    W[(size_t)c * R + perm[k]] = Y[e];
  }
  __syncthreads();
}

// Pivot search keys without FP64 instructions (a dependent FP64 compare costs ~150
// cycles here): the bit pattern of a double read as a signed 64-bit integer orders all
// non-negative values like the doubles, puts +NaN above +inf, and puts every negative
// value below zero.  A negative value can never pass the stopping test, so its order
// among the other negatives does not matter.
// A NaN of either sign maps to the largest key, so that it is picked and then stops the
// factorisation (dpstrf's DISNAN test).
__device__ __forceinline__ long long pivot_key(double v) {
  const long long k = __double_as_longlong(v);
  return (k & 0x7fffffffffffffffll) > 0x7ff0000000000000ll ? LLONG_MAX : k;
}
__device__ __forceinline__ bool key_is_nan(long long k) { return k == LLONG_MAX; }

__global__ void __launch_bounds__(FT) k_factorize(GramSet gs, int order, int skip, int R, double* __restrict__ Aglob,
                                                  double* __restrict__ U, double* __restrict__ dinv,
                                                  int* __restrict__ piv, double* __restrict__ W,
                                                  double* __restrict__ qwork, SolveInfo* info, DevCheck* chk,
                                                  int mixed, int clustered) {
  if (done_flag(chk)) return;
  if (mixed && info->refine) return;     // the FP32 sweep produced W
  if (clustered && info->swept) return;  // the cluster sweep produced W and U at full rank
  if (threadIdx.x == 0) info->refine = 0;
  extern __shared__ double smA[];
  // an odd leading dimension in shared memory keeps column accesses free of bank conflicts
  const int ld = (R <= 128) ? (R | 1) : R;
  double* A = (R <= 128) ? smA : Aglob;
  __shared__ double sv[32];
  __shared__ int si[32];
  __shared__ int s_piv[CPALS_MAX_RANK_SOLVE];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // V = ones .* G_a .* G_b ... (mode order, skipping `skip`); upper triangle only.  Eight
  // elements per thread step, so that their Gram loads are in flight together.
  for (int e0 = tid; e0 < R * R; e0 += 8 * FT) {
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = 1.0;
    for (int m = 0; m < order; ++m) {
      if (m == skip) continue;
      const double* __restrict__ G = gs.G[m];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int e = e0 + q * FT;
        if (e < R * R) v[q] *= G[e];
      }
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = e0 + q * FT;
      if (e < R * R) {
        const int r = e / R, c = e - r * R;
        if (c >= r) A[r * ld + c] = v[q];
      }
    }
  }
  for (int k = tid; k < R; k += blockDim.x) s_piv[k] = k;
  __syncthreads();

  // Pivoted symmetric sweep (Gauss-Jordan on the symmetric matrix, Goodnight 1979):
  // sweeping index k replaces A by
  //   A(i,j) - A(i,k) A(k,j) / d,  A(i,k) / d,  -1/d        (i, j != k; d = A(k,k)).
  // The unswept block always holds the Schur complement of the swept one, so its
  // diagonal is the one dpstrf (pivoted Cholesky, tol 1e-6) picks its pivots from: the
  // pivot sequence, the rank and the stopping rule are dpstrf's.  After all R indices
  // are swept, A = -V^{-1}: the solve operator comes out of the same R steps, with no
  // interchanges and no separate triangular inversion.  The rows of the Cholesky factor
  // U (needed by the leverage scores) are the Schur rows at each step, divided by the
  // square root of the pivot; they are kept unscaled and finished after the loop.
  __shared__ double s_a[CPALS_MAX_RANK_SOLVE];  // pivot row before the step
  __shared__ double s_t[CPALS_MAX_RANK_SOLVE];  // pivot row divided by the pivot
  __shared__ double s_dp[CPALS_MAX_RANK_SOLVE]; // pivot values in step order
  __shared__ unsigned char s_swept[CPALS_MAX_RANK_SOLVE];
  __shared__ double s_pv, s_pinv;               // next pivot value and its reciprocal
  __shared__ int s_p, s_stop;                   // next pivot index, stop flag
  double* Uo = qwork;                           // unscaled Schur rows, [step][original index]
  for (int k = tid; k < R; k += blockDim.x) s_swept[k] = 0;
  // Pivot search (warp 0) over the unswept diagonal entries offered by each lane.  The
  // largest wins, first index on ties (LAPACK MAXLOC); the 64-bit key is reduced as its
  // signed high word, then its low word among the lanes holding the maximum high word,
  // then the smallest index among the lanes holding the maximum key.  Lane 0 publishes
  // the pivot and its reciprocal, or the stop flag (pivot <= tol or NaN, dpstrf's rule).
  auto pick_pivot = [&](long long bk, int bi) {
    const int khi = (int)(bk >> 32);
    const int mhi = __reduce_max_sync(0xffffffffu, khi);
    const unsigned mlo = __reduce_max_sync(0xffffffffu, khi == mhi ? (unsigned)(bk & 0xffffffffll) : 0u);
    const long long mk = (long long)(((unsigned long long)(unsigned)mhi << 32) | mlo);
    const int p = __reduce_min_sync(0xffffffffu, (bi < R && bk == mk) ? bi : INT_MAX);
    if (lane == 0) {
      // for a non-NaN key, the pivot exceeds tol exactly when its key exceeds the key of
      // tol (a negative value has a negative key)
      const int stop = key_is_nan(mk) || !(mk > pivot_key(kCholTol));
      s_stop = stop;
      s_p = p;
      if (!stop) {
        const double pv = __longlong_as_double(mk);
        s_pv = pv;
        s_pinv = 1.0 / pv;
      }
    }
    __syncwarp();  // warp 0 meets the block barrier converged
  };
  __syncthreads();
  if (warp == 0) {
    long long bk = LLONG_MIN;
    int bi = R;
    for (int i = lane; i < R; i += 32) {
      const long long key = pivot_key(A[i * ld + i]);
      if (bi == R || key > bk) {  // i increases: strict > keeps the first index on ties
        bk = key;
        bi = i;
      }
    }
    pick_pivot(bk, bi);
  }
  __syncthreads();

  int rank = R;
  for (int j = 0; j < R; ++j) {
    if (s_stop) {
      rank = j;
      break;
    }
    const int k = s_p;
    const double dk = s_pinv;
    // snapshot of the pivot row (upper storage: A(k,i) sits at (min, max)); the unswept
    // part of it is row j of U times sqrt(pivot)
    for (int i = tid; i < R; i += blockDim.x) {
      const double a = (i <= k) ? A[i * ld + k] : A[k * ld + i];
      s_a[i] = a;
      s_t[i] = a * dk;
      Uo[(size_t)j * R + i] = (s_swept[i] || i == k) ? 0.0 : a;
    }
    if (tid == 0) {
      s_piv[j] = k;
      s_dp[j] = s_pv;
    }
    __syncthreads();
    if (warp == 0) {
      // the diagonal, then (look-ahead) the next pivot and its reciprocal, while the
      // other warps update the off-diagonal entries
      if (tid == 0) s_swept[k] = 1;
      long long bk = LLONG_MIN;
      int bi = R;
      for (int i = lane; i < R; i += 32) {
        if (i == k) {
          A[i * ld + i] = -dk;
          continue;
        }
        const double v = fma(-s_a[i], s_t[i], A[i * ld + i]);
        A[i * ld + i] = v;
        if (!s_swept[i]) {
          const long long key = pivot_key(v);
          if (bi == R || key > bk) {
            bk = key;
            bi = i;
          }
        }
      }
      if (j + 1 < R) pick_pivot(bk, bi);
    } else if (warp & 3) {
      // Strictly upper entries (i < c).  Row i (R-1-i entries) is paired with row R-2-i
      // (i+1 entries): R entries per pair, pair q at t < R-1-q is (q, q+1+t), else
      // (R-2-q, t).  The work units are (pair, 32 consecutive t), dealt round-robin to
      // the warps on schedulers 1-3 (warp % 4 != 0), so that warp 0's diagonal FMA and
      // reciprocal on scheduler 0 do not queue behind update FMAs; four units per thread
      // step, loads issued before the FMAs, integer index arithmetic only.  Row and
      // column k take A(i,k) / d.
      const int npair = R / 2;  // rows 0..R-2; with R even the middle row pairs with itself
      const int nchunk = (R + 31) >> 5;
      const int nunit = npair * nchunk;
      const int nwk = (blockDim.x >> 5) / 4 * 3;
      const int wk = (warp >> 2) * 3 + (warp & 3) - 1;
      for (int u0 = wk; u0 < nunit; u0 += 4 * nwk) {
        int idx[4];
        double av[4], xv[4], yv[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int u = u0 + b * nwk;
          idx[b] = -1;
          av[b] = xv[b] = yv[b] = 0.0;
          int i = -1, c = -1;
          if (u < nunit) {
            const int q = u / nchunk;
            const int t = (u - q * nchunk) * 32 + lane;
            if (t < R - 1 - q) {
              i = q;
              c = q + 1 + t;
            } else if (t < R && R - 2 - q != q) {  // the middle row of an even R is listed once
              i = R - 2 - q;
              c = i + 1 + (t - (R - 1 - q));
            }
          }
          if (i >= 0) {
            idx[b] = i * ld + c;
            if (i == k) {
              av[b] = s_t[c];  // new A(k,c) = A(k,c) / d
            } else if (c == k) {
              av[b] = s_t[i];
            } else {
              av[b] = A[idx[b]];
              xv[b] = s_a[i];
              yv[b] = s_t[c];
            }
          }
        }
#pragma unroll
        for (int b = 0; b < 4; ++b)
          if (idx[b] >= 0) A[idx[b]] = fma(-xv[b], yv[b], av[b]);
      }
    }
    __syncthreads();
  }

  if (tid == 0) {
    info->rank = rank;
    info->fallback = (rank < R) ? 1 : 0;
    info->qr_rank = rank;
  }
  // U in pivoted order, rows 0..rank-1 (the leverage scores use its leading rank x rank
  // block): U(j,j) = sqrt(d_j), U(j,c) = Uo(j, piv(c)) / sqrt(d_j) for c > j
  for (int jj = tid; jj < R; jj += blockDim.x) {
    const double ri = (jj < rank) ? rsqrt(s_dp[jj]) : 0.0;
    s_a[jj] = ri;
    dinv[jj] = ri;
    piv[jj] = s_piv[jj];
  }
  __syncthreads();
  {
    double* UT = U + (size_t)R * R;
    for (int e = tid; e < R * R; e += blockDim.x) {
      const int r = e / R, c = e - r * R;
      double u = 0.0;
      if (r < rank && c < rank) {
        if (c == r) u = s_dp[r] * s_a[r];
        else if (c > r) u = Uo[(size_t)r * R + s_piv[c]] * s_a[r];
      }
      U[e] = u;
      UT[(size_t)c * R + r] = u;
    }
  }
  if (rank == R) {
    // W = -A (symmetric; also W^T)
    for (int e = tid; e < R * R; e += blockDim.x) {
      const int r = e / R, c = e - r * R;
      W[e] = -((r <= c) ? A[r * ld + c] : A[c * ld + r]);
    }
  } else {
    if (tid == 0 && chk) atomicAdd(reinterpret_cast<unsigned long long*>(&chk->fallbacks), 1ull);
    double* B = qwork;
    double* Z = qwork + (size_t)R * R;
    double* Y = qwork + 2 * (size_t)R * R;
    double* tau = qwork + 3 * (size_t)R * R;
    int* perm = reinterpret_cast<int*>(qwork + 4 * (size_t)R * R + R);
    double* cn = qwork + 4 * (size_t)R * R + 2 * R;
    __syncthreads();
    qr_fallback(gs, order, skip, R, B, Z, Y, tau, perm, W, info, sv, si, cn);
  }
}

// ---------------- FP64 pivoted sweep over a thread-block cluster ----------------
// The same sweep as k_factorize, with the rows of V dealt to the C CTAs of one cluster, so
// that the O(R^3) FP64 FMAs of a factorisation run on C SMs instead of one.  Like
// k_factorize, only the upper triangle (c >= i) is stored and updated, each entry by the
// operation k_factorize applies to it, and the pivot search uses the same keys and tie
// rule: W, U, dinv, piv and the rank come out bit-identical.  Row i belongs to block
// b = i / C at position i % C, and goes to CTA i % C for even b, C - 1 - i % C for odd b,
// so that the upper-triangle rows (R - i entries) even out over the CTAs.  One step:
//   (a) every warp finds the pivot among the C CTAs' candidates (each CTA's largest
//       diagonal key and its index, in a table every CTA holds a copy of);
//   (b) each thread reads one entry of the pivot row, A(min(t,k), max(t,k)), from the
//       shared memory of the CTA holding it (the matrix is double-buffered by step
//       parity, so that CTA's next update goes to the other buffer); the row is kept as
//       the step's row of U, while one thread forms the pivot's reciprocal (a division is
//       a chain of dependent FP64 operations: it hides under the remote loads); then the
//       row is scaled;
//   (c) warp 0 updates the CTA's diagonal entries and writes the CTA's candidate for the
//       next pivot into every CTA's table, then all threads update the rest of the
//       CTA's upper-triangle entries into the other buffer;
//   (d) one cluster barrier (release / acquire) publishes the rows and the table.
// A rank-deficient V (the stopping rule fires before R pivots) leaves info->swept = 0, and
// the single-CTA k_factorize launched after it redoes the factorisation with its QR
// fallback; at full rank k_factorize returns at once.
constexpr int CLT = 512;        // threads per CTA of the cluster sweep
constexpr int kClMaxRank = 256; // one pivot-row entry per thread in step (b)
constexpr int kClMinRank = 40;  // below it the single CTA's steps are shorter than a cluster round trip

__device__ __forceinline__ unsigned cl_ctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// address of the same shared-memory location in CTA `rank` of the cluster
__device__ __forceinline__ unsigned cl_map(const void* p, unsigned rank) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  unsigned out;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(a), "r"(rank));
  return out;
}
__device__ __forceinline__ double cl_ld_f64(unsigned addr) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}
// all threads of all CTAs of the cluster; shared-memory writes before it are visible after it
__device__ __forceinline__ void cl_sync() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
// largest key over the warp, smallest index among the lanes holding it (LAPACK MAXLOC on the
// keys); idx = INT_MAX marks a lane with no candidate
__device__ __forceinline__ void warp_argmax_key(long long key, int idx, long long& mk, int& k) {
  const int khi = (int)(key >> 32);
  const int mhi = __reduce_max_sync(0xffffffffu, khi);
  const unsigned mlo = __reduce_max_sync(0xffffffffu, khi == mhi ? (unsigned)(key & 0xffffffffll) : 0u);
  mk = (long long)(((unsigned long long)(unsigned)mhi << 32) | mlo);
  k = (int)__reduce_min_sync(0xffffffffu, (unsigned)((idx != INT_MAX && key == mk) ? idx : INT_MAX));
}
// warp 0: this CTA's best {key, index} into slot `me` of the candidate table in every CTA
__device__ __forceinline__ void cl_st_pair(unsigned addr, long long a, long long b) {
  asm volatile("st.shared::cluster.v2.s64 [%0], {%1, %2};" ::"r"(addr), "l"(a), "l"(b) : "memory");
}
__device__ __forceinline__ void push_candidate(long long key, int idx, long long* table, int me, int C) {
  long long mk;
  int k;
  warp_argmax_key(key, idx, mk, k);
  const int lane = threadIdx.x & 31;
  if (lane < C) cl_st_pair(cl_map(table + 2 * me, (unsigned)lane), mk, (long long)k);
}
// owner CTA and local row of row i
__host__ __device__ inline int cl_owner(int i, int C) {
  const int b = i / C, p = i - b * C;
  return (b & 1) ? C - 1 - p : p;
}
__host__ __device__ inline int cl_row(int li, int me, int C) { return li * C + ((li & 1) ? C - 1 - me : me); }

// -x by flipping the sign bit: the same bits as FP64 negation, without an FP64 instruction
// (on this part one warp's FP64 instruction holds the SM's FP64 pipe for about 19 cycles)
__device__ __forceinline__ double neg_bits(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}

__host__ __device__ inline int cl_rows(int R, int C) { return (R + C - 1) / C; }
__host__ __device__ inline size_t cl_smem_bytes(int R, int C) {
  const size_t nloc = (size_t)cl_rows(R, C);
  // A[2][nloc][R], Uo[nloc][R], s_ri[nloc], (pad), cand[2][C][2] (16-byte aligned), s_na, s_t,
  // s_dp [R], s_dk | emap[nloc R], s_piv, s_swept [R]
  return sizeof(double) * (3 * nloc * R + nloc + 1 + 4 * (size_t)C + 3 * (size_t)R + 1) +
         sizeof(int) * (nloc * R + 2 * (size_t)R);
}

__global__ void __launch_bounds__(CLT) k_factorize_cluster(GramSet gs, int order, int skip, int R, int C,
                                                          double* __restrict__ U, double* __restrict__ dinv,
                                                          int* __restrict__ piv, double* __restrict__ W,
                                                          SolveInfo* info, const DevCheck* chk) {
  if (done_flag(chk)) return;  // the same flag for every CTA: the cluster leaves together
  extern __shared__ __align__(16) double clsm[];
  const int nloc = cl_rows(R, C);
  const int nent = nloc * R;
  const int me = (int)cl_ctarank();
  const int tid = threadIdx.x, lane = tid & 31;
  double* A0 = clsm;                       // [2][nloc][R]: row li holds V row cl_row(li), c >= that row
  double* Uo = A0 + 2 * (size_t)nent;      // [nloc][R]: pivot rows of steps me + C lr
  double* s_ri = Uo + (size_t)nent;        // [nloc]
  long long* cand = reinterpret_cast<long long*>(clsm + ((3 * (size_t)nent + nloc + 1) & ~(size_t)1));  // [2][C][2]
  double* s_na = reinterpret_cast<double*>(cand + 4 * C);        // the pivot row, negated
  double* s_t = s_na + R;
  double* s_dp = s_t + R;
  double* s_dk = s_dp + R;
  int* emap = reinterpret_cast<int*>(s_dk + 1);  // strictly-upper entries of the local rows: li << 16 | c
  int* s_piv = emap + nent;
  int* s_swept = s_piv + R;

  // the local strictly-upper entries, row by row (row li has R - 1 - cl_row(li) of them); the
  // diagonal entry of local row li is lane li of warp 0's
  int nup = 0;
  for (int li = 0; li < nloc; ++li) {
    const int i = cl_row(li, me, C);
    if (i >= R) continue;
    for (int c = i + 1 + tid; c < R; c += CLT) emap[nup + c - i - 1] = (li << 16) | c;
    nup += R - 1 - i;
  }
  for (int t = tid; t < R; t += CLT) s_swept[t] = 0;
  cl_sync();  // every CTA of the cluster is running before the first remote store
  // V = ones .* G_a .* G_b ... in mode order (upper triangle, as k_factorize forms it)
  auto form_v = [&](int i, int c) {
    double v = 1.0;
    for (int q = 0; q < order; ++q)
      if (q != skip) v *= gs.G[q][(size_t)i * R + c];
    return v;
  };
  for (int f = tid; f < nup; f += CLT) {
    const int m = emap[f], li = m >> 16, c = m & 0xffff;
    A0[li * R + c] = form_v(cl_row(li, me, C), c);
  }
  if (tid < 32) {
    long long key = LLONG_MIN;
    int idx = INT_MAX;
    const int i = cl_row(lane, me, C);
    if (lane < nloc && i < R) {
      const double v = form_v(i, i);
      A0[lane * R + i] = v;
      key = pivot_key(v);
      idx = i;
    }
    push_candidate(key, idx, cand, me, C);
  }
  cl_sync();

  // the thread that divides: one not needed for the row fetch when there is one
  const int div_tid = (R < CLT) ? R : 0;
  int rank = R;
  for (int j = 0; j < R; ++j) {
    const int cur = j & 1;
    const double* __restrict__ Ac = A0 + (size_t)cur * nent;
    double* __restrict__ An = A0 + (size_t)(cur ^ 1) * nent;
    // (a) pivot: largest key, first index on ties (k_factorize's pick_pivot), in every warp
    long long mk;
    int k;
    {
      const long long* cc = cand + cur * 2 * C;
      const long long key = (lane < C) ? cc[2 * lane] : LLONG_MIN;
      const int idx = (lane < C) ? (int)cc[2 * lane + 1] : INT_MAX;
      warp_argmax_key(key, idx, mk, k);
    }
    if (key_is_nan(mk) || !(mk > pivot_key(kCholTol))) {  // the same decision everywhere in the cluster
      rank = j;
      break;
    }
    const double pv = __longlong_as_double(mk);
    // (b) the pivot row, before this step's update; its reciprocal beside it
    double a = 0.0;
    if (tid < R) {
      const int lo = min(tid, k), hi = max(tid, k);
      a = cl_ld_f64(cl_map(Ac + (size_t)(lo / C) * R + hi, (unsigned)cl_owner(lo, C)));
      s_na[tid] = neg_bits(a);
      if (j % C == me) Uo[(size_t)(j / C) * R + tid] = (s_swept[tid] || tid == k) ? 0.0 : a;
      if (tid == k) s_swept[tid] = 1;
    }
    if (tid == div_tid) {
      *s_dk = 1.0 / pv;
      s_piv[j] = k;
      s_dp[j] = pv;
    }
    __syncthreads();
    const double dk = *s_dk;
    if (tid < R) s_t[tid] = a * dk;
    __syncthreads();
    // (c) this CTA's upper-triangle entries, into the other buffer (k_factorize's update).
    // One warp's FP64 instruction holds its scheduler's FP64 pipe for ~64 cycles whatever
    // its active lanes, so every entry takes the same single FMA, with the special rows
    // and columns selected after it: no divergent FP64 code.  The diagonal comes first
    // (warp 0), so that the CTA's candidate travels to the other CTAs while the rest is
    // updated.
    if (tid < 32) {
      long long key = LLONG_MIN;
      int idx = INT_MAX;
      const int i = cl_row(lane, me, C);
      if (lane < nloc && i < R) {
        const int e = lane * R + i;
        const double f = fma(s_na[i], s_t[i], Ac[e]);
        const double v = (i == k) ? neg_bits(dk) : f;
        An[e] = v;
        if (!s_swept[i]) {
          key = pivot_key(v);
          idx = i;
        }
      }
      push_candidate(key, idx, cand + (cur ^ 1) * 2 * C, me, C);
    }
    for (int f0 = tid; f0 < nup; f0 += CLT) {
      const int m = emap[f0], li = m >> 16, c = m & 0xffff, i = cl_row(li, me, C);
      const int e = li * R + c;
      const double tc = s_t[c], ti = s_t[i];
      const double f = fma(s_na[i], tc, Ac[e]);
      An[e] = (i == k) ? tc : ((c == k) ? ti : f);  // row and column k take A(i,k) / d
    }
    // (d)
    cl_sync();
  }

  if (rank == R) {
    const double* Af = A0 + (size_t)(R & 1) * nent;
    for (int lr = tid; lr < nloc; lr += CLT) {
      const int r = me + C * lr;
      if (r < R) s_ri[lr] = rsqrt(s_dp[r]);
    }
    __syncthreads();
    // W = -A = V^{-1}, both triangles
    for (int f = tid; f < nup; f += CLT) {
      const int m = emap[f], li = m >> 16, c = m & 0xffff, i = cl_row(li, me, C);
      const double w = -Af[li * R + c];
      W[(size_t)i * R + c] = w;
      W[(size_t)c * R + i] = w;
    }
    if (tid < nloc) {
      const int i = cl_row(tid, me, C);
      if (i < R) W[(size_t)i * R + i] = -Af[tid * R + i];
    }
    // rows me + C lr of U (pivoted order): U(r,r) = sqrt(d_r), U(r,c) = Uo(r, piv(c)) / sqrt(d_r) for c > r
    double* UT = U + (size_t)R * R;
    for (int e = tid; e < nent; e += CLT) {
      const int lr = e / R, c = e - lr * R, r = me + C * lr;
      if (r >= R) continue;
      const double ri = s_ri[lr];
      double u = 0.0;
      if (c == r) u = s_dp[r] * ri;
      else if (c > r) u = Uo[(size_t)lr * R + s_piv[c]] * ri;
      U[(size_t)r * R + c] = u;
      UT[(size_t)c * R + r] = u;
      if (c == 0) {
        dinv[r] = ri;
        piv[r] = s_piv[r];
      }
    }
    if (me == 0 && tid == 0) {
      info->rank = R;
      info->fallback = 0;
      info->qr_rank = R;
      info->refine = 0;
      info->swept = 1;
    }
  } else if (me == 0 && tid == 0) {
    info->swept = 0;
  }
}

// ---------------- FP32 sweep (split-BF16 path) ----------------
// A blocked symmetric sweep in FP32 (this part issues FP32 FMAs at 64x its FP64 rate).  V is
// formed in FP64 exactly as above and kept in the workspace; W = V^{-1} in FP32 goes beside
// it.  The solve then refines X once with a compensated residual (mixed-precision iterative
// refinement: X += (M - X V) W), which brings X to FP64 accuracy while kappa(V) eps_32 << 1.
// A pivot below 1e-3 of the largest diagonal entry (or a NaN) leaves info->refine = 0 and the
// FP64 pivoted sweep takes over, as it does for every rank-deficient V.
//
// The sweep operator (Goodnight 1979) on an index block P of a symmetric A, with D = A_PP:
//   A_PP <- -D^{-1},  A_iP <- A_iP D^{-1} (= B_i),  A_ij <- A_ij - B_i A_Pj   (i, j not in P)
// is the composition of the single-index sweeps over P; after every block A = -V^{-1}.  The
// indices are swept in blocks of 32 in their natural order (V is symmetric positive definite
// whenever this path is taken; any pivot order is sound because the solve refines X):
//   (a) warps 0-3 sweep D in registers (lane i holds row i, eight columns per warp), one
//       index at a time; the pivot row reaches the lanes through shared memory, one named
//       barrier per index, and per-lane selects replace a branch on lane == k;
//   (b) all warps form B = A_{.P} D^{-1} and keep A_{.P} (both transposed, 32 x R);
//   (c) all warps apply the rank-32 update to the upper half of the rest of A in 4 x 4
//       register tiles, each written with its mirror, and write the swept blocks back.
// That is three barriers per block (twelve at R = 128) instead of two per index.
constexpr int FT32 = 512;
constexpr int kBlk32 = 32;
constexpr int kSweepWarps = 4;  // warps sweeping the diagonal block (eight columns each)
// The refinement's FP32 operands, written by the FP32 sweep into the workspace after the
// FP64 factorisation's area: [W | V_hi | V_lo], each R^2 floats padded to a multiple of four
// (16-byte aligned, so the solve stages them with 16-byte asynchronous copies).  V = V_hi +
// V_lo to 2^-48 relative.
__host__ __device__ inline int rr4(int R) { return (R * R + 3) & ~3; }
__host__ __device__ inline size_t ops32_offset_doubles(int R) {
  return (5 * (size_t)R * R + 4 * (size_t)R + 64 + 1) & ~(size_t)1;
}
__host__ __device__ inline int ld32(int R) { return ((R + 3) & ~3) + 4; }  // row stride of A, B^T, C^T
__host__ __device__ inline size_t factorize32_smem_bytes(int R) {
  const int ld = ld32(R);
  return sizeof(float) * ((size_t)R * ld + 2 * (size_t)kBlk32 * ld + (size_t)kBlk32 * 33 + 96);
}
// V = Hadamard product of the other modes' Grams (FP64, in mode order, as the FP64 sweep
// forms it), written as the FP32 pair V_hi + V_lo into the refinement operands.  One
// thread per entry over the whole grid: the FP64 products run on every SM instead of on
// the sweep's single CTA.
__global__ void __launch_bounds__(256) k_form_v32(GramSet gs, int order, int skip, int R, float* __restrict__ ops,
                                                  const DevCheck* chk) {
  if (done_flag(chk)) return;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= R * R) return;
  double v = 1.0;
  for (int m = 0; m < order; ++m)
    if (m != skip) v *= gs.G[m][e];
  const float vh = (float)v;
  ops[rr4(R) + e] = vh;
  ops[2 * rr4(R) + e] = (float)(v - (double)vh);
}

__global__ void __launch_bounds__(FT32) k_factorize32(int R, float* __restrict__ ops, SolveInfo* info, DevCheck* chk) {
  if (done_flag(chk)) return;
  extern __shared__ __align__(16) float fsm[];
  const int ld = ld32(R);
  float* A = fsm;                            // R x ld, row-major, both triangles
  float* Bt = A + (size_t)R * ld;            // 32 x ld: B^T, row p = column p of B = A_{.P} D^{-1}
  float* Ct = Bt + (size_t)kBlk32 * ld;      // 32 x ld: A_{.P}^T before the block
  float* Dm = Ct + (size_t)kBlk32 * ld;      // 32 x 33: the diagonal block, swept in place
  float* misc = Dm + kBlk32 * 33;            // [0]: pivot threshold, [1]: failure flag, [32, 96): pivot rows
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
  const float* __restrict__ Vh = ops + rr4(R);  // V_hi from k_form_v32
  const int Rp = (R + 3) & ~3;
  for (int e = tid; e < R * ld; e += nt) {
    const int i = e / ld, j = e - i * ld;
    A[e] = (j < R) ? Vh[(size_t)i * R + j] : 0.f;
  }
  for (int e = tid; e < 2 * kBlk32 * ld; e += nt) Bt[e] = 0.f;  // (Ct follows Bt)
  if (warp == 0) {
    float md = 0.f;
    for (int i = lane; i < R; i += 32) md = fmaxf(md, Vh[(size_t)i * R + i]);
    for (int off = 16; off > 0; off >>= 1) md = fmaxf(md, __shfl_xor_sync(0xffffffffu, md, off));
    if (lane == 0) {
      misc[0] = 1e-3f * md;
      misc[1] = 0.f;
    }
  }
  __syncthreads();
  const int ntile = Rp / 4;
  for (int p0 = 0; p0 < R; p0 += kBlk32) {
    const int pb = min(kBlk32, R - p0);
    // (a) sweep of the diagonal block D = A_PP by warps 0-3: lane i of warp w holds row i,
    // columns 8w .. 8w+7, in registers.  Per pivot k, lane k of each warp publishes its
    // eight entries of row k in shared memory (two buffers, alternating), one named barrier
    // over the four warps, then every lane reads row k back (broadcast loads) and takes
    // D(i, k) as D(k, i), the sweep keeping the block symmetric.  Column k is set by an
    // unrolled select (no dynamically indexed registers).
    if (warp < kSweepWarps) {
      constexpr int CW = kBlk32 / kSweepWarps;  // columns per warp
      const int c0 = warp * CW;
      float r[CW];
#pragma unroll
      for (int c = 0; c < CW; ++c)
        r[c] = (lane < pb && c0 + c < pb) ? A[(size_t)(p0 + lane) * ld + p0 + c0 + c] : 0.f;
      const float thr = misc[0];
      bool bad = false;
      for (int k = 0; k < pb; ++k) {
        float* prow = misc + 32 * (1 + (k & 1));  // 16-byte aligned, two buffers
        const bool me = (lane == k);
        if (me) {
#pragma unroll
          for (int v = 0; v < CW / 4; ++v)
            reinterpret_cast<float4*>(prow + c0)[v] = make_float4(r[4 * v], r[4 * v + 1], r[4 * v + 2], r[4 * v + 3]);
        }
        __syncwarp();
        asm volatile("barrier.sync 1, %0;" ::"n"(kSweepWarps * 32) : "memory");
        float rk[CW];
#pragma unroll
        for (int v = 0; v < CW / 4; ++v) {
          const float4 x = reinterpret_cast<const float4*>(prow + c0)[v];
          rk[4 * v] = x.x;
          rk[4 * v + 1] = x.y;
          rk[4 * v + 2] = x.z;
          rk[4 * v + 3] = x.w;
        }
        const float dik = prow[lane];
        const float d = prow[k];
        bad = bad || !(d > thr) || !(d < INFINITY);
        const float rd = __frcp_rn(d);
        const float f = dik * rd;
        const float pk = me ? -rd : f;
#pragma unroll
        for (int c = 0; c < CW; ++c) {
          const float v = me ? rk[c] * rd : fmaf(-f, rk[c], r[c]);
          r[c] = (c0 + c == k) ? pk : v;
        }
      }
      if (lane < pb) {
#pragma unroll
        for (int c = 0; c < CW; ++c) Dm[lane * 33 + c0 + c] = r[c];
      }
      if (warp == 0 && lane == 0 && bad) misc[1] = 1.f;
    }
    __syncthreads();
    if (misc[1] != 0.f) break;
    // (b) B = A_{.P} D^{-1} (D^{-1} = -Dm) and C = A_{.P}, both transposed, for every row i:
    // lane q keeps column q of D^{-1} in registers, the warps take the rows
    {
      float dcol[kBlk32];
#pragma unroll
      for (int pp = 0; pp < kBlk32; ++pp) dcol[pp] = (lane < pb && pp < pb) ? -Dm[pp * 33 + lane] : 0.f;
      for (int i = warp; i < R; i += nt >> 5) {
        const float4* ai = reinterpret_cast<const float4*>(A + (size_t)i * ld + p0);
        float b4[4] = {0.f, 0.f, 0.f, 0.f};  // four independent partial sums: a short dependent chain
#pragma unroll
        for (int v = 0; v < kBlk32 / 4; ++v) {
          const float4 x = ai[v];
          b4[0] = fmaf(x.x, dcol[4 * v], b4[0]);
          b4[1] = fmaf(x.y, dcol[4 * v + 1], b4[1]);
          b4[2] = fmaf(x.z, dcol[4 * v + 2], b4[2]);
          b4[3] = fmaf(x.w, dcol[4 * v + 3], b4[3]);
        }
        Bt[(size_t)lane * ld + i] = (b4[0] + b4[1]) + (b4[2] + b4[3]);
        Ct[(size_t)lane * ld + i] = (lane < pb) ? A[(size_t)i * ld + p0 + lane] : 0.f;
      }
    }
    __syncthreads();
    // (c) the rank-pb update of the rest and the swept blocks written back, in 4 x 4 tiles
    // (tiles never straddle the block: it starts at a multiple of 32).  The matrix stays
    // symmetric, so only tiles (ti <= tj) outside the block's tile range P are computed, each
    // written with its mirror; the P row strip (the swept block and A_Pj = B_j^T) is written
    // with its mirror too.  Work items: the rank-pb update tiles first, then the strip's
    // copies, so that no thread takes two update tiles at R = 128.
    {
      const int tp0 = p0 / 4, npt = (pb + 3) / 4;
      const int m = ntile - npt;                    // tiles outside P, in each direction
      const int nexp = m * (m + 1) / 2, ncopy = npt * ntile;
      for (int u = tid; u < nexp + ncopy; u += nt) {
        float v[4][4];
        int i0, j0;
        bool mirror;
        if (u < nexp) {  // A_ij - sum_p B(i, p) C(j, p), ti <= tj, both outside P
          int a = 0, rem = u, len = m;
          while (rem >= len) {
            rem -= len;
            ++a;
            --len;
          }
          const int bb = a + rem;
          const int ti = a < tp0 ? a : a + npt, tj = bb < tp0 ? bb : bb + npt;
          i0 = 4 * ti;
          j0 = 4 * tj;
          mirror = ti != tj;
#pragma unroll
          for (int r4 = 0; r4 < 4; ++r4) {
            const float4 x = *reinterpret_cast<const float4*>(A + (size_t)(i0 + r4) * ld + j0);
            v[r4][0] = x.x;
            v[r4][1] = x.y;
            v[r4][2] = x.z;
            v[r4][3] = x.w;
          }
          for (int pp = 0; pp < pb; ++pp) {
            const float4 bi = *reinterpret_cast<const float4*>(Bt + (size_t)pp * ld + i0);
            const float4 cj = *reinterpret_cast<const float4*>(Ct + (size_t)pp * ld + j0);
            const float bv[4] = {bi.x, bi.y, bi.z, bi.w}, cv[4] = {cj.x, cj.y, cj.z, cj.w};
#pragma unroll
            for (int r4 = 0; r4 < 4; ++r4)
#pragma unroll
              for (int c4 = 0; c4 < 4; ++c4) v[r4][c4] = fmaf(-bv[r4], cv[c4], v[r4][c4]);
          }
        } else {  // the P row strip: tile (tp0 + e / ntile, e % ntile)
          const int e = u - nexp;
          const int ti = tp0 + e / ntile, tj = e - (e / ntile) * ntile;
          i0 = 4 * ti;
          j0 = 4 * tj;
          const bool inJ = (j0 >= p0 && j0 < p0 + pb);
          mirror = !inJ;
          if (inJ) {  // the swept block: -D^{-1}
#pragma unroll
            for (int r4 = 0; r4 < 4; ++r4)
#pragma unroll
              for (int c4 = 0; c4 < 4; ++c4)
                v[r4][c4] = (i0 + r4 < p0 + pb && j0 + c4 < p0 + pb) ? Dm[(i0 + r4 - p0) * 33 + (j0 + c4 - p0)] : 0.f;
          } else {  // A_Pj = B_j^T (its mirror A_jP = B_j)
#pragma unroll
            for (int r4 = 0; r4 < 4; ++r4) {
              const float4 x = *reinterpret_cast<const float4*>(Bt + (size_t)(i0 + r4 - p0) * ld + j0);
              v[r4][0] = x.x;
              v[r4][1] = x.y;
              v[r4][2] = x.z;
              v[r4][3] = x.w;
            }
          }
        }
#pragma unroll
        for (int r4 = 0; r4 < 4; ++r4)
          if (i0 + r4 < R)
            *reinterpret_cast<float4*>(A + (size_t)(i0 + r4) * ld + j0) =
                make_float4(v[r4][0], v[r4][1], v[r4][2], v[r4][3]);
        if (mirror) {
#pragma unroll
          for (int c4 = 0; c4 < 4; ++c4)
            if (j0 + c4 < R)
              *reinterpret_cast<float4*>(A + (size_t)(j0 + c4) * ld + i0) =
                  make_float4(v[0][c4], v[1][c4], v[2][c4], v[3][c4]);
        }
      }
    }
    __syncthreads();
  }
  const int ok = (misc[1] == 0.f) ? 1 : 0;
  if (tid == 0) {
    info->refine = ok;
    if (ok) {
      info->rank = R;
      info->fallback = 0;
      info->qr_rank = R;
    }
  }
  if (!ok) return;
  // W = -A (FP32): column-major = row-major (A is symmetric)
  for (int e = tid; e < R * R; e += nt) {
    const int c = e / R, i = e - c * R;
    ops[e] = -A[(size_t)i * ld + c];
  }
}

// ---------------- solve: X = M W^T ----------------
// M rows are the split-K partial sums (added in split order, FP64); W^T is the solve
// operator from the factorisation (V^{-1}, or the pivoted-QR least-squares operator),
// stored so that consecutive output columns are contiguous.  One thread per output.
// FP64 here has ~128-cycle latency and a low issue rate per warp, so every loop keeps
// many independent loads or accumulators in flight: W^T is staged in shared memory (when
// it fits) while the partial sums load, the partials are summed by eight accumulators,
// and each output by eight.  Per-row sums of M .* X (a tree over the row) feed the fit.
constexpr int SOLVE_T = 256;
constexpr int kSolveStageMaxR = 128;  // W^T (R^2 doubles) staged in shared memory up to here
// The solve of one block of RB rows (the block index `blk`); the rows' X stays in shared
// memory (sm + 2 RB R) for a caller that continues with it.
template <typename PT>
__device__ __forceinline__ void solve_rows_body(const PT* __restrict__ part, int S, int64_t In, int R, int RB,
                                                const double* __restrict__ WT, double* __restrict__ X,
                                                double* __restrict__ inner_rows, const SolveInfo* __restrict__ info,
                                                const float* __restrict__ ops, double* __restrict__ gpart, int blk,
                                                double* sm) {
  double* Ms = sm;            // RB x R
  double* Ps = sm + RB * R;   // RB x R products for the fit
  double* Xs = sm + 2 * RB * R;  // RB x R: X before the refinement
  const int fw = ((RB * R + 3) & ~3) / 2;                 // doubles per RB x R float array
  float* Fs = reinterpret_cast<float*>(sm + 3 * RB * R);  // RB x R floats: M, then the residual
  float* X0f = reinterpret_cast<float*>(sm + 3 * RB * R + fw);  // RB x R floats: X0
  const bool staged = (R <= kSolveStageMaxR);
  const bool refine = info && info->refine;
  double* St = sm + ((3 * RB * R + 2 * fw + 1) & ~1);  // staging area (16-byte aligned)
  double* Ws = St;                        // W (FP64 path)
  float* W32 = reinterpret_cast<float*>(St);  // refinement: [W | V_hi | V_lo] (FP32 sweep)
  const float* Vh = W32 + rr4(R);
  const float* Vl = W32 + 2 * rr4(R);
  const int tid = threadIdx.x;
  const int64_t r0 = (int64_t)blk * RB;
  const int rows = (In - r0 < (int64_t)RB) ? (int)(In - r0) : RB;
  const int nval = rows * R;
  const int64_t base = r0 * R;
  const int64_t sstride = In * R;
  if (refine) {
    // 16-byte asynchronous copies of [W | V_hi | V_lo]; they land while M is summed below
    const int n16 = 3 * rr4(R) / 4;
    const char* src = reinterpret_cast<const char*>(ops);
    const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(W32));
    for (int c = tid; c < n16; c += SOLVE_T)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16u * c), "l"(src + 16 * (size_t)c)
                   : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
  } else if (staged) {
    const int n = R * R;
    for (int e0 = tid; e0 < n; e0 += 8 * SOLVE_T) {
      double w[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int e = e0 + q * SOLVE_T;
        w[q] = (e < n) ? __ldg(&WT[e]) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int e = e0 + q * SOLVE_T;
        if (e < n) Ws[e] = w[q];
      }
    }
  }
  for (int e = tid; e < nval; e += SOLVE_T) {
    if constexpr (sizeof(PT) == 4) {
      // FP32 partials: a compensated (Neumaier) sum in FP32, finished in FP64.  Its error
      // is O(S eps32^2) of the summed magnitudes, and it keeps the conversions and adds
      // off the FP64 pipe, which the product below saturates.
      float sacc = 0.0f, cacc = 0.0f;
      int sp = 0;
      for (; sp + 16 <= S; sp += 16) {
        float v[16];
#pragma unroll
        for (int t = 0; t < 16; ++t) v[t] = part[(int64_t)(sp + t) * sstride + base + e];
#pragma unroll
        for (int t = 0; t < 16; ++t) {
          const float tt = sacc + v[t];
          cacc += (fabsf(sacc) >= fabsf(v[t])) ? ((sacc - tt) + v[t]) : ((v[t] - tt) + sacc);
          sacc = tt;
        }
      }
      if (sp < S) {  // the last (< 16) splits, their loads in flight together
        float v[16];
#pragma unroll
        for (int t = 0; t < 16; ++t) v[t] = (sp + t < S) ? part[(int64_t)(sp + t) * sstride + base + e] : 0.0f;
#pragma unroll
        for (int t = 0; t < 16; ++t) {
          if (sp + t < S) {
            const float tt = sacc + v[t];
            cacc += (fabsf(sacc) >= fabsf(v[t])) ? ((sacc - tt) + v[t]) : ((v[t] - tt) + sacc);
            sacc = tt;
          }
        }
      }
      Ms[e] = (double)sacc + (double)cacc;
    } else {
      double acc[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] = 0.0;
      int sp = 0;
      for (; sp + 16 <= S; sp += 16) {
        PT v[16];
#pragma unroll
        for (int t = 0; t < 16; ++t) v[t] = part[(int64_t)(sp + t) * sstride + base + e];
#pragma unroll
        for (int t = 0; t < 16; ++t) acc[t & 7] += (double)v[t];
      }
#pragma unroll
      for (int t = 0; t < 16; ++t)
        if (sp + t < S) acc[t & 7] += (double)part[(int64_t)(sp + t) * sstride + base + e];
      Ms[e] = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
    }
  }
  if (refine) asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  const double* W = staged ? Ws : WT;
  // one output of A B for the row `row` of A (RB x R in shared memory), column k of B (R x R)
  auto rowdot = [&](const double* Arow, const double* __restrict__ B, int k) {
    double a[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) a[t] = 0.0;
    int l = 0;
    for (; l + 8 <= R; l += 8) {
#pragma unroll
      for (int t = 0; t < 8; ++t) a[t] = fma(Arow[l + t], B[(size_t)(l + t) * R + k], a[t]);
    }
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (l + t < R) a[t] = fma(Arow[l + t], B[(size_t)(l + t) * R + k], a[t]);
    return ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
  };
  if (refine) {
    // Mixed-precision iterative refinement with the FP32 inverse W: only the residual needs
    // more than FP32 (it cancels); X0 and the correction carry FP32 relative error, and the
    // correction is ~kappa eps_32 smaller than X:
    //   X0 = M W (FP32),  E = M - X0 V,  X = X0 + E W (FP32 product, FP64 sum).
    // X0 V is a compensated FP32 dot product (Dot2, Ogita, Rump and Oishi 2005): X0 is
    // exact in FP32, V = V_hi + V_lo, each X0 V_hi term is split exactly into product and
    // error (one FMA) and summed with an error-free TwoSum, X0 V_lo is added in FP32.  The
    // result is as accurate as an FP64 dot product (~2^-48 relative to sum |X0| |V|), at
    // FP32 rates (this part issues FP32 64x faster than FP64).
    auto dot2 = [&](const float* x, int k) {
      float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
      auto term = [&](float xv, int l, float& s, float& c) {
        const float vh = Vh[(size_t)l * R + k];
        const float p = xv * vh;
        const float pe = fmaf(xv, vh, -p);
        const float t = s + p;
        const float z = t - s;
        const float e = (s - (t - z)) + (p - z);
        s = t;
        c = fmaf(xv, Vl[(size_t)l * R + k], c + (pe + e));
      };
      int l = 0;
      for (; l + 2 <= R; l += 2) {
        term(x[l], l, s0, c0);
        term(x[l + 1], l + 1, s1, c1);
      }
      if (l < R) term(x[l], l, s0, c0);
      return ((double)s0 + (double)s1) + ((double)c0 + (double)c1);
    };
    auto rowdot32 = [&](const float* Arow, int k) {
      float a[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) a[t] = 0.f;
      int l = 0;
      for (; l + 8 <= R; l += 8) {
#pragma unroll
        for (int t = 0; t < 8; ++t) a[t] = fmaf(Arow[l + t], W32[(size_t)(l + t) * R + k], a[t]);
      }
#pragma unroll
      for (int t = 0; t < 8; ++t)
        if (l + t < R) a[t] = fmaf(Arow[l + t], W32[(size_t)(l + t) * R + k], a[t]);
      return ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    };
    for (int e = tid; e < nval; e += SOLVE_T) Fs[e] = (float)Ms[e];
    __syncthreads();
    for (int e = tid; e < nval; e += SOLVE_T) {
      const int row = e / R, k = e % R;
      const float x0 = rowdot32(Fs + row * R, k);
      X0f[e] = x0;
      Xs[e] = (double)x0;
    }
    __syncthreads();
    for (int e = tid; e < nval; e += SOLVE_T) {
      const int row = e / R, k = e % R;
      Ps[e] = Ms[e] - dot2(X0f + row * R, k);
    }
    __syncthreads();
    for (int e = tid; e < nval; e += SOLVE_T) Fs[e] = (float)Ps[e];
    __syncthreads();
    for (int e = tid; e < nval; e += SOLVE_T) {
      const int row = e / R, k = e % R;
      const double x = Xs[e] + (double)rowdot32(Fs + row * R, k);
      X[base + e] = x;
      Xs[e] = x;  // (only this thread reads Xs[e] in this loop)
    }
  } else {
    for (int e = tid; e < nval; e += SOLVE_T) {
      const int row = e / R, k = e % R;
      const double x = rowdot(Ms + row * R, W, k);
      X[base + e] = x;
      Xs[e] = x;
    }
  }
  if (gpart) {
    // this block's share of G = X^T X: the upper triangle (rows paired: row p with row
    // R-1-p, R+1 entries per pair), two accumulators over the block's rows
    __syncthreads();
    const int T = R * (R + 1) / 2;
    double* gp = gpart + (size_t)blk * T;
    for (int e = tid; e < T; e += SOLVE_T) {
      const int p = e / (R + 1), t = e - p * (R + 1);
      int a, b;
      if (t < R - p) {
        a = p;
        b = p + t;
      } else {
        a = R - 1 - p;
        b = a + (t - (R - p));
      }
      double s0 = 0.0, s1 = 0.0;
      int row = 0;
      for (; row + 1 < rows; row += 2) {
        s0 = fma(Xs[row * R + a], Xs[row * R + b], s0);
        s1 = fma(Xs[(row + 1) * R + a], Xs[(row + 1) * R + b], s1);
      }
      if (row < rows) s0 = fma(Xs[row * R + a], Xs[row * R + b], s0);
      gp[e] = s0 + s1;
    }
  }
  if (!inner_rows) return;
  __syncthreads();
  // per-row sum of M .* X for the fit's <T, X>, exact in 128-bit fixed point (one warp per
  // row: the row's largest exponent, then the integer sum); stored as (lo, hi, base)
  const int lane = tid & 31, warp = tid >> 5, nw = SOLVE_T >> 5;
  long long* ir = reinterpret_cast<long long*>(inner_rows);
  for (int row = warp; row < rows; row += nw) {
    int emax = 1;
    for (int kk = lane; kk < R; kk += 32) emax = max(emax, fx_exp(Ms[row * R + kk] * Xs[row * R + kk]));
    emax = __reduce_max_sync(0xffffffffu, emax);
    const int base = (emax == 0x7ff) ? kFxBad : emax - kFxHead;
    __int128 q = 0;
    if (base != kFxBad)
      for (int kk = lane; kk < R; kk += 32) q += fx_term(Ms[row * R + kk] * Xs[row * R + kk], base);
    q = fx_warp_sum(q);
    if (lane == 0) {
      ir[3 * (r0 + row)] = (long long)(unsigned long long)q;
      ir[3 * (r0 + row) + 1] = (long long)(q >> 64);
      ir[3 * (r0 + row) + 2] = base;
    }
  }
}

template <typename PT>
__global__ void __launch_bounds__(SOLVE_T) k_solve_gemm(const PT* __restrict__ part, int S, int64_t In, int R, int RB,
                                                        const double* __restrict__ WT, double* __restrict__ X,
                                                        double* __restrict__ inner_rows, const DevCheck* chk,
                                                        const SolveInfo* __restrict__ info,
                                                        const float* __restrict__ ops,
                                                        double* __restrict__ gpart) {
  if (done_flag(chk)) return;
  extern __shared__ double sm[];
  solve_rows_body<PT>(part, S, In, R, RB, WT, X, inner_rows, info, ops, gpart, blockIdx.x, sm);
}

// ---------------- gram + finalize ----------------
// Block-wide helpers for the exact fixed-point sums: the largest int, and the sum of the
// threads' 128-bit values (every thread gets both).
__device__ int block_max_int(int v, int* si) {  // si: 32 ints
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = __reduce_max_sync(0xffffffffu, v);
  __syncthreads();
  if (lane == 0) si[w] = v;
  __syncthreads();
  int t = (lane < nw) ? si[lane] : INT_MIN;
  t = __reduce_max_sync(0xffffffffu, t);
  __syncthreads();
  return t;
}
__device__ __int128 block_sum_fx(__int128 q, long long* sl) {  // sl: 64 words
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  q = fx_warp_sum(q);
  __syncthreads();
  if (lane == 0) {
    sl[2 * w] = (long long)(unsigned long long)q;
    sl[2 * w + 1] = (long long)(q >> 64);
  }
  __syncthreads();
  __int128 t = 0;
  if (lane < nw)
    t = (__int128)(((unsigned __int128)(unsigned long long)sl[2 * lane + 1] << 64) |
                   (unsigned long long)sl[2 * lane]);
  t = fx_warp_sum(t);
  __syncthreads();
  return t;
}
__device__ __forceinline__ __int128 fx_join(unsigned long long lo, long long hi) {
  return (__int128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}

// The fit 1 - ||T - X|| / ||T|| with ||T - X||^2 = ||T||^2 + ||X||^2 - 2 |<T, X>|
// (fit_check.jl:26-32).  Near fit -> 1 the three terms cancel, so the combination is done
// exactly: <T, X> and ||X||^2 arrive as exact fixed-point sums, ||T||^2 (the device's own,
// when ref_norm is norm(T) to 1e-15 relative; else the exact square of ref_norm) joins them at
// a common base, and only the small result is rounded to a double.
__device__ double compensated_fit(const DevCheck& k) {
  const double rn = k.ref_norm;
  if (!(rn > 0.0)) return NAN;
  double ta, tb;
  if (k.t2_valid && fabs(rn - sqrt(k.t2_hi)) <= 1e-15 * rn) {
    ta = k.t2_hi;
    tb = k.t2_lo;
  } else {
    ta = rn * rn;
    tb = fma(rn, rn, -ta);
  }
  if (k.inner_base == kFxBad || k.fsq_base == kFxBad || !isfinite(ta)) return NAN;
  const int tbase = fx_exp(ta) - kFxHead;
  const int c = max(max(k.inner_base, k.fsq_base), tbase) + 2;  // (+2: room for the sum)
  const __int128 t2 = fx_align(fx_term(ta, tbase) + fx_term(tb, tbase), tbase, c);
  __int128 in = fx_align(fx_join(k.inner_lo, k.inner_hi), k.inner_base, c);
  if (in < 0) in = -in;
  const __int128 fs = fx_align(fx_join(k.fsq_lo, k.fsq_hi), k.fsq_base, c);
  __int128 r2 = t2 + fs - 2 * in;
  if (r2 < 0) r2 = -r2;
  const double nr = sqrt(fx_to_double(r2, c));
  return 1.0 - nr / rn;
}

// The check's update after a sweep (FitCheck fit_check.jl:24-66, NoCheck no_check.jl:11-20)
// from the terms in k; writes the trajectory entry.
__device__ void check_update(DevCheck& k, double* traj, int64_t traj_cap) {
  // CPDiffCheck / CPAngleCheck run after the sweep, on the normalised iterate (k_cpcheck.cu)
  if (k.kind == CPALS_CHECK_DIFF || k.kind == CPALS_CHECK_ANGLE) return;
  const double fit = compensated_fit(k);
  k.terms_ready = 0;
  if (k.sweeps < traj_cap) traj[k.sweeps] = fit;
  k.sweeps += 1;
  if (k.kind == CPALS_CHECK_FIT) {
    k.iter += 1;
    const double dfit = fabs(k.lastfit - fit);
    k.lastfit = fit;
    if (isnan(fit)) {
      k.nan_flag = 1;
      k.done = 1;
      return;
    }
    if (dfit < k.tol) {
      k.counter += 1;
      if (k.counter >= 2) {
        k.total_iter = k.iter;
        k.iter = 0;
        k.counter = 0;
        k.final_fit = k.lastfit;
        k.lastfit = 0.0;
        k.done = 1;
        return;
      }
    } else {
      k.counter = 0;
    }
    if (k.iter >= k.max_counter) {
      k.total_iter = k.iter;
      k.iter = 0;
      k.counter = 0;
      k.final_fit = k.lastfit;
      k.lastfit = 0.0;
    }
  } else {
    k.iter += 1;
    k.lastfit = fit;
    if (k.iter == k.max_counter) {
      k.iter = 0;
      k.done = 1;
    }
  }
}

__global__ void k_check_step(DevCheck* chk, double* traj, int64_t traj_cap) {
  if (threadIdx.x == 0 && blockIdx.x == 0) check_update(*chk, traj, traj_cap);
}

struct FinalizeArgs {
  double* lam;
  double* lam_inv;
  double* Gn;  // written here only when fpart is null (else by the normalisation kernel)
  GramSet gs;
  int order;
  int last;
  const long long* inner_rows_fx;  // per row: an exact fixed-point sum (lo, hi, base)
  int64_t In;
  DevCheck* chk;
  double* traj;
  int64_t traj_cap;
  int mode;       // the mode whose raw Gram is being finalised
  double* fpart;  // per-tile (per-block) exact shares of ||X||^2 (lo, hi, base), or null
  int ntiles;
  int run_check;  // 0: only save the fit's terms (a caller-driven sweep runs the check)
};

// lambda = sqrt(diag Graw) (one reciprocal square root per column), G_n = Graw ./
// (lambda lambda^T) by the reciprocals; on the last mode the fit (fit_check.jl:22-43)
// and the device FitCheck / NoCheck update.  One block; loads are issued eight at a
// time (a single FP64 dependent chain costs ~128 cycles per step here).  `coherent`
// reads Graw through L2 (written by other blocks of the same launch).
__device__ void finalize_fit(int R, const FinalizeArgs& fa, const double* lam);

__device__ void finalize_body(const double* __restrict__ Graw, int R, const FinalizeArgs& fa, bool coherent) {
  __shared__ double s_lam[CPALS_MAX_RANK_SOLVE];
  __shared__ double s_inv[CPALS_MAX_RANK_SOLVE];
  const int tid = threadIdx.x, nt = blockDim.x;
  auto ld = [&](const double* p) { return coherent ? __ldcg(p) : *p; };
  for (int r = tid; r < R; r += nt) {
    const double g = ld(&Graw[(size_t)r * R + r]);
    const double ri = rsqrt(g);
    const double l = g * ri;
    s_lam[r] = l;
    s_inv[r] = ri;
    fa.lam[r] = l;
    fa.lam_inv[r] = ri;
  }
  __syncthreads();
  const int n = R * R;
  for (int e0 = tid; !fa.fpart && e0 < n; e0 += 8 * nt) {
    double g[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = e0 + q * nt;
      g[q] = (e < n) ? ld(&Graw[e]) : 0.0;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = e0 + q * nt;
      if (e < n) {
        const int r = e / R, c = e - r * R;
        fa.Gn[e] = g[q] * s_inv[r] * s_inv[c];
      }
    }
  }
  if (!fa.last) return;
  finalize_fit(R, fa, s_lam);
}

// The fit's terms on the last mode (and the check's update when fa.run_check): <T, X> from the
// rows' exact sums, ||X||^2 from the per-tile (per-block) shares or, without them, from the
// Grams and lambda (lam: R values visible to the whole block).  One block.
__device__ void finalize_fit(int R, const FinalizeArgs& fa, const double* lam) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int n = R * R;
  __shared__ int si[32];
  __shared__ long long sl[64];
  // <T, X> = sum(M_N .* F_N .* lambda) = sum(M_N .* X_N)  (fit_check.jl:28): the rows' exact
  // fixed-point sums, aligned to the largest row base (+8: room for 2^36 rows) and added
  const long long* ir = fa.inner_rows_fx;
  int bmax = INT_MIN;
  for (int64_t i = tid; i < fa.In; i += nt) bmax = max(bmax, (int)__ldcg(&ir[3 * i + 2]));
  bmax = block_max_int(bmax, si);
  const int ib = (bmax == kFxBad) ? kFxBad : bmax + 8;
  __int128 qi = 0;
  if (ib != kFxBad)
    for (int64_t i = tid; i < fa.In; i += nt)
      qi += fx_align(fx_join((unsigned long long)__ldcg(&ir[3 * i]), __ldcg(&ir[3 * i + 1])), (int)__ldcg(&ir[3 * i + 2]),
                     ib);
  const __int128 inner = block_sum_fx(qi, sl);
  // ||X||^2 = lambda^T (G_1 o ... o G_N) lambda  (converge_checks.jl:5-11): with the per-tile
  // (per-block) shares of the fused path, their exact sums; otherwise each term formed here
  int fb;
  __int128 qf = 0;
  if (fa.fpart) {
    const long long* fp = reinterpret_cast<const long long*>(fa.fpart);
    int m = INT_MIN;
    for (int t = tid; t < fa.ntiles; t += nt) m = max(m, (int)__ldcg(&fp[3 * t + 2]));
    m = block_max_int(m, si);
    fb = (m == kFxBad) ? kFxBad : m + 8;
    if (fb != kFxBad)
      for (int t = tid; t < fa.ntiles; t += nt)
        qf += fx_align(fx_join((unsigned long long)__ldcg(&fp[3 * t]), __ldcg(&fp[3 * t + 1])),
                       (int)__ldcg(&fp[3 * t + 2]), fb);
  } else {
    auto term = [&](int e) {
      double h = fa.gs.G[0][e];
      for (int m = 1; m < fa.order; ++m) h *= fa.gs.G[m][e];
      const int r = e / R, c2 = e - r * R;
      return h * lam[r] * lam[c2];
    };
    int m = 1;
    for (int e = tid; e < n; e += nt) m = max(m, fx_exp(term(e)));
    m = block_max_int(m, si);
    fb = (m == 0x7ff) ? kFxBad : m - kFxHead + 8;
    if (fb != kFxBad)
      for (int e = tid; e < n; e += nt) qf += fx_term(term(e), fb);
  }
  const __int128 fact_square = block_sum_fx(qf, sl);
  if (tid != 0) return;
  DevCheck& k = *fa.chk;
  k.inner_lo = (unsigned long long)inner;
  k.inner_hi = (long long)(inner >> 64);
  k.inner_base = ib;
  k.fsq_lo = (unsigned long long)fact_square;
  k.fsq_hi = (long long)(fact_square >> 64);
  k.fsq_base = fb;
  k.terms_ready = 1;
  if (fa.run_check) check_update(k, fa.traj, fa.traj_cap);
}


constexpr int GT = 16;  // tile edge
// G = X^T X over 16x16 upper tiles and S2 row splits; the last split of each tile sums
// the S2 partials (in split order) and writes the tile and its mirror; with FIN the last
// tile to finish runs finalize_body.  Rows are loaded 64 at a time, only real rows, and
// each output keeps four accumulators.
template <bool FIN>
__global__ void __launch_bounds__(256) k_gram(const double* __restrict__ X, int64_t In, int R, int S2,
                                              int64_t rows_per_split, double* __restrict__ part,
                                              unsigned* __restrict__ counters, double* __restrict__ G,
                                              const DevCheck* chk, FinalizeArgs fa) {
  if (done_flag(chk)) return;
  __shared__ double xa[64][GT + 1];
  __shared__ double xb[64][GT + 1];
  __shared__ int s_last;
  const int nt = (R + GT - 1) / GT;
  const int ntiles = nt * (nt + 1) / 2;
  // blockIdx.x enumerates upper-triangle tiles (ti <= tj)
  int t = blockIdx.x, ti = 0;
  while (t >= nt - ti) {
    t -= nt - ti;
    ++ti;
  }
  const int tj = ti + t;
  const int tile = blockIdx.x, s = blockIdx.y;
  const int a = threadIdx.x / GT, b = threadIdx.x % GT;
  const int r1 = ti * GT + a, r2 = tj * GT + b;
  const int64_t rb = (int64_t)s * rows_per_split;
  const int64_t re = (In < rb + rows_per_split) ? In : rb + rows_per_split;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t i0 = rb; i0 < re; i0 += 64) {
    const int nr = (re - i0 < 64) ? (int)(re - i0) : 64;
    __syncthreads();
    {
      double va[4], vb[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int e = threadIdx.x + q * 256;  // 64 rows x 16 columns
        const int ii = e / GT, c = e % GT;
        const int ca = ti * GT + c, cb = tj * GT + c;
        va[q] = (ii < nr && ca < R) ? X[(i0 + ii) * R + ca] : 0.0;
        vb[q] = (ii < nr && cb < R) ? X[(i0 + ii) * R + cb] : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int e = threadIdx.x + q * 256;
        xa[e / GT][e % GT] = va[q];
        xb[e / GT][e % GT] = vb[q];
      }
    }
    __syncthreads();
    int ii = 0;
    for (; ii + 4 <= nr; ii += 4) {
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fma(xa[ii + q][a], xb[ii + q][b], acc[q]);
    }
    for (; ii < nr; ++ii) acc[0] = fma(xa[ii][a], xb[ii][b], acc[0]);
  }
  part[((size_t)tile * S2 + s) * 256 + threadIdx.x] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(&counters[tile], 1u) == (unsigned)(S2 - 1));
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double sq[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) sq[q] = 0.0;
  int q0 = 0;
  for (; q0 + 8 <= S2; q0 += 8) {
#pragma unroll
    for (int q = 0; q < 8; ++q) sq[q] += __ldcg(&part[((size_t)tile * S2 + q0 + q) * 256 + threadIdx.x]);
  }
  for (int q = 0; q0 + q < S2; ++q) sq[q] += __ldcg(&part[((size_t)tile * S2 + q0 + q) * 256 + threadIdx.x]);
  const double sum = ((sq[0] + sq[1]) + (sq[2] + sq[3])) + ((sq[4] + sq[5]) + (sq[6] + sq[7]));
  if (r1 < R && r2 < R) {
    G[(size_t)r1 * R + r2] = sum;
    G[(size_t)r2 * R + r1] = sum;
  }
  if (threadIdx.x == 0) counters[tile] = 0u;
  if (!FIN) return;
  if (fa.last) {
    // this tile's share of ||X||^2 = sum(Graw .* prod_{m != mode} G_m) (lambda_r lambda_c
    // times the normalised Gram of this mode is its raw Gram); off-diagonal tiles count twice
    // (an exact fixed-point sum: the fit's terms cancel near fit -> 1)
    double h = 0.0;
    if (r1 < R && r2 < R) {
      h = (ti == tj) ? sum : 2.0 * sum;
      for (int m = 0; m < fa.order; ++m)
        if (m != fa.mode) h *= fa.gs.G[m][(size_t)r1 * R + r2];
    }
    __shared__ int si_t[32];
    __shared__ long long sl_t[64];
    const int em = block_max_int(fx_exp(h), si_t);
    const int base = (em == 0x7ff) ? kFxBad : em - kFxHead;
    const __int128 q = block_sum_fx(base == kFxBad ? (__int128)0 : fx_term(h, base), sl_t);
    if (threadIdx.x == 0) {
      long long* fp = reinterpret_cast<long long*>(fa.fpart);
      fp[3 * tile] = (long long)(unsigned long long)q;
      fp[3 * tile + 1] = (long long)(q >> 64);
      fp[3 * tile + 2] = base;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(&counters[ntiles], 1u) == (unsigned)(ntiles - 1));
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x == 0) counters[ntiles] = 0u;
  finalize_body(G, R, fa, true);
}

// G from the solve blocks' partial Grams: 32 upper-triangle entries per block, eight
// slices of the partials per entry summed in block order and then across the slices in a
// fixed order; the block's share of ||X||^2 goes to fa.fpart, and the last block to finish
// runs finalize_body (lambda, fit, check).
__global__ void __launch_bounds__(256) k_gram_rows(const double* __restrict__ gpart, int nblk, int R,
                                                   double* __restrict__ G, unsigned* __restrict__ counter,
                                                   const DevCheck* chk, FinalizeArgs fa) {
  if (done_flag(chk)) return;
  __shared__ double red[8][33];
  __shared__ int s_last;
  const int T = R * (R + 1) / 2;
  const int lane = threadIdx.x & 31, sl = threadIdx.x >> 5;
  const int e = blockIdx.x * 32 + lane;
  // warp sl sums partials sl, sl + 8, ...: four accumulators, four loads in flight
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  if (e < T) {
    int b = sl;
    for (; b + 24 < nblk; b += 32) {
      const double v0 = gpart[(size_t)b * T + e], v1 = gpart[(size_t)(b + 8) * T + e];
      const double v2 = gpart[(size_t)(b + 16) * T + e], v3 = gpart[(size_t)(b + 24) * T + e];
      a0 += v0;
      a1 += v1;
      a2 += v2;
      a3 += v3;
    }
    for (; b < nblk; b += 8) a0 += gpart[(size_t)b * T + e];
  }
  red[sl][lane] = (a0 + a1) + (a2 + a3);
  __syncthreads();
  double h = 0.0;
  if (sl == 0 && e < T) {
    double sum = 0.0;
    for (int q = 0; q < 8; ++q) sum += red[q][lane];
    const int p = e / (R + 1), t = e - p * (R + 1);
    int a, c;
    if (t < R - p) {
      a = p;
      c = p + t;
    } else {
      a = R - 1 - p;
      c = a + (t - (R - p));
    }
    G[(size_t)a * R + c] = sum;
    G[(size_t)c * R + a] = sum;
    if (fa.last) {  // this entry's share of ||X||^2
      h = (a == c) ? sum : 2.0 * sum;
      for (int m = 0; m < fa.order; ++m)
        if (m != fa.mode) h *= fa.gs.G[m][(size_t)a * R + c];
    }
  }
  if (fa.last && sl == 0) {  // the block's 32 shares (warp 0), summed exactly in fixed point
    const int em = __reduce_max_sync(0xffffffffu, fx_exp(h));
    const int base = (em == 0x7ff) ? kFxBad : em - kFxHead;
    const __int128 q = fx_warp_sum(base == kFxBad ? (__int128)0 : fx_term(h, base));
    if (lane == 0) {
      long long* fp = reinterpret_cast<long long*>(fa.fpart);
      fp[3 * blockIdx.x] = (long long)(unsigned long long)q;
      fp[3 * blockIdx.x + 1] = (long long)(q >> 64);
      fp[3 * blockIdx.x + 2] = base;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x == 0) *counter = 0u;
  finalize_body(G, R, fa, true);
}

__global__ void __launch_bounds__(256) k_finalize(const double* __restrict__ Graw, int R, FinalizeArgs fa) {
  if (done_flag(fa.chk)) return;
  finalize_body(Graw, R, fa, false);
}

// ---------------- normalize ----------------
// Entry (i, r) of the new factor f = X(i, r) / lambda_r and its copies: the FP32 row-major
// copy, its FP32 remainder, and the BF16 hi / lo pair in the tensor-core MTTKRP's tile.
__device__ __forceinline__ void store_factor_entry(int64_t i, int r, int R, double f, double* __restrict__ F,
                                                   float* __restrict__ F32r, float* __restrict__ F32lo, int64_t rpad,
                                                   const BtileDesc& btd) {
  F[i * R + r] = f;
  if (F32r) F32r[i * rpad + r] = (float)f;
  if (F32lo) F32lo[i * rpad + r] = (float)(f - (double)(float)f);  // f = hi + lo to 2^-48
  if (btd.bt) {
    // hi = bf16(f), lo = bf16(f - hi), at row i of column r in its tile
    const __nv_bfloat16 h = __double2bfloat16(f);
    const __nv_bfloat16 l = __double2bfloat16(f - (double)__bfloat162float(h));
    const int nblk = r / btd.nb, rr = r - nblk * btd.nb;
    const int64_t fb = i >> 6;
    const int kk = (int)(i & 63);
    uint8_t* tile = btd.bt + (size_t)(fb * btd.n_blocks + nblk) * (2 * (size_t)btd.nb * 64 * 2);
    const uint32_t off = (uint32_t)rr * 128u + ((uint32_t)((kk >> 3) ^ (rr & 7)) << 4) + (uint32_t)(kk & 7) * 2u;
    *reinterpret_cast<__nv_bfloat16*>(tile + off) = h;
    *reinterpret_cast<__nv_bfloat16*>(tile + (size_t)btd.nb * 64 * 2 + off) = l;
  }
}

__global__ void k_normalize(const double* __restrict__ X, const double* __restrict__ lam_inv, int64_t In, int R,
                            double* __restrict__ F, float* __restrict__ F32r,
                            int64_t rpad, const double* __restrict__ Graw, double* __restrict__ Gn,
                            const DevCheck* chk, BtileDesc btd, float* __restrict__ F32lo) {
  if (done_flag(chk)) return;
  const int64_t n = In * R;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    const int64_t i = e / R;
    const int r = (int)(e % R);
    const double f = lam_inv ? X[e] * lam_inv[r] : X[e];
    store_factor_entry(i, r, R, f, F, F32r, F32lo, rpad, btd);
  }
  // the normalised Gram G_n = Graw ./ (lambda lambda^T), by the reciprocals
  if (Gn)
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)R * R; e += stride) {
      const int r = (int)(e / R), c = (int)(e % R);
      Gn[e] = Graw[e] * lam_inv[r] * lam_inv[c];
    }
}

// ---------------- the fused mode tail: solve, Gram, lambda, normalisation ----------------
// One cooperative launch per mode (all blocks resident) in place of the solve, the Gram
// reduction and the normalisation kernels, with two grid barriers:
//   1. each block solves its RB rows (X stays in shared memory) and writes its partial Gram;
//   2. the blocks split the R(R+1)/2 Gram entries: each sums its entries over the blocks'
//      partials, writes Graw, and lambda, 1 / lambda for the diagonal ones; on the last mode
//      also its exact share of ||X||^2;
//   3. each block normalises its rows from shared memory and writes G_n entries; on the last
//      mode block 0 then runs the finalize step (the fit and the check).
// The barrier waits are bounded: on expiry the kernel records an error and carries on (the
// host reports CPALS_E_DEVICE); it never waits forever.
constexpr uint32_t kGridSpin = 1u << 22;
__device__ __forceinline__ void grid_barrier(GridBar* b, int* err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = &b->gen;
    const unsigned g0 = *gen;
    __threadfence();
    if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
      b->count = 0u;
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      uint32_t it = 0;
      while (*gen == g0) {
        if (++it > kGridSpin) {
          atomicExch(err, 1);
          break;
        }
        if (it > 64) __nanosleep(128);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

struct TailArgs {
  const void* part;
  int part_f32, S, R, RB;
  int64_t In;
  const double* WT;
  const SolveInfo* info;
  const float* ops;
  double* X;
  double* gpart;  // nblk * R(R+1)/2 partial Grams, then 3 words per block (||X||^2 shares)
  double* F;
  float* F32r;
  float* F32lo;
  int64_t rpad;
  BtileDesc btd;
  GridBar* bar;
  int* err;
  double* Graw;
  FinalizeArgs fa;  // lambda, 1 / lambda, G_n, the Grams, the fit's inputs
};

template <typename PT>
__global__ void __launch_bounds__(SOLVE_T) k_mode_tail(TailArgs a) {
  if (done_flag(a.fa.chk)) return;  // uniform: only block 0 sets `done`, after every block passed barrier 2
  extern __shared__ double sm[];
  const int R = a.R, RB = a.RB, tid = threadIdx.x, nt = blockDim.x;
  const int nblk = gridDim.x;
  const int T = R * (R + 1) / 2;
  // ---- 1: the rows' solve (X stays in shared memory), the block's partial Gram, the rows'
  // <T, X> terms on the last mode
  double* inner = a.fa.last ? const_cast<double*>(reinterpret_cast<const double*>(a.fa.inner_rows_fx)) : nullptr;
  solve_rows_body<PT>(static_cast<const PT*>(a.part), a.S, a.In, R, RB, a.WT, a.X, inner, a.info, a.ops, a.gpart,
                      blockIdx.x, sm);
  grid_barrier(a.bar, a.err);
  // ---- 2: Gram entries [e0, e1) of this block, each summed over the blocks' partials in
  // block order (eight slices of the partials, then the slices in order), 32 entries at a time
  const int per = (T + nblk - 1) / nblk;
  const int e0 = min(T, blockIdx.x * per), e1 = min(T, e0 + per);
  __shared__ double red[8][33];
  const int lane = tid & 31, sl = tid >> 5;
  auto entry = [&](int e, int& r, int& c) {  // the upper-triangle pairing of the partial Grams
    const int p = e / (R + 1), t = e - p * (R + 1);
    if (t < R - p) {
      r = p;
      c = p + t;
    } else {
      r = R - 1 - p;
      c = r + (t - (R - p));
    }
  };
  for (int eb = e0; eb < e1; eb += 32) {
    const int e = eb + lane;
    double acc = 0.0;
    if (e < e1)
      for (int b0 = sl; b0 < nblk; b0 += 64) {  // eight loads in flight, added in block order
        double v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = (b0 + 8 * q < nblk) ? __ldcg(&a.gpart[(size_t)(b0 + 8 * q) * T + e]) : 0.0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (b0 + 8 * q < nblk) acc += v[q];
      }
    red[sl][lane] = acc;
    __syncthreads();
    if (sl == 0 && e < e1) {
      double sum = 0.0;
      for (int q = 0; q < 8; ++q) sum += red[q][lane];
      int r, c;
      entry(e, r, c);
      a.Graw[(size_t)r * R + c] = sum;
      a.Graw[(size_t)c * R + r] = sum;
      if (r == c) {
        const double ri = rsqrt(sum);
        a.fa.lam[r] = sum * ri;
        a.fa.lam_inv[r] = ri;
      }
    }
    __syncthreads();
  }
  if (a.fa.last && sl == 0) {
    // this block's share of ||X||^2 = sum over its entries of Graw .* prod_{m != mode} G_m
    // (off-diagonal entries twice), exact in fixed point; each lane reads back the entries
    // it wrote above
    auto share = [&](int e) {
      int r, c;
      entry(e, r, c);
      double v = a.Graw[(size_t)r * R + c];
      v = (r == c) ? v : 2.0 * v;
      for (int m = 0; m < a.fa.order; ++m)
        if (m != a.fa.mode) v *= a.fa.gs.G[m][(size_t)r * R + c];
      return v;
    };
    int em = 1;
    for (int e = e0 + lane; e < e1; e += 32) em = max(em, fx_exp(share(e)));
    em = __reduce_max_sync(0xffffffffu, em);
    const int base = (em == 0x7ff) ? kFxBad : em - kFxHead;
    __int128 q = 0;
    if (base != kFxBad)
      for (int e = e0 + lane; e < e1; e += 32) q += fx_term(share(e), base);
    q = fx_warp_sum(q);
    if (lane == 0) {
      long long* fp = reinterpret_cast<long long*>(a.fa.fpart);
      fp[3 * blockIdx.x] = (long long)(unsigned long long)q;
      fp[3 * blockIdx.x + 1] = (long long)(q >> 64);
      fp[3 * blockIdx.x + 2] = base;
    }
  }
  grid_barrier(a.bar, a.err);
  // ---- 3: normalise this block's rows (X in shared memory) and write G_n entries
  const int64_t r0 = (int64_t)blockIdx.x * RB;
  const int rows = (a.In - r0 < (int64_t)RB) ? (int)(a.In - r0) : RB;
  const double* Xs = sm + 2 * RB * R;
  for (int e = tid; e < rows * R; e += nt) {
    const int row = e / R, r = e - row * R;
    store_factor_entry(r0 + row, r, R, Xs[e] * __ldcg(&a.fa.lam_inv[r]), a.F, a.F32r, a.F32lo, a.rpad, a.btd);
  }
  for (int e = blockIdx.x * nt + tid; e < R * R; e += nblk * nt) {
    const int r = e / R, c = e - r * R;
    a.fa.Gn[e] = __ldcg(&a.Graw[e]) * __ldcg(&a.fa.lam_inv[r]) * __ldcg(&a.fa.lam_inv[c]);
  }
  if (a.fa.last && blockIdx.x == 0) finalize_fit(R, a.fa, nullptr);  // fpart is set: lam unused
}

__global__ void k_transpose(const double* __restrict__ src, int64_t rows, int64_t cols, double* __restrict__ dst) {
  __shared__ double tile[32][33];
  const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t r = r0 + y, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[y][threadIdx.x] = src[r * cols + c];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t c = c0 + y, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[c * rows + r] = tile[threadIdx.x][y];
  }
}

template <typename PT>
__global__ void k_reduce_partials(const PT* __restrict__ part, int S, int64_t n, double* __restrict__ M) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int sp = 0; sp < S; ++sp) s += (double)part[(int64_t)sp * n + e];
    M[e] = s;
  }
}

// ---------------- ||T||^2 as a double-double ----------------
// FP32 tensors.  GB300 issues FP64 some 60 times slower than FP32 and integer work, so the
// exact sum uses integers: an FP32 entry is m 2^(e - 150) (m: 24-bit significand, e: biased
// exponent, 1 for subnormals), its square the 48-bit integer m^2 times 2^(2(e - 150)).  With
// e_max the exponent of the largest |entry|, each square is added into a 128-bit fixed-point
// sum in units of 2^(2(e_max - 150) - 32): shifted left by 32 - 2(e_max - e) bits (right when
// negative; bits below the unit, less than 2^-78 of the largest square each, are dropped).
// A square is below 2^80 units, so 2^40 entries stay below 2^120: no overflow.  Integer sums
// are associative, so the result does not depend on the order of the atomics.
__global__ void __launch_bounds__(256) k_absmax_bits(const float* __restrict__ T, int64_t n,
                                                     unsigned* __restrict__ out) {
  unsigned m = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    m = max(m, __float_as_uint(T[i]) & 0x7fffffffu);  // |x| orders as its bit pattern
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void __launch_bounds__(256) k_sumsq_f32(const float* __restrict__ T, int64_t n,
                                                   const unsigned* __restrict__ maxbits,
                                                   unsigned long long* __restrict__ acc) {
  const unsigned mb = *maxbits;
  if (mb == 0u || mb >= 0x7f800000u) return;  // all zero, or a non-finite entry
  const int emax = (int)(mb >> 23) + ((mb >> 23) == 0u ? 1 : 0);
  // the 128-bit sum as two 64-bit words, the shifts written out (a term is below 2^80)
  unsigned long long lo = 0, hi = 0;
  auto add = [&](float x) {
    const unsigned u = __float_as_uint(x) & 0x7fffffffu;
    const unsigned e = u >> 23;
    const unsigned long long mm = (unsigned long long)((u & 0x7fffffu) | (e ? 0x800000u : 0u));
    const unsigned long long sq = mm * mm;  // < 2^48, exact
    const int sh = 32 - 2 * (emax - ((int)e + (e == 0u ? 1 : 0)));
    const unsigned long long t = (sh >= 0) ? sq : ((sh > -64) ? (sq >> (-sh)) : 0ull);
    const int sl = sh > 0 ? sh : 0;  // 0 .. 32
    const unsigned long long tlo = t << sl;
    const unsigned long long thi = sl ? (t >> (64 - sl)) : 0ull;
    lo += tlo;
    hi += thi + (lo < tlo ? 1ull : 0ull);
  };
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t tid0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool al16 = (reinterpret_cast<uintptr_t>(T) & 15) == 0;
  const int64_t n4 = al16 ? n / 4 : 0;
  for (int64_t i = tid0; i < n4; i += stride) {  // 16-byte loads
    const float4 v = reinterpret_cast<const float4*>(T)[i];
    add(v.x);
    add(v.y);
    add(v.z);
    add(v.w);
  }
  for (int64_t i = 4 * n4 + tid0; i < n; i += stride) add(T[i]);
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long olo = __shfl_xor_sync(0xffffffffu, lo, off);
    const unsigned long long ohi = __shfl_xor_sync(0xffffffffu, hi, off);
    const unsigned long long nlo = lo + olo;
    hi += ohi + (nlo < lo ? 1ull : 0ull);
    lo = nlo;
  }
  if ((threadIdx.x & 31) == 0 && (lo | hi)) {
    const unsigned long long old = atomicAdd(&acc[0], lo);
    atomicAdd(&acc[1], hi + ((old + lo) < old ? 1ull : 0ull));
  }
}

// FP64 tensors: the same two passes; each square is split exactly by TwoProduct
// (x^2 = p + e) and both parts are added in 128-bit fixed point anchored at the largest
// square (6 more bits of headroom: 2^40 entries).
__global__ void __launch_bounds__(256) k_absmax_bits64(const double* __restrict__ T, int64_t n,
                                                       unsigned long long* __restrict__ out) {
  unsigned long long m = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    m = max(m, (unsigned long long)__double_as_longlong(T[i]) & 0x7fffffffffffffffull);
  for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__device__ __forceinline__ int sumsq64_base(unsigned long long mb) {
  if (mb >= 0x7ff0000000000000ull) return kFxBad;
  const double x = __longlong_as_double((long long)mb);
  const double p = x * x;
  if (!(p < INFINITY)) return kFxBad;
  return fx_exp(p) - kFxHead + 6;
}

__global__ void __launch_bounds__(256) k_sumsq_f64(const double* __restrict__ T, int64_t n,
                                                   const unsigned long long* __restrict__ maxbits,
                                                   unsigned long long* __restrict__ acc) {
  const int base = sumsq64_base(*maxbits);
  if (base == kFxBad || *maxbits == 0ull) return;
  __int128 q = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double x = T[i];
    const double p = x * x;
    q += fx_term(p, base) + fx_term(fma(x, x, -p), base);
  }
  q = fx_warp_sum(q);
  const unsigned long long lo = (unsigned long long)q, hi = (unsigned long long)(q >> 64);
  if ((threadIdx.x & 31) == 0 && (lo | hi)) {  // 128-bit two's complement add, carry by hand
    const unsigned long long old = atomicAdd(&acc[0], lo);
    atomicAdd(&acc[1], hi + ((old + lo) < old ? 1ull : 0ull));
  }
}

// q 2^(base - 1075) as a double-double (hi rounded, lo the exact remainder rounded)
__device__ DD fx_to_dd(__int128 q, int base) {
  const double hi = fx_to_double(q, base);
  return DD{hi, fx_to_double(q - fx_term(hi, base), base)};
}

__global__ void k_norm2_finish(int is_f32, const void* __restrict__ maxbits,
                               const unsigned long long* __restrict__ acc, DevCheck* chk) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  DD t{0.0, 0.0};
  int valid = 1;
  const __int128 q = (__int128)(((unsigned __int128)acc[1] << 64) | acc[0]);
  if (is_f32) {
    const unsigned mb = *static_cast<const unsigned*>(maxbits);
    if (mb >= 0x7f800000u) {
      valid = 0;
    } else if (mb != 0u) {
      // units of 2^(2(e_max - 150) - 32) = 2^(base - 1075)
      const int emax = (int)(mb >> 23) + ((mb >> 23) == 0u ? 1 : 0);
      t = fx_to_dd(q, 2 * (emax - 150) - 32 + 1075);
    }
  } else {
    const unsigned long long mb = *static_cast<const unsigned long long*>(maxbits);
    const int base = sumsq64_base(mb);
    if (base == kFxBad)
      valid = 0;
    else if (mb != 0ull)
      t = fx_to_dd(q, base);
  }
  chk->t2_hi = t.hi;
  chk->t2_lo = t.lo;
  chk->t2_valid = valid;
}

}  // namespace

size_t norm2_scratch_doubles() { return 4; }

cudaError_t launch_tensor_norm2(const void* T, int tdtype, int64_t n, double* scratch, DevCheck* chk, int num_sms,
                                cudaStream_t st) {
  // scratch: [0, 2) the 128-bit sum, [2] the largest |entry|'s bits
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(scratch);
  void* maxbits = scratch + 2;
  const int64_t want = (n + 255) / 256;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, 8 * (int64_t)num_sms));
  cudaError_t e = cudaMemsetAsync(scratch, 0, 4 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  if (tdtype == CPALS_DTYPE_F32) {
    const float* Tf = static_cast<const float*>(T);
    k_absmax_bits<<<blocks, 256, 0, st>>>(Tf, n, static_cast<unsigned*>(maxbits));
    k_sumsq_f32<<<blocks, 256, 0, st>>>(Tf, n, static_cast<const unsigned*>(maxbits), acc);
    k_norm2_finish<<<1, 32, 0, st>>>(1, maxbits, acc, chk);
  } else {
    const double* Td = static_cast<const double*>(T);
    k_absmax_bits64<<<blocks, 256, 0, st>>>(Td, n, static_cast<unsigned long long*>(maxbits));
    k_sumsq_f64<<<blocks, 256, 0, st>>>(Td, n, static_cast<const unsigned long long*>(maxbits), acc);
    k_norm2_finish<<<1, 32, 0, st>>>(0, maxbits, acc, chk);
  }
  return cudaGetLastError();
}

size_t factorize_work_doubles(int R) { return ops32_offset_doubles(R) + (3 * (size_t)rr4(R) + 1) / 2; }

cudaError_t launch_factorize(const GramSet& gs, int order, int skip, int R, double* work, double* U, int* piv,
                             double* W, SolveInfo* info, DevCheck* chk, cudaStream_t st, int mixed) {
  // work layout: [Aglob R*R (FP64 V of the FP32 sweep when R <= 128)][dinv R][qwork 4R^2 + 3R + 64]
  double* Aglob = work;
  double* dinv = work + (size_t)R * R;
  double* qwork = dinv + R;
  const size_t smem = (R <= 128) ? (size_t)R * (R | 1) * sizeof(double) : 0;
  cudaError_t ea = set_smem_limit_once((const void*)k_factorize, 200 * 1024);
  if (ea != cudaSuccess) return ea;
  mixed = (mixed && R <= 128) ? 1 : 0;
  if (mixed) {
    float* ops = reinterpret_cast<float*>(work + ops32_offset_doubles(R));
    const size_t sm32 = factorize32_smem_bytes(R);
    cudaError_t eb = set_smem_limit_once((const void*)k_factorize32, (int)factorize32_smem_bytes(128));
    if (eb != cudaSuccess) return eb;
    k_form_v32<<<(R * R + 255) / 256, 256, 0, st>>>(gs, order, skip, R, ops, chk);
    k_factorize32<<<1, FT32, sm32, st>>>(R, ops, info, chk);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const int C = mixed ? 0 : cluster_sweep_size(R);
  if (C > 0) {
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)C);
    cfg.blockDim = dim3(CLT);
    cfg.dynamicSmemBytes = cl_smem_bytes(R, C);
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_factorize_cluster, gs, order, skip, R, C, U, dinv, piv, W, info,
                                       (const DevCheck*)chk);
    if (e != cudaSuccess) return e;
  }
  k_factorize<<<1, FT, smem, st>>>(gs, order, skip, R, Aglob, U, dinv, piv, W, qwork, info, chk, mixed, C > 0);
  return cudaGetLastError();
}

int factorize_launches(int R, int mixed) {
  if (mixed && R <= 128) return 3;
  return cluster_sweep_size(R) > 0 ? 2 : 1;
}

namespace {
std::atomic<int> g_cl_min_rank{kClMinRank};
}

int set_cluster_sweep_min_rank(int r) { return g_cl_min_rank.exchange(r); }

// Cluster size of the FP64 sweep for rank R on the current device: 16 CTAs where the device
// can place such a cluster with the sweep's shared memory (a non-portable size, which GB300
// supports), else 0 (single CTA).
int cluster_sweep_size(int R) {
  if (R < g_cl_min_rank.load() || R > kClMaxRank) return 0;
  return cluster_sweep_device_size();
}

int cluster_sweep_device_size() {
  static std::mutex mu;
  static std::map<int, int> sizes;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  std::lock_guard<std::mutex> lock(mu);
  auto it = sizes.find(dev);
  if (it != sizes.end()) return it->second;
  int best = 0, optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess &&
      cudaFuncSetAttribute(k_factorize_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    const int C = 16;
    const size_t smem = cl_smem_bytes(kClMaxRank, C);
    if (smem <= (size_t)optin &&
        cudaFuncSetAttribute(k_factorize_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
            cudaSuccess) {
      cudaLaunchConfig_t cfg{};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)C;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3((unsigned)C);
      cfg.blockDim = dim3(CLT);
      cfg.dynamicSmemBytes = smem;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int n = 0;
      if (cudaOccupancyMaxActiveClusters(&n, k_factorize_cluster, &cfg) == cudaSuccess && n > 0) best = C;
    }
  }
  (void)cudaGetLastError();  // leave no error behind for the next launch check
  sizes[dev] = best;
  return best;
}

static int solve_rows_per_block(int R) { return R >= 256 ? 1 : 256 / R; }

int solve_blocks(int64_t In, int R) {
  const int RB = solve_rows_per_block(R);
  return (int)((In + RB - 1) / RB);
}

cudaError_t launch_solve_rows(const void* part, int part_is_f32, int splits, int64_t In, int R, const double* work,
                              const double* U, const int* piv, const double* W, const SolveInfo* info, double* X,
                              double* inner_rows, const DevCheck* chk, cudaStream_t st, double* gram_part) {
  (void)U;
  (void)piv;
  const int RB = solve_rows_per_block(R);
  dim3 grid((unsigned)((In + RB - 1) / RB));
  // M, products, X (doubles), M / residual and X0 (floats), then W (FP64) or the
  // refinement's [W | V_hi | V_lo] (FP32)
  const size_t fw = (size_t)((RB * R + 3) & ~3) / 2;
  size_t smem = ((size_t)3 * RB * R + 2 * fw + 1) * sizeof(double);
  if (R <= kSolveStageMaxR) smem += std::max((size_t)R * R * sizeof(double), (size_t)3 * rr4(R) * sizeof(float));
  {
    const int mx = (3 * 256 + 2 * 128 + 1) * 8 + 3 * rr4(kSolveStageMaxR) * 4;
    cudaError_t ea = set_smem_limit_once((const void*)k_solve_gemm<float>, mx);
    if (ea == cudaSuccess) ea = set_smem_limit_once((const void*)k_solve_gemm<double>, mx);
    if (ea != cudaSuccess) return ea;
  }
  const float* ops = reinterpret_cast<const float*>(work + ops32_offset_doubles(R));
  if (part_is_f32)
    k_solve_gemm<float><<<grid, SOLVE_T, smem, st>>>(static_cast<const float*>(part), splits, In, R, RB, W, X,
                                                     inner_rows, chk, info, ops, gram_part);
  else
    k_solve_gemm<double><<<grid, SOLVE_T, smem, st>>>(static_cast<const double*>(part), splits, In, R, RB, W, X,
                                                      inner_rows, chk, info, ops, gram_part);
  return cudaGetLastError();
}

// The fused tail's shared memory is the solve's; it runs when every block of rows can be
// resident at once (a cooperative launch).  Returns cudaErrorNotSupported when it cannot,
// and the caller takes the three-kernel path.
cudaError_t launch_mode_tail(const void* part, int part_is_f32, int splits, int64_t In, int R, const double* work,
                             const double* W, const SolveInfo* info, double* X, double* gram_part, double* F,
                             float* F32r, float* F32lo, int64_t rpad, BtileDesc btd, double* Graw, double* lam,
                             double* lam_inv, double* Gn, const GramSet& gs, int order, int last,
                             const double* inner_rows, DevCheck* chk, double* traj, int64_t traj_cap, GridBar* bar,
                             int* err, int num_sms, int run_check, cudaStream_t st) {
  const int RB = solve_rows_per_block(R);
  const int nblk = solve_blocks(In, R);
  const size_t fw = (size_t)((RB * R + 3) & ~3) / 2;
  size_t smem = ((size_t)3 * RB * R + 2 * fw + 1) * sizeof(double);
  if (R <= kSolveStageMaxR) smem += std::max((size_t)R * R * sizeof(double), (size_t)3 * rr4(R) * sizeof(float));
  const void* kfn = part_is_f32 ? (const void*)k_mode_tail<float> : (const void*)k_mode_tail<double>;
  {
    const int mx = (3 * 256 + 2 * 128 + 1) * 8 + 3 * rr4(kSolveStageMaxR) * 4;
    cudaError_t ea = set_smem_limit_once(kfn, mx);
    if (ea != cudaSuccess) return ea;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, SOLVE_T, smem);
  if (e != cudaSuccess) return e;
  if ((int64_t)per_sm * num_sms < nblk) return cudaErrorNotSupported;
  const int T = R * (R + 1) / 2;
  TailArgs a{};
  a.part = part;
  a.part_f32 = part_is_f32;
  a.S = splits;
  a.R = R;
  a.RB = RB;
  a.In = In;
  a.WT = W;
  a.info = info;
  a.ops = reinterpret_cast<const float*>(work + ops32_offset_doubles(R));
  a.X = X;
  a.gpart = gram_part;
  a.F = F;
  a.F32r = F32r;
  a.F32lo = F32lo;
  a.rpad = rpad;
  a.btd = btd;
  a.bar = bar;
  a.err = err;
  a.Graw = Graw;
  // the blocks' exact shares of ||X||^2 follow the partial Grams (3 words per block)
  a.fa = FinalizeArgs{lam, lam_inv, Gn, gs, order, last, reinterpret_cast<const long long*>(inner_rows), In, chk,
                      traj, traj_cap, order - 1, gram_part + (size_t)nblk * T, nblk, run_check};
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel(kfn, dim3((unsigned)nblk), dim3(SOLVE_T), args, smem, st);
}

size_t mode_tail_part_doubles(int nblk, int R) { return (size_t)nblk * R * (R + 1) / 2 + 3 * (size_t)nblk; }

int gram_tiles(int R) {
  const int nt = (R + GT - 1) / GT;
  return nt * (nt + 1) / 2;
}

int gram_splits(int64_t In, int R, int num_sms) {
  const int tiles = gram_tiles(R);
  int64_t s = (4LL * num_sms + tiles - 1) / tiles;
  const int64_t max_s = (In + 31) / 32;
  if (s > max_s) s = max_s;
  if (s < 1) s = 1;
  if (s > 512) s = 512;
  return (int)s;
}

cudaError_t launch_gram(const double* X, int64_t In, int R, int S2, double* part, unsigned* counters, double* G,
                        const DevCheck* chk, cudaStream_t st) {
  const int64_t rps = (In + S2 - 1) / S2;
  dim3 grid((unsigned)gram_tiles(R), (unsigned)S2);
  k_gram<false><<<grid, 256, 0, st>>>(X, In, R, S2, rps, part, counters, G, chk, FinalizeArgs{});
  return cudaGetLastError();
}

size_t gram_finalize_part_doubles(int S2, int R) { return (size_t)gram_tiles(R) * ((size_t)S2 * 256 + 3); }

cudaError_t launch_gram_finalize(const double* X, int64_t In, int R, int S2, double* part, unsigned* counters,
                                 double* Graw, double* lam, double* lam_inv, double* Gn, const GramSet& gs, int order,
                                 int last, const double* inner_rows, DevCheck* chk, double* traj, int64_t traj_cap,
                                 cudaStream_t st, int run_check) {
  const int64_t rps = (In + S2 - 1) / S2;
  dim3 grid((unsigned)gram_tiles(R), (unsigned)S2);
  const int ntiles = gram_tiles(R);
  // per-tile double-double partials of ||X||^2 live after the tile partial sums
  FinalizeArgs fa{lam, lam_inv, Gn, gs, order, last, reinterpret_cast<const long long*>(inner_rows), In, chk,
                  traj, traj_cap, order - 1, part + (size_t)ntiles * S2 * 256, ntiles, run_check};
  k_gram<true><<<grid, 256, 0, st>>>(X, In, R, S2, rps, part, counters, Graw, chk, fa);
  return cudaGetLastError();
}

size_t gram_rows_part_doubles(int nblk, int R) {
  const size_t T = (size_t)R * (R + 1) / 2;
  return (size_t)nblk * T + 3 * ((T + 31) / 32);
}

cudaError_t launch_gram_rows(const double* gram_part, int nblk, int R, unsigned* counter, double* Graw, double* lam,
                             double* lam_inv, double* Gn, const GramSet& gs, int order, int last,
                             const double* inner_rows, int64_t In, DevCheck* chk, double* traj, int64_t traj_cap,
                             cudaStream_t st, int run_check) {
  const int T = R * (R + 1) / 2;
  const int blocks = (T + 31) / 32;
  // the blocks' double-double shares of ||X||^2 follow the partial Grams
  double* fpart = const_cast<double*>(gram_part) + (size_t)nblk * T;
  FinalizeArgs fa{lam, lam_inv, Gn, gs, order, last, reinterpret_cast<const long long*>(inner_rows), In, chk,
                  traj, traj_cap, order - 1, fpart, blocks, run_check};
  k_gram_rows<<<blocks, 256, 0, st>>>(gram_part, nblk, R, Graw, counter, chk, fa);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const double* Graw, int R, double* lam, double* lam_inv, double* Gn, const GramSet& gs,
                            int order, int last, const double* inner_rows, int64_t In, DevCheck* chk, double* traj,
                            int64_t traj_cap, cudaStream_t st) {
  FinalizeArgs fa{lam, lam_inv, Gn, gs, order, last, reinterpret_cast<const long long*>(inner_rows), In, chk,
                  traj, traj_cap, order - 1, nullptr, 0, 1};
  k_finalize<<<1, 256, 0, st>>>(Graw, R, fa);
  return cudaGetLastError();
}

cudaError_t launch_check_step(DevCheck* chk, double* traj, int64_t traj_cap, cudaStream_t st) {
  k_check_step<<<1, 32, 0, st>>>(chk, traj, traj_cap);
  return cudaGetLastError();
}

cudaError_t launch_normalize(const double* X, const double* lam_inv, int64_t In, int R, double* F, float* F32r,
                             int64_t rpad, const double* Graw, double* Gn, const DevCheck* chk, cudaStream_t st,
                             BtileDesc bt, float* F32lo) {
  const int64_t n = In * R;
  int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  k_normalize<<<blocks, 256, 0, st>>>(X, lam_inv, In, R, F, F32r, rpad, Graw, Gn, chk, bt, F32lo);
  return cudaGetLastError();
}

cudaError_t launch_transpose_f64(const double* src, int64_t rows, int64_t cols, double* dst, cudaStream_t st) {
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  k_transpose<<<grid, dim3(32, 8), 0, st>>>(src, rows, cols, dst);
  return cudaGetLastError();
}

cudaError_t launch_reduce_partials(const void* part, int part_is_f32, int splits, int64_t In, int R, double* M,
                                   cudaStream_t st) {
  const int64_t n = In * R;
  int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  if (part_is_f32)
    k_reduce_partials<float><<<blocks, 256, 0, st>>>(static_cast<const float*>(part), splits, n, M);
  else
    k_reduce_partials<double><<<blocks, 256, 0, st>>>(static_cast<const double*>(part), splits, n, M);
  return cudaGetLastError();
}

}  // namespace cpals
