// Convergence checks that compare consecutive iterates instead of the target:
// CPDiffCheck (src/converge_checks/cp_diff_check.jl:20-68) and CPAngleCheck
// (src/converge_checks/cp_angle_check.jl:20-68).  Both need
//
//   <T_prev, T_curr> = lam_prev^T (P_0^T F_0 .* P_1^T F_1 .* ...) lam        (cp_cp_contract,
//                                                           src/algebra/cp_contract.jl:32-52)
//   ||T_curr||^2     = lam^T (G_0 .* G_1 .* ...) lam      (norm_factors, converge_checks.jl:5-11)
//
// with P_m the previous iterate's factors and G_m = F_m^T F_m the Grams the sweep keeps.
// The cross Grams are I_m x R by I_m x R FP64 products, and FP64 issue (two DFMA per clock
// per SM) is the limit: k_cross_gram cuts every cross Gram into 32 x 32 output tiles and
// splits of 8k rows, about six blocks per SM of about 2 us each, and writes the split
// partials.  k_cp_check sums the partials of 32 entries per block over 8 thread groups
// (fixed order), forms both quadratic forms, reduces them over its blocks in block order
// (the last block to finish does this) and runs the check's update on one thread.
//
// FP64 throughout: the fit between consecutive iterates, 1 - sqrt(|a + b - 2c|) / sqrt(a),
// cancels to the size of the change, so lower precision would hide changes below 1e-4.
#include "cpals_internal.cuh"

namespace cpals {
namespace {

constexpr int XT = 32;  // output tile edge
constexpr int XK = 8;   // rows staged per step (a split is a multiple of XK rows)

__device__ double warp_block_sum(double v, double* sv) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  __syncthreads();
  if (lane == 0) sv[w] = v;
  __syncthreads();
  double t = (lane < nw) ? sv[lane] : 0.0;
  for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  __syncthreads();
  return t;
}

// grid (Smax, nt*nt, order), 256 threads.  Block (s, tile, m) computes rows [r0, r1) of
// P_m^T F_m for the 32 x 32 tile (ti, tj), two by two outputs per thread; the tile-0
// blocks also copy those rows of F_m (and block (0, 0, 0) lambda) into the buffer that
// becomes PrevCP.
__global__ void __launch_bounds__(256) k_cross_gram(CrossArgs a) {
  const DevCheck* chk = a.chk;
  if (chk->done) return;
  const int s = blockIdx.x, tile = blockIdx.y, m = blockIdx.z;
  if (s >= a.S[m]) return;
  __shared__ double ps[XK][XT];
  __shared__ double fs[XK][XT];
  const int R = a.R;
  const int nt = (R + XT - 1) / XT;
  const int ti = tile / nt, tj = tile - ti * nt;
  const int64_t In = a.dims[m];
  const int64_t r0 = min(In, (int64_t)s * a.rows), r1 = min(In, r0 + a.rows);
  const int sel = chk->psel;
  const double* __restrict__ Fm = a.F[m];
  if (tile == 0) {
    double* __restrict__ dst = a.prevF[sel ^ 1] + a.off[m];
    for (int64_t e = r0 * R + threadIdx.x; e < r1 * R; e += blockDim.x) dst[e] = Fm[e];
    if (m == 0 && s == 0)
      for (int r = threadIdx.x; r < R; r += blockDim.x) a.prevLam[sel ^ 1][r] = a.lam[r];
  }
  if (!chk->has_prev) return;
  const double* __restrict__ Pm = a.prevF[sel] + a.off[m];
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const int lk = threadIdx.x >> 5, lc = threadIdx.x & 31;  // staging: one row, one column
  const int ca = ti * XT + lc, cb = tj * XT + lc;
  double acc00 = 0.0, acc01 = 0.0, acc10 = 0.0, acc11 = 0.0;
  for (int64_t kk = r0; kk < r1; kk += XK) {
    const int64_t row = kk + lk;
    ps[lk][lc] = (row < r1 && ca < R) ? Pm[row * R + ca] : 0.0;
    fs[lk][lc] = (row < r1 && cb < R) ? Fm[row * R + cb] : 0.0;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < XK; ++k) {
      const double p0 = ps[k][ty], p1 = ps[k][ty + 16];
      const double f0 = fs[k][tx], f1 = fs[k][tx + 16];
      acc00 = fma(p0, f0, acc00);
      acc01 = fma(p0, f1, acc01);
      acc10 = fma(p1, f0, acc10);
      acc11 = fma(p1, f1, acc11);
    }
    __syncthreads();
  }
  double* __restrict__ out = a.xpart + ((int64_t)m * a.Smax + s) * (int64_t)R * R;
  const int r_0 = ti * XT + ty, r_1 = r_0 + 16, c_0 = tj * XT + tx, c_1 = c_0 + 16;
  if (r_0 < R) {
    if (c_0 < R) out[(int64_t)r_0 * R + c_0] = acc00;
    if (c_1 < R) out[(int64_t)r_0 * R + c_1] = acc01;
  }
  if (r_1 < R) {
    if (c_0 < R) out[(int64_t)r_1 * R + c_0] = acc10;
    if (c_1 < R) out[(int64_t)r_1 * R + c_1] = acc11;
  }
}

// The check's update (cp_diff_check.jl:20-68 / cp_angle_check.jl:20-68) on one thread.
__device__ void cp_check_update(DevCheck& k, double inner, double self, double* traj, int64_t traj_cap) {
  const bool angle = (k.kind == CPALS_CHECK_ANGLE);
  k.iter += 1;
  if (!k.has_prev) {  // PrevCP === nothing: store this iterate and its norm
    k.has_prev = 1;
    k.norm_prev = angle ? sqrt(self) : self;
    k.psel ^= 1;
    if (k.sweeps < traj_cap) traj[k.sweeps] = NAN;
    k.sweeps += 1;
    return;
  }
  double cur, norm_now;
  if (angle) {
    norm_now = sqrt(self);
    double theta = inner / (norm_now * k.norm_prev);
    theta = theta > 1.0 ? 1.0 : theta;  // NaN passes through, as in the reference
    cur = acos(theta);
  } else {
    norm_now = self;
    const double nres = sqrt(fabs(k.norm_prev + self - 2.0 * fabs(inner)));
    cur = 1.0 - nres / sqrt(fabs(k.norm_prev));
  }
  const double delta = fabs(k.lastfit - cur);
  k.lastfit = cur;
  k.psel ^= 1;
  k.norm_prev = norm_now;
  if (k.sweeps < traj_cap) traj[k.sweeps] = cur;
  k.sweeps += 1;
  if (delta < k.tol) {
    k.counter += 1;
    if (k.counter >= 2) {
      k.total_iter = k.iter;
      k.iter = 0;
      k.counter = 0;
      k.final_fit = k.lastfit;
      k.lastfit = 0.0;
      k.has_prev = 0;
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
    k.has_prev = 0;
  }
}

// grid ceil(R*R / 32), 256 threads: 32 entries e = (r, c) per block, 8 groups of split
// indices (s = g, g + 8, ...).  Warp 0 then forms lam_prev[r] lam[c] prod_m C_m[r][c] and
// lam[r] lam[c] prod_m G_m[r][c] for its entries.
__global__ void __launch_bounds__(256) k_cp_check(CrossArgs a) {
  DevCheck* chk = a.chk;
  if (chk->done) return;
  __shared__ double sp[8][33];
  __shared__ double sv[8];
  __shared__ int s_last;
  const int R = a.R;
  const int64_t RR = (int64_t)R * R;
  const int sel = chk->psel;
  const int has_prev = chk->has_prev;
  const int j = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int64_t e = (int64_t)blockIdx.x * 32 + j;
  const bool valid = e < RR;
  double h = 1.0;
  if (has_prev) {
    for (int m = 0; m < a.order; ++m) {
      double x = 0.0;
      if (valid) {
        const double* __restrict__ xp = a.xpart + (int64_t)m * a.Smax * RR + e;
        for (int s = g; s < a.S[m]; s += 8) x += xp[(int64_t)s * RR];
      }
      sp[g][j] = x;
      __syncthreads();
      if (g == 0) {
        double t = 0.0;
#pragma unroll
        for (int q = 0; q < 8; ++q) t += sp[q][j];
        h *= t;
      }
      __syncthreads();
    }
  }
  if (g == 0) {
    double inner = 0.0, self = 0.0;
    if (valid) {
      const int r = (int)(e / R), c = (int)(e - (int64_t)r * R);
      double gm = a.lam[r] * a.lam[c];
      for (int m = 0; m < a.order; ++m) gm *= a.G[m][e];
      self = gm;
      if (has_prev) inner = a.prevLam[sel][r] * h * a.lam[c];
    }
    for (int off = 16; off > 0; off >>= 1) {
      inner += __shfl_xor_sync(0xffffffffu, inner, off);
      self += __shfl_xor_sync(0xffffffffu, self, off);
    }
    if (j == 0) {
      a.red[2 * blockIdx.x] = inner;
      a.red[2 * blockIdx.x + 1] = self;
      __threadfence();
      s_last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double ti = 0.0, ts = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    ti += __ldcg(&a.red[2 * b]);
    ts += __ldcg(&a.red[2 * b + 1]);
  }
  ti = warp_block_sum(ti, sv);
  ts = warp_block_sum(ts, sv);
  if (threadIdx.x != 0) return;
  *a.counter = 0u;
  cp_check_update(*chk, ti, ts, a.traj, a.traj_cap);
}

}  // namespace

int64_t cross_rows(int order, const int64_t* dims, int R, int num_sms) {
  const int64_t nt = (R + XT - 1) / XT;
  int64_t units = 0;  // rows x tiles over all modes
  for (int m = 0; m < order; ++m) units += dims[m] * nt * nt;
  const int64_t target = 6 * (int64_t)num_sms;
  int64_t rows = (units + target - 1) / target;
  rows = (rows + XK - 1) / XK * XK;
  return rows < XK ? XK : rows;
}

cudaError_t launch_cp_check(const CrossArgs& a, cudaStream_t st) {
  const int nt = (a.R + XT - 1) / XT;
  k_cross_gram<<<dim3(a.Smax, nt * nt, a.order), 256, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int64_t RR = (int64_t)a.R * a.R;
  k_cp_check<<<(unsigned)((RR + 31) / 32), 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace cpals
