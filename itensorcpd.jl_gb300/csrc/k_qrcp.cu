// Column-pivoted Householder QR and the gathers that feed it, for the QR-pivoted
// projection solvers (QRPivProjected, SEQRCSPivProjected, KSEQRCSPivProjected:
// src/optimizers/als_optimizers/randomized/qr_lev_score_sampled.jl) and SE-QRCS
// (src/algebra/SEQRCS.jl).  The reference factors with LinearAlgebra's qr(A, ColumnNorm()),
// LAPACK's xGEQP3; the pivots must be the ones it picks.
//
// The factorization is Businger and Golub's (1965) QR with column pivoting.  Step j takes the
// trailing column of largest partial norm (the lowest position among equal norms, as
// IDAMAX does), swaps it to position j, reduces it with a Householder reflector
// H = I - tau v v^T (v_0 = 1, beta = -sign(alpha) ||x||, tau = (beta - alpha) / beta, the
// convention of LAPACK's xLARFG) and applies H to the trailing columns.  The partial norms are
// downdated as in xLAQP2, with the safeguard of Drmač and Bujanović (2008): after a step,
// vn1 *= sqrt(1 - (r_jc / vn1)^2) unless (1 - (r_jc / vn1)^2)(vn1 / vn2)^2 <= sqrt(eps), in which
// case the norm is recomputed from the trailing entries and vn2 is reset to it.  With the same
// rule and the same downdating, pivots agree with xGEQP3 except for columns whose norms tie to
// rounding.
//
// Data: A is m x n, column-major FP64, factored in place (R above the diagonal, v below it).
// One step is two launches: k_qrcp_reflect (one block: the pivot from the previous launch's
// per-block argmax partials, the column swap, the reflector) and k_qrcp_apply (the grid, one
// warp per trailing column: w = v^T x, x -= tau w v, the norm downdate, and this block's
// argmax partial).  The apply pass is FP64-issue bound (two FMAs per entry, plus the
// recompute pass when the safeguard fires); for columns of at most 1024 rows a warp keeps its
// column in registers, so A is read and written once per step.
#include <cfloat>
#include <cstdint>

#include "cpals_internal.cuh"

namespace cpals {
namespace {

constexpr int QW = 8;  // warps per block of the column kernels
constexpr unsigned FULL = 0xffffffffu;
constexpr double kTol3z = 1.4901161193847656e-08;  // sqrt(DBL_EPSILON)

__device__ __forceinline__ bool better(double v1, int64_t i1, double v2, int64_t i2) {
  return v1 > v2 || (v1 == v2 && i1 < i2);
}

__device__ __forceinline__ double warp_sum(double s) {
  for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(FULL, s, off);
  return s;
}

__device__ __forceinline__ void warp_best(double& v, int64_t& i) {
  for (int off = 16; off; off >>= 1) {
    const double ov = __shfl_xor_sync(FULL, v, off);
    const int64_t oi = __shfl_xor_sync(FULL, i, off);
    if (better(ov, oi, v, i)) {
      v = ov;
      i = oi;
    }
  }
}

// block-wide best over warps; every thread gets the result
__device__ void block_best(double& v, int64_t& i) {
  __shared__ double sv[32];
  __shared__ int64_t si[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  warp_best(v, i);
  __syncthreads();
  if (lane == 0) {
    sv[w] = v;
    si[w] = i;
  }
  __syncthreads();
  v = (lane < nw) ? sv[lane] : -1.0;
  i = (lane < nw) ? si[lane] : INT64_MAX;
  warp_best(v, i);
  __syncthreads();
}

__device__ double block_sum(double s) {
  __shared__ double sb[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  s = warp_sum(s);
  __syncthreads();
  if (lane == 0) sb[w] = s;
  __syncthreads();
  s = (lane < nw) ? sb[lane] : 0.0;
  s = warp_sum(s);
  __syncthreads();
  return s;
}

// Initial column norms vn1 = vn2 = ||A(:, c)|| and the per-block argmax over candidates.
__global__ void __launch_bounds__(QW * 32) k_qrcp_norms(const double* __restrict__ A, int64_t m, int64_t n,
                                                        int64_t ncand, double* __restrict__ vn1,
                                                        double* __restrict__ vn2, QrcpArg* __restrict__ part) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double bv = -1.0;
  int64_t bi = INT64_MAX;
  for (int64_t c = (int64_t)blockIdx.x * QW + w; c < n; c += (int64_t)gridDim.x * QW) {
    const double* __restrict__ x = A + c * m;
    double s = 0.0;
    for (int64_t i = lane; i < m; i += 32) s = fma(x[i], x[i], s);
    const double nrm = sqrt(warp_sum(s));
    if (lane == 0) {
      vn1[c] = nrm;
      vn2[c] = nrm;
    }
    if (c < ncand && better(nrm, c, bv, bi)) {
      bv = nrm;
      bi = c;
    }
  }
  block_best(bv, bi);
  if (threadIdx.x == 0) part[blockIdx.x] = QrcpArg{bv, bi};
}

// Step j, one block: pivot, swap, reflector.
__global__ void __launch_bounds__(1024) k_qrcp_reflect(double* __restrict__ A, int64_t m, int64_t n, int64_t ncand,
                                                       int64_t j, double* __restrict__ vn1, double* __restrict__ vn2,
                                                       int64_t* __restrict__ perm, const QrcpArg* __restrict__ part,
                                                       int nparts, double* __restrict__ vbuf, double* __restrict__ taus,
                                                       double* __restrict__ rdiag, QrcpState* st, int64_t kmax,
                                                       double stop_ratio) {
  if (st->done) return;
  __shared__ double s_beta, s_scale, s_tau;
  double bv = -1.0;
  int64_t bi = INT64_MAX;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x)
    if (better(part[q].v, part[q].i, bv, bi)) {
      bv = part[q].v;
      bi = part[q].i;
    }
  block_best(bv, bi);
  const int64_t p = (bi >= j && bi < ncand && bi < n) ? bi : j;
  double* __restrict__ xj = A + j * m;
  if (p != j) {
    double* __restrict__ xp = A + p * m;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
      const double t = xj[i];
      xj[i] = xp[i];
      xp[i] = t;
    }
    if (threadIdx.x == 0) {
      const int64_t t = perm[j];
      perm[j] = perm[p];
      perm[p] = t;
      vn1[p] = vn1[j];
      vn2[p] = vn2[j];
    }
  }
  __syncthreads();
  double s = 0.0;
  for (int64_t i = j + 1 + threadIdx.x; i < m; i += blockDim.x) s = fma(xj[i], xj[i], s);
  s = block_sum(s);
  if (threadIdx.x == 0) {
    const double alpha = xj[j];
    double beta = alpha, tau = 0.0, scale = 0.0;
    if (s > 0.0) {
      beta = -copysign(sqrt(fma(alpha, alpha, s)), alpha);
      tau = (beta - alpha) / beta;
      scale = 1.0 / (alpha - beta);
    }
    s_beta = beta;
    s_tau = tau;
    s_scale = scale;
  }
  __syncthreads();
  const double scale = s_scale;
  for (int64_t i = j + 1 + threadIdx.x; i < m; i += blockDim.x) {
    const double v = xj[i] * scale;
    xj[i] = v;
    vbuf[i] = v;
  }
  if (threadIdx.x == 0) {
    const double beta = s_beta;
    vbuf[j] = 1.0;
    xj[j] = beta;
    taus[j] = s_tau;
    rdiag[j] = beta;
    st->tau = s_tau;
    if (j == 0) st->r00 = fabs(beta);
    st->steps = j + 1;
    st->active = j + 1;  // 0: no step has run
    if (j + 1 >= kmax || (stop_ratio >= 0.0 && !(fabs(beta) > stop_ratio * st->r00))) st->done = 1;
  }
}

// xLAQP2's downdate of the partial norm of this lane's pending column pc (x0 = its new row-j
// entry, r_jc), and the column's entry into the lane's argmax.  The warp keeps one pending
// column per lane and runs the 32 downdates together, one per lane, instead of 32 copies of
// each.  xLAQP2 tests (1 - (x0/a)^2)(a/b)^2 <= sqrt(eps) and scales a by sqrt(1 - (x0/a)^2);
// here the same quantities without divisions: max(a^2 - x0^2, 0) <= sqrt(eps) b^2, and
// a = sqrt(max(a^2 - x0^2, 0)).  When the test fires the lane recomputes the norm from the
// trailing entries of its column.
__device__ __forceinline__ void downdate_lane(double px0, int64_t& pc, const double* __restrict__ A, int64_t m,
                                              int64_t j, int64_t len, double* __restrict__ vn1,
                                              double* __restrict__ vn2, int64_t ncand, double& bv, int64_t& bi) {
  __syncwarp();  // the warp's stores to its columns are visible to every lane
  if (pc >= 0 && pc < ncand) {
    double a = vn1[pc], b = vn2[pc];
    if (a != 0.0) {
      double s = fma(-px0, px0, a * a);
      s = s > 0.0 ? s : 0.0;
      if (s <= kTol3z * (b * b)) {
        const double* __restrict__ x = A + pc * m + j;
        double t0 = 0.0, t1 = 0.0;
        int64_t i = 1;
        for (; i + 1 < len; i += 2) {
          t0 = fma(x[i], x[i], t0);
          t1 = fma(x[i + 1], x[i + 1], t1);
        }
        if (i < len) t0 = fma(x[i], x[i], t0);
        a = sqrt(t0 + t1);
        b = a;
      } else {
        a = sqrt(s);
      }
      vn1[pc] = a;
      vn2[pc] = b;
    }
    if (better(a, pc, bv, bi)) {
      bv = a;
      bi = pc;
    }
  }
  pc = -1;
}

// Step j, the grid: apply H_j to columns j+1 .. n-1, downdate the candidates' norms, and write
// this block's argmax partial.  A warp takes 32 / LPC columns at a time, LPC lanes each; a lane
// holds rows j + s, j + s + LPC, ... of its column in CH registers (m - j <= LPC CH).  CH == 0
// (LPC = 32): two passes over global memory.  Two FMAs per entry (w = v^T x, then the update);
// the reduction of w takes log2(LPC) shuffle steps shared by the warp's columns, and the norm
// downdates run one per lane (downdate_lane).
template <int LPC, int CH>
__global__ void __launch_bounds__(QW * 32) k_qrcp_apply(double* __restrict__ A, int64_t m, int64_t n, int64_t ncand,
                                                        int64_t j, double* __restrict__ vn1, double* __restrict__ vn2,
                                                        const double* __restrict__ vbuf, const QrcpState* st,
                                                        QrcpArg* __restrict__ part) {
  static_assert(LPC == 8 || LPC == 16 || LPC == 32, "lanes per column");
  static_assert(CH > 0 || LPC == 32, "the two-pass form uses whole warps");
  constexpr int G = 32 / LPC;  // columns per warp step
  if (st->active != j + 1) return;  // step j's reflector was not formed
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane / LPC, sl = lane % LPC;
  const double tau = st->tau;
  const int64_t len = m - j;
  const double* __restrict__ v = vbuf + j;
  double bv = -1.0;
  int64_t bi = INT64_MAX;
  double px0 = 0.0;  // this lane's pending column and its new row-j entry
  int64_t pc = -1;
  int slot = 0;
  const int64_t wstride = (int64_t)gridDim.x * QW * G;
  for (int64_t base = j + 1 + ((int64_t)blockIdx.x * QW + w) * G; base < n; base += wstride) {
    const int64_t c = base + g;
    const bool live = c < n;
    double* __restrict__ x = A + (live ? c : base) * m + j;
    double x0;
    if constexpr (CH > 0) {
      double xr[CH];
      double d0 = 0.0, d1 = 0.0;  // two chains halve the dependent FMA latency
#pragma unroll
      for (int q = 0; q < CH; ++q) {
        const int64_t i = sl + (int64_t)LPC * q;
        const bool in = live && i < len;
        xr[q] = in ? x[i] : 0.0;
        if (in) {
          if (q & 1)
            d1 = fma(v[i], xr[q], d1);
          else
            d0 = fma(v[i], xr[q], d0);
        }
      }
      double d = d0 + d1;
#pragma unroll
      for (int off = LPC / 2; off; off >>= 1) d += __shfl_xor_sync(FULL, d, off);
      const double t = tau * d;
#pragma unroll
      for (int q = 0; q < CH; ++q) {
        const int64_t i = sl + (int64_t)LPC * q;
        if (live && i < len) {
          xr[q] = fma(-t, v[i], xr[q]);
          x[i] = xr[q];
        }
      }
      x0 = xr[0];  // row j of column c, held by sub-lane 0 of each group
    } else {
      double d0 = 0.0, d1 = 0.0;
      for (int64_t i = lane; i < len; i += 64) {
        d0 = fma(v[i], x[i], d0);
        if (i + 32 < len) d1 = fma(v[i + 32], x[i + 32], d1);
      }
      const double t = tau * warp_sum(d0 + d1);
      for (int64_t i = lane; i < len; i += 32) x[i] = fma(-t, v[i], x[i]);
      __syncwarp();
      x0 = x[0];
    }
    // hand the G new columns to lanes slot .. slot + G - 1 for their downdates
    const int rel = lane - slot;
    const bool mine = rel >= 0 && rel < G;
    const double got = __shfl_sync(FULL, x0, mine ? rel * LPC : 0);
    if (mine && base + rel < n) {
      px0 = got;
      pc = base + rel;
    }
    slot += G;
    if (slot == 32) {
      downdate_lane(px0, pc, A, m, j, len, vn1, vn2, ncand, bv, bi);
      slot = 0;
    }
  }
  if (slot > 0) downdate_lane(px0, pc, A, m, j, len, vn1, vn2, ncand, bv, bi);
  block_best(bv, bi);
  if (threadIdx.x == 0) part[blockIdx.x] = QrcpArg{bv, bi};
}

// Q = H_0 H_1 ... H_{k-1} [I; 0] by backward accumulation (as xORG2R): for j = k-1 .. 0,
// columns j .. kq-1 of Q get H_j, with v read from column j of the factored A.
__global__ void __launch_bounds__(QW * 32) k_qr_apply_q(double* __restrict__ Q, int64_t m, int64_t kq, int64_t j,
                                                        const double* __restrict__ A, const double* __restrict__ taus) {
  const double tau = taus[j];
  if (tau == 0.0) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const double* __restrict__ vt = A + j * m + j;  // v_0 = 1 is implicit
  const int64_t len = m - j;
  for (int64_t c = j + (int64_t)blockIdx.x * QW + w; c < kq; c += (int64_t)gridDim.x * QW) {
    double* __restrict__ x = Q + c * m + j;
    double d = 0.0;
    for (int64_t i = lane; i < len; i += 32) d = fma(i == 0 ? 1.0 : vt[i], x[i], d);
    const double t = tau * warp_sum(d);
    for (int64_t i = lane; i < len; i += 32) x[i] = fma(-t, i == 0 ? 1.0 : vt[i], x[i]);
  }
}

__global__ void k_eye(double* __restrict__ Q, int64_t m, int64_t kq) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m * kq; e += (int64_t)gridDim.x * blockDim.x)
    Q[e] = (e % m == e / m) ? 1.0 : 0.0;
}

__global__ void k_iota(int64_t* __restrict__ p, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) p[e] = e;
}

// Columns of the mode-k unfolding T_(k) (In x prod_{m != k} I_m): out(:, c) = T_(k)(:, cols[c])
// (cols 0-based; identity when null).  Column col starts at (col / stride) stride In +
// col % stride, stride = prod_{m < k} I_m, and steps by stride.  32 x 32 tiles through shared
// memory, so reads run along consecutive columns and writes along rows.
template <typename TT>
__global__ void k_unfold_cols(const TT* __restrict__ T, int64_t In, int64_t stride, const int64_t* __restrict__ cols,
                              int64_t ncols, double* __restrict__ out) {
  __shared__ double tile[32][33];
  for (int64_t cb = (int64_t)blockIdx.x * 32; cb < ncols; cb += (int64_t)gridDim.x * 32) {
    for (int64_t ib = (int64_t)blockIdx.y * 32; ib < In; ib += (int64_t)gridDim.y * 32) {
      const int64_t c = cb + threadIdx.x;
      int64_t base = 0;
      if (c < ncols) {
        const int64_t col = cols ? cols[c] : c;
        base = (col / stride) * stride * In + (col % stride);
      }
      for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = ib + r;
        if (c < ncols && i < In) tile[r][threadIdx.x] = (double)T[base + stride * i];
      }
      __syncthreads();
      for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int64_t cc = cb + q, i = ib + threadIdx.x;
        if (cc < ncols && i < In) out[cc * In + i] = tile[threadIdx.x][q];
      }
      __syncthreads();
    }
  }
}

// Rows of the Khatri-Rao product of the factors other than `mode`, transposed:
// out(r, c) = prod_{m != mode} F_m(i_m(col_c), r), R x ncols column-major, with col_c's
// coordinates over the other modes in increasing order, the first fastest (the row order of
// had_contract(factors[1:end .!= n], rank) reshaped to a matrix).  The product runs left to
// right from 1, as pivot_hadamard's does (src/algebra/had_contract.jl:277-295).
__global__ void k_krp_cols(FactorSet fs, int order, int mode, KrpDims kd, const int64_t* __restrict__ cols,
                           int64_t ncols, int R, double* __restrict__ out) {
  const int64_t total = ncols * (int64_t)R;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / R;
    const int r = (int)(e - c * R);
    int64_t col = cols ? cols[c] : c;
    double p = 1.0;
    for (int m = 0; m < order; ++m) {
      if (m == mode) continue;
      const int64_t d = kd.dims[m];
      const int64_t idx = col % d;
      col /= d;
      p *= fs.F[m][idx * R + r];
    }
    out[e] = p;
  }
}

// omega_hadamard (src/algebra/had_contract.jl:300-326): row j of Omega (KRP), l x R, is
// sum over the entries p of Omega's row j (seg[j] .. seg[j+1], ascending column) of
// v[p] times KRP row cols[p].  Written to out[r * sr + j * sj].
__global__ void k_omega_hadamard(FactorSet fs, int order, int mode, KrpDims kd, const int64_t* __restrict__ seg,
                                 const int64_t* __restrict__ cols, const double* __restrict__ v, int64_t l, int R,
                                 double* __restrict__ out, int64_t sr, int64_t sj) {
  for (int64_t j = blockIdx.x; j < l; j += gridDim.x) {
    const int64_t b = seg[j], e = seg[j + 1];
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
      double acc = 0.0;
      for (int64_t p = b; p < e; ++p) {
        int64_t col = cols[p];
        double prod = 1.0;
        for (int m = 0; m < order; ++m) {
          if (m == mode) continue;
          const int64_t d = kd.dims[m];
          const int64_t idx = col % d;
          col /= d;
          prod *= fs.F[m][idx * R + r];
        }
        acc = fma(v[p], prod, acc);
      }
      out[r * sr + j * sj] = acc;
    }
  }
}

int qrcp_grid(int64_t n, int num_sms) {
  const int64_t want = (n + QW - 1) / QW;
  const int64_t cap = (int64_t)QW * num_sms;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace

int qrcp_parts(int64_t n, int num_sms) { return qrcp_grid(n, num_sms); }

cudaError_t launch_qrcp_init(const QrcpJob& q, cudaStream_t st) {
  const int g = qrcp_grid(q.n, q.num_sms);
  k_iota<<<(int)std::min<int64_t>((q.n + 255) / 256, 4096), 256, 0, st>>>(q.perm, q.n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_qrcp_norms<<<g, QW * 32, 0, st>>>(q.A, q.m, q.n, q.ncand, q.vn1, q.vn2, q.part);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaMemsetAsync(q.st, 0, sizeof(QrcpState), st);
}

cudaError_t launch_qrcp_step(const QrcpJob& q, int64_t j, cudaStream_t st) {
  const int g = qrcp_grid(q.n, q.num_sms);
  k_qrcp_reflect<<<1, 1024, 0, st>>>(q.A, q.m, q.n, q.ncand, j, q.vn1, q.vn2, q.perm, q.part, g, q.vbuf, q.taus,
                                     q.rdiag, q.st, q.kmax, q.stop_ratio);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (j + 1 >= q.n) return cudaSuccess;  // no trailing columns
  const int64_t len = q.m - j;
  if (len <= 8 * 4)
    k_qrcp_apply<8, 4><<<g, QW * 32, 0, st>>>(q.A, q.m, q.n, q.ncand, j, q.vn1, q.vn2, q.vbuf, q.st, q.part);
  else if (len <= 8 * 16)
    k_qrcp_apply<8, 16><<<g, QW * 32, 0, st>>>(q.A, q.m, q.n, q.ncand, j, q.vn1, q.vn2, q.vbuf, q.st, q.part);
  else if (len <= 16 * 16)
    k_qrcp_apply<16, 16><<<g, QW * 32, 0, st>>>(q.A, q.m, q.n, q.ncand, j, q.vn1, q.vn2, q.vbuf, q.st, q.part);
  else if (len <= 16 * 32)
    k_qrcp_apply<16, 32><<<g, QW * 32, 0, st>>>(q.A, q.m, q.n, q.ncand, j, q.vn1, q.vn2, q.vbuf, q.st, q.part);
  else if (len <= 32 * 32)
    k_qrcp_apply<32, 32><<<g, QW * 32, 0, st>>>(q.A, q.m, q.n, q.ncand, j, q.vn1, q.vn2, q.vbuf, q.st, q.part);
  else
    k_qrcp_apply<32, 0><<<g, QW * 32, 0, st>>>(q.A, q.m, q.n, q.ncand, j, q.vn1, q.vn2, q.vbuf, q.st, q.part);
  return cudaGetLastError();
}

cudaError_t launch_qr_form_q(const double* A, int64_t m, int64_t k, const double* taus, double* Q, int num_sms,
                             cudaStream_t st) {
  k_eye<<<(int)std::min<int64_t>((m * k + 255) / 256, 4096), 256, 0, st>>>(Q, m, k);
  cudaError_t e = cudaGetLastError();
  for (int64_t j = k - 1; j >= 0 && e == cudaSuccess; --j) {
    k_qr_apply_q<<<qrcp_grid(k - j, num_sms), QW * 32, 0, st>>>(Q, m, k, j, A, taus);
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t launch_unfold_cols(const void* T, int tdtype, int64_t In, int64_t stride, const int64_t* cols,
                               int64_t ncols, double* out, cudaStream_t st) {
  const dim3 block(32, 8);
  const dim3 grid((unsigned)std::min<int64_t>((ncols + 31) / 32, 1 << 20),
                  (unsigned)std::min<int64_t>((In + 31) / 32, 65535));
  if (tdtype == CPALS_DTYPE_F64)
    k_unfold_cols<double><<<grid, block, 0, st>>>(static_cast<const double*>(T), In, stride, cols, ncols, out);
  else
    k_unfold_cols<float><<<grid, block, 0, st>>>(static_cast<const float*>(T), In, stride, cols, ncols, out);
  return cudaGetLastError();
}

cudaError_t launch_krp_cols(const FactorSet& fs, int order, int mode, const int64_t* dims, const int64_t* cols,
                            int64_t ncols, int R, double* out, cudaStream_t st) {
  KrpDims kd{};
  for (int m = 0; m < order; ++m) kd.dims[m] = dims[m];
  const int64_t total = ncols * (int64_t)R;
  k_krp_cols<<<(int)std::min<int64_t>((total + 255) / 256, 16384), 256, 0, st>>>(fs, order, mode, kd, cols, ncols, R,
                                                                               out);
  return cudaGetLastError();
}

cudaError_t launch_omega_hadamard(const FactorSet& fs, int order, int mode, const int64_t* dims, const int64_t* seg,
                                  const int64_t* cols, const double* v, int64_t l, int R, double* out, int64_t sr,
                                  int64_t sj, cudaStream_t st) {
  KrpDims kd{};
  for (int m = 0; m < order; ++m) kd.dims[m] = dims[m];
  const int threads = R <= 32 ? 32 : (R <= 64 ? 64 : 128);
  k_omega_hadamard<<<(int)std::min<int64_t>(l, 65535), threads, 0, st>>>(fs, order, mode, kd, seg, cols, v, l, R,
                                                                          out, sr, sj);
  return cudaGetLastError();
}

}  // namespace cpals
