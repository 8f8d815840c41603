// Gathers of the randomized leverage-score path (LevScoreSampled).
//   pivot_hadamard       : S(s, r) = prod over the other modes, in mode order, of
//                          F_m(p_m(s), r), multiplied left to right from 1
//                          (src/algebra/had_contract.jl:277-295).  Only products, no
//                          sums, so the result is bit-identical to the host loop.
//   fused_flatten_sample : T_s(i, s) = T(p_1(s), .., i, .., p_{N-1}(s)), a copy
//                          (src/algebra/pivot_mapping.jl:59-85).
//   leverage rows        : p_i = ||(F P)_i U^{-1}||^2 / min(I, R) with P^T F^T F P = U^T U,
//                          the row norms of the thin-QR Q of F
//                          (src/math_tools/probability.jl:3-10).
// Pivots are 1-based Int64, nsamps x (N-1), column-major.  Every index is checked
// on the host before launch; the kernels also guard and flag, never read out of range.
#include "cpals_internal.cuh"

namespace cpals {
namespace {

struct Dims {
  int64_t d[kMaxOrder];
  int64_t s[kMaxOrder];
};

__global__ void k_pivot_hadamard(FactorSet fs, int order, int mode, Dims dm, const int64_t* __restrict__ piv,
                                 int64_t nsamps, int R, double* __restrict__ out, int* __restrict__ err) {
  const int64_t n = nsamps * R;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = e % nsamps;
    const int r = (int)(e / nsamps);
    double prod = 1.0;
    int j = 0;
    for (int m = 0; m < order; ++m) {
      if (m == mode) continue;
      const int64_t idx = piv[s + nsamps * j] - 1;
      ++j;
      if (idx < 0 || idx >= dm.d[m]) {
        atomicExch(err, 1);
        prod = NAN;
        break;
      }
      prod = __dmul_rn(prod, fs.F[m][idx * R + r]);
    }
    out[e] = prod;  // column-major nsamps x R
  }
}

template <typename TT>
__global__ void k_fibers(const TT* __restrict__ T, int order, int mode, Dims dm, const int64_t* __restrict__ piv,
                         int64_t nsamps, TT* __restrict__ out, int* __restrict__ err) {
  const int64_t In = dm.d[mode];
  const int64_t n = In * nsamps;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % In, s = e / In;
    int64_t base = 0;
    int j = 0;
    bool ok = true;
    for (int m = 0; m < order; ++m) {
      if (m == mode) continue;
      const int64_t idx = piv[s + nsamps * j] - 1;
      ++j;
      if (idx < 0 || idx >= dm.d[m]) ok = false;
      base += idx * dm.s[m];
    }
    if (!ok) {
      atomicExch(err, 1);
      out[e] = TT(0);
      continue;
    }
    out[e] = T[base + i * dm.s[mode]];
  }
}

// row-major copy of a column-major nsamps x R matrix (for the Gram / MTTKRP of the sampled solve)
__global__ void k_colmajor_to_rowmajor(const double* __restrict__ src, int64_t rows, int R, double* __restrict__ dst) {
  const int64_t n = rows * R;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / R;
    const int r = (int)(e % R);
    dst[e] = src[i + rows * r];
  }
}

// leverage scores: warp per row, forward substitution with the pivoted Cholesky factor of F^T F
template <int RQ>
__global__ void k_leverage_rows(const double* __restrict__ F, int64_t In, int R, const double* __restrict__ U,
                                const double* __restrict__ dinv, const int* __restrict__ piv,
                                const SolveInfo* __restrict__ info, double scale, double* __restrict__ probs) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int64_t row = (int64_t)blockIdx.x * wpb + warp;
  if (row >= In) return;
  const int rank = info->rank;
  double t[RQ];
#pragma unroll
  for (int q = 0; q < RQ; ++q) {
    const int j = lane + 32 * q;
    t[q] = (j < rank) ? F[row * R + piv[j]] : 0.0;
  }
  for (int k = 0; k < rank; ++k) {
    const int qk = k >> 5, owner = k & 31;
    double tk = 0.0;
#pragma unroll
    for (int q = 0; q < RQ; ++q)
      if (q == qk) tk = t[q];
    const double c = __shfl_sync(0xffffffffu, tk * dinv[k], owner);
    const double* Uk = U + (size_t)k * R;
#pragma unroll
    for (int q = 0; q < RQ; ++q) {
      const int j = lane + 32 * q;
      if (j == k) t[q] = c;
      else if (j > k && j < rank) t[q] = fma(-c, Uk[j], t[q]);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < RQ; ++q) s = fma(t[q], t[q], s);
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if (lane == 0) probs[row] = s * scale;
}

Dims make_dims(int order, const int64_t* dims) {
  Dims d{};
  int64_t s = 1;
  for (int m = 0; m < order; ++m) {
    d.d[m] = dims[m];
    d.s[m] = s;
    s *= dims[m];
  }
  return d;
}

}  // namespace

cudaError_t launch_pivot_hadamard(const FactorSet& fs, int order, int mode, const int64_t* dims,
                                  const int64_t* piv, int64_t nsamps, int R, double* out, int* err, cudaStream_t st) {
  const int64_t n = nsamps * R;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 8192);
  k_pivot_hadamard<<<blocks, 256, 0, st>>>(fs, order, mode, make_dims(order, dims), piv, nsamps, R, out, err);
  return cudaGetLastError();
}

cudaError_t launch_fibers(const void* T, int tdtype, int order, int mode, const int64_t* dims, const int64_t* piv,
                          int64_t nsamps, void* out, int* err, cudaStream_t st) {
  const int64_t n = dims[mode] * nsamps;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 8192);
  const Dims dm = make_dims(order, dims);
  if (tdtype == CPALS_DTYPE_F64)
    k_fibers<double><<<blocks, 256, 0, st>>>(static_cast<const double*>(T), order, mode, dm, piv, nsamps,
                                             static_cast<double*>(out), err);
  else
    k_fibers<float><<<blocks, 256, 0, st>>>(static_cast<const float*>(T), order, mode, dm, piv, nsamps,
                                            static_cast<float*>(out), err);
  return cudaGetLastError();
}

cudaError_t launch_colmajor_to_rowmajor(const double* src, int64_t rows, int R, double* dst, cudaStream_t st) {
  const int64_t n = rows * R;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 8192);
  k_colmajor_to_rowmajor<<<blocks, 256, 0, st>>>(src, rows, R, dst);
  return cudaGetLastError();
}

cudaError_t launch_leverage_rows(const double* F, int64_t In, int R, const double* work, const double* U,
                                 const int* piv, const SolveInfo* info, double scale, double* probs, cudaStream_t st) {
  const double* dinv = work + (size_t)R * R;
  const int wpb = 4;
  dim3 grid((unsigned)((In + wpb - 1) / wpb));
  const int rq = (R + 31) / 32;
#define CPALS_LEV_CASE(Q)                                                                          \
  if (rq <= Q) {                                                                                   \
    k_leverage_rows<Q><<<grid, 32 * wpb, 0, st>>>(F, In, R, U, dinv, piv, info, scale, probs); \
    return cudaGetLastError();                                                                     \
  }
  CPALS_LEV_CASE(1)
  CPALS_LEV_CASE(2)
  CPALS_LEV_CASE(4)
  CPALS_LEV_CASE(8)
  CPALS_LEV_CASE(16)
#undef CPALS_LEV_CASE
  return cudaErrorInvalidValue;
}

}  // namespace cpals
