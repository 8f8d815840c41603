// Dimension-tree MTTKRP for order-4 tensors.
//
// The four MTTKRPs of a sweep share two partial contractions.  With T viewed as the
// order-3 tensors A = (I0*I1, I2, I3) and B = (I0, I1, I2*I3) (column-major, so the merged
// modes keep their element order):
//   P_L[i0 + I0 i1, r] = sum_{i2,i3} T[i0,i1,i2,i3] F2[i2,r] F3[i3,r]   (MTTKRP of A, mode 0)
//   P_R[i2 + I2 i3, r] = sum_{i0,i1} T[i0,i1,i2,i3] F0[i0,r] F1[i1,r]   (MTTKRP of B, mode 2)
//   M0 = sum_{i1} P_L F1,  M1 = sum_{i0} P_L F0,  M2 = sum_{i3} P_R F3,  M3 = sum_{i2} P_R F2.
// In ALS order P_L depends only on F2, F3 (fixed while modes 0 and 1 update) and P_R on the
// updated F0, F1 (fixed while modes 2 and 3 update), so a sweep streams T twice instead of
// four times.  The full contractions run on the same kernels as the plain path (tcgen05
// split-BF16 for FP32 tensors, the FP64 SIMT kernel otherwise).  On the FP64 path the
// split-K partials are reduced into P (FP64) and the small contractions run in FP64.  On the
// tensor-core path the FP32 partials are summed with compensation into P as an unevaluated
// FP32 pair hi + lo (no FP64 operation), and the small contractions are compensated FP32
// dot products of P with the factor's FP32 hi / lo rows: FP64-grade sums at FP32 rates.
#include <algorithm>
#include <cstring>

#include "cpals_dimtree.cuh"
#include "cpals_tc.cuh"

namespace cpals {

namespace {

__device__ __forceinline__ bool dt_done(const DevCheck* chk) { return chk != nullptr && chk->done; }

// P = sum of the FP64 split-K partials (FP64 path).
__global__ void k_dt_reduce(const double* __restrict__ part, int S, int64_t n, double* __restrict__ P,
                            const DevCheck* chk) {
  if (dt_done(chk)) return;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int sp = 0; sp < S; ++sp) s += part[(int64_t)sp * n + e];
    P[e] = s;
  }
}

// P2 = the compensated FP32 sum of the FP32 split-K partials, kept as {hi, lo} (Fast2Sum
// of the Neumaier sum and its compensation).
__global__ void k_dt_reduce_df(const float* __restrict__ part, int S, int64_t n, float2* __restrict__ P2,
                               const DevCheck* chk) {
  if (dt_done(chk)) return;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f, c = 0.0f;
    for (int sp = 0; sp < S; ++sp) {
      const float p = part[(int64_t)sp * n + e];
      const float t = s + p;
      c += (fabsf(s) >= fabsf(p)) ? ((s - t) + p) : ((p - t) + s);
      s = t;
    }
    const float hi = s + c;
    P2[e] = make_float2(hi, c - (hi - s));
  }
}

// The small contraction on the tensor-core path: out[i][r] = sum_j P[row(i, j)][r] F[j][r]
// with P = {hi, lo} and F = Fh + Fl (FP32 rows, stride rpad), as a compensated FP32 dot
// product (Dot2, Ogita, Rump and Oishi 2005: each hi x hi product split exactly by one FMA,
// summed by TwoSum; the cross terms added in FP32).  Block: two output rows x 32 ranks; warp
// w takes row 2 blockIdx.x + (w & 1) and the quarter w >> 1 of the summed index; the four
// quarters are combined in order.
__device__ __forceinline__ void dot2_term(float xh, float xl, float yh, float yl, float& s, float& c) {
  const float p = xh * yh;
  const float pe = fmaf(xh, yh, -p);
  const float t = s + p;
  const float z = t - s;
  const float e = (s - (t - z)) + (p - z);
  s = t;
  c = fmaf(xh, yl, fmaf(xl, yh, c + (pe + e)));
}
__global__ void __launch_bounds__(256) k_dt_contract_df(const float2* __restrict__ P, int64_t Ia, int64_t Ib, int R,
                                                        const float* __restrict__ Fh, const float* __restrict__ Fl,
                                                        int64_t rpad, int which, double* __restrict__ out,
                                                        const DevCheck* chk) {
  if (dt_done(chk)) return;
  __shared__ float2 red[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t nI = which ? Ib : Ia, nsum = which ? Ia : Ib;
  const int64_t i = 2 * (int64_t)blockIdx.x + (w & 1);
  const int r = blockIdx.y * 32 + lane;
  const int64_t nq = (nsum + 3) / 4;
  const int64_t j0 = (w >> 1) * nq, j1 = min(nsum, j0 + nq);
  float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
  if (i < nI && r < R) {
    int64_t j = j0;
    for (; j + 2 <= j1; j += 2) {
      const int64_t ra = which ? j + Ia * i : i + Ia * j;
      const int64_t rb = which ? (j + 1) + Ia * i : i + Ia * (j + 1);
      const float2 xa = P[ra * R + r], xb = P[rb * R + r];
      dot2_term(xa.x, xa.y, Fh[j * rpad + r], Fl[j * rpad + r], s0, c0);
      dot2_term(xb.x, xb.y, Fh[(j + 1) * rpad + r], Fl[(j + 1) * rpad + r], s1, c1);
    }
    if (j < j1) {
      const int64_t ra = which ? j + Ia * i : i + Ia * j;
      const float2 xa = P[ra * R + r];
      dot2_term(xa.x, xa.y, Fh[j * rpad + r], Fl[j * rpad + r], s0, c0);
    }
  }
  // (s0, c0) + (s1, c1) with one TwoSum
  {
    const float t = s0 + s1, z = t - s0;
    const float e = (s0 - (t - z)) + (s1 - z);
    red[w][lane] = make_float2(t, (c0 + c1) + e);
  }
  __syncthreads();
  if (w >= 2 || i >= nI || r >= R) return;
  float s = red[w][lane].x, c = red[w][lane].y;
#pragma unroll
  for (int q = 1; q < 4; ++q) {
    const float2 v = red[w + 2 * q][lane];
    const float t = s + v.x, z = t - s;
    const float e = (s - (t - z)) + (v.x - z);
    s = t;
    c += v.y + e;
  }
  out[i * R + r] = (double)s + (double)c;
}

// out[i][r] = sum_j P[(which ? j + Ia i : i + Ia j)][r] F[j][r]: contract P (rows a + Ia b)
// over b (which = 0, out rows a, F has Ib rows) or over a (which = 1, out rows b, F has Ia
// rows).  One thread per output, eight accumulators (FP64 dependent adds are slow here).
__global__ void __launch_bounds__(256) k_dt_contract(const double* __restrict__ P, int64_t Ia, int64_t Ib, int R,
                                                     const double* __restrict__ F, int which,
                                                     double* __restrict__ out, const DevCheck* chk) {
  if (dt_done(chk)) return;
  const int64_t nout = (which ? Ib : Ia) * R;
  const int64_t nsum = which ? Ia : Ib;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nout; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / R;
    const int r = (int)(e % R);
    double acc[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) acc[t] = 0.0;
    int64_t j = 0;
    for (; j + 8 <= nsum; j += 8) {
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int64_t row = which ? (j + t) + Ia * i : i + Ia * (j + t);
        acc[t] = fma(P[row * R + r], F[(j + t) * R + r], acc[t]);
      }
    }
    for (int t = 0; j < nsum; ++j, ++t) {
      const int64_t row = which ? j + Ia * i : i + Ia * j;
      acc[t] = fma(P[row * R + r], F[j * R + r], acc[t]);
    }
    out[e] = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
  }
}

int grid_for(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 8192); }

}  // namespace

struct DimTree {
  int64_t dims[4] = {};
  int64_t R = 0;
  int mmode = 0, tdtype = 0, num_sms = 0;
  int64_t rowsA = 0, rowsB = 0;  // I0*I1 and I2*I3
  // tensor-core path
  TcState* tcA = nullptr;  // view (I0*I1, I2, I3), mode 0
  TcState* tcB = nullptr;  // view (I0, I1, I2*I3), mode 2
  // FP64 path
  ModeGeom gA{}, gB{};
  int splitsA = 0, splitsB = 0;
  int64_t cpsA = 0, cpsB = 0;
  const void* dT = nullptr;  // the device tensor (FP64 path)
  void* part = nullptr;  // split-K partials of the full contractions
  double* PL = nullptr;  // [I0*I1][R] (FP64, or {hi, lo} FP32 pairs on the tensor-core path)
  double* PR = nullptr;  // [I2*I3][R]
  const float* Fh[4] = {};  // tensor-core path: the factors' FP32 rows (hi) and remainders (lo)
  const float* Fl[4] = {};
  int64_t rpad = 0;
};

int dt_create(DimTree** out, const int64_t* dims, int64_t R, int mmode, int tdtype, int num_sms) {
  *out = nullptr;
  DimTree* d = new DimTree();
  for (int m = 0; m < 4; ++m) d->dims[m] = dims[m];
  d->R = R;
  d->mmode = mmode;
  d->tdtype = tdtype;
  d->num_sms = num_sms;
  d->rowsA = dims[0] * dims[1];
  d->rowsB = dims[2] * dims[3];
  const int64_t vA[3] = {d->rowsA, dims[2], dims[3]};
  const int64_t vB[3] = {dims[0], dims[1], d->rowsB};
  size_t part_bytes = 0;
  if (mmode == CPALS_MTTKRP_BF16X3) {
    int rc = tc_create(&d->tcA, 3, vA, R, tdtype, num_sms, 1u << 0);
    if (rc == CPALS_OK) rc = tc_create(&d->tcB, 3, vB, R, tdtype, num_sms, 1u << 2);
    if (rc != CPALS_OK) {
      dt_destroy(d);
      return rc;
    }
    part_bytes = std::max((size_t)tc_splits(d->tcA, 0) * d->rowsA, (size_t)tc_splits(d->tcB, 2) * d->rowsB) * R * 4;
  } else {
    d->gA = make_geom(3, vA, 0, 32);
    d->gB = make_geom(3, vB, 2, 32);
    d->splitsA = mttkrp_f64_splits(d->gA, R, num_sms, &d->cpsA);
    d->splitsB = mttkrp_f64_splits(d->gB, R, num_sms, &d->cpsB);
    part_bytes = std::max((size_t)d->splitsA * d->rowsA, (size_t)d->splitsB * d->rowsB) * R * 8;
  }
  if (cudaMalloc(&d->part, part_bytes) != cudaSuccess || cudaMalloc(&d->PL, sizeof(double) * d->rowsA * R) != cudaSuccess ||
      cudaMalloc(&d->PR, sizeof(double) * d->rowsB * R) != cudaSuccess) {
    dt_destroy(d);
    return CPALS_E_CUDA;
  }
  *out = d;
  return CPALS_OK;
}

void dt_destroy(DimTree* d) {
  if (!d) return;
  if (d->tcA) tc_destroy(d->tcA);
  if (d->tcB) tc_destroy(d->tcB);
  cudaFree(d->part);
  cudaFree(d->PL);
  cudaFree(d->PR);
  delete d;
}

int dt_set_tensor(DimTree* d, const void* T, cudaStream_t st) {
  d->dT = T;
  if (d->tcA) {
    int rc = tc_set_tensor(d->tcA, T, st);
    if (rc == CPALS_OK) rc = tc_set_tensor(d->tcB, T, st);
    return rc;
  }
  return CPALS_OK;
}

int* dt_error_flag(DimTree* d, int which) {
  TcState* tc = which ? d->tcB : d->tcA;
  return tc ? tc_error_flag(tc) : nullptr;
}

int64_t dt_factor_rpad(const DimTree* d) { return d->tcA ? tc_factor_rpad(d->tcA) : 0; }

int dt_bind_factors(DimTree* d, const float* const* F32r, const float* const* F32lo) {
  if (!d->tcA) return CPALS_OK;
  for (int m = 0; m < 4; ++m) {
    d->Fh[m] = F32r[m];
    d->Fl[m] = F32lo[m];
  }
  d->rpad = tc_factor_rpad(d->tcA);
  // view A, mode 0: fastest reduction mode = view mode 1 (F2), outer = view mode 2 (F3)
  const float* fa[kMaxOrder] = {nullptr, F32r[2], F32r[3]};
  // view B, mode 2: fastest reduction mode = view mode 0 (F0), outer = view mode 1 (F1)
  const float* fb[kMaxOrder] = {F32r[0], F32r[1], nullptr};
  int rc = tc_bind_factors(d->tcA, fa);
  if (rc == CPALS_OK) rc = tc_bind_factors(d->tcB, fb);
  return rc;
}

cudaError_t dt_update_factor(DimTree* d, int m, const double* F, const DevCheck* chk, cudaStream_t st) {
  if (!d->tcA) return cudaSuccess;
  if (m == 2) return tc_update_factor(d->tcA, 1, F, chk, st);
  if (m == 0) return tc_update_factor(d->tcB, 0, F, chk, st);
  return cudaSuccess;
}

BtileDesc dt_btile_desc(const DimTree* d, int m) {
  if (!d->tcA) return BtileDesc{nullptr, 0, 0};
  if (m == 2) return tc_btile_desc(d->tcA, 1);
  if (m == 0) return tc_btile_desc(d->tcB, 0);
  return BtileDesc{nullptr, 0, 0};
}

int dt_launches(const DimTree* d, int n, bool reuse) {
  (void)d;
  const bool full = (n == 0 || n == 2) || !reuse;
  return (full ? 2 : 0) + 1;  // [MTTKRP, partial reduce,] contraction
}

cudaError_t dt_mttkrp(DimTree* d, int n, const double* const* F, bool reuse, double* M, const DevCheck* chk,
                      cudaStream_t st) {
  const int R = (int)d->R;
  const bool left = (n <= 1);
  const bool full = (n == 0 || n == 2) || !reuse;
  double* P = left ? d->PL : d->PR;
  const int64_t rows = left ? d->rowsA : d->rowsB;
  if (full) {
    int S = 0;
    if (d->tcA) {
      TcState* tc = left ? d->tcA : d->tcB;
      const int vm = left ? 0 : 2;
      cudaError_t e = tc_launch_mttkrp(tc, vm, static_cast<float*>(d->part), chk, st);
      if (e != cudaSuccess) return e;
      S = tc_splits(tc, vm);
      k_dt_reduce_df<<<grid_for(rows * R), 256, 0, st>>>(static_cast<const float*>(d->part), S, rows * R,
                                                          reinterpret_cast<float2*>(P), chk);
    } else {
      FactorSet fs{};
      if (left) {
        fs.F[1] = F[2];
        fs.F[2] = F[3];
      } else {
        fs.F[0] = F[0];
        fs.F[1] = F[1];
      }
      const ModeGeom& g = left ? d->gA : d->gB;
      S = left ? d->splitsA : d->splitsB;
      cudaError_t e = launch_mttkrp_f64(d->dT, d->tdtype, fs, g, R, S, left ? d->cpsA : d->cpsB,
                                        static_cast<double*>(d->part), chk, st);
      if (e != cudaSuccess) return e;
      k_dt_reduce<<<grid_for(rows * R), 256, 0, st>>>(static_cast<const double*>(d->part), S, rows * R, P, chk);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  // the small contraction
  const int64_t Ia = left ? d->dims[0] : d->dims[2];
  const int64_t Ib = left ? d->dims[1] : d->dims[3];
  const int which = (n == 1 || n == 3) ? 1 : 0;  // modes 1, 3 contract over the first index
  const int fc = (n == 0) ? 1 : (n == 1) ? 0 : (n == 2) ? 3 : 2;
  if (d->tcA) {
    const int64_t nI = which ? Ib : Ia;
    const dim3 grid((unsigned)((nI + 1) / 2), (unsigned)((R + 31) / 32));
    k_dt_contract_df<<<grid, 256, 0, st>>>(reinterpret_cast<const float2*>(P), Ia, Ib, R, d->Fh[fc], d->Fl[fc],
                                          d->rpad, which, M, chk);
  } else {
    const int64_t nout = (which ? Ib : Ia) * R;
    k_dt_contract<<<grid_for(nout), 256, 0, st>>>(P, Ia, Ib, R, F[fc], which, M, chk);
  }
  return cudaGetLastError();
}

}  // namespace cpals
