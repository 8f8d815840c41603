// CPU baseline (TEST AND BENCH INFRASTRUCTURE ONLY): normal-equation CP-ALS of an order-3
// tensor with the MTTKRP in GEMM form, multithreaded with OpenMP.  It restates the reference's
// KRPNormal path (src/algorithms/als_algorithms/standard/tensor.jl:12-20: the explicit
// Khatri-Rao product, then T_(n) * KRP, a BLAS GEMM in the reference) inside its sweep loop
// (src/optimizers/als_optimizers/optimize.jl:15-32), so the GPU engine can be timed beside a
// compiled CPU implementation of the same algorithm on the same host cores.
//
// For an order-3 tensor the GEMM T_(n) * KRP splits over the frontal slices T(:, :, k), each an
// I0 x I1 column-major matrix, so nothing of the size of T is formed:
//   M0 = sum_k [T_k F1] .* F2(k, :)      M1 = sum_k [T_k^T F0] .* F2(k, :)
//   M2(k, :) = colsum([T_k^T F0] .* F1)
// Each slice product is a small GEMM (OpenMP over slices, private accumulators).  The MTTKRP
// arithmetic runs in the tensor's element type TT; the normal equations, lambda, Grams and fit
// in FP64: V = Hadamard product of the other Grams (MttkrpAlgorithm.jl:18-31), X = M V^{-1} by
// a pivoted Cholesky with tolerance 1e-6 and a least-squares fallback (ldiv_solve.jl:13-29),
// lambda = column norms, F = X / lambda (row_norm.jl:4-24), the Gram refresh
// (standard/tensor.jl:46-49), and after the last mode the fit of fit_check.jl:24-32.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

namespace {

// Pivoted Cholesky of the symmetric positive semidefinite R x R matrix A (row-major, full):
// A(p, p) = U^T U with the largest remaining diagonal as pivot (dpstrf's rule); stops at a
// pivot <= tol * (largest initial diagonal).  Returns the rank; piv receives the order.
int pstrf(std::vector<double>& A, int R, std::vector<int>& piv, double tol) {
  piv.resize(R);
  for (int i = 0; i < R; ++i) piv[i] = i;
  double dmax = 0.0;
  for (int i = 0; i < R; ++i) dmax = std::max(dmax, A[i * R + i]);
  const double stop = tol * dmax;
  for (int j = 0; j < R; ++j) {
    int p = j;
    for (int i = j + 1; i < R; ++i)
      if (A[i * R + i] > A[p * R + p]) p = i;
    if (!(A[p * R + p] > stop)) return j;
    if (p != j) {  // symmetric swap of rows and columns j, p
      for (int c = 0; c < R; ++c) std::swap(A[j * R + c], A[p * R + c]);
      for (int r = 0; r < R; ++r) std::swap(A[r * R + j], A[r * R + p]);
      std::swap(piv[j], piv[p]);
    }
    const double d = std::sqrt(A[j * R + j]);
    A[j * R + j] = d;
    for (int c = j + 1; c < R; ++c) A[j * R + c] /= d;
    // the whole trailing Schur complement (both triangles: later swaps read both)
    for (int r = j + 1; r < R; ++r)
      for (int c = j + 1; c < R; ++c) A[r * R + c] -= A[j * R + r] * A[j * R + c];
  }
  return R;
}

// X (In x R, row-major) = M V^{-1} for symmetric V: pivoted Cholesky, and when V is rank
// deficient the minimum-norm least-squares solution from V's eigendecomposition (Jacobi),
// the role the pivoted QR plays in ldiv_solve.jl:20-21.
void solve_normal(const std::vector<double>& V, int R, const std::vector<double>& M, int64_t In,
                  std::vector<double>& X) {
  std::vector<double> A = V;
  std::vector<int> piv;
  const int rank = pstrf(A, R, piv, 1e-6);
  X.assign((size_t)In * R, 0.0);
  if (rank == R) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < In; ++i) {
      std::vector<double> y(R);
      for (int c = 0; c < R; ++c) y[c] = M[(size_t)i * R + piv[c]];
      for (int c = 0; c < R; ++c) {  // U^T y' = y
        double s = y[c];
        for (int l = 0; l < c; ++l) s -= A[l * R + c] * y[l];
        y[c] = s / A[c * R + c];
      }
      for (int c = R - 1; c >= 0; --c) {  // U x = y'
        double s = y[c];
        for (int l = c + 1; l < R; ++l) s -= A[c * R + l] * y[l];
        y[c] = s / A[c * R + c];
      }
      for (int c = 0; c < R; ++c) X[(size_t)i * R + piv[c]] = y[c];
    }
    return;
  }
  // symmetric Jacobi eigendecomposition V = Q diag(w) Q^T, pseudo-inverse on w > tol * max w
  std::vector<double> a = V, q((size_t)R * R, 0.0);
  for (int i = 0; i < R; ++i) q[i * R + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int i = 0; i < R; ++i)
      for (int j = i + 1; j < R; ++j) off += a[i * R + j] * a[i * R + j];
    if (off < 1e-30) break;
    for (int p = 0; p < R; ++p)
      for (int r = p + 1; r < R; ++r) {
        const double apr = a[p * R + r];
        if (std::fabs(apr) < 1e-300) continue;
        const double th = (a[r * R + r] - a[p * R + p]) / (2.0 * apr);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < R; ++k) {
          const double akp = a[k * R + p], akr = a[k * R + r];
          a[k * R + p] = c * akp - s * akr;
          a[k * R + r] = s * akp + c * akr;
        }
        for (int k = 0; k < R; ++k) {
          const double apk = a[p * R + k], ark = a[r * R + k];
          a[p * R + k] = c * apk - s * ark;
          a[r * R + k] = s * apk + c * ark;
        }
        for (int k = 0; k < R; ++k) {
          const double qkp = q[k * R + p], qkr = q[k * R + r];
          q[k * R + p] = c * qkp - s * qkr;
          q[k * R + r] = s * qkp + c * qkr;
        }
      }
  }
  double wmax = 0.0;
  for (int i = 0; i < R; ++i) wmax = std::max(wmax, std::fabs(a[i * R + i]));
  std::vector<double> pinv((size_t)R * R, 0.0);
  for (int e = 0; e < R; ++e) {
    const double w = a[e * R + e];
    if (std::fabs(w) <= 1e-12 * wmax) continue;
    for (int i = 0; i < R; ++i)
      for (int j = 0; j < R; ++j) pinv[i * R + j] += q[i * R + e] * q[j * R + e] / w;
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < In; ++i)
    for (int c = 0; c < R; ++c) {
      double s = 0.0;
      for (int l = 0; l < R; ++l) s += M[(size_t)i * R + l] * pinv[l * R + c];
      X[(size_t)i * R + c] = s;
    }
}

// C (m x n, column-major, ldc) = A (m x k, column-major, lda) B, with B(p, j) = B[p bp + j bj]:
// 16 x 4 tiles of C held in registers over the whole k loop (the inner loops vectorise over
// the 16 rows on either instruction set).
template <typename TT>
void gemm(int64_t m, int64_t n, int64_t k, const TT* A, int64_t lda, const TT* B, int64_t bp, int64_t bj, TT* C,
          int64_t ldc) {
  constexpr int MB = 16, NB = 4;
  for (int64_t j0 = 0; j0 < n; j0 += NB) {
    const int nj = (int)std::min<int64_t>(NB, n - j0);
    for (int64_t i0 = 0; i0 < m; i0 += MB) {
      const int mi = (int)std::min<int64_t>(MB, m - i0);
      TT acc[NB][MB] = {};
      if (mi == MB && nj == NB) {
        for (int64_t p = 0; p < k; ++p) {
          const TT* a = A + i0 + lda * p;
          const TT b0 = B[p * bp + (j0 + 0) * bj], b1 = B[p * bp + (j0 + 1) * bj];
          const TT b2 = B[p * bp + (j0 + 2) * bj], b3 = B[p * bp + (j0 + 3) * bj];
          for (int ii = 0; ii < MB; ++ii) {
            const TT av = a[ii];
            acc[0][ii] += av * b0;
            acc[1][ii] += av * b1;
            acc[2][ii] += av * b2;
            acc[3][ii] += av * b3;
          }
        }
      } else {
        for (int64_t p = 0; p < k; ++p)
          for (int jj = 0; jj < nj; ++jj) {
            const TT b = B[p * bp + (j0 + jj) * bj];
            for (int ii = 0; ii < mi; ++ii) acc[jj][ii] += A[i0 + ii + lda * p] * b;
          }
      }
      for (int jj = 0; jj < nj; ++jj)
        for (int ii = 0; ii < mi; ++ii) C[i0 + ii + ldc * (j0 + jj)] = acc[jj][ii];
    }
  }
}

template <typename TT>
void mttkrp3(const TT* T, const int64_t* d, int R, int mode, const std::vector<std::vector<TT>>& F,
             std::vector<double>& M) {
  const int64_t I0 = d[0], I1 = d[1], I2 = d[2];
  const int64_t In = d[mode];
  M.assign((size_t)In * R, 0.0);
  const int nth = omp_get_max_threads();
  std::vector<std::vector<TT>> part(nth);
#pragma omp parallel
  {
    const int tid = omp_get_thread_num();
    std::vector<TT>& acc = part[tid];
    acc.assign((size_t)In * R, TT(0));
    std::vector<TT> y((size_t)std::max(I0, I1) * R);
#pragma omp for schedule(static)
    for (int64_t k = 0; k < I2; ++k) {
      const TT* S = T + k * I0 * I1;  // T(:, :, k), I0 x I1 column-major
      if (mode == 0) {
        // y (I0 x R, column-major) = S F1, then acc += y .* F2(k, :)
        gemm<TT>(I0, R, I1, S, I0, F[1].data(), R, 1, y.data(), I0);
        const TT* f2 = F[2].data() + (size_t)k * R;
        for (int64_t i = 0; i < I0; ++i)
          for (int r = 0; r < R; ++r) acc[(size_t)i * R + r] += y[(size_t)r * I0 + i] * f2[r];
      } else {
        // y^T (R x I1, column-major, i.e. y row-major [j][r]) = F0^T S
        gemm<TT>(R, I1, I0, F[0].data(), R, S, 1, I0, y.data(), R);
        if (mode == 1) {
          const TT* f2 = F[2].data() + (size_t)k * R;
          for (int64_t j = 0; j < I1; ++j)
            for (int r = 0; r < R; ++r) acc[(size_t)j * R + r] += y[(size_t)j * R + r] * f2[r];
        } else {
          TT* out = acc.data() + (size_t)k * R;  // slice k is this thread's alone
          for (int64_t j = 0; j < I1; ++j)
            for (int r = 0; r < R; ++r) out[r] += y[(size_t)j * R + r] * F[1][(size_t)j * R + r];
        }
      }
    }
  }
  for (int t = 0; t < nth; ++t)
    if (!part[t].empty())
      for (size_t e = 0; e < M.size(); ++e) M[e] += (double)part[t][e];
}

template <typename TT>
int run(const TT* T, const int64_t* dims, int R, double* factors, double* lam, int sweeps, double ref_norm,
        double* fits) {
  const int N = 3;
  // working copies: row-major [I_m][R] in FP64 and in TT; F[3] = F0 column-major in TT
  std::vector<std::vector<double>> F64(N);
  std::vector<std::vector<TT>> Ft(3);
  int64_t off[3] = {0, dims[0] * R, (dims[0] + dims[1]) * R};
  auto refresh_tt = [&](int m) {
    Ft[m].resize((size_t)dims[m] * R);
    for (size_t e = 0; e < Ft[m].size(); ++e) Ft[m][e] = (TT)F64[m][e];
  };
  std::vector<std::vector<double>> G(N, std::vector<double>((size_t)R * R));
  auto gram = [&](int m) {
    const std::vector<double>& f = F64[m];
    for (int a = 0; a < R; ++a)
      for (int b = a; b < R; ++b) {
        double s = 0.0;
        for (int64_t i = 0; i < dims[m]; ++i) s += f[(size_t)i * R + a] * f[(size_t)i * R + b];
        G[m][a * R + b] = G[m][b * R + a] = s;
      }
  };
  for (int m = 0; m < N; ++m) {
    F64[m].resize((size_t)dims[m] * R);
    for (int64_t i = 0; i < dims[m]; ++i)
      for (int r = 0; r < R; ++r) F64[m][(size_t)i * R + r] = factors[off[m] + i + dims[m] * r];
    refresh_tt(m);
    gram(m);
  }
  std::vector<double> L(lam, lam + R), M, X, V((size_t)R * R);
  for (int s = 0; s < sweeps; ++s) {
    double inner = 0.0;
    for (int n = 0; n < N; ++n) {
      for (int e = 0; e < R * R; ++e) {
        double v = 1.0;
        for (int m = 0; m < N; ++m)
          if (m != n) v *= G[m][e];
        V[e] = v;
      }
      mttkrp3<TT>(T, dims, R, n, Ft, M);
      solve_normal(V, R, M, dims[n], X);
      if (n == N - 1)
        for (size_t e = 0; e < M.size(); ++e) inner += M[e] * X[e];
      for (int r = 0; r < R; ++r) {
        double q = 0.0;
        for (int64_t i = 0; i < dims[n]; ++i) q += X[(size_t)i * R + r] * X[(size_t)i * R + r];
        L[r] = std::sqrt(q);
      }
      for (int64_t i = 0; i < dims[n]; ++i)
        for (int r = 0; r < R; ++r) F64[n][(size_t)i * R + r] = X[(size_t)i * R + r] / L[r];
      refresh_tt(n);
      gram(n);
    }
    if (fits) {  // fit_check.jl:26-32 with norm_factors (converge_checks.jl:5-11)
      double fsq = 0.0;
      for (int a = 0; a < R; ++a)
        for (int b = 0; b < R; ++b) fsq += L[a] * L[b] * G[0][a * R + b] * G[1][a * R + b] * G[2][a * R + b];
      fits[s] = 1.0 - std::sqrt(std::fabs(ref_norm * ref_norm + fsq - 2.0 * std::fabs(inner))) / ref_norm;
    }
  }
  for (int m = 0; m < N; ++m)
    for (int64_t i = 0; i < dims[m]; ++i)
      for (int r = 0; r < R; ++r) factors[off[m] + i + dims[m] * r] = F64[m][(size_t)i * R + r];
  for (int r = 0; r < R; ++r) lam[r] = L[r];
  return 0;
}

}  // namespace

extern "C" {

// `sweeps` ALS sweeps of the order-3 column-major tensor T (dtype 0: FP64, 1: FP32) from the
// factors (F0, F1, F2 concatenated, each I_m x R column-major, FP64; updated in place) and
// lambda (R).  fits (may be NULL) receives one fit per sweep against ref_norm.  threads <= 0
// keeps OpenMP's default.  Returns 0, or -1 for a bad argument.
int cpu_als_sweeps(int dtype, const void* T, const int64_t* dims, int R, double* factors, double* lam, int sweeps,
                   double ref_norm, double* fits, int threads) {
  if (!T || !dims || !factors || !lam || R < 1 || sweeps < 0) return -1;
  for (int m = 0; m < 3; ++m)
    if (dims[m] < 1) return -1;
  if (threads > 0) omp_set_num_threads(threads);
  if (dtype == 0) return run<double>(static_cast<const double*>(T), dims, R, factors, lam, sweeps, ref_norm, fits);
  if (dtype == 1) return run<float>(static_cast<const float*>(T), dims, R, factors, lam, sweeps, ref_norm, fits);
  return -1;
}

int cpu_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
