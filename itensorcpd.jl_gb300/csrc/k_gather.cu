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
// ---------------- the sampled system's products in compensated FP32 (Dot2)
// This part issues FP64 some 60 times slower than FP32, so S^T S and T_s S (2 x 16384 x 128^2
// multiply-adds per mode update at 128^4 R = 128, 16384 samples) run as Dot2 products (Ogita,
// Rump & Oishi 2005): each FP64 operand is split once into an FP32 pair hi + lo (exact to
// 2^-48), each term's leading product split exactly by one FMA and added with TwoSum, the
// cross terms in FP32; a sum stays a pair until it is written as one FP64 partial.

// x = hi + lo (FP32 pairs) of an FP64 array
__global__ void k_split_pairs(const double* __restrict__ x, int64_t n, float2* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[e];
    const float h = (float)v;
    out[e] = make_float2(h, (float)(v - (double)h));
  }
}

__device__ __forceinline__ float2 pair_of(float v) { return make_float2(v, 0.f); }
__device__ __forceinline__ float2 pair_of(float2 v) { return v; }

// s + c += a b for pairs a, b (the _rn intrinsics keep the compiler from contracting the
// error-free steps into FMAs)
__device__ __forceinline__ void dot2_acc(float& s, float& c, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  const float e = fmaf(ah, bh, -p);
  const float t = __fadd_rn(s, p);
  const float z = __fsub_rn(t, s);
  const float r = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
  s = t;
  c += (e + r) + fmaf(ah, bl, al * bh);
}

// S (column-major nsamps x R, S(s, r) at s + nsamps r) as FP32 pairs in sample-major order,
// P[s R + r], through 32 x 32 tiles in shared memory (both sides coalesced)
__global__ void k_split_pairs_t(const double* __restrict__ S, int64_t nsamps, int R, float2* __restrict__ P) {
  __shared__ double tile[32][33];
  const int64_t s0 = (int64_t)blockIdx.x * 32;
  const int r0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 256 threads: 8 rows per pass
  for (int q = ty; q < 32; q += 8) {
    const int64_t sv = s0 + tx;
    const int r = r0 + q;
    tile[q][tx] = (sv < nsamps && r < R) ? S[sv + nsamps * r] : 0.0;
  }
  __syncthreads();
  for (int q = ty; q < 32; q += 8) {
    const int64_t sv = s0 + q;
    const int r = r0 + tx;
    if (sv < nsamps && r < R) {
      const double v = tile[tx][q];
      const float h = (float)v;
      P[sv * R + r] = make_float2(h, (float)(v - (double)h));
    }
  }
}

__device__ __forceinline__ float2 ld_pair(const float* p) { return make_float2(*p, 0.f); }
__device__ __forceinline__ float2 ld_pair(const float2* p) { return *p; }

// part[y][m][n] = sum over k in split y of A(k, m) B(k, n), A(k, m) = A[k lak + m] and
// B(k, n) = B[k lbk + n] (FP32 pairs, or FP32 values with a zero lo; m and n contiguous);
// 32 x 32 output tiles (blockIdx.x), splits of kchunk (blockIdx.y); with `upper` only tiles on
// or above the diagonal.  64 threads, each a 4 x 4 block of outputs (16 independent Dot2
// chains, the shared-memory operands read as 16-byte vectors); 32-deep K steps.  Every output
// takes its terms in k order within its split, one sum per split.
template <typename TA>
__global__ void __launch_bounds__(64) k_dot2_atb(const TA* __restrict__ A, int64_t lak, const float2* __restrict__ B,
                                                  int64_t lbk, int64_t K, int M, int N, int64_t kchunk, int upper,
                                                  double* __restrict__ part) {
  __shared__ __align__(16) float Ah[32][36], Al[32][36], Bh[32][36], Bl[32][36];  // [k][m], [k][n]
  const int tiles_n = (N + 31) / 32;
  const int mb = blockIdx.x / tiles_n, nb = blockIdx.x % tiles_n;
  if (upper && mb > nb) return;  // uniform over the block
  const int64_t k0 = (int64_t)blockIdx.y * kchunk;
  const int64_t k1 = (K < k0 + kchunk) ? K : k0 + kchunk;
  const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3;
  float s[4][4], c[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) s[i][j] = c[i][j] = 0.f;
  for (int64_t kk = k0; kk < k1; kk += 32) {
    // 32 x 32 of each operand: consecutive threads on consecutive m (n)
#pragma unroll 4
    for (int e = tid; e < 1024; e += 64) {
      const int ml = e & 31, kl = e >> 5;
      const int64_t k = kk + kl;
      const int m = mb * 32 + ml, n = nb * 32 + ml;
      const float2 a = (k < k1 && m < M) ? ld_pair(A + k * lak + m) : make_float2(0.f, 0.f);
      const float2 b = (k < k1 && n < N) ? B[k * lbk + n] : make_float2(0.f, 0.f);
      Ah[kl][ml] = a.x;
      Al[kl][ml] = a.y;
      Bh[kl][ml] = b.x;
      Bl[kl][ml] = b.y;
    }
    __syncthreads();
    const int kn = (k1 - kk < 32) ? (int)(k1 - kk) : 32;
    for (int kl = 0; kl < kn; ++kl) {
      const float4 ah = *reinterpret_cast<const float4*>(&Ah[kl][4 * ty]);
      const float4 al = *reinterpret_cast<const float4*>(&Al[kl][4 * ty]);
      const float4 bh = *reinterpret_cast<const float4*>(&Bh[kl][4 * tx]);
      const float4 bl = *reinterpret_cast<const float4*>(&Bl[kl][4 * tx]);
      const float avh[4] = {ah.x, ah.y, ah.z, ah.w}, avl[4] = {al.x, al.y, al.z, al.w};
      const float bvh[4] = {bh.x, bh.y, bh.z, bh.w}, bvl[4] = {bl.x, bl.y, bl.z, bl.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) dot2_acc(s[i][j], c[i][j], avh[i], avl[i], bvh[j], bvl[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = mb * 32 + 4 * ty + i, n = nb * 32 + 4 * tx + j;
      if (m < M && n < N) part[((size_t)blockIdx.y * M + m) * N + n] = (double)s[i][j] + (double)c[i][j];
    }
}

// G = the splits' partials summed in split order, the upper triangle mirrored
__global__ void k_reduce_gram_splits(const double* __restrict__ part, int splits, int R, double* __restrict__ G) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < R * R; e += gridDim.x * blockDim.x) {
    const int a = e / R, b = e - a * R;
    const int src = (a <= b) ? a * R + b : b * R + a;
    double v = 0.0;
    for (int y = 0; y < splits; ++y) v += part[(size_t)y * R * R + src];
    G[e] = v;
  }
}

__global__ void k_colmajor_to_rowmajor(const double* __restrict__ src, int64_t rows, int R, double* __restrict__ dst) {
  const int64_t n = rows * R;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / R;
    const int r = (int)(e % R);
    dst[e] = src[i + rows * r];
  }
}

// leverage scores: warp per row, forward substitution with the pivoted Cholesky factor of F^T F.
// With STAGED, U and dinv are first copied into shared memory (R <= 128) and the warps of a
// grid of at most one block per SM stride over the rows: the substitution's R dependent
// steps then wait on shared-memory loads instead of L2 round trips.
template <int RQ, bool STAGED>
__global__ void k_leverage_rows(const double* __restrict__ F, int64_t In, int R, const double* __restrict__ U,
                                const double* __restrict__ dinv, const int* __restrict__ piv,
                                const SolveInfo* __restrict__ info, double scale, double* __restrict__ probs) {
  extern __shared__ double lsm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int rank = info->rank;
  const double* Us = U;
  const double* ds = dinv;
  if (STAGED) {
    for (int e = threadIdx.x; e < rank * R; e += blockDim.x) lsm[e] = U[e];
    for (int e = threadIdx.x; e < rank; e += blockDim.x) lsm[R * R + e] = dinv[e];
    __syncthreads();
    Us = lsm;
    ds = lsm + R * R;
  }
  for (int64_t row = (int64_t)blockIdx.x * wpb + warp; row < In; row += (int64_t)gridDim.x * wpb) {
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
      const double c = __shfl_sync(0xffffffffu, tk * ds[k], owner);
      const double* Uk = Us + (size_t)k * R;
#pragma unroll
      for (int q = 0; q < RQ; ++q) {
        // blocks of 32 below the pivot's hold no j > k: a warp-uniform skip, so that no FP64
        // instruction issues for them (a warp's FP64 instruction holds its scheduler's FP64
        // pipe for ~64 cycles whatever its active lanes)
        if (q < qk) continue;
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

// Splits of the sampled products' K range (the samples): about 128 samples each, at least one,
// so that the 64-thread tiles of k_dot2_atb keep ~16 warps on each SM at R = 128.
int sampled_splits(int64_t nsamps) { return (int)std::max<int64_t>(1, std::min<int64_t>(256, (nsamps + 127) / 128)); }

cudaError_t launch_sampled_gram(const double* Scol, int64_t nsamps, int R, float2* Spair, double* part, double* G,
                                cudaStream_t st) {
  if (nsamps > (int64_t)INT_MAX * 32) return cudaErrorInvalidValue;
  k_split_pairs_t<<<dim3((unsigned)((nsamps + 31) / 32), (unsigned)((R + 31) / 32)), 256, 0, st>>>(Scol, nsamps, R,
                                                                                                  Spair);
  const int sp = sampled_splits(nsamps);
  const int64_t kchunk = (nsamps + sp - 1) / sp;
  const int tiles = ((R + 31) / 32) * ((R + 31) / 32);
  // S^T S: A = B = S, S(s, r) at s R + r (the sample-major pairs)
  k_dot2_atb<float2><<<dim3((unsigned)tiles, (unsigned)sp), 64, 0, st>>>(Spair, R, Spair, R, nsamps, R, R, kchunk, 1,
                                                                         part);
  k_reduce_gram_splits<<<(R * R + 255) / 256, 256, 0, st>>>(part, sp, R, G);
  return cudaGetLastError();
}

cudaError_t launch_sampled_rhs(const void* Ts, int tdtype, int64_t In, int64_t nsamps, int R, const float2* Spair,
                               float2* Tpair, double* part, int* splits_out, cudaStream_t st) {
  const int sp = sampled_splits(nsamps);
  const int64_t kchunk = (nsamps + sp - 1) / sp;
  const int tiles = (int)(((In + 31) / 32) * ((R + 31) / 32));
  if (In > INT_MAX) return cudaErrorInvalidValue;
  // T_s S: A = T_s (i, s) at i + In s, B = S (sample-major pairs)
  if (tdtype == CPALS_DTYPE_F64) {
    const int64_t n = In * nsamps;
    k_split_pairs<<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(static_cast<const double*>(Ts), n,
                                                                                  Tpair);
    k_dot2_atb<float2><<<dim3((unsigned)tiles, (unsigned)sp), 64, 0, st>>>(Tpair, In, Spair, R, nsamps, (int)In, R,
                                                                           kchunk, 0, part);
  } else {
    k_dot2_atb<float><<<dim3((unsigned)tiles, (unsigned)sp), 64, 0, st>>>(static_cast<const float*>(Ts), In, Spair, R,
                                                                          nsamps, (int)In, R, kchunk, 0, part);
  }
  *splits_out = sp;
  return cudaGetLastError();
}

cudaError_t launch_leverage_rows(const double* F, int64_t In, int R, const double* work, const double* U,
                                 const int* piv, const SolveInfo* info, double scale, double* probs, cudaStream_t st) {
  const double* dinv = work + (size_t)R * R;
  const int rq = (R + 31) / 32;
  if (R <= 128) {
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int wpb = 4;  // one row per scheduler: the substitution's FP64 chain owns its pipe
    const size_t smem = sizeof(double) * ((size_t)R * R + R);
    dim3 grid((unsigned)std::min<int64_t>((In + wpb - 1) / wpb, nsm));
#define CPALS_LEV_STAGED(Q)                                                                           \
  if (rq <= Q) {                                                                                      \
    e = set_smem_limit_once((const void*)k_leverage_rows<Q, true>, (int)(sizeof(double) * (128 * 128 + 128))); \
    if (e != cudaSuccess) return e;                                                                   \
    k_leverage_rows<Q, true><<<grid, 32 * wpb, smem, st>>>(F, In, R, U, dinv, piv, info, scale, probs); \
    return cudaGetLastError();                                                                        \
  }
    CPALS_LEV_STAGED(1)
    CPALS_LEV_STAGED(2)
    CPALS_LEV_STAGED(4)
#undef CPALS_LEV_STAGED
  }
  const int wpb = 4;
  dim3 grid((unsigned)((In + wpb - 1) / wpb));
#define CPALS_LEV_CASE(Q)                                                                                \
  if (rq <= Q) {                                                                                         \
    k_leverage_rows<Q, false><<<grid, 32 * wpb, 0, st>>>(F, In, R, U, dinv, piv, info, scale, probs); \
    return cudaGetLastError();                                                                           \
  }
  CPALS_LEV_CASE(8)
  CPALS_LEV_CASE(16)
#undef CPALS_LEV_CASE
  return cudaErrorInvalidValue;
}

}  // namespace cpals
