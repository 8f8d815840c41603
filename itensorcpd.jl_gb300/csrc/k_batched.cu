// Batched CP-ALS: thousands of small independent order-3 decompositions of uneven shape
// and rank in one persistent kernel.
//
// Each CTA pulls tensor indices from a device work queue (largest tensors first) and runs
// ALS sweeps of that tensor in shared memory -- by default until the tensor's own check
// stops it, or one (k) sweep(s) per launch -- with the reference's steps
// (src/optimizers/als_optimizers/optimize.jl:15-32) for every mode n:
//   M_n = T_(n) (F_b (.) F_a)          from the mode's own layout of T (slabs streamed through a
//                                      shared-memory ring): FP32 products, FP32 sums within a
//                                      slab, compensated FP32 pairs across slabs
//   V = G_a .* G_b                     FP64 (MttkrpAlgorithm.jl:18-31), and its pivoted
//                                      symmetric sweep (tol 1e-6) on one warp beside the MTTKRP
//   X = M_n V^{-1}                     compensated FP32 (Dot2) product
//   lambda, F_n = X / lambda, G_n      FP64 (row_norm.jl, standard/tensor.jl:46-49)
// and after the last mode the fit and the tensor's own FitCheck (fit_check.jl:24-66).
// Converged tensors are skipped.  The launch is a CUDA graph (queue reset + kernel).
//
// Shared memory per CTA (Imax = largest mode size, Rmax = largest rank of its tensors):
//   ring    two or more steps of slabs (the MTTKRP's tensor stream)
//   F32     3 Imax Rmax floats        the factors in FP32 (MTTKRP operands)
//   M       Imax Rmax float pairs     MTTKRP result (hi + lo)
//   X       Imax Rmax doubles         solve result (during the MTTKRP: partial pairs)
//   A       Rmax (Rmax|1) doubles     V, swept in place into -V^{-1}
//   G       3 Rmax^2 doubles          Grams
//   vecs    6 Rmax doubles
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "cpals_internal.cuh"

namespace cpals {

namespace {

constexpr double kBatchTol = 1e-6;  // cholesky_epsilon (src/ITensorCPD.jl:2)

struct BatchItem {
  int64_t toff;     // tensor offset (elements) in the natural layout, as uploaded
  int64_t loff[3];  // offsets of the MTTKRP's per-mode layouts (floats, 16-byte aligned)
  int64_t foff;  // factor offset (doubles): F0, F1, F2 (I_m x R column-major), lambda [R]
  int64_t goff;  // Gram offset (doubles): G0, G1, G2 (R x R each)
  int I[3];
  int R;
  double ref_norm;
};

struct BatchRun {  // the FitCheck parameters of the current optimize call (read by the sweep kernel)
  double tol;
  int max_iter;
  int sweeps_per_pull;  // sweeps a CTA runs on a tensor it pulls (stopping at its check); < 2: one
};

struct BatchCheck {  // fit_check.jl:5-20, per tensor
  int iter, counter, done, sweeps;
  int total_iter, rank_deficient, nan, pad;
  double lastfit, final_fit, fit;
};

struct SmemLayout {
  int Imax, Rmax, ld, lm;  // lm: odd leading dimension (doubles) of M and X
  size_t ring, ring_bytes, f32, M, X, A, G, vec, total;
};

__host__ __device__ inline size_t al16(size_t b) { return (b + 15) & ~size_t(15); }

// The MTTKRP's slab ring holds at least two steps of P slabs; P is chosen so that two steps
// take at most this many bytes, or P = 1 (two 96 x 96 FP32 slabs take 72 KB).
constexpr int kRingBytes = 96 * 1024;

// FP32 elements of one slab of a mode layout (In x Ia), padded to 16 bytes.
__host__ __device__ inline int64_t slab_floats(int In, int Ia) { return (((int64_t)In * Ia + 3) / 4) * 4; }

// Rank columns per MTTKRP thread: 8 unless that pads the rank further than groups of 4 do.
__host__ __device__ inline int rank_width(int R) { return ((R + 7) / 8) * 8 == ((R + 3) / 4) * 4 ? 8 : 4; }

// Slab partitions of one mode's MTTKRP (Ig output groups, Rg rank groups, In x Ia slabs, Ib of
// them): as many as keep the items at 480 or fewer (one round on the MTTKRP's 15 warps of a
// 512-thread CTA) and two steps of P slabs within kRingBytes.
__host__ __device__ inline int mttkrp_parts(int Ig, int Rg, int In, int Ia, int Ib) {
  int P = 480 / (Ig * Rg);
  const int pr = (int)(kRingBytes / (2 * 4 * slab_floats(In, Ia)));
  P = P < pr ? P : pr;
  return P < 1 ? 1 : (P > Ib ? Ib : P);
}

// How one mode's MTTKRP is split: W rank columns and Q output rows (o and o + ceil(In/Q)) per
// thread item, P slab partitions.  Two rows per item when that keeps as many items (the slab
// partitions double instead): half the steps, the Fa loads shared by two rows.  A function of
// the tensor's shape alone, so that the sums and their order do not depend on the thread count
// or the schedule.
struct MttkrpPlan {
  int W, Q, P, Rg, Ig;
};
__host__ __device__ inline MttkrpPlan mttkrp_plan(int In, int Ia, int Ib, int R) {
  MttkrpPlan m;
  m.W = rank_width(R);
  m.Rg = (R + m.W - 1) / m.W;
  const int P1 = mttkrp_parts(In, m.Rg, In, Ia, Ib);
  const int Ih = (In + 1) / 2;
  int P2 = mttkrp_parts(Ih, m.Rg, In, Ia, Ib);
  const int pp = 1 + 4096 / (In * m.Rg * m.W);  // partial pairs of p >= 1 within 32 KB
  P2 = P2 < pp ? P2 : pp;
  if (In >= 2 && Ih * m.Rg * P2 >= In * m.Rg * P1) {
    m.Q = 2, m.P = P2, m.Ig = Ih;
  } else {
    m.Q = 1, m.P = P1, m.Ig = In;
  }
  return m;
}

// Shared memory a tensor's MTTKRP needs beyond the sweep's arrays: the slab ring (two steps of
// P slabs, the largest over the modes) and the partial pairs of the partitions p >= 1.
struct MttkrpNeed {
  size_t ring = 0, part = 0;
};
inline MttkrpNeed mttkrp_need(const int I[3], int R) {
  MttkrpNeed m;
  for (int n = 0; n < 3; ++n) {
    const int ma = (n == 0) ? 1 : 0, mb = (n == 2) ? 1 : 2;
    const MttkrpPlan pl = mttkrp_plan(I[n], I[ma], I[mb], R);
    m.ring = std::max(m.ring, (size_t)2 * pl.P * slab_floats(I[n], I[ma]) * 4);
    m.part = std::max(m.part, (size_t)(pl.P - 1) * I[n] * pl.Rg * pl.W * 8);
  }
  return m;
}

// Imax, Rmax: the largest extent and rank of the tensors that use the layout; need: the
// largest of their MTTKRP needs.  The partial pairs share the space of X, which is free
// during the MTTKRP.
inline SmemLayout smem_layout(int Imax, int Rmax, MttkrpNeed need) {
  SmemLayout L{};
  L.Imax = Imax;
  L.Rmax = (Rmax + 3) & ~3;  // FP32 factor rows of 16-byte multiples (float4 loads)
  Rmax = L.Rmax;
  L.ld = Rmax | 1;
  L.lm = Rmax + 1;  // Rmax is a multiple of 4: odd, so row walks of M and X are conflict-free
  size_t o = 0;
  L.ring = o;
  L.ring_bytes = need.ring;
  o += al16(L.ring_bytes);
  L.f32 = o;
  o += al16((size_t)3 * Imax * Rmax * 4);
  L.M = o;
  o += al16((size_t)Imax * L.lm * 8);
  L.X = o;
  o += al16(std::max((size_t)Imax * L.lm * 8, need.part));
  L.A = o;
  o += al16((size_t)Rmax * L.ld * 8);
  L.G = o;
  o += al16((size_t)3 * Rmax * Rmax * 8);
  L.vec = o;
  o += al16((size_t)6 * Rmax * 8);
  L.total = o;
  return L;
}

__device__ __forceinline__ double block_sum_d(double v, double* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = (lane < nw) ? red[lane] : 0.0;
  for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  __syncthreads();
  return t;
}

// s + c += v, a compensated (Neumaier) FP32 sum: the MTTKRP's sums across slabs stay off the
// FP64 pipe (2 operations per clock per SM on this part), at FP32-product accuracy
__device__ __forceinline__ void acc2(float2& a, float v) {
  const float t = a.x + v;
  a.y += (fabsf(a.x) >= fabsf(v)) ? ((a.x - t) + v) : ((v - t) + a.x);
  a.x = t;
}

// s += v for two compensated pairs: TwoSum of the leading parts, the rest added in FP32
__device__ __forceinline__ void merge2(float2& s, const float2 v) {
  const float t = s.x + v.x;
  const float z = t - s.x;
  const float e = (s.x - (t - z)) + (v.x - z);
  s.x = t;
  s.y = (s.y + v.y) + e;
}


__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_wait_dyn(int n) {
  // wait_group takes an immediate: the ring depths that occur
  if (n <= 0) cp_async_wait<0>();
  else if (n == 1) cp_async_wait<1>();
  else if (n == 2) cp_async_wait<2>();
  else if (n == 3) cp_async_wait<3>();
  else if (n == 4) cp_async_wait<4>();
  else if (n == 5) cp_async_wait<5>();
  else cp_async_wait<6>();
}

// One mode's MTTKRP, M[o][r] = sum_b Fb[b][r] sum_a S_b[o + In a] Fa[a][r], with S_b slab b of the
// mode's own layout of T (this mode's index o fastest, a and b the other two; slabs `slab`
// floats apart, 16-byte aligned).
// Thread item (o, rank group, slab partition p): the W rank columns of output row o over the
// slabs b = p, p + P, ...; the slab's sum over a in FP32, the sum across slabs as compensated
// FP32 pairs in registers.  The slabs stream through a shared-memory ring in steps of P (slab
// s P + p for partition p), 16-byte cp.async copies by all threads, up to NS - 1 steps ahead;
// one barrier per step.  S reads are consecutive across the warp's o, Fa rows broadcast.
// Partition 0 writes M; the others write partial pairs merged into M in the order of p.
__device__ __forceinline__ void bar_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Run by threads [0, nthr) of the block (named barrier 1); the block's last warp runs the
// pivoted sweep meanwhile.
template <int W, int Q>
__device__ __forceinline__ void mttkrp_mode(const float* __restrict__ Tn, int In, int Ia, int Ib, int R,
                                            const MttkrpPlan pl, const float* Fa, const float* Fb, int Rm,
                                            float2* Mc, int lm, float2* part, float* ring, size_t ring_bytes,
                                            int tid, int nthr) {
  const int Rg = pl.Rg, P = pl.P, Ig = pl.Ig;
  const int items = Ig * Rg * P;
  const int slab = (int)slab_floats(In, Ia);
  const int stepf = P * slab;
  const int steps = (Ib + P - 1) / P;
  const int NS = (int)(ring_bytes / ((size_t)stepf * 4)) < 7 ? (int)(ring_bytes / ((size_t)stepf * 4)) : 7;
  auto copy_step = [&](int s) {
    if (s < steps) {
      const int nb = (s + 1) * P <= Ib ? P : Ib - s * P;
      const int n16 = nb * slab / 4;
      const float* src = Tn + (int64_t)s * stepf;
      float* dst = ring + (s % NS) * stepf;
      for (int c = tid; c < n16; c += nthr) cp_async16(dst + 4 * c, src + 4 * c);
    }
    cp_async_commit();  // empty groups keep the count uniform
  };
  for (int e0 = 0; e0 < items; e0 += nthr) {
    const int e = e0 + tid;
    const bool active = e < items;
    const int og = e % Ig, q = e / Ig, rg = q % Rg, p = q / Rg;
    const int r0 = rg * W;
    int orow[Q];
    bool ok[Q];
#pragma unroll
    for (int h = 0; h < Q; ++h) {
      const int o = og + h * Ig;
      ok[h] = o < In;
      orow[h] = ok[h] ? o : og;  // a row past the extent repeats row og; its sums are dropped
    }
    float2 acc[Q][W];
#pragma unroll
    for (int h = 0; h < Q; ++h)
#pragma unroll
      for (int w = 0; w < W; ++w) acc[h][w] = make_float2(0.f, 0.f);
    bar_sync(1, nthr);  // the ring's previous contents are consumed
    for (int s = 0; s < NS - 1; ++s) copy_step(s);
    for (int s = 0; s < steps; ++s) {
      cp_async_wait_dyn(NS - 2);  // this thread's copies of step s have landed
      bar_sync(1, nthr);          // everyone's have; step s - 1's slot is free
      copy_step(s + NS - 1);
      const int b = s * P + p;
      if (active && b < Ib) {
        const float* S = ring + (s % NS) * stepf + p * slab;
        float t[Q][W];
#pragma unroll
        for (int h = 0; h < Q; ++h)
#pragma unroll
          for (int w = 0; w < W; ++w) t[h][w] = 0.f;
#pragma unroll 8
        for (int a = 0; a < Ia; ++a) {
          float sv[Q];
#pragma unroll
          for (int h = 0; h < Q; ++h) sv[h] = S[orow[h] + a * In];
          const float* fr = Fa + a * Rm + r0;
#pragma unroll
          for (int w4 = 0; w4 < W; w4 += 4) {
            const float4 f = *reinterpret_cast<const float4*>(fr + w4);
#pragma unroll
            for (int h = 0; h < Q; ++h) {
              t[h][w4] = fmaf(sv[h], f.x, t[h][w4]);
              t[h][w4 + 1] = fmaf(sv[h], f.y, t[h][w4 + 1]);
              t[h][w4 + 2] = fmaf(sv[h], f.z, t[h][w4 + 2]);
              t[h][w4 + 3] = fmaf(sv[h], f.w, t[h][w4 + 3]);
            }
          }
        }
        const float* gr = Fb + b * Rm + r0;
#pragma unroll
        for (int w4 = 0; w4 < W; w4 += 4) {
          const float4 g = *reinterpret_cast<const float4*>(gr + w4);
#pragma unroll
          for (int h = 0; h < Q; ++h) {
            acc2(acc[h][w4], t[h][w4] * g.x);
            acc2(acc[h][w4 + 1], t[h][w4 + 1] * g.y);
            acc2(acc[h][w4 + 2], t[h][w4 + 2] * g.z);
            acc2(acc[h][w4 + 3], t[h][w4 + 3] * g.w);
          }
        }
      }
    }
    cp_async_wait<0>();  // no copy is left in flight (the trailing groups are empty)
    if (active) {
#pragma unroll
      for (int h = 0; h < Q; ++h) {
        if (!ok[h]) continue;
        const int o = orow[h];
        if (p == 0) {
          float2* d = Mc + o * lm + r0;
#pragma unroll
          for (int w = 0; w < W; ++w)
            if (r0 + w < R) d[w] = acc[h][w];
        } else {
          float2* d = part + ((size_t)((p - 1) * Rg + rg) * In + o) * W;
#pragma unroll
          for (int w = 0; w < W; ++w) d[w] = acc[h][w];
        }
      }
    }
  }
  if (P > 1) {
    bar_sync(1, nthr);
    for (int e = tid; e < In * R; e += nthr) {
      const int o = e / R, r = e - o * R, rg = r / W, w = r - rg * W;
      float2 sm2 = Mc[o * lm + r];
      for (int p = 1; p < P; ++p) merge2(sm2, part[((size_t)((p - 1) * Rg + rg) * In + o) * W + w]);
      Mc[o * lm + r] = sm2;
    }
  }
}

__device__ __forceinline__ long long bkey(double v) {
  const long long k = __double_as_longlong(v);
  return (k & 0x7fffffffffffffffll) > 0x7ff0000000000000ll ? LLONG_MAX : k;
}

// One ALS sweep of tensor `it` by the whole CTA.
__device__ void batch_sweep_one(const BatchItem& it, const float* __restrict__ T, double* __restrict__ Fg,
                                double* __restrict__ Gg, BatchCheck* __restrict__ chk, const SmemLayout& L,
                                unsigned char* sm, double tol, int max_iter) {
  __shared__ double red[32];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  const int R = it.R, I0 = it.I[0], I1 = it.I[1], I2 = it.I[2];
  const int Rm = L.Rmax;
  const int lm = L.lm;
  float* F32 = reinterpret_cast<float*>(sm + L.f32);  // F32 + m*Imax*Rm: [I_m][R] row-major (ld Rm)
  double* M = reinterpret_cast<double*>(sm + L.M);     // [I_n][Rm]
  double* X = reinterpret_cast<double*>(sm + L.X);     // [I_n][Rm]
  double* A = reinterpret_cast<double*>(sm + L.A);     // [R][ld]
  double* G = reinterpret_cast<double*>(sm + L.G);     // 3 x [R][R]
  double* vec = reinterpret_cast<double*>(sm + L.vec);
  double* lam = vec;          // R
  double* a_row = vec + Rm;   // pivot row
  double* t_row = vec + 2 * Rm;
  const int ld = L.ld;
  double* F0g = Fg + it.foff;
  const int64_t fo1 = (int64_t)I0 * R, fo2 = (int64_t)(I0 + I1) * R;
  double* lamg = Fg + it.foff + (int64_t)(I0 + I1 + I2) * R;
  // factors (FP32 copies, zero beyond column R) and Grams into shared memory
  for (int e = tid; e < 3 * L.Imax * Rm; e += nt) F32[e] = 0.f;
  __syncthreads();
  for (int m = 0; m < 3; ++m)
    for (int e = tid; e < it.I[m] * R; e += nt) {
      const int i = e % it.I[m], r = e / it.I[m];
      F32[(size_t)m * L.Imax * Rm + (size_t)i * Rm + r] = (float)F0g[(m == 0 ? 0 : m == 1 ? fo1 : fo2) + e];
    }
  for (int e = tid; e < 3 * R * R; e += nt) G[e] = Gg[it.goff + e];
  __syncthreads();
  double inner = 0.0;
  for (int n = 0; n < 3; ++n) {
    const int In = it.I[n];
    const int64_t fon = n == 0 ? 0 : n == 1 ? fo1 : fo2;
    // ---- MTTKRP (warps 0 .. nw-2) and, concurrently, V and its pivoted sweep (the last
    // warp): V = G_a .* G_b needs only the other modes' Grams.
    float2* Mc = reinterpret_cast<float2*>(M);
    if (warp < nwarps - 1) {
      // MTTKRP from the mode's own layout of T (this mode's index fastest): mode 0 over
      // (a, b) = (j, k), mode 1 over (i, k), mode 2 over (i, j); M as compensated FP32 pairs
      // (same bytes as the FP64 array, float2 per entry)
      const int ma = (n == 0) ? 1 : 0, mb = (n == 2) ? 1 : 2;
      const float* Tn = T + it.loff[n];
      const float* Fa = F32 + (size_t)ma * L.Imax * Rm;
      const float* Fb = F32 + (size_t)mb * L.Imax * Rm;
      float2* part = reinterpret_cast<float2*>(X);
      float* ring = reinterpret_cast<float*>(sm + L.ring);
      const MttkrpPlan pl = mttkrp_plan(In, it.I[ma], it.I[mb], R);
      if (pl.W == 8 && pl.Q == 2)
        mttkrp_mode<8, 2>(Tn, In, it.I[ma], it.I[mb], R, pl, Fa, Fb, Rm, Mc, lm, part, ring, L.ring_bytes, tid, nt - 32);
      else if (pl.W == 8)
        mttkrp_mode<8, 1>(Tn, In, it.I[ma], it.I[mb], R, pl, Fa, Fb, Rm, Mc, lm, part, ring, L.ring_bytes, tid, nt - 32);
      else if (pl.Q == 2)
        mttkrp_mode<4, 2>(Tn, In, it.I[ma], it.I[mb], R, pl, Fa, Fb, Rm, Mc, lm, part, ring, L.ring_bytes, tid, nt - 32);
      else
        mttkrp_mode<4, 1>(Tn, In, it.I[ma], it.I[mb], R, pl, Fa, Fb, Rm, Mc, lm, part, ring, L.ring_bytes, tid, nt - 32);
    } else {
      // V = G_a .* G_b (mode order), upper triangle into A
      const double* Ga = G + (size_t)(n == 0 ? 1 : 0) * R * R;
      const double* Gb = G + (size_t)(n == 2 ? 1 : 2) * R * R;
      for (int e = lane; e < R * R; e += 32) {
        const int r = e / R, c = e - r * R;
        if (c >= r) A[r * ld + c] = (1.0 * Ga[e]) * Gb[e];
      }
      // pivoted symmetric sweep (same pivot rule and tolerance as dpstrf), by this warp alone
      for (int i = lane; i < R; i += 32) vec[3 * Rm + i] = 0.0;  // swept flags
      __syncwarp();
      int rank = R;
      for (int j = 0; j < R; ++j) {
        long long bk = LLONG_MIN;
        int bi = R;
        for (int i = lane; i < R; i += 32) {
          // the unswept diagonal entries; swept ones hold negative values (-1/d)
          const double d = A[i * ld + i];
          const long long key = (vec[3 * Rm + i] != 0.0) ? LLONG_MIN : bkey(d);
          if (bi == R || key > bk) {
            bk = key;
            bi = i;
          }
        }
        const int khi = (int)(bk >> 32);
        const int mhi = __reduce_max_sync(0xffffffffu, khi);
        const unsigned mlo = __reduce_max_sync(0xffffffffu, khi == mhi ? (unsigned)(bk & 0xffffffffll) : 0u);
        const long long mk = (long long)(((unsigned long long)(unsigned)mhi << 32) | mlo);
        const int k = __reduce_min_sync(0xffffffffu, (bi < R && bk == mk) ? bi : INT_MAX);
        if ((mk == LLONG_MAX) || !(mk > bkey(kBatchTol)) || k >= R) {  // warp-uniform
          rank = j;
          break;
        }
        const double dk = 1.0 / __longlong_as_double(mk);
        for (int i = lane; i < R; i += 32) {
          const double av = (i <= k) ? A[i * ld + k] : A[k * ld + i];
          a_row[i] = av;
          t_row[i] = av * dk;
        }
        __syncwarp();
        for (int c = lane; c < R; c += 32) {
          const double tc = t_row[c];
          for (int i = 0; i <= c; ++i) {
            double v;
            if (i == k && c == k) v = -dk;
            else if (i == k) v = tc;
            else if (c == k) v = t_row[i];
            else v = fma(-a_row[i], tc, A[i * ld + c]);
            A[i * ld + c] = v;
          }
        }
        if (lane == 0) vec[3 * Rm + k] = 1.0;
        __syncwarp();
      }
      // W = -A on the swept indices.  A rank-deficient V (a pivot <= 1e-6) keeps the basic
      // solution: the unswept components of X are zero (the reference's pivoted-QR
      // fallback, ldiv_solve.jl:20-21, returns its least-squares solution instead)
      if (rank < R && lane == 0) chk->rank_deficient += 1;
    }
    __syncthreads();
    // ---- X = M W: W(l, c) = -A(min, max) for swept l, c; 0 otherwise.  M is the MTTKRP's
    // FP32 pair m = mh + ml and W is split the same way (into the space of G_n, which is
    // rewritten at the end of the mode); each product is a compensated FP32 dot product
    // (Dot2: the mh wh terms split exactly by one FMA and summed with TwoSum, the cross
    // terms added in FP32), as accurate as FP64 to ~2^-48 and off the FP64 pipe.
    float2* Wp = reinterpret_cast<float2*>(G + (size_t)n * R * R);
    for (int e = tid; e < R * R; e += nt) {
      const int l = e / R, c = e - l * R;
      const bool sw = vec[3 * Rm + c] != 0.0 && vec[3 * Rm + l] != 0.0;
      const double w = sw ? -((l <= c) ? A[l * ld + c] : A[c * ld + l]) : 0.0;
      const float wh = (float)w;
      Wp[e] = make_float2(wh, (float)(w - (double)wh));
    }
    __syncthreads();
    for (int e = tid; e < In * R; e += nt) {
      const int i = e / R, c = e - i * R;
      const float2* mrow = Mc + i * lm;
      float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
      // the _rn intrinsics keep the compiler from contracting the error-free steps into FMAs
      auto term = [&](const float2 m, const float2 w, float& sa, float& ca) {
        const float pr = __fmul_rn(m.x, w.x);
        const float pe = fmaf(m.x, w.x, -pr);
        const float t = __fadd_rn(sa, pr);
        const float z = __fsub_rn(t, sa);
        const float er = __fadd_rn(__fsub_rn(sa, __fsub_rn(t, z)), __fsub_rn(pr, z));
        sa = t;
        ca += (pe + er) + fmaf(m.x, w.y, m.y * w.x);
      };
      int l = 0;
      for (; l + 2 <= R; l += 2) {
        term(mrow[l], Wp[l * R + c], s0, c0);
        term(mrow[l + 1], Wp[(l + 1) * R + c], s1, c1);
      }
      if (l < R) term(mrow[l], Wp[l * R + c], s0, c0);
      X[i * lm + c] = ((double)s0 + (double)s1) + ((double)c0 + (double)c1);
    }
    __syncthreads();
    // ---- <T, X> on the last mode (fit_check.jl:28)
    if (n == 2) {
      double p = 0.0;
      for (int e = tid; e < In * R; e += nt) {
        const float2 m = Mc[(e / R) * lm + e % R];
        p += ((double)m.x + (double)m.y) * X[(e / R) * lm + e % R];
      }
      inner = block_sum_d(p, red);
    }
    // ---- lambda = column norms, F_n = X / lambda (row_norm.jl:4-24)
    for (int r = warp; r < R; r += nt >> 5) {
      double s = 0.0;
      for (int i = lane; i < In; i += 32) s = fma(X[i * lm + r], X[i * lm + r], s);
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (lane == 0) {
        const double l = sqrt(s);
        lam[r] = l;
        // one FP64 reciprocal per column (the FP64 divide is a long software sequence on this
        // part's FP64 pipe); a column left at zero by a rank-deficient solve (basic solution)
        // stays zero
        t_row[r] = (l > 0.0) ? 1.0 / l : 0.0;
      }
    }
    __syncthreads();
    float* Fn32 = F32 + (size_t)n * L.Imax * Rm;
    for (int e = tid; e < In * R; e += nt) {
      const int i = e / R, r = e - i * R;
      const double f = X[i * lm + r] * t_row[r];
      X[i * lm + r] = f;
      F0g[fon + i + (int64_t)In * r] = f;
      Fn32[i * Rm + r] = (float)f;
    }
    __syncthreads();
    // ---- G_n = F_n^T F_n (standard/tensor.jl:46-49)
    double* Gn = G + (size_t)n * R * R;
    for (int e = tid; e < R * R; e += nt) {
      const int r = e / R, c = e - r * R;
      if (c < r) continue;
      double s0 = 0.0, s1 = 0.0;
      int i = 0;
      for (; i + 1 < In; i += 2) {
        s0 = fma(X[i * lm + r], X[i * lm + c], s0);
        s1 = fma(X[(i + 1) * lm + r], X[(i + 1) * lm + c], s1);
      }
      if (i < In) s0 = fma(X[i * lm + r], X[i * lm + c], s0);
      Gn[r * R + c] = s0 + s1;
      Gn[c * R + r] = s0 + s1;
    }
    __syncthreads();
  }
  // ---- fit and FitCheck (fit_check.jl:24-66; converge_checks.jl:5-11)
  double pf = 0.0;
  for (int e = tid; e < R * R; e += nt) {
    const int r = e / R, c = e - r * R;
    pf += ((G[e] * G[R * R + e]) * G[2 * R * R + e]) * (lam[r] * lam[c]);
  }
  const double fact = block_sum_d(pf, red);
  for (int e = tid; e < 3 * R * R; e += nt) Gg[it.goff + e] = G[e];
  for (int r = tid; r < R; r += nt) lamg[r] = lam[r];
  if (tid == 0) {
    BatchCheck& c = *chk;
    const double rn = it.ref_norm;
    const double fit = 1.0 - sqrt(fabs(rn * rn + fact - 2.0 * fabs(inner))) / rn;
    c.fit = fit;
    c.sweeps += 1;
    c.iter += 1;
    const double dfit = fabs(c.lastfit - fit);
    c.lastfit = fit;
    if (isnan(fit)) {
      c.nan = 1;
      c.done = 1;
    } else if (dfit < tol) {
      c.counter += 1;
      if (c.counter >= 2) {
        c.total_iter = c.iter;
        c.final_fit = fit;
        c.done = 1;
      }
    } else {
      c.counter = 0;
    }
    if (!c.done && c.iter >= max_iter) {
      c.total_iter = c.iter;
      c.final_fit = fit;
      c.done = 1;
    }
  }
  __syncthreads();
}

template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_batch_sweep(const BatchItem* __restrict__ items, const int* __restrict__ order,
                                                    int count, const float* __restrict__ T, double* __restrict__ F,
                                                    double* __restrict__ G, BatchCheck* __restrict__ chk,
                                                    unsigned* __restrict__ queue, SmemLayout L,
                                                    const BatchRun* __restrict__ run) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ int s_t;
  const double tol = run->tol;
  const int max_iter = run->max_iter;
  const int spp = run->sweeps_per_pull > 1 ? run->sweeps_per_pull : 1;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_t = (int)atomicAdd(queue, 1u);
    __syncthreads();
    const int t = s_t;
    if (t >= count) break;
    const int id = order[t];
    if (chk[id].done) continue;
    // one sweep, or up to spp: each tensor's sweeps and check are its own, so running several
    // back to back in one CTA gives the same results as one launch per sweep
    for (int s = 0; s < spp; ++s) {
      batch_sweep_one(items[id], T, F, G, &chk[id], L, sm, tol, max_iter);  // ends with a block barrier
      if (*reinterpret_cast<volatile const int*>(&chk[id].done)) break;
    }
  }
}

__global__ void k_batch_reset(unsigned* queue, int nqueue, const BatchCheck* chk, int count, int* active) {
  // queue resets for the next launch, and the count of active tensors (read by the host)
  __shared__ int s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  int a = 0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) a += chk[i].done ? 0 : 1;
  atomicAdd(&s, a);
  __syncthreads();
  if (threadIdx.x < nqueue) queue[threadIdx.x] = 0u;
  if (threadIdx.x == 0) *active = s;
}

// dst[y + dx x] = src[x + sy y] for x < X, y < Y, through a 32 x 33 tile (256 threads).
__device__ void transpose_plane(const float* __restrict__ src, float* __restrict__ dst, int X, int Y, int64_t sy,
                                int64_t dx, float (*tile)[33]) {
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int y0 = 0; y0 < Y; y0 += 32)
    for (int x0 = 0; x0 < X; x0 += 32) {
      for (int yy = ty; yy < 32; yy += 8) {
        const int x = x0 + tx, y = y0 + yy;
        if (x < X && y < Y) tile[yy][tx] = src[x + sy * y];
      }
      __syncthreads();
      for (int xx = ty; xx < 32; xx += 8) {
        const int x = x0 + xx, y = y0 + tx;
        if (x < X && y < Y) dst[y + dx * x] = tile[tx][xx];
      }
      __syncthreads();
    }
}

// The MTTKRP's per-mode layouts of every tensor, from the natural one (T[i + I0 j + I0 I1 k]):
// mode n's layout holds element (o, a, b) at loff[n] + b slab + o + In a, with o mode n's index
// and (a, b) = (j, k), (i, k), (i, j) for n = 0, 1, 2; slabs are padded to 16 bytes so that the
// sweep streams them with 16-byte copies.  256 threads per block.
__global__ void k_batch_layouts(const BatchItem* __restrict__ items, int count, const float* __restrict__ T,
                                float* __restrict__ Lay) {
  __shared__ float tile[32][33];
  for (int id = blockIdx.x; id < count; id += gridDim.x) {
    const BatchItem it = items[id];
    const int I0 = it.I[0], I1 = it.I[1], I2 = it.I[2];
    const float* src = T + it.toff;
    const int64_t s0 = slab_floats(I0, I1), s1 = slab_floats(I1, I0), s2 = slab_floats(I2, I0);
    const int64_t plane = (int64_t)I0 * I1;
    for (int k = 0; k < I2; ++k)
      for (int e = threadIdx.x; e < plane; e += blockDim.x) Lay[it.loff[0] + k * s0 + e] = src[plane * k + e];
    for (int k = 0; k < I2; ++k) transpose_plane(src + plane * k, Lay + it.loff[1] + k * s1, I0, I1, I0, I1, tile);
    for (int j = 0; j < I1; ++j)
      transpose_plane(src + (int64_t)I0 * j, Lay + it.loff[2] + j * s2, I0, I2, plane, I2, tile);
  }
}

// Grams of the initial factors, and lambda / checks reset.
__global__ void k_batch_init(const BatchItem* __restrict__ items, int count, double* __restrict__ F,
                             double* __restrict__ G, BatchCheck* __restrict__ chk) {
  for (int id = blockIdx.x; id < count; id += gridDim.x) {
    const BatchItem it = items[id];
    const int R = it.R;
    int64_t off = it.foff;
    for (int m = 0; m < 3; ++m) {
      const double* Fm = F + off;
      for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        const int r = e / R, c = e % R;
        double s = 0.0;
        for (int i = 0; i < it.I[m]; ++i) s = fma(Fm[i + (int64_t)it.I[m] * r], Fm[i + (int64_t)it.I[m] * c], s);
        G[it.goff + (int64_t)m * R * R + e] = s;
      }
      off += (int64_t)it.I[m] * R;
    }
    if (threadIdx.x == 0) {
      BatchCheck c{};
      c.lastfit = 1.0;  // fit_check.jl:16-20
      chk[id] = c;
    }
  }
}

}  // namespace

}  // namespace cpals

using namespace cpals;

// A size class of the batch: the tensors order[begin, end) (largest work first), swept by one
// persistent launch with a shared-memory layout sized to the class's largest extent and rank,
// so that small tensors get several CTAs per SM.  Classes run concurrently on their own streams.
struct BatchClass {
  int begin = 0, end = 0;
  int Imax = 0, Rmax = 0;
  MttkrpNeed need;
  SmemLayout L{};
  int nt = 256;
  int ctas_per_sm = 1;
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  float ms_alone = 0.f;  // the autotuner's time for this class alone
};
constexpr int kMaxBatchClasses = 4;

struct cpals_batch {
  int device = 0;
  int64_t count = 0;
  int Imax = 0, Rmax = 0;
  MttkrpNeed need;  // the largest MTTKRP needs of the batch
  std::vector<BatchItem> items;
  std::vector<int> order;
  int64_t tot_T = 0, tot_L = 0, tot_F = 0, tot_G = 0;
  BatchItem* d_items = nullptr;
  int* d_order = nullptr;
  float* d_T = nullptr;  // the tensors as uploaded
  float* d_L = nullptr;  // the MTTKRP's per-mode layouts
  double* d_F = nullptr;
  double* d_G = nullptr;
  BatchCheck* d_chk = nullptr;
  unsigned* d_queue = nullptr;
  int* d_active = nullptr;
  int* h_active = nullptr;
  BatchRun* d_run = nullptr;  // tol and max_iter, outside the graph so that changing them keeps it
  BatchRun* h_run = nullptr;
  cudaStream_t st = nullptr;
  cudaGraphExec_t graph = nullptr;
  int nt = 256;         // threads per CTA (autotuned)
  int ctas_per_sm = 1;  // resident CTAs per SM (from the occupancy calculator)
  double tol = 1e-5;
  int max_iter = 200;
  int sweeps_per_launch = 0;  // 0: every tensor to its own stop in one launch
  int num_sms = 0;
  SmemLayout L{};
  int64_t launches = 0;
  // the schedule: one class (every tensor, layout L) or the classes by CTAs per SM
  std::vector<BatchClass> cls;
  std::vector<int> order_one, order_split;  // LPT order of the single class; by class, then LPT
  std::vector<BatchClass> split;           // the candidate classes
  cudaEvent_t fork = nullptr;
  double ms_split = -1.0;  // the autotuner's time for the split schedule (< 0: not tried)
};

namespace {

const void* sweep_fn(int nt) {
  return nt == 128 ? (const void*)k_batch_sweep<128> : nt == 256 ? (const void*)k_batch_sweep<256>
                                                                 : (const void*)k_batch_sweep<512>;
}

// One class's persistent launch on stream st (queue slot q).
int class_launch(cpals_batch* b, const BatchClass& c, int q, cudaStream_t st) {
  const int n = c.end - c.begin;
  if (n <= 0) return CPALS_OK;
  const int grid = std::min(b->num_sms * c.ctas_per_sm, n);
  const int* order = b->d_order + c.begin;
  switch (c.nt) {
    case 128:
      k_batch_sweep<128><<<grid, 128, c.L.total, st>>>(b->d_items, order, n, b->d_L, b->d_F, b->d_G, b->d_chk,
                                                          b->d_queue + q, c.L, b->d_run);
      break;
    case 256:
      k_batch_sweep<256><<<grid, 256, c.L.total, st>>>(b->d_items, order, n, b->d_L, b->d_F, b->d_G, b->d_chk,
                                                          b->d_queue + q, c.L, b->d_run);
      break;
    case 512:
      k_batch_sweep<512><<<grid, 512, c.L.total, st>>>(b->d_items, order, n, b->d_L, b->d_F, b->d_G, b->d_chk,
                                                          b->d_queue + q, c.L, b->d_run);
      break;
    default:
      return CPALS_E_ARG;
  }
  b->launches += 1;
  return cudaGetLastError() == cudaSuccess ? CPALS_OK : CPALS_E_CUDA;
}

// One sweep of every active tensor: the classes' launches forked from and joined back to the
// batch's stream, then the queue resets and the active count.
int batch_launch(cpals_batch* b) {
  const int nc = (int)b->cls.size();
  if (nc == 1) {
    int rc = class_launch(b, b->cls[0], 0, b->st);
    if (rc != CPALS_OK) return rc;
  } else {
    if (cudaEventRecord(b->fork, b->st) != cudaSuccess) return CPALS_E_CUDA;
    for (int i = 0; i < nc; ++i) {
      BatchClass& c = b->cls[i];
      if (cudaStreamWaitEvent(c.st, b->fork, 0) != cudaSuccess) return CPALS_E_CUDA;
      int rc = class_launch(b, c, i, c.st);
      if (rc != CPALS_OK) return rc;
      if (cudaEventRecord(c.done, c.st) != cudaSuccess || cudaStreamWaitEvent(b->st, c.done, 0) != cudaSuccess)
        return CPALS_E_CUDA;
    }
  }
  k_batch_reset<<<1, 1024, 0, b->st>>>(b->d_queue, kMaxBatchClasses, b->d_chk, (int)b->count, b->d_active);
  b->launches += 1;
  return cudaGetLastError() == cudaSuccess ? CPALS_OK : CPALS_E_CUDA;
}

// Thread count of class c: sets the kernel's shared-memory limit and the resident CTAs per SM.
int class_config(BatchClass& c, int nt) {
  const void* fn = sweep_fn(nt);
  // the opt-in maximum less the kernel's static shared memory
  if (set_smem_limit_once(fn, 227 * 1024) != cudaSuccess) return CPALS_E_CUDA;
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) {
    (void)cudaGetLastError();
    return CPALS_E_CUDA;
  }
  if (c.L.total > (size_t)fa.maxDynamicSharedSizeBytes) return CPALS_E_UNSUPPORTED;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, nt, c.L.total) != cudaSuccess || per_sm < 1) {
    (void)cudaGetLastError();
    return CPALS_E_UNSUPPORTED;
  }
  c.nt = nt;
  c.ctas_per_sm = per_sm;
  return CPALS_OK;
}

void drop_graph(cpals_batch* b) {
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
}

// Makes `classes` (with `order`) the schedule: uploads the order, rebuilds the graph later.
int use_schedule(cpals_batch* b, const std::vector<BatchClass>& classes, const std::vector<int>& order) {
  CPALS_CUDA_TRY(cudaStreamSynchronize(b->st));
  CPALS_CUDA_TRY(cudaMemcpy(b->d_order, order.data(), sizeof(int) * b->count, cudaMemcpyHostToDevice));
  b->cls = classes;
  drop_graph(b);
  return CPALS_OK;
}

// The single class with nt threads per CTA (the whole batch, the batch-wide layout).
int set_config(cpals_batch* b, int nt) {
  BatchClass c;
  c.begin = 0;
  c.end = (int)b->count;
  c.Imax = b->Imax;
  c.Rmax = b->Rmax;
  c.L = b->L;
  c.st = b->st;
  int rc = class_config(c, nt);
  if (rc != CPALS_OK) return rc;
  b->nt = nt;
  b->ctas_per_sm = c.ctas_per_sm;
  return use_schedule(b, {c}, b->order_one);
}

int build_graph(cpals_batch* b) {
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return CPALS_E_CUDA;
  const int64_t before = b->launches;
  int rc = batch_launch(b);
  b->launches = before;
  cudaError_t e = cudaStreamEndCapture(b->st, &g);
  if (rc != CPALS_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return rc != CPALS_OK ? rc : CPALS_E_CUDA;
  }
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  return e == cudaSuccess ? CPALS_OK : CPALS_E_CUDA;
}

}  // namespace

extern "C" {

int cpals_batch_create(cpals_batch** out, int device, int64_t count, const int64_t* dims, const int64_t* ranks,
                       const double* ref_norms) {
  if (!out || count < 1 || !dims || !ranks || !ref_norms) return CPALS_E_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CPALS_E_CUDA;
  DeviceGuard guard(device);
  cpals_batch* b = new cpals_batch();
  b->device = device;
  b->count = count;
  b->items.resize(count);
  for (int64_t t = 0; t < count; ++t) {
    BatchItem& it = b->items[t];
    for (int m = 0; m < 3; ++m) {
      if (dims[3 * t + m] < 1 || dims[3 * t + m] > 4096) {
        delete b;
        return CPALS_E_ARG;
      }
      it.I[m] = (int)dims[3 * t + m];
    }
    if (ranks[t] < 1 || ranks[t] > 64 || !(ref_norms[t] > 0.0)) {
      delete b;
      return CPALS_E_ARG;
    }
    it.R = (int)ranks[t];
    it.ref_norm = ref_norms[t];
    it.toff = b->tot_T;
    it.foff = b->tot_F;
    it.goff = b->tot_G;
    b->tot_T += (int64_t)it.I[0] * it.I[1] * it.I[2];
    it.loff[0] = b->tot_L;
    b->tot_L += it.I[2] * slab_floats(it.I[0], it.I[1]);
    it.loff[1] = b->tot_L;
    b->tot_L += it.I[2] * slab_floats(it.I[1], it.I[0]);
    it.loff[2] = b->tot_L;
    b->tot_L += it.I[1] * slab_floats(it.I[2], it.I[0]);
    b->tot_F += (int64_t)(it.I[0] + it.I[1] + it.I[2] + 1) * it.R;
    b->tot_G += (int64_t)3 * it.R * it.R;
    b->Imax = std::max({b->Imax, it.I[0], it.I[1], it.I[2]});
    b->Rmax = std::max(b->Rmax, it.R);
    const MttkrpNeed m = mttkrp_need(it.I, it.R);
    b->need.ring = std::max(b->need.ring, m.ring);
    b->need.part = std::max(b->need.part, m.part);
  }
  b->L = smem_layout(b->Imax, b->Rmax, b->need);
  if (b->L.total > 227 * 1024) {
    delete b;
    return CPALS_E_UNSUPPORTED;
  }
  // largest work first (longest-processing-time order)
  b->order.resize(count);
  std::iota(b->order.begin(), b->order.end(), 0);
  std::vector<double> work(count);
  for (int64_t t = 0; t < count; ++t) {
    const BatchItem& it = b->items[t];
    work[t] = (double)it.I[0] * it.I[1] * it.I[2] * it.R + 3.0 * it.R * it.R * it.R * 20.0;
  }
  std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int c) { return work[a] > work[c]; });
  b->order_one = b->order;
  // The candidate split: by the CTAs per SM a tensor's own layout allows (1 to 4, at the
  // batch's largest rank), one class per value; LPT order inside each class.
  {
    std::vector<int> cps(count);
    for (int64_t t = 0; t < count; ++t) {
      const BatchItem& it = b->items[t];
      const size_t tot = smem_layout(std::max({it.I[0], it.I[1], it.I[2]}), b->Rmax, mttkrp_need(it.I, it.R)).total;
      cps[t] = (int)std::max<size_t>(1, std::min<size_t>(kMaxBatchClasses, (227 * 1024) / tot));
    }
    for (int k = 1; k <= kMaxBatchClasses; ++k) {
      BatchClass c;
      c.begin = (int)b->order_split.size();
      for (int t : b->order)
        if (cps[t] == k) {
          b->order_split.push_back(t);
          c.Imax = std::max({c.Imax, b->items[t].I[0], b->items[t].I[1], b->items[t].I[2]});
          c.Rmax = std::max(c.Rmax, b->items[t].R);
          const MttkrpNeed m = mttkrp_need(b->items[t].I, b->items[t].R);
          c.need.ring = std::max(c.need.ring, m.ring);
          c.need.part = std::max(c.need.part, m.part);
        }
      c.end = (int)b->order_split.size();
      if (c.end > c.begin) {
        c.L = smem_layout(c.Imax, c.Rmax, c.need);
        b->split.push_back(c);
      }
    }
  }
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, device);
  bool ok = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&b->d_items, sizeof(BatchItem) * count) == cudaSuccess &&
            cudaMalloc(&b->d_order, sizeof(int) * count) == cudaSuccess &&
            cudaMalloc(&b->d_T, sizeof(float) * b->tot_T) == cudaSuccess &&
            cudaMalloc(&b->d_L, sizeof(float) * b->tot_L) == cudaSuccess &&
            cudaMemset(b->d_L, 0, sizeof(float) * b->tot_L) == cudaSuccess &&  // slab padding
            cudaMalloc(&b->d_F, sizeof(double) * b->tot_F) == cudaSuccess &&
            cudaMalloc(&b->d_G, sizeof(double) * b->tot_G) == cudaSuccess &&
            cudaMalloc(&b->d_chk, sizeof(BatchCheck) * count) == cudaSuccess &&
            cudaMalloc(&b->d_queue, sizeof(unsigned) * kMaxBatchClasses) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaMalloc(&b->d_active, sizeof(int)) == cudaSuccess &&
            cudaMallocHost(&b->h_active, sizeof(int)) == cudaSuccess &&
            cudaMalloc(&b->d_run, sizeof(BatchRun)) == cudaSuccess &&
            cudaMallocHost(&b->h_run, sizeof(BatchRun)) == cudaSuccess;
  for (BatchClass& c : b->split)
    ok = ok && cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cpals_batch_destroy(b);
    return CPALS_E_CUDA;
  }
  cudaMemcpy(b->d_items, b->items.data(), sizeof(BatchItem) * count, cudaMemcpyHostToDevice);
  *b->h_run = BatchRun{b->tol, b->max_iter, 1};  // what the autotuner's sweeps use
  cudaMemcpy(b->d_run, b->h_run, sizeof(BatchRun), cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_order, b->order.data(), sizeof(int) * count, cudaMemcpyHostToDevice);
  cudaMemset(b->d_queue, 0, sizeof(unsigned) * kMaxBatchClasses);
  cudaMemset(b->d_chk, 0, sizeof(BatchCheck) * count);
  int rc = set_config(b, 256);
  if (rc != CPALS_OK) rc = set_config(b, 128);
  if (rc != CPALS_OK) {
    cpals_batch_destroy(b);
    return rc;
  }
  *out = b;
  return CPALS_OK;
}

int cpals_batch_destroy(cpals_batch* b) {
  if (!b) return CPALS_OK;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->d_items);
  cudaFree(b->d_order);
  cudaFree(b->d_T);
  cudaFree(b->d_L);
  cudaFree(b->d_F);
  cudaFree(b->d_G);
  cudaFree(b->d_chk);
  cudaFree(b->d_queue);
  cudaFree(b->d_active);
  if (b->h_active) cudaFreeHost(b->h_active);
  cudaFree(b->d_run);
  if (b->h_run) cudaFreeHost(b->h_run);
  for (BatchClass& c : b->split) {
    if (c.st) cudaStreamDestroy(c.st);
    if (c.done) cudaEventDestroy(c.done);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return CPALS_OK;
}

int cpals_batch_set_tensors(cpals_batch* b, const float* host_concat) {
  if (!b || !host_concat) return CPALS_E_ARG;
  DeviceGuard guard(b->device);
  CPALS_CUDA_TRY(cudaMemcpyAsync(b->d_T, host_concat, sizeof(float) * b->tot_T, cudaMemcpyHostToDevice, b->st));
  const int blocks = (int)std::min<int64_t>(b->count, 8192);
  k_batch_layouts<<<blocks, 256, 0, b->st>>>(b->d_items, (int)b->count, b->d_T, b->d_L);
  CPALS_CUDA_TRY(cudaGetLastError());
  b->launches += 1;
  return CPALS_OK;
}

int cpals_batch_set_norms(cpals_batch* b, const double* ref_norms) {
  if (!b || !ref_norms) return CPALS_E_ARG;
  for (int64_t t = 0; t < b->count; ++t)
    if (!(ref_norms[t] > 0.0) || !std::isfinite(ref_norms[t])) return CPALS_E_ARG;
  DeviceGuard guard(b->device);
  for (int64_t t = 0; t < b->count; ++t) b->items[t].ref_norm = ref_norms[t];
  CPALS_CUDA_TRY(cudaMemcpyAsync(b->d_items, b->items.data(), sizeof(BatchItem) * b->count, cudaMemcpyHostToDevice,
                                 b->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(b->st));  // the host array is the copy's source
  return CPALS_OK;
}

int cpals_batch_set_factors(cpals_batch* b, const double* host_concat) {
  if (!b || !host_concat) return CPALS_E_ARG;
  DeviceGuard guard(b->device);
  CPALS_CUDA_TRY(cudaMemcpyAsync(b->d_F, host_concat, sizeof(double) * b->tot_F, cudaMemcpyHostToDevice, b->st));
  const int blocks = (int)std::min<int64_t>(b->count, 4096);
  k_batch_init<<<blocks, 256, 0, b->st>>>(b->d_items, (int)b->count, b->d_F, b->d_G, b->d_chk);
  CPALS_CUDA_TRY(cudaGetLastError());
  CPALS_CUDA_TRY(cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned) * kMaxBatchClasses, b->st));
  b->launches += 1;
  return CPALS_OK;
}

int cpals_batch_get_factors(cpals_batch* b, double* host_concat) {
  if (!b || !host_concat) return CPALS_E_ARG;
  DeviceGuard guard(b->device);
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_concat, b->d_F, sizeof(double) * b->tot_F, cudaMemcpyDeviceToHost, b->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(b->st));
  return CPALS_OK;
}

int cpals_batch_set_sweeps_per_launch(cpals_batch* b, int k) {
  if (!b || k < 0) return CPALS_E_ARG;
  b->sweeps_per_launch = k;
  return CPALS_OK;
}

int cpals_batch_set_threads(cpals_batch* b, int threads) {
  if (!b || (threads != 128 && threads != 256 && threads != 512)) return CPALS_E_ARG;
  DeviceGuard guard(b->device);
  return set_config(b, threads);
}

int cpals_batch_optimize(cpals_batch* b, double tol, int max_iter, int* sweeps_out, double* fits_out,
                         int* flags_out, int64_t* launches_out) {
  if (!b || max_iter < 1 || !(tol >= 0.0)) return CPALS_E_ARG;
  DeviceGuard guard(b->device);
  b->tol = tol;
  b->max_iter = max_iter;
  // By default one launch runs every tensor to its own stop: a CTA sweeps the tensor it pulls
  // until that tensor's check stops it.  Each tensor's sweeps and check are its own, so this
  // gives the results of one launch per sweep; launches of one sweep each would last as long
  // as the slowest active tensor's sweep, with most SMs idle once most tensors have stopped.
  // With sweeps_per_launch = k >= 1, k sweeps per launch and the active count polled between.
  const int spl = b->sweeps_per_launch > 0 ? std::min(b->sweeps_per_launch, max_iter) : max_iter;
  *b->h_run = BatchRun{tol, max_iter, spl};
  CPALS_CUDA_TRY(cudaMemcpyAsync(b->d_run, b->h_run, sizeof(BatchRun), cudaMemcpyHostToDevice, b->st));
  if (!b->graph) {
    int rc = build_graph(b);
    if (rc != CPALS_OK) return rc;
  }
  int launched = 0, batch = (spl == max_iter) ? 1 : 4;
  const int64_t l0 = b->launches;
  while (launched < max_iter) {
    const int n = std::min(batch, (max_iter - launched + spl - 1) / spl);
    for (int k = 0; k < n; ++k) CPALS_CUDA_TRY(cudaGraphLaunch(b->graph, b->st));
    b->launches += (int64_t)(b->cls.size() + 1) * n;
    launched += n * spl;
    CPALS_CUDA_TRY(cudaMemcpyAsync(b->h_active, b->d_active, sizeof(int), cudaMemcpyDeviceToHost, b->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(b->st));
    if (*b->h_active == 0) break;
    batch = std::min(batch * 2, 32);
  }
  if (b->h_run->sweeps_per_pull != 1) {  // one sweep per pull again (the autotuner's launches)
    b->h_run->sweeps_per_pull = 1;
    CPALS_CUDA_TRY(cudaMemcpyAsync(b->d_run, b->h_run, sizeof(BatchRun), cudaMemcpyHostToDevice, b->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(b->st));
  }
  std::vector<BatchCheck> h(b->count);
  CPALS_CUDA_TRY(cudaMemcpy(h.data(), b->d_chk, sizeof(BatchCheck) * b->count, cudaMemcpyDeviceToHost));
  int nan_any = 0;
  for (int64_t t = 0; t < b->count; ++t) {
    if (sweeps_out) sweeps_out[t] = h[t].sweeps;
    if (fits_out) fits_out[t] = h[t].done ? h[t].final_fit : h[t].fit;
    if (flags_out) flags_out[t] = (h[t].nan ? 1 : 0) | (h[t].rank_deficient ? 2 : 0) | (h[t].done ? 4 : 0);
    nan_any |= h[t].nan;
  }
  if (launches_out) *launches_out = b->launches - l0;
  return CPALS_OK;
}

// Autotuner.  Schedules tried, each timed over `sweeps` sweeps from host_factors (restored
// after every trial):
//   - one class (every tensor, the batch-wide layout) with 128, 256 and 512 threads per CTA;
//   - the split by CTAs per SM: each class's thread count chosen by timing the class alone,
//     then the classes together, concurrently on their own streams.
// The fastest schedule is kept.  ms_out (3 entries, may be null): the one-class trials.
int cpals_batch_autotune(cpals_batch* b, const double* host_factors, int sweeps, int* threads_out,
                         double* ms_out) {
  if (!b || !host_factors || sweeps < 1) return CPALS_E_ARG;
  DeviceGuard guard(b->device);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto timed = [&](float* ms) -> int {  // `sweeps` sweeps under the current schedule
    int rc = cpals_batch_set_factors(b, host_factors);
    if (rc != CPALS_OK) return rc;
    cudaEventRecord(e0, b->st);
    for (int s2 = 0; s2 < sweeps; ++s2) {
      rc = batch_launch(b);
      if (rc != CPALS_OK) return rc;
    }
    cudaEventRecord(e1, b->st);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    return CPALS_OK;
  };
  const int cand[3] = {128, 256, 512};
  float best = 3.0e38f;
  int best_nt = 0;
  for (int i = 0; i < 3; ++i) {
    if (ms_out) ms_out[i] = -1.0;
    if (set_config(b, cand[i]) != CPALS_OK) continue;
    float ms = 0.f;
    int rc = timed(&ms);
    if (rc != CPALS_OK) return rc;
    if (ms_out) ms_out[i] = ms;
    if (ms < best) {
      best = ms;
      best_nt = cand[i];
    }
  }
  b->ms_split = -1.0;
  if (b->split.size() > 1) {
    std::vector<BatchClass> sp = b->split;
    bool ok = true;
    for (BatchClass& c : sp) {
      float cbest = 3.0e38f;
      int cnt = 0;
      for (int nt : cand) {
        BatchClass t = c;
        if (class_config(t, nt) != CPALS_OK) continue;
        t.st = b->st;  // alone, on the batch's stream
        if (use_schedule(b, {t}, b->order_split) != CPALS_OK) return CPALS_E_CUDA;
        float ms = 0.f;
        int rc = timed(&ms);
        if (rc != CPALS_OK) return rc;
        if (ms < cbest) {
          cbest = ms;
          cnt = nt;
        }
      }
      if (!cnt || class_config(c, cnt) != CPALS_OK) {
        ok = false;
        break;
      }
      c.ms_alone = cbest;
    }
    if (ok) {
      if (use_schedule(b, sp, b->order_split) != CPALS_OK) return CPALS_E_CUDA;
      float ms = 0.f;
      int rc = timed(&ms);
      if (rc != CPALS_OK) return rc;
      b->ms_split = ms;
      if (ms < best) {
        best = ms;
        best_nt = 0;  // the split schedule stays in place
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int rc = CPALS_OK;
  if (best_nt) {
    rc = set_config(b, best_nt);
  } else if (best > 2.9e38f) {
    return CPALS_E_UNSUPPORTED;
  }
  if (rc == CPALS_OK) rc = cpals_batch_set_factors(b, host_factors);
  if (threads_out) {
    int nt = 0;
    for (const BatchClass& c : b->cls) nt = std::max(nt, c.nt);
    *threads_out = nt;
  }
  return rc;
}

int cpals_batch_schedule(cpals_batch* b, int* nclass, int64_t* info, double* ms_split) {
  if (!b || !nclass) return CPALS_E_ARG;
  *nclass = (int)b->cls.size();
  if (info)
    for (size_t i = 0; i < b->cls.size(); ++i) {
      const BatchClass& c = b->cls[i];
      int64_t* r = info + 6 * i;
      r[0] = c.end - c.begin;
      r[1] = c.Imax;
      r[2] = c.Rmax;
      r[3] = c.nt;
      r[4] = c.ctas_per_sm;
      r[5] = (int64_t)(1000.0 * c.ms_alone);  // microseconds, 0 when not timed alone
    }
  if (ms_split) *ms_split = b->ms_split;
  return CPALS_OK;
}

}  // extern "C"
