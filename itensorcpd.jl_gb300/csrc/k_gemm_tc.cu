// tcgen05 BF16 GEMM for the warm-start network: part[s] = A B^T over one reduction slice.
//
// One CTA per (128-row block of A, 128-row block of B, reduction slice); 6 warps.
//   warp 0   producer: per 64-wide reduction step, two 16 KB cp.async.bulk copies (the A and
//            B panel tiles) into a 4-stage mbarrier ring;
//   warp 1   MMA issuer: four tcgen05.mma.kind::f16 (M = N = 128, K = 16) per stage into one
//            TMEM accumulator of 128 FP32 columns; tcgen05.commit releases the stage;
//   warps 2-5 epilogue: tcgen05.ld of their TMEM lane quarter, FP32 stores of the slice's
//            partial sums.
// The slices are summed in a fixed order by the epilogue kernel, which also applies the
// bias and the activation and writes the next GEMM's panels.  Every wait is bounded: on
// expiry the kernel sets err[0], waits (bounded) for its own copies and MMAs in flight,
// frees TMEM and returns without writing.
#include <algorithm>

#include "cpals_internal.cuh"
#include "gemm_tc.cuh"
#include "tc_ptx.cuh"

namespace cpals {
namespace {

constexpr int kGemmStages = 4;
constexpr uint32_t kTileBytes = kPanelRows * kPanelK * 2;  // 16 KB
constexpr int kGemmThreads = 192;
constexpr size_t kGemmSmem = 1024 + (size_t)kGemmStages * 2 * kTileBytes + 256;

struct GemmTcArgs {
  const uint8_t* a;
  const uint8_t* b;
  float* part;
  int M, N, KT, MT, NT, kps;
  int* err;
};

__global__ void __launch_bounds__(kGemmThreads, 1) k_gemm_tc(GemmTcArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)kGemmStages * 2 * kTileBytes);
  uint64_t* empty = full + kGemmStages;
  uint64_t* done_bar = empty + kGemmStages;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(done_bar + 1);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done_bar + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x % g.MT;
  const int nt = (blockIdx.x / g.MT) % g.NT;
  const int sp = blockIdx.x / (g.MT * g.NT);
  const int k0 = sp * g.kps;
  const int nk = max(0, min(g.KT, k0 + g.kps) - k0);
  volatile int* never = reinterpret_cast<volatile int*>(g.err + 1);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kGemmStages; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    mbar_init(smem_u32(done_bar), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(128)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  auto stage = [&](int s) { return smem + (size_t)s * 2 * kTileBytes; };

  if (warp == 0) {
    if (lane == 0) {
      const uint8_t* pa = g.a + ((size_t)mt * g.KT + k0) * kTileBytes;
      const uint8_t* pb = g.b + ((size_t)nt * g.KT + k0) * kTileBytes;
      int issued = 0;
      for (int it = 0; it < nk; ++it) {
        const int s = it % kGemmStages;
        if (!mbar_wait(smem_u32(&empty[s]), (uint32_t)(((it / kGemmStages) & 1) ^ 1), abort_flag)) {
          atomicCAS(g.err, 0, 1);
          *abort_flag = 1;
          break;
        }
        const uint32_t bar = smem_u32(&full[s]);
        mbar_expect_tx(bar, 2 * kTileBytes);
        bulk_load(smem_u32(stage(s)), pa + (size_t)it * kTileBytes, kTileBytes, bar);
        bulk_load(smem_u32(stage(s) + kTileBytes), pb + (size_t)it * kTileBytes, kTileBytes, bar);
        issued = it + 1;
      }
      if (*abort_flag)  // this CTA's copies in flight land before the shared memory goes away
        for (int it = max(0, issued - kGemmStages); it < issued; ++it)
          (void)mbar_wait(smem_u32(&full[it % kGemmStages]), (uint32_t)((it / kGemmStages) & 1), never);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(kPanelRows, kPanelRows);
      for (int it = 0; it < nk && !*abort_flag; ++it) {
        const int s = it % kGemmStages;
        if (!mbar_wait(smem_u32(&full[s]), (uint32_t)((it / kGemmStages) & 1), abort_flag)) {
          atomicCAS(g.err, 0, 2);
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t sa = smem_u32(stage(s)), sb = sa + kTileBytes;
#pragma unroll
        for (int kk = 0; kk < kPanelK / 16; ++kk)
          umma_bf16(tmem, sw128_desc(sa + kk * 32), sw128_desc(sb + kk * 32), idesc, (it > 0 || kk > 0) ? 1u : 0u);
        umma_commit(smem_u32(&empty[s]));  // the stage is free once these MMAs have read it
      }
      umma_commit(smem_u32(done_bar));
      (void)mbar_wait(smem_u32(done_bar), 0u, never);  // every MMA issued here has finished
    }
  } else {
    const int q = warp & 3;  // TMEM lane quarter of this warp
    int ok = 0;
    if (lane == 0) ok = (nk > 0 && mbar_wait(smem_u32(done_bar), 0u, abort_flag)) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (ok) {
      tc_fence_after();
      const int64_t row = (int64_t)mt * kPanelRows + q * 32 + lane;
      const int n0 = nt * kPanelRows;
      float* out = g.part + ((int64_t)sp * g.M + row) * g.N;
#pragma unroll 1
      for (int c0 = 0; c0 < kPanelRows; c0 += 32) {
        uint32_t v[32];
        tmem_ld32_nowait(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
        tmem_wait_ld();
        if (row < g.M) {
          const int n = n0 + c0;
          if (n + 32 <= g.N && (g.N & 3) == 0) {
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              *reinterpret_cast<float4*>(out + n + j) = make_float4(__uint_as_float(v[j]), __uint_as_float(v[j + 1]),
                                                                    __uint_as_float(v[j + 2]), __uint_as_float(v[j + 3]));
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (n + j < g.N) out[n + j] = __uint_as_float(v[j]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
  }
}

__device__ __forceinline__ int64_t panel_index(int64_t row, int64_t k, int64_t KT) {
  const int64_t tile = (row >> 7) * KT + (k >> 6);
  const int r = (int)(row & 127), kk = (int)(k & 63);
  return tile * (kPanelRows * kPanelK) + r * kPanelK + ((((kk >> 3) ^ (r & 7))) << 3) + (kk & 7);
}

// Sum of the slices, bias, activation; FP32 and panel outputs over the padded domain
// [0, ceil64(M)) x [0, ceil64(N)) so that the panels' reduction padding is written as zero.
__global__ void k_gemm_epilogue(const float* __restrict__ part, int splits, int M, int N, const float* __restrict__ bias,
                                int mode, const float* __restrict__ mask, float* __restrict__ out32,
                                __nv_bfloat16* __restrict__ prm, __nv_bfloat16* __restrict__ ptr) {
  const int Mp = (prm || ptr) ? ((M + kPanelK - 1) / kPanelK) * kPanelK : M;
  const int Np = (prm || ptr) ? ((N + kPanelK - 1) / kPanelK) * kPanelK : N;
  const int64_t KTm = (N + kPanelK - 1) / kPanelK;  // prm: M rows, K = N
  const int64_t KTt = (M + kPanelK - 1) / kPanelK;  // ptr: N rows, K = M
  const int64_t total = (int64_t)Mp * Np;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(e / Np), n = (int)(e % Np);
    float v = 0.f;
    const bool in = m < M && n < N;
    if (in) {
      const int64_t o = (int64_t)m * N + n;
      for (int s = 0; s < splits; ++s) v += part[(int64_t)s * M * N + o];
      if (bias) v += bias[n];
      if (mode == 1) v = fmaxf(v, 0.f);
      if (mode == 2 && !(__bfloat162float(__float2bfloat16_rn(mask[o])) > 0.f)) v = 0.f;
      if (out32) out32[o] = v;
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    if (prm && m < M) prm[panel_index(m, n, KTm)] = h;  // rows past M are never read into an output
    if (ptr && n < N) ptr[panel_index(n, m, KTt)] = h;
  }
}

}  // namespace

cudaError_t gemm_tc_prepare() {
  return set_smem_limit_once(reinterpret_cast<const void*>(k_gemm_tc), (int)kGemmSmem);
}

int gemm_tc_splits(int M, int N, int K, int sms) {
  const int MT = (M + kPanelRows - 1) / kPanelRows, NT = (N + kPanelRows - 1) / kPanelRows;
  const int KT = (K + kPanelK - 1) / kPanelK;
  const int tiles = MT * NT;
  if (tiles >= sms || KT < 8) return 1;
  int s = std::min((sms + tiles - 1) / tiles, KT / 4);  // fill the SMs, at least 4 steps a slice
  s = std::max(s, 1);
  const int kps = (KT + s - 1) / s;
  return (KT + kps - 1) / kps;
}

cudaError_t gemm_tc_launch(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, int splits,
                           float* part, int* err, cudaStream_t st) {
  if (M < 1 || N < 1 || K < 1 || splits < 1) return cudaErrorInvalidValue;
  cudaError_t e = set_smem_limit_once(reinterpret_cast<const void*>(k_gemm_tc), (int)kGemmSmem);
  if (e != cudaSuccess) return e;
  GemmTcArgs g;
  g.a = reinterpret_cast<const uint8_t*>(A);
  g.b = reinterpret_cast<const uint8_t*>(B);
  g.part = part;
  g.M = M;
  g.N = N;
  g.KT = (K + kPanelK - 1) / kPanelK;
  g.MT = (M + kPanelRows - 1) / kPanelRows;
  g.NT = (N + kPanelRows - 1) / kPanelRows;
  g.kps = (g.KT + splits - 1) / splits;
  if ((g.KT + g.kps - 1) / g.kps != splits) return cudaErrorInvalidValue;  // every slice non-empty
  g.err = err;
  const int grid = g.MT * g.NT * splits;
  k_gemm_tc<<<grid, kGemmThreads, kGemmSmem, st>>>(g);
  return cudaGetLastError();
}

cudaError_t gemm_tc_epilogue(const float* part, int splits, int M, int N, const float* bias, int mode,
                             const float* mask, float* out32, __nv_bfloat16* prm, __nv_bfloat16* ptr, cudaStream_t st) {
  const int64_t Mp = ((M + kPanelK - 1) / kPanelK) * kPanelK, Np = ((N + kPanelK - 1) / kPanelK) * kPanelK;
  const int blocks = (int)std::min<int64_t>((Mp * Np + 255) / 256, 4096);
  k_gemm_epilogue<<<blocks, 256, 0, st>>>(part, splits, M, N, bias, mode, mask, out32, prm, ptr);
  return cudaGetLastError();
}

}  // namespace cpals
