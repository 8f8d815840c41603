// tcgen05 split-BF16 MTTKRP for FP32 (or FP64) tensors on sm_103a.
//
// M_n(i, r) = sum_k T_(n)(i, k) KRP(k, r), the contraction that
// matricize_tensor(::KRPFreeNormal / ::KRPNormal) forms
// (src/algorithms/als_algorithms/standard/tensor.jl:12-44), computed as
//   T ~ Th + Tl,  KRP ~ Kh + Kl  (BF16 hi/lo, round to nearest),
//   M ~ Th Kh + Th Kl + Tl Kh   (three BF16 tensor-core products).
//
// Chunks.  The reduction index space (every mode but n) is cut into chunks of 64
// consecutive values of the fastest reduction mode f (f = 1 for mode 0, else 0) at
// fixed values of the other ("outer") reduction modes; inside a chunk
// KRP(k, r) = F_f(k, r) * s(r), s(r) = product of the outer modes' factor rows.
//
// Layout.  HBM bandwidth bounds this kernel, so at set-up every mode gets its own copy
// of the BF16 hi/lo unfolding as 32 KB tiles -- 128 rows x 64 reduction values, hi then
// lo, each already in the SWIZZLE_128B K-major arrangement the tensor core reads --
// stored in the order the CTAs consume them.  A stage is one contiguous 32 KB bulk copy
// and every CTA streams one contiguous region (4 bytes per element, the FP32 size).
//
// CTA (6 or 10 warps).  Warp 0 is the producer: per stage it issues cp.async.bulk copies
// into a 2-4 stage mbarrier ring -- the 32 KB unfolding tile (hi, lo), the FP32 rows of the
// outer factors and, unless every factor-block tile of the CTA's N block is resident in
// shared memory (loaded once, when four stages still fit beside them), the prebuilt BF16
// hi/lo factor-block tile of F_f[k0:k0+64, n0:n0+NB] (written by k_build_btiles, or by the
// normalisation when the factor is updated in a sweep).  Warp 1 issues
// tcgen05.mma.kind::f16 (M = 128, K = 16, four steps per chunk): one N = 2 NB product
// Th [Bh | Bl] and one N = NB product Tl Bh.  The tensor core's FP32 accumulation rounds
// toward zero, which over long chains shrinks the result (about 0.5 ulp per accumulation),
// so accumulation groups stay short: each group of chunks (one chunk, or two consecutive
// factor blocks of one outer index when NB = 128) accumulates into fresh TMEM accumulators
// (2 or 4 buffers).  The drain warps (4, or 8 when NB is a multiple of 64: one or two per
// TMEM lane quarter) form the group's outer-row scale s(r) into their own shared slice,
// release the group's stages, read the accumulators with tcgen05.ld and accumulate
// s(r) (hi + cross terms) in FP32 registers with round-to-nearest adds.  The reduction
// range is split across CTAs; each writes FP32 partials part[split][I_n][R], reduced by the
// solve.  Every wait is bounded: on expiry the kernel records an error code, drains its own
// copies in flight (bounded), frees TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "cpals_tc.cuh"
#include "tc_ptx.cuh"

namespace cpals {

namespace {

constexpr int kChunk = 64;     // K values per stage (one 128-byte swizzle row of BF16)
constexpr int kBlockM = 128;   // rows per CTA (one UMMA M)
// Drain warps: one per TMEM lane quarter, or two (each taking half of the columns) when
// the N block is a multiple of 64 wide, which halves the per-chunk drain latency and the
// accumulator registers of the wide blocks.  Warps 0 and 1 produce and issue the MMAs.
template <int NB>
__host__ __device__ constexpr int tc_drain_warps() { return (NB % 64 == 0) ? 8 : 4; }
template <int NB>
__host__ __device__ constexpr int tc_threads() { return 64 + 32 * tc_drain_warps<NB>(); }
constexpr size_t kSmemLimit = 227 * 1024;

struct TcModePlan {
  int mode, fmode, n_outer, m_blocks, n_blocks, splits, stages, nb, tmem_cols, rpad;
  int64_t In, If, nfb, nchunks, chunks_per_split;
  int64_t sn, sf;              // element strides of mode n and of f in the tensor
  uint32_t stage_bytes;        // stride of the ring's stages
  // Resident factor-block tiles: all nfb B tiles of the CTA's N block are loaded once, at
  // bres_off, and a stage holds only the 32 KB unfolding tile; the outer rows then have their
  // own ring (obytes per stage, at orow_off).  ctl_off: barriers and flags.
  int bres;
  uint32_t bres_off, orow_off, obytes, ctl_off;
  // Chunks per accumulation group: consecutive factor blocks of one outer index accumulate in
  // the same TMEM buffer before one drain (1, or 2 for 128-wide N blocks).
  int grp;
  int64_t outer_dims[kMaxOrder];
  int64_t outer_stride[kMaxOrder];  // element stride of each outer mode in the tensor
  int outer_modes[kMaxOrder];
};

struct FactorPtrs32 {
  const float* F[kMaxOrder];  // row-major FP32 factor copies [I_m][rpad], zero-padded columns
};

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b, float* ra, float* rb) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  float2 f = __bfloat1622float2(h);
  *ra = a - f.x;
  *rb = b - f.y;
  return *reinterpret_cast<uint32_t*>(&h);
}

// ---------------------------------------------------------------- the kernel
template <int NBT>  // N-block width (a multiple of 16, at most 128): loops unroll exactly this far
__global__ void __launch_bounds__(tc_threads<NBT>(), 1)
    k_mttkrp_tc(const uint8_t* __restrict__ tiles, const uint8_t* __restrict__ btiles, TcModePlan p,
                FactorPtrs32 fr, int R, float* __restrict__ part, const DevCheck* __restrict__ chk,
                int* __restrict__ err) {
  if (chk && chk->done) return;
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte aligned tile region
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int S = p.stages;
  constexpr int NB = NBT;
  // Per chunk buffer: hi*hi in columns [0, NB), the small cross terms hi*lo + lo*hi in
  // [NB, 2NB).  Four buffers (when TMEM has room) let the MMAs run four chunks ahead of
  // the drain.
  constexpr int kAcc = 2;
  constexpr int kBuf = (2 * kAcc * NB <= 256) ? 4 : 2;
  constexpr uint32_t a_bytes = kBlockM * kChunk * 2;  // 16 KB: one BF16 tile (hi or lo)
  constexpr uint32_t b_bytes = NB * kChunk * 2;       // one BF16 factor-block tile (hi or lo)
  constexpr uint32_t o_bytes = NB * 4;                // one outer factor row slice
  const uint32_t stage_bytes = p.stage_bytes;
  const bool bres = p.bres != 0;
  uint8_t* ctl = smem + p.ctl_off;
  uint64_t* full_a = reinterpret_cast<uint64_t*>(ctl);  // [4] stage data landed
  uint64_t* empty = full_a + 4;                          // [4] stage consumed (MMAs done, rows read)
  uint64_t* acc_full = empty + 4;                        // [4] chunk accumulators ready
  uint64_t* acc_empty = acc_full + 4;                    // [4] chunk accumulators drained
  uint64_t* done_bar = acc_empty + 4;
  uint64_t* bres_bar = done_bar + 1;                     // resident B tiles landed
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bres_bar + 1);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bres_bar + 2);
  // where stage s keeps its unfolding tile, the B tile of chunk fb, and its outer rows
  auto stage_a = [&](int s) { return smem + (size_t)s * stage_bytes; };
  auto b_tile = [&](int s, int64_t fb) {
    return bres ? smem + p.bres_off + (size_t)fb * (2 * b_bytes) : stage_a(s) + 2 * a_bytes;
  };
  auto outer_rows = [&](int s) {
    return bres ? smem + p.orow_off + (size_t)s * p.obytes : stage_a(s) + 2 * a_bytes + 2 * b_bytes;
  };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mblk = blockIdx.x % p.m_blocks;
  const int nblk = (blockIdx.x / p.m_blocks) % p.n_blocks;
  const int split = blockIdx.x / (p.m_blocks * p.n_blocks);
  const int n0 = nblk * NB;
  const int64_t c_begin = (int64_t)split * p.chunks_per_split;
  const int64_t c_end = min(p.nchunks, c_begin + p.chunks_per_split);
  const int nloc = (c_end > c_begin) ? (int)(c_end - c_begin) : 0;
  const int nfb = (int)p.nfb;  // factor blocks of the fastest reduction mode (a few)

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(smem_u32(&full_a[s]), 1);
      mbar_init(smem_u32(&empty[s]), tc_drain_warps<NB>());
    }
    for (int b = 0; b < kBuf; ++b) {
      mbar_init(smem_u32(&acc_full[b]), 1);
      mbar_init(smem_u32(&acc_empty[b]), tc_drain_warps<NB>());
    }
    mbar_init(smem_u32(done_bar), 1);
    mbar_init(smem_u32(bres_bar), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(p.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- producer: unfolding tile, factor-block tile, outer rows
    if (lane == 0) {
      int issued = 0;
      const uint32_t tx = 2 * a_bytes + (bres ? 0u : 2 * b_bytes) + (uint32_t)p.n_outer * o_bytes;
      const uint8_t* src_tiles = tiles + ((size_t)mblk * p.nchunks + c_begin) * (2 * a_bytes);
      if (bres && nloc > 0) {  // every B tile of this N block, once
        const uint32_t bar = smem_u32(bres_bar);
        mbar_expect_tx(bar, (uint32_t)p.nfb * 2 * b_bytes);
        for (int64_t fb = 0; fb < p.nfb; ++fb)
          bulk_load(smem_u32(b_tile(0, fb)), btiles + ((size_t)fb * p.n_blocks + nblk) * (2 * b_bytes), 2 * b_bytes,
                    bar);
      }
      for (int it = 0; it < nloc; ++it) {
        const int s = it % S;
        const uint32_t ph = (uint32_t)((it / S) & 1);
        if (!mbar_wait(smem_u32(&empty[s]), ph ^ 1u, abort_flag)) {
          atomicCAS(err, 0, 1);
          *abort_flag = 1;
          break;
        }
        const int64_t c = c_begin + it;
        const int64_t fb = c % p.nfb;
        int64_t o = c / p.nfb;
        uint8_t* st = stage_a(s);
        const uint32_t bar = smem_u32(&full_a[s]);
        mbar_expect_tx(bar, tx);
        bulk_load(smem_u32(st), src_tiles + (size_t)it * (2 * a_bytes), 2 * a_bytes, bar);
        if (!bres)
          bulk_load(smem_u32(st + 2 * a_bytes), btiles + ((size_t)fb * p.n_blocks + nblk) * (2 * b_bytes),
                    2 * b_bytes, bar);
        uint8_t* orow = outer_rows(s);
        for (int j = 0; j < p.n_outer; ++j) {
          const int64_t id = o % p.outer_dims[j];
          o /= p.outer_dims[j];
          const float* src = fr.F[p.outer_modes[j]] + id * p.rpad + n0;
          bulk_load(smem_u32(orow + j * o_bytes), src, o_bytes, bar);
        }
        issued = it + 1;
      }
      if (*abort_flag) {
        // drain this CTA's own copies in flight before the shared memory goes away
        for (int it = max(0, issued - S); it < issued; ++it)
          (void)mbar_wait(smem_u32(&full_a[it % S]), (uint32_t)((it / S) & 1), reinterpret_cast<volatile int*>(err + 1));
        if (bres && nloc > 0) (void)mbar_wait(smem_u32(bres_bar), 0u, reinterpret_cast<volatile int*>(err + 1));
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer: per accumulation group g (p.grp chunks of one outer index),
    // fresh accumulators in buffer b = g % kBuf.
    // B = [Bh; Bl] stacked (2 NB rows): one N = 2 NB product gives Th Bh and Th Bl
    // together, a second N = NB product adds Tl Bh onto the cross terms.
    if (lane == 0) {
      const uint32_t idesc_w = idesc_bf16(kBlockM, 2 * NB), idesc_n = idesc_bf16(kBlockM, NB);
      if (bres && nloc > 0 && !mbar_wait(smem_u32(bres_bar), 0u, abort_flag)) {
        atomicCAS(err, 0, 2);
        *abort_flag = 1;
      }
      int fbm = (int)(c_begin % p.nfb);  // the chunk's factor block, kept without a division per chunk
      int g = 0;     // accumulation group
      int gpos = 0;  // position of the chunk in its group
      for (int it = 0; it < nloc && !*abort_flag; ++it, fbm = (fbm + 1 == nfb) ? 0 : fbm + 1) {
        const int s = it % S;
        const uint32_t ph = (uint32_t)((it / S) & 1);
        const int b = g % kBuf;
        const uint32_t uph = (uint32_t)((g / kBuf) & 1);
        const bool first = gpos == 0;
        const bool last = (it + 1 == nloc) || (gpos + 1 == p.grp) || (fbm + 1 == nfb);
        if (!mbar_wait(smem_u32(&full_a[s]), ph, abort_flag) ||
            (first && !mbar_wait(smem_u32(&acc_empty[b]), uph ^ 1u, abort_flag))) {
          atomicCAS(err, 0, 2);
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t ah = smem_u32(stage_a(s)), al = ah + a_bytes;
        const uint32_t bh = smem_u32(b_tile(s, fbm));
        const uint32_t acc_h = tmem + (uint32_t)(b * kAcc * NB), acc_l = acc_h + (uint32_t)NB;
#pragma unroll
        for (int kk = 0; kk < kChunk / 16; ++kk) {
          const uint32_t off = kk * 32;
          const uint64_t dah = sw128_desc(ah + off), dal = sw128_desc(al + off), dbh = sw128_desc(bh + off);
          umma_bf16(acc_h, dah, dbh, idesc_w, (first && kk == 0) ? 0u : 1u);  // [Th Bh | Th Bl]
          umma_bf16(acc_l, dal, dbh, idesc_n, 1u);                           // += Tl Bh
        }
        if (last) {
          umma_commit(smem_u32(&acc_full[b]));
          ++g;
        }
        gpos = last ? 0 : gpos + 1;
      }
      umma_commit(smem_u32(done_bar));
    }
  } else {
    // ---------------- drainers (warps 2..): per chunk, acc[r] += s(r) * (Th Kh + cross terms),
    // promoted from TMEM into FP32 registers with round-to-nearest adds.  Warp w reads TMEM
    // lane quarter w % 4 and, with two warps per quarter, half of the columns.
    constexpr int NH = NB * 4 / tc_drain_warps<NB>();  // columns of this warp
    const int q = warp & 3;  // this warp's TMEM lane quarter
    const int cb = ((warp - 2) >> 2) * NH;  // first column of this warp
    const int64_t row = (int64_t)mblk * kBlockM + q * 32 + lane;
    float* sw = reinterpret_cast<float*>(ctl + 256) + (warp - 2) * NH;  // this warp's scale slice
    float acc[NH];
#pragma unroll
    for (int j = 0; j < NH; ++j) acc[j] = 0.0f;
    bool ok = true;
    int fbm = (int)(c_begin % p.nfb);
    int g = 0, it0 = 0;  // accumulation group and its first chunk
    for (int it = 0; it < nloc && ok; ++it, fbm = (fbm + 1 == nfb) ? 0 : fbm + 1) {
      // the issuer's grouping: p.grp chunks, cut where the outer index changes
      if (!((it + 1 == nloc) || (it + 1 - it0 == p.grp) || (fbm + 1 == nfb))) continue;
      const int s = it % S;
      const int b = g % kBuf;
      const uint32_t uph = (uint32_t)((g / kBuf) & 1);
      int got = 0;
      if (lane == 0) got = mbar_wait(smem_u32(&acc_full[b]), uph, abort_flag) ? 1 : 0;
      got = __shfl_sync(0xffffffffu, got, 0);
      if (!got) {
        if (lane == 0) {
          atomicCAS(err, 0, 4);
          *abort_flag = 1;
        }
        ok = false;
        break;
      }
      tc_fence_after();
      // s(r), the product of the outer factor rows in mode order (one outer index per group),
      // for this warp's columns into its own shared slice, two columns per lane; then every
      // stage of the group is free: its MMAs have completed and its outer rows are read
      {
        const float* orow = reinterpret_cast<const float*>(outer_rows(s)) + cb;
        for (int j = lane; j < NH; j += 32) {
          float v = 1.0f;
          for (int jo = 0; jo < p.n_outer; ++jo) v *= orow[jo * NB + j];
          sw[j] = v;
        }
        __syncwarp();
        if (lane == 0)
          for (int j = it0; j <= it; ++j) mbar_arrive(smem_u32(&empty[j % S]));
      }
      const uint32_t base = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * kAcc * NB + cb);
      // 32 columns per TMEM load, or 16 with two drain warps per quarter (their register
      // budget is smaller: 320 threads)
      constexpr int W = (tc_drain_warps<NB>() == 8) ? 16 : 32;
#pragma unroll
      for (int c0 = 0; c0 < NH; c0 += W) {
        uint32_t vh[W], vl[W];
        const bool full = (W == 32) && (c0 + 32 <= NH);
        if (full) {
          tmem_ld32_nowait(base + (uint32_t)c0, vh);
          tmem_ld32_nowait(base + (uint32_t)(NB + c0), vl);
        } else {
          tmem_ld16_nowait(base + (uint32_t)c0, vh);
          tmem_ld16_nowait(base + (uint32_t)(NB + c0), vl);
        }
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < W; j += 4) {
          if (c0 + j < NH) {
            const float4 v4 = *reinterpret_cast<const float4*>(sw + c0 + j);  // broadcast read
            acc[c0 + j] = fmaf(v4.x, __uint_as_float(vh[j]) + __uint_as_float(vl[j]), acc[c0 + j]);
            acc[c0 + j + 1] = fmaf(v4.y, __uint_as_float(vh[j + 1]) + __uint_as_float(vl[j + 1]), acc[c0 + j + 1]);
            acc[c0 + j + 2] = fmaf(v4.z, __uint_as_float(vh[j + 2]) + __uint_as_float(vl[j + 2]), acc[c0 + j + 2]);
            acc[c0 + j + 3] = fmaf(v4.w, __uint_as_float(vh[j + 3]) + __uint_as_float(vl[j + 3]), acc[c0 + j + 3]);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&acc_empty[b]));
      ++g;
      it0 = it + 1;
    }
    if (nloc > 0 && ok) {
      int got = 0;
      if (lane == 0) got = mbar_wait(smem_u32(done_bar), 0u, abort_flag) ? 1 : 0;
      got = __shfl_sync(0xffffffffu, got, 0);
      ok = got != 0;
    }
    if (row < p.In && (ok || nloc == 0)) {
      float* out = part + ((int64_t)split * p.In + row) * R + n0 + cb;
#pragma unroll
      for (int j = 0; j < NH; ++j)
        if (n0 + cb + j < R) out[j] = acc[j];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.tmem_cols) : "memory");
  }
}

// ---------------------------------------------------------------- factor-block tiles
// For the fastest reduction mode f: per (f-block fb, N block), the NB x 64 block
// F_f[fb*64 : fb*64+64, n0 : n0+NB]^T split into BF16 hi / lo (from FP64, round to
// nearest), K-major and pre-swizzled, zero outside the factor.
__global__ void k_build_btiles(const double* __restrict__ F, int64_t If, int R, int64_t nfb, int n_blocks, int nb,
                               uint8_t* __restrict__ bt, const DevCheck* chk) {
  if (chk && chk->done) return;
  const int64_t units = nfb * n_blocks * nb * 8;  // 16-byte chunks per plane
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < units; u += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(u & 7);
    const int64_t rowg = u >> 3;  // (fb * n_blocks + nblk) * nb + r
    const int r = (int)(rowg % nb);
    const int64_t tile = rowg / nb;
    const int nblk = (int)(tile % n_blocks);
    const int64_t fb = tile / n_blocks;
    const int col = nblk * nb + r;
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      double x[2];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int64_t k = fb * kChunk + c * 8 + 2 * t + e;
        x[e] = (col < R && k < If) ? F[k * R + col] : 0.0;
      }
      __nv_bfloat162 h = __halves2bfloat162(__double2bfloat16(x[0]), __double2bfloat16(x[1]));
      __nv_bfloat162 l = __halves2bfloat162(__double2bfloat16(x[0] - (double)__bfloat162float(h.x)),
                                            __double2bfloat16(x[1] - (double)__bfloat162float(h.y)));
      hw[t] = *reinterpret_cast<uint32_t*>(&h);
      lw[t] = *reinterpret_cast<uint32_t*>(&l);
    }
    uint8_t* out = bt + (size_t)tile * (2 * (size_t)nb * kChunk * 2);
    const uint32_t off = (uint32_t)r * 128u + ((uint32_t)(c ^ (r & 7)) << 4);
    *reinterpret_cast<uint4*>(out + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *reinterpret_cast<uint4*>(out + (size_t)nb * kChunk * 2 + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
}

// ---------------------------------------------------------------- set-up: the tile stream
// One CTA per 32 KB tile (m-block, chunk): gathers the 128 x 64 block of the unfolding
// (zero outside the tensor), splits it into BF16 hi/lo and writes it pre-swizzled.
template <typename TT>
__global__ void __launch_bounds__(256) k_build_tiles(const TT* __restrict__ T, TcModePlan p, uint8_t* __restrict__ tiles) {
  __shared__ float fb_s[kBlockM][kChunk + 1];
  const int64_t tile = blockIdx.x;
  const int64_t mblk = tile / p.nchunks, c = tile % p.nchunks;
  const int64_t fb = c % p.nfb;
  int64_t o = c / p.nfb;
  int64_t base = fb * kChunk * p.sf;
  for (int j = 0; j < p.n_outer; ++j) {
    const int64_t id = o % p.outer_dims[j];
    o /= p.outer_dims[j];
    base += id * p.outer_stride[j];
  }
  const int tid = threadIdx.x;
  for (int e = tid; e < kBlockM * kChunk; e += 256) {
    int r, k;
    if (p.sf == 1) {
      r = e / kChunk;
      k = e % kChunk;
    } else {
      k = e / kBlockM;
      r = e % kBlockM;
    }
    const int64_t i = mblk * kBlockM + r, kf = fb * kChunk + k;
    float v = 0.0f;
    if (i < p.In && kf < p.If) v = (float)T[base + i * p.sn + (int64_t)k * p.sf];
    fb_s[r][k] = v;
  }
  __syncthreads();
  uint8_t* out = tiles + (size_t)tile * (2 * kBlockM * kChunk * 2);
  for (int u = tid; u < kBlockM * 8; u += 256) {
    const int r = u >> 3, cc = u & 7;
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const float x0 = fb_s[r][cc * 8 + 2 * t], x1 = fb_s[r][cc * 8 + 2 * t + 1];
      float r0, r1, d0, d1;
      hw[t] = pack_bf16x2(x0, x1, &r0, &r1);
      lw[t] = pack_bf16x2(r0, r1, &d0, &d1);
    }
    const uint32_t off = (uint32_t)r * 128u + ((uint32_t)(cc ^ (r & 7)) << 4);
    *reinterpret_cast<uint4*>(out + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *reinterpret_cast<uint4*>(out + kBlockM * kChunk * 2 + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
}

int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

}  // namespace

struct TcState {
  int order = 0, tdtype = 0, num_sms = 0;
  int64_t R = 0, rpad = 0;
  int64_t dims[kMaxOrder] = {};
  uint8_t* tiles[kMaxOrder] = {};  // per-mode tile streams
  size_t tile_bytes[kMaxOrder] = {};
  TcModePlan plan[kMaxOrder];
  uint8_t* btiles[2] = {};  // BF16 hi/lo factor-block tiles of modes 0 and 1 (the fastest reduction modes)
  size_t btile_bytes[2] = {};
  int64_t nfb_mode[2] = {};
  bool factors_bound = false;
  const float* F32r[kMaxOrder] = {};
  int* err = nullptr;  // [2]: error code, spare (never set: bounded drain flag)
  size_t smem_bytes[kMaxOrder] = {};
  bool shared = false;          // one buffer for every mode's stream, built per MTTKRP
  uint8_t* shared_buf = nullptr;
  const void* T = nullptr;      // the tensor the shared buffer's streams are built from
};

int tc_create(TcState** out, int order, const int64_t* dims, int64_t R, int tdtype, int num_sms, unsigned mode_mask,
              bool shared) {
  *out = nullptr;
  if (R > 512) return CPALS_E_UNSUPPORTED;
  TcState* s = new TcState();
  s->shared = shared;
  s->order = order;
  s->tdtype = tdtype;
  s->num_sms = num_sms;
  s->R = R;
  for (int m = 0; m < order; ++m) s->dims[m] = dims[m];
  // N blocks of at most 128 columns (a multiple of 16 each)
  const int64_t rp16 = round_up(R, 16);
  const int n_blocks = (int)((rp16 + 127) / 128);
  const int nb = (int)round_up((rp16 + n_blocks - 1) / n_blocks, 16);
  s->rpad = (int64_t)nb * n_blocks;
  int tcols = 32;
  const int kacc = 2;                             // accumulators per chunk buffer (see the kernel)
  const int kbuf = (2 * kacc * nb <= 256) ? 4 : 2;  // chunk buffers (see the kernel)
  while (tcols < kbuf * kacc * nb) tcols *= 2;
  const int usable = std::max(1, num_sms - 1);  // one SM stays free for the side-stream factorisation
  if (cudaMalloc(&s->err, 2 * sizeof(int)) != cudaSuccess) {
    tc_destroy(s);
    return CPALS_E_CUDA;
  }
  cudaMemset(s->err, 0, 2 * sizeof(int));
  int64_t strides[kMaxOrder];
  {
    int64_t st = 1;
    for (int m = 0; m < order; ++m) {
      strides[m] = st;
      st *= dims[m];
    }
  }
  for (int n = 0; n < order; ++n) {
    TcModePlan& p = s->plan[n];
    memset(&p, 0, sizeof(p));
    if (!((mode_mask >> n) & 1u)) continue;  // no tile stream for this mode
    p.mode = n;
    p.fmode = (n == 0) ? 1 : 0;
    p.In = dims[n];
    p.If = dims[p.fmode];
    p.sn = strides[n];
    p.sf = strides[p.fmode];
    p.nb = nb;
    p.n_blocks = n_blocks;
    p.rpad = (int)s->rpad;
    p.tmem_cols = tcols;
    p.nfb = (p.If + kChunk - 1) / kChunk;
    p.grp = (nb == 128) ? 2 : 1;
    int64_t outer = 1;
    for (int m = 0; m < order; ++m) {
      if (m == n || m == p.fmode) continue;
      p.outer_modes[p.n_outer] = m;
      p.outer_dims[p.n_outer] = dims[m];
      p.outer_stride[p.n_outer] = strides[m];
      ++p.n_outer;
      outer *= dims[m];
    }
    p.nchunks = p.nfb * outer;
    p.m_blocks = (int)((p.In + kBlockM - 1) / kBlockM);
    int64_t splits = std::max<int64_t>(1, usable / (p.m_blocks * p.n_blocks));
    splits = std::min<int64_t>(splits, p.nchunks);
    p.chunks_per_split = (p.nchunks + splits - 1) / splits;
    p.splits = (int)((p.nchunks + p.chunks_per_split - 1) / p.chunks_per_split);
    // Resident B tiles (all nfb of them, loaded once) when they leave room for four 32 KB
    // unfolding stages: a stage then streams 32 KB instead of 32 KB + the B tile.  With fewer
    // stages the unfolding bytes in flight drop, and the kernel is bound by them (at 512^3
    // R = 64, resident tiles with three stages took 120 us a launch against 110 us with four
    // stages of A + B).  Otherwise each stage is A hi | A lo | B hi | B lo | outer rows.
    const size_t ctl_bytes = 1024 + 256 + 16 * (size_t)nb;  // alignment slack, barriers and flags, drain scales
    const size_t a2 = (size_t)2 * kBlockM * kChunk * 2;
    const size_t b2 = (size_t)2 * nb * kChunk * 2;
    const size_t ob = (size_t)round_up((int64_t)p.n_outer * nb * 4, 16);
    const size_t bres_bytes = (size_t)p.nfb * b2;
    const size_t room = (kSmemLimit > ctl_bytes + bres_bytes + 4 * ob) ? kSmemLimit - ctl_bytes - bres_bytes - 4 * ob : 0;
    const int res_stages = (int)std::min<size_t>(4, room / a2);
    if (res_stages >= 4) {
      p.bres = 1;
      p.stages = res_stages;
      p.stage_bytes = (uint32_t)a2;
      p.bres_off = (uint32_t)(p.stages * a2);
      p.orow_off = p.bres_off + (uint32_t)bres_bytes;
      p.obytes = (uint32_t)ob;
      p.ctl_off = p.orow_off + (uint32_t)(p.stages * ob);
    } else {
      const size_t sb = a2 + b2 + (size_t)p.n_outer * nb * 4;
      p.bres = 0;
      p.stage_bytes = (uint32_t)round_up((int64_t)sb, 1024);
      p.stages = (int)std::min<size_t>(4, (kSmemLimit - ctl_bytes) / p.stage_bytes);
      p.ctl_off = (uint32_t)(p.stages * (size_t)p.stage_bytes);
    }
    if (p.stages < 2 || p.nchunks >= (int64_t(1) << 31)) {
      tc_destroy(s);
      return CPALS_E_UNSUPPORTED;
    }
    s->smem_bytes[n] = ctl_bytes + p.ctl_off;
    s->tile_bytes[n] = (size_t)p.m_blocks * p.nchunks * (2 * kBlockM * kChunk * 2);
    if (!shared && cudaMalloc(&s->tiles[n], s->tile_bytes[n]) != cudaSuccess) {
      tc_destroy(s);
      return CPALS_E_CUDA;
    }
  }
  if (shared) {
    size_t mx = 0;
    for (int n = 0; n < order; ++n) mx = std::max(mx, s->tile_bytes[n]);
    if (mx == 0 || cudaMalloc(&s->shared_buf, mx) != cudaSuccess) {
      tc_destroy(s);
      return mx == 0 ? CPALS_E_ARG : CPALS_E_CUDA;
    }
    for (int n = 0; n < order; ++n)
      if (s->tile_bytes[n]) s->tiles[n] = s->shared_buf;
  }
  for (int f = 0; f < 2; ++f) {
    bool used = false;  // is f the fastest reduction mode of a planned mode?
    for (int n = 0; n < order; ++n)
      if (((mode_mask >> n) & 1u) && ((n == 0) ? 1 : 0) == f) used = true;
    if (!used) continue;
    s->nfb_mode[f] = (dims[f] + kChunk - 1) / kChunk;
    s->btile_bytes[f] = (size_t)s->nfb_mode[f] * n_blocks * 2 * nb * kChunk * 2;
    if (cudaMalloc(&s->btiles[f], s->btile_bytes[f]) != cudaSuccess) {
      tc_destroy(s);
      return CPALS_E_CUDA;
    }
    cudaMemset(s->btiles[f], 0, s->btile_bytes[f]);
  }
  const void* kernels[8] = {(const void*)k_mttkrp_tc<16>, (const void*)k_mttkrp_tc<32>, (const void*)k_mttkrp_tc<48>,
                            (const void*)k_mttkrp_tc<64>, (const void*)k_mttkrp_tc<80>, (const void*)k_mttkrp_tc<96>,
                            (const void*)k_mttkrp_tc<112>, (const void*)k_mttkrp_tc<128>};
  for (const void* k : kernels)
    if (set_smem_limit_once(k, (int)kSmemLimit) != cudaSuccess) {
      tc_destroy(s);
      return CPALS_E_CUDA;
    }
  *out = s;
  return CPALS_OK;
}

int64_t tc_factor_rpad(const TcState* s) { return s->rpad; }

int tc_bind_factors(TcState* s, const float* const* F32r) {
  for (int m = 0; m < s->order; ++m) s->F32r[m] = F32r[m];
  s->factors_bound = true;
  return CPALS_OK;
}

BtileDesc tc_btile_desc(const TcState* s, int m) {
  if (m > 1 || !s->btiles[m]) return BtileDesc{nullptr, 0, 0};
  const TcModePlan& p = s->plan[s->plan[0].m_blocks ? 0 : (s->plan[1].m_blocks ? 1 : 2)];
  return BtileDesc{s->btiles[m], p.nb, p.n_blocks};
}

cudaError_t tc_update_factor(TcState* s, int m, const double* F, const DevCheck* chk, cudaStream_t st) {
  if (m > 1 || !s->btiles[m]) return cudaSuccess;  // only planned fastest reduction modes feed the tensor core
  const TcModePlan& p = s->plan[s->plan[0].m_blocks ? 0 : (s->plan[1].m_blocks ? 1 : 2)];
  const int64_t units = s->nfb_mode[m] * p.n_blocks * p.nb * 8;
  const int blocks = (int)std::min<int64_t>((units + 255) / 256, 4096);
  k_build_btiles<<<blocks, 256, 0, st>>>(F, s->dims[m], (int)s->R, s->nfb_mode[m], p.n_blocks, p.nb, s->btiles[m], chk);
  return cudaGetLastError();
}

void tc_destroy(TcState* s) {
  if (!s) return;
  if (s->shared)
    cudaFree(s->shared_buf);
  else
    for (int m = 0; m < kMaxOrder; ++m) cudaFree(s->tiles[m]);
  cudaFree(s->btiles[0]);
  cudaFree(s->btiles[1]);
  cudaFree(s->err);
  delete s;
}

static int build_mode(TcState* s, int n, const void* T, cudaStream_t st) {
  const TcModePlan& p = s->plan[n];
  if (!p.m_blocks) return 0;  // mode not planned
  const int64_t ntiles = (int64_t)p.m_blocks * p.nchunks;
  if (ntiles >= (int64_t(1) << 31)) return CPALS_E_UNSUPPORTED;
  if (s->tdtype == CPALS_DTYPE_F64)
    k_build_tiles<double><<<(unsigned)ntiles, 256, 0, st>>>(static_cast<const double*>(T), p, s->tiles[n]);
  else
    k_build_tiles<float><<<(unsigned)ntiles, 256, 0, st>>>(static_cast<const float*>(T), p, s->tiles[n]);
  return cudaGetLastError() == cudaSuccess ? 1 : CPALS_E_CUDA;
}

int tc_set_tensor(TcState* s, const void* T, cudaStream_t st) {
  s->T = T;
  if (s->shared) return CPALS_OK;  // built per MTTKRP
  for (int n = 0; n < s->order; ++n) {
    const int rc = build_mode(s, n, T, st);
    if (rc < 0) return rc;
  }
  return CPALS_OK;
}

int tc_prepare_mode(TcState* s, int n, cudaStream_t st) {
  if (!s->shared) return 0;
  if (!s->T) return CPALS_E_STATE;
  return build_mode(s, n, s->T, st);
}

int tc_splits(const TcState* s, int n) { return s->plan[n].splits; }
int* tc_error_flag(TcState* s) { return s->err; }

cudaError_t tc_launch_mttkrp(TcState* s, int n, float* part, const DevCheck* chk, cudaStream_t st) {
  if (!s->factors_bound) return cudaErrorInvalidValue;
  const TcModePlan& p = s->plan[n];
  if (!p.m_blocks || !s->btiles[p.fmode]) return cudaErrorInvalidValue;  // mode not planned
  FactorPtrs32 fr{};
  for (int m = 0; m < s->order; ++m) fr.F[m] = s->F32r[m];
  const unsigned grid = (unsigned)(p.m_blocks * p.n_blocks * p.splits);
  switch (p.nb) {
#define CPALS_TC_CASE(W)                                                                                           \
  case W:                                                                                                          \
    k_mttkrp_tc<W><<<grid, tc_threads<W>(), s->smem_bytes[n], st>>>(s->tiles[n], s->btiles[p.fmode], p, fr,       \
                                                                    (int)s->R,                                  \
                                                            part, chk, s->err);                                   \
    break;
    CPALS_TC_CASE(16)
    CPALS_TC_CASE(32)
    CPALS_TC_CASE(48)
    CPALS_TC_CASE(64)
    CPALS_TC_CASE(80)
    CPALS_TC_CASE(96)
    CPALS_TC_CASE(112)
    CPALS_TC_CASE(128)
#undef CPALS_TC_CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace cpals
