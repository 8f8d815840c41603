// Plain FP64 MTTKRP on CUDA cores: the parity path and the FP64 comparator.
//
// Computes M_n(i, r) = sum_{k} T_(n)(i, k) * KRP(k, r) for the mode-n unfolding of
// a column-major tensor (the product that matricize_tensor(::KRPFreeNormal) forms
// with R tensor-times-vector chains, src/algorithms/als_algorithms/standard/tensor.jl:32-44,
// and matricize_tensor(::KRPNormal) with an explicit KRP, tensor.jl:12-20).
//
// The reduction index space is cut into chunks of CH consecutive values of the
// fastest reduction mode f at fixed values of the other reduction modes.  Inside
// a chunk KRP(k, r) = F_f(k, r) * s(r), where s(r) is the product of the other
// reduction modes' factor rows, so each chunk is a small dense GEMM.  The chunk
// range is split across CTAs (split-K); partial sums go to part[split][In][R]
// and are reduced, in FP64 and in split order, by the solve kernel.
// The tensor may be FP32 (converted exactly on load) or FP64.
#include <algorithm>
#include <atomic>

#include "cpals_internal.cuh"

namespace cpals {
namespace {

constexpr int BM = 64, BN = 64, CH = 32, NT = 256;

// kColMajor: factors are read column-major (I_m x R, first index fastest) instead of
// the engine's row-major copies.
template <typename TT, bool kColMajor = false>
__global__ void __launch_bounds__(NT) k_mttkrp_f64(const TT* __restrict__ T, FactorSet fs, ModeGeom g, int64_t R,
                                                   int64_t chunks_per_split, double* __restrict__ part,
                                                   const DevCheck* __restrict__ chk) {
  if (chk && chk->done) return;
  __shared__ __align__(16) double As[CH][BM + 2];
  __shared__ __align__(16) double Bs[CH][BN + 2];
  __shared__ double s_scale[BN];

  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t i0 = (int64_t)blockIdx.x * BM, r0 = (int64_t)blockIdx.y * BN;
  const int64_t c_begin = (int64_t)blockIdx.z * chunks_per_split;
  const int64_t c_end = min(g.nchunks, c_begin + chunks_per_split);
  const double* __restrict__ Ff = fs.F[g.fmode];
  const int64_t sn = g.strides[g.mode], sf = g.strides[g.fmode];

  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;

  for (int64_t c = c_begin; c < c_end; ++c) {
    const int64_t fb = c % g.nfb;
    int64_t o = c / g.nfb;
    int64_t base = fb * CH * sf;
    int64_t oidx[kMaxOrder];
    for (int j = 0; j < g.n_outer; ++j) {
      const int m = g.outer_modes[j];
      oidx[j] = o % g.dims[m];
      o /= g.dims[m];
      base += oidx[j] * g.strides[m];
    }
    __syncthreads();  // the previous chunk is done with As / Bs / s_scale
    if (tid < BN) {
      const int64_t r = r0 + tid;
      double s = 1.0;
      if (r < R) {
        for (int j = 0; j < g.n_outer; ++j) {
          const int m = g.outer_modes[j];
          s *= fs.F[m][kColMajor ? (oidx[j] + g.dims[m] * r) : (oidx[j] * R + r)];
        }
      } else {
        s = 0.0;
      }
      s_scale[tid] = s;
    }
    const int64_t kf0 = fb * CH;
    if (sf == 1) {
      // reduction index contiguous: lanes walk k, warps walk rows
      const int lane = tid & 31, w = tid >> 5;
      const bool kok = (kf0 + lane) < g.If;
      for (int rr = w; rr < BM; rr += NT / 32) {
        const int64_t i = i0 + rr;
        double v = 0.0;
        if (kok && i < g.In) v = (double)T[base + i * sn + lane];
        As[lane][rr] = v;
      }
    } else {
      // row index contiguous (mode 0): lanes walk rows
      for (int e = tid; e < BM * CH; e += NT) {
        const int rr = e % BM, k = e / BM;
        const int64_t i = i0 + rr;
        double v = 0.0;
        if ((kf0 + k) < g.If && i < g.In) v = (double)T[base + i * sn + (int64_t)k * sf];
        As[k][rr] = v;
      }
    }
    __syncthreads();  // s_scale visible
    for (int e = tid; e < CH * BN; e += NT) {
      const int cc = e % BN, k = e / BN;
      const int64_t kf = kf0 + k, r = r0 + cc;
      double v = 0.0;
      if (kf < g.If && r < R) v = Ff[kColMajor ? (kf + g.If * r) : (kf * R + r)] * s_scale[cc];
      Bs[k][cc] = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < CH; ++k) {
      const double2 a01 = *reinterpret_cast<const double2*>(&As[k][ty * 4]);
      const double2 a23 = *reinterpret_cast<const double2*>(&As[k][ty * 4 + 2]);
      const double2 b01 = *reinterpret_cast<const double2*>(&Bs[k][tx * 4]);
      const double2 b23 = *reinterpret_cast<const double2*>(&Bs[k][tx * 4 + 2]);
      const double av[4] = {a01.x, a01.y, a23.x, a23.y};
      const double bv[4] = {b01.x, b01.y, b23.x, b23.y};
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
    }
  }
  double* out = part + (int64_t)blockIdx.z * g.In * R;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int64_t i = i0 + ty * 4 + a;
    if (i >= g.In) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t r = r0 + tx * 4 + b;
      if (r < R) out[i * R + r] = acc[a][b];
    }
  }
}

}  // namespace

int mttkrp_f64_splits(const ModeGeom& g, int64_t R, int num_sms, int64_t* chunks_per_split) {
  const int64_t tiles = ((g.In + BM - 1) / BM) * ((R + BN - 1) / BN);
  int64_t want = (2LL * num_sms + tiles - 1) / tiles;
  if (want < 1) want = 1;
  if (want > g.nchunks) want = g.nchunks;
  if (want > 4096) want = 4096;
  const int64_t cps = (g.nchunks + want - 1) / want;
  *chunks_per_split = cps;
  return (int)((g.nchunks + cps - 1) / cps);
}

cudaError_t launch_mttkrp_f64(const void* T, int tdtype, const FactorSet& fs, const ModeGeom& g, int64_t R,
                              int splits, int64_t chunks_per_split, double* part, const DevCheck* chk,
                              cudaStream_t st) {
  dim3 grid((unsigned)((g.In + BM - 1) / BM), (unsigned)((R + BN - 1) / BN), (unsigned)splits);
  if (tdtype == CPALS_DTYPE_F64)
    k_mttkrp_f64<double><<<grid, NT, 0, st>>>(static_cast<const double*>(T), fs, g, R, chunks_per_split, part, chk);
  else
    k_mttkrp_f64<float><<<grid, NT, 0, st>>>(static_cast<const float*>(T), fs, g, R, chunks_per_split, part, chk);
  return cudaGetLastError();
}

}  // namespace cpals

// ---------------------------------------------------------------------------
// MTTKRP without any allocation
// ---------------------------------------------------------------------------
// Some callers cannot allocate GPU memory at the time they need an MTTKRP: code that
// runs under a caching allocator's lock or inside a memory-budgeted service, plugins
// that are handed a stream and device buffers by their host, and code paths that must
// not synchronise the device (cudaMalloc and cudaFree can).  cpals_mttkrp_fp64_noalloc
// serves them: the caller passes the tensor, the factors and the output as device
// buffers, and the split-K partial sums live in the fixed array below instead of a
// handle's buffers.  The array is 16 MiB, held by every GPU that loads the library
// until the process exits.
namespace cpals {
namespace {

constexpr int64_t kNoAllocScratchDoubles = int64_t(1) << 21;  // 16 MiB of FP64 partials
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kNoAllocMaxDevices = 64;
// Device address of g_noalloc_scratch per device, fetched once per device.
std::atomic<double*> g_noalloc_ptr[kNoAllocMaxDevices];

__global__ void k_noalloc_reduce(const double* __restrict__ part, int S, int64_t In, int64_t R,
                                 double* __restrict__ out) {
  // partials are [split][In][R]; the output is column-major In x R
  const int64_t n = In * R;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / R, r = e % R;
    double s = 0.0;
    for (int sp = 0; sp < S; ++sp) s += part[(int64_t)sp * n + e];
    out[i + In * r] = s;
  }
}

}  // namespace
}  // namespace cpals

extern "C" int cpals_mttkrp_fp64_noalloc(int order, const int64_t* dims, int64_t rank, int mode, int tensor_dtype,
                                         const void* d_tensor, const double* const* d_factors, double* d_out,
                                         void* stream) {
  using namespace cpals;
  if (order < 2 || order > kMaxOrder || !dims || !d_factors || !d_tensor || !d_out) return CPALS_E_ARG;
  if (mode < 0 || mode >= order || rank < 1) return CPALS_E_ARG;
  if (tensor_dtype != CPALS_DTYPE_F64 && tensor_dtype != CPALS_DTYPE_F32) return CPALS_E_ARG;
  int64_t numel = 1;
  for (int m = 0; m < order; ++m) {
    if (dims[m] < 1 || dims[m] > (int64_t(1) << 31)) return CPALS_E_ARG;
    if (m != mode && !d_factors[m]) return CPALS_E_ARG;
    if (dims[m] > (int64_t(1) << 40) / numel) return CPALS_E_ARG;  // at most 2^40 elements
    numel *= dims[m];
  }
  // The partial sums of one split need In * R doubles; the array must hold at least one.
  // Compared by division: In * rank could overflow for a huge rank.
  if (rank > kNoAllocScratchDoubles / dims[mode]) {
    fprintf(stderr,
            "libcpals: cpals_mttkrp_fp64_noalloc: I_mode = %lld times rank = %lld exceeds the %lld-double scratch "
            "array\n",
            (long long)dims[mode], (long long)rank, (long long)kNoAllocScratchDoubles);
    return CPALS_E_ARG;
  }
  int dev = 0;
  CPALS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return CPALS_E_UNSUPPORTED;
  double* scratch = g_noalloc_ptr[dev].load();
  if (!scratch) {
    // First call on this device (the current device): look up the array's device address.
    CPALS_CUDA_TRY(cudaGetSymbolAddress(reinterpret_cast<void**>(&scratch), g_noalloc_scratch));
    g_noalloc_ptr[dev].store(scratch);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int num_sms = 0;
  CPALS_CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
  const ModeGeom g = make_geom(order, dims, mode, CH);
  int64_t cps = 0;
  int splits = mttkrp_f64_splits(g, rank, num_sms, &cps);
  const int64_t per_split = g.In * rank;
  const int64_t max_splits = kNoAllocScratchDoubles / per_split;
  if (splits > max_splits) {
    // fewer, longer splits so that every split's partials fit the array
    cps = (g.nchunks + max_splits - 1) / max_splits;
    splits = (int)((g.nchunks + cps - 1) / cps);
  }
  FactorSet fs{};
  for (int m = 0; m < order; ++m) fs.F[m] = d_factors[m];
  dim3 grid((unsigned)((g.In + BM - 1) / BM), (unsigned)((rank + BN - 1) / BN), (unsigned)splits);
  // Every split writes all of its In x R partials, so nothing in the array needs clearing.
  if (tensor_dtype == CPALS_DTYPE_F64)
    k_mttkrp_f64<double, true><<<grid, NT, 0, st>>>(static_cast<const double*>(d_tensor), fs, g, rank, cps, scratch,
                                                    nullptr);
  else
    k_mttkrp_f64<float, true><<<grid, NT, 0, st>>>(static_cast<const float*>(d_tensor), fs, g, rank, cps, scratch,
                                                   nullptr);
  CPALS_CUDA_TRY(cudaGetLastError());
  const int64_t n = per_split;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  k_noalloc_reduce<<<blocks, 256, 0, st>>>(scratch, splits, g.In, rank, d_out);
  CPALS_CUDA_TRY(cudaGetLastError());
  return CPALS_OK;
}

