// Oblivious sparse sign embeddings and the sketched matricization A_sk = T_(k) Omega^T.
//
// The generator follows the two layouts of the reference's C generators
// (src/algebra/sparse_sign.c, src/algebra/sparsestack.c): zeta nonzeros per column of the
// l x n embedding, each +-1/sqrt(zeta), at zeta distinct uniform rows (sparse_sign) or at one
// uniform row in each of zeta near-equal row blocks (sparsestack: block j has q + 1 rows for
// j < r and q rows after, l = q zeta + r).  The reference draws from rand(); here every
// column draws from its own counter-based stream (SplitMix64, Steele, Lea and Flood 2014,
// keyed by the seed and the column), so a column is one thread's work and the embedding is
// reproducible on any device.  Uniform integers use Lemire's multiply-shift with rejection
// (Lemire 2019), so they are unbiased like the reference's rejection sampling.
//
// The sketched matricization (src/algebra/pivot_mapping.jl:111-140) gathers, for each output
// column j, the tensor fibres of the columns that Omega maps to j and sums them weighted by
// Omega's values, in entry order (the reference's order).  The host groups the entries by
// output column (as the reference's dict_rows does) and passes the fibre base positions.
#include <cmath>

#include "cpals_internal.cuh"

namespace cpals {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// one column's stream: word t of column c
struct ColumnStream {
  uint64_t key, t;
  __device__ uint64_t next() { return mix64(key + 0x632BE59BD9B4E019ull * (++t)); }
  // uniform in [0, n), n >= 1 (Lemire: multiply-shift, reject the biased low products)
  __device__ uint32_t below(uint32_t n) {
    uint64_t m = (uint64_t)(uint32_t)next() * n;
    uint32_t lo = (uint32_t)m;
    if (lo < n) {
      const uint32_t thr = (uint32_t)(-n) % n;
      for (int tries = 0; lo < thr && tries < 64; ++tries) {  // expected < 1 extra draw
        m = (uint64_t)(uint32_t)next() * n;
        lo = (uint32_t)m;
      }
    }
    return (uint32_t)(m >> 32);
  }
};

__global__ void k_sparse_sign(int64_t l, int64_t n, int zeta, int injective, uint64_t seed, double a,
                              int32_t* __restrict__ rows, double* __restrict__ vals) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    ColumnStream rs{mix64(seed ^ mix64((uint64_t)c)), 0};
    int32_t* rc = rows + c * zeta;
    double* vc = vals + c * zeta;
    if (injective) {
      const int64_t q = l / zeta, r = l % zeta;
      for (int j = 0; j < zeta; ++j) {
        const int64_t size = q + (j < r ? 1 : 0);
        const int64_t start = (j < r) ? j * (q + 1) : r * (q + 1) + (j - r) * q;
        rc[j] = (int32_t)(start + rs.below((uint32_t)size));
      }
    } else {
      for (int j = 0; j < zeta; ++j) {
        // redraw on a repeat (the reference's rule); after 64 repeats take the smallest row
        // not used yet, so the loop always ends
        int32_t v = 0;
        bool fresh = false;
        for (int tries = 0; tries < 64 && !fresh; ++tries) {
          v = (int32_t)rs.below((uint32_t)l);
          fresh = true;
          for (int k = 0; k < j; ++k) fresh = fresh && (rc[k] != v);
        }
        for (v = fresh ? v : 0; !fresh; ++v) {
          fresh = true;
          for (int k = 0; k < j; ++k) fresh = fresh && (rc[k] != v);
          if (fresh) break;
        }
        rc[j] = v;
      }
    }
    uint64_t bits = 0;
    for (int j = 0; j < zeta; ++j) {
      if ((j & 63) == 0) bits = rs.next();
      vc[j] = (bits & 1ull) ? a : -a;
      bits >>= 1;
    }
  }
}

// out[j * In + i] = sum_{p in segment j} v[p] T[pos[p] + stride * i]
template <typename TT>
__global__ void k_sketch_gather(const TT* __restrict__ T, int64_t In, int64_t stride, const int64_t* __restrict__ seg,
                                const int64_t* __restrict__ pos, const double* __restrict__ v, int64_t l,
                                double* __restrict__ out) {
  for (int64_t j = blockIdx.x; j < l; j += gridDim.x) {
    const int64_t b = seg[j], e = seg[j + 1];
    for (int64_t i = threadIdx.x; i < In; i += blockDim.x) {
      double acc = 0.0;
      for (int64_t p = b; p < e; ++p) acc = fma(v[p], (double)T[pos[p] + stride * i], acc);
      out[j * In + i] = acc;
    }
  }
}

}  // namespace

cudaError_t launch_sparse_sign(int64_t l, int64_t n, int zeta, int injective, uint64_t seed, int32_t* rows,
                               double* vals, cudaStream_t st) {
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 8192);
  k_sparse_sign<<<blocks, 256, 0, st>>>(l, n, zeta, injective, seed, 1.0 / std::sqrt((double)zeta), rows, vals);
  return cudaGetLastError();
}

cudaError_t launch_sketch_gather(const void* T, int tdtype, int64_t In, int64_t stride, const int64_t* seg,
                                 const int64_t* pos, const double* v, int64_t l, double* out, cudaStream_t st) {
  const int threads = (int)std::min<int64_t>(512, std::max<int64_t>(32, (In + 31) / 32 * 32));
  const int blocks = (int)std::min<int64_t>(l, 65535);
  if (tdtype == CPALS_DTYPE_F64)
    k_sketch_gather<double><<<blocks, threads, 0, st>>>(static_cast<const double*>(T), In, stride, seg, pos, v, l, out);
  else
    k_sketch_gather<float><<<blocks, threads, 0, st>>>(static_cast<const float*>(T), In, stride, seg, pos, v, l, out);
  return cudaGetLastError();
}

}  // namespace cpals
