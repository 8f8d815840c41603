// C ABI of libcpals: handle state, the per-sweep launch sequence, CUDA-graph replay
// and the device-side FitCheck loop.  The steps follow optimize()
// (src/optimizers/als_optimizers/optimize.jl:6-35):
//   per mode n: compute_krp (Hadamard of Grams) -> matricize_tensor (MTTKRP) ->
//   solve_ls_problem -> row_norm -> post_solve (Gram); after the last mode check_converge.
// The O(R^3) factorisation of mode n depends only on the Grams, so it runs on a side
// stream concurrently with the MTTKRP of mode n; events fork and join the streams, and
// a whole sweep is captured once into a CUDA graph and replayed.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <set>
#include <vector>

#include "cpals_internal.cuh"
#include "cpals_dimtree.cuh"
#include "cpals_tc.cuh"

using namespace cpals;

struct cpals_ctx {
  int device = 0, order = 0, tdtype = 0, mmode = 0, flags = 0, num_sms = 0;
  int64_t R = 0;
  int64_t dims[kMaxOrder] = {};
  int64_t numel = 0, maxI = 0;
  cudaStream_t st = nullptr, side = nullptr;
  cudaEvent_t ev_main[kMaxOrder] = {}, ev_side[kMaxOrder] = {};
  const void* dT = nullptr;
  void* dT_owned = nullptr;
  bool T_set = false, F_set = false;
  double* F[kMaxOrder] = {};
  float* F32r[kMaxOrder] = {};  // row-major FP32 copies (tensor-core path)
  float* F32lo[kMaxOrder] = {};  // their FP32 remainders F - F32r (dimension tree, tensor-core path)
  int64_t rpad = 0;
  double* G[kMaxOrder] = {};
  double* lam = nullptr;
  double* lam_inv = nullptr;
  double* X = nullptr;
  double* Graw = nullptr;
  void* part = nullptr;
  int part_f32 = 0;
  int splits[kMaxOrder] = {};
  int64_t cps[kMaxOrder] = {};
  ModeGeom geom[kMaxOrder];
  double* work = nullptr;
  double* U = nullptr;
  int* piv = nullptr;
  double* W = nullptr;
  SolveInfo* info = nullptr;
  double* gpart = nullptr;
  double* rgpart = nullptr;  // the solve blocks' partial Grams (null: the tiled Gram kernel)
  unsigned* gcnt = nullptr;
  int gS2[kMaxOrder] = {};
  double* inner_rows = nullptr;  // three words per row: an exact fixed-point row sum
  // the fused mode tail (one cooperative launch per mode): its grid barrier, its error word,
  // whether it is in use, and per mode whether its blocks fit on the device at once
  GridBar* gbar = nullptr;
  int* tail_err = nullptr;
  bool fused_tail = true;
  bool tail_fits[kMaxOrder] = {};
  double* nrm = nullptr;         // scratch of the ||T||^2 kernels
  DevCheck* chk = nullptr;
  DevCheck* hchk = nullptr;  // pinned mirror
  double* traj = nullptr;
  int64_t traj_cap = 0;
  cudaGraphExec_t graph = nullptr;
  const void* graph_dT = nullptr;  // the tensor address the graph's kernels were captured with
  // randomized path
  int64_t* dpiv = nullptr;
  int64_t piv_cap = 0;
  double* Scol = nullptr;
  float2* Spair = nullptr;  // the samples' S as FP32 pairs (the compensated sampled products)
  float2* Tpair = nullptr;  // T_s as FP32 pairs, for FP64 tensors
  void* Ts = nullptr;
  double* Spart = nullptr;
  size_t spart_cap = 0;
  int64_t samp_cap = 0;
  int* derr = nullptr;
  // tensor-core path
  TcState* tc = nullptr;
  // order-4 dimension tree (CPALS_FLAG_DIMTREE): its own contraction plans, and M_n in FP64
  DimTree* dt = nullptr;
  double* Mdt = nullptr;
  // measurement
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  bool profiling = false;
  std::vector<cudaEvent_t> prof_ev;  // pairs
  int64_t prof_used = 0;
  std::vector<cudaEvent_t> samp_ev;  // per sampled update: start, gathers start, gathers end, end
  int64_t samp_used = 0;
  int64_t launches = 0;
  int64_t sweep_launches = 0;  // kernel launches of one sweep (set when the graph is built)
  // CPDiffCheck / CPAngleCheck: two previous-iterate buffers, the split cross Grams, the
  // check kernel's block partials; cross_on appends the check to every sweep
  double* prevF[2] = {};
  double* prevLam[2] = {};
  double* xpart = nullptr;
  double* xred = nullptr;
  unsigned* xcnt = nullptr;
  int64_t xrows = 0;
  int xS[kMaxOrder] = {};
  int xSmax = 0;
  int64_t prev_off[kMaxOrder] = {};
  bool cross_on = false;
  bool prev_valid = false;
};

cudaError_t cpals::set_smem_limit_once(const void* kernel, int bytes) {
  static std::mutex mu;
  static std::set<std::pair<int, const void*>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (done.count({dev, kernel})) return cudaSuccess;
  // the opt-in limit covers static and dynamic shared memory together
  cudaFuncAttributes fa{};
  int optin = 0;
  e = cudaFuncGetAttributes(&fa, kernel);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) {
    bytes = std::min(bytes, optin - (int)fa.sharedSizeBytes);
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  }
  if (e == cudaSuccess)
    done.insert({dev, kernel});
  else
    (void)cudaGetLastError();  // leave no error behind for the next launch check
  return e;
}

namespace {

FactorSet factor_set(const cpals_ctx* c) {
  FactorSet fs{};
  for (int m = 0; m < c->order; ++m) fs.F[m] = c->F[m];
  return fs;
}
GramSet gram_set(const cpals_ctx* c) {
  GramSet gs{};
  for (int m = 0; m < c->order; ++m) gs.G[m] = c->G[m];
  return gs;
}

template <typename T>
int dmalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) {
    fprintf(stderr, "libcpals: cudaMalloc(%zu bytes) failed: %s\n", count * sizeof(T), cudaGetErrorString(e));
    return CPALS_E_CUDA;
  }
  return CPALS_OK;
}

void invalidate_graph(cpals_ctx* c) {
  if (c->graph) cudaGraphExecDestroy(c->graph);
  c->graph = nullptr;
}

// The FP32/BF16 copies a new factor of mode m feeds (tensor-core and dimension-tree paths).
cudaError_t update_factor_tiles(cpals_ctx* c, int m, const DevCheck* chk) {
  if (c->tc) return tc_update_factor(c->tc, m, c->F[m], chk, c->st);
  if (c->dt) return dt_update_factor(c->dt, m, c->F[m], chk, c->st);
  return cudaSuccess;
}

cudaError_t enqueue_mttkrp(cpals_ctx* c, int n, const DevCheck* chk) {
  if (c->mmode == CPALS_MTTKRP_FP64)
    return launch_mttkrp_f64(c->dT, c->tdtype, factor_set(c), c->geom[n], c->R, c->splits[n], c->cps[n],
                             static_cast<double*>(c->part), chk, c->st);
  // CPALS_FLAG_LOWMEM: mode n's tile stream is built into the shared buffer first
  const int k = tc_prepare_mode(c->tc, n, c->st);
  if (k < 0) return cudaErrorInvalidValue;
  c->launches += k;
  return tc_launch_mttkrp(c->tc, n, static_cast<float*>(c->part), chk, c->st);
}

int ensure_cross(cpals_ctx* c) {
  if (c->xpart) return CPALS_OK;
  const int R = (int)c->R;
  int64_t tot = 0;
  for (int m = 0; m < c->order; ++m) {
    c->prev_off[m] = tot;
    tot += c->dims[m] * R;
  }
  const int64_t rows = cross_rows(c->order, c->dims, R, c->num_sms);
  int smax = 1;
  for (int m = 0; m < c->order; ++m) {
    c->xS[m] = (int)((c->dims[m] + rows - 1) / rows);
    smax = std::max(smax, c->xS[m]);
  }
  const int64_t RR = (int64_t)R * R;
  if (dmalloc(&c->prevF[0], tot) != CPALS_OK || dmalloc(&c->prevF[1], tot) != CPALS_OK ||
      dmalloc(&c->prevLam[0], R) != CPALS_OK || dmalloc(&c->prevLam[1], R) != CPALS_OK ||
      dmalloc(&c->xred, 2 * ((RR + 31) / 32)) != CPALS_OK || dmalloc(&c->xcnt, 1) != CPALS_OK ||
      dmalloc(&c->xpart, (int64_t)c->order * smax * RR) != CPALS_OK)
    return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemsetAsync(c->xcnt, 0, sizeof(unsigned), c->st));
  c->xrows = rows;
  c->xSmax = smax;
  return CPALS_OK;
}

CrossArgs cross_args(const cpals_ctx* c) {
  CrossArgs a{};
  for (int m = 0; m < c->order; ++m) {
    a.F[m] = c->F[m];
    a.G[m] = c->G[m];
    a.dims[m] = c->dims[m];
    a.off[m] = c->prev_off[m];
    a.S[m] = c->xS[m];
  }
  a.lam = c->lam;
  a.prevF[0] = c->prevF[0];
  a.prevF[1] = c->prevF[1];
  a.prevLam[0] = c->prevLam[0];
  a.prevLam[1] = c->prevLam[1];
  a.order = c->order;
  a.R = (int)c->R;
  a.rows = c->xrows;
  a.Smax = c->xSmax;
  a.xpart = c->xpart;
  a.red = c->xred;
  a.counter = c->xcnt;
  a.chk = c->chk;
  a.traj = c->traj;
  a.traj_cap = c->traj_cap;
  return a;
}

bool is_cross_kind(int kind) { return kind == CPALS_CHECK_DIFF || kind == CPALS_CHECK_ANGLE; }

bool stream_capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

// One mode of the sweep: compute_krp, matricize_tensor, solve_ls_problem, row_norm and
// post_solve of optimize (optimize.jl:19-27).  On the last mode the fit's terms are saved in
// the device check; run_check = 1 also runs the check's update there (the fused sweep),
// run_check = 0 leaves it to launch_check_step (a caller-driven sweep).
int enqueue_mode(cpals_ctx* c, int n, int run_check) {
  const int N = c->order;
  const int R = (int)c->R;
  const GramSet gs = gram_set(c);
  {
    const int last = (n == N - 1);
    const int64_t In = c->dims[n];
    CPALS_CUDA_TRY(cudaEventRecord(c->ev_main[n], c->st));
    CPALS_CUDA_TRY(cudaStreamWaitEvent(c->side, c->ev_main[n], 0));
    const int mixed = (c->mmode == CPALS_MTTKRP_BF16X3 && R <= 128) ? 1 : 0;
    CPALS_CUDA_TRY(launch_factorize(gs, N, n, R, c->work, c->U, c->piv, c->W, c->info, c->chk, c->side, mixed));
    c->launches += factorize_launches(R, mixed) - 1;  // the FP32 sweep and its V, or the cluster sweep
    CPALS_CUDA_TRY(cudaEventRecord(c->ev_side[n], c->side));
    const bool prof = c->profiling && c->prof_used + 2 <= (int64_t)c->prof_ev.size();
    if (prof) CPALS_CUDA_TRY(cudaEventRecord(c->prof_ev[c->prof_used], c->st));
    if (c->dt) {
      const double* fp[kMaxOrder] = {};
      for (int m = 0; m < N; ++m) fp[m] = c->F[m];
      CPALS_CUDA_TRY(dt_mttkrp(c->dt, n, fp, true, c->Mdt, c->chk, c->st));
      c->launches += dt_launches(c->dt, n, true) - 1;
    } else {
      CPALS_CUDA_TRY(enqueue_mttkrp(c, n, c->chk));
    }
    if (prof) {
      CPALS_CUDA_TRY(cudaEventRecord(c->prof_ev[c->prof_used + 1], c->st));
      c->prof_used += 2;
    }
    CPALS_CUDA_TRY(cudaStreamWaitEvent(c->st, c->ev_side[n], 0));
    // factorize, MTTKRP, solve, gram+finalize, normalize (which also writes the BF16 factor tiles)
    c->launches += 5;
    double* rg = c->rgpart;  // Gram partials from the solve blocks, reduced by launch_gram_rows
    const BtileDesc btd = c->tc ? tc_btile_desc(c->tc, n) : c->dt ? dt_btile_desc(c->dt, n) : BtileDesc{nullptr, 0, 0};
    if (rg && c->fused_tail && c->tail_fits[n]) {
      // solve, Gram, lambda, normalisation (and the fit on the last mode) in one launch
      const void* part = c->dt ? (const void*)c->Mdt : c->part;
      const int pf32 = c->dt ? 0 : c->part_f32;
      const int sp = c->dt ? 1 : c->splits[n];
      cudaError_t e = launch_mode_tail(part, pf32, sp, In, R, c->work, c->W, c->info, c->X, rg, c->F[n], c->F32r[n],
                                       c->F32lo[n], c->rpad, btd, c->Graw, c->lam, c->lam_inv, c->G[n], gs, N, last,
                                       c->inner_rows, c->chk, c->traj, c->traj_cap, c->gbar, c->tail_err,
                                       c->num_sms, run_check, c->st);
      if (e == cudaSuccess) {
        c->launches -= 2;  // factorize, MTTKRP and the tail: three launches, not five
        return CPALS_OK;
      }
      if (e != cudaErrorNotSupported) {
        (void)cudaGetLastError();
        fprintf(stderr, "libcpals: fused mode tail refused (%s); using the separate kernels\n", cudaGetErrorString(e));
        return CPALS_E_UNSUPPORTED;  // the caller retries without it
      }
      c->tail_fits[n] = false;
    }
    if (c->dt)
      CPALS_CUDA_TRY(launch_solve_rows(c->Mdt, 0, 1, In, R, c->work, c->U, c->piv, c->W, c->info, c->X,
                                       last ? c->inner_rows : nullptr, c->chk, c->st, rg));
    else
      CPALS_CUDA_TRY(launch_solve_rows(c->part, c->part_f32, c->splits[n], In, R, c->work, c->U, c->piv, c->W,
                                       c->info, c->X, last ? c->inner_rows : nullptr, c->chk, c->st, rg));
    if (rg)
      CPALS_CUDA_TRY(launch_gram_rows(rg, solve_blocks(In, R), R, c->gcnt + gram_tiles(R), c->Graw, c->lam,
                                      c->lam_inv, c->G[n], gs, N, last, c->inner_rows, In, c->chk, c->traj,
                                      c->traj_cap, c->st, run_check));
    else
      CPALS_CUDA_TRY(launch_gram_finalize(c->X, In, R, c->gS2[n], c->gpart, c->gcnt, c->Graw, c->lam, c->lam_inv,
                                          c->G[n], gs, N, last, c->inner_rows, c->chk, c->traj, c->traj_cap, c->st,
                                          run_check));
    // The last mode's normalisation ignores `done`: it is idempotent (X and lambda are
    // left untouched by the early-returning kernels of later sweeps).
    // the BF16 factor tiles the tensor-core MTTKRP reads are written by the same kernel
    CPALS_CUDA_TRY(launch_normalize(c->X, c->lam_inv, In, R, c->F[n], c->F32r[n], c->rpad,
                                    c->Graw, c->G[n], last ? nullptr : c->chk, c->st, btd, c->F32lo[n]));
  }
  return CPALS_OK;
}

int enqueue_sweep(cpals_ctx* c) {
  for (int n = 0; n < c->order; ++n) {
    int rc = enqueue_mode(c, n, 1);
    if (rc == CPALS_E_UNSUPPORTED && c->fused_tail && !stream_capturing(c->st)) {
      c->fused_tail = false;  // the cooperative launch was refused: the separate kernels from now on
      rc = enqueue_mode(c, n, 1);
    }
    if (rc != CPALS_OK) return rc;
  }
  if (c->cross_on) {  // check_converge of a CPDiffCheck / CPAngleCheck on the new iterate
    CPALS_CUDA_TRY(launch_cp_check(cross_args(c), c->st));
    c->launches += 2;
  }
  return CPALS_OK;
}

int build_graph(cpals_ctx* c) {
  invalidate_graph(c);
  cudaGraph_t g = nullptr;
  CPALS_CUDA_TRY(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
  const int64_t before = c->launches;
  int rc = enqueue_sweep(c);
  c->sweep_launches = c->launches - before;
  c->launches = before;  // capture enqueues nothing; replays are counted
  cudaError_t e = cudaStreamEndCapture(c->st, &g);
  if (rc == CPALS_E_UNSUPPORTED && c->fused_tail) {
    // the cooperative tail could not be captured: capture the separate kernels instead
    if (g) cudaGraphDestroy(g);
    (void)cudaGetLastError();
    c->fused_tail = false;
    return build_graph(c);
  }
  if (rc != CPALS_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  CPALS_CUDA_TRY(e);
  e = cudaGraphInstantiate(&c->graph, g, 0);
  cudaGraphDestroy(g);
  CPALS_CUDA_TRY(e);
  c->graph_dT = c->dT;
  return CPALS_OK;
}

int ensure_traj(cpals_ctx* c, int64_t need) {
  if (need <= c->traj_cap) return CPALS_OK;
  int64_t cap = std::max<int64_t>(need, 2 * c->traj_cap);
  if (c->traj) cudaFree(c->traj);
  c->traj = nullptr;
  c->traj_cap = 0;
  if (dmalloc(&c->traj, cap) != CPALS_OK) return CPALS_E_CUDA;
  c->traj_cap = cap;
  invalidate_graph(c);
  return CPALS_OK;
}

int validate_pivots(const cpals_ctx* c, int mode, const int64_t* pivots, int64_t nsamps) {
  int j = 0;
  for (int m = 0; m < c->order; ++m) {
    if (m == mode) continue;
    const int64_t* col = pivots + nsamps * j;
    for (int64_t s = 0; s < nsamps; ++s)
      if (col[s] < 1 || col[s] > c->dims[m]) return CPALS_E_ARG;
    ++j;
  }
  return CPALS_OK;
}

int ensure_sample_buffers(cpals_ctx* c, int64_t nsamps) {
  if (nsamps <= c->samp_cap) return CPALS_OK;
  cudaFree(c->dpiv);
  cudaFree(c->Scol);
  cudaFree(c->Spair);
  cudaFree(c->Tpair);
  cudaFree(c->Ts);
  c->dpiv = nullptr;
  c->Scol = nullptr;
  c->Spair = c->Tpair = nullptr;
  c->Ts = nullptr;
  c->samp_cap = 0;
  const size_t esz = c->tdtype == CPALS_DTYPE_F64 ? 8 : 4;
  if (dmalloc(&c->dpiv, (size_t)nsamps * (c->order - 1)) || dmalloc(&c->Scol, (size_t)nsamps * c->R) ||
      dmalloc(&c->Spair, (size_t)nsamps * c->R))
    return CPALS_E_CUDA;
  if (c->tdtype == CPALS_DTYPE_F64 && dmalloc(&c->Tpair, (size_t)c->maxI * nsamps)) return CPALS_E_CUDA;
  char* ts = nullptr;
  if (dmalloc(&ts, (size_t)c->maxI * nsamps * esz)) return CPALS_E_CUDA;
  c->Ts = ts;
  c->samp_cap = nsamps;
  return CPALS_OK;
}

int upload_pivots(cpals_ctx* c, int mode, const int64_t* pivots, int64_t nsamps) {
  if (!pivots || nsamps <= 0) return CPALS_E_ARG;
  if (mode < 0 || mode >= c->order) return CPALS_E_ARG;
  if (validate_pivots(c, mode, pivots, nsamps) != CPALS_OK) return CPALS_E_ARG;
  if (ensure_sample_buffers(c, nsamps) != CPALS_OK) return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->dpiv, pivots, sizeof(int64_t) * nsamps * (c->order - 1), cudaMemcpyHostToDevice,
                                 c->st));
  CPALS_CUDA_TRY(cudaMemsetAsync(c->derr, 0, sizeof(int), c->st));
  return CPALS_OK;
}

// Reads and clears the tensor-core kernels' and the fused tail's error words (after a
// stream sync).
int check_tc_err(cpals_ctx* c) {
  if (c->tail_err) {
    int h = 0;
    CPALS_CUDA_TRY(cudaMemcpy(&h, c->tail_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
      fprintf(stderr, "libcpals: a grid barrier of the fused mode tail gave up (bounded wait expired)\n");
      CPALS_CUDA_TRY(cudaMemset(c->tail_err, 0, sizeof(int)));
      return CPALS_E_DEVICE;
    }
  }
  int* flags[2] = {c->tc ? tc_error_flag(c->tc) : nullptr, nullptr};
  if (c->dt) {
    flags[0] = dt_error_flag(c->dt, 0);
    flags[1] = dt_error_flag(c->dt, 1);
  }
  for (int* f : flags) {
    if (!f) continue;
    int h = 0;
    CPALS_CUDA_TRY(cudaMemcpy(&h, f, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
      fprintf(stderr, "libcpals: tensor-core MTTKRP reported error %d (bounded wait expired)\n", h);
      CPALS_CUDA_TRY(cudaMemset(f, 0, sizeof(int)));
      return CPALS_E_DEVICE;
    }
  }
  return CPALS_OK;
}

int check_derr(cpals_ctx* c) {
  int h = 0;
  CPALS_CUDA_TRY(cudaMemcpyAsync(&h, c->derr, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  return h ? CPALS_E_DEVICE : CPALS_OK;
}

void colmajor_to_rowmajor_host(const double* src, int64_t rows, int64_t cols, double* dst) {
  for (int64_t i = 0; i < rows; ++i)
    for (int64_t r = 0; r < cols; ++r) dst[i * cols + r] = src[i + rows * r];
}
void rowmajor_to_colmajor_host(const double* src, int64_t rows, int64_t cols, double* dst) {
  for (int64_t i = 0; i < rows; ++i)
    for (int64_t r = 0; r < cols; ++r) dst[i + rows * r] = src[i * cols + r];
}

}  // namespace

extern "C" {

int cpals_version(void) { return 100; }

const char* cpals_status_string(int s) {
  switch (s) {
    case CPALS_OK: return "ok";
    case CPALS_E_ARG: return "bad argument";
    case CPALS_E_CUDA: return "CUDA runtime error";
    case CPALS_E_NAN: return "Error NAN: the fit became NaN";
    case CPALS_E_STATE: return "call out of order (tensor or factors not set)";
    case CPALS_E_UNSUPPORTED: return "unsupported shape or option";
    case CPALS_E_DEVICE: return "a kernel reported an error status";
    default: return "unknown status";
  }
}

int cpals_destroy(cpals_ctx* c) {
  if (!c) return CPALS_OK;
  DeviceGuard g(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->side) cudaStreamSynchronize(c->side);
  invalidate_graph(c);
  if (c->tc) tc_destroy(c->tc);
  if (c->dt) dt_destroy(c->dt);
  cudaFree(c->Mdt);
  for (int m = 0; m < kMaxOrder; ++m) {
    cudaFree(c->F[m]);
    cudaFree(c->F32r[m]);
    cudaFree(c->F32lo[m]);
    cudaFree(c->G[m]);
    if (c->ev_main[m]) cudaEventDestroy(c->ev_main[m]);
    if (c->ev_side[m]) cudaEventDestroy(c->ev_side[m]);
  }
  cudaFree(c->dT_owned);
  cudaFree(c->lam);
  cudaFree(c->lam_inv);
  cudaFree(c->X);
  cudaFree(c->Graw);
  cudaFree(c->part);
  cudaFree(c->work);
  cudaFree(c->U);
  cudaFree(c->piv);
  cudaFree(c->W);
  cudaFree(c->info);
  cudaFree(c->gpart);
  cudaFree(c->rgpart);
  cudaFree(c->gcnt);
  cudaFree(c->inner_rows);
  cudaFree(c->nrm);
  cudaFree(c->gbar);
  cudaFree(c->tail_err);
  cudaFree(c->chk);
  if (c->hchk) cudaFreeHost(c->hchk);
  cudaFree(c->traj);
  cudaFree(c->dpiv);
  cudaFree(c->Scol);
  cudaFree(c->Spair);
  cudaFree(c->Tpair);
  cudaFree(c->Ts);
  cudaFree(c->Spart);
  cudaFree(c->derr);
  for (int b = 0; b < 2; ++b) {
    cudaFree(c->prevF[b]);
    cudaFree(c->prevLam[b]);
  }
  cudaFree(c->xpart);
  cudaFree(c->xred);
  cudaFree(c->xcnt);
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  for (cudaEvent_t e : c->prof_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : c->samp_ev) cudaEventDestroy(e);
  if (c->st) cudaStreamDestroy(c->st);
  if (c->side) cudaStreamDestroy(c->side);
  delete c;
  return CPALS_OK;
}

int cpals_create(cpals_ctx** out, int device, int order, const int64_t* dims, int64_t rank, int tensor_dtype,
                 int mttkrp_mode, int flags) {
  if (!out) return CPALS_E_ARG;
  *out = nullptr;
  if (order < 2 || order > kMaxOrder || !dims) return CPALS_E_ARG;
  if (rank < 1 || rank > CPALS_MAX_RANK_SOLVE) return CPALS_E_ARG;
  if (tensor_dtype != CPALS_DTYPE_F64 && tensor_dtype != CPALS_DTYPE_F32) return CPALS_E_ARG;
  if (mttkrp_mode != CPALS_MTTKRP_FP64 && mttkrp_mode != CPALS_MTTKRP_BF16X3) return CPALS_E_ARG;
  // the shared tile buffer belongs to the plain split-BF16 engine's tile streams
  if ((flags & CPALS_FLAG_LOWMEM) && (mttkrp_mode != CPALS_MTTKRP_BF16X3 || (flags & CPALS_FLAG_DIMTREE)))
    return CPALS_E_ARG;
  int64_t numel = 1, maxI = 0;
  for (int m = 0; m < order; ++m) {
    if (dims[m] < 1 || dims[m] > (int64_t(1) << 31)) return CPALS_E_ARG;
    if (dims[m] > (int64_t(1) << 40) / numel) return CPALS_E_ARG;  // at most 2^40 elements
    numel *= dims[m];
    maxI = std::max(maxI, dims[m]);
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CPALS_E_CUDA;
  DeviceGuard guard(device);
  cpals_ctx* c = new cpals_ctx();
  c->device = device;
  c->order = order;
  c->tdtype = tensor_dtype;
  c->mmode = mttkrp_mode;
  c->flags = flags;
  c->R = rank;
  c->numel = numel;
  c->maxI = maxI;
  for (int m = 0; m < order; ++m) c->dims[m] = dims[m];
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  {
    // the cluster sweep's device query (function attributes, occupancy) runs here, never
    // inside the capture of a sweep graph
    DeviceGuard g(device);
    (void)cluster_sweep_device_size();
  }
  int rc = CPALS_OK;
#define CK(x)                \
  do {                       \
    rc = (x);                \
    if (rc != CPALS_OK) {    \
      cpals_destroy(c);      \
      return rc;             \
    }                        \
  } while (0)
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess) {
    cpals_destroy(c);
    return CPALS_E_CUDA;
  }
  for (int m = 0; m < order; ++m) {
    if (cudaEventCreateWithFlags(&c->ev_main[m], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_side[m], cudaEventDisableTiming) != cudaSuccess) {
      cpals_destroy(c);
      return CPALS_E_CUDA;
    }
  }
  const int64_t R = rank;
  if (flags & CPALS_FLAG_DIMTREE) {
    if (order != 4) {
      cpals_destroy(c);
      return CPALS_E_UNSUPPORTED;
    }
    rc = dt_create(&c->dt, dims, R, mttkrp_mode, tensor_dtype, c->num_sms);
    if (rc != CPALS_OK) {
      cpals_destroy(c);
      return rc;
    }
  } else if (mttkrp_mode == CPALS_MTTKRP_BF16X3) {
    rc = tc_create(&c->tc, order, dims, R, tensor_dtype, c->num_sms, ~0u, (flags & CPALS_FLAG_LOWMEM) != 0);
    if (rc != CPALS_OK) {
      cpals_destroy(c);
      return rc;
    }
  }
  size_t part_elems = 0;
  for (int m = 0; m < order; ++m) {
    if (c->dt) {
      c->splits[m] = 1;  // M_n arrives reduced, in FP64
    } else if (mttkrp_mode == CPALS_MTTKRP_FP64) {
      c->geom[m] = make_geom(order, dims, m, 32);
      c->splits[m] = mttkrp_f64_splits(c->geom[m], R, c->num_sms, &c->cps[m]);
    } else {
      c->splits[m] = tc_splits(c->tc, m);
    }
    part_elems = std::max(part_elems, (size_t)c->splits[m] * dims[m] * R);
    c->gS2[m] = gram_splits(dims[m], (int)R, c->num_sms);
    CK(dmalloc(&c->F[m], (size_t)dims[m] * R));
    if (c->tc || (c->dt && mttkrp_mode == CPALS_MTTKRP_BF16X3)) {
      c->rpad = c->tc ? tc_factor_rpad(c->tc) : dt_factor_rpad(c->dt);
      CK(dmalloc(&c->F32r[m], (size_t)dims[m] * c->rpad));
      CPALS_CUDA_TRY(cudaMemset(c->F32r[m], 0, sizeof(float) * dims[m] * c->rpad));
      if (c->dt) {
        CK(dmalloc(&c->F32lo[m], (size_t)dims[m] * c->rpad));
        CPALS_CUDA_TRY(cudaMemset(c->F32lo[m], 0, sizeof(float) * dims[m] * c->rpad));
      }
    }
    CK(dmalloc(&c->G[m], (size_t)R * R));
  }
  if (c->tc || c->dt) {
    const float* fr[kMaxOrder] = {};
    const float* fl[kMaxOrder] = {};
    for (int m = 0; m < order; ++m) {
      fr[m] = c->F32r[m];
      fl[m] = c->F32lo[m];
    }
    CK(c->tc ? tc_bind_factors(c->tc, fr) : dt_bind_factors(c->dt, fr, fl));
  }
  if (c->dt) CK(dmalloc(&c->Mdt, (size_t)maxI * R));
  c->part_f32 = (mttkrp_mode == CPALS_MTTKRP_BF16X3) && !c->dt;
  {
    char* p = nullptr;
    CK(dmalloc(&p, part_elems * (c->part_f32 ? 4 : 8)));
    c->part = p;
  }
  int maxS2 = 1;
  for (int m = 0; m < order; ++m) maxS2 = std::max(maxS2, c->gS2[m]);
  CK(dmalloc(&c->lam, R));
  CK(dmalloc(&c->lam_inv, R));
  CK(dmalloc(&c->X, (size_t)maxI * R));
  CK(dmalloc(&c->Graw, (size_t)R * R));
  CK(dmalloc(&c->work, factorize_work_doubles((int)R)));
  CK(dmalloc(&c->U, 2 * (size_t)R * R));  // U and its transpose
  CK(dmalloc(&c->piv, R));
  CK(dmalloc(&c->W, (size_t)R * R));
  CK(dmalloc(&c->info, 1));
  CK(dmalloc(&c->gpart, gram_finalize_part_doubles(maxS2, (int)R)));
  CK(dmalloc(&c->gcnt, gram_tiles((int)R) + 1));
  {
    // partial Grams of the solve blocks, when they stay small (16M doubles)
    size_t need = 0;
    for (int m = 0; m < order; ++m) {
      const int nb = solve_blocks(dims[m], (int)R);
      need = std::max({need, gram_rows_part_doubles(nb, (int)R), mode_tail_part_doubles(nb, (int)R)});
      c->tail_fits[m] = true;  // until a launch says otherwise
    }
    if (need <= (size_t(1) << 24)) CK(dmalloc(&c->rgpart, need));
  }
  CPALS_CUDA_TRY(cudaMemset(c->gcnt, 0, sizeof(unsigned) * (gram_tiles((int)R) + 1)));
  CK(dmalloc(&c->inner_rows, 3 * maxI));
  CK(dmalloc(&c->nrm, norm2_scratch_doubles()));
  CK(dmalloc(&c->gbar, 1));
  CK(dmalloc(&c->tail_err, 1));
  CPALS_CUDA_TRY(cudaMemset(c->gbar, 0, sizeof(GridBar)));
  CPALS_CUDA_TRY(cudaMemset(c->tail_err, 0, sizeof(int)));
  if (flags & CPALS_FLAG_FUSED_TAIL) {  // opt-in: the three kernels measured faster
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
    c->fused_tail = coop != 0;
  } else {
    c->fused_tail = false;
  }
  CK(dmalloc(&c->chk, 1));
  CPALS_CUDA_TRY(cudaMemset(c->chk, 0, sizeof(DevCheck)));
  CK(dmalloc(&c->derr, 1));
  if (cudaMallocHost(&c->hchk, sizeof(DevCheck)) != cudaSuccess) {
    cpals_destroy(c);
    return CPALS_E_CUDA;
  }
  memset(c->hchk, 0, sizeof(DevCheck));
  CK(ensure_traj(c, 1024));
#undef CK
  *out = c;
  return CPALS_OK;
}

static int after_tensor_set(cpals_ctx* c) {
  c->T_set = true;
  // The sweep graph reads the tensor only through its address (FP64 MTTKRP) or through the
  // tile streams rebuilt in place below, so a new tensor at the same address keeps it.
  if (c->graph_dT != c->dT) invalidate_graph(c);
  // ||T||^2 as a double-double, for the compensated fit
  CPALS_CUDA_TRY(launch_tensor_norm2(c->dT, c->tdtype, c->numel, c->nrm, c->chk, c->num_sms, c->st));
  c->launches += 3;
  if (c->tc) {
    int rc = tc_set_tensor(c->tc, c->dT, c->st);
    if (rc != CPALS_OK) return rc;
  }
  if (c->dt) {
    int rc = dt_set_tensor(c->dt, c->dT, c->st);
    if (rc != CPALS_OK) return rc;
  }
  return CPALS_OK;
}

int cpals_set_tensor(cpals_ctx* c, const void* host_tensor) {
  if (!c || !host_tensor) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  const size_t bytes = (size_t)c->numel * (c->tdtype == CPALS_DTYPE_F64 ? 8 : 4);
  if (!c->dT_owned) {
    char* p = nullptr;
    if (dmalloc(&p, bytes) != CPALS_OK) return CPALS_E_CUDA;
    c->dT_owned = p;
  }
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->dT_owned, host_tensor, bytes, cudaMemcpyHostToDevice, c->st));
  c->dT = c->dT_owned;
  int rc = after_tensor_set(c);
  if (rc != CPALS_OK) return rc;
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  return CPALS_OK;
}

int cpals_set_tensor_device(cpals_ctx* c, const void* device_tensor) {
  if (!c || !device_tensor) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  c->dT = device_tensor;
  int rc = after_tensor_set(c);
  if (rc != CPALS_OK) return rc;
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  return CPALS_OK;
}

int cpals_tensor_device(cpals_ctx* c, const void** device_tensor) {
  if (!c || !device_tensor) return CPALS_E_ARG;
  if (!c->T_set || !c->dT) return CPALS_E_STATE;
  *device_tensor = c->dT;
  return CPALS_OK;
}

int cpals_set_factors(cpals_ctx* c, const double* const* host_factors, const double* host_lambda) {
  if (!c || !host_factors) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  const int R = (int)c->R;
  std::vector<double> tmp;
  for (int m = 0; m < c->order; ++m) {
    if (!host_factors[m]) return CPALS_E_ARG;
    tmp.resize((size_t)c->dims[m] * R);
    colmajor_to_rowmajor_host(host_factors[m], c->dims[m], R, tmp.data());
    CPALS_CUDA_TRY(cudaMemcpyAsync(c->F[m], tmp.data(), sizeof(double) * tmp.size(), cudaMemcpyHostToDevice, c->st));
    CPALS_CUDA_TRY(launch_normalize(c->F[m], nullptr, c->dims[m], R, c->F[m], c->F32r[m],
                                    c->rpad, nullptr, nullptr, nullptr, c->st, BtileDesc{nullptr, 0, 0},
                                    c->F32lo[m]));
    CPALS_CUDA_TRY(update_factor_tiles(c, m, nullptr));
    CPALS_CUDA_TRY(launch_gram(c->F[m], c->dims[m], R, c->gS2[m], c->gpart, c->gcnt, c->G[m], nullptr, c->st));
    c->launches += 2;
    CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));  // tmp is reused for the next mode
  }
  if (host_lambda) {
    CPALS_CUDA_TRY(cudaMemcpyAsync(c->lam, host_lambda, sizeof(double) * R, cudaMemcpyHostToDevice, c->st));
  } else {
    std::vector<double> ones(R, 1.0);
    CPALS_CUDA_TRY(cudaMemcpyAsync(c->lam, ones.data(), sizeof(double) * R, cudaMemcpyHostToDevice, c->st));
  }
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  c->F_set = true;
  return CPALS_OK;
}

int cpals_get_factors(cpals_ctx* c, double* const* host_factors, double* host_lambda) {
  if (!c) return CPALS_E_ARG;
  if (!c->F_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  const int R = (int)c->R;
  std::vector<double> tmp;
  for (int m = 0; m < c->order; ++m) {
    if (!host_factors || !host_factors[m]) continue;
    tmp.resize((size_t)c->dims[m] * R);
    CPALS_CUDA_TRY(cudaMemcpyAsync(tmp.data(), c->F[m], sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, c->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
    rowmajor_to_colmajor_host(tmp.data(), c->dims[m], R, host_factors[m]);
  }
  if (host_lambda) {
    CPALS_CUDA_TRY(cudaMemcpyAsync(host_lambda, c->lam, sizeof(double) * R, cudaMemcpyDeviceToHost, c->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  }
  return CPALS_OK;
}

int cpals_get_gram(cpals_ctx* c, int mode, double* host_gram) {
  if (!c || !host_gram || mode < 0 || mode >= c->order) return CPALS_E_ARG;
  if (!c->F_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_gram, c->G[mode], sizeof(double) * c->R * c->R, cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  return CPALS_OK;  // symmetric: row-major == column-major
}

int cpals_mttkrp(cpals_ctx* c, int mode, double* host_out) {
  if (!c || !host_out || mode < 0 || mode >= c->order) return CPALS_E_ARG;
  if (!c->T_set || !c->F_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  const int R = (int)c->R;
  const int64_t In = c->dims[mode];
  if (c->dt) {
    const double* fp[kMaxOrder] = {};
    for (int m = 0; m < c->order; ++m) fp[m] = c->F[m];
    CPALS_CUDA_TRY(dt_mttkrp(c->dt, mode, fp, false, c->X, nullptr, c->st));
    c->launches += dt_launches(c->dt, mode, false);
  } else {
    CPALS_CUDA_TRY(enqueue_mttkrp(c, mode, nullptr));
    c->launches += 2;
    CPALS_CUDA_TRY(launch_reduce_partials(c->part, c->part_f32, c->splits[mode], In, R, c->X, c->st));
  }
  std::vector<double> tmp((size_t)In * R);
  CPALS_CUDA_TRY(cudaMemcpyAsync(tmp.data(), c->X, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  rowmajor_to_colmajor_host(tmp.data(), In, R, host_out);
  return check_tc_err(c);
}

int cpals_mode_update(cpals_ctx* c, int mode, double* host_solution) {
  if (!c || mode < 0 || mode >= c->order) return CPALS_E_ARG;
  if (!c->T_set || !c->F_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  // A converged cpals_optimize leaves `done` set, which makes the sweep kernels return at
  // once; a caller-driven sweep has no such stop.
  CPALS_CUDA_TRY(cudaMemsetAsync(&c->chk->done, 0, sizeof(int), c->st));
  int rc = enqueue_mode(c, mode, 0);
  if (rc == CPALS_E_UNSUPPORTED && c->fused_tail) {
    c->fused_tail = false;
    rc = enqueue_mode(c, mode, 0);
  }
  if (rc != CPALS_OK) return rc;
  if (host_solution) {
    const int64_t In = c->dims[mode];
    std::vector<double> tmp((size_t)In * c->R);
    CPALS_CUDA_TRY(cudaMemcpyAsync(tmp.data(), c->X, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, c->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
    rowmajor_to_colmajor_host(tmp.data(), In, c->R, host_solution);
    return check_tc_err(c);
  }
  return CPALS_OK;
}

int cpals_tensor_norm(cpals_ctx* c, double* norm, double* norm2) {
  if (!c || !norm) return CPALS_E_ARG;
  if (!c->T_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->hchk, c->chk, sizeof(DevCheck), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  const DevCheck& h = *c->hchk;
  if (!h.t2_valid) return CPALS_E_NAN;
  // sqrt of the double-double with one Newton correction
  double r = std::sqrt(h.t2_hi);
  if (r > 0.0) {
    const double rr = r * r, rre = std::fma(r, r, -rr);
    r += (((h.t2_hi - rr) - rre) + h.t2_lo) / (2.0 * r);
  }
  *norm = r;
  if (norm2) {
    norm2[0] = h.t2_hi;
    norm2[1] = h.t2_lo;
  }
  return CPALS_OK;
}

int cpals_optimize(cpals_ctx* c, cpals_check* check, double* fit_trajectory, int64_t traj_capacity) {
  if (!c || !check) return CPALS_E_ARG;
  if (check->kind != CPALS_CHECK_NONE && check->kind != CPALS_CHECK_FIT && !is_cross_kind(check->kind))
    return CPALS_E_ARG;
  if (check->max_counter < 0) return CPALS_E_ARG;
  if (!c->T_set || !c->F_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  const bool cross = is_cross_kind(check->kind);
  if (cross && check->has_prev && !c->prev_valid) return CPALS_E_STATE;
  const int64_t nmax = (int64_t)check->max_counter - check->iter;
  check->sweeps_run = 0;
  if (nmax <= 0) return CPALS_OK;
  if (ensure_traj(c, nmax) != CPALS_OK) return CPALS_E_CUDA;
  if (cross && ensure_cross(c) != CPALS_OK) return CPALS_E_CUDA;
  if (cross != c->cross_on) {
    invalidate_graph(c);
    c->cross_on = cross;
  }
  // keep the device fallback counter, reset the rest from the host check
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->hchk, c->chk, sizeof(DevCheck), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  DevCheck& h = *c->hchk;
  h.kind = check->kind;
  h.iter = check->iter;
  h.counter = check->counter;
  h.max_counter = check->max_counter;
  h.tol = check->tolerance;
  h.ref_norm = check->ref_norm;
  h.lastfit = check->lastfit;
  h.final_fit = check->final_fit;
  h.total_iter = check->total_iter;
  h.done = 0;
  h.nan_flag = 0;
  h.sweeps = 0;
  h.norm_prev = check->norm_prev;
  h.has_prev = cross ? check->has_prev : 0;
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->chk, c->hchk, sizeof(DevCheck), cudaMemcpyHostToDevice, c->st));
  const bool use_graph = !(c->flags & CPALS_FLAG_NO_GRAPH) && !c->profiling;
  if (use_graph && !c->graph) {
    int rc = build_graph(c);
    if (rc != CPALS_OK) return rc;
  }
  int64_t launched = 0, batch = 4;
  while (launched < nmax) {
    const int64_t b = std::min(batch, nmax - launched);
    for (int64_t k = 0; k < b; ++k) {
      if (use_graph) {
        CPALS_CUDA_TRY(cudaGraphLaunch(c->graph, c->st));
        c->launches += c->sweep_launches;
      } else {
        int rc = enqueue_sweep(c);
        if (rc != CPALS_OK) return rc;
      }
    }
    launched += b;
    batch = std::min<int64_t>(batch * 2, 64);
    CPALS_CUDA_TRY(cudaMemcpyAsync(&c->hchk->done, &c->chk->done, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
    if (c->hchk->done) break;
  }
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->hchk, c->chk, sizeof(DevCheck), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  check->iter = h.iter;
  check->counter = h.counter;
  check->lastfit = h.lastfit;
  check->final_fit = h.final_fit;
  check->total_iter = h.total_iter;
  check->sweeps_run = h.sweeps;
  if (cross) {
    check->norm_prev = h.norm_prev;
    check->has_prev = h.has_prev;
    c->prev_valid = h.has_prev != 0;
  }
  if (fit_trajectory && traj_capacity > 0) {
    const int64_t n = std::min<int64_t>({(int64_t)h.sweeps, traj_capacity, c->traj_cap});
    if (n > 0) {
      CPALS_CUDA_TRY(cudaMemcpyAsync(fit_trajectory, c->traj, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st));
      CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
    }
  }
  if (h.nan_flag) return CPALS_E_NAN;
  return check_tc_err(c);
}

int cpals_check_converge(cpals_ctx* c, cpals_check* check, int* converged, double* value) {
  if (!c || !check || !converged || check->max_counter < 0) return CPALS_E_ARG;
  const bool cross = is_cross_kind(check->kind);
  if (!cross && check->kind != CPALS_CHECK_FIT && check->kind != CPALS_CHECK_NONE) return CPALS_E_ARG;
  if (!c->F_set) return CPALS_E_STATE;
  if (cross && check->has_prev && !c->prev_valid) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  if (ensure_traj(c, 1) != CPALS_OK || (cross && ensure_cross(c) != CPALS_OK)) return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->hchk, c->chk, sizeof(DevCheck), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  DevCheck& h = *c->hchk;
  // FitCheck / NoCheck read the terms the last mode's cpals_mode_update saved
  if (!cross && !h.terms_ready) return CPALS_E_STATE;
  h.kind = check->kind;
  h.iter = check->iter;
  h.counter = check->counter;
  h.max_counter = check->max_counter;
  h.tol = check->tolerance;
  h.ref_norm = check->ref_norm;
  h.lastfit = check->lastfit;
  h.final_fit = check->final_fit;
  h.total_iter = check->total_iter;
  h.norm_prev = check->norm_prev;
  h.has_prev = check->has_prev;
  h.done = 0;
  h.nan_flag = 0;
  h.sweeps = 0;
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->chk, c->hchk, sizeof(DevCheck), cudaMemcpyHostToDevice, c->st));
  if (cross) {
    CPALS_CUDA_TRY(launch_cp_check(cross_args(c), c->st));
    c->launches += 2;
  } else {
    CPALS_CUDA_TRY(launch_check_step(c->chk, c->traj, c->traj_cap, c->st));
    c->launches += 1;
  }
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->hchk, c->chk, sizeof(DevCheck), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  check->iter = h.iter;
  check->counter = h.counter;
  check->lastfit = h.lastfit;
  check->final_fit = h.final_fit;
  check->total_iter = h.total_iter;
  check->sweeps_run = 0;
  if (cross) {
    check->norm_prev = h.norm_prev;
    check->has_prev = h.has_prev;
    c->prev_valid = h.has_prev != 0;
  }
  *converged = h.done;
  if (value) {
    CPALS_CUDA_TRY(cudaMemcpyAsync(value, c->traj, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  }
  if (h.nan_flag && check->kind == CPALS_CHECK_FIT) return CPALS_E_NAN;
  return CPALS_OK;
}

int cpals_get_prev(cpals_ctx* c, double* const* host_factors, double* host_lambda) {
  if (!c) return CPALS_E_ARG;
  if (!c->prev_valid) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->hchk, c->chk, sizeof(DevCheck), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  const int sel = c->hchk->psel;
  const int R = (int)c->R;
  std::vector<double> tmp;
  for (int m = 0; m < c->order; ++m) {
    if (!host_factors || !host_factors[m]) continue;
    tmp.resize((size_t)c->dims[m] * R);
    CPALS_CUDA_TRY(cudaMemcpyAsync(tmp.data(), c->prevF[sel] + c->prev_off[m], sizeof(double) * tmp.size(),
                                   cudaMemcpyDeviceToHost, c->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
    rowmajor_to_colmajor_host(tmp.data(), c->dims[m], R, host_factors[m]);
  }
  if (host_lambda) {
    CPALS_CUDA_TRY(cudaMemcpyAsync(host_lambda, c->prevLam[sel], sizeof(double) * R, cudaMemcpyDeviceToHost, c->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  }
  return CPALS_OK;
}

int cpals_set_prev(cpals_ctx* c, const double* const* host_factors, const double* host_lambda) {
  if (!c || !host_factors || !host_lambda) return CPALS_E_ARG;
  for (int m = 0; m < c->order; ++m)
    if (!host_factors[m]) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  if (ensure_cross(c) != CPALS_OK) return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->hchk, c->chk, sizeof(DevCheck), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  const int sel = c->hchk->psel;
  const int R = (int)c->R;
  std::vector<double> tmp;
  for (int m = 0; m < c->order; ++m) {
    tmp.resize((size_t)c->dims[m] * R);
    colmajor_to_rowmajor_host(host_factors[m], c->dims[m], R, tmp.data());
    CPALS_CUDA_TRY(cudaMemcpyAsync(c->prevF[sel] + c->prev_off[m], tmp.data(), sizeof(double) * tmp.size(),
                                   cudaMemcpyHostToDevice, c->st));
    CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));  // tmp is reused for the next mode
  }
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->prevLam[sel], host_lambda, sizeof(double) * R, cudaMemcpyHostToDevice, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  c->prev_valid = true;
  return CPALS_OK;
}

int cpals_sparse_sign(int device, int64_t l, int64_t n, int zeta, int injective, uint64_t seed, int32_t* rows,
                      double* vals, int32_t* colstarts) {
  if (l < 1 || l > INT32_MAX || n < 0 || zeta < 1 || !rows || !vals) return CPALS_E_ARG;
  if (zeta > l) zeta = (int)l;  // as the reference's generators clamp it
  if (colstarts)
    for (int64_t c = 0; c <= n; ++c) colstarts[c] = (int32_t)(c * zeta);
  if (n == 0) return CPALS_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CPALS_E_CUDA;
  DeviceGuard g(device);
  const size_t nnz = (size_t)n * zeta;
  int32_t* drows = nullptr;
  double* dvals = nullptr;
  int rc = CPALS_OK;
  if (dmalloc(&drows, nnz) != CPALS_OK || dmalloc(&dvals, nnz) != CPALS_OK) {
    rc = CPALS_E_CUDA;
  } else {
    cudaError_t e = launch_sparse_sign(l, n, zeta, injective ? 1 : 0, seed, drows, dvals, 0);
    if (e == cudaSuccess) e = cudaMemcpy(rows, drows, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(vals, dvals, sizeof(double) * nnz, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      fprintf(stderr, "libcpals: sparse sign embedding failed: %s\n", cudaGetErrorString(e));
      rc = CPALS_E_CUDA;
    }
  }
  cudaFree(drows);
  cudaFree(dvals);
  return rc;
}

int cpals_sketched_matricization(cpals_ctx* c, int mode, int64_t l, int zeta, const int32_t* rows,
                                 const double* vals, double* host_out) {
  if (!c || mode < 0 || mode >= c->order || l < 1 || zeta < 1 || zeta > l || !rows || !vals || !host_out)
    return CPALS_E_ARG;
  if (!c->T_set) return CPALS_E_STATE;
  const int64_t In = c->dims[mode];
  int64_t n = 1, stride = 1;
  for (int m = 0; m < c->order; ++m)
    if (m != mode) n *= c->dims[m];
  for (int m = 0; m < mode; ++m) stride *= c->dims[m];
  const int64_t nnz = n * zeta;
  // group the entries by output column, keeping entry order (the reference's dict_rows)
  std::vector<int64_t> seg((size_t)l + 1, 0);
  for (int64_t p = 0; p < nnz; ++p) {
    if (rows[p] < 0 || rows[p] >= l) return CPALS_E_ARG;
    ++seg[(size_t)rows[p] + 1];
  }
  for (int64_t j = 0; j < l; ++j) seg[(size_t)j + 1] += seg[(size_t)j];
  std::vector<int64_t> fill(seg.begin(), seg.end() - 1), pos((size_t)std::max<int64_t>(nnz, 1));
  std::vector<double> v((size_t)std::max<int64_t>(nnz, 1));
  for (int64_t p = 0; p < nnz; ++p) {
    const int64_t col = p / zeta;  // column of Omega = fused index of the other modes
    const int64_t slot = fill[(size_t)rows[p]]++;
    pos[(size_t)slot] = (col / stride) * stride * In + (col % stride);
    v[(size_t)slot] = vals[p];
  }
  DeviceGuard g(c->device);
  int64_t *dseg = nullptr, *dpos = nullptr;
  double *dv = nullptr, *dout = nullptr;
  int rc = CPALS_OK;
  if (dmalloc(&dseg, (size_t)l + 1) != CPALS_OK || dmalloc(&dpos, pos.size()) != CPALS_OK ||
      dmalloc(&dv, v.size()) != CPALS_OK || dmalloc(&dout, (size_t)(In * l)) != CPALS_OK) {
    rc = CPALS_E_CUDA;
  } else {
    cudaError_t e = cudaMemcpyAsync(dseg, seg.data(), sizeof(int64_t) * seg.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dpos, pos.data(), sizeof(int64_t) * pos.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dv, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = launch_sketch_gather(c->dT, c->tdtype, In, stride, dseg, dpos, dv, l, dout, c->st);
    if (e == cudaSuccess) {
      c->launches += 1;
      e = cudaMemcpyAsync(host_out, dout, sizeof(double) * (size_t)(In * l), cudaMemcpyDeviceToHost, c->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
      fprintf(stderr, "libcpals: sketched matricization failed: %s\n", cudaGetErrorString(e));
      rc = CPALS_E_CUDA;
    }
  }
  cudaFree(dseg);
  cudaFree(dpos);
  cudaFree(dv);
  cudaFree(dout);
  return rc;
}

// ---- column-pivoted QR, SE-QRCS ----
}  // extern "C"

namespace {

// Device buffers of one column-pivoted QR of an m x n matrix (filled by the caller into A).
struct QrcpBuffers {
  double *A = nullptr, *vn1 = nullptr, *vn2 = nullptr, *vbuf = nullptr, *taus = nullptr, *rdiag = nullptr;
  double* Q = nullptr;
  int64_t* perm = nullptr;
  QrcpArg* part = nullptr;
  QrcpState* st = nullptr;
  QrcpBuffers() = default;
  QrcpBuffers(const QrcpBuffers&) = delete;
  QrcpBuffers& operator=(const QrcpBuffers&) = delete;
  ~QrcpBuffers() {
    cudaFree(A);
    cudaFree(vn1);
    cudaFree(vn2);
    cudaFree(vbuf);
    cudaFree(taus);
    cudaFree(rdiag);
    cudaFree(Q);
    cudaFree(perm);
    cudaFree(part);
    cudaFree(st);
  }
  int alloc(int64_t m, int64_t n, int64_t kmax, int num_sms) {
    if (dmalloc(&A, (size_t)(m * n)) != CPALS_OK || dmalloc(&vn1, (size_t)n) != CPALS_OK ||
        dmalloc(&vn2, (size_t)n) != CPALS_OK || dmalloc(&vbuf, (size_t)m) != CPALS_OK ||
        dmalloc(&taus, (size_t)kmax) != CPALS_OK || dmalloc(&rdiag, (size_t)kmax) != CPALS_OK ||
        dmalloc(&perm, (size_t)n) != CPALS_OK || dmalloc(&part, (size_t)qrcp_parts(n, num_sms)) != CPALS_OK ||
        dmalloc(&st, 1) != CPALS_OK)
      return CPALS_E_CUDA;
    return CPALS_OK;
  }
};

int64_t qrcp_kmax(int64_t m, int64_t ncand, int64_t max_steps) {
  int64_t k = std::min(m, ncand);
  if (max_steps > 0) k = std::min(k, max_steps);
  return k;
}

// Factors b.A (m x n, filled) and copies out: perm0 (n, 0-based original column of each
// position), rdiag (steps), steps, and when non-null R (steps x n, column-major, zero below
// the diagonal) and Q (m x steps).
int qrcp_run(QrcpBuffers& b, int64_t m, int64_t n, int64_t ncand, int64_t kmax, double stop_ratio, int num_sms,
             cudaStream_t st, int64_t* perm0, double* rdiag, int64_t* steps, double* R, double* Q) {
  QrcpJob q{};
  q.A = b.A;
  q.m = m;
  q.n = n;
  q.ncand = ncand;
  q.kmax = kmax;
  q.stop_ratio = stop_ratio;
  q.vn1 = b.vn1;
  q.vn2 = b.vn2;
  q.vbuf = b.vbuf;
  q.taus = b.taus;
  q.rdiag = b.rdiag;
  q.perm = b.perm;
  q.part = b.part;
  q.st = b.st;
  q.num_sms = num_sms;
  CPALS_CUDA_TRY(launch_qrcp_init(q, st));
  QrcpState hs{};
  for (int64_t j = 0; j < kmax;) {
    // with a stopping ratio, look at the state every 32 steps; the steps after a stop return at once
    const int64_t j1 = stop_ratio >= 0.0 ? std::min(kmax, j + 32) : kmax;
    for (; j < j1; ++j) CPALS_CUDA_TRY(launch_qrcp_step(q, j, st));
    if (j < kmax) {
      CPALS_CUDA_TRY(cudaMemcpyAsync(&hs, b.st, sizeof(QrcpState), cudaMemcpyDeviceToHost, st));
      CPALS_CUDA_TRY(cudaStreamSynchronize(st));
      if (hs.done) break;
    }
  }
  CPALS_CUDA_TRY(cudaMemcpyAsync(&hs, b.st, sizeof(QrcpState), cudaMemcpyDeviceToHost, st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(st));
  const int64_t k = hs.steps;
  *steps = k;
  CPALS_CUDA_TRY(cudaMemcpyAsync(perm0, b.perm, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st));
  if (k > 0) CPALS_CUDA_TRY(cudaMemcpyAsync(rdiag, b.rdiag, sizeof(double) * k, cudaMemcpyDeviceToHost, st));
  if (R && k > 0)
    CPALS_CUDA_TRY(cudaMemcpy2DAsync(R, sizeof(double) * k, b.A, sizeof(double) * m, sizeof(double) * k, n,
                                     cudaMemcpyDeviceToHost, st));
  if (Q && k > 0) {
    if (dmalloc(&b.Q, (size_t)(m * k)) != CPALS_OK) return CPALS_E_CUDA;
    CPALS_CUDA_TRY(launch_qr_form_q(b.A, m, k, b.taus, b.Q, num_sms, st));
    CPALS_CUDA_TRY(cudaMemcpyAsync(Q, b.Q, sizeof(double) * m * k, cudaMemcpyDeviceToHost, st));
  }
  CPALS_CUDA_TRY(cudaStreamSynchronize(st));
  if (R)
    for (int64_t c = 0; c < std::min(k, n); ++c)
      for (int64_t r = c + 1; r < k; ++r) R[c * k + r] = 0.0;
  return CPALS_OK;
}

int64_t other_extent(const cpals_ctx* c, int mode) {
  int64_t n = 1;
  for (int m = 0; m < c->order; ++m)
    if (m != mode) n *= c->dims[m];
  return n;
}

// Validates 1-based column ids (or none) and uploads them 0-based; ncols <= 0 with no ids
// means every column.
int upload_cols(int64_t n, int64_t ncols, const int64_t* cols1, int64_t** dcols, int64_t* count, cudaStream_t st) {
  *dcols = nullptr;
  if (!cols1) {
    if (ncols > 0 && ncols != n) return CPALS_E_ARG;
    *count = n;
    return CPALS_OK;
  }
  if (ncols <= 0) return CPALS_E_ARG;
  std::vector<int64_t> h((size_t)ncols);
  for (int64_t i = 0; i < ncols; ++i) {
    if (cols1[i] < 1 || cols1[i] > n) return CPALS_E_ARG;
    h[(size_t)i] = cols1[i] - 1;
  }
  if (dmalloc(dcols, (size_t)ncols) != CPALS_OK) return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemcpyAsync(*dcols, h.data(), sizeof(int64_t) * ncols, cudaMemcpyHostToDevice, st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(st));
  *count = ncols;
  return CPALS_OK;
}

// Fills dst (m x ncols) with columns dcols (0-based; all when null) of the mode unfolding
// (source 0) or of the transposed Khatri-Rao product of the other factors (source 1).
cudaError_t fill_columns(cpals_ctx* c, int source, int mode, const int64_t* dcols, int64_t ncols, double* dst) {
  if (source == 0) {
    int64_t stride = 1;
    for (int m = 0; m < mode; ++m) stride *= c->dims[m];
    return launch_unfold_cols(c->dT, c->tdtype, c->dims[mode], stride, dcols, ncols, dst, c->st);
  }
  return launch_krp_cols(factor_set(c), c->order, mode, c->dims, dcols, ncols, (int)c->R, dst, c->st);
}

int source_ready(const cpals_ctx* c, int source) {
  if (source == 0) return c->T_set ? CPALS_OK : CPALS_E_STATE;
  if (source == 1) return c->F_set ? CPALS_OK : CPALS_E_STATE;
  return CPALS_E_ARG;
}

int matrix_qrcp(cpals_ctx* c, int source, int mode, int64_t ncols, const int64_t* cols1, int64_t ncand,
                int64_t max_steps, double stop_ratio, int64_t* perm, double* rdiag, int64_t* steps, double* R,
                double* Q) {
  if (!c || mode < 0 || mode >= c->order || !perm || !rdiag || !steps) return CPALS_E_ARG;
  int rc = source_ready(c, source);
  if (rc != CPALS_OK) return rc;
  DeviceGuard g(c->device);
  const int64_t m = source == 0 ? c->dims[mode] : c->R;
  int64_t* dcols = nullptr;
  int64_t n = 0;
  rc = upload_cols(other_extent(c, mode), ncols, cols1, &dcols, &n, c->st);
  if (rc == CPALS_OK) {
    ncand = (ncand <= 0 || ncand > n) ? n : ncand;
    const int64_t kmax = qrcp_kmax(m, ncand, max_steps);
    QrcpBuffers b;
    std::vector<int64_t> p0((size_t)n);
    rc = b.alloc(m, n, kmax, c->num_sms);
    if (rc == CPALS_OK) {
      cudaError_t e = fill_columns(c, source, mode, dcols, n, b.A);
      rc = (e == cudaSuccess) ? qrcp_run(b, m, n, ncand, kmax, stop_ratio, c->num_sms, c->st, p0.data(), rdiag, steps,
                                         R, Q)
                              : CPALS_E_CUDA;
      if (e != cudaSuccess) fprintf(stderr, "libcpals: column gather failed: %s\n", cudaGetErrorString(e));
    }
    if (rc == CPALS_OK)
      for (int64_t i = 0; i < n; ++i) perm[i] = p0[(size_t)i] + 1;
  }
  cudaFree(dcols);
  return rc;
}

// Entries of Omega grouped by row, each row's entries in ascending column (entry) order.
struct OmegaRows {
  std::vector<int64_t> seg, col;
  std::vector<double> val;
};
int group_omega_rows(int64_t l, int64_t n, int zeta, const int32_t* rows, const double* vals, OmegaRows& o) {
  const int64_t nnz = n * zeta;
  o.seg.assign((size_t)l + 1, 0);
  for (int64_t p = 0; p < nnz; ++p) {
    if (rows[p] < 0 || rows[p] >= l) return CPALS_E_ARG;
    ++o.seg[(size_t)rows[p] + 1];
  }
  for (int64_t j = 0; j < l; ++j) o.seg[(size_t)j + 1] += o.seg[(size_t)j];
  std::vector<int64_t> fill(o.seg.begin(), o.seg.end() - 1);
  o.col.assign((size_t)std::max<int64_t>(nnz, 1), 0);
  o.val.assign((size_t)std::max<int64_t>(nnz, 1), 0.0);
  for (int64_t p = 0; p < nnz; ++p) {
    const int64_t slot = fill[(size_t)rows[p]]++;
    o.col[(size_t)slot] = p / zeta;
    o.val[(size_t)slot] = vals[p];
  }
  return CPALS_OK;
}

// The columns of Omega (0-based) with an entry in one of the rows psk[0..t) (0-based), in pivot
// order then column order with repeats dropped (SEQRCS.jl:158-159), or in column order
// (sorted, SEQRCS.jl:109-111, 205-207); in[col] marks the members.
void seqrcs_subset(int64_t l, int64_t n, int zeta, const int32_t* rows, const OmegaRows& o, int64_t t,
                   const int64_t* psk, int sorted, std::vector<int64_t>& subset, std::vector<char>& in) {
  subset.clear();
  in.assign((size_t)n, 0);
  if (sorted) {
    std::vector<char> sel((size_t)l, 0);
    for (int64_t q = 0; q < t; ++q) sel[(size_t)psk[q]] = 1;
    for (int64_t col = 0; col < n; ++col)
      for (int k = 0; k < zeta; ++k)
        if (sel[(size_t)rows[col * zeta + k]]) {
          in[(size_t)col] = 1;
          subset.push_back(col);
          break;
        }
  } else {
    for (int64_t q = 0; q < t; ++q) {
      const int64_t row = psk[q];
      for (int64_t p = o.seg[(size_t)row]; p < o.seg[(size_t)row + 1]; ++p) {
        const int64_t col = o.col[(size_t)p];
        if (!in[(size_t)col]) {
          in[(size_t)col] = 1;
          subset.push_back(col);
        }
      }
    }
  }
}

// The sketch of SE-QRCS into b.A (m x l): T_(mode) Omega^T (source 0) or (Omega KRP)^T (source 1).
int fill_sketch(cpals_ctx* c, int source, int mode, int64_t l, const OmegaRows& o, double* dst) {
  int64_t *dseg = nullptr, *dcol = nullptr;
  double* dv = nullptr;
  int rc = CPALS_OK;
  std::vector<int64_t> pos;
  if (source == 0) {
    int64_t stride = 1;
    for (int m = 0; m < mode; ++m) stride *= c->dims[m];
    const int64_t In = c->dims[mode];
    pos.resize(o.col.size());
    for (size_t p = 0; p < o.col.size(); ++p) pos[p] = (o.col[p] / stride) * stride * In + (o.col[p] % stride);
  }
  const std::vector<int64_t>& idx = source == 0 ? pos : o.col;
  if (dmalloc(&dseg, o.seg.size()) != CPALS_OK || dmalloc(&dcol, idx.size()) != CPALS_OK ||
      dmalloc(&dv, o.val.size()) != CPALS_OK) {
    rc = CPALS_E_CUDA;
  } else {
    cudaError_t e = cudaMemcpyAsync(dseg, o.seg.data(), sizeof(int64_t) * o.seg.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dcol, idx.data(), sizeof(int64_t) * idx.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dv, o.val.data(), sizeof(double) * o.val.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) {
      if (source == 0) {
        int64_t stride = 1;
        for (int m = 0; m < mode; ++m) stride *= c->dims[m];
        e = launch_sketch_gather(c->dT, c->tdtype, c->dims[mode], stride, dseg, dcol, dv, l, dst, c->st);
      } else {
        e = launch_omega_hadamard(factor_set(c), c->order, mode, c->dims, dseg, dcol, dv, l, (int)c->R, dst, 1,
                                  c->R, c->st);
      }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
      fprintf(stderr, "libcpals: SE-QRCS sketch failed: %s\n", cudaGetErrorString(e));
      rc = CPALS_E_CUDA;
    }
  }
  cudaFree(dseg);
  cudaFree(dcol);
  cudaFree(dv);
  return rc;
}

}  // namespace

extern "C" {

int cpals_seqrcs_subset(int64_t l, int64_t n, int zeta, const int32_t* rows, int64_t t, const int64_t* psk,
                        int sorted_subset, int64_t* subset, int64_t* nsubset) {
  if (l < 1 || n < 0 || zeta < 1 || zeta > l || (n > 0 && !rows) || t < 1 || !psk || !subset || !nsubset)
    return CPALS_E_ARG;
  std::vector<int64_t> p0((size_t)t);
  for (int64_t q = 0; q < t; ++q) {
    if (psk[q] < 1 || psk[q] > l) return CPALS_E_ARG;
    p0[(size_t)q] = psk[q] - 1;
  }
  OmegaRows o;
  const int rc = group_omega_rows(l, n, zeta, rows, std::vector<double>((size_t)(n * zeta), 0.0).data(), o);
  if (rc != CPALS_OK) return rc;
  std::vector<int64_t> sub;
  std::vector<char> in;
  seqrcs_subset(l, n, zeta, rows, o, t, p0.data(), sorted_subset, sub, in);
  for (size_t i = 0; i < sub.size(); ++i) subset[i] = sub[i] + 1;
  *nsubset = (int64_t)sub.size();
  return CPALS_OK;
}

int cpals_qrcp(int device, int64_t m, int64_t n, const double* A, int64_t ncand, int64_t max_steps,
               double stop_ratio, int64_t* perm, double* rdiag, int64_t* steps, double* R, double* Q) {
  if (m < 1 || n < 1 || !A || !perm || !rdiag || !steps) return CPALS_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CPALS_E_CUDA;
  DeviceGuard guard(device);
  int num_sms = 0;
  if (cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return CPALS_E_CUDA;
  ncand = (ncand <= 0 || ncand > n) ? n : ncand;
  const int64_t kmax = qrcp_kmax(m, ncand, max_steps);
  QrcpBuffers b;
  if (b.alloc(m, n, kmax, num_sms) != CPALS_OK) return CPALS_E_CUDA;
  CPALS_CUDA_TRY(cudaMemcpy(b.A, A, sizeof(double) * m * n, cudaMemcpyHostToDevice));
  std::vector<int64_t> p0((size_t)n);
  const int rc = qrcp_run(b, m, n, ncand, kmax, stop_ratio, num_sms, 0, p0.data(), rdiag, steps, R, Q);
  if (rc == CPALS_OK)
    for (int64_t i = 0; i < n; ++i) perm[i] = p0[(size_t)i] + 1;
  return rc;
}

int cpals_unfolding_qrcp(cpals_ctx* c, int mode, int64_t ncols, const int64_t* cols, int64_t ncand, int64_t max_steps,
                         double stop_ratio, int64_t* perm, double* rdiag, int64_t* steps, double* R, double* Q) {
  return matrix_qrcp(c, 0, mode, ncols, cols, ncand, max_steps, stop_ratio, perm, rdiag, steps, R, Q);
}

int cpals_krp_qrcp(cpals_ctx* c, int mode, int64_t ncols, const int64_t* cols, int64_t ncand, int64_t max_steps,
                   double stop_ratio, int64_t* perm, double* rdiag, int64_t* steps, double* R, double* Q) {
  return matrix_qrcp(c, 1, mode, ncols, cols, ncand, max_steps, stop_ratio, perm, rdiag, steps, R, Q);
}

int cpals_omega_hadamard(cpals_ctx* c, int mode, int64_t l, int zeta, const int32_t* rows, const double* vals,
                         double* host_out) {
  if (!c || mode < 0 || mode >= c->order || l < 1 || zeta < 1 || zeta > l || !rows || !vals || !host_out)
    return CPALS_E_ARG;
  if (!c->F_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  OmegaRows o;
  int rc = group_omega_rows(l, other_extent(c, mode), zeta, rows, vals, o);
  if (rc != CPALS_OK) return rc;
  double* dout = nullptr;
  if (dmalloc(&dout, (size_t)(l * c->R)) != CPALS_OK) return CPALS_E_CUDA;
  // l x R column-major: entry (j, r) at j + l r
  int64_t *dseg = nullptr, *dcol = nullptr;
  double* dv = nullptr;
  if (dmalloc(&dseg, o.seg.size()) != CPALS_OK || dmalloc(&dcol, o.col.size()) != CPALS_OK ||
      dmalloc(&dv, o.val.size()) != CPALS_OK) {
    rc = CPALS_E_CUDA;
  } else {
    cudaError_t e = cudaMemcpyAsync(dseg, o.seg.data(), sizeof(int64_t) * o.seg.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dcol, o.col.data(), sizeof(int64_t) * o.col.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dv, o.val.data(), sizeof(double) * o.val.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess)
      e = launch_omega_hadamard(factor_set(c), c->order, mode, c->dims, dseg, dcol, dv, l, (int)c->R, dout, l, 1,
                                c->st);
    if (e == cudaSuccess) {
      c->launches += 1;
      e = cudaMemcpyAsync(host_out, dout, sizeof(double) * l * c->R, cudaMemcpyDeviceToHost, c->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
      fprintf(stderr, "libcpals: omega_hadamard failed: %s\n", cudaGetErrorString(e));
      rc = CPALS_E_CUDA;
    }
  }
  cudaFree(dseg);
  cudaFree(dcol);
  cudaFree(dv);
  cudaFree(dout);
  return rc;
}

int cpals_seqrcs(cpals_ctx* c, int source, int mode, int64_t l, int zeta, const int32_t* rows, const double* vals,
                 int64_t t, int sorted_subset, int compute_r, double stop_ratio, int64_t* perm, double* rdiag,
                 int64_t* steps, int64_t* nsubset, double* R, double* Q) {
  if (!c || mode < 0 || mode >= c->order || l < 1 || zeta < 1 || zeta > l || !rows || !vals || t < 1 || t > l ||
      !perm || !rdiag || !steps || !nsubset)
    return CPALS_E_ARG;
  if (compute_r && (!R || !Q)) return CPALS_E_ARG;
  int rc = source_ready(c, source);
  if (rc != CPALS_OK) return rc;
  DeviceGuard g(c->device);
  const int64_t m = source == 0 ? c->dims[mode] : c->R;
  const int64_t n = other_extent(c, mode);
  OmegaRows o;
  rc = group_omega_rows(l, n, zeta, rows, vals, o);
  if (rc != CPALS_OK) return rc;
  // stage 1: pivoted QR of the sketch (m x l); its first t pivots are rows of Omega
  std::vector<int64_t> psk((size_t)l);
  {
    QrcpBuffers b;
    const int64_t kmax = qrcp_kmax(m, l, t);
    if (b.alloc(m, l, kmax, c->num_sms) != CPALS_OK) return CPALS_E_CUDA;
    rc = fill_sketch(c, source, mode, l, o, b.A);
    if (rc != CPALS_OK) return rc;
    std::vector<double> rd1((size_t)kmax);
    int64_t k1 = 0;
    rc = qrcp_run(b, m, l, l, kmax, -1.0, c->num_sms, c->st, psk.data(), rd1.data(), &k1, nullptr, nullptr);
    if (rc != CPALS_OK) return rc;
  }
  std::vector<int64_t> subset;
  std::vector<char> in;
  seqrcs_subset(l, n, zeta, rows, o, t, psk.data(), sorted_subset, subset, in);
  const int64_t nsub = (int64_t)subset.size();
  *nsubset = nsub;
  std::vector<int64_t> order = subset;  // matrix columns: the subset, then (with R) the rest ascending
  if (compute_r)
    for (int64_t col = 0; col < n; ++col)
      if (!in[(size_t)col]) order.push_back(col);
  const int64_t ncols = (int64_t)order.size();
  if (nsub == 0) {  // no column reaches the selected rows: p is every column ascending
    *steps = 0;
    for (int64_t col = 0; col < n; ++col) perm[col] = col + 1;
    return CPALS_OK;
  }
  // stage 2: pivoted QR of those columns, pivots among the subset
  int64_t* dcols = nullptr;
  if (dmalloc(&dcols, (size_t)ncols) != CPALS_OK) return CPALS_E_CUDA;
  std::vector<int64_t> p0((size_t)ncols);
  {
    QrcpBuffers b;
    const int64_t kmax = qrcp_kmax(m, nsub, 0);
    rc = b.alloc(m, ncols, kmax, c->num_sms);
    if (rc == CPALS_OK) {
      cudaError_t e = cudaMemcpyAsync(dcols, order.data(), sizeof(int64_t) * ncols, cudaMemcpyHostToDevice, c->st);
      if (e == cudaSuccess) e = fill_columns(c, source, mode, dcols, ncols, b.A);
      rc = (e == cudaSuccess) ? qrcp_run(b, m, ncols, nsub, kmax, compute_r ? -1.0 : stop_ratio, c->num_sms, c->st,
                                         p0.data(), rdiag, steps, compute_r ? R : nullptr, compute_r ? Q : nullptr)
                              : CPALS_E_CUDA;
    }
  }
  cudaFree(dcols);
  if (rc != CPALS_OK) return rc;
  // p = vcat(subset[p_subset], the other columns ascending)
  int64_t w = 0;
  for (int64_t q = 0; q < nsub; ++q) perm[w++] = order[(size_t)p0[(size_t)q]] + 1;
  for (int64_t col = 0; col < n; ++col)
    if (!in[(size_t)col]) perm[w++] = col + 1;
  return CPALS_OK;
}

int cpals_fallback_count(cpals_ctx* c, int64_t* count) {
  if (!c || !count) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  CPALS_CUDA_TRY(cudaMemcpyAsync(c->hchk, c->chk, sizeof(DevCheck), cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  *count = c->hchk->fallbacks;
  return CPALS_OK;
}

int cpals_synchronize(cpals_ctx* c) {
  if (!c) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->side));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  return CPALS_OK;
}

int cpals_timer_start(cpals_ctx* c) {
  if (!c) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  if (!c->t0) {
    CPALS_CUDA_TRY(cudaEventCreate(&c->t0));
    CPALS_CUDA_TRY(cudaEventCreate(&c->t1));
  }
  CPALS_CUDA_TRY(cudaEventRecord(c->t0, c->st));
  return CPALS_OK;
}

int cpals_timer_stop(cpals_ctx* c, double* elapsed_ms) {
  if (!c || !elapsed_ms || !c->t0) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  CPALS_CUDA_TRY(cudaEventRecord(c->t1, c->st));
  CPALS_CUDA_TRY(cudaEventSynchronize(c->t1));
  float ms = 0.0f;
  CPALS_CUDA_TRY(cudaEventElapsedTime(&ms, c->t0, c->t1));
  *elapsed_ms = ms;
  return CPALS_OK;
}

int cpals_set_profiling(cpals_ctx* c, int on) {
  if (!c) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  if (on && c->prof_ev.empty()) {
    c->prof_ev.resize(2 * 8192);
    for (auto& e : c->prof_ev) CPALS_CUDA_TRY(cudaEventCreate(&e));
    c->samp_ev.resize(4 * 1024);
    for (auto& e : c->samp_ev) CPALS_CUDA_TRY(cudaEventCreate(&e));
  }
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  c->profiling = on != 0;
  c->prof_used = 0;
  c->samp_used = 0;
  return CPALS_OK;
}

int cpals_profile_read_sampled(cpals_ctx* c, double* update_ms, double* gather_ms, int64_t* updates) {
  if (!c || !update_ms || !gather_ms || !updates) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  double tu = 0.0, tg = 0.0;
  for (int64_t k = 0; k + 3 < c->samp_used; k += 4) {
    float a = 0.0f, b = 0.0f;
    CPALS_CUDA_TRY(cudaEventElapsedTime(&a, c->samp_ev[k], c->samp_ev[k + 3]));
    CPALS_CUDA_TRY(cudaEventElapsedTime(&b, c->samp_ev[k + 1], c->samp_ev[k + 2]));
    tu += a;
    tg += b;
  }
  *update_ms = tu;
  *gather_ms = tg;
  *updates = c->samp_used / 4;
  return CPALS_OK;
}

int cpals_profile_read(cpals_ctx* c, double* mttkrp_ms, int64_t* launches) {
  if (!c || !mttkrp_ms || !launches) return CPALS_E_ARG;
  DeviceGuard g(c->device);
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  double tot = 0.0;
  for (int64_t k = 0; k + 1 < c->prof_used; k += 2) {
    float ms = 0.0f;
    CPALS_CUDA_TRY(cudaEventElapsedTime(&ms, c->prof_ev[k], c->prof_ev[k + 1]));
    tot += ms;
  }
  *mttkrp_ms = tot;
  *launches = c->prof_used / 2;
  return CPALS_OK;
}

int cpals_set_cluster_sweep_min_rank(int min_rank) { return set_cluster_sweep_min_rank(min_rank); }

int cpals_launch_count(cpals_ctx* c, int64_t* launches) {
  if (!c || !launches) return CPALS_E_ARG;
  *launches = c->launches;
  return CPALS_OK;
}

int cpals_pivot_hadamard(cpals_ctx* c, int mode, const int64_t* pivots, int64_t nsamps, double* host_out) {
  if (!c || !host_out) return CPALS_E_ARG;
  if (!c->F_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  int rc = upload_pivots(c, mode, pivots, nsamps);
  if (rc != CPALS_OK) return rc;
  CPALS_CUDA_TRY(launch_pivot_hadamard(factor_set(c), c->order, mode, c->dims, c->dpiv, nsamps, (int)c->R, c->Scol,
                                       c->derr, c->st));
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_out, c->Scol, sizeof(double) * nsamps * c->R, cudaMemcpyDeviceToHost, c->st));
  return check_derr(c);
}

int cpals_fused_flatten_sample(cpals_ctx* c, int mode, const int64_t* pivots, int64_t nsamps, void* host_out) {
  if (!c || !host_out) return CPALS_E_ARG;
  if (!c->T_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  int rc = upload_pivots(c, mode, pivots, nsamps);
  if (rc != CPALS_OK) return rc;
  CPALS_CUDA_TRY(launch_fibers(c->dT, c->tdtype, c->order, mode, c->dims, c->dpiv, nsamps, c->Ts, c->derr, c->st));
  const size_t esz = c->tdtype == CPALS_DTYPE_F64 ? 8 : 4;
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_out, c->Ts, esz * c->dims[mode] * nsamps, cudaMemcpyDeviceToHost, c->st));
  return check_derr(c);
}

int cpals_leverage_scores(cpals_ctx* c, int mode, double* host_probs) {
  if (!c || !host_probs || mode < 0 || mode >= c->order) return CPALS_E_ARG;
  if (!c->F_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  const int R = (int)c->R;
  const int64_t In = c->dims[mode];
  double* probs = c->inner_rows;  // maxI doubles, free outside a sweep
  CPALS_CUDA_TRY(launch_gram(c->F[mode], In, R, c->gS2[mode], c->gpart, c->gcnt, c->Graw, nullptr, c->st));
  GramSet one{};
  one.G[0] = c->Graw;
  CPALS_CUDA_TRY(launch_factorize(one, 1, -1, R, c->work, c->U, c->piv, c->W, c->info, nullptr, c->st));
  const double scale = 1.0 / (double)std::min<int64_t>(In, R);
  CPALS_CUDA_TRY(launch_leverage_rows(c->F[mode], In, R, c->work, c->U, c->piv, c->info, scale, probs, c->st));
  CPALS_CUDA_TRY(cudaMemcpyAsync(host_probs, probs, sizeof(double) * In, cudaMemcpyDeviceToHost, c->st));
  CPALS_CUDA_TRY(cudaStreamSynchronize(c->st));
  return CPALS_OK;
}

int cpals_sampled_update(cpals_ctx* c, int mode, const int64_t* pivots, int64_t nsamps, int normal) {
  (void)normal;  // both forms solve the FP64 normal equations of the sampled system
  if (!c) return CPALS_E_ARG;
  if (!c->T_set || !c->F_set) return CPALS_E_STATE;
  DeviceGuard g(c->device);
  // profiling: device time of the whole update (pivot upload included) and of the gathers
  const bool prof = c->profiling && c->samp_used + 4 <= (int64_t)c->samp_ev.size();
  cudaEvent_t* ev = prof ? &c->samp_ev[c->samp_used] : nullptr;
  if (prof) CPALS_CUDA_TRY(cudaEventRecord(ev[0], c->st));
  int rc = upload_pivots(c, mode, pivots, nsamps);
  if (rc != CPALS_OK) return rc;
  const int R = (int)c->R;
  const int64_t In = c->dims[mode];
  // S (sampled KRP rows) and T_s (sampled fibres)
  if (prof) CPALS_CUDA_TRY(cudaEventRecord(ev[1], c->st));
  CPALS_CUDA_TRY(launch_pivot_hadamard(factor_set(c), c->order, mode, c->dims, c->dpiv, nsamps, R, c->Scol, c->derr,
                                       c->st));
  CPALS_CUDA_TRY(launch_fibers(c->dT, c->tdtype, c->order, mode, c->dims, c->dpiv, nsamps, c->Ts, c->derr, c->st));
  if (prof) CPALS_CUDA_TRY(cudaEventRecord(ev[2], c->st));
  // A = S^T S and the split-K partials of B = T_s S, both as compensated FP32 (Dot2) products
  // summed into FP64 (FP64 runs some 60 times slower than FP32 on this part)
  const int sp = sampled_splits(nsamps);
  const size_t need = (size_t)sp * std::max<int64_t>(In, R) * R;
  if (need > c->spart_cap) {
    cudaFree(c->Spart);
    c->Spart = nullptr;
    c->spart_cap = 0;
    if (dmalloc(&c->Spart, need) != CPALS_OK) return CPALS_E_CUDA;
    c->spart_cap = need;
  }
  CPALS_CUDA_TRY(launch_sampled_gram(c->Scol, nsamps, R, c->Spair, c->Spart, c->Graw, c->st));
  GramSet one{};
  one.G[0] = c->Graw;
  CPALS_CUDA_TRY(launch_factorize(one, 1, -1, R, c->work, c->U, c->piv, c->W, c->info, nullptr, c->st));
  int sp_rhs = 0;
  CPALS_CUDA_TRY(launch_sampled_rhs(c->Ts, c->tdtype, In, nsamps, R, c->Spair, c->Tpair, c->Spart, &sp_rhs, c->st));
  CPALS_CUDA_TRY(launch_solve_rows(c->Spart, 0, sp_rhs, In, R, c->work, c->U, c->piv, c->W, c->info, c->X, nullptr,
                                   nullptr, c->st));
  // row_norm, Gram refresh, FP32 copy
  CPALS_CUDA_TRY(launch_gram(c->X, In, R, c->gS2[mode], c->gpart, c->gcnt, c->Graw, nullptr, c->st));
  const GramSet gs = gram_set(c);
  CPALS_CUDA_TRY(launch_finalize(c->Graw, R, c->lam, c->lam_inv, c->G[mode], gs, c->order, 0, nullptr, In, nullptr,
                                 c->traj, c->traj_cap, c->st));
  CPALS_CUDA_TRY(launch_normalize(c->X, c->lam_inv, In, R, c->F[mode], c->F32r[mode],
                                  c->rpad, nullptr, nullptr, nullptr, c->st, BtileDesc{nullptr, 0, 0},
                                  c->F32lo[mode]));
  CPALS_CUDA_TRY(update_factor_tiles(c, mode, nullptr));
  if (prof) {
    CPALS_CUDA_TRY(cudaEventRecord(ev[3], c->st));
    c->samp_used += 4;
  }
  return check_derr(c);
}

}  // extern "C"
