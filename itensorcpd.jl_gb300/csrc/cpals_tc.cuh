// Interface of the tcgen05 split-BF16 MTTKRP (k_mttkrp_tc.cu).
#pragma once
#include "cpals_internal.cuh"

namespace cpals {

struct TcState;

// Plan the tensor-core MTTKRP for the modes of an order-`order` tensor set in `mode_mask`
// (bit n = mode n); only those modes get a tile stream.  `shared`: one buffer, the size of the
// largest stream, holds the stream of the mode being computed (built by tc_prepare_mode).
int tc_create(TcState** out, int order, const int64_t* dims, int64_t R, int tdtype, int num_sms,
              unsigned mode_mask = ~0u, bool shared = false);
void tc_destroy(TcState* s);
// Split the (FP32 or FP64) tensor into BF16 hi/lo planes in the layouts the kernel streams
// (with a shared buffer: only remember T, which must stay at its address).
int tc_set_tensor(TcState* s, const void* T, cudaStream_t st);
// With a shared buffer: build mode n's stream from the remembered tensor (stream-ordered before
// the MTTKRP that reads it); otherwise nothing.  Returns the launches enqueued (0 or 1), or a
// negative CPALS_E_* code.
int tc_prepare_mode(TcState* s, int n, cudaStream_t st);
// Split-K slices of mode n (partials are float [splits][I_n][R]).
int tc_splits(const TcState* s, int n);
// Device error word of the tensor-core kernel (0 = ok; non-zero = a bounded wait expired).
int* tc_error_flag(TcState* s);
// Column count (>= R, zero padded) of the row-major FP32 factor copies.
int64_t tc_factor_rpad(const TcState* s);
// Register the row-major FP32 factor copies F32r[m] ([I_m][tc_factor_rpad()], zero padded) the
// kernel reads the outer factor rows from.
int tc_bind_factors(TcState* s, const float* const* F32r);
// Rebuild the BF16 hi/lo factor-block tiles of mode m (a no-op unless m is 0 or 1) from the FP64
// row-major factor; skipped when the device check is done.
cudaError_t tc_update_factor(TcState* s, int m, const double* F, const DevCheck* chk, cudaStream_t st);
// Layout of mode m's BF16 factor tiles (bt null unless m is a planned fastest reduction
// mode), for a kernel that writes them while it writes the factor.
BtileDesc tc_btile_desc(const TcState* s, int m);
// Launch the MTTKRP of mode n with the bound factor copies.
cudaError_t tc_launch_mttkrp(TcState* s, int n, float* part, const DevCheck* chk, cudaStream_t st);

}  // namespace cpals
