// Interface of the tcgen05 split-BF16 MTTKRP (k_mttkrp_tc.cu).
#pragma once
#include "cpals_internal.cuh"

namespace cpals {

struct TcState;

// Plan the tensor-core MTTKRP for every mode of an order-`order` tensor.
int tc_create(TcState** out, int order, const int64_t* dims, int64_t R, int tdtype, int num_sms);
void tc_destroy(TcState* s);
// Split the (FP32 or FP64) tensor into BF16 hi/lo planes in the two layouts the kernel streams.
int tc_set_tensor(TcState* s, const void* T, cudaStream_t st);
// Split-K slices of mode n (partials are float [splits][I_n][R]).
int tc_splits(const TcState* s, int n);
// Leading dimension (>= I_m, zero padded) of the FP32 column-major factor copies.
int64_t tc_factor_ld(const TcState* s, int m);
// Launch the MTTKRP of mode n; F32t[m] are the FP32 column-major factor copies.
cudaError_t tc_launch_mttkrp(TcState* s, int n, const float* const* F32t, float* part, const DevCheck* chk,
                             cudaStream_t st);

}  // namespace cpals
