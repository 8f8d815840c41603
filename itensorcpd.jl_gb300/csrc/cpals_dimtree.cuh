// Interface of the order-4 dimension-tree MTTKRP (k_dimtree.cu).
#pragma once
#include "cpals_internal.cuh"

namespace cpals {

struct DimTree;

// Plan both partial contractions of an order-4 tensor (mmode: CPALS_MTTKRP_*).
int dt_create(DimTree** out, const int64_t* dims, int64_t R, int mmode, int tdtype, int num_sms);
void dt_destroy(DimTree* d);
// Record the device tensor and (tensor-core path) build the two views' tile streams.
int dt_set_tensor(DimTree* d, const void* T, cudaStream_t st);
// Error word of the tensor-core kernel of view A (which = 0) or B (1); null on the FP64 path.
int* dt_error_flag(DimTree* d, int which);
// Column count of the row-major FP32 factor copies (tensor-core path; 0 otherwise).
int64_t dt_factor_rpad(const DimTree* d);
// Register the row-major FP32 factor copies of the four modes (tensor-core path).
int dt_bind_factors(DimTree* d, const float* const* F32r, const float* const* F32lo);
// Layout of the BF16 factor tiles mode m's new factor feeds (modes 0 and 2; else bt null).
BtileDesc dt_btile_desc(const DimTree* d, int m);
// Rebuild the BF16 factor tiles that mode m's new factor feeds (modes 0 and 2).
cudaError_t dt_update_factor(DimTree* d, int m, const double* F, const DevCheck* chk, cudaStream_t st);
// M_n (FP64 row-major [I_n][R]) from the FP64 row-major factors F.  Modes 0 and 2 (and 1,
// 3 when `reuse` is false) first recompute their partial contraction; modes 1 and 3 with
// `reuse` use the one computed for mode 0 / 2 (valid in ALS order).
cudaError_t dt_mttkrp(DimTree* d, int n, const double* const* F, bool reuse, double* M, const DevCheck* chk,
                      cudaStream_t st);
// Kernel launches of one dt_mttkrp call.
int dt_launches(const DimTree* d, int n, bool reuse);

}  // namespace cpals
