// tcgen05 split-BF16 MTTKRP (placeholder until the tensor-core kernel lands).
#include "cpals_tc.cuh"

namespace cpals {
struct TcState {
  int dummy;
};
int tc_create(TcState** out, int, const int64_t*, int64_t, int, int) {
  *out = nullptr;
  return CPALS_E_UNSUPPORTED;
}
void tc_destroy(TcState* s) { delete s; }
int tc_set_tensor(TcState*, const void*, cudaStream_t) { return CPALS_E_UNSUPPORTED; }
int tc_splits(const TcState*, int) { return 1; }
int64_t tc_factor_ld(const TcState*, int) { return 1; }
cudaError_t tc_launch_mttkrp(TcState*, int, const float* const*, float*, const DevCheck*, cudaStream_t) {
  return cudaErrorNotSupported;
}
}  // namespace cpals
