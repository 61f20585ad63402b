// Split-precision contraction path (ITG_PREC_SPLIT).
#include "itg_internal.cuh"

struct ContractPlan;

int itg_split_gemm(itg_handle* h, const ContractPlan& p, const double* A, const double* B, double* C,
                   double alpha, double beta) {
  (void)p; (void)A; (void)B; (void)C; (void)alpha; (void)beta;
  return itg_fail(h, ITG_ERR_UNSUPPORTED, "split-precision contraction not built yet");
}

extern "C" double itg_split_error_bound(int64_t K) {
  (void)K;
  return 0.0;
}
