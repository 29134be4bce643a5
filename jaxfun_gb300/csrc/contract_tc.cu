// Placeholder replaced by the tcgen05 kernel.
#include "jfg_internal.cuh"

namespace jfg {
int contract_tc(const jfg_contract_desc& d, const float* op_hi, const float* op_lo,
                const float* in, float* out, cudaStream_t st) {
  (void)d; (void)op_hi; (void)op_lo; (void)in; (void)out; (void)st;
  return JFG_ERR_UNSUPPORTED;
}
}  // namespace jfg

extern "C" int jfg_contract_tc(const jfg_contract_desc* d, const float* op_hi,
                               const float* op_lo, const float* in, float* out, void* stream) {
  if (!d) return JFG_ERR_ARG;
  return jfg::contract_tc(*d, op_hi, op_lo, in, out, (cudaStream_t)stream);
}
