// eval_mixed.cu -- mixed-precision rule evaluation (FP32 integrand).
#include "g3l_device.cuh"

namespace g3l {
void *evalmx_kernel(int, int) { return nullptr; }
}  // namespace g3l
