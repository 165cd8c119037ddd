// Tensor-core (tcgen05) filter HX: placeholder until the kernel lands.
#include "internal.h"

namespace chefsi {
void prepare_tensor_mats(chefsi_operator_s*, cudaStream_t) {}
bool hx_tc(chefsi_operator_s*, const float*, int64_t, float*, int64_t, int, double, bool,
           cudaStream_t) {
  return false;
}
}  // namespace chefsi
