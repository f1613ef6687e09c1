// Tensor-core (tcgen05) DFT correlation. Declared here; the engine is selected
// per pass only when correlate_tensor_supported() accepts the pass.
#include "piv_common.cuh"
#include "piv_internal.h"

namespace piv {

bool correlate_tensor_supported(const CorrArgs& a) {
  (void)a;
  return false;
}

int correlate_tensor(const CorrArgs& a, cudaStream_t stream) {
  (void)a;
  (void)stream;
  return set_error(PIV_E_UNSUPPORTED, "tensor-core correlation is not available for this pass");
}

}  // namespace piv
