// Instantiations of the per-view RL kernel for tap counts T = 3 and 5.
#include "mlf_view.cuh"

namespace mlf {
MLF_INSTANTIATE_VIEW(3)
MLF_INSTANTIATE_VIEW(5)
}  // namespace mlf
