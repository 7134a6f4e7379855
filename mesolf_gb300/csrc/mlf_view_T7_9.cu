// Instantiations of the per-view RL kernel for tap counts T = 7 and 9.
#include "mlf_view.cuh"

namespace mlf {
MLF_INSTANTIATE_VIEW(7)
MLF_INSTANTIATE_VIEW(9)
}  // namespace mlf
