// Instantiations of the per-view RL kernel for tap counts T = 15 and 17.
#include "mlf_view.cuh"

namespace mlf {
MLF_INSTANTIATE_VIEW(15)
MLF_INSTANTIATE_VIEW(17)
}  // namespace mlf
