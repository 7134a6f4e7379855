// Instantiations of the per-view RL kernel for tap counts T = 11 and 13.
#include "mlf_view.cuh"

namespace mlf {
MLF_INSTANTIATE_VIEW(11)
MLF_INSTANTIATE_VIEW(13)
}  // namespace mlf
