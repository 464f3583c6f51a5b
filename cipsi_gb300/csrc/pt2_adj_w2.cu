// pt2_adj_w2.cu -- the adjoint launch of k_pt2, plain form, two 64-bit
// words per spin string (norb 65..128), 1..8 roots; a unit of its own so
// that the build compiles it beside pt2_adj.cu.
#include "pt2_kernel.cuh"

namespace cipsi_dev {
template cudaError_t launch_pt2<2, 1, false, true>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 2, false, true>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 4, false, true>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 8, false, true>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
}  // namespace cipsi_dev
