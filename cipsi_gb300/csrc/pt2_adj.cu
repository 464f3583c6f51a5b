// pt2_adj.cu -- the adjoint launch of k_pt2 (dE2/d integrals and root
// energies), plain form, one 64-bit word per spin string, 1..8 roots
// (pt2_adj_w2.cu: two words).
#include "pt2_kernel.cuh"

namespace cipsi_dev {
template cudaError_t launch_pt2<1, 1, false, true>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 2, false, true>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 4, false, true>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 8, false, true>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
}  // namespace cipsi_dev
