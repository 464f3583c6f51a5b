// pt2_w2.cu -- k_pt2 for two 64-bit words per spin string (norb 65..128),
// plain and batched, for 1, 2, 4 and 8 roots.
#include "pt2_kernel.cuh"

namespace cipsi_dev {
template cudaError_t launch_pt2<2, 1, false, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 1, true, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 2, false, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 2, true, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 4, false, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 4, true, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 8, false, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<2, 8, true, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
}  // namespace cipsi_dev
