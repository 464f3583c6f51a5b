// pt2_w1.cu -- k_pt2 for one 64-bit word per spin string (norb <= 64),
// plain and batched, for 1, 2, 4 and 8 roots.
#include "pt2_kernel.cuh"

namespace cipsi_dev {
template cudaError_t launch_pt2<1, 1, false, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 1, true, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 2, false, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 2, true, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 4, false, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 4, true, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 8, false, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
template cudaError_t launch_pt2<1, 8, true, false>(const Params&, const BatchArgs&, int, size_t, cudaStream_t);
}  // namespace cipsi_dev
