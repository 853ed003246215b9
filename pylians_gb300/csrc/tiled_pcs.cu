// The tiled mass-assignment pipeline instantiated for PCS.  One unit per MAS so
// that the deposit kernels compile in parallel.
#include "tiled_impl.cuh"

namespace pyl {
template int launch_tiled<PYL_MAS_PCS>(const float *, const float *, long long, float *, float *, int, float, float, void *, OutScale,
                                  cudaStream_t, unsigned *, const RsdArgs *, Owned);
}  // namespace pyl
