// vxc_mixed.cu -- tensor-core (tcgen05) XC quadrature path.  Not yet enabled: the C ABI
// rejects CALCHEM_XC_MIXED with -1 while mixed_supported() returns 0.
#include <cuda_runtime.h>

#include "common.cuh"

namespace cxc {

int mixed_supported(int) { return 0; }
size_t mixed_slab_doubles(int) { return 1; }
int mixed_ctas_per_sm() { return 1; }
cudaError_t launch_mixed(const DevGrid&, const EvalArgs&, int, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t launch_mixed_prepare(const double*, int, void*, cudaStream_t) { return cudaErrorNotSupported; }

}  // namespace cxc
