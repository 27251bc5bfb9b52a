// Tensor-core (tcgen05) DST-I GEMMs: placeholder until the sm_103a kernel lands.
#include "qg_internal.cuh"

namespace qg {

cudaError_t gemm_tc_init() { return cudaErrorNotSupported; }
int gemm_tc_tile_n(int) { return 128; }
cudaError_t launch_gemm_tc(const GemmArgs&, int, int, cudaStream_t) { return cudaErrorNotSupported; }

}  // namespace qg
