// placeholder until the mixed-precision kernels land
#include "jsh_launch.h"
#include "jsh_context.h"
int jsh_prepare_mixed(JshRequest*, const double*) { jsh_set_error("mixed precision not available"); return JSH_ERR_INVALID; }
cudaError_t jsh_launch_transfer_mixed(const JshRequest*, int, int, bool, uint64_t, const JshLaunchShape&, unsigned int*, int, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t jsh_launch_transfer_persistent64(const JshRequest*, int, uint64_t, const JshLaunchShape&, unsigned int*, int, cudaStream_t) { return cudaErrorNotSupported; }
int jsh_persistent_occupancy(int, bool, int) { return 0; }
