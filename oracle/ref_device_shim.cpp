// Linked into the reference's own GPU build (oracle/build_ref_gpu.sh) in
// place of cudaSetDevice, which the reference's sources call with their
// hard-coded CUDA_DEVICE 1 (include/params.cuh:40): the build renames those
// calls to this function, which selects device 0, the one GPU of the
// machines that run it.  Measurement infrastructure only.
#include <cuda_runtime_api.h>

extern "C" cudaError_t mistic_ref_set_device(int) { return cudaSetDevice(0); }
