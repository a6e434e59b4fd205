// kernels for __half population storage (see rr_inst.inc): all but the tile step and the batch
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#define RR_STORE __half
#define RR_OPS_NAME ops_f16
#define RR_IMPL_NS impl_f16
#define RR_PART 2
#include "rr_inst.inc"
