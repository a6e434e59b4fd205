// kernels for __nv_bfloat16 population storage (see rr_inst.inc): the tile step and the batch
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#define RR_STORE __nv_bfloat16
#define RR_OPS_NAME ops_bf16
#define RR_IMPL_NS impl_bf16
#define RR_PART 1
#include "rr_inst.inc"
