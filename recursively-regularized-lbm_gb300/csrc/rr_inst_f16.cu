// kernels for __half population storage (see rr_inst.inc)
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#define RR_STORE __half
#define RR_OPS_NAME ops_f16
#include "rr_inst.inc"
