// kernels for float population storage (see rr_inst.inc)
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#define RR_STORE float
#define RR_OPS_NAME ops_f32
#include "rr_inst.inc"
