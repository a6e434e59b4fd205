// kernels for double population storage (see rr_inst.inc)
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#define RR_STORE double
#define RR_OPS_NAME ops_f64
#define RR_IMPL_NS impl_f64
#include "rr_inst.inc"
