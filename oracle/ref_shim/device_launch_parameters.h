/* empty host stand-in (see cuda_runtime.h in this directory) */
