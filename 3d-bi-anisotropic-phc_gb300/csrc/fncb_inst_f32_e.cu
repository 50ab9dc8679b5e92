// Instantiates the fncB / curl-transform kernels for float at n = 64.
#include "fncb_impl.cuh"

FAME_INST_SIZE(float, 64)
