// Instantiates the fncB / curl-transform kernels for double at n = 64.
#include "fncb_impl.cuh"

FAME_INST_SIZE(double, 64)
