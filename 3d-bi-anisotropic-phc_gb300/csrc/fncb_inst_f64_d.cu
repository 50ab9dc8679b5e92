// Instantiates the fncB / curl-transform kernels for double at n = 60.
#include "fncb_impl.cuh"

FAME_INST_SIZE(double, 60)
