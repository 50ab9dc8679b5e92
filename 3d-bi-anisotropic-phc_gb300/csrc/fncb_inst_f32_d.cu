// Instantiates the fncB / curl-transform kernels for float at n = 60.
#include "fncb_impl.cuh"

FAME_INST_SIZE(float, 60)
