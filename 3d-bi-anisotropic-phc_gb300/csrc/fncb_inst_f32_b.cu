// Instantiates the fncB / curl-transform kernels for float at n = 24, 30, 32, 36.
#include "fncb_impl.cuh"

FAME_INST_SIZE(float, 24)
FAME_INST_SIZE(float, 30)
FAME_INST_SIZE(float, 32)
FAME_INST_SIZE(float, 36)
