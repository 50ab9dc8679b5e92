// Instantiates the fncB / curl-transform kernels for double at n = 24, 30, 32, 36.
#include "fncb_impl.cuh"

FAME_INST_SIZE(double, 24)
FAME_INST_SIZE(double, 30)
FAME_INST_SIZE(double, 32)
FAME_INST_SIZE(double, 36)
