// Instantiates the fncB / curl-transform kernels for double at n = 40, 48, 50.
#include "fncb_impl.cuh"

FAME_INST_SIZE(double, 40)
FAME_INST_SIZE(double, 48)
FAME_INST_SIZE(double, 50)
