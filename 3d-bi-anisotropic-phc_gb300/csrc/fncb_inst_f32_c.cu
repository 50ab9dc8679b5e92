// Instantiates the fncB / curl-transform kernels for float at n = 40, 48, 50.
#include "fncb_impl.cuh"

FAME_INST_SIZE(float, 40)
FAME_INST_SIZE(float, 48)
FAME_INST_SIZE(float, 50)
