// Instantiates the fncB / curl-transform kernels for float at n = 4, 6, 8, 10, 12, 16, 18, 20.
#include "fncb_impl.cuh"

FAME_INST_SIZE(float, 4)
FAME_INST_SIZE(float, 6)
FAME_INST_SIZE(float, 8)
FAME_INST_SIZE(float, 10)
FAME_INST_SIZE(float, 12)
FAME_INST_SIZE(float, 16)
FAME_INST_SIZE(float, 18)
FAME_INST_SIZE(float, 20)
