// Instantiates the fncB / curl-transform kernels for double at n = 4, 6, 8, 10, 12, 16, 18, 20.
#include "fncb_impl.cuh"

FAME_INST_SIZE(double, 4)
FAME_INST_SIZE(double, 6)
FAME_INST_SIZE(double, 8)
FAME_INST_SIZE(double, 10)
FAME_INST_SIZE(double, 12)
FAME_INST_SIZE(double, 16)
FAME_INST_SIZE(double, 18)
FAME_INST_SIZE(double, 20)
