// Instantiates the double-single fncB at n = 12 and 24.
#include "fncb_impl.cuh"

FAME_INST_DS(12)
FAME_INST_DS(24)
