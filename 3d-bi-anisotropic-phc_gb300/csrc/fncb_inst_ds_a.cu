// Instantiates the double-single fncB at n = 12.
#include "fncb_impl.cuh"

FAME_INST_DS(12)
