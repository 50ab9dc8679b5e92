// Instantiates the double-single fncB at n = 60.
#include "fncb_impl.cuh"

FAME_INST_DS(60)
