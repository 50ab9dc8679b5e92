// Instantiates the double-single fncB at n = 40 and 48.
#include "fncb_impl.cuh"

FAME_INST_DS(40)
FAME_INST_DS(48)
