// k_res_c.cu — resident engine instantiations for cluster sizes 5 and 6.
#include "k_resident.cuh"

SRS_RESIDENT_DEFINE(5)
SRS_RESIDENT_DEFINE(6)
