// k_res_b.cu — resident engine instantiations for cluster sizes 3 and 4.
#include "k_resident.cuh"

SRS_RESIDENT_DEFINE(3)
SRS_RESIDENT_DEFINE(4)
