// k_res_a.cu — resident engine instantiations for cluster sizes 1 and 2.
#include "k_resident.cuh"

SRS_RESIDENT_DEFINE(1)
SRS_RESIDENT_DEFINE(2)
