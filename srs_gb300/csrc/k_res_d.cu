// k_res_d.cu — resident engine instantiations for cluster sizes 8 and 16.
#include "k_resident.cuh"

SRS_RESIDENT_DEFINE(8)
SRS_RESIDENT_DEFINE(16)
