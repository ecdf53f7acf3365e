// rowstep_d34.cu -- row-kernel instantiations: double, three and four species.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST_NC34(double)
