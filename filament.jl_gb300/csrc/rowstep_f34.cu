// rowstep_f34.cu -- row-kernel instantiations: float, three and four species.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST_NC34(float)
