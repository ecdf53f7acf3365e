// rowstep_f.cu -- row-kernel instantiations: float.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST(float, false)
