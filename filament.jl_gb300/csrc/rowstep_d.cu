// rowstep_d.cu -- row-kernel instantiations: double.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST(double, false)
