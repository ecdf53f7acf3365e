// rowstep_f_ram.cu -- row-kernel instantiations: float, with the Raman channel.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST(float, true)
