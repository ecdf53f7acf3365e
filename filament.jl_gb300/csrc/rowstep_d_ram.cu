// rowstep_d_ram.cu -- row-kernel instantiations: double, with the Raman channel.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST(double, true)
