// rowstage_d.cu -- non-paraxial stage kernel instantiations: double.
#include "rowstep_inst.cuh"

FIL_ROWSTAGE_INST(double)
