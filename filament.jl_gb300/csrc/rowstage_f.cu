// rowstage_f.cu -- non-paraxial stage kernel instantiations: float.
#include "rowstep_inst.cuh"

FIL_ROWSTAGE_INST(float)
