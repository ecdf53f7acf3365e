// rowstep_ts_f.cu -- row-kernel instantiations: float, Tsitouras methods.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST_TS(float, false)
