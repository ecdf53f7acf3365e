// rowstep_ts_d.cu -- row-kernel instantiations: double, Tsitouras methods.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST_TS(double, false)
