// rowstep_ts_f_ram.cu -- row-kernel instantiations: float, Tsitouras methods, with the Raman channel.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST_TS(float, true)
