// rowstep_ts_d_ram.cu -- row-kernel instantiations: double, Tsitouras methods, with the Raman channel.
#include "rowstep_inst.cuh"

FIL_ROWSTEP_INST_TS(double, true)
