// surrogate_consts.h -- shape of the learned plasma surrogate (surrogate.cuh)
// and the range of its output, shared with the row kernel that uses it.
#pragma once

#define NN_IN 3       // input channels
#define NN_CH 64      // hidden channels
#define NN_K 9        // kernel width
#define NN_HALF 4
#define NN_LAYERS 4
// range of the network output g used by the density (the avalanche term's
// amplification e^g stays within [e^-2, e^4]; the physical value,
// ln(rho / rho_photoionised), is small and non-negative)
#define NN_G_LO (-2.0f)
#define NN_G_HI 4.0f
