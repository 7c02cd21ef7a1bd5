#define MWF_T double
#define MWF_SUF f64
#include "kernels_inst.cuh"
