#define MWF_T float
#define MWF_SUF f32
#include "kernels_inst.cuh"
