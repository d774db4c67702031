// grad_dd_0.cu -- double-float gradient kernels of the classes with id % 4 == 0.
#define SF_DD_PART 0
#include "grad_dd_part.cuh"
