// grad_dd_1.cu -- double-float gradient kernels of the classes with id % 4 == 1.
#define SF_DD_PART 1
#include "grad_dd_part.cuh"
