// grad_dd_3.cu -- double-float gradient kernels of the classes with id % 4 == 3.
#define SF_DD_PART 3
#include "grad_dd_part.cuh"
