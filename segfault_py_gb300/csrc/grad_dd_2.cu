// grad_dd_2.cu -- double-float gradient kernels of the classes with id % 4 == 2.
#define SF_DD_PART 2
#include "grad_dd_part.cuh"
