/* k_precision.cu -- placeholder translation unit */
#include "glint_internal.cuh"
