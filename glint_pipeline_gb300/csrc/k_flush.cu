/* k_flush.cu -- placeholder translation unit */
#include "glint_internal.cuh"
