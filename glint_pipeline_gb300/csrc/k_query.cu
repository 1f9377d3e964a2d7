/* k_query.cu -- placeholder translation unit */
#include "glint_internal.cuh"
