/* glint_types.h -- pulls the public C ABI types into the CUDA sources. */
#ifndef GLINT_TYPES_H_
#define GLINT_TYPES_H_
#include <string.h>
#include "glint.h"
#endif
