/* gpu_array_base.h -- the reference header name; see gpu_array.h. */
#include "gpu_array.h"
