/* dim3.h -- the reference header name; the types live in tde_types.h. */
#include "tde_types.h"
