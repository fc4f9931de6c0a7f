/* base_point_types.h -- the reference header name; the types live in tde_types.h. */
#include "tde_types.h"
