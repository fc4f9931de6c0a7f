/* elementary_points.h -- the reference header name; the types live in tde_types.h. */
#include "tde_types.h"
