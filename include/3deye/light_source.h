/* light_source.h -- the reference header name; the type lives in tde_types.h. */
#include "tde_types.h"
