/* atan_product.c -- the library's gatan2 (box2c_gb300/csrc/b2g_math.h) compiled for the
 * host, for tests/c/atan_check.c. */
#include "b2g_math.h"

float pt_atan2( float y, float x ) { return gatan2( y, x ); }
