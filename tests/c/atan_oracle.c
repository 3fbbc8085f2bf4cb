/* atan_oracle.c -- the oracle's o_atan2 (oracle/b2o_math.h, -DB2O_OWN_ATAN2 build) for
 * tests/c/atan_check.c. */
#define B2O_OWN_ATAN2
#include "b2o_math.h"

float ot_atan2( float y, float x ) { return o_atan2( y, x ); }
