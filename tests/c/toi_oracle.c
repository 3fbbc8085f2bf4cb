/*
 * toi_oracle.c -- flat-array wrapper of the oracle's continuous collision arithmetic
 * (oracle/b2o_toi.c) for tests/c/toi_check.c; same layout as toi_product.c.
 */
#include "b2o.h"

static oSweep sweep_of( const float* s )
{
	oSweep w;
	w.localCenter = ov( s[0], s[1] );
	w.c1 = ov( s[2], s[3] );
	w.c2 = ov( s[4], s[5] );
	w.q1 = orot( s[6], s[7] );
	w.q2 = orot( s[8], s[9] );
	return w;
}

float ot_toi( const float* ptsA, int nA, float rA, const float* sweepA, const float* ptsB, int nB, float rB, const float* sweepB,
			  float tMax, int* state )
{
	oProxy A = o_make_proxy( (const oVec*)ptsA, nA, rA );
	oProxy B = o_make_proxy( (const oVec*)ptsB, nB, rB );
	oSweep sA = sweep_of( sweepA ), sB = sweep_of( sweepB );
	return o_time_of_impact( &A, &sA, &B, &sB, tMax, state );
}

float ot_distance( const float* ptsA, int nA, const float* xfA, const float* ptsB, int nB, const float* xfB )
{
	oProxy A = o_make_proxy( (const oVec*)ptsA, nA, 0.0f );
	oProxy B = o_make_proxy( (const oVec*)ptsB, nB, 0.0f );
	oXf a = { ov( xfA[0], xfA[1] ), orot( xfA[2], xfA[3] ) };
	oXf b = { ov( xfB[0], xfB[1] ), orot( xfB[2], xfB[3] ) };
	oDistCache cache = { 0, { 0, 0, 0 }, { 0, 0, 0 } };
	return o_distance( &cache, &A, a, &B, b, NULL, NULL );
}
