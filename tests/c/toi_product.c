/*
 * toi_product.c -- flat-array wrapper of the library's continuous collision arithmetic
 * (box2c_gb300/csrc/b2g_toi.h, compiled for the host) for tests/c/toi_check.c.
 * sweep: localCenter.xy, c1.xy, c2.xy, q1.cs, q2.cs.
 */
#include "b2g_toi.h"

static b2gSweep sweep_of( const float* s )
{
	b2gSweep w;
	w.localCenter = gv( s[0], s[1] );
	w.c1 = gv( s[2], s[3] );
	w.c2 = gv( s[4], s[5] );
	w.q1 = grot( s[6], s[7] );
	w.q2 = grot( s[8], s[9] );
	return w;
}

float pt_toi( const float* ptsA, int nA, float rA, const float* sweepA, const float* ptsB, int nB, float rB, const float* sweepB,
			  float tMax, int* state )
{
	b2gProxy A = gproxy_points( (const b2gVec*)ptsA, nA, rA );
	b2gProxy B = gproxy_points( (const b2gVec*)ptsB, nB, rB );
	b2gSweep sA = sweep_of( sweepA ), sB = sweep_of( sweepB );
	return gtime_of_impact( &A, &sA, &B, &sB, tMax, state );
}

float pt_distance( const float* ptsA, int nA, const float* xfA, const float* ptsB, int nB, const float* xfB )
{
	b2gProxy A = gproxy_points( (const b2gVec*)ptsA, nA, 0.0f );
	b2gProxy B = gproxy_points( (const b2gVec*)ptsB, nB, 0.0f );
	b2gXf a = { gv( xfA[0], xfA[1] ), grot( xfA[2], xfA[3] ) };
	b2gXf b = { gv( xfB[0], xfB[1] ), grot( xfB[2], xfB[3] ) };
	b2gDistCache cache;
	cache.count = 0;
	return gdistance( &cache, &A, a, &B, b );
}
