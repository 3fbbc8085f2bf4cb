/*
 * toi_check.c -- the library's time of impact and closest-point distance
 * (box2c_gb300/csrc/b2g_toi.h) against the oracle's (oracle/b2o_toi.c, pinned to the
 * reference through the stepped scenes): seeded random convex proxies (points, segments,
 * boxes, regular polygons; with and without radius) on random sweeps must give the same
 * time bits and the same outcome, and the same distance bits at random poses.  Also
 * checks that every outcome occurs.  Prints "ok" and exits 0, or the first difference.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

float pt_toi( const float* ptsA, int nA, float rA, const float* sweepA, const float* ptsB, int nB, float rB, const float* sweepB,
			  float tMax, int* state );
float pt_distance( const float* ptsA, int nA, const float* xfA, const float* ptsB, int nB, const float* xfB );
float ot_toi( const float* ptsA, int nA, float rA, const float* sweepA, const float* ptsB, int nB, float rB, const float* sweepB,
			  float tMax, int* state );
float ot_distance( const float* ptsA, int nA, const float* xfA, const float* ptsB, int nB, const float* xfB );

static uint64_t s_rng = 0x9e3779b97f4a7c15ull;
static float uni( float lo, float hi )
{
	s_rng = s_rng * 6364136223846793005ull + 1442695040888963407ull;
	float u = (float)( s_rng >> 40 ) * ( 1.0f / 16777216.0f );
	return lo + ( hi - lo ) * u;
}

/* random convex proxy: 1 point, a segment, a box or a regular polygon of 3..8 sides */
static int proxy( float* pts, float* radius )
{
	int kind = (int)uni( 0.0f, 4.0f );
	float s = uni( 0.1f, 1.0f );
	*radius = uni( 0.0f, 1.0f ) < 0.5f ? 0.0f : uni( 0.01f, 0.3f );
	if ( kind == 0 )
	{
		pts[0] = uni( -0.2f, 0.2f );
		pts[1] = uni( -0.2f, 0.2f );
		if ( *radius == 0.0f )
			*radius = uni( 0.05f, 0.5f );
		return 1;
	}
	if ( kind == 1 )
	{
		pts[0] = -s;
		pts[1] = uni( -0.1f, 0.1f );
		pts[2] = s;
		pts[3] = uni( -0.1f, 0.1f );
		return 2;
	}
	if ( kind == 2 )
	{
		float h = uni( 0.1f, 1.0f );
		float v[8] = { -s, -h, s, -h, s, h, -s, h };
		memcpy( pts, v, sizeof( v ) );
		return 4;
	}
	int n = 3 + (int)uni( 0.0f, 6.0f );
	for ( int i = 0; i < n; ++i )
	{
		float a = 6.2831853f * (float)i / (float)n;
		pts[2 * i] = s * cosf( a );
		pts[2 * i + 1] = s * sinf( a );
	}
	return n;
}

static void sweep( float* w, int moving )
{
	w[0] = uni( -0.1f, 0.1f );
	w[1] = uni( -0.1f, 0.1f );
	w[2] = uni( -3.0f, 3.0f );
	w[3] = uni( -3.0f, 3.0f );
	float a1 = uni( -3.0f, 3.0f );
	w[6] = cosf( a1 );
	w[7] = sinf( a1 );
	if ( moving )
	{
		w[4] = uni( -3.0f, 3.0f );
		w[5] = uni( -3.0f, 3.0f );
		float a2 = a1 + uni( -1.0f, 1.0f );
		w[8] = cosf( a2 );
		w[9] = sinf( a2 );
	}
	else
	{
		w[4] = w[2];
		w[5] = w[3];
		w[8] = w[6];
		w[9] = w[7];
	}
}

int main( void )
{
	int seen[5] = { 0 };
	for ( int k = 0; k < 200000; ++k )
	{
		float pa[16], pb[16], ra, rb, sa[10], sb[10];
		int na = proxy( pa, &ra );
		int nb = proxy( pb, &rb );
		sweep( sa, k % 3 == 0 );
		sweep( sb, 1 );
		float tMax = k % 4 == 0 ? uni( 0.2f, 1.0f ) : 1.0f;
		int s1, s2;
		float t1 = pt_toi( pa, na, ra, sa, pb, nb, rb, sb, tMax, &s1 );
		float t2 = ot_toi( pa, na, ra, sa, pb, nb, rb, sb, tMax, &s2 );
		if ( memcmp( &t1, &t2, 4 ) != 0 || s1 != s2 )
		{
			printf( "case %d: toi %.9g (%d) vs oracle %.9g (%d)\n", k, t1, s1, t2, s2 );
			return 1;
		}
		if ( s1 >= 0 && s1 < 5 )
			seen[s1] += 1;
		float xa[4] = { sa[2], sa[3], sa[6], sa[7] }, xb[4] = { sb[4], sb[5], sb[8], sb[9] };
		float d1 = pt_distance( pa, na, xa, pb, nb, xb );
		float d2 = ot_distance( pa, na, xa, pb, nb, xb );
		if ( memcmp( &d1, &d2, 4 ) != 0 )
		{
			printf( "case %d: distance %.9g vs oracle %.9g\n", k, d1, d2 );
			return 1;
		}
	}
	for ( int s = 2; s < 5; ++s )
		if ( seen[s] == 0 )
		{
			printf( "outcome %d never occurred\n", s );
			return 1;
		}
	printf( "ok failed=%d overlapped=%d hit=%d separated=%d\n", seen[1], seen[2], seen[3], seen[4] );
	return 0;
}
