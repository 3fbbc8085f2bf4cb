/*
 * atan_check.c -- the library's atan2 for the revolute joint angle: bit-identical to the
 * oracle's copy (the checker the device is stepped against on joint springs and
 * limits), within one float ulp of the C library's atan2f (which the reference calls),
 * and equal to atan2 evaluated in double and rounded to float (correctly rounded but
 * for rare midpoint cases).  Inputs: the sine/cosine pairs of relative rotations
 * (unit vectors with rounding noise), general pairs over many binades, and the signed
 * zero and axis cases.  Prints "ok ..." and exits 0, or the first failure.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

float pt_atan2( float y, float x );
float ot_atan2( float y, float x );

static uint64_t s_rng = 0x243f6a8885a308d3ull;
static uint32_t next( void )
{
	s_rng = s_rng * 6364136223846793005ull + 1442695040888963407ull;
	return (uint32_t)( s_rng >> 32 );
}
static float uni( float lo, float hi ) { return lo + ( hi - lo ) * ( (float)( next() >> 8 ) * ( 1.0f / 16777216.0f ) ); }

static int64_t ordered( float f )
{
	int32_t i;
	memcpy( &i, &f, 4 );
	return i < 0 ? (int64_t)INT32_MIN - i : i;
}

static long s_glibcDiff, s_roundDiff, s_count;

static int check( float y, float x )
{
	float a = pt_atan2( y, x );
	float b = ot_atan2( y, x );
	float g = atan2f( y, x );
	float d = (float)atan2( (double)y, (double)x );
	if ( memcmp( &a, &b, 4 ) != 0 )
	{
		printf( "atan2(%a, %a): library %a, oracle %a\n", y, x, a, b );
		return 1;
	}
	int64_t u = ordered( a ) - ordered( g );
	if ( u > 1 || u < -1 )
	{
		printf( "atan2(%a, %a): library %a, atan2f %a (%lld ulp)\n", y, x, a, g, (long long)u );
		return 1;
	}
	s_glibcDiff += u != 0;
	s_roundDiff += memcmp( &a, &d, 4 ) != 0;
	s_count += 1;
	return 0;
}

int main( void )
{
	const float z = 0.0f;
	float special[][2] = { { 0.0f, 1.0f }, { -z, 1.0f }, { 0.0f, -1.0f }, { -z, -1.0f }, { 1.0f, 0.0f }, { -1.0f, 0.0f },
						   { 1.0f, -z },   { -1.0f, -z }, { 0.0f, 0.0f },  { -z, 0.0f },   { 0.0f, -z },  { -z, -z },
						   { 1.0f, 1.0f }, { -1.0f, 1.0f }, { 1.0f, -1.0f }, { -1.0f, -1.0f } };
	for ( int i = 0; i < (int)( sizeof( special ) / sizeof( special[0] ) ); ++i )
		if ( check( special[i][0], special[i][1] ) )
			return 1;
	for ( int i = 0; i < 4000000; ++i )
	{
		float a = uni( -3.14159265f, 3.14159265f );
		float s = sinf( a ), c = cosf( a );
		float e = 1.0f + uni( -1e-6f, 1e-6f );
		if ( check( s * e, c * e ) )
			return 1;
		/* small relative angles, where joint limits sit */
		float t = uni( -1e-3f, 1e-3f );
		if ( check( t, 1.0f - 0.5f * t * t ) )
			return 1;
		float y = ldexpf( uni( -1.0f, 1.0f ), (int)( next() % 40 ) - 20 );
		float x = ldexpf( uni( -1.0f, 1.0f ), (int)( next() % 40 ) - 20 );
		if ( check( y, x ) )
			return 1;
	}
	printf( "ok %ld inputs, %ld differ from atan2f by one ulp, %ld from double atan2 rounded\n", s_count, s_glibcDiff,
			s_roundDiff );
	return 0;
}
