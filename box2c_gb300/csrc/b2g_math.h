/*
 * b2g_math.h -- single-precision 2D math shared by the host C code and the sm_103a
 * kernels of the GB300 step pipeline.
 *
 * Every helper evaluates in the operand order of the matching reference helper
 * (include/box2d/math_functions.h:118-540, src/math_functions.c:55-93).  Host files are
 * compiled with -ffp-contract=off and device code with --fmad=false, so no multiply-add
 * is fused and results are bit-identical to the reference's non-FMA build.  sqrtf and
 * division are the IEEE-754 correctly rounded operations on both sides.
 */
#pragma once

#include <float.h>
#include <math.h>
#include <stdbool.h>
#include <stdint.h>

#if defined( __CUDACC__ )
	#define B2G_HD __host__ __device__ __forceinline__
#else
	#define B2G_HD static inline
#endif

#define B2G_PI 3.14159265359f
#define B2G_LINEAR_SLOP 0.005f
#define B2G_SPECULATIVE ( 4.0f * B2G_LINEAR_SLOP )
#define B2G_AABB_MARGIN 0.1f
#define B2G_MAX_TRANSLATION 4.0f
#define B2G_MAX_ROTATION ( 0.25f * B2G_PI )
#define B2G_HUGE 100000.0f
#define B2G_COLORS 12
#define B2G_OVERFLOW 11
#define B2G_NULL ( -1 )

typedef struct b2gVec
{
	float x, y;
} b2gVec;

typedef struct b2gRot
{
	float c, s;
} b2gRot;

typedef struct b2gXf
{
	b2gVec p;
	b2gRot q;
} b2gXf;

typedef struct b2gBox
{
	b2gVec lo, hi;
} b2gBox;

B2G_HD b2gVec gv( float x, float y )
{
	b2gVec v;
	v.x = x;
	v.y = y;
	return v;
}
B2G_HD b2gRot grot( float c, float s )
{
	b2gRot q;
	q.c = c;
	q.s = s;
	return q;
}
B2G_HD float gmin( float a, float b ) { return a < b ? a : b; }
B2G_HD float gmax( float a, float b ) { return a > b ? a : b; }
B2G_HD float gabs( float a ) { return a < 0 ? -a : a; }
B2G_HD float gclamp( float a, float lo, float hi ) { return a < lo ? lo : ( a > hi ? hi : a ); }
B2G_HD float gdot( b2gVec a, b2gVec b ) { return a.x * b.x + a.y * b.y; }
B2G_HD float gcross( b2gVec a, b2gVec b ) { return a.x * b.y - a.y * b.x; }
B2G_HD b2gVec gcross_sv( float s, b2gVec v ) { return gv( -s * v.y, s * v.x ); }
B2G_HD b2gVec gright( b2gVec v ) { return gv( v.y, -v.x ); }
B2G_HD b2gVec gleft( b2gVec v ) { return gv( -v.y, v.x ); }
B2G_HD b2gVec gadd( b2gVec a, b2gVec b ) { return gv( a.x + b.x, a.y + b.y ); }
B2G_HD b2gVec gsub( b2gVec a, b2gVec b ) { return gv( a.x - b.x, a.y - b.y ); }
B2G_HD b2gVec gneg( b2gVec a ) { return gv( -a.x, -a.y ); }
B2G_HD b2gVec glerp( b2gVec a, b2gVec b, float t ) { return gv( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y ); }
B2G_HD b2gVec gmulsv( float s, b2gVec v ) { return gv( s * v.x, s * v.y ); }
B2G_HD b2gVec gmuladd( b2gVec a, float s, b2gVec b ) { return gv( a.x + s * b.x, a.y + s * b.y ); }
B2G_HD b2gVec gmulsub( b2gVec a, float s, b2gVec b ) { return gv( a.x - s * b.x, a.y - s * b.y ); }
B2G_HD b2gVec gminv( b2gVec a, b2gVec b ) { return gv( gmin( a.x, b.x ), gmin( a.y, b.y ) ); }
B2G_HD b2gVec gmaxv( b2gVec a, b2gVec b ) { return gv( gmax( a.x, b.x ), gmax( a.y, b.y ) ); }
B2G_HD float glen( b2gVec v ) { return sqrtf( v.x * v.x + v.y * v.y ); }
B2G_HD float glen2( b2gVec v ) { return v.x * v.x + v.y * v.y; }
B2G_HD float gdist2( b2gVec a, b2gVec b )
{
	b2gVec c = gv( b.x - a.x, b.y - a.y );
	return c.x * c.x + c.y * c.y;
}
B2G_HD b2gVec gnormalize( b2gVec v )
{
	float length = glen( v );
	if ( length < FLT_EPSILON )
		return gv( 0.0f, 0.0f );
	float inv = 1.0f / length;
	return gv( inv * v.x, inv * v.y );
}
B2G_HD b2gVec glen_normalize( float* length, b2gVec v )
{
	*length = glen( v );
	if ( *length < FLT_EPSILON )
		return gv( 0.0f, 0.0f );
	float inv = 1.0f / *length;
	return gv( inv * v.x, inv * v.y );
}
B2G_HD b2gRot gnormrot( b2gRot q )
{
	float mag = sqrtf( q.s * q.s + q.c * q.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	return grot( q.c * inv, q.s * inv );
}
B2G_HD b2gRot gintrot( b2gRot q1, float da )
{
	b2gRot q2 = grot( q1.c - da * q1.s, q1.s + da * q1.c );
	float mag = sqrtf( q2.s * q2.s + q2.c * q2.c );
	float inv = mag > 0.0f ? 1.0f / mag : 0.0f;
	return grot( q2.c * inv, q2.s * inv );
}
B2G_HD b2gRot gmulrot( b2gRot q, b2gRot r )
{
	b2gRot qr;
	qr.s = q.s * r.c + q.c * r.s;
	qr.c = q.c * r.c - q.s * r.s;
	return qr;
}
B2G_HD b2gRot ginvmulrot( b2gRot q, b2gRot r )
{
	b2gRot qr;
	qr.s = q.c * r.s - q.s * r.c;
	qr.c = q.c * r.c + q.s * r.s;
	return qr;
}
B2G_HD b2gVec grotate( b2gRot q, b2gVec v ) { return gv( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y ); }
B2G_HD b2gVec ginvrotate( b2gRot q, b2gVec v ) { return gv( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y ); }
B2G_HD b2gVec gxfpoint( b2gXf t, b2gVec p )
{
	return gv( ( t.q.c * p.x - t.q.s * p.y ) + t.p.x, ( t.q.s * p.x + t.q.c * p.y ) + t.p.y );
}
B2G_HD b2gXf ginvmulxf( b2gXf A, b2gXf B )
{
	b2gXf C;
	C.q = ginvmulrot( A.q, B.q );
	C.p = ginvrotate( A.q, gsub( B.p, A.p ) );
	return C;
}
/* atan2 of finite arguments, in single precision, evaluated in double with IEEE
 * operations only (no library call), so host and device compute the same bits.  Method:
 * reduce to z = min(|x|,|y|) / max(|x|,|y|) in [0, 1]; take the nearest table point
 * c = k/8 and t = (z - c) / (1 + z c), |t| <= 1/16, so atan z = atan c + atan t by the
 * arctangent addition formula; atan t by its Taylor series to t^13 (truncation below
 * 2^-56 relative); then undo the octant reduction.  The table holds atan(k/8) rounded
 * to double.  The double result is within a few double ulps of the true value, so the
 * returned float is the correctly rounded atan2 except in rare midpoint cases; it is
 * within one float ulp of glibc's atan2f. */
B2G_HD float gatan2( float y, float x )
{
	const double atanTable[9] = { 0.0,
								  0x1.fd5ba9aac2f6ep-4,
								  0x1.f5b75f92c80ddp-3,
								  0x1.6f61941e4def1p-2,
								  0x1.dac670561bb4fp-2,
								  0x1.1e00babdefeb4p-1,
								  0x1.4978fa3269ee1p-1,
								  0x1.700a7c5784634p-1,
								  0x1.921fb54442d18p-1 };
	const double pi = 0x1.921fb54442d18p+1, halfPi = 0x1.921fb54442d18p+0;
	double ax = x < 0.0f ? -(double)x : (double)x;
	double ay = y < 0.0f ? -(double)y : (double)y;
	bool negX = signbit( x ) != 0, negY = signbit( y ) != 0;
	double r;
	if ( ax == 0.0 && ay == 0.0 )
		r = negX ? pi : 0.0;
	else
	{
		bool swap = ay > ax;
		double z = swap ? ax / ay : ay / ax;
		int k = (int)( z * 8.0 + 0.5 );
		double c = (double)k * 0.125;
		double t = ( z - c ) / ( 1.0 + z * c );
		double t2 = t * t;
		double p = 0x1.3b13b13b13b14p-4;
		p = p * t2 - 0x1.745d1745d1746p-4;
		p = p * t2 + 0x1.c71c71c71c71cp-4;
		p = p * t2 - 0x1.2492492492492p-3;
		p = p * t2 + 0x1.999999999999ap-3;
		p = p * t2 - 0x1.5555555555555p-2;
		r = atanTable[k] + ( t + t * ( t2 * p ) );
		if ( swap )
			r = halfPi - r;
		if ( negX )
			r = pi - r;
	}
	return (float)( negY ? -r : r );
}

B2G_HD bool gbox_contains( b2gBox a, b2gBox b )
{
	return a.lo.x <= b.lo.x && a.lo.y <= b.lo.y && b.hi.x <= a.hi.x && b.hi.y <= a.hi.y;
}
B2G_HD b2gBox gbox_union( b2gBox a, b2gBox b )
{
	b2gBox c;
	c.lo.x = gmin( a.lo.x, b.lo.x );
	c.lo.y = gmin( a.lo.y, b.lo.y );
	c.hi.x = gmax( a.hi.x, b.hi.x );
	c.hi.y = gmax( a.hi.y, b.hi.y );
	return c;
}
B2G_HD bool gbox_overlaps( b2gBox a, b2gBox b )
{
	float d1x = b.lo.x - a.hi.x, d1y = b.lo.y - a.hi.y;
	float d2x = a.lo.x - b.hi.x, d2y = a.lo.y - b.hi.y;
	if ( d1x > 0.0f || d1y > 0.0f )
		return false;
	if ( d2x > 0.0f || d2y > 0.0f )
		return false;
	return true;
}
