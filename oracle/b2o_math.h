/*
 * b2o_math.h -- scalar vector math of the plain-C oracle.
 *
 * TEST INFRASTRUCTURE: part of the CPU restatement used only by tests/, the smoke check
 * and the benchmark's CPU baseline.  `b2r` is float by default (bit-exact with the
 * reference) and double when compiled with -DB2O_F64 (the FP64 re-implementation used
 * to check gradients).  Every helper evaluates in the operand order of the matching
 * reference helper in include/box2d/math_functions.h:118-540 and src/math_functions.c:
 * 55-93, with no fused multiply-add (build with -ffp-contract=off).
 */
#pragma once

#include <float.h>
#include <math.h>
#include <stdbool.h>
#include <stdint.h>

#ifdef B2O_F64
typedef double b2r;
	#define RSQRT( x ) sqrt( x )
	#define RATAN2( y, x ) atan2( y, x )
	#define RCOS( x ) cos( x )
	#define RSIN( x ) sin( x )
#elif defined( B2O_OWN_ATAN2 )
typedef float b2r;
	#define RSQRT( x ) sqrtf( x )
	#define RATAN2( y, x ) o_atan2( y, x )
	#define RCOS( x ) cosf( x )
	#define RSIN( x ) sinf( x )
#else
typedef float b2r;
	#define RSQRT( x ) sqrtf( x )
	#define RATAN2( y, x ) atan2f( y, x )
	#define RCOS( x ) cosf( x )
	#define RSIN( x ) sinf( x )
#endif

#define R( x ) ( (b2r)( x ) )

#ifdef B2O_OWN_ATAN2
/* The float build that checks the library on joint springs and limits replaces the C
 * library's atan2f (which the reference calls, and which differs from the device's by a
 * float ulp at times) with the library's own atan2: double evaluation with IEEE
 * operations only; reduction to [0, 1], the arctangent addition formula around the
 * nearest k/8 with a table of atan(k/8), and the Taylor series of atan to t^13 for
 * |t| <= 1/16.  Same operations in the same order as the library's gatan2. */
static inline float o_atan2( float y, float x )
{
	static const double table[9] = { 0.0,
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
	int negX = signbit( x ) != 0, negY = signbit( y ) != 0;
	double r;
	if ( ax == 0.0 && ay == 0.0 )
		r = negX ? pi : 0.0;
	else
	{
		int swap = ay > ax;
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
		r = table[k] + ( t + t * ( t2 * p ) );
		if ( swap )
			r = halfPi - r;
		if ( negX )
			r = pi - r;
	}
	return (float)( negY ? -r : r );
}
#endif
#define O_PI R( 3.14159265359f )
#define O_EPS R( FLT_EPSILON )
#define O_MAX R( FLT_MAX )

/* Tuning constants of the reference src/core.h:110-151 with one length unit per meter. */
#define O_LINEAR_SLOP R( 0.005f )
#define O_SPECULATIVE ( R( 4.0f ) * O_LINEAR_SLOP )
#define O_AABB_MARGIN R( 0.1f )
#define O_MAX_TRANSLATION R( 4.0f )
#define O_MAX_ROTATION ( R( 0.25f ) * O_PI )
#define O_HUGE R( 100000.0f )
#define O_COLORS 12
#define O_OVERFLOW 11
#define O_NULL ( -1 )

typedef struct oVec
{
	b2r x, y;
} oVec;

typedef struct oRot
{
	b2r c, s;
} oRot;

typedef struct oXf
{
	oVec p;
	oRot q;
} oXf;

typedef struct oBox
{
	oVec lo, hi;
} oBox;

static inline oVec ov( b2r x, b2r y )
{
	oVec v = { x, y };
	return v;
}
static inline b2r omin( b2r a, b2r b ) { return a < b ? a : b; }
static inline b2r omax( b2r a, b2r b ) { return a > b ? a : b; }
static inline b2r oabs( b2r a ) { return a < 0 ? -a : a; }
static inline b2r oclamp( b2r a, b2r lo, b2r hi ) { return a < lo ? lo : ( a > hi ? hi : a ); }
static inline b2r odot( oVec a, oVec b ) { return a.x * b.x + a.y * b.y; }
static inline b2r ocross( oVec a, oVec b ) { return a.x * b.y - a.y * b.x; }
static inline oVec ocross_vs( oVec v, b2r s ) { return ov( s * v.y, -s * v.x ); }
static inline oVec ocross_sv( b2r s, oVec v ) { return ov( -s * v.y, s * v.x ); }
static inline oVec oright( oVec v ) { return ov( v.y, -v.x ); }
static inline oVec oadd( oVec a, oVec b ) { return ov( a.x + b.x, a.y + b.y ); }
static inline oVec osub( oVec a, oVec b ) { return ov( a.x - b.x, a.y - b.y ); }
static inline oVec oneg( oVec a ) { return ov( -a.x, -a.y ); }
static inline oVec olerp( oVec a, oVec b, b2r t ) { return ov( ( R( 1 ) - t ) * a.x + t * b.x, ( R( 1 ) - t ) * a.y + t * b.y ); }
static inline oVec omulsv( b2r s, oVec v ) { return ov( s * v.x, s * v.y ); }
static inline oVec omuladd( oVec a, b2r s, oVec b ) { return ov( a.x + s * b.x, a.y + s * b.y ); }
static inline oVec omulsub( oVec a, b2r s, oVec b ) { return ov( a.x - s * b.x, a.y - s * b.y ); }
static inline oVec ominv( oVec a, oVec b ) { return ov( omin( a.x, b.x ), omin( a.y, b.y ) ); }
static inline oVec omaxv( oVec a, oVec b ) { return ov( omax( a.x, b.x ), omax( a.y, b.y ) ); }
static inline b2r olen( oVec v ) { return RSQRT( v.x * v.x + v.y * v.y ); }
static inline b2r olen2( oVec v ) { return v.x * v.x + v.y * v.y; }
static inline b2r odist2( oVec a, oVec b )
{
	oVec c = ov( b.x - a.x, b.y - a.y );
	return c.x * c.x + c.y * c.y;
}

static inline oVec onormalize( oVec v )
{
	b2r length = olen( v );
	if ( length < O_EPS )
		return ov( 0, 0 );
	b2r inv = R( 1 ) / length;
	return ov( inv * v.x, inv * v.y );
}

static inline oVec olen_normalize( b2r* length, oVec v )
{
	*length = olen( v );
	if ( *length < O_EPS )
		return ov( 0, 0 );
	b2r inv = R( 1 ) / *length;
	return ov( inv * v.x, inv * v.y );
}

static inline oRot orot( b2r c, b2r s )
{
	oRot q = { c, s };
	return q;
}
static inline oRot onormrot( oRot q )
{
	b2r mag = RSQRT( q.s * q.s + q.c * q.c );
	b2r inv = mag > R( 0 ) ? R( 1 ) / mag : R( 0 );
	return orot( q.c * inv, q.s * inv );
}
static inline oRot ointrot( oRot q1, b2r da )
{
	oRot q2 = { q1.c - da * q1.s, q1.s + da * q1.c };
	b2r mag = RSQRT( q2.s * q2.s + q2.c * q2.c );
	b2r inv = mag > R( 0 ) ? R( 1 ) / mag : R( 0 );
	return orot( q2.c * inv, q2.s * inv );
}
static inline oRot omulrot( oRot q, oRot r )
{
	oRot qr;
	qr.s = q.s * r.c + q.c * r.s;
	qr.c = q.c * r.c - q.s * r.s;
	return qr;
}
static inline oRot oinvmulrot( oRot q, oRot r )
{
	oRot qr;
	qr.s = q.c * r.s - q.s * r.c;
	qr.c = q.c * r.c + q.s * r.s;
	return qr;
}
static inline b2r orelangle( oRot b, oRot a )
{
	b2r s = b.s * a.c - b.c * a.s;
	b2r c = b.c * a.c + b.s * a.s;
	return RATAN2( s, c );
}
static inline b2r ounwind( b2r a )
{
	if ( a < -O_PI )
		return a + R( 2 ) * O_PI;
	if ( a > O_PI )
		return a - R( 2 ) * O_PI;
	return a;
}
static inline oVec orotate( oRot q, oVec v ) { return ov( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y ); }
static inline oVec oinvrotate( oRot q, oVec v ) { return ov( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y ); }
static inline oVec oxfpoint( oXf t, oVec p )
{
	return ov( ( t.q.c * p.x - t.q.s * p.y ) + t.p.x, ( t.q.s * p.x + t.q.c * p.y ) + t.p.y );
}
static inline oXf oinvmulxf( oXf A, oXf B )
{
	oXf C;
	C.q = oinvmulrot( A.q, B.q );
	C.p = oinvrotate( A.q, osub( B.p, A.p ) );
	return C;
}

static inline bool obox_contains( oBox a, oBox b )
{
	return a.lo.x <= b.lo.x && a.lo.y <= b.lo.y && b.hi.x <= a.hi.x && b.hi.y <= a.hi.y;
}
static inline oVec obox_center( oBox a ) { return ov( R( 0.5f ) * ( a.lo.x + a.hi.x ), R( 0.5f ) * ( a.lo.y + a.hi.y ) ); }
static inline oBox obox_union( oBox a, oBox b )
{
	oBox c;
	c.lo.x = omin( a.lo.x, b.lo.x );
	c.lo.y = omin( a.lo.y, b.lo.y );
	c.hi.x = omax( a.hi.x, b.hi.x );
	c.hi.y = omax( a.hi.y, b.hi.y );
	return c;
}
static inline b2r obox_perimeter( oBox a )
{
	b2r wx = a.hi.x - a.lo.x;
	b2r wy = a.hi.y - a.lo.y;
	return R( 2 ) * ( wx + wy );
}
static inline bool obox_enlarge( oBox* a, oBox b )
{
	bool changed = false;
	if ( b.lo.x < a->lo.x )
	{
		a->lo.x = b.lo.x;
		changed = true;
	}
	if ( b.lo.y < a->lo.y )
	{
		a->lo.y = b.lo.y;
		changed = true;
	}
	if ( a->hi.x < b.hi.x )
	{
		a->hi.x = b.hi.x;
		changed = true;
	}
	if ( a->hi.y < b.hi.y )
	{
		a->hi.y = b.hi.y;
		changed = true;
	}
	return changed;
}
static inline bool obox_overlaps( oBox a, oBox b )
{
	oVec d1 = ov( b.lo.x - a.hi.x, b.lo.y - a.hi.y );
	oVec d2 = ov( a.lo.x - b.hi.x, a.lo.y - b.hi.y );
	if ( d1.x > R( 0 ) || d1.y > R( 0 ) )
		return false;
	if ( d2.x > R( 0 ) || d2.y > R( 0 ) )
		return false;
	return true;
}
