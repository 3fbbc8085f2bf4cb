/*
 * b2g_dual.h -- forward-mode dual numbers and a dual copy of the polygon narrowphase,
 * for the derivatives of a contact manifold with respect to the two bodies' centres
 * and angles (used by the step adjoint).
 *
 * Dual<N> carries a value and N directional derivatives.  Every routine below performs
 * the value arithmetic in the operand order of its b2g_math.h / b2g_collide.h twin, so
 * the values equal the narrowphase's results bit for bit and every branch (reference
 * and incident edge, clipping case, vertex case) goes the same way; the derivative
 * parts differentiate that same piecewise-smooth path.  Restates the reference
 * src/manifold.c b2ClipPolygons (:276-411), b2FindMaxSeparation (:414-450),
 * b2CollidePolygons (:470-700) and src/distance.c b2SegmentDistance (:32-107).
 */
#pragma once

#include "b2g_collide.h"

template <int N>
struct Dual
{
	float v;
	float d[N];
};

template <int N>
__device__ __forceinline__ Dual<N> dc( float v )
{
	Dual<N> r;
	r.v = v;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = 0.0f;
	return r;
}

template <int N>
__device__ __forceinline__ Dual<N> operator+( const Dual<N>& a, const Dual<N>& b )
{
	Dual<N> r;
	r.v = a.v + b.v;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = a.d[i] + b.d[i];
	return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-( const Dual<N>& a, const Dual<N>& b )
{
	Dual<N> r;
	r.v = a.v - b.v;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = a.d[i] - b.d[i];
	return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-( const Dual<N>& a, float b )
{
	Dual<N> r = a;
	r.v = a.v - b;
	return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-( float a, const Dual<N>& b )
{
	Dual<N> r;
	r.v = a - b.v;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = -b.d[i];
	return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-( const Dual<N>& a )
{
	Dual<N> r;
	r.v = -a.v;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = -a.d[i];
	return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*( const Dual<N>& a, const Dual<N>& b )
{
	Dual<N> r;
	r.v = a.v * b.v;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = a.d[i] * b.v + a.v * b.d[i];
	return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*( float s, const Dual<N>& b )
{
	Dual<N> r;
	r.v = s * b.v;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = s * b.d[i];
	return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*( const Dual<N>& a, float s )
{
	Dual<N> r;
	r.v = a.v * s;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = a.d[i] * s;
	return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/( const Dual<N>& a, const Dual<N>& b )
{
	Dual<N> r;
	r.v = a.v / b.v;
	float inv = 1.0f / b.v;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = ( a.d[i] - r.v * b.d[i] ) * inv;
	return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dsqrt( const Dual<N>& a )
{
	Dual<N> r;
	r.v = sqrtf( a.v );
	float k = r.v > 0.0f ? 0.5f / r.v : 0.0f;
#pragma unroll
	for ( int i = 0; i < N; ++i )
		r.d[i] = k * a.d[i];
	return r;
}
/* gclamp( a, lo, hi ) with constant bounds */
template <int N>
__device__ __forceinline__ Dual<N> dclamp01( const Dual<N>& a )
{
	return a.v < 0.0f ? dc<N>( 0.0f ) : ( a.v > 1.0f ? dc<N>( 1.0f ) : a );
}

template <int N>
struct DVec
{
	Dual<N> x, y;
};
template <int N>
struct DRot
{
	Dual<N> c, s;
};
template <int N>
struct DXf
{
	DVec<N> p;
	DRot<N> q;
};

template <int N>
__device__ __forceinline__ DVec<N> dv( const Dual<N>& x, const Dual<N>& y )
{
	DVec<N> r;
	r.x = x;
	r.y = y;
	return r;
}
template <int N>
__device__ __forceinline__ DVec<N> dvc( b2gVec a )
{
	return dv( dc<N>( a.x ), dc<N>( a.y ) );
}
template <int N>
__device__ __forceinline__ Dual<N> ddot( const DVec<N>& a, const DVec<N>& b )
{
	return a.x * b.x + a.y * b.y;
}
template <int N>
__device__ __forceinline__ DVec<N> dadd( const DVec<N>& a, const DVec<N>& b )
{
	return dv( a.x + b.x, a.y + b.y );
}
template <int N>
__device__ __forceinline__ DVec<N> dsub( const DVec<N>& a, const DVec<N>& b )
{
	return dv( a.x - b.x, a.y - b.y );
}
template <int N>
__device__ __forceinline__ DVec<N> dneg( const DVec<N>& a )
{
	return dv( -a.x, -a.y );
}
template <int N>
__device__ __forceinline__ DVec<N> dlerp( const DVec<N>& a, const DVec<N>& b, const Dual<N>& t )
{
	return dv( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y );
}
template <int N>
__device__ __forceinline__ DVec<N> dlerp_f( const DVec<N>& a, const DVec<N>& b, float t )
{
	return dv( ( 1.0f - t ) * a.x + t * b.x, ( 1.0f - t ) * a.y + t * b.y );
}
template <int N>
__device__ __forceinline__ DVec<N> dmuladd( const DVec<N>& a, const Dual<N>& s, const DVec<N>& b )
{
	return dv( a.x + s * b.x, a.y + s * b.y );
}
template <int N>
__device__ __forceinline__ DVec<N> dmuladd_f( const DVec<N>& a, float s, const DVec<N>& b )
{
	return dv( a.x + s * b.x, a.y + s * b.y );
}
template <int N>
__device__ __forceinline__ DVec<N> drotate( const DRot<N>& q, const DVec<N>& v )
{
	return dv( q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y );
}
template <int N>
__device__ __forceinline__ DVec<N> dinvrotate( const DRot<N>& q, const DVec<N>& v )
{
	return dv( q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y );
}
template <int N>
__device__ __forceinline__ DVec<N> dxfpoint( const DXf<N>& t, const DVec<N>& p )
{
	return dv( ( t.q.c * p.x - t.q.s * p.y ) + t.p.x, ( t.q.s * p.x + t.q.c * p.y ) + t.p.y );
}
template <int N>
__device__ __forceinline__ DXf<N> dinvmulxf( const DXf<N>& A, const DXf<N>& B )
{
	DXf<N> C;
	C.q.s = A.q.c * B.q.s - A.q.s * B.q.c;
	C.q.c = A.q.c * B.q.c + A.q.s * B.q.s;
	C.p = dinvrotate( A.q, dsub( B.p, A.p ) );
	return C;
}

template <int N>
struct DPoint
{
	DVec<N> anchorA, anchorB;
	Dual<N> separation;
	uint16_t id;
};

template <int N>
struct DManifold
{
	DPoint<N> pts[2];
	DVec<N> normal;
	int count;
};

template <int N>
struct DPoly
{
	DVec<N> v[8];
	DVec<N> n[8];
	float radius;
	int count;
};

template <int N>
__device__ Dual<N> dfind_max_separation( int* edgeIndex, const DPoly<N>& p1, const DPoly<N>& p2 )
{
	int best = 0;
	Dual<N> maxSep = dc<N>( -FLT_MAX );
	for ( int i = 0; i < p1.count; ++i )
	{
		Dual<N> si = dc<N>( FLT_MAX );
		for ( int j = 0; j < p2.count; ++j )
		{
			Dual<N> sij = ddot( p1.n[i], dsub( p2.v[j], p1.v[i] ) );
			if ( sij.v < si.v )
				si = sij;
		}
		if ( si.v > maxSep.v )
		{
			maxSep = si;
			best = i;
		}
	}
	*edgeIndex = best;
	return maxSep;
}

template <int N>
__device__ void dclip_polygons( DManifold<N>& m, const DPoly<N>& pA, const DPoly<N>& pB, int edgeA, int edgeB, bool flip )
{
	const DPoly<N>* poly1;
	const DPoly<N>* poly2;
	int i11, i12, i21, i22;
	if ( flip )
	{
		poly1 = &pB;
		poly2 = &pA;
		i11 = edgeB;
		i12 = edgeB + 1 < pB.count ? edgeB + 1 : 0;
		i21 = edgeA;
		i22 = edgeA + 1 < pA.count ? edgeA + 1 : 0;
	}
	else
	{
		poly1 = &pA;
		poly2 = &pB;
		i11 = edgeA;
		i12 = edgeA + 1 < pA.count ? edgeA + 1 : 0;
		i21 = edgeB;
		i22 = edgeB + 1 < pB.count ? edgeB + 1 : 0;
	}
	DVec<N> normal = poly1->n[i11];
	DVec<N> v11 = poly1->v[i11], v12 = poly1->v[i12];
	DVec<N> v21 = poly2->v[i21], v22 = poly2->v[i22];
	/* gcross_sv( 1.0f, normal ) */
	DVec<N> tangent = dv( -1.0f * normal.y, 1.0f * normal.x );
	Dual<N> lower1 = dc<N>( 0.0f );
	Dual<N> upper1 = ddot( dsub( v12, v11 ), tangent );
	Dual<N> upper2 = ddot( dsub( v21, v11 ), tangent );
	Dual<N> lower2 = ddot( dsub( v22, v11 ), tangent );
	DVec<N> vLower, vUpper;
	if ( lower2.v < lower1.v && ( upper2 - lower2 ).v > FLT_EPSILON )
		vLower = dlerp( v22, v21, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vLower = v22;
	if ( upper2.v > upper1.v && ( upper2 - lower2 ).v > FLT_EPSILON )
		vUpper = dlerp( v22, v21, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vUpper = v21;
	Dual<N> sepLower = ddot( dsub( vLower, v11 ), normal );
	Dual<N> sepUpper = ddot( dsub( vUpper, v11 ), normal );
	float r1 = poly1->radius, r2 = poly2->radius;
	vLower = dmuladd( vLower, 0.5f * ( ( r1 - r2 ) - sepLower ), normal );
	vUpper = dmuladd( vUpper, 0.5f * ( ( r1 - r2 ) - sepUpper ), normal );
	float radius = r1 + r2;
	if ( flip == false )
	{
		m.normal = normal;
		m.pts[0].anchorA = vLower;
		m.pts[0].separation = sepLower - radius;
		m.pts[0].id = B2G_MAKE_ID( i11, i22 );
		m.pts[1].anchorA = vUpper;
		m.pts[1].separation = sepUpper - radius;
		m.pts[1].id = B2G_MAKE_ID( i12, i21 );
	}
	else
	{
		m.normal = dneg( normal );
		m.pts[0].anchorA = vUpper;
		m.pts[0].separation = sepUpper - radius;
		m.pts[0].id = B2G_MAKE_ID( i21, i12 );
		m.pts[1].anchorA = vLower;
		m.pts[1].separation = sepLower - radius;
		m.pts[1].id = B2G_MAKE_ID( i22, i11 );
	}
	m.count = 2;
}

template <int N>
struct DSegDist
{
	DVec<N> c1, c2;
	Dual<N> f1, f2, dist2;
};

template <int N>
__device__ DSegDist<N> dsegment_distance( const DVec<N>& p1, const DVec<N>& q1, const DVec<N>& p2, const DVec<N>& q2 )
{
	DSegDist<N> r;
	DVec<N> d1 = dsub( q1, p1 );
	DVec<N> d2 = dsub( q2, p2 );
	DVec<N> rr = dsub( p1, p2 );
	Dual<N> dd1 = ddot( d1, d1 );
	Dual<N> dd2 = ddot( d2, d2 );
	Dual<N> rd2 = ddot( rr, d2 );
	Dual<N> rd1 = ddot( rr, d1 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	if ( dd1.v < epsSqr || dd2.v < epsSqr )
	{
		if ( dd1.v >= epsSqr )
		{
			r.f1 = dclamp01( -rd1 / dd1 );
			r.f2 = dc<N>( 0.0f );
		}
		else if ( dd2.v >= epsSqr )
		{
			r.f1 = dc<N>( 0.0f );
			r.f2 = dclamp01( rd2 / dd2 );
		}
		else
		{
			r.f1 = dc<N>( 0.0f );
			r.f2 = dc<N>( 0.0f );
		}
	}
	else
	{
		Dual<N> d12 = ddot( d1, d2 );
		Dual<N> denom = dd1 * dd2 - d12 * d12;
		Dual<N> f1 = dc<N>( 0.0f );
		if ( denom.v != 0.0f )
			f1 = dclamp01( ( d12 * rd2 - rd1 * dd2 ) / denom );
		Dual<N> f2 = ( d12 * f1 + rd2 ) / dd2;
		if ( f2.v < 0.0f )
		{
			f2 = dc<N>( 0.0f );
			f1 = dclamp01( -rd1 / dd1 );
		}
		else if ( f2.v > 1.0f )
		{
			f2 = dc<N>( 1.0f );
			f1 = dclamp01( ( d12 - rd1 ) / dd1 );
		}
		r.f1 = f1;
		r.f2 = f2;
	}
	r.c1 = dmuladd( p1, r.f1, d1 );
	r.c2 = dmuladd( p2, r.f2, d2 );
	DVec<N> c = dv( r.c2.x - r.c1.x, r.c2.y - r.c1.y );
	r.dist2 = c.x * c.x + c.y * c.y;
	return r;
}

template <int N>
__device__ bool dvertex_manifold( DManifold<N>& m, const DVec<N>& vA, const DVec<N>& vB, const Dual<N>& dist2, float rA, float rB,
								  float radius, uint16_t id )
{
	DVec<N> normal = dsub( vB, vA );
	Dual<N> distance = dsqrt( dist2 );
	if ( distance.v > B2G_SPECULATIVE + radius )
		return false;
	Dual<N> inv = dc<N>( 1.0f ) / distance;
	normal.x = normal.x * inv;
	normal.y = normal.y * inv;
	DVec<N> c1 = dmuladd_f( vA, rA, normal );
	DVec<N> c2 = dmuladd_f( vB, -rB, normal );
	m.normal = normal;
	m.pts[0].anchorA = dlerp_f( c1, c2, 0.5f );
	m.pts[0].separation = distance - radius;
	m.pts[0].id = id;
	m.count = 1;
	return true;
}

/* Dual twin of gcollide_polygons: anchors relative to the body origins, as the float
 * routine leaves them (reference src/manifold.c:470-700). */
template <int N>
__device__ void dcollide_polygons( DManifold<N>& m, const b2gPoly& polyA, const DXf<N>& xfA, const b2gPoly& polyB, const DXf<N>& xfB )
{
	m.count = 0;
	b2gVec origin = polyA.v[0];
	DXf<N> sfA;
	sfA.p = dadd( xfA.p, drotate( xfA.q, dvc<N>( origin ) ) );
	sfA.q = xfA.q;
	DXf<N> xf = dinvmulxf( sfA, xfB );

	DPoly<N> A, B;
	A.count = polyA.count;
	A.radius = polyA.radius;
	A.v[0] = dvc<N>( gv( 0.0f, 0.0f ) );
	A.n[0] = dvc<N>( polyA.n[0] );
	for ( int i = 1; i < A.count; ++i )
	{
		A.v[i] = dvc<N>( gsub( polyA.v[i], origin ) );
		A.n[i] = dvc<N>( polyA.n[i] );
	}
	B.count = polyB.count;
	B.radius = polyB.radius;
	for ( int i = 0; i < B.count; ++i )
	{
		B.v[i] = dxfpoint( xf, dvc<N>( polyB.v[i] ) );
		B.n[i] = drotate( xf.q, dvc<N>( polyB.n[i] ) );
	}

	int edgeA = 0;
	Dual<N> sepA = dfind_max_separation( &edgeA, A, B );
	int edgeB = 0;
	Dual<N> sepB = dfind_max_separation( &edgeB, B, A );
	float radius = A.radius + B.radius;
	if ( sepA.v > B2G_SPECULATIVE + radius || sepB.v > B2G_SPECULATIVE + radius )
		return;

	bool flip;
	if ( sepA.v >= sepB.v )
	{
		flip = false;
		DVec<N> search = A.n[edgeA];
		edgeB = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < B.count; ++i )
		{
			float d = ddot( search, B.n[i] ).v;
			if ( d < minDot )
			{
				minDot = d;
				edgeB = i;
			}
		}
	}
	else
	{
		flip = true;
		DVec<N> search = B.n[edgeB];
		edgeA = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < A.count; ++i )
		{
			float d = ddot( search, A.n[i] ).v;
			if ( d < minDot )
			{
				minDot = d;
				edgeA = i;
			}
		}
	}

	if ( sepA.v > 0.1f * B2G_LINEAR_SLOP || sepB.v > 0.1f * B2G_LINEAR_SLOP )
	{
		int i11 = edgeA;
		int i12 = edgeA + 1 < A.count ? edgeA + 1 : 0;
		int i21 = edgeB;
		int i22 = edgeB + 1 < B.count ? edgeB + 1 : 0;
		DVec<N> v11 = A.v[i11], v12 = A.v[i12], v21 = B.v[i21], v22 = B.v[i22];
		DSegDist<N> r = dsegment_distance( v11, v12, v21, v22 );
		bool ok = true;
		if ( r.f1.v == 0.0f && r.f2.v == 0.0f )
			ok = dvertex_manifold( m, v11, v21, r.dist2, A.radius, B.radius, radius, B2G_MAKE_ID( i11, i21 ) );
		else if ( r.f1.v == 0.0f && r.f2.v == 1.0f )
			ok = dvertex_manifold( m, v11, v22, r.dist2, A.radius, B.radius, radius, B2G_MAKE_ID( i11, i22 ) );
		else if ( r.f1.v == 1.0f && r.f2.v == 0.0f )
			ok = dvertex_manifold( m, v12, v21, r.dist2, A.radius, B.radius, radius, B2G_MAKE_ID( i12, i21 ) );
		else if ( r.f1.v == 1.0f && r.f2.v == 1.0f )
			ok = dvertex_manifold( m, v12, v22, r.dist2, A.radius, B.radius, radius, B2G_MAKE_ID( i12, i22 ) );
		else
			dclip_polygons( m, A, B, edgeA, edgeB, flip );
		if ( ok == false )
			return;
	}
	else
		dclip_polygons( m, A, B, edgeA, edgeB, flip );

	if ( m.count > 0 )
	{
		m.normal = drotate( xfA.q, m.normal );
		for ( int i = 0; i < m.count; ++i )
		{
			DPoint<N>* mp = m.pts + i;
			mp->anchorA = drotate( xfA.q, dadd( mp->anchorA, dvc<N>( origin ) ) );
			mp->anchorB = dadd( mp->anchorA, dsub( xfA.p, xfB.p ) );
		}
	}
}

/* ------------------------------------------------------------------ circle manifolds */
/* Dual-number twins of the circle manifolds of b2g_collide.h (reference
 * src/manifold.c:36-250): the same operations in the same order, so the values are the
 * forward manifold's bits and the derivatives follow the chosen branch. */
template <int N>
__device__ __forceinline__ DVec<N> dmulsub_f( const DVec<N>& a, float s, const DVec<N>& b )
{
	return dv( a.x - s * b.x, a.y - s * b.y );
}

template <int N>
__device__ __forceinline__ DVec<N> dlen_normalize( Dual<N>& length, const DVec<N>& v )
{
	length = dsqrt( v.x * v.x + v.y * v.y );
	if ( length.v < FLT_EPSILON )
		return dvc<N>( gv( 0.0f, 0.0f ) );
	Dual<N> inv = dc<N>( 1.0f ) / length;
	return dv( inv * v.x, inv * v.y );
}

template <int N>
__device__ __forceinline__ void done_point( DManifold<N>& m, const DXf<N>& xfA, const DXf<N>& xfB, const DVec<N>& localNormal,
											const DVec<N>& contactPointA, const Dual<N>& separation )
{
	m.normal = drotate( xfA.q, localNormal );
	DPoint<N>* mp = m.pts;
	mp->anchorA = drotate( xfA.q, contactPointA );
	mp->anchorB = dadd( mp->anchorA, dsub( xfA.p, xfB.p ) );
	mp->separation = separation;
	mp->id = 0;
	m.count = 1;
}

/* the closing part of the circle-circle and capsule-circle manifolds, from the closest
 * point pA on A and the circle centre pB (A's frame) */
template <int N>
__device__ __forceinline__ void dround_pair( DManifold<N>& m, const DVec<N>& pA, const DVec<N>& pB, float rA, float rB, const DXf<N>& xfA,
											 const DXf<N>& xfB )
{
	Dual<N> distance;
	DVec<N> normal = dlen_normalize( distance, dsub( pB, pA ) );
	Dual<N> separation = distance - rA - rB;
	if ( separation.v > B2G_SPECULATIVE )
		return;
	DVec<N> cA = dmuladd_f( pA, rA, normal );
	DVec<N> cB = dmuladd_f( pB, -rB, normal );
	done_point( m, xfA, xfB, normal, dlerp_f( cA, cB, 0.5f ), separation );
}

template <int N>
__device__ void dcollide_circles( DManifold<N>& m, b2gVec centerA, float rA, const DXf<N>& xfA, b2gVec centerB, float rB, const DXf<N>& xfB )
{
	m.count = 0;
	DXf<N> xf = dinvmulxf( xfA, xfB );
	DVec<N> pB = dxfpoint( xf, dvc<N>( centerB ) );
	dround_pair( m, dvc<N>( centerA ), pB, rA, rB, xfA, xfB );
}

template <int N>
__device__ void dcollide_capsule_circle( DManifold<N>& m, b2gVec p1, b2gVec p2, float rA, const DXf<N>& xfA, b2gVec centerB, float rB,
										 const DXf<N>& xfB )
{
	m.count = 0;
	DXf<N> xf = dinvmulxf( xfA, xfB );
	DVec<N> pB = dxfpoint( xf, dvc<N>( centerB ) );
	b2gVec e = gsub( p2, p1 );
	DVec<N> E = dvc<N>( e );
	Dual<N> s1 = ddot( dsub( pB, dvc<N>( p1 ) ), E );
	Dual<N> s2 = ddot( dsub( dvc<N>( p2 ), pB ), E );
	DVec<N> pA;
	if ( s1.v < 0.0f )
		pA = dvc<N>( p1 );
	else if ( s2.v < 0.0f )
		pA = dvc<N>( p2 );
	else
	{
		Dual<N> s = s1 / dc<N>( gdot( e, e ) );
		pA = dmuladd( dvc<N>( p1 ), s, E );
	}
	dround_pair( m, pA, pB, rA, rB, xfA, xfB );
}

template <int N>
__device__ void dcollide_polygon_circle( DManifold<N>& m, const b2gPoly& a, const DXf<N>& xfA, b2gVec centerB, float rB, const DXf<N>& xfB )
{
	m.count = 0;
	DXf<N> xf = dinvmulxf( xfA, xfB );
	DVec<N> c = dxfpoint( xf, dvc<N>( centerB ) );
	float rA = a.radius;
	float radius = rA + rB;
	int normalIndex = 0;
	Dual<N> separation = dc<N>( -FLT_MAX );
	for ( int i = 0; i < a.count; ++i )
	{
		Dual<N> s = ddot( dvc<N>( a.n[i] ), dsub( c, dvc<N>( a.v[i] ) ) );
		if ( s.v > separation.v )
		{
			separation = s;
			normalIndex = i;
		}
	}
	if ( separation.v > radius + B2G_SPECULATIVE )
		return;
	int i1 = normalIndex;
	int i2 = i1 + 1 < a.count ? i1 + 1 : 0;
	b2gVec v1 = a.v[i1], v2 = a.v[i2];
	Dual<N> u1 = ddot( dsub( c, dvc<N>( v1 ) ), dvc<N>( gsub( v2, v1 ) ) );
	Dual<N> u2 = ddot( dsub( c, dvc<N>( v2 ) ), dvc<N>( gsub( v1, v2 ) ) );
	if ( ( u1.v < 0.0f && separation.v > FLT_EPSILON ) || ( u2.v < 0.0f && separation.v > FLT_EPSILON ) )
	{
		/* vertex region: the first of the two tests that holds picks the vertex */
		b2gVec v = u1.v < 0.0f ? v1 : v2;
		Dual<N> len;
		DVec<N> d = dsub( c, dvc<N>( v ) );
		DVec<N> normal = dlen_normalize( len, d );
		Dual<N> sep = ddot( d, normal );
		if ( sep.v > radius + B2G_SPECULATIVE )
			return;
		DVec<N> cA = dmuladd_f( dvc<N>( v ), rA, normal );
		DVec<N> cB = dmulsub_f( c, rB, normal );
		done_point( m, xfA, xfB, normal, dlerp_f( cA, cB, 0.5f ), ddot( dsub( cB, cA ), normal ) );
		return;
	}
	DVec<N> normal = dvc<N>( a.n[normalIndex] );
	DVec<N> cA = dmuladd( c, dc<N>( rA ) - ddot( dsub( c, dvc<N>( v1 ) ), normal ), normal );
	DVec<N> cB = dmulsub_f( c, rB, normal );
	done_point( m, xfA, xfB, normal, dlerp_f( cA, cB, 0.5f ), separation - radius );
}
