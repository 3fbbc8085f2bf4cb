/*
 * b2g_collide.h -- contact manifolds, shared by the narrowphase kernel and the public
 * host functions b2Collide* (one source for both).
 *
 * Restates the reference src/manifold.c: b2MakeCapsule (:14-30), b2CollideCircles
 * (:36-70), b2CollideCapsuleAndCircle (:73-135), b2CollidePolygonAndCircle (:137-253),
 * b2ClipPolygons (:276-411), b2FindMaxSeparation (:414-450), b2CollidePolygons
 * (:470-700), the smooth (chain) segment manifolds b2CollideSmoothSegmentAndCircle
 * (:714-800), b2ClipSegments (:809-874), b2ClassifyNormal (:876-934) and
 * b2CollideSmoothSegmentAndPolygon (:944-1333), with b2SegmentDistance from
 * src/distance.c:32-107.  Feature ids (B2_MAKE_ID, manifold.c:12) and operand order are
 * kept so warm starting matches.
 */
#pragma once

#include "b2g_math.h"
#include "b2g_toi.h"
#include "b2g_types.h"

typedef struct b2gPoly
{
	b2gVec v[8];
	b2gVec n[8];
	float radius;
	int count;
} b2gPoly;

typedef struct b2gSegDist
{
	b2gVec c1, c2;
	float f1, f2, dist2;
} b2gSegDist;

#define B2G_MAKE_ID( A, B ) ( (uint16_t)( ( (uint8_t)( A ) << 8 ) | (uint8_t)( B ) ) )

B2G_HD void gmanifold_clear( b2gManifold* m )
{
	for ( int i = 0; i < 2; ++i )
	{
		b2gPoint* p = m->pts + i;
		p->anchorA = gv( 0.0f, 0.0f );
		p->anchorB = gv( 0.0f, 0.0f );
		p->point = gv( 0.0f, 0.0f );
		p->separation = 0.0f;
		p->normalImpulse = 0.0f;
		p->tangentImpulse = 0.0f;
		p->maxNormalImpulse = 0.0f;
		p->normalVelocity = 0.0f;
		p->id = 0;
		p->persisted = 0;
		p->pad = 0;
	}
	m->normal = gv( 0.0f, 0.0f );
	m->count = 0;
}

B2G_HD b2gSegDist gsegment_distance( b2gVec p1, b2gVec q1, b2gVec p2, b2gVec q2 )
{
	b2gSegDist r;
	b2gVec d1 = gsub( q1, p1 );
	b2gVec d2 = gsub( q2, p2 );
	b2gVec rr = gsub( p1, p2 );
	float dd1 = gdot( d1, d1 );
	float dd2 = gdot( d2, d2 );
	float rd2 = gdot( rr, d2 );
	float rd1 = gdot( rr, d1 );
	const float epsSqr = FLT_EPSILON * FLT_EPSILON;
	if ( dd1 < epsSqr || dd2 < epsSqr )
	{
		if ( dd1 >= epsSqr )
		{
			r.f1 = gclamp( -rd1 / dd1, 0.0f, 1.0f );
			r.f2 = 0.0f;
		}
		else if ( dd2 >= epsSqr )
		{
			r.f1 = 0.0f;
			r.f2 = gclamp( rd2 / dd2, 0.0f, 1.0f );
		}
		else
		{
			r.f1 = 0.0f;
			r.f2 = 0.0f;
		}
	}
	else
	{
		float d12 = gdot( d1, d2 );
		float denom = dd1 * dd2 - d12 * d12;
		float f1 = 0.0f;
		if ( denom != 0.0f )
			f1 = gclamp( ( d12 * rd2 - rd1 * dd2 ) / denom, 0.0f, 1.0f );
		float f2 = ( d12 * f1 + rd2 ) / dd2;
		if ( f2 < 0.0f )
		{
			f2 = 0.0f;
			f1 = gclamp( -rd1 / dd1, 0.0f, 1.0f );
		}
		else if ( f2 > 1.0f )
		{
			f2 = 1.0f;
			f1 = gclamp( ( d12 - rd1 ) / dd1, 0.0f, 1.0f );
		}
		r.f1 = f1;
		r.f2 = f2;
	}
	r.c1 = gmuladd( p1, r.f1, d1 );
	r.c2 = gmuladd( p2, r.f2, d2 );
	r.dist2 = gdist2( r.c1, r.c2 );
	return r;
}

B2G_HD void gmake_capsule( b2gPoly* s, b2gVec p1, b2gVec p2, float radius )
{
	s->v[0] = p1;
	s->v[1] = p2;
	b2gVec axis = gnormalize( gsub( p2, p1 ) );
	b2gVec normal = gright( axis );
	s->n[0] = normal;
	s->n[1] = gneg( normal );
	s->count = 2;
	s->radius = radius;
}

/* Writes the single manifold point of the circle-type manifolds. */
B2G_HD void gone_point( b2gManifold* m, b2gXf xfA, b2gXf xfB, b2gVec localNormal, b2gVec contactPointA, float separation )
{
	m->normal = grotate( xfA.q, localNormal );
	b2gPoint* mp = m->pts;
	mp->anchorA = grotate( xfA.q, contactPointA );
	mp->anchorB = gadd( mp->anchorA, gsub( xfA.p, xfB.p ) );
	mp->point = gadd( xfA.p, mp->anchorA );
	mp->separation = separation;
	mp->id = 0;
	m->count = 1;
}

B2G_HD void gcollide_circles( b2gManifold* m, b2gVec centerA, float rA, b2gXf xfA, b2gVec centerB, float rB, b2gXf xfB )
{
	gmanifold_clear( m );
	b2gXf xf = ginvmulxf( xfA, xfB );
	b2gVec pA = centerA;
	b2gVec pB = gxfpoint( xf, centerB );
	float distance;
	b2gVec normal = glen_normalize( &distance, gsub( pB, pA ) );
	float separation = distance - rA - rB;
	if ( separation > B2G_SPECULATIVE )
		return;
	b2gVec cA = gmuladd( pA, rA, normal );
	b2gVec cB = gmuladd( pB, -rB, normal );
	gone_point( m, xfA, xfB, normal, glerp( cA, cB, 0.5f ), separation );
}

B2G_HD void gcollide_capsule_circle( b2gManifold* m, b2gVec p1, b2gVec p2, float rA, b2gXf xfA, b2gVec centerB, float rB,
									b2gXf xfB )
{
	gmanifold_clear( m );
	b2gXf xf = ginvmulxf( xfA, xfB );
	b2gVec pB = gxfpoint( xf, centerB );
	b2gVec e = gsub( p2, p1 );
	b2gVec pA;
	float s1 = gdot( gsub( pB, p1 ), e );
	float s2 = gdot( gsub( p2, pB ), e );
	if ( s1 < 0.0f )
		pA = p1;
	else if ( s2 < 0.0f )
		pA = p2;
	else
	{
		float s = s1 / gdot( e, e );
		pA = gmuladd( p1, s, e );
	}
	float distance;
	b2gVec normal = glen_normalize( &distance, gsub( pB, pA ) );
	float separation = distance - rA - rB;
	if ( separation > B2G_SPECULATIVE )
		return;
	b2gVec cA = gmuladd( pA, rA, normal );
	b2gVec cB = gmuladd( pB, -rB, normal );
	gone_point( m, xfA, xfB, normal, glerp( cA, cB, 0.5f ), separation );
}

B2G_HD void gcollide_polygon_circle( b2gManifold* m, const b2gPoly* a, b2gXf xfA, b2gVec centerB, float rB, b2gXf xfB )
{
	gmanifold_clear( m );
	b2gXf xf = ginvmulxf( xfA, xfB );
	b2gVec c = gxfpoint( xf, centerB );
	float rA = a->radius;
	float radius = rA + rB;
	int normalIndex = 0;
	float separation = -FLT_MAX;
	for ( int i = 0; i < a->count; ++i )
	{
		float s = gdot( a->n[i], gsub( c, a->v[i] ) );
		if ( s > separation )
		{
			separation = s;
			normalIndex = i;
		}
	}
	if ( separation > radius + B2G_SPECULATIVE )
		return;
	int i1 = normalIndex;
	int i2 = i1 + 1 < a->count ? i1 + 1 : 0;
	b2gVec v1 = a->v[i1], v2 = a->v[i2];
	float u1 = gdot( gsub( c, v1 ), gsub( v2, v1 ) );
	float u2 = gdot( gsub( c, v2 ), gsub( v1, v2 ) );
	if ( u1 < 0.0f && separation > FLT_EPSILON )
	{
		b2gVec normal = gnormalize( gsub( c, v1 ) );
		separation = gdot( gsub( c, v1 ), normal );
		if ( separation > radius + B2G_SPECULATIVE )
			return;
		b2gVec cA = gmuladd( v1, rA, normal );
		b2gVec cB = gmulsub( c, rB, normal );
		gone_point( m, xfA, xfB, normal, glerp( cA, cB, 0.5f ), gdot( gsub( cB, cA ), normal ) );
	}
	else if ( u2 < 0.0f && separation > FLT_EPSILON )
	{
		b2gVec normal = gnormalize( gsub( c, v2 ) );
		separation = gdot( gsub( c, v2 ), normal );
		if ( separation > radius + B2G_SPECULATIVE )
			return;
		b2gVec cA = gmuladd( v2, rA, normal );
		b2gVec cB = gmulsub( c, rB, normal );
		gone_point( m, xfA, xfB, normal, glerp( cA, cB, 0.5f ), gdot( gsub( cB, cA ), normal ) );
	}
	else
	{
		b2gVec normal = a->n[normalIndex];
		b2gVec cA = gmuladd( c, rA - gdot( gsub( c, v1 ), normal ), normal );
		b2gVec cB = gmulsub( c, rB, normal );
		gone_point( m, xfA, xfB, normal, glerp( cA, cB, 0.5f ), separation - radius );
	}
}

B2G_HD float gfind_max_separation( int* edgeIndex, const b2gPoly* p1, const b2gPoly* p2 )
{
	int best = 0;
	float maxSep = -FLT_MAX;
	for ( int i = 0; i < p1->count; ++i )
	{
		b2gVec n = p1->n[i];
		b2gVec v1 = p1->v[i];
		float si = FLT_MAX;
		for ( int j = 0; j < p2->count; ++j )
		{
			float sij = gdot( n, gsub( p2->v[j], v1 ) );
			if ( sij < si )
				si = sij;
		}
		if ( si > maxSep )
		{
			maxSep = si;
			best = i;
		}
	}
	*edgeIndex = best;
	return maxSep;
}

B2G_HD void gclip_polygons( b2gManifold* m, const b2gPoly* pA, const b2gPoly* pB, int edgeA, int edgeB, bool flip )
{
	const b2gPoly *poly1, *poly2;
	int i11, i12, i21, i22;
	if ( flip )
	{
		poly1 = pB;
		poly2 = pA;
		i11 = edgeB;
		i12 = edgeB + 1 < pB->count ? edgeB + 1 : 0;
		i21 = edgeA;
		i22 = edgeA + 1 < pA->count ? edgeA + 1 : 0;
	}
	else
	{
		poly1 = pA;
		poly2 = pB;
		i11 = edgeA;
		i12 = edgeA + 1 < pA->count ? edgeA + 1 : 0;
		i21 = edgeB;
		i22 = edgeB + 1 < pB->count ? edgeB + 1 : 0;
	}
	b2gVec normal = poly1->n[i11];
	b2gVec v11 = poly1->v[i11], v12 = poly1->v[i12];
	b2gVec v21 = poly2->v[i21], v22 = poly2->v[i22];
	b2gVec tangent = gcross_sv( 1.0f, normal );
	float lower1 = 0.0f;
	float upper1 = gdot( gsub( v12, v11 ), tangent );
	float upper2 = gdot( gsub( v21, v11 ), tangent );
	float lower2 = gdot( gsub( v22, v11 ), tangent );
	b2gVec vLower, vUpper;
	if ( lower2 < lower1 && upper2 - lower2 > FLT_EPSILON )
		vLower = glerp( v22, v21, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vLower = v22;
	if ( upper2 > upper1 && upper2 - lower2 > FLT_EPSILON )
		vUpper = glerp( v22, v21, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vUpper = v21;
	float sepLower = gdot( gsub( vLower, v11 ), normal );
	float sepUpper = gdot( gsub( vUpper, v11 ), normal );
	float r1 = poly1->radius, r2 = poly2->radius;
	vLower = gmuladd( vLower, 0.5f * ( r1 - r2 - sepLower ), normal );
	vUpper = gmuladd( vUpper, 0.5f * ( r1 - r2 - sepUpper ), normal );
	float radius = r1 + r2;
	if ( flip == false )
	{
		m->normal = normal;
		m->pts[0].anchorA = vLower;
		m->pts[0].separation = sepLower - radius;
		m->pts[0].id = B2G_MAKE_ID( i11, i22 );
		m->pts[1].anchorA = vUpper;
		m->pts[1].separation = sepUpper - radius;
		m->pts[1].id = B2G_MAKE_ID( i12, i21 );
	}
	else
	{
		m->normal = gneg( normal );
		m->pts[0].anchorA = vUpper;
		m->pts[0].separation = sepUpper - radius;
		m->pts[0].id = B2G_MAKE_ID( i21, i12 );
		m->pts[1].anchorA = vLower;
		m->pts[1].separation = sepLower - radius;
		m->pts[1].id = B2G_MAKE_ID( i22, i11 );
	}
	m->count = 2;
}

B2G_HD bool gvertex_manifold( b2gManifold* m, b2gVec vA, b2gVec vB, float dist2, float rA, float rB, float radius, uint16_t id )
{
	b2gVec normal = gsub( vB, vA );
	float distance = sqrtf( dist2 );
	if ( distance > B2G_SPECULATIVE + radius )
		return false;
	float inv = 1.0f / distance;
	normal.x *= inv;
	normal.y *= inv;
	b2gVec c1 = gmuladd( vA, rA, normal );
	b2gVec c2 = gmuladd( vB, -rB, normal );
	m->normal = normal;
	m->pts[0].anchorA = glerp( c1, c2, 0.5f );
	m->pts[0].separation = distance - radius;
	m->pts[0].id = id;
	m->count = 1;
	return true;
}

/* Polygon (or capsule / segment cast as a polygon) against polygon, on the vertex and
 * normal arrays of either a b2gPoly or a polygon shape (no copy of the shapes). */
B2G_HD void gcollide_polygons_raw( b2gManifold* m, const b2gVec* vA, const b2gVec* nA, int countA, float radiusA, b2gXf xfA,
								   const b2gVec* vB, const b2gVec* nB, int countB, float radiusB, b2gXf xfB )
{
	gmanifold_clear( m );
	b2gVec origin = vA[0];
	b2gXf sfA;
	sfA.p = gadd( xfA.p, grotate( xfA.q, origin ) );
	sfA.q = xfA.q;
	b2gXf xf = ginvmulxf( sfA, xfB );

	b2gPoly A, B;
	A.count = countA;
	A.radius = radiusA;
	A.v[0] = gv( 0.0f, 0.0f );
	A.n[0] = nA[0];
	for ( int i = 1; i < A.count; ++i )
	{
		A.v[i] = gsub( vA[i], origin );
		A.n[i] = nA[i];
	}
	B.count = countB;
	B.radius = radiusB;
	for ( int i = 0; i < B.count; ++i )
	{
		B.v[i] = gxfpoint( xf, vB[i] );
		B.n[i] = grotate( xf.q, nB[i] );
	}

	int edgeA = 0;
	float sepA = gfind_max_separation( &edgeA, &A, &B );
	int edgeB = 0;
	float sepB = gfind_max_separation( &edgeB, &B, &A );
	float radius = A.radius + B.radius;
	if ( sepA > B2G_SPECULATIVE + radius || sepB > B2G_SPECULATIVE + radius )
		return;

	bool flip;
	if ( sepA >= sepB )
	{
		flip = false;
		b2gVec search = A.n[edgeA];
		edgeB = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < B.count; ++i )
		{
			float d = gdot( search, B.n[i] );
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
		b2gVec search = B.n[edgeB];
		edgeA = 0;
		float minDot = FLT_MAX;
		for ( int i = 0; i < A.count; ++i )
		{
			float d = gdot( search, A.n[i] );
			if ( d < minDot )
			{
				minDot = d;
				edgeA = i;
			}
		}
	}

	if ( sepA > 0.1f * B2G_LINEAR_SLOP || sepB > 0.1f * B2G_LINEAR_SLOP )
	{
		int i11 = edgeA;
		int i12 = edgeA + 1 < A.count ? edgeA + 1 : 0;
		int i21 = edgeB;
		int i22 = edgeB + 1 < B.count ? edgeB + 1 : 0;
		b2gVec v11 = A.v[i11], v12 = A.v[i12], v21 = B.v[i21], v22 = B.v[i22];
		b2gSegDist r = gsegment_distance( v11, v12, v21, v22 );
		if ( r.f1 == 0.0f && r.f2 == 0.0f )
		{
			if ( !gvertex_manifold( m, v11, v21, r.dist2, A.radius, B.radius, radius, B2G_MAKE_ID( i11, i21 ) ) )
				return;
		}
		else if ( r.f1 == 0.0f && r.f2 == 1.0f )
		{
			if ( !gvertex_manifold( m, v11, v22, r.dist2, A.radius, B.radius, radius, B2G_MAKE_ID( i11, i22 ) ) )
				return;
		}
		else if ( r.f1 == 1.0f && r.f2 == 0.0f )
		{
			if ( !gvertex_manifold( m, v12, v21, r.dist2, A.radius, B.radius, radius, B2G_MAKE_ID( i12, i21 ) ) )
				return;
		}
		else if ( r.f1 == 1.0f && r.f2 == 1.0f )
		{
			if ( !gvertex_manifold( m, v12, v22, r.dist2, A.radius, B.radius, radius, B2G_MAKE_ID( i12, i22 ) ) )
				return;
		}
		else
		{
			gclip_polygons( m, &A, &B, edgeA, edgeB, flip );
		}
	}
	else
	{
		gclip_polygons( m, &A, &B, edgeA, edgeB, flip );
	}

	if ( m->count > 0 )
	{
		m->normal = grotate( xfA.q, m->normal );
		for ( int i = 0; i < m->count; ++i )
		{
			b2gPoint* mp = m->pts + i;
			mp->anchorA = grotate( xfA.q, gadd( mp->anchorA, origin ) );
			mp->anchorB = gadd( mp->anchorA, gsub( xfA.p, xfB.p ) );
			mp->point = gadd( xfA.p, mp->anchorA );
		}
	}
}

B2G_HD void gcollide_polygons( b2gManifold* m, const b2gPoly* polyA, b2gXf xfA, const b2gPoly* polyB, b2gXf xfB )
{
	gcollide_polygons_raw( m, polyA->v, polyA->n, polyA->count, polyA->radius, xfA, polyB->v, polyB->n, polyB->count, polyB->radius,
						   xfB );
}

/* Shape as a polygon for the polygon path: capsules and segments become 2-gons. */
B2G_HD void gshape_poly( b2gPoly* p, const b2gShapeGeo* g )
{
	if ( g->type == 3 /* polygon */ )
	{
		p->count = g->count;
		p->radius = g->radius;
		for ( int i = 0; i < g->count; ++i )
		{
			p->v[i] = g->v[i];
			p->n[i] = g->n[i];
		}
	}
	else
	{
		/* capsule (radius) or segment (radius 0) */
		gmake_capsule( p, g->v[0], g->v[1], g->type == 1 ? g->radius : 0.0f );
	}
}

/* ------------------------------------------------------------ smooth segments
 * A smooth segment (a link of a chain) collides on its right side only, and its ghost
 * vertices (the neighbouring links' far ends) decide which normals it may produce. */
typedef struct b2gSmooth
{
	b2gVec ghost1, p1, p2, ghost2;
} b2gSmooth;

B2G_HD b2gSmooth gsmooth_of( const b2gShapeGeo* g )
{
	b2gSmooth s;
	s.p1 = g->v[0];
	s.p2 = g->v[1];
	s.ghost1 = g->v[2];
	s.ghost2 = g->v[3];
	return s;
}

B2G_HD void gcollide_smooth_circle( b2gManifold* m, const b2gSmooth* sA, b2gXf xfA, b2gVec centerB, float radiusB, b2gXf xfB )
{
	gmanifold_clear( m );
	b2gXf xf = ginvmulxf( xfA, xfB );
	b2gVec pB = gxfpoint( xf, centerB );
	b2gVec p1 = sA->p1;
	b2gVec p2 = sA->p2;
	b2gVec e = gsub( p2, p1 );
	float offset = gdot( gright( e ), gsub( pB, p1 ) );
	if ( offset < 0.0f )
		return;
	float u = gdot( e, gsub( p2, pB ) );
	float v = gdot( e, gsub( pB, p1 ) );
	b2gVec pA;
	if ( v <= 0.0f )
	{
		b2gVec prevEdge = gsub( p1, sA->ghost1 );
		float uPrev = gdot( prevEdge, gsub( pB, p1 ) );
		if ( uPrev <= 0.0f )
			return;
		pA = p1;
	}
	else if ( u <= 0.0f )
	{
		b2gVec nextEdge = gsub( sA->ghost2, p2 );
		float vNext = gdot( nextEdge, gsub( pB, p2 ) );
		if ( vNext > 0.0f )
			return;
		pA = p2;
	}
	else
	{
		float ee = gdot( e, e );
		pA = gv( u * p1.x + v * p2.x, u * p1.y + v * p2.y );
		pA = ee > 0.0f ? gmulsv( 1.0f / ee, pA ) : p1;
	}
	float distance;
	b2gVec normal = glen_normalize( &distance, gsub( pB, pA ) );
	float separation = distance - radiusB;
	if ( separation > B2G_SPECULATIVE )
		return;
	b2gVec cA = pA;
	b2gVec cB = gmuladd( pB, -radiusB, normal );
	b2gVec contactPointA = glerp( cA, cB, 0.5f );
	m->normal = grotate( xfA.q, normal );
	b2gPoint* mp = m->pts + 0;
	mp->anchorA = grotate( xfA.q, contactPointA );
	mp->anchorB = gadd( mp->anchorA, gsub( xfA.p, xfB.p ) );
	mp->point = gadd( xfA.p, mp->anchorA );
	mp->separation = separation;
	mp->id = 0;
	m->count = 1;
}

/* Two-point manifold of segment a1-a2 (reference side) against b1-b2 (incident, opposite
 * winding), points at the midpoints accounting for the radii, in frame A. */
B2G_HD void gclip_segments( b2gManifold* m, b2gVec a1, b2gVec a2, b2gVec b1, b2gVec b2, b2gVec normal, float ra, float rb, uint16_t id1,
							uint16_t id2 )
{
	gmanifold_clear( m );
	b2gVec tangent = gleft( normal );
	float lower1 = 0.0f;
	float upper1 = gdot( gsub( a2, a1 ), tangent );
	float upper2 = gdot( gsub( b1, a1 ), tangent );
	float lower2 = gdot( gsub( b2, a1 ), tangent );
	if ( upper2 < lower1 || upper1 < lower2 )
		return;
	b2gVec vLower;
	if ( lower2 < lower1 && upper2 - lower2 > FLT_EPSILON )
		vLower = glerp( b2, b1, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vLower = b2;
	b2gVec vUpper;
	if ( upper2 > upper1 && upper2 - lower2 > FLT_EPSILON )
		vUpper = glerp( b2, b1, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vUpper = b1;
	float separationLower = gdot( gsub( vLower, a1 ), normal );
	float separationUpper = gdot( gsub( vUpper, a1 ), normal );
	vLower = gmuladd( vLower, 0.5f * ( ra - rb - separationLower ), normal );
	vUpper = gmuladd( vUpper, 0.5f * ( ra - rb - separationUpper ), normal );
	float radius = ra + rb;
	m->normal = normal;
	m->pts[0].anchorA = vLower;
	m->pts[0].separation = separationLower - radius;
	m->pts[0].id = id1;
	m->pts[1].anchorA = vUpper;
	m->pts[1].separation = separationUpper - radius;
	m->pts[1].id = id2;
	m->count = 2;
}

enum
{
	B2G_NORMAL_SKIP = 0,
	B2G_NORMAL_ADMIT = 1,
	B2G_NORMAL_SNAP = 2,
};

typedef struct b2gSmoothParams
{
	b2gVec edge1, normal0, normal2;
	bool convex1, convex2;
} b2gSmoothParams;

/* Gauss-map test of a candidate normal against the neighbouring links. */
B2G_HD int gclassify_normal( const b2gSmoothParams* params, b2gVec normal )
{
	const float sinTol = 0.01f;
	if ( gdot( normal, params->edge1 ) <= 0.0f )
	{
		if ( params->convex1 )
		{
			if ( gcross( normal, params->normal0 ) > sinTol )
				return B2G_NORMAL_SKIP;
			return B2G_NORMAL_ADMIT;
		}
		return B2G_NORMAL_SNAP;
	}
	if ( params->convex2 )
	{
		if ( gcross( params->normal2, normal ) > sinTol )
			return B2G_NORMAL_SKIP;
		return B2G_NORMAL_ADMIT;
	}
	return B2G_NORMAL_SNAP;
}

/* The frame-A manifold of a clip to world anchors and points. */
B2G_HD void gsmooth_finish( b2gManifold* m, b2gXf xfA, b2gXf xfB, b2gVec normalA )
{
	m->normal = grotate( xfA.q, normalA );
	m->pts[0].anchorA = grotate( xfA.q, m->pts[0].anchorA );
	m->pts[1].anchorA = grotate( xfA.q, m->pts[1].anchorA );
	b2gVec pAB = gsub( xfA.p, xfB.p );
	m->pts[0].anchorB = gadd( m->pts[0].anchorA, pAB );
	m->pts[1].anchorB = gadd( m->pts[1].anchorA, pAB );
	m->pts[0].point = gadd( xfA.p, m->pts[0].anchorA );
	m->pts[1].point = gadd( xfA.p, m->pts[1].anchorA );
}

/* Smooth segment against a polygon (capsules enter as rounded 2-gons); `cache` is the
 * contact's closest-feature cache, read and updated. */
B2G_HD void gcollide_smooth_polygon( b2gManifold* m, const b2gSmooth* sA, b2gXf xfA, const b2gVec* vB, const b2gVec* nB, int count,
									 float radiusB, b2gVec centroidB0, b2gXf xfB, b2gDistCache* cache )
{
	gmanifold_clear( m );
	b2gXf xf = ginvmulxf( xfA, xfB );
	b2gVec centroidB = gxfpoint( xf, centroidB0 );
	b2gVec p1 = sA->p1;
	b2gVec p2 = sA->p2;
	b2gVec edge1 = gnormalize( gsub( p2, p1 ) );

	b2gSmoothParams sp;
	sp.edge1 = edge1;
	const float convexTol = 0.01f;
	b2gVec edge0 = gnormalize( gsub( p1, sA->ghost1 ) );
	sp.normal0 = gright( edge0 );
	sp.convex1 = gcross( edge0, edge1 ) >= convexTol;
	b2gVec edge2 = gnormalize( gsub( sA->ghost2, p2 ) );
	sp.normal2 = gright( edge2 );
	sp.convex2 = gcross( edge1, edge2 ) >= convexTol;

	b2gVec normal1 = gright( edge1 );
	bool behind1 = gdot( normal1, gsub( centroidB, p1 ) ) < 0.0f;
	bool behind0 = true;
	bool behind2 = true;
	if ( sp.convex1 )
		behind0 = gdot( sp.normal0, gsub( centroidB, p1 ) ) < 0.0f;
	if ( sp.convex2 )
		behind2 = gdot( sp.normal2, gsub( centroidB, p2 ) ) < 0.0f;
	if ( behind1 && behind0 && behind2 )
		return;

	b2gVec vertices[8];
	b2gVec normals[8];
	for ( int i = 0; i < count; ++i )
	{
		vertices[i] = gxfpoint( xf, vB[i] );
		normals[i] = grotate( xf.q, nB[i] );
	}

	b2gVec segPts[2] = { p1, p2 };
	b2gProxy proxyA = gproxy_points( segPts, 2, 0.0f );
	b2gProxy proxyB = gproxy_points( vertices, count, 0.0f );
	b2gXf identity;
	identity.p = gv( 0.0f, 0.0f );
	identity.q = grot( 1.0f, 0.0f );
	b2gVec pointA, pointB;
	float distance = gdistance_points( cache, &proxyA, identity, &proxyB, identity, &pointA, &pointB );
	if ( distance > radiusB + B2G_SPECULATIVE )
		return;

	b2gVec n0 = sp.convex1 ? sp.normal0 : normal1;
	b2gVec n2 = sp.convex2 ? sp.normal2 : normal1;
	int incidentIndex = -1;
	int incidentNormal = -1;

	if ( behind1 == false && distance > 0.1f * B2G_LINEAR_SLOP )
	{
		if ( cache->count == 1 )
		{
			/* vertex-vertex */
			b2gVec pA = pointA;
			b2gVec pB = pointB;
			b2gVec normal = gnormalize( gsub( pB, pA ) );
			int type = gclassify_normal( &sp, normal );
			if ( type == B2G_NORMAL_SKIP )
				return;
			if ( type == B2G_NORMAL_ADMIT )
			{
				m->normal = grotate( xfA.q, normal );
				b2gPoint* cp = m->pts + 0;
				cp->anchorA = grotate( xfA.q, pA );
				cp->anchorB = gadd( cp->anchorA, gsub( xfA.p, xfB.p ) );
				cp->point = gadd( xfA.p, cp->anchorA );
				cp->separation = distance - radiusB;
				cp->id = B2G_MAKE_ID( cache->indexA[0], cache->indexB[0] );
				m->count = 1;
				return;
			}
			incidentIndex = cache->indexB[0];
		}
		else
		{
			/* vertex-edge */
			int ia1 = cache->indexA[0];
			int ia2 = cache->indexA[1];
			int ib1 = cache->indexB[0];
			int ib2 = cache->indexB[1];
			if ( ia1 == ia2 )
			{
				/* one point on A, two on B */
				b2gVec normalB = gsub( pointA, pointB );
				float dot1 = gdot( normalB, normals[ib1] );
				float dot2 = gdot( normalB, normals[ib2] );
				int ib = dot1 > dot2 ? ib1 : ib2;
				normalB = normals[ib];
				int type = gclassify_normal( &sp, gneg( normalB ) );
				if ( type == B2G_NORMAL_SKIP )
					return;
				if ( type == B2G_NORMAL_ADMIT )
				{
					ib1 = ib;
					ib2 = ib < count - 1 ? ib + 1 : 0;
					b2gVec b1 = vertices[ib1];
					b2gVec b2 = vertices[ib2];
					dot1 = gdot( normalB, gsub( p1, b1 ) );
					dot2 = gdot( normalB, gsub( p2, b1 ) );
					if ( dot1 < dot2 )
					{
						if ( gdot( n0, normalB ) < gdot( normal1, normalB ) )
							return;
					}
					else
					{
						if ( gdot( n2, normalB ) < gdot( normal1, normalB ) )
							return;
					}
					gclip_segments( m, b1, b2, p1, p2, normalB, radiusB, 0.0f, B2G_MAKE_ID( ib1, 1 ), B2G_MAKE_ID( ib2, 0 ) );
					gsmooth_finish( m, xfA, xfB, gneg( normalB ) );
					return;
				}
				incidentNormal = ib;
			}
			else
			{
				float dot1 = gdot( normal1, gsub( vertices[ib1], p1 ) );
				float dot2 = gdot( normal1, gsub( vertices[ib2], p2 ) );
				incidentIndex = dot1 < dot2 ? ib1 : ib2;
			}
		}
	}
	else
	{
		/* SAT: the segment normal */
		float edgeSeparation = FLT_MAX;
		for ( int i = 0; i < count; ++i )
		{
			float sep = gdot( normal1, gsub( vertices[i], p1 ) );
			if ( sep < edgeSeparation )
			{
				edgeSeparation = sep;
				incidentIndex = i;
			}
		}
		/* convex neighbours */
		if ( sp.convex1 )
		{
			float s0 = FLT_MAX;
			for ( int i = 0; i < count; ++i )
			{
				float sep = gdot( sp.normal0, gsub( vertices[i], p1 ) );
				if ( sep < s0 )
					s0 = sep;
			}
			if ( s0 > edgeSeparation )
			{
				edgeSeparation = s0;
				incidentIndex = -1;
			}
		}
		if ( sp.convex2 )
		{
			float s2 = FLT_MAX;
			for ( int i = 0; i < count; ++i )
			{
				float sep = gdot( sp.normal2, gsub( vertices[i], p2 ) );
				if ( sep < s2 )
					s2 = sep;
			}
			if ( s2 > edgeSeparation )
			{
				edgeSeparation = s2;
				incidentIndex = -1;
			}
		}
		/* SAT: the polygon's admitted normals */
		float polygonSeparation = -FLT_MAX;
		int referenceIndex = -1;
		for ( int i = 0; i < count; ++i )
		{
			b2gVec n = normals[i];
			int type = gclassify_normal( &sp, gneg( n ) );
			if ( type != B2G_NORMAL_ADMIT )
				continue;
			b2gVec p = vertices[i];
			float sep = gmin( gdot( n, gsub( p2, p ) ), gdot( n, gsub( p1, p ) ) );
			if ( sep > polygonSeparation )
			{
				polygonSeparation = sep;
				referenceIndex = i;
			}
		}
		if ( polygonSeparation > edgeSeparation )
		{
			int ia1 = referenceIndex;
			int ia2 = ia1 < count - 1 ? ia1 + 1 : 0;
			b2gVec a1 = vertices[ia1];
			b2gVec a2 = vertices[ia2];
			b2gVec n = normals[ia1];
			float dot1 = gdot( n, gsub( p1, a1 ) );
			float dot2 = gdot( n, gsub( p2, a1 ) );
			if ( dot1 < dot2 )
			{
				if ( gdot( n0, n ) < gdot( normal1, n ) )
					return;
			}
			else
			{
				if ( gdot( n2, n ) < gdot( normal1, n ) )
					return;
			}
			gclip_segments( m, a1, a2, p1, p2, normals[ia1], radiusB, 0.0f, B2G_MAKE_ID( ia1, 1 ), B2G_MAKE_ID( ia2, 0 ) );
			gsmooth_finish( m, xfA, xfB, gneg( normals[ia1] ) );
			return;
		}
		if ( incidentIndex == -1 )
			return;
	}

	/* the segment normal is the reference: find the incident polygon edge */
	b2gVec b1, b2;
	int ib1, ib2;
	if ( incidentNormal != -1 )
	{
		ib1 = incidentNormal;
		ib2 = ib1 < count - 1 ? ib1 + 1 : 0;
		b1 = vertices[ib1];
		b2 = vertices[ib2];
	}
	else
	{
		int i2 = incidentIndex;
		int i1 = i2 > 0 ? i2 - 1 : count - 1;
		float d1 = gdot( normal1, normals[i1] );
		float d2 = gdot( normal1, normals[i2] );
		if ( d1 < d2 )
		{
			ib1 = i1;
			ib2 = i2;
		}
		else
		{
			ib1 = i2;
			ib2 = i2 < count - 1 ? i2 + 1 : 0;
		}
		b1 = vertices[ib1];
		b2 = vertices[ib2];
	}
	gclip_segments( m, p1, p2, b1, b2, normal1, 0.0f, radiusB, B2G_MAKE_ID( 0, ib2 ), B2G_MAKE_ID( 1, ib1 ) );
	gsmooth_finish( m, xfA, xfB, m->normal );
}

/* Manifold of a registered shape pair with A the primary type (reference
 * src/contact.c:150-183): circle=0 capsule=1 segment=2 polygon=3 smooth segment=4.
 * `cache` (smooth segments only) is the contact's closest-feature cache. */
B2G_HD void gcollide_shapes( b2gManifold* m, const b2gShapeGeo* a, b2gXf xfA, const b2gShapeGeo* b, b2gXf xfB,
							 b2gDistCache* cache )
{
	if ( a->type == 4 )
	{
		b2gSmooth sa = gsmooth_of( a );
		if ( b->type == 0 )
			gcollide_smooth_circle( m, &sa, xfA, b->v[0], b->radius, xfB );
		else
		{
			/* polygon, or a capsule as a rounded 2-gon (reference b2MakeCapsule) */
			b2gPoly pb;
			gshape_poly( &pb, b );
			b2gVec centroid = b->type == 3 ? b->centroid : glerp( b->v[0], b->v[1], 0.5f );
			gcollide_smooth_polygon( m, &sa, xfA, pb.v, pb.n, pb.count, pb.radius, centroid, xfB, cache );
		}
		return;
	}
	if ( b->type == 0 )
	{
		/* B is a circle */
		if ( a->type == 0 )
			gcollide_circles( m, a->v[0], a->radius, xfA, b->v[0], b->radius, xfB );
		else if ( a->type == 1 )
			gcollide_capsule_circle( m, a->v[0], a->v[1], a->radius, xfA, b->v[0], b->radius, xfB );
		else if ( a->type == 2 )
			gcollide_capsule_circle( m, a->v[0], a->v[1], 0.0f, xfA, b->v[0], b->radius, xfB );
		else
		{
			b2gPoly pa;
			gshape_poly( &pa, a );
			gcollide_polygon_circle( m, &pa, xfA, b->v[0], b->radius, xfB );
		}
		return;
	}
	if ( a->type == 3 && b->type == 3 )
	{
		gcollide_polygons_raw( m, a->v, a->n, a->count, a->radius, xfA, b->v, b->n, b->count, b->radius, xfB );
		return;
	}
	b2gPoly pa, pb;
	gshape_poly( &pa, a );
	gshape_poly( &pb, b );
	gcollide_polygons( m, &pa, xfA, &pb, xfB );
}
