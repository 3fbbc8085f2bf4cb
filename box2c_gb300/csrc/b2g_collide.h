/*
 * b2g_collide.h -- contact manifolds, shared by the narrowphase kernel and the public
 * host functions b2Collide* (one source for both).
 *
 * Restates the reference src/manifold.c: b2MakeCapsule (:14-30), b2CollideCircles
 * (:36-70), b2CollideCapsuleAndCircle (:73-135), b2CollidePolygonAndCircle (:137-253),
 * b2ClipPolygons (:276-411), b2FindMaxSeparation (:414-450), b2CollidePolygons
 * (:470-700), with b2SegmentDistance from src/distance.c:32-107.  Feature ids
 * (B2_MAKE_ID, manifold.c:12) and operand order are kept so warm starting matches.
 */
#pragma once

#include "b2g_math.h"
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

/* Manifold of a registered shape pair with A the primary type (reference
 * src/contact.c:150-183): circle=0 capsule=1 segment=2 polygon=3. */
B2G_HD void gcollide_shapes( b2gManifold* m, const b2gShapeGeo* a, b2gXf xfA, const b2gShapeGeo* b, b2gXf xfB )
{
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
