/*
 * b2o_geometry.c -- shapes, mass, bounding boxes and contact manifolds of the plain-C
 * oracle (TEST INFRASTRUCTURE).
 *
 * Restates reference src/geometry.c:127-430 (box makers, mass, AABBs), src/shape.c:
 * 551-630 (extents), src/distance.c:32-107 (segment distance) and src/manifold.c:14-700
 * (circle, capsule and polygon manifolds with the same feature ids and operand order).
 * The public geometry entry points of include/box2d/collision.h are exported from here
 * so scenes built against the oracle get the same polygons as against the reference.
 */
#include "b2o.h"

#include <string.h>

oVec ovf( b2Vec2 v ) { return ov( (b2r)v.x, (b2r)v.y ); }
b2Vec2 vfo( oVec v )
{
	b2Vec2 r = { (float)v.x, (float)v.y };
	return r;
}

#define MAKE_ID( A, B ) ( (uint16_t)( ( (uint8_t)( A ) << 8 ) | (uint8_t)( B ) ) )

/* ------------------------------------------------------------ public geometry API */
b2Polygon b2MakeBox( float hx, float hy )
{
	b2Polygon p;
	memset( &p, 0, sizeof( p ) );
	p.count = 4;
	p.vertices[0] = ( b2Vec2 ){ -hx, -hy };
	p.vertices[1] = ( b2Vec2 ){ hx, -hy };
	p.vertices[2] = ( b2Vec2 ){ hx, hy };
	p.vertices[3] = ( b2Vec2 ){ -hx, hy };
	p.normals[0] = ( b2Vec2 ){ 0.0f, -1.0f };
	p.normals[1] = ( b2Vec2 ){ 1.0f, 0.0f };
	p.normals[2] = ( b2Vec2 ){ 0.0f, 1.0f };
	p.normals[3] = ( b2Vec2 ){ -1.0f, 0.0f };
	return p;
}

b2Polygon b2MakeSquare( float h ) { return b2MakeBox( h, h ); }

b2Polygon b2MakeRoundedBox( float hx, float hy, float radius )
{
	b2Polygon p = b2MakeBox( hx, hy );
	p.radius = radius;
	return p;
}

b2Polygon b2MakeOffsetBox( float hx, float hy, b2Vec2 center, float angle )
{
	b2Transform xf;
	xf.p = center;
	xf.q = b2MakeRot( angle );
	b2Polygon p;
	memset( &p, 0, sizeof( p ) );
	p.count = 4;
	p.vertices[0] = b2TransformPoint( xf, ( b2Vec2 ){ -hx, -hy } );
	p.vertices[1] = b2TransformPoint( xf, ( b2Vec2 ){ hx, -hy } );
	p.vertices[2] = b2TransformPoint( xf, ( b2Vec2 ){ hx, hy } );
	p.vertices[3] = b2TransformPoint( xf, ( b2Vec2 ){ -hx, hy } );
	p.normals[0] = b2RotateVector( xf.q, ( b2Vec2 ){ 0.0f, -1.0f } );
	p.normals[1] = b2RotateVector( xf.q, ( b2Vec2 ){ 1.0f, 0.0f } );
	p.normals[2] = b2RotateVector( xf.q, ( b2Vec2 ){ 0.0f, 1.0f } );
	p.normals[3] = b2RotateVector( xf.q, ( b2Vec2 ){ -1.0f, 0.0f } );
	p.centroid = center;
	return p;
}

b2Polygon b2TransformPolygon( b2Transform transform, const b2Polygon* polygon )
{
	b2Polygon p = *polygon;
	for ( int i = 0; i < p.count; ++i )
	{
		p.vertices[i] = b2TransformPoint( transform, p.vertices[i] );
		p.normals[i] = b2RotateVector( transform.q, p.normals[i] );
	}
	p.centroid = b2TransformPoint( transform, p.centroid );
	return p;
}

/* ------------------------------------------------------------ mass */
typedef struct oMass
{
	b2r mass;
	oVec center;
	b2r I;
} oMass;

static oMass circle_mass( oVec center, b2r radius, b2r density )
{
	b2r rr = radius * radius;
	oMass m;
	m.mass = density * O_PI * rr;
	m.center = center;
	m.I = m.mass * ( R( 0.5f ) * rr + odot( center, center ) );
	return m;
}

static oMass capsule_mass( oVec p1, oVec p2, b2r radius, b2r density )
{
	b2r rr = radius * radius;
	b2r length = olen( osub( p2, p1 ) );
	b2r ll = length * length;
	b2r circleMass = density * ( O_PI * radius * radius );
	b2r boxMass = density * ( R( 2 ) * radius * length );
	oMass m;
	m.mass = circleMass + boxMass;
	m.center = ov( R( 0.5f ) * ( p1.x + p2.x ), R( 0.5f ) * ( p1.y + p2.y ) );
	b2r lc = R( 4 ) * radius / ( R( 3 ) * O_PI );
	b2r h = R( 0.5f ) * length;
	b2r circleInertia = circleMass * ( R( 0.5f ) * rr + h * h + R( 2 ) * h * lc );
	b2r boxInertia = boxMass * ( R( 4 ) * rr + ll ) / R( 12 );
	m.I = circleInertia + boxInertia;
	m.I += m.mass * odot( m.center, m.center );
	return m;
}

static oMass polygon_mass( const oPolygon* s, b2r density )
{
	if ( s->count == 1 )
		return circle_mass( s->v[0], s->radius, density );
	if ( s->count == 2 )
		return capsule_mass( s->v[0], s->v[1], s->radius, density );

	oVec vs[8] = { { 0 } };
	int count = s->count;
	if ( s->radius > R( 0 ) )
	{
		b2r sqrt2 = R( 1.412f );
		for ( int i = 0; i < count; ++i )
		{
			int j = i == 0 ? count - 1 : i - 1;
			oVec mid = onormalize( oadd( s->n[j], s->n[i] ) );
			vs[i] = omuladd( s->v[i], sqrt2 * s->radius, mid );
		}
	}
	else
	{
		for ( int i = 0; i < count; ++i )
			vs[i] = s->v[i];
	}

	oVec center = ov( 0, 0 );
	b2r area = 0, I = 0;
	oVec r = vs[0];
	const b2r inv3 = R( 1.0f ) / R( 3.0f );
	for ( int i = 1; i < count - 1; ++i )
	{
		oVec e1 = osub( vs[i], r );
		oVec e2 = osub( vs[i + 1], r );
		b2r D = ocross( e1, e2 );
		b2r triArea = R( 0.5f ) * D;
		area += triArea;
		center = omuladd( center, triArea * inv3, oadd( e1, e2 ) );
		b2r ex1 = e1.x, ey1 = e1.y, ex2 = e2.x, ey2 = e2.y;
		b2r intx2 = ex1 * ex1 + ex2 * ex1 + ex2 * ex2;
		b2r inty2 = ey1 * ey1 + ey2 * ey1 + ey2 * ey2;
		I += ( R( 0.25f ) * inv3 * D ) * ( intx2 + inty2 );
	}
	oMass m;
	m.mass = density * area;
	b2r invArea = R( 1 ) / area;
	center.x *= invArea;
	center.y *= invArea;
	m.center = oadd( r, center );
	m.I = density * I;
	m.I += m.mass * ( odot( m.center, m.center ) - odot( center, center ) );
	return m;
}

static oPolygon poly_from( const b2Polygon* p )
{
	oPolygon o;
	memset( &o, 0, sizeof( o ) );
	o.count = p->count;
	o.radius = p->radius;
	o.centroid = ovf( p->centroid );
	for ( int i = 0; i < p->count; ++i )
	{
		o.v[i] = ovf( p->vertices[i] );
		o.n[i] = ovf( p->normals[i] );
	}
	return o;
}

static b2MassData mass_out( oMass m )
{
	b2MassData d;
	d.mass = (float)m.mass;
	d.center = vfo( m.center );
	d.rotationalInertia = (float)m.I;
	return d;
}

b2MassData b2ComputePolygonMass( const b2Polygon* shape, float density )
{
	oPolygon p = poly_from( shape );
	return mass_out( polygon_mass( &p, density ) );
}

b2MassData b2ComputeCircleMass( const b2Circle* shape, float density )
{
	return mass_out( circle_mass( ovf( shape->center ), shape->radius, density ) );
}

b2MassData b2ComputeCapsuleMass( const b2Capsule* shape, float density )
{
	return mass_out( capsule_mass( ovf( shape->center1 ), ovf( shape->center2 ), shape->radius, density ) );
}

/* ------------------------------------------------------------ bounding boxes */
static oBox polygon_aabb( const oPolygon* s, oXf xf )
{
	oVec lo = oxfpoint( xf, s->v[0] );
	oVec hi = lo;
	for ( int i = 1; i < s->count; ++i )
	{
		oVec v = oxfpoint( xf, s->v[i] );
		lo = ominv( lo, v );
		hi = omaxv( hi, v );
	}
	oVec r = ov( s->radius, s->radius );
	oBox b = { osub( lo, r ), oadd( hi, r ) };
	return b;
}

oBox o_shape_aabb( const oShape* s, oXf xf )
{
	switch ( s->type )
	{
		case b2_circleShape:
		{
			oVec p = oxfpoint( xf, s->circle.center );
			b2r r = s->circle.radius;
			oBox b = { ov( p.x - r, p.y - r ), ov( p.x + r, p.y + r ) };
			return b;
		}
		case b2_capsuleShape:
		{
			oVec v1 = oxfpoint( xf, s->capsule.c1 );
			oVec v2 = oxfpoint( xf, s->capsule.c2 );
			oVec r = ov( s->capsule.radius, s->capsule.radius );
			oBox b = { osub( ominv( v1, v2 ), r ), oadd( omaxv( v1, v2 ), r ) };
			return b;
		}
		case b2_polygonShape:
			return polygon_aabb( &s->polygon, xf );
		case b2_segmentShape:
		{
			oVec v1 = oxfpoint( xf, s->segment.p1 );
			oVec v2 = oxfpoint( xf, s->segment.p2 );
			oBox b = { ominv( v1, v2 ), omaxv( v1, v2 ) };
			return b;
		}
		case b2_smoothSegmentShape:
		{
			oVec v1 = oxfpoint( xf, s->smooth.p1 );
			oVec v2 = oxfpoint( xf, s->smooth.p2 );
			oBox b = { ominv( v1, v2 ), omaxv( v1, v2 ) };
			return b;
		}
		default:
		{
			oBox b = { xf.p, xf.p };
			return b;
		}
	}
}

static oXf xf_from( b2Transform t )
{
	oXf x;
	x.p = ovf( t.p );
	x.q = orot( t.q.c, t.q.s );
	return x;
}

static b2AABB box_out( oBox b )
{
	b2AABB a;
	a.lowerBound = vfo( b.lo );
	a.upperBound = vfo( b.hi );
	return a;
}

b2AABB b2ComputePolygonAABB( const b2Polygon* shape, b2Transform xf )
{
	oPolygon p = poly_from( shape );
	return box_out( polygon_aabb( &p, xf_from( xf ) ) );
}

b2AABB b2ComputeCircleAABB( const b2Circle* shape, b2Transform xf )
{
	oShape s;
	s.type = b2_circleShape;
	s.circle.center = ovf( shape->center );
	s.circle.radius = shape->radius;
	return box_out( o_shape_aabb( &s, xf_from( xf ) ) );
}

b2AABB b2ComputeCapsuleAABB( const b2Capsule* shape, b2Transform xf )
{
	oShape s;
	s.type = b2_capsuleShape;
	s.capsule.c1 = ovf( shape->center1 );
	s.capsule.c2 = ovf( shape->center2 );
	s.capsule.radius = shape->radius;
	return box_out( o_shape_aabb( &s, xf_from( xf ) ) );
}

b2AABB b2ComputeSegmentAABB( const b2Segment* shape, b2Transform xf )
{
	oShape s;
	s.type = b2_segmentShape;
	s.segment.p1 = ovf( shape->point1 );
	s.segment.p2 = ovf( shape->point2 );
	return box_out( o_shape_aabb( &s, xf_from( xf ) ) );
}

/* ------------------------------------------------------------ body mass update */
typedef struct oExtent
{
	b2r minExtent, maxExtent;
} oExtent;

static oExtent shape_extent( const oShape* s, oVec lc )
{
	oExtent e = { 0, 0 };
	switch ( s->type )
	{
		case b2_capsuleShape:
		{
			b2r r = s->capsule.radius;
			e.minExtent = r;
			oVec c1 = osub( s->capsule.c1, lc );
			oVec c2 = osub( s->capsule.c2, lc );
			e.maxExtent = RSQRT( omax( olen2( c1 ), olen2( c2 ) ) ) + r;
			break;
		}
		case b2_circleShape:
		{
			b2r r = s->circle.radius;
			e.minExtent = r;
			e.maxExtent = olen( osub( s->circle.center, lc ) ) + r;
			break;
		}
		case b2_polygonShape:
		{
			const oPolygon* p = &s->polygon;
			b2r minE = O_HUGE, maxE2 = 0;
			for ( int i = 0; i < p->count; ++i )
			{
				oVec v = p->v[i];
				b2r planeOffset = odot( p->n[i], osub( v, p->centroid ) );
				minE = omin( minE, planeOffset );
				maxE2 = omax( maxE2, olen2( osub( v, lc ) ) );
			}
			e.minExtent = minE + p->radius;
			e.maxExtent = RSQRT( maxE2 ) + p->radius;
			break;
		}
		case b2_segmentShape:
		{
			e.minExtent = 0;
			oVec c1 = osub( s->segment.p1, lc );
			oVec c2 = osub( s->segment.p2, lc );
			e.maxExtent = RSQRT( omax( olen2( c1 ), olen2( c2 ) ) );
			break;
		}
		case b2_smoothSegmentShape:
		{
			e.minExtent = 0;
			oVec c1 = osub( s->smooth.p1, lc );
			oVec c2 = osub( s->smooth.p2, lc );
			e.maxExtent = RSQRT( omax( olen2( c1 ), olen2( c2 ) ) );
			break;
		}
		default:
			break;
	}
	return e;
}

static oMass shape_mass( const oShape* s )
{
	switch ( s->type )
	{
		case b2_capsuleShape:
			return capsule_mass( s->capsule.c1, s->capsule.c2, s->capsule.radius, s->density );
		case b2_circleShape:
			return circle_mass( s->circle.center, s->circle.radius, s->density );
		case b2_polygonShape:
			return polygon_mass( &s->polygon, s->density );
		default:
		{
			oMass m = { 0, { 0, 0 }, 0 };
			return m;
		}
	}
}

/* Reference src/body.c:516-617. */
void o_update_body_mass( oWorld* w, oBody* b )
{
	b->mass = 0;
	b->invMass = 0;
	b->inertia = 0;
	b->invI = 0;
	b->localCenter = ov( 0, 0 );
	b->minExtent = O_HUGE;
	b->maxExtent = 0;

	if ( b->type != b2_dynamicBody )
	{
		b->center = b->xf.p;
		if ( b->type == b2_kinematicBody )
		{
			for ( int sid = b->headShape; sid != O_NULL; sid = w->shapes[sid].next )
			{
				oExtent e = shape_extent( w->shapes + sid, ov( 0, 0 ) );
				b->minExtent = omin( b->minExtent, e.minExtent );
				b->maxExtent = omax( b->maxExtent, e.maxExtent );
			}
		}
		return;
	}

	oVec lc = ov( 0, 0 );
	for ( int sid = b->headShape; sid != O_NULL; sid = w->shapes[sid].next )
	{
		const oShape* s = w->shapes + sid;
		if ( s->density == R( 0 ) )
			continue;
		oMass m = shape_mass( s );
		b->mass += m.mass;
		lc = omuladd( lc, m.mass, m.center );
		b->inertia += m.I;
	}
	if ( b->mass > R( 0 ) )
	{
		b->invMass = R( 1 ) / b->mass;
		lc = omulsv( b->invMass, lc );
	}
	if ( b->inertia > R( 0 ) && b->fixedRotation == false )
	{
		b->inertia -= b->mass * odot( lc, lc );
		b->invI = R( 1 ) / b->inertia;
	}
	else
	{
		b->inertia = 0;
		b->invI = 0;
	}
	oVec oldCenter = b->center;
	b->localCenter = lc;
	b->center = oxfpoint( b->xf, b->localCenter );
	oVec dl = ocross_sv( b->w, osub( b->center, oldCenter ) );
	b->v = oadd( b->v, dl );
	for ( int sid = b->headShape; sid != O_NULL; sid = w->shapes[sid].next )
	{
		oExtent e = shape_extent( w->shapes + sid, lc );
		b->minExtent = omin( b->minExtent, e.minExtent );
		b->maxExtent = omax( b->maxExtent, e.maxExtent );
	}
}

/* ------------------------------------------------------------ segment distance */
oSegDist o_segment_distance( oVec p1, oVec q1, oVec p2, oVec q2 )
{
	oSegDist r;
	memset( &r, 0, sizeof( r ) );
	oVec d1 = osub( q1, p1 );
	oVec d2 = osub( q2, p2 );
	oVec rr = osub( p1, p2 );
	b2r dd1 = odot( d1, d1 );
	b2r dd2 = odot( d2, d2 );
	b2r rd2 = odot( rr, d2 );
	b2r rd1 = odot( rr, d1 );
	const b2r epsSqr = O_EPS * O_EPS;
	if ( dd1 < epsSqr || dd2 < epsSqr )
	{
		if ( dd1 >= epsSqr )
		{
			r.f1 = oclamp( -rd1 / dd1, R( 0 ), R( 1 ) );
			r.f2 = 0;
		}
		else if ( dd2 >= epsSqr )
		{
			r.f1 = 0;
			r.f2 = oclamp( rd2 / dd2, R( 0 ), R( 1 ) );
		}
		else
		{
			r.f1 = 0;
			r.f2 = 0;
		}
	}
	else
	{
		b2r d12 = odot( d1, d2 );
		b2r denom = dd1 * dd2 - d12 * d12;
		b2r f1 = 0;
		if ( denom != R( 0 ) )
			f1 = oclamp( ( d12 * rd2 - rd1 * dd2 ) / denom, R( 0 ), R( 1 ) );
		b2r f2 = ( d12 * f1 + rd2 ) / dd2;
		if ( f2 < R( 0 ) )
		{
			f2 = 0;
			f1 = oclamp( -rd1 / dd1, R( 0 ), R( 1 ) );
		}
		else if ( f2 > R( 1 ) )
		{
			f2 = 1;
			f1 = oclamp( ( d12 - rd1 ) / dd1, R( 0 ), R( 1 ) );
		}
		r.f1 = f1;
		r.f2 = f2;
	}
	r.c1 = omuladd( p1, r.f1, d1 );
	r.c2 = omuladd( p2, r.f2, d2 );
	r.dist2 = odist2( r.c1, r.c2 );
	return r;
}

b2SegmentDistanceResult b2SegmentDistance( b2Vec2 p1, b2Vec2 q1, b2Vec2 p2, b2Vec2 q2 )
{
	oSegDist d = o_segment_distance( ovf( p1 ), ovf( q1 ), ovf( p2 ), ovf( q2 ) );
	b2SegmentDistanceResult r;
	r.closest1 = vfo( d.c1 );
	r.closest2 = vfo( d.c2 );
	r.fraction1 = (float)d.f1;
	r.fraction2 = (float)d.f2;
	r.distanceSquared = (float)d.dist2;
	return r;
}

/* ------------------------------------------------------------ manifolds */
static oManifold empty_manifold( void )
{
	oManifold m;
	memset( &m, 0, sizeof( m ) );
	return m;
}

/* One-point manifold from local contact point `local` (in A's frame) and normal. */
static void finish_one_point( oManifold* m, oXf xfA, oXf xfB, oVec localNormal, oVec contactPointA, b2r separation )
{
	m->normal = orotate( xfA.q, localNormal );
	oMPoint* mp = m->pts;
	mp->anchorA = orotate( xfA.q, contactPointA );
	mp->anchorB = oadd( mp->anchorA, osub( xfA.p, xfB.p ) );
	mp->point = oadd( xfA.p, mp->anchorA );
	mp->separation = separation;
	mp->id = 0;
	m->count = 1;
}

oManifold o_collide_circles( const oCircle* a, oXf xfA, const oCircle* b, oXf xfB )
{
	oManifold m = empty_manifold();
	oXf xf = oinvmulxf( xfA, xfB );
	oVec pA = a->center;
	oVec pB = oxfpoint( xf, b->center );
	b2r distance;
	oVec normal = olen_normalize( &distance, osub( pB, pA ) );
	b2r rA = a->radius, rB = b->radius;
	b2r separation = distance - rA - rB;
	if ( separation > O_SPECULATIVE )
		return m;
	oVec cA = omuladd( pA, rA, normal );
	oVec cB = omuladd( pB, -rB, normal );
	finish_one_point( &m, xfA, xfB, normal, olerp( cA, cB, R( 0.5f ) ), separation );
	return m;
}

oManifold o_collide_capsule_circle( const oCapsule* a, oXf xfA, const oCircle* b, oXf xfB )
{
	oManifold m = empty_manifold();
	oXf xf = oinvmulxf( xfA, xfB );
	oVec pB = oxfpoint( xf, b->center );
	oVec p1 = a->c1, p2 = a->c2;
	oVec e = osub( p2, p1 );
	oVec pA;
	b2r s1 = odot( osub( pB, p1 ), e );
	b2r s2 = odot( osub( p2, pB ), e );
	if ( s1 < R( 0 ) )
		pA = p1;
	else if ( s2 < R( 0 ) )
		pA = p2;
	else
	{
		b2r s = s1 / odot( e, e );
		pA = omuladd( p1, s, e );
	}
	b2r distance;
	oVec normal = olen_normalize( &distance, osub( pB, pA ) );
	b2r rA = a->radius, rB = b->radius;
	b2r separation = distance - rA - rB;
	if ( separation > O_SPECULATIVE )
		return m;
	oVec cA = omuladd( pA, rA, normal );
	oVec cB = omuladd( pB, -rB, normal );
	finish_one_point( &m, xfA, xfB, normal, olerp( cA, cB, R( 0.5f ) ), separation );
	return m;
}

oManifold o_collide_polygon_circle( const oPolygon* a, oXf xfA, const oCircle* b, oXf xfB )
{
	oManifold m = empty_manifold();
	oXf xf = oinvmulxf( xfA, xfB );
	oVec c = oxfpoint( xf, b->center );
	b2r rA = a->radius, rB = b->radius;
	b2r radius = rA + rB;
	int normalIndex = 0;
	b2r separation = -O_MAX;
	for ( int i = 0; i < a->count; ++i )
	{
		b2r s = odot( a->n[i], osub( c, a->v[i] ) );
		if ( s > separation )
		{
			separation = s;
			normalIndex = i;
		}
	}
	if ( separation > radius + O_SPECULATIVE )
		return m;
	int i1 = normalIndex;
	int i2 = i1 + 1 < a->count ? i1 + 1 : 0;
	oVec v1 = a->v[i1], v2 = a->v[i2];
	b2r u1 = odot( osub( c, v1 ), osub( v2, v1 ) );
	b2r u2 = odot( osub( c, v2 ), osub( v1, v2 ) );
	if ( u1 < R( 0 ) && separation > O_EPS )
	{
		oVec normal = onormalize( osub( c, v1 ) );
		separation = odot( osub( c, v1 ), normal );
		if ( separation > radius + O_SPECULATIVE )
			return m;
		oVec cA = omuladd( v1, rA, normal );
		oVec cB = omulsub( c, rB, normal );
		finish_one_point( &m, xfA, xfB, normal, olerp( cA, cB, R( 0.5f ) ), odot( osub( cB, cA ), normal ) );
	}
	else if ( u2 < R( 0 ) && separation > O_EPS )
	{
		oVec normal = onormalize( osub( c, v2 ) );
		separation = odot( osub( c, v2 ), normal );
		if ( separation > radius + O_SPECULATIVE )
			return m;
		oVec cA = omuladd( v2, rA, normal );
		oVec cB = omulsub( c, rB, normal );
		finish_one_point( &m, xfA, xfB, normal, olerp( cA, cB, R( 0.5f ) ), odot( osub( cB, cA ), normal ) );
	}
	else
	{
		oVec normal = a->n[normalIndex];
		oVec cA = omuladd( c, rA - odot( osub( c, v1 ), normal ), normal );
		oVec cB = omulsub( c, rB, normal );
		finish_one_point( &m, xfA, xfB, normal, olerp( cA, cB, R( 0.5f ) ), separation - radius );
	}
	return m;
}

oPolygon o_make_capsule( oVec p1, oVec p2, b2r radius )
{
	oPolygon s;
	memset( &s, 0, sizeof( s ) );
	s.v[0] = p1;
	s.v[1] = p2;
	s.centroid = olerp( p1, p2, R( 0.5f ) );
	oVec axis = onormalize( osub( p2, p1 ) );
	oVec normal = oright( axis );
	s.n[0] = normal;
	s.n[1] = oneg( normal );
	s.count = 2;
	s.radius = radius;
	return s;
}

static b2r find_max_separation( int* edgeIndex, const oPolygon* p1, const oPolygon* p2 )
{
	int best = 0;
	b2r maxSep = -O_MAX;
	for ( int i = 0; i < p1->count; ++i )
	{
		oVec n = p1->n[i];
		oVec v1 = p1->v[i];
		b2r si = O_MAX;
		for ( int j = 0; j < p2->count; ++j )
		{
			b2r sij = odot( n, osub( p2->v[j], v1 ) );
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

static oManifold clip_polygons( const oPolygon* pA, const oPolygon* pB, int edgeA, int edgeB, bool flip )
{
	oManifold m = empty_manifold();
	const oPolygon *poly1, *poly2;
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
	oVec normal = poly1->n[i11];
	oVec v11 = poly1->v[i11], v12 = poly1->v[i12];
	oVec v21 = poly2->v[i21], v22 = poly2->v[i22];
	oVec tangent = ocross_sv( R( 1 ), normal );
	b2r lower1 = 0;
	b2r upper1 = odot( osub( v12, v11 ), tangent );
	b2r upper2 = odot( osub( v21, v11 ), tangent );
	b2r lower2 = odot( osub( v22, v11 ), tangent );
	oVec vLower, vUpper;
	if ( lower2 < lower1 && upper2 - lower2 > O_EPS )
		vLower = olerp( v22, v21, ( lower1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vLower = v22;
	if ( upper2 > upper1 && upper2 - lower2 > O_EPS )
		vUpper = olerp( v22, v21, ( upper1 - lower2 ) / ( upper2 - lower2 ) );
	else
		vUpper = v21;
	b2r sepLower = odot( osub( vLower, v11 ), normal );
	b2r sepUpper = odot( osub( vUpper, v11 ), normal );
	b2r r1 = poly1->radius, r2 = poly2->radius;
	vLower = omuladd( vLower, R( 0.5f ) * ( r1 - r2 - sepLower ), normal );
	vUpper = omuladd( vUpper, R( 0.5f ) * ( r1 - r2 - sepUpper ), normal );
	b2r radius = r1 + r2;
	if ( flip == false )
	{
		m.normal = normal;
		m.pts[0].anchorA = vLower;
		m.pts[0].separation = sepLower - radius;
		m.pts[0].id = MAKE_ID( i11, i22 );
		m.pts[1].anchorA = vUpper;
		m.pts[1].separation = sepUpper - radius;
		m.pts[1].id = MAKE_ID( i12, i21 );
	}
	else
	{
		m.normal = oneg( normal );
		m.pts[0].anchorA = vUpper;
		m.pts[0].separation = sepUpper - radius;
		m.pts[0].id = MAKE_ID( i21, i12 );
		m.pts[1].anchorA = vLower;
		m.pts[1].separation = sepLower - radius;
		m.pts[1].id = MAKE_ID( i22, i11 );
	}
	m.count = 2;
	return m;
}

/* Vertex-vertex contact between local vertices vA (on A) and vB (on B). */
static bool vertex_manifold( oManifold* m, oVec vA, oVec vB, b2r dist2, b2r rA, b2r rB, b2r radius, uint16_t id )
{
	oVec normal = osub( vB, vA );
	b2r distance = RSQRT( dist2 );
	if ( distance > O_SPECULATIVE + radius )
		return false;
	b2r inv = R( 1 ) / distance;
	normal.x *= inv;
	normal.y *= inv;
	oVec c1 = omuladd( vA, rA, normal );
	oVec c2 = omuladd( vB, -rB, normal );
	m->normal = normal;
	m->pts[0].anchorA = olerp( c1, c2, R( 0.5f ) );
	m->pts[0].separation = distance - radius;
	m->pts[0].id = id;
	m->count = 1;
	return true;
}

oManifold o_collide_polygons( const oPolygon* polyA, oXf xfA, const oPolygon* polyB, oXf xfB )
{
	oVec origin = polyA->v[0];
	oXf sfA;
	sfA.p = oadd( xfA.p, orotate( xfA.q, origin ) );
	sfA.q = xfA.q;
	oXf xf = oinvmulxf( sfA, xfB );

	oPolygon A, B;
	A.count = polyA->count;
	A.radius = polyA->radius;
	A.v[0] = ov( 0, 0 );
	A.n[0] = polyA->n[0];
	for ( int i = 1; i < A.count; ++i )
	{
		A.v[i] = osub( polyA->v[i], origin );
		A.n[i] = polyA->n[i];
	}
	B.count = polyB->count;
	B.radius = polyB->radius;
	for ( int i = 0; i < B.count; ++i )
	{
		B.v[i] = oxfpoint( xf, polyB->v[i] );
		B.n[i] = orotate( xf.q, polyB->n[i] );
	}

	int edgeA = 0;
	b2r sepA = find_max_separation( &edgeA, &A, &B );
	int edgeB = 0;
	b2r sepB = find_max_separation( &edgeB, &B, &A );
	b2r radius = A.radius + B.radius;
	if ( sepA > O_SPECULATIVE + radius || sepB > O_SPECULATIVE + radius )
		return empty_manifold();

	bool flip;
	if ( sepA >= sepB )
	{
		flip = false;
		oVec search = A.n[edgeA];
		edgeB = 0;
		b2r minDot = O_MAX;
		for ( int i = 0; i < B.count; ++i )
		{
			b2r d = odot( search, B.n[i] );
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
		oVec search = B.n[edgeB];
		edgeA = 0;
		b2r minDot = O_MAX;
		for ( int i = 0; i < A.count; ++i )
		{
			b2r d = odot( search, A.n[i] );
			if ( d < minDot )
			{
				minDot = d;
				edgeA = i;
			}
		}
	}

	oManifold m = empty_manifold();
	if ( sepA > R( 0.1f ) * O_LINEAR_SLOP || sepB > R( 0.1f ) * O_LINEAR_SLOP )
	{
		int i11 = edgeA;
		int i12 = edgeA + 1 < A.count ? edgeA + 1 : 0;
		int i21 = edgeB;
		int i22 = edgeB + 1 < B.count ? edgeB + 1 : 0;
		oVec v11 = A.v[i11], v12 = A.v[i12], v21 = B.v[i21], v22 = B.v[i22];
		oSegDist r = o_segment_distance( v11, v12, v21, v22 );
		if ( r.f1 == R( 0 ) && r.f2 == R( 0 ) )
		{
			if ( !vertex_manifold( &m, v11, v21, r.dist2, A.radius, B.radius, radius, MAKE_ID( i11, i21 ) ) )
				return m;
		}
		else if ( r.f1 == R( 0 ) && r.f2 == R( 1 ) )
		{
			if ( !vertex_manifold( &m, v11, v22, r.dist2, A.radius, B.radius, radius, MAKE_ID( i11, i22 ) ) )
				return m;
		}
		else if ( r.f1 == R( 1 ) && r.f2 == R( 0 ) )
		{
			if ( !vertex_manifold( &m, v12, v21, r.dist2, A.radius, B.radius, radius, MAKE_ID( i12, i21 ) ) )
				return m;
		}
		else if ( r.f1 == R( 1 ) && r.f2 == R( 1 ) )
		{
			if ( !vertex_manifold( &m, v12, v22, r.dist2, A.radius, B.radius, radius, MAKE_ID( i12, i22 ) ) )
				return m;
		}
		else
		{
			m = clip_polygons( &A, &B, edgeA, edgeB, flip );
		}
	}
	else
	{
		m = clip_polygons( &A, &B, edgeA, edgeB, flip );
	}

	if ( m.count > 0 )
	{
		m.normal = orotate( xfA.q, m.normal );
		for ( int i = 0; i < m.count; ++i )
		{
			oMPoint* mp = m.pts + i;
			mp->anchorA = orotate( xfA.q, oadd( mp->anchorA, origin ) );
			mp->anchorB = oadd( mp->anchorA, osub( xfA.p, xfB.p ) );
			mp->point = oadd( xfA.p, mp->anchorA );
		}
	}
	return m;
}

/* ------------------------------------------------------------ smooth segments
 * Chain links collide on their right side only; the ghost vertices decide which normals a
 * link may produce (reference src/manifold.c:714-1333). */
static oVec o_leftperp( oVec v ) { return ov( -v.y, v.x ); }

oManifold o_collide_smooth_circle( const oSmooth* a, oXf xfA, const oCircle* b, oXf xfB )
{
	oManifold m = empty_manifold();
	oXf xf = oinvmulxf( xfA, xfB );
	oVec pB = oxfpoint( xf, b->center );
	oVec p1 = a->p1;
	oVec p2 = a->p2;
	oVec e = osub( p2, p1 );
	b2r offset = odot( oright( e ), osub( pB, p1 ) );
	if ( offset < R( 0 ) )
		return m;
	b2r u = odot( e, osub( p2, pB ) );
	b2r v = odot( e, osub( pB, p1 ) );
	oVec pA;
	if ( v <= R( 0 ) )
	{
		oVec prevEdge = osub( p1, a->ghost1 );
		b2r uPrev = odot( prevEdge, osub( pB, p1 ) );
		if ( uPrev <= R( 0 ) )
			return m;
		pA = p1;
	}
	else if ( u <= R( 0 ) )
	{
		oVec nextEdge = osub( a->ghost2, p2 );
		b2r vNext = odot( nextEdge, osub( pB, p2 ) );
		if ( vNext > R( 0 ) )
			return m;
		pA = p2;
	}
	else
	{
		b2r ee = odot( e, e );
		pA = ov( u * p1.x + v * p2.x, u * p1.y + v * p2.y );
		pA = ee > R( 0 ) ? omulsv( R( 1 ) / ee, pA ) : p1;
	}
	b2r distance;
	oVec normal = olen_normalize( &distance, osub( pB, pA ) );
	b2r radius = b->radius;
	b2r separation = distance - radius;
	if ( separation > O_SPECULATIVE )
		return m;
	oVec cA = pA;
	oVec cB = omuladd( pB, -radius, normal );
	oVec contactPointA = olerp( cA, cB, R( 0.5f ) );
	m.normal = orotate( xfA.q, normal );
	oMPoint* mp = m.pts + 0;
	mp->anchorA = orotate( xfA.q, contactPointA );
	mp->anchorB = oadd( mp->anchorA, osub( xfA.p, xfB.p ) );
	mp->point = oadd( xfA.p, mp->anchorA );
	mp->separation = separation;
	mp->id = 0;
	m.count = 1;
	return m;
}

static oManifold o_clip_segments( oVec a1, oVec a2, oVec b1, oVec b2, oVec normal, b2r ra, b2r rb, uint16_t id1, uint16_t id2 )
{
	oManifold m = empty_manifold();
	oVec tangent = o_leftperp( normal );
	b2r lower1 = 0;
	b2r upper1 = odot( osub( a2, a1 ), tangent );
	b2r upper2 = odot( osub( b1, a1 ), tangent );
	b2r lower2 = odot( osub( b2, a1 ), tangent );
	if ( upper2 < lower1 || upper1 < lower2 )
		return m;
	oVec vLower = ( lower2 < lower1 && upper2 - lower2 > O_EPS ) ? olerp( b2, b1, ( lower1 - lower2 ) / ( upper2 - lower2 ) ) : b2;
	oVec vUpper = ( upper2 > upper1 && upper2 - lower2 > O_EPS ) ? olerp( b2, b1, ( upper1 - lower2 ) / ( upper2 - lower2 ) ) : b1;
	b2r separationLower = odot( osub( vLower, a1 ), normal );
	b2r separationUpper = odot( osub( vUpper, a1 ), normal );
	vLower = omuladd( vLower, R( 0.5f ) * ( ra - rb - separationLower ), normal );
	vUpper = omuladd( vUpper, R( 0.5f ) * ( ra - rb - separationUpper ), normal );
	b2r radius = ra + rb;
	m.normal = normal;
	m.pts[0].anchorA = vLower;
	m.pts[0].separation = separationLower - radius;
	m.pts[0].id = id1;
	m.pts[1].anchorA = vUpper;
	m.pts[1].separation = separationUpper - radius;
	m.pts[1].id = id2;
	m.count = 2;
	return m;
}

enum
{
	O_NORMAL_SKIP,
	O_NORMAL_ADMIT,
	O_NORMAL_SNAP
};

typedef struct oSmoothParams
{
	oVec edge1, normal0, normal2;
	bool convex1, convex2;
} oSmoothParams;

static int o_classify_normal( const oSmoothParams* p, oVec normal )
{
	const b2r sinTol = R( 0.01f );
	if ( odot( normal, p->edge1 ) <= R( 0 ) )
	{
		if ( p->convex1 )
			return ocross( normal, p->normal0 ) > sinTol ? O_NORMAL_SKIP : O_NORMAL_ADMIT;
		return O_NORMAL_SNAP;
	}
	if ( p->convex2 )
		return ocross( p->normal2, normal ) > sinTol ? O_NORMAL_SKIP : O_NORMAL_ADMIT;
	return O_NORMAL_SNAP;
}

/* frame-A clip result to anchors and points, normal as given (in frame A) */
static void o_smooth_finish( oManifold* m, oXf xfA, oXf xfB, oVec normalA )
{
	m->normal = orotate( xfA.q, normalA );
	m->pts[0].anchorA = orotate( xfA.q, m->pts[0].anchorA );
	m->pts[1].anchorA = orotate( xfA.q, m->pts[1].anchorA );
	oVec pAB = osub( xfA.p, xfB.p );
	m->pts[0].anchorB = oadd( m->pts[0].anchorA, pAB );
	m->pts[1].anchorB = oadd( m->pts[1].anchorA, pAB );
	m->pts[0].point = oadd( xfA.p, m->pts[0].anchorA );
	m->pts[1].point = oadd( xfA.p, m->pts[1].anchorA );
}

#define O_MAKE_ID( A, B ) ( (uint16_t)( ( (uint8_t)( A ) << 8 ) | (uint8_t)( B ) ) )

oManifold o_collide_smooth_polygon( const oSmooth* a, oXf xfA, const oPolygon* b, oXf xfB, oDistCache* cache )
{
	oManifold m = empty_manifold();
	oXf xf = oinvmulxf( xfA, xfB );
	oVec centroidB = oxfpoint( xf, b->centroid );
	b2r radiusB = b->radius;
	oVec p1 = a->p1;
	oVec p2 = a->p2;
	oVec edge1 = onormalize( osub( p2, p1 ) );
	oSmoothParams sp;
	memset( &sp, 0, sizeof( sp ) );
	sp.edge1 = edge1;
	const b2r convexTol = R( 0.01f );
	oVec edge0 = onormalize( osub( p1, a->ghost1 ) );
	sp.normal0 = oright( edge0 );
	sp.convex1 = ocross( edge0, edge1 ) >= convexTol;
	oVec edge2 = onormalize( osub( a->ghost2, p2 ) );
	sp.normal2 = oright( edge2 );
	sp.convex2 = ocross( edge1, edge2 ) >= convexTol;

	oVec normal1 = oright( edge1 );
	bool behind1 = odot( normal1, osub( centroidB, p1 ) ) < R( 0 );
	bool behind0 = true;
	bool behind2 = true;
	if ( sp.convex1 )
		behind0 = odot( sp.normal0, osub( centroidB, p1 ) ) < R( 0 );
	if ( sp.convex2 )
		behind2 = odot( sp.normal2, osub( centroidB, p2 ) ) < R( 0 );
	if ( behind1 && behind0 && behind2 )
		return m;

	int count = b->count;
	oVec vertices[8];
	oVec normals[8];
	for ( int i = 0; i < count; ++i )
	{
		vertices[i] = oxfpoint( xf, b->v[i] );
		normals[i] = orotate( xf.q, b->n[i] );
	}
	oVec segPts[2] = { p1, p2 };
	oProxy proxyA = o_make_proxy( segPts, 2, R( 0 ) );
	oProxy proxyB = o_make_proxy( vertices, count, R( 0 ) );
	oXf identity;
	identity.p = ov( 0, 0 );
	identity.q = orot( 1, 0 );
	oVec pointA, pointB;
	b2r distance = o_distance( cache, &proxyA, identity, &proxyB, identity, &pointA, &pointB );
	if ( distance > radiusB + O_SPECULATIVE )
		return m;

	oVec n0 = sp.convex1 ? sp.normal0 : normal1;
	oVec n2 = sp.convex2 ? sp.normal2 : normal1;
	int incidentIndex = -1;
	int incidentNormal = -1;
	if ( behind1 == false && distance > R( 0.1f ) * O_LINEAR_SLOP )
	{
		if ( cache->count == 1 )
		{
			oVec normal = onormalize( osub( pointB, pointA ) );
			int type = o_classify_normal( &sp, normal );
			if ( type == O_NORMAL_SKIP )
				return m;
			if ( type == O_NORMAL_ADMIT )
			{
				m.normal = orotate( xfA.q, normal );
				oMPoint* cp = m.pts + 0;
				cp->anchorA = orotate( xfA.q, pointA );
				cp->anchorB = oadd( cp->anchorA, osub( xfA.p, xfB.p ) );
				cp->point = oadd( xfA.p, cp->anchorA );
				cp->separation = distance - radiusB;
				cp->id = O_MAKE_ID( cache->indexA[0], cache->indexB[0] );
				m.count = 1;
				return m;
			}
			incidentIndex = cache->indexB[0];
		}
		else
		{
			int ia1 = cache->indexA[0], ia2 = cache->indexA[1];
			int ib1 = cache->indexB[0], ib2 = cache->indexB[1];
			if ( ia1 == ia2 )
			{
				oVec normalB = osub( pointA, pointB );
				b2r dot1 = odot( normalB, normals[ib1] );
				b2r dot2 = odot( normalB, normals[ib2] );
				int ib = dot1 > dot2 ? ib1 : ib2;
				normalB = normals[ib];
				int type = o_classify_normal( &sp, oneg( normalB ) );
				if ( type == O_NORMAL_SKIP )
					return m;
				if ( type == O_NORMAL_ADMIT )
				{
					ib1 = ib;
					ib2 = ib < count - 1 ? ib + 1 : 0;
					oVec b1 = vertices[ib1];
					oVec b2 = vertices[ib2];
					dot1 = odot( normalB, osub( p1, b1 ) );
					dot2 = odot( normalB, osub( p2, b1 ) );
					if ( dot1 < dot2 )
					{
						if ( odot( n0, normalB ) < odot( normal1, normalB ) )
							return m;
					}
					else if ( odot( n2, normalB ) < odot( normal1, normalB ) )
						return m;
					m = o_clip_segments( b1, b2, p1, p2, normalB, radiusB, 0, O_MAKE_ID( ib1, 1 ), O_MAKE_ID( ib2, 0 ) );
					o_smooth_finish( &m, xfA, xfB, oneg( normalB ) );
					return m;
				}
				incidentNormal = ib;
			}
			else
			{
				b2r dot1 = odot( normal1, osub( vertices[ib1], p1 ) );
				b2r dot2 = odot( normal1, osub( vertices[ib2], p2 ) );
				incidentIndex = dot1 < dot2 ? ib1 : ib2;
			}
		}
	}
	else
	{
		b2r edgeSeparation = O_MAX;
		for ( int i = 0; i < count; ++i )
		{
			b2r sep = odot( normal1, osub( vertices[i], p1 ) );
			if ( sep < edgeSeparation )
			{
				edgeSeparation = sep;
				incidentIndex = i;
			}
		}
		if ( sp.convex1 )
		{
			b2r s0 = O_MAX;
			for ( int i = 0; i < count; ++i )
			{
				b2r sep = odot( sp.normal0, osub( vertices[i], p1 ) );
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
			b2r s2 = O_MAX;
			for ( int i = 0; i < count; ++i )
			{
				b2r sep = odot( sp.normal2, osub( vertices[i], p2 ) );
				if ( sep < s2 )
					s2 = sep;
			}
			if ( s2 > edgeSeparation )
			{
				edgeSeparation = s2;
				incidentIndex = -1;
			}
		}
		b2r polygonSeparation = -O_MAX;
		int referenceIndex = -1;
		for ( int i = 0; i < count; ++i )
		{
			oVec n = normals[i];
			if ( o_classify_normal( &sp, oneg( n ) ) != O_NORMAL_ADMIT )
				continue;
			oVec p = vertices[i];
			b2r sep = omin( odot( n, osub( p2, p ) ), odot( n, osub( p1, p ) ) );
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
			oVec a1 = vertices[ia1];
			oVec a2 = vertices[ia2];
			oVec n = normals[ia1];
			b2r dot1 = odot( n, osub( p1, a1 ) );
			b2r dot2 = odot( n, osub( p2, a1 ) );
			if ( dot1 < dot2 )
			{
				if ( odot( n0, n ) < odot( normal1, n ) )
					return m;
			}
			else if ( odot( n2, n ) < odot( normal1, n ) )
				return m;
			m = o_clip_segments( a1, a2, p1, p2, normals[ia1], radiusB, 0, O_MAKE_ID( ia1, 1 ), O_MAKE_ID( ia2, 0 ) );
			o_smooth_finish( &m, xfA, xfB, oneg( normals[ia1] ) );
			return m;
		}
		if ( incidentIndex == -1 )
			return m;
	}

	oVec b1, b2;
	int ib1, ib2;
	if ( incidentNormal != -1 )
	{
		ib1 = incidentNormal;
		ib2 = ib1 < count - 1 ? ib1 + 1 : 0;
	}
	else
	{
		int i2 = incidentIndex;
		int i1 = i2 > 0 ? i2 - 1 : count - 1;
		b2r d1 = odot( normal1, normals[i1] );
		b2r d2 = odot( normal1, normals[i2] );
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
	}
	b1 = vertices[ib1];
	b2 = vertices[ib2];
	m = o_clip_segments( p1, p2, b1, b2, normal1, 0, radiusB, O_MAKE_ID( 0, ib2 ), O_MAKE_ID( 1, ib1 ) );
	o_smooth_finish( &m, xfA, xfB, m.normal );
	return m;
}

/* ------------------------------------------------------------ public manifold API */
static b2Manifold manifold_out( oManifold m )
{
	b2Manifold r;
	memset( &r, 0, sizeof( r ) );
	r.normal = vfo( m.normal );
	r.pointCount = m.count;
	for ( int i = 0; i < 2; ++i )
	{
		r.points[i].point = vfo( m.pts[i].point );
		r.points[i].anchorA = vfo( m.pts[i].anchorA );
		r.points[i].anchorB = vfo( m.pts[i].anchorB );
		r.points[i].separation = (float)m.pts[i].separation;
		r.points[i].id = m.pts[i].id;
	}
	return r;
}

static oCircle circle_from( const b2Circle* c )
{
	oCircle o = { ovf( c->center ), c->radius };
	return o;
}

static oCapsule capsule_from( const b2Capsule* c )
{
	oCapsule o = { ovf( c->center1 ), ovf( c->center2 ), c->radius };
	return o;
}

b2Manifold b2CollideCircles( const b2Circle* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	oCircle ca = circle_from( a ), cb = circle_from( b );
	return manifold_out( o_collide_circles( &ca, xf_from( xfA ), &cb, xf_from( xfB ) ) );
}

b2Manifold b2CollideCapsuleAndCircle( const b2Capsule* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	oCapsule ca = capsule_from( a );
	oCircle cb = circle_from( b );
	return manifold_out( o_collide_capsule_circle( &ca, xf_from( xfA ), &cb, xf_from( xfB ) ) );
}

b2Manifold b2CollideSegmentAndCircle( const b2Segment* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	oCapsule ca = { ovf( a->point1 ), ovf( a->point2 ), 0 };
	oCircle cb = circle_from( b );
	return manifold_out( o_collide_capsule_circle( &ca, xf_from( xfA ), &cb, xf_from( xfB ) ) );
}

b2Manifold b2CollidePolygonAndCircle( const b2Polygon* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	oPolygon pa = poly_from( a );
	oCircle cb = circle_from( b );
	return manifold_out( o_collide_polygon_circle( &pa, xf_from( xfA ), &cb, xf_from( xfB ) ) );
}

b2Manifold b2CollideCapsules( const b2Capsule* a, b2Transform xfA, const b2Capsule* b, b2Transform xfB )
{
	oPolygon pa = o_make_capsule( ovf( a->center1 ), ovf( a->center2 ), a->radius );
	oPolygon pb = o_make_capsule( ovf( b->center1 ), ovf( b->center2 ), b->radius );
	return manifold_out( o_collide_polygons( &pa, xf_from( xfA ), &pb, xf_from( xfB ) ) );
}

b2Manifold b2CollideSegmentAndCapsule( const b2Segment* a, b2Transform xfA, const b2Capsule* b, b2Transform xfB )
{
	oPolygon pa = o_make_capsule( ovf( a->point1 ), ovf( a->point2 ), 0 );
	oPolygon pb = o_make_capsule( ovf( b->center1 ), ovf( b->center2 ), b->radius );
	return manifold_out( o_collide_polygons( &pa, xf_from( xfA ), &pb, xf_from( xfB ) ) );
}

b2Manifold b2CollidePolygonAndCapsule( const b2Polygon* a, b2Transform xfA, const b2Capsule* b, b2Transform xfB )
{
	oPolygon pa = poly_from( a );
	oPolygon pb = o_make_capsule( ovf( b->center1 ), ovf( b->center2 ), b->radius );
	return manifold_out( o_collide_polygons( &pa, xf_from( xfA ), &pb, xf_from( xfB ) ) );
}

b2Manifold b2CollidePolygons( const b2Polygon* a, b2Transform xfA, const b2Polygon* b, b2Transform xfB )
{
	oPolygon pa = poly_from( a ), pb = poly_from( b );
	return manifold_out( o_collide_polygons( &pa, xf_from( xfA ), &pb, xf_from( xfB ) ) );
}

b2Manifold b2CollideSegmentAndPolygon( const b2Segment* a, b2Transform xfA, const b2Polygon* b, b2Transform xfB )
{
	oPolygon pa = o_make_capsule( ovf( a->point1 ), ovf( a->point2 ), 0 );
	oPolygon pb = poly_from( b );
	return manifold_out( o_collide_polygons( &pa, xf_from( xfA ), &pb, xf_from( xfB ) ) );
}

static oSmooth smooth_from( const b2SmoothSegment* a )
{
	oSmooth o;
	o.ghost1 = ovf( a->ghost1 );
	o.p1 = ovf( a->segment.point1 );
	o.p2 = ovf( a->segment.point2 );
	o.ghost2 = ovf( a->ghost2 );
	o.chainId = a->chainId;
	return o;
}

static oDistCache cache_from( const b2DistanceCache* c )
{
	oDistCache o;
	memset( &o, 0, sizeof( o ) );
	if ( c != NULL )
	{
		o.count = c->count;
		for ( int i = 0; i < 3; ++i )
		{
			o.indexA[i] = c->indexA[i];
			o.indexB[i] = c->indexB[i];
		}
	}
	return o;
}

static void cache_to( b2DistanceCache* c, const oDistCache* o )
{
	if ( c == NULL )
		return;
	c->count = (uint16_t)o->count;
	for ( int i = 0; i < 3; ++i )
	{
		c->indexA[i] = (uint8_t)( i < o->count ? o->indexA[i] : 0 );
		c->indexB[i] = (uint8_t)( i < o->count ? o->indexB[i] : 0 );
	}
}

b2Manifold b2CollideSmoothSegmentAndCircle( const b2SmoothSegment* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	oSmooth sa = smooth_from( a );
	oCircle cb = circle_from( b );
	return manifold_out( o_collide_smooth_circle( &sa, xf_from( xfA ), &cb, xf_from( xfB ) ) );
}

b2Manifold b2CollideSmoothSegmentAndCapsule( const b2SmoothSegment* a, b2Transform xfA, const b2Capsule* b, b2Transform xfB,
											 b2DistanceCache* cache )
{
	oSmooth sa = smooth_from( a );
	oPolygon pb = o_make_capsule( ovf( b->center1 ), ovf( b->center2 ), b->radius );
	oDistCache c = cache_from( cache );
	b2Manifold r = manifold_out( o_collide_smooth_polygon( &sa, xf_from( xfA ), &pb, xf_from( xfB ), &c ) );
	cache_to( cache, &c );
	return r;
}

b2Manifold b2CollideSmoothSegmentAndPolygon( const b2SmoothSegment* a, b2Transform xfA, const b2Polygon* b, b2Transform xfB,
											 b2DistanceCache* cache )
{
	oSmooth sa = smooth_from( a );
	oPolygon pb = poly_from( b );
	oDistCache c = cache_from( cache );
	b2Manifold r = manifold_out( o_collide_smooth_polygon( &sa, xf_from( xfA ), &pb, xf_from( xfB ), &c ) );
	cache_to( cache, &c );
	return r;
}
