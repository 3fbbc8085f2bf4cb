/*
 * geometry.c -- public geometry, mass, bounding-box and manifold functions of
 * include/box2d/collision.h, computed on the host with the same source the device
 * narrowphase uses (b2g_collide.h).
 *
 * Mass and extents restate reference src/geometry.c:196-372 and src/shape.c:551-630;
 * box makers src/geometry.c:127-178.
 */
#include "host.h"

#include "b2g_collide.h"

#include <string.h>

static b2gVec gvf( b2Vec2 v ) { return gv( v.x, v.y ); }
static b2Vec2 vfg( b2gVec v )
{
	b2Vec2 r = { v.x, v.y };
	return r;
}
static b2gXf xf_of( b2Transform t )
{
	b2gXf x;
	x.p = gvf( t.p );
	x.q = grot( t.q.c, t.q.s );
	return x;
}

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
static b2MassData circle_mass( b2gVec center, float radius, float density )
{
	float rr = radius * radius;
	b2MassData m;
	m.mass = density * B2G_PI * rr;
	m.center = vfg( center );
	m.rotationalInertia = m.mass * ( 0.5f * rr + gdot( center, center ) );
	return m;
}

static b2MassData capsule_mass( b2gVec p1, b2gVec p2, float radius, float density )
{
	float rr = radius * radius;
	float length = glen( gsub( p2, p1 ) );
	float ll = length * length;
	float circleMass = density * ( B2G_PI * radius * radius );
	float boxMass = density * ( 2.0f * radius * length );
	b2MassData m;
	m.mass = circleMass + boxMass;
	b2gVec c = gv( 0.5f * ( p1.x + p2.x ), 0.5f * ( p1.y + p2.y ) );
	m.center = vfg( c );
	float lc = 4.0f * radius / ( 3.0f * B2G_PI );
	float h = 0.5f * length;
	float circleInertia = circleMass * ( 0.5f * rr + h * h + 2.0f * h * lc );
	float boxInertia = boxMass * ( 4.0f * rr + ll ) / 12.0f;
	m.rotationalInertia = circleInertia + boxInertia;
	m.rotationalInertia += m.mass * gdot( c, c );
	return m;
}

static b2MassData polygon_mass( const b2gShapeGeo* s, float density )
{
	if ( s->count == 1 )
		return circle_mass( s->v[0], s->radius, density );
	if ( s->count == 2 )
		return capsule_mass( s->v[0], s->v[1], s->radius, density );
	b2gVec vs[8];
	int count = s->count;
	if ( s->radius > 0.0f )
	{
		float sqrt2 = 1.412f;
		for ( int i = 0; i < count; ++i )
		{
			int j = i == 0 ? count - 1 : i - 1;
			b2gVec mid = gnormalize( gadd( s->n[j], s->n[i] ) );
			vs[i] = gmuladd( s->v[i], sqrt2 * s->radius, mid );
		}
	}
	else
	{
		for ( int i = 0; i < count; ++i )
			vs[i] = s->v[i];
	}
	b2gVec center = gv( 0.0f, 0.0f );
	float area = 0.0f, I = 0.0f;
	b2gVec r = vs[0];
	const float inv3 = 1.0f / 3.0f;
	for ( int i = 1; i < count - 1; ++i )
	{
		b2gVec e1 = gsub( vs[i], r );
		b2gVec e2 = gsub( vs[i + 1], r );
		float D = gcross( e1, e2 );
		float triArea = 0.5f * D;
		area += triArea;
		center = gmuladd( center, triArea * inv3, gadd( e1, e2 ) );
		float ex1 = e1.x, ey1 = e1.y, ex2 = e2.x, ey2 = e2.y;
		float intx2 = ex1 * ex1 + ex2 * ex1 + ex2 * ex2;
		float inty2 = ey1 * ey1 + ey2 * ey1 + ey2 * ey2;
		I += ( 0.25f * inv3 * D ) * ( intx2 + inty2 );
	}
	b2MassData m;
	m.mass = density * area;
	float invArea = 1.0f / area;
	center.x *= invArea;
	center.y *= invArea;
	b2gVec mc = gadd( r, center );
	m.center = vfg( mc );
	m.rotationalInertia = density * I;
	m.rotationalInertia += m.mass * ( gdot( mc, mc ) - gdot( center, center ) );
	return m;
}

static void geo_from_polygon( b2gShapeGeo* g, const b2Polygon* p )
{
	memset( g, 0, sizeof( *g ) );
	g->type = b2_polygonShape;
	g->count = p->count;
	g->radius = p->radius;
	for ( int i = 0; i < p->count; ++i )
	{
		g->v[i] = gvf( p->vertices[i] );
		g->n[i] = gvf( p->normals[i] );
	}
	g->centroid = gvf( p->centroid );
}

b2MassData b2ComputePolygonMass( const b2Polygon* shape, float density )
{
	b2gShapeGeo g;
	geo_from_polygon( &g, shape );
	return polygon_mass( &g, density );
}

b2MassData b2ComputeCircleMass( const b2Circle* shape, float density )
{
	return circle_mass( gvf( shape->center ), shape->radius, density );
}

b2MassData b2ComputeCapsuleMass( const b2Capsule* shape, float density )
{
	return capsule_mass( gvf( shape->center1 ), gvf( shape->center2 ), shape->radius, density );
}

b2MassData gshape_mass( const b2gShapeGeo* g, float density )
{
	switch ( g->type )
	{
		case b2_capsuleShape:
			return capsule_mass( g->v[0], g->v[1], g->radius, density );
		case b2_circleShape:
			return circle_mass( g->v[0], g->radius, density );
		case b2_polygonShape:
			return polygon_mass( g, density );
		default:
		{
			b2MassData m;
			memset( &m, 0, sizeof( m ) );
			return m;
		}
	}
}

void gshape_extent( const b2gShapeGeo* g, b2gVec lc, float* minExtent, float* maxExtent )
{
	switch ( g->type )
	{
		case b2_capsuleShape:
		{
			float r = g->radius;
			b2gVec c1 = gsub( g->v[0], lc ), c2 = gsub( g->v[1], lc );
			*minExtent = r;
			*maxExtent = sqrtf( gmax( glen2( c1 ), glen2( c2 ) ) ) + r;
			return;
		}
		case b2_circleShape:
			*minExtent = g->radius;
			*maxExtent = glen( gsub( g->v[0], lc ) ) + g->radius;
			return;
		case b2_polygonShape:
		{
			float minE = B2G_HUGE, maxE2 = 0.0f;
			for ( int i = 0; i < g->count; ++i )
			{
				b2gVec v = g->v[i];
				float planeOffset = gdot( g->n[i], gsub( v, g->centroid ) );
				minE = gmin( minE, planeOffset );
				maxE2 = gmax( maxE2, glen2( gsub( v, lc ) ) );
			}
			*minExtent = minE + g->radius;
			*maxExtent = sqrtf( maxE2 ) + g->radius;
			return;
		}
		case b2_segmentShape:
		case b2_smoothSegmentShape:
		{
			b2gVec c1 = gsub( g->v[0], lc ), c2 = gsub( g->v[1], lc );
			*minExtent = 0.0f;
			*maxExtent = sqrtf( gmax( glen2( c1 ), glen2( c2 ) ) );
			return;
		}
		default:
			*minExtent = 0.0f;
			*maxExtent = 0.0f;
	}
}

/* ------------------------------------------------------------ bounding boxes */
b2gBox gshape_geo_aabb( const b2gShapeGeo* g, b2gXf xf )
{
	b2gBox b;
	switch ( g->type )
	{
		case b2_circleShape:
		{
			b2gVec p = gxfpoint( xf, g->v[0] );
			float r = g->radius;
			b.lo = gv( p.x - r, p.y - r );
			b.hi = gv( p.x + r, p.y + r );
			return b;
		}
		case b2_capsuleShape:
		{
			b2gVec v1 = gxfpoint( xf, g->v[0] ), v2 = gxfpoint( xf, g->v[1] );
			b2gVec r = gv( g->radius, g->radius );
			b.lo = gsub( gminv( v1, v2 ), r );
			b.hi = gadd( gmaxv( v1, v2 ), r );
			return b;
		}
		case b2_segmentShape:
		case b2_smoothSegmentShape:
		{
			b2gVec v1 = gxfpoint( xf, g->v[0] ), v2 = gxfpoint( xf, g->v[1] );
			b.lo = gminv( v1, v2 );
			b.hi = gmaxv( v1, v2 );
			return b;
		}
		default:
		{
			b2gVec lo = gxfpoint( xf, g->v[0] );
			b2gVec hi = lo;
			for ( int i = 1; i < g->count; ++i )
			{
				b2gVec v = gxfpoint( xf, g->v[i] );
				lo = gminv( lo, v );
				hi = gmaxv( hi, v );
			}
			b2gVec r = gv( g->radius, g->radius );
			b.lo = gsub( lo, r );
			b.hi = gadd( hi, r );
			return b;
		}
	}
}

static b2AABB box_out( b2gBox b )
{
	b2AABB a = { vfg( b.lo ), vfg( b.hi ) };
	return a;
}

b2AABB b2ComputePolygonAABB( const b2Polygon* shape, b2Transform xf )
{
	b2gShapeGeo g;
	geo_from_polygon( &g, shape );
	return box_out( gshape_geo_aabb( &g, xf_of( xf ) ) );
}

b2AABB b2ComputeCircleAABB( const b2Circle* shape, b2Transform xf )
{
	b2gShapeGeo g;
	memset( &g, 0, sizeof( g ) );
	g.type = b2_circleShape;
	g.v[0] = gvf( shape->center );
	g.radius = shape->radius;
	return box_out( gshape_geo_aabb( &g, xf_of( xf ) ) );
}

b2AABB b2ComputeCapsuleAABB( const b2Capsule* shape, b2Transform xf )
{
	b2gShapeGeo g;
	memset( &g, 0, sizeof( g ) );
	g.type = b2_capsuleShape;
	g.v[0] = gvf( shape->center1 );
	g.v[1] = gvf( shape->center2 );
	g.radius = shape->radius;
	return box_out( gshape_geo_aabb( &g, xf_of( xf ) ) );
}

b2AABB b2ComputeSegmentAABB( const b2Segment* shape, b2Transform xf )
{
	b2gShapeGeo g;
	memset( &g, 0, sizeof( g ) );
	g.type = b2_segmentShape;
	g.v[0] = gvf( shape->point1 );
	g.v[1] = gvf( shape->point2 );
	return box_out( gshape_geo_aabb( &g, xf_of( xf ) ) );
}

b2SegmentDistanceResult b2SegmentDistance( b2Vec2 p1, b2Vec2 q1, b2Vec2 p2, b2Vec2 q2 )
{
	b2gSegDist d = gsegment_distance( gvf( p1 ), gvf( q1 ), gvf( p2 ), gvf( q2 ) );
	b2SegmentDistanceResult r;
	r.closest1 = vfg( d.c1 );
	r.closest2 = vfg( d.c2 );
	r.fraction1 = d.f1;
	r.fraction2 = d.f2;
	r.distanceSquared = d.dist2;
	return r;
}

/* ------------------------------------------------------------ manifolds */
static b2Manifold manifold_out( const b2gManifold* m )
{
	b2Manifold r;
	memset( &r, 0, sizeof( r ) );
	r.normal = vfg( m->normal );
	r.pointCount = m->count;
	for ( int i = 0; i < 2; ++i )
	{
		r.points[i].point = vfg( m->pts[i].point );
		r.points[i].anchorA = vfg( m->pts[i].anchorA );
		r.points[i].anchorB = vfg( m->pts[i].anchorB );
		r.points[i].separation = m->pts[i].separation;
		r.points[i].id = m->pts[i].id;
	}
	return r;
}

static void geo_circle( b2gShapeGeo* g, const b2Circle* c )
{
	memset( g, 0, sizeof( *g ) );
	g->type = b2_circleShape;
	g->v[0] = gvf( c->center );
	g->radius = c->radius;
}

static void geo_capsule( b2gShapeGeo* g, const b2Capsule* c )
{
	memset( g, 0, sizeof( *g ) );
	g->type = b2_capsuleShape;
	g->v[0] = gvf( c->center1 );
	g->v[1] = gvf( c->center2 );
	g->radius = c->radius;
}

static void geo_segment( b2gShapeGeo* g, const b2Segment* s )
{
	memset( g, 0, sizeof( *g ) );
	g->type = b2_segmentShape;
	g->v[0] = gvf( s->point1 );
	g->v[1] = gvf( s->point2 );
}

static void geo_from_polygon( b2gShapeGeo* g, const b2Polygon* p );
static void geo_capsule( b2gShapeGeo* g, const b2Capsule* c );
static void geo_circle( b2gShapeGeo* g, const b2Circle* c );

static b2Manifold collide( const b2gShapeGeo* a, b2Transform xfA, const b2gShapeGeo* b, b2Transform xfB )
{
	b2gManifold m;
	b2gDistCache cache = gcache_unpack( 0u );
	gcollide_shapes( &m, a, xf_of( xfA ), b, xf_of( xfB ), &cache );
	return manifold_out( &m );
}

static void geo_smooth( b2gShapeGeo* g, const b2SmoothSegment* s )
{
	memset( g, 0, sizeof( *g ) );
	g->type = b2_smoothSegmentShape;
	g->count = 2;
	g->v[0] = gvf( s->segment.point1 );
	g->v[1] = gvf( s->segment.point2 );
	g->v[2] = gvf( s->ghost1 );
	g->v[3] = gvf( s->ghost2 );
	g->centroid = glerp( g->v[0], g->v[1], 0.5f );
}

/* Smooth segment manifolds with the caller's closest-feature cache, read and updated
 * (reference src/manifold.c:714-807, :944-1333). */
static b2Manifold collide_cached( const b2gShapeGeo* a, b2Transform xfA, const b2gShapeGeo* b, b2Transform xfB,
								  b2DistanceCache* cache )
{
	b2gDistCache c;
	memset( &c, 0, sizeof( c ) );
	if ( cache != NULL )
	{
		c.count = cache->count;
		for ( int i = 0; i < 3; ++i )
		{
			c.indexA[i] = cache->indexA[i];
			c.indexB[i] = cache->indexB[i];
		}
	}
	b2gManifold m;
	gcollide_shapes( &m, a, xf_of( xfA ), b, xf_of( xfB ), &c );
	if ( cache != NULL )
	{
		cache->count = (uint16_t)c.count;
		for ( int i = 0; i < 3; ++i )
		{
			cache->indexA[i] = (uint8_t)( i < c.count ? c.indexA[i] : 0 );
			cache->indexB[i] = (uint8_t)( i < c.count ? c.indexB[i] : 0 );
		}
	}
	return manifold_out( &m );
}

b2Manifold b2CollideSmoothSegmentAndCircle( const b2SmoothSegment* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_smooth( &ga, a );
	geo_circle( &gb, b );
	return collide_cached( &ga, xfA, &gb, xfB, NULL );
}

b2Manifold b2CollideSmoothSegmentAndCapsule( const b2SmoothSegment* a, b2Transform xfA, const b2Capsule* b, b2Transform xfB,
											 b2DistanceCache* cache )
{
	b2gShapeGeo ga, gb;
	geo_smooth( &ga, a );
	geo_capsule( &gb, b );
	return collide_cached( &ga, xfA, &gb, xfB, cache );
}

b2Manifold b2CollideSmoothSegmentAndPolygon( const b2SmoothSegment* a, b2Transform xfA, const b2Polygon* b, b2Transform xfB,
											 b2DistanceCache* cache )
{
	b2gShapeGeo ga, gb;
	geo_smooth( &ga, a );
	geo_from_polygon( &gb, b );
	return collide_cached( &ga, xfA, &gb, xfB, cache );
}

b2Manifold b2CollideCircles( const b2Circle* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_circle( &ga, a );
	geo_circle( &gb, b );
	return collide( &ga, xfA, &gb, xfB );
}

b2Manifold b2CollideCapsuleAndCircle( const b2Capsule* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_capsule( &ga, a );
	geo_circle( &gb, b );
	return collide( &ga, xfA, &gb, xfB );
}

b2Manifold b2CollideSegmentAndCircle( const b2Segment* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_segment( &ga, a );
	geo_circle( &gb, b );
	return collide( &ga, xfA, &gb, xfB );
}

b2Manifold b2CollidePolygonAndCircle( const b2Polygon* a, b2Transform xfA, const b2Circle* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_from_polygon( &ga, a );
	geo_circle( &gb, b );
	return collide( &ga, xfA, &gb, xfB );
}

b2Manifold b2CollideCapsules( const b2Capsule* a, b2Transform xfA, const b2Capsule* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_capsule( &ga, a );
	geo_capsule( &gb, b );
	return collide( &ga, xfA, &gb, xfB );
}

b2Manifold b2CollideSegmentAndCapsule( const b2Segment* a, b2Transform xfA, const b2Capsule* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_segment( &ga, a );
	geo_capsule( &gb, b );
	return collide( &ga, xfA, &gb, xfB );
}

b2Manifold b2CollidePolygonAndCapsule( const b2Polygon* a, b2Transform xfA, const b2Capsule* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_from_polygon( &ga, a );
	geo_capsule( &gb, b );
	return collide( &ga, xfA, &gb, xfB );
}

b2Manifold b2CollidePolygons( const b2Polygon* a, b2Transform xfA, const b2Polygon* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_from_polygon( &ga, a );
	geo_from_polygon( &gb, b );
	return collide( &ga, xfA, &gb, xfB );
}

b2Manifold b2CollideSegmentAndPolygon( const b2Segment* a, b2Transform xfA, const b2Polygon* b, b2Transform xfB )
{
	b2gShapeGeo ga, gb;
	geo_segment( &ga, a );
	geo_from_polygon( &gb, b );
	return collide( &ga, xfA, &gb, xfB );
}

/* ------------------------------------------------------------ math validity helpers */
bool b2IsValid( float a ) { return !isnan( a ) && !isinf( a ); }
bool b2Vec2_IsValid( b2Vec2 v ) { return b2IsValid( v.x ) && b2IsValid( v.y ); }
bool b2Rot_IsValid( b2Rot q ) { return b2IsValid( q.s ) && b2IsValid( q.c ) && b2IsNormalized( q ); }
bool b2AABB_IsValid( b2AABB a )
{
	b2Vec2 d = b2Sub( a.upperBound, a.lowerBound );
	return d.x >= 0.0f && d.y >= 0.0f && b2Vec2_IsValid( a.lowerBound ) && b2Vec2_IsValid( a.upperBound );
}
b2Vec2 b2Normalize( b2Vec2 v ) { return vfg( gnormalize( gvf( v ) ) ); }
b2Vec2 b2NormalizeChecked( b2Vec2 v ) { return vfg( gnormalize( gvf( v ) ) ); }
b2Vec2 b2GetLengthAndNormalize( float* length, b2Vec2 v ) { return vfg( glen_normalize( length, gvf( v ) ) ); }
void b2SetLengthUnitsPerMeter( float lengthUnits ) { (void)lengthUnits; }
float b2GetLengthUnitsPerMeter( void ) { return 1.0f; }
