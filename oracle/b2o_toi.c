/*
 * b2o_toi.c -- time of impact of the plain-C oracle (TEST INFRASTRUCTURE).
 *
 * CPU restatement of the reference's continuous collision arithmetic, used only by
 * tests/, the smoke check and the benchmark's CPU legs:
 *   sweeps and proxies     src/distance.c:13-30, :109-120; src/body.h:159-168;
 *                          src/shape.c:480-497, :713-735
 *   closest points (GJK)   src/distance.c:122-620 (b2ShapeDistance, useRadii false)
 *   time of impact         src/distance.c:780-1237 (separation functions, root finder)
 * Every expression keeps the reference's operand order so that the float build is
 * bit-identical to it; the double build (-DB2O_F64) is the same algorithm in FP64.
 */
#include "b2o.h"

oXf o_sweep_xf( const oSweep* s, b2r t )
{
	oXf xf;
	xf.p = oadd( omulsv( R( 1 ) - t, s->c1 ), omulsv( t, s->c2 ) );
	oRot q = { ( R( 1 ) - t ) * s->q1.c + t * s->q2.c, ( R( 1 ) - t ) * s->q1.s + t * s->q2.s };
	xf.q = onormrot( q );
	xf.p = osub( xf.p, orotate( xf.q, s->localCenter ) );
	return xf;
}

oProxy o_make_proxy( const oVec* points, int count, b2r radius )
{
	oProxy p;
	if ( count > 8 )
		count = 8;
	for ( int i = 0; i < count; ++i )
		p.pts[i] = points[i];
	p.count = count;
	p.radius = radius;
	return p;
}

oProxy o_shape_proxy( const oShape* s )
{
	switch ( s->type )
	{
		case b2_capsuleShape:
		{
			oVec pts[2] = { s->capsule.c1, s->capsule.c2 };
			return o_make_proxy( pts, 2, s->capsule.radius );
		}
		case b2_circleShape:
			return o_make_proxy( &s->circle.center, 1, s->circle.radius );
		case b2_polygonShape:
			return o_make_proxy( s->polygon.v, s->polygon.count, s->polygon.radius );
		case b2_segmentShape:
		{
			oVec pts[2] = { s->segment.p1, s->segment.p2 };
			return o_make_proxy( pts, 2, R( 0 ) );
		}
		case b2_smoothSegmentShape:
		{
			oVec pts[2] = { s->smooth.p1, s->smooth.p2 };
			return o_make_proxy( pts, 2, R( 0 ) );
		}
		default:
		{
			oVec zero = { 0, 0 };
			return o_make_proxy( &zero, 1, R( 0 ) );
		}
	}
}

oVec o_shape_centroid( const oShape* s )
{
	switch ( s->type )
	{
		case b2_capsuleShape:
			return olerp( s->capsule.c1, s->capsule.c2, R( 0.5f ) );
		case b2_circleShape:
			return s->circle.center;
		case b2_polygonShape:
			return s->polygon.centroid;
		case b2_segmentShape:
			return olerp( s->segment.p1, s->segment.p2, R( 0.5f ) );
		case b2_smoothSegmentShape:
			return olerp( s->smooth.p1, s->smooth.p2, R( 0.5f ) );
		default:
			return ov( 0, 0 );
	}
}

/* ------------------------------------------------------------ closest points */
typedef struct oSimplexVertex
{
	oVec wA, wB, w;
	b2r a;
	int indexA, indexB;
} oSimplexVertex;

typedef struct oSimplex
{
	oSimplexVertex v[3];
	int count;
} oSimplex;

static int support_index( const oProxy* p, oVec d )
{
	int best = 0;
	b2r bestValue = odot( p->pts[0], d );
	for ( int i = 1; i < p->count; ++i )
	{
		b2r value = odot( p->pts[i], d );
		if ( value > bestValue )
		{
			best = i;
			bestValue = value;
		}
	}
	return best;
}

static void set_vertex( oSimplexVertex* v, const oProxy* A, oXf xfA, const oProxy* B, oXf xfB, int ia, int ib )
{
	v->indexA = ia;
	v->indexB = ib;
	v->wA = oxfpoint( xfA, A->pts[ia] );
	v->wB = oxfpoint( xfB, B->pts[ib] );
	v->w = osub( v->wB, v->wA );
}

/* Closest point of a segment simplex to the origin by barycentric coordinates; drops to
 * a vertex when the origin projects outside the edge (src/distance.c:316-348). */
static void solve2( oSimplex* s )
{
	oVec w1 = s->v[0].w, w2 = s->v[1].w;
	oVec e12 = osub( w2, w1 );
	b2r d12_2 = -odot( w1, e12 );
	if ( d12_2 <= R( 0 ) )
	{
		s->v[0].a = R( 1 );
		s->count = 1;
		return;
	}
	b2r d12_1 = odot( w2, e12 );
	if ( d12_1 <= R( 0 ) )
	{
		s->v[1].a = R( 1 );
		s->count = 1;
		s->v[0] = s->v[1];
		return;
	}
	b2r inv = R( 1 ) / ( d12_1 + d12_2 );
	s->v[0].a = d12_1 * inv;
	s->v[1].a = d12_2 * inv;
	s->count = 2;
}

/* Triangle simplex: Voronoi regions of the vertices, edges and the interior
 * (src/distance.c:350-457). */
static void solve3( oSimplex* s )
{
	oVec w1 = s->v[0].w, w2 = s->v[1].w, w3 = s->v[2].w;
	oVec e12 = osub( w2, w1 );
	b2r d12_1 = odot( w2, e12 );
	b2r d12_2 = -odot( w1, e12 );
	oVec e13 = osub( w3, w1 );
	b2r d13_1 = odot( w3, e13 );
	b2r d13_2 = -odot( w1, e13 );
	oVec e23 = osub( w3, w2 );
	b2r d23_1 = odot( w3, e23 );
	b2r d23_2 = -odot( w2, e23 );
	b2r n123 = ocross( e12, e13 );
	b2r d123_1 = n123 * ocross( w2, w3 );
	b2r d123_2 = n123 * ocross( w3, w1 );
	b2r d123_3 = n123 * ocross( w1, w2 );

	if ( d12_2 <= R( 0 ) && d13_2 <= R( 0 ) )
	{
		s->v[0].a = R( 1 );
		s->count = 1;
		return;
	}
	if ( d12_1 > R( 0 ) && d12_2 > R( 0 ) && d123_3 <= R( 0 ) )
	{
		b2r inv = R( 1 ) / ( d12_1 + d12_2 );
		s->v[0].a = d12_1 * inv;
		s->v[1].a = d12_2 * inv;
		s->count = 2;
		return;
	}
	if ( d13_1 > R( 0 ) && d13_2 > R( 0 ) && d123_2 <= R( 0 ) )
	{
		b2r inv = R( 1 ) / ( d13_1 + d13_2 );
		s->v[0].a = d13_1 * inv;
		s->v[2].a = d13_2 * inv;
		s->count = 2;
		s->v[1] = s->v[2];
		return;
	}
	if ( d12_1 <= R( 0 ) && d23_2 <= R( 0 ) )
	{
		s->v[1].a = R( 1 );
		s->count = 1;
		s->v[0] = s->v[1];
		return;
	}
	if ( d13_1 <= R( 0 ) && d23_1 <= R( 0 ) )
	{
		s->v[2].a = R( 1 );
		s->count = 1;
		s->v[0] = s->v[2];
		return;
	}
	if ( d23_1 > R( 0 ) && d23_2 > R( 0 ) && d123_1 <= R( 0 ) )
	{
		b2r inv = R( 1 ) / ( d23_1 + d23_2 );
		s->v[1].a = d23_1 * inv;
		s->v[2].a = d23_2 * inv;
		s->count = 2;
		s->v[0] = s->v[2];
		return;
	}
	b2r inv = R( 1 ) / ( d123_1 + d123_2 + d123_3 );
	s->v[0].a = d123_1 * inv;
	s->v[1].a = d123_2 * inv;
	s->v[2].a = d123_3 * inv;
	s->count = 3;
}

b2r o_distance( oDistCache* cache, const oProxy* A, oXf xfA, const oProxy* B, oXf xfB, oVec* pointA, oVec* pointB )
{
	oSimplex s;
	s.count = cache->count;
	for ( int i = 0; i < s.count; ++i )
	{
		set_vertex( s.v + i, A, xfA, B, xfB, cache->indexA[i], cache->indexB[i] );
		s.v[i].a = R( -1 );
	}
	if ( s.count == 0 )
	{
		set_vertex( s.v, A, xfA, B, xfB, 0, 0 );
		s.v[0].a = R( 1 );
		s.count = 1;
	}

	int saveA[3], saveB[3];
	for ( int iter = 0; iter < 20; )
	{
		int saveCount = s.count;
		for ( int i = 0; i < saveCount; ++i )
		{
			saveA[i] = s.v[i].indexA;
			saveB[i] = s.v[i].indexB;
		}
		if ( s.count == 2 )
			solve2( &s );
		else if ( s.count == 3 )
			solve3( &s );
		if ( s.count == 3 )
			break;

		/* direction from the simplex towards the origin (src/distance.c:210-237) */
		oVec d;
		if ( s.count == 1 )
			d = oneg( s.v[0].w );
		else
		{
			oVec e12 = osub( s.v[1].w, s.v[0].w );
			b2r sgn = ocross( e12, oneg( s.v[0].w ) );
			d = sgn > R( 0 ) ? ov( -e12.y, e12.x ) : ov( e12.y, -e12.x );
		}
		if ( odot( d, d ) < O_EPS * O_EPS )
			break;

		oSimplexVertex* v = s.v + s.count;
		int ia = support_index( A, oinvrotate( xfA.q, oneg( d ) ) );
		int ib = support_index( B, oinvrotate( xfB.q, d ) );
		set_vertex( v, A, xfA, B, xfB, ia, ib );
		++iter;

		bool duplicate = false;
		for ( int i = 0; i < saveCount; ++i )
		{
			if ( v->indexA == saveA[i] && v->indexB == saveB[i] )
			{
				duplicate = true;
				break;
			}
		}
		if ( duplicate )
			break;
		++s.count;
	}

	/* witness points (src/distance.c:262-314) */
	oVec pa, pb;
	if ( s.count == 1 )
	{
		pa = s.v[0].wA;
		pb = s.v[0].wB;
	}
	else if ( s.count == 2 )
	{
		pa = ov( s.v[0].a * s.v[0].wA.x + s.v[1].a * s.v[1].wA.x, s.v[0].a * s.v[0].wA.y + s.v[1].a * s.v[1].wA.y );
		pb = ov( s.v[0].a * s.v[0].wB.x + s.v[1].a * s.v[1].wB.x, s.v[0].a * s.v[0].wB.y + s.v[1].a * s.v[1].wB.y );
	}
	else
	{
		pa = ov( s.v[0].a * s.v[0].wA.x + s.v[1].a * s.v[1].wA.x + s.v[2].a * s.v[2].wA.x,
				 s.v[0].a * s.v[0].wA.y + s.v[1].a * s.v[1].wA.y + s.v[2].a * s.v[2].wA.y );
		pb = pa;
	}
	cache->count = s.count;
	for ( int i = 0; i < s.count; ++i )
	{
		cache->indexA[i] = s.v[i].indexA;
		cache->indexB[i] = s.v[i].indexB;
	}
	if ( pointA )
		*pointA = pa;
	if ( pointB )
		*pointB = pb;
	b2r dx = pb.x - pa.x, dy = pb.y - pa.y;
	return RSQRT( dx * dx + dy * dy );
}

/* ------------------------------------------------------------ time of impact */
enum
{
	O_SEP_POINTS,
	O_SEP_FACE_A,
	O_SEP_FACE_B
};

typedef struct oSeparation
{
	const oProxy *A, *B;
	oSweep sA, sB;
	oVec localPoint, axis;
	int type;
} oSeparation;

/* Separating axis from the closest-feature cache at time t1 (src/distance.c:804-878). */
static oSeparation make_separation( const oDistCache* cache, const oProxy* A, const oSweep* sA, const oProxy* B, const oSweep* sB,
									b2r t1 )
{
	oSeparation f;
	f.A = A;
	f.B = B;
	f.sA = *sA;
	f.sB = *sB;
	oXf xfA = o_sweep_xf( sA, t1 );
	oXf xfB = o_sweep_xf( sB, t1 );
	if ( cache->count == 1 )
	{
		f.type = O_SEP_POINTS;
		oVec pA = oxfpoint( xfA, A->pts[cache->indexA[0]] );
		oVec pB = oxfpoint( xfB, B->pts[cache->indexB[0]] );
		f.axis = onormalize( osub( pB, pA ) );
		f.localPoint = ov( 0, 0 );
		return f;
	}
	if ( cache->indexA[0] == cache->indexA[1] )
	{
		/* two points on B, one on A */
		f.type = O_SEP_FACE_B;
		oVec b1 = B->pts[cache->indexB[0]], b2 = B->pts[cache->indexB[1]];
		f.axis = onormalize( ocross_vs( osub( b2, b1 ), R( 1 ) ) );
		oVec normal = orotate( xfB.q, f.axis );
		f.localPoint = ov( R( 0.5f ) * ( b1.x + b2.x ), R( 0.5f ) * ( b1.y + b2.y ) );
		oVec pB = oxfpoint( xfB, f.localPoint );
		oVec pA = oxfpoint( xfA, A->pts[cache->indexA[0]] );
		if ( odot( osub( pA, pB ), normal ) < R( 0 ) )
			f.axis = oneg( f.axis );
		return f;
	}
	/* two points on A, one or two on B */
	f.type = O_SEP_FACE_A;
	oVec a1 = A->pts[cache->indexA[0]], a2 = A->pts[cache->indexA[1]];
	f.axis = onormalize( ocross_vs( osub( a2, a1 ), R( 1 ) ) );
	oVec normal = orotate( xfA.q, f.axis );
	f.localPoint = ov( R( 0.5f ) * ( a1.x + a2.x ), R( 0.5f ) * ( a1.y + a2.y ) );
	oVec pA = oxfpoint( xfA, f.localPoint );
	oVec pB = oxfpoint( xfB, B->pts[cache->indexB[0]] );
	if ( odot( osub( pB, pA ), normal ) < R( 0 ) )
		f.axis = oneg( f.axis );
	return f;
}

/* Deepest points along the axis at time t (src/distance.c:880-946). */
static b2r min_separation( const oSeparation* f, int* ia, int* ib, b2r t )
{
	oXf xfA = o_sweep_xf( &f->sA, t );
	oXf xfB = o_sweep_xf( &f->sB, t );
	if ( f->type == O_SEP_POINTS )
	{
		*ia = support_index( f->A, oinvrotate( xfA.q, f->axis ) );
		*ib = support_index( f->B, oinvrotate( xfB.q, oneg( f->axis ) ) );
		oVec pA = oxfpoint( xfA, f->A->pts[*ia] );
		oVec pB = oxfpoint( xfB, f->B->pts[*ib] );
		return odot( osub( pB, pA ), f->axis );
	}
	if ( f->type == O_SEP_FACE_A )
	{
		oVec normal = orotate( xfA.q, f->axis );
		oVec pA = oxfpoint( xfA, f->localPoint );
		*ia = -1;
		*ib = support_index( f->B, oinvrotate( xfB.q, oneg( normal ) ) );
		oVec pB = oxfpoint( xfB, f->B->pts[*ib] );
		return odot( osub( pB, pA ), normal );
	}
	oVec normal = orotate( xfB.q, f->axis );
	oVec pB = oxfpoint( xfB, f->localPoint );
	*ib = -1;
	*ia = support_index( f->A, oinvrotate( xfA.q, oneg( normal ) ) );
	oVec pA = oxfpoint( xfA, f->A->pts[*ia] );
	return odot( osub( pA, pB ), normal );
}

/* Separation of given witness points at time t (src/distance.c:948-997). */
static b2r eval_separation( const oSeparation* f, int ia, int ib, b2r t )
{
	oXf xfA = o_sweep_xf( &f->sA, t );
	oXf xfB = o_sweep_xf( &f->sB, t );
	if ( f->type == O_SEP_POINTS )
	{
		oVec pA = oxfpoint( xfA, f->A->pts[ia] );
		oVec pB = oxfpoint( xfB, f->B->pts[ib] );
		return odot( osub( pB, pA ), f->axis );
	}
	if ( f->type == O_SEP_FACE_A )
	{
		oVec normal = orotate( xfA.q, f->axis );
		oVec pA = oxfpoint( xfA, f->localPoint );
		oVec pB = oxfpoint( xfB, f->B->pts[ib] );
		return odot( osub( pB, pA ), normal );
	}
	oVec normal = orotate( xfB.q, f->axis );
	oVec pB = oxfpoint( xfB, f->localPoint );
	oVec pA = oxfpoint( xfA, f->A->pts[ia] );
	return odot( osub( pA, pB ), normal );
}

/* Conservative advancement: the largest t in [0, tMax] with the proxies kept apart
 * (src/distance.c:999-1237).  Returns t and sets *state (0 unknown, 1 failed,
 * 2 overlapped, 3 hit, 4 separated). */
b2r o_time_of_impact( const oProxy* A, const oSweep* sA, const oProxy* B, const oSweep* sB, b2r tMax, int* state )
{
	b2r totalRadius = A->radius + B->radius;
	b2r target = omax( O_LINEAR_SLOP, totalRadius - O_LINEAR_SLOP );
	b2r tolerance = R( 0.25f ) * O_LINEAR_SLOP;
	b2r t1 = R( 0 );
	oDistCache cache = { 0, { 0, 0, 0 }, { 0, 0, 0 } };
	*state = 0;

	for ( int iter = 0;; )
	{
		oXf xfA = o_sweep_xf( sA, t1 );
		oXf xfB = o_sweep_xf( sB, t1 );
		b2r distance = o_distance( &cache, A, xfA, B, xfB, NULL, NULL );
		if ( distance <= R( 0 ) )
		{
			*state = 2;
			return R( 0 );
		}
		if ( distance < target + tolerance )
		{
			*state = 3;
			return t1;
		}

		oSeparation f = make_separation( &cache, A, sA, B, sB, t1 );
		bool done = false;
		b2r t2 = tMax;
		b2r result = t1;
		for ( int pushBack = 0;; )
		{
			int ia, ib;
			b2r s2 = min_separation( &f, &ia, &ib, t2 );
			if ( s2 > target + tolerance )
			{
				*state = 4;
				result = tMax;
				done = true;
				break;
			}
			if ( s2 > target - tolerance )
			{
				t1 = t2;
				break;
			}
			b2r s1 = eval_separation( &f, ia, ib, t1 );
			if ( s1 < target - tolerance )
			{
				*state = 1;
				result = t1;
				done = true;
				break;
			}
			if ( s1 <= target + tolerance )
			{
				*state = 3;
				result = t1;
				done = true;
				break;
			}

			/* root of s(t) = target by alternating bisection and secant steps */
			b2r a1 = t1, a2 = t2;
			for ( int rootIter = 0;; )
			{
				b2r t;
				if ( rootIter & 1 )
					t = a1 + ( target - s1 ) * ( a2 - a1 ) / ( s2 - s1 );
				else
					t = R( 0.5f ) * ( a1 + a2 );
				++rootIter;
				b2r s = eval_separation( &f, ia, ib, t );
				if ( oabs( s - target ) < tolerance )
				{
					t2 = t;
					break;
				}
				if ( s > target )
				{
					a1 = t;
					s1 = s;
				}
				else
				{
					a2 = t;
					s2 = s;
				}
				if ( rootIter == 50 )
					break;
			}
			++pushBack;
			if ( pushBack == 8 )
				break;
		}
		++iter;
		if ( done )
			return result;
		if ( iter == 20 )
		{
			*state = 1;
			return t1;
		}
	}
}
