/*
 * b2g_toi.h -- continuous collision arithmetic shared by host C code and sm_103a kernels:
 * body sweeps, shape proxies, closest points of two convex proxies (GJK) and the time of
 * impact of two sweeping proxies by conservative advancement along separating axes.
 *
 * Reference: src/distance.c:13-30 (sweep transform), :109-620 (proxies, simplex solver,
 * b2ShapeDistance without radii), :780-1237 (separation functions and b2TimeOfImpact),
 * src/shape.c:480-497, :713-735 (shape centroid and proxy), src/body.h:159-168 (sweep).
 * The results feed body positions, so every expression keeps the reference's operand
 * order; with no fused multiply-add (host -ffp-contract=off, device --fmad=false) the
 * times of impact are bit-identical to the reference's.
 */
#pragma once

#include "b2g_types.h"

typedef struct b2gSweep
{
	b2gVec localCenter, c1, c2;
	b2gRot q1, q2;
} b2gSweep;

typedef struct b2gProxy
{
	b2gVec pts[8];
	int count;
	float radius;
} b2gProxy;

typedef struct b2gDistCache
{
	int count;
	int indexA[3], indexB[3];
} b2gDistCache;

/* A closest-feature cache in one word: the count in bits 0-1, the three vertex indices
 * of A in 3 bits each from bit 2, those of B from bit 11 (polygons have at most 8). */
B2G_HD b2gDistCache gcache_unpack( uint32_t packed )
{
	b2gDistCache c;
	c.count = (int)( packed & 3u );
	for ( int i = 0; i < 3; ++i )
	{
		c.indexA[i] = (int)( ( packed >> ( 2 + 3 * i ) ) & 7u );
		c.indexB[i] = (int)( ( packed >> ( 11 + 3 * i ) ) & 7u );
	}
	return c;
}

B2G_HD uint32_t gcache_pack( const b2gDistCache* c )
{
	uint32_t packed = (uint32_t)c->count;
	for ( int i = 0; i < c->count; ++i )
	{
		packed |= (uint32_t)c->indexA[i] << ( 2 + 3 * i );
		packed |= (uint32_t)c->indexB[i] << ( 11 + 3 * i );
	}
	return packed;
}

/* Time-of-impact outcomes (reference b2TOIState). */
enum
{
	B2G_TOI_UNKNOWN = 0,
	B2G_TOI_FAILED = 1,
	B2G_TOI_OVERLAPPED = 2,
	B2G_TOI_HIT = 3,
	B2G_TOI_SEPARATED = 4,
};

/* Transform of a sweep at time t in [0, 1]. */
B2G_HD b2gXf gsweep_xf( const b2gSweep* s, float t )
{
	b2gXf xf;
	xf.p = gadd( gmulsv( 1.0f - t, s->c1 ), gmulsv( t, s->c2 ) );
	xf.q = gnormrot( grot( ( 1.0f - t ) * s->q1.c + t * s->q2.c, ( 1.0f - t ) * s->q1.s + t * s->q2.s ) );
	xf.p = gsub( xf.p, grotate( xf.q, s->localCenter ) );
	return xf;
}

B2G_HD b2gProxy gproxy_points( const b2gVec* pts, int count, float radius )
{
	b2gProxy p;
	count = count < 8 ? count : 8;
	for ( int i = 0; i < count; ++i )
		p.pts[i] = pts[i];
	p.count = count;
	p.radius = radius;
	return p;
}

/* Distance proxy of a shape in its body frame (type: circle 0, capsule 1, segment 2,
 * polygon 3). */
B2G_HD b2gProxy gproxy_shape( const b2gShapeGeo* g )
{
	if ( g->type == 3 )
		return gproxy_points( g->v, g->count, g->radius );
	if ( g->type == 0 )
		return gproxy_points( g->v, 1, g->radius );
	return gproxy_points( g->v, 2, g->type == 1 ? g->radius : 0.0f );
}

B2G_HD b2gVec gshape_centroid( const b2gShapeGeo* g )
{
	if ( g->type == 3 )
		return g->centroid;
	if ( g->type == 0 )
		return g->v[0];
	return glerp( g->v[0], g->v[1], 0.5f );
}

B2G_HD int gsupport( const b2gProxy* p, b2gVec d )
{
	int best = 0;
	float bestValue = gdot( p->pts[0], d );
	for ( int i = 1; i < p->count; ++i )
	{
		float value = gdot( p->pts[i], d );
		if ( value > bestValue )
		{
			best = i;
			bestValue = value;
		}
	}
	return best;
}

/* ------------------------------------------------------------ closest points */
typedef struct b2gSimplexVertex
{
	b2gVec wA, wB, w;
	float a;
	int indexA, indexB;
} b2gSimplexVertex;

B2G_HD void gsimplex_vertex( b2gSimplexVertex* v, const b2gProxy* A, b2gXf xfA, const b2gProxy* B, b2gXf xfB, int ia, int ib )
{
	v->indexA = ia;
	v->indexB = ib;
	v->wA = gxfpoint( xfA, A->pts[ia] );
	v->wB = gxfpoint( xfB, B->pts[ib] );
	v->w = gsub( v->wB, v->wA );
}

/* Segment simplex reduced to the part nearest the origin. */
B2G_HD void gsimplex2( b2gSimplexVertex* v, int* count )
{
	b2gVec w1 = v[0].w, w2 = v[1].w;
	b2gVec e12 = gsub( w2, w1 );
	float d12_2 = -gdot( w1, e12 );
	if ( d12_2 <= 0.0f )
	{
		v[0].a = 1.0f;
		*count = 1;
		return;
	}
	float d12_1 = gdot( w2, e12 );
	if ( d12_1 <= 0.0f )
	{
		v[1].a = 1.0f;
		*count = 1;
		v[0] = v[1];
		return;
	}
	float inv = 1.0f / ( d12_1 + d12_2 );
	v[0].a = d12_1 * inv;
	v[1].a = d12_2 * inv;
	*count = 2;
}

/* Triangle simplex reduced to the vertex, edge or interior region holding the point
 * nearest the origin. */
B2G_HD void gsimplex3( b2gSimplexVertex* v, int* count )
{
	b2gVec w1 = v[0].w, w2 = v[1].w, w3 = v[2].w;
	b2gVec e12 = gsub( w2, w1 );
	float d12_1 = gdot( w2, e12 );
	float d12_2 = -gdot( w1, e12 );
	b2gVec e13 = gsub( w3, w1 );
	float d13_1 = gdot( w3, e13 );
	float d13_2 = -gdot( w1, e13 );
	b2gVec e23 = gsub( w3, w2 );
	float d23_1 = gdot( w3, e23 );
	float d23_2 = -gdot( w2, e23 );
	float n123 = gcross( e12, e13 );
	float d123_1 = n123 * gcross( w2, w3 );
	float d123_2 = n123 * gcross( w3, w1 );
	float d123_3 = n123 * gcross( w1, w2 );

	if ( d12_2 <= 0.0f && d13_2 <= 0.0f )
	{
		v[0].a = 1.0f;
		*count = 1;
		return;
	}
	if ( d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f )
	{
		float inv = 1.0f / ( d12_1 + d12_2 );
		v[0].a = d12_1 * inv;
		v[1].a = d12_2 * inv;
		*count = 2;
		return;
	}
	if ( d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f )
	{
		float inv = 1.0f / ( d13_1 + d13_2 );
		v[0].a = d13_1 * inv;
		v[2].a = d13_2 * inv;
		*count = 2;
		v[1] = v[2];
		return;
	}
	if ( d12_1 <= 0.0f && d23_2 <= 0.0f )
	{
		v[1].a = 1.0f;
		*count = 1;
		v[0] = v[1];
		return;
	}
	if ( d13_1 <= 0.0f && d23_1 <= 0.0f )
	{
		v[2].a = 1.0f;
		*count = 1;
		v[0] = v[2];
		return;
	}
	if ( d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f )
	{
		float inv = 1.0f / ( d23_1 + d23_2 );
		v[1].a = d23_1 * inv;
		v[2].a = d23_2 * inv;
		*count = 2;
		v[0] = v[2];
		return;
	}
	float inv = 1.0f / ( d123_1 + d123_2 + d123_3 );
	v[0].a = d123_1 * inv;
	v[1].a = d123_2 * inv;
	v[2].a = d123_3 * inv;
	*count = 3;
}

/* Distance between two proxies (radii not applied), warm-started and updated through
 * `cache`; at most 20 support evaluations.  The closest points go to *pointA and *pointB. */
B2G_HD float gdistance_points( b2gDistCache* cache, const b2gProxy* A, b2gXf xfA, const b2gProxy* B, b2gXf xfB, b2gVec* pointA,
							   b2gVec* pointB )
{
	b2gSimplexVertex v[3];
	int count = cache->count;
	for ( int i = 0; i < count; ++i )
	{
		gsimplex_vertex( v + i, A, xfA, B, xfB, cache->indexA[i], cache->indexB[i] );
		v[i].a = -1.0f;
	}
	if ( count == 0 )
	{
		gsimplex_vertex( v, A, xfA, B, xfB, 0, 0 );
		v[0].a = 1.0f;
		count = 1;
	}

	int saveA[3], saveB[3];
	for ( int iter = 0; iter < 20; )
	{
		int saveCount = count;
		for ( int i = 0; i < saveCount; ++i )
		{
			saveA[i] = v[i].indexA;
			saveB[i] = v[i].indexB;
		}
		if ( count == 2 )
			gsimplex2( v, &count );
		else if ( count == 3 )
			gsimplex3( v, &count );
		if ( count == 3 )
			break;

		b2gVec d;
		if ( count == 1 )
			d = gneg( v[0].w );
		else
		{
			b2gVec e12 = gsub( v[1].w, v[0].w );
			float sgn = gcross( e12, gneg( v[0].w ) );
			d = sgn > 0.0f ? gv( -e12.y, e12.x ) : gv( e12.y, -e12.x );
		}
		if ( gdot( d, d ) < FLT_EPSILON * FLT_EPSILON )
			break;

		int ia = gsupport( A, ginvrotate( xfA.q, gneg( d ) ) );
		int ib = gsupport( B, ginvrotate( xfB.q, d ) );
		gsimplex_vertex( v + count, A, xfA, B, xfB, ia, ib );
		++iter;

		bool duplicate = false;
		for ( int i = 0; i < saveCount; ++i )
		{
			if ( ia == saveA[i] && ib == saveB[i] )
			{
				duplicate = true;
				break;
			}
		}
		if ( duplicate )
			break;
		++count;
	}

	b2gVec pa, pb;
	if ( count == 1 )
	{
		pa = v[0].wA;
		pb = v[0].wB;
	}
	else if ( count == 2 )
	{
		pa = gv( v[0].a * v[0].wA.x + v[1].a * v[1].wA.x, v[0].a * v[0].wA.y + v[1].a * v[1].wA.y );
		pb = gv( v[0].a * v[0].wB.x + v[1].a * v[1].wB.x, v[0].a * v[0].wB.y + v[1].a * v[1].wB.y );
	}
	else
	{
		pa = gv( v[0].a * v[0].wA.x + v[1].a * v[1].wA.x + v[2].a * v[2].wA.x,
				 v[0].a * v[0].wA.y + v[1].a * v[1].wA.y + v[2].a * v[2].wA.y );
		pb = pa;
	}
	cache->count = count;
	for ( int i = 0; i < count; ++i )
	{
		cache->indexA[i] = v[i].indexA;
		cache->indexB[i] = v[i].indexB;
	}
	*pointA = pa;
	*pointB = pb;
	float dx = pb.x - pa.x, dy = pb.y - pa.y;
	return sqrtf( dx * dx + dy * dy );
}

B2G_HD float gdistance( b2gDistCache* cache, const b2gProxy* A, b2gXf xfA, const b2gProxy* B, b2gXf xfB )
{
	b2gVec pa, pb;
	return gdistance_points( cache, A, xfA, B, xfB, &pa, &pb );
}

/* ------------------------------------------------------------ time of impact */
enum
{
	B2G_SEP_POINTS = 0,
	B2G_SEP_FACE_A = 1,
	B2G_SEP_FACE_B = 2,
};

typedef struct b2gSeparation
{
	const b2gProxy *A, *B;
	const b2gSweep *sA, *sB;
	b2gVec localPoint, axis;
	int type;
} b2gSeparation;

B2G_HD void gseparation_init( b2gSeparation* f, const b2gDistCache* cache, const b2gProxy* A, const b2gSweep* sA, const b2gProxy* B,
							  const b2gSweep* sB, float t1 )
{
	f->A = A;
	f->B = B;
	f->sA = sA;
	f->sB = sB;
	b2gXf xfA = gsweep_xf( sA, t1 );
	b2gXf xfB = gsweep_xf( sB, t1 );
	if ( cache->count == 1 )
	{
		f->type = B2G_SEP_POINTS;
		b2gVec pA = gxfpoint( xfA, A->pts[cache->indexA[0]] );
		b2gVec pB = gxfpoint( xfB, B->pts[cache->indexB[0]] );
		f->axis = gnormalize( gsub( pB, pA ) );
		f->localPoint = gv( 0.0f, 0.0f );
		return;
	}
	if ( cache->indexA[0] == cache->indexA[1] )
	{
		f->type = B2G_SEP_FACE_B;
		b2gVec b1 = B->pts[cache->indexB[0]], b2 = B->pts[cache->indexB[1]];
		b2gVec e = gsub( b2, b1 );
		f->axis = gnormalize( gv( 1.0f * e.y, -1.0f * e.x ) );
		b2gVec normal = grotate( xfB.q, f->axis );
		f->localPoint = gv( 0.5f * ( b1.x + b2.x ), 0.5f * ( b1.y + b2.y ) );
		b2gVec pB = gxfpoint( xfB, f->localPoint );
		b2gVec pA = gxfpoint( xfA, A->pts[cache->indexA[0]] );
		if ( gdot( gsub( pA, pB ), normal ) < 0.0f )
			f->axis = gneg( f->axis );
		return;
	}
	f->type = B2G_SEP_FACE_A;
	b2gVec a1 = A->pts[cache->indexA[0]], a2 = A->pts[cache->indexA[1]];
	b2gVec e = gsub( a2, a1 );
	f->axis = gnormalize( gv( 1.0f * e.y, -1.0f * e.x ) );
	b2gVec normal = grotate( xfA.q, f->axis );
	f->localPoint = gv( 0.5f * ( a1.x + a2.x ), 0.5f * ( a1.y + a2.y ) );
	b2gVec pA = gxfpoint( xfA, f->localPoint );
	b2gVec pB = gxfpoint( xfB, B->pts[cache->indexB[0]] );
	if ( gdot( gsub( pB, pA ), normal ) < 0.0f )
		f->axis = gneg( f->axis );
}

/* Deepest points along the separating axis at time t and their separation. */
B2G_HD float gseparation_min( const b2gSeparation* f, int* ia, int* ib, float t )
{
	b2gXf xfA = gsweep_xf( f->sA, t );
	b2gXf xfB = gsweep_xf( f->sB, t );
	if ( f->type == B2G_SEP_POINTS )
	{
		*ia = gsupport( f->A, ginvrotate( xfA.q, f->axis ) );
		*ib = gsupport( f->B, ginvrotate( xfB.q, gneg( f->axis ) ) );
		b2gVec pA = gxfpoint( xfA, f->A->pts[*ia] );
		b2gVec pB = gxfpoint( xfB, f->B->pts[*ib] );
		return gdot( gsub( pB, pA ), f->axis );
	}
	if ( f->type == B2G_SEP_FACE_A )
	{
		b2gVec normal = grotate( xfA.q, f->axis );
		b2gVec pA = gxfpoint( xfA, f->localPoint );
		*ia = -1;
		*ib = gsupport( f->B, ginvrotate( xfB.q, gneg( normal ) ) );
		b2gVec pB = gxfpoint( xfB, f->B->pts[*ib] );
		return gdot( gsub( pB, pA ), normal );
	}
	b2gVec normal = grotate( xfB.q, f->axis );
	b2gVec pB = gxfpoint( xfB, f->localPoint );
	*ib = -1;
	*ia = gsupport( f->A, ginvrotate( xfA.q, gneg( normal ) ) );
	b2gVec pA = gxfpoint( xfA, f->A->pts[*ia] );
	return gdot( gsub( pA, pB ), normal );
}

/* Separation of fixed witness points at time t. */
B2G_HD float gseparation_eval( const b2gSeparation* f, int ia, int ib, float t )
{
	b2gXf xfA = gsweep_xf( f->sA, t );
	b2gXf xfB = gsweep_xf( f->sB, t );
	if ( f->type == B2G_SEP_POINTS )
	{
		b2gVec pA = gxfpoint( xfA, f->A->pts[ia] );
		b2gVec pB = gxfpoint( xfB, f->B->pts[ib] );
		return gdot( gsub( pB, pA ), f->axis );
	}
	if ( f->type == B2G_SEP_FACE_A )
	{
		b2gVec normal = grotate( xfA.q, f->axis );
		b2gVec pA = gxfpoint( xfA, f->localPoint );
		b2gVec pB = gxfpoint( xfB, f->B->pts[ib] );
		return gdot( gsub( pB, pA ), normal );
	}
	b2gVec normal = grotate( xfB.q, f->axis );
	b2gVec pB = gxfpoint( xfB, f->localPoint );
	b2gVec pA = gxfpoint( xfA, f->A->pts[ia] );
	return gdot( gsub( pA, pB ), normal );
}

/* Largest t in [0, tMax] up to which the proxies stay apart by the target distance
 * (total radius less one linear slop).  Iterations are bounded: 20 separating axes,
 * 8 push-backs per axis, 50 root steps. */
B2G_HD float gtime_of_impact( const b2gProxy* A, const b2gSweep* sA, const b2gProxy* B, const b2gSweep* sB, float tMax, int* state )
{
	float totalRadius = A->radius + B->radius;
	float target = gmax( B2G_LINEAR_SLOP, totalRadius - B2G_LINEAR_SLOP );
	float tolerance = 0.25f * B2G_LINEAR_SLOP;
	float t1 = 0.0f;
	b2gDistCache cache;
	cache.count = 0;
	*state = B2G_TOI_UNKNOWN;

	for ( int iter = 0;; )
	{
		b2gXf xfA = gsweep_xf( sA, t1 );
		b2gXf xfB = gsweep_xf( sB, t1 );
		float distance = gdistance( &cache, A, xfA, B, xfB );
		if ( distance <= 0.0f )
		{
			*state = B2G_TOI_OVERLAPPED;
			return 0.0f;
		}
		if ( distance < target + tolerance )
		{
			*state = B2G_TOI_HIT;
			return t1;
		}

		b2gSeparation f;
		gseparation_init( &f, &cache, A, sA, B, sB, t1 );
		float t2 = tMax;
		for ( int pushBack = 0; pushBack < 8; ++pushBack )
		{
			int ia, ib;
			float s2 = gseparation_min( &f, &ia, &ib, t2 );
			if ( s2 > target + tolerance )
			{
				*state = B2G_TOI_SEPARATED;
				return tMax;
			}
			if ( s2 > target - tolerance )
			{
				t1 = t2;
				break;
			}
			float s1 = gseparation_eval( &f, ia, ib, t1 );
			if ( s1 < target - tolerance )
			{
				*state = B2G_TOI_FAILED;
				return t1;
			}
			if ( s1 <= target + tolerance )
			{
				*state = B2G_TOI_HIT;
				return t1;
			}
			float a1 = t1, a2 = t2;
			for ( int rootIter = 0;; )
			{
				float t;
				if ( rootIter & 1 )
					t = a1 + ( target - s1 ) * ( a2 - a1 ) / ( s2 - s1 );
				else
					t = 0.5f * ( a1 + a2 );
				++rootIter;
				float s = gseparation_eval( &f, ia, ib, t );
				if ( gabs( s - target ) < tolerance )
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
		}
		++iter;
		if ( iter == 20 )
		{
			*state = B2G_TOI_FAILED;
			return t1;
		}
	}
}
