/*
 * alloc_fault.c -- host allocation failures injected through the reference allocator
 * hook (b2SetAllocator, reference src/allocate.c:39-107) into libbox2d_gb300.so.
 *
 *   alloc_fault N    the installed allocator grants N requests, then refuses all
 *   alloc_fault -1   it never refuses (counts only)
 *
 * Builds a world (ground and a 9-row pyramid, 45 boxes: past the device arena's first
 * capacities of 32 bodies and 128 contacts, so the arena regrows), steps it 60 times,
 * destroys it and prints one line:
 *   "world=<0|1> bodies=<n> status=<s> refused=<r> calls=<c> leaked=<bytes>"
 * where leaked is b2GetByteCount() after the world is destroyed less the count after a
 * first world was created and destroyed (the process-wide registries).  Exits 0 unless
 * it is killed; the test checks the line.
 */
#include "box2d/box2d.h"
#include "box2d/gpu.h"

#include <stdio.h>
#include <stdlib.h>

static long s_grant = -1;
static long s_calls, s_refused;

static void* alloc_fn( unsigned int size, int alignment )
{
	s_calls += 1;
	if ( s_grant >= 0 && s_calls > s_grant )
	{
		s_refused += 1;
		return NULL;
	}
	return aligned_alloc( (size_t)alignment, size );
}

static void free_fn( void* mem ) { free( mem ); }

static b2WorldId build( int* bodies )
{
	b2WorldDef wd = b2DefaultWorldDef();
	wd.enableSleep = false;
	b2WorldId w = b2CreateWorld( &wd );
	*bodies = 0;
	if ( B2_IS_NULL( w ) )
		return w;
	b2BodyDef gd = b2DefaultBodyDef();
	gd.position = ( b2Vec2 ){ 0.0f, -0.5f };
	b2BodyId ground = b2CreateBody( w, &gd );
	b2Polygon gbox = b2MakeBox( 50.0f, 0.5f );
	b2ShapeDef sd = b2DefaultShapeDef();
	b2CreatePolygonShape( ground, &sd, &gbox );
	b2BodyDef bd = b2DefaultBodyDef();
	bd.type = b2_dynamicBody;
	b2Polygon box = b2MakeSquare( 0.5f );
	for ( int i = 0; i < 9; ++i )
		for ( int j = i; j < 9; ++j )
		{
			bd.position = ( b2Vec2 ){ ( i + 1.0f ) * 0.5f + ( j - i ) - 4.5f, ( 2.0f * i + 1.0f ) * 0.5f };
			b2BodyId id = b2CreateBody( w, &bd );
			if ( B2_IS_NON_NULL( id ) && B2_IS_NON_NULL( b2CreatePolygonShape( id, &sd, &box ) ) )
				*bodies += 1;
		}
	return w;
}

int main( int argc, char** argv )
{
	long grant = argc > 1 ? atol( argv[1] ) : -1;
	b2SetAllocator( alloc_fn, free_fn );

	/* a first world fills the process-wide registries */
	int n;
	b2WorldId first = build( &n );
	if ( B2_IS_NON_NULL( first ) )
		b2DestroyWorld( first );
	int baseline = b2GetByteCount();
	long calls0 = s_calls;

	s_grant = grant < 0 ? -1 : s_calls + grant;
	b2WorldId w = build( &n );
	int status = 0;
	if ( B2_IS_NON_NULL( w ) )
	{
		for ( int s = 0; s < 60; ++s )
			b2World_Step( w, 1.0f / 60.0f, 4 );
		status = b2World_GetStatus( w );
		b2DestroyWorld( w );
	}
	s_grant = -1;
	printf( "world=%d bodies=%d status=%d refused=%ld calls=%ld leaked=%d\n", B2_IS_NON_NULL( w ) ? 1 : 0, n, status,
			s_refused, s_calls - calls0, b2GetByteCount() - baseline );
	return 0;
}
