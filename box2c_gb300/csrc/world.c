/*
 * world.c -- world / body / shape / joint part of the box2d C API on the GB300 backend.
 *
 * Creation functions follow the reference bookkeeping exactly where it decides ids and
 * orders (LIFO id pools src/id_pool.c:21-45; body creation src/body.c:178-318; shape
 * creation and proxies src/shape.c:38-153, :692-702; joint creation src/joint.c:140-270,
 * :458-511; colouring of joints src/constraint_graph.c:216-267).  Numeric body and shape
 * data are written to pinned host mirrors in device layout and uploaded in bulk before
 * the next step; after a step the device copy is authoritative and the mirrors are
 * refreshed lazily when a getter or a mutation needs them.
 */
#include "host.h"

#include "box2d/gpu.h"
#include "box2d/inspect.h"

#include <cuda_runtime_api.h>

#include <stdio.h>
#include <string.h>
#include <time.h>

#define G_MAX_WORLDS 65535

static gWorld** s_worlds;
static int s_worldCap;
static b2AssertFcn* s_assertFcn;

double b2g_now_ms( void )
{
	struct timespec ts;
	clock_gettime( CLOCK_MONOTONIC, &ts );
	return 1e3 * (double)ts.tv_sec + 1e-6 * (double)ts.tv_nsec;
}

void b2SetAssertFcn( b2AssertFcn* fcn ) { s_assertFcn = fcn; }

bool gworld_out_of_memory( gWorld* w, int before )
{
	if ( b2g_alloc_failures() == before )
		return false;
	if ( w->status == 0 )
		w->status = B2_STATUS_OUT_OF_HOST_MEMORY;
	return true;
}
b2Version b2GetVersion( void )
{
	b2Version v = { 3, 0, 0 };
	return v;
}

void gworld_fail( const char* what )
{
	if ( s_assertFcn )
		s_assertFcn( what, __FILE__, 0 );
	else
		fprintf( stderr, "box2d-gb300: %s\n", what );
}

gWorld* gworld_get( b2WorldId id ) { return s_worlds[id.index1 - 1]; }
gWorld* gworld_slot( int slot ) { return s_worlds[slot]; }

/* ------------------------------------------------------------ defaults (reference src/types.c:8-63) */
b2WorldDef b2DefaultWorldDef( void )
{
	b2WorldDef d;
	memset( &d, 0, sizeof( d ) );
	d.gravity.y = -10.0f;
	d.hitEventThreshold = 1.0f;
	d.restitutionThreshold = 1.0f;
	d.contactPushoutVelocity = 3.0f;
	d.contactHertz = 30.0f;
	d.contactDampingRatio = 10.0f;
	d.jointHertz = 60.0f;
	d.jointDampingRatio = 2.0f;
	d.enableSleep = true;
	d.enableContinous = true;
	d.internalValue = 1152023;
	return d;
}

b2BodyDef b2DefaultBodyDef( void )
{
	b2BodyDef d;
	memset( &d, 0, sizeof( d ) );
	d.type = b2_staticBody;
	d.rotation.c = 1.0f;
	d.sleepThreshold = 0.05f;
	d.gravityScale = 1.0f;
	d.enableSleep = true;
	d.isAwake = true;
	d.isEnabled = true;
	d.automaticMass = true;
	d.internalValue = 1152023;
	return d;
}

b2Filter b2DefaultFilter( void )
{
	b2Filter f = { 1u, 0xFFFFFFFFu, 0 };
	return f;
}

b2QueryFilter b2DefaultQueryFilter( void )
{
	b2QueryFilter f = { 1u, 0xFFFFFFFFu };
	return f;
}

b2ShapeDef b2DefaultShapeDef( void )
{
	b2ShapeDef d;
	memset( &d, 0, sizeof( d ) );
	d.friction = 0.6f;
	d.density = 1.0f;
	d.filter = b2DefaultFilter();
	d.enableSensorEvents = true;
	d.enableContactEvents = true;
	d.internalValue = 1152023;
	return d;
}

b2ChainDef b2DefaultChainDef( void )
{
	b2ChainDef d;
	memset( &d, 0, sizeof( d ) );
	d.friction = 0.6f;
	d.filter = b2DefaultFilter();
	d.internalValue = 1152023;
	return d;
}

/* ------------------------------------------------------------ pinned mirrors */
static int grow_cap( int have, int need )
{
	int c = have < 64 ? 64 : have;
	while ( c < need )
		c *= 2;
	return c;
}

/* Grows a group of pinned mirrors together: every new buffer is allocated before any
 * old one is released, so a failed request leaves the group as it was. */
static bool grow_pinned( void** ptrs[], const size_t oldBytes[], const size_t newBytes[], int n )
{
	void* fresh[12];
	for ( int i = 0; i < n; ++i )
	{
		fresh[i] = NULL;
		if ( cudaHostAlloc( &fresh[i], newBytes[i], cudaHostAllocDefault ) != cudaSuccess )
		{
			for ( int k = 0; k < i; ++k )
				cudaFreeHost( fresh[k] );
			b2g_note_alloc_failure();
			return false;
		}
		memset( fresh[i], 0, newBytes[i] );
		if ( *ptrs[i] )
			memcpy( fresh[i], *ptrs[i], oldBytes[i] );
	}
	for ( int i = 0; i < n; ++i )
	{
		if ( *ptrs[i] )
			cudaFreeHost( *ptrs[i] );
		*ptrs[i] = fresh[i];
	}
	return true;
}

bool gworld_reserve_mirrors( gWorld* w )
{
	int needB = w->bodyIds.next;
	if ( needB > w->mirrorCap )
	{
		int nc = grow_cap( w->mirrorCap, needB );
		size_t o4 = 16u * (size_t)w->mirrorCap, n4 = 16u * (size_t)nc;
		void** ptrs[] = { (void**)&w->hState, (void**)&w->hXf, (void**)&w->hCenters, (void**)&w->hPrev,
						  (void**)&w->hMass,  (void**)&w->hForce, (void**)&w->hExtent, (void**)&w->hInfo };
		size_t ob[] = { 2 * o4, o4, o4, o4, o4, o4, o4, 4u * (size_t)w->mirrorCap };
		size_t nb[] = { 2 * n4, n4, n4, n4, n4, n4, n4, 4u * (size_t)nc };
		if ( grow_pinned( ptrs, ob, nb, 8 ) == false )
			return false;
		w->mirrorCap = nc;
	}
	int needS = w->shapeIds.next;
	if ( needS > w->shapeMirrorCap )
	{
		int nc = grow_cap( w->shapeMirrorCap, needS );
		void** ptrs[] = { (void**)&w->hGeo, (void**)&w->hAabb, (void**)&w->hFat };
		size_t ob[] = { sizeof( b2gShapeGeo ) * (size_t)w->shapeMirrorCap, 16u * (size_t)w->shapeMirrorCap,
						16u * (size_t)w->shapeMirrorCap };
		size_t nb[] = { sizeof( b2gShapeGeo ) * (size_t)nc, 16u * (size_t)nc, 16u * (size_t)nc };
		if ( grow_pinned( ptrs, ob, nb, 3 ) == false )
			return false;
		w->shapeMirrorCap = nc;
	}
	int needJ = w->jointIds.next;
	if ( needJ > w->jointMirrorCap )
	{
		int nc = grow_cap( w->jointMirrorCap, needJ );
		void** ptrs[] = { (void**)&w->hJoints };
		size_t ob[] = { sizeof( b2gJointDev ) * (size_t)w->jointMirrorCap };
		size_t nb[] = { sizeof( b2gJointDev ) * (size_t)nc };
		if ( grow_pinned( ptrs, ob, nb, 1 ) == false )
			return false;
		w->jointMirrorCap = nc;
	}
	return true;
}

/* Refreshes the host body mirror from the device after a step. */
void gworld_ensure_mirror( gWorld* w )
{
	/* staged body operations reach the device before anything reads or writes a body
	 * there */
	if ( w->bodyOps.count > 0 )
	{
		int e = gbody_flush_ops( w );
		if ( e )
			w->status = e;
	}
	if ( w->mirrorStale == false )
		return;
	int n = w->bodyIds.next;
	int e = b2gd_download_bodies( &w->dev, w->hState, w->hXf, w->hCenters, n );
	if ( e )
		w->status = e;
	/* finalisation zeroes forces and advances the sweep start to the current pose */
	for ( int i = 0; i < n; ++i )
	{
		float* f = w->hForce + 4 * i;
		f[0] = f[1] = f[2] = 0.0f;
		float* p = w->hPrev + 4 * i;
		const float* c = w->hCenters + 4 * i;
		const float* x = w->hXf + 4 * i;
		if ( w->bodies[i].id == i && w->bodies[i].type != b2_staticBody )
		{
			p[0] = c[0];
			p[1] = c[1];
			p[2] = x[2];
			p[3] = x[3];
		}
	}
	w->mirrorStale = false;
}

void gworld_ensure_shape_mirror( gWorld* w )
{
	if ( w->shapeMirrorStale == false )
		return;
	int e = b2gd_download_shapes( &w->dev, w->hAabb, w->hFat, w->shapeIds.next );
	if ( e )
		w->status = e;
	w->shapeMirrorStale = false;
}

static void ensure_joint_mirror( gWorld* w )
{
	if ( w->jointMirrorStale == false )
		return;
	int e = b2gd_download_joints( &w->dev, w->hJoints, w->jointIds.next );
	if ( e )
		w->status = e;
	w->jointMirrorStale = false;
}

/* Uploads every dirty host-side table before a step. */
void gworld_flush( gWorld* w )
{
	int nb = w->bodyIds.next, ns = w->shapeIds.next, nj = w->jointIds.next;
	int e = b2gd_reserve( &w->dev, &w->io, nb, ns, w->contactIds.next, nj, w->contactIds.next, ns );
	/* body operations first: the full upload below carries a mirror that already
	 * reflects them */
	e |= gbody_flush_ops( w );
	if ( w->enableSleep )
		e |= b2gd_reserve_sleep( &w->dev, &w->io );
	if ( w->bodiesDirty )
	{
		e |= b2gd_upload_bodies( &w->dev, w->hState, w->hXf, w->hCenters, w->hPrev, w->hMass, w->hForce, w->hExtent, w->hInfo, nb );
		w->bodiesDirty = false;
	}
	if ( w->awakeDirty )
	{
		e |= b2gd_upload_awake( &w->dev, w->awake.data, w->awake.count );
		w->awakeDirty = false;
	}
	if ( w->shapesDirty )
	{
		e |= b2gd_upload_shapes( &w->dev, w->hGeo, w->hAabb, w->hFat, ns );
		w->shapesDirty = false;
	}
	if ( w->shapeListsDirty )
	{
		int* range = (int*)b2g_alloc( sizeof( int ) * 2 * (size_t)( nb > 0 ? nb : 1 ) );
		int* list = (int*)b2g_alloc( sizeof( int ) * (size_t)( ns > 0 ? ns : 1 ) );
		if ( range == NULL || list == NULL )
		{
			b2g_free( range );
			b2g_free( list );
			w->status = w->status ? w->status : B2_STATUS_OUT_OF_HOST_MEMORY;
			return;
		}
		int n = 0;
		for ( int i = 0; i < nb; ++i )
		{
			range[2 * i] = n;
			int c = 0;
			if ( w->bodies[i].id == i )
			{
				for ( int s = w->bodies[i].headShape; s != B2G_NULL; s = w->shapes[s].next )
				{
					list[n++] = s;
					c += 1;
				}
			}
			range[2 * i + 1] = c;
		}
		e |= b2gd_upload_shape_lists( &w->dev, range, nb, list, n );
		e |= b2gd_sync( &w->dev );
		b2g_free( range );
		b2g_free( list );
		w->shapeListsDirty = false;
	}
	if ( w->jointsDirty )
	{
		e |= b2gd_upload_joints( &w->dev, w->hJoints, nj );
		w->jointsDirty = false;
	}
	if ( e )
		w->status = e;
}

/* ------------------------------------------------------------ world */
b2WorldId b2CreateWorld( const b2WorldDef* def )
{
	if ( b2gd_device_ok() == 0 )
	{
		gworld_fail( "b2CreateWorld: no CUDA device; this library has no CPU fallback" );
		return b2_nullWorldId;
	}
	int slot = -1;
	for ( int i = 0; i < s_worldCap; ++i )
	{
		if ( s_worlds[i] == NULL || s_worlds[i]->inUse == false )
		{
			slot = i;
			break;
		}
	}
	if ( slot < 0 )
	{
		if ( s_worldCap >= G_MAX_WORLDS )
			return b2_nullWorldId;
		int nc = s_worldCap ? 2 * s_worldCap : 16;
		if ( nc > G_MAX_WORLDS )
			nc = G_MAX_WORLDS;
		gWorld** grown = (gWorld**)b2g_realloc( s_worlds, sizeof( gWorld* ) * (size_t)nc );
		if ( grown == NULL )
			return b2_nullWorldId;
		s_worlds = grown;
		memset( s_worlds + s_worldCap, 0, sizeof( gWorld* ) * (size_t)( nc - s_worldCap ) );
		slot = s_worldCap;
		s_worldCap = nc;
	}
	if ( s_worlds[slot] == NULL )
		s_worlds[slot] = (gWorld*)b2g_calloc( 1, sizeof( gWorld ) );
	if ( s_worlds[slot] == NULL )
		return b2_nullWorldId;
	int failures = b2g_alloc_failures();
	gWorld* w = s_worlds[slot];
	uint16_t revision = w->revision;
	memset( w, 0, sizeof( *w ) );
	w->revision = revision;
	if ( b2gd_init( &w->dev, &w->io ) != 0 )
	{
		gworld_fail( "b2CreateWorld: device arena initialisation failed" );
		return b2_nullWorldId;
	}
	w->inUse = true;
	w->slot = slot;
	for ( int i = 0; i < 3; ++i )
		gtree_init( w->trees + i );
	w->gravity = gv( def->gravity.x, def->gravity.y );
	w->hitThreshold = def->hitEventThreshold;
	w->restitutionThreshold = def->restitutionThreshold;
	w->pushout = def->contactPushoutVelocity;
	w->contactHertz = def->contactHertz;
	w->contactDamping = def->contactDampingRatio;
	w->jointHertz = def->jointHertz;
	w->jointDamping = def->jointDampingRatio;
	w->enableSleep = def->enableSleep;
	w->enableWarmStarting = true;
	w->enableContinuous = def->enableContinous;
	gislands_init( w );
	b2WorldId id = { (uint16_t)( slot + 1 ), w->revision };
	if ( b2g_alloc_failures() != failures )
	{
		b2DestroyWorld( id );
		return b2_nullWorldId;
	}
	return id;
}

void b2DestroyWorld( b2WorldId worldId )
{
	if ( b2World_IsValid( worldId ) == false )
		return;
	gWorld* w = gworld_get( worldId );
	gtape_free( w );
	b2gd_pair_query_free( w->pairQuery );
	w->pairQuery = NULL;
	for ( int i = 0; i < w->pairListCap; ++i )
	{
		b2g_free( w->pairLists[i].a );
		b2g_free( w->pairLists[i].b );
	}
	b2g_free( w->pairLists );
	b2gd_free( &w->dev, &w->io );
	for ( int i = 0; i < 3; ++i )
		gtree_free( w->trees + i );
	for ( int i = 0; i < B2G_COLORS; ++i )
	{
		gbits_free( &w->colors[i].bodySet );
		gia_free( &w->colors[i].contacts );
		gia_free( &w->colors[i].joints );
	}
	gia_free( &w->bodyIds.freeIds );
	gia_free( &w->shapeIds.freeIds );
	gia_free( &w->contactIds.freeIds );
	gia_free( &w->jointIds.freeIds );
	gia_free( &w->awake );
	gia_free( &w->nonTouching );
	gislands_free( w );
	gia_free( &w->moveArray );
	gia_free( &w->solveList );
	gia_free( &w->jointList );
	gset_free( &w->moveSet );
	gset_free( &w->pairSet );
	b2g_free( w->bodies );
	b2g_free( w->shapes );
	b2g_free( w->contacts );
	b2g_free( w->joints );
	for ( int i = 0; i < w->chainCap; ++i )
		if ( w->chains[i].id != B2G_NULL )
			b2g_free( w->chains[i].shapeIndices );
	b2g_free( w->chains );
	gia_free( &w->chainIds.freeIds );
	b2g_free( w->pending );
	b2g_free( w->scratch );
	b2g_free( w->recordSort );
	b2g_free( w->recordBucket );
	b2g_free( w->beginEvents );
	b2g_free( w->endEvents );
	b2g_free( w->hitEvents );
	b2g_free( w->sensorBeginEvents );
	b2g_free( w->sensorEndEvents );
	void* pinned[] = { w->hState, w->hXf, w->hCenters, w->hPrev, w->hMass, w->hForce, w->hExtent, w->hInfo, w->hGeo, w->hAabb, w->hFat, w->hJoints };
	for ( size_t i = 0; i < sizeof( pinned ) / sizeof( pinned[0] ); ++i )
		if ( pinned[i] )
			cudaFreeHost( pinned[i] );
	uint16_t revision = w->revision;
	memset( w, 0, sizeof( *w ) );
	w->revision = (uint16_t)( revision + 1 );
}

bool b2World_IsValid( b2WorldId id )
{
	if ( id.index1 < 1 || id.index1 > s_worldCap )
		return false;
	gWorld* w = s_worlds[id.index1 - 1];
	return w && w->inUse && w->revision == id.revision;
}

/* Turning sleep off wakes every sleeping set (reference src/world.c:1568-1594). */
void b2World_EnableSleeping( b2WorldId id, bool flag )
{
	gWorld* w = gworld_get( id );
	if ( w->locked || flag == w->enableSleep )
		return;
	w->enableSleep = flag;
	if ( flag == false )
	{
		for ( int i = G_SET_FIRST_SLEEPING; i < w->setCap; ++i )
			if ( w->sets[i].setIndex != B2G_NULL && w->sets[i].bodies.count > 0 )
				gsolver_set_wake( w, i );
	}
}
void b2World_EnableContinuous( b2WorldId id, bool flag ) { gworld_get( id )->enableContinuous = flag; }
void b2World_EnableWarmStarting( b2WorldId id, bool flag ) { gworld_get( id )->enableWarmStarting = flag; }
void b2World_SetRestitutionThreshold( b2WorldId id, float v ) { gworld_get( id )->restitutionThreshold = v; }
void b2World_SetHitEventThreshold( b2WorldId id, float v ) { gworld_get( id )->hitThreshold = v; }
void b2World_SetGravity( b2WorldId id, b2Vec2 g ) { gworld_get( id )->gravity = gv( g.x, g.y ); }
b2Vec2 b2World_GetGravity( b2WorldId id )
{
	b2gVec g = gworld_get( id )->gravity;
	b2Vec2 r = { g.x, g.y };
	return r;
}
void b2World_SetContactTuning( b2WorldId id, float hertz, float damping, float push )
{
	gWorld* w = gworld_get( id );
	w->contactHertz = gmin( hertz, 1e30f );
	w->contactDamping = damping;
	w->pushout = push;
}
b2Profile b2World_GetProfile( b2WorldId id ) { return gworld_get( id )->profile; }

b2ContactEvents b2World_GetContactEvents( b2WorldId id )
{
	gWorld* w = gworld_get( id );
	b2ContactEvents e;
	memset( &e, 0, sizeof( e ) );
	e.beginEvents = w->beginEvents;
	e.beginCount = w->beginCount;
	e.endEvents = w->endEvents;
	e.endCount = w->endCount;
	e.hitEvents = w->hitEvents;
	e.hitCount = w->hitCount;
	return e;
}

b2SensorEvents b2World_GetSensorEvents( b2WorldId id )
{
	gWorld* w = gworld_get( id );
	b2SensorEvents e = { w->sensorBeginEvents, w->sensorEndEvents, w->sensorBeginCount, w->sensorEndCount };
	return e;
}

b2Counters b2World_GetCounters( b2WorldId id )
{
	gWorld* w = gworld_get( id );
	b2Counters c;
	memset( &c, 0, sizeof( c ) );
	int staticCount = 0;
	for ( int i = 0; i < w->bodyIds.next; ++i )
		if ( w->bodies[i].id == i && w->bodies[i].type == b2_staticBody )
			staticCount += 1;
	c.staticBodyCount = staticCount;
	c.bodyCount = gid_count( &w->bodyIds );
	c.shapeCount = gid_count( &w->shapeIds );
	c.contactCount = gid_count( &w->contactIds );
	c.jointCount = gid_count( &w->jointIds );
	c.islandCount = gid_count( &w->islandIds );
	c.staticTreeHeight = gtree_height( w->trees + b2_staticBody );
	int hd = gtree_height( w->trees + b2_dynamicBody );
	int hk = gtree_height( w->trees + b2_kinematicBody );
	c.treeHeight = hd > hk ? hd : hk;
	for ( int i = 0; i < B2G_COLORS; ++i )
		c.colorCounts[i] = w->colors[i].contacts.count + w->colors[i].joints.count;
	return c;
}

/* ------------------------------------------------------------ bodies */
/* Grows a record array to `need` entries (new entries free); ok becomes false, and
 * the array stays as it was, when memory ran out. */
#define GROW_RECORDS( ptr, cap, need, T, ok )                                                                                    \
	do                                                                                                                           \
	{                                                                                                                            \
		if ( ( need ) > ( cap ) )                                                                                                \
		{                                                                                                                        \
			int nc = ( cap ) < 16 ? 16 : ( cap );                                                                                \
			while ( nc < ( need ) )                                                                                              \
				nc *= 2;                                                                                                         \
			T* _p = (T*)b2g_realloc( ptr, sizeof( T ) * (size_t)nc );                                                            \
			if ( _p == NULL )                                                                                                    \
				ok = false;                                                                                                      \
			else                                                                                                                 \
			{                                                                                                                    \
				ptr = _p;                                                                                                        \
				memset( ptr + ( cap ), 0, sizeof( T ) * (size_t)( nc - ( cap ) ) );                                              \
				for ( int _i = ( cap ); _i < nc; ++_i )                                                                          \
					ptr[_i].id = B2G_NULL;                                                                                       \
				cap = nc;                                                                                                        \
			}                                                                                                                    \
		}                                                                                                                        \
	}                                                                                                                            \
	while ( 0 )

static gBody* get_body( b2BodyId id ) { return s_worlds[id.world0]->bodies + ( id.index1 - 1 ); }
static gWorld* body_world( b2BodyId id ) { return s_worlds[id.world0]; }

b2BodyId b2CreateBody( b2WorldId worldId, const b2BodyDef* def )
{
	if ( b2World_IsValid( worldId ) == false )
		return b2_nullBodyId;
	gWorld* w = gworld_get( worldId );
	if ( w->locked )
		return b2_nullBodyId;
	gworld_ensure_mirror( w );
	int id = gid_alloc( &w->bodyIds );
	bool ok = true;
	GROW_RECORDS( w->bodies, w->bodyCap, id + 1, gBody, ok );
	if ( ok == false || gworld_reserve_mirrors( w ) == false )
	{
		gid_unalloc( &w->bodyIds, id );
		w->status = w->status ? w->status : B2_STATUS_OUT_OF_HOST_MEMORY;
		return b2_nullBodyId;
	}
	gBody* b = w->bodies + id;
	uint16_t rev = b->revision;
	memset( b, 0, sizeof( *b ) );
	b->id = id;
	b->revision = (uint16_t)( rev + 1 );
	b->type = def->type;
	b->userData = def->userData;
	b->headShape = B2G_NULL;
	b->headContactKey = B2G_NULL;
	b->headJointKey = B2G_NULL;
	b->headChainId = B2G_NULL;
	b->fixedRotation = def->fixedRotation;
	b->isBullet = def->isBullet;
	b->enableSleep = def->enableSleep;
	b->automaticMass = def->automaticMass;
	b->sleepThreshold = def->sleepThreshold;

	float* st = w->hState + 8 * id;
	float* xf = w->hXf + 4 * id;
	float* ce = w->hCenters + 4 * id;
	float* pr = w->hPrev + 4 * id;
	float* ma = w->hMass + 4 * id;
	float* fo = w->hForce + 4 * id;
	float* ex = w->hExtent + 4 * id;
	memset( st, 0, 32 );
	st[6] = 1.0f;
	xf[0] = def->position.x;
	xf[1] = def->position.y;
	xf[2] = def->rotation.c;
	xf[3] = def->rotation.s;
	ce[0] = def->position.x;
	ce[1] = def->position.y;
	ce[2] = 0.0f;
	ce[3] = 0.0f;
	pr[0] = def->position.x;
	pr[1] = def->position.y;
	pr[2] = def->rotation.c;
	pr[3] = def->rotation.s;
	memset( ma, 0, 16 );
	fo[0] = fo[1] = fo[2] = 0.0f;
	fo[3] = def->gravityScale;
	ex[0] = def->linearDamping;
	ex[1] = def->angularDamping;
	ex[2] = B2G_HUGE;
	ex[3] = 0.0f;
	/* solver set (reference src/body.c:196-228): static, awake, or a sleeping set of its
	 * own; only an awake body keeps the definition's velocity */
	int info = (int)def->type;
	b->awakeIndex = B2G_NULL;
	b->setLocal = B2G_NULL;
	b->islandId = B2G_NULL;
	b->islandPrev = B2G_NULL;
	b->islandNext = B2G_NULL;
	bool isAwake = def->isAwake || def->enableSleep == false;
	if ( def->type == b2_staticBody )
	{
		b->setIndex = G_SET_STATIC;
	}
	else if ( isAwake )
	{
		b->setIndex = G_SET_AWAKE;
		b->awakeIndex = w->awake.count;
		gia_push( &w->awake, id );
		w->awakeDirty = true;
		info |= B2G_B_AWAKE;
		st[0] = def->linearVelocity.x;
		st[1] = def->linearVelocity.y;
		st[2] = def->angularVelocity;
	}
	else
	{
		int setId = gsolver_set_create( w );
		if ( setId == B2G_NULL )
		{
			gid_unalloc( &w->bodyIds, id );
			b->id = B2G_NULL;
			w->status = w->status ? w->status : B2_STATUS_OUT_OF_HOST_MEMORY;
			return b2_nullBodyId;
		}
		b->setIndex = setId;
		b->setLocal = w->sets[setId].bodies.count;
		gia_push( &w->sets[setId].bodies, id );
	}
	if ( b->setIndex >= G_SET_AWAKE )
		gisland_create_for_body( w, b->setIndex, b );
	/* the spare lane of the velocity float4 carries the sleep threshold */
	st[3] = def->sleepThreshold;
	if ( def->isBullet )
		info |= B2G_B_BULLET;
	if ( def->enableSleep )
		info |= B2G_B_SLEEP_OK;
	w->hInfo[id] = info;
	w->bodiesDirty = true;
	/* a new body's sleep timer starts at zero (a world without timers yet gets them
	 * zeroed); the upload that follows the operation restores the definition's velocity */
	if ( b->setIndex != G_SET_STATIC && w->dev.sleepTime != NULL )
		gbody_stage_new( w, id, b->setIndex == G_SET_AWAKE ? B2G_BODY_WAKE : B2G_BODY_SLEEP );
	b2BodyId bid = { id + 1, (uint16_t)w->slot, b->revision };
	return bid;
}

bool b2Body_IsValid( b2BodyId id )
{
	if ( id.world0 >= s_worldCap || s_worlds[id.world0] == NULL || !s_worlds[id.world0]->inUse )
		return false;
	gWorld* w = s_worlds[id.world0];
	if ( id.index1 < 1 || id.index1 > w->bodyCap )
		return false;
	gBody* b = w->bodies + id.index1 - 1;
	return b->id == id.index1 - 1 && b->revision == id.revision;
}

b2BodyType b2Body_GetType( b2BodyId id ) { return get_body( id )->type; }
void b2Body_SetUserData( b2BodyId id, void* u ) { get_body( id )->userData = u; }
void* b2Body_GetUserData( b2BodyId id ) { return get_body( id )->userData; }

b2Transform b2Body_GetTransform( b2BodyId id )
{
	gWorld* w = body_world( id );
	gworld_ensure_mirror( w );
	const float* x = w->hXf + 4 * ( id.index1 - 1 );
	b2Transform t = { { x[0], x[1] }, { x[2], x[3] } };
	return t;
}
b2Vec2 b2Body_GetPosition( b2BodyId id ) { return b2Body_GetTransform( id ).p; }
b2Rot b2Body_GetRotation( b2BodyId id ) { return b2Body_GetTransform( id ).q; }
b2Vec2 b2Body_GetLocalPoint( b2BodyId id, b2Vec2 p ) { return b2InvTransformPoint( b2Body_GetTransform( id ), p ); }
b2Vec2 b2Body_GetWorldPoint( b2BodyId id, b2Vec2 p ) { return b2TransformPoint( b2Body_GetTransform( id ), p ); }

/* Velocities live in the awake set only (reference src/body.c:729-787): a body that is
 * not awake reports zero, and a non-zero velocity wakes it first. */
b2Vec2 b2Body_GetLinearVelocity( b2BodyId id )
{
	gWorld* w = body_world( id );
	if ( get_body( id )->setIndex != G_SET_AWAKE )
		return b2Vec2_zero;
	gworld_ensure_mirror( w );
	const float* s = w->hState + 8 * ( id.index1 - 1 );
	b2Vec2 v = { s[0], s[1] };
	return v;
}

float b2Body_GetAngularVelocity( b2BodyId id )
{
	gWorld* w = body_world( id );
	if ( get_body( id )->setIndex != G_SET_AWAKE )
		return 0.0f;
	gworld_ensure_mirror( w );
	return w->hState[8 * ( id.index1 - 1 ) + 2];
}

static void set_velocity( b2BodyId id, const float* v, int mask )
{
	gWorld* w = body_world( id );
	gBody* b = get_body( id );
	bool moving = ( mask & 1 ) ? v[0] * v[0] + v[1] * v[1] > 0.0f : v[2] != 0.0f;
	if ( moving )
		gbody_wake( w, b );
	if ( b->setIndex != G_SET_AWAKE )
		return;
	gworld_ensure_mirror( w );
	float* s = w->hState + 8 * b->id;
	if ( mask & 1 )
	{
		s[0] = v[0];
		s[1] = v[1];
	}
	if ( mask & 2 )
		s[2] = v[2];
	if ( b2gd_reserve( &w->dev, &w->io, w->bodyIds.next, w->shapeIds.next, w->contactIds.next, w->jointIds.next,
					   w->contactIds.next, w->shapeIds.next ) == 0 )
		b2gd_upload_body_velocity( &w->dev, b->id, s );
}

void b2Body_SetLinearVelocity( b2BodyId id, b2Vec2 v )
{
	float t[3] = { v.x, v.y, 0.0f };
	set_velocity( id, t, 1 );
}

void b2Body_SetAngularVelocity( b2BodyId id, float a )
{
	float t[3] = { 0.0f, 0.0f, a };
	set_velocity( id, t, 2 );
}

/* Sleep (reference src/body.c:1358-1433). */
bool b2Body_IsAwake( b2BodyId id ) { return get_body( id )->setIndex == G_SET_AWAKE; }

void b2Body_SetAwake( b2BodyId id, bool awake )
{
	gWorld* w = body_world( id );
	if ( w->locked )
		return;
	gBody* b = get_body( id );
	if ( awake && b->setIndex >= G_SET_FIRST_SLEEPING )
		gbody_wake( w, b );
	else if ( awake == false && b->setIndex == G_SET_AWAKE )
	{
		if ( w->islands[b->islandId].constraintRemoveCount > 0 )
			gisland_split( w, b->islandId );
		gisland_try_sleep( w, b->islandId );
	}
}

bool b2Body_IsSleepEnabled( b2BodyId id ) { return get_body( id )->enableSleep; }

void b2Body_SetSleepThreshold( b2BodyId id, float sleepVelocity )
{
	gWorld* w = body_world( id );
	gBody* b = get_body( id );
	b->sleepThreshold = sleepVelocity;
	/* the threshold rides in the velocity record's spare lane */
	gworld_ensure_mirror( w );
	w->hState[8 * b->id + 3] = sleepVelocity;
	w->bodiesDirty = true;
}

float b2Body_GetSleepThreshold( b2BodyId id ) { return get_body( id )->sleepThreshold; }

void b2Body_EnableSleep( b2BodyId id, bool enableSleep )
{
	gWorld* w = body_world( id );
	if ( w->locked )
		return;
	gBody* b = get_body( id );
	b->enableSleep = enableSleep;
	if ( enableSleep )
		w->hInfo[b->id] |= B2G_B_SLEEP_OK;
	else
		w->hInfo[b->id] &= ~B2G_B_SLEEP_OK;
	gworld_ensure_mirror( w );
	w->bodiesDirty = true;
	if ( enableSleep == false )
		gbody_wake( w, b );
}

float b2Body_GetMass( b2BodyId id ) { return body_world( id )->hMass[4 * ( id.index1 - 1 )]; }
float b2Body_GetInertiaTensor( b2BodyId id ) { return body_world( id )->hMass[4 * ( id.index1 - 1 ) + 2]; }
b2Vec2 b2Body_GetLocalCenterOfMass( b2BodyId id )
{
	const float* c = body_world( id )->hCenters + 4 * ( id.index1 - 1 );
	b2Vec2 v = { c[2], c[3] };
	return v;
}
b2Vec2 b2Body_GetWorldCenterOfMass( b2BodyId id )
{
	gWorld* w = body_world( id );
	gworld_ensure_mirror( w );
	const float* c = w->hCenters + 4 * ( id.index1 - 1 );
	b2Vec2 v = { c[0], c[1] };
	return v;
}
float b2Body_GetLinearDamping( b2BodyId id ) { return body_world( id )->hExtent[4 * ( id.index1 - 1 )]; }
float b2Body_GetAngularDamping( b2BodyId id ) { return body_world( id )->hExtent[4 * ( id.index1 - 1 ) + 1]; }
float b2Body_GetGravityScale( b2BodyId id ) { return body_world( id )->hForce[4 * ( id.index1 - 1 ) + 3]; }
int b2Body_GetShapeCount( b2BodyId id ) { return get_body( id )->shapeCount; }
int b2Body_GetShapes( b2BodyId id, b2ShapeId* out, int capacity )
{
	gWorld* w = body_world( id );
	gBody* b = get_body( id );
	int n = 0;
	for ( int s = b->headShape; s != B2G_NULL && n < capacity; s = w->shapes[s].next )
		out[n++] = ( b2ShapeId ){ s + 1, id.world0, w->shapes[s].revision };
	return n;
}
int b2Body_GetJointCount( b2BodyId id ) { return get_body( id )->jointCount; }
int b2Body_GetContactCapacity( b2BodyId id ) { return get_body( id )->contactCount; }

int b2Body_GetContactData( b2BodyId id, b2ContactData* out, int capacity )
{
	gWorld* w = body_world( id );
	gBody* b = get_body( id );
	int nc = w->contactIds.next;
	b2gManifold* ms = (b2gManifold*)b2g_alloc( sizeof( b2gManifold ) * (size_t)( nc > 0 ? nc : 1 ) );
	if ( ms == NULL || ( nc > 0 && b2gd_download_manifolds( &w->dev, ms, NULL, nc ) != 0 ) )
	{
		b2g_free( ms );
		return 0;
	}
	int n = 0;
	for ( int key = b->headContactKey; key != B2G_NULL && n < capacity; )
	{
		gContact* c = w->contacts + ( key >> 1 );
		if ( c->flags & G_TOUCHING )
		{
			const b2gManifold* m = ms + c->id;
			b2ContactData* d = out + n++;
			memset( d, 0, sizeof( *d ) );
			d->shapeIdA = ( b2ShapeId ){ c->shapeIdA + 1, id.world0, w->shapes[c->shapeIdA].revision };
			d->shapeIdB = ( b2ShapeId ){ c->shapeIdB + 1, id.world0, w->shapes[c->shapeIdB].revision };
			d->manifold.normal = ( b2Vec2 ){ m->normal.x, m->normal.y };
			d->manifold.pointCount = m->count;
			for ( int i = 0; i < 2; ++i )
			{
				const b2gPoint* p = m->pts + i;
				b2ManifoldPoint* q = d->manifold.points + i;
				q->point = ( b2Vec2 ){ p->point.x, p->point.y };
				q->anchorA = ( b2Vec2 ){ p->anchorA.x, p->anchorA.y };
				q->anchorB = ( b2Vec2 ){ p->anchorB.x, p->anchorB.y };
				q->separation = p->separation;
				q->normalImpulse = p->normalImpulse;
				q->tangentImpulse = p->tangentImpulse;
				q->maxNormalImpulse = p->maxNormalImpulse;
				q->normalVelocity = p->normalVelocity;
				q->id = p->id;
				q->persisted = p->persisted != 0;
			}
		}
		key = c->edges[key & 1].nextKey;
	}
	b2g_free( ms );
	return n;
}

/* Reference src/body.c:516-617, reading shape geometry from the host mirror. */
b2MassData gshape_mass( const b2gShapeGeo* g, float density );
void gshape_extent( const b2gShapeGeo* g, b2gVec lc, float* minExtent, float* maxExtent );

void gbody_update_mass( gWorld* w, gBody* b )
{
	float* ma = w->hMass + 4 * b->id;
	float* ce = w->hCenters + 4 * b->id;
	float* ex = w->hExtent + 4 * b->id;
	float* xf = w->hXf + 4 * b->id;
	float* st = w->hState + 8 * b->id;
	float mass = 0.0f, invMass = 0.0f, inertia = 0.0f, invI = 0.0f;
	b2gVec localCenter = gv( 0.0f, 0.0f );
	float minExtent = B2G_HUGE, maxExtent = 0.0f;
	b2gXf x;
	x.p = gv( xf[0], xf[1] );
	x.q = grot( xf[2], xf[3] );

	if ( b->type != b2_dynamicBody )
	{
		ce[0] = x.p.x;
		ce[1] = x.p.y;
		if ( b->type == b2_kinematicBody )
		{
			for ( int s = b->headShape; s != B2G_NULL; s = w->shapes[s].next )
			{
				float mn, mx;
				gshape_extent( w->hGeo + s, gv( 0.0f, 0.0f ), &mn, &mx );
				minExtent = gmin( minExtent, mn );
				maxExtent = gmax( maxExtent, mx );
			}
		}
		ma[0] = ma[1] = ma[2] = ma[3] = 0.0f;
		ce[2] = ce[3] = 0.0f;
		ex[2] = minExtent;
		ex[3] = maxExtent;
		return;
	}

	for ( int s = b->headShape; s != B2G_NULL; s = w->shapes[s].next )
	{
		const gShape* sh = w->shapes + s;
		if ( sh->density == 0.0f )
			continue;
		b2MassData md = gshape_mass( w->hGeo + s, sh->density );
		mass += md.mass;
		localCenter = gmuladd( localCenter, md.mass, gv( md.center.x, md.center.y ) );
		inertia += md.rotationalInertia;
	}
	if ( mass > 0.0f )
	{
		invMass = 1.0f / mass;
		localCenter = gmulsv( invMass, localCenter );
	}
	if ( inertia > 0.0f && b->fixedRotation == false )
	{
		inertia -= mass * gdot( localCenter, localCenter );
		invI = 1.0f / inertia;
	}
	else
	{
		inertia = 0.0f;
		invI = 0.0f;
	}
	b2gVec oldCenter = gv( ce[0], ce[1] );
	b2gVec center = gxfpoint( x, localCenter );
	ce[0] = center.x;
	ce[1] = center.y;
	ce[2] = localCenter.x;
	ce[3] = localCenter.y;
	b2gVec dl = gcross_sv( st[2], gsub( center, oldCenter ) );
	st[0] = st[0] + dl.x;
	st[1] = st[1] + dl.y;
	for ( int s = b->headShape; s != B2G_NULL; s = w->shapes[s].next )
	{
		float mn, mx;
		gshape_extent( w->hGeo + s, localCenter, &mn, &mx );
		minExtent = gmin( minExtent, mn );
		maxExtent = gmax( maxExtent, mx );
	}
	ma[0] = mass;
	ma[1] = invMass;
	ma[2] = inertia;
	ma[3] = invI;
	ex[2] = minExtent;
	ex[3] = maxExtent;
	/* the reference keeps the previous-pose centre of a new body at its origin until the
	 * first finalisation */
	w->bodiesDirty = true;
}

/* ------------------------------------------------------------ shapes */
void gbuffer_move( gWorld* w, int proxyKey )
{
	if ( gset_add( &w->moveSet, (uint64_t)( proxyKey + 1 ) ) == false )
		gia_push( &w->moveArray, proxyKey );
}

/* Shape creation (reference src/shape.c:62-170); chains skip the mass update as the
 * reference's b2CreateShapeInternal does. */
static b2ShapeId create_shape_internal( b2BodyId bodyId, const b2ShapeDef* def, b2ShapeType type, const b2gShapeGeo* geo,
										bool updateMass )
{
	/* an invalid body (a null id from a failed creation included) gets no shape */
	if ( b2Body_IsValid( bodyId ) == false )
		return b2_nullShapeId;
	gWorld* w = body_world( bodyId );
	if ( w->locked )
		return b2_nullShapeId;
	gworld_ensure_mirror( w );
	gworld_ensure_shape_mirror( w );
	int id = gid_alloc( &w->shapeIds );
	bool ok = true;
	GROW_RECORDS( w->shapes, w->shapeCap, id + 1, gShape, ok );
	if ( ok == false || gworld_reserve_mirrors( w ) == false )
	{
		gid_unalloc( &w->shapeIds, id );
		w->status = w->status ? w->status : B2_STATUS_OUT_OF_HOST_MEMORY;
		return b2_nullShapeId;
	}
	gBody* body = get_body( bodyId );
	gShape* s = w->shapes + id;
	uint16_t rev = s->revision;
	memset( s, 0, sizeof( *s ) );
	s->revision = (uint16_t)( rev + 1 );
	s->id = id;
	s->bodyId = body->id;
	s->type = type;
	s->density = def->density;
	s->friction = def->friction;
	s->restitution = def->restitution;
	s->filter = def->filter;
	s->userData = def->userData;
	s->isSensor = def->isSensor;
	s->enableSensorEvents = def->enableSensorEvents;
	s->enableContactEvents = def->enableContactEvents;
	s->enableHitEvents = def->enableHitEvents;
	if ( def->enableHitEvents )
		w->hitShapes += 1;
	s->enablePreSolveEvents = def->enablePreSolveEvents;
	b2gShapeGeo* g = w->hGeo + id;
	*g = *geo;
	g->type = type;
	g->bodyId = body->id;
	g->enableHitEvents = def->enableHitEvents;
	g->isSensor = def->isSensor;

	/* proxy (reference src/shape.c:38-59, :692-702, src/broad_phase.c:91-102) */
	const float* xf = w->hXf + 4 * body->id;
	b2gXf x;
	x.p = gv( xf[0], xf[1] );
	x.q = grot( xf[2], xf[3] );
	b2gBox aabb = gshape_geo_aabb( g, x );
	aabb.lo.x -= B2G_SPECULATIVE;
	aabb.lo.y -= B2G_SPECULATIVE;
	aabb.hi.x += B2G_SPECULATIVE;
	aabb.hi.y += B2G_SPECULATIVE;
	float margin = body->type == b2_staticBody ? B2G_SPECULATIVE : B2G_AABB_MARGIN;
	b2gBox fat;
	fat.lo.x = aabb.lo.x - margin;
	fat.lo.y = aabb.lo.y - margin;
	fat.hi.x = aabb.hi.x + margin;
	fat.hi.y = aabb.hi.y + margin;
	float* a4 = w->hAabb + 4 * id;
	float* f4 = w->hFat + 4 * id;
	a4[0] = aabb.lo.x;
	a4[1] = aabb.lo.y;
	a4[2] = aabb.hi.x;
	a4[3] = aabb.hi.y;
	f4[0] = fat.lo.x;
	f4[1] = fat.lo.y;
	f4[2] = fat.hi.x;
	f4[3] = fat.hi.y;
	int proxyType = (int)body->type;
	int proxyId = gtree_create_proxy( w->trees + proxyType, fat, s->filter.categoryBits, id );
	if ( proxyId == B2G_NULL )
	{
		/* the tree had no memory for the proxy: nothing links the shape yet */
		s->id = B2G_NULL;
		gid_unalloc( &w->shapeIds, id );
		w->status = w->status ? w->status : B2_STATUS_OUT_OF_HOST_MEMORY;
		return b2_nullShapeId;
	}
	s->proxyKey = ( proxyId << 2 ) | proxyType;
	s->chainId = B2G_NULL;
	if ( proxyType != b2_staticBody || def->forceContactCreation )
		gbuffer_move( w, s->proxyKey );

	if ( body->headShape != B2G_NULL )
		w->shapes[body->headShape].prev = id;
	s->prev = B2G_NULL;
	s->next = body->headShape;
	body->headShape = id;
	body->shapeCount += 1;

	if ( updateMass && body->automaticMass )
		gbody_update_mass( w, body );
	w->shapesDirty = true;
	w->shapeListsDirty = true;
	w->bodiesDirty = true;
	b2ShapeId sid = { id + 1, bodyId.world0, s->revision };
	return sid;
}

static b2ShapeId create_shape( b2BodyId bodyId, const b2ShapeDef* def, b2ShapeType type, const b2gShapeGeo* geo )
{
	return create_shape_internal( bodyId, def, type, geo, true );
}

b2ShapeId b2CreatePolygonShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Polygon* p )
{
	b2gShapeGeo g;
	memset( &g, 0, sizeof( g ) );
	g.count = p->count;
	g.radius = p->radius;
	for ( int i = 0; i < p->count; ++i )
	{
		g.v[i] = gv( p->vertices[i].x, p->vertices[i].y );
		g.n[i] = gv( p->normals[i].x, p->normals[i].y );
	}
	g.centroid = gv( p->centroid.x, p->centroid.y );
	return create_shape( bodyId, def, b2_polygonShape, &g );
}

b2ShapeId b2CreateCircleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Circle* c )
{
	b2gShapeGeo g;
	memset( &g, 0, sizeof( g ) );
	g.v[0] = gv( c->center.x, c->center.y );
	g.radius = c->radius;
	g.centroid = g.v[0];
	return create_shape( bodyId, def, b2_circleShape, &g );
}

b2ShapeId b2CreateCapsuleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Capsule* c )
{
	float lengthSqr = b2DistanceSquared( c->center1, c->center2 );
	if ( lengthSqr <= B2G_LINEAR_SLOP * B2G_LINEAR_SLOP )
	{
		b2Circle circle = { b2Lerp( c->center1, c->center2, 0.5f ), c->radius };
		return b2CreateCircleShape( bodyId, def, &circle );
	}
	b2gShapeGeo g;
	memset( &g, 0, sizeof( g ) );
	g.v[0] = gv( c->center1.x, c->center1.y );
	g.v[1] = gv( c->center2.x, c->center2.y );
	g.radius = c->radius;
	g.centroid = glerp( g.v[0], g.v[1], 0.5f );
	return create_shape( bodyId, def, b2_capsuleShape, &g );
}

b2ShapeId b2CreateSegmentShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Segment* sgm )
{
	float lengthSqr = b2DistanceSquared( sgm->point1, sgm->point2 );
	if ( lengthSqr <= B2G_LINEAR_SLOP * B2G_LINEAR_SLOP )
	{
		gworld_fail( "b2CreateSegmentShape: segment too short" );
		return b2_nullShapeId;
	}
	b2gShapeGeo g;
	memset( &g, 0, sizeof( g ) );
	g.v[0] = gv( sgm->point1.x, sgm->point1.y );
	g.v[1] = gv( sgm->point2.x, sgm->point2.y );
	g.centroid = glerp( g.v[0], g.v[1], 0.5f );
	return create_shape( bodyId, def, b2_segmentShape, &g );
}

static gShape* get_shape( b2ShapeId id ) { return s_worlds[id.world0]->shapes + ( id.index1 - 1 ); }

bool b2Shape_IsValid( b2ShapeId id )
{
	if ( id.world0 >= s_worldCap || s_worlds[id.world0] == NULL || !s_worlds[id.world0]->inUse )
		return false;
	gWorld* w = s_worlds[id.world0];
	if ( id.index1 < 1 || id.index1 > w->shapeCap )
		return false;
	gShape* s = w->shapes + id.index1 - 1;
	return s->id == id.index1 - 1 && s->revision == id.revision;
}
b2ShapeType b2Shape_GetType( b2ShapeId id ) { return get_shape( id )->type; }
b2BodyId b2Shape_GetBody( b2ShapeId id )
{
	gWorld* w = s_worlds[id.world0];
	gShape* s = get_shape( id );
	b2BodyId b = { s->bodyId + 1, id.world0, w->bodies[s->bodyId].revision };
	return b;
}
float b2Shape_GetDensity( b2ShapeId id ) { return get_shape( id )->density; }
void b2Shape_SetFriction( b2ShapeId id, float f ) { get_shape( id )->friction = f; }
float b2Shape_GetFriction( b2ShapeId id ) { return get_shape( id )->friction; }
void b2Shape_SetRestitution( b2ShapeId id, float r ) { get_shape( id )->restitution = r; }
float b2Shape_GetRestitution( b2ShapeId id ) { return get_shape( id )->restitution; }
b2Filter b2Shape_GetFilter( b2ShapeId id ) { return get_shape( id )->filter; }
b2Polygon b2Shape_GetPolygon( b2ShapeId id )
{
	const b2gShapeGeo* g = s_worlds[id.world0]->hGeo + ( id.index1 - 1 );
	b2Polygon p;
	memset( &p, 0, sizeof( p ) );
	p.count = g->count;
	p.radius = g->radius;
	p.centroid = ( b2Vec2 ){ g->centroid.x, g->centroid.y };
	for ( int i = 0; i < g->count; ++i )
	{
		p.vertices[i] = ( b2Vec2 ){ g->v[i].x, g->v[i].y };
		p.normals[i] = ( b2Vec2 ){ g->n[i].x, g->n[i].y };
	}
	return p;
}
b2Segment b2Shape_GetSegment( b2ShapeId id )
{
	const b2gShapeGeo* g = s_worlds[id.world0]->hGeo + ( id.index1 - 1 );
	b2Segment r = { { g->v[0].x, g->v[0].y }, { g->v[1].x, g->v[1].y } };
	return r;
}

b2SmoothSegment b2Shape_GetSmoothSegment( b2ShapeId id )
{
	gWorld* w = s_worlds[id.world0];
	const b2gShapeGeo* g = w->hGeo + ( id.index1 - 1 );
	b2SmoothSegment r;
	r.ghost1 = ( b2Vec2 ){ g->v[2].x, g->v[2].y };
	r.segment.point1 = ( b2Vec2 ){ g->v[0].x, g->v[0].y };
	r.segment.point2 = ( b2Vec2 ){ g->v[1].x, g->v[1].y };
	r.ghost2 = ( b2Vec2 ){ g->v[3].x, g->v[3].y };
	r.chainId = w->shapes[id.index1 - 1].chainId;
	return r;
}

b2Capsule b2Shape_GetCapsule( b2ShapeId id )
{
	const b2gShapeGeo* g = s_worlds[id.world0]->hGeo + ( id.index1 - 1 );
	b2Capsule r = { { g->v[0].x, g->v[0].y }, { g->v[1].x, g->v[1].y }, g->radius };
	return r;
}

b2Circle b2Shape_GetCircle( b2ShapeId id )
{
	const b2gShapeGeo* g = s_worlds[id.world0]->hGeo + ( id.index1 - 1 );
	b2Circle c = { { g->v[0].x, g->v[0].y }, g->radius };
	return c;
}
b2AABB b2Shape_GetAABB( b2ShapeId id )
{
	gWorld* w = s_worlds[id.world0];
	gworld_ensure_shape_mirror( w );
	const float* a = w->hAabb + 4 * ( id.index1 - 1 );
	b2AABB r = { { a[0], a[1] }, { a[2], a[3] } };
	return r;
}

/* ------------------------------------------------------------ joints */
int gassign_joint_color( gWorld* w, int bodyIdA, int bodyIdB, bool staticA, bool staticB )
{
	for ( int i = 0; i < B2G_COLORS; ++i )
	{
		gBits* set = &w->colors[i].bodySet;
		if ( staticA == false && staticB == false )
		{
			if ( gbits_get( set, bodyIdA ) || gbits_get( set, bodyIdB ) )
				continue;
			gbits_set( set, bodyIdA );
			gbits_set( set, bodyIdB );
			return i;
		}
		else if ( staticA == false )
		{
			if ( gbits_get( set, bodyIdA ) )
				continue;
			gbits_set( set, bodyIdA );
			return i;
		}
		else if ( staticB == false )
		{
			if ( gbits_get( set, bodyIdB ) )
				continue;
			gbits_set( set, bodyIdB );
			return i;
		}
		else
			break;
	}
	return B2G_OVERFLOW;
}

/* Joint record shared by every joint type (reference src/joint.c:140-288): allocates the
 * id, links the joint into both bodies' joint lists and puts it in the constraint graph.
 * Returns the joint's zeroed device record with its type and bodies set, or NULL when the
 * world or a body is invalid, the world is locked, or host memory ran out. */
b2gJointDev* gjoint_create( b2WorldId worldId, b2BodyId bodyIdA, b2BodyId bodyIdB, b2JointType type, bool collideConnected,
							void* userData, b2JointId* out )
{
	*out = b2_nullJointId;
	if ( b2World_IsValid( worldId ) == false || b2Body_IsValid( bodyIdA ) == false || b2Body_IsValid( bodyIdB ) == false )
		return NULL;
	gWorld* w = gworld_get( worldId );
	if ( w->locked )
		return NULL;
	ensure_joint_mirror( w );
	gBody* a = get_body( bodyIdA );
	gBody* b = get_body( bodyIdB );
	int id = gid_alloc( &w->jointIds );
	bool ok = true;
	GROW_RECORDS( w->joints, w->jointCap, id + 1, gJoint, ok );
	if ( ok == false || gworld_reserve_mirrors( w ) == false )
	{
		gid_unalloc( &w->jointIds, id );
		w->status = w->status ? w->status : B2_STATUS_OUT_OF_HOST_MEMORY;
		return NULL;
	}
	gJoint* j = w->joints + id;
	uint16_t rev = j->revision;
	memset( j, 0, sizeof( *j ) );
	j->id = id;
	j->revision = (uint16_t)( rev + 1 );
	j->type = type;
	j->bodyIdA = a->id;
	j->bodyIdB = b->id;
	j->userData = userData;
	j->collideConnected = collideConnected;

	j->edges[0].bodyId = a->id;
	j->edges[0].prevKey = B2G_NULL;
	j->edges[0].nextKey = a->headJointKey;
	int keyA = ( id << 1 ) | 0;
	if ( a->headJointKey != B2G_NULL )
		w->joints[a->headJointKey >> 1].edges[a->headJointKey & 1].prevKey = keyA;
	a->headJointKey = keyA;
	a->jointCount += 1;

	j->edges[1].bodyId = b->id;
	j->edges[1].prevKey = B2G_NULL;
	j->edges[1].nextKey = b->headJointKey;
	int keyB = ( id << 1 ) | 1;
	if ( b->headJointKey != B2G_NULL )
		w->joints[b->headJointKey >> 1].edges[b->headJointKey & 1].prevKey = keyB;
	b->headJointKey = keyB;
	b->jointCount += 1;

	j->islandId = B2G_NULL;
	j->islandPrev = B2G_NULL;
	j->islandNext = B2G_NULL;
	j->colorIndex = B2G_NULL;

	/* solver set (reference src/joint.c:198-283): between static bodies the static set;
	 * touching the awake set the constraint graph, after waking a sleeping partner;
	 * otherwise the sleeping set, merging two sleeping sets */
	int maxSetIndex = a->setIndex > b->setIndex ? a->setIndex : b->setIndex;
	if ( a->setIndex == G_SET_STATIC && b->setIndex == G_SET_STATIC )
	{
		j->setIndex = G_SET_STATIC;
		j->localIndex = w->staticJoints.count;
		gia_push( &w->staticJoints, id );
	}
	else if ( a->setIndex == G_SET_AWAKE || b->setIndex == G_SET_AWAKE )
	{
		if ( maxSetIndex >= G_SET_FIRST_SLEEPING )
			gsolver_set_wake( w, maxSetIndex );
		j->setIndex = G_SET_AWAKE;
		bool staticA = a->setIndex == G_SET_STATIC;
		bool staticB = b->setIndex == G_SET_STATIC;
		int color = gassign_joint_color( w, a->id, b->id, staticA, staticB );
		j->colorIndex = color;
		j->localIndex = w->colors[color].joints.count;
		gia_push( &w->colors[color].joints, id );
		w->solveDirty = true;
	}
	else
	{
		j->setIndex = maxSetIndex;
		j->localIndex = w->sets[maxSetIndex].joints.count;
		gia_push( &w->sets[maxSetIndex].joints, id );
		if ( a->setIndex != b->setIndex && a->setIndex >= G_SET_FIRST_SLEEPING && b->setIndex >= G_SET_FIRST_SLEEPING )
			gsolver_set_merge( w, a->setIndex, b->setIndex );
	}
	if ( j->setIndex > G_SET_DISABLED )
		gisland_link_joint( w, j );

	b2gJointDev* d = w->hJoints + id;
	memset( d, 0, sizeof( *d ) );
	d->type = (int32_t)type;
	d->bodyIdA = a->id;
	d->bodyIdB = b->id;
	d->indexA = B2G_NULL;
	d->indexB = B2G_NULL;
	w->jointsDirty = true;
	b2JointId jid = { id + 1, (uint16_t)w->slot, j->revision };
	*out = jid;
	return d;
}

/* Destroys the contacts between a joint's two bodies (reference src/joint.c:290-322),
 * walking the shorter contact list. */
void gjoint_disconnect_bodies( gWorld* w, int bodyIdA, int bodyIdB )
{
	gBody* a = w->bodies + bodyIdA;
	gBody* b = w->bodies + bodyIdB;
	int key, other;
	if ( a->contactCount < b->contactCount )
	{
		key = a->headContactKey;
		other = b->id;
	}
	else
	{
		key = b->headContactKey;
		other = a->id;
	}
	while ( key != B2G_NULL )
	{
		gContact* c = w->contacts + ( key >> 1 );
		int e = key & 1;
		key = c->edges[e].nextKey;
		if ( c->edges[e ^ 1].bodyId == other )
			gcontact_destroy( w, c, false );
	}
}

void gworld_ensure_joint_mirror( gWorld* w ) { ensure_joint_mirror( w ); }

static gJoint* get_joint( b2JointId id ) { return s_worlds[id.world0]->joints + ( id.index1 - 1 ); }

bool b2Joint_IsValid( b2JointId id )
{
	if ( id.world0 >= s_worldCap || s_worlds[id.world0] == NULL || !s_worlds[id.world0]->inUse )
		return false;
	gWorld* w = s_worlds[id.world0];
	if ( id.index1 < 1 || id.index1 > w->jointCap )
		return false;
	return w->joints[id.index1 - 1].id == id.index1 - 1 && w->joints[id.index1 - 1].revision == id.revision;
}

/* ------------------------------------------------------------ introspection */
int b2World_InspectBodies( b2WorldId worldId, float* out, int capacity )
{
	gWorld* w = gworld_get( worldId );
	gworld_ensure_mirror( w );
	int count = w->bodyIds.next;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		float* o = out + B2_INSPECT_BODY_FLOATS * i;
		if ( w->bodies[i].id != i )
		{
			for ( int k = 0; k < B2_INSPECT_BODY_FLOATS; ++k )
				o[k] = NAN;
			continue;
		}
		const float* x = w->hXf + 4 * i;
		const float* s = w->hState + 8 * i;
		/* velocities live in the awake set only */
		bool moving = w->bodies[i].setIndex == G_SET_AWAKE;
		o[0] = x[0];
		o[1] = x[1];
		o[2] = x[2];
		o[3] = x[3];
		o[4] = moving ? s[0] : 0.0f;
		o[5] = moving ? s[1] : 0.0f;
		o[6] = moving ? s[2] : 0.0f;
		o[7] = (float)w->bodies[i].type;
	}
	return count;
}

int b2World_InspectIslands( b2WorldId worldId, int* out, int capacity )
{
	gWorld* w = gworld_get( worldId );
	int count = w->bodyIds.next;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		const gBody* b = w->bodies + i;
		out[2 * i] = b->id == i ? b->setIndex : -1;
		out[2 * i + 1] = b->id == i ? b->islandId : -1;
	}
	return count;
}

int b2World_InspectShapes( b2WorldId worldId, b2InspectShape* out, int capacity )
{
	gWorld* w = gworld_get( worldId );
	gworld_ensure_shape_mirror( w );
	int count = w->shapeIds.next;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		b2InspectShape* o = out + i;
		memset( o, 0, sizeof( *o ) );
		if ( w->shapes[i].id != i )
		{
			o->proxyKey = -1;
			o->bodyId = -1;
			continue;
		}
		memcpy( o->aabb, w->hAabb + 4 * i, 16 );
		memcpy( o->fatAABB, w->hFat + 4 * i, 16 );
		o->proxyKey = w->shapes[i].proxyKey;
		o->bodyId = w->shapes[i].bodyId;
	}
	return count;
}

int b2World_InspectContacts( b2WorldId worldId, b2InspectContact* out, int capacity )
{
	gWorld* w = gworld_get( worldId );
	int nc = w->contactIds.next;
	b2gManifold* ms = NULL;
	int n = 0;
	for ( int i = 0; i < nc; ++i )
	{
		gContact* c = w->contacts + i;
		if ( c->id != i )
			continue;
		if ( n < capacity )
		{
			if ( ms == NULL )
			{
				ms = (b2gManifold*)b2g_alloc( sizeof( b2gManifold ) * (size_t)nc );
				if ( ms == NULL || b2gd_download_manifolds( &w->dev, ms, NULL, nc ) != 0 )
				{
					b2g_free( ms );
					return 0;
				}
			}
			const b2gManifold* m = ms + i;
			b2InspectContact* o = out + n;
			memset( o, 0, sizeof( *o ) );
			o->contactId = i;
			o->shapeIdA = c->shapeIdA;
			o->shapeIdB = c->shapeIdB;
			o->colorIndex = c->colorIndex;
			o->localIndex = c->localIndex;
			o->touching = ( c->flags & G_TOUCHING ) ? 1 : 0;
			o->pointCount = m->count;
			o->normal[0] = m->normal.x;
			o->normal[1] = m->normal.y;
			o->friction = c->friction;
			o->restitution = c->restitution;
			for ( int k = 0; k < 2; ++k )
			{
				const b2gPoint* mp = m->pts + k;
				b2InspectPoint* p = o->points + k;
				p->anchorA[0] = mp->anchorA.x;
				p->anchorA[1] = mp->anchorA.y;
				p->anchorB[0] = mp->anchorB.x;
				p->anchorB[1] = mp->anchorB.y;
				p->point[0] = mp->point.x;
				p->point[1] = mp->point.y;
				p->separation = mp->separation;
				p->normalImpulse = mp->normalImpulse;
				p->tangentImpulse = mp->tangentImpulse;
				p->maxNormalImpulse = mp->maxNormalImpulse;
				p->normalVelocity = mp->normalVelocity;
				p->id = mp->id;
				p->persisted = mp->persisted;
			}
		}
		n += 1;
	}
	b2g_free( ms );
	return n;
}

/* ------------------------------------------------------------ box2d/gpu.h */
int b2World_GetStatus( b2WorldId worldId ) { return gworld_get( worldId )->status; }

int b2World_GetToiEventCount( b2WorldId worldId ) { return gworld_get( worldId )->toiEvents; }

void b2World_EnableDeviceTiming( b2WorldId worldId, bool flag )
{
	gWorld* w = gworld_get( worldId );
	b2gd_enable_timing( &w->dev, flag ? 1 : 0 );
}

b2DeviceTimes b2World_GetDeviceTimes( b2WorldId worldId )
{
	gWorld* w = gworld_get( worldId );
	b2DeviceTimes t;
	memset( &t, 0, sizeof( t ) );
	b2gd_stage_times( &w->dev, &t.step, &t.collide, &t.solve, &t.finalize );
	t.eventCount = w->lastEventCount;
	t.recordCount = w->lastRecordCount;
	t.launches = w->dev.launches;
	t.fusedSolver = w->dev.fusedUsed;
	t.hostToDeviceBytes = w->dev.h2dBytes;
	t.deviceToHostBytes = w->dev.d2hBytes;
	t.hostPairQuery = w->hostMs[0];
	t.hostPairRules = w->hostMs[1];
	t.hostContactCreate = w->hostMs[2];
	t.hostEvents = w->hostMs[3];
	t.hostSolveLists = w->hostMs[4];
	t.hostTreeRebuild = w->hostMs[5];
	t.hostRecords = w->hostMs[6];
	t.hostContinuous = w->hostMs[7];
	return t;
}

void b2World_EnableFusedSolver( b2WorldId worldId, bool flag )
{
	gWorld* w = gworld_get( worldId );
	w->dev.fused = flag ? 1 : 0;
}

int b2World_GetBodyStates( b2WorldId worldId, float* out, int capacity )
{
	gWorld* w = gworld_get( worldId );
	gworld_ensure_mirror( w );
	int n = w->bodyIds.next;
	for ( int i = 0; i < n && i < capacity; ++i )
	{
		const float* x = w->hXf + 4 * i;
		const float* s = w->hState + 8 * i;
		bool moving = w->bodies[i].id == i && w->bodies[i].type != b2_staticBody;
		float* o = out + 7 * i;
		o[0] = x[0];
		o[1] = x[1];
		o[2] = x[2];
		o[3] = x[3];
		o[4] = moving ? s[0] : 0.0f;
		o[5] = moving ? s[1] : 0.0f;
		o[6] = moving ? s[2] : 0.0f;
	}
	return n;
}

/* Diagnostics: raw copy of a device array of the world (see b2gd_debug_read). */
int b2gd_debug_read( b2gDevWorld* w, int which, void* out, int count );
int b2World_DebugRead( b2WorldId worldId, int which, void* out, int count )
{
	return b2gd_debug_read( &gworld_get( worldId )->dev, which, out, count );
}

int b2gd_debug_collide( b2gDevWorld* w, int id, float* hostOut );
int b2World_DebugCollide( b2WorldId worldId, int contactId, float* out64 )
{
	return b2gd_debug_collide( &gworld_get( worldId )->dev, contactId, out64 );
}

/* ------------------------------------------------------------ destruction
 * Reference src/body.c:161-176, :336-430 (b2DestroyBody), src/shape.c:220-290
 * (b2DestroyShapeInternal, b2DestroyShape), src/shape.c:704-711 with
 * src/broad_phase.c:71-116 (proxy destruction and the move-buffer purge),
 * src/joint.c:657-768 (b2DestroyJointInternal) with src/constraint_graph.c:297-324.
 * Islands and sleep are not built, so waking the bodies touched is a no-op.  Device
 * records of destroyed ids stay in place unused: contacts are retired before the next
 * narrowphase, and the awake list, shape lists and solve lists that the kernels walk
 * are rebuilt without them. */
static void unbuffer_move( gWorld* w, int proxyKey )
{
	if ( gset_remove( &w->moveSet, (uint64_t)( proxyKey + 1 ) ) == false )
		return;
	for ( int i = 0; i < w->moveArray.count; ++i )
	{
		if ( w->moveArray.data[i] == proxyKey )
		{
			gia_remove_swap( &w->moveArray, i );
			break;
		}
	}
}

static void destroy_proxy( gWorld* w, gShape* s )
{
	if ( s->proxyKey == B2G_NULL )
		return;
	unbuffer_move( w, s->proxyKey );
	gtree_destroy_proxy( w->trees + ( s->proxyKey & 3 ), s->proxyKey >> 2 );
	s->proxyKey = B2G_NULL;
}

static void unlink_joint_edge( gWorld* w, gJoint* j, int e )
{
	gEdge* edge = j->edges + e;
	gBody* body = w->bodies + edge->bodyId;
	if ( edge->prevKey != B2G_NULL )
		w->joints[edge->prevKey >> 1].edges[edge->prevKey & 1].nextKey = edge->nextKey;
	if ( edge->nextKey != B2G_NULL )
		w->joints[edge->nextKey >> 1].edges[edge->nextKey & 1].prevKey = edge->prevKey;
	int key = ( j->id << 1 ) | e;
	if ( body->headJointKey == key )
		body->headJointKey = edge->nextKey;
	body->jointCount -= 1;
}

/* Reference src/joint.c:657-752. */
static void destroy_joint( gWorld* w, gJoint* j, bool wakeBodies )
{
	int bodyIdA = j->edges[0].bodyId;
	int bodyIdB = j->edges[1].bodyId;
	unlink_joint_edge( w, j, 0 );
	unlink_joint_edge( w, j, 1 );
	gisland_unlink_joint( w, j );
	if ( j->setIndex != G_SET_AWAKE )
	{
		gIntArray* list = gsolver_set_joints( w, j->setIndex );
		int moved = gia_remove_swap( list, j->localIndex );
		if ( moved != B2G_NULL )
			w->joints[list->data[j->localIndex]].localIndex = j->localIndex;
	}
	else
	{
		/* swap-remove from the colour: the overflow colour is solved in array order */
		gColor* color = w->colors + j->colorIndex;
		if ( j->colorIndex != B2G_OVERFLOW )
		{
			gbits_clear( &color->bodySet, j->edges[0].bodyId );
			gbits_clear( &color->bodySet, j->edges[1].bodyId );
		}
		int moved = gia_remove_swap( &color->joints, j->localIndex );
		if ( moved != B2G_NULL )
			w->joints[color->joints.data[j->localIndex]].localIndex = j->localIndex;
		w->solveDirty = true;
	}
	int id = j->id;
	j->setIndex = B2G_NULL;
	j->colorIndex = B2G_NULL;
	j->localIndex = B2G_NULL;
	j->id = B2G_NULL;
	gid_free( &w->jointIds, id );
	if ( wakeBodies )
	{
		gbody_wake( w, w->bodies + bodyIdA );
		gbody_wake( w, w->bodies + bodyIdB );
	}
}

void b2DestroyJoint( b2JointId jointId )
{
	if ( b2Joint_IsValid( jointId ) == false )
		return;
	gWorld* w = s_worlds[jointId.world0];
	if ( w->locked )
		return;
	destroy_joint( w, get_joint( jointId ), true );
}

/* Unlinks and frees a shape with its proxy and contacts (reference
 * src/shape.c:220-269). */
static void destroy_shape_internal( gWorld* w, gShape* s, gBody* b, bool wakeBodies )
{
	int id = s->id;
	if ( s->prev != B2G_NULL )
		w->shapes[s->prev].next = s->next;
	if ( s->next != B2G_NULL )
		w->shapes[s->next].prev = s->prev;
	if ( b->headShape == id )
		b->headShape = s->next;
	b->shapeCount -= 1;
	destroy_proxy( w, s );
	int key = b->headContactKey;
	while ( key != B2G_NULL )
	{
		gContact* c = w->contacts + ( key >> 1 );
		key = c->edges[key & 1].nextKey;
		if ( c->shapeIdA == id || c->shapeIdB == id )
			gcontact_destroy( w, c, wakeBodies );
	}
	gid_free( &w->shapeIds, id );
	s->id = B2G_NULL;
	if ( s->enableHitEvents )
		w->hitShapes -= 1;
	w->shapeListsDirty = true;
}

void b2DestroyShape( b2ShapeId shapeId )
{
	if ( b2Shape_IsValid( shapeId ) == false )
		return;
	gWorld* w = s_worlds[shapeId.world0];
	if ( w->locked )
		return;
	gworld_ensure_mirror( w );
	gworld_ensure_shape_mirror( w );
	gShape* s = get_shape( shapeId );
	gBody* b = w->bodies + s->bodyId;
	destroy_shape_internal( w, s, b, true );
	if ( b->automaticMass )
		gbody_update_mass( w, b );
	w->bodiesDirty = true;
}

/* ------------------------------------------------------------ chains */
/* Chain creation (reference src/shape.c:292-403): one smooth segment per link, each
 * with the neighbouring points as ghost vertices; a loop closes on its first point. */
b2ChainId b2CreateChain( b2BodyId bodyId, const b2ChainDef* def )
{
	if ( b2Body_IsValid( bodyId ) == false || def->count < 4 || def->points == NULL )
		return b2_nullChainId;
	gWorld* w = body_world( bodyId );
	if ( w->locked )
		return b2_nullChainId;
	gworld_ensure_mirror( w );
	int n = def->count;
	int links = def->isLoop ? n : n - 3;
	int* indices = (int*)b2g_alloc( sizeof( int ) * (size_t)n );
	int chainId = gid_alloc( &w->chainIds );
	bool ok = indices != NULL;
	if ( ok )
		GROW_RECORDS( w->chains, w->chainCap, chainId + 1, gChain, ok );
	if ( ok == false )
	{
		b2g_free( indices );
		gid_unalloc( &w->chainIds, chainId );
		w->status = w->status ? w->status : B2_STATUS_OUT_OF_HOST_MEMORY;
		return b2_nullChainId;
	}
	gBody* body = get_body( bodyId );
	gChain* chain = w->chains + chainId;
	uint16_t rev = chain->revision;
	memset( chain, 0, sizeof( *chain ) );
	chain->revision = (uint16_t)( rev + 1 );
	chain->id = chainId;
	chain->bodyId = body->id;
	chain->nextChainId = body->headChainId;
	chain->shapeIndices = indices;
	chain->count = links;
	body->headChainId = chainId;

	b2ShapeDef sd = b2DefaultShapeDef();
	sd.userData = def->userData;
	sd.restitution = def->restitution;
	sd.friction = def->friction;
	sd.filter = def->filter;
	sd.enableContactEvents = false;
	sd.enableHitEvents = false;
	sd.enableSensorEvents = false;

	const b2Vec2* pts = def->points;
	for ( int i = 0; i < links; ++i )
	{
		/* ghost1, point1, point2, ghost2 of link i */
		int i0, i1, i2, i3;
		if ( def->isLoop )
		{
			i1 = i;
			i2 = ( i + 1 ) % n;
			i0 = ( i + n - 1 ) % n;
			i3 = ( i + 2 ) % n;
		}
		else
		{
			i0 = i;
			i1 = i + 1;
			i2 = i + 2;
			i3 = i + 3;
		}
		b2gShapeGeo g;
		memset( &g, 0, sizeof( g ) );
		g.count = 2;
		g.v[0] = gv( pts[i1].x, pts[i1].y );
		g.v[1] = gv( pts[i2].x, pts[i2].y );
		g.v[2] = gv( pts[i0].x, pts[i0].y );
		g.v[3] = gv( pts[i3].x, pts[i3].y );
		g.centroid = glerp( g.v[0], g.v[1], 0.5f );
		b2ShapeId sid = create_shape_internal( bodyId, &sd, b2_smoothSegmentShape, &g, false );
		int shapeId = sid.index1 - 1;
		indices[i] = shapeId;
		if ( shapeId >= 0 )
			w->shapes[shapeId].chainId = chainId;
	}
	b2ChainId id = { chainId + 1, (uint16_t)w->slot, chain->revision };
	return id;
}

static gChain* get_chain( b2ChainId id ) { return s_worlds[id.world0]->chains + ( id.index1 - 1 ); }

bool b2Chain_IsValid( b2ChainId id )
{
	if ( id.world0 >= s_worldCap || s_worlds[id.world0] == NULL || !s_worlds[id.world0]->inUse )
		return false;
	gWorld* w = s_worlds[id.world0];
	if ( id.index1 < 1 || id.index1 > w->chainCap )
		return false;
	gChain* c = w->chains + ( id.index1 - 1 );
	return c->id == id.index1 - 1 && c->revision == id.revision;
}

/* Chain destruction (reference src/shape.c:405-451). */
void b2DestroyChain( b2ChainId chainId )
{
	if ( b2Chain_IsValid( chainId ) == false )
		return;
	gWorld* w = s_worlds[chainId.world0];
	if ( w->locked )
		return;
	gworld_ensure_mirror( w );
	gworld_ensure_shape_mirror( w );
	gChain* chain = get_chain( chainId );
	gBody* body = w->bodies + chain->bodyId;
	int* link = &body->headChainId;
	while ( *link != B2G_NULL && *link != chain->id )
		link = &w->chains[*link].nextChainId;
	if ( *link == B2G_NULL )
		return;
	*link = chain->nextChainId;
	for ( int i = 0; i < chain->count; ++i )
	{
		int sid = chain->shapeIndices[i];
		if ( sid >= 0 && w->shapes[sid].id == sid )
			destroy_shape_internal( w, w->shapes + sid, body, true );
	}
	b2g_free( chain->shapeIndices );
	chain->shapeIndices = NULL;
	gid_free( &w->chainIds, chain->id );
	chain->id = B2G_NULL;
}

void b2Chain_SetFriction( b2ChainId chainId, float friction )
{
	gWorld* w = s_worlds[chainId.world0];
	if ( w->locked )
		return;
	gChain* chain = get_chain( chainId );
	for ( int i = 0; i < chain->count; ++i )
		w->shapes[chain->shapeIndices[i]].friction = friction;
}

void b2Chain_SetRestitution( b2ChainId chainId, float restitution )
{
	gWorld* w = s_worlds[chainId.world0];
	if ( w->locked )
		return;
	gChain* chain = get_chain( chainId );
	for ( int i = 0; i < chain->count; ++i )
		w->shapes[chain->shapeIndices[i]].restitution = restitution;
}

b2ChainId b2Shape_GetParentChain( b2ShapeId shapeId )
{
	gWorld* w = s_worlds[shapeId.world0];
	gShape* s = get_shape( shapeId );
	if ( s->type == b2_smoothSegmentShape && s->chainId != B2G_NULL )
	{
		b2ChainId id = { s->chainId + 1, shapeId.world0, w->chains[s->chainId].revision };
		return id;
	}
	return b2_nullChainId;
}

void b2DestroyBody( b2BodyId bodyId )
{
	if ( b2Body_IsValid( bodyId ) == false )
		return;
	gWorld* w = body_world( bodyId );
	if ( w->locked )
		return;
	gworld_ensure_mirror( w );
	gBody* b = get_body( bodyId );
	/* bodies attached through joints and contacts wake, even when this one is static */
	int key = b->headJointKey;
	while ( key != B2G_NULL )
	{
		gJoint* j = w->joints + ( key >> 1 );
		key = j->edges[key & 1].nextKey;
		destroy_joint( w, j, true );
	}
	key = b->headContactKey;
	while ( key != B2G_NULL )
	{
		gContact* c = w->contacts + ( key >> 1 );
		key = c->edges[key & 1].nextKey;
		gcontact_destroy( w, c, true );
	}
	for ( int sid = b->headShape; sid != B2G_NULL; )
	{
		gShape* s = w->shapes + sid;
		destroy_proxy( w, s );
		gid_free( &w->shapeIds, sid );
		s->id = B2G_NULL;
		if ( s->enableHitEvents )
			w->hitShapes -= 1;
		sid = s->next;
	}
	/* the chains' shapes went with the body's shapes above (reference src/body.c:381-395) */
	for ( int cid = b->headChainId; cid != B2G_NULL; )
	{
		gChain* chain = w->chains + cid;
		b2g_free( chain->shapeIndices );
		chain->shapeIndices = NULL;
		gid_free( &w->chainIds, cid );
		chain->id = B2G_NULL;
		cid = chain->nextChainId;
	}
	/* the body's set drops it by moving its last body into the slot */
	gisland_remove_body( w, b );
	gbody_remove_from_set( w, b );
	w->hInfo[b->id] = 0;
	gid_free( &w->bodyIds, b->id );
	b->setIndex = B2G_NULL;
	b->awakeIndex = B2G_NULL;
	b->id = B2G_NULL;
	w->bodiesDirty = true;
	w->shapeListsDirty = true;
	w->solveDirty = true;
}
