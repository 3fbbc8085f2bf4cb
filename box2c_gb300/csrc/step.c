/*
 * step.c -- b2World_Step on the GB300: host bookkeeping around two device stages.
 *
 *   1. broadphase pairs (host trees, reference src/broad_phase.c:162-436) create contacts
 *      in the reference order; their sim records are staged for the device;
 *   2. device: contact creation + narrowphase over every live contact (kernels.cu);
 *      meanwhile the host rebuilds the trees (src/dynamic_tree.c:1811-1925);
 *   3. host: begin/end/disjoint events in ascending contact id, contact destruction and
 *      graph colouring (src/world.c:489-667, src/constraint_graph.c:64-214);
 *   4. device: the soft-step solver, colour by colour, and body finalisation;
 *   5. host: proxy enlargement in awake order and the fast-body pass
 *      (src/solver.c:1741-1954).
 * Steps 3 and 5 only touch the few contacts and proxies whose state changed.
 */
#include "host.h"
#include "b2g_toi.h"
#include "box2d/gpu.h"

#include <string.h>

#define PAIR_KEY( K1, K2 ) ( ( K1 ) < ( K2 ) ? (uint64_t)( K1 ) << 32 | (uint64_t)( K2 ) : (uint64_t)( K2 ) << 32 | (uint64_t)( K1 ) )

/* ------------------------------------------------------------ event lists */
static void push_begin( gWorld* w, int a, int b )
{
	if ( w->beginCount == w->beginCap )
	{
		int cap = w->beginCap ? 2 * w->beginCap : 16;
		void* p = b2g_realloc( w->beginEvents, sizeof( b2ContactBeginTouchEvent ) * (size_t)cap );
		if ( p == NULL )
			return;
		w->beginEvents = p;
		w->beginCap = cap;
	}
	b2ContactBeginTouchEvent* e = w->beginEvents + w->beginCount++;
	e->shapeIdA = ( b2ShapeId ){ a + 1, (uint16_t)w->slot, w->shapes[a].revision };
	e->shapeIdB = ( b2ShapeId ){ b + 1, (uint16_t)w->slot, w->shapes[b].revision };
}

static void push_end( gWorld* w, int a, int b )
{
	if ( w->endCount == w->endCap )
	{
		int cap = w->endCap ? 2 * w->endCap : 16;
		void* p = b2g_realloc( w->endEvents, sizeof( b2ContactEndTouchEvent ) * (size_t)cap );
		if ( p == NULL )
			return;
		w->endEvents = p;
		w->endCap = cap;
	}
	b2ContactEndTouchEvent* e = w->endEvents + w->endCount++;
	e->shapeIdA = ( b2ShapeId ){ a + 1, (uint16_t)w->slot, w->shapes[a].revision };
	e->shapeIdB = ( b2ShapeId ){ b + 1, (uint16_t)w->slot, w->shapes[b].revision };
}

static b2ShapeId shape_id( gWorld* w, int s ) { return ( b2ShapeId ){ s + 1, (uint16_t)w->slot, w->shapes[s].revision }; }

/* Sensor overlap events (reference src/world.c:563-580, :606-624): one per sensor shape
 * of the pair, the sensor first. */
static void push_sensor( gWorld* w, bool begin, int sensor, int visitor )
{
	if ( begin )
	{
		if ( w->sensorBeginCount == w->sensorBeginCap )
		{
			int cap = w->sensorBeginCap ? 2 * w->sensorBeginCap : 16;
			void* p = b2g_realloc( w->sensorBeginEvents, sizeof( b2SensorBeginTouchEvent ) * (size_t)cap );
			if ( p == NULL )
				return;
			w->sensorBeginEvents = p;
			w->sensorBeginCap = cap;
		}
		b2SensorBeginTouchEvent* e = w->sensorBeginEvents + w->sensorBeginCount++;
		e->sensorShapeId = shape_id( w, sensor );
		e->visitorShapeId = shape_id( w, visitor );
	}
	else
	{
		if ( w->sensorEndCount == w->sensorEndCap )
		{
			int cap = w->sensorEndCap ? 2 * w->sensorEndCap : 16;
			void* p = b2g_realloc( w->sensorEndEvents, sizeof( b2SensorEndTouchEvent ) * (size_t)cap );
			if ( p == NULL )
				return;
			w->sensorEndEvents = p;
			w->sensorEndCap = cap;
		}
		b2SensorEndTouchEvent* e = w->sensorEndEvents + w->sensorEndCount++;
		e->sensorShapeId = shape_id( w, sensor );
		e->visitorShapeId = shape_id( w, visitor );
	}
}

static void sensor_events( gWorld* w, gContact* c, bool begin )
{
	if ( ( c->flags & G_ENABLE_SENSOR_EVENTS ) == 0 )
		return;
	if ( w->shapes[c->shapeIdA].isSensor )
		push_sensor( w, begin, c->shapeIdA, c->shapeIdB );
	if ( w->shapes[c->shapeIdB].isSensor )
		push_sensor( w, begin, c->shapeIdB, c->shapeIdA );
}

/* Hit events of the step (reference src/solver.c:1670-1723): the contacts of the graph
 * colours in colour and array order whose shapes enable hit events, tested on the
 * device against their solved manifolds. */
static void report_hits( gWorld* w )
{
	if ( w->hitShapes == 0 )
		return;
	int n = 0;
	for ( int i = 0; i < B2G_COLORS; ++i )
		n += w->colors[i].contacts.count;
	if ( n == 0 || b2gd_reserve_hits( &w->io, n ) != 0 )
		return;
	n = 0;
	for ( int i = 0; i < B2G_COLORS; ++i )
	{
		gIntArray* a = &w->colors[i].contacts;
		for ( int j = 0; j < a->count; ++j )
		{
			gContact* c = w->contacts + a->data[j];
			if ( w->shapes[c->shapeIdA].enableHitEvents || w->shapes[c->shapeIdB].enableHitEvents )
				w->io.hitIds[n++] = c->id;
		}
	}
	if ( n == 0 )
		return;
	int e = b2gd_hit_events( &w->dev, &w->io, n, w->hitThreshold );
	if ( e )
	{
		w->status = e;
		return;
	}
	for ( int k = 0; k < n; ++k )
	{
		const float* r = w->io.hitOut + 8 * k;
		if ( r[0] == 0.0f )
			continue;
		if ( w->hitCount == w->hitCap )
		{
			int cap = w->hitCap ? 2 * w->hitCap : 16;
			void* p = b2g_realloc( w->hitEvents, sizeof( b2ContactHitEvent ) * (size_t)cap );
			if ( p == NULL )
				return;
			w->hitEvents = p;
			w->hitCap = cap;
		}
		gContact* c = w->contacts + w->io.hitIds[k];
		b2ContactHitEvent* h = w->hitEvents + w->hitCount++;
		h->shapeIdA = shape_id( w, c->shapeIdA );
		h->shapeIdB = shape_id( w, c->shapeIdB );
		h->point = ( b2Vec2 ){ r[2], r[3] };
		h->normal = ( b2Vec2 ){ r[4], r[5] };
		h->approachSpeed = r[1];
	}
}

/* ------------------------------------------------------------ contacts */
/* Contact records staged for the device, applied in order before the next narrowphase
 * (creation, or retirement of a contact destroyed outside the narrowphase). */
static b2gContactInit* push_pending( gWorld* w )
{
	if ( w->pendingCount == w->pendingCap )
	{
		int cap = w->pendingCap ? 2 * w->pendingCap : 256;
		b2gContactInit* p = (b2gContactInit*)b2g_realloc( w->pending, sizeof( b2gContactInit ) * (size_t)cap );
		if ( p == NULL )
		{
			/* out of memory: the record is written nowhere and the world fails at the
			 * next check of its API call */
			static _Thread_local b2gContactInit sink;
			return &sink;
		}
		w->pending = p;
		w->pendingCap = cap;
	}
	return w->pending + w->pendingCount++;
}

/* Keeps only the last staged record of each contact id (ids can be freed and reused
 * between two steps), so the device can apply them in parallel.  A set record (the
 * contact moved into or out of the awake set) that follows a creation or another set
 * record of the same contact folds into it. */
static int compact_pending( gWorld* w )
{
	int n = w->pendingCount;
	int ids = w->contactIds.next > 0 ? w->contactIds.next : 1;
	for ( int i = 0; i < n; ++i )
		if ( w->pending[i].id + 1 > ids )
			ids = w->pending[i].id + 1;
	if ( ids > w->scratchCap )
	{
		int* p = (int*)b2g_realloc( w->scratch, sizeof( int ) * (size_t)ids );
		if ( p == NULL )
			return -1;
		w->scratch = p;
		w->scratchCap = ids;
	}
	for ( int i = 0; i < n; ++i )
		w->scratch[w->pending[i].id] = B2G_NULL;
	for ( int i = 0; i < n; ++i )
	{
		b2gContactInit* r = w->pending + i;
		int last = w->scratch[r->id];
		if ( ( r->flags & B2G_INIT_SET ) && last != B2G_NULL && ( w->pending[last].flags & B2G_INIT_KILL ) == 0 )
		{
			b2gContactInit* base = w->pending + last;
			base->flags = ( base->flags & ~B2G_INIT_ASLEEP ) | ( r->flags & B2G_INIT_ASLEEP );
			r->flags = B2G_INIT_KILL | B2G_INIT_SET; /* folded: dropped below */
			continue;
		}
		w->scratch[r->id] = i;
	}
	int m = 0;
	for ( int i = 0; i < n; ++i )
		if ( w->scratch[w->pending[i].id] == i )
			w->pending[m++] = w->pending[i];
	return m;
}

/* Registered shape pairs and primary order (reference src/contact.c:150-183). */
static int registered( b2ShapeType a, b2ShapeType b, bool* primary )
{
	static const int table[5][5] = {
		{ 1, -1, -1, -1, -1 }, { 1, 1, -1, -1, -1 }, { 1, 1, 0, 1, 0 }, { 1, 1, -1, 1, -1 }, { 1, 1, 0, 1, 0 },
	};
	int v = table[a][b];
	if ( v == 0 )
		return 0;
	*primary = v > 0;
	return 1;
}

void gcontact_create( gWorld* w, gShape* shapeA, gShape* shapeB )
{
	bool primary;
	if ( registered( shapeA->type, shapeB->type, &primary ) == 0 )
		return;
	if ( primary == false )
	{
		gcontact_create( w, shapeB, shapeA );
		return;
	}
	gBody* bodyA = w->bodies + shapeA->bodyId;
	gBody* bodyB = w->bodies + shapeB->bodyId;
	int id = gid_alloc( &w->contactIds );
	if ( id + 1 > w->contactCap )
	{
		int nc = w->contactCap < 64 ? 64 : w->contactCap;
		while ( nc < id + 1 )
			nc *= 2;
		gContact* p = (gContact*)b2g_realloc( w->contacts, sizeof( gContact ) * (size_t)nc );
		if ( p == NULL )
		{
			gid_unalloc( &w->contactIds, id );
			return;
		}
		w->contacts = p;
		for ( int i = w->contactCap; i < nc; ++i )
			w->contacts[i].id = B2G_NULL;
		w->contactCap = nc;
	}
	gContact* c = w->contacts + id;
	memset( c, 0, sizeof( *c ) );
	c->id = id;
	/* non-touching contacts of two bodies that are not awake live in the disabled set
	 * (reference src/contact.c:210-222) */
	int setIndex = bodyA->setIndex == G_SET_AWAKE || bodyB->setIndex == G_SET_AWAKE ? G_SET_AWAKE : G_SET_DISABLED;
	gIntArray* list = gsolver_set_contacts( w, setIndex );
	c->setIndex = setIndex;
	c->colorIndex = B2G_NULL;
	c->localIndex = list->count;
	c->islandId = B2G_NULL;
	c->islandPrev = B2G_NULL;
	c->islandNext = B2G_NULL;
	c->shapeIdA = shapeA->id;
	c->shapeIdB = shapeB->id;
	if ( shapeA->isSensor || shapeB->isSensor )
		c->flags |= G_SENSOR;
	if ( shapeA->enableSensorEvents || shapeB->enableSensorEvents )
		c->flags |= G_ENABLE_SENSOR_EVENTS;
	if ( shapeA->enableContactEvents || shapeB->enableContactEvents )
		c->flags |= G_ENABLE_CONTACT_EVENTS;
	c->friction = sqrtf( shapeA->friction * shapeB->friction );
	c->restitution = shapeA->restitution > shapeB->restitution ? shapeA->restitution : shapeB->restitution;

	c->edges[0].bodyId = shapeA->bodyId;
	c->edges[0].prevKey = B2G_NULL;
	c->edges[0].nextKey = bodyA->headContactKey;
	int keyA = ( id << 1 ) | 0;
	if ( bodyA->headContactKey != B2G_NULL )
		w->contacts[bodyA->headContactKey >> 1].edges[bodyA->headContactKey & 1].prevKey = keyA;
	bodyA->headContactKey = keyA;
	bodyA->contactCount += 1;

	c->edges[1].bodyId = shapeB->bodyId;
	c->edges[1].prevKey = B2G_NULL;
	c->edges[1].nextKey = bodyB->headContactKey;
	int keyB = ( id << 1 ) | 1;
	if ( bodyB->headContactKey != B2G_NULL )
		w->contacts[bodyB->headContactKey >> 1].edges[bodyB->headContactKey & 1].prevKey = keyB;
	bodyB->headContactKey = keyB;
	bodyB->contactCount += 1;

	gset_add( &w->pairSet, PAIR_KEY( (uint64_t)shapeA->id, (uint64_t)shapeB->id ) );
	w->pairSetVersion += 1;
	gia_push( list, id );

	b2gContactInit* init = push_pending( w );
	init->id = id;
	init->shapeA = shapeA->id;
	init->shapeB = shapeB->id;
	init->friction = c->friction;
	init->restitution = c->restitution;
	init->flags = setIndex == G_SET_AWAKE ? 0u : B2G_INIT_ASLEEP;
}

void gcontact_stage_set( gWorld* w, int contactId, bool asleep )
{
	b2gContactInit* r = push_pending( w );
	memset( r, 0, sizeof( *r ) );
	r->id = contactId;
	r->flags = B2G_INIT_SET | ( asleep ? B2G_INIT_ASLEEP : 0u );
}

static void remove_non_touching( gWorld* w, int localIndex )
{
	int moved = gia_remove_swap( &w->nonTouching, localIndex );
	if ( moved != B2G_NULL )
		w->contacts[w->nonTouching.data[localIndex]].localIndex = localIndex;
}

void gcontact_remove_from_graph( gWorld* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex )
{
	gColor* color = w->colors + colorIndex;
	if ( colorIndex != B2G_OVERFLOW )
	{
		gbits_clear( &color->bodySet, bodyIdA );
		gbits_clear( &color->bodySet, bodyIdB );
	}
	int moved = gia_remove_swap( &color->contacts, localIndex );
	if ( moved != B2G_NULL )
		w->contacts[color->contacts.data[localIndex]].localIndex = localIndex;
	w->solveDirty = true;
}

static void unlink_edge( gWorld* w, gContact* c, int e )
{
	gEdge* edge = c->edges + e;
	gBody* body = w->bodies + edge->bodyId;
	if ( edge->prevKey != B2G_NULL )
		w->contacts[edge->prevKey >> 1].edges[edge->prevKey & 1].nextKey = edge->nextKey;
	if ( edge->nextKey != B2G_NULL )
		w->contacts[edge->nextKey >> 1].edges[edge->nextKey & 1].prevKey = edge->prevKey;
	int key = ( c->id << 1 ) | e;
	if ( body->headContactKey == key )
		body->headContactKey = edge->nextKey;
	body->contactCount -= 1;
}

/* Reference src/contact.c:320-449.  The device record is retired by the narrowphase
 * (disjoint) or ignored once its id is free. */
void gcontact_destroy( gWorld* w, gContact* c, bool wakeBodies )
{
	gset_remove( &w->pairSet, PAIR_KEY( (uint64_t)c->shapeIdA, (uint64_t)c->shapeIdB ) );
	w->pairSetVersion += 1;
	int bodyIdA = c->edges[0].bodyId;
	int bodyIdB = c->edges[1].bodyId;
	unlink_edge( w, c, 0 );
	unlink_edge( w, c, 1 );
	if ( c->islandId != B2G_NULL )
		gisland_unlink_contact( w, c );
	if ( c->colorIndex != B2G_NULL )
		gcontact_remove_from_graph( w, bodyIdA, bodyIdB, c->colorIndex, c->localIndex );
	else
	{
		gIntArray* list = gsolver_set_contacts( w, c->setIndex );
		int moved = gia_remove_swap( list, c->localIndex );
		if ( moved != B2G_NULL )
			w->contacts[list->data[c->localIndex]].localIndex = c->localIndex;
	}
	int id = c->id;
	c->id = B2G_NULL;
	c->setIndex = B2G_NULL;
	c->colorIndex = B2G_NULL;
	c->localIndex = B2G_NULL;
	gid_free( &w->contactIds, id );
	if ( wakeBodies )
	{
		gbody_wake( w, w->bodies + bodyIdA );
		gbody_wake( w, w->bodies + bodyIdB );
	}
	/* retire the device record before the next narrowphase */
	b2gContactInit* kill = push_pending( w );
	memset( kill, 0, sizeof( *kill ) );
	kill->id = id;
	kill->flags = B2G_INIT_KILL;
}

/* Greedy first-fit colouring keyed by body id (reference src/constraint_graph.c:64-183). */
void gcontact_add_to_graph( gWorld* w, gContact* c )
{
	int colorIndex = B2G_OVERFLOW;
	int a = c->edges[0].bodyId;
	int b = c->edges[1].bodyId;
	bool staticA = w->bodies[a].type == b2_staticBody;
	bool staticB = w->bodies[b].type == b2_staticBody;
	if ( staticA == false && staticB == false )
	{
		for ( int i = 0; i < B2G_OVERFLOW; ++i )
		{
			gBits* set = &w->colors[i].bodySet;
			if ( gbits_get( set, a ) || gbits_get( set, b ) )
				continue;
			gbits_set( set, a );
			gbits_set( set, b );
			colorIndex = i;
			break;
		}
	}
	else if ( staticA == false )
	{
		for ( int i = 1; i < B2G_OVERFLOW; ++i )
		{
			gBits* set = &w->colors[i].bodySet;
			if ( gbits_get( set, a ) )
				continue;
			gbits_set( set, a );
			colorIndex = i;
			break;
		}
	}
	else if ( staticB == false )
	{
		for ( int i = 1; i < B2G_OVERFLOW; ++i )
		{
			gBits* set = &w->colors[i].bodySet;
			if ( gbits_get( set, b ) )
				continue;
			gbits_set( set, b );
			colorIndex = i;
			break;
		}
	}
	gColor* color = w->colors + colorIndex;
	c->colorIndex = colorIndex;
	c->localIndex = color->contacts.count;
	gia_push( &color->contacts, c->id );
	w->solveDirty = true;
}

/* ------------------------------------------------------------ broadphase pairs */
typedef struct gQueryCtx
{
	gWorld* w;
	gPairList* list;
	int queryTreeType, queryProxyKey, queryShapeIndex;
} gQueryCtx;

static bool should_shapes_collide( b2Filter a, b2Filter b )
{
	if ( a.groupIndex == b.groupIndex && a.groupIndex != 0 )
		return a.groupIndex > 0;
	return ( a.maskBits & b.categoryBits ) != 0 && ( a.categoryBits & b.maskBits ) != 0;
}

static bool should_bodies_collide( gWorld* w, gBody* a, gBody* b )
{
	if ( a->type != b2_dynamicBody && b->type != b2_dynamicBody )
		return false;
	int key, other;
	if ( a->jointCount < b->jointCount )
	{
		key = a->headJointKey;
		other = b->id;
	}
	else
	{
		key = b->headJointKey;
		other = a->id;
	}
	while ( key != B2G_NULL )
	{
		gJoint* j = w->joints + ( key >> 1 );
		int e = key & 1;
		if ( j->collideConnected == false && j->edges[e ^ 1].bodyId == other )
			return false;
		key = j->edges[e].nextKey;
	}
	return true;
}

static bool pair_query( int proxyId, int shapeId, void* context )
{
	gQueryCtx* q = (gQueryCtx*)context;
	gWorld* w = q->w;
	int proxyKey = ( proxyId << 2 ) | q->queryTreeType;
	if ( proxyKey == q->queryProxyKey )
		return true;
	if ( q->queryTreeType != b2_staticBody )
	{
		bool moved = gset_contains( &w->moveSet, (uint64_t)( proxyKey + 1 ) );
		if ( moved && proxyKey < q->queryProxyKey )
			return true;
	}
	if ( gset_contains( &w->pairSet, PAIR_KEY( (uint64_t)shapeId, (uint64_t)q->queryShapeIndex ) ) )
		return true;
	int idA, idB;
	if ( proxyKey < q->queryProxyKey )
	{
		idA = shapeId;
		idB = q->queryShapeIndex;
	}
	else
	{
		idA = q->queryShapeIndex;
		idB = shapeId;
	}
	gShape* sA = w->shapes + idA;
	gShape* sB = w->shapes + idB;
	if ( sA->bodyId == sB->bodyId )
		return true;
	if ( should_shapes_collide( sA->filter, sB->filter ) == false )
		return true;
	if ( sA->isSensor && sB->isSensor )
		return true;
	if ( should_bodies_collide( w, w->bodies + sA->bodyId, w->bodies + sB->bodyId ) == false )
		return true;
	gPairList* l = q->list;
	if ( l->count == l->capacity )
	{
		int cap = l->capacity ? 2 * l->capacity : 16;
		int* a = (int*)b2g_realloc( l->a, sizeof( int ) * (size_t)cap );
		if ( a != NULL )
			l->a = a;
		int* b = a != NULL ? (int*)b2g_realloc( l->b, sizeof( int ) * (size_t)cap ) : NULL;
		if ( b == NULL )
			return false;
		l->b = b;
		l->capacity = cap;
	}
	l->a[l->count] = idA;
	l->b[l->count] = idB;
	l->count += 1;
	return true;
}

/* Moved proxies from which the tree query runs on the device: below this a host query
 * costs less than the device round trip (upload, launch, synchronise). */
#define DEVICE_QUERY_MIN_MOVES 256
/* Moved proxies per chunk when the pair rules run on the host pool, and the host tree
 * walks below which the rules run on the calling thread. */
#define PAIR_GRAIN 64
#define PAIR_POOL_MIN_WALKS 32

typedef struct gPairCtx
{
	gWorld* w;
	gPairList* lists;
	const int* cand;
	const int* counts;
} gPairCtx;

/* Pairs of moved proxies [begin, end): the device's candidates, or a host tree walk,
 * through pair_query.  Reads the trees, move and pair sets, shapes, bodies and joints,
 * writes only the proxies' own lists, so ranges run in parallel. */
static void query_moved( int begin, int end, void* arg )
{
	gPairCtx* c = (gPairCtx*)arg;
	gWorld* w = c->w;
	for ( int i = begin; i < end; ++i )
	{
		int proxyKey = w->moveArray.data[i];
		if ( proxyKey == B2G_NULL )
			continue;
		int proxyType = proxyKey & 3;
		int proxyId = proxyKey >> 2;
		const gTree* base = w->trees + proxyType;
		b2gBox fat = base->nodes[proxyId].box;
		gQueryCtx q;
		q.w = w;
		q.list = c->lists + i;
		q.queryProxyKey = proxyKey;
		q.queryShapeIndex = base->nodes[proxyId].userData;
		if ( c->counts != NULL && c->counts[i] >= 0 )
		{
			const int* cand = c->cand + 2 * B2G_QUERY_SLOTS * i;
			for ( int k = 0; k < c->counts[i]; ++k )
			{
				q.queryTreeType = cand[2 * k] & 3;
				pair_query( cand[2 * k] >> 2, cand[2 * k + 1], &q );
			}
			continue;
		}
		if ( proxyType == b2_dynamicBody )
		{
			q.queryTreeType = b2_kinematicBody;
			gtree_query( w->trees + b2_kinematicBody, fat, 0xFFFFFFFFu, pair_query, &q );
			q.queryTreeType = b2_staticBody;
			gtree_query( w->trees + b2_staticBody, fat, 0xFFFFFFFFu, pair_query, &q );
		}
		q.queryTreeType = b2_dynamicBody;
		gtree_query( w->trees + b2_dynamicBody, fat, 0xFFFFFFFFu, pair_query, &q );
	}
}

/* All moved proxies are queried before any contact is created (reference
 * src/broad_phase.c:333-436, the queries as parallel tasks); each proxy's pairs are then
 * created in move order, in reverse discovery order (the reference prepends to a list).
 * With many moved proxies the tree walks run on the device (pairs.cu) and their
 * candidate leaves pass through pair_query in the order the host walk would report
 * them; the pair rules run on the host pool when it is free.  Returns 0 or a CUDA
 * error. */
static int update_pairs( gWorld* w )
{
	int moveCount = w->moveArray.count;
	if ( moveCount == 0 )
		return 0;
	gPairCtx c;
	c.w = w;
	c.cand = NULL;
	c.counts = NULL;
	double t0 = b2g_now_ms();
	if ( moveCount >= DEVICE_QUERY_MIN_MOVES )
	{
		const b2gTreeNode* nodes[3];
		int capacity[3], root[3];
		for ( int t = 0; t < 3; ++t )
		{
			nodes[t] = w->trees[t].nodes;
			capacity[t] = w->trees[t].capacity;
			root[t] = w->trees[t].root;
		}
		int e = b2gd_pair_query( &w->dev, &w->pairQuery, nodes, capacity, root, w->moveArray.data, moveCount,
								 (const unsigned long long*)w->pairSet.keys, w->pairSet.capacity, w->pairSetVersion, &c.cand,
								 &c.counts );
		if ( e )
			return e;
	}
	double t1 = b2g_now_ms();
	if ( moveCount > w->pairListCap )
	{
		int cap = w->pairListCap < 64 ? 64 : w->pairListCap;
		while ( cap < moveCount )
			cap *= 2;
		gPairList* lists = (gPairList*)b2g_realloc( w->pairLists, sizeof( gPairList ) * (size_t)cap );
		if ( lists == NULL )
			return -1;
		memset( lists + w->pairListCap, 0, sizeof( gPairList ) * (size_t)( cap - w->pairListCap ) );
		w->pairLists = lists;
		w->pairListCap = cap;
	}
	c.lists = w->pairLists;
	for ( int i = 0; i < moveCount; ++i )
		c.lists[i].count = 0;
	/* After the device walk only candidates that pass its rules remain, and the host work
	 * per proxy is a few loads: the pool pays only when proxies fall back to host walks. */
	int hostWalks = moveCount;
	if ( c.counts != NULL )
	{
		hostWalks = 0;
		for ( int i = 0; i < moveCount; ++i )
			hostWalks += c.counts[i] < 0;
	}
	if ( hostWalks < PAIR_POOL_MIN_WALKS || gpool_try_for( moveCount, PAIR_GRAIN, query_moved, &c ) == false )
		query_moved( 0, moveCount, &c );
	double t2 = b2g_now_ms();
	for ( int i = 0; i < moveCount; ++i )
	{
		gPairList* l = c.lists + i;
		for ( int k = l->count - 1; k >= 0; --k )
			gcontact_create( w, w->shapes + l->a[k], w->shapes + l->b[k] );
	}
	w->moveArray.count = 0;
	gset_clear( &w->moveSet );
	double t3 = b2g_now_ms();
	w->hostMs[0] = (float)( t1 - t0 );
	w->hostMs[1] = (float)( t2 - t1 );
	w->hostMs[2] = (float)( t3 - t2 );
	return 0;
}

/* ------------------------------------------------------------ narrowphase events */
static int cmp_int( const void* a, const void* b )
{
	int x = *(const int*)a, y = *(const int*)b;
	return ( x > y ) - ( x < y );
}

static void process_events( gWorld* w, int count )
{
	int* ev = w->io.events;
	qsort( ev, (size_t)count, sizeof( int ), cmp_int );
	for ( int i = 0; i < count; ++i )
	{
		int id = ev[i] >> 2;
		int code = ev[i] & 3;
		gContact* c = w->contacts + id;
		uint32_t flags = c->flags;
		if ( code == B2G_EV_DISJOINT )
		{
			if ( ( flags & G_TOUCHING ) && ( flags & G_ENABLE_CONTACT_EVENTS ) )
				push_end( w, c->shapeIdA, c->shapeIdB );
			c->flags &= ~G_TOUCHING;
			gcontact_destroy( w, c, false );
		}
		else if ( code == B2G_EV_STARTED )
		{
			if ( flags & G_SENSOR )
			{
				sensor_events( w, c, true );
				c->flags |= G_SENSOR_TOUCHING;
				continue;
			}
			if ( flags & G_ENABLE_CONTACT_EVENTS )
				push_begin( w, c->shapeIdA, c->shapeIdB );
			/* link first: it may wake a sleeping set, which appends to the awake lists
			 * and leaves this contact's place unchanged */
			c->flags |= G_TOUCHING;
			gisland_link_contact( w, c );
			int localIndex = c->localIndex;
			gcontact_add_to_graph( w, c );
			remove_non_touching( w, localIndex );
		}
		else if ( code == B2G_EV_STOPPED )
		{
			if ( flags & G_SENSOR )
			{
				c->flags &= ~G_SENSOR_TOUCHING;
				sensor_events( w, c, false );
				continue;
			}
			c->flags &= ~G_TOUCHING;
			if ( c->flags & G_ENABLE_CONTACT_EVENTS )
				push_end( w, c->shapeIdA, c->shapeIdB );
			gisland_unlink_contact( w, c );
			int a = c->edges[0].bodyId, b = c->edges[1].bodyId;
			int colorIndex = c->colorIndex, localIndex = c->localIndex;
			c->setIndex = G_SET_AWAKE;
			c->colorIndex = B2G_NULL;
			c->localIndex = w->nonTouching.count;
			gia_push( &w->nonTouching, id );
			gcontact_remove_from_graph( w, a, b, colorIndex, localIndex );
		}
	}
}

/* ------------------------------------------------------------ finalisation records */
static int cmp_record( const void* a, const void* b )
{
	const b2gRecord* x = (const b2gRecord*)a;
	const b2gRecord* y = (const b2gRecord*)b;
	if ( x->awakeIndex != y->awakeIndex )
		return ( x->awakeIndex > y->awakeIndex ) - ( x->awakeIndex < y->awakeIndex );
	return ( x->slot > y->slot ) - ( x->slot < y->slot );
}

static b2gBox box4( const float* f )
{
	b2gBox b;
	b.lo = gv( f[0], f[1] );
	b.hi = gv( f[2], f[3] );
	return b;
}

/* Continuous collision of one fast body (reference src/solver.c:787-1105): the static
 * shapes (and, for a bullet, kinematic and dynamic shapes) its shapes sweep over, in the
 * host trees' query order, lower the body's time-of-impact fraction. */
typedef struct gSweepCtx
{
	gWorld* w;
	gShape* fast;
	gBody* fastBody;
	b2gSweep sweep;
	b2gVec centroid1, centroid2; /* the fast shape's centroid at the sweep's ends */
	float fraction;
} gSweepCtx;

/* Sweep of a body from the host mirrors: static bodies never move; the others are read
 * after the mirrors were refreshed from the device. */
static b2gSweep mirror_sweep( const gWorld* w, int bodyId )
{
	const float* x = w->hXf + 4 * bodyId;
	const float* c = w->hCenters + 4 * bodyId;
	const float* p = w->hPrev + 4 * bodyId;
	b2gSweep s;
	s.c1 = gv( p[0], p[1] );
	s.c2 = gv( c[0], c[1] );
	s.q1 = grot( p[2], p[3] );
	s.q2 = grot( x[2], x[3] );
	s.localCenter = gv( c[2], c[3] );
	return s;
}

static bool sweep_query( int proxyId, int shapeId, void* context )
{
	(void)proxyId;
	gSweepCtx* q = (gSweepCtx*)context;
	gWorld* w = q->w;
	if ( shapeId == q->fast->id )
		return true;
	gShape* s = w->shapes + shapeId;
	if ( s->bodyId == q->fast->bodyId )
		return true;
	if ( should_shapes_collide( q->fast->filter, s->filter ) == false )
		return true;
	if ( s->isSensor )
		return true;
	gBody* body = w->bodies + s->bodyId;
	if ( body->isBullet )
		return true;
	if ( should_bodies_collide( w, q->fastBody, body ) == false )
		return true;
	/* a chain link is passed over when the fast shape starts behind it or ends in front
	 * of it, so bodies do not pause at link junctions (reference src/solver.c:869-885) */
	if ( s->type == b2_smoothSegmentShape )
	{
		const float* x = w->hXf + 4 * s->bodyId;
		b2gXf t;
		t.p = gv( x[0], x[1] );
		t.q = grot( x[2], x[3] );
		const b2gShapeGeo* g = w->hGeo + shapeId;
		b2gVec p1 = gxfpoint( t, g->v[0] );
		b2gVec p2 = gxfpoint( t, g->v[1] );
		b2gVec e = gsub( p2, p1 );
		float offset1 = gcross( gsub( q->centroid1, p1 ), e );
		float offset2 = gcross( gsub( q->centroid2, p1 ), e );
		if ( offset1 < 0.0f || offset2 > 0.0f )
			return true;
	}

	b2gProxy pa = gproxy_shape( w->hGeo + shapeId );
	b2gProxy pb = gproxy_shape( w->hGeo + q->fast->id );
	b2gSweep sa = mirror_sweep( w, s->bodyId );
	int state;
	float t = gtime_of_impact( &pa, &sa, &pb, &q->sweep, q->fraction, &state );
	if ( 0.0f < t && t < q->fraction )
		q->fraction = t;
	else if ( 0.0f == t )
	{
		/* fall back to a small circle around the fast shape's centroid */
		b2gVec centroid = gshape_centroid( w->hGeo + q->fast->id );
		pb = gproxy_points( &centroid, 1, B2G_SPECULATIVE );
		t = gtime_of_impact( &pa, &sa, &pb, &q->sweep, q->fraction, &state );
		if ( 0.0f < t && t < q->fraction )
			q->fraction = t;
	}
	return true;
}

/* recs: the body's records (one per shape, in shape-list order).  With an impact the
 * body is moved back along its sweep on the device and the records carry the fat boxes
 * of the new pose; without one the device's pose and boxes stand. */
static void solve_continuous( gWorld* w, b2gRecord* recs, int n, bool bullet )
{
	int bodyId = w->awake.data[recs[0].awakeIndex];
	gBody* b = w->bodies + bodyId;
	gSweepCtx q;
	q.w = w;
	q.fastBody = b;
	q.fraction = 1.0f;
	q.sweep.c1 = gv( recs[0].pose1[0], recs[0].pose1[1] );
	q.sweep.q1 = grot( recs[0].pose1[2], recs[0].pose1[3] );
	q.sweep.c2 = gv( recs[0].pose2[0], recs[0].pose2[1] );
	q.sweep.q2 = grot( recs[0].pose2[2], recs[0].pose2[3] );
	q.sweep.localCenter = gv( w->hCenters[4 * bodyId + 2], w->hCenters[4 * bodyId + 3] );
	b2gXf xf1, xf2;
	xf1.q = q.sweep.q1;
	xf1.p = gsub( q.sweep.c1, grotate( q.sweep.q1, q.sweep.localCenter ) );
	xf2.q = q.sweep.q2;
	xf2.p = gsub( q.sweep.c2, grotate( q.sweep.q2, q.sweep.localCenter ) );
	for ( int k = 0; k < n; ++k )
	{
		gShape* s = w->shapes + recs[k].shapeId;
		q.centroid1 = gxfpoint( xf1, gshape_centroid( w->hGeo + s->id ) );
		q.centroid2 = gxfpoint( xf2, gshape_centroid( w->hGeo + s->id ) );
		if ( s->isSensor )
			continue;
		q.fast = s;
		b2gBox sweep = box4( recs[k].sweep );
		gtree_query( w->trees + b2_staticBody, sweep, 0xFFFFFFFFu, sweep_query, &q );
		if ( bullet )
		{
			gtree_query( w->trees + b2_kinematicBody, sweep, 0xFFFFFFFFu, sweep_query, &q );
			gtree_query( w->trees + b2_dynamicBody, sweep, 0xFFFFFFFFu, sweep_query, &q );
		}
	}
	if ( q.fraction >= 1.0f )
		return;

	/* time-of-impact event */
	float f = q.fraction;
	b2gRot rq = gnormrot( grot( ( 1.0f - f ) * q.sweep.q1.c + f * q.sweep.q2.c, ( 1.0f - f ) * q.sweep.q1.s + f * q.sweep.q2.s ) );
	b2gVec c = glerp( q.sweep.c1, q.sweep.c2, f );
	b2gXf xf;
	xf.q = rq;
	xf.p = gsub( c, grotate( rq, q.sweep.localCenter ) );
	float xf4[4] = { xf.p.x, xf.p.y, rq.c, rq.s };
	float center4[4] = { c.x, c.y, q.sweep.localCenter.x, q.sweep.localCenter.y };
	float prev4[4] = { c.x, c.y, rq.c, rq.s };
	int e = b2gd_upload_pose( &w->dev, bodyId, xf4, center4, prev4 );
	if ( w->mirrorStale == false )
	{
		memcpy( w->hXf + 4 * bodyId, xf4, 16 );
		memcpy( w->hCenters + 4 * bodyId, center4, 16 );
		memcpy( w->hPrev + 4 * bodyId, prev4, 16 );
	}
	for ( int k = 0; k < n; ++k )
	{
		b2gRecord* r = recs + k;
		b2gBox aabb = gshape_geo_aabb( w->hGeo + r->shapeId, xf );
		aabb.lo.x -= B2G_SPECULATIVE;
		aabb.lo.y -= B2G_SPECULATIVE;
		aabb.hi.x += B2G_SPECULATIVE;
		aabb.hi.y += B2G_SPECULATIVE;
		b2gBox fat = box4( w->hFat + 4 * r->shapeId );
		r->flags &= ~B2G_R_FAST_ENLARGED;
		if ( gbox_contains( fat, aabb ) == false )
		{
			fat.lo.x = aabb.lo.x - B2G_AABB_MARGIN;
			fat.lo.y = aabb.lo.y - B2G_AABB_MARGIN;
			fat.hi.x = aabb.hi.x + B2G_AABB_MARGIN;
			fat.hi.y = aabb.hi.y + B2G_AABB_MARGIN;
			r->flags |= B2G_R_FAST_ENLARGED;
		}
		float aabb4[4] = { aabb.lo.x, aabb.lo.y, aabb.hi.x, aabb.hi.y };
		float fat4[4] = { fat.lo.x, fat.lo.y, fat.hi.x, fat.hi.y };
		memcpy( r->fat, fat4, 16 );
		e |= b2gd_upload_shape_boxes( &w->dev, r->shapeId, aabb4, fat4 );
	}
	if ( e )
		w->status = e;
	w->toiEvents += 1;
	if ( w->tape )
		w->tapeToiEvents += 1;
}

/* Continuous collision of the fast bodies of one class (bullets or not), then their
 * grown fat boxes into the dynamic tree (reference src/solver.c:1839-1950: fast bodies
 * first, then bullets, which see the fast bodies' proxies). */
static void continuous_pass( gWorld* w, b2gRecord* rec, int count, bool bullets )
{
	bool mirrored = false;
	for ( int i = 0; i < count; )
	{
		b2gRecord* r = rec + i;
		int end = i + 1;
		while ( end < count && rec[end].awakeIndex == r->awakeIndex )
			++end;
		if ( ( r->flags & B2G_R_FAST ) && ( ( r->flags & B2G_R_BULLET ) != 0 ) == bullets )
		{
			if ( bullets && mirrored == false )
			{
				/* a bullet sweeps against moving bodies: their poses after this step */
				w->mirrorStale = true;
				gworld_ensure_mirror( w );
				mirrored = true;
			}
			solve_continuous( w, r, end - i, bullets );
		}
		i = end;
	}
	for ( int i = 0; i < count; ++i )
	{
		b2gRecord* r = rec + i;
		if ( ( r->flags & B2G_R_FAST ) == 0 || ( ( r->flags & B2G_R_BULLET ) != 0 ) != bullets )
			continue;
		if ( r->flags & B2G_R_FAST_ENLARGED )
		{
			gShape* s = w->shapes + r->shapeId;
			memcpy( w->hFat + 4 * r->shapeId, r->fat, 16 );
			gtree_enlarge_proxy( w->trees + b2_dynamicBody, s->proxyKey >> 2, box4( r->fat ) );
		}
	}
}

/* Records sorted by awake index with a counting sort.  A body's records come from one
 * device thread in slot order, so the sort, which is stable, leaves them in slot order.
 * Falls back to a comparison sort in place when memory for the buckets runs out. */
static b2gRecord* sort_records( gWorld* w, int count )
{
	b2gRecord* rec = w->io.records;
	int n = w->awake.count + 1;
	if ( count > w->recordSortCap )
	{
		b2gRecord* p = (b2gRecord*)b2g_realloc( w->recordSort, sizeof( b2gRecord ) * (size_t)count );
		if ( p != NULL )
		{
			w->recordSort = p;
			w->recordSortCap = count;
		}
	}
	if ( n > w->recordBucketCap )
	{
		int* p = (int*)b2g_realloc( w->recordBucket, sizeof( int ) * (size_t)n );
		if ( p != NULL )
		{
			w->recordBucket = p;
			w->recordBucketCap = n;
		}
	}
	if ( count > w->recordSortCap || n > w->recordBucketCap )
	{
		qsort( rec, (size_t)count, sizeof( b2gRecord ), cmp_record );
		return rec;
	}
	int* first = w->recordBucket;
	memset( first, 0, sizeof( int ) * (size_t)n );
	for ( int i = 0; i < count; ++i )
		first[rec[i].awakeIndex + 1] += 1;
	for ( int k = 1; k < n; ++k )
		first[k] += first[k - 1];
	b2gRecord* out = w->recordSort;
	for ( int i = 0; i < count; ++i )
		out[first[rec[i].awakeIndex]++] = rec[i];
	return out;
}

static void process_records( gWorld* w, int count )
{
	b2gRecord* rec = sort_records( w, count );
	/* proxy enlargement and move buffer in awake order (reference src/solver.c:1741-1797) */
	for ( int i = 0; i < count; ++i )
	{
		b2gRecord* r = rec + i;
		gShape* s = w->shapes + r->shapeId;
		if ( r->flags & B2G_R_ENLARGED )
		{
			memcpy( w->hFat + 4 * r->shapeId, r->fat, 16 );
			gtree_enlarge_proxy( w->trees + ( s->proxyKey & 3 ), s->proxyKey >> 2, box4( r->fat ) );
			gbuffer_move( w, s->proxyKey );
		}
		else if ( r->flags & B2G_R_FAST )
		{
			gbuffer_move( w, s->proxyKey );
		}
	}
	double t0 = b2g_now_ms();
	continuous_pass( w, rec, count, false );
	continuous_pass( w, rec, count, true );
	w->hostMs[7] = (float)( b2g_now_ms() - t0 );
}

/* ------------------------------------------------------------ step */
static void make_soft( float hertz, float zeta, float h, float* out )
{
	if ( hertz == 0.0f )
	{
		out[0] = 0.0f;
		out[1] = 1.0f;
		out[2] = 0.0f;
		return;
	}
	float omega = 2.0f * B2G_PI * hertz;
	float a1 = 2.0f * zeta + h * omega;
	float a2 = h * omega * a1;
	float a3 = 1.0f / ( 1.0f + a2 );
	out[0] = omega / a1;
	out[1] = a2 * a3;
	out[2] = a3;
}

/* Owner CTA of a contact row in the fused solver: the block of its first non-static
 * body. */
static int row_owner( gWorld* w, const gContact* c, int block )
{
	int a = c->edges[0].bodyId, b = c->edges[1].bodyId;
	int key = w->bodies[a].type != b2_staticBody ? a : b;
	int o = key / block;
	return o < B2G_FUSED_CTAS ? o : B2G_FUSED_CTAS - 1;
}

/* Colour-major solve lists.  Within a graph colour the order of rows does not change any
 * result (no two rows of a colour share a non-static body), so rows are grouped by owner
 * CTA (a stable counting sort); the overflow colour keeps its order, which is the order
 * it is solved in.  Rebuilt only when the colouring or the body count changed. */
static void build_solve_lists( gWorld* w, b2gSolvePlan* plan )
{
	int bodyIdCount = w->bodyIds.next;
	int block = ( bodyIdCount + B2G_FUSED_CTAS - 1 ) / B2G_FUSED_CTAS;
	if ( block < 1 )
		block = 1;
	if ( w->solveDirty == false && w->solvePlan.bodyBlock == block )
	{
		*plan = w->solvePlan;
		return;
	}
	memset( plan, 0, sizeof( *plan ) );
	int rows = 0, joints = 0;
	for ( int c = 0; c < B2G_COLORS; ++c )
	{
		rows += w->colors[c].contacts.count;
		joints += w->colors[c].joints.count;
	}
	if ( gia_reserve( &w->solveList, rows ) == false || gia_reserve( &w->jointList, joints ) == false )
		return; /* out of memory: counted, and the caller fails the world before the plan is used */
	plan->bodyBlock = block;
	w->solveList.count = 0;
	w->jointList.count = 0;
	for ( int c = 0; c < B2G_COLORS; ++c )
	{
		plan->colorStart[c] = w->solveList.count;
		plan->jointStart[c] = w->jointList.count;
		gIntArray* ca = &w->colors[c].contacts;
		gIntArray* ja = &w->colors[c].joints;
		if ( c < B2G_OVERFLOW && ca->count > 0 )
		{
			int* split = plan->rowSplit[c];
			for ( int k = 0; k < ca->count; ++k )
				split[row_owner( w, w->contacts + ca->data[k], block )] += 1;
			int offset[B2G_FUSED_CTAS];
			int start = w->solveList.count;
			for ( int o = 0, n = 0; o < B2G_FUSED_CTAS; ++o )
			{
				offset[o] = start + n;
				n += split[o];
			}
			for ( int k = 0; k < ca->count; ++k )
				gia_push( &w->solveList, 0 );
			for ( int k = 0; k < ca->count; ++k )
			{
				int id = ca->data[k];
				w->solveList.data[offset[row_owner( w, w->contacts + id, block )]++] = id;
			}
		}
		else
		{
			for ( int k = 0; k < ca->count; ++k )
				gia_push( &w->solveList, ca->data[k] );
		}
		for ( int k = 0; k < ja->count; ++k )
			gia_push( &w->jointList, ja->data[k] );
		if ( c < B2G_OVERFLOW && ca->count + ja->count > 0 )
			plan->active[plan->activeCount++] = c;
	}
	plan->colorStart[B2G_COLORS] = w->solveList.count;
	plan->jointStart[B2G_COLORS] = w->jointList.count;
	w->solvePlan = *plan;
	w->solveDirty = false;
	w->solveUploaded = false;
}

/* Host work before the narrowphase: pair update, device capacity, contact staging.
 * Returns the number of staged contact records, or -1 after a device failure. */
int gstep_begin( gWorld* w )
{
	double t0 = b2g_now_ms();
	int failures = b2g_alloc_failures();
	int pe = update_pairs( w );
	if ( pe )
	{
		w->status = pe;
		return -1;
	}
	double t1 = b2g_now_ms();
	w->profile.pairs = (float)( t1 - t0 );
	w->stepStart = t1;

	int idCount = w->contactIds.next;
	int e = b2gd_reserve( &w->dev, &w->io, w->bodyIds.next, w->shapeIds.next, idCount, w->jointIds.next, idCount, w->shapeIds.next );
	if ( e )
	{
		w->status = e;
		return -1;
	}
	int staged = compact_pending( w );
	if ( staged < 0 || gworld_out_of_memory( w, failures ) )
	{
		/* nothing reaches the device from a step whose host state is incomplete */
		if ( w->status == 0 )
			w->status = B2_STATUS_OUT_OF_HOST_MEMORY;
		return -1;
	}
	if ( staged > 0 )
		memcpy( w->io.newContacts, w->pending, sizeof( b2gContactInit ) * (size_t)staged );
	w->pendingCount = 0;
	w->stepIdCount = idCount;
	return staged;
}

/* Runs while the device narrowphase is in flight (reference src/world.c:420). */
void gstep_rebuild_trees( gWorld* w )
{
	double t0 = b2g_now_ms();
	gtree_rebuild( w->trees + b2_dynamicBody );
	gtree_rebuild( w->trees + b2_kinematicBody );
	w->hostMs[5] = (float)( b2g_now_ms() - t0 );
}

/* Host work between the narrowphase and the solver: events in contact-id order, step
 * constants, solve lists.  Returns 1 when the solver stage has to run. */
/* Step constants (reference src/world.c:715-757). */
static void step_constants( gWorld* w, float dt, int subSteps, b2gStepConst* sc )
{
	memset( sc, 0, sizeof( *sc ) );
	sc->subSteps = subSteps < 1 ? 1 : subSteps;
	sc->dt = dt;
	sc->inv_dt = 1.0f / dt;
	sc->h = dt / (float)sc->subSteps;
	sc->inv_h = (float)sc->subSteps * sc->inv_dt;
	w->inv_h = sc->inv_h;
	float contactHertz = gmin( w->contactHertz, 0.25f * sc->inv_h );
	float jointHertz = gmin( w->jointHertz, 0.125f * sc->inv_h );
	make_soft( contactHertz, w->contactDamping, sc->h, sc->contactSoft );
	make_soft( 2.0f * contactHertz, w->contactDamping, sc->h, sc->staticSoft );
	make_soft( jointHertz, w->jointDamping, sc->h, sc->jointSoft );
	sc->restitutionThreshold = w->restitutionThreshold;
	sc->pushout = w->pushout;
	sc->gravity = w->gravity;
	sc->enableWarmStarting = w->enableWarmStarting;
	sc->enableContinuous = w->enableContinuous;
	sc->enableSleep = w->enableSleep;
}

int gstep_after_collide( gWorld* w, float dt, int subSteps, b2gStepConst* sc, b2gSolvePlan* plan )
{
	int failures = b2g_alloc_failures();
	int eventCount = w->io.counters[0];
	w->lastEventCount = eventCount;
	/* events reach the host through mapped memory */
	w->dev.d2hBytes += 4 * (long long)( eventCount < w->dev.eventCap ? eventCount : w->dev.eventCap );
	double te = b2g_now_ms();
	process_events( w, eventCount < w->dev.eventCap ? eventCount : w->dev.eventCap );
	double t2 = b2g_now_ms();
	w->hostMs[3] = (float)( t2 - te );
	w->profile.collide = (float)( t2 - w->stepStart );
	w->stepStart = t2;

	if ( dt <= 0.0f )
		return 0;

	/* islands joined since the last step merge at the start of the solve; the previous
	 * step's split candidate splits before the bodies are finalised (reference
	 * src/solver.c:1114, :1395-1410, :1614-1620) */
	gislands_merge_awake( w );
	if ( w->awake.count > 0 )
	{
		if ( w->splitIslandId != B2G_NULL )
			gisland_split( w, w->splitIslandId );
		w->splitIslandId = B2G_NULL;
	}
	/* bodies woken by this step's events join the solve */
	int fe = gbody_flush_ops( w );
	if ( fe )
	{
		w->status = fe;
		return 0;
	}

	step_constants( w, dt, subSteps, sc );

	if ( w->awake.count == 0 )
	{
		if ( w->tape )
			gtape_record( w, NULL, sc, 0 );
		return 0;
	}

	double tl = b2g_now_ms();
	build_solve_lists( w, plan );
	if ( gworld_out_of_memory( w, failures ) )
		return 0;
	plan->awakeCount = w->awake.count;
	plan->bodyIdCount = w->bodyIds.next;
	if ( w->solveUploaded == false )
	{
		int e = b2gd_upload_solve_lists( &w->dev, w->solveList.data, w->solveList.count, w->jointList.data, w->jointList.count );
		if ( e )
		{
			w->status = e;
			return 0;
		}
		w->solveUploaded = true;
	}
	w->hostMs[4] = (float)( b2g_now_ms() - tl );
	if ( w->tape )
		gtape_record( w, plan, sc, 1 );
	return 1;
}

/* Host work after the solver stage: finalisation records in the reference's awake order
 * (proxy enlargement, move buffer). */
void gstep_finish( gWorld* w )
{
	double t3 = b2g_now_ms();
	w->profile.solve = (float)( t3 - w->stepStart );
	int recordCount = w->io.counters[1];
	w->lastRecordCount = recordCount;
	report_hits( w );
	double tr = b2g_now_ms();
	/* records reach the host through mapped memory: 48 bytes, 80 for fast shapes */
	for ( int i = 0; i < ( recordCount < w->dev.recordCap ? recordCount : w->dev.recordCap ); ++i )
		w->dev.d2hBytes += ( w->io.records[i].flags & B2G_R_FAST ) ? 80 : 48;
	process_records( w, recordCount < w->dev.recordCap ? recordCount : w->dev.recordCap );
	/* island sleep comes last: it moves bodies out of the awake set */
	gislands_sleep_step( w );
	w->profile.broadphase = (float)( b2g_now_ms() - t3 );
	w->profile.continuous = w->hostMs[7];
	w->hostMs[6] = (float)( b2g_now_ms() - tr ) - w->hostMs[7];
}

/* Whether the solver stage can be launched behind the narrowphase before its events are
 * known: the solve lists on the device are current (no event can have been processed
 * yet, so they are what the host would use after a step without events), the world
 * solves, nothing records the step, and the last step had no events either (a world
 * whose contacts change every step would waste the launches). */
static bool can_speculate( const gWorld* w, float dt )
{
	int block = ( w->bodyIds.next + B2G_FUSED_CTAS - 1 ) / B2G_FUSED_CTAS;
	block = block < 1 ? 1 : block;
	return dt > 0.0f && w->awake.count > 0 && w->tape == NULL && w->dev.fused && w->lastEventCount == 0 &&
		   w->solveDirty == false && w->solveUploaded && w->solvePlan.bodyBlock == block;
}

void gstep_run( gWorld* w, float dt, int subSteps )
{
	int staged = gstep_begin( w );
	if ( staged < 0 )
		return;
	int e = b2gd_collide( &w->dev, &w->io, staged, w->stepIdCount );
	b2gStepConst sc;
	b2gSolvePlan plan;
	int speculated = 0;
	if ( e == 0 && can_speculate( w, dt ) )
	{
		step_constants( w, dt, subSteps, &sc );
		plan = w->solvePlan;
		plan.awakeCount = w->awake.count;
		plan.bodyIdCount = w->bodyIds.next;
		speculated = b2gd_solve_speculative( &w->dev, &w->io, &plan, &sc );
	}
	/* The partial rebuild of the trees (reference src/world.c:420, finished before the
	 * proxies are enlarged, src/solver.c:1725) runs on the host while the device works:
	 * beside the whole launch sequence when the solver went out speculatively, else
	 * beside the solver stage, which takes longer than the narrowphase.  Nothing in
	 * between reads the trees. */
	bool rebuilt = false;
	if ( speculated > 0 )
	{
		gstep_rebuild_trees( w );
		rebuilt = true;
	}
	e |= b2gd_sync( &w->dev );
	if ( e || speculated < 0 )
	{
		w->status = e ? e : -1;
		return;
	}
	if ( speculated > 0 && w->io.counters[0] == 0 )
	{
		/* no events: the solver stage has run on the lists the host would have used */
		gstep_after_collide( w, dt, subSteps, &sc, &plan );
		gstep_finish( w );
		return;
	}
	if ( gstep_after_collide( w, dt, subSteps, &sc, &plan ) == 0 )
	{
		if ( rebuilt == false )
			gstep_rebuild_trees( w );
		return;
	}
	e = b2gd_solve( &w->dev, &w->io, &plan, &sc );
	if ( rebuilt == false )
		gstep_rebuild_trees( w );
	e |= b2gd_sync( &w->dev );
	if ( e )
	{
		w->status = e;
		return;
	}
	gstep_finish( w );
}

void b2World_Step( b2WorldId worldId, float timeStep, int subStepCount )
{
	if ( b2World_IsValid( worldId ) == false )
		return;
	gWorld* w = gworld_get( worldId );
	if ( w->locked )
		return;
	w->beginCount = 0;
	w->endCount = 0;
	w->hitCount = 0;
	w->sensorBeginCount = 0;
	w->sensorEndCount = 0;
	memset( &w->profile, 0, sizeof( w->profile ) );
	if ( timeStep == 0.0f || w->status != 0 )
		return;
	double t0 = b2g_now_ms();
	int failures = b2g_alloc_failures();
	w->locked = true;
	w->dev.h2dBytes = 0;
	w->dev.d2hBytes = 0;
	memset( w->hostMs, 0, sizeof( w->hostMs ) );
	b2gd_mark( &w->dev, 0 );
	gworld_flush( w );
	if ( w->status == 0 )
		gstep_run( w, timeStep, subStepCount );
	b2gd_mark( &w->dev, 6 );
	w->mirrorStale = true;
	w->shapeMirrorStale = true;
	w->jointMirrorStale = true;
	w->locked = false;
	w->profile.step = (float)( b2g_now_ms() - t0 );
	gworld_out_of_memory( w, failures );
	if ( w->status )
		gworld_fail( b2gd_last_error() );
}
