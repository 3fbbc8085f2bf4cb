/*
 * b2o_world.c -- world, body, shape, joint and contact bookkeeping, broadphase pairs,
 * narrowphase and constraint-graph colouring of the plain-C oracle
 * (TEST INFRASTRUCTURE).
 *
 * Restates the reference: world creation (src/world.c:80-208), the step driver
 * (:676-776), narrowphase and contact state processing (:290-674); body creation
 * (src/body.c:178-318); shape creation and proxies (src/shape.c:38-153, :692-702);
 * contact creation / destruction / update (src/contact.c:185-582); broadphase pair
 * finding (src/broad_phase.c:91-436); colouring (src/constraint_graph.c:64-267) and
 * joint creation (src/joint.c:140-655, src/joint.c:458-511).
 */
#include "b2o.h"

#include <string.h>

#define O_MAX_WORLDS 65535

static oWorld** s_worlds;
static int s_worldCap;

oWorld* o_world_index( int index ) { return s_worlds[index]; }

oWorld* o_world( b2WorldId id ) { return s_worlds[id.index1 - 1]; }

static b2AssertFcn* s_assert;
void b2SetAssertFcn( b2AssertFcn* fcn ) { s_assert = fcn; }
void b2SetAllocator( b2AllocFcn* a, b2FreeFcn* f )
{
	(void)a;
	(void)f;
}
int b2GetByteCount( void ) { return 0; }
b2Version b2GetVersion( void )
{
	b2Version v = { 3, 0, 0 };
	return v;
}

static void o_fail( const char* what )
{
	if ( s_assert )
		s_assert( what, __FILE__, 0 );
}

/* ------------------------------------------------------------ defaults (src/types.c) */
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

/* ------------------------------------------------------------ math API of math_functions.h */
bool b2IsValid( float a ) { return !isnan( a ) && !isinf( a ); }
bool b2Vec2_IsValid( b2Vec2 v ) { return b2IsValid( v.x ) && b2IsValid( v.y ); }
bool b2Rot_IsValid( b2Rot q ) { return b2IsValid( q.s ) && b2IsValid( q.c ) && b2IsNormalized( q ); }
bool b2AABB_IsValid( b2AABB a )
{
	b2Vec2 d = b2Sub( a.upperBound, a.lowerBound );
	return d.x >= 0.0f && d.y >= 0.0f && b2Vec2_IsValid( a.lowerBound ) && b2Vec2_IsValid( a.upperBound );
}
b2Vec2 b2Normalize( b2Vec2 v ) { return vfo( onormalize( ovf( v ) ) ); }
b2Vec2 b2NormalizeChecked( b2Vec2 v ) { return vfo( onormalize( ovf( v ) ) ); }
b2Vec2 b2GetLengthAndNormalize( float* length, b2Vec2 v )
{
	b2r l;
	oVec n = olen_normalize( &l, ovf( v ) );
	*length = (float)l;
	return vfo( n );
}
void b2SetLengthUnitsPerMeter( float u ) { (void)u; }
float b2GetLengthUnitsPerMeter( void ) { return 1.0f; }

/* ------------------------------------------------------------ record storage */
#define GROW( ptr, cap, need, T )                                                                                                \
	do                                                                                                                           \
	{                                                                                                                            \
		if ( ( need ) > ( cap ) )                                                                                                \
		{                                                                                                                        \
			int nc = ( cap ) < 16 ? 16 : ( cap );                                                                                \
			while ( nc < ( need ) )                                                                                              \
				nc *= 2;                                                                                                         \
			ptr = (T*)realloc( ptr, sizeof( T ) * (size_t)nc );                                                                  \
			memset( ptr + ( cap ), 0, sizeof( T ) * (size_t)( nc - ( cap ) ) );                                                  \
			for ( int _i = ( cap ); _i < nc; ++_i )                                                                              \
				ptr[_i].id = O_NULL;                                                                                             \
			cap = nc;                                                                                                            \
		}                                                                                                                        \
	}                                                                                                                            \
	while ( 0 )

static void add_event_begin( oWorld* w, int a, int b )
{
	if ( w->beginCount == w->beginCap )
	{
		w->beginCap = w->beginCap ? 2 * w->beginCap : 16;
		w->beginEvents = realloc( w->beginEvents, sizeof( b2ContactBeginTouchEvent ) * (size_t)w->beginCap );
	}
	b2ContactBeginTouchEvent* e = w->beginEvents + w->beginCount++;
	e->shapeIdA = ( b2ShapeId ){ a + 1, (uint16_t)w->slot, w->shapes[a].revision };
	e->shapeIdB = ( b2ShapeId ){ b + 1, (uint16_t)w->slot, w->shapes[b].revision };
}

static void add_event_end( oWorld* w, int a, int b )
{
	if ( w->endCount == w->endCap )
	{
		w->endCap = w->endCap ? 2 * w->endCap : 16;
		w->endEvents = realloc( w->endEvents, sizeof( b2ContactEndTouchEvent ) * (size_t)w->endCap );
	}
	b2ContactEndTouchEvent* e = w->endEvents + w->endCount++;
	e->shapeIdA = ( b2ShapeId ){ a + 1, (uint16_t)w->slot, w->shapes[a].revision };
	e->shapeIdB = ( b2ShapeId ){ b + 1, (uint16_t)w->slot, w->shapes[b].revision };
}

static b2ShapeId shape_id( oWorld* w, int s ) { return ( b2ShapeId ){ s + 1, (uint16_t)w->slot, w->shapes[s].revision }; }

static void add_sensor_event( oWorld* w, bool begin, int sensor, int visitor )
{
	if ( begin )
	{
		if ( w->sensorBeginCount == w->sensorBeginCap )
		{
			w->sensorBeginCap = w->sensorBeginCap ? 2 * w->sensorBeginCap : 16;
			w->sensorBeginEvents = realloc( w->sensorBeginEvents, sizeof( b2SensorBeginTouchEvent ) * (size_t)w->sensorBeginCap );
		}
		b2SensorBeginTouchEvent* e = w->sensorBeginEvents + w->sensorBeginCount++;
		e->sensorShapeId = shape_id( w, sensor );
		e->visitorShapeId = shape_id( w, visitor );
	}
	else
	{
		if ( w->sensorEndCount == w->sensorEndCap )
		{
			w->sensorEndCap = w->sensorEndCap ? 2 * w->sensorEndCap : 16;
			w->sensorEndEvents = realloc( w->sensorEndEvents, sizeof( b2SensorEndTouchEvent ) * (size_t)w->sensorEndCap );
		}
		b2SensorEndTouchEvent* e = w->sensorEndEvents + w->sensorEndCount++;
		e->sensorShapeId = shape_id( w, sensor );
		e->visitorShapeId = shape_id( w, visitor );
	}
}

/* Hit events of the step (reference src/solver.c:1670-1723): contacts of the colours in
 * colour and array order whose touching shapes enable hit events; the point of the
 * fastest approach above the world's threshold among points that carry an impulse. */
void o_report_hits( oWorld* w )
{
	for ( int i = 0; i < O_COLORS; ++i )
	{
		oIntArray* a = &w->colors[i].contacts;
		for ( int j = 0; j < a->count; ++j )
		{
			oContact* c = w->contacts + a->data[j];
			if ( ( c->simFlags & OS_HIT ) == 0 )
				continue;
			b2ContactHitEvent e;
			memset( &e, 0, sizeof( e ) );
			b2r approach = R( w->hitThreshold );
			bool hit = false;
			for ( int k = 0; k < c->manifold.count; ++k )
			{
				oMPoint* mp = c->manifold.pts + k;
				b2r s = -mp->normalVelocity;
				if ( s > approach && mp->normalImpulse > R( 0 ) )
				{
					approach = s;
					e.point = ( b2Vec2 ){ (float)mp->point.x, (float)mp->point.y };
					hit = true;
				}
			}
			if ( hit == false )
				continue;
			e.approachSpeed = (float)approach;
			e.normal = ( b2Vec2 ){ (float)c->manifold.normal.x, (float)c->manifold.normal.y };
			e.shapeIdA = shape_id( w, c->shapeIdA );
			e.shapeIdB = shape_id( w, c->shapeIdB );
			if ( w->hitCount == w->hitCap )
			{
				w->hitCap = w->hitCap ? 2 * w->hitCap : 16;
				w->hitEvents = realloc( w->hitEvents, sizeof( b2ContactHitEvent ) * (size_t)w->hitCap );
			}
			w->hitEvents[w->hitCount++] = e;
		}
	}
}

/* ------------------------------------------------------------ world */
b2WorldId b2CreateWorld( const b2WorldDef* def )
{
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
		if ( s_worldCap >= O_MAX_WORLDS )
			return b2_nullWorldId;
		int nc = s_worldCap ? 2 * s_worldCap : 16;
		if ( nc > O_MAX_WORLDS )
			nc = O_MAX_WORLDS;
		s_worlds = (oWorld**)realloc( s_worlds, sizeof( oWorld* ) * (size_t)nc );
		memset( s_worlds + s_worldCap, 0, sizeof( oWorld* ) * (size_t)( nc - s_worldCap ) );
		slot = s_worldCap;
		s_worldCap = nc;
	}
	if ( s_worlds[slot] == NULL )
		s_worlds[slot] = (oWorld*)calloc( 1, sizeof( oWorld ) );
	oWorld* w = s_worlds[slot];
	uint16_t revision = w->revision;
	memset( w, 0, sizeof( *w ) );
	w->revision = revision;
	w->inUse = true;
	w->slot = slot;
	for ( int i = 0; i < 3; ++i )
		otree_init( w->trees + i );
	w->gravity = ovf( def->gravity );
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
	o_islands_init( w );
	b2WorldId id = { (uint16_t)( slot + 1 ), w->revision };
	return id;
}

void b2DestroyWorld( b2WorldId worldId )
{
	oWorld* w = o_world( worldId );
	for ( int i = 0; i < 3; ++i )
		otree_free( w->trees + i );
	for ( int i = 0; i < O_COLORS; ++i )
	{
		obits_free( &w->colors[i].bodySet );
		oia_free( &w->colors[i].contacts );
		oia_free( &w->colors[i].joints );
	}
	oia_free( &w->bodyIds.freeIds );
	oia_free( &w->shapeIds.freeIds );
	oia_free( &w->contactIds.freeIds );
	oia_free( &w->jointIds.freeIds );
	oia_free( &w->awake );
	oia_free( &w->staticBodies );
	oia_free( &w->nonTouching );
	o_islands_free( w );
	oia_free( &w->moveArray );
	oset_free( &w->moveSet );
	oset_free( &w->pairSet );
	free( w->bodies );
	free( w->shapes );
	free( w->contacts );
	free( w->joints );
	for ( int i = 0; i < w->chainCap; ++i )
		if ( w->chains[i].id != O_NULL )
			free( w->chains[i].shapeIndices );
	free( w->chains );
	oia_free( &w->chainIds.freeIds );
	free( w->beginEvents );
	free( w->endEvents );
	free( w->hitEvents );
	free( w->sensorBeginEvents );
	free( w->sensorEndEvents );
	uint16_t revision = w->revision;
	memset( w, 0, sizeof( *w ) );
	w->revision = (uint16_t)( revision + 1 );
}

bool b2World_IsValid( b2WorldId id )
{
	if ( id.index1 < 1 || id.index1 > s_worldCap )
		return false;
	oWorld* w = s_worlds[id.index1 - 1];
	return w && w->inUse && w->revision == id.revision;
}

/* reference src/world.c:1568-1594: turning sleep off wakes every sleeping set */
void b2World_EnableSleeping( b2WorldId id, bool flag )
{
	oWorld* w = o_world( id );
	if ( w->locked || flag == w->enableSleep )
		return;
	w->enableSleep = flag;
	if ( flag == false )
	{
		for ( int i = O_SET_FIRST_SLEEPING; i < w->setCap; ++i )
			if ( w->sets[i].bodies.count > 0 )
				o_wake_solver_set( w, i );
	}
}
void b2World_EnableContinuous( b2WorldId id, bool flag ) { o_world( id )->enableContinuous = flag; }
void b2World_EnableWarmStarting( b2WorldId id, bool flag ) { o_world( id )->enableWarmStarting = flag; }
void b2World_SetRestitutionThreshold( b2WorldId id, float v ) { o_world( id )->restitutionThreshold = v; }
void b2World_SetHitEventThreshold( b2WorldId id, float v ) { o_world( id )->hitThreshold = v; }
void b2World_SetGravity( b2WorldId id, b2Vec2 g ) { o_world( id )->gravity = ovf( g ); }
b2Vec2 b2World_GetGravity( b2WorldId id ) { return vfo( o_world( id )->gravity ); }
void b2World_SetContactTuning( b2WorldId id, float hertz, float damping, float push )
{
	oWorld* w = o_world( id );
	w->contactHertz = omin( hertz, R( 1e30f ) );
	w->contactDamping = damping;
	w->pushout = push;
}
b2Profile b2World_GetProfile( b2WorldId id ) { return o_world( id )->profile; }

b2ContactEvents b2World_GetContactEvents( b2WorldId id )
{
	oWorld* w = o_world( id );
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
	oWorld* w = o_world( id );
	b2SensorEvents e = { w->sensorBeginEvents, w->sensorEndEvents, w->sensorBeginCount, w->sensorEndCount };
	return e;
}

b2Counters b2World_GetCounters( b2WorldId id )
{
	oWorld* w = o_world( id );
	b2Counters c;
	memset( &c, 0, sizeof( c ) );
	c.staticBodyCount = w->staticBodies.count;
	c.bodyCount = oid_count( &w->bodyIds );
	c.shapeCount = oid_count( &w->shapeIds );
	c.contactCount = oid_count( &w->contactIds );
	c.jointCount = oid_count( &w->jointIds );
	c.islandCount = oid_count( &w->islandIds );
	c.staticTreeHeight = otree_height( w->trees + b2_staticBody );
	int hd = otree_height( w->trees + b2_dynamicBody );
	int hk = otree_height( w->trees + b2_kinematicBody );
	c.treeHeight = hd > hk ? hd : hk;
	for ( int i = 0; i < O_COLORS; ++i )
		c.colorCounts[i] = w->colors[i].contacts.count + w->colors[i].joints.count;
	return c;
}

/* ------------------------------------------------------------ bodies */
static oBody* get_body( b2BodyId id ) { return s_worlds[id.world0]->bodies + ( id.index1 - 1 ); }
static oWorld* body_world( b2BodyId id ) { return s_worlds[id.world0]; }

b2BodyId b2CreateBody( b2WorldId worldId, const b2BodyDef* def )
{
	oWorld* w = o_world( worldId );
	if ( w->locked )
		return b2_nullBodyId;
	int id = oid_alloc( &w->bodyIds );
	GROW( w->bodies, w->bodyCap, id + 1, oBody );
	oBody* b = w->bodies + id;
	uint16_t rev = b->revision;
	memset( b, 0, sizeof( *b ) );
	b->id = id;
	b->revision = (uint16_t)( rev + 1 );
	b->type = def->type;
	b->userData = def->userData;
	b->headShape = O_NULL;
	b->headContactKey = O_NULL;
	b->headJointKey = O_NULL;
	b->headChainId = O_NULL;
	b->fixedRotation = def->fixedRotation;
	b->isBullet = def->isBullet;
	b->enableSleep = def->enableSleep;
	b->automaticMass = def->automaticMass;
	b->sleepThreshold = def->sleepThreshold;
	b->xf.p = ovf( def->position );
	b->xf.q = orot( def->rotation.c, def->rotation.s );
	b->center = b->xf.p;
	b->rot0 = b->xf.q;
	b->center0 = b->center;
	b->minExtent = O_HUGE;
	b->linearDamping = def->linearDamping;
	b->angularDamping = def->angularDamping;
	b->gravityScale = def->gravityScale;
	b->dq = orot( 1, 0 );
	b->islandId = O_NULL;
	b->islandPrev = O_NULL;
	b->islandNext = O_NULL;
	/* solver set (reference src/body.c:196-228): static, awake, or a new sleeping set of
	 * its own; only an awake body keeps the definition's velocity */
	bool isAwake = def->isAwake || def->enableSleep == false;
	int setId;
	if ( def->type == b2_staticBody )
		setId = O_SET_STATIC;
	else if ( isAwake )
		setId = O_SET_AWAKE;
	else
		setId = o_create_sleeping_set( w );
	b->setIndex = setId;
	b->awakeIndex = O_NULL;
	b->setLocal = O_NULL;
	if ( setId == O_SET_AWAKE )
	{
		b->awakeIndex = w->awake.count;
		b->v = ovf( def->linearVelocity );
		b->w = def->angularVelocity;
	}
	else
		b->setLocal = o_set_bodies( w, setId )->count;
	oia_push( o_set_bodies( w, setId ), id );
	if ( setId >= O_SET_AWAKE )
		o_create_island_for_body( w, setId, b );
	b2BodyId bid = { id + 1, (uint16_t)w->slot, b->revision };
	return bid;
}

bool b2Body_IsValid( b2BodyId id )
{
	if ( id.world0 >= s_worldCap || s_worlds[id.world0] == NULL || !s_worlds[id.world0]->inUse )
		return false;
	oWorld* w = s_worlds[id.world0];
	if ( id.index1 < 1 || id.index1 > w->bodyCap )
		return false;
	oBody* b = w->bodies + id.index1 - 1;
	return b->id == id.index1 - 1 && b->revision == id.revision;
}

b2BodyType b2Body_GetType( b2BodyId id ) { return get_body( id )->type; }
void b2Body_SetUserData( b2BodyId id, void* u ) { get_body( id )->userData = u; }
void* b2Body_GetUserData( b2BodyId id ) { return get_body( id )->userData; }
b2Vec2 b2Body_GetPosition( b2BodyId id ) { return vfo( get_body( id )->xf.p ); }
b2Rot b2Body_GetRotation( b2BodyId id )
{
	oBody* b = get_body( id );
	b2Rot q = { (float)b->xf.q.c, (float)b->xf.q.s };
	return q;
}
b2Transform b2Body_GetTransform( b2BodyId id )
{
	b2Transform t;
	t.p = b2Body_GetPosition( id );
	t.q = b2Body_GetRotation( id );
	return t;
}
b2Vec2 b2Body_GetLocalPoint( b2BodyId id, b2Vec2 p ) { return b2InvTransformPoint( b2Body_GetTransform( id ), p ); }
b2Vec2 b2Body_GetWorldPoint( b2BodyId id, b2Vec2 p ) { return b2TransformPoint( b2Body_GetTransform( id ), p ); }
/* Velocities live in the awake set only (reference src/body.c:729-787): a body that is
 * not awake reports zero, and a non-zero velocity wakes it first. */
b2Vec2 b2Body_GetLinearVelocity( b2BodyId id )
{
	oBody* b = get_body( id );
	return b->setIndex == O_SET_AWAKE ? vfo( b->v ) : b2Vec2_zero;
}
float b2Body_GetAngularVelocity( b2BodyId id )
{
	oBody* b = get_body( id );
	return b->setIndex == O_SET_AWAKE ? (float)b->w : 0.0f;
}
void b2Body_SetLinearVelocity( b2BodyId id, b2Vec2 v )
{
	oWorld* w = body_world( id );
	oBody* b = get_body( id );
	if ( v.x * v.x + v.y * v.y > 0.0f )
		o_wake_body( w, b );
	if ( b->setIndex == O_SET_AWAKE )
		b->v = ovf( v );
}
void b2Body_SetAngularVelocity( b2BodyId id, float a )
{
	oWorld* w = body_world( id );
	oBody* b = get_body( id );
	if ( a != 0.0f )
		o_wake_body( w, b );
	if ( b->setIndex == O_SET_AWAKE )
		b->w = a;
}

/* reference src/body.c:1358-1433 */
bool b2Body_IsAwake( b2BodyId id ) { return get_body( id )->setIndex == O_SET_AWAKE; }
void b2Body_SetAwake( b2BodyId id, bool awake )
{
	oWorld* w = body_world( id );
	if ( w->locked )
		return;
	oBody* b = get_body( id );
	if ( awake && b->setIndex >= O_SET_FIRST_SLEEPING )
		o_wake_body( w, b );
	else if ( awake == false && b->setIndex == O_SET_AWAKE )
	{
		if ( w->islands[b->islandId].constraintRemoveCount > 0 )
			o_split_island( w, b->islandId );
		o_try_sleep_island( w, b->islandId );
	}
}
bool b2Body_IsSleepEnabled( b2BodyId id ) { return get_body( id )->enableSleep; }
void b2Body_SetSleepThreshold( b2BodyId id, float v ) { get_body( id )->sleepThreshold = v; }
float b2Body_GetSleepThreshold( b2BodyId id ) { return (float)get_body( id )->sleepThreshold; }
void b2Body_EnableSleep( b2BodyId id, bool enableSleep )
{
	oWorld* w = body_world( id );
	if ( w->locked )
		return;
	oBody* b = get_body( id );
	b->enableSleep = enableSleep;
	if ( enableSleep == false )
		o_wake_body( w, b );
}
float b2Body_GetMass( b2BodyId id ) { return (float)get_body( id )->mass; }
float b2Body_GetInertiaTensor( b2BodyId id ) { return (float)get_body( id )->inertia; }
b2Vec2 b2Body_GetLocalCenterOfMass( b2BodyId id ) { return vfo( get_body( id )->localCenter ); }
b2Vec2 b2Body_GetWorldCenterOfMass( b2BodyId id ) { return vfo( get_body( id )->center ); }
float b2Body_GetLinearDamping( b2BodyId id ) { return (float)get_body( id )->linearDamping; }
float b2Body_GetAngularDamping( b2BodyId id ) { return (float)get_body( id )->angularDamping; }
float b2Body_GetGravityScale( b2BodyId id ) { return (float)get_body( id )->gravityScale; }
int b2Body_GetShapeCount( b2BodyId id ) { return get_body( id )->shapeCount; }
int b2Body_GetShapes( b2BodyId id, b2ShapeId* out, int capacity )
{
	oWorld* w = body_world( id );
	oBody* b = get_body( id );
	int n = 0;
	for ( int s = b->headShape; s != O_NULL && n < capacity; s = w->shapes[s].next )
		out[n++] = ( b2ShapeId ){ s + 1, id.world0, w->shapes[s].revision };
	return n;
}
int b2Body_GetJointCount( b2BodyId id ) { return get_body( id )->jointCount; }
int b2Body_GetContactCapacity( b2BodyId id ) { return get_body( id )->contactCount; }

int b2Body_GetContactData( b2BodyId id, b2ContactData* out, int capacity )
{
	oWorld* w = body_world( id );
	oBody* b = get_body( id );
	int n = 0;
	for ( int key = b->headContactKey; key != O_NULL && n < capacity; )
	{
		oContact* c = w->contacts + ( key >> 1 );
		if ( c->flags & OC_TOUCHING )
		{
			b2ContactData* d = out + n++;
			memset( d, 0, sizeof( *d ) );
			d->shapeIdA = ( b2ShapeId ){ c->shapeIdA + 1, id.world0, w->shapes[c->shapeIdA].revision };
			d->shapeIdB = ( b2ShapeId ){ c->shapeIdB + 1, id.world0, w->shapes[c->shapeIdB].revision };
			d->manifold.normal = vfo( c->manifold.normal );
			d->manifold.pointCount = c->manifold.count;
			for ( int i = 0; i < 2; ++i )
			{
				const oMPoint* p = c->manifold.pts + i;
				b2ManifoldPoint* q = d->manifold.points + i;
				q->point = vfo( p->point );
				q->anchorA = vfo( p->anchorA );
				q->anchorB = vfo( p->anchorB );
				q->separation = (float)p->separation;
				q->normalImpulse = (float)p->normalImpulse;
				q->tangentImpulse = (float)p->tangentImpulse;
				q->maxNormalImpulse = (float)p->maxNormalImpulse;
				q->normalVelocity = (float)p->normalVelocity;
				q->id = p->id;
				q->persisted = p->persisted;
			}
		}
		key = c->edges[key & 1].nextKey;
	}
	return n;
}

/* ------------------------------------------------------------ shapes */
static void buffer_move( oWorld* w, int proxyKey )
{
	if ( oset_add( &w->moveSet, (uint64_t)( proxyKey + 1 ) ) == false )
		oia_push( &w->moveArray, proxyKey );
}

void o_buffer_move( oWorld* w, int proxyKey ) { buffer_move( w, proxyKey ); }

static b2ShapeId create_shape_internal( b2BodyId bodyId, const b2ShapeDef* def, b2ShapeType type, const void* geometry,
										bool updateMass )
{
	oWorld* w = body_world( bodyId );
	if ( w->locked )
		return b2_nullShapeId;
	oBody* body = get_body( bodyId );
	int id = oid_alloc( &w->shapeIds );
	GROW( w->shapes, w->shapeCap, id + 1, oShape );
	body = get_body( bodyId );
	oShape* s = w->shapes + id;
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
	s->enablePreSolveEvents = def->enablePreSolveEvents;
	s->proxyKey = O_NULL;
	switch ( type )
	{
		case b2_polygonShape:
		{
			const b2Polygon* p = (const b2Polygon*)geometry;
			s->polygon.count = p->count;
			s->polygon.radius = p->radius;
			s->polygon.centroid = ovf( p->centroid );
			for ( int i = 0; i < p->count; ++i )
			{
				s->polygon.v[i] = ovf( p->vertices[i] );
				s->polygon.n[i] = ovf( p->normals[i] );
			}
			s->localCentroid = s->polygon.centroid;
			break;
		}
		case b2_circleShape:
		{
			const b2Circle* c = (const b2Circle*)geometry;
			s->circle.center = ovf( c->center );
			s->circle.radius = c->radius;
			s->localCentroid = s->circle.center;
			break;
		}
		case b2_capsuleShape:
		{
			const b2Capsule* c = (const b2Capsule*)geometry;
			s->capsule.c1 = ovf( c->center1 );
			s->capsule.c2 = ovf( c->center2 );
			s->capsule.radius = c->radius;
			s->localCentroid = olerp( s->capsule.c1, s->capsule.c2, R( 0.5f ) );
			break;
		}
		case b2_segmentShape:
		{
			const b2Segment* g = (const b2Segment*)geometry;
			s->segment.p1 = ovf( g->point1 );
			s->segment.p2 = ovf( g->point2 );
			s->localCentroid = olerp( s->segment.p1, s->segment.p2, R( 0.5f ) );
			break;
		}
		case b2_smoothSegmentShape:
		{
			const b2SmoothSegment* g = (const b2SmoothSegment*)geometry;
			s->smooth.ghost1 = ovf( g->ghost1 );
			s->smooth.p1 = ovf( g->segment.point1 );
			s->smooth.p2 = ovf( g->segment.point2 );
			s->smooth.ghost2 = ovf( g->ghost2 );
			s->smooth.chainId = g->chainId;
			s->localCentroid = olerp( s->smooth.p1, s->smooth.p2, R( 0.5f ) );
			break;
		}
		default:
			break;
	}

	/* proxy (reference src/shape.c:38-59, :692-702, src/broad_phase.c:91-102) */
	{
		b2BodyType proxyType = body->type;
		oBox aabb = o_shape_aabb( s, body->xf );
		aabb.lo.x -= O_SPECULATIVE;
		aabb.lo.y -= O_SPECULATIVE;
		aabb.hi.x += O_SPECULATIVE;
		aabb.hi.y += O_SPECULATIVE;
		s->aabb = aabb;
		b2r margin = proxyType == b2_staticBody ? O_SPECULATIVE : O_AABB_MARGIN;
		s->fatAABB.lo.x = aabb.lo.x - margin;
		s->fatAABB.lo.y = aabb.lo.y - margin;
		s->fatAABB.hi.x = aabb.hi.x + margin;
		s->fatAABB.hi.y = aabb.hi.y + margin;
		int proxyId = otree_create_proxy( w->trees + proxyType, s->fatAABB, s->filter.categoryBits, id );
		s->proxyKey = ( proxyId << 2 ) | proxyType;
		if ( proxyType != b2_staticBody || def->forceContactCreation )
			buffer_move( w, s->proxyKey );
	}

	if ( body->headShape != O_NULL )
		w->shapes[body->headShape].prev = id;
	s->prev = O_NULL;
	s->next = body->headShape;
	body->headShape = id;
	body->shapeCount += 1;

	if ( updateMass && body->automaticMass )
		o_update_body_mass( w, body );

	b2ShapeId sid = { id + 1, bodyId.world0, s->revision };
	return sid;
}

static b2ShapeId create_shape( b2BodyId bodyId, const b2ShapeDef* def, b2ShapeType type, const void* geometry )
{
	return create_shape_internal( bodyId, def, type, geometry, true );
}

b2ShapeId b2CreatePolygonShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Polygon* polygon )
{
	return create_shape( bodyId, def, b2_polygonShape, polygon );
}

b2ShapeId b2CreateCircleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Circle* circle )
{
	return create_shape( bodyId, def, b2_circleShape, circle );
}

b2ShapeId b2CreateCapsuleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Capsule* capsule )
{
	float lengthSqr = b2DistanceSquared( capsule->center1, capsule->center2 );
	if ( lengthSqr <= 0.005f * 0.005f )
	{
		b2Circle circle = { b2Lerp( capsule->center1, capsule->center2, 0.5f ), capsule->radius };
		return create_shape( bodyId, def, b2_circleShape, &circle );
	}
	return create_shape( bodyId, def, b2_capsuleShape, capsule );
}

b2ShapeId b2CreateSegmentShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Segment* segment )
{
	float lengthSqr = b2DistanceSquared( segment->point1, segment->point2 );
	if ( lengthSqr <= 0.005f * 0.005f )
	{
		o_fail( "segment too short" );
		return b2_nullShapeId;
	}
	return create_shape( bodyId, def, b2_segmentShape, segment );
}

static oShape* get_shape( b2ShapeId id ) { return s_worlds[id.world0]->shapes + ( id.index1 - 1 ); }

bool b2Shape_IsValid( b2ShapeId id )
{
	if ( id.world0 >= s_worldCap || s_worlds[id.world0] == NULL || !s_worlds[id.world0]->inUse )
		return false;
	oWorld* w = s_worlds[id.world0];
	if ( id.index1 < 1 || id.index1 > w->shapeCap )
		return false;
	oShape* s = w->shapes + id.index1 - 1;
	return s->id == id.index1 - 1 && s->revision == id.revision;
}
b2ShapeType b2Shape_GetType( b2ShapeId id ) { return get_shape( id )->type; }
b2BodyId b2Shape_GetBody( b2ShapeId id )
{
	oWorld* w = s_worlds[id.world0];
	oShape* s = get_shape( id );
	b2BodyId b = { s->bodyId + 1, id.world0, w->bodies[s->bodyId].revision };
	return b;
}
float b2Shape_GetDensity( b2ShapeId id ) { return (float)get_shape( id )->density; }
void b2Shape_SetFriction( b2ShapeId id, float f ) { get_shape( id )->friction = f; }
float b2Shape_GetFriction( b2ShapeId id ) { return (float)get_shape( id )->friction; }
void b2Shape_SetRestitution( b2ShapeId id, float r ) { get_shape( id )->restitution = r; }
float b2Shape_GetRestitution( b2ShapeId id ) { return (float)get_shape( id )->restitution; }
b2Filter b2Shape_GetFilter( b2ShapeId id ) { return get_shape( id )->filter; }
b2Polygon b2Shape_GetPolygon( b2ShapeId id )
{
	oShape* s = get_shape( id );
	b2Polygon p;
	memset( &p, 0, sizeof( p ) );
	p.count = s->polygon.count;
	p.radius = (float)s->polygon.radius;
	p.centroid = vfo( s->polygon.centroid );
	for ( int i = 0; i < p.count; ++i )
	{
		p.vertices[i] = vfo( s->polygon.v[i] );
		p.normals[i] = vfo( s->polygon.n[i] );
	}
	return p;
}
b2Circle b2Shape_GetCircle( b2ShapeId id )
{
	oShape* s = get_shape( id );
	b2Circle c = { vfo( s->circle.center ), (float)s->circle.radius };
	return c;
}
b2AABB b2Shape_GetAABB( b2ShapeId id )
{
	oShape* s = get_shape( id );
	b2AABB a = { vfo( s->aabb.lo ), vfo( s->aabb.hi ) };
	return a;
}

/* ------------------------------------------------------------ contacts */
#define PAIR_KEY( K1, K2 ) ( ( K1 ) < ( K2 ) ? (uint64_t)( K1 ) << 32 | (uint64_t)( K2 ) : (uint64_t)( K2 ) << 32 | (uint64_t)( K1 ) )

/* Which shape-type pairs have a manifold function, and which order is primary
 * (reference src/contact.c:150-183). */
static int registered( b2ShapeType a, b2ShapeType b, bool* primary )
{
	static const int table[5][5] = {
		/*            circle capsule segment polygon smooth */
		/* circle  */ { 1, -1, -1, -1, -1 },
		/* capsule */ { 1, 1, -1, -1, -1 },
		/* segment */ { 1, 1, 0, 1, 0 },
		/* polygon */ { 1, 1, -1, 1, -1 },
		/* smooth  */ { 1, 1, 0, 1, 0 },
	};
	int v = table[a][b];
	if ( v == 0 )
		return 0;
	*primary = v > 0;
	return 1;
}

void o_create_contact( oWorld* w, oShape* shapeA, oShape* shapeB )
{
	bool primary;
	if ( registered( shapeA->type, shapeB->type, &primary ) == 0 )
		return;
	if ( primary == false )
	{
		o_create_contact( w, shapeB, shapeA );
		return;
	}
	oBody* bodyA = w->bodies + shapeA->bodyId;
	oBody* bodyB = w->bodies + shapeB->bodyId;
	int id = oid_alloc( &w->contactIds );
	GROW( w->contacts, w->contactCap, id + 1, oContact );
	oContact* c = w->contacts + id;
	memset( c, 0, sizeof( *c ) );
	c->id = id;
	/* non-touching contacts of two bodies that are not awake live in the disabled set
	 * (reference src/contact.c:210-222) */
	int setIndex = bodyA->setIndex == O_SET_AWAKE || bodyB->setIndex == O_SET_AWAKE ? O_SET_AWAKE : O_SET_DISABLED;
	c->setIndex = setIndex;
	c->colorIndex = O_NULL;
	c->localIndex = o_set_contacts( w, setIndex )->count;
	c->islandId = O_NULL;
	c->islandPrev = O_NULL;
	c->islandNext = O_NULL;
	c->shapeIdA = shapeA->id;
	c->shapeIdB = shapeB->id;
	if ( shapeA->isSensor || shapeB->isSensor )
		c->flags |= OC_SENSOR;
	if ( shapeA->enableSensorEvents || shapeB->enableSensorEvents )
		c->flags |= OC_ENABLE_SENSOR_EVENTS;
	if ( shapeA->enableContactEvents || shapeB->enableContactEvents )
		c->flags |= OC_ENABLE_CONTACT_EVENTS;

	c->edges[0].bodyId = shapeA->bodyId;
	c->edges[0].prevKey = O_NULL;
	c->edges[0].nextKey = bodyA->headContactKey;
	int keyA = ( id << 1 ) | 0;
	if ( bodyA->headContactKey != O_NULL )
		w->contacts[bodyA->headContactKey >> 1].edges[bodyA->headContactKey & 1].prevKey = keyA;
	bodyA->headContactKey = keyA;
	bodyA->contactCount += 1;

	c->edges[1].bodyId = shapeB->bodyId;
	c->edges[1].prevKey = O_NULL;
	c->edges[1].nextKey = bodyB->headContactKey;
	int keyB = ( id << 1 ) | 1;
	if ( bodyB->headContactKey != O_NULL )
		w->contacts[bodyB->headContactKey >> 1].edges[bodyB->headContactKey & 1].prevKey = keyB;
	bodyB->headContactKey = keyB;
	bodyB->contactCount += 1;

	oset_add( &w->pairSet, PAIR_KEY( (uint64_t)shapeA->id, (uint64_t)shapeB->id ) );
	oia_push( o_set_contacts( w, setIndex ), id );

	c->simIndexA = O_NULL;
	c->simIndexB = O_NULL;
	c->friction = RSQRT( shapeA->friction * shapeB->friction );
	c->restitution = shapeA->restitution > shapeB->restitution ? shapeA->restitution : shapeB->restitution;
}

static void remove_non_touching( oWorld* w, int localIndex )
{
	int moved = oia_remove_swap( &w->nonTouching, localIndex );
	if ( moved != O_NULL )
		w->contacts[w->nonTouching.data[localIndex]].localIndex = localIndex;
}

static void unlink_edge( oWorld* w, oContact* c, int e )
{
	oEdge* edge = c->edges + e;
	oBody* body = w->bodies + edge->bodyId;
	if ( edge->prevKey != O_NULL )
		w->contacts[edge->prevKey >> 1].edges[edge->prevKey & 1].nextKey = edge->nextKey;
	if ( edge->nextKey != O_NULL )
		w->contacts[edge->nextKey >> 1].edges[edge->nextKey & 1].prevKey = edge->prevKey;
	int key = ( c->id << 1 ) | e;
	if ( body->headContactKey == key )
		body->headContactKey = edge->nextKey;
	body->contactCount -= 1;
}

/* reference src/contact.c:320-449 */
void o_destroy_contact( oWorld* w, oContact* c, bool wakeBodies )
{
	oset_remove( &w->pairSet, PAIR_KEY( (uint64_t)c->shapeIdA, (uint64_t)c->shapeIdB ) );
	int bodyIdA = c->edges[0].bodyId;
	int bodyIdB = c->edges[1].bodyId;
	unlink_edge( w, c, 0 );
	unlink_edge( w, c, 1 );
	if ( c->islandId != O_NULL )
		o_unlink_contact( w, c );
	if ( c->colorIndex != O_NULL )
		o_remove_contact_from_graph( w, bodyIdA, bodyIdB, c->colorIndex, c->localIndex );
	else
	{
		oIntArray* list = o_set_contacts( w, c->setIndex );
		int moved = oia_remove_swap( list, c->localIndex );
		if ( moved != O_NULL )
			w->contacts[list->data[c->localIndex]].localIndex = c->localIndex;
	}
	int id = c->id;
	c->id = O_NULL;
	c->setIndex = O_NULL;
	c->colorIndex = O_NULL;
	c->localIndex = O_NULL;
	oid_free( &w->contactIds, id );
	if ( wakeBodies )
	{
		o_wake_body( w, w->bodies + bodyIdA );
		o_wake_body( w, w->bodies + bodyIdB );
	}
}

/* ------------------------------------------------------------ colouring */
void o_add_contact_to_graph( oWorld* w, oContact* c )
{
	int colorIndex = O_OVERFLOW;
	int a = c->edges[0].bodyId;
	int b = c->edges[1].bodyId;
	bool staticA = w->bodies[a].type == b2_staticBody;
	bool staticB = w->bodies[b].type == b2_staticBody;
	if ( staticA == false && staticB == false )
	{
		for ( int i = 0; i < O_OVERFLOW; ++i )
		{
			oBits* set = &w->colors[i].bodySet;
			if ( obits_get( set, a ) || obits_get( set, b ) )
				continue;
			obits_set( set, a );
			obits_set( set, b );
			colorIndex = i;
			break;
		}
	}
	else if ( staticA == false )
	{
		for ( int i = 1; i < O_OVERFLOW; ++i )
		{
			oBits* set = &w->colors[i].bodySet;
			if ( obits_get( set, a ) )
				continue;
			obits_set( set, a );
			colorIndex = i;
			break;
		}
	}
	else if ( staticB == false )
	{
		for ( int i = 1; i < O_OVERFLOW; ++i )
		{
			oBits* set = &w->colors[i].bodySet;
			if ( obits_get( set, b ) )
				continue;
			obits_set( set, b );
			colorIndex = i;
			break;
		}
	}
	oColor* color = w->colors + colorIndex;
	c->colorIndex = colorIndex;
	c->localIndex = color->contacts.count;
	oia_push( &color->contacts, c->id );
	oBody* bodyA = w->bodies + a;
	oBody* bodyB = w->bodies + b;
	c->simIndexA = staticA ? O_NULL : a;
	c->invMassA = staticA ? R( 0 ) : bodyA->invMass;
	c->invIA = staticA ? R( 0 ) : bodyA->invI;
	c->simIndexB = staticB ? O_NULL : b;
	c->invMassB = staticB ? R( 0 ) : bodyB->invMass;
	c->invIB = staticB ? R( 0 ) : bodyB->invI;
}

void o_remove_contact_from_graph( oWorld* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex )
{
	oColor* color = w->colors + colorIndex;
	if ( colorIndex != O_OVERFLOW )
	{
		obits_clear( &color->bodySet, bodyIdA );
		obits_clear( &color->bodySet, bodyIdB );
	}
	int moved = oia_remove_swap( &color->contacts, localIndex );
	if ( moved != O_NULL )
		w->contacts[color->contacts.data[localIndex]].localIndex = localIndex;
}

int o_assign_joint_color( oWorld* w, int bodyIdA, int bodyIdB, bool staticA, bool staticB )
{
	for ( int i = 0; i < O_COLORS; ++i )
	{
		oBits* set = &w->colors[i].bodySet;
		if ( staticA == false && staticB == false )
		{
			if ( obits_get( set, bodyIdA ) || obits_get( set, bodyIdB ) )
				continue;
			obits_set( set, bodyIdA );
			obits_set( set, bodyIdB );
			return i;
		}
		else if ( staticA == false )
		{
			if ( obits_get( set, bodyIdA ) )
				continue;
			obits_set( set, bodyIdA );
			return i;
		}
		else if ( staticB == false )
		{
			if ( obits_get( set, bodyIdB ) )
				continue;
			obits_set( set, bodyIdB );
			return i;
		}
		else
			break;
	}
	return O_OVERFLOW;
}

/* ------------------------------------------------------------ joints */
bool o_should_bodies_collide( oWorld* w, oBody* a, oBody* b )
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
	while ( key != O_NULL )
	{
		oJoint* j = w->joints + ( key >> 1 );
		int e = key & 1;
		if ( j->collideConnected == false && j->edges[e ^ 1].bodyId == other )
			return false;
		key = j->edges[e].nextKey;
	}
	return true;
}

/* Joint record shared by every type (reference src/joint.c:140-288): id, body joint
 * lists, constraint graph colour.  Returns NULL when the world is locked. */
oJoint* o_create_joint( b2WorldId worldId, b2BodyId bodyIdA, b2BodyId bodyIdB, b2JointType type, bool collideConnected,
						void* userData, b2JointId* out )
{
	*out = b2_nullJointId;
	oWorld* w = o_world( worldId );
	if ( w->locked )
		return NULL;
	oBody* a = get_body( bodyIdA );
	oBody* b = get_body( bodyIdB );
	int id = oid_alloc( &w->jointIds );
	GROW( w->joints, w->jointCap, id + 1, oJoint );
	oJoint* j = w->joints + id;
	uint16_t rev = j->revision;
	memset( j, 0, sizeof( *j ) );
	j->id = id;
	j->revision = (uint16_t)( rev + 1 );
	j->type = type;
	j->bodyIdA = a->id;
	j->bodyIdB = b->id;
	j->userData = userData;
	j->collideConnected = collideConnected;
	j->indexA = O_NULL;
	j->indexB = O_NULL;

	j->edges[0].bodyId = a->id;
	j->edges[0].prevKey = O_NULL;
	j->edges[0].nextKey = a->headJointKey;
	int keyA = ( id << 1 ) | 0;
	if ( a->headJointKey != O_NULL )
		w->joints[a->headJointKey >> 1].edges[a->headJointKey & 1].prevKey = keyA;
	a->headJointKey = keyA;
	a->jointCount += 1;

	j->edges[1].bodyId = b->id;
	j->edges[1].prevKey = O_NULL;
	j->edges[1].nextKey = b->headJointKey;
	int keyB = ( id << 1 ) | 1;
	if ( b->headJointKey != O_NULL )
		w->joints[b->headJointKey >> 1].edges[b->headJointKey & 1].prevKey = keyB;
	b->headJointKey = keyB;
	b->jointCount += 1;

	j->islandId = O_NULL;
	j->islandPrev = O_NULL;
	j->islandNext = O_NULL;
	j->colorIndex = O_NULL;

	/* solver set (reference src/joint.c:198-283): between static bodies the static set;
	 * touching the awake set the constraint graph, waking a sleeping partner first;
	 * otherwise the sleeping set, merging two sleeping sets */
	int maxSetIndex = a->setIndex > b->setIndex ? a->setIndex : b->setIndex;
	if ( a->setIndex == O_SET_STATIC && b->setIndex == O_SET_STATIC )
	{
		j->setIndex = O_SET_STATIC;
		j->localIndex = w->sets[O_SET_STATIC].joints.count;
		oia_push( &w->sets[O_SET_STATIC].joints, id );
	}
	else if ( a->setIndex == O_SET_AWAKE || b->setIndex == O_SET_AWAKE )
	{
		if ( maxSetIndex >= O_SET_FIRST_SLEEPING )
			o_wake_solver_set( w, maxSetIndex );
		j->setIndex = O_SET_AWAKE;
		bool staticA = a->setIndex == O_SET_STATIC;
		bool staticB = b->setIndex == O_SET_STATIC;
		int color = o_assign_joint_color( w, a->id, b->id, staticA, staticB );
		j->colorIndex = color;
		j->localIndex = w->colors[color].joints.count;
		oia_push( &w->colors[color].joints, id );
	}
	else
	{
		j->setIndex = maxSetIndex;
		j->localIndex = w->sets[maxSetIndex].joints.count;
		oia_push( &w->sets[maxSetIndex].joints, id );
		if ( a->setIndex != b->setIndex && a->setIndex >= O_SET_FIRST_SLEEPING && b->setIndex >= O_SET_FIRST_SLEEPING )
			o_merge_solver_sets( w, a->setIndex, b->setIndex );
	}
	if ( j->setIndex > O_SET_DISABLED )
		o_link_joint( w, j );
	b2JointId jid = { id + 1, worldId.index1 - 1, j->revision };
	*out = jid;
	return j;
}

/* Destroys the contacts between two bodies, walking the shorter contact list (reference
 * src/joint.c:290-322). */
void o_destroy_contacts_between( oWorld* w, int bodyIdA, int bodyIdB )
{
	oBody* a = w->bodies + bodyIdA;
	oBody* b = w->bodies + bodyIdB;
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
	while ( key != O_NULL )
	{
		oContact* c = w->contacts + ( key >> 1 );
		int e = key & 1;
		key = c->edges[e].nextKey;
		if ( c->edges[e ^ 1].bodyId == other )
			o_destroy_contact( w, c, false );
	}
}

bool b2Joint_IsValid( b2JointId id )
{
	if ( id.world0 >= s_worldCap || s_worlds[id.world0] == NULL || !s_worlds[id.world0]->inUse )
		return false;
	oWorld* w = s_worlds[id.world0];
	if ( id.index1 < 1 || id.index1 > w->jointCap )
		return false;
	return w->joints[id.index1 - 1].id == id.index1 - 1 && w->joints[id.index1 - 1].revision == id.revision;
}

/* ------------------------------------------------------------ broadphase pairs */
typedef struct oPairList
{
	int* a;
	int* b;
	int count, capacity;
} oPairList;

typedef struct oQueryCtx
{
	oWorld* w;
	oPairList* list;
	int queryTreeType;
	int queryProxyKey;
	int queryShapeIndex;
} oQueryCtx;

static bool pair_query( int proxyId, int shapeId, void* context )
{
	oQueryCtx* q = (oQueryCtx*)context;
	oWorld* w = q->w;
	int proxyKey = ( proxyId << 2 ) | q->queryTreeType;
	if ( proxyKey == q->queryProxyKey )
		return true;
	if ( q->queryTreeType != b2_staticBody )
	{
		bool moved = oset_contains( &w->moveSet, (uint64_t)( proxyKey + 1 ) );
		if ( moved && proxyKey < q->queryProxyKey )
			return true;
	}
	uint64_t pairKey = PAIR_KEY( (uint64_t)shapeId, (uint64_t)q->queryShapeIndex );
	if ( oset_contains( &w->pairSet, pairKey ) )
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
	oShape* sA = w->shapes + idA;
	oShape* sB = w->shapes + idB;
	if ( sA->bodyId == sB->bodyId )
		return true;
	/* shape filter (reference src/contact.c:450-459) */
	if ( sA->filter.groupIndex == sB->filter.groupIndex && sA->filter.groupIndex != 0 )
	{
		if ( sA->filter.groupIndex <= 0 )
			return true;
	}
	else if ( ( sA->filter.maskBits & sB->filter.categoryBits ) == 0 || ( sA->filter.categoryBits & sB->filter.maskBits ) == 0 )
		return true;
	if ( sA->isSensor && sB->isSensor )
		return true;
	if ( o_should_bodies_collide( w, w->bodies + sA->bodyId, w->bodies + sB->bodyId ) == false )
		return true;
	oPairList* l = q->list;
	if ( l->count == l->capacity )
	{
		l->capacity = l->capacity ? 2 * l->capacity : 16;
		l->a = (int*)realloc( l->a, sizeof( int ) * (size_t)l->capacity );
		l->b = (int*)realloc( l->b, sizeof( int ) * (size_t)l->capacity );
	}
	l->a[l->count] = idA;
	l->b[l->count] = idB;
	l->count += 1;
	return true;
}

/* Reference src/broad_phase.c:278-436: query every moved proxy first, then create the
 * contacts serially, per proxy in reverse discovery order (the reference prepends). */
void o_update_pairs( oWorld* w )
{
	int moveCount = w->moveArray.count;
	if ( moveCount == 0 )
		return;
	oPairList* lists = (oPairList*)calloc( (size_t)moveCount, sizeof( oPairList ) );
	/* the queries only read the world and fill their own lists (reference
	 * src/broad_phase.c:278-331 and :361-362 runs them as parallel tasks); pairs are created below in
	 * move order */
#pragma omp parallel for if ( o_threads > 1 && moveCount >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( dynamic, 16 )
	for ( int i = 0; i < moveCount; ++i )
	{
		int proxyKey = w->moveArray.data[i];
		if ( proxyKey == O_NULL )
			continue;
		int proxyType = proxyKey & 3;
		int proxyId = proxyKey >> 2;
		const oTree* base = w->trees + proxyType;
		oBox fat = base->nodes[proxyId].box;
		oQueryCtx q;
		q.w = w;
		q.list = lists + i;
		q.queryProxyKey = proxyKey;
		q.queryShapeIndex = base->nodes[proxyId].userData;
		if ( proxyType == b2_dynamicBody )
		{
			q.queryTreeType = b2_kinematicBody;
			otree_query( w->trees + b2_kinematicBody, fat, 0xFFFFFFFFu, pair_query, &q );
			q.queryTreeType = b2_staticBody;
			otree_query( w->trees + b2_staticBody, fat, 0xFFFFFFFFu, pair_query, &q );
		}
		q.queryTreeType = b2_dynamicBody;
		otree_query( w->trees + b2_dynamicBody, fat, 0xFFFFFFFFu, pair_query, &q );
	}
	for ( int i = 0; i < moveCount; ++i )
	{
		oPairList* l = lists + i;
		for ( int k = l->count - 1; k >= 0; --k )
			o_create_contact( w, w->shapes + l->a[k], w->shapes + l->b[k] );
		free( l->a );
		free( l->b );
	}
	free( lists );
	w->moveArray.count = 0;
	oset_clear( &w->moveSet );
}

/* ------------------------------------------------------------ narrowphase */
static bool update_contact( oWorld* w, oContact* c, oShape* sA, oXf xfA, oVec offA, oShape* sB, oXf xfB, oVec offB )
{
	if ( sA->isSensor || sB->isSensor )
	{
		/* sensors: overlap of the shapes, no manifold (reference src/contact.c:476-503) */
		oProxy pa = o_shape_proxy( sA ), pb = o_shape_proxy( sB );
		b2r d = o_distance( &c->cache, &pa, xfA, &pb, xfB, NULL, NULL );
		if ( d < O_EPS )
			d = R( 0 );
		else
			d = omax( R( 0 ), d - pa.radius - pb.radius );
		bool overlap = d < R( 10.0f ) * O_EPS;
		if ( overlap )
			c->simFlags |= OS_TOUCHING;
		else
			c->simFlags &= ~OS_TOUCHING;
		return overlap;
	}
	oManifold old = c->manifold;
	oManifold m;
	switch ( sA->type )
	{
		case b2_circleShape:
			m = o_collide_circles( &sA->circle, xfA, &sB->circle, xfB );
			break;
		case b2_capsuleShape:
			if ( sB->type == b2_circleShape )
				m = o_collide_capsule_circle( &sA->capsule, xfA, &sB->circle, xfB );
			else
			{
				oPolygon pa = o_make_capsule( sA->capsule.c1, sA->capsule.c2, sA->capsule.radius );
				oPolygon pb = o_make_capsule( sB->capsule.c1, sB->capsule.c2, sB->capsule.radius );
				m = o_collide_polygons( &pa, xfA, &pb, xfB );
			}
			break;
		case b2_segmentShape:
		{
			if ( sB->type == b2_circleShape )
			{
				oCapsule ca = { sA->segment.p1, sA->segment.p2, 0 };
				m = o_collide_capsule_circle( &ca, xfA, &sB->circle, xfB );
			}
			else
			{
				oPolygon pa = o_make_capsule( sA->segment.p1, sA->segment.p2, 0 );
				oPolygon pb;
				if ( sB->type == b2_capsuleShape )
					pb = o_make_capsule( sB->capsule.c1, sB->capsule.c2, sB->capsule.radius );
				else
					pb = sB->polygon;
				m = o_collide_polygons( &pa, xfA, &pb, xfB );
			}
			break;
		}
		case b2_smoothSegmentShape:
			/* chain links keep the contact's closest-feature cache (reference
			 * src/contact.c:131-148) */
			if ( sB->type == b2_circleShape )
				m = o_collide_smooth_circle( &sA->smooth, xfA, &sB->circle, xfB );
			else if ( sB->type == b2_capsuleShape )
			{
				oPolygon pb = o_make_capsule( sB->capsule.c1, sB->capsule.c2, sB->capsule.radius );
				m = o_collide_smooth_polygon( &sA->smooth, xfA, &pb, xfB, &c->cache );
			}
			else
				m = o_collide_smooth_polygon( &sA->smooth, xfA, &sB->polygon, xfB, &c->cache );
			break;
		case b2_polygonShape:
			if ( sB->type == b2_circleShape )
				m = o_collide_polygon_circle( &sA->polygon, xfA, &sB->circle, xfB );
			else if ( sB->type == b2_capsuleShape )
			{
				oPolygon pb = o_make_capsule( sB->capsule.c1, sB->capsule.c2, sB->capsule.radius );
				m = o_collide_polygons( &sA->polygon, xfA, &pb, xfB );
			}
			else
				m = o_collide_polygons( &sA->polygon, xfA, &sB->polygon, xfB );
			break;
		default:
			memset( &m, 0, sizeof( m ) );
			break;
	}
	c->manifold = m;
	int pointCount = m.count;
	bool touching = pointCount > 0;
	if ( touching && ( sA->enableHitEvents || sB->enableHitEvents ) )
		c->simFlags |= OS_HIT;
	else
		c->simFlags &= ~OS_HIT;
	for ( int i = 0; i < pointCount; ++i )
	{
		oMPoint* mp2 = c->manifold.pts + i;
		mp2->anchorA = osub( mp2->anchorA, offA );
		mp2->anchorB = osub( mp2->anchorB, offB );
		mp2->normalImpulse = 0;
		mp2->tangentImpulse = 0;
		mp2->maxNormalImpulse = 0;
		mp2->normalVelocity = 0;
		mp2->persisted = false;
		for ( int j = 0; j < old.count; ++j )
		{
			oMPoint* mp1 = old.pts + j;
			if ( mp1->id == mp2->id )
			{
				mp2->normalImpulse = mp1->normalImpulse;
				mp2->tangentImpulse = mp1->tangentImpulse;
				mp2->persisted = true;
				break;
			}
		}
	}
	if ( touching )
		c->simFlags |= OS_TOUCHING;
	else
		c->simFlags &= ~OS_TOUCHING;
	return touching;
}

/* Narrowphase of one contact; returns whether its state changed (disjoint, started or
 * stopped touching). */
static bool collide_one( oWorld* w, oContact* c )
{
	oShape* sA = w->shapes + c->shapeIdA;
	oShape* sB = w->shapes + c->shapeIdB;
	if ( obox_overlaps( sA->fatAABB, sB->fatAABB ) == false )
	{
		c->simFlags |= OS_DISJOINT;
		c->simFlags &= ~OS_TOUCHING;
		return true;
	}
	bool wasTouching = ( c->simFlags & OS_TOUCHING ) != 0;
	oBody* bA = w->bodies + sA->bodyId;
	oBody* bB = w->bodies + sB->bodyId;
	c->simIndexA = bA->awakeIndex != O_NULL ? bA->id : O_NULL;
	c->invMassA = bA->invMass;
	c->invIA = bA->invI;
	c->simIndexB = bB->awakeIndex != O_NULL ? bB->id : O_NULL;
	c->invMassB = bB->invMass;
	c->invIB = bB->invI;
	oVec offA = orotate( bA->xf.q, bA->localCenter );
	oVec offB = orotate( bB->xf.q, bB->localCenter );
	bool touching = update_contact( w, c, sA, bA->xf, offA, sB, bB->xf, offB );
	if ( touching && !wasTouching )
	{
		c->simFlags |= OS_STARTED;
		return true;
	}
	else if ( !touching && wasTouching )
	{
		c->simFlags |= OS_STOPPED;
		return true;
	}
	return false;
}

/* Contacts [0, count) of a list through the narrowphase (in parallel: each touches only
 * its own contact), then their state changes into the bitset in list order. */
static void collide_list( oWorld* w, const int* ids, int count, oBits* changed )
{
	uint8_t* flag = (uint8_t*)malloc( (size_t)( count > 0 ? count : 1 ) );
#pragma omp parallel for if ( o_threads > 1 && count >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( static )
	for ( int k = 0; k < count; ++k )
		flag[k] = collide_one( w, w->contacts + ids[k] ) ? 1 : 0;
	for ( int k = 0; k < count; ++k )
		if ( flag[k] )
			obits_set( changed, ids[k] );
	free( flag );
}

/* Reference src/world.c:410-674. */
void o_collide( oWorld* w )
{
	/* the tree rebuild runs here in the reference (async task started at :420) */
	otree_rebuild( w->trees + b2_dynamicBody );
	otree_rebuild( w->trees + b2_kinematicBody );

	oBits changed = { 0 };
	for ( int i = 0; i < O_COLORS; ++i )
		collide_list( w, w->colors[i].contacts.data, w->colors[i].contacts.count, &changed );
	collide_list( w, w->nonTouching.data, w->nonTouching.count, &changed );

	for ( int word = 0; word < changed.wordCount; ++word )
	{
		uint64_t bits = changed.words[word];
		while ( bits )
		{
			int ctz = __builtin_ctzll( bits );
			int id = 64 * word + ctz;
			bits &= bits - 1;
			oContact* c = w->contacts + id;
			uint32_t flags = c->flags;
			uint32_t simFlags = c->simFlags;
			if ( simFlags & OS_DISJOINT )
			{
				if ( ( flags & OC_TOUCHING ) && ( flags & OC_ENABLE_CONTACT_EVENTS ) )
					add_event_end( w, c->shapeIdA, c->shapeIdB );
				c->flags &= ~OC_TOUCHING;
				o_destroy_contact( w, c, false );
			}
			else if ( simFlags & OS_STARTED )
			{
				if ( flags & OC_SENSOR )
				{
					if ( flags & OC_ENABLE_SENSOR_EVENTS )
					{
						if ( w->shapes[c->shapeIdA].isSensor )
							add_sensor_event( w, true, c->shapeIdA, c->shapeIdB );
						if ( w->shapes[c->shapeIdB].isSensor )
							add_sensor_event( w, true, c->shapeIdB, c->shapeIdA );
					}
					c->simFlags &= ~OS_STARTED;
					c->flags |= OC_SENSOR_TOUCHING;
				}
				else
				{
					if ( flags & OC_ENABLE_CONTACT_EVENTS )
						add_event_begin( w, c->shapeIdA, c->shapeIdB );
					/* link first: it may wake a sleeping set, which appends to the awake
					 * lists and leaves this contact's place unchanged */
					c->flags |= OC_TOUCHING;
					o_link_contact( w, c );
					c->simFlags &= ~OS_STARTED;
					int localIndex = c->localIndex;
					o_add_contact_to_graph( w, c );
					remove_non_touching( w, localIndex );
				}
			}
			else if ( simFlags & OS_STOPPED )
			{
				c->simFlags &= ~OS_STOPPED;
				if ( flags & OC_SENSOR )
				{
					c->flags &= ~OC_SENSOR_TOUCHING;
					if ( flags & OC_ENABLE_SENSOR_EVENTS )
					{
						if ( w->shapes[c->shapeIdA].isSensor )
							add_sensor_event( w, false, c->shapeIdA, c->shapeIdB );
						if ( w->shapes[c->shapeIdB].isSensor )
							add_sensor_event( w, false, c->shapeIdB, c->shapeIdA );
					}
				}
				else
				{
					c->flags &= ~OC_TOUCHING;
					if ( c->flags & OC_ENABLE_CONTACT_EVENTS )
						add_event_end( w, c->shapeIdA, c->shapeIdB );
					o_unlink_contact( w, c );
					int a = c->edges[0].bodyId, b = c->edges[1].bodyId;
					int colorIndex = c->colorIndex, localIndex = c->localIndex;
					c->setIndex = O_SET_AWAKE;
					c->colorIndex = O_NULL;
					c->localIndex = w->nonTouching.count;
					oia_push( &w->nonTouching, id );
					o_remove_contact_from_graph( w, a, b, colorIndex, localIndex );
				}
			}
		}
	}
	obits_free( &changed );
}

void b2World_Step( b2WorldId worldId, float timeStep, int subStepCount )
{
	oWorld* w = o_world( worldId );
	if ( w->locked )
		return;
	w->beginCount = 0;
	w->endCount = 0;
	w->hitCount = 0;
	w->sensorBeginCount = 0;
	w->sensorEndCount = 0;
	memset( &w->profile, 0, sizeof( w->profile ) );
	if ( timeStep == 0.0f )
		return;
	w->locked = true;
	o_step( w, timeStep, subStepCount );
	w->locked = false;
}

/* ------------------------------------------------------------ destruction
 * reference src/body.c:161-176, :336-430 (b2DestroyBody), src/shape.c:220-290
 * (b2DestroyShapeInternal, b2DestroyShape), src/shape.c:704-711 and
 * src/broad_phase.c:71-116 (proxy destruction with the move-buffer purge),
 * src/joint.c:657-768 (b2DestroyJointInternal) and src/constraint_graph.c:297-324.
 * Destruction unlinks islands and wakes the bodies it touches, as the reference does. */
static void unbuffer_move( oWorld* w, int proxyKey )
{
	if ( oset_remove( &w->moveSet, (uint64_t)( proxyKey + 1 ) ) == false )
		return;
	for ( int i = 0; i < w->moveArray.count; ++i )
	{
		if ( w->moveArray.data[i] == proxyKey )
		{
			oia_remove_swap( &w->moveArray, i );
			break;
		}
	}
}

static void destroy_proxy( oWorld* w, oShape* s )
{
	if ( s->proxyKey == O_NULL )
		return;
	unbuffer_move( w, s->proxyKey );
	otree_destroy_proxy( w->trees + ( s->proxyKey & 3 ), s->proxyKey >> 2 );
	s->proxyKey = O_NULL;
}

static void unlink_joint_edge( oWorld* w, oJoint* j, int e )
{
	oEdge* edge = j->edges + e;
	oBody* body = w->bodies + edge->bodyId;
	if ( edge->prevKey != O_NULL )
		w->joints[edge->prevKey >> 1].edges[edge->prevKey & 1].nextKey = edge->nextKey;
	if ( edge->nextKey != O_NULL )
		w->joints[edge->nextKey >> 1].edges[edge->nextKey & 1].prevKey = edge->prevKey;
	int key = ( j->id << 1 ) | e;
	if ( body->headJointKey == key )
		body->headJointKey = edge->nextKey;
	body->jointCount -= 1;
}

/* reference src/joint.c:657-752 */
static void destroy_joint( oWorld* w, oJoint* j, bool wakeBodies )
{
	int bodyIdA = j->edges[0].bodyId;
	int bodyIdB = j->edges[1].bodyId;
	unlink_joint_edge( w, j, 0 );
	unlink_joint_edge( w, j, 1 );
	o_unlink_joint( w, j );
	if ( j->setIndex != O_SET_AWAKE )
	{
		oIntArray* list = o_set_joints( w, j->setIndex );
		int moved = oia_remove_swap( list, j->localIndex );
		if ( moved != O_NULL )
			w->joints[list->data[j->localIndex]].localIndex = j->localIndex;
	}
	else
	{
		oColor* color = w->colors + j->colorIndex;
		if ( j->colorIndex != O_OVERFLOW )
		{
			obits_clear( &color->bodySet, j->edges[0].bodyId );
			obits_clear( &color->bodySet, j->edges[1].bodyId );
		}
		int moved = oia_remove_swap( &color->joints, j->localIndex );
		if ( moved != O_NULL )
			w->joints[color->joints.data[j->localIndex]].localIndex = j->localIndex;
	}
	int id = j->id;
	j->setIndex = O_NULL;
	j->colorIndex = O_NULL;
	j->localIndex = O_NULL;
	j->id = O_NULL;
	oid_free( &w->jointIds, id );
	if ( wakeBodies )
	{
		o_wake_body( w, w->bodies + bodyIdA );
		o_wake_body( w, w->bodies + bodyIdB );
	}
}

void b2DestroyJoint( b2JointId jointId )
{
	if ( b2Joint_IsValid( jointId ) == false )
		return;
	oWorld* w = s_worlds[jointId.world0];
	if ( w->locked )
		return;
	destroy_joint( w, w->joints + ( jointId.index1 - 1 ), true );
}

/* Unlinks and frees a shape with its proxy and contacts (reference src/shape.c:220-269). */
static void destroy_shape_internal( oWorld* w, oShape* s, oBody* b, bool wakeBodies )
{
	int id = s->id;
	if ( s->prev != O_NULL )
		w->shapes[s->prev].next = s->next;
	if ( s->next != O_NULL )
		w->shapes[s->next].prev = s->prev;
	if ( b->headShape == id )
		b->headShape = s->next;
	b->shapeCount -= 1;
	destroy_proxy( w, s );
	int key = b->headContactKey;
	while ( key != O_NULL )
	{
		oContact* c = w->contacts + ( key >> 1 );
		key = c->edges[key & 1].nextKey;
		if ( c->shapeIdA == id || c->shapeIdB == id )
			o_destroy_contact( w, c, wakeBodies );
	}
	oid_free( &w->shapeIds, id );
	s->id = O_NULL;
}

void b2DestroyShape( b2ShapeId shapeId )
{
	if ( b2Shape_IsValid( shapeId ) == false )
		return;
	oWorld* w = s_worlds[shapeId.world0];
	if ( w->locked )
		return;
	oShape* s = get_shape( shapeId );
	oBody* b = w->bodies + s->bodyId;
	destroy_shape_internal( w, s, b, true );
	if ( b->automaticMass )
		o_update_body_mass( w, b );
}

/* ------------------------------------------------------------ chains */
b2ChainDef b2DefaultChainDef( void )
{
	b2ChainDef d;
	memset( &d, 0, sizeof( d ) );
	d.friction = 0.6f;
	d.filter = b2DefaultFilter();
	d.internalValue = 1152023;
	return d;
}

/* reference src/shape.c:292-403 */
b2ChainId b2CreateChain( b2BodyId bodyId, const b2ChainDef* def )
{
	oWorld* w = body_world( bodyId );
	if ( w->locked || def->count < 4 )
		return b2_nullChainId;
	oBody* body = get_body( bodyId );
	int chainId = oid_alloc( &w->chainIds );
	GROW( w->chains, w->chainCap, chainId + 1, oChain );
	oChain* chain = w->chains + chainId;
	uint16_t rev = chain->revision;
	memset( chain, 0, sizeof( *chain ) );
	chain->revision = (uint16_t)( rev + 1 );
	chain->id = chainId;
	chain->bodyId = body->id;
	chain->nextChainId = body->headChainId;
	body->headChainId = chainId;

	b2ShapeDef sd = b2DefaultShapeDef();
	sd.userData = def->userData;
	sd.restitution = def->restitution;
	sd.friction = def->friction;
	sd.filter = def->filter;
	sd.enableContactEvents = false;
	sd.enableHitEvents = false;
	sd.enableSensorEvents = false;

	int n = def->count;
	const b2Vec2* points = def->points;
	chain->shapeIndices = (int*)malloc( sizeof( int ) * (size_t)n );
	b2SmoothSegment seg;
	seg.chainId = chainId;
	if ( def->isLoop )
	{
		chain->count = n;
		int prevIndex = n - 1;
		for ( int i = 0; i < n - 2; ++i )
		{
			seg.ghost1 = points[prevIndex];
			seg.segment.point1 = points[i];
			seg.segment.point2 = points[i + 1];
			seg.ghost2 = points[i + 2];
			prevIndex = i;
			chain->shapeIndices[i] = create_shape_internal( bodyId, &sd, b2_smoothSegmentShape, &seg, false ).index1 - 1;
		}
		seg.ghost1 = points[n - 3];
		seg.segment.point1 = points[n - 2];
		seg.segment.point2 = points[n - 1];
		seg.ghost2 = points[0];
		chain->shapeIndices[n - 2] = create_shape_internal( bodyId, &sd, b2_smoothSegmentShape, &seg, false ).index1 - 1;
		seg.ghost1 = points[n - 2];
		seg.segment.point1 = points[n - 1];
		seg.segment.point2 = points[0];
		seg.ghost2 = points[1];
		chain->shapeIndices[n - 1] = create_shape_internal( bodyId, &sd, b2_smoothSegmentShape, &seg, false ).index1 - 1;
	}
	else
	{
		chain->count = n - 3;
		for ( int i = 0; i < n - 3; ++i )
		{
			seg.ghost1 = points[i];
			seg.segment.point1 = points[i + 1];
			seg.segment.point2 = points[i + 2];
			seg.ghost2 = points[i + 3];
			chain->shapeIndices[i] = create_shape_internal( bodyId, &sd, b2_smoothSegmentShape, &seg, false ).index1 - 1;
		}
	}
	b2ChainId id = { chainId + 1, bodyId.world0, chain->revision };
	return id;
}

bool b2Chain_IsValid( b2ChainId id )
{
	if ( id.world0 >= s_worldCap || s_worlds[id.world0] == NULL || !s_worlds[id.world0]->inUse )
		return false;
	oWorld* w = s_worlds[id.world0];
	if ( id.index1 < 1 || id.index1 > w->chainCap )
		return false;
	oChain* c = w->chains + ( id.index1 - 1 );
	return c->id == id.index1 - 1 && c->revision == id.revision;
}

/* reference src/shape.c:405-451 */
void b2DestroyChain( b2ChainId chainId )
{
	if ( b2Chain_IsValid( chainId ) == false )
		return;
	oWorld* w = s_worlds[chainId.world0];
	if ( w->locked )
		return;
	oChain* chain = w->chains + ( chainId.index1 - 1 );
	oBody* body = w->bodies + chain->bodyId;
	int* link = &body->headChainId;
	while ( *link != O_NULL && *link != chain->id )
		link = &w->chains[*link].nextChainId;
	if ( *link == O_NULL )
		return;
	*link = chain->nextChainId;
	for ( int i = 0; i < chain->count; ++i )
		destroy_shape_internal( w, w->shapes + chain->shapeIndices[i], body, true );
	free( chain->shapeIndices );
	chain->shapeIndices = NULL;
	oid_free( &w->chainIds, chain->id );
	chain->id = O_NULL;
}

void b2Chain_SetFriction( b2ChainId chainId, float friction )
{
	oWorld* w = s_worlds[chainId.world0];
	oChain* chain = w->chains + ( chainId.index1 - 1 );
	for ( int i = 0; i < chain->count; ++i )
		w->shapes[chain->shapeIndices[i]].friction = friction;
}

void b2Chain_SetRestitution( b2ChainId chainId, float restitution )
{
	oWorld* w = s_worlds[chainId.world0];
	oChain* chain = w->chains + ( chainId.index1 - 1 );
	for ( int i = 0; i < chain->count; ++i )
		w->shapes[chain->shapeIndices[i]].restitution = restitution;
}

b2ChainId b2Shape_GetParentChain( b2ShapeId shapeId )
{
	oWorld* w = s_worlds[shapeId.world0];
	oShape* s = get_shape( shapeId );
	if ( s->type == b2_smoothSegmentShape && s->smooth.chainId != O_NULL )
	{
		b2ChainId id = { s->smooth.chainId + 1, shapeId.world0, w->chains[s->smooth.chainId].revision };
		return id;
	}
	return b2_nullChainId;
}

b2Segment b2Shape_GetSegment( b2ShapeId id )
{
	oShape* s = get_shape( id );
	b2Segment r = { vfo( s->segment.p1 ), vfo( s->segment.p2 ) };
	return r;
}

b2SmoothSegment b2Shape_GetSmoothSegment( b2ShapeId id )
{
	oShape* s = get_shape( id );
	b2SmoothSegment r;
	r.ghost1 = vfo( s->smooth.ghost1 );
	r.segment.point1 = vfo( s->smooth.p1 );
	r.segment.point2 = vfo( s->smooth.p2 );
	r.ghost2 = vfo( s->smooth.ghost2 );
	r.chainId = s->smooth.chainId;
	return r;
}

b2Capsule b2Shape_GetCapsule( b2ShapeId id )
{
	oShape* s = get_shape( id );
	b2Capsule r = { vfo( s->capsule.c1 ), vfo( s->capsule.c2 ), (float)s->capsule.radius };
	return r;
}

void b2DestroyBody( b2BodyId bodyId )
{
	if ( b2Body_IsValid( bodyId ) == false )
		return;
	oWorld* w = body_world( bodyId );
	if ( w->locked )
		return;
	oBody* b = get_body( bodyId );
	int key = b->headJointKey;
	while ( key != O_NULL )
	{
		oJoint* j = w->joints + ( key >> 1 );
		key = j->edges[key & 1].nextKey;
		destroy_joint( w, j, true );
	}
	key = b->headContactKey;
	while ( key != O_NULL )
	{
		oContact* c = w->contacts + ( key >> 1 );
		key = c->edges[key & 1].nextKey;
		o_destroy_contact( w, c, true );
	}
	for ( int sid = b->headShape; sid != O_NULL; )
	{
		oShape* s = w->shapes + sid;
		destroy_proxy( w, s );
		oid_free( &w->shapeIds, sid );
		s->id = O_NULL;
		sid = s->next;
	}
	for ( int cid = b->headChainId; cid != O_NULL; )
	{
		oChain* chain = w->chains + cid;
		free( chain->shapeIndices );
		chain->shapeIndices = NULL;
		oid_free( &w->chainIds, cid );
		chain->id = O_NULL;
		cid = chain->nextChainId;
	}
	/* the body's set drops it by moving its last body into the slot */
	o_remove_body_from_island( w, b );
	o_remove_body_from_set( w, b );
	oid_free( &w->bodyIds, b->id );
	b->setIndex = O_NULL;
	b->awakeIndex = O_NULL;
	b->setLocal = O_NULL;
	b->id = O_NULL;
}
