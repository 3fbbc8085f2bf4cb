/*
 * host.h -- host-side records of the GB300 step driver.
 *
 * The host keeps what is serial and order-sensitive in the reference step: id pools
 * (src/id_pool.c), body/shape/contact/joint bookkeeping and linked lists
 * (src/body.c, src/shape.c, src/contact.c, src/joint.c), the three broadphase trees and
 * move buffer (src/dynamic_tree.c, src/broad_phase.c) and the constraint-graph colour
 * arrays (src/constraint_graph.c).  Numeric state (body motion, shape boxes, manifolds,
 * impulses) lives in the device arena (b2g_types.h) and is mirrored into pinned host
 * arrays only for setup and read-back.
 */
#pragma once

#include "b2g_device.h"
#include "b2g_math.h"
#include "b2g_types.h"

#include "box2d/box2d.h"

#include <stdlib.h>

/* ---------------------------------------------------------------- containers */
typedef struct gIntArray
{
	int* data;
	int count;
	int capacity;
} gIntArray;

void gia_push( gIntArray* a, int v );
int gia_remove_swap( gIntArray* a, int index ); /* returns the moved index or -1 */
bool gia_reserve( gIntArray* a, int count );   /* false when memory ran out */

/* Host memory through the caller's allocator (util.c, reference src/allocate.c):
 * b2g_realloc keeps the old block when it fails; every failure is counted. */
void* b2g_alloc( size_t size );
void* b2g_realloc( void* p, size_t size );
int b2g_alloc_failures( void );
void b2g_note_alloc_failure( void );
void gia_free( gIntArray* a );

typedef struct gSet
{
	uint64_t* keys;
	int capacity;
	int count;
} gSet;

bool gset_add( gSet* s, uint64_t key ); /* true if already present */
bool gset_remove( gSet* s, uint64_t key );
bool gset_contains( const gSet* s, uint64_t key );
void gset_clear( gSet* s );
void gset_free( gSet* s );

typedef struct gIdPool
{
	gIntArray freeIds;
	int next;
} gIdPool;

int gid_alloc( gIdPool* p );
void gid_free( gIdPool* p, int id );
/* Returns an id a failed creation took: the pool is as before the gid_alloc. */
void gid_unalloc( gIdPool* p, int id );
int gid_count( const gIdPool* p );

typedef struct gBits
{
	uint64_t* words;
	int wordCount;
} gBits;

bool gbits_get( const gBits* b, int i );
void gbits_set( gBits* b, int i );
void gbits_clear( gBits* b, int i );
void gbits_free( gBits* b );

/* ---------------------------------------------------------------- tree */
typedef b2gTreeNode gNode;

typedef struct gTree
{
	gNode* nodes;
	int root;
	int nodeCount;
	int capacity; /* nodes in the pool (used or on the free list) */
	int reserved; /* nodes the allocation holds, at least capacity */
	int freeList;
	int proxyCount;
	int* leafIndices;
	b2gVec* leafCenters;
	int rebuildCapacity;
} gTree;

static inline float gbox_perimeter( b2gBox a )
{
	float wx = a.hi.x - a.lo.x;
	float wy = a.hi.y - a.lo.y;
	return 2.0f * ( wx + wy );
}

static inline b2gVec gbox_center( b2gBox a ) { return gv( 0.5f * ( a.lo.x + a.hi.x ), 0.5f * ( a.lo.y + a.hi.y ) ); }

static inline bool gbox_enlarge( b2gBox* a, b2gBox b )
{
	bool changed = false;
	if ( b.lo.x < a->lo.x )
	{
		a->lo.x = b.lo.x;
		changed = true;
	}
	if ( b.lo.y < a->lo.y )
	{
		a->lo.y = b.lo.y;
		changed = true;
	}
	if ( a->hi.x < b.hi.x )
	{
		a->hi.x = b.hi.x;
		changed = true;
	}
	if ( a->hi.y < b.hi.y )
	{
		a->hi.y = b.hi.y;
		changed = true;
	}
	return changed;
}

void gtree_init( gTree* t );
void gtree_free( gTree* t );
int gtree_create_proxy( gTree* t, b2gBox box, uint32_t category, int userData );
void gtree_destroy_proxy( gTree* t, int proxyId );
void gtree_move_proxy( gTree* t, int proxyId, b2gBox box );
void gtree_enlarge_proxy( gTree* t, int proxyId, b2gBox box );
void gtree_rebuild( gTree* t );
int gtree_height( const gTree* t );
typedef bool gQueryFcn( int proxyId, int userData, void* ctx );
void gtree_query( const gTree* t, b2gBox box, uint32_t mask, gQueryFcn* fcn, void* ctx );

/* ---------------------------------------------------------------- records */
typedef struct gBody
{
	int id; /* -1 when free */
	b2BodyType type;
	int awakeIndex;
	int headShape, shapeCount;
	int headContactKey, contactCount;
	int headJointKey, jointCount;
	int headChainId;
	void* userData;
	uint16_t revision;
	bool fixedRotation, isBullet, enableSleep, automaticMass;
	float sleepThreshold;
	int setIndex; /* solver set: G_SET_STATIC, G_SET_AWAKE or a sleeping set */
	int setLocal; /* position in a sleeping set's body list */
	int islandId, islandPrev, islandNext;
	bool isMarked;
} gBody;

typedef struct gShape
{
	int id;
	int bodyId;
	int prev, next;
	b2ShapeType type;
	float density, friction, restitution;
	b2Filter filter;
	void* userData;
	int proxyKey;
	int chainId; /* smooth segments of a chain: the chain, else -1 */
	uint16_t revision;
	bool isSensor, enableContactEvents, enableSensorEvents, enableHitEvents, enablePreSolveEvents;
} gShape;

/* A chain: the smooth segments made from one point list (reference src/shape.h:52-60). */
typedef struct gChain
{
	int id; /* -1 when free */
	int bodyId;
	int nextChainId;
	int* shapeIndices;
	int count;
	uint16_t revision;
} gChain;

typedef struct gEdge
{
	int bodyId, prevKey, nextKey;
} gEdge;

enum
{
	G_TOUCHING = 1,
	G_SENSOR = 4,
	G_ENABLE_SENSOR_EVENTS = 0x10,
	G_ENABLE_CONTACT_EVENTS = 0x20,
	G_SENSOR_TOUCHING = 0x40,
};

typedef struct gContact
{
	int id;
	int setIndex; /* awake, disabled (non-touching between bodies not awake) or sleeping */
	int colorIndex, localIndex;
	int islandId, islandPrev, islandNext;
	bool isMarked;
	gEdge edges[2];
	int shapeIdA, shapeIdB;
	uint32_t flags;
	float friction, restitution;
} gContact;

typedef struct gJoint
{
	int id;
	b2JointType type;
	int bodyIdA, bodyIdB;
	gEdge edges[2];
	int setIndex;
	int colorIndex, localIndex;
	int islandId, islandPrev, islandNext;
	bool isMarked;
	bool collideConnected;
	uint16_t revision;
	void* userData;
} gJoint;

/* Solver sets (reference src/solver_set.h:11-30): static, disabled, awake, then one per
 * group of sleeping islands. */
enum
{
	G_SET_STATIC = 0,
	G_SET_DISABLED = 1,
	G_SET_AWAKE = 2,
	G_SET_FIRST_SLEEPING = 3,
};

/* A persistent island (reference src/island.h:32-56): its bodies, touching contacts and
 * joints as linked lists through the records, and a union-find parent for islands that
 * a new constraint joined since the last merge. */
typedef struct gIsland
{
	int setIndex, localIndex, islandId;
	int headBody, tailBody, bodyCount;
	int headContact, tailContact, contactCount;
	int headJoint, tailJoint, jointCount;
	int parentIsland;
	int constraintRemoveCount;
} gIsland;

/* The members of a sleeping set in set order; the awake set's are the awake lists and
 * the graph colours. */
typedef struct gSolverSet
{
	int setIndex; /* -1 when free */
	gIntArray bodies, contacts, joints, islands;
} gSolverSet;

/* Pairs found from one moved proxy (kept across steps, only the count is reset). */
typedef struct gPairList
{
	int* a;
	int* b;
	int count, capacity;
} gPairList;

typedef struct gColor
{
	gBits bodySet;
	gIntArray contacts;
	gIntArray joints;
} gColor;

typedef struct gWorld
{
	bool inUse;
	uint16_t revision;
	int slot;

	gIdPool bodyIds, shapeIds, contactIds, jointIds, chainIds;
	gBody* bodies;
	int bodyCap;
	gShape* shapes;
	int shapeCap;
	gContact* contacts;
	int contactCap;
	gJoint* joints;
	int jointCap;
	gChain* chains;
	int chainCap;

	/* pinned host mirrors in device layout, indexed by id */
	float* hState; /* 8 per body */
	float* hXf;
	float* hCenters;
	float* hPrev;
	float* hMass;
	float* hForce;
	float* hExtent;
	int* hInfo;
	int mirrorCap;
	b2gShapeGeo* hGeo;
	float* hAabb;
	float* hFat;
	int shapeMirrorCap;
	b2gJointDev* hJoints;
	int jointMirrorCap;

	gIntArray awake;
	gIntArray nonTouching;
	gColor colors[B2G_COLORS];

	/* islands and solver sets (island.c) */
	gIntArray disabledContacts; /* non-touching contacts whose bodies are both not awake */
	gIntArray staticJoints;		/* joints between two static bodies */
	gIntArray awakeIslands;		/* awake island ids in set order */
	gIsland* islands;
	int islandCap;
	gIdPool islandIds;
	gSolverSet* sets; /* by set id; entries below G_SET_FIRST_SLEEPING unused */
	int setCap;
	gIdPool setIds;
	int splitIslandId;	  /* island to split at the next solve, or -1 */
	gIntArray bodyOps;	  /* device body operations staged since the last flush */
	int* bodyOpSlot;	  /* per body id: its op's position in bodyOps, or -1 */
	int bodyOpSlotCap;
	int* islandSleepy;	  /* per awake island: bodies past the sleep time this step */
	int islandSleepyCap;

	gTree trees[3];
	gIntArray moveArray;
	gSet moveSet;
	gSet pairSet;
	unsigned pairSetVersion; /* changes with every pair added or removed */

	/* step staging */
	b2gContactInit* pending;
	int pendingCount, pendingCap;
	int* scratch;
	int scratchCap;
	b2gRecord* recordSort; /* finalisation records in awake order */
	int recordSortCap;
	int* recordBucket; /* per awake index: first sorted record */
	int recordBucketCap;
	gIntArray solveList;
	gIntArray jointList;
	b2gSolvePlan solvePlan; /* plan of the current solve lists */
	bool solveUploaded;		/* solve lists on the device match the host's */
	b2gPairQuery* pairQuery; /* device pair query buffers, made on first use */
	gPairList* pairLists;	 /* per moved proxy, reused every step */
	int pairListCap;

	b2gVec gravity;
	float restitutionThreshold, pushout, hitThreshold, contactHertz, contactDamping, jointHertz, jointDamping;
	float inv_h;
	bool enableSleep, enableWarmStarting, enableContinuous, locked;

	/* dirty / stale tracking */
	bool bodiesDirty, awakeDirty, shapesDirty, shapeListsDirty, jointsDirty, solveDirty;
	bool mirrorStale, shapeMirrorStale, jointMirrorStale;

	b2ContactBeginTouchEvent* beginEvents;
	int beginCount, beginCap;
	b2ContactEndTouchEvent* endEvents;
	int endCount, endCap;
	b2ContactHitEvent* hitEvents;
	int hitCount, hitCap;
	b2SensorBeginTouchEvent* sensorBeginEvents;
	int sensorBeginCount, sensorBeginCap;
	b2SensorEndTouchEvent* sensorEndEvents;
	int sensorEndCount, sensorEndCap;
	int hitShapes; /* live shapes with hit events enabled */

	b2Profile profile;
	/* host phases of the last step in ms (b2DeviceTimes order): pair query, pair rules,
	 * contact creation, events, solve lists, tree rebuild, records, continuous */
	float hostMs[8];
	int status; /* last CUDA error or 0 */
	int toiEvents;	   /* time-of-impact events since the world was created */
	int tapeToiEvents; /* time-of-impact events while the tape records */
	int lastEventCount, lastRecordCount;
	double stepStart; /* host clock at the start of the current step phase */
	int stepIdCount;  /* contact ids of the current step's narrowphase */
	struct gTape* tape; /* recording for b2World_StepBackward, or null */
	bool batching;		/* inside b2World_StepBatch: tape records go into the batch's graph */
	void* tapeBodyDst;	/* this step's tape destinations while batching */
	void* tapeRowDst;
	int tapeRowCount;

	b2gDevWorld dev;
	b2gHostIO io;
} gWorld;

gWorld* gworld_get( b2WorldId id );
gWorld* gworld_slot( int slot );
void gworld_fail( const char* what );

/* True (and the world marked failed) when a host allocation failed since
 * b2g_alloc_failures() returned `before`. */
bool gworld_out_of_memory( gWorld* w, int before );

void gworld_ensure_mirror( gWorld* w );
void gworld_ensure_shape_mirror( gWorld* w );
bool gworld_reserve_mirrors( gWorld* w ); /* false when pinned memory ran out */
void gworld_flush( gWorld* w );

void gstep_run( gWorld* w, float dt, int subSteps );

/* Phases of one step, driven by gstep_run for one world and by b2World_StepBatch for
 * many: begin (pairs, staging) -> narrowphase on the device (trees rebuilt meanwhile)
 * -> after_collide (events, constants, solve lists) -> solver on the device -> finish
 * (records). */
int gstep_begin( gWorld* w );

/* Fork-join pool for per-world host work (pool.c). */
typedef void gTaskFn( int begin, int end, void* ctx );
void gpool_for( int count, int grain, gTaskFn* fn, void* ctx );
bool gpool_try_for( int count, int grain, gTaskFn* fn, void* ctx );
int gpool_threads( void );
void gstep_rebuild_trees( gWorld* w );
int gstep_after_collide( gWorld* w, float dt, int subSteps, b2gStepConst* sc, b2gSolvePlan* plan );
void gstep_finish( gWorld* w );

/* Adjoint tape (adjoint.c): records the solver inputs of the current step when the
 * world is recording; frees a world's tape. */
void gtape_record( gWorld* w, const b2gSolvePlan* plan, const b2gStepConst* sc, int solve );
void gtape_free( gWorld* w );
void gcontact_create( gWorld* w, gShape* a, gShape* b );
void gcontact_destroy( gWorld* w, gContact* c, bool wakeBodies );
void gcontact_add_to_graph( gWorld* w, gContact* c );
void gcontact_remove_from_graph( gWorld* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex );
/* Stages the move of a live contact into (asleep false) or out of the awake set for the
 * device narrowphase. */
void gcontact_stage_set( gWorld* w, int contactId, bool asleep );

/* Islands, solver sets and sleep (island.c; reference src/island.c, src/solver_set.c,
 * src/body.c:84-159). */
void gislands_init( gWorld* w );
void gislands_free( gWorld* w );
void gisland_create_for_body( gWorld* w, int setIndex, gBody* b );
void gisland_remove_body( gWorld* w, gBody* b );
void gisland_link_contact( gWorld* w, gContact* c );
void gisland_unlink_contact( gWorld* w, gContact* c );
void gisland_link_joint( gWorld* w, gJoint* j );
void gisland_unlink_joint( gWorld* w, gJoint* j );
void gislands_merge_awake( gWorld* w );
void gisland_split( gWorld* w, int baseId );
void gsolver_set_wake( gWorld* w, int setIndex );
void gisland_try_sleep( gWorld* w, int islandId );
void gsolver_set_merge( gWorld* w, int setId1, int setId2 );
int gsolver_set_create( gWorld* w );
bool gbody_wake( gWorld* w, gBody* b );
void gbody_remove_from_set( gWorld* w, gBody* b );
gIntArray* gsolver_set_bodies( gWorld* w, int setIndex );
gIntArray* gsolver_set_contacts( gWorld* w, int setIndex );
gIntArray* gsolver_set_joints( gWorld* w, int setIndex );
/* Stages a device body operation (B2G_BODY_SLEEP or B2G_BODY_WAKE); the last one staged
 * for a body wins.  The host mirror follows at once. */
void gbody_stage_op( gWorld* w, int bodyId, int code );
/* The same for a body being created, whose mirror the caller writes in full. */
void gbody_stage_new( gWorld* w, int bodyId, int code );
/* Applies the staged body operations and the awake list on the device. */
int gbody_flush_ops( gWorld* w );
/* End of a step: the sleepy bodies the device reported, the split candidate and the
 * islands that fall asleep (reference src/solver.c:1956-2001). */
void gislands_sleep_step( gWorld* w );
int gassign_joint_color( gWorld* w, int bodyIdA, int bodyIdB, bool staticA, bool staticB );

/* Joints (world.c: the record shared by every type; joint.c: the per-type API). */
b2gJointDev* gjoint_create( b2WorldId worldId, b2BodyId bodyIdA, b2BodyId bodyIdB, b2JointType type, bool collideConnected,
							void* userData, b2JointId* out );
void gjoint_disconnect_bodies( gWorld* w, int bodyIdA, int bodyIdB );
void gworld_ensure_joint_mirror( gWorld* w );
void gbuffer_move( gWorld* w, int proxyKey );

b2gBox gshape_geo_aabb( const b2gShapeGeo* g, b2gXf xf );
void gbody_update_mass( gWorld* w, gBody* b );
double b2g_now_ms( void );
