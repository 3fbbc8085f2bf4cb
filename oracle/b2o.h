/*
 * b2o.h -- internal types of the plain-C oracle (a scalar CPU restatement of the
 * reference's per-step contact pipeline).
 *
 * TEST INFRASTRUCTURE ONLY: tests/, the smoke check and the benchmark's CPU-baseline leg
 * load this code as the checker; the GPU library never links it.  It restates the
 * reference algorithms (cited per function in the .c files) with its own data layout:
 * body, shape, contact and joint records are indexed by their stable ids, and the
 * reference's moving arrays (constraint-graph colours, the non-touching contact array,
 * the awake body set) are kept as arrays of ids with the same swap-remove order, because
 * that order fixes contact ids, colours and the overflow solve order.
 */
#pragma once

#include "b2o_math.h"

#include "box2d/box2d.h"

#include <stdlib.h>

/* ---------------------------------------------------------------- small containers */
typedef struct oIntArray
{
	int* data;
	int count;
	int capacity;
} oIntArray;

void oia_push( oIntArray* a, int v );
int oia_remove_swap( oIntArray* a, int index ); /* returns the moved index or -1 */
void oia_free( oIntArray* a );

/* Open-addressing set of non-zero 64-bit keys (membership only; its iteration order is
 * never observed, as in the reference src/table.c). */
typedef struct oSet
{
	uint64_t* keys;
	int capacity;
	int count;
} oSet;

bool oset_add( oSet* s, uint64_t key ); /* returns true if it was already present */
bool oset_remove( oSet* s, uint64_t key );
bool oset_contains( const oSet* s, uint64_t key );
void oset_clear( oSet* s );
void oset_free( oSet* s );

/* LIFO id pool (reference src/id_pool.c:21-45; a freed id is always pushed). */
typedef struct oIdPool
{
	oIntArray freeIds;
	int next;
} oIdPool;

int oid_alloc( oIdPool* p );
void oid_free( oIdPool* p, int id );
int oid_count( const oIdPool* p );

/* Threads of the oracle's independent loops (the rows of one colour, bodies, contacts of
 * the narrowphase), set by b2o_SetThreads; 1, the default, runs everything on the
 * calling thread.  The loops' iterations touch disjoint data, so any count gives the
 * same bits.  Loops shorter than O_PARALLEL_MIN stay serial. */
extern int o_threads;
#define O_PARALLEL_MIN 64

typedef struct oBits
{
	uint64_t* words;
	int wordCount;
} oBits;

bool obits_get( const oBits* b, int i );
void obits_set( oBits* b, int i ); /* grows */
void obits_clear( oBits* b, int i );
void obits_free( oBits* b );

/* ---------------------------------------------------------------- dynamic tree */
typedef struct oNode
{
	oBox box;
	uint32_t category;
	int parent; /* also the free-list link */
	int child1, child2;
	int userData;
	int16_t height; /* 0 leaf, -1 free */
	bool enlarged;
} oNode;

typedef struct oTree
{
	oNode* nodes;
	int root;
	int nodeCount;
	int capacity;
	int freeList;
	int proxyCount;
	int* leafIndices;
	oVec* leafCenters;
	int rebuildCapacity;
} oTree;

void otree_init( oTree* t );
void otree_free( oTree* t );
int otree_create_proxy( oTree* t, oBox box, uint32_t category, int userData );
void otree_destroy_proxy( oTree* t, int proxyId );
void otree_move_proxy( oTree* t, int proxyId, oBox box );
void otree_enlarge_proxy( oTree* t, int proxyId, oBox box );
void otree_rebuild( oTree* t );
int otree_height( const oTree* t );
typedef bool oQueryFcn( int proxyId, int userData, void* ctx );
void otree_query( const oTree* t, oBox box, uint32_t mask, oQueryFcn* fcn, void* ctx );

/* ---------------------------------------------------------------- geometry */
typedef struct oPolygon
{
	oVec v[8];
	oVec n[8];
	oVec centroid;
	b2r radius;
	int count;
} oPolygon;

typedef struct oCircle
{
	oVec center;
	b2r radius;
} oCircle;

typedef struct oCapsule
{
	oVec c1, c2;
	b2r radius;
} oCapsule;

typedef struct oSegment
{
	oVec p1, p2;
} oSegment;

/* Chain link (reference b2SmoothSegment, include/box2d/collision.h:159-172). */
typedef struct oSmooth
{
	oVec ghost1, p1, p2, ghost2;
	int chainId;
} oSmooth;

typedef struct oMPoint
{
	oVec point, anchorA, anchorB;
	b2r separation, normalImpulse, tangentImpulse, maxNormalImpulse, normalVelocity;
	uint16_t id;
	bool persisted;
} oMPoint;

typedef struct oManifold
{
	oMPoint pts[2];
	oVec normal;
	int count;
} oManifold;

oManifold o_collide_circles( const oCircle* a, oXf xfA, const oCircle* b, oXf xfB );
oManifold o_collide_capsule_circle( const oCapsule* a, oXf xfA, const oCircle* b, oXf xfB );
oManifold o_collide_polygon_circle( const oPolygon* a, oXf xfA, const oCircle* b, oXf xfB );
oManifold o_collide_polygons( const oPolygon* a, oXf xfA, const oPolygon* b, oXf xfB );
oPolygon o_make_capsule( oVec p1, oVec p2, b2r radius );

typedef struct oSegDist
{
	oVec c1, c2;
	b2r f1, f2, dist2;
} oSegDist;
oSegDist o_segment_distance( oVec p1, oVec q1, oVec p2, oVec q2 );

/* Closest-feature cache of the GJK distance (reference include/box2d/collision.h
 * b2DistanceCache); kept per contact for the sensor overlap test. */
typedef struct oDistCache
{
	int count;
	int indexA[3], indexB[3];
} oDistCache;

oManifold o_collide_smooth_circle( const oSmooth* a, oXf xfA, const oCircle* b, oXf xfB );
oManifold o_collide_smooth_polygon( const oSmooth* a, oXf xfA, const oPolygon* b, oXf xfB, oDistCache* cache );

/* ---------------------------------------------------------------- world records */
typedef struct oShape
{
	int id; /* -1 when free */
	int bodyId;
	int prev, next;
	b2ShapeType type;
	b2r density, friction, restitution;
	oBox aabb, fatAABB;
	oVec localCentroid;
	int proxyKey;
	b2Filter filter;
	void* userData;
	union
	{
		oPolygon polygon;
		oCircle circle;
		oCapsule capsule;
		oSegment segment;
		oSmooth smooth;
	};
	uint16_t revision;
	bool isSensor, enableContactEvents, enableSensorEvents, enableHitEvents, enablePreSolveEvents;
	bool enlargedAABB, isFast;
} oShape;

typedef struct oBody
{
	int id; /* -1 when free */
	b2BodyType type;
	int awakeIndex; /* position in the awake list, -1 for static */
	int headShape, shapeCount;
	int headContactKey, contactCount;
	int headJointKey, jointCount;
	int headChainId;
	void* userData;
	uint16_t revision;
	bool fixedRotation, isBullet, enableSleep, isSpeedCapped, automaticMass;
	b2r sleepThreshold, sleepTime;
	int setIndex;	/* solver set (O_SET_*); sleeping sets from O_SET_FIRST_SLEEPING */
	int setLocal;	/* position in a non-awake set's body list */
	int islandId, islandPrev, islandNext;
	bool isMarked;

	/* simulation record (reference src/body.h:95-133) */
	oXf xf;
	oVec center, center0, localCenter, force;
	oRot rot0;
	b2r torque, mass, invMass, inertia, invI, minExtent, maxExtent;
	b2r linearDamping, angularDamping, gravityScale;
	bool isFast, simSpeedCapped, enlargeAABB;

	/* solver record (reference src/body.h:76-91) */
	oVec v, dp;
	b2r w;
	oRot dq;
} oBody;

enum
{
	OC_TOUCHING = 1,
	OC_SENSOR = 4,
	OC_ENABLE_SENSOR_EVENTS = 0x10,
	OC_ENABLE_CONTACT_EVENTS = 0x20,
	OC_SENSOR_TOUCHING = 0x40,

	OS_TOUCHING = 0x10000,
	OS_DISJOINT = 0x20000,
	OS_STARTED = 0x40000,
	OS_STOPPED = 0x80000,
	OS_HIT = 0x100000,
};

typedef struct oEdge
{
	int bodyId, prevKey, nextKey;
} oEdge;

typedef struct oContact
{
	int id; /* -1 when free */
	int setIndex; /* awake, disabled (non-touching, both bodies asleep) or a sleeping set */
	int colorIndex, localIndex;
	int islandId, islandPrev, islandNext;
	bool isMarked;
	oEdge edges[2];
	int shapeIdA, shapeIdB;
	uint32_t flags;

	/* simulation record (reference src/contact.h:107-141) */
	int simIndexA, simIndexB; /* body ids of awake bodies, -1 for static */
	b2r invMassA, invIA, invMassB, invIB;
	oManifold manifold;
	b2r friction, restitution;
	uint32_t simFlags;
	oDistCache cache; /* sensor overlap test (reference src/contact.h:136) */
} oContact;

/* A chain of smooth segments (reference src/shape.h:52-60). */
typedef struct oChain
{
	int id; /* -1 when free */
	int bodyId;
	int nextChainId;
	int* shapeIndices;
	int count;
	uint16_t revision;
} oChain;

typedef struct oSoft
{
	b2r biasRate, massScale, impulseScale;
} oSoft;

typedef struct oMat22
{
	oVec cx, cy;
} oMat22;

/* Per-type joint records (reference src/joint.h:56-234). */
typedef struct oDistanceJoint
{
	b2r length, hertz, dampingRatio, minLength, maxLength, maxMotorForce, motorSpeed;
	b2r impulse, lowerImpulse, upperImpulse, motorImpulse;
	oVec anchorA, anchorB, deltaCenter;
	oSoft distanceSoftness;
	b2r axialMass;
	bool enableSpring, enableLimit, enableMotor;
} oDistanceJoint;

typedef struct oMotorJoint
{
	oVec linearOffset;
	b2r angularOffset;
	oVec linearImpulse;
	b2r angularImpulse, maxForce, maxTorque, correctionFactor;
	oVec anchorA, anchorB, deltaCenter;
	b2r deltaAngle;
	oMat22 linearMass;
	b2r angularMass;
} oMotorJoint;

typedef struct oMouseJoint
{
	oVec targetA;
	b2r hertz, dampingRatio, maxForce;
	oVec linearImpulse;
	b2r angularImpulse;
	oSoft linearSoftness, angularSoftness;
	oVec anchorB, deltaCenter;
	oMat22 linearMass;
} oMouseJoint;

typedef struct oPrismaticJoint
{
	oVec localAxisA, impulse;
	b2r springImpulse, motorImpulse, lowerImpulse, upperImpulse;
	b2r hertz, dampingRatio, maxMotorForce, motorSpeed, referenceAngle, lowerTranslation, upperTranslation;
	oVec anchorA, anchorB, axisA, deltaCenter;
	b2r deltaAngle, axialMass;
	oSoft springSoftness;
	bool enableSpring, enableLimit, enableMotor;
} oPrismaticJoint;

typedef struct oRevoluteJoint
{
	oVec linearImpulse;
	b2r springImpulse, motorImpulse, lowerImpulse, upperImpulse;
	b2r hertz, dampingRatio, maxMotorTorque, motorSpeed, referenceAngle, lowerAngle, upperAngle;
	oVec anchorA, anchorB, deltaCenter;
	b2r deltaAngle, axialMass;
	oSoft springSoftness;
	bool enableSpring, enableMotor, enableLimit;
} oRevoluteJoint;

typedef struct oWeldJoint
{
	b2r referenceAngle, linearHertz, linearDampingRatio, angularHertz, angularDampingRatio;
	oSoft linearSoftness, angularSoftness;
	oVec linearImpulse;
	b2r angularImpulse;
	oVec anchorA, anchorB, deltaCenter;
	b2r deltaAngle, axialMass;
} oWeldJoint;

typedef struct oWheelJoint
{
	oVec localAxisA;
	b2r perpImpulse, motorImpulse, springImpulse, lowerImpulse, upperImpulse;
	b2r maxMotorTorque, motorSpeed, lowerTranslation, upperTranslation, hertz, dampingRatio;
	oVec anchorA, anchorB, axisA, deltaCenter;
	b2r perpMass, motorMass, axialMass;
	oSoft springSoftness;
	bool enableSpring, enableMotor, enableLimit;
} oWheelJoint;

typedef struct oJoint
{
	int id;
	b2JointType type;
	int bodyIdA, bodyIdB;
	oEdge edges[2];
	int setIndex;
	int colorIndex, localIndex;
	int islandId, islandPrev, islandNext;
	bool isMarked;
	oVec localAnchorA, localAnchorB; /* reference localOriginAnchorA/B */
	b2r invMassA, invMassB, invIA, invIB;
	int indexA, indexB; /* awake body ids, -1 for a body that is not awake */
	union
	{
		oDistanceJoint distance;
		oMotorJoint motor;
		oMouseJoint mouse;
		oPrismaticJoint prismatic;
		oRevoluteJoint revolute;
		oWeldJoint weld;
		oWheelJoint wheel;
	};
	bool collideConnected;
	uint16_t revision;
	void* userData;
} oJoint;

typedef struct oColor
{
	oBits bodySet;
	oIntArray contacts; /* contact ids in colour array order */
	oIntArray joints;
} oColor;

/* Per-constraint solver data (overflow path: reference src/contact_solver.h:11-35; the
 * coloured path keeps the same fields per lane of the 8-wide record). */
typedef struct oCPoint
{
	oVec anchorA, anchorB;
	b2r baseSeparation, relativeVelocity, normalImpulse, tangentImpulse, maxNormalImpulse, normalMass, tangentMass;
} oCPoint;

typedef struct oConstraint
{
	int contactId;
	int indexA, indexB;
	oCPoint pts[2];
	oVec normal;
	b2r invMassA, invMassB, invIA, invIB, friction, restitution;
	oSoft soft;
	int pointCount;
} oConstraint;

/* Solver sets (reference src/solver_set.h): static, disabled, awake, then sleeping sets. */
enum
{
	O_SET_STATIC = 0,
	O_SET_DISABLED = 1,
	O_SET_AWAKE = 2,
	O_SET_FIRST_SLEEPING = 3,
};

/* A persistent island: bodies, contacts and joints linked through the records
 * (reference src/island.h:32-56). */
typedef struct oIsland
{
	int setIndex, localIndex, islandId;
	int headBody, tailBody, bodyCount;
	int headContact, tailContact, contactCount;
	int headJoint, tailJoint, jointCount;
	int parentIsland;
	int constraintRemoveCount;
} oIsland;

/* A sleeping set's members in set order (the awake set's are the awake lists). */
typedef struct oSolverSet
{
	int setIndex; /* -1 when free */
	oIntArray bodies, contacts, joints, islands;
} oSolverSet;

typedef struct oWorld
{
	bool inUse;
	uint16_t revision;
	int slot;

	oIdPool bodyIds, shapeIds, contactIds, jointIds, chainIds;
	oBody* bodies;
	int bodyCap;
	oShape* shapes;
	int shapeCap;
	oContact* contacts;
	int contactCap;
	oJoint* joints;
	int jointCap;
	struct oChain* chains;
	int chainCap;

	oIntArray awake;		 /* awake body ids in solver order */
	oIntArray staticBodies;	 /* static body ids */
	oIntArray nonTouching;	 /* awake non-touching contact ids */
	oIntArray disabledContacts; /* non-touching contacts whose bodies both sleep */
	oIntArray awakeIslands;	 /* awake island ids in set order */
	oIsland* islands;
	int islandCap;
	oIdPool islandIds;
	oSolverSet* sets; /* indexed by set id; entries below O_SET_FIRST_SLEEPING unused */
	int setCap;
	oIdPool setIds;
	int splitIslandId;
	oColor colors[O_COLORS];

	oTree trees[3];
	oIntArray moveArray;
	oSet moveSet;
	oSet pairSet;

	oVec gravity;
	b2r restitutionThreshold, pushout, hitThreshold, contactHertz, contactDamping, jointHertz, jointDamping;
	bool enableSleep, enableWarmStarting, enableContinuous, locked;

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

	b2Profile profile;
	uint64_t stepIndex;
	b2r inv_h;
	int toiEvents; /* time-of-impact events (fast bodies moved back along their sweep) */
} oWorld;

oWorld* o_world( b2WorldId id );
oWorld* o_world_index( int index );
void o_step( oWorld* w, b2r dt, int subSteps );
void o_update_pairs( oWorld* w );
void o_collide( oWorld* w );
void o_solve( oWorld* w, b2r dt, int subSteps );
void o_create_contact( oWorld* w, oShape* a, oShape* b );
void o_destroy_contact( oWorld* w, oContact* c, bool wakeBodies );
void o_add_contact_to_graph( oWorld* w, oContact* c );
void o_remove_contact_from_graph( oWorld* w, int bodyIdA, int bodyIdB, int colorIndex, int localIndex );
int o_assign_joint_color( oWorld* w, int bodyIdA, int bodyIdB, bool staticA, bool staticB );

oBox o_shape_aabb( const oShape* s, oXf xf );
void o_update_body_mass( oWorld* w, oBody* b );
oSoft o_make_soft( b2r hertz, b2r zeta, b2r h );
bool o_should_bodies_collide( oWorld* w, oBody* a, oBody* b );
void o_report_hits( oWorld* w );

/* Step constants (reference b2StepContext, src/solver.h:76-140). */
typedef struct oStep
{
	b2r dt, inv_dt, h, inv_h;
	int subSteps;
	oSoft contactSoft, staticSoft, jointSoft;
	b2r restitutionThreshold, pushout;
	bool enableWarmStarting;
} oStep;

/* Solver view of one body (reference b2BodyState, src/body.h:76-91); the identity state
 * stands in for a static body. */
typedef struct oState
{
	oVec v;
	b2r w;
	oVec dp;
	oRot dq;
} oState;

/* Joints of every type (b2o_joint.c; reference src/joint.c:983-1108 and the per-type
 * prepare, warm start and solve functions). */
void o_prepare_joint( oWorld* w, const oStep* st, oJoint* j );

/* Islands and sleep (b2o_island.c; reference src/island.c, src/solver_set.c). */
void o_islands_init( oWorld* w );
void o_islands_free( oWorld* w );
void o_create_island_for_body( oWorld* w, int setIndex, oBody* b );
void o_remove_body_from_island( oWorld* w, oBody* b );
void o_remove_body_from_set( oWorld* w, oBody* b );
void o_link_contact( oWorld* w, oContact* c );
void o_unlink_contact( oWorld* w, oContact* c );
void o_link_joint( oWorld* w, oJoint* j );
void o_unlink_joint( oWorld* w, oJoint* j );
void o_merge_awake_islands( oWorld* w );
void o_split_island( oWorld* w, int baseId );
void o_wake_solver_set( oWorld* w, int setIndex );
void o_try_sleep_island( oWorld* w, int islandId );
void o_merge_solver_sets( oWorld* w, int setId1, int setId2 );
int o_create_sleeping_set( oWorld* w );
bool o_wake_body( oWorld* w, oBody* b );
oIntArray* o_set_bodies( oWorld* w, int setIndex );
oIntArray* o_set_contacts( oWorld* w, int setIndex );
oIntArray* o_set_joints( oWorld* w, int setIndex );
oJoint* o_create_joint( b2WorldId worldId, b2BodyId bodyIdA, b2BodyId bodyIdB, b2JointType type, bool collideConnected,
						void* userData, b2JointId* out );
void o_destroy_contacts_between( oWorld* w, int bodyIdA, int bodyIdB );
void o_buffer_move( oWorld* w, int proxyKey );
void o_warm_start_joint( oJoint* j, oState* a, oState* b );
void o_solve_joint( oJoint* j, const oStep* st, oState* a, oState* b, bool useBias );

/* ---------------------------------------------------------------- time of impact
 * (b2o_toi.c; reference src/distance.c, src/shape.c:480-497, :713-735) */
typedef struct oSweep
{
	oVec localCenter, c1, c2;
	oRot q1, q2;
} oSweep;

typedef struct oProxy
{
	oVec pts[8];
	int count;
	b2r radius;
} oProxy;

oXf o_sweep_xf( const oSweep* s, b2r t );
oProxy o_make_proxy( const oVec* points, int count, b2r radius );
oProxy o_shape_proxy( const oShape* s );
oVec o_shape_centroid( const oShape* s );
b2r o_distance( oDistCache* cache, const oProxy* A, oXf xfA, const oProxy* B, oXf xfB, oVec* pointA, oVec* pointB );
b2r o_time_of_impact( const oProxy* A, const oSweep* sA, const oProxy* B, const oSweep* sB, b2r tMax, int* state );

oVec ovf( b2Vec2 v );
b2Vec2 vfo( oVec v );
