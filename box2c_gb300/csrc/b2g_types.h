/*
 * b2g_types.h -- data layout shared by the host C code and the sm_103a kernels.
 *
 * Device memory of one world ("arena") holds structure-of-arrays records indexed by the
 * stable ids of the C API:
 *   bodies   : solver state (2 x float4: v.x v.y w flags | dp.x dp.y dq.c dq.s, the
 *              32-byte b2BodyState of reference src/body.h:76-91), transform, centre,
 *              previous pose, mass, force, damping/extent (float4 each)
 *   shapes   : geometry (160 B), tight and fat AABB (float4 each)
 *   contacts : shape pair, mixed friction/restitution, flags, manifold (112 B)
 *   solver   : per-step constraint rows in colour-major order (see kernels.cu)
 * The host keeps pinned mirrors of the body arrays with the same layout, so setup data
 * and read-back move with single contiguous copies.
 */
#pragma once

#include "b2g_math.h"

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Dynamic-tree node (reference include/box2d/collision.h:600-635 b2TreeNode fields the
 * path uses): fat box, category bits, links, shape id of a leaf, height (0 for leaves).
 * The host trees use this layout, so a tree is copied to the device as it is. */
typedef struct b2gTreeNode
{
	b2gBox box;
	uint32_t category;
	int32_t parent;
	int32_t child1, child2;
	int32_t userData;
	int16_t height;
	bool enlarged;
} b2gTreeNode;

/* Shape geometry record (160 bytes).  Polygons use v/n/centroid/count/radius; circles
 * v[0] and radius; capsules v[0], v[1] and radius; segments v[0], v[1]. */
typedef struct b2gShapeGeo
{
	int32_t type;
	int32_t count;
	float radius;
	int32_t bodyId;
	b2gVec v[8];
	b2gVec n[8];
	b2gVec centroid;
	int32_t enableHitEvents;
	int32_t isSensor;
} b2gShapeGeo;

typedef struct b2gPoint
{
	b2gVec point, anchorA, anchorB;
	float separation, normalImpulse, tangentImpulse, maxNormalImpulse, normalVelocity;
	uint16_t id;
	uint8_t persisted;
	uint8_t pad;
} b2gPoint;

/* Contact manifold (108 bytes): the layout of the public b2Manifold
 * (include/box2d/collision.h, reference include/box2d/collision.h:474-520), so device
 * manifolds can be handed to callers as b2Manifold arrays. */
typedef struct b2gManifold
{
	b2gPoint pts[2];
	b2gVec normal;
	int32_t count;
} b2gManifold;

/* Contact flags kept on the device (reference src/contact.h:85-104). */
enum
{
	B2G_C_LIVE = 0x1,
	B2G_C_ASLEEP = 0x2, /* outside the awake set: skipped by the narrowphase */
	B2G_C_TOUCHING = 0x10000,
	B2G_C_HIT = 0x100000,
};

/* Narrowphase event codes, packed as (contactId << 2) | code. */
enum
{
	B2G_EV_DISJOINT = 1,
	B2G_EV_STARTED = 2,
	B2G_EV_STOPPED = 3,
};

/* Body info bits (bodyInfo array). */
enum
{
	B2G_B_TYPE_MASK = 0x3,
	B2G_B_AWAKE = 0x4,
	B2G_B_BULLET = 0x8,
	B2G_B_SLEEP_OK = 0x10,
};

/* Staged contact record: a contact created by the host broadphase (flags 0, or
 * B2G_INIT_ASLEEP when it starts outside the awake set), the retirement of a destroyed
 * contact id (flags B2G_INIT_KILL), or a move of a live contact into or out of the awake
 * set (B2G_INIT_SET, with B2G_INIT_ASLEEP when it leaves it). */
#define B2G_INIT_KILL 0x80000000u
#define B2G_INIT_SET 0x40000000u
#define B2G_INIT_ASLEEP 0x20000000u

/* Seconds a body must stay below its sleep velocity before its island may sleep
 * (reference src/core.h b2_timeToSleep). */
#define B2G_TIME_TO_SLEEP 0.5f

/* Body operations staged by the host, applied on the device before the next kernel that
 * reads the body: (bodyId << 2) | code. */
enum
{
	B2G_BODY_SLEEP = 0, /* leaves the awake set */
	B2G_BODY_WAKE = 1,	/* joins the awake set with zero velocity and a zero sleep timer */
};

typedef struct b2gContactInit
{
	int32_t id;
	int32_t shapeA;
	int32_t shapeB;
	float friction;
	float restitution;
	uint32_t flags;
} b2gContactInit;

/* Finalisation record for a shape whose broadphase proxy needs host attention. */
enum
{
	B2G_R_ENLARGED = 0x1,	   /* non-fast shape with a grown fat box */
	B2G_R_FAST = 0x2,		   /* shape of a fast body: moved to the move buffer */
	B2G_R_FAST_ENLARGED = 0x4, /* fast shape whose fat box grew after the sweep */
	B2G_R_BULLET = 0x8,
};

typedef struct b2gRecord
{
	int32_t awakeIndex;
	int32_t slot; /* position of the shape in its body's shape list */
	int32_t shapeId;
	int32_t flags;
	float fat[4];
	float sweep[4]; /* swept box of a fast shape (union of old and new boxes) */
	/* fast shapes only: the body's sweep, start (centre0, rotation0) and end (centre,
	 * rotation) of the step, for continuous collision on the host */
	float pose1[4];
	float pose2[4];
} b2gRecord;

/* Joint types, numbered as the reference's b2JointType (include/box2d/types.h:446-455). */
enum
{
	B2G_J_DISTANCE = 0,
	B2G_J_MOTOR = 1,
	B2G_J_MOUSE = 2,
	B2G_J_PRISMATIC = 3,
	B2G_J_REVOLUTE = 4,
	B2G_J_WELD = 5,
	B2G_J_WHEEL = 6,
};

/* One joint of any type: configuration (host-owned) and solver state (device-owned).
 * The reference keeps a union of per-type structs (src/joint.h:56-263); this record is
 * their union by meaning, one field per quantity, so every type is one 256-byte record
 * and one code path loads it.  Fields a type does not use stay zero. */
typedef struct b2gJointDev
{
	int32_t bodyIdA, bodyIdB;
	int32_t indexA, indexB; /* awake body ids, -1 for a body that is not awake */
	int32_t type;			/* b2JointType */
	int32_t enableSpring, enableMotor, enableLimit;
	b2gVec localAnchorA, localAnchorB;
	b2gVec localAxisA; /* prismatic, wheel: unit axis in body A's frame */
	b2gVec target;	   /* mouse: target point (targetA); motor: linear offset */
	float hertz, dampingRatio; /* spring (revolute, prismatic, wheel, distance); linear softness (weld, mouse) */
	float angularHertz, angularDampingRatio; /* weld */
	float maxMotor;		  /* revolute, wheel: max motor torque; prismatic, distance: max motor force; motor, mouse: max force */
	float maxTorque;	  /* motor joint */
	float motorSpeed;
	float referenceAngle; /* revolute, prismatic, weld; motor joint: angular offset */
	float lower, upper;	  /* limits: angles (revolute), translations (prismatic, wheel), lengths (distance) */
	float length;		  /* distance */
	float correctionFactor; /* motor joint */

	/* solver state */
	float invMassA, invMassB, invIA, invIB;
	b2gVec linearImpulse; /* point constraint (revolute, weld, motor, mouse); prismatic: (perpendicular, angular) */
	float impulse;		  /* distance: spring or rigid impulse */
	float perpImpulse;	  /* wheel: point-to-line impulse */
	float angularImpulse; /* weld, motor, mouse */
	float springImpulse, motorImpulse, lowerImpulse, upperImpulse;
	b2gVec anchorA, anchorB, deltaCenter, axisA;
	float deltaAngle;
	float axialMass; /* motor joint: its angular mass */
	float perpMass, motorMass; /* wheel */
	float linearMass[4]; /* motor, mouse: inverse of K as cx.x cx.y cy.x cy.y */
	float springSoft[3]; /* biasRate massScale impulseScale: spring; weld and mouse: linear softness */
	float angularSoft[3]; /* weld, mouse */
	int32_t pad;
} b2gJointDev;

/* Step constants (reference b2StepContext, src/solver.h:76-140). */
typedef struct b2gStepConst
{
	float dt, inv_dt, h, inv_h;
	int32_t subSteps;
	float contactSoft[3]; /* biasRate, massScale, impulseScale */
	float staticSoft[3];
	float jointSoft[3];
	float restitutionThreshold, pushout;
	b2gVec gravity;
	int32_t enableWarmStarting, enableContinuous, enableSleep;
} b2gStepConst;

/* Device arena of one world: raw device pointers and capacities. */
/* float4 arrays of one constraint row: indices, normal/friction/restitution, masses,
 * two anchor pairs, two coefficient sets, two impulse sets (144 bytes) */
#define B2G_ROW_FLOAT4 9

typedef struct b2gDevWorld
{
	int bodyCap, shapeCap, contactCap, jointCap, solveCap, listCap;

	/* bodies, indexed by body id */
	void* state;   /* float4[2*bodyCap] */
	void* xf;	   /* float4: p.x p.y q.c q.s */
	void* centers; /* float4: center.x center.y localCenter.x localCenter.y */
	void* prev;	   /* float4: center0.x center0.y rot0.c rot0.s */
	void* mass;	   /* float4: mass invMass inertia invI */
	void* force;   /* float4: force.x force.y torque gravityScale */
	void* extent;  /* float4: linearDamping angularDamping minExtent maxExtent */
	int* bodyInfo;
	float* sleepTime; /* seconds below the sleep velocity, by body id (null until the world steps with sleep on) */
	int* bodyOps;	  /* staged body operations ((bodyId << 2) | B2G_BODY_*), one per body at most */
	int bodyOpsCap;
	int* awake;		 /* awake body ids in solver order */
	int* shapeRange; /* 2 per body: start, count into shapeList */
	int* shapeList;

	/* shapes, indexed by shape id */
	b2gShapeGeo* geo;
	void* aabb; /* float4 */
	void* fat;	/* float4 */

	/* contacts, indexed by contact id */
	int* cShapes;	/* 2 per contact */
	float* cMix;	/* friction, restitution */
	uint32_t* cFlags;
	uint32_t* cCache; /* sensor contacts: the GJK closest-feature cache, packed */
	int* cBodies; /* 2 per contact: awake body id or -1 */
	b2gManifold* manifold;

	/* colour-major solve lists */
	int* solveList; /* contact ids */
	int* jointList; /* joint ids */

	/* constraint rows (B2G_ROW_FLOAT4 arrays; the softness follows from whether a body
	 * is static and is not stored) */
	void* kIdx;	 /* int4: indexA indexB contactId pointCount */
	void* kNF;	 /* float4: normal.x normal.y friction restitution */
	void* kMass; /* float4: mA iA mB iB */
	void* kAnchor[2];
	void* kCoef[2]; /* baseSeparation normalMass tangentMass relativeVelocity */
	void* kImp[2];	/* normalImpulse tangentImpulse maxNormalImpulse 0 */

	b2gJointDev* joints;

	/* staging and outputs */
	b2gContactInit* newContacts;
	int newCap;
	int* counters;	   /* device: [0] events, [1] records, [2] status, [3] sleepy bodies */
	int* events;	   /* device view of the mapped event buffer */
	b2gRecord* records; /* device view of the mapped record buffer */
	int* sleepy;	   /* device view of the mapped sleepy-body buffer: 2 ints per body (awake index, sleep time bits) */
	int eventCap, recordCap, sleepyCap;
	void* stream; /* cudaStream_t */
	void* timers[8]; /* cudaEvent_t: step start, collide start/end, solve start/end, finalize end, step end */
	int timing;
	int launches;
	long long h2dBytes, d2hBytes; /* host <-> device bytes of the current step */
	int fused;	   /* use the fused cluster solver when the world fits on chip */
	int fusedUsed; /* the last step's solver stage ran fused */
	/* set for a solver stage launched before the host has seen the narrowphase's events:
	 * its kernels return at once when the narrowphase reported any (counters[0] != 0) */
	int guardEvents;
	void* stage;   /* fused solver: per-CTA shared-memory images */
	size_t stageBytes;
} b2gDevWorld;

#ifdef __cplusplus
}
#endif
