/*
 * box2d/types.h -- definition structs, enums, events and statistics of the C API.
 *
 * Every struct here keeps the field order and types of the reference
 * `include/box2d/types.h` (b2WorldDef :64-113, b2BodyDef :130-190, b2ShapeDef :256-300,
 * b2Profile :397-421, b2Counters :424-438, joint defs :464-853, events :900-1010)
 * so that a caller compiled against the reference headers passes them to this library
 * unchanged.  Defaults come from b2Default*Def (reference src/types.c:8-63).
 */
#pragma once

#include "base.h"
#include "collision.h"
#include "id.h"
#include "math_functions.h"

#include <stdbool.h>
#include <stdint.h>

/* Task-system hooks (reference types.h:30-48).  Accepted and stored; the device path
 * does not call them. */
typedef void b2TaskCallback( int32_t startIndex, int32_t endIndex, uint32_t workerIndex, void* taskContext );
typedef void* b2EnqueueTaskCallback( b2TaskCallback* task, int32_t itemCount, int32_t minRange, void* taskContext,
									 void* userContext );
typedef void b2FinishTaskCallback( void* userTask, void* userContext );

typedef struct b2RayResult
{
	b2ShapeId shapeId;
	b2Vec2 point;
	b2Vec2 normal;
	float fraction;
	bool hit;
} b2RayResult;

typedef struct b2WorldDef
{
	b2Vec2 gravity;
	float restitutionThreshold;
	float contactPushoutVelocity;
	float hitEventThreshold;
	float contactHertz;
	float contactDampingRatio;
	float jointHertz;
	float jointDampingRatio;
	bool enableSleep;
	bool enableContinous;
	int32_t workerCount;
	b2EnqueueTaskCallback* enqueueTask;
	b2FinishTaskCallback* finishTask;
	void* userTaskContext;
	int32_t internalValue;
} b2WorldDef;

B2_API b2WorldDef b2DefaultWorldDef( void );

typedef enum b2BodyType
{
	b2_staticBody = 0,
	b2_kinematicBody = 1,
	b2_dynamicBody = 2,
	b2_bodyTypeCount,
} b2BodyType;

typedef struct b2BodyDef
{
	b2BodyType type;
	b2Vec2 position;
	b2Rot rotation;
	b2Vec2 linearVelocity;
	float angularVelocity;
	float linearDamping;
	float angularDamping;
	float gravityScale;
	float sleepThreshold;
	void* userData;
	bool enableSleep;
	bool isAwake;
	bool fixedRotation;
	bool isBullet;
	bool isEnabled;
	bool automaticMass;
	int32_t internalValue;
} b2BodyDef;

B2_API b2BodyDef b2DefaultBodyDef( void );

typedef struct b2Filter
{
	uint32_t categoryBits;
	uint32_t maskBits;
	int32_t groupIndex;
} b2Filter;

B2_API b2Filter b2DefaultFilter( void );

typedef struct b2QueryFilter
{
	uint32_t categoryBits;
	uint32_t maskBits;
} b2QueryFilter;

B2_API b2QueryFilter b2DefaultQueryFilter( void );

typedef enum b2ShapeType
{
	b2_circleShape,
	b2_capsuleShape,
	b2_segmentShape,
	b2_polygonShape,
	b2_smoothSegmentShape,
	b2_shapeTypeCount
} b2ShapeType;

typedef struct b2ShapeDef
{
	void* userData;
	float friction;
	float restitution;
	float density;
	b2Filter filter;
	uint32_t customColor;
	bool isSensor;
	bool enableSensorEvents;
	bool enableContactEvents;
	bool enableHitEvents;
	bool enablePreSolveEvents;
	bool forceContactCreation;
	int32_t internalValue;
} b2ShapeDef;

B2_API b2ShapeDef b2DefaultShapeDef( void );

/* Per-stage timings in milliseconds of the last step (reference types.h:397-421). */
typedef struct b2Profile
{
	float step;
	float pairs;
	float collide;
	float solve;
	float buildIslands;
	float solveConstraints;
	float prepareTasks;
	float solverTasks;
	float prepareConstraints;
	float integrateVelocities;
	float warmStart;
	float solveVelocities;
	float integratePositions;
	float relaxVelocities;
	float applyRestitution;
	float storeImpulses;
	float finalizeBodies;
	float splitIslands;
	float sleepIslands;
	float hitEvents;
	float broadphase;
	float continuous;
} b2Profile;

typedef struct b2Counters
{
	int32_t staticBodyCount;
	int32_t bodyCount;
	int32_t shapeCount;
	int32_t contactCount;
	int32_t jointCount;
	int32_t islandCount;
	int32_t stackUsed;
	int32_t staticTreeHeight;
	int32_t treeHeight;
	int32_t byteCount;
	int32_t taskCount;
	int32_t colorCounts[12];
} b2Counters;

typedef enum b2JointType
{
	b2_distanceJoint,
	b2_motorJoint,
	b2_mouseJoint,
	b2_prismaticJoint,
	b2_revoluteJoint,
	b2_weldJoint,
	b2_wheelJoint,
} b2JointType;

typedef struct b2RevoluteJointDef
{
	b2BodyId bodyIdA;
	b2BodyId bodyIdB;
	b2Vec2 localAnchorA;
	b2Vec2 localAnchorB;
	float referenceAngle;
	bool enableSpring;
	float hertz;
	float dampingRatio;
	bool enableLimit;
	float lowerAngle;
	float upperAngle;
	bool enableMotor;
	float maxMotorTorque;
	float motorSpeed;
	float drawSize;
	bool collideConnected;
	void* userData;
	int32_t internalValue;
} b2RevoluteJointDef;

B2_API b2RevoluteJointDef b2DefaultRevoluteJointDef( void );

/* Chain definition (reference types.h:364-393): at least four points; a loop connects
 * the last point to the first. */
typedef struct b2ChainDef
{
	void* userData;
	const b2Vec2* points;
	int32_t count;
	float friction;
	float restitution;
	b2Filter filter;
	bool isLoop;
	int32_t internalValue;
} b2ChainDef;

B2_API b2ChainDef b2DefaultChainDef( void );

/* Distance joint definition (reference types.h:464-517). */
typedef struct b2DistanceJointDef
{
	b2BodyId bodyIdA;
	b2BodyId bodyIdB;
	b2Vec2 localAnchorA;
	b2Vec2 localAnchorB;
	float length;
	bool enableSpring;
	float hertz;
	float dampingRatio;
	bool enableLimit;
	float minLength;
	float maxLength;
	bool enableMotor;
	float maxMotorForce;
	float motorSpeed;
	bool collideConnected;
	void* userData;
	int32_t internalValue;
} b2DistanceJointDef;

B2_API b2DistanceJointDef b2DefaultDistanceJointDef( void );

/* Motor joint definition (reference types.h:527-558). */
typedef struct b2MotorJointDef
{
	b2BodyId bodyIdA;
	b2BodyId bodyIdB;
	b2Vec2 linearOffset;
	float angularOffset;
	float maxForce;
	float maxTorque;
	float correctionFactor;
	bool collideConnected;
	void* userData;
	int32_t internalValue;
} b2MotorJointDef;

B2_API b2MotorJointDef b2DefaultMotorJointDef( void );

/* Mouse joint definition (reference types.h:569-597). */
typedef struct b2MouseJointDef
{
	b2BodyId bodyIdA;
	b2BodyId bodyIdB;
	b2Vec2 target;
	float hertz;
	float dampingRatio;
	float maxForce;
	bool collideConnected;
	void* userData;
	int32_t internalValue;
} b2MouseJointDef;

B2_API b2MouseJointDef b2DefaultMouseJointDef( void );

/* Prismatic joint definition (reference types.h:610-665). */
typedef struct b2PrismaticJointDef
{
	b2BodyId bodyIdA;
	b2BodyId bodyIdB;
	b2Vec2 localAnchorA;
	b2Vec2 localAnchorB;
	b2Vec2 localAxisA;
	float referenceAngle;
	bool enableSpring;
	float hertz;
	float dampingRatio;
	bool enableLimit;
	float lowerTranslation;
	float upperTranslation;
	bool enableMotor;
	float maxMotorForce;
	float motorSpeed;
	bool collideConnected;
	void* userData;
	int32_t internalValue;
} b2PrismaticJointDef;

B2_API b2PrismaticJointDef b2DefaultPrismaticJointDef( void );

/* Weld joint definition (reference types.h:751-788). */
typedef struct b2WeldJointDef
{
	b2BodyId bodyIdA;
	b2BodyId bodyIdB;
	b2Vec2 localAnchorA;
	b2Vec2 localAnchorB;
	float referenceAngle;
	float linearHertz;
	float angularHertz;
	float linearDampingRatio;
	float angularDampingRatio;
	bool collideConnected;
	void* userData;
	int32_t internalValue;
} b2WeldJointDef;

B2_API b2WeldJointDef b2DefaultWeldJointDef( void );

/* Wheel joint definition (reference types.h:801-853). */
typedef struct b2WheelJointDef
{
	b2BodyId bodyIdA;
	b2BodyId bodyIdB;
	b2Vec2 localAnchorA;
	b2Vec2 localAnchorB;
	b2Vec2 localAxisA;
	bool enableSpring;
	float hertz;
	float dampingRatio;
	bool enableLimit;
	float lowerTranslation;
	float upperTranslation;
	bool enableMotor;
	float maxMotorTorque;
	float motorSpeed;
	bool collideConnected;
	void* userData;
	int32_t internalValue;
} b2WheelJointDef;

B2_API b2WheelJointDef b2DefaultWheelJointDef( void );

/* Sensor overlap events (reference types.h:877-912): the sensor shape and the shape that
 * began or stopped overlapping it. */
typedef struct b2SensorBeginTouchEvent
{
	b2ShapeId sensorShapeId;
	b2ShapeId visitorShapeId;
} b2SensorBeginTouchEvent;

typedef struct b2SensorEndTouchEvent
{
	b2ShapeId sensorShapeId;
	b2ShapeId visitorShapeId;
} b2SensorEndTouchEvent;

typedef struct b2SensorEvents
{
	b2SensorBeginTouchEvent* beginEvents;
	b2SensorEndTouchEvent* endEvents;
	int32_t beginCount;
	int32_t endCount;
} b2SensorEvents;

typedef struct b2ContactBeginTouchEvent
{
	b2ShapeId shapeIdA;
	b2ShapeId shapeIdB;
} b2ContactBeginTouchEvent;

typedef struct b2ContactEndTouchEvent
{
	b2ShapeId shapeIdA;
	b2ShapeId shapeIdB;
} b2ContactEndTouchEvent;

typedef struct b2ContactHitEvent
{
	b2ShapeId shapeIdA;
	b2ShapeId shapeIdB;
	b2Vec2 point;
	b2Vec2 normal;
	float approachSpeed;
} b2ContactHitEvent;

typedef struct b2ContactEvents
{
	b2ContactBeginTouchEvent* beginEvents;
	b2ContactEndTouchEvent* endEvents;
	b2ContactHitEvent* hitEvents;
	int32_t beginCount;
	int32_t endCount;
	int32_t hitCount;
} b2ContactEvents;

typedef struct b2ContactData
{
	b2ShapeId shapeIdA;
	b2ShapeId shapeIdB;
	b2Manifold manifold;
} b2ContactData;

typedef bool b2CustomFilterFcn( b2ShapeId shapeIdA, b2ShapeId shapeIdB, void* context );
typedef bool b2PreSolveFcn( b2ShapeId shapeIdA, b2ShapeId shapeIdB, b2Manifold* manifold, void* context );
