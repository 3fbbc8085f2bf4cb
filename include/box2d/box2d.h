/*
 * box2d/box2d.h -- the world / body / shape / joint C API served by the GB300 backend.
 *
 * Each declaration has the signature of the same-named function in the reference
 * `include/box2d/box2d.h` (line numbers cited per group).  A C program written against
 * the reference links this library instead and keeps its source unchanged for the
 * functions below.  b2World_Step runs the per-step contact pipeline (broadphase pairs,
 * narrowphase manifolds, graph colouring, soft-step solver) on the GPU.
 *
 * Error convention (reference core.h:80-91): invalid input trips B2_ASSERT through the
 * b2SetAssertFcn hook; create functions return a null id on failure.  Device failures
 * never abort the process: they are reported by b2World_GetStatus (box2d/gpu.h).
 */
#pragma once

#include "base.h"
#include "collision.h"
#include "id.h"
#include "types.h"

/* World (reference box2d.h:27-160) */
B2_API b2WorldId b2CreateWorld( const b2WorldDef* def );
B2_API void b2DestroyWorld( b2WorldId worldId );
B2_API bool b2World_IsValid( b2WorldId id );
B2_API void b2World_Step( b2WorldId worldId, float timeStep, int subStepCount );
/* Events of the last step (reference box2d.h:48, :51): contact begin/end touch and hit
 * events, sensor begin/end overlap events; valid until the next step. */
B2_API b2SensorEvents b2World_GetSensorEvents( b2WorldId worldId );
B2_API b2ContactEvents b2World_GetContactEvents( b2WorldId worldId );
B2_API void b2World_EnableSleeping( b2WorldId worldId, bool flag );
B2_API void b2World_EnableContinuous( b2WorldId worldId, bool flag );
B2_API void b2World_SetRestitutionThreshold( b2WorldId worldId, float value );
B2_API void b2World_SetHitEventThreshold( b2WorldId worldId, float value );
B2_API void b2World_SetGravity( b2WorldId worldId, b2Vec2 gravity );
B2_API b2Vec2 b2World_GetGravity( b2WorldId worldId );
B2_API void b2World_SetContactTuning( b2WorldId worldId, float hertz, float dampingRatio, float pushVelocity );
B2_API void b2World_EnableWarmStarting( b2WorldId worldId, bool flag );
B2_API b2Profile b2World_GetProfile( b2WorldId worldId );
B2_API b2Counters b2World_GetCounters( b2WorldId worldId );

/* Body (reference box2d.h:175-405) */
B2_API b2BodyId b2CreateBody( b2WorldId worldId, const b2BodyDef* def );
/* Destroys a body with its shapes, contacts and joints (reference box2d.h:179).  The
 * last awake body takes the destroyed one's place in the awake order, as in the
 * reference, so the following steps stay bit-identical to it. */
B2_API void b2DestroyBody( b2BodyId bodyId );
B2_API bool b2Body_IsValid( b2BodyId id );
B2_API b2BodyType b2Body_GetType( b2BodyId bodyId );
B2_API void b2Body_SetUserData( b2BodyId bodyId, void* userData );
B2_API void* b2Body_GetUserData( b2BodyId bodyId );
B2_API b2Vec2 b2Body_GetPosition( b2BodyId bodyId );
B2_API b2Rot b2Body_GetRotation( b2BodyId bodyId );
B2_API b2Transform b2Body_GetTransform( b2BodyId bodyId );
B2_API b2Vec2 b2Body_GetLocalPoint( b2BodyId bodyId, b2Vec2 worldPoint );
B2_API b2Vec2 b2Body_GetWorldPoint( b2BodyId bodyId, b2Vec2 localPoint );
B2_API b2Vec2 b2Body_GetLinearVelocity( b2BodyId bodyId );
B2_API float b2Body_GetAngularVelocity( b2BodyId bodyId );
B2_API void b2Body_SetLinearVelocity( b2BodyId bodyId, b2Vec2 linearVelocity );
B2_API void b2Body_SetAngularVelocity( b2BodyId bodyId, float angularVelocity );
B2_API float b2Body_GetMass( b2BodyId bodyId );
B2_API float b2Body_GetInertiaTensor( b2BodyId bodyId );
B2_API b2Vec2 b2Body_GetLocalCenterOfMass( b2BodyId bodyId );
B2_API b2Vec2 b2Body_GetWorldCenterOfMass( b2BodyId bodyId );
B2_API float b2Body_GetLinearDamping( b2BodyId bodyId );
B2_API float b2Body_GetAngularDamping( b2BodyId bodyId );
B2_API float b2Body_GetGravityScale( b2BodyId bodyId );
B2_API int b2Body_GetShapeCount( b2BodyId bodyId );
B2_API int b2Body_GetShapes( b2BodyId bodyId, b2ShapeId* shapeArray, int capacity );
B2_API int b2Body_GetJointCount( b2BodyId bodyId );
B2_API int b2Body_GetContactCapacity( b2BodyId bodyId );
B2_API int b2Body_GetContactData( b2BodyId bodyId, b2ContactData* contactData, int capacity );
/* Sleep (reference box2d.h:342-359).  A body sleeps with its whole island: SetAwake(false)
 * splits the island first when constraints were removed from it, and a body that is not
 * awake reports zero velocity. */
B2_API bool b2Body_IsAwake( b2BodyId bodyId );
B2_API void b2Body_SetAwake( b2BodyId bodyId, bool awake );
B2_API void b2Body_EnableSleep( b2BodyId bodyId, bool enableSleep );
B2_API bool b2Body_IsSleepEnabled( b2BodyId bodyId );
B2_API void b2Body_SetSleepThreshold( b2BodyId bodyId, float sleepVelocity );
B2_API float b2Body_GetSleepThreshold( b2BodyId bodyId );

/* Shape (reference box2d.h:423-571) */
B2_API b2ShapeId b2CreateCircleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Circle* circle );
B2_API b2ShapeId b2CreateSegmentShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Segment* segment );
B2_API b2ShapeId b2CreateCapsuleShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Capsule* capsule );
B2_API b2ShapeId b2CreatePolygonShape( b2BodyId bodyId, const b2ShapeDef* def, const b2Polygon* polygon );
/* Destroys a shape and its contacts and updates the body's mass when it is automatic
 * (reference box2d.h:441). */
B2_API void b2DestroyShape( b2ShapeId shapeId );
B2_API bool b2Shape_IsValid( b2ShapeId id );
B2_API b2ShapeType b2Shape_GetType( b2ShapeId shapeId );
B2_API b2BodyId b2Shape_GetBody( b2ShapeId shapeId );
B2_API float b2Shape_GetDensity( b2ShapeId shapeId );
B2_API void b2Shape_SetFriction( b2ShapeId shapeId, float friction );
B2_API float b2Shape_GetFriction( b2ShapeId shapeId );
B2_API void b2Shape_SetRestitution( b2ShapeId shapeId, float restitution );
B2_API float b2Shape_GetRestitution( b2ShapeId shapeId );
B2_API b2Filter b2Shape_GetFilter( b2ShapeId shapeId );
B2_API b2Polygon b2Shape_GetPolygon( b2ShapeId shapeId );
B2_API b2Circle b2Shape_GetCircle( b2ShapeId shapeId );
B2_API b2Segment b2Shape_GetSegment( b2ShapeId shapeId );
B2_API b2SmoothSegment b2Shape_GetSmoothSegment( b2ShapeId shapeId );
B2_API b2Capsule b2Shape_GetCapsule( b2ShapeId shapeId );
B2_API b2ChainId b2Shape_GetParentChain( b2ShapeId shapeId );

/* Chains of smooth segments (reference box2d.h:576-594). */
B2_API b2ChainId b2CreateChain( b2BodyId bodyId, const b2ChainDef* def );
B2_API void b2DestroyChain( b2ChainId chainId );
B2_API void b2Chain_SetFriction( b2ChainId chainId, float friction );
B2_API void b2Chain_SetRestitution( b2ChainId chainId, float restitution );
B2_API bool b2Chain_IsValid( b2ChainId id );
B2_API b2AABB b2Shape_GetAABB( b2ShapeId shapeId );

/* Joints: generic (reference box2d.h:605-646). */
B2_API void b2DestroyJoint( b2JointId jointId );
B2_API bool b2Joint_IsValid( b2JointId id );
B2_API b2JointType b2Joint_GetType( b2JointId jointId );
B2_API b2BodyId b2Joint_GetBodyA( b2JointId jointId );
B2_API b2BodyId b2Joint_GetBodyB( b2JointId jointId );
B2_API b2Vec2 b2Joint_GetLocalAnchorA( b2JointId jointId );
B2_API b2Vec2 b2Joint_GetLocalAnchorB( b2JointId jointId );
B2_API void b2Joint_SetCollideConnected( b2JointId jointId, bool shouldCollide );
B2_API bool b2Joint_GetCollideConnected( b2JointId jointId );
B2_API void b2Joint_SetUserData( b2JointId jointId, void* userData );
B2_API void* b2Joint_GetUserData( b2JointId jointId );
B2_API void b2Joint_WakeBodies( b2JointId jointId );
B2_API b2Vec2 b2Joint_GetConstraintForce( b2JointId jointId );
B2_API float b2Joint_GetConstraintTorque( b2JointId jointId );

/* Distance joint (reference box2d.h:654-720). */
B2_API b2JointId b2CreateDistanceJoint( b2WorldId worldId, const b2DistanceJointDef* def );
B2_API void b2DistanceJoint_SetLength( b2JointId jointId, float length );
B2_API float b2DistanceJoint_GetLength( b2JointId jointId );
B2_API void b2DistanceJoint_EnableSpring( b2JointId jointId, bool enableSpring );
B2_API bool b2DistanceJoint_IsSpringEnabled( b2JointId jointId );
B2_API void b2DistanceJoint_SetSpringHertz( b2JointId jointId, float hertz );
B2_API void b2DistanceJoint_SetSpringDampingRatio( b2JointId jointId, float dampingRatio );
B2_API float b2DistanceJoint_GetHertz( b2JointId jointId );
B2_API float b2DistanceJoint_GetDampingRatio( b2JointId jointId );
B2_API void b2DistanceJoint_EnableLimit( b2JointId jointId, bool enableLimit );
B2_API bool b2DistanceJoint_IsLimitEnabled( b2JointId jointId );
B2_API void b2DistanceJoint_SetLengthRange( b2JointId jointId, float minLength, float maxLength );
B2_API float b2DistanceJoint_GetMinLength( b2JointId jointId );
B2_API float b2DistanceJoint_GetMaxLength( b2JointId jointId );
B2_API float b2DistanceJoint_GetCurrentLength( b2JointId jointId );
B2_API void b2DistanceJoint_EnableMotor( b2JointId jointId, bool enableMotor );
B2_API bool b2DistanceJoint_IsMotorEnabled( b2JointId jointId );
B2_API void b2DistanceJoint_SetMotorSpeed( b2JointId jointId, float motorSpeed );
B2_API float b2DistanceJoint_GetMotorSpeed( b2JointId jointId );
B2_API void b2DistanceJoint_SetMaxMotorForce( b2JointId jointId, float force );
B2_API float b2DistanceJoint_GetMaxMotorForce( b2JointId jointId );
B2_API float b2DistanceJoint_GetMotorForce( b2JointId jointId );

/* Motor joint (reference box2d.h:736-766). */
B2_API b2JointId b2CreateMotorJoint( b2WorldId worldId, const b2MotorJointDef* def );
B2_API void b2MotorJoint_SetLinearOffset( b2JointId jointId, b2Vec2 linearOffset );
B2_API b2Vec2 b2MotorJoint_GetLinearOffset( b2JointId jointId );
B2_API void b2MotorJoint_SetAngularOffset( b2JointId jointId, float angularOffset );
B2_API float b2MotorJoint_GetAngularOffset( b2JointId jointId );
B2_API void b2MotorJoint_SetMaxForce( b2JointId jointId, float maxForce );
B2_API float b2MotorJoint_GetMaxForce( b2JointId jointId );
B2_API void b2MotorJoint_SetMaxTorque( b2JointId jointId, float maxTorque );
B2_API float b2MotorJoint_GetMaxTorque( b2JointId jointId );
B2_API void b2MotorJoint_SetCorrectionFactor( b2JointId jointId, float correctionFactor );
B2_API float b2MotorJoint_GetCorrectionFactor( b2JointId jointId );

/* Mouse joint (reference box2d.h:781-805). */
B2_API b2JointId b2CreateMouseJoint( b2WorldId worldId, const b2MouseJointDef* def );
B2_API void b2MouseJoint_SetTarget( b2JointId jointId, b2Vec2 target );
B2_API b2Vec2 b2MouseJoint_GetTarget( b2JointId jointId );
B2_API void b2MouseJoint_SetSpringHertz( b2JointId jointId, float hertz );
B2_API float b2MouseJoint_GetSpringHertz( b2JointId jointId );
B2_API void b2MouseJoint_SetSpringDampingRatio( b2JointId jointId, float dampingRatio );
B2_API float b2MouseJoint_GetSpringDampingRatio( b2JointId jointId );
B2_API void b2MouseJoint_SetMaxForce( b2JointId jointId, float maxForce );
B2_API float b2MouseJoint_GetMaxForce( b2JointId jointId );

/* Prismatic joint (reference box2d.h:820-876). */
B2_API b2JointId b2CreatePrismaticJoint( b2WorldId worldId, const b2PrismaticJointDef* def );
B2_API void b2PrismaticJoint_EnableSpring( b2JointId jointId, bool enableSpring );
B2_API bool b2PrismaticJoint_IsSpringEnabled( b2JointId jointId );
B2_API void b2PrismaticJoint_SetSpringHertz( b2JointId jointId, float hertz );
B2_API float b2PrismaticJoint_GetSpringHertz( b2JointId jointId );
B2_API void b2PrismaticJoint_SetSpringDampingRatio( b2JointId jointId, float dampingRatio );
B2_API float b2PrismaticJoint_GetSpringDampingRatio( b2JointId jointId );
B2_API void b2PrismaticJoint_EnableLimit( b2JointId jointId, bool enableLimit );
B2_API bool b2PrismaticJoint_IsLimitEnabled( b2JointId jointId );
B2_API float b2PrismaticJoint_GetLowerLimit( b2JointId jointId );
B2_API float b2PrismaticJoint_GetUpperLimit( b2JointId jointId );
B2_API void b2PrismaticJoint_SetLimits( b2JointId jointId, float lower, float upper );
B2_API void b2PrismaticJoint_EnableMotor( b2JointId jointId, bool enableMotor );
B2_API bool b2PrismaticJoint_IsMotorEnabled( b2JointId jointId );
B2_API void b2PrismaticJoint_SetMotorSpeed( b2JointId jointId, float motorSpeed );
B2_API float b2PrismaticJoint_GetMotorSpeed( b2JointId jointId );
B2_API void b2PrismaticJoint_SetMaxMotorForce( b2JointId jointId, float force );
B2_API float b2PrismaticJoint_GetMaxMotorForce( b2JointId jointId );
B2_API float b2PrismaticJoint_GetMotorForce( b2JointId jointId );

/* Revolute joint (reference box2d.h:891-946). */
B2_API b2JointId b2CreateRevoluteJoint( b2WorldId worldId, const b2RevoluteJointDef* def );
B2_API void b2RevoluteJoint_EnableSpring( b2JointId jointId, bool enableSpring );
B2_API bool b2RevoluteJoint_IsSpringEnabled( b2JointId jointId );
B2_API void b2RevoluteJoint_SetSpringHertz( b2JointId jointId, float hertz );
B2_API float b2RevoluteJoint_GetSpringHertz( b2JointId jointId );
B2_API void b2RevoluteJoint_SetSpringDampingRatio( b2JointId jointId, float dampingRatio );
B2_API float b2RevoluteJoint_GetSpringDampingRatio( b2JointId jointId );
B2_API float b2RevoluteJoint_GetAngle( b2JointId jointId );
B2_API void b2RevoluteJoint_EnableLimit( b2JointId jointId, bool enableLimit );
B2_API bool b2RevoluteJoint_IsLimitEnabled( b2JointId jointId );
B2_API float b2RevoluteJoint_GetLowerLimit( b2JointId jointId );
B2_API float b2RevoluteJoint_GetUpperLimit( b2JointId jointId );
B2_API void b2RevoluteJoint_SetLimits( b2JointId jointId, float lower, float upper );
B2_API void b2RevoluteJoint_EnableMotor( b2JointId jointId, bool enableMotor );
B2_API bool b2RevoluteJoint_IsMotorEnabled( b2JointId jointId );
B2_API void b2RevoluteJoint_SetMotorSpeed( b2JointId jointId, float motorSpeed );
B2_API float b2RevoluteJoint_GetMotorSpeed( b2JointId jointId );
B2_API float b2RevoluteJoint_GetMotorTorque( b2JointId jointId );
B2_API void b2RevoluteJoint_SetMaxMotorTorque( b2JointId jointId, float torque );
B2_API float b2RevoluteJoint_GetMaxMotorTorque( b2JointId jointId );

/* Weld joint (reference box2d.h:963-987). */
B2_API b2JointId b2CreateWeldJoint( b2WorldId worldId, const b2WeldJointDef* def );
B2_API void b2WeldJoint_SetLinearHertz( b2JointId jointId, float hertz );
B2_API float b2WeldJoint_GetLinearHertz( b2JointId jointId );
B2_API void b2WeldJoint_SetLinearDampingRatio( b2JointId jointId, float dampingRatio );
B2_API float b2WeldJoint_GetLinearDampingRatio( b2JointId jointId );
B2_API void b2WeldJoint_SetAngularHertz( b2JointId jointId, float hertz );
B2_API float b2WeldJoint_GetAngularHertz( b2JointId jointId );
B2_API void b2WeldJoint_SetAngularDampingRatio( b2JointId jointId, float dampingRatio );
B2_API float b2WeldJoint_GetAngularDampingRatio( b2JointId jointId );

/* Wheel joint (reference box2d.h:1003-1057). */
B2_API b2JointId b2CreateWheelJoint( b2WorldId worldId, const b2WheelJointDef* def );
B2_API void b2WheelJoint_EnableSpring( b2JointId jointId, bool enableSpring );
B2_API bool b2WheelJoint_IsSpringEnabled( b2JointId jointId );
B2_API void b2WheelJoint_SetSpringHertz( b2JointId jointId, float hertz );
B2_API float b2WheelJoint_GetSpringHertz( b2JointId jointId );
B2_API void b2WheelJoint_SetSpringDampingRatio( b2JointId jointId, float dampingRatio );
B2_API float b2WheelJoint_GetSpringDampingRatio( b2JointId jointId );
B2_API void b2WheelJoint_EnableLimit( b2JointId jointId, bool enableLimit );
B2_API bool b2WheelJoint_IsLimitEnabled( b2JointId jointId );
B2_API float b2WheelJoint_GetLowerLimit( b2JointId jointId );
B2_API float b2WheelJoint_GetUpperLimit( b2JointId jointId );
B2_API void b2WheelJoint_SetLimits( b2JointId jointId, float lower, float upper );
B2_API void b2WheelJoint_EnableMotor( b2JointId jointId, bool enableMotor );
B2_API bool b2WheelJoint_IsMotorEnabled( b2JointId jointId );
B2_API void b2WheelJoint_SetMotorSpeed( b2JointId jointId, float motorSpeed );
B2_API float b2WheelJoint_GetMotorSpeed( b2JointId jointId );
B2_API void b2WheelJoint_SetMaxMotorTorque( b2JointId jointId, float torque );
B2_API float b2WheelJoint_GetMaxMotorTorque( b2JointId jointId );
B2_API float b2WheelJoint_GetMotorTorque( b2JointId jointId );
