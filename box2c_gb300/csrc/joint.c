/*
 * joint.c -- the joint API of every joint type: default definitions, creation, the
 * generic joint queries and each type's getters and setters.
 *
 * Creation follows reference src/joint.c:331-655 (the record itself comes from
 * gjoint_create in world.c, src/joint.c:140-288); the per-type API follows
 * src/distance_joint.c:18-211, src/motor_joint.c:14-83, src/mouse_joint.c:14-75,
 * src/prismatic_joint.c:16-165, src/revolute_joint.c:16-146, src/weld_joint.c:16-75 and
 * src/wheel_joint.c:16-163, including which setters reset which accumulated impulses.
 * Joint configuration lives in the host table of device joint records (w->hJoints); a
 * setter downloads the device's solver state first, so impulses it keeps survive, and
 * marks the table for upload before the next step.
 */
#include "host.h"

#include <math.h>
#include <string.h>

#define B2G_COOKIE 1152023

_Static_assert( B2G_J_DISTANCE == (int)b2_distanceJoint && B2G_J_MOTOR == (int)b2_motorJoint &&
					B2G_J_MOUSE == (int)b2_mouseJoint && B2G_J_PRISMATIC == (int)b2_prismaticJoint &&
					B2G_J_REVOLUTE == (int)b2_revoluteJoint && B2G_J_WELD == (int)b2_weldJoint &&
					B2G_J_WHEEL == (int)b2_wheelJoint,
				"device joint type numbers follow b2JointType" );
_Static_assert( sizeof( b2gJointDev ) == 256, "joint record layout" );

/* ------------------------------------------------------------ default definitions */
b2DistanceJointDef b2DefaultDistanceJointDef( void )
{
	b2DistanceJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.length = 1.0f;
	d.maxLength = B2G_HUGE;
	d.internalValue = B2G_COOKIE;
	return d;
}

b2MotorJointDef b2DefaultMotorJointDef( void )
{
	b2MotorJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.maxForce = 1.0f;
	d.maxTorque = 1.0f;
	d.correctionFactor = 0.3f;
	d.internalValue = B2G_COOKIE;
	return d;
}

b2MouseJointDef b2DefaultMouseJointDef( void )
{
	b2MouseJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.hertz = 4.0f;
	d.dampingRatio = 1.0f;
	d.maxForce = 1.0f;
	d.internalValue = B2G_COOKIE;
	return d;
}

b2PrismaticJointDef b2DefaultPrismaticJointDef( void )
{
	b2PrismaticJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.localAxisA.x = 1.0f;
	d.internalValue = B2G_COOKIE;
	return d;
}

b2RevoluteJointDef b2DefaultRevoluteJointDef( void )
{
	b2RevoluteJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.drawSize = 0.25f;
	d.internalValue = B2G_COOKIE;
	return d;
}

b2WeldJointDef b2DefaultWeldJointDef( void )
{
	b2WeldJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.internalValue = B2G_COOKIE;
	return d;
}

b2WheelJointDef b2DefaultWheelJointDef( void )
{
	b2WheelJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.localAxisA.y = 1.0f;
	d.enableSpring = true;
	d.hertz = 1.0f;
	d.dampingRatio = 0.7f;
	d.internalValue = B2G_COOKIE;
	return d;
}

/* ------------------------------------------------------------ helpers */
static gWorld* joint_world( b2JointId id ) { return gworld_slot( id.world0 ); }
static gJoint* joint_rec( b2JointId id ) { return joint_world( id )->joints + ( id.index1 - 1 ); }

/* The joint's device record for reading: solver state as of the last step. */
static const b2gJointDev* joint_read( b2JointId id )
{
	gWorld* w = joint_world( id );
	gworld_ensure_joint_mirror( w );
	return w->hJoints + ( id.index1 - 1 );
}

/* The joint's device record for writing: uploaded again before the next step. */
static b2gJointDev* joint_write( b2JointId id )
{
	gWorld* w = joint_world( id );
	gworld_ensure_joint_mirror( w );
	w->jointsDirty = true;
	return w->hJoints + ( id.index1 - 1 );
}

static b2Transform body_transform( gWorld* w, int bodyId )
{
	gworld_ensure_mirror( w );
	const float* x = w->hXf + 4 * bodyId;
	b2Transform t = { { x[0], x[1] }, { x[2], x[3] } };
	return t;
}

static b2gVec gvec( b2Vec2 v ) { return gv( v.x, v.y ); }
static b2Vec2 bvec( b2gVec v )
{
	b2Vec2 r = { v.x, v.y };
	return r;
}

/* Relative angle with the C library's atan2f, as the reference's queries compute it
 * (include/box2d/math_functions.h:386-394). */
static float host_relative_angle( b2Rot b, b2Rot a )
{
	float s = b.s * a.c - b.c * a.s;
	float c = b.c * a.c + b.s * a.s;
	return atan2f( s, c );
}

static float host_unwind( float a )
{
	if ( a < -B2G_PI )
		return a + 2.0f * B2G_PI;
	if ( a > B2G_PI )
		return a - 2.0f * B2G_PI;
	return a;
}

/* Finishes a creation: the contacts between the two bodies go when the joint keeps them
 * from colliding (reference src/joint.c:370-374 and the same step of every type). */
static b2JointId joint_finish( b2JointId id, bool collideConnected )
{
	if ( collideConnected == false )
	{
		gWorld* w = joint_world( id );
		gJoint* j = joint_rec( id );
		gjoint_disconnect_bodies( w, j->bodyIdA, j->bodyIdB );
	}
	return id;
}

/* ------------------------------------------------------------ creation */
b2JointId b2CreateDistanceJoint( b2WorldId worldId, const b2DistanceJointDef* def )
{
	b2JointId id;
	b2gJointDev* d = gjoint_create( worldId, def->bodyIdA, def->bodyIdB, b2_distanceJoint, def->collideConnected, def->userData, &id );
	if ( d == NULL )
		return id;
	d->localAnchorA = gvec( def->localAnchorA );
	d->localAnchorB = gvec( def->localAnchorB );
	d->length = gmax( def->length, B2G_LINEAR_SLOP );
	d->hertz = def->hertz;
	d->dampingRatio = def->dampingRatio;
	d->lower = gmax( def->minLength, B2G_LINEAR_SLOP );
	d->upper = gmax( def->minLength, def->maxLength );
	d->maxMotor = def->maxMotorForce;
	d->motorSpeed = def->motorSpeed;
	d->enableSpring = def->enableSpring;
	d->enableLimit = def->enableLimit;
	d->enableMotor = def->enableMotor;
	return joint_finish( id, def->collideConnected );
}

b2JointId b2CreateMotorJoint( b2WorldId worldId, const b2MotorJointDef* def )
{
	b2JointId id;
	b2gJointDev* d = gjoint_create( worldId, def->bodyIdA, def->bodyIdB, b2_motorJoint, def->collideConnected, def->userData, &id );
	if ( d == NULL )
		return id;
	d->target = gvec( def->linearOffset );
	d->referenceAngle = def->angularOffset;
	d->maxMotor = def->maxForce;
	d->maxTorque = def->maxTorque;
	d->correctionFactor = gclamp( def->correctionFactor, 0.0f, 1.0f );
	return joint_finish( id, def->collideConnected );
}

b2JointId b2CreateMouseJoint( b2WorldId worldId, const b2MouseJointDef* def )
{
	b2JointId id;
	if ( b2World_IsValid( worldId ) == false || b2Body_IsValid( def->bodyIdA ) == false || b2Body_IsValid( def->bodyIdB ) == false )
		return b2_nullJointId;
	gWorld* w = gworld_get( worldId );
	b2Transform xfA = body_transform( w, def->bodyIdA.index1 - 1 );
	b2Transform xfB = body_transform( w, def->bodyIdB.index1 - 1 );
	b2gJointDev* d = gjoint_create( worldId, def->bodyIdA, def->bodyIdB, b2_mouseJoint, def->collideConnected, def->userData, &id );
	if ( d == NULL )
		return id;
	d->localAnchorA = gvec( b2InvTransformPoint( xfA, def->target ) );
	d->localAnchorB = gvec( b2InvTransformPoint( xfB, def->target ) );
	d->target = gvec( def->target );
	d->hertz = def->hertz;
	d->dampingRatio = def->dampingRatio;
	d->maxMotor = def->maxForce;
	/* the reference keeps the contacts of a mouse joint's bodies (src/joint.c:422-456) */
	return id;
}

b2JointId b2CreatePrismaticJoint( b2WorldId worldId, const b2PrismaticJointDef* def )
{
	b2JointId id;
	b2gJointDev* d =
		gjoint_create( worldId, def->bodyIdA, def->bodyIdB, b2_prismaticJoint, def->collideConnected, def->userData, &id );
	if ( d == NULL )
		return id;
	d->localAnchorA = gvec( def->localAnchorA );
	d->localAnchorB = gvec( def->localAnchorB );
	d->localAxisA = gnormalize( gvec( def->localAxisA ) );
	d->referenceAngle = def->referenceAngle;
	d->hertz = def->hertz;
	d->dampingRatio = def->dampingRatio;
	d->lower = def->lowerTranslation;
	d->upper = def->upperTranslation;
	d->maxMotor = def->maxMotorForce;
	d->motorSpeed = def->motorSpeed;
	d->enableSpring = def->enableSpring;
	d->enableLimit = def->enableLimit;
	d->enableMotor = def->enableMotor;
	return joint_finish( id, def->collideConnected );
}

b2JointId b2CreateRevoluteJoint( b2WorldId worldId, const b2RevoluteJointDef* def )
{
	b2JointId id;
	b2gJointDev* d =
		gjoint_create( worldId, def->bodyIdA, def->bodyIdB, b2_revoluteJoint, def->collideConnected, def->userData, &id );
	if ( d == NULL )
		return id;
	d->localAnchorA = gvec( def->localAnchorA );
	d->localAnchorB = gvec( def->localAnchorB );
	d->referenceAngle = gclamp( def->referenceAngle, -B2G_PI, B2G_PI );
	d->hertz = def->hertz;
	d->dampingRatio = def->dampingRatio;
	d->lower = gmin( def->lowerAngle, def->upperAngle );
	d->upper = gmax( def->lowerAngle, def->upperAngle );
	d->lower = gclamp( d->lower, -B2G_PI, B2G_PI );
	d->upper = gclamp( d->upper, -B2G_PI, B2G_PI );
	d->maxMotor = def->maxMotorTorque;
	d->motorSpeed = def->motorSpeed;
	d->enableSpring = def->enableSpring;
	d->enableLimit = def->enableLimit;
	d->enableMotor = def->enableMotor;
	return joint_finish( id, def->collideConnected );
}

b2JointId b2CreateWeldJoint( b2WorldId worldId, const b2WeldJointDef* def )
{
	b2JointId id;
	b2gJointDev* d = gjoint_create( worldId, def->bodyIdA, def->bodyIdB, b2_weldJoint, def->collideConnected, def->userData, &id );
	if ( d == NULL )
		return id;
	d->localAnchorA = gvec( def->localAnchorA );
	d->localAnchorB = gvec( def->localAnchorB );
	d->referenceAngle = def->referenceAngle;
	d->hertz = def->linearHertz;
	d->dampingRatio = def->linearDampingRatio;
	d->angularHertz = def->angularHertz;
	d->angularDampingRatio = def->angularDampingRatio;
	return joint_finish( id, def->collideConnected );
}

b2JointId b2CreateWheelJoint( b2WorldId worldId, const b2WheelJointDef* def )
{
	b2JointId id;
	b2gJointDev* d = gjoint_create( worldId, def->bodyIdA, def->bodyIdB, b2_wheelJoint, def->collideConnected, def->userData, &id );
	if ( d == NULL )
		return id;
	d->localAnchorA = gvec( def->localAnchorA );
	d->localAnchorB = gvec( def->localAnchorB );
	d->localAxisA = gnormalize( gvec( def->localAxisA ) );
	d->lower = def->lowerTranslation;
	d->upper = def->upperTranslation;
	d->maxMotor = def->maxMotorTorque;
	d->motorSpeed = def->motorSpeed;
	d->hertz = def->hertz;
	d->dampingRatio = def->dampingRatio;
	d->enableSpring = def->enableSpring;
	d->enableLimit = def->enableLimit;
	d->enableMotor = def->enableMotor;
	return joint_finish( id, def->collideConnected );
}

/* ------------------------------------------------------------ generic queries */
b2JointType b2Joint_GetType( b2JointId id ) { return joint_rec( id )->type; }

b2BodyId b2Joint_GetBodyA( b2JointId id )
{
	gWorld* w = joint_world( id );
	gJoint* j = joint_rec( id );
	b2BodyId b = { j->bodyIdA + 1, id.world0, w->bodies[j->bodyIdA].revision };
	return b;
}

b2BodyId b2Joint_GetBodyB( b2JointId id )
{
	gWorld* w = joint_world( id );
	gJoint* j = joint_rec( id );
	b2BodyId b = { j->bodyIdB + 1, id.world0, w->bodies[j->bodyIdB].revision };
	return b;
}

b2Vec2 b2Joint_GetLocalAnchorA( b2JointId id ) { return bvec( joint_read( id )->localAnchorA ); }
b2Vec2 b2Joint_GetLocalAnchorB( b2JointId id ) { return bvec( joint_read( id )->localAnchorB ); }

void b2Joint_SetCollideConnected( b2JointId id, bool shouldCollide )
{
	gWorld* w = joint_world( id );
	if ( w->locked )
		return;
	gJoint* j = joint_rec( id );
	if ( j->collideConnected == shouldCollide )
		return;
	j->collideConnected = shouldCollide;
	gBody* a = w->bodies + j->edges[0].bodyId;
	gBody* b = w->bodies + j->edges[1].bodyId;
	if ( shouldCollide )
	{
		/* look for new pairs from the body with fewer shapes (reference src/joint.c:826-842) */
		int shapeId = a->shapeCount < b->shapeCount ? a->headShape : b->headShape;
		while ( shapeId != B2G_NULL )
		{
			gShape* s = w->shapes + shapeId;
			if ( s->proxyKey != B2G_NULL )
				gbuffer_move( w, s->proxyKey );
			shapeId = s->next;
		}
	}
	else
		gjoint_disconnect_bodies( w, a->id, b->id );
}

bool b2Joint_GetCollideConnected( b2JointId id ) { return joint_rec( id )->collideConnected; }
void b2Joint_SetUserData( b2JointId id, void* userData ) { joint_rec( id )->userData = userData; }
void* b2Joint_GetUserData( b2JointId id ) { return joint_rec( id )->userData; }

/* Every body is awake (sleep is not simulated), so waking is a no-op. */
/* reference src/joint.c:874-888 */
void b2Joint_WakeBodies( b2JointId id )
{
	gWorld* w = joint_world( id );
	if ( w->locked )
		return;
	gJoint* j = w->joints + ( id.index1 - 1 );
	gbody_wake( w, w->bodies + j->edges[0].bodyId );
	gbody_wake( w, w->bodies + j->edges[1].bodyId );
}

b2Vec2 b2Joint_GetConstraintForce( b2JointId id )
{
	gWorld* w = joint_world( id );
	const b2gJointDev* d = joint_read( id );
	float inv_h = w->inv_h;
	switch ( (b2JointType)d->type )
	{
		case b2_distanceJoint:
		{
			/* src/distance_joint.c:183-196 */
			b2Transform xfA = body_transform( w, d->bodyIdA );
			b2Transform xfB = body_transform( w, d->bodyIdB );
			b2Vec2 pA = b2TransformPoint( xfA, bvec( d->localAnchorA ) );
			b2Vec2 pB = b2TransformPoint( xfB, bvec( d->localAnchorB ) );
			b2gVec axis = gnormalize( gv( pB.x - pA.x, pB.y - pA.y ) );
			float force = ( d->impulse + d->lowerImpulse - d->upperImpulse + d->motorImpulse ) * inv_h;
			return bvec( gmulsv( force, axis ) );
		}
		case b2_prismaticJoint:
		{
			/* src/prismatic_joint.c:144-160 */
			b2Transform xfA = body_transform( w, d->bodyIdA );
			b2gVec axisA = grotate( grot( xfA.q.c, xfA.q.s ), d->localAxisA );
			b2gVec perpA = gv( -axisA.y, axisA.x );
			float perpForce = inv_h * d->linearImpulse.x;
			float axialForce = inv_h * ( d->motorImpulse + d->lowerImpulse - d->upperImpulse );
			return bvec( gadd( gmulsv( perpForce, perpA ), gmulsv( axialForce, axisA ) ) );
		}
		case b2_wheelJoint:
		{
			/* src/wheel_joint.c:145-158: the axis of the last step */
			b2gVec axisA = d->axisA;
			b2gVec perpA = gv( -axisA.y, axisA.x );
			float perpForce = inv_h * d->perpImpulse;
			float axialForce = inv_h * ( d->springImpulse + d->lowerImpulse - d->upperImpulse );
			return bvec( gadd( gmulsv( perpForce, perpA ), gmulsv( axialForce, axisA ) ) );
		}
		default:
			/* revolute, weld, motor, mouse: inv_h * linearImpulse */
			return bvec( gmulsv( inv_h, d->linearImpulse ) );
	}
}

float b2Joint_GetConstraintTorque( b2JointId id )
{
	gWorld* w = joint_world( id );
	const b2gJointDev* d = joint_read( id );
	float inv_h = w->inv_h;
	switch ( (b2JointType)d->type )
	{
		case b2_distanceJoint:
			return 0.0f;
		case b2_prismaticJoint:
			return inv_h * d->linearImpulse.y;
		case b2_revoluteJoint:
			return inv_h * ( d->motorImpulse + d->lowerImpulse - d->upperImpulse );
		case b2_wheelJoint:
			return inv_h * d->motorImpulse;
		default:
			/* weld, motor, mouse */
			return inv_h * d->angularImpulse;
	}
}

/* ------------------------------------------------------------ distance joint */
void b2DistanceJoint_SetLength( b2JointId id, float length )
{
	b2gJointDev* d = joint_write( id );
	d->length = gclamp( length, B2G_LINEAR_SLOP, B2G_HUGE );
	d->impulse = 0.0f;
	d->lowerImpulse = 0.0f;
	d->upperImpulse = 0.0f;
}
float b2DistanceJoint_GetLength( b2JointId id ) { return joint_read( id )->length; }
void b2DistanceJoint_EnableSpring( b2JointId id, bool enableSpring ) { joint_write( id )->enableSpring = enableSpring; }
bool b2DistanceJoint_IsSpringEnabled( b2JointId id ) { return joint_read( id )->enableSpring != 0; }
void b2DistanceJoint_SetSpringHertz( b2JointId id, float hertz ) { joint_write( id )->hertz = hertz; }
void b2DistanceJoint_SetSpringDampingRatio( b2JointId id, float dampingRatio ) { joint_write( id )->dampingRatio = dampingRatio; }
float b2DistanceJoint_GetHertz( b2JointId id ) { return joint_read( id )->hertz; }
float b2DistanceJoint_GetDampingRatio( b2JointId id ) { return joint_read( id )->dampingRatio; }
void b2DistanceJoint_EnableLimit( b2JointId id, bool enableLimit ) { joint_write( id )->enableLimit = enableLimit; }
bool b2DistanceJoint_IsLimitEnabled( b2JointId id ) { return joint_read( id )->enableLimit != 0; }
void b2DistanceJoint_SetLengthRange( b2JointId id, float minLength, float maxLength )
{
	b2gJointDev* d = joint_write( id );
	minLength = gclamp( minLength, B2G_LINEAR_SLOP, B2G_HUGE );
	maxLength = gclamp( maxLength, B2G_LINEAR_SLOP, B2G_HUGE );
	d->lower = gmin( minLength, maxLength );
	d->upper = gmax( minLength, maxLength );
	d->impulse = 0.0f;
	d->lowerImpulse = 0.0f;
	d->upperImpulse = 0.0f;
}
float b2DistanceJoint_GetMinLength( b2JointId id ) { return joint_read( id )->lower; }
float b2DistanceJoint_GetMaxLength( b2JointId id ) { return joint_read( id )->upper; }
float b2DistanceJoint_GetCurrentLength( b2JointId id )
{
	gWorld* w = joint_world( id );
	if ( w->locked )
		return 0.0f;
	const b2gJointDev* d = joint_read( id );
	b2Vec2 pA = b2TransformPoint( body_transform( w, d->bodyIdA ), bvec( d->localAnchorA ) );
	b2Vec2 pB = b2TransformPoint( body_transform( w, d->bodyIdB ), bvec( d->localAnchorB ) );
	return glen( gv( pB.x - pA.x, pB.y - pA.y ) );
}
void b2DistanceJoint_EnableMotor( b2JointId id, bool enableMotor )
{
	b2gJointDev* d = joint_write( id );
	if ( enableMotor != ( d->enableMotor != 0 ) )
	{
		d->enableMotor = enableMotor;
		d->motorImpulse = 0.0f;
	}
}
bool b2DistanceJoint_IsMotorEnabled( b2JointId id ) { return joint_read( id )->enableMotor != 0; }
void b2DistanceJoint_SetMotorSpeed( b2JointId id, float motorSpeed ) { joint_write( id )->motorSpeed = motorSpeed; }
float b2DistanceJoint_GetMotorSpeed( b2JointId id ) { return joint_read( id )->motorSpeed; }
float b2DistanceJoint_GetMotorForce( b2JointId id ) { return joint_world( id )->inv_h * joint_read( id )->motorImpulse; }
void b2DistanceJoint_SetMaxMotorForce( b2JointId id, float force ) { joint_write( id )->maxMotor = force; }
float b2DistanceJoint_GetMaxMotorForce( b2JointId id ) { return joint_read( id )->maxMotor; }

/* ------------------------------------------------------------ motor joint */
void b2MotorJoint_SetLinearOffset( b2JointId id, b2Vec2 linearOffset ) { joint_write( id )->target = gvec( linearOffset ); }
b2Vec2 b2MotorJoint_GetLinearOffset( b2JointId id ) { return bvec( joint_read( id )->target ); }
void b2MotorJoint_SetAngularOffset( b2JointId id, float angularOffset )
{
	joint_write( id )->referenceAngle = gclamp( angularOffset, -B2G_PI, B2G_PI );
}
float b2MotorJoint_GetAngularOffset( b2JointId id ) { return joint_read( id )->referenceAngle; }
void b2MotorJoint_SetMaxForce( b2JointId id, float maxForce ) { joint_write( id )->maxMotor = gmax( 0.0f, maxForce ); }
float b2MotorJoint_GetMaxForce( b2JointId id ) { return joint_read( id )->maxMotor; }
void b2MotorJoint_SetMaxTorque( b2JointId id, float maxTorque ) { joint_write( id )->maxTorque = gmax( 0.0f, maxTorque ); }
float b2MotorJoint_GetMaxTorque( b2JointId id ) { return joint_read( id )->maxTorque; }
void b2MotorJoint_SetCorrectionFactor( b2JointId id, float correctionFactor )
{
	joint_write( id )->correctionFactor = gclamp( correctionFactor, 0.0f, 1.0f );
}
float b2MotorJoint_GetCorrectionFactor( b2JointId id ) { return joint_read( id )->correctionFactor; }

/* ------------------------------------------------------------ mouse joint */
void b2MouseJoint_SetTarget( b2JointId id, b2Vec2 target ) { joint_write( id )->target = gvec( target ); }
b2Vec2 b2MouseJoint_GetTarget( b2JointId id ) { return bvec( joint_read( id )->target ); }
void b2MouseJoint_SetSpringHertz( b2JointId id, float hertz ) { joint_write( id )->hertz = hertz; }
float b2MouseJoint_GetSpringHertz( b2JointId id ) { return joint_read( id )->hertz; }
void b2MouseJoint_SetSpringDampingRatio( b2JointId id, float dampingRatio ) { joint_write( id )->dampingRatio = dampingRatio; }
float b2MouseJoint_GetSpringDampingRatio( b2JointId id ) { return joint_read( id )->dampingRatio; }
void b2MouseJoint_SetMaxForce( b2JointId id, float maxForce ) { joint_write( id )->maxMotor = maxForce; }
float b2MouseJoint_GetMaxForce( b2JointId id ) { return joint_read( id )->maxMotor; }

/* ------------------------------------------------------------ spring / limit / motor setters
 * shared by the prismatic, revolute and wheel joints (same fields, same impulse resets) */
static void enable_spring( b2JointId id, bool enable )
{
	b2gJointDev* d = joint_write( id );
	if ( enable != ( d->enableSpring != 0 ) )
	{
		d->enableSpring = enable;
		d->springImpulse = 0.0f;
	}
}

static void enable_limit( b2JointId id, bool enable )
{
	b2gJointDev* d = joint_write( id );
	if ( enable != ( d->enableLimit != 0 ) )
	{
		d->enableLimit = enable;
		d->lowerImpulse = 0.0f;
		d->upperImpulse = 0.0f;
	}
}

static void set_limits( b2JointId id, float lower, float upper )
{
	b2gJointDev* d = joint_write( id );
	if ( lower != d->lower || upper != d->upper )
	{
		d->lower = gmin( lower, upper );
		d->upper = gmax( lower, upper );
		d->lowerImpulse = 0.0f;
		d->upperImpulse = 0.0f;
	}
}

static void enable_motor( b2JointId id, bool enable )
{
	b2gJointDev* d = joint_write( id );
	if ( enable != ( d->enableMotor != 0 ) )
	{
		d->enableMotor = enable;
		d->motorImpulse = 0.0f;
	}
}

/* ------------------------------------------------------------ prismatic joint */
void b2PrismaticJoint_EnableSpring( b2JointId id, bool enableSpring ) { enable_spring( id, enableSpring ); }
bool b2PrismaticJoint_IsSpringEnabled( b2JointId id ) { return joint_read( id )->enableSpring != 0; }
void b2PrismaticJoint_SetSpringHertz( b2JointId id, float hertz ) { joint_write( id )->hertz = hertz; }
float b2PrismaticJoint_GetSpringHertz( b2JointId id ) { return joint_read( id )->hertz; }
void b2PrismaticJoint_SetSpringDampingRatio( b2JointId id, float dampingRatio ) { joint_write( id )->dampingRatio = dampingRatio; }
float b2PrismaticJoint_GetSpringDampingRatio( b2JointId id ) { return joint_read( id )->dampingRatio; }
void b2PrismaticJoint_EnableLimit( b2JointId id, bool enableLimit ) { enable_limit( id, enableLimit ); }
bool b2PrismaticJoint_IsLimitEnabled( b2JointId id ) { return joint_read( id )->enableLimit != 0; }
float b2PrismaticJoint_GetLowerLimit( b2JointId id ) { return joint_read( id )->lower; }
float b2PrismaticJoint_GetUpperLimit( b2JointId id ) { return joint_read( id )->upper; }
void b2PrismaticJoint_SetLimits( b2JointId id, float lower, float upper ) { set_limits( id, lower, upper ); }
void b2PrismaticJoint_EnableMotor( b2JointId id, bool enableMotor ) { enable_motor( id, enableMotor ); }
bool b2PrismaticJoint_IsMotorEnabled( b2JointId id ) { return joint_read( id )->enableMotor != 0; }
void b2PrismaticJoint_SetMotorSpeed( b2JointId id, float motorSpeed ) { joint_write( id )->motorSpeed = motorSpeed; }
float b2PrismaticJoint_GetMotorSpeed( b2JointId id ) { return joint_read( id )->motorSpeed; }
void b2PrismaticJoint_SetMaxMotorForce( b2JointId id, float force ) { joint_write( id )->maxMotor = force; }
float b2PrismaticJoint_GetMaxMotorForce( b2JointId id ) { return joint_read( id )->maxMotor; }
float b2PrismaticJoint_GetMotorForce( b2JointId id ) { return joint_world( id )->inv_h * joint_read( id )->motorImpulse; }

/* ------------------------------------------------------------ revolute joint */
void b2RevoluteJoint_EnableSpring( b2JointId id, bool enableSpring ) { enable_spring( id, enableSpring ); }
bool b2RevoluteJoint_IsSpringEnabled( b2JointId id ) { return joint_read( id )->enableSpring != 0; }
void b2RevoluteJoint_SetSpringHertz( b2JointId id, float hertz ) { joint_write( id )->hertz = hertz; }
float b2RevoluteJoint_GetSpringHertz( b2JointId id ) { return joint_read( id )->hertz; }
void b2RevoluteJoint_SetSpringDampingRatio( b2JointId id, float dampingRatio ) { joint_write( id )->dampingRatio = dampingRatio; }
float b2RevoluteJoint_GetSpringDampingRatio( b2JointId id ) { return joint_read( id )->dampingRatio; }
float b2RevoluteJoint_GetAngle( b2JointId id )
{
	gWorld* w = joint_world( id );
	const b2gJointDev* d = joint_read( id );
	b2Transform xfA = body_transform( w, d->bodyIdA );
	b2Transform xfB = body_transform( w, d->bodyIdB );
	float angle = host_relative_angle( xfB.q, xfA.q ) - d->referenceAngle;
	return host_unwind( angle );
}
void b2RevoluteJoint_EnableLimit( b2JointId id, bool enableLimit ) { enable_limit( id, enableLimit ); }
bool b2RevoluteJoint_IsLimitEnabled( b2JointId id ) { return joint_read( id )->enableLimit != 0; }
float b2RevoluteJoint_GetLowerLimit( b2JointId id ) { return joint_read( id )->lower; }
float b2RevoluteJoint_GetUpperLimit( b2JointId id ) { return joint_read( id )->upper; }
void b2RevoluteJoint_SetLimits( b2JointId id, float lower, float upper ) { set_limits( id, lower, upper ); }
void b2RevoluteJoint_EnableMotor( b2JointId id, bool enableMotor ) { enable_motor( id, enableMotor ); }
bool b2RevoluteJoint_IsMotorEnabled( b2JointId id ) { return joint_read( id )->enableMotor != 0; }
void b2RevoluteJoint_SetMotorSpeed( b2JointId id, float motorSpeed ) { joint_write( id )->motorSpeed = motorSpeed; }
float b2RevoluteJoint_GetMotorSpeed( b2JointId id ) { return joint_read( id )->motorSpeed; }
float b2RevoluteJoint_GetMotorTorque( b2JointId id ) { return joint_world( id )->inv_h * joint_read( id )->motorImpulse; }
void b2RevoluteJoint_SetMaxMotorTorque( b2JointId id, float torque ) { joint_write( id )->maxMotor = torque; }
float b2RevoluteJoint_GetMaxMotorTorque( b2JointId id ) { return joint_read( id )->maxMotor; }

/* ------------------------------------------------------------ weld joint */
void b2WeldJoint_SetLinearHertz( b2JointId id, float hertz ) { joint_write( id )->hertz = hertz; }
float b2WeldJoint_GetLinearHertz( b2JointId id ) { return joint_read( id )->hertz; }
void b2WeldJoint_SetLinearDampingRatio( b2JointId id, float dampingRatio ) { joint_write( id )->dampingRatio = dampingRatio; }
float b2WeldJoint_GetLinearDampingRatio( b2JointId id ) { return joint_read( id )->dampingRatio; }
void b2WeldJoint_SetAngularHertz( b2JointId id, float hertz ) { joint_write( id )->angularHertz = hertz; }
float b2WeldJoint_GetAngularHertz( b2JointId id ) { return joint_read( id )->angularHertz; }
void b2WeldJoint_SetAngularDampingRatio( b2JointId id, float dampingRatio ) { joint_write( id )->angularDampingRatio = dampingRatio; }
float b2WeldJoint_GetAngularDampingRatio( b2JointId id ) { return joint_read( id )->angularDampingRatio; }

/* ------------------------------------------------------------ wheel joint */
void b2WheelJoint_EnableSpring( b2JointId id, bool enableSpring ) { enable_spring( id, enableSpring ); }
bool b2WheelJoint_IsSpringEnabled( b2JointId id ) { return joint_read( id )->enableSpring != 0; }
void b2WheelJoint_SetSpringHertz( b2JointId id, float hertz ) { joint_write( id )->hertz = hertz; }
float b2WheelJoint_GetSpringHertz( b2JointId id ) { return joint_read( id )->hertz; }
void b2WheelJoint_SetSpringDampingRatio( b2JointId id, float dampingRatio ) { joint_write( id )->dampingRatio = dampingRatio; }
float b2WheelJoint_GetSpringDampingRatio( b2JointId id ) { return joint_read( id )->dampingRatio; }
void b2WheelJoint_EnableLimit( b2JointId id, bool enableLimit ) { enable_limit( id, enableLimit ); }
bool b2WheelJoint_IsLimitEnabled( b2JointId id ) { return joint_read( id )->enableLimit != 0; }
float b2WheelJoint_GetLowerLimit( b2JointId id ) { return joint_read( id )->lower; }
float b2WheelJoint_GetUpperLimit( b2JointId id ) { return joint_read( id )->upper; }
void b2WheelJoint_SetLimits( b2JointId id, float lower, float upper ) { set_limits( id, lower, upper ); }
void b2WheelJoint_EnableMotor( b2JointId id, bool enableMotor ) { enable_motor( id, enableMotor ); }
bool b2WheelJoint_IsMotorEnabled( b2JointId id ) { return joint_read( id )->enableMotor != 0; }
void b2WheelJoint_SetMotorSpeed( b2JointId id, float motorSpeed ) { joint_write( id )->motorSpeed = motorSpeed; }
float b2WheelJoint_GetMotorSpeed( b2JointId id ) { return joint_read( id )->motorSpeed; }
void b2WheelJoint_SetMaxMotorTorque( b2JointId id, float torque ) { joint_write( id )->maxMotor = torque; }
float b2WheelJoint_GetMaxMotorTorque( b2JointId id ) { return joint_read( id )->maxMotor; }
float b2WheelJoint_GetMotorTorque( b2JointId id ) { return joint_world( id )->inv_h * joint_read( id )->motorImpulse; }
