/*
 * b2o_joint.c -- joints of every type for the plain-C oracle (TEST INFRASTRUCTURE):
 * default definitions, creation, the joint API, and each type's prepare, warm start and
 * solve.
 *
 * Restates the reference: creation src/joint.c:331-655 (the shared record is
 * o_create_joint in b2o_world.c, src/joint.c:140-288); the generic queries
 * src/joint.c:771-973; the type dispatch src/joint.c:983-1108; and per type
 *   distance   src/distance_joint.c:18-495
 *   motor      src/motor_joint.c:14-273
 *   mouse      src/mouse_joint.c:14-230
 *   prismatic  src/prismatic_joint.c:16-551
 *   revolute   src/revolute_joint.c:16-470
 *   weld       src/weld_joint.c:16-307
 *   wheel      src/wheel_joint.c:16-506
 * expression by expression in b2r (float, or double in the FP64 build).
 */
#include "b2o.h"

#include <string.h>

#define O_COOKIE 1152023

/* ------------------------------------------------------------ default definitions */
b2DistanceJointDef b2DefaultDistanceJointDef( void )
{
	b2DistanceJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.length = 1.0f;
	d.maxLength = 100000.0f;
	d.internalValue = O_COOKIE;
	return d;
}

b2MotorJointDef b2DefaultMotorJointDef( void )
{
	b2MotorJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.maxForce = 1.0f;
	d.maxTorque = 1.0f;
	d.correctionFactor = 0.3f;
	d.internalValue = O_COOKIE;
	return d;
}

b2MouseJointDef b2DefaultMouseJointDef( void )
{
	b2MouseJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.hertz = 4.0f;
	d.dampingRatio = 1.0f;
	d.maxForce = 1.0f;
	d.internalValue = O_COOKIE;
	return d;
}

b2PrismaticJointDef b2DefaultPrismaticJointDef( void )
{
	b2PrismaticJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.localAxisA.x = 1.0f;
	d.internalValue = O_COOKIE;
	return d;
}

b2RevoluteJointDef b2DefaultRevoluteJointDef( void )
{
	b2RevoluteJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.drawSize = 0.25f;
	d.internalValue = O_COOKIE;
	return d;
}

b2WeldJointDef b2DefaultWeldJointDef( void )
{
	b2WeldJointDef d;
	memset( &d, 0, sizeof( d ) );
	d.internalValue = O_COOKIE;
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
	d.internalValue = O_COOKIE;
	return d;
}

/* ------------------------------------------------------------ helpers */
static oWorld* jworld( b2JointId id ) { return o_world_index( id.world0 ); }
static oJoint* jget( b2JointId id ) { return jworld( id )->joints + ( id.index1 - 1 ); }
static oVec ovf2( b2Vec2 v ) { return ov( v.x, v.y ); }
static b2Vec2 fvec( oVec v )
{
	b2Vec2 r = { (float)v.x, (float)v.y };
	return r;
}
static oVec oleft( oVec v ) { return ov( -v.y, v.x ); }

/* b2Solve22 / b2GetInverse22 / b2MulMV (reference include/box2d/math_functions.h:461-499) */
static oVec osolve22( oMat22 A, oVec b )
{
	b2r a11 = A.cx.x, a12 = A.cy.x, a21 = A.cx.y, a22 = A.cy.y;
	b2r det = a11 * a22 - a12 * a21;
	if ( det != R( 0 ) )
		det = R( 1 ) / det;
	return ov( det * ( a22 * b.x - a12 * b.y ), det * ( a11 * b.y - a21 * b.x ) );
}

static oMat22 oinverse22( oMat22 A )
{
	b2r a = A.cx.x, b = A.cy.x, c = A.cx.y, d = A.cy.y;
	b2r det = a * d - b * c;
	if ( det != R( 0 ) )
		det = R( 1 ) / det;
	oMat22 B;
	B.cx = ov( det * d, -det * c );
	B.cy = ov( -det * b, det * a );
	return B;
}

static oVec omulmv( oMat22 A, oVec v ) { return ov( A.cx.x * v.x + A.cy.x * v.y, A.cx.y * v.x + A.cy.y * v.y ); }

static oXf body_xf( oWorld* w, int bodyId ) { return w->bodies[bodyId].xf; }

static oVec xf_point( oXf t, oVec p ) { return oadd( orotate( t.q, p ), t.p ); }

static b2JointId finish( b2JointId id, bool collideConnected )
{
	if ( collideConnected == false )
	{
		oJoint* j = jget( id );
		o_destroy_contacts_between( jworld( id ), j->bodyIdA, j->bodyIdB );
	}
	return id;
}

/* ------------------------------------------------------------ creation */
b2JointId b2CreateDistanceJoint( b2WorldId worldId, const b2DistanceJointDef* def )
{
	b2JointId id;
	oJoint* j = o_create_joint( worldId, def->bodyIdA, def->bodyIdB, b2_distanceJoint, def->collideConnected, def->userData, &id );
	if ( j == NULL )
		return id;
	j->localAnchorA = ovf2( def->localAnchorA );
	j->localAnchorB = ovf2( def->localAnchorB );
	oDistanceJoint* d = &j->distance;
	d->length = omax( def->length, O_LINEAR_SLOP );
	d->hertz = def->hertz;
	d->dampingRatio = def->dampingRatio;
	d->minLength = omax( def->minLength, O_LINEAR_SLOP );
	d->maxLength = omax( def->minLength, def->maxLength );
	d->maxMotorForce = def->maxMotorForce;
	d->motorSpeed = def->motorSpeed;
	d->enableSpring = def->enableSpring;
	d->enableLimit = def->enableLimit;
	d->enableMotor = def->enableMotor;
	return finish( id, def->collideConnected );
}

b2JointId b2CreateMotorJoint( b2WorldId worldId, const b2MotorJointDef* def )
{
	b2JointId id;
	oJoint* j = o_create_joint( worldId, def->bodyIdA, def->bodyIdB, b2_motorJoint, def->collideConnected, def->userData, &id );
	if ( j == NULL )
		return id;
	oMotorJoint* m = &j->motor;
	m->linearOffset = ovf2( def->linearOffset );
	m->angularOffset = def->angularOffset;
	m->maxForce = def->maxForce;
	m->maxTorque = def->maxTorque;
	m->correctionFactor = oclamp( def->correctionFactor, R( 0 ), R( 1 ) );
	return finish( id, def->collideConnected );
}

b2JointId b2CreateMouseJoint( b2WorldId worldId, const b2MouseJointDef* def )
{
	oWorld* w = o_world( worldId );
	oXf xfA = body_xf( w, def->bodyIdA.index1 - 1 );
	oXf xfB = body_xf( w, def->bodyIdB.index1 - 1 );
	b2JointId id;
	oJoint* j = o_create_joint( worldId, def->bodyIdA, def->bodyIdB, b2_mouseJoint, def->collideConnected, def->userData, &id );
	if ( j == NULL )
		return id;
	oVec target = ovf2( def->target );
	j->localAnchorA = oinvrotate( xfA.q, osub( target, xfA.p ) );
	j->localAnchorB = oinvrotate( xfB.q, osub( target, xfB.p ) );
	oMouseJoint* m = &j->mouse;
	m->targetA = target;
	m->hertz = def->hertz;
	m->dampingRatio = def->dampingRatio;
	m->maxForce = def->maxForce;
	return id;
}

b2JointId b2CreatePrismaticJoint( b2WorldId worldId, const b2PrismaticJointDef* def )
{
	b2JointId id;
	oJoint* j = o_create_joint( worldId, def->bodyIdA, def->bodyIdB, b2_prismaticJoint, def->collideConnected, def->userData, &id );
	if ( j == NULL )
		return id;
	j->localAnchorA = ovf2( def->localAnchorA );
	j->localAnchorB = ovf2( def->localAnchorB );
	oPrismaticJoint* p = &j->prismatic;
	p->localAxisA = onormalize( ovf2( def->localAxisA ) );
	p->referenceAngle = def->referenceAngle;
	p->hertz = def->hertz;
	p->dampingRatio = def->dampingRatio;
	p->lowerTranslation = def->lowerTranslation;
	p->upperTranslation = def->upperTranslation;
	p->maxMotorForce = def->maxMotorForce;
	p->motorSpeed = def->motorSpeed;
	p->enableSpring = def->enableSpring;
	p->enableLimit = def->enableLimit;
	p->enableMotor = def->enableMotor;
	return finish( id, def->collideConnected );
}

b2JointId b2CreateRevoluteJoint( b2WorldId worldId, const b2RevoluteJointDef* def )
{
	b2JointId id;
	oJoint* j = o_create_joint( worldId, def->bodyIdA, def->bodyIdB, b2_revoluteJoint, def->collideConnected, def->userData, &id );
	if ( j == NULL )
		return id;
	j->localAnchorA = ovf2( def->localAnchorA );
	j->localAnchorB = ovf2( def->localAnchorB );
	oRevoluteJoint* r = &j->revolute;
	r->referenceAngle = oclamp( def->referenceAngle, -O_PI, O_PI );
	r->hertz = def->hertz;
	r->dampingRatio = def->dampingRatio;
	r->lowerAngle = omin( def->lowerAngle, def->upperAngle );
	r->upperAngle = omax( def->lowerAngle, def->upperAngle );
	r->lowerAngle = oclamp( r->lowerAngle, -O_PI, O_PI );
	r->upperAngle = oclamp( r->upperAngle, -O_PI, O_PI );
	r->maxMotorTorque = def->maxMotorTorque;
	r->motorSpeed = def->motorSpeed;
	r->enableSpring = def->enableSpring;
	r->enableLimit = def->enableLimit;
	r->enableMotor = def->enableMotor;
	return finish( id, def->collideConnected );
}

b2JointId b2CreateWeldJoint( b2WorldId worldId, const b2WeldJointDef* def )
{
	b2JointId id;
	oJoint* j = o_create_joint( worldId, def->bodyIdA, def->bodyIdB, b2_weldJoint, def->collideConnected, def->userData, &id );
	if ( j == NULL )
		return id;
	j->localAnchorA = ovf2( def->localAnchorA );
	j->localAnchorB = ovf2( def->localAnchorB );
	oWeldJoint* wj = &j->weld;
	wj->referenceAngle = def->referenceAngle;
	wj->linearHertz = def->linearHertz;
	wj->linearDampingRatio = def->linearDampingRatio;
	wj->angularHertz = def->angularHertz;
	wj->angularDampingRatio = def->angularDampingRatio;
	return finish( id, def->collideConnected );
}

b2JointId b2CreateWheelJoint( b2WorldId worldId, const b2WheelJointDef* def )
{
	b2JointId id;
	oJoint* j = o_create_joint( worldId, def->bodyIdA, def->bodyIdB, b2_wheelJoint, def->collideConnected, def->userData, &id );
	if ( j == NULL )
		return id;
	j->localAnchorA = ovf2( def->localAnchorA );
	j->localAnchorB = ovf2( def->localAnchorB );
	oWheelJoint* h = &j->wheel;
	h->localAxisA = onormalize( ovf2( def->localAxisA ) );
	h->lowerTranslation = def->lowerTranslation;
	h->upperTranslation = def->upperTranslation;
	h->maxMotorTorque = def->maxMotorTorque;
	h->motorSpeed = def->motorSpeed;
	h->hertz = def->hertz;
	h->dampingRatio = def->dampingRatio;
	h->enableSpring = def->enableSpring;
	h->enableLimit = def->enableLimit;
	h->enableMotor = def->enableMotor;
	return finish( id, def->collideConnected );
}

/* ------------------------------------------------------------ generic queries */
b2JointType b2Joint_GetType( b2JointId id ) { return jget( id )->type; }
b2BodyId b2Joint_GetBodyA( b2JointId id )
{
	oJoint* j = jget( id );
	b2BodyId b = { j->bodyIdA + 1, id.world0, jworld( id )->bodies[j->bodyIdA].revision };
	return b;
}
b2BodyId b2Joint_GetBodyB( b2JointId id )
{
	oJoint* j = jget( id );
	b2BodyId b = { j->bodyIdB + 1, id.world0, jworld( id )->bodies[j->bodyIdB].revision };
	return b;
}
b2Vec2 b2Joint_GetLocalAnchorA( b2JointId id ) { return fvec( jget( id )->localAnchorA ); }
b2Vec2 b2Joint_GetLocalAnchorB( b2JointId id ) { return fvec( jget( id )->localAnchorB ); }

void b2Joint_SetCollideConnected( b2JointId id, bool shouldCollide )
{
	oWorld* w = jworld( id );
	if ( w->locked )
		return;
	oJoint* j = jget( id );
	if ( j->collideConnected == shouldCollide )
		return;
	j->collideConnected = shouldCollide;
	oBody* a = w->bodies + j->edges[0].bodyId;
	oBody* b = w->bodies + j->edges[1].bodyId;
	if ( shouldCollide )
	{
		int shapeId = a->shapeCount < b->shapeCount ? a->headShape : b->headShape;
		while ( shapeId != O_NULL )
		{
			oShape* s = w->shapes + shapeId;
			if ( s->proxyKey != O_NULL )
				o_buffer_move( w, s->proxyKey );
			shapeId = s->next;
		}
	}
	else
		o_destroy_contacts_between( w, a->id, b->id );
}

bool b2Joint_GetCollideConnected( b2JointId id ) { return jget( id )->collideConnected; }
void b2Joint_SetUserData( b2JointId id, void* userData ) { jget( id )->userData = userData; }
void* b2Joint_GetUserData( b2JointId id ) { return jget( id )->userData; }
/* reference src/joint.c:874-888 */
void b2Joint_WakeBodies( b2JointId id )
{
	oWorld* w = jworld( id );
	if ( w->locked )
		return;
	oJoint* j = jget( id );
	o_wake_body( w, w->bodies + j->edges[0].bodyId );
	o_wake_body( w, w->bodies + j->edges[1].bodyId );
}

b2Vec2 b2Joint_GetConstraintForce( b2JointId id )
{
	oWorld* w = jworld( id );
	oJoint* j = jget( id );
	b2r inv_h = w->inv_h;
	switch ( j->type )
	{
		case b2_distanceJoint:
		{
			oDistanceJoint* d = &j->distance;
			oVec pA = xf_point( body_xf( w, j->bodyIdA ), j->localAnchorA );
			oVec pB = xf_point( body_xf( w, j->bodyIdB ), j->localAnchorB );
			oVec axis = onormalize( osub( pB, pA ) );
			b2r force = ( d->impulse + d->lowerImpulse - d->upperImpulse + d->motorImpulse ) * inv_h;
			return fvec( omulsv( force, axis ) );
		}
		case b2_motorJoint:
			return fvec( omulsv( inv_h, j->motor.linearImpulse ) );
		case b2_mouseJoint:
			return fvec( omulsv( inv_h, j->mouse.linearImpulse ) );
		case b2_prismaticJoint:
		{
			oPrismaticJoint* p = &j->prismatic;
			oVec axisA = orotate( body_xf( w, j->bodyIdA ).q, p->localAxisA );
			oVec perpA = oleft( axisA );
			b2r perpForce = inv_h * p->impulse.x;
			b2r axialForce = inv_h * ( p->motorImpulse + p->lowerImpulse - p->upperImpulse );
			return fvec( oadd( omulsv( perpForce, perpA ), omulsv( axialForce, axisA ) ) );
		}
		case b2_revoluteJoint:
			return fvec( omulsv( inv_h, j->revolute.linearImpulse ) );
		case b2_weldJoint:
			return fvec( omulsv( inv_h, j->weld.linearImpulse ) );
		case b2_wheelJoint:
		{
			oWheelJoint* h = &j->wheel;
			oVec perpA = oleft( h->axisA );
			b2r perpForce = inv_h * h->perpImpulse;
			b2r axialForce = inv_h * ( h->springImpulse + h->lowerImpulse - h->upperImpulse );
			return fvec( oadd( omulsv( perpForce, perpA ), omulsv( axialForce, h->axisA ) ) );
		}
		default:
		{
			b2Vec2 z = { 0.0f, 0.0f };
			return z;
		}
	}
}

float b2Joint_GetConstraintTorque( b2JointId id )
{
	oWorld* w = jworld( id );
	oJoint* j = jget( id );
	b2r inv_h = w->inv_h;
	switch ( j->type )
	{
		case b2_motorJoint:
			return (float)( inv_h * j->motor.angularImpulse );
		case b2_mouseJoint:
			return (float)( inv_h * j->mouse.angularImpulse );
		case b2_prismaticJoint:
			return (float)( inv_h * j->prismatic.impulse.y );
		case b2_revoluteJoint:
			return (float)( inv_h * ( j->revolute.motorImpulse + j->revolute.lowerImpulse - j->revolute.upperImpulse ) );
		case b2_weldJoint:
			return (float)( inv_h * j->weld.angularImpulse );
		case b2_wheelJoint:
			return (float)( inv_h * j->wheel.motorImpulse );
		default:
			return 0.0f;
	}
}

/* ------------------------------------------------------------ distance joint API */
#define DJ( id ) ( &jget( id )->distance )
void b2DistanceJoint_SetLength( b2JointId id, float length )
{
	oDistanceJoint* d = DJ( id );
	d->length = oclamp( length, O_LINEAR_SLOP, O_HUGE );
	d->impulse = 0;
	d->lowerImpulse = 0;
	d->upperImpulse = 0;
}
float b2DistanceJoint_GetLength( b2JointId id ) { return (float)DJ( id )->length; }
void b2DistanceJoint_EnableSpring( b2JointId id, bool f ) { DJ( id )->enableSpring = f; }
bool b2DistanceJoint_IsSpringEnabled( b2JointId id ) { return DJ( id )->enableSpring; }
void b2DistanceJoint_SetSpringHertz( b2JointId id, float hertz ) { DJ( id )->hertz = hertz; }
void b2DistanceJoint_SetSpringDampingRatio( b2JointId id, float zeta ) { DJ( id )->dampingRatio = zeta; }
float b2DistanceJoint_GetHertz( b2JointId id ) { return (float)DJ( id )->hertz; }
float b2DistanceJoint_GetDampingRatio( b2JointId id ) { return (float)DJ( id )->dampingRatio; }
void b2DistanceJoint_EnableLimit( b2JointId id, bool f ) { DJ( id )->enableLimit = f; }
bool b2DistanceJoint_IsLimitEnabled( b2JointId id ) { return DJ( id )->enableLimit; }
void b2DistanceJoint_SetLengthRange( b2JointId id, float minLength, float maxLength )
{
	oDistanceJoint* d = DJ( id );
	b2r lo = oclamp( minLength, O_LINEAR_SLOP, O_HUGE );
	b2r hi = oclamp( maxLength, O_LINEAR_SLOP, O_HUGE );
	d->minLength = omin( lo, hi );
	d->maxLength = omax( lo, hi );
	d->impulse = 0;
	d->lowerImpulse = 0;
	d->upperImpulse = 0;
}
float b2DistanceJoint_GetMinLength( b2JointId id ) { return (float)DJ( id )->minLength; }
float b2DistanceJoint_GetMaxLength( b2JointId id ) { return (float)DJ( id )->maxLength; }
float b2DistanceJoint_GetCurrentLength( b2JointId id )
{
	oWorld* w = jworld( id );
	oJoint* j = jget( id );
	oVec pA = xf_point( body_xf( w, j->bodyIdA ), j->localAnchorA );
	oVec pB = xf_point( body_xf( w, j->bodyIdB ), j->localAnchorB );
	return (float)olen( osub( pB, pA ) );
}
void b2DistanceJoint_EnableMotor( b2JointId id, bool f )
{
	oDistanceJoint* d = DJ( id );
	if ( f != d->enableMotor )
	{
		d->enableMotor = f;
		d->motorImpulse = 0;
	}
}
bool b2DistanceJoint_IsMotorEnabled( b2JointId id ) { return DJ( id )->enableMotor; }
void b2DistanceJoint_SetMotorSpeed( b2JointId id, float s ) { DJ( id )->motorSpeed = s; }
float b2DistanceJoint_GetMotorSpeed( b2JointId id ) { return (float)DJ( id )->motorSpeed; }
float b2DistanceJoint_GetMotorForce( b2JointId id ) { return (float)( jworld( id )->inv_h * DJ( id )->motorImpulse ); }
void b2DistanceJoint_SetMaxMotorForce( b2JointId id, float f ) { DJ( id )->maxMotorForce = f; }
float b2DistanceJoint_GetMaxMotorForce( b2JointId id ) { return (float)DJ( id )->maxMotorForce; }

/* ------------------------------------------------------------ motor joint API */
#define MJ( id ) ( &jget( id )->motor )
void b2MotorJoint_SetLinearOffset( b2JointId id, b2Vec2 v ) { MJ( id )->linearOffset = ovf2( v ); }
b2Vec2 b2MotorJoint_GetLinearOffset( b2JointId id ) { return fvec( MJ( id )->linearOffset ); }
void b2MotorJoint_SetAngularOffset( b2JointId id, float a ) { MJ( id )->angularOffset = oclamp( a, -O_PI, O_PI ); }
float b2MotorJoint_GetAngularOffset( b2JointId id ) { return (float)MJ( id )->angularOffset; }
void b2MotorJoint_SetMaxForce( b2JointId id, float f ) { MJ( id )->maxForce = omax( R( 0 ), f ); }
float b2MotorJoint_GetMaxForce( b2JointId id ) { return (float)MJ( id )->maxForce; }
void b2MotorJoint_SetMaxTorque( b2JointId id, float t ) { MJ( id )->maxTorque = omax( R( 0 ), t ); }
float b2MotorJoint_GetMaxTorque( b2JointId id ) { return (float)MJ( id )->maxTorque; }
void b2MotorJoint_SetCorrectionFactor( b2JointId id, float c ) { MJ( id )->correctionFactor = oclamp( c, R( 0 ), R( 1 ) ); }
float b2MotorJoint_GetCorrectionFactor( b2JointId id ) { return (float)MJ( id )->correctionFactor; }

/* ------------------------------------------------------------ mouse joint API */
#define OJ( id ) ( &jget( id )->mouse )
void b2MouseJoint_SetTarget( b2JointId id, b2Vec2 t ) { OJ( id )->targetA = ovf2( t ); }
b2Vec2 b2MouseJoint_GetTarget( b2JointId id ) { return fvec( OJ( id )->targetA ); }
void b2MouseJoint_SetSpringHertz( b2JointId id, float h ) { OJ( id )->hertz = h; }
float b2MouseJoint_GetSpringHertz( b2JointId id ) { return (float)OJ( id )->hertz; }
void b2MouseJoint_SetSpringDampingRatio( b2JointId id, float z ) { OJ( id )->dampingRatio = z; }
float b2MouseJoint_GetSpringDampingRatio( b2JointId id ) { return (float)OJ( id )->dampingRatio; }
void b2MouseJoint_SetMaxForce( b2JointId id, float f ) { OJ( id )->maxForce = f; }
float b2MouseJoint_GetMaxForce( b2JointId id ) { return (float)OJ( id )->maxForce; }

/* ------------------------------------------------------------ prismatic joint API */
#define PJ( id ) ( &jget( id )->prismatic )
void b2PrismaticJoint_EnableSpring( b2JointId id, bool f )
{
	oPrismaticJoint* p = PJ( id );
	if ( f != p->enableSpring )
	{
		p->enableSpring = f;
		p->springImpulse = 0;
	}
}
bool b2PrismaticJoint_IsSpringEnabled( b2JointId id ) { return PJ( id )->enableSpring; }
void b2PrismaticJoint_SetSpringHertz( b2JointId id, float h ) { PJ( id )->hertz = h; }
float b2PrismaticJoint_GetSpringHertz( b2JointId id ) { return (float)PJ( id )->hertz; }
void b2PrismaticJoint_SetSpringDampingRatio( b2JointId id, float z ) { PJ( id )->dampingRatio = z; }
float b2PrismaticJoint_GetSpringDampingRatio( b2JointId id ) { return (float)PJ( id )->dampingRatio; }
void b2PrismaticJoint_EnableLimit( b2JointId id, bool f )
{
	oPrismaticJoint* p = PJ( id );
	if ( f != p->enableLimit )
	{
		p->enableLimit = f;
		p->lowerImpulse = 0;
		p->upperImpulse = 0;
	}
}
bool b2PrismaticJoint_IsLimitEnabled( b2JointId id ) { return PJ( id )->enableLimit; }
float b2PrismaticJoint_GetLowerLimit( b2JointId id ) { return (float)PJ( id )->lowerTranslation; }
float b2PrismaticJoint_GetUpperLimit( b2JointId id ) { return (float)PJ( id )->upperTranslation; }
void b2PrismaticJoint_SetLimits( b2JointId id, float lower, float upper )
{
	oPrismaticJoint* p = PJ( id );
	if ( lower != p->lowerTranslation || upper != p->upperTranslation )
	{
		p->lowerTranslation = omin( lower, upper );
		p->upperTranslation = omax( lower, upper );
		p->lowerImpulse = 0;
		p->upperImpulse = 0;
	}
}
void b2PrismaticJoint_EnableMotor( b2JointId id, bool f )
{
	oPrismaticJoint* p = PJ( id );
	if ( f != p->enableMotor )
	{
		p->enableMotor = f;
		p->motorImpulse = 0;
	}
}
bool b2PrismaticJoint_IsMotorEnabled( b2JointId id ) { return PJ( id )->enableMotor; }
void b2PrismaticJoint_SetMotorSpeed( b2JointId id, float s ) { PJ( id )->motorSpeed = s; }
float b2PrismaticJoint_GetMotorSpeed( b2JointId id ) { return (float)PJ( id )->motorSpeed; }
void b2PrismaticJoint_SetMaxMotorForce( b2JointId id, float f ) { PJ( id )->maxMotorForce = f; }
float b2PrismaticJoint_GetMaxMotorForce( b2JointId id ) { return (float)PJ( id )->maxMotorForce; }
float b2PrismaticJoint_GetMotorForce( b2JointId id ) { return (float)( jworld( id )->inv_h * PJ( id )->motorImpulse ); }

/* ------------------------------------------------------------ revolute joint API */
#define RJ( id ) ( &jget( id )->revolute )
void b2RevoluteJoint_EnableSpring( b2JointId id, bool f )
{
	oRevoluteJoint* r = RJ( id );
	if ( f != r->enableSpring )
	{
		r->enableSpring = f;
		r->springImpulse = 0;
	}
}
bool b2RevoluteJoint_IsSpringEnabled( b2JointId id ) { return RJ( id )->enableSpring; }
void b2RevoluteJoint_SetSpringHertz( b2JointId id, float h ) { RJ( id )->hertz = h; }
float b2RevoluteJoint_GetSpringHertz( b2JointId id ) { return (float)RJ( id )->hertz; }
void b2RevoluteJoint_SetSpringDampingRatio( b2JointId id, float z ) { RJ( id )->dampingRatio = z; }
float b2RevoluteJoint_GetSpringDampingRatio( b2JointId id ) { return (float)RJ( id )->dampingRatio; }
float b2RevoluteJoint_GetAngle( b2JointId id )
{
	oWorld* w = jworld( id );
	oJoint* j = jget( id );
	b2r angle = orelangle( body_xf( w, j->bodyIdB ).q, body_xf( w, j->bodyIdA ).q ) - j->revolute.referenceAngle;
	return (float)ounwind( angle );
}
void b2RevoluteJoint_EnableLimit( b2JointId id, bool f )
{
	oRevoluteJoint* r = RJ( id );
	if ( f != r->enableLimit )
	{
		r->enableLimit = f;
		r->lowerImpulse = 0;
		r->upperImpulse = 0;
	}
}
bool b2RevoluteJoint_IsLimitEnabled( b2JointId id ) { return RJ( id )->enableLimit; }
float b2RevoluteJoint_GetLowerLimit( b2JointId id ) { return (float)RJ( id )->lowerAngle; }
float b2RevoluteJoint_GetUpperLimit( b2JointId id ) { return (float)RJ( id )->upperAngle; }
void b2RevoluteJoint_SetLimits( b2JointId id, float lower, float upper )
{
	oRevoluteJoint* r = RJ( id );
	if ( lower != r->lowerAngle || upper != r->upperAngle )
	{
		r->lowerAngle = omin( lower, upper );
		r->upperAngle = omax( lower, upper );
		r->lowerImpulse = 0;
		r->upperImpulse = 0;
	}
}
void b2RevoluteJoint_EnableMotor( b2JointId id, bool f )
{
	oRevoluteJoint* r = RJ( id );
	if ( f != r->enableMotor )
	{
		r->enableMotor = f;
		r->motorImpulse = 0;
	}
}
bool b2RevoluteJoint_IsMotorEnabled( b2JointId id ) { return RJ( id )->enableMotor; }
void b2RevoluteJoint_SetMotorSpeed( b2JointId id, float s ) { RJ( id )->motorSpeed = s; }
float b2RevoluteJoint_GetMotorSpeed( b2JointId id ) { return (float)RJ( id )->motorSpeed; }
float b2RevoluteJoint_GetMotorTorque( b2JointId id ) { return (float)( jworld( id )->inv_h * RJ( id )->motorImpulse ); }
void b2RevoluteJoint_SetMaxMotorTorque( b2JointId id, float t ) { RJ( id )->maxMotorTorque = t; }
float b2RevoluteJoint_GetMaxMotorTorque( b2JointId id ) { return (float)RJ( id )->maxMotorTorque; }

/* ------------------------------------------------------------ weld joint API */
#define WJ( id ) ( &jget( id )->weld )
void b2WeldJoint_SetLinearHertz( b2JointId id, float h ) { WJ( id )->linearHertz = h; }
float b2WeldJoint_GetLinearHertz( b2JointId id ) { return (float)WJ( id )->linearHertz; }
void b2WeldJoint_SetLinearDampingRatio( b2JointId id, float z ) { WJ( id )->linearDampingRatio = z; }
float b2WeldJoint_GetLinearDampingRatio( b2JointId id ) { return (float)WJ( id )->linearDampingRatio; }
void b2WeldJoint_SetAngularHertz( b2JointId id, float h ) { WJ( id )->angularHertz = h; }
float b2WeldJoint_GetAngularHertz( b2JointId id ) { return (float)WJ( id )->angularHertz; }
void b2WeldJoint_SetAngularDampingRatio( b2JointId id, float z ) { WJ( id )->angularDampingRatio = z; }
float b2WeldJoint_GetAngularDampingRatio( b2JointId id ) { return (float)WJ( id )->angularDampingRatio; }

/* ------------------------------------------------------------ wheel joint API */
#define HJ( id ) ( &jget( id )->wheel )
void b2WheelJoint_EnableSpring( b2JointId id, bool f )
{
	oWheelJoint* h = HJ( id );
	if ( f != h->enableSpring )
	{
		h->enableSpring = f;
		h->springImpulse = 0;
	}
}
bool b2WheelJoint_IsSpringEnabled( b2JointId id ) { return HJ( id )->enableSpring; }
void b2WheelJoint_SetSpringHertz( b2JointId id, float x ) { HJ( id )->hertz = x; }
float b2WheelJoint_GetSpringHertz( b2JointId id ) { return (float)HJ( id )->hertz; }
void b2WheelJoint_SetSpringDampingRatio( b2JointId id, float z ) { HJ( id )->dampingRatio = z; }
float b2WheelJoint_GetSpringDampingRatio( b2JointId id ) { return (float)HJ( id )->dampingRatio; }
void b2WheelJoint_EnableLimit( b2JointId id, bool f )
{
	oWheelJoint* h = HJ( id );
	if ( h->enableLimit != f )
	{
		h->lowerImpulse = 0;
		h->upperImpulse = 0;
		h->enableLimit = f;
	}
}
bool b2WheelJoint_IsLimitEnabled( b2JointId id ) { return HJ( id )->enableLimit; }
float b2WheelJoint_GetLowerLimit( b2JointId id ) { return (float)HJ( id )->lowerTranslation; }
float b2WheelJoint_GetUpperLimit( b2JointId id ) { return (float)HJ( id )->upperTranslation; }
void b2WheelJoint_SetLimits( b2JointId id, float lower, float upper )
{
	oWheelJoint* h = HJ( id );
	if ( lower != h->lowerTranslation || upper != h->upperTranslation )
	{
		h->lowerTranslation = omin( lower, upper );
		h->upperTranslation = omax( lower, upper );
		h->lowerImpulse = 0;
		h->upperImpulse = 0;
	}
}
void b2WheelJoint_EnableMotor( b2JointId id, bool f )
{
	oWheelJoint* h = HJ( id );
	if ( h->enableMotor != f )
	{
		h->motorImpulse = 0;
		h->enableMotor = f;
	}
}
bool b2WheelJoint_IsMotorEnabled( b2JointId id ) { return HJ( id )->enableMotor; }
void b2WheelJoint_SetMotorSpeed( b2JointId id, float s ) { HJ( id )->motorSpeed = s; }
float b2WheelJoint_GetMotorSpeed( b2JointId id ) { return (float)HJ( id )->motorSpeed; }
void b2WheelJoint_SetMaxMotorTorque( b2JointId id, float t ) { HJ( id )->maxMotorTorque = t; }
float b2WheelJoint_GetMaxMotorTorque( b2JointId id ) { return (float)HJ( id )->maxMotorTorque; }
float b2WheelJoint_GetMotorTorque( b2JointId id ) { return (float)( jworld( id )->inv_h * HJ( id )->motorImpulse ); }

/* ------------------------------------------------------------ prepare */
void o_prepare_joint( oWorld* w, const oStep* st, oJoint* j )
{
	oBody* a = w->bodies + j->bodyIdA;
	oBody* b = w->bodies + j->bodyIdB;
	b2r mA = a->invMass, iA = a->invI, mB = b->invMass, iB = b->invI;
	j->indexA = a->awakeIndex != O_NULL ? a->id : O_NULL;
	j->indexB = b->awakeIndex != O_NULL ? b->id : O_NULL;
	bool warm = st->enableWarmStarting;

	if ( j->type == b2_mouseJoint )
	{
		/* src/mouse_joint.c:77-135 */
		oMouseJoint* m = &j->mouse;
		j->invMassB = mB;
		j->invIB = iB;
		m->anchorB = orotate( b->xf.q, osub( j->localAnchorB, b->localCenter ) );
		m->linearSoftness = o_make_soft( m->hertz, m->dampingRatio, st->h );
		m->angularSoftness = o_make_soft( R( 0.5f ), R( 0.1f ), st->h );
		oVec rB = m->anchorB;
		oMat22 K;
		K.cx.x = mB + iB * rB.y * rB.y;
		K.cx.y = -iB * rB.x * rB.y;
		K.cy.x = K.cx.y;
		K.cy.y = mB + iB * rB.x * rB.x;
		m->linearMass = oinverse22( K );
		m->deltaCenter = osub( b->center, m->targetA );
		if ( warm == false )
		{
			m->linearImpulse = ov( 0, 0 );
			m->angularImpulse = 0;
		}
		return;
	}

	j->invMassA = mA;
	j->invMassB = mB;
	j->invIA = iA;
	j->invIB = iB;
	oVec anchorA = orotate( a->xf.q, osub( j->localAnchorA, a->localCenter ) );
	oVec anchorB = orotate( b->xf.q, osub( j->localAnchorB, b->localCenter ) );
	oVec deltaCenter = osub( b->center, a->center );

	switch ( j->type )
	{
		case b2_distanceJoint:
		{
			/* src/distance_joint.c:213-283 */
			oDistanceJoint* d = &j->distance;
			d->anchorA = anchorA;
			d->anchorB = anchorB;
			d->deltaCenter = deltaCenter;
			oVec rA = anchorA, rB = anchorB;
			oVec separation = oadd( osub( rB, rA ), deltaCenter );
			oVec axis = onormalize( separation );
			b2r crA = ocross( rA, axis );
			b2r crB = ocross( rB, axis );
			b2r k = mA + mB + iA * crA * crA + iB * crB * crB;
			d->axialMass = k > R( 0 ) ? R( 1 ) / k : R( 0 );
			d->distanceSoftness = o_make_soft( d->hertz, d->dampingRatio, st->h );
			if ( warm == false )
			{
				d->impulse = 0;
				d->lowerImpulse = 0;
				d->upperImpulse = 0;
				d->motorImpulse = 0;
			}
			break;
		}
		case b2_motorJoint:
		{
			/* src/motor_joint.c:99-170 */
			oMotorJoint* m = &j->motor;
			m->anchorA = anchorA;
			m->anchorB = anchorB;
			m->deltaCenter = osub( osub( b->center, a->center ), m->linearOffset );
			m->deltaAngle = orelangle( b->xf.q, a->xf.q ) - m->angularOffset;
			m->deltaAngle = ounwind( m->deltaAngle );
			oVec rA = anchorA, rB = anchorB;
			oMat22 K;
			K.cx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
			K.cx.y = -rA.y * rA.x * iA - rB.y * rB.x * iB;
			K.cy.x = K.cx.y;
			K.cy.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
			m->linearMass = oinverse22( K );
			b2r ka = iA + iB;
			m->angularMass = ka > R( 0 ) ? R( 1 ) / ka : R( 0 );
			if ( warm == false )
			{
				m->linearImpulse = ov( 0, 0 );
				m->angularImpulse = 0;
			}
			break;
		}
		case b2_prismaticJoint:
		{
			/* src/prismatic_joint.c:212-289 */
			oPrismaticJoint* p = &j->prismatic;
			p->anchorA = anchorA;
			p->anchorB = anchorB;
			p->axisA = orotate( a->xf.q, p->localAxisA );
			p->deltaCenter = deltaCenter;
			p->deltaAngle = orelangle( b->xf.q, a->xf.q ) - p->referenceAngle;
			oVec rA = anchorA, rB = anchorB;
			oVec d = oadd( p->deltaCenter, osub( rB, rA ) );
			b2r a1 = ocross( oadd( d, rA ), p->axisA );
			b2r a2 = ocross( rB, p->axisA );
			b2r k = mA + mB + iA * a1 * a1 + iB * a2 * a2;
			p->axialMass = k > R( 0 ) ? R( 1 ) / k : R( 0 );
			p->springSoftness = o_make_soft( p->hertz, p->dampingRatio, st->h );
			if ( warm == false )
			{
				p->impulse = ov( 0, 0 );
				p->springImpulse = 0;
				p->motorImpulse = 0;
				p->lowerImpulse = 0;
				p->upperImpulse = 0;
			}
			break;
		}
		case b2_revoluteJoint:
		{
			/* src/revolute_joint.c:201-270 */
			oRevoluteJoint* r = &j->revolute;
			r->anchorA = anchorA;
			r->anchorB = anchorB;
			r->deltaCenter = deltaCenter;
			r->deltaAngle = orelangle( b->xf.q, a->xf.q ) - r->referenceAngle;
			r->deltaAngle = ounwind( r->deltaAngle );
			b2r k = iA + iB;
			r->axialMass = k > R( 0 ) ? R( 1 ) / k : R( 0 );
			r->springSoftness = o_make_soft( r->hertz, r->dampingRatio, st->h );
			if ( warm == false )
			{
				r->linearImpulse = ov( 0, 0 );
				r->springImpulse = 0;
				r->motorImpulse = 0;
				r->lowerImpulse = 0;
				r->upperImpulse = 0;
			}
			break;
		}
		case b2_weldJoint:
		{
			/* src/weld_joint.c:93-177 */
			oWeldJoint* wj = &j->weld;
			wj->anchorA = anchorA;
			wj->anchorB = anchorB;
			wj->deltaCenter = deltaCenter;
			wj->deltaAngle = orelangle( b->xf.q, a->xf.q ) - wj->referenceAngle;
			b2r ka = iA + iB;
			wj->axialMass = ka > R( 0 ) ? R( 1 ) / ka : R( 0 );
			wj->linearSoftness =
				wj->linearHertz == R( 0 ) ? st->jointSoft : o_make_soft( wj->linearHertz, wj->linearDampingRatio, st->h );
			wj->angularSoftness =
				wj->angularHertz == R( 0 ) ? st->jointSoft : o_make_soft( wj->angularHertz, wj->angularDampingRatio, st->h );
			if ( warm == false )
			{
				wj->linearImpulse = ov( 0, 0 );
				wj->angularImpulse = 0;
			}
			break;
		}
		case b2_wheelJoint:
		{
			/* src/wheel_joint.c:181-271 */
			oWheelJoint* h = &j->wheel;
			h->anchorA = anchorA;
			h->anchorB = anchorB;
			h->axisA = orotate( a->xf.q, h->localAxisA );
			h->deltaCenter = deltaCenter;
			oVec rA = anchorA, rB = anchorB;
			oVec d = oadd( h->deltaCenter, osub( rB, rA ) );
			oVec axisA = h->axisA;
			oVec perpA = oleft( axisA );
			b2r s1 = ocross( oadd( d, rA ), perpA );
			b2r s2 = ocross( rB, perpA );
			b2r kp = mA + mB + iA * s1 * s1 + iB * s2 * s2;
			h->perpMass = kp > R( 0 ) ? R( 1 ) / kp : R( 0 );
			b2r a1 = ocross( oadd( d, rA ), axisA );
			b2r a2 = ocross( rB, axisA );
			b2r ka = mA + mB + iA * a1 * a1 + iB * a2 * a2;
			h->axialMass = ka > R( 0 ) ? R( 1 ) / ka : R( 0 );
			h->springSoftness = o_make_soft( h->hertz, h->dampingRatio, st->h );
			b2r km = iA + iB;
			h->motorMass = km > R( 0 ) ? R( 1 ) / km : R( 0 );
			if ( warm == false )
			{
				h->perpImpulse = 0;
				h->springImpulse = 0;
				h->motorImpulse = 0;
				h->lowerImpulse = 0;
				h->upperImpulse = 0;
			}
			break;
		}
		default:
			break;
	}
}

/* ------------------------------------------------------------ warm start */
void o_warm_start_joint( oJoint* j, oState* sA, oState* sB )
{
	b2r mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	switch ( j->type )
	{
		case b2_distanceJoint:
		{
			oDistanceJoint* d = &j->distance;
			oVec rA = orotate( sA->dq, d->anchorA );
			oVec rB = orotate( sB->dq, d->anchorB );
			oVec ds = oadd( osub( sB->dp, sA->dp ), osub( rB, rA ) );
			oVec separation = oadd( d->deltaCenter, ds );
			oVec axis = onormalize( separation );
			b2r axialImpulse = d->impulse + d->lowerImpulse - d->upperImpulse + d->motorImpulse;
			oVec P = omulsv( axialImpulse, axis );
			sA->v = omulsub( sA->v, mA, P );
			sA->w -= iA * ocross( rA, P );
			sB->v = omuladd( sB->v, mB, P );
			sB->w += iB * ocross( rB, P );
			break;
		}
		case b2_motorJoint:
		{
			oMotorJoint* m = &j->motor;
			oVec rA = orotate( sA->dq, m->anchorA );
			oVec rB = orotate( sB->dq, m->anchorB );
			sA->v = omulsub( sA->v, mA, m->linearImpulse );
			sA->w -= iA * ( ocross( rA, m->linearImpulse ) + m->angularImpulse );
			sB->v = omuladd( sB->v, mB, m->linearImpulse );
			sB->w += iB * ( ocross( rB, m->linearImpulse ) + m->angularImpulse );
			break;
		}
		case b2_mouseJoint:
		{
			oMouseJoint* m = &j->mouse;
			oVec rB = orotate( sB->dq, m->anchorB );
			sB->v = omuladd( sB->v, mB, m->linearImpulse );
			sB->w += iB * ( ocross( rB, m->linearImpulse ) + m->angularImpulse );
			break;
		}
		case b2_prismaticJoint:
		{
			oPrismaticJoint* p = &j->prismatic;
			oVec rA = orotate( sA->dq, p->anchorA );
			oVec rB = orotate( sB->dq, p->anchorB );
			oVec d = oadd( oadd( osub( sB->dp, sA->dp ), p->deltaCenter ), osub( rB, rA ) );
			oVec axisA = orotate( sA->dq, p->axisA );
			b2r a1 = ocross( oadd( d, rA ), axisA );
			b2r a2 = ocross( rB, axisA );
			b2r axialImpulse = p->springImpulse + p->motorImpulse + p->lowerImpulse - p->upperImpulse;
			oVec perpA = oleft( axisA );
			b2r s1 = ocross( oadd( d, rA ), perpA );
			b2r s2 = ocross( rB, perpA );
			b2r perpImpulse = p->impulse.x;
			b2r angleImpulse = p->impulse.y;
			oVec P = oadd( omulsv( axialImpulse, axisA ), omulsv( perpImpulse, perpA ) );
			b2r LA = axialImpulse * a1 + perpImpulse * s1 + angleImpulse;
			b2r LB = axialImpulse * a2 + perpImpulse * s2 + angleImpulse;
			sA->v = omulsub( sA->v, mA, P );
			sA->w -= iA * LA;
			sB->v = omuladd( sB->v, mB, P );
			sB->w += iB * LB;
			break;
		}
		case b2_revoluteJoint:
		{
			oRevoluteJoint* r = &j->revolute;
			oVec rA = orotate( sA->dq, r->anchorA );
			oVec rB = orotate( sB->dq, r->anchorB );
			b2r axial = r->springImpulse + r->motorImpulse + r->lowerImpulse - r->upperImpulse;
			sA->v = omulsub( sA->v, mA, r->linearImpulse );
			sA->w -= iA * ( ocross( rA, r->linearImpulse ) + axial );
			sB->v = omuladd( sB->v, mB, r->linearImpulse );
			sB->w += iB * ( ocross( rB, r->linearImpulse ) + axial );
			break;
		}
		case b2_weldJoint:
		{
			oWeldJoint* wj = &j->weld;
			oVec rA = orotate( sA->dq, wj->anchorA );
			oVec rB = orotate( sB->dq, wj->anchorB );
			sA->v = omulsub( sA->v, mA, wj->linearImpulse );
			sA->w -= iA * ( ocross( rA, wj->linearImpulse ) + wj->angularImpulse );
			sB->v = omuladd( sB->v, mB, wj->linearImpulse );
			sB->w += iB * ( ocross( rB, wj->linearImpulse ) + wj->angularImpulse );
			break;
		}
		case b2_wheelJoint:
		{
			oWheelJoint* h = &j->wheel;
			oVec rA = orotate( sA->dq, h->anchorA );
			oVec rB = orotate( sB->dq, h->anchorB );
			oVec d = oadd( oadd( osub( sB->dp, sA->dp ), h->deltaCenter ), osub( rB, rA ) );
			oVec axisA = orotate( sA->dq, h->axisA );
			oVec perpA = oleft( axisA );
			b2r a1 = ocross( oadd( d, rA ), axisA );
			b2r a2 = ocross( rB, axisA );
			b2r s1 = ocross( oadd( d, rA ), perpA );
			b2r s2 = ocross( rB, perpA );
			b2r axialImpulse = h->springImpulse + h->lowerImpulse - h->upperImpulse;
			oVec P = oadd( omulsv( axialImpulse, axisA ), omulsv( h->perpImpulse, perpA ) );
			b2r LA = axialImpulse * a1 + h->perpImpulse * s1 + h->motorImpulse;
			b2r LB = axialImpulse * a2 + h->perpImpulse * s2 + h->motorImpulse;
			sA->v = omulsub( sA->v, mA, P );
			sA->w -= iA * LA;
			sB->v = omuladd( sB->v, mB, P );
			sB->w += iB * LB;
			break;
		}
		default:
			break;
	}
}

/* ------------------------------------------------------------ solve */
static void solve_distance( oJoint* j, const oStep* st, oState* sA, oState* sB, bool useBias )
{
	oDistanceJoint* jd = &j->distance;
	b2r mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	oVec vA = sA->v, vB = sB->v;
	b2r wA = sA->w, wB = sB->w;
	oVec rA = orotate( sA->dq, jd->anchorA );
	oVec rB = orotate( sB->dq, jd->anchorB );
	oVec ds = oadd( osub( sB->dp, sA->dp ), osub( rB, rA ) );
	oVec separation = oadd( jd->deltaCenter, ds );
	b2r length = olen( separation );
	oVec axis = onormalize( separation );

	if ( jd->enableSpring && ( jd->minLength < jd->maxLength || jd->enableLimit == false ) )
	{
		if ( jd->hertz > R( 0 ) )
		{
			oVec vr = oadd( osub( vB, vA ), osub( ocross_sv( wB, rB ), ocross_sv( wA, rA ) ) );
			b2r Cdot = odot( axis, vr );
			b2r C = length - jd->length;
			b2r bias = jd->distanceSoftness.biasRate * C;
			b2r m = jd->distanceSoftness.massScale * jd->axialMass;
			b2r impulse = -m * ( Cdot + bias ) - jd->distanceSoftness.impulseScale * jd->impulse;
			jd->impulse += impulse;
			oVec P = omulsv( impulse, axis );
			vA = omulsub( vA, mA, P );
			wA -= iA * ocross( rA, P );
			vB = omuladd( vB, mB, P );
			wB += iB * ocross( rB, P );
		}
		if ( jd->enableLimit )
		{
			{
				oVec vr = oadd( osub( vB, vA ), osub( ocross_sv( wB, rB ), ocross_sv( wA, rA ) ) );
				b2r Cdot = odot( axis, vr );
				b2r C = length - jd->minLength;
				b2r bias = 0, massCoeff = 1, impulseCoeff = 0;
				if ( C > R( 0 ) )
					bias = C * st->inv_h;
				else if ( useBias )
				{
					bias = st->jointSoft.biasRate * C;
					massCoeff = st->jointSoft.massScale;
					impulseCoeff = st->jointSoft.impulseScale;
				}
				b2r impulse = -massCoeff * jd->axialMass * ( Cdot + bias ) - impulseCoeff * jd->lowerImpulse;
				b2r newImpulse = omax( R( 0 ), jd->lowerImpulse + impulse );
				impulse = newImpulse - jd->lowerImpulse;
				jd->lowerImpulse = newImpulse;
				oVec P = omulsv( impulse, axis );
				vA = omulsub( vA, mA, P );
				wA -= iA * ocross( rA, P );
				vB = omuladd( vB, mB, P );
				wB += iB * ocross( rB, P );
			}
			{
				oVec vr = oadd( osub( vA, vB ), osub( ocross_sv( wA, rA ), ocross_sv( wB, rB ) ) );
				b2r Cdot = odot( axis, vr );
				b2r C = jd->maxLength - length;
				b2r bias = 0, massScale = 1, impulseScale = 0;
				if ( C > R( 0 ) )
					bias = C * st->inv_h;
				else if ( useBias )
				{
					bias = st->jointSoft.biasRate * C;
					massScale = st->jointSoft.massScale;
					impulseScale = st->jointSoft.impulseScale;
				}
				b2r impulse = -massScale * jd->axialMass * ( Cdot + bias ) - impulseScale * jd->upperImpulse;
				b2r newImpulse = omax( R( 0 ), jd->upperImpulse + impulse );
				impulse = newImpulse - jd->upperImpulse;
				jd->upperImpulse = newImpulse;
				oVec P = omulsv( -impulse, axis );
				vA = omulsub( vA, mA, P );
				wA -= iA * ocross( rA, P );
				vB = omuladd( vB, mB, P );
				wB += iB * ocross( rB, P );
			}
		}
		if ( jd->enableMotor )
		{
			oVec vr = oadd( osub( vB, vA ), osub( ocross_sv( wB, rB ), ocross_sv( wA, rA ) ) );
			b2r Cdot = odot( axis, vr );
			b2r impulse = jd->axialMass * ( jd->motorSpeed - Cdot );
			b2r oldImpulse = jd->motorImpulse;
			b2r maxImpulse = st->h * jd->maxMotorForce;
			jd->motorImpulse = oclamp( jd->motorImpulse + impulse, -maxImpulse, maxImpulse );
			impulse = jd->motorImpulse - oldImpulse;
			oVec P = omulsv( impulse, axis );
			vA = omulsub( vA, mA, P );
			wA -= iA * ocross( rA, P );
			vB = omuladd( vB, mB, P );
			wB += iB * ocross( rB, P );
		}
	}
	else
	{
		oVec vr = oadd( osub( vB, vA ), osub( ocross_sv( wB, rB ), ocross_sv( wA, rA ) ) );
		b2r Cdot = odot( axis, vr );
		b2r C = length - jd->length;
		b2r bias = 0, massScale = 1, impulseScale = 0;
		if ( useBias )
		{
			bias = st->jointSoft.biasRate * C;
			massScale = st->jointSoft.massScale;
			impulseScale = st->jointSoft.impulseScale;
		}
		b2r impulse = -massScale * jd->axialMass * ( Cdot + bias ) - impulseScale * jd->impulse;
		jd->impulse += impulse;
		oVec P = omulsv( impulse, axis );
		vA = omulsub( vA, mA, P );
		wA -= iA * ocross( rA, P );
		vB = omuladd( vB, mB, P );
		wB += iB * ocross( rB, P );
	}
	sA->v = vA;
	sA->w = wA;
	sB->v = vB;
	sB->w = wB;
}

static void solve_motor( oJoint* j, const oStep* st, oState* sA, oState* sB )
{
	oMotorJoint* m = &j->motor;
	b2r mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	oVec vA = sA->v, vB = sB->v;
	b2r wA = sA->w, wB = sB->w;
	{
		b2r angularSeparation = orelangle( sB->dq, sA->dq ) + m->deltaAngle;
		angularSeparation = ounwind( angularSeparation );
		b2r angularBias = st->inv_h * m->correctionFactor * angularSeparation;
		b2r Cdot = wB - wA;
		b2r impulse = -m->angularMass * ( Cdot + angularBias );
		b2r oldImpulse = m->angularImpulse;
		b2r maxImpulse = st->h * m->maxTorque;
		m->angularImpulse = oclamp( m->angularImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = m->angularImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		oVec rA = orotate( sA->dq, m->anchorA );
		oVec rB = orotate( sB->dq, m->anchorB );
		oVec ds = oadd( osub( sB->dp, sA->dp ), osub( rB, rA ) );
		oVec linearSeparation = oadd( m->deltaCenter, ds );
		oVec linearBias = omulsv( st->inv_h * m->correctionFactor, linearSeparation );
		oVec Cdot = osub( oadd( vB, ocross_sv( wB, rB ) ), oadd( vA, ocross_sv( wA, rA ) ) );
		oVec b = omulmv( m->linearMass, oadd( Cdot, linearBias ) );
		oVec impulse = ov( -b.x, -b.y );
		oVec oldImpulse = m->linearImpulse;
		b2r maxImpulse = st->h * m->maxForce;
		m->linearImpulse = oadd( m->linearImpulse, impulse );
		if ( olen2( m->linearImpulse ) > maxImpulse * maxImpulse )
		{
			m->linearImpulse = onormalize( m->linearImpulse );
			m->linearImpulse.x *= maxImpulse;
			m->linearImpulse.y *= maxImpulse;
		}
		impulse = osub( m->linearImpulse, oldImpulse );
		vA = omulsub( vA, mA, impulse );
		wA -= iA * ocross( rA, impulse );
		vB = omuladd( vB, mB, impulse );
		wB += iB * ocross( rB, impulse );
	}
	sA->v = vA;
	sA->w = wA;
	sB->v = vB;
	sB->w = wB;
}

static void solve_mouse( oJoint* j, const oStep* st, oState* sB )
{
	oMouseJoint* m = &j->mouse;
	b2r mB = j->invMassB, iB = j->invIB;
	oVec vB = sB->v;
	b2r wB = sB->w;
	{
		b2r massScale = m->angularSoftness.massScale;
		b2r impulseScale = m->angularSoftness.impulseScale;
		b2r impulse = iB > R( 0 ) ? -wB / iB : R( 0 );
		impulse = massScale * impulse - impulseScale * m->angularImpulse;
		m->angularImpulse += impulse;
		wB += iB * impulse;
	}
	b2r maxImpulse = m->maxForce * st->h;
	{
		oVec rB = orotate( sB->dq, m->anchorB );
		oVec Cdot = oadd( vB, ocross_sv( wB, rB ) );
		oVec separation = oadd( oadd( sB->dp, rB ), m->deltaCenter );
		oVec bias = omulsv( m->linearSoftness.biasRate, separation );
		b2r massScale = m->linearSoftness.massScale;
		b2r impulseScale = m->linearSoftness.impulseScale;
		oVec b = omulmv( m->linearMass, oadd( Cdot, bias ) );
		oVec impulse;
		impulse.x = -massScale * b.x - impulseScale * m->linearImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * m->linearImpulse.y;
		oVec oldImpulse = m->linearImpulse;
		m->linearImpulse.x += impulse.x;
		m->linearImpulse.y += impulse.y;
		b2r mag = olen( m->linearImpulse );
		if ( mag > maxImpulse )
			m->linearImpulse = omulsv( maxImpulse, onormalize( m->linearImpulse ) );
		impulse.x = m->linearImpulse.x - oldImpulse.x;
		impulse.y = m->linearImpulse.y - oldImpulse.y;
		vB = omuladd( vB, mB, impulse );
		wB += iB * ocross( rB, impulse );
	}
	sB->v = vB;
	sB->w = wB;
}

static void solve_prismatic( oJoint* j, const oStep* st, oState* sA, oState* sB, bool useBias )
{
	oPrismaticJoint* p = &j->prismatic;
	b2r mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	oVec vA = sA->v, vB = sB->v;
	b2r wA = sA->w, wB = sB->w;
	oVec rA = orotate( sA->dq, p->anchorA );
	oVec rB = orotate( sB->dq, p->anchorB );
	oVec d = oadd( oadd( osub( sB->dp, sA->dp ), p->deltaCenter ), osub( rB, rA ) );
	oVec axisA = orotate( sA->dq, p->axisA );
	b2r translation = odot( axisA, d );
	b2r a1 = ocross( oadd( d, rA ), axisA );
	b2r a2 = ocross( rB, axisA );

	if ( p->enableSpring )
	{
		b2r C = translation;
		b2r bias = p->springSoftness.biasRate * C;
		b2r massScale = p->springSoftness.massScale;
		b2r impulseScale = p->springSoftness.impulseScale;
		b2r Cdot = odot( axisA, osub( vB, vA ) ) + a2 * wB - a1 * wA;
		b2r impulse = -massScale * p->axialMass * ( Cdot + bias ) - impulseScale * p->springImpulse;
		p->springImpulse += impulse;
		oVec P = omulsv( impulse, axisA );
		b2r LA = impulse * a1;
		b2r LB = impulse * a2;
		vA = omulsub( vA, mA, P );
		wA -= iA * LA;
		vB = omuladd( vB, mB, P );
		wB += iB * LB;
	}
	if ( p->enableMotor )
	{
		b2r Cdot = odot( axisA, osub( vB, vA ) ) + a2 * wB - a1 * wA;
		b2r impulse = p->axialMass * ( p->motorSpeed - Cdot );
		b2r oldImpulse = p->motorImpulse;
		b2r maxImpulse = st->h * p->maxMotorForce;
		p->motorImpulse = oclamp( p->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = p->motorImpulse - oldImpulse;
		oVec P = omulsv( impulse, axisA );
		b2r LA = impulse * a1;
		b2r LB = impulse * a2;
		vA = omulsub( vA, mA, P );
		wA -= iA * LA;
		vB = omuladd( vB, mB, P );
		wB += iB * LB;
	}
	if ( p->enableLimit )
	{
		{
			b2r C = translation - p->lowerTranslation;
			b2r bias = 0, massScale = 1, impulseScale = 0;
			if ( C > R( 0 ) )
				bias = C * st->inv_h;
			else if ( useBias )
			{
				bias = st->jointSoft.biasRate * C;
				massScale = st->jointSoft.massScale;
				impulseScale = st->jointSoft.impulseScale;
			}
			b2r oldImpulse = p->lowerImpulse;
			b2r Cdot = odot( axisA, osub( vB, vA ) ) + a2 * wB - a1 * wA;
			b2r impulse = -p->axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
			p->lowerImpulse = omax( oldImpulse + impulse, R( 0 ) );
			impulse = p->lowerImpulse - oldImpulse;
			oVec P = omulsv( impulse, axisA );
			b2r LA = impulse * a1;
			b2r LB = impulse * a2;
			vA = omulsub( vA, mA, P );
			wA -= iA * LA;
			vB = omuladd( vB, mB, P );
			wB += iB * LB;
		}
		{
			b2r C = p->upperTranslation - translation;
			b2r bias = 0, massScale = 1, impulseScale = 0;
			if ( C > R( 0 ) )
				bias = C * st->inv_h;
			else if ( useBias )
			{
				bias = st->jointSoft.biasRate * C;
				massScale = st->jointSoft.massScale;
				impulseScale = st->jointSoft.impulseScale;
			}
			b2r oldImpulse = p->upperImpulse;
			b2r Cdot = odot( axisA, osub( vA, vB ) ) + a1 * wA - a2 * wB;
			b2r impulse = -p->axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
			p->upperImpulse = omax( oldImpulse + impulse, R( 0 ) );
			impulse = p->upperImpulse - oldImpulse;
			oVec P = omulsv( impulse, axisA );
			b2r LA = impulse * a1;
			b2r LB = impulse * a2;
			vA = omuladd( vA, mA, P );
			wA += iA * LA;
			vB = omulsub( vB, mB, P );
			wB -= iB * LB;
		}
	}
	{
		oVec perpA = oleft( axisA );
		b2r s1 = ocross( oadd( d, rA ), perpA );
		b2r s2 = ocross( rB, perpA );
		oVec Cdot;
		Cdot.x = odot( perpA, osub( vB, vA ) ) + s2 * wB - s1 * wA;
		Cdot.y = wB - wA;
		oVec bias = ov( 0, 0 );
		b2r massScale = 1, impulseScale = 0;
		if ( useBias )
		{
			oVec C;
			C.x = odot( perpA, d );
			C.y = orelangle( sB->dq, sA->dq ) + p->deltaAngle;
			bias = omulsv( st->jointSoft.biasRate, C );
			massScale = st->jointSoft.massScale;
			impulseScale = st->jointSoft.impulseScale;
		}
		b2r k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
		b2r k12 = iA * s1 + iB * s2;
		b2r k22 = iA + iB;
		if ( k22 == R( 0 ) )
			k22 = R( 1 );
		oMat22 K;
		K.cx = ov( k11, k12 );
		K.cy = ov( k12, k22 );
		oVec b = osolve22( K, oadd( Cdot, bias ) );
		oVec impulse;
		impulse.x = -massScale * b.x - impulseScale * p->impulse.x;
		impulse.y = -massScale * b.y - impulseScale * p->impulse.y;
		p->impulse.x += impulse.x;
		p->impulse.y += impulse.y;
		oVec P = omulsv( impulse.x, perpA );
		b2r LA = impulse.x * s1 + impulse.y;
		b2r LB = impulse.x * s2 + impulse.y;
		vA = omulsub( vA, mA, P );
		wA -= iA * LA;
		vB = omuladd( vB, mB, P );
		wB += iB * LB;
	}
	sA->v = vA;
	sA->w = wA;
	sB->v = vB;
	sB->w = wB;
}

static void solve_revolute( oJoint* j, const oStep* st, oState* sA, oState* sB, bool useBias )
{
	oRevoluteJoint* r = &j->revolute;
	b2r mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	oVec vA = sA->v, vB = sB->v;
	b2r wA = sA->w, wB = sB->w;
	bool fixedRotation = ( iA + iB == R( 0 ) );

	if ( r->enableSpring && fixedRotation == false )
	{
		b2r C = orelangle( sB->dq, sA->dq ) + r->deltaAngle;
		b2r bias = r->springSoftness.biasRate * C;
		b2r Cdot = wB - wA;
		b2r impulse = -r->springSoftness.massScale * r->axialMass * ( Cdot + bias ) - r->springSoftness.impulseScale * r->springImpulse;
		r->springImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( r->enableMotor && fixedRotation == false )
	{
		b2r Cdot = wB - wA - r->motorSpeed;
		b2r impulse = -r->axialMass * Cdot;
		b2r old = r->motorImpulse;
		b2r maxImpulse = st->h * r->maxMotorTorque;
		r->motorImpulse = oclamp( r->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = r->motorImpulse - old;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( r->enableLimit && fixedRotation == false )
	{
		b2r angle = orelangle( sB->dq, sA->dq ) + r->deltaAngle;
		angle = ounwind( angle );
		{
			b2r C = angle - r->lowerAngle;
			b2r bias = 0, massScale = 1, impulseScale = 0;
			if ( C > R( 0 ) )
				bias = C * st->inv_h;
			else if ( useBias )
			{
				bias = st->jointSoft.biasRate * C;
				massScale = st->jointSoft.massScale;
				impulseScale = st->jointSoft.impulseScale;
			}
			b2r Cdot = wB - wA;
			b2r impulse = -massScale * r->axialMass * ( Cdot + bias ) - impulseScale * r->lowerImpulse;
			b2r old = r->lowerImpulse;
			r->lowerImpulse = omax( r->lowerImpulse + impulse, R( 0 ) );
			impulse = r->lowerImpulse - old;
			wA -= iA * impulse;
			wB += iB * impulse;
		}
		{
			b2r C = r->upperAngle - angle;
			b2r bias = 0, massScale = 1, impulseScale = 0;
			if ( C > R( 0 ) )
				bias = C * st->inv_h;
			else if ( useBias )
			{
				bias = st->jointSoft.biasRate * C;
				massScale = st->jointSoft.massScale;
				impulseScale = st->jointSoft.impulseScale;
			}
			b2r Cdot = wA - wB;
			/* the reference scales the upper-limit term by lowerImpulse (revolute_joint.c:409) */
			b2r impulse = -massScale * r->axialMass * ( Cdot + bias ) - impulseScale * r->lowerImpulse;
			b2r old = r->upperImpulse;
			r->upperImpulse = omax( r->upperImpulse + impulse, R( 0 ) );
			impulse = r->upperImpulse - old;
			wA += iA * impulse;
			wB -= iB * impulse;
		}
	}
	{
		oVec rA = orotate( sA->dq, r->anchorA );
		oVec rB = orotate( sB->dq, r->anchorB );
		oVec Cdot = osub( oadd( vB, ocross_sv( wB, rB ) ), oadd( vA, ocross_sv( wA, rA ) ) );
		oVec bias = ov( 0, 0 );
		b2r massScale = 1, impulseScale = 0;
		if ( useBias )
		{
			oVec sep = oadd( oadd( osub( sB->dp, sA->dp ), osub( rB, rA ) ), r->deltaCenter );
			bias = omulsv( st->jointSoft.biasRate, sep );
			massScale = st->jointSoft.massScale;
			impulseScale = st->jointSoft.impulseScale;
		}
		oMat22 K;
		K.cx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		K.cy.x = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		K.cx.y = K.cy.x;
		K.cy.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		oVec b = osolve22( K, oadd( Cdot, bias ) );
		oVec impulse;
		impulse.x = -massScale * b.x - impulseScale * r->linearImpulse.x;
		impulse.y = -massScale * b.y - impulseScale * r->linearImpulse.y;
		r->linearImpulse.x += impulse.x;
		r->linearImpulse.y += impulse.y;
		vA = omulsub( vA, mA, impulse );
		wA -= iA * ocross( rA, impulse );
		vB = omuladd( vB, mB, impulse );
		wB += iB * ocross( rB, impulse );
	}
	sA->v = vA;
	sA->w = wA;
	sB->v = vB;
	sB->w = wB;
}

static void solve_weld( oJoint* j, oState* sA, oState* sB, bool useBias )
{
	oWeldJoint* wj = &j->weld;
	b2r mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	oVec vA = sA->v, vB = sB->v;
	b2r wA = sA->w, wB = sB->w;
	{
		b2r bias = 0, massScale = 1, impulseScale = 0;
		if ( useBias || wj->angularHertz > R( 0 ) )
		{
			b2r C = orelangle( sB->dq, sA->dq ) + wj->deltaAngle;
			bias = wj->angularSoftness.biasRate * C;
			massScale = wj->angularSoftness.massScale;
			impulseScale = wj->angularSoftness.impulseScale;
		}
		b2r Cdot = wB - wA;
		b2r impulse = -massScale * wj->axialMass * ( Cdot + bias ) - impulseScale * wj->angularImpulse;
		wj->angularImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		oVec rA = orotate( sA->dq, wj->anchorA );
		oVec rB = orotate( sB->dq, wj->anchorB );
		oVec bias = ov( 0, 0 );
		b2r massScale = 1, impulseScale = 0;
		if ( useBias || wj->linearHertz > R( 0 ) )
		{
			oVec dcA = sA->dp;
			oVec dcB = sB->dp;
			oVec C = oadd( oadd( osub( dcB, dcA ), osub( rB, rA ) ), wj->deltaCenter );
			bias = omulsv( wj->linearSoftness.biasRate, C );
			massScale = wj->linearSoftness.massScale;
			impulseScale = wj->linearSoftness.impulseScale;
		}
		oVec Cdot = osub( oadd( vB, ocross_sv( wB, rB ) ), oadd( vA, ocross_sv( wA, rA ) ) );
		oMat22 K;
		K.cx.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		K.cy.x = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		K.cx.y = K.cy.x;
		K.cy.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		oVec b = osolve22( K, oadd( Cdot, bias ) );
		oVec impulse = ov( -massScale * b.x - impulseScale * wj->linearImpulse.x, -massScale * b.y - impulseScale * wj->linearImpulse.y );
		wj->linearImpulse = oadd( wj->linearImpulse, impulse );
		vA = omulsub( vA, mA, impulse );
		wA -= iA * ocross( rA, impulse );
		vB = omuladd( vB, mB, impulse );
		wB += iB * ocross( rB, impulse );
	}
	sA->v = vA;
	sA->w = wA;
	sB->v = vB;
	sB->w = wB;
}

static void solve_wheel( oJoint* j, const oStep* st, oState* sA, oState* sB, bool useBias )
{
	oWheelJoint* h = &j->wheel;
	b2r mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	oVec vA = sA->v, vB = sB->v;
	b2r wA = sA->w, wB = sB->w;
	bool fixedRotation = ( iA + iB == R( 0 ) );
	oVec rA = orotate( sA->dq, h->anchorA );
	oVec rB = orotate( sB->dq, h->anchorB );
	oVec d = oadd( oadd( osub( sB->dp, sA->dp ), h->deltaCenter ), osub( rB, rA ) );
	oVec axisA = orotate( sA->dq, h->axisA );
	b2r translation = odot( axisA, d );
	b2r a1 = ocross( oadd( d, rA ), axisA );
	b2r a2 = ocross( rB, axisA );

	if ( h->enableMotor && fixedRotation == false )
	{
		b2r Cdot = wB - wA - h->motorSpeed;
		b2r impulse = -h->motorMass * Cdot;
		b2r oldImpulse = h->motorImpulse;
		b2r maxImpulse = st->h * h->maxMotorTorque;
		h->motorImpulse = oclamp( h->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = h->motorImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( h->enableSpring )
	{
		b2r C = translation;
		b2r bias = h->springSoftness.biasRate * C;
		b2r massScale = h->springSoftness.massScale;
		b2r impulseScale = h->springSoftness.impulseScale;
		b2r Cdot = odot( axisA, osub( vB, vA ) ) + a2 * wB - a1 * wA;
		b2r impulse = -massScale * h->axialMass * ( Cdot + bias ) - impulseScale * h->springImpulse;
		h->springImpulse += impulse;
		oVec P = omulsv( impulse, axisA );
		b2r LA = impulse * a1;
		b2r LB = impulse * a2;
		vA = omulsub( vA, mA, P );
		wA -= iA * LA;
		vB = omuladd( vB, mB, P );
		wB += iB * LB;
	}
	if ( h->enableLimit )
	{
		b2r tr = odot( axisA, d );
		{
			b2r C = tr - h->lowerTranslation;
			b2r bias = 0, massScale = 1, impulseScale = 0;
			if ( C > R( 0 ) )
				bias = C * st->inv_h;
			else if ( useBias )
			{
				bias = st->jointSoft.biasRate * C;
				massScale = st->jointSoft.massScale;
				impulseScale = st->jointSoft.impulseScale;
			}
			b2r Cdot = odot( axisA, osub( vB, vA ) ) + a2 * wB - a1 * wA;
			b2r impulse = -massScale * h->axialMass * ( Cdot + bias ) - impulseScale * h->lowerImpulse;
			b2r oldImpulse = h->lowerImpulse;
			h->lowerImpulse = omax( oldImpulse + impulse, R( 0 ) );
			impulse = h->lowerImpulse - oldImpulse;
			oVec P = omulsv( impulse, axisA );
			b2r LA = impulse * a1;
			b2r LB = impulse * a2;
			vA = omulsub( vA, mA, P );
			wA -= iA * LA;
			vB = omuladd( vB, mB, P );
			wB += iB * LB;
		}
		{
			b2r C = h->upperTranslation - tr;
			b2r bias = 0, massScale = 1, impulseScale = 0;
			if ( C > R( 0 ) )
				bias = C * st->inv_h;
			else if ( useBias )
			{
				bias = st->jointSoft.biasRate * C;
				massScale = st->jointSoft.massScale;
				impulseScale = st->jointSoft.impulseScale;
			}
			b2r Cdot = odot( axisA, osub( vA, vB ) ) + a1 * wA - a2 * wB;
			b2r impulse = -massScale * h->axialMass * ( Cdot + bias ) - impulseScale * h->upperImpulse;
			b2r oldImpulse = h->upperImpulse;
			h->upperImpulse = omax( oldImpulse + impulse, R( 0 ) );
			impulse = h->upperImpulse - oldImpulse;
			oVec P = omulsv( impulse, axisA );
			b2r LA = impulse * a1;
			b2r LB = impulse * a2;
			vA = omuladd( vA, mA, P );
			wA += iA * LA;
			vB = omulsub( vB, mB, P );
			wB -= iB * LB;
		}
	}
	{
		oVec perpA = oleft( axisA );
		b2r bias = 0, massScale = 1, impulseScale = 0;
		if ( useBias )
		{
			b2r C = odot( perpA, d );
			bias = st->jointSoft.biasRate * C;
			massScale = st->jointSoft.massScale;
			impulseScale = st->jointSoft.impulseScale;
		}
		b2r s1 = ocross( oadd( d, rA ), perpA );
		b2r s2 = ocross( rB, perpA );
		b2r Cdot = odot( perpA, osub( vB, vA ) ) + s2 * wB - s1 * wA;
		b2r impulse = -massScale * h->perpMass * ( Cdot + bias ) - impulseScale * h->perpImpulse;
		h->perpImpulse += impulse;
		oVec P = omulsv( impulse, perpA );
		b2r LA = impulse * s1;
		b2r LB = impulse * s2;
		vA = omulsub( vA, mA, P );
		wA -= iA * LA;
		vB = omuladd( vB, mB, P );
		wB += iB * LB;
	}
	sA->v = vA;
	sA->w = wA;
	sB->v = vB;
	sB->w = wB;
}

void o_solve_joint( oJoint* j, const oStep* st, oState* a, oState* b, bool useBias )
{
	switch ( j->type )
	{
		case b2_distanceJoint:
			solve_distance( j, st, a, b, useBias );
			break;
		case b2_motorJoint:
			solve_motor( j, st, a, b );
			break;
		case b2_mouseJoint:
			solve_mouse( j, st, b );
			break;
		case b2_prismaticJoint:
			solve_prismatic( j, st, a, b, useBias );
			break;
		case b2_revoluteJoint:
			solve_revolute( j, st, a, b, useBias );
			break;
		case b2_weldJoint:
			solve_weld( j, a, b, useBias );
			break;
		case b2_wheelJoint:
			solve_wheel( j, st, a, b, useBias );
			break;
		default:
			break;
	}
}
