/*
 * b2g_joints.h -- joint preparation and solver arithmetic for every joint type, on
 * values already in registers (the joint record and the two body states it couples).
 *
 * Included by b2g_solve.h after DevState.  Each routine restates the reference's
 * per-type functions expression by expression (compiled with --fmad=false):
 *   distance   src/distance_joint.c:213-495
 *   motor      src/motor_joint.c:99-273
 *   mouse      src/mouse_joint.c:77-230
 *   prismatic  src/prismatic_joint.c:212-551
 *   revolute   src/revolute_joint.c:201-470
 *   weld       src/weld_joint.c:93-307
 *   wheel      src/wheel_joint.c:181-506
 * and the type switch of src/joint.c:983-1108.  Static bodies enter as the identity
 * state; a body the reference never touches (body A of a mouse joint) is returned as it
 * came in, so storing it back changes nothing.
 */
#pragma once

/* Joint softness coefficients (reference b2Softness, src/solver.h:144-156). */
struct JSoft
{
	float biasRate, massScale, impulseScale;
};

__device__ __forceinline__ JSoft jsoft( float hertz, float zeta, float h )
{
	JSoft s;
	if ( hertz == 0.0f )
	{
		s.biasRate = 0.0f;
		s.massScale = 1.0f;
		s.impulseScale = 0.0f;
		return s;
	}
	float omega = 2.0f * B2G_PI * hertz;
	float a1 = 2.0f * zeta + h * omega;
	float a2 = h * omega * a1;
	float a3 = 1.0f / ( 1.0f + a2 );
	s.biasRate = omega / a1;
	s.massScale = a2 * a3;
	s.impulseScale = a3;
	return s;
}

__device__ __forceinline__ void jsoft_store( float* out, JSoft s )
{
	out[0] = s.biasRate;
	out[1] = s.massScale;
	out[2] = s.impulseScale;
}

__device__ __forceinline__ JSoft step_joint_soft( const b2gStepConst& sc )
{
	JSoft s;
	s.biasRate = sc.jointSoft[0];
	s.massScale = sc.jointSoft[1];
	s.impulseScale = sc.jointSoft[2];
	return s;
}

/* Relative angle of two rotations (reference include/box2d/math_functions.h:386-394).
 * The reference calls the C library's atan2f; the device uses gatan2, which is within one
 * float ulp of it and gives the same bits on host and device. */
__device__ __forceinline__ float rel_angle( b2gRot b, b2gRot a )
{
	float s = b.s * a.c - b.c * a.s;
	float c = b.c * a.c + b.s * a.s;
	return gatan2( s, c );
}

__device__ __forceinline__ float unwind( float a )
{
	if ( a < -B2G_PI )
		return a + 2.0f * B2G_PI;
	if ( a > B2G_PI )
		return a - 2.0f * B2G_PI;
	return a;
}

/* b2Solve22 and b2GetInverse22 (reference include/box2d/math_functions.h:471-499) on a
 * matrix given by its columns cx = (a11, a21), cy = (a12, a22). */
__device__ __forceinline__ b2gVec solve22( float a11, float a21, float a12, float a22, b2gVec b )
{
	float det = a11 * a22 - a12 * a21;
	if ( det != 0.0f )
		det = 1.0f / det;
	return gv( det * ( a22 * b.x - a12 * b.y ), det * ( a11 * b.y - a21 * b.x ) );
}

__device__ __forceinline__ void inverse22( float a, float c, float b, float d, float* out )
{
	/* a = cx.x, c = cx.y, b = cy.x, d = cy.y; out = cx.x cx.y cy.x cy.y */
	float det = a * d - b * c;
	if ( det != 0.0f )
		det = 1.0f / det;
	out[0] = det * d;
	out[1] = -det * c;
	out[2] = -det * b;
	out[3] = det * a;
}

/* b2MulMV with the matrix stored as cx.x cx.y cy.x cy.y */
__device__ __forceinline__ b2gVec mulmv( const float* m, b2gVec v )
{
	return gv( m[0] * v.x + m[2] * v.y, m[1] * v.x + m[3] * v.y );
}

/* Mass properties and pose of a joint's two bodies at the start of the step. */
struct JointBodies
{
	float mA, iA, mB, iB;
	b2gRot qA, qB;
	b2gVec cA, cB;	 /* centres of mass */
	b2gVec lcA, lcB; /* local centres */
};

/* ------------------------------------------------------------------ preparation */
__device__ __forceinline__ void joint_prepare( b2gJointDev* j, const JointBodies& jb, const b2gStepConst& sc )
{
	float mA = jb.mA, iA = jb.iA, mB = jb.mB, iB = jb.iB;
	int type = j->type;
	if ( type == B2G_J_MOUSE )
	{
		/* src/mouse_joint.c:77-135: body B only */
		j->invMassB = mB;
		j->invIB = iB;
		j->anchorB = grotate( jb.qB, gsub( j->localAnchorB, jb.lcB ) );
		jsoft_store( j->springSoft, jsoft( j->hertz, j->dampingRatio, sc.h ) );
		jsoft_store( j->angularSoft, jsoft( 0.5f, 0.1f, sc.h ) );
		b2gVec rB = j->anchorB;
		float kxx = mB + iB * rB.y * rB.y;
		float kxy = -iB * rB.x * rB.y;
		float kyy = mB + iB * rB.x * rB.x;
		inverse22( kxx, kxy, kxy, kyy, j->linearMass );
		j->deltaCenter = gsub( jb.cB, j->target );
		if ( sc.enableWarmStarting == 0 )
		{
			j->linearImpulse = gv( 0.0f, 0.0f );
			j->angularImpulse = 0.0f;
		}
		return;
	}

	j->invMassA = mA;
	j->invMassB = mB;
	j->invIA = iA;
	j->invIB = iB;
	j->anchorA = grotate( jb.qA, gsub( j->localAnchorA, jb.lcA ) );
	j->anchorB = grotate( jb.qB, gsub( j->localAnchorB, jb.lcB ) );
	j->deltaCenter = gsub( jb.cB, jb.cA );
	b2gVec rA = j->anchorA;
	b2gVec rB = j->anchorB;
	bool warm = sc.enableWarmStarting != 0;

	switch ( type )
	{
		case B2G_J_DISTANCE:
		{
			b2gVec separation = gadd( gsub( rB, rA ), j->deltaCenter );
			b2gVec axis = gnormalize( separation );
			float crA = gcross( rA, axis );
			float crB = gcross( rB, axis );
			float k = mA + mB + iA * crA * crA + iB * crB * crB;
			j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
			jsoft_store( j->springSoft, jsoft( j->hertz, j->dampingRatio, sc.h ) );
			if ( warm == false )
			{
				j->impulse = 0.0f;
				j->lowerImpulse = 0.0f;
				j->upperImpulse = 0.0f;
				j->motorImpulse = 0.0f;
			}
			break;
		}
		case B2G_J_MOTOR:
		{
			j->deltaCenter = gsub( gsub( jb.cB, jb.cA ), j->target );
			j->deltaAngle = rel_angle( jb.qB, jb.qA ) - j->referenceAngle;
			j->deltaAngle = unwind( j->deltaAngle );
			float kxx = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
			float kxy = -rA.y * rA.x * iA - rB.y * rB.x * iB;
			float kyy = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
			inverse22( kxx, kxy, kxy, kyy, j->linearMass );
			float ka = iA + iB;
			j->axialMass = ka > 0.0f ? 1.0f / ka : 0.0f;
			if ( warm == false )
			{
				j->linearImpulse = gv( 0.0f, 0.0f );
				j->angularImpulse = 0.0f;
			}
			break;
		}
		case B2G_J_PRISMATIC:
		{
			j->axisA = grotate( jb.qA, j->localAxisA );
			j->deltaAngle = rel_angle( jb.qB, jb.qA ) - j->referenceAngle;
			b2gVec d = gadd( j->deltaCenter, gsub( rB, rA ) );
			float a1 = gcross( gadd( d, rA ), j->axisA );
			float a2 = gcross( rB, j->axisA );
			float k = mA + mB + iA * a1 * a1 + iB * a2 * a2;
			j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
			jsoft_store( j->springSoft, jsoft( j->hertz, j->dampingRatio, sc.h ) );
			if ( warm == false )
			{
				j->linearImpulse = gv( 0.0f, 0.0f );
				j->springImpulse = 0.0f;
				j->motorImpulse = 0.0f;
				j->lowerImpulse = 0.0f;
				j->upperImpulse = 0.0f;
			}
			break;
		}
		case B2G_J_REVOLUTE:
		{
			j->deltaAngle = rel_angle( jb.qB, jb.qA ) - j->referenceAngle;
			j->deltaAngle = unwind( j->deltaAngle );
			float k = iA + iB;
			j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
			jsoft_store( j->springSoft, jsoft( j->hertz, j->dampingRatio, sc.h ) );
			if ( warm == false )
			{
				j->linearImpulse = gv( 0.0f, 0.0f );
				j->springImpulse = 0.0f;
				j->motorImpulse = 0.0f;
				j->lowerImpulse = 0.0f;
				j->upperImpulse = 0.0f;
			}
			break;
		}
		case B2G_J_WELD:
		{
			j->deltaAngle = rel_angle( jb.qB, jb.qA ) - j->referenceAngle;
			float ka = iA + iB;
			j->axialMass = ka > 0.0f ? 1.0f / ka : 0.0f;
			JSoft js = step_joint_soft( sc );
			jsoft_store( j->springSoft, j->hertz == 0.0f ? js : jsoft( j->hertz, j->dampingRatio, sc.h ) );
			jsoft_store( j->angularSoft, j->angularHertz == 0.0f ? js : jsoft( j->angularHertz, j->angularDampingRatio, sc.h ) );
			if ( warm == false )
			{
				j->linearImpulse = gv( 0.0f, 0.0f );
				j->angularImpulse = 0.0f;
			}
			break;
		}
		case B2G_J_WHEEL:
		{
			j->axisA = grotate( jb.qA, j->localAxisA );
			b2gVec d = gadd( j->deltaCenter, gsub( rB, rA ) );
			b2gVec axisA = j->axisA;
			b2gVec perpA = gleft( axisA );
			float s1 = gcross( gadd( d, rA ), perpA );
			float s2 = gcross( rB, perpA );
			float kp = mA + mB + iA * s1 * s1 + iB * s2 * s2;
			j->perpMass = kp > 0.0f ? 1.0f / kp : 0.0f;
			float a1 = gcross( gadd( d, rA ), axisA );
			float a2 = gcross( rB, axisA );
			float ka = mA + mB + iA * a1 * a1 + iB * a2 * a2;
			j->axialMass = ka > 0.0f ? 1.0f / ka : 0.0f;
			jsoft_store( j->springSoft, jsoft( j->hertz, j->dampingRatio, sc.h ) );
			float km = iA + iB;
			j->motorMass = km > 0.0f ? 1.0f / km : 0.0f;
			if ( warm == false )
			{
				j->perpImpulse = 0.0f;
				j->springImpulse = 0.0f;
				j->motorImpulse = 0.0f;
				j->lowerImpulse = 0.0f;
				j->upperImpulse = 0.0f;
			}
			break;
		}
		default:
			break;
	}
}

/* ------------------------------------------------------------------ warm start */
/* Apply an impulse P at the anchors with angular parts LA, LB. */
__device__ __forceinline__ void apply_axial( const b2gJointDev* j, DevState& a, DevState& b, b2gVec P, float LA, float LB )
{
	a.v = gmulsub( a.v, j->invMassA, P );
	a.w -= j->invIA * LA;
	b.v = gmuladd( b.v, j->invMassB, P );
	b.w += j->invIB * LB;
}

/* Joint phases are out of line: joints are few, and inlining their rows would raise the
 * register count and spills of the contact sweep in every solver kernel. */
static __device__ __noinline__ void joint_warm_state( const b2gJointDev* j, DevState& a, DevState& b )
{
	switch ( j->type )
	{
		case B2G_J_DISTANCE:
		{
			b2gVec rA = grotate( a.dq, j->anchorA );
			b2gVec rB = grotate( b.dq, j->anchorB );
			b2gVec ds = gadd( gsub( b.dp, a.dp ), gsub( rB, rA ) );
			b2gVec separation = gadd( j->deltaCenter, ds );
			b2gVec axis = gnormalize( separation );
			float axialImpulse = j->impulse + j->lowerImpulse - j->upperImpulse + j->motorImpulse;
			b2gVec P = gmulsv( axialImpulse, axis );
			apply_axial( j, a, b, P, gcross( rA, P ), gcross( rB, P ) );
			break;
		}
		case B2G_J_MOUSE:
		{
			b2gVec rB = grotate( b.dq, j->anchorB );
			b.v = gmuladd( b.v, j->invMassB, j->linearImpulse );
			b.w += j->invIB * ( gcross( rB, j->linearImpulse ) + j->angularImpulse );
			break;
		}
		case B2G_J_MOTOR:
		case B2G_J_WELD:
		{
			b2gVec rA = grotate( a.dq, j->anchorA );
			b2gVec rB = grotate( b.dq, j->anchorB );
			a.v = gmulsub( a.v, j->invMassA, j->linearImpulse );
			a.w -= j->invIA * ( gcross( rA, j->linearImpulse ) + j->angularImpulse );
			b.v = gmuladd( b.v, j->invMassB, j->linearImpulse );
			b.w += j->invIB * ( gcross( rB, j->linearImpulse ) + j->angularImpulse );
			break;
		}
		case B2G_J_PRISMATIC:
		case B2G_J_WHEEL:
		{
			b2gVec rA = grotate( a.dq, j->anchorA );
			b2gVec rB = grotate( b.dq, j->anchorB );
			b2gVec d = gadd( gadd( gsub( b.dp, a.dp ), j->deltaCenter ), gsub( rB, rA ) );
			b2gVec axisA = grotate( a.dq, j->axisA );
			float a1 = gcross( gadd( d, rA ), axisA );
			float a2 = gcross( rB, axisA );
			b2gVec perpA = gleft( axisA );
			float s1 = gcross( gadd( d, rA ), perpA );
			float s2 = gcross( rB, perpA );
			b2gVec P;
			float LA, LB;
			if ( j->type == B2G_J_PRISMATIC )
			{
				float axialImpulse = j->springImpulse + j->motorImpulse + j->lowerImpulse - j->upperImpulse;
				float perpImpulse = j->linearImpulse.x;
				float angleImpulse = j->linearImpulse.y;
				P = gadd( gmulsv( axialImpulse, axisA ), gmulsv( perpImpulse, perpA ) );
				LA = axialImpulse * a1 + perpImpulse * s1 + angleImpulse;
				LB = axialImpulse * a2 + perpImpulse * s2 + angleImpulse;
			}
			else
			{
				float axialImpulse = j->springImpulse + j->lowerImpulse - j->upperImpulse;
				P = gadd( gmulsv( axialImpulse, axisA ), gmulsv( j->perpImpulse, perpA ) );
				LA = axialImpulse * a1 + j->perpImpulse * s1 + j->motorImpulse;
				LB = axialImpulse * a2 + j->perpImpulse * s2 + j->motorImpulse;
			}
			apply_axial( j, a, b, P, LA, LB );
			break;
		}
		case B2G_J_REVOLUTE:
		{
			b2gVec rA = grotate( a.dq, j->anchorA );
			b2gVec rB = grotate( b.dq, j->anchorB );
			float axial = j->springImpulse + j->motorImpulse + j->lowerImpulse - j->upperImpulse;
			a.v = gmulsub( a.v, j->invMassA, j->linearImpulse );
			a.w -= j->invIA * ( gcross( rA, j->linearImpulse ) + axial );
			b.v = gmuladd( b.v, j->invMassB, j->linearImpulse );
			b.w += j->invIB * ( gcross( rB, j->linearImpulse ) + axial );
			break;
		}
		default:
			break;
	}
}

/* ------------------------------------------------------------------ solve */
/* Limit rows share one shape: speculative when separated, soft (with bias) or rigid
 * (relax) when violated; returns the bias and the mass and impulse scales. */
__device__ __forceinline__ void limit_coefs( float C, bool useBias, const b2gStepConst& sc, float& bias, float& massScale,
											 float& impulseScale )
{
	bias = 0.0f;
	massScale = 1.0f;
	impulseScale = 0.0f;
	if ( C > 0.0f )
		bias = C * sc.inv_h;
	else if ( useBias )
	{
		bias = sc.jointSoft[0] * C;
		massScale = sc.jointSoft[1];
		impulseScale = sc.jointSoft[2];
	}
}

__device__ __forceinline__ void solve_distance( b2gJointDev* j, DevState& a, DevState& b, bool useBias, const b2gStepConst& sc )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	b2gVec vA = a.v, vB = b.v;
	float wA = a.w, wB = b.w;
	b2gVec rA = grotate( a.dq, j->anchorA );
	b2gVec rB = grotate( b.dq, j->anchorB );
	b2gVec ds = gadd( gsub( b.dp, a.dp ), gsub( rB, rA ) );
	b2gVec separation = gadd( j->deltaCenter, ds );
	float length = glen( separation );
	b2gVec axis = gnormalize( separation );

	if ( j->enableSpring && ( j->lower < j->upper || j->enableLimit == 0 ) )
	{
		if ( j->hertz > 0.0f )
		{
			b2gVec vr = gadd( gsub( vB, vA ), gsub( gcross_sv( wB, rB ), gcross_sv( wA, rA ) ) );
			float Cdot = gdot( axis, vr );
			float C = length - j->length;
			float bias = j->springSoft[0] * C;
			float m = j->springSoft[1] * j->axialMass;
			float impulse = -m * ( Cdot + bias ) - j->springSoft[2] * j->impulse;
			j->impulse += impulse;
			b2gVec P = gmulsv( impulse, axis );
			vA = gmulsub( vA, mA, P );
			wA -= iA * gcross( rA, P );
			vB = gmuladd( vB, mB, P );
			wB += iB * gcross( rB, P );
		}
		if ( j->enableLimit )
		{
			{
				b2gVec vr = gadd( gsub( vB, vA ), gsub( gcross_sv( wB, rB ), gcross_sv( wA, rA ) ) );
				float Cdot = gdot( axis, vr );
				float C = length - j->lower;
				float bias, massScale, impulseScale;
				limit_coefs( C, useBias, sc, bias, massScale, impulseScale );
				float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->lowerImpulse;
				float newImpulse = gmax( 0.0f, j->lowerImpulse + impulse );
				impulse = newImpulse - j->lowerImpulse;
				j->lowerImpulse = newImpulse;
				b2gVec P = gmulsv( impulse, axis );
				vA = gmulsub( vA, mA, P );
				wA -= iA * gcross( rA, P );
				vB = gmuladd( vB, mB, P );
				wB += iB * gcross( rB, P );
			}
			{
				b2gVec vr = gadd( gsub( vA, vB ), gsub( gcross_sv( wA, rA ), gcross_sv( wB, rB ) ) );
				float Cdot = gdot( axis, vr );
				float C = j->upper - length;
				float bias, massScale, impulseScale;
				limit_coefs( C, useBias, sc, bias, massScale, impulseScale );
				float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->upperImpulse;
				float newImpulse = gmax( 0.0f, j->upperImpulse + impulse );
				impulse = newImpulse - j->upperImpulse;
				j->upperImpulse = newImpulse;
				b2gVec P = gmulsv( -impulse, axis );
				vA = gmulsub( vA, mA, P );
				wA -= iA * gcross( rA, P );
				vB = gmuladd( vB, mB, P );
				wB += iB * gcross( rB, P );
			}
		}
		if ( j->enableMotor )
		{
			b2gVec vr = gadd( gsub( vB, vA ), gsub( gcross_sv( wB, rB ), gcross_sv( wA, rA ) ) );
			float Cdot = gdot( axis, vr );
			float impulse = j->axialMass * ( j->motorSpeed - Cdot );
			float oldImpulse = j->motorImpulse;
			float maxImpulse = sc.h * j->maxMotor;
			j->motorImpulse = gclamp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
			impulse = j->motorImpulse - oldImpulse;
			b2gVec P = gmulsv( impulse, axis );
			vA = gmulsub( vA, mA, P );
			wA -= iA * gcross( rA, P );
			vB = gmuladd( vB, mB, P );
			wB += iB * gcross( rB, P );
		}
	}
	else
	{
		b2gVec vr = gadd( gsub( vB, vA ), gsub( gcross_sv( wB, rB ), gcross_sv( wA, rA ) ) );
		float Cdot = gdot( axis, vr );
		float C = length - j->length;
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			bias = sc.jointSoft[0] * C;
			massScale = sc.jointSoft[1];
			impulseScale = sc.jointSoft[2];
		}
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->impulse;
		j->impulse += impulse;
		b2gVec P = gmulsv( impulse, axis );
		vA = gmulsub( vA, mA, P );
		wA -= iA * gcross( rA, P );
		vB = gmuladd( vB, mB, P );
		wB += iB * gcross( rB, P );
	}
	a.v = vA;
	a.w = wA;
	b.v = vB;
	b.w = wB;
}

__device__ __forceinline__ void solve_motor( b2gJointDev* j, DevState& a, DevState& b, const b2gStepConst& sc )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	b2gVec vA = a.v, vB = b.v;
	float wA = a.w, wB = b.w;
	{
		float angularSeparation = rel_angle( b.dq, a.dq ) + j->deltaAngle;
		angularSeparation = unwind( angularSeparation );
		float angularBias = sc.inv_h * j->correctionFactor * angularSeparation;
		float Cdot = wB - wA;
		float impulse = -j->axialMass * ( Cdot + angularBias );
		float oldImpulse = j->angularImpulse;
		float maxImpulse = sc.h * j->maxTorque;
		j->angularImpulse = gclamp( j->angularImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->angularImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		b2gVec rA = grotate( a.dq, j->anchorA );
		b2gVec rB = grotate( b.dq, j->anchorB );
		b2gVec ds = gadd( gsub( b.dp, a.dp ), gsub( rB, rA ) );
		b2gVec linearSeparation = gadd( j->deltaCenter, ds );
		b2gVec linearBias = gmulsv( sc.inv_h * j->correctionFactor, linearSeparation );
		b2gVec Cdot = gsub( gadd( vB, gcross_sv( wB, rB ) ), gadd( vA, gcross_sv( wA, rA ) ) );
		b2gVec bb = mulmv( j->linearMass, gadd( Cdot, linearBias ) );
		b2gVec impulse = gv( -bb.x, -bb.y );
		b2gVec oldImpulse = j->linearImpulse;
		float maxImpulse = sc.h * j->maxMotor;
		j->linearImpulse = gadd( j->linearImpulse, impulse );
		if ( glen2( j->linearImpulse ) > maxImpulse * maxImpulse )
		{
			j->linearImpulse = gnormalize( j->linearImpulse );
			j->linearImpulse.x *= maxImpulse;
			j->linearImpulse.y *= maxImpulse;
		}
		impulse = gsub( j->linearImpulse, oldImpulse );
		vA = gmulsub( vA, mA, impulse );
		wA -= iA * gcross( rA, impulse );
		vB = gmuladd( vB, mB, impulse );
		wB += iB * gcross( rB, impulse );
	}
	a.v = vA;
	a.w = wA;
	b.v = vB;
	b.w = wB;
}

__device__ __forceinline__ void solve_mouse( b2gJointDev* j, DevState& b, const b2gStepConst& sc )
{
	float mB = j->invMassB, iB = j->invIB;
	b2gVec vB = b.v;
	float wB = b.w;
	{
		float massScale = j->angularSoft[1];
		float impulseScale = j->angularSoft[2];
		float impulse = iB > 0.0f ? -wB / iB : 0.0f;
		impulse = massScale * impulse - impulseScale * j->angularImpulse;
		j->angularImpulse += impulse;
		wB += iB * impulse;
	}
	float maxImpulse = j->maxMotor * sc.h;
	{
		b2gVec rB = grotate( b.dq, j->anchorB );
		b2gVec Cdot = gadd( vB, gcross_sv( wB, rB ) );
		b2gVec separation = gadd( gadd( b.dp, rB ), j->deltaCenter );
		b2gVec bias = gmulsv( j->springSoft[0], separation );
		float massScale = j->springSoft[1];
		float impulseScale = j->springSoft[2];
		b2gVec bb = mulmv( j->linearMass, gadd( Cdot, bias ) );
		b2gVec impulse;
		impulse.x = -massScale * bb.x - impulseScale * j->linearImpulse.x;
		impulse.y = -massScale * bb.y - impulseScale * j->linearImpulse.y;
		b2gVec oldImpulse = j->linearImpulse;
		j->linearImpulse.x += impulse.x;
		j->linearImpulse.y += impulse.y;
		float mag = glen( j->linearImpulse );
		if ( mag > maxImpulse )
			j->linearImpulse = gmulsv( maxImpulse, gnormalize( j->linearImpulse ) );
		impulse.x = j->linearImpulse.x - oldImpulse.x;
		impulse.y = j->linearImpulse.y - oldImpulse.y;
		vB = gmuladd( vB, mB, impulse );
		wB += iB * gcross( rB, impulse );
	}
	b.v = vB;
	b.w = wB;
}

/* Axial rows of the prismatic and wheel joints: J = [-axis, -a1, axis, a2]. */
__device__ __forceinline__ float axial_cdot( b2gVec axisA, b2gVec vA, float wA, b2gVec vB, float wB, float a1, float a2 )
{
	return gdot( axisA, gsub( vB, vA ) ) + a2 * wB - a1 * wA;
}

/* Spring (always soft, also in relax), motor and limit rows of the prismatic and wheel
 * joints; the wheel joint's motor is rotational and is solved by its caller. */
__device__ __forceinline__ void slider_rows( b2gJointDev* j, b2gVec axisA, float translation, float a1, float a2, b2gVec& vA,
											 float& wA, b2gVec& vB, float& wB, bool linearMotor, bool useBias,
											 const b2gStepConst& sc )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	if ( j->enableSpring )
	{
		float C = translation;
		float bias = j->springSoft[0] * C;
		float massScale = j->springSoft[1];
		float impulseScale = j->springSoft[2];
		float Cdot = axial_cdot( axisA, vA, wA, vB, wB, a1, a2 );
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->springImpulse;
		j->springImpulse += impulse;
		b2gVec P = gmulsv( impulse, axisA );
		float LA = impulse * a1;
		float LB = impulse * a2;
		vA = gmulsub( vA, mA, P );
		wA -= iA * LA;
		vB = gmuladd( vB, mB, P );
		wB += iB * LB;
	}
	if ( linearMotor && j->enableMotor )
	{
		float Cdot = axial_cdot( axisA, vA, wA, vB, wB, a1, a2 );
		float impulse = j->axialMass * ( j->motorSpeed - Cdot );
		float oldImpulse = j->motorImpulse;
		float maxImpulse = sc.h * j->maxMotor;
		j->motorImpulse = gclamp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - oldImpulse;
		b2gVec P = gmulsv( impulse, axisA );
		float LA = impulse * a1;
		float LB = impulse * a2;
		vA = gmulsub( vA, mA, P );
		wA -= iA * LA;
		vB = gmuladd( vB, mB, P );
		wB += iB * LB;
	}
	if ( j->enableLimit )
	{
		{
			float C = translation - j->lower;
			float bias, massScale, impulseScale;
			limit_coefs( C, useBias, sc, bias, massScale, impulseScale );
			float oldImpulse = j->lowerImpulse;
			float Cdot = axial_cdot( axisA, vA, wA, vB, wB, a1, a2 );
			float impulse = -j->axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->lowerImpulse = gmax( oldImpulse + impulse, 0.0f );
			impulse = j->lowerImpulse - oldImpulse;
			b2gVec P = gmulsv( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = gmulsub( vA, mA, P );
			wA -= iA * LA;
			vB = gmuladd( vB, mB, P );
			wB += iB * LB;
		}
		{
			float C = j->upper - translation;
			float bias, massScale, impulseScale;
			limit_coefs( C, useBias, sc, bias, massScale, impulseScale );
			float oldImpulse = j->upperImpulse;
			float Cdot = gdot( axisA, gsub( vA, vB ) ) + a1 * wA - a2 * wB;
			float impulse = -j->axialMass * massScale * ( Cdot + bias ) - impulseScale * oldImpulse;
			j->upperImpulse = gmax( oldImpulse + impulse, 0.0f );
			impulse = j->upperImpulse - oldImpulse;
			b2gVec P = gmulsv( impulse, axisA );
			float LA = impulse * a1;
			float LB = impulse * a2;
			vA = gmuladd( vA, mA, P );
			wA += iA * LA;
			vB = gmulsub( vB, mB, P );
			wB -= iB * LB;
		}
	}
}

__device__ __forceinline__ void solve_prismatic( b2gJointDev* j, DevState& a, DevState& b, bool useBias, const b2gStepConst& sc )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	b2gVec vA = a.v, vB = b.v;
	float wA = a.w, wB = b.w;
	b2gVec rA = grotate( a.dq, j->anchorA );
	b2gVec rB = grotate( b.dq, j->anchorB );
	b2gVec d = gadd( gadd( gsub( b.dp, a.dp ), j->deltaCenter ), gsub( rB, rA ) );
	b2gVec axisA = grotate( a.dq, j->axisA );
	float translation = gdot( axisA, d );
	float a1 = gcross( gadd( d, rA ), axisA );
	float a2 = gcross( rB, axisA );

	slider_rows( j, axisA, translation, a1, a2, vA, wA, vB, wB, true, useBias, sc );

	{
		b2gVec perpA = gleft( axisA );
		float s1 = gcross( gadd( d, rA ), perpA );
		float s2 = gcross( rB, perpA );
		b2gVec Cdot;
		Cdot.x = gdot( perpA, gsub( vB, vA ) ) + s2 * wB - s1 * wA;
		Cdot.y = wB - wA;
		b2gVec bias = gv( 0.0f, 0.0f );
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			b2gVec C;
			C.x = gdot( perpA, d );
			C.y = rel_angle( b.dq, a.dq ) + j->deltaAngle;
			bias = gmulsv( sc.jointSoft[0], C );
			massScale = sc.jointSoft[1];
			impulseScale = sc.jointSoft[2];
		}
		float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
		float k12 = iA * s1 + iB * s2;
		float k22 = iA + iB;
		if ( k22 == 0.0f )
			k22 = 1.0f;
		b2gVec bb = solve22( k11, k12, k12, k22, gadd( Cdot, bias ) );
		b2gVec impulse;
		impulse.x = -massScale * bb.x - impulseScale * j->linearImpulse.x;
		impulse.y = -massScale * bb.y - impulseScale * j->linearImpulse.y;
		j->linearImpulse.x += impulse.x;
		j->linearImpulse.y += impulse.y;
		b2gVec P = gmulsv( impulse.x, perpA );
		float LA = impulse.x * s1 + impulse.y;
		float LB = impulse.x * s2 + impulse.y;
		vA = gmulsub( vA, mA, P );
		wA -= iA * LA;
		vB = gmuladd( vB, mB, P );
		wB += iB * LB;
	}
	a.v = vA;
	a.w = wA;
	b.v = vB;
	b.w = wB;
}

__device__ __forceinline__ void solve_revolute( b2gJointDev* j, DevState& a, DevState& b, bool useBias, const b2gStepConst& sc )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	b2gVec vA = a.v, vB = b.v;
	float wA = a.w, wB = b.w;
	bool fixedRotation = ( iA + iB == 0.0f );
	if ( j->enableSpring && fixedRotation == false )
	{
		float C = rel_angle( b.dq, a.dq ) + j->deltaAngle;
		float bias = j->springSoft[0] * C;
		float Cdot = wB - wA;
		float impulse = -j->springSoft[1] * j->axialMass * ( Cdot + bias ) - j->springSoft[2] * j->springImpulse;
		j->springImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableMotor && fixedRotation == false )
	{
		float Cdot = wB - wA - j->motorSpeed;
		float impulse = -j->axialMass * Cdot;
		float old = j->motorImpulse;
		float maxImpulse = sc.h * j->maxMotor;
		j->motorImpulse = gclamp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - old;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableLimit && fixedRotation == false )
	{
		float angle = unwind( rel_angle( b.dq, a.dq ) + j->deltaAngle );
		{
			float C = angle - j->lower;
			float bias, massScale, impulseScale;
			limit_coefs( C, useBias, sc, bias, massScale, impulseScale );
			float Cdot = wB - wA;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->lowerImpulse;
			float old = j->lowerImpulse;
			j->lowerImpulse = gmax( j->lowerImpulse + impulse, 0.0f );
			impulse = j->lowerImpulse - old;
			wA -= iA * impulse;
			wB += iB * impulse;
		}
		{
			float C = j->upper - angle;
			float bias, massScale, impulseScale;
			limit_coefs( C, useBias, sc, bias, massScale, impulseScale );
			float Cdot = wA - wB;
			/* upper limit scaled by lowerImpulse, as in the reference (revolute_joint.c:409) */
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->lowerImpulse;
			float old = j->upperImpulse;
			j->upperImpulse = gmax( j->upperImpulse + impulse, 0.0f );
			impulse = j->upperImpulse - old;
			wA += iA * impulse;
			wB -= iB * impulse;
		}
	}
	{
		b2gVec rA = grotate( a.dq, j->anchorA );
		b2gVec rB = grotate( b.dq, j->anchorB );
		b2gVec Cdot = gsub( gadd( vB, gcross_sv( wB, rB ) ), gadd( vA, gcross_sv( wA, rA ) ) );
		b2gVec bias = gv( 0.0f, 0.0f );
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			b2gVec sep = gadd( gadd( gsub( b.dp, a.dp ), gsub( rB, rA ) ), j->deltaCenter );
			bias = gmulsv( sc.jointSoft[0], sep );
			massScale = sc.jointSoft[1];
			impulseScale = sc.jointSoft[2];
		}
		float k11 = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		float k12 = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		float k22 = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		b2gVec x = solve22( k11, k12, k12, k22, gadd( Cdot, bias ) );
		b2gVec impulse;
		impulse.x = -massScale * x.x - impulseScale * j->linearImpulse.x;
		impulse.y = -massScale * x.y - impulseScale * j->linearImpulse.y;
		j->linearImpulse.x += impulse.x;
		j->linearImpulse.y += impulse.y;
		vA = gmulsub( vA, mA, impulse );
		wA -= iA * gcross( rA, impulse );
		vB = gmuladd( vB, mB, impulse );
		wB += iB * gcross( rB, impulse );
	}
	a.v = vA;
	a.w = wA;
	b.v = vB;
	b.w = wB;
}

__device__ __forceinline__ void solve_weld( b2gJointDev* j, DevState& a, DevState& b, bool useBias )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	b2gVec vA = a.v, vB = b.v;
	float wA = a.w, wB = b.w;
	{
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || j->angularHertz > 0.0f )
		{
			float C = rel_angle( b.dq, a.dq ) + j->deltaAngle;
			bias = j->angularSoft[0] * C;
			massScale = j->angularSoft[1];
			impulseScale = j->angularSoft[2];
		}
		float Cdot = wB - wA;
		float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->angularImpulse;
		j->angularImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	{
		b2gVec rA = grotate( a.dq, j->anchorA );
		b2gVec rB = grotate( b.dq, j->anchorB );
		b2gVec bias = gv( 0.0f, 0.0f );
		float massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias || j->hertz > 0.0f )
		{
			b2gVec C = gadd( gadd( gsub( b.dp, a.dp ), gsub( rB, rA ) ), j->deltaCenter );
			bias = gmulsv( j->springSoft[0], C );
			massScale = j->springSoft[1];
			impulseScale = j->springSoft[2];
		}
		b2gVec Cdot = gsub( gadd( vB, gcross_sv( wB, rB ) ), gadd( vA, gcross_sv( wA, rA ) ) );
		float kxx = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
		float kyx = -rA.y * rA.x * iA - rB.y * rB.x * iB;
		float kyy = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
		b2gVec bb = solve22( kxx, kyx, kyx, kyy, gadd( Cdot, bias ) );
		b2gVec impulse = gv( -massScale * bb.x - impulseScale * j->linearImpulse.x,
							 -massScale * bb.y - impulseScale * j->linearImpulse.y );
		j->linearImpulse = gadd( j->linearImpulse, impulse );
		vA = gmulsub( vA, mA, impulse );
		wA -= iA * gcross( rA, impulse );
		vB = gmuladd( vB, mB, impulse );
		wB += iB * gcross( rB, impulse );
	}
	a.v = vA;
	a.w = wA;
	b.v = vB;
	b.w = wB;
}

__device__ __forceinline__ void solve_wheel( b2gJointDev* j, DevState& a, DevState& b, bool useBias, const b2gStepConst& sc )
{
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	b2gVec vA = a.v, vB = b.v;
	float wA = a.w, wB = b.w;
	bool fixedRotation = ( iA + iB == 0.0f );
	b2gVec rA = grotate( a.dq, j->anchorA );
	b2gVec rB = grotate( b.dq, j->anchorB );
	b2gVec d = gadd( gadd( gsub( b.dp, a.dp ), j->deltaCenter ), gsub( rB, rA ) );
	b2gVec axisA = grotate( a.dq, j->axisA );
	float translation = gdot( axisA, d );
	float a1 = gcross( gadd( d, rA ), axisA );
	float a2 = gcross( rB, axisA );

	if ( j->enableMotor && fixedRotation == false )
	{
		float Cdot = wB - wA - j->motorSpeed;
		float impulse = -j->motorMass * Cdot;
		float oldImpulse = j->motorImpulse;
		float maxImpulse = sc.h * j->maxMotor;
		j->motorImpulse = gclamp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - oldImpulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}

	slider_rows( j, axisA, translation, a1, a2, vA, wA, vB, wB, false, useBias, sc );

	{
		b2gVec perpA = gleft( axisA );
		float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( useBias )
		{
			float C = gdot( perpA, d );
			bias = sc.jointSoft[0] * C;
			massScale = sc.jointSoft[1];
			impulseScale = sc.jointSoft[2];
		}
		float s1 = gcross( gadd( d, rA ), perpA );
		float s2 = gcross( rB, perpA );
		float Cdot = gdot( perpA, gsub( vB, vA ) ) + s2 * wB - s1 * wA;
		float impulse = -massScale * j->perpMass * ( Cdot + bias ) - impulseScale * j->perpImpulse;
		j->perpImpulse += impulse;
		b2gVec P = gmulsv( impulse, perpA );
		float LA = impulse * s1;
		float LB = impulse * s2;
		vA = gmulsub( vA, mA, P );
		wA -= iA * LA;
		vB = gmuladd( vB, mB, P );
		wB += iB * LB;
	}
	a.v = vA;
	a.w = wA;
	b.v = vB;
	b.w = wB;
}

/* One solve or relax pass of a joint (reference src/joint.c:1073-1108). */
static __device__ __noinline__ void joint_solve_state( b2gJointDev* j, DevState& a, DevState& b, bool useBias, const b2gStepConst& sc )
{
	switch ( j->type )
	{
		case B2G_J_DISTANCE:
			solve_distance( j, a, b, useBias, sc );
			break;
		case B2G_J_MOTOR:
			solve_motor( j, a, b, sc );
			break;
		case B2G_J_MOUSE:
			solve_mouse( j, b, sc );
			break;
		case B2G_J_PRISMATIC:
			solve_prismatic( j, a, b, useBias, sc );
			break;
		case B2G_J_REVOLUTE:
			solve_revolute( j, a, b, useBias, sc );
			break;
		case B2G_J_WELD:
			solve_weld( j, a, b, useBias );
			break;
		case B2G_J_WHEEL:
			solve_wheel( j, a, b, useBias, sc );
			break;
		default:
			break;
	}
}
