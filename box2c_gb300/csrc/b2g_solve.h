/*
 * b2g_solve.h -- per-constraint solver arithmetic shared by the per-phase kernels
 * (kernels.cu) and the fused cluster solver (fused.cu).
 *
 * Every routine works on values already loaded into registers: one constraint row
 * (Row) or joint (b2gJointDev), and the two body states it couples (DevState).
 * Loading and storing is the caller's business, so the same arithmetic serves body
 * states in global memory and in distributed shared memory.  Operand order follows the
 * reference expression by expression (compiled with --fmad=false):
 *   8-lane contact path   src/contact_solver.c:810-1178
 *   scalar overflow path  src/contact_solver.c:149-440
 *   joints                b2g_joints.h (every joint type)
 */
#pragma once

#include "b2g_math.h"
#include "b2g_types.h"

/* Solver view of one body: v, w, dp, dq, and the state's fourth word (the sleep
 * threshold), carried so that a store rewrites the whole float4. */
struct DevState
{
	b2gVec v;
	float w;
	float tag;
	b2gVec dp;
	b2gRot dq;
};

__device__ __forceinline__ DevState identity_state()
{
	DevState s;
	s.v = gv( 0.0f, 0.0f );
	s.w = 0.0f;
	s.tag = 0.0f;
	s.dp = gv( 0.0f, 0.0f );
	s.dq = grot( 1.0f, 0.0f );
	return s;
}

__device__ __forceinline__ DevState state_of( float4 a, float4 c )
{
	DevState s;
	s.v = gv( a.x, a.y );
	s.w = a.z;
	s.tag = a.w;
	s.dp = gv( c.x, c.y );
	s.dq = grot( c.z, c.w );
	return s;
}

__device__ __forceinline__ float4 velocity_word( const DevState& s ) { return make_float4( s.v.x, s.v.y, s.w, s.tag ); }

/* One constraint row held in registers. */
struct Row
{
	int ia, ib, count;
	b2gVec n;
	float friction, restitution;
	float biasRate, massScale, impulseScale;
	float mA, iA, mB, iB;
	b2gVec rA[2], rB[2];
	float base[2], nMass[2], tMass[2], relVel[2];
	float ni[2], ti[2], maxNi[2];
};

/* Constraint row of one contact (reference src/contact_solver.c:597-808 for the 8-lane
 * layout; the scalar prepare, :21-147, computes the same values).  Points beyond the
 * manifold's count stay zero, like the reference's SIMD remainder data. */
__device__ __forceinline__ void prepare_row( Row& r, const b2gManifold* m, int ia, int ib, float4 massA, float4 massB,
											 const DevState& sA, const DevState& sB, float friction, float restitution,
											 const float* soft, float warm )
{
	r.ia = ia;
	r.ib = ib;
	r.count = m->count;
	r.n = m->normal;
	r.friction = friction;
	r.restitution = restitution;
	r.biasRate = soft[0];
	r.massScale = soft[1];
	r.impulseScale = soft[2];
	float mA = massA.y, iA = massA.w, mB = massB.y, iB = massB.w;
	r.mA = mA;
	r.iA = iA;
	r.mB = mB;
	r.iB = iB;
	b2gVec n = r.n;
	b2gVec t = gright( n );
	for ( int j = 0; j < 2; ++j )
	{
		r.rA[j] = gv( 0.0f, 0.0f );
		r.rB[j] = gv( 0.0f, 0.0f );
		r.base[j] = 0.0f;
		r.nMass[j] = 0.0f;
		r.tMass[j] = 0.0f;
		r.relVel[j] = 0.0f;
		r.ni[j] = 0.0f;
		r.ti[j] = 0.0f;
		r.maxNi[j] = 0.0f;
		if ( j < r.count )
		{
			const b2gPoint* mp = m->pts + j;
			b2gVec rA = mp->anchorA, rB = mp->anchorB;
			r.rA[j] = rA;
			r.rB[j] = rB;
			r.base[j] = mp->separation - gdot( gsub( rB, rA ), n );
			float rnA = gcross( rA, n ), rnB = gcross( rB, n );
			float kN = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
			float rtA = gcross( rA, t ), rtB = gcross( rB, t );
			float kT = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
			b2gVec vrA = gadd( sA.v, gcross_sv( sA.w, rA ) );
			b2gVec vrB = gadd( sB.v, gcross_sv( sB.w, rB ) );
			r.nMass[j] = kN > 0.0f ? 1.0f / kN : 0.0f;
			r.tMass[j] = kT > 0.0f ? 1.0f / kT : 0.0f;
			r.relVel[j] = gdot( n, gsub( vrB, vrA ) );
			r.ni[j] = warm * mp->normalImpulse;
			r.ti[j] = warm * mp->tangentImpulse;
		}
	}
}

/* ------------------------------------------------------------------ 8-lane path */
__device__ __forceinline__ void lane_apply( DevState& a, DevState& b, const Row& r, b2gVec rA, b2gVec rB, float Px, float Py )
{
	a.v.x = a.v.x - r.mA * Px;
	a.v.y = a.v.y - r.mA * Py;
	a.w = a.w - r.iA * ( rA.x * Py - rA.y * Px );
	b.v.x = b.v.x + r.mB * Px;
	b.v.y = b.v.y + r.mB * Py;
	b.w = b.w + r.iB * ( rB.x * Py - rB.y * Px );
}

__device__ __forceinline__ void warm_lane( const Row& r, DevState& a, DevState& b )
{
	float tX = r.n.y;
	float tY = 0.0f - r.n.x;
	for ( int j = 0; j < 2; ++j )
	{
		b2gVec rA = r.rA[j], rB = r.rB[j];
		float Px = r.ni[j] * r.n.x + r.ti[j] * tX;
		float Py = r.ni[j] * r.n.y + r.ti[j] * tY;
		a.w = a.w - r.iA * ( rA.x * Py - rA.y * Px );
		a.v.x = a.v.x - r.mA * Px;
		a.v.y = a.v.y - r.mA * Py;
		b.w = b.w + r.iB * ( rB.x * Py - rB.y * Px );
		b.v.x = b.v.x + r.mB * Px;
		b.v.y = b.v.y + r.mB * Py;
	}
}

__device__ __forceinline__ void solve_lane( Row& r, DevState& a, DevState& b, bool useBias, float inv_h, float pushout )
{
	float biasRate = useBias ? r.biasRate : 0.0f;
	float massScale = useBias ? r.massScale : 1.0f;
	float impulseScale = useBias ? r.impulseScale : 0.0f;
	float minBias = -pushout;
	b2gVec dp = gv( b.dp.x - a.dp.x, b.dp.y - a.dp.y );
	b2gVec n = r.n;
	for ( int j = 0; j < 2; ++j )
	{
		b2gVec aA = r.rA[j], aB = r.rB[j];
		b2gVec rsA = gv( a.dq.c * aA.x - a.dq.s * aA.y, a.dq.s * aA.x + a.dq.c * aA.y );
		b2gVec rsB = gv( b.dq.c * aB.x - b.dq.s * aB.y, b.dq.s * aB.x + b.dq.c * aB.y );
		b2gVec ds = gv( dp.x + ( rsB.x - rsA.x ), dp.y + ( rsB.y - rsA.y ) );
		float s = ( n.x * ds.x + n.y * ds.y ) + r.base[j];
		float specBias = s * inv_h;
		float softBias = gmax( biasRate * s, minBias );
		float bias = s > 0.0f ? specBias : softBias;
		float dvx = ( b.v.x - b.w * aB.y ) - ( a.v.x - a.w * aA.y );
		float dvy = ( b.v.y + b.w * aB.x ) - ( a.v.y + a.w * aA.x );
		float vn = dvx * n.x + dvy * n.y;
		float negImpulse = r.nMass[j] * ( massScale * ( vn + bias ) ) + impulseScale * r.ni[j];
		float newImpulse = gmax( r.ni[j] - negImpulse, 0.0f );
		float impulse = newImpulse - r.ni[j];
		r.ni[j] = newImpulse;
		r.maxNi[j] = gmax( r.maxNi[j], newImpulse );
		lane_apply( a, b, r, aA, aB, impulse * n.x, impulse * n.y );
	}
	float tX = n.y;
	float tY = 0.0f - n.x;
	for ( int j = 0; j < 2; ++j )
	{
		b2gVec aA = r.rA[j], aB = r.rB[j];
		float dvx = ( b.v.x - b.w * aB.y ) - ( a.v.x - a.w * aA.y );
		float dvy = ( b.v.y + b.w * aB.x ) - ( a.v.y + a.w * aA.x );
		float vt = dvx * tX + dvy * tY;
		float negImpulse = r.tMass[j] * vt;
		float maxFriction = r.friction * r.ni[j];
		float newImpulse = r.ti[j] - negImpulse;
		float lo = 0.0f - maxFriction;
		float mn = newImpulse < maxFriction ? newImpulse : maxFriction;
		newImpulse = lo > mn ? lo : mn;
		float impulse = newImpulse - r.ti[j];
		r.ti[j] = newImpulse;
		lane_apply( a, b, r, aA, aB, impulse * tX, impulse * tY );
	}
}

__device__ __forceinline__ void restitution_lane( Row& r, DevState& a, DevState& b, float threshold )
{
	b2gVec n = r.n;
	for ( int j = 0; j < 2; ++j )
	{
		bool skip = ( r.relVel[j] + threshold > 0.0f ) || ( r.maxNi[j] == 0.0f );
		float mass = skip ? 0.0f : r.nMass[j];
		b2gVec aA = r.rA[j], aB = r.rB[j];
		float dvx = ( b.v.x - b.w * aB.y ) - ( a.v.x - a.w * aA.y );
		float dvy = ( b.v.y + b.w * aB.x ) - ( a.v.y + a.w * aA.x );
		float vn = dvx * n.x + dvy * n.y;
		float negImpulse = mass * ( vn + r.restitution * r.relVel[j] );
		float newImpulse = gmax( r.ni[j] - negImpulse, 0.0f );
		float impulse = newImpulse - r.ni[j];
		r.ni[j] = newImpulse;
		lane_apply( a, b, r, aA, aB, impulse * n.x, impulse * n.y );
	}
}

/* ------------------------------------------------------------------ scalar overflow path */
/* Only the manifold's points, with the scalar path's operand grouping. */
__device__ __forceinline__ void warm_scalar( const Row& r, DevState& a, DevState& b )
{
	b2gVec t = gright( r.n );
	/* constant bounds keep the row's arrays in registers; points past count are skipped */
#pragma unroll
	for ( int j = 0; j < 2; ++j )
	{
		if ( j >= r.count )
			break;
		b2gVec P = gadd( gmulsv( r.ni[j], r.n ), gmulsv( r.ti[j], t ) );
		a.w -= r.iA * gcross( r.rA[j], P );
		a.v = gmuladd( a.v, -r.mA, P );
		b.w += r.iB * gcross( r.rB[j], P );
		b.v = gmuladd( b.v, r.mB, P );
	}
}

__device__ __forceinline__ void solve_scalar( Row& r, DevState& a, DevState& b, bool useBias, float inv_h, float pushout )
{
	b2gVec dp = gsub( b.dp, a.dp );
	b2gVec n = r.n, t = gright( n );
	/* constant bounds keep the row's arrays in registers; points past count are skipped */
#pragma unroll
	for ( int j = 0; j < 2; ++j )
	{
		if ( j >= r.count )
			break;
		b2gVec rA = r.rA[j], rB = r.rB[j];
		b2gVec ds = gadd( dp, gsub( grotate( b.dq, rB ), grotate( a.dq, rA ) ) );
		float s = gdot( ds, n ) + r.base[j];
		float velocityBias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
		if ( s > 0.0f )
			velocityBias = s * inv_h;
		else if ( useBias )
		{
			velocityBias = gmax( r.biasRate * s, -pushout );
			massScale = r.massScale;
			impulseScale = r.impulseScale;
		}
		b2gVec vrA = gadd( a.v, gcross_sv( a.w, rA ) );
		b2gVec vrB = gadd( b.v, gcross_sv( b.w, rB ) );
		float vn = gdot( gsub( vrB, vrA ), n );
		float impulse = -r.nMass[j] * massScale * ( vn + velocityBias ) - impulseScale * r.ni[j];
		float newImpulse = gmax( r.ni[j] + impulse, 0.0f );
		impulse = newImpulse - r.ni[j];
		r.ni[j] = newImpulse;
		r.maxNi[j] = gmax( r.maxNi[j], impulse );
		b2gVec P = gmulsv( impulse, n );
		a.v = gmulsub( a.v, r.mA, P );
		a.w -= r.iA * gcross( rA, P );
		b.v = gmuladd( b.v, r.mB, P );
		b.w += r.iB * gcross( rB, P );
	}
	/* constant bounds keep the row's arrays in registers; points past count are skipped */
#pragma unroll
	for ( int j = 0; j < 2; ++j )
	{
		if ( j >= r.count )
			break;
		b2gVec rA = r.rA[j], rB = r.rB[j];
		b2gVec vrB = gadd( b.v, gcross_sv( b.w, rB ) );
		b2gVec vrA = gadd( a.v, gcross_sv( a.w, rA ) );
		float vt = gdot( gsub( vrB, vrA ), t );
		float impulse = r.tMass[j] * ( -vt );
		float maxFriction = r.friction * r.ni[j];
		float newImpulse = gclamp( r.ti[j] + impulse, -maxFriction, maxFriction );
		impulse = newImpulse - r.ti[j];
		r.ti[j] = newImpulse;
		b2gVec P = gmulsv( impulse, t );
		a.v = gmulsub( a.v, r.mA, P );
		a.w -= r.iA * gcross( rA, P );
		b.v = gmuladd( b.v, r.mB, P );
		b.w += r.iB * gcross( rB, P );
	}
}

/* Returns false when the row has no restitution (the reference skips it entirely). */
__device__ __forceinline__ bool restitution_scalar( Row& r, DevState& a, DevState& b, float threshold )
{
	if ( r.restitution == 0.0f )
		return false;
	b2gVec n = r.n;
	/* constant bounds keep the row's arrays in registers; points past count are skipped */
#pragma unroll
	for ( int j = 0; j < 2; ++j )
	{
		if ( j >= r.count )
			break;
		if ( r.relVel[j] > -threshold || r.maxNi[j] == 0.0f )
			continue;
		b2gVec rA = r.rA[j], rB = r.rB[j];
		b2gVec vrB = gadd( b.v, gcross_sv( b.w, rB ) );
		b2gVec vrA = gadd( a.v, gcross_sv( a.w, rA ) );
		float vn = gdot( gsub( vrB, vrA ), n );
		float impulse = -r.nMass[j] * ( vn + r.restitution * r.relVel[j] );
		float newImpulse = gmax( r.ni[j] + impulse, 0.0f );
		impulse = newImpulse - r.ni[j];
		r.ni[j] = newImpulse;
		r.maxNi[j] = gmax( r.maxNi[j], impulse );
		b2gVec P = gmulsv( impulse, n );
		a.v = gmulsub( a.v, r.mA, P );
		a.w -= r.iA * gcross( rA, P );
		b.v = gmuladd( b.v, r.mB, P );
		b.w += r.iB * gcross( rB, P );
	}
	return true;
}

/* ------------------------------------------------------------------ joints */
#include "b2g_joints.h"

/* ------------------------------------------------------------------ body integration */
/* Per-step velocity increments of one body (reference src/solver.c:34-93): the same
 * values every substep, so they are computed once per step. */
struct VelocityTerms
{
	b2gVec lvd;
	float avd, ld, ad;
};

__device__ __forceinline__ VelocityTerms velocity_terms( float4 ms, float4 fo, float4 ex, const b2gStepConst& sc )
{
	float h = sc.h;
	VelocityTerms t;
	t.ld = 1.0f / ( 1.0f + h * ex.x );
	t.ad = 1.0f / ( 1.0f + h * ex.y );
	t.lvd = gmulsv( h * ms.y, gmuladd( gv( fo.x, fo.y ), ms.x * fo.w, sc.gravity ) );
	t.avd = h * ms.w * fo.z;
	return t;
}

__device__ __forceinline__ void integrate_velocity( DevState& s, const VelocityTerms& t, const b2gStepConst& sc )
{
	float maxLin = B2G_MAX_TRANSLATION * sc.inv_dt;
	float maxAng = B2G_MAX_ROTATION * sc.inv_dt;
	float maxLin2 = maxLin * maxLin, maxAng2 = maxAng * maxAng;
	b2gVec v = gmuladd( t.lvd, t.ld, s.v );
	float w = t.avd + t.ad * s.w;
	if ( gdot( v, v ) > maxLin2 )
	{
		float ratio = maxLin / glen( v );
		v = gmulsv( ratio, v );
	}
	if ( w * w > maxAng2 )
	{
		float ratio = maxAng / gabs( w );
		w *= ratio;
	}
	s.v = v;
	s.w = w;
}

__device__ __forceinline__ void integrate_position( DevState& s, float h )
{
	s.dq = gintrot( s.dq, h * s.w );
	s.dp = gmuladd( s.dp, h, s.v );
}

/* Body states in one CTA's shared memory, by index (a body id or a slot); -1 is a static
 * body.  Stores write the velocity word only: no row or joint phase changes dp or dq. */
struct SharedBodies
{
	float4* st0;
	float4* st1;
	__device__ __forceinline__ DevState load( int b ) const
	{
		return b < 0 ? identity_state() : state_of( st0[b], st1[b] );
	}
	__device__ __forceinline__ DevState load_velocity( int b ) const
	{
		return b < 0 ? identity_state() : state_of( st0[b], make_float4( 0.0f, 0.0f, 1.0f, 0.0f ) );
	}
	__device__ __forceinline__ void store( int b, const DevState& x ) const
	{
		if ( b >= 0 )
			st0[b] = velocity_word( x );
	}
};
