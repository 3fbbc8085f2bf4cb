/*
 * kernels.cu -- sm_103a kernels of the per-step contact pipeline and their launch
 * sequences.
 *
 * Stage                reference                                  kernel
 * contact creation     src/contact.c:185-332 (sim part)           k_scatter_contacts
 * narrowphase          src/world.c:290-365, src/contact.c:493-582 k_collide
 * prepare contacts     src/contact_solver.c:21-147, :597-808       k_prepare
 * prepare joints       src/revolute_joint.c:201-270                k_prepare_joints
 * integrate velocities src/solver.c:34-93                          k_integrate_velocities
 * warm start / solve / relax / restitution
 *                      src/contact_solver.c:149-440 (overflow)     k_overflow (serial)
 *                      src/contact_solver.c:810-1178 (8-lane)      k_color (one colour)
 *                      src/revolute_joint.c:272-470                (joints inside both)
 * integrate positions  src/solver.c:146-163                        k_integrate_positions
 * store impulses       src/contact_solver.c:442-471, :1180-1293    k_store
 * finalize bodies      src/solver.c:165-351 (+ fast-body sweep
 *                      boxes, :787-1105)                           k_finalize
 *
 * Within one graph colour no two constraints share a non-static body
 * (src/constraint_graph.c:84-131), so a colour runs fully in parallel and still gives
 * the reference's results bit for bit: one thread owns one constraint row (or joint),
 * gathers the two 32-byte body states with float4 loads, and scatters the velocities.
 * All arithmetic keeps the reference operand order; this file is compiled with
 * --fmad=false so no multiply-add is contracted.
 */
#include "b2g_collide.h"
#include "b2g_device.h"

#include <cuda_runtime.h>

#include <stdio.h>

#define BLOCK 256

/* ------------------------------------------------------------------ state access */
struct DevState
{
	b2gVec v;
	float w;
	b2gVec dp;
	b2gRot dq;
};

__device__ __forceinline__ DevState load_state( const b2gDevWorld& W, int b )
{
	DevState s;
	if ( b < 0 )
	{
		s.v = gv( 0.0f, 0.0f );
		s.w = 0.0f;
		s.dp = gv( 0.0f, 0.0f );
		s.dq = grot( 1.0f, 0.0f );
		return s;
	}
	const float4* st = (const float4*)W.state;
	float4 a = st[2 * b];
	float4 c = st[2 * b + 1];
	s.v = gv( a.x, a.y );
	s.w = a.z;
	s.dp = gv( c.x, c.y );
	s.dq = grot( c.z, c.w );
	return s;
}

__device__ __forceinline__ void store_velocity( const b2gDevWorld& W, int b, b2gVec v, float w )
{
	if ( b < 0 )
		return;
	float4* st = (float4*)W.state;
	float4 a = st[2 * b];
	a.x = v.x;
	a.y = v.y;
	a.z = w;
	st[2 * b] = a;
}

__device__ __forceinline__ b2gBox box_of( float4 f )
{
	b2gBox b;
	b.lo = gv( f.x, f.y );
	b.hi = gv( f.z, f.w );
	return b;
}

__device__ __forceinline__ float4 f4_of( b2gBox b ) { return make_float4( b.lo.x, b.lo.y, b.hi.x, b.hi.y ); }

/* Shape AABB (reference src/geometry.c:385-430, src/shape.c:457-478). */
__device__ b2gBox shape_aabb( const b2gShapeGeo& g, b2gXf xf )
{
	b2gBox b;
	switch ( g.type )
	{
		case 0:
		{
			b2gVec p = gxfpoint( xf, g.v[0] );
			float r = g.radius;
			b.lo = gv( p.x - r, p.y - r );
			b.hi = gv( p.x + r, p.y + r );
			return b;
		}
		case 1:
		{
			b2gVec v1 = gxfpoint( xf, g.v[0] );
			b2gVec v2 = gxfpoint( xf, g.v[1] );
			b2gVec r = gv( g.radius, g.radius );
			b.lo = gsub( gminv( v1, v2 ), r );
			b.hi = gadd( gmaxv( v1, v2 ), r );
			return b;
		}
		case 2:
		{
			b2gVec v1 = gxfpoint( xf, g.v[0] );
			b2gVec v2 = gxfpoint( xf, g.v[1] );
			b.lo = gminv( v1, v2 );
			b.hi = gmaxv( v1, v2 );
			return b;
		}
		default:
		{
			b2gVec lo = gxfpoint( xf, g.v[0] );
			b2gVec hi = lo;
			for ( int i = 1; i < g.count; ++i )
			{
				b2gVec v = gxfpoint( xf, g.v[i] );
				lo = gminv( lo, v );
				hi = gmaxv( hi, v );
			}
			b2gVec r = gv( g.radius, g.radius );
			b.lo = gsub( lo, r );
			b.hi = gadd( hi, r );
			return b;
		}
	}
}

/* ------------------------------------------------------------------ contact creation */
__global__ void k_scatter_contacts( b2gDevWorld W, const b2gContactInit* inits, int n )
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if ( t >= n )
		return;
	b2gContactInit c = inits[t];
	int id = c.id;
	if ( c.flags & B2G_INIT_KILL )
	{
		W.cFlags[id] = 0;
		return;
	}
	W.cShapes[2 * id] = c.shapeA;
	W.cShapes[2 * id + 1] = c.shapeB;
	W.cMix[2 * id] = c.friction;
	W.cMix[2 * id + 1] = c.restitution;
	W.cFlags[id] = B2G_C_LIVE;
	W.cBodies[2 * id] = -1;
	W.cBodies[2 * id + 1] = -1;
	b2gManifold m;
	gmanifold_clear( &m );
	W.manifold[id] = m;
}

/* ------------------------------------------------------------------ narrowphase */
/* Manifold of one shape pair; sensors never generate points.  Kept behind a call
 * boundary: inlined into k_collide, this routine returned empty manifolds for touching
 * boxes on sm_103a (nvcc 13.0.88, -O3 --fmad=false) while the same source called from a
 * one-thread kernel, or on the host, was correct; the non-inlined form is correct in
 * both kernels and bit-identical to the reference. */
__device__ __noinline__ void narrowphase( b2gManifold* m, const b2gShapeGeo* gA, b2gXf xfA, const b2gShapeGeo* gB, b2gXf xfB )
{
	if ( gA->isSensor || gB->isSensor )
		gmanifold_clear( m );
	else
		gcollide_shapes( m, gA, xfA, gB, xfB );
}

__device__ __forceinline__ void emit_event( const b2gDevWorld& W, int id, int code )
{
	int slot = atomicAdd( W.counters + 0, 1 );
	if ( slot < W.eventCap )
		W.events[slot] = ( id << 2 ) | code;
}

__global__ void __launch_bounds__( BLOCK ) k_collide( b2gDevWorld W, int idCount )
{
	int id = blockIdx.x * blockDim.x + threadIdx.x;
	if ( id >= idCount )
		return;
	uint32_t flags = W.cFlags[id];
	if ( ( flags & B2G_C_LIVE ) == 0 )
		return;
	int sA = W.cShapes[2 * id];
	int sB = W.cShapes[2 * id + 1];
	const float4* fat = (const float4*)W.fat;
	if ( gbox_overlaps( box_of( fat[sA] ), box_of( fat[sB] ) ) == false )
	{
		/* the host destroys the contact while processing this event */
		W.cFlags[id] = 0;
		emit_event( W, id, B2G_EV_DISJOINT );
		return;
	}
	bool wasTouching = ( flags & B2G_C_TOUCHING ) != 0;
	const b2gShapeGeo* gA = W.geo + sA;
	const b2gShapeGeo* gB = W.geo + sB;
	int bA = gA->bodyId;
	int bB = gB->bodyId;
	int infoA = W.bodyInfo[bA];
	int infoB = W.bodyInfo[bB];
	W.cBodies[2 * id] = ( infoA & B2G_B_AWAKE ) ? bA : -1;
	W.cBodies[2 * id + 1] = ( infoB & B2G_B_AWAKE ) ? bB : -1;
	const float4* xf = (const float4*)W.xf;
	const float4* centers = (const float4*)W.centers;
	float4 xa = xf[bA], xb = xf[bB];
	b2gXf xfA, xfB;
	xfA.p = gv( xa.x, xa.y );
	xfA.q = grot( xa.z, xa.w );
	xfB.p = gv( xb.x, xb.y );
	xfB.q = grot( xb.z, xb.w );
	float4 ca = centers[bA], cb = centers[bB];
	b2gVec offA = grotate( xfA.q, gv( ca.z, ca.w ) );
	b2gVec offB = grotate( xfB.q, gv( cb.z, cb.w ) );

	b2gManifold old = W.manifold[id];
	b2gManifold m;
	narrowphase( &m, gA, xfA, gB, xfB );

	int pointCount = m.count;
	bool touching = pointCount > 0;
	for ( int i = 0; i < pointCount; ++i )
	{
		b2gPoint* mp2 = m.pts + i;
		mp2->anchorA = gsub( mp2->anchorA, offA );
		mp2->anchorB = gsub( mp2->anchorB, offB );
		mp2->normalImpulse = 0.0f;
		mp2->tangentImpulse = 0.0f;
		mp2->maxNormalImpulse = 0.0f;
		mp2->normalVelocity = 0.0f;
		mp2->persisted = 0;
		for ( int j = 0; j < old.count; ++j )
		{
			if ( old.pts[j].id == mp2->id )
			{
				mp2->normalImpulse = old.pts[j].normalImpulse;
				mp2->tangentImpulse = old.pts[j].tangentImpulse;
				mp2->persisted = 1;
				break;
			}
		}
	}
	W.manifold[id] = m;
	uint32_t nf = B2G_C_LIVE | ( touching ? B2G_C_TOUCHING : 0u );
	if ( touching && ( gA->enableHitEvents || gB->enableHitEvents ) )
		nf |= B2G_C_HIT;
	W.cFlags[id] = nf;
	if ( touching && !wasTouching )
		emit_event( W, id, B2G_EV_STARTED );
	else if ( !touching && wasTouching )
		emit_event( W, id, B2G_EV_STOPPED );
}

/* ------------------------------------------------------------------ constraint rows */
__global__ void __launch_bounds__( BLOCK ) k_prepare( b2gDevWorld W, int total, b2gStepConst sc )
{
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if ( k >= total )
		return;
	/* a null solve list means rows are the contacts in order */
	int cid = W.solveList ? W.solveList[k] : k;
	const b2gManifold* m = W.manifold + cid;
	int ia = W.cBodies[2 * cid];
	int ib = W.cBodies[2 * cid + 1];
	/* inverse masses of the reference's contact sim: the body's, zero for static bodies */
	const float4* mass = (const float4*)W.mass;
	float4 ma = ia >= 0 ? mass[ia] : make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	float4 mb = ib >= 0 ? mass[ib] : make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	float mA = ma.y, iA = ma.w, mB = mb.y, iB = mb.w;
	float friction = W.cMix[2 * cid];
	float restitution = W.cMix[2 * cid + 1];
	DevState sA = load_state( W, ia );
	DevState sB = load_state( W, ib );
	const float* soft = ( ia < 0 || ib < 0 ) ? sc.staticSoft : sc.contactSoft;
	b2gVec n = m->normal;
	int count = m->count;
	float warm = sc.enableWarmStarting ? 1.0f : 0.0f;

	( (int4*)W.kIdx )[k] = make_int4( ia, ib, cid, count );
	( (float4*)W.kNF )[k] = make_float4( n.x, n.y, friction, restitution );
	( (float4*)W.kSoft )[k] = make_float4( soft[0], soft[1], soft[2], 0.0f );
	( (float4*)W.kMass )[k] = make_float4( mA, iA, mB, iB );
	b2gVec t = gright( n );
	for ( int j = 0; j < 2; ++j )
	{
		float4 anchor = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		float4 coef = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		float4 imp = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		if ( j < count )
		{
			const b2gPoint* mp = m->pts + j;
			b2gVec rA = mp->anchorA, rB = mp->anchorB;
			float base = mp->separation - gdot( gsub( rB, rA ), n );
			float rnA = gcross( rA, n ), rnB = gcross( rB, n );
			float kN = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
			float rtA = gcross( rA, t ), rtB = gcross( rB, t );
			float kT = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
			b2gVec vrA = gadd( sA.v, gcross_sv( sA.w, rA ) );
			b2gVec vrB = gadd( sB.v, gcross_sv( sB.w, rB ) );
			float relVel = gdot( n, gsub( vrB, vrA ) );
			anchor = make_float4( rA.x, rA.y, rB.x, rB.y );
			coef = make_float4( base, kN > 0.0f ? 1.0f / kN : 0.0f, kT > 0.0f ? 1.0f / kT : 0.0f, relVel );
			imp = make_float4( warm * mp->normalImpulse, warm * mp->tangentImpulse, 0.0f, 0.0f );
		}
		( (float4*)W.kAnchor[j] )[k] = anchor;
		( (float4*)W.kCoef[j] )[k] = coef;
		( (float4*)W.kImp[j] )[k] = imp;
	}
}

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

__device__ __forceinline__ void load_row( const b2gDevWorld& W, int k, Row& r )
{
	int4 idx = ( (const int4*)W.kIdx )[k];
	float4 nf = ( (const float4*)W.kNF )[k];
	float4 so = ( (const float4*)W.kSoft )[k];
	float4 ms = ( (const float4*)W.kMass )[k];
	r.ia = idx.x;
	r.ib = idx.y;
	r.count = idx.w;
	r.n = gv( nf.x, nf.y );
	r.friction = nf.z;
	r.restitution = nf.w;
	r.biasRate = so.x;
	r.massScale = so.y;
	r.impulseScale = so.z;
	r.mA = ms.x;
	r.iA = ms.y;
	r.mB = ms.z;
	r.iB = ms.w;
	for ( int j = 0; j < 2; ++j )
	{
		float4 a = ( (const float4*)W.kAnchor[j] )[k];
		float4 c = ( (const float4*)W.kCoef[j] )[k];
		float4 i = ( (const float4*)W.kImp[j] )[k];
		r.rA[j] = gv( a.x, a.y );
		r.rB[j] = gv( a.z, a.w );
		r.base[j] = c.x;
		r.nMass[j] = c.y;
		r.tMass[j] = c.z;
		r.relVel[j] = c.w;
		r.ni[j] = i.x;
		r.ti[j] = i.y;
		r.maxNi[j] = i.z;
	}
}

__device__ __forceinline__ void store_impulses( const b2gDevWorld& W, int k, const Row& r )
{
	for ( int j = 0; j < 2; ++j )
		( (float4*)W.kImp[j] )[k] = make_float4( r.ni[j], r.ti[j], r.maxNi[j], 0.0f );
}

/* 8-lane path: both point slots are evaluated (slot 1 of a one-point manifold carries
 * zeros, like the reference's SIMD remainder data). */
__device__ __forceinline__ void lane_apply( DevState& a, DevState& b, const Row& r, b2gVec rA, b2gVec rB, float Px, float Py )
{
	a.v.x = a.v.x - r.mA * Px;
	a.v.y = a.v.y - r.mA * Py;
	a.w = a.w - r.iA * ( rA.x * Py - rA.y * Px );
	b.v.x = b.v.x + r.mB * Px;
	b.v.y = b.v.y + r.mB * Py;
	b.w = b.w + r.iB * ( rB.x * Py - rB.y * Px );
}

__device__ void lane_warm( const b2gDevWorld& W, int k )
{
	Row r;
	load_row( W, k, r );
	DevState a = load_state( W, r.ia );
	DevState b = load_state( W, r.ib );
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
	store_velocity( W, r.ia, a.v, a.w );
	store_velocity( W, r.ib, b.v, b.w );
}

__device__ void lane_solve( const b2gDevWorld& W, int k, bool useBias, float inv_h, float pushout )
{
	Row r;
	load_row( W, k, r );
	DevState a = load_state( W, r.ia );
	DevState b = load_state( W, r.ib );
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
	store_velocity( W, r.ia, a.v, a.w );
	store_velocity( W, r.ib, b.v, b.w );
	store_impulses( W, k, r );
}

__device__ void lane_restitution( const b2gDevWorld& W, int k, float threshold )
{
	Row r;
	load_row( W, k, r );
	DevState a = load_state( W, r.ia );
	DevState b = load_state( W, r.ib );
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
	store_velocity( W, r.ia, a.v, a.w );
	store_velocity( W, r.ib, b.v, b.w );
	store_impulses( W, k, r );
}

/* Overflow (scalar) path: only the manifold's points, different operand grouping. */
__device__ void ovf_warm( const b2gDevWorld& W, int k )
{
	Row r;
	load_row( W, k, r );
	DevState a = load_state( W, r.ia );
	DevState b = load_state( W, r.ib );
	b2gVec t = gright( r.n );
	for ( int j = 0; j < r.count; ++j )
	{
		b2gVec P = gadd( gmulsv( r.ni[j], r.n ), gmulsv( r.ti[j], t ) );
		a.w -= r.iA * gcross( r.rA[j], P );
		a.v = gmuladd( a.v, -r.mA, P );
		b.w += r.iB * gcross( r.rB[j], P );
		b.v = gmuladd( b.v, r.mB, P );
	}
	store_velocity( W, r.ia, a.v, a.w );
	store_velocity( W, r.ib, b.v, b.w );
}

__device__ void ovf_solve( const b2gDevWorld& W, int k, bool useBias, float inv_h, float pushout )
{
	Row r;
	load_row( W, k, r );
	DevState a = load_state( W, r.ia );
	DevState b = load_state( W, r.ib );
	b2gVec dp = gsub( b.dp, a.dp );
	b2gVec n = r.n, t = gright( n );
	for ( int j = 0; j < r.count; ++j )
	{
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
	for ( int j = 0; j < r.count; ++j )
	{
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
	store_velocity( W, r.ia, a.v, a.w );
	store_velocity( W, r.ib, b.v, b.w );
	store_impulses( W, k, r );
}

__device__ void ovf_restitution( const b2gDevWorld& W, int k, float threshold )
{
	Row r;
	load_row( W, k, r );
	if ( r.restitution == 0.0f )
		return;
	DevState a = load_state( W, r.ia );
	DevState b = load_state( W, r.ib );
	b2gVec n = r.n;
	for ( int j = 0; j < r.count; ++j )
	{
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
	store_velocity( W, r.ia, a.v, a.w );
	store_velocity( W, r.ib, b.v, b.w );
	store_impulses( W, k, r );
}

/* ------------------------------------------------------------------ revolute joint */
__device__ float rel_angle( b2gRot b, b2gRot a )
{
	float s = b.s * a.c - b.c * a.s;
	float c = b.c * a.c + b.s * a.s;
	return atan2f( s, c );
}

__device__ float unwind( float a )
{
	if ( a < -B2G_PI )
		return a + 2.0f * B2G_PI;
	if ( a > B2G_PI )
		return a - 2.0f * B2G_PI;
	return a;
}

__device__ void make_soft( float hertz, float zeta, float h, float* out )
{
	if ( hertz == 0.0f )
	{
		out[0] = 0.0f;
		out[1] = 1.0f;
		out[2] = 0.0f;
		return;
	}
	float omega = 2.0f * B2G_PI * hertz;
	float a1 = 2.0f * zeta + h * omega;
	float a2 = h * omega * a1;
	float a3 = 1.0f / ( 1.0f + a2 );
	out[0] = omega / a1;
	out[1] = a2 * a3;
	out[2] = a3;
}

__global__ void k_prepare_joints( b2gDevWorld W, int count, b2gStepConst sc )
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if ( t >= count )
		return;
	b2gJointDev* j = W.joints + W.jointList[t];
	const float4* mass = (const float4*)W.mass;
	const float4* xf = (const float4*)W.xf;
	const float4* centers = (const float4*)W.centers;
	int a = j->bodyIdA, b = j->bodyIdB;
	float4 ma = mass[a], mb = mass[b];
	j->invMassA = ma.y;
	j->invMassB = mb.y;
	j->invIA = ma.w;
	j->invIB = mb.w;
	j->indexA = ( W.bodyInfo[a] & B2G_B_AWAKE ) ? a : -1;
	j->indexB = ( W.bodyInfo[b] & B2G_B_AWAKE ) ? b : -1;
	float4 xa = xf[a], xb = xf[b];
	float4 ca = centers[a], cb = centers[b];
	b2gRot qA = grot( xa.z, xa.w ), qB = grot( xb.z, xb.w );
	j->anchorA = grotate( qA, gsub( j->localAnchorA, gv( ca.z, ca.w ) ) );
	j->anchorB = grotate( qB, gsub( j->localAnchorB, gv( cb.z, cb.w ) ) );
	j->deltaCenter = gsub( gv( cb.x, cb.y ), gv( ca.x, ca.y ) );
	j->deltaAngle = rel_angle( qB, qA ) - j->referenceAngle;
	j->deltaAngle = unwind( j->deltaAngle );
	float k = j->invIA + j->invIB;
	j->axialMass = k > 0.0f ? 1.0f / k : 0.0f;
	float s[3];
	make_soft( j->hertz, j->dampingRatio, sc.h, s );
	j->springBias = s[0];
	j->springMass = s[1];
	j->springImpulseScale = s[2];
	if ( sc.enableWarmStarting == 0 )
	{
		j->linearImpulse = gv( 0.0f, 0.0f );
		j->springImpulse = 0.0f;
		j->motorImpulse = 0.0f;
		j->lowerImpulse = 0.0f;
		j->upperImpulse = 0.0f;
	}
}

__device__ void joint_warm( const b2gDevWorld& W, int jid )
{
	b2gJointDev* j = W.joints + jid;
	DevState a = load_state( W, j->indexA );
	DevState b = load_state( W, j->indexB );
	b2gVec rA = grotate( a.dq, j->anchorA );
	b2gVec rB = grotate( b.dq, j->anchorB );
	float axial = j->springImpulse + j->motorImpulse + j->lowerImpulse - j->upperImpulse;
	a.v = gmulsub( a.v, j->invMassA, j->linearImpulse );
	a.w -= j->invIA * ( gcross( rA, j->linearImpulse ) + axial );
	b.v = gmuladd( b.v, j->invMassB, j->linearImpulse );
	b.w += j->invIB * ( gcross( rB, j->linearImpulse ) + axial );
	store_velocity( W, j->indexA, a.v, a.w );
	store_velocity( W, j->indexB, b.v, b.w );
}

__device__ void joint_solve( const b2gDevWorld& W, int jid, bool useBias, const b2gStepConst& sc )
{
	b2gJointDev* j = W.joints + jid;
	float mA = j->invMassA, mB = j->invMassB, iA = j->invIA, iB = j->invIB;
	DevState a = load_state( W, j->indexA );
	DevState b = load_state( W, j->indexB );
	b2gVec vA = a.v, vB = b.v;
	float wA = a.w, wB = b.w;
	bool fixedRotation = ( iA + iB == 0.0f );
	if ( j->enableSpring && fixedRotation == false )
	{
		float C = rel_angle( b.dq, a.dq ) + j->deltaAngle;
		float bias = j->springBias * C;
		float Cdot = wB - wA;
		float impulse = -j->springMass * j->axialMass * ( Cdot + bias ) - j->springImpulseScale * j->springImpulse;
		j->springImpulse += impulse;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableMotor && fixedRotation == false )
	{
		float Cdot = wB - wA - j->motorSpeed;
		float impulse = -j->axialMass * Cdot;
		float old = j->motorImpulse;
		float maxImpulse = sc.h * j->maxMotorTorque;
		j->motorImpulse = gclamp( j->motorImpulse + impulse, -maxImpulse, maxImpulse );
		impulse = j->motorImpulse - old;
		wA -= iA * impulse;
		wB += iB * impulse;
	}
	if ( j->enableLimit && fixedRotation == false )
	{
		float angle = unwind( rel_angle( b.dq, a.dq ) + j->deltaAngle );
		{
			float C = angle - j->lowerAngle;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * sc.inv_h;
			else if ( useBias )
			{
				bias = sc.jointSoft[0] * C;
				massScale = sc.jointSoft[1];
				impulseScale = sc.jointSoft[2];
			}
			float Cdot = wB - wA;
			float impulse = -massScale * j->axialMass * ( Cdot + bias ) - impulseScale * j->lowerImpulse;
			float old = j->lowerImpulse;
			j->lowerImpulse = gmax( j->lowerImpulse + impulse, 0.0f );
			impulse = j->lowerImpulse - old;
			wA -= iA * impulse;
			wB += iB * impulse;
		}
		{
			float C = j->upperAngle - angle;
			float bias = 0.0f, massScale = 1.0f, impulseScale = 0.0f;
			if ( C > 0.0f )
				bias = C * sc.inv_h;
			else if ( useBias )
			{
				bias = sc.jointSoft[0] * C;
				massScale = sc.jointSoft[1];
				impulseScale = sc.jointSoft[2];
			}
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
		b2gVec rhs = gadd( Cdot, bias );
		float det = k11 * k22 - k12 * k12;
		if ( det != 0.0f )
			det = 1.0f / det;
		b2gVec x = gv( det * ( k22 * rhs.x - k12 * rhs.y ), det * ( k11 * rhs.y - k12 * rhs.x ) );
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
	store_velocity( W, j->indexA, vA, wA );
	store_velocity( W, j->indexB, vB, wB );
}

/* ------------------------------------------------------------------ phases */
enum
{
	PH_WARM = 0,
	PH_SOLVE = 1,
	PH_RELAX = 2,
	PH_RESTITUTION = 3,
};

/* One graph colour: threads [0, jointCount) run joints, the rest run contact rows. */
__global__ void __launch_bounds__( BLOCK )
	k_color( b2gDevWorld W, int phase, int jointStart, int jointCount, int rowStart, int rowCount, b2gStepConst sc )
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if ( t < jointCount )
	{
		int jid = W.jointList[jointStart + t];
		if ( phase == PH_WARM )
			joint_warm( W, jid );
		else if ( phase == PH_SOLVE )
			joint_solve( W, jid, true, sc );
		else if ( phase == PH_RELAX )
			joint_solve( W, jid, false, sc );
		return;
	}
	t -= jointCount;
	if ( t >= rowCount )
		return;
	int k = rowStart + t;
	if ( phase == PH_WARM )
		lane_warm( W, k );
	else if ( phase == PH_SOLVE )
		lane_solve( W, k, true, sc.inv_h, sc.pushout );
	else if ( phase == PH_RELAX )
		lane_solve( W, k, false, sc.inv_h, sc.pushout );
	else
		lane_restitution( W, k, sc.restitutionThreshold );
}

/* Overflow constraints share bodies, so they run serially in list order (joints first). */
__global__ void k_overflow( b2gDevWorld W, int phase, int jointStart, int jointCount, int rowStart, int rowCount, b2gStepConst sc )
{
	if ( threadIdx.x != 0 || blockIdx.x != 0 )
		return;
	if ( phase != PH_RESTITUTION )
	{
		for ( int i = 0; i < jointCount; ++i )
		{
			int jid = W.jointList[jointStart + i];
			if ( phase == PH_WARM )
				joint_warm( W, jid );
			else
				joint_solve( W, jid, phase == PH_SOLVE, sc );
		}
	}
	for ( int i = 0; i < rowCount; ++i )
	{
		int k = rowStart + i;
		if ( phase == PH_WARM )
			ovf_warm( W, k );
		else if ( phase == PH_SOLVE )
			ovf_solve( W, k, true, sc.inv_h, sc.pushout );
		else if ( phase == PH_RELAX )
			ovf_solve( W, k, false, sc.inv_h, sc.pushout );
		else
			ovf_restitution( W, k, sc.restitutionThreshold );
	}
}

/* ------------------------------------------------------------------ bodies */
__global__ void __launch_bounds__( BLOCK ) k_integrate_velocities( b2gDevWorld W, int awakeCount, b2gStepConst sc )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= awakeCount )
		return;
	int b = W.awake[i];
	float4* st = (float4*)W.state;
	float4 s0 = st[2 * b];
	float4 ms = ( (const float4*)W.mass )[b];
	float4 fo = ( (const float4*)W.force )[b];
	float4 ex = ( (const float4*)W.extent )[b];
	float h = sc.h;
	float maxLin = B2G_MAX_TRANSLATION * sc.inv_dt;
	float maxAng = B2G_MAX_ROTATION * sc.inv_dt;
	float maxLin2 = maxLin * maxLin, maxAng2 = maxAng * maxAng;
	b2gVec v = gv( s0.x, s0.y );
	float w = s0.z;
	float ld = 1.0f / ( 1.0f + h * ex.x );
	float ad = 1.0f / ( 1.0f + h * ex.y );
	b2gVec lvd = gmulsv( h * ms.y, gmuladd( gv( fo.x, fo.y ), ms.x * fo.w, sc.gravity ) );
	float avd = h * ms.w * fo.z;
	v = gmuladd( lvd, ld, v );
	w = avd + ad * w;
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
	s0.x = v.x;
	s0.y = v.y;
	s0.z = w;
	st[2 * b] = s0;
}

__global__ void __launch_bounds__( BLOCK ) k_integrate_positions( b2gDevWorld W, int awakeCount, b2gStepConst sc )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= awakeCount )
		return;
	int b = W.awake[i];
	float4* st = (float4*)W.state;
	float4 s0 = st[2 * b];
	float4 s1 = st[2 * b + 1];
	b2gRot dq = gintrot( grot( s1.z, s1.w ), sc.h * s0.z );
	b2gVec dp = gmuladd( gv( s1.x, s1.y ), sc.h, gv( s0.x, s0.y ) );
	st[2 * b + 1] = make_float4( dp.x, dp.y, dq.c, dq.s );
}

__global__ void __launch_bounds__( BLOCK ) k_store( b2gDevWorld W, int total, int overflowStart )
{
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if ( k >= total )
		return;
	int4 idx = ( (const int4*)W.kIdx )[k];
	b2gManifold* m = W.manifold + idx.z;
	int n = k < overflowStart ? 2 : idx.w;
	for ( int j = 0; j < n; ++j )
	{
		float4 imp = ( (const float4*)W.kImp[j] )[k];
		float4 coef = ( (const float4*)W.kCoef[j] )[k];
		m->pts[j].normalImpulse = imp.x;
		m->pts[j].tangentImpulse = imp.y;
		m->pts[j].maxNormalImpulse = imp.z;
		m->pts[j].normalVelocity = coef.w;
	}
}

__device__ __forceinline__ void emit_record( const b2gDevWorld& W, int awakeIndex, int slot, int shapeId, int flags, b2gBox fat,
											 b2gBox sweep )
{
	int r = atomicAdd( W.counters + 1, 1 );
	if ( r >= W.recordCap )
		return;
	b2gRecord rec;
	rec.awakeIndex = awakeIndex;
	rec.slot = slot;
	rec.shapeId = shapeId;
	rec.flags = flags;
	rec.fat[0] = fat.lo.x;
	rec.fat[1] = fat.lo.y;
	rec.fat[2] = fat.hi.x;
	rec.fat[3] = fat.hi.y;
	rec.sweep[0] = sweep.lo.x;
	rec.sweep[1] = sweep.lo.y;
	rec.sweep[2] = sweep.hi.x;
	rec.sweep[3] = sweep.hi.y;
	W.records[r] = rec;
}

__global__ void __launch_bounds__( BLOCK ) k_finalize( b2gDevWorld W, int awakeCount, b2gStepConst sc )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= awakeCount )
		return;
	int b = W.awake[i];
	float4* st = (float4*)W.state;
	float4 s0 = st[2 * b];
	float4 s1 = st[2 * b + 1];
	float4* xfs = (float4*)W.xf;
	float4* cen = (float4*)W.centers;
	float4* prev = (float4*)W.prev;
	float4 x = xfs[b];
	float4 c = cen[b];
	float4 ex = ( (const float4*)W.extent )[b];
	int info = W.bodyInfo[b];

	b2gVec v = gv( s0.x, s0.y );
	float w = s0.z;
	b2gVec dp = gv( s1.x, s1.y );
	b2gRot dq = grot( s1.z, s1.w );
	b2gVec center = gadd( gv( c.x, c.y ), dp );
	b2gRot q = gnormrot( gmulrot( dq, grot( x.z, x.w ) ) );
	float maxExtent = ex.w, minExtent = ex.z;
	float maxVelocity = glen( v ) + gabs( w ) * maxExtent;
	float maxDeltaPosition = glen( dp ) + gabs( dq.s ) * maxExtent;
	float sleepVelocity = gmax( maxVelocity, 0.5f * sc.inv_dt * maxDeltaPosition );
	st[2 * b + 1] = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
	b2gVec p = gsub( center, grotate( q, gv( c.z, c.w ) ) );
	b2gXf xf;
	xf.p = p;
	xf.q = q;
	xfs[b] = make_float4( p.x, p.y, q.c, q.s );
	cen[b] = make_float4( center.x, center.y, c.z, c.w );
	float4* fo = (float4*)W.force;
	float4 f = fo[b];
	fo[b] = make_float4( 0.0f, 0.0f, 0.0f, f.w );

	bool isFast = false;
	float sleepThreshold = s0.w;
	if ( sc.enableSleep == 0 || ( info & B2G_B_SLEEP_OK ) == 0 || sleepVelocity > sleepThreshold )
	{
		if ( ( info & B2G_B_TYPE_MASK ) == 2 && sc.enableContinuous && maxVelocity * sc.dt > 0.5f * minExtent )
			isFast = true;
	}
	/* with no time-of-impact event the fast body also advances its sweep start */
	prev[b] = make_float4( center.x, center.y, q.c, q.s );

	int start = W.shapeRange[2 * b];
	int count = W.shapeRange[2 * b + 1];
	float4* aabbs = (float4*)W.aabb;
	float4* fats = (float4*)W.fat;
	int bullet = ( info & B2G_B_BULLET ) ? B2G_R_BULLET : 0;
	for ( int slot = 0; slot < count; ++slot )
	{
		int sid = W.shapeList[start + slot];
		b2gShapeGeo g = W.geo[sid];
		b2gBox fat = box_of( fats[sid] );
		if ( isFast )
		{
			b2gBox box1 = box_of( aabbs[sid] );
			b2gBox box2 = shape_aabb( g, xf );
			aabbs[sid] = f4_of( box2 );
			int flags = B2G_R_FAST | bullet;
			if ( gbox_contains( fat, box2 ) == false )
			{
				fat.lo.x = box2.lo.x - B2G_AABB_MARGIN;
				fat.lo.y = box2.lo.y - B2G_AABB_MARGIN;
				fat.hi.x = box2.hi.x + B2G_AABB_MARGIN;
				fat.hi.y = box2.hi.y + B2G_AABB_MARGIN;
				fats[sid] = f4_of( fat );
				flags |= B2G_R_FAST_ENLARGED;
			}
			emit_record( W, i, slot, sid, flags, fat, gbox_union( box1, box2 ) );
		}
		else
		{
			b2gBox aabb = shape_aabb( g, xf );
			aabb.lo.x -= B2G_SPECULATIVE;
			aabb.lo.y -= B2G_SPECULATIVE;
			aabb.hi.x += B2G_SPECULATIVE;
			aabb.hi.y += B2G_SPECULATIVE;
			aabbs[sid] = f4_of( aabb );
			if ( gbox_contains( fat, aabb ) == false )
			{
				fat.lo.x = aabb.lo.x - B2G_AABB_MARGIN;
				fat.lo.y = aabb.lo.y - B2G_AABB_MARGIN;
				fat.hi.x = aabb.hi.x + B2G_AABB_MARGIN;
				fat.hi.y = aabb.hi.y + B2G_AABB_MARGIN;
				fats[sid] = f4_of( fat );
				emit_record( W, i, slot, sid, B2G_R_ENLARGED, fat, aabb );
			}
		}
	}
}

/* ------------------------------------------------------------------ launch sequences */
static inline int blocks_for( int n ) { return n > 0 ? ( n + BLOCK - 1 ) / BLOCK : 0; }

static cudaError_t s_lastError = cudaSuccess;

extern "C" const char* b2gd_last_error( void ) { return cudaGetErrorString( s_lastError ); }

static int check( cudaError_t e )
{
	if ( e != cudaSuccess )
	{
		s_lastError = e;
		return (int)e;
	}
	return 0;
}

extern "C" int b2gd_collide( b2gDevWorld* w, b2gHostIO* io, int newCount, int idCount )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	w->launches = 0;
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[1], s );
	cudaMemsetAsync( w->counters, 0, 4 * sizeof( int ), s );
	if ( newCount > 0 )
	{
		cudaMemcpyAsync( w->newContacts, io->newContacts, sizeof( b2gContactInit ) * (size_t)newCount, cudaMemcpyHostToDevice, s );
		k_scatter_contacts<<<blocks_for( newCount ), BLOCK, 0, s>>>( *w, w->newContacts, newCount );
		w->launches += 1;
	}
	if ( idCount > 0 )
	{
		k_collide<<<blocks_for( idCount ), BLOCK, 0, s>>>( *w, idCount );
		w->launches += 1;
	}
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[2], s );
	cudaMemcpyAsync( io->counters, w->counters, 4 * sizeof( int ), cudaMemcpyDeviceToHost, s );
	return check( cudaGetLastError() );
}

/* Prepare .. store impulses on the world's stream (no body finalisation).  Returns the
 * number of kernels launched. */
extern "C" int b2gd_contact_solver( b2gDevWorld* w, const b2gSolvePlan* plan, const b2gStepConst* scp )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	b2gStepConst sc = *scp;
	const int* cs = plan->colorStart;
	const int* js = plan->jointStart;
	int rows = cs[B2G_COLORS];
	int joints = js[B2G_COLORS];
	int awake = plan->awakeCount;
	int ovRow = cs[B2G_OVERFLOW], ovRows = cs[B2G_COLORS] - cs[B2G_OVERFLOW];
	int ovJoint = js[B2G_OVERFLOW], ovJoints = js[B2G_COLORS] - js[B2G_OVERFLOW];
	bool overflow = ovRows + ovJoints > 0;
	int launches = 0;

	if ( rows > 0 )
	{
		k_prepare<<<blocks_for( rows ), BLOCK, 0, s>>>( *w, rows, sc );
		launches += 1;
	}
	if ( joints > 0 )
	{
		k_prepare_joints<<<blocks_for( joints ), BLOCK, 0, s>>>( *w, joints, sc );
		launches += 1;
	}
	for ( int sub = 0; sub < sc.subSteps; ++sub )
	{
		if ( awake > 0 )
		{
			k_integrate_velocities<<<blocks_for( awake ), BLOCK, 0, s>>>( *w, awake, sc );
			launches += 1;
		}
		for ( int phase = PH_WARM; phase <= PH_SOLVE; ++phase )
		{
			if ( overflow )
			{
				k_overflow<<<1, 32, 0, s>>>( *w, phase, ovJoint, ovJoints, ovRow, ovRows, sc );
				launches += 1;
			}
			if ( phase == PH_WARM && sc.enableWarmStarting == 0 )
				continue;
			for ( int a = 0; a < plan->activeCount; ++a )
			{
				int c = plan->active[a];
				int nj = js[c + 1] - js[c], nr = cs[c + 1] - cs[c];
				k_color<<<blocks_for( nj + nr ), BLOCK, 0, s>>>( *w, phase, js[c], nj, cs[c], nr, sc );
				launches += 1;
			}
		}
		if ( awake > 0 )
		{
			k_integrate_positions<<<blocks_for( awake ), BLOCK, 0, s>>>( *w, awake, sc );
			launches += 1;
		}
		if ( overflow )
		{
			k_overflow<<<1, 32, 0, s>>>( *w, PH_RELAX, ovJoint, ovJoints, ovRow, ovRows, sc );
			launches += 1;
		}
		for ( int a = 0; a < plan->activeCount; ++a )
		{
			int c = plan->active[a];
			int nj = js[c + 1] - js[c], nr = cs[c + 1] - cs[c];
			k_color<<<blocks_for( nj + nr ), BLOCK, 0, s>>>( *w, PH_RELAX, js[c], nj, cs[c], nr, sc );
			launches += 1;
		}
	}
	if ( ovRows > 0 )
	{
		k_overflow<<<1, 32, 0, s>>>( *w, PH_RESTITUTION, ovJoint, 0, ovRow, ovRows, sc );
		launches += 1;
	}
	for ( int a = 0; a < plan->activeCount; ++a )
	{
		int c = plan->active[a];
		int nr = cs[c + 1] - cs[c];
		if ( nr > 0 )
		{
			k_color<<<blocks_for( nr ), BLOCK, 0, s>>>( *w, PH_RESTITUTION, 0, 0, cs[c], nr, sc );
			launches += 1;
		}
	}
	if ( rows > 0 )
	{
		k_store<<<blocks_for( rows ), BLOCK, 0, s>>>( *w, rows, ovRow );
		launches += 1;
	}
	return launches;
}

extern "C" int b2gd_solve( b2gDevWorld* w, b2gHostIO* io, const b2gSolvePlan* plan, const b2gStepConst* scp )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int awake = plan->awakeCount;
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[3], s );
	cudaMemsetAsync( w->counters + 1, 0, sizeof( int ), s );
	w->launches += b2gd_contact_solver( w, plan, scp );
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[4], s );
	if ( awake > 0 )
	{
		k_finalize<<<blocks_for( awake ), BLOCK, 0, s>>>( *w, awake, *scp );
		w->launches += 1;
	}
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[5], s );
	cudaMemcpyAsync( io->counters, w->counters, 4 * sizeof( int ), cudaMemcpyDeviceToHost, s );
	return check( cudaGetLastError() );
}

/* ------------------------------------------------------------------ diagnostics */
/* Replays the narrowphase of one contact and writes its inputs and manifold to out:
 * [0..3] shape ids / flags, [4..11] xfA xfB, [12..39] manifold (28 words). */
__global__ void k_debug_collide( b2gDevWorld W, int id, float* out )
{
	if ( threadIdx.x != 0 || blockIdx.x != 0 )
		return;
	int sA = W.cShapes[2 * id];
	int sB = W.cShapes[2 * id + 1];
	const b2gShapeGeo* gA = W.geo + sA;
	const b2gShapeGeo* gB = W.geo + sB;
	const float4* xf = (const float4*)W.xf;
	float4 xa = xf[gA->bodyId], xb = xf[gB->bodyId];
	if ( out[40] != 0.0f )
	{
		/* caller-supplied transforms in out[41..48] */
		xa = make_float4( out[41], out[42], out[43], out[44] );
		xb = make_float4( out[45], out[46], out[47], out[48] );
	}
	b2gXf xfA, xfB;
	xfA.p = gv( xa.x, xa.y );
	xfA.q = grot( xa.z, xa.w );
	xfB.p = gv( xb.x, xb.y );
	xfB.q = grot( xb.z, xb.w );
	b2gManifold m;
	narrowphase( &m, gA, xfA, gB, xfB );
	int* oi = (int*)out;
	oi[0] = sA;
	oi[1] = sB;
	oi[2] = (int)W.cFlags[id];
	oi[3] = gA->isSensor | ( gB->isSensor << 1 );
	out[4] = xa.x;
	out[5] = xa.y;
	out[6] = xa.z;
	out[7] = xa.w;
	out[8] = xb.x;
	out[9] = xb.y;
	out[10] = xb.z;
	out[11] = xb.w;
	const float* mf = (const float*)&m;
	for ( int i = 0; i < (int)( sizeof( b2gManifold ) / 4 ); ++i )
		out[12 + i] = mf[i];
}

extern "C" int b2gd_debug_collide( b2gDevWorld* w, int id, float* hostOut )
{
	float* d = nullptr;
	cudaMalloc( &d, 64 * sizeof( float ) );
	cudaMemcpy( d, hostOut, 64 * sizeof( float ), cudaMemcpyHostToDevice );
	k_debug_collide<<<1, 1, 0, (cudaStream_t)w->stream>>>( *w, id, d );
	cudaError_t e = cudaGetLastError();
	cudaMemcpyAsync( hostOut, d, 64 * sizeof( float ), cudaMemcpyDeviceToHost, (cudaStream_t)w->stream );
	cudaStreamSynchronize( (cudaStream_t)w->stream );
	cudaFree( d );
	return (int)e;
}
