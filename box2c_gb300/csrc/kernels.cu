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
#include "b2g_solve.h"

#include <cuda_runtime.h>

#include <stdio.h>

#define BLOCK 256

/* ------------------------------------------------------------------ state access */
__device__ __forceinline__ DevState load_state( const b2gDevWorld& W, int b )
{
	if ( b < 0 )
		return identity_state();
	const float4* st = (const float4*)W.state;
	return state_of( st[2 * b], st[2 * b + 1] );
}

__device__ __forceinline__ void store_velocity( const b2gDevWorld& W, int b, const DevState& s )
{
	if ( b < 0 )
		return;
	( (float4*)W.state )[2 * b] = velocity_word( s );
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
	int ia = W.cBodies[2 * cid];
	int ib = W.cBodies[2 * cid + 1];
	/* inverse masses of the reference's contact sim: the body's, zero for static bodies */
	const float4* mass = (const float4*)W.mass;
	float4 zero = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	Row r;
	prepare_row( r, W.manifold + cid, ia, ib, ia >= 0 ? mass[ia] : zero, ib >= 0 ? mass[ib] : zero, load_state( W, ia ),
				 load_state( W, ib ), W.cMix[2 * cid], W.cMix[2 * cid + 1], ( ia < 0 || ib < 0 ) ? sc.staticSoft : sc.contactSoft,
				 sc.enableWarmStarting ? 1.0f : 0.0f );
	( (int4*)W.kIdx )[k] = make_int4( ia, ib, cid, r.count );
	( (float4*)W.kNF )[k] = make_float4( r.n.x, r.n.y, r.friction, r.restitution );
	( (float4*)W.kSoft )[k] = make_float4( r.biasRate, r.massScale, r.impulseScale, 0.0f );
	( (float4*)W.kMass )[k] = make_float4( r.mA, r.iA, r.mB, r.iB );
	for ( int j = 0; j < 2; ++j )
	{
		( (float4*)W.kAnchor[j] )[k] = make_float4( r.rA[j].x, r.rA[j].y, r.rB[j].x, r.rB[j].y );
		( (float4*)W.kCoef[j] )[k] = make_float4( r.base[j], r.nMass[j], r.tMass[j], r.relVel[j] );
		( (float4*)W.kImp[j] )[k] = make_float4( r.ni[j], r.ti[j], r.maxNi[j], 0.0f );
	}
}

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

/* Row phases over global body state: load, solve in registers, store. */
__device__ void row_phase( const b2gDevWorld& W, int k, int phase, bool scalar, const b2gStepConst& sc )
{
	Row r;
	load_row( W, k, r );
	DevState a = load_state( W, r.ia );
	DevState b = load_state( W, r.ib );
	bool changed = true;
	if ( phase == 0 )
		scalar ? warm_scalar( r, a, b ) : warm_lane( r, a, b );
	else if ( phase == 1 || phase == 2 )
		scalar ? solve_scalar( r, a, b, phase == 1, sc.inv_h, sc.pushout ) : solve_lane( r, a, b, phase == 1, sc.inv_h, sc.pushout );
	else if ( scalar )
		changed = restitution_scalar( r, a, b, sc.restitutionThreshold );
	else
		restitution_lane( r, a, b, sc.restitutionThreshold );
	if ( changed == false )
		return;
	store_velocity( W, r.ia, a );
	store_velocity( W, r.ib, b );
	if ( phase != 0 )
		store_impulses( W, k, r );
}

/* ------------------------------------------------------------------ revolute joint */
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

__device__ void joint_phase( const b2gDevWorld& W, int jid, int phase, const b2gStepConst& sc )
{
	b2gJointDev* j = W.joints + jid;
	DevState a = load_state( W, j->indexA );
	DevState b = load_state( W, j->indexB );
	if ( phase == 0 )
		joint_warm_state( j, a, b );
	else
		joint_solve_state( j, a, b, phase == 1, sc );
	store_velocity( W, j->indexA, a );
	store_velocity( W, j->indexB, b );
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
		joint_phase( W, W.jointList[jointStart + t], phase, sc );
		return;
	}
	t -= jointCount;
	if ( t >= rowCount )
		return;
	row_phase( W, rowStart + t, phase, false, sc );
}

/* Overflow constraints share bodies, so they run serially in list order (joints first). */
__global__ void k_overflow( b2gDevWorld W, int phase, int jointStart, int jointCount, int rowStart, int rowCount, b2gStepConst sc )
{
	if ( threadIdx.x != 0 || blockIdx.x != 0 )
		return;
	if ( phase != PH_RESTITUTION )
	{
		for ( int i = 0; i < jointCount; ++i )
			joint_phase( W, W.jointList[jointStart + i], phase, sc );
	}
	for ( int i = 0; i < rowCount; ++i )
		row_phase( W, rowStart + i, phase, true, sc );
}

/* ------------------------------------------------------------------ bodies */
__global__ void __launch_bounds__( BLOCK ) k_integrate_velocities( b2gDevWorld W, int awakeCount, b2gStepConst sc )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= awakeCount )
		return;
	int b = W.awake[i];
	DevState s = load_state( W, b );
	VelocityTerms t = velocity_terms( ( (const float4*)W.mass )[b], ( (const float4*)W.force )[b], ( (const float4*)W.extent )[b], sc );
	integrate_velocity( s, t, sc );
	store_velocity( W, b, s );
}

__global__ void __launch_bounds__( BLOCK ) k_integrate_positions( b2gDevWorld W, int awakeCount, b2gStepConst sc )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= awakeCount )
		return;
	int b = W.awake[i];
	DevState s = load_state( W, b );
	integrate_position( s, sc.h );
	( (float4*)W.state )[2 * b + 1] = make_float4( s.dp.x, s.dp.y, s.dq.c, s.dq.s );
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

/* Prepares the step's joints (all colours); used by the fused solver, which runs
 * everything else of the solver stage. */
extern "C" int b2gd_prepare_joints( b2gDevWorld* w, int joints, const b2gStepConst* sc )
{
	if ( joints <= 0 )
		return 0;
	k_prepare_joints<<<blocks_for( joints ), BLOCK, 0, (cudaStream_t)w->stream>>>( *w, joints, *sc );
	return 1;
}

extern "C" int b2gd_solver_fused( b2gDevWorld* w, const b2gSolvePlan* plan, const b2gStepConst* sc );

extern "C" int b2gd_solve( b2gDevWorld* w, b2gHostIO* io, const b2gSolvePlan* plan, const b2gStepConst* scp )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int awake = plan->awakeCount;
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[3], s );
	cudaMemsetAsync( w->counters + 1, 0, sizeof( int ), s );
	int fused = w->fused ? b2gd_solver_fused( w, plan, scp ) : 0;
	if ( fused < 0 )
		return check( cudaGetLastError() );
	w->fusedUsed = fused > 0;
	w->launches += fused > 0 ? fused : b2gd_contact_solver( w, plan, scp );
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
