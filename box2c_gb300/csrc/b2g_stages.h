/*
 * b2g_stages.h -- the per-item work of each device stage, as device functions over one
 * world descriptor: contact creation, narrowphase, row and joint preparation, body
 * integration, impulse storage and body finalisation.
 *
 * kernels.cu wraps them in one-launch-per-stage kernels for a single world; batch.cu
 * calls the same functions from the batched kernels that step many worlds per launch,
 * so both give the same bits.
 *
 * Stage                reference
 * contact creation     src/contact.c:185-332 (sim part)
 * narrowphase          src/world.c:290-365, src/contact.c:493-582
 * prepare contacts     src/contact_solver.c:21-147, :597-808
 * prepare joints       src/joint.c:983-1018 (per type: b2g_joints.h)
 * integrate velocities src/solver.c:34-93
 * integrate positions  src/solver.c:146-163
 * store impulses       src/contact_solver.c:442-471, :1180-1293
 * finalize bodies      src/solver.c:165-351 (+ fast-body sweep boxes, :787-1105)
 */
#pragma once

#include "b2g_collide.h"
#include "b2g_device.h"
#include "b2g_solve.h"
#include "b2g_toi.h"

#include <cuda_runtime.h>

/* ------------------------------------------------------------------ state access */
static __device__ __forceinline__ DevState load_state( const b2gDevWorld& W, int b )
{
	if ( b < 0 )
		return identity_state();
	const float4* st = (const float4*)W.state;
	return state_of( st[2 * b], st[2 * b + 1] );
}

static __device__ __forceinline__ void store_velocity( const b2gDevWorld& W, int b, const DevState& s )
{
	if ( b < 0 )
		return;
	( (float4*)W.state )[2 * b] = velocity_word( s );
}

static __device__ __forceinline__ b2gBox box_of( float4 f )
{
	b2gBox b;
	b.lo = gv( f.x, f.y );
	b.hi = gv( f.z, f.w );
	return b;
}

static __device__ __forceinline__ float4 f4_of( b2gBox b ) { return make_float4( b.lo.x, b.lo.y, b.hi.x, b.hi.y ); }

/* Shape AABB (reference src/geometry.c:385-430, src/shape.c:457-478). */
static __device__ b2gBox shape_aabb( const b2gShapeGeo& g, b2gXf xf )
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

/* ------------------------------------------------------------------ sleep and wake */
/* A staged body operation (reference src/solver_set.c:50-58, :190-214): a woken body
 * starts from the identity state (zero velocity, no pending motion) with a zero sleep
 * timer; a sleeping body stops being integrated.  The sleep threshold in the velocity's
 * spare lane stays. */
static __device__ __forceinline__ void apply_body_op( const b2gDevWorld& W, int op )
{
	int b = op >> 2;
	if ( ( op & 3 ) == B2G_BODY_WAKE )
	{
		float4* st = (float4*)W.state;
		float threshold = st[2 * b].w;
		st[2 * b] = make_float4( 0.0f, 0.0f, 0.0f, threshold );
		st[2 * b + 1] = make_float4( 0.0f, 0.0f, 1.0f, 0.0f );
		if ( W.sleepTime != nullptr )
			W.sleepTime[b] = 0.0f;
		W.bodyInfo[b] |= B2G_B_AWAKE;
	}
	else
	{
		W.bodyInfo[b] &= ~B2G_B_AWAKE;
	}
}

/* ------------------------------------------------------------------ contact creation */
static __device__ __forceinline__ void scatter_contact( const b2gDevWorld& W, const b2gContactInit* inits, int t )
{
	b2gContactInit c = inits[t];
	int id = c.id;
	if ( c.flags & B2G_INIT_KILL )
	{
		W.cFlags[id] = 0;
		return;
	}
	uint32_t asleep = ( c.flags & B2G_INIT_ASLEEP ) ? B2G_C_ASLEEP : 0u;
	if ( c.flags & B2G_INIT_SET )
	{
		/* the contact moved into or out of the awake set: only its set bit changes */
		W.cFlags[id] = ( W.cFlags[id] & ~(uint32_t)B2G_C_ASLEEP ) | asleep;
		return;
	}
	W.cShapes[2 * id] = c.shapeA;
	W.cShapes[2 * id + 1] = c.shapeB;
	W.cMix[2 * id] = c.friction;
	W.cMix[2 * id + 1] = c.restitution;
	W.cFlags[id] = B2G_C_LIVE | asleep;
	W.cCache[id] = 0u;
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
static __device__ __noinline__ void narrowphase_polygons( b2gManifold* m, const b2gShapeGeo* gA, b2gXf xfA, const b2gShapeGeo* gB,
														  b2gXf xfB )
{
	gcollide_polygons_raw( m, gA->v, gA->n, gA->count, gA->radius, xfA, gB->v, gB->n, gB->count, gB->radius, xfB );
}

/* Other pairs; a smooth segment (chain link) reads and updates the contact's
 * closest-feature cache (reference src/contact.c:138-148, the cache argument). */
static __device__ __noinline__ void narrowphase_shapes( b2gManifold* m, const b2gShapeGeo* gA, b2gXf xfA, const b2gShapeGeo* gB,
														b2gXf xfB, uint32_t* packedCache )
{
	b2gDistCache cache = gcache_unpack( gA->type == 4 ? *packedCache : 0u );
	gcollide_shapes( m, gA, xfA, gB, xfB, &cache );
	if ( gA->type == 4 )
		*packedCache = gcache_pack( &cache );
}

/* Polygon pairs (the common case) take their own call, whose frame holds only the two
 * polygons in the contact frame; the other pairs' polygon copies stay out of it. */
static __device__ __noinline__ void narrowphase( b2gManifold* m, const b2gShapeGeo* gA, b2gXf xfA, const b2gShapeGeo* gB, b2gXf xfB,
												 uint32_t* packedCache )
{
	if ( gA->isSensor || gB->isSensor )
		gmanifold_clear( m );
	else if ( gA->type == 3 && gB->type == 3 )
		narrowphase_polygons( m, gA, xfA, gB, xfB );
	else
		narrowphase_shapes( m, gA, xfA, gB, xfB, packedCache );
}

/* Sensor contacts: whether the shapes overlap, by their GJK distance with radii,
 * warm-started from the contact's closest-feature cache and updating it (reference
 * src/contact.c:476-503).  The cache packs its count in bits 0-1 and the six vertex
 * indices in 3 bits each from bit 2. */
static __device__ __noinline__ bool sensor_overlap( const b2gDevWorld& W, int id, const b2gShapeGeo* gA, b2gXf xfA,
													const b2gShapeGeo* gB, b2gXf xfB )
{
	b2gDistCache cache = gcache_unpack( W.cCache[id] );
	b2gProxy pa = gproxy_shape( gA );
	b2gProxy pb = gproxy_shape( gB );
	float d = gdistance( &cache, &pa, xfA, &pb, xfB );
	W.cCache[id] = gcache_pack( &cache );
	if ( d < FLT_EPSILON )
		d = 0.0f;
	else
		d = gmax( 0.0f, d - pa.radius - pb.radius );
	return d < 10.0f * FLT_EPSILON;
}

static __device__ __forceinline__ void emit_event( const b2gDevWorld& W, int id, int code )
{
	int slot = atomicAdd( W.counters + 0, 1 );
	if ( slot < W.eventCap )
		W.events[slot] = ( id << 2 ) | code;
}

static __device__ void collide_contact( const b2gDevWorld& W, int id )
{
	uint32_t flags = W.cFlags[id];
	/* only the awake set's contacts are updated (reference src/world.c:436-466) */
	if ( ( flags & B2G_C_LIVE ) == 0 || ( flags & B2G_C_ASLEEP ) != 0 )
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
	/* solver rows address a body by id unless it is static: a contact joins the graph
	 * only with awake or static bodies, including a body woken by the contact itself
	 * after this narrowphase (reference src/constraint_graph.c:141-170) */
	int infoA = W.bodyInfo[bA];
	int infoB = W.bodyInfo[bB];
	W.cBodies[2 * id] = ( infoA & B2G_B_TYPE_MASK ) != 0 ? bA : -1;
	W.cBodies[2 * id + 1] = ( infoB & B2G_B_TYPE_MASK ) != 0 ? bB : -1;
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

	if ( gA->isSensor || gB->isSensor )
	{
		/* sensors generate no manifold and no hit events */
		bool overlap = sensor_overlap( W, id, gA, xfA, gB, xfB );
		W.cFlags[id] = B2G_C_LIVE | ( overlap ? B2G_C_TOUCHING : 0u );
		if ( overlap && !wasTouching )
			emit_event( W, id, B2G_EV_STARTED );
		else if ( !overlap && wasTouching )
			emit_event( W, id, B2G_EV_STOPPED );
		return;
	}

	/* the previous manifold's feature ids and impulses, for warm starting */
	const b2gManifold* prev = W.manifold + id;
	const int oldCount = prev->count;
	const uint16_t oldId0 = prev->pts[0].id, oldId1 = prev->pts[1].id;
	const float oldN0 = prev->pts[0].normalImpulse, oldT0 = prev->pts[0].tangentImpulse;
	const float oldN1 = prev->pts[1].normalImpulse, oldT1 = prev->pts[1].tangentImpulse;
	b2gManifold m;
	narrowphase( &m, gA, xfA, gB, xfB, W.cCache + id );

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
		/* first old point with the same id (reference src/contact.c:539-570) */
		if ( oldCount > 0 && oldId0 == mp2->id )
		{
			mp2->normalImpulse = oldN0;
			mp2->tangentImpulse = oldT0;
			mp2->persisted = 1;
		}
		else if ( oldCount > 1 && oldId1 == mp2->id )
		{
			mp2->normalImpulse = oldN1;
			mp2->tangentImpulse = oldT1;
			mp2->persisted = 1;
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
static __device__ void prepare_contact_row( const b2gDevWorld& W, int k, const b2gStepConst& sc )
{
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
	( (float4*)W.kMass )[k] = make_float4( r.mA, r.iA, r.mB, r.iB );
	for ( int j = 0; j < 2; ++j )
	{
		( (float4*)W.kAnchor[j] )[k] = make_float4( r.rA[j].x, r.rA[j].y, r.rB[j].x, r.rB[j].y );
		( (float4*)W.kCoef[j] )[k] = make_float4( r.base[j], r.nMass[j], r.tMass[j], r.relVel[j] );
		( (float4*)W.kImp[j] )[k] = make_float4( r.ni[j], r.ti[j], r.maxNi[j], 0.0f );
	}
}

/* Row k for one phase (0 warm start, 1 solve, 2 relax, 3 restitution): the softness
 * comes from the step constants (a static body's rows use the static softness, as
 * prepare chose it), and warm starting, which reads no coefficients, skips them. */
static __device__ __forceinline__ void load_row( const b2gDevWorld& W, int k, int phase, const b2gStepConst& sc, Row& r )
{
	int4 idx = ( (const int4*)W.kIdx )[k];
	float4 nf = ( (const float4*)W.kNF )[k];
	float4 ms = ( (const float4*)W.kMass )[k];
	r.ia = idx.x;
	r.ib = idx.y;
	r.count = idx.w;
	r.n = gv( nf.x, nf.y );
	r.friction = nf.z;
	r.restitution = nf.w;
	const float* soft = ( idx.x < 0 || idx.y < 0 ) ? sc.staticSoft : sc.contactSoft;
	r.biasRate = soft[0];
	r.massScale = soft[1];
	r.impulseScale = soft[2];
	r.mA = ms.x;
	r.iA = ms.y;
	r.mB = ms.z;
	r.iB = ms.w;
	for ( int j = 0; j < 2; ++j )
	{
		float4 a = ( (const float4*)W.kAnchor[j] )[k];
		float4 c = phase == 0 ? make_float4( 0.0f, 0.0f, 0.0f, 0.0f ) : ( (const float4*)W.kCoef[j] )[k];
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

static __device__ __forceinline__ void store_impulses( const b2gDevWorld& W, int k, const Row& r )
{
	for ( int j = 0; j < 2; ++j )
		( (float4*)W.kImp[j] )[k] = make_float4( r.ni[j], r.ti[j], r.maxNi[j], 0.0f );
}

/* Row phases over global body state: load, solve in registers, store. */
/* Body-state views for the row and joint work below. */
struct GlobalBodies
{
	const b2gDevWorld* W;
	__device__ __forceinline__ DevState load( int b ) const { return load_state( *W, b ); }
	__device__ __forceinline__ DevState load_velocity( int b ) const { return load_state( *W, b ); }
	__device__ __forceinline__ void store( int b, const DevState& x ) const { store_velocity( *W, b, x ); }
};

/* One row phase (0 warm start, 1 solve, 2 relax, 3 restitution): row from the world's
 * row arrays, bodies through B. */
template <class Bodies>
static __device__ __forceinline__ void row_work( const b2gDevWorld& W, const Bodies& B, int k, int phase, bool scalar,
												 const b2gStepConst& sc )
{
	Row r;
	load_row( W, k, phase, sc, r );
	bool delta = phase == 1 || phase == 2;
	DevState a = delta ? B.load( r.ia ) : B.load_velocity( r.ia );
	DevState b = delta ? B.load( r.ib ) : B.load_velocity( r.ib );
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
	B.store( r.ia, a );
	B.store( r.ib, b );
	if ( phase != 0 )
		store_impulses( W, k, r );
}

static __device__ void row_phase( const b2gDevWorld& W, int k, int phase, bool scalar, const b2gStepConst& sc )
{
	row_work( W, GlobalBodies{ &W }, k, phase, scalar, sc );
}

/* ------------------------------------------------------------------ joints */
/* Joint preparation (reference src/joint.c:983-1018 and the per-type prepare functions):
 * gathers the two bodies' mass and pose, then the type's own preparation. */
static __device__ void prepare_joint( const b2gDevWorld& W, int t, const b2gStepConst& sc )
{
	b2gJointDev* j = W.joints + W.jointList[t];
	const float4* mass = (const float4*)W.mass;
	const float4* xf = (const float4*)W.xf;
	const float4* centers = (const float4*)W.centers;
	int a = j->bodyIdA, b = j->bodyIdB;
	float4 ma = mass[a], mb = mass[b];
	float4 xa = xf[a], xb = xf[b];
	float4 ca = centers[a], cb = centers[b];
	/* a joint in the graph has awake or static bodies */
	j->indexA = ( W.bodyInfo[a] & B2G_B_TYPE_MASK ) != 0 ? a : -1;
	j->indexB = ( W.bodyInfo[b] & B2G_B_TYPE_MASK ) != 0 ? b : -1;
	JointBodies jb;
	jb.mA = ma.y;
	jb.iA = ma.w;
	jb.mB = mb.y;
	jb.iB = mb.w;
	jb.qA = grot( xa.z, xa.w );
	jb.qB = grot( xb.z, xb.w );
	jb.cA = gv( ca.x, ca.y );
	jb.cB = gv( cb.x, cb.y );
	jb.lcA = gv( ca.z, ca.w );
	jb.lcB = gv( cb.z, cb.w );
	joint_prepare( j, jb, sc );
}

template <class Bodies>
static __device__ __forceinline__ void joint_work( const b2gDevWorld& W, const Bodies& B, int jid, int phase, const b2gStepConst& sc )
{
	b2gJointDev* j = W.joints + jid;
	DevState a = B.load( j->indexA );
	DevState b = B.load( j->indexB );
	if ( phase == 0 )
		joint_warm_state( j, a, b );
	else
		joint_solve_state( j, a, b, phase == 1, sc );
	B.store( j->indexA, a );
	B.store( j->indexB, b );
}

static __device__ void joint_phase( const b2gDevWorld& W, int jid, int phase, const b2gStepConst& sc )
{
	joint_work( W, GlobalBodies{ &W }, jid, phase, sc );
}

/* ------------------------------------------------------------------ bodies */
static __device__ __forceinline__ void integrate_body_velocity( const b2gDevWorld& W, int i, const b2gStepConst& sc )
{
	int b = W.awake[i];
	DevState s = load_state( W, b );
	VelocityTerms t = velocity_terms( ( (const float4*)W.mass )[b], ( (const float4*)W.force )[b], ( (const float4*)W.extent )[b], sc );
	integrate_velocity( s, t, sc );
	store_velocity( W, b, s );
}

static __device__ __forceinline__ void integrate_body_position( const b2gDevWorld& W, int i, const b2gStepConst& sc )
{
	int b = W.awake[i];
	DevState s = load_state( W, b );
	integrate_position( s, sc.h );
	( (float4*)W.state )[2 * b + 1] = make_float4( s.dp.x, s.dp.y, s.dq.c, s.dq.s );
}

static __device__ __forceinline__ void store_row( const b2gDevWorld& W, int k, int overflowStart )
{
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

/* Appends a finalisation record; the sweep poses are written for fast shapes only. */
static __device__ __forceinline__ void emit_record( const b2gDevWorld& W, int awakeIndex, int slot, int shapeId, int flags, b2gBox fat,
											 b2gBox sweep, const float4* pose1 = nullptr, const float4* pose2 = nullptr )
{
	int r = atomicAdd( W.counters + 1, 1 );
	if ( r >= W.recordCap )
		return;
	float4* o = (float4*)( W.records + r );
	o[0] = make_float4( __int_as_float( awakeIndex ), __int_as_float( slot ), __int_as_float( shapeId ), __int_as_float( flags ) );
	o[1] = make_float4( fat.lo.x, fat.lo.y, fat.hi.x, fat.hi.y );
	o[2] = make_float4( sweep.lo.x, sweep.lo.y, sweep.hi.x, sweep.hi.y );
	if ( pose1 != nullptr )
	{
		o[3] = *pose1;
		o[4] = *pose2;
	}
}

static __device__ void finalize_body( const b2gDevWorld& W, int i, const b2gStepConst& sc )
{
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
	float sleepTime = 0.0f;
	if ( sc.enableSleep == 0 || ( info & B2G_B_SLEEP_OK ) == 0 || sleepVelocity > sleepThreshold )
	{
		if ( ( info & B2G_B_TYPE_MASK ) == 2 && sc.enableContinuous && maxVelocity * sc.dt > 0.5f * minExtent )
			isFast = true;
	}
	else if ( W.sleepTime != nullptr )
	{
		sleepTime = W.sleepTime[b] + sc.dt;
	}
	/* a world that never stepped with sleep on keeps no timers; elsewhere a body past the
	 * sleep time no longer keeps its island awake: the host learns of it and decides the
	 * island's sleep (reference src/solver.c:281-298) */
	if ( W.sleepTime != nullptr )
		W.sleepTime[b] = sleepTime;
	if ( sleepTime >= B2G_TIME_TO_SLEEP )
	{
		int slot = atomicAdd( W.counters + 3, 1 );
		if ( slot < W.sleepyCap )
		{
			W.sleepy[2 * slot] = i;
			W.sleepy[2 * slot + 1] = __float_as_int( sleepTime );
		}
	}
	/* with no time-of-impact event the fast body also advances its sweep start; the host
	 * moves it back along the sweep when continuous collision finds an impact */
	float4 pose1 = prev[b];
	float4 pose2 = make_float4( center.x, center.y, q.c, q.s );
	prev[b] = pose2;

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
			emit_record( W, i, slot, sid, flags, fat, gbox_union( box1, box2 ), &pose1, &pose2 );
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

/* Adjoint tape record of one step (item t of max(bodies, rows)): body state, transform,
 * centre, awake flag and applied force per body id; the solver rows with their input
 * manifolds. */
static __device__ __forceinline__ void tape_record_one( const b2gDevWorld& W, float4* bodies, int bodyCount, b2gTapeRow* rows, int rowCount,
														int t )
{
	if ( t < bodyCount )
	{
		const float4* st = (const float4*)W.state;
		float4 f = ( (const float4*)W.force )[t];
		float awake = ( W.bodyInfo[t] & B2G_B_AWAKE ) ? 1.0f : 0.0f;
		float4* o = bodies + B2G_TAPE_BODY_FLOAT4 * t;
		o[0] = st[2 * t];
		o[1] = ( (const float4*)W.xf )[t];
		o[2] = ( (const float4*)W.centers )[t];
		o[3] = make_float4( awake, f.x, f.y, f.z );
	}
	if ( t < rowCount )
	{
		int cid = W.solveList[t];
		b2gTapeRow r;
		r.cid = cid;
		r.ia = W.cBodies[2 * cid];
		r.ib = W.cBodies[2 * cid + 1];
		r.shapeA = W.cShapes[2 * cid];
		r.shapeB = W.cShapes[2 * cid + 1];
		r.pad = 0;
		r.friction = W.cMix[2 * cid];
		r.restitution = W.cMix[2 * cid + 1];
		r.m = W.manifold[cid];
		r.pad2[0] = 0.0f;
		rows[t] = r;
	}
}
