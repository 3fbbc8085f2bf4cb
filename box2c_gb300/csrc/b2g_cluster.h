/*
 * b2g_cluster.h -- solver rows in shared memory and body states spread over the CTAs of
 * a thread-block cluster; shared by the fused single-world solver (fused.cu) and the
 * batched solver (batch.cu, rows of a world that fits in one CTA's shared memory).
 *
 * Rows use nine float4 arrays (structure of arrays): indices, normal / friction /
 * restitution, inverse masses, two anchor pairs, two coefficient sets, two impulse
 * sets; the softness follows from whether a body is static.  Body b lives in CTA
 * b / slots at slot b % slots; a body of the calling CTA is read and written in local
 * shared memory, any other through distributed shared memory.
 */
#pragma once

#include "b2g_solve.h"

#include <cooperative_groups.h>

namespace cg = cooperative_groups;

enum
{
	F_WARM = 0,
	F_SOLVE = 1,
	F_RELAX = 2,
	F_RESTITUTION = 3,
};

struct SmemRows
{
	int4* idx;	   /* ia ib contactId count */
	float4* nf;	   /* n.x n.y friction restitution */
	float4* ms;	   /* mA iA mB iB */
	float4* anc0;  /* rA.x rA.y rB.x rB.y of point 0 */
	float4* anc1;  /* point 1 */
	float4* coef0; /* base normalMass tangentMass relativeVelocity */
	float4* coef1;
	float4* imp0; /* normalImpulse tangentImpulse maxNormalImpulse 0 */
	float4* imp1;
};

/* Body states of the cluster: body b lives in CTA b / slots at slot b % slots.  A body
 * of this CTA is read and written in local shared memory, any other through
 * distributed shared memory. */
struct ClusterBodies
{
	cg::cluster_group cl;
	float4* st0;
	float4* st1;
	int slots;
	int rank;
	unsigned slotsInv; /* ceil(2^32 / slots) for slots > 1: b / slots = umulhi(b, slotsInv) for b, slots < 2^16 */

	__device__ __forceinline__ float4* word( float4* base, int b ) const
	{
		int r = slots == 1 ? b : (int)__umulhi( (unsigned)b, slotsInv );
		int s = b - r * slots;
		return r == rank ? base + s : cl.map_shared_rank( base + s, (unsigned)r );
	}

	/* full state (solve, relax, joints) */
	__device__ __forceinline__ DevState load( int b ) const
	{
		if ( b < 0 )
			return identity_state();
		return state_of( *word( st0, b ), *word( st1, b ) );
	}

	/* velocity only (warm start, restitution): dp and dq are not read */
	__device__ __forceinline__ DevState load_velocity( int b ) const
	{
		if ( b < 0 )
			return identity_state();
		return state_of( *word( st0, b ), make_float4( 0.0f, 0.0f, 1.0f, 0.0f ) );
	}

	__device__ __forceinline__ void store( int b, const DevState& x ) const
	{
		if ( b < 0 )
			return;
		*word( st0, b ) = velocity_word( x );
	}
};

__device__ __forceinline__ void load_row_smem( const SmemRows& m, int k, const b2gStepConst& sc, Row& r )
{
	int4 idx = m.idx[k];
	float4 nf = m.nf[k];
	float4 ms = m.ms[k];
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
	float4 a0 = m.anc0[k], a1 = m.anc1[k], c0 = m.coef0[k], c1 = m.coef1[k], i0 = m.imp0[k], i1 = m.imp1[k];
	r.rA[0] = gv( a0.x, a0.y );
	r.rB[0] = gv( a0.z, a0.w );
	r.rA[1] = gv( a1.x, a1.y );
	r.rB[1] = gv( a1.z, a1.w );
	r.base[0] = c0.x;
	r.nMass[0] = c0.y;
	r.tMass[0] = c0.z;
	r.relVel[0] = c0.w;
	r.base[1] = c1.x;
	r.nMass[1] = c1.y;
	r.tMass[1] = c1.z;
	r.relVel[1] = c1.w;
	r.ni[0] = i0.x;
	r.ti[0] = i0.y;
	r.maxNi[0] = i0.z;
	r.ni[1] = i1.x;
	r.ti[1] = i1.y;
	r.maxNi[1] = i1.z;
}

__device__ __forceinline__ void store_row_smem( const SmemRows& m, int k, int cid, const Row& r )
{
	m.idx[k] = make_int4( r.ia, r.ib, cid, r.count );
	m.nf[k] = make_float4( r.n.x, r.n.y, r.friction, r.restitution );
	m.ms[k] = make_float4( r.mA, r.iA, r.mB, r.iB );
	m.anc0[k] = make_float4( r.rA[0].x, r.rA[0].y, r.rB[0].x, r.rB[0].y );
	m.anc1[k] = make_float4( r.rA[1].x, r.rA[1].y, r.rB[1].x, r.rB[1].y );
	m.coef0[k] = make_float4( r.base[0], r.nMass[0], r.tMass[0], r.relVel[0] );
	m.coef1[k] = make_float4( r.base[1], r.nMass[1], r.tMass[1], r.relVel[1] );
	m.imp0[k] = make_float4( r.ni[0], r.ti[0], r.maxNi[0], 0.0f );
	m.imp1[k] = make_float4( r.ni[1], r.ti[1], r.maxNi[1], 0.0f );
}

/* One row phase on a row in shared memory; Bodies is ClusterBodies (states spread over
 * the cluster) or SharedBodies (states of one CTA, by body id). */
template <class Bodies>
__device__ __forceinline__ void row_step( const SmemRows& m, const Bodies& B, int k, int phase, bool scalar, const b2gStepConst& sc )
{
	Row r;
	load_row_smem( m, k, sc, r );
	bool delta = phase == F_SOLVE || phase == F_RELAX;
	DevState a = delta ? B.load( r.ia ) : B.load_velocity( r.ia );
	DevState b = delta ? B.load( r.ib ) : B.load_velocity( r.ib );
	bool changed = true;
	if ( phase == F_WARM )
		scalar ? warm_scalar( r, a, b ) : warm_lane( r, a, b );
	else if ( phase == F_SOLVE || phase == F_RELAX )
		scalar ? solve_scalar( r, a, b, phase == F_SOLVE, sc.inv_h, sc.pushout )
			   : solve_lane( r, a, b, phase == F_SOLVE, sc.inv_h, sc.pushout );
	else if ( scalar )
		changed = restitution_scalar( r, a, b, sc.restitutionThreshold );
	else
		restitution_lane( r, a, b, sc.restitutionThreshold );
	if ( changed == false )
		return;
	B.store( r.ia, a );
	B.store( r.ib, b );
	if ( phase != F_WARM )
	{
		m.imp0[k] = make_float4( r.ni[0], r.ti[0], r.maxNi[0], 0.0f );
		m.imp1[k] = make_float4( r.ni[1], r.ti[1], r.maxNi[1], 0.0f );
	}
}

/* One joint phase with its bodies at B-indices ia and ib (-1 for a static body). */
template <class Bodies>
__device__ __forceinline__ void joint_step_at( const b2gDevWorld& W, const Bodies& B, int jid, int ia, int ib, int phase,
											   const b2gStepConst& sc )
{
	b2gJointDev* j = W.joints + jid;
	DevState a = B.load( ia );
	DevState b = B.load( ib );
	if ( phase == F_WARM )
		joint_warm_state( j, a, b );
	else
		joint_solve_state( j, a, b, phase == F_SOLVE, sc );
	B.store( ia, a );
	B.store( ib, b );
}

template <class Bodies>
__device__ __forceinline__ void joint_step( const b2gDevWorld& W, const Bodies& B, int jid, int phase, const b2gStepConst& sc )
{
	const b2gJointDev* j = W.joints + jid;
	joint_step_at( W, B, jid, j->indexA, j->indexB, phase, sc );
}

