/*
 * fused.cu -- the whole solver stage of one step in one launch: a thread-block cluster
 * of CL CTAs that keeps body states and constraint rows on chip and separates the
 * dependent phases with hardware cluster barriers.
 *
 * Why: a step of the reference solver (src/solver.c:559-731) is a chain of ~110
 * dependent sweeps (per substep: integrate, warm start per colour, solve per colour,
 * integrate positions, relax per colour; then restitution per colour), each moving
 * well under a megabyte.  One kernel launch per sweep leaves the GPU waiting on launch
 * latency; a barrier inside one resident cluster costs a small fraction of that.
 *
 * Layout (dynamic shared memory of every CTA, rank r of CL):
 *   bodies  body id b lives in CTA b % CL at slot b / CL: two state float4 (v, w, tag |
 *           dp, dq), the per-step velocity terms (float4 + float), and the CTA's list
 *           of awake slots.  Rows reach a body in another CTA through distributed
 *           shared memory.
 *   rows    row i of colour c lives in CTA i % CL at local index base[c] + i / CL, as
 *           nine float4 arrays (structure of arrays, conflict-free).  The overflow
 *           colour's rows all live in CTA 0 and thread 0 of CTA 0 solves them serially.
 *   joints  stay in global memory; joint i of colour c is always handled by the same
 *           thread (CTA i % CL), so only that thread reads and writes it.
 *
 * Arithmetic is b2g_solve.h's, shared with the per-phase kernels, so both paths give
 * the same bits.  Within a colour no two constraints share a non-static body
 * (src/constraint_graph.c:84-131), so a colour's rows run in parallel without
 * conflicts.  There is no spin-wait: every wait is a hardware barrier.
 */
#include "b2g_device.h"
#include "b2g_solve.h"

#include <cooperative_groups.h>
#include <cuda_runtime.h>

namespace cg = cooperative_groups;

#define FUSED_THREADS 256
#define FUSED_CLUSTER 16
/* dynamic shared memory per CTA, leaving 1 KB of the 227 KB opt-in limit for statics */
#define FUSED_SMEM_MAX ( 226 * 1024 )

enum
{
	F_WARM = 0,
	F_SOLVE = 1,
	F_RELAX = 2,
	F_RESTITUTION = 3,
};

struct FusedPlan
{
	int colorStart[B2G_COLORS + 1];
	int jointStart[B2G_COLORS + 1];
	int active[B2G_COLORS];
	int activeCount;
	int awakeCount;
	int bodyIdCount;
	int bodySlots; /* body slots per CTA */
	int rowCap;	   /* row slots per CTA */
};

/* Shared-memory carve-up; every CTA uses the same offsets, so a local address maps to
 * the same object in another CTA. */
struct FusedSmem
{
	float4* st0;   /* v.x v.y w tag */
	float4* st1;   /* dp.x dp.y dq.c dq.s */
	float4* term;  /* lvd.x lvd.y avd ld */
	float* ad;	   /* angular damping factor */
	int* awake;	   /* local awake slots */
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

static __host__ __device__ size_t fused_smem_bytes( int bodySlots, int rowCap )
{
	return (size_t)bodySlots * ( 3 * 16 + 4 + 4 ) + (size_t)rowCap * ( 9 * 16 ) + 64;
}

__device__ __forceinline__ FusedSmem carve( float4* base, int BS, int RC )
{
	FusedSmem m;
	m.idx = (int4*)base;
	m.nf = base + RC;
	m.ms = base + 2 * RC;
	m.anc0 = base + 3 * RC;
	m.anc1 = base + 4 * RC;
	m.coef0 = base + 5 * RC;
	m.coef1 = base + 6 * RC;
	m.imp0 = base + 7 * RC;
	m.imp1 = base + 8 * RC;
	m.st0 = base + 9 * RC;
	m.st1 = m.st0 + BS;
	m.term = m.st1 + BS;
	m.ad = (float*)( m.term + BS );
	m.awake = (int*)( m.ad + BS );
	return m;
}

template <int CL>
struct ClusterBodies
{
	cg::cluster_group cl;
	float4* st0;
	float4* st1;

	__device__ __forceinline__ DevState load( int b ) const
	{
		if ( b < 0 )
			return identity_state();
		unsigned r = (unsigned)b % CL;
		int s = b / CL;
		const float4* p0 = cl.map_shared_rank( st0 + s, r );
		const float4* p1 = cl.map_shared_rank( st1 + s, r );
		return state_of( *p0, *p1 );
	}

	__device__ __forceinline__ void store( int b, const DevState& x ) const
	{
		if ( b < 0 )
			return;
		float4* p0 = cl.map_shared_rank( st0 + b / CL, (unsigned)b % CL );
		*p0 = velocity_word( x );
	}
};

__device__ __forceinline__ void load_row_smem( const FusedSmem& m, int k, const b2gStepConst& sc, Row& r )
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

__device__ __forceinline__ void store_row_smem( const FusedSmem& m, int k, int cid, const Row& r )
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

template <int CL>
__device__ __forceinline__ void row_step( const FusedSmem& m, const ClusterBodies<CL>& B, int k, int phase, bool scalar,
										  const b2gStepConst& sc )
{
	Row r;
	load_row_smem( m, k, sc, r );
	DevState a = B.load( r.ia );
	DevState b = B.load( r.ib );
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

template <int CL>
__device__ __forceinline__ void joint_step( const b2gDevWorld& W, const ClusterBodies<CL>& B, int jid, int phase,
											const b2gStepConst& sc )
{
	b2gJointDev* j = W.joints + jid;
	DevState a = B.load( j->indexA );
	DevState b = B.load( j->indexB );
	if ( phase == F_WARM )
		joint_warm_state( j, a, b );
	else
		joint_solve_state( j, a, b, phase == F_SOLVE, sc );
	B.store( j->indexA, a );
	B.store( j->indexB, b );
}

__device__ __forceinline__ int local_count( int n, int rank, int CL ) { return n > rank ? ( n - rank + CL - 1 ) / CL : 0; }

/* One stage over all colours: the overflow set first (serially, CTA 0 thread 0), then
 * each active colour with a cluster barrier after it. */
template <int CL>
__device__ void run_stage( const b2gDevWorld& W, const FusedPlan& P, const FusedSmem& m, const ClusterBodies<CL>& B,
						   const int* base, int rank, int phase, const b2gStepConst& sc )
{
	const int* cs = P.colorStart;
	const int* js = P.jointStart;
	int ovRows = cs[B2G_COLORS] - cs[B2G_OVERFLOW];
	int ovJointsAll = js[B2G_COLORS] - js[B2G_OVERFLOW];
	int ovJoints = phase == F_RESTITUTION ? 0 : ovJointsAll;
	/* the per-phase path runs the overflow set when it has any constraint, and for
	 * restitution when it has contacts */
	bool overflow = phase == F_RESTITUTION ? ovRows > 0 : ovRows + ovJointsAll > 0;
	if ( overflow )
	{
		if ( rank == 0 && threadIdx.x == 0 )
		{
			for ( int i = 0; i < ovJoints; ++i )
				joint_step<CL>( W, B, W.jointList[js[B2G_OVERFLOW] + i], phase, sc );
			for ( int i = 0; i < ovRows; ++i )
				row_step<CL>( m, B, base[B2G_OVERFLOW] + i, phase, true, sc );
		}
		B.cl.sync();
	}
	if ( phase == F_WARM && sc.enableWarmStarting == 0 )
		return;
	for ( int a = 0; a < P.activeCount; ++a )
	{
		int c = P.active[a];
		int nr = local_count( cs[c + 1] - cs[c], rank, CL );
		int nj = phase == F_RESTITUTION ? 0 : local_count( js[c + 1] - js[c], rank, CL );
		if ( phase == F_RESTITUTION && cs[c + 1] == cs[c] )
			continue;
		for ( int j = threadIdx.x; j < nr; j += FUSED_THREADS )
			row_step<CL>( m, B, base[c] + j, phase, false, sc );
		for ( int j = threadIdx.x; j < nj; j += FUSED_THREADS )
			joint_step<CL>( W, B, W.jointList[js[c] + rank + j * CL], phase, sc );
		B.cl.sync();
	}
}

template <int CL>
__global__ void __launch_bounds__( FUSED_THREADS ) k_solve_fused( b2gDevWorld W, FusedPlan P, b2gStepConst sc )
{
	extern __shared__ float4 smem[];
	__shared__ int base[B2G_COLORS + 1];
	__shared__ int awakeLocal;
	cg::cluster_group cl = cg::this_cluster();
	const int rank = (int)cl.block_rank();
	const int tid = threadIdx.x;
	const int BS = P.bodySlots;
	FusedSmem m = carve( smem, BS, P.rowCap );
	const int* cs = P.colorStart;

	if ( tid == 0 )
	{
		/* local row bases: active colours in order, then the overflow set (CTA 0 only) */
		int n = 0;
		for ( int c = 0; c <= B2G_COLORS; ++c )
			base[c] = 0;
		for ( int a = 0; a < P.activeCount; ++a )
		{
			int c = P.active[a];
			base[c] = n;
			n += local_count( cs[c + 1] - cs[c], rank, CL );
		}
		base[B2G_OVERFLOW] = n;
		awakeLocal = 0;
	}

	/* owned body states */
	const float4* gst = (const float4*)W.state;
	for ( int s = tid; s < BS; s += FUSED_THREADS )
	{
		int b = s * CL + rank;
		if ( b < P.bodyIdCount )
		{
			m.st0[s] = gst[2 * b];
			m.st1[s] = gst[2 * b + 1];
		}
	}
	__syncthreads();

	/* owned awake bodies and their per-step velocity terms */
	for ( int i = tid; i < P.awakeCount; i += FUSED_THREADS )
	{
		int b = W.awake[i];
		if ( b % CL != rank )
			continue;
		int s = b / CL;
		int slot = atomicAdd( &awakeLocal, 1 );
		m.awake[slot] = s;
		VelocityTerms t = velocity_terms( ( (const float4*)W.mass )[b], ( (const float4*)W.force )[b],
										  ( (const float4*)W.extent )[b], sc );
		m.term[s] = make_float4( t.lvd.x, t.lvd.y, t.avd, t.ld );
		m.ad[s] = t.ad;
	}

	/* constraint rows (reference src/contact_solver.c:597-808), from the global state */
	const float4* mass = (const float4*)W.mass;
	const float4 zero = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
	const float warm = sc.enableWarmStarting ? 1.0f : 0.0f;
	for ( int a = -1; a < P.activeCount; ++a )
	{
		int c = a < 0 ? B2G_OVERFLOW : P.active[a];
		int n = cs[c + 1] - cs[c];
		int local = c == B2G_OVERFLOW ? ( rank == 0 ? n : 0 ) : local_count( n, rank, CL );
		for ( int j = tid; j < local; j += FUSED_THREADS )
		{
			int i = c == B2G_OVERFLOW ? j : rank + j * CL;
			int cid = W.solveList[cs[c] + i];
			int ia = W.cBodies[2 * cid];
			int ib = W.cBodies[2 * cid + 1];
			DevState sA = ia >= 0 ? state_of( gst[2 * ia], gst[2 * ia + 1] ) : identity_state();
			DevState sB = ib >= 0 ? state_of( gst[2 * ib], gst[2 * ib + 1] ) : identity_state();
			Row r;
			prepare_row( r, W.manifold + cid, ia, ib, ia >= 0 ? mass[ia] : zero, ib >= 0 ? mass[ib] : zero, sA, sB,
						 W.cMix[2 * cid], W.cMix[2 * cid + 1], ( ia < 0 || ib < 0 ) ? sc.staticSoft : sc.contactSoft, warm );
			store_row_smem( m, base[c] + j, cid, r );
		}
	}
	ClusterBodies<CL> B{ cl, m.st0, m.st1 };
	cl.sync();

	for ( int sub = 0; sub < sc.subSteps; ++sub )
	{
		for ( int j = tid; j < awakeLocal; j += FUSED_THREADS )
		{
			int s = m.awake[j];
			DevState x = state_of( m.st0[s], m.st1[s] );
			float4 t4 = m.term[s];
			VelocityTerms t;
			t.lvd = gv( t4.x, t4.y );
			t.avd = t4.z;
			t.ld = t4.w;
			t.ad = m.ad[s];
			integrate_velocity( x, t, sc );
			m.st0[s] = velocity_word( x );
		}
		cl.sync();
		run_stage<CL>( W, P, m, B, base, rank, F_WARM, sc );
		run_stage<CL>( W, P, m, B, base, rank, F_SOLVE, sc );
		for ( int j = tid; j < awakeLocal; j += FUSED_THREADS )
		{
			int s = m.awake[j];
			DevState x = state_of( m.st0[s], m.st1[s] );
			integrate_position( x, sc.h );
			m.st1[s] = make_float4( x.dp.x, x.dp.y, x.dq.c, x.dq.s );
		}
		cl.sync();
		run_stage<CL>( W, P, m, B, base, rank, F_RELAX, sc );
	}
	run_stage<CL>( W, P, m, B, base, rank, F_RESTITUTION, sc );

	/* store impulses (reference src/contact_solver.c:442-471, :1180-1293): colour rows
	 * write both point slots, overflow rows their points */
	int localRows = base[B2G_OVERFLOW] + ( rank == 0 ? cs[B2G_COLORS] - cs[B2G_OVERFLOW] : 0 );
	for ( int k = tid; k < localRows; k += FUSED_THREADS )
	{
		int4 idx = m.idx[k];
		b2gManifold* mf = W.manifold + idx.z;
		int n = k < base[B2G_OVERFLOW] ? 2 : idx.w;
		float4 imp[2] = { m.imp0[k], m.imp1[k] };
		float4 coef[2] = { m.coef0[k], m.coef1[k] };
		for ( int j = 0; j < n; ++j )
		{
			mf->pts[j].normalImpulse = imp[j].x;
			mf->pts[j].tangentImpulse = imp[j].y;
			mf->pts[j].maxNormalImpulse = imp[j].z;
			mf->pts[j].normalVelocity = coef[j].w;
		}
	}
	/* owned awake body states back to global memory for finalisation */
	float4* gout = (float4*)W.state;
	for ( int j = tid; j < awakeLocal; j += FUSED_THREADS )
	{
		int s = m.awake[j];
		int b = s * CL + rank;
		gout[2 * b] = m.st0[s];
		gout[2 * b + 1] = m.st1[s];
	}
}

/* Launches the fused solver when the world fits on chip; returns the number of launches,
 * or 0 when the world does not fit (or clusters of FUSED_CLUSTER are unavailable) and the
 * caller must use the per-phase kernels. */
extern "C" int b2gd_prepare_joints( b2gDevWorld* w, int joints, const b2gStepConst* sc );

extern "C" int b2gd_solver_fused( b2gDevWorld* w, const b2gSolvePlan* plan, const b2gStepConst* sc )
{
	/* per device: 0 unknown, 1 available, -1 unavailable */
	static int s_readyByDevice[64];
	const int CL = FUSED_CLUSTER;
	int dev = 0;
	if ( cudaGetDevice( &dev ) != cudaSuccess || dev < 0 || dev >= 64 )
		return 0;
	int& s_ready = s_readyByDevice[dev];
	if ( plan->bodyIdCount <= 0 )
		return 0;
	FusedPlan P;
	for ( int c = 0; c <= B2G_COLORS; ++c )
	{
		P.colorStart[c] = plan->colorStart[c];
		P.jointStart[c] = plan->jointStart[c];
	}
	for ( int c = 0; c < B2G_COLORS; ++c )
		P.active[c] = plan->active[c];
	P.activeCount = plan->activeCount;
	P.awakeCount = plan->awakeCount;
	P.bodyIdCount = plan->bodyIdCount;
	P.bodySlots = ( plan->bodyIdCount + CL - 1 ) / CL;
	int rows = 0;
	for ( int a = 0; a < plan->activeCount; ++a )
	{
		int c = plan->active[a];
		rows += ( plan->colorStart[c + 1] - plan->colorStart[c] + CL - 1 ) / CL;
	}
	rows += plan->colorStart[B2G_COLORS] - plan->colorStart[B2G_OVERFLOW];
	P.rowCap = rows > 0 ? rows : 1;
	size_t bytes = fused_smem_bytes( P.bodySlots, P.rowCap );
	if ( bytes > FUSED_SMEM_MAX )
		return 0;

	auto kernel = k_solve_fused<FUSED_CLUSTER>;
	if ( s_ready == 0 )
	{
		s_ready = -1;
		if ( cudaFuncSetAttribute( kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1 ) == cudaSuccess &&
			 cudaFuncSetAttribute( kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, FUSED_SMEM_MAX ) == cudaSuccess )
		{
			cudaLaunchConfig_t cfg = {};
			cudaLaunchAttribute attr[1];
			attr[0].id = cudaLaunchAttributeClusterDimension;
			attr[0].val.clusterDim.x = CL;
			attr[0].val.clusterDim.y = 1;
			attr[0].val.clusterDim.z = 1;
			cfg.gridDim = dim3( CL, 1, 1 );
			cfg.blockDim = dim3( FUSED_THREADS, 1, 1 );
			cfg.dynamicSmemBytes = FUSED_SMEM_MAX;
			cfg.attrs = attr;
			cfg.numAttrs = 1;
			int clusters = 0;
			if ( cudaOccupancyMaxActiveClusters( &clusters, kernel, &cfg ) == cudaSuccess && clusters >= 1 )
				s_ready = 1;
		}
		cudaGetLastError();
	}
	if ( s_ready != 1 )
		return 0;

	cudaLaunchConfig_t cfg = {};
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = CL;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.gridDim = dim3( CL, 1, 1 );
	cfg.blockDim = dim3( FUSED_THREADS, 1, 1 );
	cfg.dynamicSmemBytes = bytes;
	cfg.stream = (cudaStream_t)w->stream;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	int launches = b2gd_prepare_joints( w, plan->jointStart[B2G_COLORS], sc );
	if ( cudaLaunchKernelEx( &cfg, kernel, *w, P, *sc ) != cudaSuccess )
		return -1;
	return launches + 1;
}
