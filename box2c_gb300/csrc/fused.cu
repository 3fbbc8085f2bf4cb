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
 *   bodies  body ids are cut into CL contiguous blocks of bodySlots: body b lives in CTA
 *           b / bodySlots at slot b % bodySlots (the owner is found by a multiply-high
 *           with a host-computed reciprocal): two state float4 (v, w, tag | dp, dq), the
 *           per-step velocity terms (float4 + float), an awake flag, and the CTA's list
 *           of awake slots.  Rows reach a body of another CTA through distributed
 *           shared memory.
 *   rows    the host groups each colour's rows by the CTA owning their first
 *           non-static body (rows of one colour share no body, so the order within a
 *           colour changes no result); CTA o holds rows [split[c][o], split[c][o+1]) of
 *           colour c from local index ctaBase[c][o], as nine float4 arrays (structure of
 *           arrays, conflict-free).  Most body accesses of a row are then local.  The
 *           overflow colour's rows all live in CTA 0; thread 0 of CTA 0 solves them
 *           serially on CTA-local copies of their bodies.
 *   joints  stay in global memory; joint i of colour c is always handled by the same
 *           thread (CTA i % CL), so only that thread reads and writes it.
 *
 * Arithmetic is b2g_solve.h's, shared with the per-phase kernels, so both paths give
 * the same bits.  Within a colour no two constraints share a non-static body
 * (src/constraint_graph.c:84-131), so a colour's rows run in parallel without
 * conflicts.  There is no spin-wait: every wait is a hardware barrier.
 */
#include "b2g_cluster.h"
#include "b2g_device.h"

#include <cuda_runtime.h>

#include <string.h>

#define FUSED_THREADS 256
#define FUSED_CLUSTER B2G_FUSED_CTAS
/* dynamic shared memory per CTA, leaving 1 KB of the 227 KB opt-in limit for statics */
#define FUSED_SMEM_MAX ( 226 * 1024 )


struct FusedPlan
{
	int colorStart[B2G_COLORS + 1];
	int jointStart[B2G_COLORS + 1];
	int active[B2G_COLORS];
	int activeCount;
	int bodyIdCount;
	int bodySlots; /* body slots per CTA: body b lives in CTA b / bodySlots */
	int rowCap;	   /* row slots per CTA */
	int imageFloat4;
	/* rows of colour c owned by CTA o: offsets [split[c][o], split[c][o+1]) within the
	 * colour, stored from local index ctaBase[c][o]; the overflow rows live in CTA 0 from
	 * ctaBase[B2G_OVERFLOW][0] */
	int split[B2G_OVERFLOW][B2G_FUSED_CTAS + 1];
	int ctaBase[B2G_COLORS][B2G_FUSED_CTAS];
	/* overflow set solved on local copies of its bodies in CTA 0 (1) or in place (0);
	 * the copies and their index tables start at float4 offset ovOffset */
	int ovCached;
	int ovOffset;
	unsigned bodySlotsInv; /* ceil(2^32 / bodySlots), for the owner of a body id */
};

/* Shared-memory carve-up; every CTA uses the same offsets, so a local address maps to
 * the same object in another CTA.  The first imageFloat4 float4 are the image the
 * staging kernel writes to global memory (rows, bodies, awake flags); the local awake
 * list follows it. */
struct FusedSmem : SmemRows
{
	float4* st0;  /* v.x v.y w tag */
	float4* st1;  /* dp.x dp.y dq.c dq.s */
	float4* term; /* lvd.x lvd.y avd ld */
	float* ad;	  /* angular damping factor */
	int* flags;	  /* 1 for an awake body */
	int* awake;	  /* local awake slots */
};

static __host__ __device__ int image_float4( int bodySlots, int rowCap )
{
	/* 9 row arrays, 3 body float4 arrays, two body 4-byte arrays */
	return 9 * rowCap + 3 * bodySlots + ( 2 * bodySlots + 3 ) / 4;
}

static size_t fused_smem_bytes( int bodySlots, int rowCap )
{
	return 16 * (size_t)image_float4( bodySlots, rowCap ) + 4 * (size_t)bodySlots + 16;
}

/* Overflow cache of CTA 0: for R overflow rows and J overflow joints with E = 2 (R + J)
 * body ends, the rows' indices with body slots (int4 x R), slot states (2 x float4 x E),
 * slot bodies, first occurrences and slots per end (3 x int x E), joint slots (int2 x J). */
#define FUSED_OVERFLOW_MAX 512

struct OverflowCache
{
	int4* idx;
	float4* st0;
	float4* st1;
	int* body;
	int* first;
	int* slot;
	int2* jslot;
};

static __host__ __device__ size_t overflow_bytes( int R, int J )
{
	size_t E = 2u * (size_t)( R + J );
	return 16u * ( (size_t)R + 2u * E ) + 4u * ( 3u * E + 2u * (size_t)J );
}

__device__ __forceinline__ OverflowCache carve_overflow( float4* base, int R, int J )
{
	int E = 2 * ( R + J );
	OverflowCache o;
	o.idx = (int4*)base;
	o.st0 = base + R;
	o.st1 = o.st0 + E;
	o.body = (int*)( o.st1 + E );
	o.first = o.body + E;
	o.slot = o.first + E;
	o.jslot = (int2*)( o.slot + E );
	return o;
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
	m.flags = (int*)( m.ad + BS );
	m.awake = (int*)( base + image_float4( BS, RC ) );
	return m;
}

__device__ __forceinline__ int local_count( int n, int rank, int CL ) { return n > rank ? ( n - rank + CL - 1 ) / CL : 0; }

/* One stage over all colours: the overflow set first (serially, CTA 0 thread 0), then
 * each active colour with a cluster barrier after it.  JOINTS false compiles the joint
 * calls out, so a world without joints runs the contact sweep alone. */
template <int CL, bool JOINTS>
__device__ void run_stage( const b2gDevWorld& W, const FusedPlan& P, const FusedSmem& m, const ClusterBodies& B, int rank,
						   int phase, const b2gStepConst& sc, const OverflowCache& ov, int ovSlots )
{
	const int* cs = P.colorStart;
	const int* js = P.jointStart;
	int ovRows = cs[B2G_COLORS] - cs[B2G_OVERFLOW];
	int ovJointsAll = JOINTS ? js[B2G_COLORS] - js[B2G_OVERFLOW] : 0;
	int ovJoints = phase == F_RESTITUTION ? 0 : ovJointsAll;
	/* the per-phase path runs the overflow set when it has any constraint, and for
	 * restitution when it has contacts */
	bool overflow = phase == F_RESTITUTION ? ovRows > 0 : ovRows + ovJointsAll > 0;
	if ( overflow )
	{
		int base = P.ctaBase[B2G_OVERFLOW][0];
		if ( rank == 0 && P.ovCached )
		{
			/* the set's bodies to local slots, the serial pass on them, velocities back:
			 * nothing else touches a body while the set runs */
			for ( int s = threadIdx.x; s < ovSlots; s += FUSED_THREADS )
			{
				int b = ov.body[s];
				ov.st0[s] = *B.word( B.st0, b );
				ov.st1[s] = *B.word( B.st1, b );
			}
			__syncthreads();
			if ( threadIdx.x == 0 )
			{
				SharedBodies OB{ ov.st0, ov.st1 };
				for ( int i = 0; i < ovJoints; ++i )
					joint_step_at( W, OB, W.jointList[js[B2G_OVERFLOW] + i], ov.jslot[i].x, ov.jslot[i].y, phase, sc );
				SmemRows mo;
				mo.idx = ov.idx;
				mo.nf = m.nf + base;
				mo.ms = m.ms + base;
				mo.anc0 = m.anc0 + base;
				mo.anc1 = m.anc1 + base;
				mo.coef0 = m.coef0 + base;
				mo.coef1 = m.coef1 + base;
				mo.imp0 = m.imp0 + base;
				mo.imp1 = m.imp1 + base;
				for ( int i = 0; i < ovRows; ++i )
					row_step( mo, OB, i, phase, true, sc );
			}
			__syncthreads();
			for ( int s = threadIdx.x; s < ovSlots; s += FUSED_THREADS )
				*B.word( B.st0, ov.body[s] ) = ov.st0[s];
		}
		else if ( rank == 0 && threadIdx.x == 0 )
		{
			for ( int i = 0; i < ovJoints; ++i )
				joint_step( W, B, W.jointList[js[B2G_OVERFLOW] + i], phase, sc );
			for ( int i = 0; i < ovRows; ++i )
				row_step( m, B, base + i, phase, true, sc );
		}
		B.cl.sync();
	}
	if ( phase == F_WARM && sc.enableWarmStarting == 0 )
		return;
	for ( int a = 0; a < P.activeCount; ++a )
	{
		int c = P.active[a];
		if ( phase == F_RESTITUTION && cs[c + 1] == cs[c] )
			continue;
		int base = P.ctaBase[c][rank];
		int nr = P.split[c][rank + 1] - P.split[c][rank];
		int nj = ( JOINTS == false || phase == F_RESTITUTION ) ? 0 : local_count( js[c + 1] - js[c], rank, CL );
		for ( int j = threadIdx.x; j < nr; j += FUSED_THREADS )
			row_step( m, B, base + j, phase, false, sc );
		for ( int j = threadIdx.x; j < nj; j += FUSED_THREADS )
			joint_step( W, B, W.jointList[js[c] + rank + j * CL], phase, sc );
		B.cl.sync();
	}
}

/* Staging: writes every CTA's shared-memory image (constraint rows, reference
 * src/contact_solver.c:597-808 and :21-147; body states; per-step velocity terms,
 * src/solver.c:34-93) to global memory, one thread per row and per body id. */
__global__ void __launch_bounds__( 128 ) k_fused_stage( b2gDevWorld W, FusedPlan P, b2gStepConst sc, float4* image )
{
	if ( W.guardEvents && W.counters[0] != 0 )
		return;
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	const int* cs = P.colorStart;
	const int BS = P.bodySlots, RC = P.rowCap;
	const float4* gst = (const float4*)W.state;
	const float4* mass = (const float4*)W.mass;
	if ( t < cs[B2G_COLORS] )
	{
		int c = 0;
		while ( cs[c + 1] <= t )
			++c;
		int o = 0, local;
		if ( c == B2G_OVERFLOW )
			local = P.ctaBase[B2G_OVERFLOW][0] + ( t - cs[B2G_OVERFLOW] );
		else
		{
			int i = t - cs[c];
			while ( P.split[c][o + 1] <= i )
				++o;
			local = P.ctaBase[c][o] + ( i - P.split[c][o] );
		}
		FusedSmem m = carve( image + (size_t)o * P.imageFloat4, BS, RC );
		int cid = W.solveList[t];
		int ia = W.cBodies[2 * cid];
		int ib = W.cBodies[2 * cid + 1];
		float4 zero = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		DevState sA = ia >= 0 ? state_of( gst[2 * ia], gst[2 * ia + 1] ) : identity_state();
		DevState sB = ib >= 0 ? state_of( gst[2 * ib], gst[2 * ib + 1] ) : identity_state();
		Row r;
		prepare_row( r, W.manifold + cid, ia, ib, ia >= 0 ? mass[ia] : zero, ib >= 0 ? mass[ib] : zero, sA, sB,
					 W.cMix[2 * cid], W.cMix[2 * cid + 1], ( ia < 0 || ib < 0 ) ? sc.staticSoft : sc.contactSoft,
					 sc.enableWarmStarting ? 1.0f : 0.0f );
		store_row_smem( m, local, cid, r );
	}
	if ( t < P.bodyIdCount )
	{
		int o = t / BS;
		int s = t - o * BS;
		FusedSmem m = carve( image + (size_t)o * P.imageFloat4, BS, RC );
		m.st0[s] = gst[2 * t];
		m.st1[s] = gst[2 * t + 1];
		bool awake = ( W.bodyInfo[t] & B2G_B_AWAKE ) != 0;
		m.flags[s] = awake ? 1 : 0;
		if ( awake )
		{
			VelocityTerms v = velocity_terms( mass[t], ( (const float4*)W.force )[t], ( (const float4*)W.extent )[t], sc );
			m.term[s] = make_float4( v.lvd.x, v.lvd.y, v.avd, v.ld );
			m.ad[s] = v.ad;
		}
	}
}

template <int CL, bool JOINTS>
__global__ void __launch_bounds__( FUSED_THREADS, 1 ) k_solve_fused( b2gDevWorld W, FusedPlan P, b2gStepConst sc, const float4* image )
{
	/* every CTA of the cluster takes the same branch: no barrier is left waiting */
	if ( W.guardEvents && W.counters[0] != 0 )
		return;
	extern __shared__ float4 smem[];
	__shared__ int awakeLocal;
	cg::cluster_group cl = cg::this_cluster();
	const int rank = (int)cl.block_rank();
	const int tid = threadIdx.x;
	const int BS = P.bodySlots;
	FusedSmem m = carve( smem, BS, P.rowCap );
	const int* cs = P.colorStart;

	/* this CTA's image: rows, owned bodies, velocity terms, awake flags */
	const float4* src = image + (size_t)rank * P.imageFloat4;
	const int n4 = P.imageFloat4;
#pragma unroll 4
	for ( int i = tid; i < n4; i += FUSED_THREADS )
		smem[i] = src[i];
	if ( tid == 0 )
		awakeLocal = 0;
	__syncthreads();
	int bodies = P.bodyIdCount - rank * BS;
	bodies = bodies < 0 ? 0 : ( bodies > BS ? BS : bodies );
	for ( int s = tid; s < bodies; s += FUSED_THREADS )
	{
		if ( m.flags[s] )
			m.awake[atomicAdd( &awakeLocal, 1 )] = s;
	}
	/* overflow cache: distinct bodies of the set's ends get slots in end order */
	const int ovR = cs[B2G_COLORS] - cs[B2G_OVERFLOW];
	const int ovJ = JOINTS ? P.jointStart[B2G_COLORS] - P.jointStart[B2G_OVERFLOW] : 0;
	const int ovBase = P.ctaBase[B2G_OVERFLOW][0];
	OverflowCache ov = carve_overflow( smem + P.ovOffset, ovR, ovJ );
	__shared__ int ovSlots;
	if ( rank == 0 && P.ovCached )
	{
		const int E = 2 * ( ovR + ovJ );
		auto end_body = [&]( int e ) {
			if ( e < 2 * ovJ )
			{
				const b2gJointDev* j = W.joints + W.jointList[P.jointStart[B2G_OVERFLOW] + ( e >> 1 )];
				return ( e & 1 ) ? j->indexB : j->indexA;
			}
			int4 ix = m.idx[ovBase + ( ( e - 2 * ovJ ) >> 1 )];
			return ( e & 1 ) ? ix.y : ix.x;
		};
		for ( int e = tid; e < E; e += FUSED_THREADS )
		{
			int b = end_body( e );
			int f = -1;
			if ( b >= 0 )
			{
				f = e;
				for ( int e2 = 0; e2 < e; ++e2 )
				{
					if ( end_body( e2 ) == b )
					{
						f = e2;
						break;
					}
				}
			}
			ov.first[e] = f;
		}
		__syncthreads();
		if ( tid == 0 )
		{
			int K = 0;
			for ( int e = 0; e < E; ++e )
			{
				if ( ov.first[e] == e )
				{
					ov.slot[e] = K;
					ov.body[K++] = end_body( e );
				}
			}
			ovSlots = K;
		}
		__syncthreads();
		for ( int e = tid; e < E; e += FUSED_THREADS )
		{
			int f = ov.first[e];
			int s = f < 0 ? -1 : ov.slot[f];
			if ( e < 2 * ovJ )
			{
				if ( e & 1 )
					ov.jslot[e >> 1].y = s;
				else
					ov.jslot[e >> 1].x = s;
			}
			else
			{
				int r = ( e - 2 * ovJ ) >> 1;
				if ( e & 1 )
					ov.idx[r].y = s;
				else
				{
					int4 ix = m.idx[ovBase + r];
					ov.idx[r].x = s;
					ov.idx[r].z = ix.z;
					ov.idx[r].w = ix.w;
				}
			}
		}
	}
	ClusterBodies B{ cl, m.st0, m.st1, BS, rank, P.bodySlotsInv };
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
		run_stage<CL, JOINTS>( W, P, m, B, rank, F_WARM, sc, ov, ovSlots );
		run_stage<CL, JOINTS>( W, P, m, B, rank, F_SOLVE, sc, ov, ovSlots );
		for ( int j = tid; j < awakeLocal; j += FUSED_THREADS )
		{
			int s = m.awake[j];
			DevState x = state_of( m.st0[s], m.st1[s] );
			integrate_position( x, sc.h );
			m.st1[s] = make_float4( x.dp.x, x.dp.y, x.dq.c, x.dq.s );
		}
		cl.sync();
		run_stage<CL, JOINTS>( W, P, m, B, rank, F_RELAX, sc, ov, ovSlots );
	}
	run_stage<CL, JOINTS>( W, P, m, B, rank, F_RESTITUTION, sc, ov, ovSlots );

	/* store impulses (reference src/contact_solver.c:442-471, :1180-1293): colour rows
	 * write both point slots, overflow rows their points */
	int colourRows = 0;
	for ( int a = 0; a < P.activeCount; ++a )
	{
		int c = P.active[a];
		colourRows += P.split[c][rank + 1] - P.split[c][rank];
	}
	int localRows = colourRows + ( rank == 0 ? cs[B2G_COLORS] - cs[B2G_OVERFLOW] : 0 );
	for ( int k = tid; k < localRows; k += FUSED_THREADS )
	{
		int4 idx = m.idx[k];
		b2gManifold* mf = W.manifold + idx.z;
		int n = k < colourRows ? 2 : idx.w;
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
		int b = rank * BS + s;
		gout[2 * b] = m.st0[s];
		gout[2 * b + 1] = m.st1[s];
	}
}

extern "C" int b2gd_prepare_joints( b2gDevWorld* w, int joints, const b2gStepConst* sc );

static cudaLaunchConfig_t cluster_config( cudaLaunchAttribute* attr, size_t smem, cudaStream_t stream )
{
	cudaLaunchConfig_t cfg = {};
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = FUSED_CLUSTER;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.gridDim = dim3( FUSED_CLUSTER, 1, 1 );
	cfg.blockDim = dim3( FUSED_THREADS, 1, 1 );
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	return cfg;
}

/* Launches the fused solver when the world fits on chip; returns the number of launches,
 * 0 when it does not fit (or clusters of FUSED_CLUSTER CTAs are unavailable) and the
 * caller must use the per-phase kernels, or -1 on a launch error. */
extern "C" int b2gd_solver_fused( b2gDevWorld* w, const b2gSolvePlan* plan, const b2gStepConst* sc )
{
	/* per device: 0 unknown, 1 available, -1 unavailable */
	static int s_readyByDevice[64];
	const int CL = FUSED_CLUSTER;
	/* body ids and slots below 2^16: the owner division is one multiply-high */
	if ( plan->bodyIdCount <= 0 || plan->bodyBlock <= 0 || plan->bodyIdCount >= 65536 )
		return 0;
	int dev = 0;
	if ( cudaGetDevice( &dev ) != cudaSuccess || dev < 0 || dev >= 64 )
		return 0;
	int& ready = s_readyByDevice[dev];

	FusedPlan P;
	memset( &P, 0, sizeof( P ) );
	for ( int c = 0; c <= B2G_COLORS; ++c )
	{
		P.colorStart[c] = plan->colorStart[c];
		P.jointStart[c] = plan->jointStart[c];
	}
	for ( int c = 0; c < B2G_COLORS; ++c )
		P.active[c] = plan->active[c];
	P.activeCount = plan->activeCount;
	P.bodyIdCount = plan->bodyIdCount;
	P.bodySlots = plan->bodyBlock;
	P.bodySlotsInv = P.bodySlots > 1 ? (unsigned)( ( ( 1ull << 32 ) + (unsigned long long)P.bodySlots - 1 ) / (unsigned long long)P.bodySlots ) : 0u;
	int perCta[B2G_FUSED_CTAS] = { 0 };
	for ( int c = 0; c < B2G_OVERFLOW; ++c )
	{
		int n = 0;
		for ( int o = 0; o < CL; ++o )
		{
			P.split[c][o] = n;
			n += plan->rowSplit[c][o];
		}
		P.split[c][CL] = n;
		if ( n != plan->colorStart[c + 1] - plan->colorStart[c] )
			return 0; /* rows not grouped by owner */
	}
	for ( int a = 0; a < plan->activeCount; ++a )
	{
		int c = plan->active[a];
		for ( int o = 0; o < CL; ++o )
		{
			P.ctaBase[c][o] = perCta[o];
			perCta[o] += plan->rowSplit[c][o];
		}
	}
	P.ctaBase[B2G_OVERFLOW][0] = perCta[0];
	perCta[0] += plan->colorStart[B2G_COLORS] - plan->colorStart[B2G_OVERFLOW];
	int rowCap = 1;
	for ( int o = 0; o < CL; ++o )
		rowCap = perCta[o] > rowCap ? perCta[o] : rowCap;
	P.rowCap = rowCap;
	P.imageFloat4 = image_float4( P.bodySlots, P.rowCap );
	size_t bytes = fused_smem_bytes( P.bodySlots, P.rowCap );
	if ( bytes > FUSED_SMEM_MAX )
		return 0;
	int ovR = plan->colorStart[B2G_COLORS] - plan->colorStart[B2G_OVERFLOW];
	int ovJ = plan->jointStart[B2G_COLORS] - plan->jointStart[B2G_OVERFLOW];
	size_t ovAt = ( bytes + 15 ) / 16;
	size_t withCache = 16 * ovAt + overflow_bytes( ovR, ovJ );
	if ( ovR + ovJ > 0 && ovR + ovJ <= FUSED_OVERFLOW_MAX && withCache <= FUSED_SMEM_MAX )
	{
		P.ovCached = 1;
		P.ovOffset = (int)ovAt;
		bytes = withCache;
	}

	auto plain = k_solve_fused<FUSED_CLUSTER, false>;
	auto jointed = k_solve_fused<FUSED_CLUSTER, true>;
	auto kernel = plan->jointStart[B2G_COLORS] > 0 ? jointed : plain;
	if ( ready == 0 )
	{
		ready = -1;
		bool ok = true;
		for ( auto k : { plain, jointed } )
		{
			ok = ok && cudaFuncSetAttribute( k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1 ) == cudaSuccess &&
				 cudaFuncSetAttribute( k, cudaFuncAttributeMaxDynamicSharedMemorySize, FUSED_SMEM_MAX ) == cudaSuccess;
			cudaLaunchAttribute attr[1];
			cudaLaunchConfig_t cfg = cluster_config( attr, FUSED_SMEM_MAX, nullptr );
			int clusters = 0;
			ok = ok && cudaOccupancyMaxActiveClusters( &clusters, k, &cfg ) == cudaSuccess && clusters >= 1;
		}
		if ( ok )
			ready = 1;
		cudaGetLastError();
	}
	if ( ready != 1 )
		return 0;

	size_t stage = 16 * (size_t)P.imageFloat4 * CL;
	if ( w->stageBytes < stage )
	{
		if ( w->stage )
			cudaFree( w->stage );
		w->stage = nullptr;
		w->stageBytes = 0;
		if ( cudaMalloc( &w->stage, stage ) != cudaSuccess )
			return -1;
		w->stageBytes = stage;
	}
	cudaStream_t s = (cudaStream_t)w->stream;
	int launches = b2gd_prepare_joints( w, plan->jointStart[B2G_COLORS], sc );
	int rows = plan->colorStart[B2G_COLORS];
	int threads = rows > plan->bodyIdCount ? rows : plan->bodyIdCount;
	k_fused_stage<<<( threads + 127 ) / 128, 128, 0, s>>>( *w, P, *sc, (float4*)w->stage );
	cudaLaunchAttribute attr[1];
	cudaLaunchConfig_t cfg = cluster_config( attr, bytes, s );
	if ( cudaLaunchKernelEx( &cfg, kernel, *w, P, *sc, (const float4*)w->stage ) != cudaSuccess )
		return -1;
	return launches + 2;
}
