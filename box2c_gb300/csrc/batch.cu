/*
 * batch.cu -- device side of b2World_StepBatch: many independent worlds per launch.
 *
 * Narrowphase: two grid-stride kernels over the concatenated contact records and
 * contact ids of all worlds (a flat index finds its world by binary search over the
 * prefix sums).  Solver: one persistent kernel; each CTA takes the next pack from a
 * queue: worlds of similar size side by side, each on a group of threads (one warp, a
 * named-barrier group or the whole CTA) that runs the world's whole solver stage and
 * finalisation with the group's barrier between the dependent phases.  Body states
 * always live in shared memory; a world whose constraint rows fit beside them keeps the
 * rows there too, a larger one in its own row arrays.  The per-row work is
 * b2g_stages.h's and b2g_cluster.h's, the same functions the single-world kernels use,
 * so every world gets the bits it would get from b2World_Step alone.
 *
 * A step's worlds run in two halves, each with its own graphs (uploads, kernels,
 * counter download), captured once and replayed every step, so that the host work of
 * one half overlaps the device work of the other; the kernels read their counts from
 * device memory, so the graphs do not change while the number of worlds and the
 * shared-memory size stay the same.  The solver's launch shape (threads per CTA, CTAs
 * per SM and so shared memory per world) is chosen by timing the candidates on the
 * first steps (any choice gives the same results).
 */
#include "b2g_cluster.h"
#include "b2g_packs.h"
#include "b2g_stages.h"

#include <cuda_runtime.h>

#include <stdlib.h>
#include <string.h>

#define BATCH_GRID_THREADS 256
#define TUNE_CANDIDATES 6
/* The candidates are timed round-robin, one per step, for TUNE_ROUNDS rounds: round 0
 * warms each one up (graph instantiation, first launch) and is not counted, so every
 * candidate is measured on a similar spread of the first steps' changing workload. */
#define TUNE_ROUNDS 3
#define B2G_BATCH_HALVES 2
#define SM_SHARED_BYTES ( 228u * 1024u ) /* shared memory of one SM */
/* dynamic shared memory one solver CTA may take: the 227 KB opt-in limit covers the
 * kernel's static shared memory too (the groups' items, up to 12.3 KB at 512 threads),
 * so leave room for it */
#define CTA_SHARED_MAX ( 214u * 1024u )
/* static shared memory of a solver CTA of T threads, with the 1 KB the system reserves */
#define SOLVE_STATIC_BYTES( T ) ( (size_t)( ( T ) / 32 ) * sizeof( b2gBatchItem ) + 1024u + 64u )

/* One half of a batched step's worlds: its own graphs, prefix sums, packs, queue and
 * timing events, so that the host phases of one half overlap the other's device work. */
struct BatchHalf
{
	int* hPrefix; /* scatter prefix [n+1], then narrowphase prefix [n+1] */
	int* dPrefix;
	int* hOrder; /* [0] = packs to solve, then PACK_INTS ints per pack; then scratch */
	int* dOrder;
	int* hScratch; /* 5 ints per item */
	int* dQueue;
	cudaEvent_t ev[4]; /* narrowphase start / end, solver start / end */

	cudaGraphExec_t collideExec;
	int collideFirst, collideN;
	cudaGraphExec_t solveExec[TUNE_CANDIDATES];
	int solveFirst[TUNE_CANDIDATES];
	int solveN[TUNE_CANDIDATES];
	int solveSmem[TUNE_CANDIDATES];
	int solvePerSm[TUNE_CANDIDATES]; /* resident CTAs per SM of each captured launch */
	int collideTimed, solveTimed;
};

struct b2gBatch
{
	cudaStream_t stream;
	int capacity;
	b2gBatchItem* hItems;
	b2gBatchItem* dItems;
	int* hCounters; /* 4 per item */
	int* dCounters;
	int sms;
	BatchHalf half[B2G_BATCH_HALVES];

	int tuned, choice, tuneStep;
	float tuneMs[TUNE_CANDIDATES];
	float collideMs, solveMs;
	int launches;
};


/* largest w with prefix[w] <= t, given prefix[0] <= t < prefix[n] */
__device__ __forceinline__ int find_world( const int* prefix, int n, int t )
{
	int lo = 0, hi = n;
	while ( hi - lo > 1 )
	{
		int mid = ( lo + hi ) >> 1;
		if ( prefix[mid] <= t )
			lo = mid;
		else
			hi = mid;
	}
	return lo;
}

__global__ void __launch_bounds__( BATCH_GRID_THREADS ) k_batch_scatter( const b2gBatchItem* items, const int* prefix, int n )
{
	int total = prefix[n];
	for ( int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x )
	{
		int w = find_world( prefix, n, t );
		const b2gDevWorld& W = items[w].W;
		scatter_contact( W, W.newContacts, t - prefix[w] );
	}
}

__global__ void __launch_bounds__( BATCH_GRID_THREADS, 4 ) k_batch_collide( const b2gBatchItem* items, const int* prefix, int n )
{
	int total = prefix[n];
	for ( int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x )
	{
		int w = find_world( prefix, n, t );
		collide_contact( items[w].W, t - prefix[w] );
	}
}

/* Adjoint tape records of the worlds that are recording (one CTA per world in turn). */
__global__ void __launch_bounds__( BATCH_GRID_THREADS ) k_batch_tape( const b2gBatchItem* items, int n )
{
	for ( int w = blockIdx.x; w < n; w += gridDim.x )
	{
		const b2gBatchItem& it = items[w];
		if ( it.tapeBodies == nullptr || it.solve == 0 )
			continue;
		int count = it.bodyIdCount > it.tapeRows ? it.bodyIdCount : it.tapeRows;
		for ( int t = threadIdx.x; t < count; t += blockDim.x )
			tape_record_one( it.W, (float4*)it.tapeBodies, it.bodyIdCount, (b2gTapeRow*)it.tapeRowDst, it.tapeRows, t );
	}
}

struct WorldImage
{
	SharedBodies B;
	SmemRows m;
};

/* Asks L2 for rows [first, first + n) of the world's row arrays: one bulk prefetch per
 * array, nothing to wait for. */
__device__ __forceinline__ void prefetch_rows( const b2gDevWorld& W, int first, int n )
{
	const void* arrays[B2G_ROW_FLOAT4] = { W.kIdx, W.kNF, W.kMass, W.kAnchor[0], W.kAnchor[1], W.kCoef[0], W.kCoef[1], W.kImp[0], W.kImp[1] };
	unsigned bytes = 16u * (unsigned)n;
	for ( int i = 0; i < B2G_ROW_FLOAT4; ++i )
	{
		const char* p = (const char*)arrays[i] + 16u * (size_t)first;
		asm volatile( "cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"( p ), "r"( bytes ) : "memory" );
	}
}

/* One row phase: the row in shared memory (ONCHIP) or in the world's row arrays. */
template <bool ONCHIP>
__device__ __forceinline__ void world_row( const b2gDevWorld& W, const WorldImage& s, int k, int phase, bool scalar,
										   const b2gStepConst& sc )
{
	if constexpr ( ONCHIP )
		row_step( s.m, s.B, k, phase, scalar, sc );
	else
		row_work( W, s.B, k, phase, scalar, sc );
}

/* The threads that solve one world: g consecutive threads of the CTA (a warp, a named-
 * barrier group of 64 or 128, or the whole CTA), group number gi, own index t. */
struct Group
{
	int g, gi, t;
};

/* Barrier of one group: every thread of the group reaches each of these at the same
 * point of its world's (group-uniform) control flow. */
template <int T>
__device__ __forceinline__ void group_sync( const Group& G )
{
	if ( G.g == 32 )
		__syncwarp();
	else if ( G.g == T )
		__syncthreads();
	else
		asm volatile( "bar.sync %0, %1;" ::"r"( G.gi + 1 ), "r"( G.g ) : "memory" );
}

/* One stage over all colours of one world (overflow first, serially), the group's
 * threads sharing each colour, a group barrier after each. */
template <int T, bool ONCHIP>
__device__ void world_stage( const b2gBatchItem& it, const WorldImage& s, const Group& G, int phase, const b2gStepConst& sc )
{
	const b2gDevWorld& W = it.W;
	const int* cs = it.colorStart;
	const int* js = it.jointStart;
	int ovRows = cs[B2G_COLORS] - cs[B2G_OVERFLOW];
	int ovJointsAll = js[B2G_COLORS] - js[B2G_OVERFLOW];
	bool overflow = phase == F_RESTITUTION ? ovRows > 0 : ovRows + ovJointsAll > 0;
	if ( overflow )
	{
		if ( G.t == 0 )
		{
			if ( phase != F_RESTITUTION )
				for ( int i = 0; i < ovJointsAll; ++i )
					joint_work( W, s.B, W.jointList[js[B2G_OVERFLOW] + i], phase, sc );
			for ( int i = 0; i < ovRows; ++i )
				world_row<ONCHIP>( W, s, cs[B2G_OVERFLOW] + i, phase, true, sc );
		}
		group_sync<T>( G );
	}
	if ( phase == F_WARM && sc.enableWarmStarting == 0 )
		return;
	for ( int a = 0; a < it.activeCount; ++a )
	{
		int c = it.active[a];
		int nr = cs[c + 1] - cs[c];
		int nj = phase == F_RESTITUTION ? 0 : js[c + 1] - js[c];
		if ( phase == F_RESTITUTION && nr == 0 )
			continue;
		if constexpr ( ONCHIP == false )
		{
			/* the colour after this one (the next stage starts again at the first) */
			if ( G.t == G.g - 1 )
			{
				int cn = it.active[a + 1 < it.activeCount ? a + 1 : 0];
				if ( cs[cn + 1] > cs[cn] )
					prefetch_rows( W, cs[cn], cs[cn + 1] - cs[cn] );
			}
		}
		for ( int t = G.t; t < nj + nr; t += G.g )
		{
			if ( t < nj )
				joint_work( W, s.B, W.jointList[js[c] + t], phase, sc );
			else
				world_row<ONCHIP>( W, s, cs[c] + t - nj, phase, false, sc );
		}
		group_sync<T>( G );
	}
}

/* The solver stage and finalisation of one world by one group (reference src/solver.c
 * stage order: prepare, substeps of integrate velocities / warm start / solve /
 * integrate positions / relax, restitution, store impulses, finalize bodies).  With
 * ONCHIP the rows are prepared straight into shared memory (reference
 * src/contact_solver.c:597-808) and only their impulses go back to the manifolds. */
template <int T, bool ONCHIP>
__device__ void solve_world( const b2gBatchItem& it, const b2gStepConst& sc, float4* sm, const Group& G )
{
	const b2gDevWorld& W = it.W;
	const int tid = G.t;
	const int step = G.g;
	const int N = it.bodyIdCount;
	const int rows = it.colorStart[B2G_COLORS];
	WorldImage s;
	s.B = SharedBodies{ sm, sm + N };
	float4* rb = sm + body_float4s( N );
	s.m.idx = (int4*)rb;
	s.m.nf = rb + rows;
	s.m.ms = rb + 2 * rows;
	s.m.anc0 = rb + 3 * rows;
	s.m.anc1 = rb + 4 * rows;
	s.m.coef0 = rb + 5 * rows;
	s.m.coef1 = rb + 6 * rows;
	s.m.imp0 = rb + 7 * rows;
	s.m.imp1 = rb + 8 * rows;
	float4* st0 = s.B.st0;
	float4* st1 = s.B.st1;
	float4* gst = (float4*)W.state;
	const float4* mass = (const float4*)W.mass;

	if ( tid == 0 )
	{
		W.counters[1] = 0;
		W.counters[3] = 0;
	}
	for ( int b = tid; b < N; b += step )
	{
		st0[b] = gst[2 * b];
		st1[b] = gst[2 * b + 1];
	}
	const int awake = it.awakeCount;
	if constexpr ( ONCHIP )
	{
		const float4 zero = make_float4( 0.0f, 0.0f, 0.0f, 0.0f );
		const float warm = sc.enableWarmStarting ? 1.0f : 0.0f;
		for ( int k = tid; k < rows; k += step )
		{
			int cid = W.solveList[k];
			int ia = W.cBodies[2 * cid];
			int ib = W.cBodies[2 * cid + 1];
			DevState sA = ia >= 0 ? state_of( gst[2 * ia], gst[2 * ia + 1] ) : identity_state();
			DevState sB = ib >= 0 ? state_of( gst[2 * ib], gst[2 * ib + 1] ) : identity_state();
			Row r;
			prepare_row( r, W.manifold + cid, ia, ib, ia >= 0 ? mass[ia] : zero, ib >= 0 ? mass[ib] : zero, sA, sB, W.cMix[2 * cid],
						 W.cMix[2 * cid + 1], ( ia < 0 || ib < 0 ) ? sc.staticSoft : sc.contactSoft, warm );
			store_row_smem( s.m, k, cid, r );
		}
	}
	else
	{
		for ( int k = tid; k < rows; k += step )
			prepare_contact_row( W, k, sc );
	}
	const int joints = it.jointStart[B2G_COLORS];
	for ( int t = tid; t < joints; t += step )
		prepare_joint( W, t, sc );
	group_sync<T>( G );

	for ( int sub = 0; sub < sc.subSteps; ++sub )
	{
		for ( int i = tid; i < awake; i += step )
		{
			int b = W.awake[i];
			DevState x = state_of( st0[b], st1[b] );
			VelocityTerms v = velocity_terms( mass[b], ( (const float4*)W.force )[b], ( (const float4*)W.extent )[b], sc );
			integrate_velocity( x, v, sc );
			st0[b] = velocity_word( x );
		}
		group_sync<T>( G );
		world_stage<T, ONCHIP>( it, s, G, F_WARM, sc );
		world_stage<T, ONCHIP>( it, s, G, F_SOLVE, sc );
		for ( int i = tid; i < awake; i += step )
		{
			int b = W.awake[i];
			DevState x = state_of( st0[b], st1[b] );
			integrate_position( x, sc.h );
			st1[b] = make_float4( x.dp.x, x.dp.y, x.dq.c, x.dq.s );
		}
		group_sync<T>( G );
		world_stage<T, ONCHIP>( it, s, G, F_RELAX, sc );
	}
	world_stage<T, ONCHIP>( it, s, G, F_RESTITUTION, sc );

	if constexpr ( ONCHIP )
	{
		/* colour rows store both point slots, overflow rows their points (as store_row) */
		const int ov = it.colorStart[B2G_OVERFLOW];
		for ( int k = tid; k < rows; k += step )
		{
			int4 idx = s.m.idx[k];
			b2gManifold* mf = W.manifold + idx.z;
			int n = k < ov ? 2 : idx.w;
			float4 imp[2] = { s.m.imp0[k], s.m.imp1[k] };
			float4 coef[2] = { s.m.coef0[k], s.m.coef1[k] };
			for ( int j = 0; j < n; ++j )
			{
				mf->pts[j].normalImpulse = imp[j].x;
				mf->pts[j].tangentImpulse = imp[j].y;
				mf->pts[j].maxNormalImpulse = imp[j].z;
				mf->pts[j].normalVelocity = coef[j].w;
			}
		}
	}
	else
	{
		for ( int k = tid; k < rows; k += step )
			store_row( W, k, it.colorStart[B2G_OVERFLOW] );
	}
	for ( int i = tid; i < awake; i += step )
	{
		int b = W.awake[i];
		gst[2 * b] = st0[b];
		gst[2 * b + 1] = st1[b];
	}
	group_sync<T>( G );
	for ( int i = tid; i < awake; i += step )
		finalize_body( W, i, sc );
}


/* Persistent: each CTA takes the next pack from the queue (packs[0] packs, then
 * PACK_INTS ints each: group size, item indices or -1). */
template <int T, int MINB>
__global__ void __launch_bounds__( T, MINB ) k_batch_solve( const b2gBatchItem* items, const int* packs, int* queue, int smemFloat4 )
{
	extern __shared__ float4 sm[];
	__shared__ int s_next;
	/* each group's item in shared memory: its counts, colour offsets and array pointers
	 * are read again after every group barrier */
	__shared__ b2gBatchItem s_it[T / 32];
	const int m = packs[0];
	for ( ;; )
	{
		if ( threadIdx.x == 0 )
			s_next = atomicAdd( queue, 1 );
		__syncthreads();
		int q = s_next;
		if ( q >= m )
			break;
		const int* p = packs + 1 + PACK_INTS * q;
		Group G;
		G.g = p[0];
		G.gi = threadIdx.x / G.g;
		G.t = threadIdx.x - G.gi * G.g;
		int w = G.gi < PACK_WORLDS ? p[1 + G.gi] : -1;
		if ( w >= 0 )
		{
			b2gBatchItem& it = s_it[G.gi];
			for ( int i = G.t; i < (int)( sizeof( b2gBatchItem ) / 4 ); i += G.g )
				( (int*)&it )[i] = ( (const int*)( items + w ) )[i];
			group_sync<T>( G );
			float4* region = sm + ( smemFloat4 / ( T / G.g ) ) * G.gi;
			if ( it.rowsOnChip )
				solve_world<T, true>( it, it.sc, region, G );
			else
				solve_world<T, false>( it, it.sc, region, G );
		}
		__syncthreads();
	}
}

static_assert( PACK_WORLDS * 32 >= 512, "a pack holds a world for every warp of the largest CTA" );

/* ------------------------------------------------------------------ host side */
template <int T, int MINB>
static int solve_occupancy( size_t smem )
{
	int blocks = 0;
	/* the default carve-out: the L1 left beside shared memory caches the row arrays of
	 * the worlds whose rows stay in global memory (a maximal shared carve-out measured
	 * 20% slower) */
	cudaFuncSetAttribute( k_batch_solve<T, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem );
	if ( cudaOccupancyMaxActiveBlocksPerMultiprocessor( &blocks, k_batch_solve<T, MINB>, T, smem ) != cudaSuccess )
		return 0;
	return blocks;
}

template <int T, int MINB>
static void launch_solve( b2gBatch* b, int grid, size_t smem, const int* packs, int* queue )
{
	k_batch_solve<T, MINB><<<grid, T, smem, b->stream>>>( b->dItems, packs, queue, (int)( smem / 16u ) );
}

/* Solver launch shapes tried on the first steps: threads per CTA and CTAs per SM (which
 * also caps the registers per thread and sets the shared memory per world). */
struct TuneCandidate
{
	int threads, perSM;
	int ( *occupancy )( size_t smem );
	void ( *launch )( b2gBatch* b, int grid, size_t smem, const int* packs, int* queue );
};
#define TUNE_SHAPE( T, B ) { T, B, solve_occupancy<T, B>, launch_solve<T, B> }
static const TuneCandidate s_tune[TUNE_CANDIDATES] = { TUNE_SHAPE( 128, 6 ), TUNE_SHAPE( 512, 1 ), TUNE_SHAPE( 128, 8 ),
													   TUNE_SHAPE( 512, 2 ), TUNE_SHAPE( 256, 3 ), TUNE_SHAPE( 128, 4 ) };
#undef TUNE_SHAPE

extern "C" b2gBatch* b2gd_batch_create( void )
{
	b2gBatch* b = (b2gBatch*)b2g_calloc( 1, sizeof( b2gBatch ) );
	if ( b == nullptr )
		return nullptr;
	if ( cudaStreamCreateWithFlags( &b->stream, cudaStreamNonBlocking ) != cudaSuccess )
	{
		b2g_free( b );
		return nullptr;
	}
	int dev = 0;
	cudaGetDevice( &dev );
	cudaDeviceGetAttribute( &b->sms, cudaDevAttrMultiProcessorCount, dev );
	for ( int h = 0; h < B2G_BATCH_HALVES; ++h )
	{
		for ( int i = 0; i < 4; ++i )
			cudaEventCreate( &b->half[h].ev[i] );
		cudaMalloc( &b->half[h].dQueue, sizeof( int ) );
	}
	return b;
}

static void release_graphs( b2gBatch* b )
{
	for ( int h = 0; h < B2G_BATCH_HALVES; ++h )
	{
		BatchHalf& H = b->half[h];
		if ( H.collideExec )
			cudaGraphExecDestroy( H.collideExec );
		H.collideExec = nullptr;
		for ( int i = 0; i < TUNE_CANDIDATES; ++i )
		{
			if ( H.solveExec[i] )
				cudaGraphExecDestroy( H.solveExec[i] );
			H.solveExec[i] = nullptr;
		}
	}
}

static void release_buffers( b2gBatch* b )
{
	cudaFreeHost( b->hItems );
	cudaFreeHost( b->hCounters );
	cudaFree( b->dItems );
	cudaFree( b->dCounters );
	b->hItems = b->dItems = nullptr;
	b->hCounters = b->dCounters = nullptr;
	for ( int h = 0; h < B2G_BATCH_HALVES; ++h )
	{
		BatchHalf& H = b->half[h];
		cudaFreeHost( H.hPrefix );
		cudaFreeHost( H.hOrder );
		cudaFreeHost( H.hScratch );
		cudaFree( H.dPrefix );
		cudaFree( H.dOrder );
		H.hPrefix = H.dPrefix = H.hOrder = H.dOrder = H.hScratch = nullptr;
	}
	b->capacity = 0;
}

extern "C" void b2gd_batch_destroy( b2gBatch* b )
{
	if ( b == nullptr )
		return;
	cudaStreamSynchronize( b->stream );
	release_graphs( b );
	release_buffers( b );
	for ( int h = 0; h < B2G_BATCH_HALVES; ++h )
	{
		cudaFree( b->half[h].dQueue );
		for ( int i = 0; i < 4; ++i )
			cudaEventDestroy( b->half[h].ev[i] );
	}
	cudaStreamDestroy( b->stream );
	b2g_free( b );
}

extern "C" b2gBatchItem* b2gd_batch_items( b2gBatch* b, int count )
{
	if ( count <= b->capacity )
		return b->hItems;
	cudaStreamSynchronize( b->stream );
	release_graphs( b );
	release_buffers( b );
	int cap = count < 64 ? 64 : count;
	size_t ints = (size_t)cap + 1;
	bool ok = cudaMallocHost( &b->hItems, sizeof( b2gBatchItem ) * cap ) == cudaSuccess &&
			  cudaMallocHost( &b->hCounters, sizeof( int ) * 4 * cap ) == cudaSuccess &&
			  cudaMalloc( &b->dItems, sizeof( b2gBatchItem ) * cap ) == cudaSuccess &&
			  cudaMalloc( &b->dCounters, sizeof( int ) * 4 * cap ) == cudaSuccess;
	for ( int h = 0; h < B2G_BATCH_HALVES && ok; ++h )
	{
		BatchHalf& H = b->half[h];
		ok = cudaMallocHost( &H.hPrefix, sizeof( int ) * 2 * ints ) == cudaSuccess &&
			 cudaMallocHost( &H.hOrder, sizeof( int ) * ( 1u + 2u * PACK_INTS * ints ) ) == cudaSuccess && /* packs + scratch */
			 cudaMallocHost( &H.hScratch, sizeof( int ) * 5u * ints ) == cudaSuccess &&
			 cudaMalloc( &H.dPrefix, sizeof( int ) * 2 * ints ) == cudaSuccess &&
			 cudaMalloc( &H.dOrder, sizeof( int ) * ( 1u + PACK_INTS * ints ) ) == cudaSuccess;
	}
	if ( ok == false )
	{
		release_buffers( b );
		return nullptr;
	}
	memset( b->hCounters, 0, sizeof( int ) * 4 * cap );
	b->capacity = cap;
	return b->hItems;
}

extern "C" void* b2gd_batch_stream( b2gBatch* b ) { return (void*)b->stream; }

/* Largest body-id count the batched solver holds (bodies in shared memory, 32 bytes each,
 * rounded up to 256 ids). */
extern "C" int b2gd_batch_max_bodies( void ) { return (int)( CTA_SHARED_MAX / 32u / 256u * 256u ); }

extern "C" const int* b2gd_batch_counters( b2gBatch* b, int i ) { return b->hCounters + 4 * i; }

extern "C" int b2gd_stage_contacts( b2gDevWorld* w, b2gHostIO* io, int count )
{
	if ( count <= 0 )
		return 0;
	return (int)cudaMemcpyAsync( w->newContacts, io->newContacts, sizeof( b2gContactInit ) * (size_t)count,
								 cudaMemcpyHostToDevice, (cudaStream_t)w->stream );
}

static void point_counters( b2gBatch* b, int first, int count )
{
	for ( int i = first; i < first + count; ++i )
		b->hItems[i].W.counters = b->dCounters + 4 * i;
}

/* Ends a capture; on a failed launch or capture nothing is instantiated. */
static cudaError_t finish_capture( cudaStream_t s, cudaError_t launch, cudaGraphExec_t* exec )
{
	cudaGraph_t g = nullptr;
	cudaError_t e = cudaStreamEndCapture( s, &g );
	if ( launch != cudaSuccess || e != cudaSuccess )
	{
		if ( g )
			cudaGraphDestroy( g );
		return launch != cudaSuccess ? launch : e;
	}
	e = cudaGraphInstantiate( exec, g, 0 );
	cudaGraphDestroy( g );
	return e;
}

extern "C" void b2gd_batch_begin_step( b2gBatch* b )
{
	b->choice = b->tuned ? b->choice : b->tuneStep % TUNE_CANDIDATES;
	b->launches = 0;
	for ( int h = 0; h < B2G_BATCH_HALVES; ++h )
		b->half[h].collideTimed = b->half[h].solveTimed = 0;
}

extern "C" int b2gd_batch_collide( b2gBatch* b, int h, int first, int n )
{
	if ( n <= 0 )
		return 0;
	BatchHalf& H = b->half[h];
	point_counters( b, first, n );
	int* ps = H.hPrefix;
	int* pc = H.hPrefix + n + 1;
	ps[0] = 0;
	pc[0] = 0;
	for ( int i = 0; i < n; ++i )
	{
		ps[i + 1] = ps[i] + b->hItems[first + i].staged;
		pc[i + 1] = pc[i] + b->hItems[first + i].idCount;
	}
	if ( H.collideExec == nullptr || H.collideN != n || H.collideFirst != first )
	{
		if ( H.collideExec )
			cudaGraphExecDestroy( H.collideExec );
		H.collideExec = nullptr;
		int grid = b->sms * 8;
		const b2gBatchItem* items = b->dItems + first;
		cudaGetLastError();
		cudaStreamBeginCapture( b->stream, cudaStreamCaptureModeThreadLocal );
		cudaMemcpyAsync( b->dItems + first, b->hItems + first, sizeof( b2gBatchItem ) * n, cudaMemcpyHostToDevice, b->stream );
		cudaMemcpyAsync( H.dPrefix, H.hPrefix, sizeof( int ) * 2 * ( n + 1 ), cudaMemcpyHostToDevice, b->stream );
		cudaMemsetAsync( b->dCounters + 4 * first, 0, sizeof( int ) * 4 * n, b->stream );
		k_batch_scatter<<<grid, BATCH_GRID_THREADS, 0, b->stream>>>( items, H.dPrefix, n );
		k_batch_collide<<<grid, BATCH_GRID_THREADS, 0, b->stream>>>( items, H.dPrefix + n + 1, n );
		cudaError_t launch = cudaGetLastError();
		cudaMemcpyAsync( b->hCounters + 4 * first, b->dCounters + 4 * first, sizeof( int ) * 4 * n, cudaMemcpyDeviceToHost, b->stream );
		cudaError_t e = finish_capture( b->stream, launch, &H.collideExec );
		if ( e != cudaSuccess )
			return (int)e;
		H.collideN = n;
		H.collideFirst = first;
	}
	cudaEventRecord( H.ev[0], b->stream );
	cudaError_t e = cudaGraphLaunch( H.collideExec, b->stream );
	cudaEventRecord( H.ev[1], b->stream );
	H.collideTimed = 1;
	b->launches += 2;
	return (int)e;
}

extern "C" int b2gd_batch_solve( b2gBatch* b, int h, int first, int n )
{
	if ( n <= 0 )
		return 0;
	BatchHalf& H = b->half[h];
	point_counters( b, first, n );
	const int choice = b->choice;
	const TuneCandidate tc = s_tune[choice];
	/* shared memory per CTA: the candidate's share of the SM (less the per-CTA
	 * reservation), or more when the largest world needs it for its bodies (rounded up
	 * to 256 body ids so that growing worlds rarely recapture) */
	size_t target = ( SM_SHARED_BYTES / (size_t)tc.perSM - SOLVE_STATIC_BYTES( tc.threads ) ) / 256u * 256u;
	target = target < CTA_SHARED_MAX ? target : CTA_SHARED_MAX;
	int top = 0;
	for ( int i = first; i < first + n; ++i )
		if ( b->hItems[i].solve )
			top = b->hItems[i].bodyIdCount > top ? b->hItems[i].bodyIdCount : top;
	size_t smem = 16u * (size_t)body_float4s( ( top + 255 ) / 256 * 256 );
	smem = smem > target ? smem : target;
	if ( smem > CTA_SHARED_MAX )
		return (int)cudaErrorInvalidValue;
	b2g_build_packs( b->hItems, first, n, tc.threads, smem, H.hScratch, H.hOrder );

	if ( H.solveExec[choice] == nullptr || H.solveN[choice] != n || H.solveFirst[choice] != first || H.solveSmem[choice] != (int)smem )
	{
		if ( H.solveExec[choice] )
			cudaGraphExecDestroy( H.solveExec[choice] );
		H.solveExec[choice] = nullptr;
		int occ = tc.occupancy( smem );
		if ( occ <= 0 )
			return (int)cudaErrorInvalidConfiguration;
		occ = occ < tc.perSM ? occ : tc.perSM;
		H.solvePerSm[choice] = occ;
		int grid = b->sms * occ;
		cudaGetLastError();
		cudaStreamBeginCapture( b->stream, cudaStreamCaptureModeThreadLocal );
		cudaMemcpyAsync( b->dItems + first, b->hItems + first, sizeof( b2gBatchItem ) * n, cudaMemcpyHostToDevice, b->stream );
		cudaMemcpyAsync( H.dOrder, H.hOrder, sizeof( int ) * ( 1 + PACK_INTS * (size_t)n ), cudaMemcpyHostToDevice, b->stream );
		cudaMemsetAsync( H.dQueue, 0, sizeof( int ), b->stream );
		k_batch_tape<<<b->sms * 4, BATCH_GRID_THREADS, 0, b->stream>>>( b->dItems + first, n );
		tc.launch( b, grid, smem, H.dOrder, H.dQueue );
		cudaError_t launch = cudaGetLastError();
		cudaMemcpyAsync( b->hCounters + 4 * first, b->dCounters + 4 * first, sizeof( int ) * 4 * n, cudaMemcpyDeviceToHost, b->stream );
		cudaError_t e = finish_capture( b->stream, launch, &H.solveExec[choice] );
		if ( e != cudaSuccess )
			return (int)e;
		H.solveN[choice] = n;
		H.solveFirst[choice] = first;
		H.solveSmem[choice] = (int)smem;
	}
	cudaEventRecord( H.ev[2], b->stream );
	cudaError_t e = cudaGraphLaunch( H.solveExec[choice], b->stream );
	cudaEventRecord( H.ev[3], b->stream );
	H.solveTimed = 1;
	b->launches += 2; /* tape records, solver */
	return (int)e;
}

extern "C" int b2gd_batch_wait_collide( b2gBatch* b, int h )
{
	if ( b->half[h].collideTimed == 0 )
		return 0;
	return (int)cudaEventSynchronize( b->half[h].ev[1] );
}

extern "C" int b2gd_batch_wait_solve( b2gBatch* b, int h )
{
	if ( b->half[h].solveTimed == 0 )
		return 0;
	return (int)cudaEventSynchronize( b->half[h].ev[3] );
}

extern "C" int b2gd_batch_end_step( b2gBatch* b )
{
	cudaError_t e = cudaStreamSynchronize( b->stream );
	if ( e != cudaSuccess )
		return (int)e;
	float collide = 0.0f, solve = 0.0f;
	int solved = 0;
	for ( int h = 0; h < B2G_BATCH_HALVES; ++h )
	{
		BatchHalf& H = b->half[h];
		float ms = 0.0f;
		if ( H.collideTimed && cudaEventElapsedTime( &ms, H.ev[0], H.ev[1] ) == cudaSuccess )
			collide += ms;
		if ( H.solveTimed && cudaEventElapsedTime( &ms, H.ev[2], H.ev[3] ) == cudaSuccess )
		{
			solve += ms;
			solved = 1;
		}
	}
	b->collideMs = collide;
	b->solveMs = solve;
	if ( solved && b->tuned == 0 )
	{
		if ( b->tuneStep >= TUNE_CANDIDATES )
			b->tuneMs[b->choice] += solve;
		b->tuneStep += 1;
		if ( b->tuneStep == TUNE_ROUNDS * TUNE_CANDIDATES )
		{
			int best = 0;
			for ( int i = 1; i < TUNE_CANDIDATES; ++i )
				best = b->tuneMs[i] < b->tuneMs[best] ? i : best;
			b->choice = best;
			b->tuned = 1;
			for ( int h = 0; h < B2G_BATCH_HALVES; ++h )
			{
				for ( int i = 0; i < TUNE_CANDIDATES; ++i )
				{
					if ( i != best && b->half[h].solveExec[i] )
					{
						cudaGraphExecDestroy( b->half[h].solveExec[i] );
						b->half[h].solveExec[i] = nullptr;
					}
				}
			}
		}
	}
	return (int)cudaGetLastError();
}

extern "C" void b2gd_batch_stats( b2gBatch* b, float* collideMs, float* solveMs, int* threads, int* ctasPerSm, int* launches )
{
	*collideMs = b->collideMs;
	*solveMs = b->solveMs;
	*threads = b->tuned ? s_tune[b->choice].threads : 0;
	*ctasPerSm = b->tuned ? b->half[0].solvePerSm[b->choice] : 0;
	*launches = b->launches;
}
