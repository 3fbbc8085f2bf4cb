/*
 * kernels.cu -- sm_103a kernels of the per-step contact pipeline and their launch
 * sequences.
 *
 * Stage                reference                                  kernel
 * contact creation     src/contact.c:185-332 (sim part)           k_scatter_contacts
 * narrowphase          src/world.c:290-365, src/contact.c:493-582 k_collide
 * prepare contacts     src/contact_solver.c:21-147, :597-808       k_prepare
 * prepare joints       src/joint.c:983-1018 (b2g_joints.h)        k_prepare_joints
 * integrate velocities src/solver.c:34-93                          k_integrate_velocities
 * warm start / solve / relax / restitution
 *                      src/contact_solver.c:149-440 (overflow)     k_overflow (serial)
 *                      src/contact_solver.c:810-1178 (8-lane)      k_color (one colour)
 *                      src/joint.c:1028-1108 (b2g_joints.h)       (joints inside both)
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
#include "b2g_stages.h"

#include <cuda_runtime.h>

#include <stdio.h>

#define BLOCK 128

/* ------------------------------------------------------------------ single-world kernels */
__global__ void k_scatter_contacts( b2gDevWorld W, const b2gContactInit* inits, int n )
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if ( t < n )
		scatter_contact( W, inits, t );
}

__global__ void k_body_ops( b2gDevWorld W, const int* ops, int n )
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if ( t < n )
		apply_body_op( W, ops[t] );
}

__global__ void __launch_bounds__( BLOCK ) k_collide( b2gDevWorld W, int idCount )
{
	int id = blockIdx.x * blockDim.x + threadIdx.x;
	if ( id < idCount )
		collide_contact( W, id );
}

__global__ void __launch_bounds__( BLOCK ) k_prepare( b2gDevWorld W, int total, b2gStepConst sc )
{
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if ( k < total )
		prepare_contact_row( W, k, sc );
}

__global__ void k_prepare_joints( b2gDevWorld W, int count, b2gStepConst sc )
{
	if ( W.guardEvents && W.counters[0] != 0 )
		return;
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if ( t < count )
		prepare_joint( W, t, sc );
}

__global__ void __launch_bounds__( BLOCK ) k_integrate_velocities( b2gDevWorld W, int awakeCount, b2gStepConst sc )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < awakeCount )
		integrate_body_velocity( W, i, sc );
}

__global__ void __launch_bounds__( BLOCK ) k_integrate_positions( b2gDevWorld W, int awakeCount, b2gStepConst sc )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < awakeCount )
		integrate_body_position( W, i, sc );
}

__global__ void __launch_bounds__( BLOCK ) k_store( b2gDevWorld W, int total, int overflowStart )
{
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if ( k < total )
		store_row( W, k, overflowStart );
}

__global__ void __launch_bounds__( BLOCK ) k_finalize( b2gDevWorld W, int awakeCount, b2gStepConst sc )
{
	if ( W.guardEvents && W.counters[0] != 0 )
		return;
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < awakeCount )
		finalize_body( W, i, sc );
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
		w->h2dBytes += (long long)( sizeof( b2gContactInit ) * (size_t)newCount );
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
	w->d2hBytes += 4 * sizeof( int );
	return check( cudaGetLastError() );
}

/* Applies staged body operations (one per body) on the world's stream, ahead of every
 * later copy or kernel that reads the bodies. */
extern "C" int b2gd_body_ops( b2gDevWorld* w, const int* ops, int count )
{
	if ( count <= 0 )
		return 0;
	cudaStream_t s = (cudaStream_t)w->stream;
	int e = b2gd_reserve_body_ops( w, count );
	if ( e )
		return e;
	cudaMemcpyAsync( w->bodyOps, ops, sizeof( int ) * (size_t)count, cudaMemcpyHostToDevice, s );
	w->h2dBytes += (long long)( sizeof( int ) * (size_t)count );
	k_body_ops<<<blocks_for( count ), BLOCK, 0, s>>>( *w, w->bodyOps, count );
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
	cudaMemsetAsync( w->counters + 3, 0, sizeof( int ), s );
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
	w->d2hBytes += 4 * sizeof( int );
	return check( cudaGetLastError() );
}

/* The fused solver stage and finalisation launched right behind the narrowphase, before
 * the host has read its events: with no event the colouring and solve lists are the
 * ones the host would use, and the step needs no synchronisation in between; with an
 * event every kernel returns at once and the host solves again after processing them.
 * Returns 1 when launched, 0 when the world does not fit the fused solver (nothing
 * launched), or -1 on a launch error. */
extern "C" int b2gd_solve_speculative( b2gDevWorld* w, b2gHostIO* io, const b2gSolvePlan* plan, const b2gStepConst* scp )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int awake = plan->awakeCount;
	if ( w->fused == 0 || awake <= 0 )
		return 0;
	w->guardEvents = 1;
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[3], s );
	cudaMemsetAsync( w->counters + 1, 0, sizeof( int ), s );
	cudaMemsetAsync( w->counters + 3, 0, sizeof( int ), s );
	int fused = b2gd_solver_fused( w, plan, scp );
	if ( fused <= 0 )
	{
		w->guardEvents = 0;
		return fused < 0 ? -1 : 0;
	}
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[4], s );
	k_finalize<<<blocks_for( awake ), BLOCK, 0, s>>>( *w, awake, *scp );
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[5], s );
	cudaMemcpyAsync( io->counters, w->counters, 4 * sizeof( int ), cudaMemcpyDeviceToHost, s );
	w->d2hBytes += 4 * sizeof( int );
	w->guardEvents = 0;
	w->fusedUsed = 1;
	w->launches += fused + 1;
	return cudaGetLastError() == cudaSuccess ? 1 : -1;
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
	uint32_t cache = W.cCache[id]; /* a copy: the contact's own cache stays as it was */
	narrowphase( &m, gA, xfA, gB, xfB, &cache );
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
