/*
 * arena.cu -- device memory of one world: allocation, growth, host<->device copies and
 * the mapped pinned buffers through which the narrowphase and the finalisation kernel
 * hand their (rare) events to the host without an extra copy.
 *
 * Every array grows geometrically and keeps its contents; growth only happens while
 * the host adds bodies, shapes or contacts, never inside a kernel sequence.
 */
#include "b2g_device.h"

#include <cuda_runtime.h>

#include <stdlib.h>
#include <string.h>

static cudaError_t s_err = cudaSuccess;

static int ok( cudaError_t e )
{
	if ( e != cudaSuccess )
	{
		s_err = e;
		return (int)e;
	}
	return 0;
}

extern "C" int b2gd_device_ok( void )
{
	int n = 0;
	if ( cudaGetDeviceCount( &n ) != cudaSuccess )
		return 0;
	return n > 0;
}

/* Reallocates a device array from oldBytes to newBytes keeping the prefix.  Stream
 * ordered (the device's default memory pool): no host synchronisation, so growing the
 * arenas of many worlds in one batched step does not serialise on the host. */
static int grow( void** ptr, size_t oldBytes, size_t newBytes, cudaStream_t s )
{
	if ( newBytes <= oldBytes && *ptr != nullptr )
		return 0;
	void* p = nullptr;
	int e = ok( cudaMallocAsync( &p, newBytes, s ) );
	if ( e )
		return e;
	cudaMemsetAsync( p, 0, newBytes, s );
	if ( *ptr != nullptr )
	{
		if ( oldBytes > 0 )
			cudaMemcpyAsync( p, *ptr, oldBytes, cudaMemcpyDeviceToDevice, s );
		cudaFreeAsync( *ptr, s );
	}
	*ptr = p;
	return 0;
}

static int grow_host_mapped( void** hptr, void** dptr, size_t bytes )
{
	if ( *hptr )
		cudaFreeHost( *hptr );
	*hptr = nullptr;
	*dptr = nullptr;
	int e = ok( cudaHostAlloc( hptr, bytes, cudaHostAllocMapped ) );
	if ( e )
		return e;
	memset( *hptr, 0, bytes );
	return ok( cudaHostGetDevicePointer( dptr, *hptr, 0 ) );
}

extern "C" int b2gd_init( b2gDevWorld* w, b2gHostIO* io )
{
	memset( w, 0, sizeof( *w ) );
	memset( io, 0, sizeof( *io ) );
	cudaStream_t s;
	int e = ok( cudaStreamCreateWithFlags( &s, cudaStreamNonBlocking ) );
	if ( e )
		return e;
	w->stream = (void*)s;
	w->fused = 1;
	e = ok( cudaMallocAsync( (void**)&w->counters, 4 * sizeof( int ), s ) );
	if ( e )
		return e;
	e = ok( cudaHostAlloc( (void**)&io->counters, 4 * sizeof( int ), cudaHostAllocDefault ) );
	if ( e )
		return e;
	memset( io->counters, 0, 4 * sizeof( int ) );
	e = ok( cudaMemsetAsync( w->counters, 0, 4 * sizeof( int ), s ) );
	if ( e )
		return e;
	/* room for small worlds from the start, so that their first steps allocate nothing */
	return b2gd_reserve( w, io, 32, 32, 128, 4, 128, 32 );
}

#define FREE_DEV( p )                                                                                                            \
	do                                                                                                                           \
	{                                                                                                                            \
		if ( p )                                                                                                                 \
			cudaFreeAsync( (void*)( p ), (cudaStream_t)w->stream );                                                              \
		p = nullptr;                                                                                                             \
	}                                                                                                                            \
	while ( 0 )

extern "C" void b2gd_free( b2gDevWorld* w, b2gHostIO* io )
{
	if ( w->stream )
		cudaStreamSynchronize( (cudaStream_t)w->stream );
	FREE_DEV( w->state );
	FREE_DEV( w->xf );
	FREE_DEV( w->centers );
	FREE_DEV( w->prev );
	FREE_DEV( w->mass );
	FREE_DEV( w->force );
	FREE_DEV( w->extent );
	FREE_DEV( w->bodyInfo );
	FREE_DEV( w->sleepTime );
	FREE_DEV( w->bodyOps );
	FREE_DEV( w->awake );
	FREE_DEV( w->shapeRange );
	FREE_DEV( w->shapeList );
	FREE_DEV( w->geo );
	FREE_DEV( w->aabb );
	FREE_DEV( w->fat );
	FREE_DEV( w->cShapes );
	FREE_DEV( w->cMix );
	FREE_DEV( w->cFlags );
	FREE_DEV( w->cCache );
	FREE_DEV( w->cBodies );
	FREE_DEV( w->manifold );
	FREE_DEV( w->solveList );
	FREE_DEV( w->jointList );
	FREE_DEV( w->kIdx );
	FREE_DEV( w->kNF );
	FREE_DEV( w->kMass );
	for ( int j = 0; j < 2; ++j )
	{
		FREE_DEV( w->kAnchor[j] );
		FREE_DEV( w->kCoef[j] );
		FREE_DEV( w->kImp[j] );
	}
	FREE_DEV( w->joints );
	FREE_DEV( w->newContacts );
	FREE_DEV( w->counters );
	for ( int i = 0; i < 8; ++i )
		if ( w->timers[i] )
			cudaEventDestroy( (cudaEvent_t)w->timers[i] );
	if ( io->events )
		cudaFreeHost( io->events );
	if ( io->records )
		cudaFreeHost( io->records );
	if ( io->sleepy )
		cudaFreeHost( io->sleepy );
	if ( io->counters )
		cudaFreeHost( io->counters );
	if ( io->newContacts )
		cudaFreeHost( io->newContacts );
	if ( io->hitIds )
		cudaFreeHost( io->hitIds );
	if ( io->hitOut )
		cudaFreeHost( io->hitOut );
	if ( w->stage )
		cudaFree( w->stage );
	if ( w->stream )
		cudaStreamDestroy( (cudaStream_t)w->stream );
	memset( w, 0, sizeof( *w ) );
	memset( io, 0, sizeof( *io ) );
}

static int next_cap( int have, int need )
{
	if ( need <= have )
		return have;
	int c = have < 64 ? 64 : have;
	while ( c < need )
		c *= 2;
	return c;
}

extern "C" int b2gd_reserve( b2gDevWorld* w, b2gHostIO* io, int bodyCap, int shapeCap, int contactCap, int jointCap, int solveCap,
							 int listCap )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int e = 0;
	if ( bodyCap <= w->bodyCap && shapeCap <= w->shapeCap && contactCap <= w->contactCap && solveCap <= w->solveCap &&
		 jointCap <= w->jointCap )
		return 0;
	if ( bodyCap > w->bodyCap )
	{
		int nc = next_cap( w->bodyCap, bodyCap );
		size_t o4 = 16u * (size_t)w->bodyCap, n4 = 16u * (size_t)nc;
		e |= grow( &w->state, 2 * o4, 2 * n4, s );
		e |= grow( &w->xf, o4, n4, s );
		e |= grow( &w->centers, o4, n4, s );
		e |= grow( &w->prev, o4, n4, s );
		e |= grow( &w->mass, o4, n4, s );
		e |= grow( &w->force, o4, n4, s );
		e |= grow( &w->extent, o4, n4, s );
		e |= grow( (void**)&w->bodyInfo, 4u * (size_t)w->bodyCap, 4u * (size_t)nc, s );
		/* sleep timers only in worlds that have had sleep on (b2gd_reserve_sleep) */
		if ( w->sleepTime != nullptr )
			e |= grow( (void**)&w->sleepTime, 4u * (size_t)w->bodyCap, 4u * (size_t)nc, s );
		e |= grow( (void**)&w->awake, 4u * (size_t)w->bodyCap, 4u * (size_t)nc, s );
		e |= grow( (void**)&w->shapeRange, 8u * (size_t)w->bodyCap, 8u * (size_t)nc, s );
		w->bodyCap = nc;
	}
	if ( shapeCap > w->shapeCap )
	{
		int nc = next_cap( w->shapeCap, shapeCap );
		e |= grow( (void**)&w->geo, sizeof( b2gShapeGeo ) * (size_t)w->shapeCap, sizeof( b2gShapeGeo ) * (size_t)nc, s );
		e |= grow( &w->aabb, 16u * (size_t)w->shapeCap, 16u * (size_t)nc, s );
		e |= grow( &w->fat, 16u * (size_t)w->shapeCap, 16u * (size_t)nc, s );
		e |= grow( (void**)&w->shapeList, 4u * (size_t)w->shapeCap, 4u * (size_t)nc, s );
		/* two records at most per shape and step */
		e |= grow_host_mapped( (void**)&io->records, (void**)&w->records, sizeof( b2gRecord ) * 2u * (size_t)nc );
		w->recordCap = 2 * nc;
		w->shapeCap = nc;
	}
	if ( contactCap > w->contactCap )
	{
		int nc = next_cap( w->contactCap, contactCap );
		size_t o = (size_t)w->contactCap, n = (size_t)nc;
		e |= grow( (void**)&w->cShapes, 8u * o, 8u * n, s );
		e |= grow( (void**)&w->cMix, 8u * o, 8u * n, s );
		e |= grow( (void**)&w->cFlags, 4u * o, 4u * n, s );
		e |= grow( (void**)&w->cCache, 4u * o, 4u * n, s );
		e |= grow( (void**)&w->cBodies, 8u * o, 8u * n, s );
		e |= grow( (void**)&w->manifold, sizeof( b2gManifold ) * o, sizeof( b2gManifold ) * n, s );
		e |= grow_host_mapped( (void**)&io->events, (void**)&w->events, 4u * n );
		w->eventCap = nc;
		/* new contacts per step are bounded by the contact capacity */
		if ( io->newContacts )
			cudaFreeHost( io->newContacts );
		e |= ok( cudaHostAlloc( (void**)&io->newContacts, sizeof( b2gContactInit ) * n, cudaHostAllocDefault ) );
		e |= grow( (void**)&w->newContacts, sizeof( b2gContactInit ) * o, sizeof( b2gContactInit ) * n, s );
		w->newCap = nc;
		w->contactCap = nc;
	}
	if ( solveCap > w->solveCap )
	{
		int nc = next_cap( w->solveCap, solveCap );
		size_t o = (size_t)w->solveCap, n = (size_t)nc;
		e |= grow( (void**)&w->solveList, 4u * o, 4u * n, s );
		e |= grow( &w->kIdx, 16u * o, 16u * n, s );
		e |= grow( &w->kNF, 16u * o, 16u * n, s );
		e |= grow( &w->kMass, 16u * o, 16u * n, s );
		for ( int j = 0; j < 2; ++j )
		{
			e |= grow( &w->kAnchor[j], 16u * o, 16u * n, s );
			e |= grow( &w->kCoef[j], 16u * o, 16u * n, s );
			e |= grow( &w->kImp[j], 16u * o, 16u * n, s );
		}
		w->solveCap = nc;
	}
	if ( jointCap > w->jointCap )
	{
		int nc = next_cap( w->jointCap, jointCap );
		e |= grow( (void**)&w->joints, sizeof( b2gJointDev ) * (size_t)w->jointCap, sizeof( b2gJointDev ) * (size_t)nc, s );
		e |= grow( (void**)&w->jointList, 4u * (size_t)w->jointCap, 4u * (size_t)nc, s );
		w->jointCap = nc;
	}
	(void)listCap;
	/* new arrays are cleared and filled in stream order; the host reads device arrays
	 * only through copies on the same stream */
	return e;
}

/* Copies between host and device on stream s, counted in the world's transfer totals. */
static int h2d( b2gDevWorld* w, void* dst, const void* src, size_t bytes, cudaStream_t s )
{
	if ( bytes == 0 )
		return 0;
	w->h2dBytes += (long long)bytes;
	return ok( cudaMemcpyAsync( dst, src, bytes, cudaMemcpyHostToDevice, s ) );
}

static int d2h( b2gDevWorld* w, void* dst, const void* src, size_t bytes, cudaStream_t s )
{
	if ( bytes == 0 )
		return 0;
	w->d2hBytes += (long long)bytes;
	return ok( cudaMemcpyAsync( dst, src, bytes, cudaMemcpyDeviceToHost, s ) );
}

extern "C" int b2gd_upload_bodies( b2gDevWorld* w, const float* state, const float* xf, const float* centers, const float* prev,
								   const float* mass, const float* force, const float* extent, const int* info, int count )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	size_t n4 = 16u * (size_t)count;
	int e = 0;
	e |= h2d( w, w->state, state, 2 * n4, s );
	e |= h2d( w, w->xf, xf, n4, s );
	e |= h2d( w, w->centers, centers, n4, s );
	e |= h2d( w, w->prev, prev, n4, s );
	e |= h2d( w, w->mass, mass, n4, s );
	e |= h2d( w, w->force, force, n4, s );
	e |= h2d( w, w->extent, extent, n4, s );
	e |= h2d( w, w->bodyInfo, info, 4u * (size_t)count, s );
	return e;
}

/* Sleep timers (zero) and the mapped list of bodies past the sleep time, made when a
 * world first steps with sleep on; a world that never sleeps holds neither and its
 * finalisation skips the timers. */
extern "C" int b2gd_reserve_sleep( b2gDevWorld* w, b2gHostIO* io )
{
	int e = 0;
	if ( w->sleepTime == nullptr )
		e |= grow( (void**)&w->sleepTime, 0, 4u * (size_t)w->bodyCap, (cudaStream_t)w->stream );
	if ( w->sleepyCap < w->bodyCap || io->sleepy == nullptr )
	{
		e |= grow_host_mapped( (void**)&io->sleepy, (void**)&w->sleepy, 8u * (size_t)w->bodyCap );
		w->sleepyCap = e == 0 ? w->bodyCap : 0;
	}
	return e;
}

/* Device staging of body operations, grown on demand. */
extern "C" int b2gd_reserve_body_ops( b2gDevWorld* w, int count )
{
	if ( count <= w->bodyOpsCap && w->bodyOps != nullptr )
		return 0;
	int cap = w->bodyOpsCap < 64 ? 64 : w->bodyOpsCap;
	while ( cap < count )
		cap *= 2;
	int e = grow( (void**)&w->bodyOps, 0, 4u * (size_t)cap, (cudaStream_t)w->stream );
	w->bodyOpsCap = e == 0 ? cap : 0;
	return e;
}

extern "C" int b2gd_upload_awake( b2gDevWorld* w, const int* awake, int count )
{
	return h2d( w, w->awake, awake, 4u * (size_t)count, (cudaStream_t)w->stream );
}

extern "C" int b2gd_upload_shapes( b2gDevWorld* w, const b2gShapeGeo* geo, const float* aabb, const float* fat, int count )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int e = h2d( w, w->geo, geo, sizeof( b2gShapeGeo ) * (size_t)count, s );
	e |= h2d( w, w->aabb, aabb, 16u * (size_t)count, s );
	e |= h2d( w, w->fat, fat, 16u * (size_t)count, s );
	return e;
}

extern "C" int b2gd_upload_shape_lists( b2gDevWorld* w, const int* range, int bodyCount, const int* list, int listCount )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int e = h2d( w, w->shapeRange, range, 8u * (size_t)bodyCount, s );
	e |= h2d( w, w->shapeList, list, 4u * (size_t)listCount, s );
	return e;
}

extern "C" int b2gd_upload_joints( b2gDevWorld* w, const b2gJointDev* joints, int count )
{
	return h2d( w, w->joints, joints, sizeof( b2gJointDev ) * (size_t)count, (cudaStream_t)w->stream );
}

extern "C" int b2gd_upload_solve_lists( b2gDevWorld* w, const int* solveList, int solveCount, const int* jointList, int jointCount )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int e = h2d( w, w->solveList, solveList, 4u * (size_t)solveCount, s );
	e |= h2d( w, w->jointList, jointList, 4u * (size_t)jointCount, s );
	return e;
}

extern "C" int b2gd_upload_fat( b2gDevWorld* w, int shapeId, const float* fat4 )
{
	return h2d( w, (char*)w->fat + 16u * (size_t)shapeId, fat4, 16u, (cudaStream_t)w->stream );
}

extern "C" int b2gd_upload_pose( b2gDevWorld* w, int bodyId, const float* xf4, const float* center4, const float* prev4 )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	size_t at = 16u * (size_t)bodyId;
	int e = h2d( w, (char*)w->xf + at, xf4, 16u, s );
	e |= h2d( w, (char*)w->centers + at, center4, 16u, s );
	e |= h2d( w, (char*)w->prev + at, prev4, 16u, s );
	return e;
}

extern "C" int b2gd_upload_shape_boxes( b2gDevWorld* w, int shapeId, const float* aabb4, const float* fat4 )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	size_t at = 16u * (size_t)shapeId;
	int e = h2d( w, (char*)w->aabb + at, aabb4, 16u, s );
	e |= h2d( w, (char*)w->fat + at, fat4, 16u, s );
	return e;
}

extern "C" int b2gd_upload_body_velocity( b2gDevWorld* w, int bodyId, const float* v3 )
{
	return h2d( w, (char*)w->state + 32u * (size_t)bodyId, v3, 12u, (cudaStream_t)w->stream );
}

extern "C" int b2gd_download_bodies( b2gDevWorld* w, float* state, float* xf, float* centers, int count )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	size_t n4 = 16u * (size_t)count;
	int e = d2h( w, state, w->state, 2 * n4, s );
	e |= d2h( w, xf, w->xf, n4, s );
	e |= d2h( w, centers, w->centers, n4, s );
	e |= ok( cudaStreamSynchronize( s ) );
	return e;
}

/* Hit test of one contact (reference src/solver.c:1688-1712): the point with the largest
 * approach speed above the threshold among the points that carry a normal impulse. */
__global__ void k_hit_events( const b2gManifold* manifolds, const int* ids, int n, float threshold, float4* out )
{
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if ( k >= n )
		return;
	const b2gManifold* m = manifolds + ids[k];
	float approach = threshold;
	float hit = 0.0f;
	b2gVec point = gv( 0.0f, 0.0f );
	for ( int j = 0; j < m->count; ++j )
	{
		const b2gPoint* mp = m->pts + j;
		float s = -mp->normalVelocity;
		if ( s > approach && mp->normalImpulse > 0.0f )
		{
			approach = s;
			point = mp->point;
			hit = 1.0f;
		}
	}
	out[2 * k] = make_float4( hit, approach, point.x, point.y );
	out[2 * k + 1] = make_float4( m->normal.x, m->normal.y, 0.0f, 0.0f );
}

extern "C" int b2gd_reserve_hits( b2gHostIO* io, int n )
{
	if ( n <= io->hitCap )
		return 0;
	int cap = n < 256 ? 256 : n + n / 2;
	if ( io->hitIds )
		cudaFreeHost( io->hitIds );
	if ( io->hitOut )
		cudaFreeHost( io->hitOut );
	io->hitIds = nullptr;
	io->hitOut = nullptr;
	io->hitCap = 0;
	int e = ok( cudaHostAlloc( (void**)&io->hitIds, sizeof( int ) * (size_t)cap, cudaHostAllocMapped ) );
	e |= ok( cudaHostAlloc( (void**)&io->hitOut, sizeof( float ) * 8u * (size_t)cap, cudaHostAllocMapped ) );
	if ( e == 0 )
		io->hitCap = cap;
	return e;
}

extern "C" int b2gd_hit_events( b2gDevWorld* w, b2gHostIO* io, int n, float threshold )
{
	if ( n <= 0 )
		return 0;
	cudaStream_t s = (cudaStream_t)w->stream;
	int* dIds = nullptr;
	float4* dOut = nullptr;
	int e = ok( cudaHostGetDevicePointer( (void**)&dIds, io->hitIds, 0 ) );
	e |= ok( cudaHostGetDevicePointer( (void**)&dOut, io->hitOut, 0 ) );
	if ( e )
		return e;
	k_hit_events<<<( n + 127 ) / 128, 128, 0, s>>>( w->manifold, dIds, n, threshold, dOut );
	w->launches += 1;
	w->h2dBytes += 4 * (long long)n;
	w->d2hBytes += 32 * (long long)n;
	e = ok( cudaGetLastError() );
	e |= ok( cudaStreamSynchronize( s ) );
	return e;
}

extern "C" int b2gd_download_manifolds( b2gDevWorld* w, b2gManifold* out, uint32_t* flags, int count )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int e = d2h( w, out, w->manifold, sizeof( b2gManifold ) * (size_t)count, s );
	if ( flags )
		e |= d2h( w, flags, w->cFlags, 4u * (size_t)count, s );
	e |= ok( cudaStreamSynchronize( s ) );
	return e;
}

extern "C" int b2gd_download_shapes( b2gDevWorld* w, float* aabb, float* fat, int count )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int e = d2h( w, aabb, w->aabb, 16u * (size_t)count, s );
	e |= d2h( w, fat, w->fat, 16u * (size_t)count, s );
	e |= ok( cudaStreamSynchronize( s ) );
	return e;
}

extern "C" int b2gd_download_joints( b2gDevWorld* w, b2gJointDev* joints, int count )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	int e = d2h( w, joints, w->joints, sizeof( b2gJointDev ) * (size_t)count, s );
	e |= ok( cudaStreamSynchronize( s ) );
	return e;
}

extern "C" int b2gd_sync( b2gDevWorld* w )
{
	return ok( cudaStreamSynchronize( (cudaStream_t)w->stream ) );
}

extern "C" void b2gd_enable_timing( b2gDevWorld* w, int flag )
{
	if ( flag && w->timers[0] == nullptr )
	{
		for ( int i = 0; i < 8; ++i )
		{
			cudaEvent_t e;
			cudaEventCreate( &e );
			w->timers[i] = (void*)e;
		}
	}
	w->timing = flag && w->timers[0] != nullptr;
}

static float elapsed( void* a, void* b )
{
	float ms = 0.0f;
	if ( cudaEventElapsedTime( &ms, (cudaEvent_t)a, (cudaEvent_t)b ) != cudaSuccess )
		return 0.0f;
	return ms;
}

extern "C" void b2gd_mark( b2gDevWorld* w, int slot )
{
	if ( w->timing )
		cudaEventRecord( (cudaEvent_t)w->timers[slot], (cudaStream_t)w->stream );
}

extern "C" void b2gd_stage_times( b2gDevWorld* w, float* stepMs, float* collideMs, float* solveMs, float* finalizeMs )
{
	*stepMs = *collideMs = *solveMs = *finalizeMs = 0.0f;
	if ( w->timing == 0 )
		return;
	cudaEventSynchronize( (cudaEvent_t)w->timers[6] );
	*stepMs = elapsed( w->timers[0], w->timers[6] );
	*collideMs = elapsed( w->timers[1], w->timers[2] );
	*solveMs = elapsed( w->timers[3], w->timers[4] );
	*finalizeMs = elapsed( w->timers[4], w->timers[5] );
}

/* Raw device readback for diagnostics: 0 contact flags (u32), 1 shape geometry,
 * 2 contact shape pairs (2 x i32), 3 body info (i32). */
extern "C" int b2gd_debug_read( b2gDevWorld* w, int which, void* out, int count )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	const void* src = nullptr;
	size_t bytes = 0;
	switch ( which )
	{
		case 0:
			src = w->cFlags;
			bytes = 4u * (size_t)count;
			break;
		case 1:
			src = w->geo;
			bytes = sizeof( b2gShapeGeo ) * (size_t)count;
			break;
		case 2:
			src = w->cShapes;
			bytes = 8u * (size_t)count;
			break;
		case 3:
			src = w->bodyInfo;
			bytes = 4u * (size_t)count;
			break;
		case 4:
			src = w->counters;
			bytes = 16u;
			break;
		default:
			return -1;
	}
	if ( src == nullptr )
		return -2;
	int e = ok( cudaMemcpyAsync( out, src, bytes, cudaMemcpyDeviceToHost, s ) );
	e |= ok( cudaStreamSynchronize( s ) );
	return e;
}
