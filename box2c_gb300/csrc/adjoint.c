/*
 * adjoint.c -- host side of differentiable stepping: per-world tapes and the
 * b2World_StepBackward / b2World_StepBackwardBatch entry points (include/box2d/gpu.h).
 *
 * A tape is one device buffer per world.  Each recorded step appends its body records
 * (4 float4 per body id) and solver rows (b2gTapeRow) on the world's stream and keeps a
 * host header (b2gTapeStep) with their offsets, the solve plan and the step constants.
 * The backward call uploads the headers, the loss gradient and the shape frictions of
 * every world, launches the backward kernel (one warp per world) and downloads the
 * gradients.
 */
#include "host.h"

#include "box2d/gpu.h"

#include <cuda_runtime_api.h>

#include <stdlib.h>
#include <string.h>

typedef struct gTape
{
	int maxSteps, steps;
	int bodies;	 /* body ids when recording began */
	int maxRows; /* most rows of a recorded step */
	char* dev;
	size_t cap, used;
	b2gTapeStep* hdr;
} gTape;

void gtape_free( gWorld* w )
{
	gTape* t = w->tape;
	if ( t == NULL )
		return;
	if ( t->dev )
		cudaFree( t->dev );
	b2g_free( t->hdr );
	b2g_free( t );
	w->tape = NULL;
}

void b2World_BeginTape( b2WorldId worldId, int maxSteps )
{
	if ( b2World_IsValid( worldId ) == false )
		return;
	gWorld* w = gworld_get( worldId );
	if ( maxSteps <= 0 )
	{
		gtape_free( w );
		return;
	}
	gTape* t = w->tape;
	if ( t == NULL )
	{
		t = (gTape*)b2g_calloc( 1, sizeof( gTape ) );
		if ( t == NULL )
			return;
		w->tape = t;
	}
	if ( maxSteps > t->maxSteps )
	{
		b2gTapeStep* h = (b2gTapeStep*)b2g_realloc( t->hdr, sizeof( b2gTapeStep ) * (size_t)maxSteps );
		if ( h == NULL )
			return;
		t->hdr = h;
	}
	t->maxSteps = maxSteps;
	t->steps = 0;
	t->used = 0;
	t->maxRows = 0;
	t->bodies = w->bodyIds.next;
	w->tapeToiEvents = 0;
}

int b2World_GetTapeSteps( b2WorldId worldId )
{
	if ( b2World_IsValid( worldId ) == false )
		return 0;
	gTape* t = gworld_get( worldId )->tape;
	return t ? t->steps : 0;
}

static size_t round_up( size_t v, size_t a ) { return ( v + a - 1 ) / a * a; }

void gtape_record( gWorld* w, const b2gSolvePlan* plan, const b2gStepConst* sc, int solve )
{
	gTape* t = w->tape;
	if ( t == NULL || t->steps >= t->maxSteps || w->status != 0 )
		return;
	int bodies = w->bodyIds.next;
	int rows = solve ? plan->colorStart[B2G_COLORS] : 0;
	if ( bodies != t->bodies )
	{
		/* bodies created or destroyed while recording: the tape ends here */
		t->maxSteps = t->steps;
		return;
	}
	size_t rowByte = round_up( t->used, sizeof( b2gTapeRow ) );
	size_t bodyByte = round_up( rowByte + sizeof( b2gTapeRow ) * (size_t)rows, 64 );
	size_t end = bodyByte + 64u * (size_t)bodies;
	if ( end > t->cap )
	{
		size_t cap = t->cap < ( 1u << 20 ) ? ( 1u << 20 ) : t->cap;
		while ( cap < end )
			cap *= 2;
		char* p = NULL;
		if ( cudaMalloc( (void**)&p, cap ) != cudaSuccess )
		{
			w->status = -1;
			return;
		}
		if ( t->dev )
		{
			cudaStreamSynchronize( (cudaStream_t)w->dev.stream );
			cudaMemcpy( p, t->dev, t->used, cudaMemcpyDeviceToDevice );
			cudaFree( t->dev );
		}
		t->dev = p;
		t->cap = cap;
	}
	b2gTapeStep* h = t->hdr + t->steps;
	memset( h, 0, sizeof( *h ) );
	h->bodyOff = (int64_t)( bodyByte / 16 );
	h->rowOff = (int64_t)( rowByte / sizeof( b2gTapeRow ) );
	h->bodies = bodies;
	h->rows = rows;
	h->solve = solve;
	h->sc = *sc;
	if ( solve )
	{
		memcpy( h->colorStart, plan->colorStart, sizeof( h->colorStart ) );
		memcpy( h->jointStart, plan->jointStart, sizeof( h->jointStart ) );
		memcpy( h->active, plan->active, sizeof( h->active ) );
		h->activeCount = plan->activeCount;
		h->awakeCount = plan->awakeCount;
	}
	if ( w->batching )
	{
		/* recorded by the batch's solver graph */
		w->tapeBodyDst = t->dev + bodyByte;
		w->tapeRowDst = t->dev + rowByte;
		w->tapeRowCount = rows;
	}
	else
	{
		int e = b2gd_tape_record( &w->dev, t->dev + bodyByte, bodies, t->dev + rowByte, rows );
		if ( e )
		{
			w->status = e;
			return;
		}
	}
	t->used = end;
	t->maxRows = rows > t->maxRows ? rows : t->maxRows;
	t->steps += 1;
}

/* ------------------------------------------------------------------ backward */
typedef struct gAdjointCtx
{
	cudaStream_t stream;
	b2gAdjointItem* hItems;
	b2gAdjointItem* dItems;
	int itemCap;
	char* hBuf; /* pinned staging: headers, gradients, frictions, statuses */
	char* dBuf;
	size_t bufCap;
	float* scratch;
	size_t scratchCap;
} gAdjointCtx;

static gAdjointCtx s_adj;
static int s_lastCheck[2];

void b2World_GetBackwardCheck( int* manifoldMismatches, int* replayMismatches )
{
	*manifoldMismatches = s_lastCheck[0];
	*replayMismatches = s_lastCheck[1];
}

static int ensure_ctx( int count, size_t bufBytes, size_t scratchFloats )
{
	if ( s_adj.stream == NULL && cudaStreamCreateWithFlags( &s_adj.stream, cudaStreamNonBlocking ) != cudaSuccess )
		return -1;
	if ( count > s_adj.itemCap )
	{
		cudaFreeHost( s_adj.hItems );
		cudaFree( s_adj.dItems );
		s_adj.hItems = NULL;
		s_adj.dItems = NULL;
		s_adj.itemCap = 0;
		if ( cudaMallocHost( (void**)&s_adj.hItems, sizeof( b2gAdjointItem ) * (size_t)count ) != cudaSuccess ||
			 cudaMalloc( (void**)&s_adj.dItems, sizeof( b2gAdjointItem ) * (size_t)count ) != cudaSuccess )
			return -1;
		s_adj.itemCap = count;
	}
	if ( bufBytes > s_adj.bufCap )
	{
		cudaFreeHost( s_adj.hBuf );
		cudaFree( s_adj.dBuf );
		s_adj.hBuf = NULL;
		s_adj.dBuf = NULL;
		s_adj.bufCap = 0;
		if ( cudaMallocHost( (void**)&s_adj.hBuf, bufBytes ) != cudaSuccess || cudaMalloc( (void**)&s_adj.dBuf, bufBytes ) != cudaSuccess )
			return -1;
		s_adj.bufCap = bufBytes;
	}
	if ( scratchFloats > s_adj.scratchCap )
	{
		cudaFree( s_adj.scratch );
		s_adj.scratch = NULL;
		s_adj.scratchCap = 0;
		if ( cudaMalloc( (void**)&s_adj.scratch, sizeof( float ) * scratchFloats ) != cudaSuccess )
			return -1;
		s_adj.scratchCap = scratchFloats;
	}
	return 0;
}

int b2World_StepBackwardBatch( const b2WorldId* worldIds, int count, int bodyStride, int shapeStride, const float* gradFinal,
							   float* gradInitial, float* gradFriction )
{
	if ( worldIds == NULL || count <= 0 || gradFinal == NULL || gradInitial == NULL )
		return -1;
	size_t headerBytes = 0, scratchFloats = 0;
	for ( int i = 0; i < count; ++i )
	{
		if ( b2World_IsValid( worldIds[i] ) == false )
			return -1;
		gWorld* w = gworld_get( worldIds[i] );
		gTape* t = w->tape;
		if ( t == NULL || t->steps == 0 || t->bodies > bodyStride || w->shapeIds.next > shapeStride || w->status != 0 )
			return -1;
		headerBytes += sizeof( b2gTapeStep ) * (size_t)t->steps;
		scratchFloats += b2gd_adjoint_scratch( t->bodies, t->maxRows, w->dev.contactCap, 16 );
	}
	size_t gradBytes = sizeof( float ) * (size_t)count * ( 12u * (size_t)bodyStride + 2u * (size_t)shapeStride );
	size_t statusBytes = sizeof( int ) * 4u * (size_t)count;
	size_t bufBytes = round_up( headerBytes, 256 ) + round_up( gradBytes, 256 ) + statusBytes;
	if ( ensure_ctx( count, bufBytes, scratchFloats ) != 0 )
		return -1;

	char* hb = s_adj.hBuf;
	char* db = s_adj.dBuf;
	size_t gradOff = round_up( headerBytes, 256 );
	size_t statusOff = gradOff + round_up( gradBytes, 256 );
	float* hGrad = (float*)( hb + gradOff );
	float* dGrad = (float*)( db + gradOff );
	/* per world: gradFinal (6 x bodyStride), gradInitial (6 x bodyStride), shape friction
	 * (shapeStride), friction gradient (shapeStride) */
	size_t perWorld = 12u * (size_t)bodyStride + 2u * (size_t)shapeStride;
	size_t hdrOff = 0, scratchOff = 0;
	for ( int i = 0; i < count; ++i )
	{
		gWorld* w = gworld_get( worldIds[i] );
		gTape* t = w->tape;
		memcpy( hb + hdrOff, t->hdr, sizeof( b2gTapeStep ) * (size_t)t->steps );
		float* g = hGrad + perWorld * (size_t)i;
		memcpy( g, gradFinal + 6u * (size_t)bodyStride * (size_t)i, sizeof( float ) * 6u * (size_t)t->bodies );
		float* fric = g + 12u * (size_t)bodyStride;
		for ( int s = 0; s < w->shapeIds.next; ++s )
			fric[s] = w->shapes[s].id == s ? w->shapes[s].friction : 0.0f;

		b2gAdjointItem* it = s_adj.hItems + i;
		memset( it, 0, sizeof( *it ) );
		it->W = w->dev;
		it->tapeBodies = (const float*)t->dev;
		it->tapeRows = (const b2gTapeRow*)t->dev;
		it->steps = (const b2gTapeStep*)( db + hdrOff );
		it->stepCount = t->steps;
		it->bodies = t->bodies;
		it->shapes = w->shapeIds.next;
		it->maxRows = t->maxRows;
		it->contactCap = w->dev.contactCap;
		float* dg = dGrad + perWorld * (size_t)i;
		it->gradFinal = dg;
		it->gradInitial = dg + 6u * (size_t)bodyStride;
		it->shapeFriction = dg + 12u * (size_t)bodyStride;
		it->gradFriction = dg + 12u * (size_t)bodyStride + (size_t)shapeStride;
		it->scratch = s_adj.scratch + scratchOff;
		it->status = (int*)( db + statusOff ) + 4 * i;
		hdrOff += sizeof( b2gTapeStep ) * (size_t)t->steps;
		scratchOff += b2gd_adjoint_scratch( t->bodies, t->maxRows, w->dev.contactCap, 16 );
	}
	/* the recordings were made on the worlds' streams */
	if ( cudaDeviceSynchronize() != cudaSuccess )
		return (int)cudaGetLastError();
	cudaStream_t s = s_adj.stream;
	cudaMemcpyAsync( db, hb, statusOff, cudaMemcpyHostToDevice, s );
	cudaMemcpyAsync( s_adj.dItems, s_adj.hItems, sizeof( b2gAdjointItem ) * (size_t)count, cudaMemcpyHostToDevice, s );
	int e = b2gd_adjoint_launch( s_adj.dItems, count, (void*)s );
	cudaMemcpyAsync( hb + gradOff, db + gradOff, statusOff + statusBytes - gradOff, cudaMemcpyDeviceToHost, s );
	cudaError_t se = cudaStreamSynchronize( s );
	if ( e != 0 )
		return e;
	if ( se != cudaSuccess )
		return (int)se;

	int result = 0;
	s_lastCheck[0] = s_lastCheck[1] = 0;
	const int* status = (const int*)( hb + statusOff );
	for ( int i = 0; i < count; ++i )
	{
		gWorld* w = gworld_get( worldIds[i] );
		const float* g = hGrad + perWorld * (size_t)i;
		memcpy( gradInitial + 6u * (size_t)bodyStride * (size_t)i, g + 6u * (size_t)bodyStride, sizeof( float ) * 6u * (size_t)w->tape->bodies );
		if ( gradFriction )
			memcpy( gradFriction + (size_t)shapeStride * (size_t)i, g + 12u * (size_t)bodyStride + (size_t)shapeStride,
					sizeof( float ) * (size_t)w->shapeIds.next );
		s_lastCheck[0] += status[4 * i + 2];
		s_lastCheck[1] += status[4 * i + 3];
		/* a time-of-impact event moved a body outside the recorded solver stage */
		if ( status[4 * i] != 0 || w->tapeToiEvents != 0 )
			result = B2_ADJOINT_UNSUPPORTED;
		else if ( status[4 * i + 1] != 0 && result == 0 )
			result = B2_ADJOINT_REPLAY_MISMATCH;
	}
	return result;
}

int b2World_StepBackward( b2WorldId worldId, const float* gradFinal, float* gradInitial, float* gradFriction )
{
	if ( b2World_IsValid( worldId ) == false )
		return -1;
	gWorld* w = gworld_get( worldId );
	if ( w->tape == NULL )
		return -1;
	return b2World_StepBackwardBatch( &worldId, 1, w->tape->bodies, w->shapeIds.next, gradFinal, gradInitial, gradFriction );
}
