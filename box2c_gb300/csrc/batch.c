/*
 * batch.c -- b2World_StepBatch: one step of many independent worlds with the device
 * work of all of them in two replayed CUDA graphs (narrowphase, then solver and
 * finalisation).
 *
 * The host work of each world is the single-world step's, phase by phase (step.c:
 * gstep_begin, gstep_rebuild_trees, gstep_after_collide, gstep_finish); only the device
 * launches are shared.  While the batch runs, every world's uploads go to the batch's
 * stream, so they are ordered before the graphs that read them.
 */
#include "host.h"

#include "box2d/gpu.h"

#include <stdlib.h>
#include <string.h>

/* A step is split in two halves only when its worlds hold at least this many bodies:
 * below it the device work is too short to hide the host work of the other half behind,
 * and the second set of launches and waits costs more than the overlap gains. */
#define BATCH_SPLIT_BODIES 100000

static b2gBatch* s_batch;
static gWorld** s_worlds;
static void** s_streams;
static b2WorldId* s_alone; /* worlds too large for the batched solver, stepped alone */
static int s_cap;

static bool reserve_worlds( int count )
{
	if ( count <= s_cap )
		return true;
	int cap = count < 64 ? 64 : count;
	gWorld** w = (gWorld**)b2g_realloc( s_worlds, sizeof( gWorld* ) * (size_t)cap );
	if ( w == NULL )
		return false;
	s_worlds = w;
	void** s = (void**)b2g_realloc( s_streams, sizeof( void* ) * (size_t)cap );
	if ( s == NULL )
		return false;
	s_streams = s;
	b2WorldId* a = (b2WorldId*)b2g_realloc( s_alone, sizeof( b2WorldId ) * (size_t)cap );
	if ( a == NULL )
		return false;
	s_alone = a;
	s_cap = cap;
	return true;
}

static void fill_item( b2gBatchItem* it, gWorld* w )
{
	it->W = w->dev;
	it->bodyIdCount = w->bodyIds.next;
}

/* One half of the step's worlds: s_worlds[first .. first + count). */
typedef struct BatchCtx
{
	b2gBatchItem* items;
	void* stream;
	float timeStep;
	int subStepCount;
	int first, count;
	int error;
} BatchCtx;

static void begin_worlds( int begin, int end, void* arg )
{
	BatchCtx* c = (BatchCtx*)arg;
	for ( int k = c->first + begin; k < c->first + end; ++k )
	{
		gWorld* w = s_worlds[k];
		b2gBatchItem* it = c->items + k;
		memset( it, 0, sizeof( *it ) );
		w->beginCount = 0;
		w->endCount = 0;
		memset( &w->profile, 0, sizeof( w->profile ) );
		s_streams[k] = w->dev.stream;
		w->dev.stream = c->stream;
		w->batching = true;
		w->tapeBodyDst = NULL;
		w->dev.h2dBytes = 0;
		w->dev.d2hBytes = 0;
		gworld_flush( w );
		int staged = gstep_begin( w );
		if ( staged < 0 )
			continue;
		if ( b2gd_stage_contacts( &w->dev, &w->io, staged ) != 0 )
		{
			w->status = -1;
			continue;
		}
		fill_item( it, w );
		it->idCount = w->stepIdCount;
		it->staged = staged;
	}
}

static void rebuild_worlds( int begin, int end, void* arg )
{
	BatchCtx* c = (BatchCtx*)arg;
	for ( int k = c->first + begin; k < c->first + end; ++k )
		if ( s_worlds[k]->status == 0 )
			gstep_rebuild_trees( s_worlds[k] );
}

static void middle_worlds( int begin, int end, void* arg )
{
	BatchCtx* c = (BatchCtx*)arg;
	for ( int k = c->first + begin; k < c->first + end; ++k )
	{
		gWorld* w = s_worlds[k];
		b2gBatchItem* it = c->items + k;
		if ( c->error != 0 )
			w->status = c->error;
		if ( w->status != 0 )
		{
			it->solve = 0;
			continue;
		}
		w->io.counters[0] = b2gd_batch_counters( s_batch, k )[0];
		b2gStepConst sc;
		b2gSolvePlan plan;
		int run = gstep_after_collide( w, c->timeStep, c->subStepCount, &sc, &plan );
		/* uploads above may have grown the arena: copy the descriptor again */
		fill_item( it, w );
		it->solve = run && w->status == 0;
		if ( it->solve == 0 )
			continue;
		it->sc = sc;
		memcpy( it->colorStart, plan.colorStart, sizeof( it->colorStart ) );
		memcpy( it->jointStart, plan.jointStart, sizeof( it->jointStart ) );
		memcpy( it->active, plan.active, sizeof( it->active ) );
		it->activeCount = plan.activeCount;
		it->awakeCount = plan.awakeCount;
		it->bodyIdCount = plan.bodyIdCount;
		it->widest = 0;
		for ( int a = 0; a < plan.activeCount; ++a )
		{
			int col = plan.active[a];
			int nr = plan.colorStart[col + 1] - plan.colorStart[col] + plan.jointStart[col + 1] - plan.jointStart[col];
			it->widest = nr > it->widest ? nr : it->widest;
		}
		if ( w->tapeBodyDst )
		{
			it->tapeBodies = w->tapeBodyDst;
			it->tapeRowDst = w->tapeRowDst;
			it->tapeRows = w->tapeRowCount;
			w->tapeBodyDst = NULL;
		}
	}
}

static void finish_worlds( int begin, int end, void* arg )
{
	BatchCtx* c = (BatchCtx*)arg;
	for ( int k = c->first + begin; k < c->first + end; ++k )
	{
		gWorld* w = s_worlds[k];
		if ( c->error != 0 && w->status == 0 )
			w->status = c->error;
		if ( c->items[k].solve && w->status == 0 )
		{
			w->io.counters[1] = b2gd_batch_counters( s_batch, k )[1];
			w->io.counters[3] = b2gd_batch_counters( s_batch, k )[3];
			gstep_finish( w );
		}
		w->dev.stream = s_streams[k];
		w->batching = false;
		w->dev.launches = 0;
		w->dev.fusedUsed = 0;
		w->mirrorStale = true;
		w->shapeMirrorStale = true;
		w->jointMirrorStale = true;
	}
}

static float s_hostMs[5];

void b2World_StepBatch( const b2WorldId* worldIds, int count, float timeStep, int subStepCount )
{
	if ( worldIds == NULL || count <= 0 || timeStep == 0.0f )
		return;
	if ( s_batch == NULL )
	{
		s_batch = b2gd_batch_create();
		if ( s_batch == NULL )
			return;
	}
	if ( reserve_worlds( count ) == false )
		return;

	/* valid, healthy, distinct worlds; the ones whose bodies do not fit the batched
	 * solver's shared memory are stepped alone after the batch */
	int n = 0, alone = 0;
	const int maxBodies = b2gd_batch_max_bodies();
	for ( int i = 0; i < count; ++i )
	{
		if ( b2World_IsValid( worldIds[i] ) == false )
			continue;
		gWorld* w = gworld_get( worldIds[i] );
		if ( w->locked || w->status != 0 )
			continue;
		w->locked = true;
		if ( w->bodyIds.next > maxBodies )
			s_alone[alone++] = worldIds[i];
		else
			s_worlds[n++] = w;
	}
	for ( int k = 0; k < alone; ++k )
	{
		gworld_get( s_alone[k] )->locked = false;
		b2World_Step( s_alone[k], timeStep, subStepCount );
	}
	if ( n == 0 )
		return;
	b2gBatchItem* items = b2gd_batch_items( s_batch, n );
	if ( items == NULL )
	{
		for ( int k = 0; k < n; ++k )
			s_worlds[k]->locked = false;
		return;
	}
	/* two halves (one when there are few worlds): the host phases of one half run while
	 * the device works on the other */
	BatchCtx c[2];
	long long bodies = 0;
	for ( int k = 0; k < n; ++k )
		bodies += s_worlds[k]->bodyIds.next;
	int split = n >= 2 && bodies >= BATCH_SPLIT_BODIES ? n / 2 : n;
	for ( int h = 0; h < 2; ++h )
	{
		c[h].items = items;
		c[h].stream = b2gd_batch_stream( s_batch );
		c[h].timeStep = timeStep;
		c[h].subStepCount = subStepCount;
		c[h].first = h == 0 ? 0 : split;
		c[h].count = h == 0 ? split : n - split;
		c[h].error = 0;
	}
	const int grain = 16;
	b2gd_batch_begin_step( s_batch );

	double t0 = b2g_now_ms();
	gpool_for( c[0].count, grain, begin_worlds, &c[0] );
	double t1 = b2g_now_ms();
	c[0].error = b2gd_batch_collide( s_batch, 0, c[0].first, c[0].count );
	gpool_for( c[1].count, grain, begin_worlds, &c[1] );
	c[1].error = b2gd_batch_collide( s_batch, 1, c[1].first, c[1].count );
	gpool_for( c[0].count, grain, rebuild_worlds, &c[0] );
	gpool_for( c[1].count, grain, rebuild_worlds, &c[1] );
	double t2 = b2g_now_ms();
	for ( int h = 0; h < 2; ++h )
	{
		c[h].error |= b2gd_batch_wait_collide( s_batch, h );
		gpool_for( c[h].count, grain, middle_worlds, &c[h] );
		if ( c[h].error == 0 )
			c[h].error = b2gd_batch_solve( s_batch, h, c[h].first, c[h].count );
	}
	double t3 = b2g_now_ms();
	for ( int h = 0; h < 2; ++h )
	{
		c[h].error |= b2gd_batch_wait_solve( s_batch, h );
		gpool_for( c[h].count, grain, finish_worlds, &c[h] );
	}
	double t4 = b2g_now_ms();
	int e = b2gd_batch_end_step( s_batch );
	double t5 = b2g_now_ms();
	if ( e != 0 )
	{
		for ( int k = 0; k < n; ++k )
			if ( s_worlds[k]->status == 0 )
				s_worlds[k]->status = e;
	}
	s_hostMs[0] = (float)( t1 - t0 );
	s_hostMs[1] = (float)( t2 - t1 );
	s_hostMs[2] = (float)( t3 - t2 );
	s_hostMs[3] = (float)( t4 - t3 );
	s_hostMs[4] = (float)( t5 - t4 );
	for ( int k = 0; k < n; ++k )
	{
		gWorld* w = s_worlds[k];
		w->locked = false;
		w->profile.step = (float)( t5 - t0 ) / (float)n;
		if ( w->status )
			gworld_fail( b2gd_last_error() );
	}
}

b2BatchStats b2World_GetBatchStats( void )
{
	b2BatchStats s;
	memset( &s, 0, sizeof( s ) );
	if ( s_batch != NULL )
		b2gd_batch_stats( s_batch, &s.collide, &s.solve, &s.solveThreads, &s.solveCtasPerSm, &s.launches );
	s.hostBegin = s_hostMs[0];
	s.hostCollide = s_hostMs[1];
	s.hostMiddle = s_hostMs[2];
	s.hostSolve = s_hostMs[3];
	s.hostFinish = s_hostMs[4];
	s.hostThreads = gpool_threads();
	return s;
}
