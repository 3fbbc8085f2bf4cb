/*
 * pool.c -- a small fork-join thread pool for the host side of batched steps: the
 * per-world host work of b2World_StepBatch is independent between worlds, and touching
 * thousands of separately allocated worlds is bound by memory latency, so it spreads
 * over the host's cores.
 *
 * gpool_for( count, grain, fn, ctx ) calls fn( begin, end, ctx ) over [0, count) in
 * chunks of `grain`, on the calling thread and the pool's workers, and returns when all
 * chunks are done.  One job runs at a time: gpool_for waits for the pool, gpool_try_for
 * returns false at once when the pool is busy (another thread's job, or a call from
 * inside a job) and the caller runs the range itself.  gpool_for must not nest.
 */
#include "host.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <unistd.h>

#define POOL_MAX_THREADS 32

typedef struct gPool
{
	pthread_t threads[POOL_MAX_THREADS];
	int workers;
	pthread_mutex_t lock;
	pthread_cond_t wake;
	pthread_cond_t done;
	uint64_t generation;
	gTaskFn* fn;
	void* ctx;
	int count, grain;
	atomic_int next;
	int active; /* workers still inside the current job */
} gPool;

static gPool s_pool;
static pthread_once_t s_once = PTHREAD_ONCE_INIT;
static pthread_mutex_t s_job = PTHREAD_MUTEX_INITIALIZER; /* held while a job runs */

static void run_chunks( gPool* p )
{
	for ( ;; )
	{
		int begin = atomic_fetch_add( &p->next, p->grain );
		if ( begin >= p->count )
			break;
		int end = begin + p->grain < p->count ? begin + p->grain : p->count;
		p->fn( begin, end, p->ctx );
	}
}

static void* worker( void* arg )
{
	gPool* p = (gPool*)arg;
	uint64_t seen = 0;
	pthread_mutex_lock( &p->lock );
	for ( ;; )
	{
		while ( p->generation == seen )
			pthread_cond_wait( &p->wake, &p->lock );
		seen = p->generation;
		pthread_mutex_unlock( &p->lock );
		run_chunks( p );
		pthread_mutex_lock( &p->lock );
		p->active -= 1;
		if ( p->active == 0 )
			pthread_cond_signal( &p->done );
	}
	return NULL;
}

static void pool_start( void )
{
	gPool* p = &s_pool;
	pthread_mutex_init( &p->lock, NULL );
	pthread_cond_init( &p->wake, NULL );
	pthread_cond_init( &p->done, NULL );
	long cores = sysconf( _SC_NPROCESSORS_ONLN );
	int n = cores > 1 ? (int)cores - 1 : 0;
	n = n > POOL_MAX_THREADS ? POOL_MAX_THREADS : n;
	int started = 0;
	for ( int i = 0; i < n; ++i )
	{
		if ( pthread_create( p->threads + started, NULL, worker, p ) == 0 )
			started += 1;
	}
	p->workers = started;
}

int gpool_threads( void )
{
	pthread_once( &s_once, pool_start );
	return s_pool.workers + 1;
}

static void run_job( int count, int grain, gTaskFn* fn, void* ctx )
{
	gPool* p = &s_pool;
	pthread_mutex_lock( &p->lock );
	p->fn = fn;
	p->ctx = ctx;
	p->count = count;
	p->grain = grain;
	atomic_store( &p->next, 0 );
	p->active = p->workers;
	p->generation += 1;
	pthread_cond_broadcast( &p->wake );
	pthread_mutex_unlock( &p->lock );
	run_chunks( p );
	pthread_mutex_lock( &p->lock );
	while ( p->active > 0 )
		pthread_cond_wait( &p->done, &p->lock );
	pthread_mutex_unlock( &p->lock );
}

void gpool_for( int count, int grain, gTaskFn* fn, void* ctx )
{
	if ( count <= 0 )
		return;
	grain = grain < 1 ? 1 : grain;
	pthread_once( &s_once, pool_start );
	if ( s_pool.workers == 0 || count <= grain )
	{
		fn( 0, count, ctx );
		return;
	}
	pthread_mutex_lock( &s_job );
	run_job( count, grain, fn, ctx );
	pthread_mutex_unlock( &s_job );
}

bool gpool_try_for( int count, int grain, gTaskFn* fn, void* ctx )
{
	if ( count <= 0 )
		return true;
	grain = grain < 1 ? 1 : grain;
	pthread_once( &s_once, pool_start );
	if ( s_pool.workers == 0 || count <= grain )
		return false;
	if ( pthread_mutex_trylock( &s_job ) != 0 )
		return false;
	run_job( count, grain, fn, ctx );
	pthread_mutex_unlock( &s_job );
	return true;
}
